"""Parity of the GB300 force kernel against the reference's CPU_AOS outputs
(golden fixtures), the CPU oracle and an FP64 all-pairs sum."""
import numpy as np
import pytest

from conftest import GOLDEN_FORCE_CASES, golden
from oracle import oracle as O

import nbody_gb300 as nb

pytestmark = pytest.mark.gpu

# Per-body |F - F_ref| / |F_ref| against the reference's CPU_AOS (the path's
# accuracy gate), and against the FP64 all-pairs sum of the same FP32 inputs.
# On the golden fixtures the reference's own CPU_AOS is up to 1.8e-6 (RMS
# 1.7e-7) from FP64 and a sequential IEEE binary32 sum up to 3.1e-6 (RMS
# 9.6e-7); the bounds below sit above both.
TOL_VS_REFERENCE = 1e-5
TOL_VS_FP64 = 5e-6
RMS_VS_FP64 = 1e-6


def _gpu_force(pm_np, eps2, config=-1, nsplit=-1):
    import torch
    pm = torch.from_numpy(np.ascontiguousarray(pm_np, np.float32)).cuda()
    f = nb.force(pm, eps2, config=config, nsplit=nsplit)
    torch.cuda.synchronize()
    assert nb.last_status() == 0
    return f.cpu().numpy()


def _within_reference(out, ref, f64, tol=TOL_VS_REFERENCE):
    """Per body |F - F_ref| <= tol |F_ref| + |F_ref - F_64|: the gate against
    the reference, not counting the reference's own distance from the exact
    (FP64) sum against the kernel.  That distance matters only for bodies
    whose force nearly cancels (|F| a few % of the mean), where a binary32
    sequential sum is itself up to ~1e-5 off and so is any other order of
    summation."""
    d = np.linalg.norm(out[:, :3] - ref[:, :3], axis=1)
    r = np.linalg.norm(ref[:, :3], axis=1)
    own = np.linalg.norm(ref[:, :3] - f64[:, :3], axis=1)
    return bool(np.all(d <= tol * r + own))


def _f64_as4(pm, eps2, idx=None):
    f = O.ieee().forces_f64(pm, float(np.float32(eps2)), idx)
    out = np.zeros((f.shape[0], 4))
    out[:, :3] = f
    return out


@pytest.mark.parametrize("case", GOLDEN_FORCE_CASES)
def test_drop_in_entry_matches_reference(cuda, case):
    import torch
    g = golden(case)
    pm = torch.from_numpy(g["posMass"]).cuda()
    n = pm.shape[0]
    f = torch.full((n, 4), 7.0, device="cuda")
    ms = nb.ComputeGravitation_GPU_GB300(f, pm, float(g["eps2"]), n)
    assert ms > 0.0
    out = f.cpu().numpy()
    assert np.all(out[:, 3] == 0.0)
    mx, rms = O.per_body_rel_error(out, g["force_aos"])
    assert mx <= TOL_VS_REFERENCE, (mx, rms)
    mx64, rms64 = O.per_body_rel_error(out, g["force_f64"])
    assert mx64 <= TOL_VS_FP64 and rms64 <= RMS_VS_FP64
    # the reference's own crosscheck metric is reported, not asserted, by the
    # reference (src/nbody.cu:1049-1050); same here, but it must be finite
    assert np.isfinite(nb.crosscheck_max_rel_error(out, g["force_aos"]))


NUM_CONFIGS = 48
LOG_DOMAIN_CONFIGS = range(27, 48)  # every fourth source pair in the log domain
NEGATIVE_MASS = 0x8  # NBGB_STATUS_NEGATIVE_MASS


def test_configuration_table_size():
    assert len(nb.force_config_names()) == NUM_CONFIGS
    assert all(nb.force_config_names()[c].endswith("log4") for c in LOG_DOMAIN_CONFIGS)


@pytest.mark.parametrize("config", range(NUM_CONFIGS))
@pytest.mark.parametrize("nsplit", [1, 2, 3, 7])
def test_every_configuration_and_split(cuda, config, nsplit):
    g = golden("plummer4096")
    out = _gpu_force(g["posMass"], float(g["eps2"]), config, nsplit)
    assert O.per_body_rel_error(out, g["force_aos"])[0] <= TOL_VS_REFERENCE
    assert O.per_body_rel_error(out, g["force_f64"])[0] <= TOL_VS_FP64


@pytest.mark.parametrize("n", [1, 2, 3, 31, 33, 255, 257, 1000, 1023, 1025, 4097, 9001])
def test_ragged_sizes(cuda, n):
    pm, _ = nb.ic_uniform_ball(n, 1000 + n, 1.0, 0.5, 1.5)
    out = _gpu_force(pm, 1e-4)
    if n == 1:
        assert np.all(out[0, :3] == 0.0)  # only the self term, exactly 0
        return
    ref = O.ieee().forces_aos(pm, 1e-4)
    assert O.per_body_rel_error(out, ref)[0] <= TOL_VS_REFERENCE
    assert O.per_body_rel_error(out, _f64_as4(pm, 1e-4))[0] <= TOL_VS_FP64


def test_plain_16k_case(cuda):
    """N = 16,384 uniform ball, m = 1/N, eps2 = 1e-4 (the plain parity case)."""
    n = 16384
    pm, _ = nb.ic_uniform_ball(n, 16384)
    out = _gpu_force(pm, 1e-4)
    ref = O.ieee().forces_aos(pm, 1e-4)
    f64 = _f64_as4(pm, 1e-4)
    assert _within_reference(out, ref, f64)
    # all but the few near-cancelling bodies also directly within 1e-5
    d = np.linalg.norm(out[:, :3] - ref[:, :3], axis=1) / np.linalg.norm(ref[:, :3], axis=1)
    assert np.mean(d <= TOL_VS_REFERENCE) >= 0.999
    mx, rms = O.per_body_rel_error(out, f64)
    assert mx <= TOL_VS_FP64 and rms <= RMS_VS_FP64


def test_million_body_plummer_properties(cuda):
    """N = 1,048,576 Plummer sphere: FP64 and CPU_AOS on a subsample,
    Newton's third law, exact mass scaling, determinism."""
    n = 1 << 20
    _, _, pm, _ = nb.ic_plummer(n, 20)
    out = _gpu_force(pm, 1e-4)
    idx = np.random.default_rng(1).choice(n, 512, replace=False)
    f64 = _f64_as4(pm, 1e-4, idx)
    mx, rms = nb.force_error_stats(out, f64[:, :3], idx)
    assert mx <= TOL_VS_FP64 and rms <= RMS_VS_FP64, (mx, rms)
    # the CPU_AOS restatements built on this host, on the same targets: at
    # this size a sequential binary32 sum over 2^20 sources (the IEEE build)
    # is itself up to ~1e-4 from FP64, and the reference-flag build on
    # aarch64 (-mlow-precision-recip-sqrt) up to ~2e-5, so both are gated net
    # of their own distance from FP64; the direct gate against the
    # reference's own compiled CPU_AOS is test_million_body_against_reference
    for impl in (O.ieee(), O.fast()):
        assert _within_reference(out[idx], impl.forces_aos_idx(pm, 1e-4, idx), f64)
    # total momentum change sum_i m_i F_i vanishes (pairwise antisymmetry)
    m = pm[:, 3:4].astype(np.float64)
    tot = (m * out[:, :3]).sum(0)
    scale = (m * np.abs(out[:, :3])).sum(0)
    assert np.all(np.abs(tot) <= 1e-5 * scale)
    # doubling every mass doubles every force: exactly with rsqrt-only pairs
    # (power-of-two scaling), to rounding with log-domain pairs (log2 2m =
    # log2 m + 1 enters a rounded exponent sum)
    pm2 = pm.copy()
    pm2[:, 3] *= 2.0
    out2 = _gpu_force(pm2, 1e-4)
    assert O.per_body_rel_error(out2, 2.0 * out)[0] <= 1e-6
    r1 = _gpu_force(pm, 1e-4, config=25)
    r2 = _gpu_force(pm2, 1e-4, config=25)
    assert np.array_equal(r2[:, :3], 2.0 * r1[:, :3])
    # bit-identical on repeat (fixed-order combination of j-splits)
    assert np.array_equal(_gpu_force(pm, 1e-4), out)


def test_million_body_against_reference(cuda):
    """N = 1,048,576 Plummer sphere (the plain large system's own input):
    the drop-in's forces against the reference's compiled CPU_AOS
    (src/nbody_CPU_AOS.cpp:51-98, built with its flags; forces of all N
    bodies computed when the fixture was made, a seeded 1,024-body sample
    kept), per body, directly: max <= 1e-5; and against FP64 <= 5e-6."""
    import hashlib

    import torch
    g = golden("c2_plummer1m_sample")
    n, seed = int(g["n"]), int(g["seed"])
    _, _, pm_np, _ = nb.ic_plummer(n, seed)
    assert hashlib.sha256(pm_np.tobytes()).hexdigest() == g["posMass_sha256"].item().decode(), \
        "this host's Plummer input differs from the fixture's"
    pm = torch.from_numpy(pm_np).cuda()
    f = torch.zeros_like(pm)
    assert nb.ComputeGravitation_GPU_GB300(f, pm, float(g["eps2"]), n) > 0.0
    out = f.cpu().numpy()[g["idx"]]
    mx, rms = O.per_body_rel_error(out, g["force_aos"])
    assert mx <= TOL_VS_REFERENCE, (mx, rms)
    t64 = np.zeros((out.shape[0], 4))
    t64[:, :3] = g["force_f64"]
    mx64, rms64 = O.per_body_rel_error(out, t64)
    assert mx64 <= TOL_VS_FP64 and rms64 <= RMS_VS_FP64, (mx64, rms64)


@pytest.mark.parametrize("n", [155677, 163877, 311300])
def test_tail_split_plans(cuda, n):
    """Sizes whose i-blocks overflow whole waves of CTA slots: the planner
    splits the j-range of the leftover i-blocks only (whole i-blocks first,
    (i-block, slice) units after).  Results agree with the same
    configuration unsplit to rounding, and with FP64 on a sample."""
    _, _, pm, _ = nb.ic_plummer(n, n)
    cfg, ns, _ = nb.force_plan(n)
    out = _gpu_force(pm, 1e-4)
    whole = _gpu_force(pm, 1e-4, config=cfg, nsplit=1)
    assert O.per_body_rel_error(out, whole)[0] <= 1e-6
    idx = np.random.default_rng(n).choice(n, 256, replace=False)
    mx, rms = nb.force_error_stats(out, _f64_as4(pm, 1e-4, idx)[:, :3], idx)
    assert mx <= TOL_VS_FP64 and rms <= RMS_VS_FP64
    assert np.array_equal(_gpu_force(pm, 1e-4), out)  # deterministic


def test_forced_tail_only_splits(cuda):
    """nsplit <= -2 forces whole i-blocks for the whole rounds of CTA slots
    and only the leftover i-blocks split -nsplit ways: a different workspace
    from splitting every i-block, results equal to the unsplit plan to
    rounding, deterministic."""
    n = 311300
    _, _, pm, _ = nb.ic_plummer(n, 5)
    cfg = nb.force_config_names().index("w8_k2_jt1024_s3_log4")
    _, s_tail, ws_tail = nb.force_plan(n, cfg, -16)
    _, s_all, ws_all = nb.force_plan(n, cfg, 16)
    assert s_tail == s_all == 16 and ws_tail < ws_all
    whole = _gpu_force(pm, 1e-4, config=cfg, nsplit=1)
    for ns in (-2, -16, -64):
        out = _gpu_force(pm, 1e-4, config=cfg, nsplit=ns)
        assert O.per_body_rel_error(out, whole)[0] <= 1e-6, ns
        assert np.array_equal(_gpu_force(pm, 1e-4, config=cfg, nsplit=ns), out)


def test_split_choice_changes_only_rounding(cuda):
    g = golden("ball2048")
    a = _gpu_force(g["posMass"], 1e-4, 0, 1)
    b = _gpu_force(g["posMass"], 1e-4, 0, 4)
    assert O.per_body_rel_error(a, b)[0] <= 1e-6


def test_workspace_and_argument_errors(cuda):
    import torch
    lib = nb.load()
    pm = torch.zeros((1024, 4), device="cuda")
    f = torch.zeros((1024, 4), device="cuda")
    need = lib.nbgb_force_workspace_bytes(1024)
    assert need > 0
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert lib.nbgb_force(f.data_ptr(), pm.data_ptr(), 1e-4, 1024, ws.data_ptr(), need - 16,
                          s) == -2
    assert lib.nbgb_force(f.data_ptr(), pm.data_ptr(), 1e-4, 1024, None, 0, s) == -2
    assert lib.nbgb_force(f.data_ptr() + 4, pm.data_ptr(), 1e-4, 1024, ws.data_ptr(), need,
                          s) == -1
    assert lib.nbgb_force(f.data_ptr(), pm.data_ptr(), 1e-4, 1024, ws.data_ptr(), need, s) == 0
    assert lib.nbgb_force(f.data_ptr(), pm.data_ptr(), 1e-4, 0, None, 0, s) == 0
    assert nb.ComputeGravitation_GPU_GB300(f, pm, 1e-4, 0) == 0.0
    torch.cuda.synchronize()
    assert nb.last_status() == 0


def test_plan_fills_the_gpu(cuda):
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    for n in (16384, 262144, 1 << 20):
        c, s, w = nb.force_plan(n)
        assert s >= 1 and w > 0
        assert 0 <= c < len(nb.force_config_names())


def _with_negative_masses(n=3000, seed=77):
    pm, _ = nb.ic_uniform_ball(n, seed, 1.0, 0.5, 1.5)
    pm = pm.copy()
    pm[0, 3] = -pm[0, 3]       # pair 0: a log-domain pair in mode-6 plans
    pm[n // 2, 3] *= -0.5
    return pm


def test_negative_masses_through_the_drop_in(cuda):
    """Masses < 0 have no logarithm: the drop-in sees the status bit of a
    log-domain plan and evaluates again with rsqrt only, so its result is the
    reference's formula for any sign."""
    import torch
    pm_np = _with_negative_masses()
    n = pm_np.shape[0]
    pm = torch.from_numpy(pm_np).cuda()
    f = torch.zeros((n, 4), device="cuda")
    assert nb.ComputeGravitation_GPU_GB300(f, pm, 1e-4, n) > 0.0
    assert nb.last_status() == 0
    ref = O.ieee().forces_aos(pm_np, 1e-4)
    assert O.per_body_rel_error(f.cpu().numpy(), ref)[0] <= TOL_VS_REFERENCE


def test_negative_masses_stream_ordered(cuda):
    """nbgb_force with a log-domain plan flags masses < 0 (NaN forces and
    NBGB_STATUS_NEGATIVE_MASS); an rsqrt-only configuration takes them."""
    import torch
    pm_np = _with_negative_masses()
    pm = torch.from_numpy(pm_np).cuda()
    out = nb.force(pm, 1e-4, config=27)
    torch.cuda.synchronize()
    assert nb.last_status() & NEGATIVE_MASS
    assert np.isnan(out.cpu().numpy()[:, :3]).any()
    ok = _gpu_force(pm_np, 1e-4, config=25)
    ref = O.ieee().forces_aos(pm_np, 1e-4)
    assert O.per_body_rel_error(ok, ref)[0] <= TOL_VS_REFERENCE


def test_log_domain_pairs_accuracy_16k(cuda):
    """The log-domain form keeps the per-body gates on a 16k ball whose masses
    span six decades (where a binary32 sequential sum is itself up to 1.2e-4
    from FP64)."""
    n = 16384
    pm, _ = nb.ic_uniform_ball(n, 4242)
    pm = pm.copy()
    pm[:, 3] = np.float32(1.0 / n) * np.exp(np.random.default_rng(5).uniform(-7, 7, n)).astype(
        np.float32)
    ref = O.ieee().forces_aos(pm, 1e-4)
    f64 = _f64_as4(pm, 1e-4)
    for c in (25,) + tuple(LOG_DOMAIN_CONFIGS):
        out = _gpu_force(pm, 1e-4, config=c)
        assert _within_reference(out, ref, f64), c
        mx, rms = O.per_body_rel_error(out, f64)
        assert mx <= TOL_VS_FP64 and rms <= RMS_VS_FP64, (c, mx, rms)
