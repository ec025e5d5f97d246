"""The force planner without a GPU (nbgb_force_plan_on) against a GB300's
SM count and occupancy table (tests/golden/gb300_force_occupancy.json, made
by tests/golden/gen_gb300_force_occupancy.py on a GB300).  The pinned plans
are the ones the planner takes on the GPU and that
`python -m nbody_gb300.plancheck` timed against a grid of forced plans."""
import json
import os

import pytest

import nbody_gb300 as nb

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gb300():
    t = json.load(open(os.path.join(HERE, "golden", "gb300_force_occupancy.json")))
    assert t["configs"] == nb.force_config_names(), "configuration table changed: regenerate"
    return t["sms"], t["occupancy"]


def _plan(dev, n, config=-1, nsplit=-1):
    c, s, f, w = nb.force_plan_on(n, dev[0], dev[1], config, nsplit)
    return nb.force_config_names()[c], s, f, w


@pytest.mark.parametrize("n,config,nsplit,nfull", [
    (1, "w4_k2_jt256_s4_log4", 1, 1),
    (1000, "w4_k2_jt256_s4_log4", 4, 0),
    (4096, "w4_k2_jt256_s4_log4", 8, 0),
    (16384, "w4_k2_jt256_s4_log4", 16, 0),
    (20000, "w4_k2_jt256_s4_log4", 20, 0),
    (32768, "w8_k2_jt1024_s3_log4", 16, 0),
    (65536, "w8_k2_jt1024_s3_log4", 32, 0),
    (155677, "w8_k2_jt1024_s3_log4", 51, 304),
    (262144, "w8_k2_jt1024_s3_log4", 16, 304),
    (1048576, "w8_k2_jt1024_s3_log4", 19, 1824),
])
def test_gb300_plans(gb300, n, config, nsplit, nfull):
    name, s, f, w = _plan(gb300, n)
    assert (name, s, f) == (config, nsplit, nfull)
    assert _plan(gb300, n) == (name, s, f, w)  # deterministic


def test_workspace_holds_stream_and_partials(gb300):
    n = 1048576
    name, s, f, w = _plan(gb300, n)
    bi, jt = 512, 1024  # w8_k2 (8 warps x 32 x 2 targets), 1024-body tiles
    nb_blocks = n // bi
    stream = -(-n // jt) * jt * 16
    partials = 2 * s * (nb_blocks - f) * bi * 16
    assert w >= stream + partials
    assert partials == 2 * 19 * 224 * 512 * 16  # 69.7 MB


def test_forced_plans(gb300):
    c45 = nb.force_config_names().index("w8_k2_jt1024_s3_log4")
    n = 1048576
    name, s, f, w = _plan(gb300, n, c45, 16)  # every i-block split
    assert (s, f) == (16, 0)
    name, s, f, w_tail = _plan(gb300, n, c45, -16)  # leftover i-blocks only
    assert (s, f) == (16, 1824) and w_tail < w
    name, s, f, w = _plan(gb300, 2000, c45, -16)  # no whole round: every block split
    assert (s, f) == (2, 0)  # two 1024-body tiles
    name, s, f, w = _plan(gb300, n, c45, 1)
    assert (s, f) == (1, 2048)


def test_plan_follows_the_device(gb300):
    """Half the SMs: the whole rounds hold half the i-blocks."""
    c, s, f, w = nb.force_plan_on(1048576, 76, gb300[1])
    assert f > 0 and f % (76 * gb300[1][c]) == 0


def test_argument_errors(gb300):
    sms, occ = gb300
    with pytest.raises(nb.NbgbError):
        nb.force_plan_on(0, sms, occ)
    with pytest.raises(nb.NbgbError):
        nb.force_plan_on(1000, 0, occ)
    with pytest.raises(nb.NbgbError):
        nb.force_plan_on(1000, sms, occ[:-1])
    with pytest.raises(nb.NbgbError):
        nb.force_plan_on(1000, sms, [-1] + occ[1:])
    with pytest.raises(nb.NbgbError):
        nb.force_plan_on(1000, sms, occ, len(occ))
