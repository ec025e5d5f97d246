"""The C ABI library loads and exports every symbol include/*.h declares
(no compute calls: these run without a GPU)."""
import ctypes
import glob
import os
import re
import subprocess

import numpy as np

from conftest import ROOT, golden

import nbody_gb300 as nb
from nbody_gb300 import _lib


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"NBGB_API\s+[\w\s\*]+?\b(\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_header_declares_the_drop_in_signature():
    names = declared_symbols()
    assert "ComputeGravitation_GPU_GB300" in names
    text = open(os.path.join(ROOT, "include", "nbody_gb300.h")).read()
    # the reference's pfnComputeGravitation_AOS_t (src/nbody.h:68)
    assert re.search(r"float\s+ComputeGravitation_GPU_GB300\(float \*force, float \*posMass, "
                     r"float softeningSquared,\s+size_t N\)", text)


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_lib.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_exports_are_c_linkage_and_nothing_else_leaks():
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert declared_symbols() == exported


def test_python_binding_covers_the_header():
    assert declared_symbols() == set(_lib.SIGNATURES)


def test_version_and_status_strings():
    assert b"sm_103a" in _lib.load().nbgb_version()
    assert _lib.load().nbgb_status_string(0) == b"ok"
    assert b"workspace" in _lib.load().nbgb_status_string(-2)


def test_library_is_built_for_sm_103a_only():
    import nbody_gb300.build as B
    assert B.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_host_ic_reference_matches_reference_bodies():
    g = golden("refic1024_seed7")
    pm, vm = nb.ic_reference(1024, 7)
    assert np.array_equal(pm, g["posMass"]) and np.array_equal(vm, g["velInvMass"])


def test_host_crosscheck_metric_matches_oracle():
    from oracle import oracle as O
    g = golden("ball2048")
    f = O.ieee().forces_aos(g["posMass"], float(g["eps2"]))
    assert nb.crosscheck_max_rel_error(f, g["force_aos"]) == O.ieee().max_rel_error(
        f, g["force_aos"])


def test_host_error_stats_match_numpy():
    from oracle import oracle as O
    g = golden("plummer4096")
    mx, rms = nb.force_error_stats(g["force_aos"], g["force_f64"][:, :3])
    mx2, rms2 = O.per_body_rel_error(g["force_aos"], g["force_f64"])
    assert abs(mx - mx2) <= 1e-12 and abs(rms - rms2) <= 1e-12
