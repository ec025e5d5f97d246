"""The command-line driver keeps the reference's flags and output line."""
import re
import subprocess
import sys

import pytest

from conftest import ROOT

# the regular expression of the reference's scripts/nbody-stats.py (line 9)
LINE_RE = re.compile(
    r'^\s*(?P<algorithm>[\w\s]+):\s*(?P<ms>[\d.]+)\s*ms\s*=\s*(?P<interactions>[\d\.x^]+)'
    r'\s*interactions/s+\s*\(\s*(?P<gflops>[\d.]+)\s*GFLOPS\)'
    r'(?:\s*\(Rel\. error:\s*(?P<error>[\d\.E+-]+)\))?$')


def _run(*args):
    return subprocess.run([sys.executable, "-m", "nbody_gb300", *args], cwd=ROOT,
                          capture_output=True, text=True, timeout=300)


def test_reference_line_parses_with_the_stats_regex():
    import nbody_gb300 as nb
    for rel in (None, 3.2e-6):
        line = nb.reference_line("GPU_GB300", 16384, 0.12, rel, 9)
        m = LINE_RE.search(line.rstrip())
        assert m and m.group("algorithm").strip() == "GPU_GB300"
        assert float(m.group("gflops")) > 0
    # small rates switch to x10^6 like the reference (src/nbody.cu:1042-1048)
    assert "x10^6" in nb.reference_line("GPU_GB300", 1024, 10.0)


def test_flag_errors_and_list():
    assert _run("--bodies", "0").returncode == 1
    assert _run("--seed", "0").returncode == 1
    assert _run("--algorithm", "NoSuchAlgorithm").returncode == 1
    r = _run("--list")
    assert r.returncode == 0 and "0 - GPU_GB300" in r.stdout
    assert "1 - GPU_GB300_Newton3" in r.stdout
    from nbody_gb300 import cli
    assert cli.resolve_algorithm("GPU_GB300") == 0
    assert cli.resolve_algorithm("gpu_gb300_newton3") == 1
    assert cli.resolve_algorithm("1") == 1 and cli.resolve_algorithm("2") is None


@pytest.mark.gpu
def test_cli_runs_and_reports(cuda):
    r = _run("--bodies", "2", "--iterations", "3", "--verbose")
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.replace("\r", "\n").splitlines() if l.strip()]
    assert len(lines) == 3
    for l in lines:
        m = LINE_RE.search(l)
        assert m and float(m.group("ms")) > 0
        assert float(m.group("error")) < 1e-2  # per-component relError vs FP64
    assert "Running simulation with 2048 particles, crosscheck enabled" in r.stderr


@pytest.mark.gpu
def test_cli_cycles_through_both_rows(cuda):
    """--cycle-after 2 --iterations 1: two steps of each row, as the
    reference's driver cycles its algorithm table."""
    r = _run("--bodies", "2", "--iterations", "1", "--cycle-after", "2", "--verbose")
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.replace("\r", "\n").splitlines() if l.strip()]
    names = [LINE_RE.search(l).group("algorithm").strip() for l in lines]
    assert names == ["GPU_GB300"] * 2 + ["GPU_GB300_Newton3"] * 2
    for l in lines:
        assert float(LINE_RE.search(l).group("error")) < 1e-2
