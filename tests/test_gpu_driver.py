"""The lulesh-gb300 program: the reference's command line and outputs on the GPU."""
from __future__ import annotations

import re
import subprocess

import pytest

from conftest import PKG_DIR

pytestmark = pytest.mark.gpu

EXE = PKG_DIR / "lulesh-gb300"


def _golden(golden_results, s, r=11):
    return next(g for g in golden_results if g["s"] == s and g["r"] == r and "its" not in g)


@pytest.mark.parametrize("extra", [[], ["--graph"], ["--precision", "fp64_exact"]])
def test_report_matches_reference(lulesh, golden_results, extra):
    g = _golden(golden_results, 16)
    out = subprocess.run([str(EXE), "--s", "16", "--r", "11", "--p", *extra], capture_output=True,
                         text=True, check=True).stdout
    assert "Iteration count     =  434" in out
    m = re.search(r"RESULT s=16 cycles=(\d+) e0=(\S+)", out)
    assert int(m.group(1)) == g["cycles"]
    assert abs(float(m.group(2)) - float(g["e0"])) / float(g["e0"]) <= 1e-10
    assert "cycle = 400," in out  # --p progress every 100 cycles


def test_quiet_prints_the_reference_csv_line(lulesh, golden_results):
    g = _golden(golden_results, 12, r=21)
    out = subprocess.run([str(EXE), "--s", "12", "--r", "21", "--q", "--hpx:threads=4"],
                         capture_output=True, text=True, check=True).stdout.strip()
    s, r, cycles, threads, elapsed, e0 = out.split(",")
    assert (s, r, cycles, threads) == ("12", "21", str(g["cycles"]), "1")
    assert float(elapsed) > 0
    assert e0.strip() == f"{float(g['e0']):.6e}"


def test_equals_form_and_ignored_flags(lulesh, golden_results):
    """--name=value as the reference's option parser takes it, and the
    reference's viz and HPX task-size flags accepted (no effect here)."""
    g = _golden(golden_results, 12, r=21)
    out = subprocess.run([str(EXE), "--s=12", "--r=21", "--q", "--f", "2", "--elems-per-task=64",
                          "--task-size", "4", "--hpx:threads=2"],
                         capture_output=True, text=True, check=True).stdout.strip()
    s, r, cycles = out.split(",")[:3]
    assert (s, r, cycles) == ("12", "21", str(g["cycles"]))


def test_iteration_cap(lulesh):
    out = subprocess.run([str(EXE), "--s", "10", "--i", "37", "--q"], capture_output=True, text=True,
                         check=True).stdout
    assert out.split(",")[2] == "37"
