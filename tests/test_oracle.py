"""The CPU oracle against the reference's own outputs.

Pins the oracle (oracle/lulesh_oracle.c) to the golden fixtures that
tests/golden/make_golden.py recorded from the unmodified reference sources,
bit for bit, and - where the reference sources exist - against the reference
binary directly on further configurations.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle  # noqa: E402  (on sys.path through conftest)
from conftest import golden_dump

FAST_RUNS = [(8, 11, 1, 1), (10, 11, 1, 1), (12, 21, 1, 1), (12, 1, 1, 1), (9, 16, 2, 2),
             (16, 11, 1, 1), (20, 11, 1, 1)]
DUMPS = ["dump_s8_r11_b1_c1_i1.npz", "dump_s8_r11_b1_c1_i100.npz", "dump_s12_r21_b1_c1_i50.npz",
         "dump_s10_r1_b1_c1_i30.npz"]


def _golden(golden_results, s, r, b, c):
    for g in golden_results:
        if (g["s"], g["r"], g["b"], g["c"]) == (s, r, b, c):
            return g
    raise KeyError((s, r, b, c))


@pytest.mark.parametrize("s,r,b,c", FAST_RUNS)
def test_full_run_matches_reference(oracle_mod, golden_results, s, r, b, c):
    g = _golden(golden_results, s, r, b, c)
    o = oracle_mod.Oracle(s, r, b, c, threads=4)
    assert o.run() == 0
    assert o.cycle == g["cycles"]
    assert o.field("e")[0] == float(g["e0"])  # bit for bit: 17 significant digits round-trip
    sym = o.symmetry()
    assert sym == (float(g["maxabs"]), float(g["totabs"]), float(g["maxrel"]))
    assert o.scalar("deltatime") == float(g["dt"])


def test_s30_known_answer(oracle_mod, golden_results):
    """The headline known answer: --s 30 --r 11 runs 932 cycles to e(0)=2.02507478507199121e+05."""
    g = _golden(golden_results, 30, 11, 1, 1)
    o = oracle_mod.Oracle(30, 11, 1, 1, threads=os.cpu_count() or 4)
    assert o.run() == 0
    assert o.cycle == g["cycles"] == 932
    assert o.field("e")[0] == float(g["e0"])
    assert o.symmetry() == (float(g["maxabs"]), float(g["totabs"]), float(g["maxrel"]))


@pytest.mark.parametrize("name", DUMPS)
def test_fields_match_reference_dump(oracle_mod, name):
    d = golden_dump(name)
    tag = Path(name).stem.split("_")[1:]
    s, r, b, c, its = (int(t[1:]) for t in tag)
    o = oracle_mod.Oracle(s, r, b, c, threads=2)
    assert o.run(its) == 0
    assert o.cycle == int(d["cycle"]) == its
    for f in oracle_mod.NODE_FIELDS + oracle_mod.ELEM_FIELDS:
        np.testing.assert_array_equal(o.field(f), d[f], err_msg=f)
    for k in ("time", "deltatime", "dtcourant", "dthydro"):
        assert o.scalar(k) == float(d[k]), k


def test_thread_count_does_not_change_bits(oracle_mod):
    runs = []
    for t in (1, 3):
        o = oracle_mod.Oracle(11, 11, 1, 1, threads=t)
        assert o.run(60) == 0
        runs.append({f: o.field(f).copy() for f in oracle_mod.NODE_FIELDS + oracle_mod.ELEM_FIELDS})
    for f in runs[0]:
        np.testing.assert_array_equal(runs[0][f], runs[1][f], err_msg=f)


# the last three run to stoptime (--i above their cycle counts): one element
# (one step), two and three elements a side
REF_CASES = [(7, 11, 1, 1, 40), (13, 16, 2, 3, 25), (6, 5, 0, 0, 60), (1, 11, 1, 1, 10), (2, 1, 1, 1, 10),
             (3, 21, 2, 2, 100)]


@pytest.mark.skipif(not (oracle.REF_SOURCES / "lulesh.cc").exists(),
                    reason="reference sources not present on this machine")
@pytest.mark.parametrize("s,r,b,c,its", REF_CASES)
def test_oracle_equals_reference_binary(oracle_mod, tmp_path, s, r, b, c, its):
    """Dumps of the reference binary and the oracle CLI are byte-identical."""
    if not oracle_mod.REF_BIN.exists():
        oracle_mod.build(ref=True)
    env = dict(os.environ)
    args = ["--s", str(s), "--r", str(r), "--b", str(b), "--c", str(c), "--i", str(its)]
    env["LULESH_DUMP"] = str(tmp_path / "ref.bin")
    subprocess.run([str(oracle_mod.REF_BIN), *args], env=env, check=True, capture_output=True)
    env["LULESH_DUMP"] = str(tmp_path / "port.bin")
    subprocess.run([str(oracle_mod.CLI_PATH), *args, "--threads", "2"], env=env, check=True,
                   capture_output=True)
    assert (tmp_path / "ref.bin").read_bytes() == (tmp_path / "port.bin").read_bytes()


def test_energy_scale_changes_only_the_deposit(oracle_mod):
    a = oracle_mod.Oracle(6, 11, 1, 1)
    b = oracle_mod.Oracle(6, 11, 1, 1, energy_scale=1.7)
    assert b.field("e")[0] == a.field("e")[0] * 1.7
    assert b.scalar("deltatime") < a.scalar("deltatime")
    np.testing.assert_array_equal(a.field("x"), b.field("x"))


@pytest.mark.skipif(not (oracle.REF_SOURCES / "lulesh.cc").exists()
                    or oracle.REF_SOURCES.resolve() == oracle.REF_INSTALLED.resolve(),
                    reason="the reference checkout is not on this machine")
def test_installed_reference_is_the_unmodified_sources(oracle_mod):
    """make install-ref copies the reference's sources into baseline/_ref
    (where a machine without the checkout builds and times them) byte for
    byte, and nothing else."""
    subprocess.run(["make", "-s", "-C", str(oracle_mod.HERE), "install-ref"], check=True)
    files = ("lulesh.cc", "lulesh.h", "lulesh-init.cc", "lulesh-util.cc", "lulesh-viz.cc", "LICENSE")
    assert sorted(p.name for p in oracle_mod.REF_INSTALLED.iterdir()) == sorted(files)
    for f in files:
        assert (oracle_mod.REF_INSTALLED / f).read_bytes() == (oracle_mod.REF_SOURCES / f).read_bytes(), f
