"""Batched ensembles: many problems in one device pool, one CUDA graph per cycle.

Each problem in a batch runs the same per-element code with its own dt and
its own exact dt minima, so its result must equal the same problem run alone
bit for bit - whatever else is in the batch, when it was admitted, and how
the launch shapes were tuned.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "xd", "yd", "zd", "xdd", "fx", "e", "p", "q", "ql", "qq", "v", "vnew",
          "delv", "vdov", "arealg", "ss")


def _alone(lulesh, precision, s, nr=11, balance=1, cost=1, energy_scale=1.0, its=9999999):
    dom = lulesh.HostDomain(s, nr, balance, cost, energy_scale)
    dev = lulesh.Device(dom, precision)
    n = dev.run(its)
    dev.download()
    return dom, n


def _assert_same(a, b):
    for f in FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)


def _run_to_end(batch, chunk=64, limit=100000):
    total = 0
    while total < limit:
        active, _ = batch.run(chunk)
        total += chunk
        if active == 0:
            return
    raise AssertionError("batch did not finish")


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp64_exact"])
def test_each_problem_equals_its_solo_run(lulesh, precision):
    specs = [dict(s=8), dict(s=11, nr=21), dict(s=9, nr=16, balance=2, cost=2),
             dict(s=12, energy_scale=0.7), dict(s=10, nr=1, energy_scale=1.3)]
    b = lulesh.Batch(precision, pool_bytes=256 << 20, max_slots=8)
    slots = [b.admit(**sp) for sp in specs]
    _run_to_end(b)
    st = {x["slot"]: x for x in b.status()}
    for slot, sp in zip(slots, specs):
        alone, n = _alone(lulesh, precision, **sp)
        assert st[slot]["cycle"] == n and st[slot]["err"] == 0
        _assert_same(b.download(slot), alone)
        # final report of the slot computed on the device
        vr = b.verify(slot)
        assert vr["cycle"] == n and vr["nx"] == sp["s"] and vr["e0"] == alone.e[0]
        assert (vr["maxabs"], vr["totabs"], vr["maxrel"]) == alone.symmetry()
    assert b.launches > 0


def test_per_problem_limits_and_late_admission(lulesh):
    """Continuous batching: a problem admitted while others are mid-run, and
    problems with their own cycle limit and stoptime, all finish exactly as
    they do alone."""
    b = lulesh.Batch("fp64", pool_bytes=256 << 20, max_slots=4)
    a = b.admit(s=10)
    c = b.admit(s=8, max_cycles=50)
    b.run(30)
    late = b.admit(s=9, nr=21)
    d = b.admit(s=8, stoptime=5e-3)
    _run_to_end(b)
    st = {x["slot"]: x for x in b.status()}
    assert st[c]["cycle"] == 50
    _assert_same(b.download(c), _alone(lulesh, "fp64", 8, its=50)[0])
    _assert_same(b.download(a), _alone(lulesh, "fp64", 10)[0])
    _assert_same(b.download(late), _alone(lulesh, "fp64", 9, nr=21)[0])
    solo = lulesh.HostDomain(8)
    solo.time_state.stoptime = 5e-3
    dev = lulesh.Device(solo, "fp64")
    n = dev.run()
    dev.download()
    assert st[d]["cycle"] == n and st[d]["time"] == pytest.approx(5e-3)
    _assert_same(b.download(d), solo)


def test_retire_frees_pool_and_slot(lulesh):
    need = lulesh.Batch.footprint("fp64", 12)
    b = lulesh.Batch("fp64", pool_bytes=2 * need + 4096, max_slots=3)
    s0 = b.admit(s=12)
    s1 = b.admit(s=12)
    assert b.try_admit(s=12) is None  # pool full
    b.run(5)
    b.retire(s0)
    s2 = b.admit(s=12)
    assert s2 == s0
    _run_to_end(b)
    st = {x["slot"]: x for x in b.status()}
    assert st[s1]["cycle"] == st[s2]["cycle"] == 297


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_autotune_keeps_results(lulesh, precision):
    b = lulesh.Batch(precision, pool_bytes=512 << 20, max_slots=8)
    slots = [b.admit(s=s, nr=r) for s, r in ((14, 11), (9, 21), (12, 16))]
    b.run(3)
    tuning = b.autotune(cycles=1)
    assert tuning["ms_per_cycle"] > 0
    b.run(0)  # refresh the status from the device
    st0 = {x["slot"]: x["cycle"] for x in b.status()}
    assert all(c == 3 for c in st0.values())  # tuning did not advance the problems
    _run_to_end(b)
    for slot, (s, r) in zip(slots, ((14, 11), (9, 21), (12, 16))):
        _assert_same(b.download(slot), _alone(lulesh, precision, s, nr=r)[0])


def test_mixed_ensemble_against_double(lulesh):
    """Ensemble problems of the benchmark's kind (s in [16, 64], regions in
    {11, 16, 21}, lognormal(0, 0.25) energy scale, seeded) run in one mixed
    batch and in one double batch. Every problem keeps the double run's cycle
    count. The mixed e(0) stays within 1e-5 of the double one: most sizes
    land near 1e-8, but at some sizes the mixed state's drift (about 1e-7 of
    e after a few hundred cycles) moves an element's vdov across zero, where
    the monotonic Q switches off (lulesh.cc:1618-1621), and e(0) then moves by
    up to about 5e-6."""
    rng = np.random.default_rng(2024)
    n = 8
    specs = [dict(s=int(a), nr=int(b), energy_scale=float(c))
             for a, b, c in zip(rng.integers(16, 65, n), rng.choice([11, 16, 21], n),
                                rng.lognormal(0.0, 0.25, n))]
    out = {}
    for prec in ("fp64", "mixed"):
        need = sum(lulesh.Batch.footprint(prec, sp["s"]) for sp in specs)
        b = lulesh.Batch(prec, pool_bytes=need + (64 << 20), max_slots=n)
        slots = [b.admit(**sp) for sp in specs]
        _run_to_end(b)
        st = {x["slot"]: x for x in b.status()}
        out[prec] = [(st[sl]["cycle"], st[sl]["err"], b.verify(sl)["e0"]) for sl in slots]
        b.close()
    for sp, (c64, err64, e64), (cm, errm, em) in zip(specs, out["fp64"], out["mixed"]):
        assert err64 == errm == 0, sp
        assert cm == c64, sp
        assert abs(em - e64) / abs(e64) <= 1e-5, (sp, em, e64)
