"""Serving loop with continuous batching (lulesh_serve).

Requests arrive on a seeded Poisson schedule while earlier ones are running;
the loop admits them as slots and pool memory free up and retires each at its
stoptime. Every request's result (cycle count, final origin energy and the
plane-0 symmetry diffs computed on the device) must be the same as the same
problem run alone - bit for bit, since each problem keeps its own dt and
exact dt minima inside the batch.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(n, seed, smin, smax, mean_gap):
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(mean_gap, n))
    s = rng.integers(smin, smax + 1, n)
    r = rng.choice([11, 21], n)
    scale = rng.lognormal(0.0, 0.25, n)
    return [{"s": int(a), "nr": int(b), "energy_scale": float(c), "arrival_s": float(d)}
            for a, b, c, d in zip(s, r, scale, t)]


def _solo(lulesh, precision, req):
    dom = lulesh.HostDomain(req["s"], req["nr"], 1, 1, req["energy_scale"])
    dev = lulesh.Device(dom, precision)
    n = dev.run()
    dev.download()
    return n, float(dom.e[0]), dom.symmetry()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_each_request_equals_its_solo_run(lulesh, precision):
    reqs = _requests(10, seed=5, smin=6, smax=14, mean_gap=0.03)
    budget = 3 * lulesh.Batch.footprint(precision, 14) + (1 << 20)
    results, stats = lulesh.serve(reqs, precision, hbm_budget=budget, max_slots=3, sync_ms=5.0)
    assert stats["served"] == len(reqs)
    assert 2 <= stats["max_resident"] <= 3  # requests overlapped on the device
    for req, res in zip(reqs, results):
        assert res["err"] == 0
        assert res["admitted_s"] >= req["arrival_s"] - 1e-9
        assert res["finished_s"] >= res["admitted_s"]
        assert res["time_to_solution_s"] == pytest.approx(res["finished_s"] - req["arrival_s"])
        n, e0, sym = _solo(lulesh, precision, req)
        assert res["cycles"] == n
        assert res["e0"] == e0
        # the symmetry check is computed on the device at retire
        assert (res["maxabs"], res["totabs"], res["maxrel"]) == sym
        assert res["zone_cycles"] == req["s"] ** 3 * n
    assert 0 < stats["p50_s"] <= stats["p99_s"]
    assert stats["zone_cycles"] == sum(r["zone_cycles"] for r in results)
    # admission by footprint: the resident problems never held more than the budget
    assert 0 < stats["peak_resident_bytes"] <= budget
    assert 0 <= stats["p50_queue_s"] <= stats["p99_queue_s"]


def test_request_larger_than_the_budget_is_refused(lulesh):
    big = lulesh.Batch.footprint("mixed", 20)
    with pytest.raises(lulesh.LuleshError) as ei:
        lulesh.serve([{"s": 20, "arrival_s": 0.0}], "mixed", hbm_budget=big - 4096, max_slots=2)
    assert ei.value.status == lulesh.EINVAL
