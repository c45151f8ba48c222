"""The allocation-free time-step constraint entry point.

lulesh_dt_constraints_noalloc serves callers that cannot allocate device
memory - a host framework that owns every device allocation through its own
pool or budget, or a loop that cannot afford cudaMalloc's possible device-wide
synchronization. Its only working memory is a fixed 256 KiB array inside the
library. These tests call it through the C ABI on device arrays owned by the
caller (torch tensors here) and check both minima against what the existing
entry point, lulesh_dev_step, returns for the same state, on two cycles in a
row (bit for bit, on a double and a mixed handle), run it at its size limit,
and check that sizes above LULESH_NOALLOC_MAX_ELEMS are refused.

This file is collected last on purpose, so a run that stops at the first
failure has already run every other test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_ELEMS = 4194304  # LULESH_NOALLOC_MAX_ELEMS
EINVAL = -10


def _bind(lib):
    fn = lib.lulesh_dt_constraints_noalloc
    fn.restype = C.c_int32
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_double, C.c_double,
                   C.c_void_p, C.c_void_p]
    return fn


def _host_minima(ss, vdov, arealg, qqc, dvovmax, n):
    ss, vdov, arealg = ss[:n], vdov[:n], arealg[:n]
    live = vdov != 0.0
    dtf = ss * ss + np.where(vdov < 0.0, 64.0 * qqc * qqc * arealg * arealg * vdov * vdov, 0.0)
    dtc = np.min(np.where(live, arealg / np.sqrt(dtf), 1e20), initial=1e20)
    dth = np.min(np.where(live, dvovmax / (np.abs(vdov) + 1e-20), 1e20), initial=1e20)
    return dtc, dth


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_minima_match_step_on_consecutive_cycles(lulesh, precision):
    torch = pytest.importorskip("torch")
    lulesh.set_device(0)
    torch.cuda.set_device(0)
    fn = _bind(lulesh.library())
    dom = lulesh.HostDomain(20, 11, 1, 1)
    dev = lulesh.Device(dom, precision)
    assert dev.run(40) == 40  # let the blast spread over many elements
    prm = dom.view.params
    out = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
    for _ in range(2):
        dom.time_increment()
        dtc, dth = dev.step(dom.time_state.deltatime)
        dom.time_state.dtcourant, dom.time_state.dthydro = dtc, dth
        dev.download(lulesh.F_SS | lulesh.F_KIN)
        ss = torch.from_numpy(dom.ss.copy()).cuda()
        vdov = torch.from_numpy(dom.vdov.copy()).cuda()
        arealg = torch.from_numpy(dom.arealg.copy()).cuda()
        torch.cuda.synchronize()
        st = fn(ss.data_ptr(), vdov.data_ptr(), arealg.data_ptr(), dom.numElem, prm.qqc,
                prm.dvovmax, out.data_ptr(), None)
        assert st == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        # the same per-element arithmetic as the step's material kernel, and
        # exact minima: equal bit for bit
        assert got[0] == dtc
        assert got[1] == dth
        # a smaller size right after: the counter is cleared per call. The
        # host minima use correctly rounded divide and square root, the
        # device its reciprocal forms (within about one ulp).
        n = dom.numElem // 3
        assert fn(ss.data_ptr(), vdov.data_ptr(), arealg.data_ptr(), n, prm.qqc, prm.dvovmax,
                  out.data_ptr(), None) == 0
        torch.cuda.synchronize()
        want = _host_minima(dom.ss, dom.vdov, dom.arealg, prm.qqc, prm.dvovmax, n)
        got = out.cpu().numpy()
        assert got[0] == pytest.approx(want[0], rel=1e-13)
        assert got[1] == pytest.approx(want[1], rel=1e-13)


def test_noalloc_at_its_size_limit(lulesh):
    """numElem = LULESH_NOALLOC_MAX_ELEMS fills every partial slot of the
    fixed scratch: the smallest Courant candidate sits in the last element
    and the smallest hydro candidate in block 0, and both must come out, on
    two calls in a row."""
    torch = pytest.importorskip("torch")
    lulesh.set_device(0)
    torch.cuda.set_device(0)
    fn = _bind(lulesh.library())
    n = MAX_ELEMS
    rng = np.random.default_rng(11)
    ss = rng.uniform(1.0, 2.0, n)
    arealg = rng.uniform(0.5, 1.0, n)
    vdov = rng.uniform(-1.0, 1.0, n)
    vdov[rng.integers(0, n, 1000)] = 0.0  # elements that do not constrain
    arealg[n - 1], ss[n - 1], vdov[n - 1] = 1e-3, 1.0, -1e-3  # smallest Courant
    vdov[17] = 50.0  # largest |vdov| in block 0: smallest hydro
    qqc, dvovmax = 2.0, 0.1
    want = _host_minima(ss, vdov, arealg, qqc, dvovmax, n)
    assert want[0] == pytest.approx(arealg[n - 1] / np.sqrt(ss[n - 1] ** 2 + 256 * 1e-6 * 1e-6))
    assert want[1] == pytest.approx(dvovmax / 50.0)
    d = [torch.from_numpy(a).cuda() for a in (ss, vdov, arealg)]
    out = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
    for _ in range(2):
        out.fill_(-1.0)
        torch.cuda.synchronize()
        assert fn(d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), n, qqc, dvovmax,
                  out.data_ptr(), None) == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert got[0] == pytest.approx(want[0], rel=1e-13)
        assert got[1] == pytest.approx(want[1], rel=1e-13)


def test_noalloc_refuses_sizes_above_its_fixed_scratch(lulesh):
    torch = pytest.importorskip("torch")
    lulesh.set_device(0)
    fn = _bind(lulesh.library())
    buf = torch.zeros(4, dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    assert fn(p, p, p, MAX_ELEMS + 1, 2.0, 0.1, p, None) == EINVAL
    assert fn(p, p, p, 0, 2.0, 0.1, p, None) == EINVAL
    assert fn(None, p, p, 4, 2.0, 0.1, p, None) == EINVAL
