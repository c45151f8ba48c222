"""Host side of the product on CPU: the C ABI loads and exports what
include/lulesh_gb300.h declares, the host Domain equals the oracle's initial
state bit for bit, host TimeIncrement equals the oracle's, argument checks
reject bad input before any device work, and without a GPU the device entry
points fail loudly (no CPU fallback)."""
from __future__ import annotations

import ctypes as C
import math
import re

import numpy as np
import pytest

from conftest import ROOT, gpu_available

HEADER = ROOT / "include" / "lulesh_gb300.h"


def declared_functions(header=HEADER) -> list[str]:
    text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(lulesh_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lulesh):
    lib = lulesh.library()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_probes_live_in_their_own_library(lulesh):
    """The measurement probes are not part of the step's ABI: the product
    library does not export them, liblulesh_probe.so exports what its header
    declares."""
    probe_header = ROOT / "lulesh-task-based-hpx_gb300" / "csrc" / "lulesh_probe.h"
    names = declared_functions(probe_header)
    assert names == ["lulesh_probe_dadd", "lulesh_probe_dmul", "lulesh_probe_math", "lulesh_probe_pipe_rates"]
    plib = lulesh.probe_library()
    assert all(hasattr(plib, n) for n in names)
    product = C.CDLL(str(lulesh.LIB_PATH))
    assert not any(hasattr(product, n) for n in names)
    assert not set(names) & set(declared_functions())


@pytest.mark.parametrize("s,r,b,c", [(5, 11, 1, 1), (9, 21, 1, 2), (8, 1, 1, 1), (7, 16, 2, 3)])
def test_host_domain_equals_oracle_initial_state(lulesh, oracle_mod, s, r, b, c):
    d = lulesh.HostDomain(s, r, b, c)
    o = oracle_mod.Oracle(s, r, b, c)
    for f in ("x", "y", "z", "xd", "yd", "zd", "nodalMass", "e", "p", "q", "v", "volo",
              "elemMass", "ss"):
        np.testing.assert_array_equal(getattr(d, f), o.field(f), err_msg=f)
    for f in ("nodelist", "nodeElemStart", "nodeElemCornerList", "regNumList"):
        np.testing.assert_array_equal(getattr(d, f), o.field(f), err_msg=f)
    v = d.view
    for f in ("lxim", "lxip", "letam", "letap", "lzetam", "lzetap", "elemBC"):
        arr = np.ctypeslib.as_array(getattr(v, f), shape=(d.numElem,))
        np.testing.assert_array_equal(arr, o.field(f), err_msg=f)
    for f in ("symmX", "symmY", "symmZ"):
        arr = np.ctypeslib.as_array(getattr(v, f), shape=(v.numSymmX,))
        np.testing.assert_array_equal(arr, o.field(f), err_msg=f)
    ts = d.time_state
    for k in ("time", "deltatime", "dtcourant", "dthydro", "stoptime", "dtmax", "dtfixed"):
        assert getattr(ts, k) == o.scalar(k), k
    assert ts.cycle == 0


def test_energy_scale(lulesh, oracle_mod):
    d = lulesh.HostDomain(6, energy_scale=0.8)
    o = oracle_mod.Oracle(6, energy_scale=0.8)
    assert d.e[0] == o.field("e")[0]
    assert d.time_state.deltatime == o.scalar("deltatime")


def _random_states(rng, n):
    for _ in range(n):
        st = {
            "time": rng.uniform(0, 1e-2),
            "deltatime": 10 ** rng.uniform(-7, -4),
            "dtcourant": 10 ** rng.uniform(-7, -3),
            "dthydro": 10 ** rng.uniform(-7, -3),
            "stoptime": 1e-2,
            "dtmax": 1e-2,
            "dtfixed": -1e-6,
            "cycle": int(rng.integers(0, 3)),
        }
        if rng.random() < 0.2:
            st["dtcourant"] = 1e20
        if rng.random() < 0.2:
            st["time"] = st["stoptime"] - st["deltatime"] * rng.uniform(0.5, 1.5)
        yield st


def test_time_increment_equals_oracle(lulesh, oracle_mod):
    rng = np.random.default_rng(7)
    d = lulesh.HostDomain(4)
    o = oracle_mod.Oracle(4)
    for st in _random_states(rng, 2000):
        ts = d.time_state
        for k, val in st.items():
            setattr(ts, k, val)
            o.set_scalar(k, float(val))
        d.time_increment()
        o.time_increment()
        for k in ("time", "deltatime"):
            assert getattr(ts, k) == o.scalar(k), (k, st)
        assert ts.cycle == o.cycle


def test_portable_cbrt_bitwise_and_accurate(lulesh, oracle_mod):
    rng = np.random.default_rng(3)
    xs = np.concatenate([10 ** rng.uniform(-300, 300, 20000), rng.uniform(1e-9, 1e-5, 20000),
                         [1.0, 8.0, 27.0, 1e-310, 5e-324, 2.0 ** -1074]])
    lib = oracle_mod.library()
    worst = 0.0
    for x in xs:
        a = lulesh.cbrt_portable(float(x))
        b = lib.lo_portable_cbrt(float(x))
        assert a == b, x
        ref = np.cbrt(x)
        worst = max(worst, abs(a - ref) / math.ulp(ref))
    assert worst <= 1.0, worst
    assert lulesh.cbrt_portable(-8.0) == -2.0 and lulesh.cbrt_portable(0.0) == 0.0


def test_domain_create_rejects_bad_sizes(lulesh):
    lib = lulesh.library()
    h = C.c_void_p()
    for args in [(0, 11, 1, 1, 1.0), (4, 0, 1, 1, 1.0), (4, 11, -1, 1, 1.0), (4, 11, 1, 1, 0.0),
                 (700, 11, 1, 1, 1.0)]:
        assert lib.lulesh_domain_create(*args, C.byref(h)) == lulesh.EINVAL, args


def test_dev_create_rejects_corrupt_topology(lulesh):
    """Index checks run on the host before any device work, so an out-of-range
    node, neighbour or corner index never reaches a kernel."""
    d = lulesh.HostDomain(4)
    lib = lulesh.library()
    h = C.c_void_p()
    for arr, bad in ((d.nodelist, d.numNode), (d.nodeElemCornerList, 8 * d.numElem),
                     (d.regNumList, 0), (d.nodeElemStart, -5)):
        i = len(arr) // 2
        old = arr[i]
        arr[i] = bad
        try:
            assert lib.lulesh_dev_create(d.view_ptr, 0, C.byref(h)) == lulesh.EINVAL
        finally:
            arr[i] = old
    lxim = np.ctypeslib.as_array(d.view.lxim, shape=(d.numElem,))
    lxim[3] = -1
    assert lib.lulesh_dev_create(d.view_ptr, 0, C.byref(h)) == lulesh.EINVAL
    lxim[3] = 2
    assert lib.lulesh_dev_create(d.view_ptr, 7, C.byref(h)) == lulesh.EINVAL


@pytest.mark.skipif(gpu_available(), reason="a GPU is present")
def test_device_path_fails_loudly_without_gpu(lulesh):
    d = lulesh.HostDomain(4)
    with pytest.raises(lulesh.LuleshError) as ei:
        lulesh.Device(d, "fp64")
    assert ei.value.status == lulesh.ENODEV


def test_symmetry_matches_oracle(lulesh, oracle_mod):
    d = lulesh.HostDomain(6)
    o = oracle_mod.Oracle(6)
    rng = np.random.default_rng(1)
    vals = rng.uniform(-1, 1, d.numElem)
    d.e[:] = vals
    o.field("e")[:] = vals
    assert d.symmetry() == o.symmetry()


def test_batch_footprint_and_loud_failure_without_gpu(lulesh):
    f = [lulesh.Batch.footprint(p, s) for p in ("fp64", "mixed") for s in (16, 64, 150)]
    assert f[0] < f[1] < f[2] and f[3] < f[4] < f[5]
    assert f[5] < f[2]  # float temporaries take less memory
    # bytes per element of the double path: about 560 of state and scratch,
    # plus 384 of element geometry kept from kinematics to the next forces
    assert f[2] / 150 ** 3 < 1000
    assert f[5] / 150 ** 3 < 600  # the mixed path keeps no geometry
    with pytest.raises(lulesh.LuleshError) as ei:
        lulesh.Batch.footprint("fp64", 0)
    assert ei.value.status == lulesh.EINVAL
    if not gpu_available():
        with pytest.raises(lulesh.LuleshError) as ei:
            lulesh.Batch("fp64", 1 << 20, 4)
        assert ei.value.status == lulesh.ENODEV


def test_largest_problem_size(lulesh):
    """Indices are int32 as in the reference (Index_t): the 8 s^3 corner
    entries fit up to s = 645, and the library takes s <= 640, refusing
    larger cubes before any allocation. At s = 640 the double path's problem
    takes 248 GB, within a GB300's 280 GB."""
    assert 8 * 645 ** 3 < 2 ** 31 <= 8 * 646 ** 3
    f = lulesh.Batch.footprint("fp64", 640)
    assert 240e9 < f < 260e9
    for call in (lambda: lulesh.Batch.footprint("fp64", 641), lambda: lulesh.HostDomain(641)):
        with pytest.raises(lulesh.LuleshError) as ei:
            call()
        assert ei.value.status == lulesh.EINVAL


def test_driver_refuses_viz_flag(lulesh):
    """The reference refuses -v when built without viz output
    (lulesh-util.cc:48-54: a message and exit(-1)); the driver does the same
    before any device work, so it needs no GPU."""
    import subprocess

    exe = ROOT / "lulesh-task-based-hpx_gb300" / "lulesh-gb300"
    r = subprocess.run([str(exe), "--s", "5", "--v"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 255  # exit(-1)
    assert "requires a build with viz output" in r.stdout
