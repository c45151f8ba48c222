"""Problems built on the device (lulesh_dev_create_problem, and every batch
admission through lulesh_batch_admit) against the host build of
Domain::Domain (lulesh-init.cc:10-183), which itself equals the oracle's
initial state bit for bit (tests/test_host.py).

Bar: every array, constant and mutable, and the initial time state equal
bit for bit; the exact variant then runs identically from either build.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NODE = ("x", "y", "z", "xd", "yd", "zd", "xdd", "ydd", "zdd", "fx", "fy", "fz")
ELEM = ("e", "p", "q", "ql", "qq", "v", "vnew", "delv", "vdov", "arealg", "ss")
MESH = ("nodalMass", "volo", "elemMass", "nodelist", "lxim", "lxip", "letam", "letap", "lzetam",
        "lzetap", "elemBC", "nodeElemStart", "nodeElemCornerList")
TIME = ("time", "deltatime", "dtcourant", "dthydro", "dtfixed", "deltatimemultlb",
        "deltatimemultub", "dtmax", "stoptime", "cycle")

PROBLEMS = [(1, 1, 1, 1, 1.0), (2, 11, 1, 1, 1.0), (8, 11, 1, 1, 1.0), (12, 21, 1, 1, 1.0),
            (9, 16, 2, 2, 1.0), (10, 1, 1, 1, 1.3), (7, 11, 0, 3, 0.7), (31, 21, 1, 1, 1.0)]


def _fresh_view(lulesh, s, nr, b, c, scale):
    """A host Domain of the same problem with every array it will receive
    poisoned, so a field the download misses shows up."""
    dom = lulesh.HostDomain(s, nr, b, c, scale)
    for f in NODE + ELEM + ("nodalMass", "volo", "elemMass"):
        getattr(dom, f)[:] = np.nan
    for f in MESH[3:]:
        getattr(dom, f)[:] = -7
    return dom


@pytest.mark.parametrize("problem", PROBLEMS, ids=[f"s{p[0]}r{p[1]}b{p[2]}c{p[3]}" for p in PROBLEMS])
def test_device_build_equals_host_build(lulesh, problem):
    s, nr, b, c, scale = problem
    host = lulesh.HostDomain(s, nr, b, c, scale)
    dev = lulesh.Device.from_problem(s, nr, b, c, scale, "fp64_exact")
    for f in TIME:
        assert getattr(dev.dom.time_state, f) == getattr(host.time_state, f), f
    got = _fresh_view(lulesh, s, nr, b, c, scale)
    dev.download(lulesh.F_ALL | lulesh.F_MESH, into=got)
    for f in NODE + ELEM + MESH:
        np.testing.assert_array_equal(getattr(got, f), getattr(host, f), err_msg=f)
    dev.close()


@pytest.mark.parametrize("precision", ["fp64_exact", "fp64", "mixed"])
def test_device_built_run_equals_host_built_run(lulesh, precision):
    """The derived arrays of the build (repeat counts, repeat-count order,
    symmetry bits, 1/mass, float-pair mirrors) are exercised by running:
    the device-built problem runs bit for bit as the host-built one."""
    s, nr, b, c, scale = 11, 21, 1, 2, 1.1
    host = lulesh.HostDomain(s, nr, b, c, scale)
    ref = lulesh.Device(host, precision)
    dev = lulesh.Device.from_problem(s, nr, b, c, scale, precision)
    n_ref, n_dev = ref.run(60), dev.run(60)
    assert n_ref == n_dev == 60
    for f in TIME:
        assert getattr(dev.dom.time_state, f) == getattr(host.time_state, f), f
    ref.download()
    got = _fresh_view(lulesh, s, nr, b, c, scale)
    dev.download(into=got)
    for f in NODE + ELEM:
        np.testing.assert_array_equal(getattr(got, f), getattr(host, f), err_msg=f)
    assert dev.verify() == ref.verify()
    ref.close()
    dev.close()


def test_device_build_with_stoptime_and_limits(lulesh):
    dev = lulesh.Device.from_problem(6, stoptime=2e-3)
    assert dev.dom.time_state.stoptime == 2e-3
    n = dev.run()
    solo = lulesh.HostDomain(6)
    solo.time_state.stoptime = 2e-3
    ref = lulesh.Device(solo)
    assert n == ref.run() and dev.verify() == ref.verify()
    with pytest.raises(lulesh.LuleshError):
        lulesh.Device.from_problem(0)
    with pytest.raises(lulesh.LuleshError):
        lulesh.Device.from_problem(8, nr=0)
    with pytest.raises(ValueError):
        dev.download()  # no host arrays: a view must be given
    with pytest.raises(lulesh.LuleshError):
        ref.upload(lulesh.F_MESH)  # the mesh is fixed at creation
