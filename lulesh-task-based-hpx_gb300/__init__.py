"""Python binding of the GB300 LULESH Lagrange-leapfrog step (ctypes over the C ABI).

The library (liblulesh_gb300.so, built in-tree by build.py) is the product:
hand-written sm_103a kernels behind the C ABI declared in
include/lulesh_gb300.h. This module only marshals pointers; it has no compute
of its own and no CPU fallback: if the library is missing or no GPU is
present, the device calls raise.

    dom = HostDomain(s=30, nr=11)           # Domain::Domain (lulesh-init.cc:10-183)
    dev = Device(dom, precision="fp64")     # device mirrors of the Domain arrays
    cycles = dev.run()                       # time loop of hpx_main (lulesh.cc:2374-2386)
    dev.download()                           # fields back into dom's arrays
    dom.e[0], dom.symmetry()                 # VerifyAndWriteFinalOutput's checks
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liblulesh_gb300.so"

OK, EVOLUME, EQSTOP, EINVAL, ECUDA, ENOMEM, ENODEV, ETIMEOUT = 0, -1, -2, -10, -11, -12, -13, -14
PRECISION = {"fp64": 0, "fp64_exact": 1, "mixed": 2}

F_POS, F_VEL, F_ACC, F_FORCE, F_EPQ, F_V, F_QLQQ, F_KIN, F_SS = (1 << k for k in range(9))
F_STEP_IN = F_POS | F_VEL | F_EPQ | F_V | F_SS
F_STEP_OUT = F_POS | F_VEL | F_ACC | F_FORCE | F_EPQ | F_V | F_QLQQ | F_KIN | F_SS
F_ALL = 0x1FF
F_MESH = 0x200  # the constant mesh arrays, download only

PHASE_FORCES, PHASE_NODES, PHASE_KINEMATICS, PHASE_MATERIAL = range(4)

NODE_FIELDS = ("x", "y", "z", "xd", "yd", "zd", "xdd", "ydd", "zdd", "fx", "fy", "fz")
ELEM_FIELDS = ("e", "p", "q", "ql", "qq", "v", "vnew", "delv", "vdov", "arealg", "ss")


class LuleshError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {status} ({_strerror(status)})")


class Params(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "e_cut", "p_cut", "q_cut", "v_cut", "u_cut", "hgcoef", "ss4o3", "qstop", "monoq_max_slope",
        "monoq_limiter_mult", "qlc_monoq", "qqc_monoq", "qqc", "eosvmax", "eosvmin", "pmin", "emin",
        "dvovmax", "refdens")]


class TimeState(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "time", "deltatime", "dtcourant", "dthydro", "dtfixed", "deltatimemultlb", "deltatimemultub",
        "dtmax", "stoptime")] + [("cycle", C.c_int32), ("pad_", C.c_int32)]


_PD, _PI = C.POINTER(C.c_double), C.POINTER(C.c_int32)


class Profile(C.Structure):
    _fields_ = [("total_ms", C.c_double), ("kernel_ms", C.c_double * 4), ("cycles", C.c_int64),
                ("launches", C.c_int64)]


KERNELS = ("forces", "nodes", "kinematics", "material")

TL_MAX = 96
# stage kinds of lulesh_leapfrog's timeline (LULESH_TL_*)
TL_STAGES = {1: "upload", 2: "forces", 3: "energy_up", 4: "nodes", 5: "nodes_down", 6: "kinematics",
             7: "kinematics_down", 8: "material", 9: "material_down", 10: "end"}


class Timeline(C.Structure):
    _fields_ = [("n", C.c_int32), ("stage", C.c_int32 * TL_MAX), ("index", C.c_int32 * TL_MAX),
                ("ms", C.c_float * TL_MAX), ("wall_ms", C.c_double)]


class Problem(C.Structure):
    _fields_ = [("s", C.c_int32), ("nr", C.c_int32), ("balance", C.c_int32), ("cost", C.c_int32),
                ("energy_scale", C.c_double), ("stoptime", C.c_double), ("max_cycles", C.c_int32),
                ("pad_", C.c_int32)]


class SlotStatus(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("in_use", "active", "cycle", "err", "err_elem", "numElem", "s",
                                          "pad_")] + \
               [(n, C.c_double) for n in ("time", "deltatime", "dtcourant", "dthydro")]


class BatchTuning(C.Structure):
    _fields_ = [("block", C.c_int32 * 4), ("blocks_per_sm", C.c_int32 * 4), ("grab", C.c_int32 * 4),
                ("tile", C.c_int32), ("pad_", C.c_int32), ("ms_per_cycle", C.c_double)]


class Request(C.Structure):
    _fields_ = [("problem", Problem), ("arrival_s", C.c_double)]


class RequestResult(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("cycles", "err", "s", "pad_")] + \
               [(n, C.c_double) for n in ("arrival_s", "admitted_s", "finished_s", "time_to_solution_s",
                                          "e0", "maxabs", "totabs", "maxrel")] + [("zone_cycles", C.c_int64)]


class VerifyResult(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("e0", "maxabs", "totabs", "maxrel")] + \
               [("cycle", C.c_int32), ("nx", C.c_int32)]


def _verify_dict(r: VerifyResult) -> dict:
    return {k: getattr(r, k) for k, _ in VerifyResult._fields_}


class ServeStats(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("wall_s", "device_s", "zone_cycles_per_s", "p50_s", "p99_s",
                                          "mean_s")] + \
               [("zone_cycles", C.c_int64), ("launches", C.c_int64), ("served", C.c_int32),
                ("max_resident", C.c_int32), ("peak_resident_bytes", C.c_int64), ("p50_queue_s", C.c_double),
                ("p99_queue_s", C.c_double)]


class DomainView(C.Structure):
    _fields_ = (
        [(n, C.c_int32) for n in ("numElem", "numNode", "sizeX", "numReg", "cost", "numSymmX",
                                   "numSymmY", "numSymmZ")]
        + [(n, _PD) for n in NODE_FIELDS]
        + [("nodalMass", _PD), ("symmX", _PI), ("symmY", _PI), ("symmZ", _PI), ("nodelist", _PI)]
        + [(n, _PI) for n in ("lxim", "lxip", "letam", "letap", "lzetam", "lzetap", "elemBC")]
        + [(n, _PD) for n in ELEM_FIELDS]
        + [("volo", _PD), ("elemMass", _PD), ("nodeElemStart", _PI), ("nodeElemCornerList", _PI),
           ("regNumList", _PI), ("params", Params), ("time", C.POINTER(TimeState))]
    )


_lib = None


def library() -> C.CDLL:
    """Loads liblulesh_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is not built: run __graft_entry__.build() or "
                           f"python {HERE / 'build.py'}")
    lib = C.CDLL(str(LIB_PATH))
    vp, i32, i64, u32, dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_uint32, C.c_double
    sig = {
        "lulesh_domain_create": (i32, [i32, i32, i32, i32, dbl, C.POINTER(vp)]),
        "lulesh_domain_get_view": (C.POINTER(DomainView), [vp]),
        "lulesh_domain_destroy": (None, [vp]),
        "lulesh_time_increment": (i32, [C.POINTER(TimeState)]),
        "lulesh_symmetry": (i32, [C.POINTER(DomainView), C.POINTER(dbl)]),
        "lulesh_dev_create": (i32, [C.POINTER(DomainView), i32, C.POINTER(vp)]),
        "lulesh_dev_destroy": (None, [vp]),
        "lulesh_dev_create_problem": (i32, [C.POINTER(Problem), i32, C.POINTER(TimeState), C.POINTER(vp)]),
        "lulesh_dev_upload": (i32, [vp, C.POINTER(DomainView), u32]),
        "lulesh_dev_download": (i32, [vp, C.POINTER(DomainView), u32]),
        "lulesh_dev_verify": (i32, [vp, i32, C.POINTER(VerifyResult)]),
        "lulesh_dev_step": (i32, [vp, dbl, C.POINTER(dbl), C.POINTER(dbl)]),
        "lulesh_leapfrog": (i32, [vp, C.POINTER(DomainView)]),
        "lulesh_dev_run": (i32, [vp, C.POINTER(TimeState), i32, C.POINTER(i32)]),
        "lulesh_dev_run_graph": (i32, [vp, C.POINTER(TimeState), i32, i32, C.POINTER(i32)]),
        "lulesh_dev_phase": (i32, [vp, i32, dbl]),
        "lulesh_dev_corner_forces": (i32, [vp, _PD, _PD, _PD]),
        "lulesh_dev_gradients": (i32, [vp, _PD]),
        "lulesh_dev_error_elem": (i32, [vp]),
        "lulesh_dev_launch_count": (i64, [vp]),
        "lulesh_dev_profile_begin": (i32, [vp]),
        "lulesh_dev_profile_end": (i32, [vp, C.POINTER(Profile)]),
        "lulesh_leapfrog_timeline": (i32, [vp, i32]),
        "lulesh_leapfrog_timeline_read": (i32, [vp, C.POINTER(Timeline)]),
        "lulesh_domain_pin": (i32, [vp, i32]),
        "lulesh_set_device": (i32, [i32]),
        "lulesh_batch_create": (i32, [i32, C.c_uint64, i32, C.POINTER(vp)]),
        "lulesh_batch_destroy": (None, [vp]),
        "lulesh_batch_footprint": (i32, [i32, i32, C.POINTER(C.c_uint64)]),
        "lulesh_batch_admit": (i32, [vp, C.POINTER(Problem), C.POINTER(i32)]),
        "lulesh_batch_retire": (i32, [vp, i32]),
        "lulesh_batch_run": (i32, [vp, i32, C.POINTER(i32), C.POINTER(dbl)]),
        "lulesh_batch_status": (i32, [vp, C.POINTER(SlotStatus), i32]),
        "lulesh_batch_download": (i32, [vp, i32, C.POINTER(DomainView), u32]),
        "lulesh_batch_verify": (i32, [vp, i32, C.POINTER(VerifyResult)]),
        "lulesh_batch_autotune": (i32, [vp, i32, C.POINTER(BatchTuning)]),
        "lulesh_batch_get_tuning": (i32, [vp, C.POINTER(BatchTuning)]),
        "lulesh_batch_set_tuning": (i32, [vp, C.POINTER(BatchTuning)]),
        "lulesh_batch_launch_count": (i64, [vp]),
        "lulesh_batch_admit_view": (i32, [vp, C.POINTER(DomainView), dbl, i32, C.POINTER(i32)]),
        "lulesh_batch_origin_energy": (i32, [vp, i32, C.POINTER(dbl)]),
        "lulesh_serve": (i32, [i32, C.c_uint64, i32, C.POINTER(Request), i32, dbl,
                               C.POINTER(RequestResult), C.POINTER(ServeStats)]),
        "lulesh_cbrt_portable": (dbl, [dbl]),
        "lulesh_strerror": (C.c_char_p, [i32]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _strerror(status: int) -> str:
    try:
        return library().lulesh_strerror(status).decode()
    except Exception:  # library not loadable: plain code
        return "status"


def _check(status: int, what: str) -> None:
    if status != OK:
        raise LuleshError(status, what)


def _np(ptr, n: int, dtype) -> np.ndarray:
    return np.ctypeslib.as_array(ptr, shape=(n,)).view(dtype)


class HostDomain:
    """The Sedov problem of Domain::Domain built by the library's host code.

    Field arrays (numpy views onto the library's host vectors): the node fields
    x y z xd yd zd xdd ydd zdd fx fy fz nodalMass and the element fields
    e p q ql qq v vnew delv vdov arealg ss volo elemMass, plus the index
    arrays nodelist nodeElemStart nodeElemCornerList regNumList, the face
    neighbours lxim lxip letam letap lzetam lzetap and elemBC.
    """

    def __init__(self, s: int, nr: int = 11, balance: int = 1, cost: int = 1,
                 energy_scale: float = 1.0):
        lib = library()
        h = C.c_void_p()
        _check(lib.lulesh_domain_create(s, nr, balance, cost, energy_scale, C.byref(h)),
               "lulesh_domain_create")
        self._h = h
        self._lib = lib
        self.s, self.nr, self.balance, self.cost = s, nr, balance, cost
        self.view_ptr = lib.lulesh_domain_get_view(h)
        v = self.view_ptr.contents
        self.view = v
        self.numElem, self.numNode = v.numElem, v.numNode
        for f in NODE_FIELDS:
            setattr(self, f, _np(getattr(v, f), v.numNode, np.float64))
        for f in ELEM_FIELDS:
            setattr(self, f, _np(getattr(v, f), v.numElem, np.float64))
        self.nodalMass = _np(v.nodalMass, v.numNode, np.float64)
        self.volo = _np(v.volo, v.numElem, np.float64)
        self.elemMass = _np(v.elemMass, v.numElem, np.float64)
        self.nodelist = _np(v.nodelist, 8 * v.numElem, np.int32)
        self.nodeElemStart = _np(v.nodeElemStart, v.numNode + 1, np.int32)
        self.nodeElemCornerList = _np(v.nodeElemCornerList, 8 * v.numElem, np.int32)
        self.regNumList = _np(v.regNumList, v.numElem, np.int32)
        for f in ("lxim", "lxip", "letam", "letap", "lzetam", "lzetap", "elemBC"):
            setattr(self, f, _np(getattr(v, f), v.numElem, np.int32))
        self.time_state = v.time.contents

    def symmetry(self) -> tuple[float, float, float]:
        out = (C.c_double * 3)()
        _check(self._lib.lulesh_symmetry(self.view_ptr, out), "lulesh_symmetry")
        return out[0], out[1], out[2]

    def time_increment(self) -> None:
        _check(self._lib.lulesh_time_increment(C.byref(self.time_state)), "lulesh_time_increment")

    @property
    def cycle(self) -> int:
        return self.time_state.cycle

    def pin(self, on: bool = True) -> None:
        """Page-locks the mutable host arrays (fast copies for Device.leapfrog)."""
        _check(self._lib.lulesh_domain_pin(self._h, 1 if on else 0), "lulesh_domain_pin")
        self._pinned = on

    def close(self) -> None:
        if getattr(self, "_h", None):
            if getattr(self, "_pinned", False):
                self._lib.lulesh_domain_pin(self._h, 0)
            self._lib.lulesh_domain_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class DeviceBuilt:
    """Time state of a problem built on the device (Device.from_problem): it
    has no host arrays; download into the view of a HostDomain of the same
    problem when fields are needed."""

    view_ptr = None

    def __init__(self, s: int):
        self.s = s
        self.time_state = TimeState()

    @property
    def cycle(self) -> int:
        return self.time_state.cycle


class Device:
    """Device mirror of a HostDomain; every method runs the sm_103a kernels."""

    @classmethod
    def from_problem(cls, s: int, nr: int = 11, balance: int = 1, cost: int = 1,
                     energy_scale: float = 1.0, precision: str = "fp64", stoptime: float = 0.0) -> "Device":
        """Builds the problem directly in device memory (lulesh_dev_create_problem):
        no host Domain is built and nothing but the region runs is uploaded."""
        lib = library()
        self = cls.__new__(cls)
        state = DeviceBuilt(s)
        prob = Problem(s, nr, balance, cost, energy_scale, stoptime, 0, 0)
        h = C.c_void_p()
        _check(lib.lulesh_dev_create_problem(C.byref(prob), PRECISION[precision], C.byref(state.time_state),
                                             C.byref(h)), "lulesh_dev_create_problem")
        self._h = h
        self._lib = lib
        self.dom = state
        self.precision = precision
        return self

    def __init__(self, dom: HostDomain, precision: str = "fp64"):
        lib = library()
        h = C.c_void_p()
        _check(lib.lulesh_dev_create(dom.view_ptr, PRECISION[precision], C.byref(h)),
               "lulesh_dev_create")
        self._h = h
        self._lib = lib
        self.dom = dom
        self.precision = precision

    def upload(self, mask: int = F_ALL) -> None:
        _check(self._lib.lulesh_dev_upload(self._h, self.dom.view_ptr, mask), "lulesh_dev_upload")

    def download(self, mask: int = F_ALL, into: "HostDomain | None" = None) -> None:
        """Device fields -> the host view of self.dom, or of `into` (a HostDomain
        of the same problem; needed for a device-built problem)."""
        target = self.dom if into is None else into
        if target.view_ptr is None:
            raise ValueError("a device-built problem has no host arrays: pass into=HostDomain(...)")
        _check(self._lib.lulesh_dev_download(self._h, target.view_ptr, mask), "lulesh_dev_download")

    def verify(self) -> dict:
        """Final report computed on the device (lulesh_dev_verify): e0,
        maxabs, totabs, maxrel, cycle, nx; no field is downloaded."""
        r = VerifyResult()
        _check(self._lib.lulesh_dev_verify(self._h, self.dom.time_state.cycle, C.byref(r)),
               "lulesh_dev_verify")
        return _verify_dict(r)

    def step(self, dt: float) -> tuple[float, float]:
        dtc, dth = C.c_double(), C.c_double()
        _check(self._lib.lulesh_dev_step(self._h, dt, C.byref(dtc), C.byref(dth)), "lulesh_dev_step")
        return dtc.value, dth.value

    def leapfrog(self) -> None:
        """Drop-in LagrangeLeapFrog on the host Domain (upload, step, download)."""
        _check(self._lib.lulesh_leapfrog(self._h, self.dom.view_ptr), "lulesh_leapfrog")

    def run(self, max_cycles: int = 9999999) -> int:
        n = C.c_int32()
        _check(self._lib.lulesh_dev_run(self._h, C.byref(self.dom.time_state), max_cycles, C.byref(n)),
               "lulesh_dev_run")
        return n.value

    def run_graph(self, max_cycles: int = 9999999, sync_every: int = 32) -> int:
        n = C.c_int32()
        _check(self._lib.lulesh_dev_run_graph(self._h, C.byref(self.dom.time_state), max_cycles,
                                              sync_every, C.byref(n)), "lulesh_dev_run_graph")
        return n.value

    def phase(self, phase: int, dt: float = 0.0) -> None:
        _check(self._lib.lulesh_dev_phase(self._h, phase, dt), "lulesh_dev_phase")

    def corner_forces(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        n = 8 * self.dom.numElem
        out = [np.empty(n, np.float64) for _ in range(3)]
        ptrs = [o.ctypes.data_as(_PD) for o in out]
        _check(self._lib.lulesh_dev_corner_forces(self._h, *ptrs), "lulesh_dev_corner_forces")
        return tuple(out)

    def gradients(self) -> np.ndarray:
        out = np.empty(6 * self.dom.numElem, np.float64)
        _check(self._lib.lulesh_dev_gradients(self._h, out.ctypes.data_as(_PD)), "lulesh_dev_gradients")
        return out.reshape(6, self.dom.numElem)

    def profile_begin(self) -> None:
        _check(self._lib.lulesh_dev_profile_begin(self._h), "lulesh_dev_profile_begin")

    def profile_end(self) -> dict:
        p = Profile()
        _check(self._lib.lulesh_dev_profile_end(self._h, C.byref(p)), "lulesh_dev_profile_end")
        return {"total_ms": p.total_ms, "kernel_ms": dict(zip(KERNELS, list(p.kernel_ms))),
                "cycles": p.cycles, "launches": p.launches}

    def timeline(self, on: bool = True) -> None:
        """Records the stage boundaries of the following leapfrog calls."""
        _check(self._lib.lulesh_leapfrog_timeline(self._h, 1 if on else 0), "lulesh_leapfrog_timeline")

    def timeline_read(self) -> dict:
        """The last leapfrog call's stage marks: [(stage, index, ms after the
        call's first device work)] and the call's host wall time."""
        t = Timeline()
        _check(self._lib.lulesh_leapfrog_timeline_read(self._h, C.byref(t)), "lulesh_leapfrog_timeline_read")
        marks = [(TL_STAGES.get(t.stage[k], str(t.stage[k])), t.index[k], t.ms[k]) for k in range(t.n)]
        return {"marks": marks, "wall_ms": t.wall_ms}

    @property
    def error_elem(self) -> int:
        return self._lib.lulesh_dev_error_elem(self._h)

    @property
    def launches(self) -> int:
        if not self._h:
            raise RuntimeError("launch count of a closed handle")
        return self._lib.lulesh_dev_launch_count(self._h)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.lulesh_dev_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def cbrt_portable(x: float) -> float:
    return library().lulesh_cbrt_portable(x)


def set_device(device: int) -> None:
    _check(library().lulesh_set_device(device), "lulesh_set_device")


_probe_lib = None
PROBE_LIB_PATH = HERE / "liblulesh_probe.so"


def probe_library() -> C.CDLL:
    """Loads liblulesh_probe.so, the measurement probes (not part of the
    step's C ABI; the benchmark and the accuracy tests use it)."""
    global _probe_lib
    if _probe_lib is None:
        if not PROBE_LIB_PATH.exists():
            raise RuntimeError(f"{PROBE_LIB_PATH} is not built: run __graft_entry__.build()")
        lib = C.CDLL(str(PROBE_LIB_PATH))
        lib.lulesh_probe_pipe_rates.restype = C.c_int32
        lib.lulesh_probe_pipe_rates.argtypes = [C.POINTER(C.c_double)]
        lib.lulesh_probe_math.restype = C.c_int32
        lib.lulesh_probe_math.argtypes = [C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                          C.c_int64]
        for name in ("lulesh_probe_dmul", "lulesh_probe_dadd"):
            getattr(lib, name).restype = C.c_int32
            getattr(lib, name).argtypes = [C.POINTER(C.c_double)] * 4 + [C.c_int64]
        _probe_lib = lib
    return _probe_lib


def pipe_rates() -> dict:
    """Measured rates (ops/s) of the current GPU: double FMA, add, divide, sqrt,
    float FMA, double multiplies on the FP64 pipe, on the integer pipes
    (dmul_ipipe) and on both at once, and double adds on the integer pipes
    (dadd_ipipe) and on both at once."""
    out = (C.c_double * 10)()
    _check(probe_library().lulesh_probe_pipe_rates(out), "lulesh_probe_pipe_rates")
    return dict(zip(("dfma", "dadd", "ddiv", "dsqrt", "ffma", "dmul", "dmul_ipipe", "dmul_both", "dadd_ipipe",
                     "dadd_both"), list(out)))


MATH_FUNCTIONS = {"rcp": 0, "rcbrt": 1, "sqrt": 2, "rsqrt": 3, "rcp_seed": 4, "narrow": 5, "split_hi": 6,
                  "split_lo": 7}


def probe_math(fn: str, x):
    """The fast variants' helper `fn` (MATH_FUNCTIONS) evaluated on the
    device for the doubles x; returns a numpy array."""
    import numpy as np

    xs = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(xs)
    _check(probe_library().lulesh_probe_math(MATH_FUNCTIONS[fn], xs.ctypes.data_as(C.POINTER(C.c_double)),
                                       out.ctypes.data_as(C.POINTER(C.c_double)), xs.size),
           "lulesh_probe_math")
    return out


def _probe_pair(name: str, a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    native, ipipe = np.empty_like(a), np.empty_like(a)
    pd = C.POINTER(C.c_double)
    _check(getattr(probe_library(), name)(a.ctypes.data_as(pd), b.ctypes.data_as(pd),
                                          native.ctypes.data_as(pd), ipipe.ctypes.data_as(pd), a.size), name)
    return native, ipipe


def probe_dmul(a, b):
    """The products a * b on the device by the FP64 pipe's multiply and by the
    integer-pipe multiply the step kernels use; returns (native, ipipe)."""
    return _probe_pair("lulesh_probe_dmul", a, b)


def probe_dadd(a, b):
    """The sums a + b on the device by the FP64 pipe's add and by the
    integer-pipe add of the probes (dadd_ipipe); returns (native, ipipe)."""
    return _probe_pair("lulesh_probe_dadd", a, b)


def serve(requests: list[dict], precision: str = "mixed", hbm_budget: int = 160 << 30,
          max_slots: int = 256, sync_ms: float = 20.0) -> tuple[list[dict], dict]:
    """Continuous-batching serving loop (lulesh_serve). Each request is a dict
    with s, nr, balance, cost, energy_scale, stoptime, max_cycles (as
    Batch.admit) and arrival_s (seconds after the call starts)."""
    n = len(requests)
    arr = (Request * n)()
    for i, r in enumerate(requests):
        arr[i].problem = Problem(r["s"], r.get("nr", 11), r.get("balance", 1), r.get("cost", 1),
                                 r.get("energy_scale", 1.0), r.get("stoptime", 0.0),
                                 r.get("max_cycles", 0), 0)
        arr[i].arrival_s = r["arrival_s"]
    res = (RequestResult * n)()
    st = ServeStats()
    _check(library().lulesh_serve(PRECISION[precision], hbm_budget, max_slots, arr, n, sync_ms, res,
                                  C.byref(st)), "lulesh_serve")
    out = [{k: getattr(x, k) for k, _ in RequestResult._fields_ if k != "pad_"} for x in res]
    stats = {k: getattr(st, k) for k, _ in ServeStats._fields_}
    return out, stats


def _tuning_dict(t: BatchTuning) -> dict:
    return {"block": list(t.block), "blocks_per_sm": list(t.blocks_per_sm), "grab": list(t.grab),
            "tile": t.tile, "ms_per_cycle": t.ms_per_cycle}


class Batch:
    """A device pool of independent Sedov problems, one CUDA graph per cycle.

    Problems are admitted into slots (each built by Domain::Domain's set-up,
    optionally with a scaled deposit, its own stoptime and cycle limit), all
    active slots advance together with run(), and finished slots are retired
    to free their pool memory.
    """

    def __init__(self, precision: str = "fp64", pool_bytes: int = 8 << 30, max_slots: int = 64):
        lib = library()
        h = C.c_void_p()
        _check(lib.lulesh_batch_create(PRECISION[precision], pool_bytes, max_slots, C.byref(h)),
               "lulesh_batch_create")
        self._h = h
        self._lib = lib
        self.precision = precision
        self.max_slots = max_slots
        self.specs: dict[int, dict] = {}

    @staticmethod
    def footprint(precision: str, s: int) -> int:
        out = C.c_uint64()
        _check(library().lulesh_batch_footprint(PRECISION[precision], s, C.byref(out)),
               "lulesh_batch_footprint")
        return out.value

    def admit(self, s: int, nr: int = 11, balance: int = 1, cost: int = 1, energy_scale: float = 1.0,
              stoptime: float = 0.0, max_cycles: int = 0) -> int:
        p = Problem(s, nr, balance, cost, energy_scale, stoptime, max_cycles, 0)
        slot = C.c_int32()
        _check(self._lib.lulesh_batch_admit(self._h, C.byref(p), C.byref(slot)), "lulesh_batch_admit")
        self.specs[slot.value] = {"s": s, "nr": nr, "balance": balance, "cost": cost,
                                  "energy_scale": energy_scale}
        return slot.value

    def try_admit(self, **kw) -> int | None:
        """admit(), or None when the pool or the slots are full."""
        try:
            return self.admit(**kw)
        except LuleshError as e:
            if e.status == ENOMEM:
                return None
            raise

    def retire(self, slot: int) -> None:
        _check(self._lib.lulesh_batch_retire(self._h, slot), "lulesh_batch_retire")
        self.specs.pop(slot, None)

    def run(self, cycles: int) -> tuple[int, float]:
        """Replays `cycles` cycles; returns (slots still active, device ms)."""
        active, ms = C.c_int32(), C.c_double()
        _check(self._lib.lulesh_batch_run(self._h, cycles, C.byref(active), C.byref(ms)),
               "lulesh_batch_run")
        return active.value, ms.value

    def status(self) -> list[dict]:
        arr = (SlotStatus * self.max_slots)()
        _check(self._lib.lulesh_batch_status(self._h, arr, self.max_slots), "lulesh_batch_status")
        out = []
        for i, st in enumerate(arr):
            if st.in_use:
                out.append({"slot": i, **{k: getattr(st, k) for k, _ in SlotStatus._fields_ if k != "pad_"}})
        return out

    def download(self, slot: int, mask: int = F_ALL) -> HostDomain:
        """Fields of a slot, in a fresh HostDomain of the same problem."""
        sp = self.specs[slot]
        dom = HostDomain(sp["s"], sp["nr"], sp["balance"], sp["cost"], sp["energy_scale"])
        _check(self._lib.lulesh_batch_download(self._h, slot, dom.view_ptr, mask), "lulesh_batch_download")
        return dom

    def verify(self, slot: int) -> dict:
        """Final report of a slot computed on the device (lulesh_batch_verify)."""
        r = VerifyResult()
        _check(self._lib.lulesh_batch_verify(self._h, slot, C.byref(r)), "lulesh_batch_verify")
        return _verify_dict(r)

    def autotune(self, cycles: int = 2) -> dict:
        t = BatchTuning()
        _check(self._lib.lulesh_batch_autotune(self._h, cycles, C.byref(t)), "lulesh_batch_autotune")
        return _tuning_dict(t)

    def tuning(self) -> dict:
        t = BatchTuning()
        _check(self._lib.lulesh_batch_get_tuning(self._h, C.byref(t)), "lulesh_batch_get_tuning")
        return _tuning_dict(t)

    def set_tuning(self, block, blocks_per_sm, tile: int, grab=(1, 1, 1, 1)) -> None:
        t = BatchTuning((C.c_int32 * 4)(*block), (C.c_int32 * 4)(*blocks_per_sm), (C.c_int32 * 4)(*grab),
                        tile, 0, 0.0)
        _check(self._lib.lulesh_batch_set_tuning(self._h, C.byref(t)), "lulesh_batch_set_tuning")

    @property
    def launches(self) -> int:
        if not self._h:
            raise RuntimeError("launch count of a closed handle")
        return self._lib.lulesh_batch_launch_count(self._h)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.lulesh_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
