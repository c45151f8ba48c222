"""ctypes wrapper of the CPU oracle (liblulesh_oracle.so) - TEST INFRASTRUCTURE.

The oracle is a C restatement of the reference algorithm
(esa-tu-darmstadt/lulesh-task-based-hpx lulesh.cc / lulesh-init.cc), checked
bit for bit against the reference's own sources (tests/test_oracle.py and the
golden fixtures in tests/golden/). Only tests/, __graft_entry__.smoke() and
bench.py's CPU baseline use it, to compare results with; the GPU product never
does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liblulesh_oracle.so"
CLI_PATH = HERE / "lulesh-oracle"
REF_BIN = HERE / "_ref" / "lulesh-ref"


def _ref_sources() -> Path:
    """The reference checkout the recipe builds from (LULESH_REF_DIR, else the
    default oracle/Makefile names)."""
    r = subprocess.run(["make", "-s", "--no-print-directory", "-C", str(HERE), "print-ref-dir"],
                       capture_output=True, text=True)
    return Path(r.stdout.strip() or "/nonexistent")


REF_SOURCES = _ref_sources()

NODE_FIELDS = ("x", "y", "z", "xd", "yd", "zd", "xdd", "ydd", "zdd", "fx", "fy", "fz")
ELEM_FIELDS = ("e", "p", "q", "ql", "qq", "v", "vnew", "delv", "vdov", "arealg", "ss")


# The installed copy of the reference (oracle/Makefile install-ref): its
# unmodified sources, for machines without the checkout.
REF_INSTALLED = HERE.parent / "baseline" / "_ref"


def build(ref: bool | None = None) -> None:
    """Builds the port (always) and the reference binary (when its sources
    exist). Where the checkout exists, its sources are also installed into
    baseline/_ref, so that a machine without it (the GPU host) can build and
    time the reference's own code. With ref=None (build it where the sources
    are) a failed reference build only prints a message: the binary is an
    optional checker and baseline; ref=True makes it an error."""
    subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)
    required = ref is True
    if ref is None:
        ref = REF_SOURCES.is_dir()
    if not ref:
        return
    r = subprocess.run(["make", "-s", "-j2", "-C", str(HERE), "ref", f"REF_DIR={REF_SOURCES}"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        if required:
            raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")
        print(f"oracle: the reference binary was not built ({REF_SOURCES}): {r.stderr.strip()[-300:]}")
        return
    if REF_SOURCES.resolve() != REF_INSTALLED.resolve():
        subprocess.run(["make", "-s", "-C", str(HERE), "install-ref"], check=True)


_lib = None


def library() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build(ref=False)
        lib = C.CDLL(str(LIB_PATH))
        vp, i32, dbl = C.c_void_p, C.c_int, C.c_double
        sig = {
            "lo_create": (vp, [i32, i32, i32, i32, dbl]),
            "lo_destroy": (None, [vp]),
            "lo_set_threads": (None, [i32]),
            "lo_get_threads": (i32, []),
            "lo_set_cbrt_mode": (None, [i32]),
            "lo_portable_cbrt": (dbl, [dbl]),
            "lo_time_increment": (None, [vp]),
            "lo_leapfrog": (i32, [vp]),
            "lo_run": (i32, [vp, i32]),
            "lo_symmetry": (None, [vp, C.POINTER(dbl)]),
            "lo_dump": (i32, [vp, C.c_char_p]),
            "lo_field": (C.c_void_p, [vp, C.c_char_p, C.POINTER(C.c_long), C.POINTER(i32)]),
            "lo_get_scalar": (dbl, [vp, i32]),
            "lo_set_scalar": (None, [vp, i32, dbl]),
            "lo_num_elem": (i32, [vp]),
            "lo_num_node": (i32, [vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


SCALARS = {"time": 0, "deltatime": 1, "dtcourant": 2, "dthydro": 3, "stoptime": 4, "dtmax": 5,
           "dtfixed": 6, "cycle": 7}


class Oracle:
    """One Sedov problem on the CPU oracle."""

    def __init__(self, s: int, nr: int = 11, balance: int = 1, cost: int = 1,
                 energy_scale: float = 1.0, threads: int = 0, portable_cbrt: bool = False):
        self.lib = library()
        if threads:
            self.lib.lo_set_threads(threads)
        self.lib.lo_set_cbrt_mode(1 if portable_cbrt else 0)
        self.h = self.lib.lo_create(s, nr, balance, cost, energy_scale)
        if not self.h:
            raise ValueError("bad problem size")
        self.s = s
        self.numElem = self.lib.lo_num_elem(self.h)
        self.numNode = self.lib.lo_num_node(self.h)

    def field(self, name: str) -> np.ndarray:
        n, is_int = C.c_long(), C.c_int()
        p = self.lib.lo_field(self.h, name.encode(), C.byref(n), C.byref(is_int))
        if not p:
            raise KeyError(name)
        ct = C.c_int32 if is_int.value else C.c_double
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), shape=(n.value,))

    def scalar(self, name: str) -> float:
        return self.lib.lo_get_scalar(self.h, SCALARS[name])

    def set_scalar(self, name: str, v: float) -> None:
        self.lib.lo_set_scalar(self.h, SCALARS[name], v)

    @property
    def cycle(self) -> int:
        return int(self.scalar("cycle"))

    def time_increment(self) -> None:
        self.lib.lo_time_increment(self.h)

    def leapfrog(self) -> int:
        return self.lib.lo_leapfrog(self.h)

    def run(self, max_cycles: int = 9999999) -> int:
        return self.lib.lo_run(self.h, max_cycles)

    def symmetry(self) -> tuple[float, float, float]:
        out = (C.c_double * 3)()
        self.lib.lo_symmetry(self.h, out)
        return out[0], out[1], out[2]

    def dump(self, path: str | os.PathLike) -> None:
        if self.lib.lo_dump(self.h, str(path).encode()) != 0:
            raise OSError(f"dump to {path} failed")

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.lo_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def read_dump(path: str | os.PathLike) -> dict:
    """Reads a LULESHD1 field dump (written by the reference harness or the oracle)."""
    raw = Path(path).read_bytes()
    if raw[:8] != b"LULESHD1":
        raise ValueError(f"{path}: not a LULESHD1 dump")
    hdr = np.frombuffer(raw, np.int32, 6, 8)
    s, ne, nn, cycle, nreg = (int(v) for v in hdr[:5])
    t = np.frombuffer(raw, np.float64, 4, 32)
    out = {"s": s, "numElem": ne, "numNode": nn, "cycle": cycle, "numReg": nreg,
           "time": t[0], "deltatime": t[1], "dtcourant": t[2], "dthydro": t[3]}
    off = 64
    for f in NODE_FIELDS:
        out[f] = np.frombuffer(raw, np.float64, nn, off).copy()
        off += 8 * nn
    for f in ELEM_FIELDS:
        out[f] = np.frombuffer(raw, np.float64, ne, off).copy()
        off += 8 * ne
    return out
