"""In-tree build of the GB300 LULESH library and command-line driver.

Compiles every translation unit under csrc/ for sm_103a with nvcc (in
parallel), links liblulesh_gb300.so next to this file, the lulesh-gb300
executable (the reference's command line on top of the C ABI) and
liblulesh_probe.so (measurement probes for the benchmark and tests only).

Floating-point contraction is part of the numerics contract:
  * fp64_exact.cu, time_increment.cu, verify.cu and device_init.cu are
    built with --fmad=false, so the exact double path, the device
    TimeIncrement, the device final report and the device problem build
    round every operation separately, as the reference source is written;
  * domain.cpp (problem set-up, host TimeIncrement) is built with
    -ffp-contract=off so the host numbers do not depend on whether the host
    compiler fuses multiply-adds (GCC does by default on aarch64).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "liblulesh_gb300.so"
EXE = HERE / "lulesh-gb300"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                      f"-I{ROOT / 'include'}", f"-I{CSRC}"]

# (source, extra nvcc flags)
UNITS = [
    ("fp64_fast.cu", []),
    ("fp64_exact.cu", ["--fmad=false"]),
    ("mixed.cu", []),
    ("time_increment.cu", ["--fmad=false"]),
    ("verify.cu", ["--fmad=false"]),
    ("device_init.cu", ["--fmad=false"]),
    ("capi.cu", []),
    ("noalloc.cu", []),
    ("batch.cu", []),
    ("serve.cu", []),
    ("domain.cpp", ["-x", "cu", "--fmad=false"]),
]
# The measurement probes (pipe rates, the fast helpers' accuracy) form their
# own library for the benchmark and the accuracy tests; the product library
# does not contain them.
PROBE_UNITS = [
    ("probe.cu", []),
    ("probe_math.cu", []),
]
PROBE_LIB = HERE / "liblulesh_probe.so"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build lulesh_gb300")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Builds liblulesh_gb300.so and lulesh-gb300; returns the library path."""
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "lulesh_gb300.h"]
    jobs = []
    objs, probe_objs = [], []
    for units, out in ((UNITS, objs), (PROBE_UNITS, probe_objs)):
        for src, extra in units:
            s = CSRC / src
            o = BUILD / (src + ".o")
            out.append(o)
            if force or _stale(o, [s] + headers):
                jobs.append([cc, *NVCC_COMMON, *extra, "-c", str(s), "-o", str(o)])
    with ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        for cmd in jobs:
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
        list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        _run([cc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart", "-lpthread"])
    if force or jobs or _stale(PROBE_LIB, probe_objs):
        _run([cc, *ARCH, "-shared", "-o", str(PROBE_LIB), *map(str, probe_objs), "-lcudart"])
    drv = CSRC / "driver.cpp"
    if drv.exists() and (force or _stale(EXE, [drv, LIB] + headers)):
        _run([cc, *ARCH, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off", f"-I{ROOT / 'include'}",
              "-x", "cu", str(drv), "-o", str(EXE), f"-L{HERE}", "-llulesh_gb300",
              f"-Xlinker", f"-rpath,{HERE}"])
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    print(LIB)
