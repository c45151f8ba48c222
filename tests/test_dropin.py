"""The drop-in adapter compiled against the reference itself.

lulesh-task-based-hpx_gb300/dropin/lulesh_gb300_dropin.h is what a
maintainer includes after the reference's lulesh.h to call the GB300 step in
place of LagrangeLeapFrogWithTasks (lulesh.cc:1977, called at 2374-2379);
lulesh_dropin.cc is the reference's time loop with that call swapped. This
test compiles both against the reference's unmodified lulesh.h, lulesh.cc,
lulesh-init.cc, lulesh-util.cc and lulesh-viz.cc (with the sequential HPX
stand-in of oracle/hpx_shim), links liblulesh_gb300.so, and runs the
program's host-only check: the view it makes of the reference's own Domain
equals this library's host Domain of the same problem, every array bit for
bit, so the adapter needs no edit of lulesh.h. It runs where the reference
sources are (the build machine) and is skipped elsewhere.
"""
from __future__ import annotations

import subprocess

import pytest

from conftest import ROOT

PKG = ROOT / "lulesh-task-based-hpx_gb300"
DROPIN = PKG / "dropin"


@pytest.fixture(scope="module")
def dropin_exe(oracle_mod, lulesh, tmp_path_factory):
    ref = oracle_mod.REF_SOURCES
    if not (ref / "lulesh.h").is_file():
        pytest.skip("the reference sources are not on this machine")
    out = tmp_path_factory.mktemp("dropin")
    inc = [f"-I{ROOT / 'oracle' / 'hpx_shim'}", f"-I{ref}", f"-I{ROOT / 'include'}", f"-I{DROPIN}"]
    cxx = ["g++", "-std=c++17", "-O1", "-w", *inc]
    objs = []
    # lulesh.cc defines the reference's own main: renamed, so the drop-in's runs
    for src, extra in (("lulesh.cc", ["-Dmain=lulesh_reference_main"]), ("lulesh-init.cc", []),
                       ("lulesh-util.cc", []), ("lulesh-viz.cc", [])):
        o = out / (src + ".o")
        subprocess.run([*cxx, *extra, "-c", str(ref / src), "-o", str(o)], check=True)
        objs.append(str(o))
    exe = out / "lulesh-dropin"
    subprocess.run([*cxx, str(DROPIN / "lulesh_dropin.cc"), *objs, f"-L{PKG}", "-llulesh_gb300",
                    f"-Wl,-rpath,{PKG}", "-o", str(exe)], check=True)
    return exe


@pytest.mark.parametrize("args", [("--s", "5"), ("--s", "9", "--r", "21", "--c", "2"),
                                  ("--s", "8", "--r", "1", "--b", "2", "--c", "3"), ("--s", "12", "--r", "16")])
def test_view_of_reference_domain_equals_library_domain(dropin_exe, args):
    r = subprocess.run([str(dropin_exe), "--check", *args], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("view ok")


def test_dropin_fails_loudly_without_gpu(dropin_exe):
    from conftest import gpu_available

    if gpu_available():
        pytest.skip("a GPU is present")
    r = subprocess.run([str(dropin_exe), "--s", "5", "--i", "2"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 2 and "lulesh_dev_create" in r.stderr
