"""Shared fixtures: the product package (lulesh-task-based-hpx_gb300, loaded
under the import name lulesh_gb300), the CPU oracle, and the golden data.

Markers: tests marked `gpu` need a CUDA device; everything else runs on CPU.
"""
from __future__ import annotations

import importlib.util
import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG_DIR = ROOT / "lulesh-task-based-hpx_gb300"
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: long-running case")


def load_package():
    if "lulesh_gb300" in sys.modules:
        return sys.modules["lulesh_gb300"]
    spec = importlib.util.spec_from_file_location(
        "lulesh_gb300", PKG_DIR / "__init__.py", submodule_search_locations=[str(PKG_DIR)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["lulesh_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


_built = False


def ensure_built():
    """Builds the product library and the oracle port once per session."""
    global _built
    if _built:
        return
    bspec = importlib.util.spec_from_file_location("lulesh_gb300_build", PKG_DIR / "build.py")
    bmod = importlib.util.module_from_spec(bspec)
    bspec.loader.exec_module(bmod)
    bmod.build()
    import oracle

    oracle.build(ref=oracle.REF_SOURCES.is_dir() and not oracle.REF_BIN.exists())
    _built = True


@pytest.fixture(scope="session")
def lulesh():
    ensure_built()
    return load_package()


@pytest.fixture(scope="session")
def oracle_mod():
    ensure_built()
    import oracle

    return oracle


@pytest.fixture(scope="session")
def golden_results():
    return json.loads((GOLDEN / "results.json").read_text())


def golden_dump(name: str) -> dict:
    with np.load(GOLDEN / name) as z:
        return {k: z[k] for k in z.files}


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def rel_err(a, b) -> float:
    """max |a - b| / max |b| (normwise relative error)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = float(np.max(np.abs(b))) if b.size else 0.0
    if scale == 0.0:
        return float(np.max(np.abs(a))) if a.size else 0.0
    return float(np.max(np.abs(a - b))) / scale
