"""Generates the golden fixtures of tests/golden/ from the reference itself.

Runs the UNMODIFIED reference sources (esa-tu-darmstadt/lulesh-task-based-hpx
lulesh.cc, lulesh-init.cc, lulesh-viz.cc), compiled by oracle/Makefile against
the sequential HPX stand-in into oracle/_ref/lulesh-ref (-O3
-ffp-contract=off), and records:

  results.json   full-precision final report (cycles, e(0), plane-0 symmetry
                 diffs, time, dt) of whole runs, as VerifyAndWriteFinalOutput
                 computes them (lulesh-util.cc:60-115)
  dump_*.npz     every node and element field after a fixed number of cycles

  s150_r21.json  the s=150 r=21 run to stoptime (5,382 cycles, about 1.7e10
                 zone-cycles): hours for the single-threaded reference binary,
                 so it comes from the oracle port with OpenMP threads, which
                 equals the reference binary byte for byte on every golden run
                 and dump (tests/test_oracle.py) at any thread count

Needs the reference sources, so it runs in the build container only; the
fixtures it writes are committed and used everywhere else.

    python tests/golden/make_golden.py           # results.json and the dumps
    python tests/golden/make_golden.py --s150    # s150_r21.json (about 30 min on 8 cores)
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "oracle"))
import oracle  # noqa: E402

# whole runs to stoptime: (s, r, b, c); cycle-capped runs: (s, r, b, c, its)
RUNS = [(8, 11, 1, 1), (10, 11, 1, 1), (12, 21, 1, 1), (12, 1, 1, 1), (9, 16, 2, 2),
        (16, 11, 1, 1), (20, 11, 1, 1), (30, 11, 1, 1), (45, 11, 1, 1)]
CAPPED = [(90, 11, 1, 1, 1000)]
# field dumps after a fixed number of cycles: (s, r, b, c, cycles)
DUMPS = [(8, 11, 1, 1, 1), (8, 11, 1, 1, 100), (12, 21, 1, 1, 50), (10, 1, 1, 1, 30)]

_RES = re.compile(r"RESULT (.*)")


def run_ref(s, r, b, c, its=None, dump=None) -> dict:
    args = [str(oracle.REF_BIN), "--s", str(s), "--r", str(r), "--b", str(b), "--c", str(c)]
    if its is not None:
        args += ["--i", str(its)]
    env = dict(os.environ)
    if dump:
        env["LULESH_DUMP"] = str(dump)
    out = subprocess.run(args, capture_output=True, text=True, env=env, check=True).stdout
    m = _RES.search(out)
    kv = dict(t.split("=", 1) for t in m.group(1).split())
    return {"s": s, "r": r, "b": b, "c": c, "cycles": int(kv["cycles"]), "e0": kv["e0"],
            "maxabs": kv["maxabs"], "totabs": kv["totabs"], "maxrel": kv["maxrel"],
            "time": kv["time"], "dt": kv["dt"]}


def run_s150(threads: int) -> dict:
    """The s=150 r=21 run to stoptime through the oracle port's command line
    (the reference's flags and report fields)."""
    oracle.build(ref=False)
    args = [str(oracle.HERE / "lulesh-oracle"), "--s", "150", "--r", "21", "--threads", str(threads)]
    out = subprocess.run(args, capture_output=True, text=True, check=True).stdout
    kv = dict(t.split("=", 1) for t in _RES.search(out).group(1).split())
    return {"s": 150, "r": 21, "b": 1, "c": 1, "cycles": int(kv["cycles"]), "e0": kv["e0"],
            "maxabs": kv["maxabs"], "totabs": kv["totabs"], "maxrel": kv["maxrel"],
            "time": kv["time"], "dt": kv["dt"], "source": "oracle port (lulesh-oracle), "
            f"{threads} OpenMP threads, libm cube root", "command": " ".join(args[1:])}


def main() -> None:
    if "--s150" in sys.argv:
        res = run_s150(os.cpu_count() or 1)
        print(res, flush=True)
        (HERE / "s150_r21.json").write_text(json.dumps(res, indent=1) + "\n")
        return
    if not oracle.REF_SOURCES.is_dir():
        sys.exit("the reference sources are needed to generate the fixtures")
    oracle.build(ref=True)
    results = []
    for s, r, b, c in RUNS:
        res = run_ref(s, r, b, c)
        print(res, flush=True)
        results.append(res)
    for s, r, b, c, its in CAPPED:
        res = run_ref(s, r, b, c, its=its)
        res["its"] = its
        print(res, flush=True)
        results.append(res)
    (HERE / "results.json").write_text(json.dumps(results, indent=1) + "\n")
    with tempfile.TemporaryDirectory() as td:
        for s, r, b, c, its in DUMPS:
            path = Path(td) / "d.bin"
            run_ref(s, r, b, c, its=its, dump=path)
            d = oracle.read_dump(path)
            name = HERE / f"dump_s{s}_r{r}_b{b}_c{c}_i{its}.npz"
            np.savez_compressed(name, **{k: np.asarray(v) for k, v in d.items()})
            print(name.name, name.stat().st_size, flush=True)


if __name__ == "__main__":
    main()
