"""Multi-process host logic of bench.py on CPU (world size 2, gloo).

bench.py runs one rank per GPU under torchrun: each rank solves its own
problem (replicas, no data-path collective), the timed region is bracketed
by a barrier, and rank 0 prints the max over ranks. The reference arm runs on
rank 0 only. These tests exercise that host logic with CPU ranks; the GPU
work of each rank is covered by the -m gpu tests.
"""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _cpu_only():
    import torch

    if torch.cuda.is_available():
        pytest.skip("gloo rank test for machines without GPUs (bench picks nccl when CUDA is present)")


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    r, w, local = bench.dist_init()
    bench.barrier(w)
    # each rank times a different duration; every rank must see the max
    m = bench.max_over_ranks(1.5 + rank, w)
    backend = dist.get_backend()
    bench.barrier(w)
    dist.destroy_process_group()
    Path(out_dir, f"rank{rank}.json").write_text(
        json.dumps({"rank": r, "world": w, "local": local, "max": m, "backend": backend}))


def test_rank_setup_barrier_and_max_over_ranks(tmp_path):
    _cpu_only()
    import torch.multiprocessing as mp

    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    for rank in range(2):
        d = json.loads((tmp_path / f"rank{rank}.json").read_text())
        assert d == {"rank": rank, "world": 2, "local": rank, "max": 2.5, "backend": "gloo"}


def test_reference_arm_prints_once_under_torchrun():
    """torchrun's launch line with N=2: rank 0 times the reference's
    CPU path and prints one JSON line; rank 1 exits 0 without work."""
    _cpu_only()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--size", "8", "--steps", "2", "--warmup", "3"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["steps"] == 2 and d["warmup"] == 3
    assert d["unit"] == "zone-cycles/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["config"]["elements"] == 8 ** 3


def test_roofline_arithmetic():
    """bench.roofline: dominant kernel, HBM fraction and the FP64-pipe roof
    from the per-unit constants."""
    sys.path.insert(0, str(ROOT))
    import bench

    ne, nn, cycles = 3_375_000, 3_442_951, 10
    prof = {"kernel_ms": {"forces": 42.6, "nodes": 2.4, "kinematics": 20.6, "material": 14.7},
            "cycles": cycles}
    rl = bench.roofline(prof, "fp64", ne, nn, 3.26, fp64_peak=1.2, fp64_kind="test", ms_per_step=8.5)
    assert rl["kernel"] == "forces" and rl["bound"] == "hbm" and rl["unit"] == "GB/s"
    launch_s = 42.6 / cycles / 1e3
    assert rl["avg_launch_ms"] == pytest.approx(4.26)
    # the algorithmic bytes of the four-kernel step: 320 per element for forces
    assert bench.BYTES_PER_UNIT["fp64"]["forces"] == 320
    assert sum(bench.BYTES_PER_UNIT["fp64"].values()) == bench.STEP_BYTES_PER_ZONE_CYCLE["fp64"] == 1020
    assert sum(bench.BYTES_PER_UNIT["mixed"].values()) == bench.STEP_BYTES_PER_ZONE_CYCLE["mixed"] == 780
    assert rl["bytes_per_launch"] == 320 * ne
    assert rl["achieved"] == pytest.approx(rl["bytes_per_launch"] / launch_s / 1e9, rel=1e-3)
    assert rl["frac"] == pytest.approx(rl["achieved"] / rl["peak"], rel=1e-3)
    lay = bench.LAYOUT_BYTES_PER_UNIT["fp64"]["forces"] * ne / launch_s / 1e9
    assert rl["frac_layout"] == pytest.approx(lay / rl["peak"], rel=1e-3)
    step_gbs = 1020 * ne / 8.5e-3 / 1e9
    assert rl["step"]["achieved"] == pytest.approx(step_gbs, rel=1e-3)
    assert rl["step"]["frac"] == pytest.approx(step_gbs / rl["peak"], rel=1e-3)
    assert rl["traffic"] == bench.TRAFFIC_PER_UNIT["fp64"]["forces"] * ne
    fp = rl["fp64_pipe"]
    rate = bench.FP64_INSTR_PER_UNIT["fp64"]["forces"] * ne / launch_s
    assert fp["achieved_ginst_s"] == pytest.approx(rate / 1e9, rel=1e-3)
    assert fp["frac"] == pytest.approx(rate / 0.6e12, rel=1e-3)
    assert sum(rl["kernel_share"].values()) == pytest.approx(1.0, abs=1e-3)
    # every kernel of both paths carries its measured FP64-pipe count
    prof["kernel_ms"]["material"] = 99.0
    rl = bench.roofline(prof, "mixed", ne, nn, 3.26)
    assert rl["kernel"] == "material" and rl["fp64_pipe"]["instr_per_unit"] == bench.FP64_INSTR_PER_UNIT["mixed"]["material"]


def test_fom_matches_reference_report_formula():
    """bench.fom: grind time = elapsed us / cycles / elements and FOM =
    1000 / grind, as lulesh-util.cc:70-112 prints them (one rank)."""
    sys.path.insert(0, str(ROOT))
    import bench

    elapsed_s, cycles, elements = 12.5, 932, 27_000
    rate = elements * cycles / elapsed_s
    f = bench.fom(rate)
    grind = elapsed_s * 1e6 / cycles / elements
    assert f["grind_time_us_per_zone_cycle"] == pytest.approx(grind, rel=1e-5)
    assert f["fom"] == pytest.approx(1000.0 / grind, rel=1e-5)


def test_mixed_error_summary():
    """bench.mixed_error: relative e(0) error of mixed runs against double runs
    of the same problems, and the cycle-count mismatches."""
    sys.path.insert(0, str(ROOT))
    import bench

    ref = [(100, 2.0), (200, 4.0), (300, 1.0)]
    mixed = [(100, 2.0 * (1 + 1e-8)), (201, 4.0 * (1 - 3e-6)), (300, 1.0)]
    d = bench.mixed_error(ref, mixed)
    assert d["problems"] == 3 and d["cycle_mismatches"] == 1 and d["above_1e-6"] == 1
    assert d["e0_rel_max"] == pytest.approx(3e-6, rel=1e-3)
    assert d["e0_rel_median"] == pytest.approx(1e-8, rel=1e-3)


def test_gpus_flag_must_match_world_size():
    """bench.py --gpus N without N launched ranks is refused, not run as one replica."""
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--gpus", "2", "--skip-cpu"],
                       capture_output=True, text=True, timeout=120, cwd=ROOT,
                       env={k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK")})
    assert r.returncode != 0
    assert "WORLD_SIZE is 1" in r.stderr


def test_reference_code_rate_reads_the_reference_timer():
    """bench.reference_code_rate runs the reference's own binary (its
    unmodified sources, built where they are) and takes the elapsed time the
    reference prints for its time loop: one thread, elements x cycles / that
    time."""
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "oracle"))
    import bench
    import oracle

    if not (oracle.REF_SOURCES / "lulesh.cc").exists():
        pytest.skip("the reference sources are not on this machine")
    r = bench.reference_code_rate(24, 11, 6)
    assert r is not None and r["threads"] == 1 and r["unit"] == bench.UNIT
    elapsed = float(r["sample"].split("(")[1].split(" s")[0])
    assert elapsed > 0
    assert r["value"] == pytest.approx(24 ** 3 * 6 / elapsed, rel=0.05)
