#!/usr/bin/env python
"""Benchmark of the GB300 LULESH Lagrange-leapfrog step.

Workload: the Sedov blast at --s 150 --r 21 (3,375,000 hex elements,
3,442,951 nodes; regions, balance 1 and cost 1 as Domain::Domain builds them),
the size the reference's headline metric is quoted on. One step = one
LagrangeLeapFrog cycle (plus the host TimeIncrement before it) over the whole
mesh. Metric: zone-cycles per second (elements x cycles / seconds).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours (default) prints one JSON line:
  value          plain double path (LULESH_FP64), state resident in HBM,
                 device time over K cycles (CUDA events on the library's own
                 stream, host TimeIncrement and the per-cycle dt readback
                 included)
  e2e            the same metric through lulesh_leapfrog, the drop-in for
                 LagrangeLeapFrog(Domain&): every cycle uploads the state a
                 step reads from pinned host arrays and downloads everything
                 it writes; wall clock
  mixed, graph   the mixed-precision form and the CUDA-graph time loop
  batched        64 problems of uneven sizes (s in [16, 64], seeded) in one
                 device pool to their stoptimes, double and mixed; beside
                 the s=150 ratio, vs_solo_runs = the same problems run one at
                 a time on the single-problem path over the batch
  serving        the continuous-batching loop on Poisson arrivals: p50/p99
                 time to solution and zone-cycles/s
  roofline       dominant kernel vs the measured HBM copy bandwidth, plus its
                 FP64-pipe roof (the bound that actually applies)
  fom            the reference's report figures for value (and mixed):
                 grind time in us per zone-cycle and FOM = 1000 / grind
  cpu_baseline   the CPU oracle (a bit-exact restatement of the reference's
                 code) on this machine's host cores, bounded sample (the
                 reference's reduced s=150 cap of 180 cycles); its sweep
                 adds the single-thread rate, and reference_code_1_thread
                 the reference's own sources built on this host (sequential
                 HPX stand-in) where they are installed
reference: the reference's CPU algorithm (the oracle port) on all host cores,
same workload, same metric (plus reference_code_1_thread).

Multi-GPU: the step does not shard inside one problem (replicas only); with
N ranks every rank runs its own s=150 problem and value sums them (weak
scaling). Rank r uses GPU LOCAL_RANK.
"""
from __future__ import annotations

import argparse
import gc
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG_DIR = ROOT / "lulesh-task-based-hpx_gb300"
sys.path.insert(0, str(ROOT / "oracle"))

METRIC = "FOM zone-cycles/s at s=150 (FP64 vs mixed) + batched-ensemble zone-cycles/s"
UNIT = "zone-cycles/s"

# Algorithmic HBM bytes per unit (element, or node for the node kernel) of the
# four-kernel step: the compulsory traffic of the step's own arrays, each
# touched once per launch, node fields once per node (N_n / N_e ~ 1),
# neighbour re-reads as L2 hits. Double: force 320 (node list 32, node
# positions and velocities 48, p q v volo ss elemMass 48, 24 corner forces
# 192), nodes 332, kinematics + Q gradients 184, material 184: 1,020 bytes per
# zone-cycle. Mixed: float corner forces (-96 in forces and nodes) and float
# Q gradients (-24 in kinematics and material): 780.
BYTES_PER_UNIT = {
    "fp64": {"forces": 320, "nodes": 332, "kinematics": 184, "material": 184},
    "mixed": {"forces": 224, "nodes": 236, "kinematics": 160, "material": 160},
}
STEP_BYTES_PER_ZONE_CYCLE = {"fp64": 1020, "mixed": 780}
# What this implementation's layout moves on top of that: the double path's
# resident loop passes 48 doubles of element geometry per element from
# kinematics (written) to the next force phase (read instead of the node
# positions), and the mixed path reads float-pair node mirrors.
LAYOUT_BYTES_PER_UNIT = {
    "fp64": {"forces": 680, "nodes": 381, "kinematics": 568, "material": 204},
    "mixed": {"forces": 224, "nodes": 333, "kinematics": 184, "material": 180},
}
# DRAM bytes (read + write) and FP64-pipe instructions (thread level:
# sm__inst_executed_pipe_fp64 x 32) per unit, measured by ncu on this
# workload (s=150 r=21, the third cycle); every array a kernel streams is
# larger than L2. The material kernel's count depends on the state (EOS
# passes, compressing elements); these are early cycles of the run. The FP64
# pipe carries only part of the double arithmetic: the fast kernels run many
# of their multiplies on the integer pipes (dmul_ipipe).
TRAFFIC_PER_UNIT = {
    "fp64": {"forces": 672, "nodes": 368, "kinematics": 563, "material": 230},
    "mixed": {"forces": 215, "nodes": 315, "kinematics": 178, "material": 199},
}
FP64_INSTR_PER_UNIT = {
    "fp64": {"forces": 449.0, "nodes": 32.7, "kinematics": 320.0, "material": 136.1},
    "mixed": {"forces": 8.0, "nodes": 24.0, "kinematics": 76.0, "material": 115.1},
}
# Double-precision operations per unit of the reference's formulation (adds,
# multiplies, divides, square and cube roots each counted once), from
# counting its arithmetic at s=30 r=11; the material kernel adds 68 per EOS
# pass. Divided by the launch time this is an effective rate of the
# reference's arithmetic, not a pipe load: the fast kernels fuse and share
# many of these operations.
FLOPS_PER_UNIT = {"forces": 1809, "nodes": 63, "kinematics": 864, "material_base": 69,
                  "material_per_rep": 68}
# Measured on a GB300 of this machine (DFMA throughput probe): 597 G FMA/s.
FP64_PEAK_TFLOPS = 1.194
HBM_FALLBACK_GBS = 6800.0


def load_package():
    spec = importlib.util.spec_from_file_location(
        "lulesh_gb300", PKG_DIR / "__init__.py", submodule_search_locations=[str(PKG_DIR)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["lulesh_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def hbm_peak() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self) -> dict:
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        rows = []
        try:
            for line in Path(self.path).read_text().splitlines():
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
            os.unlink(self.path)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "", 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": float(rows[0][2]) if rows[0][2].replace(".", "", 1).isdigit() else None,
                "reasons": reasons, "samples": len(rows)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sync():
    import torch

    if torch.cuda.is_available():
        torch.cuda.synchronize()


def mean_rep(lul, dom) -> float:
    import numpy as np

    reg = dom.regNumList - 1
    nr = dom.nr
    rep = np.where(reg < nr // 2, 1,
                   np.where(reg < nr - (nr + 15) // 20, 1 + dom.cost, 10 * (1 + dom.cost)))
    return float(rep.mean())


def sig4(x: float) -> float:
    """x rounded to 4 significant digits."""
    return float(f"{x:.4g}")


def roofline(prof: dict, precision: str, ne: int, nn: int, rep_avg: float,
             fp64_peak: float = FP64_PEAK_TFLOPS, fp64_kind: str = "earlier probe",
             ms_per_step: float | None = None) -> dict:
    km = prof["kernel_ms"]
    cyc = max(prof["cycles"], 1)
    dom = max(km, key=km.get)
    units = nn if dom == "nodes" else ne
    avg_s = km[dom] / cyc / 1e3
    bytes_launch = BYTES_PER_UNIT[precision][dom] * units
    layout_launch = LAYOUT_BYTES_PER_UNIT[precision][dom] * units
    peak, kind = hbm_peak()
    achieved = bytes_launch / avg_s / 1e9
    step = None
    if ms_per_step:
        step_gbs = STEP_BYTES_PER_ZONE_CYCLE[precision] * ne / (ms_per_step / 1e3) / 1e9
        step = {"achieved": round(step_gbs, 1), "frac": sig4(step_gbs / peak),
                "bytes_per_zone_cycle": STEP_BYTES_PER_ZONE_CYCLE[precision],
                "note": "the whole cycle: algorithmic bytes per zone-cycle x elements / ms_per_step"}
    if dom == "material":
        flops = FLOPS_PER_UNIT["material_base"] + FLOPS_PER_UNIT["material_per_rep"] * rep_avg
    else:
        flops = FLOPS_PER_UNIT[dom]
    tflops = flops * units / avg_s / 1e12
    tpu = TRAFFIC_PER_UNIT.get(precision, {}).get(dom)
    ipu = FP64_INSTR_PER_UNIT.get(precision, {}).get(dom)
    fp64_pipe = None
    if ipu:
        rate = ipu * units / avg_s  # FP64-pipe thread instructions per second
        peak_rate = fp64_peak * 1e12 / 2  # DFMA thread instructions per second
        fp64_pipe = {"achieved_ginst_s": round(rate / 1e9, 1), "peak_ginst_s": round(peak_rate / 1e9, 1),
                     "frac": round(rate / peak_rate, 4), "instr_per_unit": ipu,
                     "note": "FP64-pipe instructions per unit (ncu, this workload) x units / launch time; peak = "
                             f"DFMA issue rate, {fp64_kind} (lulesh_probe_pipe_rates)"}
    return {
        "bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
        "unit": "GB/s", "frac": sig4(achieved / peak),
        "traffic": tpu * units if tpu else None,
        "traffic_note": "ncu dram bytes per unit on this workload x units per launch" if tpu else None,
        "peak_kind": f"{kind} ({'MEASURED_PEAKS.json hbm_gbs' if kind == 'measured' else 'recipe fallback'})",
        "bytes_per_launch": bytes_launch, "bytes_per_unit": BYTES_PER_UNIT[precision][dom],
        "avg_launch_ms": round(km[dom] / cyc, 4),
        "frac_layout": sig4(layout_launch / avg_s / 1e9 / peak),
        "layout_bytes_per_unit": LAYOUT_BYTES_PER_UNIT[precision][dom],
        "step": step,
        "kernel_share": {k: round(v / max(sum(km.values()), 1e-30), 4) for k, v in km.items()},
        "reference_flops_tflops": round(tflops, 4),
        "fp64_pipe": fp64_pipe,
    }


def time_device(lul, dom, dev, steps: int, world: int, graph: bool = False) -> dict:
    barrier(world)
    sync()
    dev.profile_begin()
    if graph:
        n = dev.run_graph(dom.cycle + steps, 8)
    else:
        n = dev.run(dom.cycle + steps)
    prof = dev.profile_end()
    sync()
    barrier(world)
    if n != steps:
        raise RuntimeError(f"ran {n} of {steps} cycles (stoptime reached?)")
    prof["max_ms"] = max_over_ranks(prof["total_ms"], world)
    return prof


def workload(s: int, r: int) -> str:
    """The workload name both arms print (config.workload)."""
    return f"Sedov blast --s {s} --r {r} (b=1, c=1), one LagrangeLeapFrog cycle per step"


def fom(value: float) -> dict:
    """The reference's report figures (lulesh-util.cc:70-112) for a
    zone-cycles/s rate: grind time = us per zone-cycle, FOM = 1000 / grind
    (zone-cycles per millisecond; the reference labels it z/s)."""
    grind = 1e6 / value
    return {"grind_time_us_per_zone_cycle": float(f"{grind:.6g}"), "fom": float(f"{1e3 / grind:.6g}")}


def cpu_oracle_rate(s: int, r: int, cycles: int, threads: int) -> tuple[float, float]:
    import oracle

    o = oracle.Oracle(s, r, 1, 1, threads=threads)
    o.run(1)  # warm caches and page in the arrays
    t0 = time.perf_counter()
    o.run(o.cycle + cycles)
    dt = time.perf_counter() - t0
    ne = o.numElem
    o.close()
    return ne * cycles / dt, dt


def link_rates(device: int, mb: int = 256, reps: int = 3) -> dict:
    """Pinned host<->device copy rates of this machine (GB/s, best of reps):
    device to host, host to device, and both directions at once (half the
    bytes each way on two streams, total bytes over the time). The drop-in
    call's copies run over this link."""
    import torch

    n = (mb << 20) // 8
    h = torch.empty(n, dtype=torch.float64, pin_memory=True)
    d = torch.empty(n, dtype=torch.float64, device=f"cuda:{device}")
    s1, s2 = torch.cuda.Stream(device), torch.cuda.Stream(device)

    def best(fn):
        t = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record(s1)
            s2.wait_event(a)
            fn()
            s1.wait_stream(s2)
            b.record(s1)
            b.synchronize()
            t.append(a.elapsed_time(b) / 1e3)
        return n * 8 / min(t) / 1e9

    def d2h():
        with torch.cuda.stream(s1):
            h.copy_(d, non_blocking=True)

    def h2d():
        with torch.cuda.stream(s1):
            d.copy_(h, non_blocking=True)

    def both():
        with torch.cuda.stream(s1):
            h[: n // 2].copy_(d[: n // 2], non_blocking=True)
        with torch.cuda.stream(s2):
            d[n // 2:].copy_(h[n // 2:], non_blocking=True)

    out = {"d2h": round(best(d2h), 1), "h2d": round(best(h2d), 1), "both": round(best(both), 1),
           "bytes": n * 8, "how": "pinned torch copies, CUDA events, best of 3"}
    del h, d
    return out


def reference_code_rate(s: int, r: int, cycles: int) -> dict | None:
    """The reference's own code on this host: its unmodified lulesh.cc,
    lulesh-init.cc and lulesh-viz.cc built here against the sequential HPX
    stand-in (oracle/_ref/lulesh-ref, from the checkout or its installed copy
    in baseline/_ref), so one thread. Rate = elements x cycles / the elapsed
    time the reference itself measures around its time loop
    (lulesh.cc:2388-2392). None where the sources are not on this machine."""
    import oracle

    if not oracle.REF_BIN.exists():
        if not (oracle.REF_SOURCES / "lulesh.cc").exists():
            return None
        oracle.build(ref=True)
    r_ = subprocess.run([str(oracle.REF_BIN), "--s", str(s), "--r", str(r), "--i", str(cycles)],
                        capture_output=True, text=True, timeout=600)
    line = next((x for x in r_.stdout.splitlines() if x.startswith("RESULT ")), None)
    if r_.returncode != 0 or line is None:
        return None
    kv = dict(x.split("=", 1) for x in line.split()[1:])
    elapsed = float(kv["elapsed"])
    return {"value": round(s ** 3 * cycles / elapsed, 1), "unit": UNIT, "threads": 1,
            "sample": f"{cycles} cycles of s={s} r={r} ({elapsed:.3f} s by the reference's own timer)",
            "code": "the reference's unmodified sources with the sequential HPX stand-in, built on this "
                    "host (-O3 -ffp-contract=off)"}


def run_ours(args) -> None:
    rank, world, local = dist_init()
    lul = load_package()
    lul.set_device(local)
    import torch

    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    s, r, K, W = args.size, args.regions, args.steps, args.warmup

    rates = lul.pipe_rates()
    fp64_peak = 2.0 * rates["dfma"] / 1e12
    dom = lul.HostDomain(s, r, 1, 1)
    ne, nn = dom.numElem, dom.numNode
    rep_avg = mean_rep(lul, dom)
    dev = lul.Device(dom, "fp64")
    dev.run(dom.cycle + W)  # warm-up cycles (untimed)

    clocks = ClockSampler(local)
    clocks.start()
    prof = time_device(lul, dom, dev, K, world)
    clk = clocks.stop()
    value = world * ne * K / (prof["max_ms"] / 1e3)
    launches = prof["launches"]

    # graph form of the same time loop, same handle, continuing the run
    gprof = time_device(lul, dom, dev, K, world, graph=True)
    gvalue = world * ne * K / (gprof["max_ms"] / 1e3)

    # end to end through the drop-in call on pinned host buffers
    dev.download()
    dom.pin(True)
    for _ in range(2):
        dom.time_increment()
        dev.leapfrog()
    barrier(world)
    sync()
    gc.disable()  # the host loop's timing without collector pauses, as timeit takes it
    t0 = time.perf_counter()
    call_ms = []
    for _ in range(K):
        t1 = time.perf_counter()
        dom.time_increment()
        dev.leapfrog()
        call_ms.append(1e3 * (time.perf_counter() - t1))
    sync()
    e2e_end = time.perf_counter()
    gc.enable()
    e2e_s = max_over_ranks(e2e_end - t0, world)
    barrier(world)
    e2e_value = world * ne * K / e2e_s
    call_ms.sort()
    h2d = (6 * nn + 5 * ne) * 8
    d2h = (12 * nn + 11 * ne) * 8 + 16
    link = link_rates(local)
    dev.close()
    dom.close()

    mixed = None
    if not args.skip_mixed:
        mdom = lul.HostDomain(s, r, 1, 1)
        mdev = lul.Device(mdom, "mixed")
        mdev.run(mdom.cycle + W)
        mprof = time_device(lul, mdom, mdev, K, world)
        mvalue = world * ne * K / (mprof["max_ms"] / 1e3)
        mgprof = time_device(lul, mdom, mdev, K, world, graph=True)
        mgvalue = world * ne * K / (mgprof["max_ms"] / 1e3)
        # the mixed path through the drop-in call (same copies as the double one)
        mdev.download()
        mdom.pin(True)
        for _ in range(2):
            mdom.time_increment()
            mdev.leapfrog()
        barrier(world)
        sync()
        gc.disable()
        t0 = time.perf_counter()
        for _ in range(K):
            mdom.time_increment()
            mdev.leapfrog()
        sync()
        me2e_end = time.perf_counter()
        gc.enable()
        me2e_s = max_over_ranks(me2e_end - t0, world)
        barrier(world)
        mixed = {"value": round(mvalue, 1), "unit": UNIT, "dtype": "f32 temporaries + f64 state",
                 "ms_per_step": round(mprof["max_ms"] / K, 4),
                 "speedup_vs_fp64": round(mvalue / value, 3), "fom": fom(mvalue),
                 "graph": {"value": round(mgvalue, 1), "unit": UNIT, "ms_per_step": round(mgprof["max_ms"] / K, 4),
                           "speedup_vs_fp64_graph": round(mgvalue / gvalue, 3),
                           "how": "device TimeIncrement, each cycle replayed from one CUDA graph"},
                 "e2e": {"value": round(world * ne * K / me2e_s, 1), "unit": UNIT,
                         "ms_per_step": round(1e3 * me2e_s / K, 4), "h2d_bytes_per_step": h2d,
                         "d2h_bytes_per_step": d2h,
                         "how": "lulesh_leapfrog as for the double path: the same bytes over the host link, "
                                "which bounds this call (the link floor above), not the GPU"},
                 "kernel_ms_per_step": {k: round(v / K, 4) for k, v in mprof["kernel_ms"].items()},
                 "roofline": roofline(mprof, "mixed", ne, nn, rep_avg, fp64_peak, "measured live",
                                      ms_per_step=mprof["max_ms"] / K)}
        mdev.close()
        mdom.close()

    batched = None
    if not args.skip_batch:
        batched = {}
        for prec in ("fp64", "mixed"):
            res = run_batched(lul, prec, args.batch_problems, args.batch_seed + rank, tune=True)
            single = value / world if prec == "fp64" else (mixed["value"] / world if mixed else None)
            if single:
                # against the s=150 r=21 problem (fewer EOS passes per element
                # than this ensemble's mix, so conservative)
                res["vs_single_problem"] = round(res["value"] / single, 3)
            res["value_all_ranks"] = round(res["value"] * world, 1)
            batched[prec] = res
        # the mixed ensemble against the double ensemble of the same seed
        batched["mixed"]["error_vs_fp64"] = mixed_error(batched["fp64"].pop("results"),
                                                        batched["mixed"].pop("results"))

    serving = None
    if not args.skip_serve and mixed:
        serving = run_serving(lul, args.serve_requests, args.batch_seed + 7 + rank, mixed["value"] / world)

    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        threads = os.cpu_count() or 1
        rate, secs = cpu_oracle_rate(s, r, args.cpu_cycles, threads)
        cpu = {"value": round(rate, 1), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{args.cpu_cycles} cycles of s={s} r={r} after 1 warm-up cycle "
                         f"({secs:.1f} s), OpenMP over all host threads"}
        if args.cpu_cycles_1t > 0:
            # the reference's thread sweep, its two ends: 1 thread and all cores
            rate1, secs1 = cpu_oracle_rate(s, r, args.cpu_cycles_1t, 1)
            cpu["sweep"] = {"threads": [1, threads], "value": [round(rate1, 1), round(rate, 1)],
                            "sample_1_thread": f"{args.cpu_cycles_1t} cycles of s={s} r={r} after 1 "
                                               f"warm-up cycle ({secs1:.1f} s)"}
            # the reference's own code at one thread, beside the port's
            refc = reference_code_rate(s, r, args.cpu_cycles_1t)
            if refc:
                refc["port_1_thread_over_reference"] = round(rate1 / refc["value"], 3)
                cpu["reference_code_1_thread"] = refc

    if rank != 0:
        return
    out = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": round(prof["max_ms"] / K, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload(s, r),
                   "path": "plain double path (LULESH_FP64), host TimeIncrement per cycle",
                   "elements": ne, "nodes": nn, "mean_eos_rep": round(rep_avg, 3),
                   "parallelism": "replicas only (one independent problem per GPU)",
                   "l2": f"no flush: working set {lul.Batch.footprint('fp64', args.size) / 1e9:.2f} GB "
                         "per GPU >> 129 MB L2"},
        "e2e": {"value": round(e2e_value, 1), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "how": "lulesh_leapfrog per cycle: upload step inputs from pinned host arrays, "
                       "run, download every field the step writes; wall clock",
                "ms_per_step": round(1e3 * e2e_s / K, 4),
                "call_ms": {"min": round(call_ms[0], 3), "median": round(call_ms[len(call_ms) // 2], 3),
                            "max": round(call_ms[-1], 3),
                            "note": "wall time of each timed call (value uses the whole window); the host "
                                    "side of this figure has varied between boxes"},
                "link_gbs": link,
                "link_floor_ms": round(1e3 * d2h / (link["d2h"] * 1e9), 3),
                "link_floor_note": "the step's downloads alone at the measured device-to-host rate"},
        "gpu_launches": launches,
        "fom": fom(value),
        "kernel_ms_per_step": {k: round(v / K, 4) for k, v in prof["kernel_ms"].items()},
        "roofline": roofline(prof, "fp64", ne, nn, rep_avg, fp64_peak, "measured live",
                             ms_per_step=prof["max_ms"] / K),
        "pipe_rates_per_s": {k: float(f"{v:.4g}") for k, v in rates.items()},
        "graph": {"value": round(gvalue, 1), "unit": UNIT,
                  "ms_per_step": round(gprof["max_ms"] / K, 4),
                  "how": "device TimeIncrement, each cycle replayed from one CUDA graph"},
        "mixed": mixed,
        "batched": batched,
        "serving": serving,
        "cpu_baseline": cpu,
        "clocks": clk,
    }
    print(json.dumps(out), flush=True)


def ensemble_specs(n: int, seed: int) -> list[dict]:
    """The batched-ensemble workload: n Sedov problems with s uniform in
    [16, 64], regions uniform in {11, 16, 21}, deposited energy scaled by a
    lognormal(0, 0.25) factor, each to its own stoptime 1e-2 (seeded)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    s = rng.integers(16, 65, n)
    r = rng.choice([11, 16, 21], n)
    scale = rng.lognormal(0.0, 0.25, n)
    return [{"s": int(a), "nr": int(b), "energy_scale": float(c)} for a, b, c in zip(s, r, scale)]


def run_batched(lul, precision: str, n: int, seed: int, tune: bool) -> dict:
    specs = ensemble_specs(n, seed)
    need = sum(lul.Batch.footprint(precision, sp["s"]) for sp in specs)
    b = lul.Batch(precision, pool_bytes=int(need * 1.05) + (64 << 20), max_slots=n)
    t0 = time.perf_counter()
    for sp in specs:
        b.admit(**sp)
    admit_s = time.perf_counter() - t0
    tuning = b.autotune(cycles=3) if tune else b.tuning()
    launches0 = b.launches
    total_ms, rounds = 0.0, 0
    while True:
        active, ms = b.run(64)
        total_ms += ms
        rounds += 1
        if active == 0:
            break
    st = b.status()
    zc = sum(x["numElem"] * x["cycle"] for x in st)
    errs = sum(1 for x in st if x["err"] != 0)
    launches = b.launches - launches0
    # per problem, in admission order: cycles run and final origin energy
    # (computed on the device)
    results = [(x["cycle"], b.verify(x["slot"])["e0"]) for x in sorted(st, key=lambda x: x["slot"])]
    b.close()
    # the same problems run one at a time through the single-problem path
    # (device-built handle, CUDA-graph time loop): device time
    solo_ms = 0.0
    for sp in specs:
        dev = lul.Device.from_problem(sp["s"], sp["nr"], 1, 1, sp["energy_scale"], precision)
        dev.profile_begin()
        dev.run_graph(10 ** 7, 64)
        solo_ms += dev.profile_end()["total_ms"]
        dev.close()
    out = {"value": round(zc / (total_ms / 1e3), 1), "unit": UNIT, "problems": n, "seed": seed,
           "zone_cycles": zc, "device_s": round(total_ms / 1e3, 3),
           "cycles_min_max": [min(x["cycle"] for x in st), max(x["cycle"] for x in st)],
           "elements": sum(x["numElem"] for x in st), "errors": errs,
           "gpu_launches": launches, "admit_s": round(admit_s, 2),
           "tuning": tuning, "results": results,
           "solo_device_s": round(solo_ms / 1e3, 3),
           "vs_solo_runs": round(solo_ms / total_ms, 3),
           "how": "all problems admitted into one pool, cycles replayed from one CUDA graph "
                  "(64 per host sync) until every problem reached its stoptime; device time. "
                  "vs_solo_runs: the same problems run one after another on the single-problem "
                  "path (graph time loop) over the batch, same zone-cycles"}
    return out


def mixed_error(ref: list, mixed: list) -> dict:
    """Relative e(0) error of mixed runs against double runs of the same
    problems, and the count of problems whose cycle counts differ."""
    import numpy as np

    err = np.array([abs(m[1] - r[1]) / abs(r[1]) for r, m in zip(ref, mixed)])
    return {"problems": len(err), "e0_rel_max": float(f"{err.max():.3g}"),
            "e0_rel_p99": float(f"{np.quantile(err, 0.99):.3g}"),
            "e0_rel_median": float(f"{np.median(err):.3g}"),
            "above_1e-6": int((err > 1e-6).sum()),
            "cycle_mismatches": sum(1 for r, m in zip(ref, mixed) if r[0] != m[0])}


def run_serving(lul, n: int, seed: int, single_rate: float, budget_gb: float = 160.0,
                check_max_s: int = 64) -> dict:
    """Serving workload: n requests with s uniform in [20, 120], regions in
    {11, 21}, energy x lognormal(0, 0.25), mixed precision, Poisson arrivals at
    twice the single-problem throughput, under a budget_gb HBM pool. The
    single-problem throughput is 1 / mean solo time, the solo time of a
    request being its zone-cycles (s^3 x 34 s cycles, the observed cycles to
    stoptime) at the measured single-problem mixed rate."""
    import numpy as np

    rng = np.random.default_rng(seed)
    s = rng.integers(20, 121, n)
    r = rng.choice([11, 21], n)
    scale = rng.lognormal(0.0, 0.25, n)
    solo_s = (s.astype(float) ** 3) * 34.0 * s / single_rate
    rate = 2.0 / float(solo_s.mean())  # requests per second
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
    reqs = [{"s": int(a), "nr": int(b), "energy_scale": float(c), "arrival_s": float(d)}
            for a, b, c, d in zip(s, r, scale, arrivals)]
    results, st = lul.serve(reqs, "mixed", hbm_budget=int(budget_gb * (1 << 30)), max_slots=256,
                            sync_ms=20.0)
    # the served (mixed) results against double runs of the same problems, for
    # the requests with s <= check_max_s (one double batch, untimed)
    pick = [i for i, q in enumerate(reqs) if q["s"] <= check_max_s]
    need = sum(lul.Batch.footprint("fp64", reqs[i]["s"]) for i in pick)
    b = lul.Batch("fp64", pool_bytes=int(need * 1.05) + (64 << 20), max_slots=max(len(pick), 1))
    slots = [b.admit(s=reqs[i]["s"], nr=reqs[i]["nr"], energy_scale=reqs[i]["energy_scale"]) for i in pick]
    while b.run(64)[0]:
        pass
    cyc = {x["slot"]: x["cycle"] for x in b.status()}
    ref = [(cyc[sl], b.verify(sl)["e0"]) for sl in slots]
    b.close()
    check = mixed_error(ref, [(results[i]["cycles"], results[i]["e0"]) for i in pick])
    check["requests_checked"] = f"the {len(pick)} requests with s <= {check_max_s}"
    return {"requests": n, "seed": seed, "arrival_rate_per_s": round(rate, 4),
            "budget_gb": budget_gb, "precision": "mixed",
            "p50_time_to_solution_s": round(st["p50_s"], 3), "p99_time_to_solution_s": round(st["p99_s"], 3),
            "mean_time_to_solution_s": round(st["mean_s"], 3),
            "value": round(st["zone_cycles_per_s"], 1), "unit": UNIT, "wall_s": round(st["wall_s"], 2),
            "device_s": round(st["device_s"], 2), "zone_cycles": st["zone_cycles"],
            "max_resident": st["max_resident"], "served": st["served"],
            "peak_resident_gb": round(st["peak_resident_bytes"] / (1 << 30), 2),
            "p50_queue_s": round(st["p50_queue_s"], 3), "p99_queue_s": round(st["p99_queue_s"], 3),
            "error_vs_fp64": check,
            "errors": sum(1 for x in results if x["err"] != 0), "gpu_launches": st["launches"],
            "how": "lulesh_serve: arrived requests are admitted by HBM footprint, each built on the "
                   "device in its pool block, ~20 ms graph chunks replay every resident problem, each "
                   "retires at stoptime with its report computed on the device; wall clock"}


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle

    s, r, K, W = args.size, args.regions, args.steps, args.warmup
    threads = os.cpu_count() or 1
    o = oracle.Oracle(s, r, 1, 1, threads=threads)
    o.run(W)
    t0 = time.perf_counter()
    o.run(o.cycle + K)
    secs = time.perf_counter() - t0
    ne = o.numElem
    value = ne * K / secs
    out = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": K, "warmup": W, "ms_per_step": round(1e3 * secs / K, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": workload(s, r), "path": "the reference's CPU algorithm",
                   "elements": ne},
        "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{K} cycles of s={s} r={r} after {W} warm-up cycles; the "
                                   "reference's algorithm as the bit-exact C oracle, OpenMP over all "
                                   "host threads (HPX is not installed, so the reference's own code "
                                   "runs here only sequentially: reference_code_1_thread)"},
        "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if args.cpu_cycles_1t > 0:
        refc = reference_code_rate(s, r, args.cpu_cycles_1t)
        if refc:
            out["cpu_baseline"]["reference_code_1_thread"] = refc
    print(json.dumps(out), flush=True)


def run_timeline(args) -> None:
    """--timeline: the drop-in call's stage timeline at --size (double and
    mixed), from CUDA events on the streams that do the work; after 3
    resident and 3 drop-in warm-up cycles, the last of --steps timed calls.
    Prints one JSON line: per stage kind its first and last mark (ms after
    the call's first device work), the marks themselves, the call's wall
    time."""
    lul = load_package()
    lul.set_device(0)
    out = {"workload": workload(args.size, args.regions), "timeline": {}}
    for prec in ("fp64", "mixed"):
        dom = lul.HostDomain(args.size, args.regions, 1, 1)
        dev = lul.Device(dom, prec)
        dev.run(dom.cycle + 3)
        dev.download()
        dom.pin(True)
        for _ in range(3):
            dom.time_increment()
            dev.leapfrog()
        dev.timeline(True)
        walls = []
        for _ in range(max(args.steps, 1)):
            dom.time_increment()
            dev.leapfrog()
            walls.append(dev.timeline_read()["wall_ms"])
        t = dev.timeline_read()
        stages = {}
        for name, _, ms in t["marks"]:
            lo, hi = stages.get(name, (ms, ms))
            stages[name] = (min(lo, ms), max(hi, ms))
        out["timeline"][prec] = {
            "stages_first_last_ms": {k: [round(a, 3), round(b, 3)] for k, (a, b) in stages.items()},
            "marks": [[n, i, round(ms, 3)] for n, i, ms in t["marks"]],
            "wall_ms_last": round(t["wall_ms"], 3), "wall_ms_median": round(sorted(walls)[len(walls) // 2], 3)}
        dev.close()
        dom.close()
    print(json.dumps(out), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--size", type=int, default=150)
    ap.add_argument("--regions", type=int, default=21)
    ap.add_argument("--cpu-cycles", type=int, default=180)
    ap.add_argument("--cpu-cycles-1t", type=int, default=6)
    ap.add_argument("--skip-mixed", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-batch", action="store_true")
    ap.add_argument("--skip-serve", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=64)
    ap.add_argument("--batch-problems", type=int, default=64)
    ap.add_argument("--batch-seed", type=int, default=2024)
    ap.add_argument("--timeline", action="store_true",
                    help="print the drop-in call's stage timeline (double and mixed) instead")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.gpus != world:
        ap.error(f"--gpus {args.gpus} but WORLD_SIZE is {world}: launch N > 1 GPUs with "
                 f"torch.distributed.run --nproc-per-node {args.gpus}")
    import oracle

    if not oracle.LIB_PATH.exists():
        oracle.build(ref=False)
    if args.timeline:
        run_timeline(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
