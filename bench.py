#!/usr/bin/env python
"""Benchmark: shallow-water RK4 steps/s at l_max=127 on one GB300.

Workload: Gauss 192x384 grid, l_max=127 (the 3/2-rule product grid equals the
state grid), a batch of independent members, each a Williamson-2 state plus
a seeded (l+1)^-2 perturbation at 1 % of the base RMS, g = 9.80616,
Omega = 7.292e-5, a = 6.371e6, dt = 240 s.  One "step" = one classical RK4
step of the whole member batch (4 fused tendency chains).  Synthetic inputs
(no dataset exists for this path).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--members B]
                  [--precision fp64|split] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is device-timed with the state
resident in HBM (CUDA events around each step, L2 flushed between steps);
`e2e` goes through the public API with the state copied host->device from
pinned memory and back every step.  `--impl reference` times the
reference's algorithm (dense complex basis matrix-vector transforms, the
CPU restatement in oracle/) on the host cores over a bounded row sample.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

os.environ.setdefault("OPENBLAS_NUM_THREADS", str(os.cpu_count() or 1))
os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "SWE RK4 steps/s at lmax=127, split-prec vs FP64 on 1 GB300 @ rel-L2≤1e-10"
UNIT = "steps/s"
NLAT, NLON, LMAX, DT = 192, 384, 127, 240.0
PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
FP64_NOMINAL_GFLOPS = 1250.0  # GB300 FP64 (no measured figure in MEASURED_PEAKS.json)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--members", type=int, default=64)
    ap.add_argument("--precision", choices=["fp64", "split"], default="fp64")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-flush", action="store_true")
    ap.add_argument("--cpu-rows", type=int, default=8, help="latitude rows in the CPU sample")
    return ap.parse_args()


def workload_config(args, B):
    return {"workload": f"swe_rk4_gauss{NLAT}x{NLON}_lmax{LMAX}_members{B}",
            "grid": f"gauss {NLAT}x{NLON}", "l_max": LMAX, "members": B, "dt_s": DT,
            "initial_state": "williamson2 + 1% seeded (l+1)^-2 perturbation per member",
            "precision": args.precision, "global_batch": B * max(args.gpus, 1),
            "parallelism": f"replicas x{max(args.gpus, 1)} (members shard, no collective)"}


# ------------------------------------------------------------ CPU baseline
def cpu_reference_sample(B: int, rows: int, reps: int = 1):
    """Time the reference algorithm for one RK4 step on a row sample.

    The reference's SWE tendency (physics/shallow_water.py:347-418) performs
    12 dense syntheses (2 complex GEMVs each, fast_geodesic_sh.py:89-107) and
    4 dense analyses (a conjugated basis copy + GEMV, :68-87) over the full
    basis matrix; the oracle restatement runs exactly that on `rows` of the
    192 Gauss rows (cost is linear in the point count), and the result is
    scaled to the full grid, 4 stages and B members.  Returns (steps/s,
    description, seconds of CPU work).
    """
    import oracle
    from oracle import models as om
    from aeolus_gb300 import workloads as W

    lat, lon, _, w_point = oracle.gauss_latlon(NLAT, NLON)
    sel = np.linspace(0, NLAT - 1, rows).round().astype(int)
    plat = np.repeat(lat[sel], NLON)
    plon = np.tile(lon, rows)
    pw = np.repeat(w_point.reshape(NLAT, NLON)[sel, 0], NLON)
    sh = oracle.PointSetSH(plat, plon, LMAX, weights=pw)
    ops = oracle.Operators(sh, W.EARTH_RADIUS)
    s0, depth = W.perturbed_williamson2(LMAX, seed=0)
    model = om.SWE(ops, W.EARTH_OMEGA, W.GRAVITY, depth)
    model.tendency(s0)  # warm-up
    t0 = time.perf_counter()
    for _ in range(reps):
        model.tendency(s0)
    t = (time.perf_counter() - t0) / reps
    step_member = t * (NLAT / rows) * 4.0
    desc = (f"reference dense-basis SWE tendency (12 syntheses x 2 GEMV + 4 analyses) on {rows} of {NLAT} "
            f"Gauss rows ({rows * NLON} points x {oracle.n_coeff(LMAX)} modes), timed {reps}x, scaled x{NLAT / rows:g} "
            f"rows x4 stages x{B} members")
    return 1.0 / (step_member * B), desc, t * reps


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    B = args.members
    cores = int(os.environ.get("OPENBLAS_NUM_THREADS", os.cpu_count() or 1))
    if args.warmup > 0:
        cpu_reference_sample(B, max(2, args.cpu_rows // 4), 1)
    vals = []
    desc = ""
    for _ in range(max(args.steps, 1)):
        v, desc, _ = cpu_reference_sample(B, args.cpu_rows, 1)
        vals.append(v)
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, B),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = ROOT / "gpurun_out" / f"clocks_rank{index}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return None
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------ GPU arm
def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    import aeolus_gb300 as ae
    from aeolus_gb300 import _lib, workloads as W
    from aeolus_gb300.shallow_water import ShallowWaterModel

    lib = _lib.load()
    B = args.members
    planet = ae.make_planet("latlon", nlat=NLAT, nlon=NLON, l_max=LMAX, device=dev)
    states, depth = W.member_states(LMAX, B, seed=1000 * rank)
    model = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth)
    if args.precision == "split":
        planet.so._product_space.sh.plan.set_precision(_lib.PREC_SPLIT_BF16)
    y0 = torch.as_tensor(states, device=dev)
    y = y0.clone()
    flush = None if args.no_flush else torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    # warm-up
    for _ in range(max(args.warmup, 3)):
        y = model.rk4(y, DT, 1, check=False)
    barrier()

    # device-timed region: per-step events, L2 flush between steps
    stream = torch.cuda.current_stream(dev)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    lib.aeolus_profile_reset()
    lib.aeolus_profile_enable(1)
    with ClockSampler(local) as clk:
        barrier()
        for i in range(args.steps):
            if flush is not None:
                flush.zero_()
            evs[i][0].record(stream)
            y = model.rk4(y, DT, 1, check=False)
            evs[i][1].record(stream)
        barrier()
    lib.aeolus_profile_enable(0)
    buf = __import__("ctypes").create_string_buffer(1 << 16)
    _lib.check(lib.aeolus_profile_collect(buf, len(buf)))
    kstats = {}
    for line in buf.value.decode().splitlines():
        name, n, ms = line.split()
        kstats[name] = (int(n), float(ms))
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([total_ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * args.steps / (total_ms / 1000.0)

    # end-to-end through the public API: pinned host state in, state out
    host_in = torch.as_tensor(states).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    dev_state = torch.empty_like(y0)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_wall = time.perf_counter()
    e0.record(stream)
    for _ in range(args.steps):
        dev_state.copy_(host_in, non_blocking=True)
        out = model.rk4(dev_state, DT, 1, check=True)   # reads the status word back
        host_out.copy_(out, non_blocking=True)
    e1.record(stream)
    barrier()
    e2e_ms = e0.elapsed_time(e1)
    e2e_wall_ms = (time.perf_counter() - t_wall) * 1000.0
    if world > 1:
        t = torch.tensor([e2e_ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    bytes_state = host_in.numel() * host_in.element_size()

    # roofline of the dominant kernel (algorithmic work per launch)
    dom = max(kstats.items(), key=lambda kv: kv[1][1]) if kstats else None
    roof = None
    if dom is not None:
        name, (n, ms) = dom
        per_launch_s = ms / n / 1000.0
        nh = NLAT // 2
        ftx = 2.0 * NLAT * (LMAX + 1) * (LMAX + 2)  # flops of one real-field Legendre transform
        fields = {"legendre_synth_f64": 9, "legendre_analysis_f64": 4}.get(name)
        peaks = json.loads(PEAKS_FILE.read_text()) if PEAKS_FILE.exists() else {}
        if fields is not None:
            flops = ftx * fields * B
            achieved = flops / per_launch_s / 1e12
            roof = {"kernel": name, "bound": "fp64", "achieved": achieved, "peak": FP64_NOMINAL_GFLOPS / 1000.0,
                    "unit": "TFLOP/s", "frac": achieved / (FP64_NOMINAL_GFLOPS / 1000.0), "traffic": None,
                    "peak_source": "nominal GB300 FP64 (not in MEASURED_PEAKS.json)",
                    "work_per_launch": f"{fields} fields x {B} members x 2*nlat*(L+1)(L+2) flops",
                    "launch_ms": per_launch_s * 1000.0}
        else:
            # row kernel: HBM-bound view -- read F blocks, write G blocks
            byt = B * NLAT * (9 + 4) * (LMAX + 1) * 16.0
            achieved = byt / per_launch_s / 1e9
            pk = peaks.get("hbm_gbs", 6800.0)
            roof = {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": pk, "unit": "GB/s",
                    "frac": achieved / pk, "traffic": None, "launch_ms": per_launch_s * 1000.0}
    launches = sum(n for n, _ in kstats.values())

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, desc, _ = cpu_reference_sample(B, args.cpu_rows, 1)
        cpu = {"value": v, "unit": UNIT, "cores": int(os.environ.get("OPENBLAS_NUM_THREADS", "1")),
               "kind": "port", "sample": desc}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": dict(workload_config(args, B), l2="flushed between steps (256 MiB write)"
                               if flush is not None else "not flushed"),
                "member_steps_per_s": value * B,
                "e2e": {"value": world * args.steps / (e2e_ms / 1000.0), "unit": UNIT,
                        "h2d_bytes_per_step": bytes_state, "d2h_bytes_per_step": bytes_state + 4 * B,
                        "wall_ms": e2e_wall_ms},
                "gpu_launches": launches,
                "kernels": {k: {"launches": n, "ms": ms} for k, (n, ms) in kstats.items()},
                "roofline": roof, "cpu_baseline": cpu, "clocks": clk.summary()}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
