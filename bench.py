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

Rank 0 prints two JSON lines: first the side measurements (configs c3-c5,
the primitive equations, the directly timed c1/c2 steps beside the
reference's own, per-kernel times), then the headline line, last.  `value`
is the split-precision path (bf16-digit tcgen05 contractions, fixed-point
longitude stage); `split_vs_fp64` times the plain FP64 path on the same
states and reports the per-field relative L2 between the two after the
timed steps.  `value` is device-timed
with the state resident in HBM (CUDA events around each step, L2 flushed
between steps);
`e2e` goes through the public API with the state copied host->device from
pinned memory and back every step.  `--impl reference` (and the
`cpu_baseline` key) times the reference's own SWE tendency on the host cores
over a bounded row sample: its package installed unmodified in baseline/_ref
and run with NumPy in place of CuPy (baseline/reference_timing.py), or the
CPU restatement in oracle/ where that package is absent ("kind": "port").
"""
from __future__ import annotations

import argparse
import json
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
    ap.add_argument("--precision", choices=["fp64", "split"], default="split")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-flush", action="store_true")
    ap.add_argument("--cpu-rows", type=int, default=8, help="latitude rows in the CPU sample")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the ensemble (uneven l_max BVE) and adjoint (SWE gradient) side measurements")
    ap.add_argument("--side", choices=["ensemble", "adjoint", "geodesic", "pe"], default=None,
                    help="run only this side measurement (one JSON object); for profiling runs")
    ap.add_argument("--geo-res", type=int, default=6, help="geodesic level of --side geodesic (profiling runs)")
    ap.add_argument("--geo-lmax", type=int, default=127, help="l_max of --side geodesic (profiling runs)")
    ap.add_argument("--knobs", default="",
                    help="launch shapes of the measured model as 5 comma-separated ints (bc_synth, bc_anal, "
                         "row_threads, slice_synth, slice_anal) instead of autotuning; for profiling runs")
    return ap.parse_args()


def workload_config(args, B):
    return {"workload": f"swe_rk4_gauss{NLAT}x{NLON}_lmax{LMAX}_members{B}",
            "grid": f"gauss {NLAT}x{NLON}", "l_max": LMAX, "members": B, "dt_s": DT,
            "initial_state": "williamson2 + 1% seeded (l+1)^-2 perturbation per member",
            "precision": args.precision, "global_batch": B * max(args.gpus, 1),
            "parallelism": f"replicas x{max(args.gpus, 1)} (members shard, no collective)"}


E2E_CHUNKS = 2   # member groups of the end-to-end step (ShallowWaterModel.rk4_host)

# ------------------------------------------------------------ side measurements
ENSEMBLE_GROUPS = [(42, 64, 128, 52), (63, 96, 192, 51), (85, 128, 256, 51), (106, 160, 320, 51),
                   (127, 192, 384, 51)]   # (l_max, nlat, nlon, members): 256 BVE members


def ensemble_measure(dev, steps: int = 10, dt: float = 600.0):
    """256 BVE members over l_max 42..127 on matching Gauss grids (nu = 1e5):
    autotuned grouped launches, one RK4 step captured in a CUDA graph and
    replayed `steps` times, FP64 and split precision; members*steps/s."""
    import torch
    import aeolus_gb300 as ae
    from aeolus_gb300 import _lib, workloads as W
    from aeolus_gb300.barotropic import BarotropicVorticity
    from aeolus_gb300.ensemble import BarotropicEnsemble

    out = {"workload": "bve_ensemble_256members_lmax42-127", "groups": [
        {"l_max": L, "grid": f"{nlat}x{nlon}", "members": B} for L, nlat, nlon, B in ENSEMBLE_GROUPS],
        "dt_s": dt, "viscosity": 1e5, "steps": steps}
    finals = {}
    for prec in ("fp64", "split"):
        models = []
        for L, nlat, nlon, _ in ENSEMBLE_GROUPS:
            planet = ae.make_planet("latlon", nlat=nlat, nlon=nlon, l_max=L, device=dev)
            if prec == "split":
                planet.so._product_space.sh.plan.set_precision(_lib.PREC_SPLIT_BF16)
            models.append(BarotropicVorticity(planet, viscosity=1e5))
        ens = BarotropicEnsemble(models, [g[3] for g in ENSEMBLE_GROUPS])
        init = [torch.as_tensor(np.stack([W.bve_vorticity(L, 7919 * g + b) for b in range(B)]), device=dev)
                for g, (L, _, _, B) in enumerate(ENSEMBLE_GROUPS)]
        states = [x.clone() for x in init]
        report = ens.autotune(states)
        ens.rk4(states, dt, 3)                       # warm-up
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        lib = _lib.load()
        lib.aeolus_profile_reset()
        lib.aeolus_profile_enable(1)
        e0.record()
        ens.rk4(states, dt, steps)
        e1.record()
        torch.cuda.synchronize(dev)
        lib.aeolus_profile_enable(0)
        kstats = _collect_kernels(lib, _lib)
        direct_ms = e0.elapsed_time(e1)
        graph_states = [x.clone() for x in init]
        ens.capture(graph_states, dt)
        ens.replay(3)                                # warm-up
        torch.cuda.synchronize(dev)
        e0.record()
        ens.replay(steps)
        e1.record()
        torch.cuda.synchronize(dev)
        graph_ms = e0.elapsed_time(e1)
        # same trajectory through both paths: compare after 3 + steps steps
        same = all(torch.equal(a, b) for a, b in zip(states, graph_states))
        finals[prec] = states
        out[prec] = {"members_per_s": ens.members * steps / (graph_ms / 1000.0),
                     "ms_per_step_graph": graph_ms / steps, "ms_per_step_direct": direct_ms / steps,
                     "graph_equals_direct": bool(same), "autotune": report.strip().splitlines(),
                     "kernel_ms_per_stage": {k: round(ms / n, 4) for k, (n, ms) in kstats.items()}}
        ens.close()
    rel = []
    for a, b in zip(finals["split"], finals["fp64"]):
        rel.append(float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b)))
    out["rel_l2_split_vs_fp64_per_group"] = rel
    out["split_vs_fp64_speedup"] = out["fp64"]["ms_per_step_graph"] / out["split"]["ms_per_step_graph"]
    return out


def adjoint_measure(dev, members: int = 8, nsteps: int = 48, every: int = 8, dt: float = 240.0):
    """Gradient of the area-weighted final-geopotential misfit through 48 SWE
    RK4 steps (192x384, l_max 127, checkpoints every 8 steps) for `members`
    independent initial states per evaluation; FP64 and split precision."""
    import torch
    import aeolus_gb300 as ae
    from aeolus_gb300 import _lib, workloads as W
    from aeolus_gb300.adjoint import swe_rk4_checkpointed, weighted_phi_misfit
    from aeolus_gb300.ops import synthesize
    from aeolus_gb300.shallow_water import ShallowWaterModel

    out = {"workload": f"swe_adjoint_gauss{NLAT}x{NLON}_lmax{LMAX}_{nsteps}steps_ckpt{every}",
           "members_per_evaluation": members, "dt_s": dt}
    grads = {}
    for prec in ("fp64", "split"):
        planet = ae.make_planet("latlon", nlat=NLAT, nlon=NLON, l_max=LMAX, device=dev)
        if prec == "split":
            planet.so._product_space.sh.plan.set_precision(_lib.PREC_SPLIT_BF16)
        s0, depth = W.member_states(LMAX, members, seed=11)
        st, _ = W.member_states(LMAX, members, seed=12)
        model = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth)
        y0 = torch.as_tensor(s0, device=dev)
        target = synthesize(model._state_plan.id, model.rk4(torch.as_tensor(st, device=dev), dt, nsteps,
                                                            check=False)[:, 2])

        def evaluate():
            y = y0.clone().requires_grad_(True)
            J = weighted_phi_misfit(model, swe_rk4_checkpointed(model, y, dt, nsteps, every), target).sum()
            (g,) = torch.autograd.grad(J, y)
            return g

        evaluate()                                   # warm-up
        torch.cuda.synchronize(dev)
        torch.cuda.reset_peak_memory_stats(dev)
        t0 = time.perf_counter()
        reps = 2
        for _ in range(reps):
            g = evaluate()
        torch.cuda.synchronize(dev)
        sec = (time.perf_counter() - t0) / reps
        grads[prec] = g
        out[prec] = {"gradient_evaluations_per_s": members / sec, "seconds_per_batch": sec,
                     "peak_memory_bytes": int(torch.cuda.max_memory_allocated(dev))}
    d = grads["split"] - grads["fp64"]
    out["rel_l2_split_vs_fp64_gradient"] = [
        float(torch.linalg.vector_norm(d[:, f]) / torch.linalg.vector_norm(grads["fp64"][:, f])) for f in range(3)]
    return out


def geodesic_measure(dev, fields: int = 64, reps: int = 3, res: int = 6, lmax: int = 127):
    """Config c3: level-6 icosahedral grid (40,962 points, Voronoi weights),
    l_max 127 (16,384 real basis columns), one synthesis and one quadrature
    analysis of `fields` seeded fields, FP64 basis GEMMs vs the bf16-digit
    tcgen05 products; ms per (synthesis + analysis) and the split error."""
    import torch
    from aeolus_gb300 import _lib, workloads as W
    from aeolus_gb300.geodesic_grid import GeodesicGridGeometry, GeodesicSphericalHarmonics
    from aeolus_gb300.ops import Plan, analyze, synthesize

    t0 = time.perf_counter()
    sh = GeodesicSphericalHarmonics(GeodesicGridGeometry(res, 6.371e6, dev), lmax, weights="voronoi")
    p64 = sh.plan
    psp = Plan.points(sh.latitudes.cpu().numpy(), sh.longitudes.cpu().numpy(), sh.weights.cpu().numpy(), lmax,
                      device=dev)
    psp.set_precision(_lib.PREC_SPLIT_BF16)
    torch.cuda.synchronize(dev)
    build_s = time.perf_counter() - t0
    rng = np.random.default_rng(5)
    a = torch.as_tensor(np.stack([W.random_spectrum(rng, lmax, -1.5, 1.0, zero_monopole=False)
                                  for _ in range(fields)]), device=dev)
    ncols = (lmax + 1) ** 2
    out = {"workload": f"geodesic_level{res}_{p64.n_points}pts_lmax{lmax}_{fields}fields", "points": p64.n_points,
           "basis_columns": ncols, "fields": fields, "plans_build_s": build_s}
    res = {}
    for name, plan in (("fp64", p64), ("split", psp)):
        g = synthesize(plan.id, a)
        c = analyze(plan.id, g)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            g = synthesize(plan.id, a)
            c = analyze(plan.id, g)
        e1.record()
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / reps
        useful = 2.0 * 2.0 * p64.n_points * ncols * fields
        res[name] = (g, c)
        out[name] = {"ms_synthesis_plus_analysis": ms, "useful_tflops": useful / ms / 1e9}
    out["rel_l2_split_vs_fp64"] = {
        "synthesis": float(torch.linalg.vector_norm(res["split"][0] - res["fp64"][0])
                           / torch.linalg.vector_norm(res["fp64"][0])),
        "analysis": float(torch.linalg.vector_norm(res["split"][1] - res["fp64"][1])
                          / torch.linalg.vector_norm(res["fp64"][1]))}
    out["split_vs_fp64_speedup"] = out["fp64"]["ms_synthesis_plus_analysis"] / out["split"]["ms_synthesis_plus_analysis"]
    return out


def pe_measure(dev, members: int = 4, nlev: int = 20, reps: int = 5):
    """Dry hydrostatic primitive-equation tendency (physics/primitive_equations.py
    :727-753) on the headline grid: Gauss 192x384, l_max 127, `nlev` uniform
    sigma levels, `members` perturbed isothermal states, FP64; tendency
    evaluations/s and the library kernels' share (their own CUDA events)."""
    import torch
    import aeolus_gb300 as ae
    from aeolus_gb300 import _lib
    from aeolus_gb300.primitive_equations import PrimitiveEquationsModel, SigmaGrid, isothermal_rest_state

    L, K = LMAX, nlev
    planet = ae.make_planet("latlon", nlat=NLAT, nlon=NLON, l_max=L, device=dev)
    model = PrimitiveEquationsModel(planet, SigmaGrid.uniform(K))
    rng = np.random.default_rng(17)
    n, cut = L + 1, (2 * L) // 3
    states = []
    for b in range(members):
        st = isothermal_rest_state(L, K, temperature=260.0, surface_pressure=101325.0, device=dev).coeffs
        for i in range(3 * K + 1):
            a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
            a[:, 0] = a[:, 0].real
            a *= np.tril(np.ones((n, n)))
            a[cut + 1:] = 0
            if i < 2 * K or i == 3 * K:
                a[0, 0] = 0
            st[i] += torch.as_tensor(a * (2e-6 if i < 2 * K else (0.5 if i < 3 * K else 1e-3)), device=dev)
        states.append(st)
    x = torch.stack(states)
    lib = _lib.load()
    out = {"workload": f"pe_tendency_gauss{NLAT}x{NLON}_lmax{L}_{K}levels_members{members}",
           "transforms_per_tendency": {"syntheses": members * (10 * K + 2),
                                       "analyses": members * (4 * K + 1) + 2 * members * K}}
    res = {}
    for prec in ("fp64", "split"):
        # split: the product plan's Legendre contractions on the bf16-digit
        # tensor-core path; the degree-(L+1) vector analysis stays FP64
        model._plan.set_precision(_lib.PREC_SPLIT_BF16 if prec == "split" else _lib.PREC_FP64)
        model.tendency(x)
        torch.cuda.synchronize(dev)
        lib.aeolus_profile_reset()
        lib.aeolus_profile_enable(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            y = model.tendency(x)
        e1.record()
        torch.cuda.synchronize(dev)
        lib.aeolus_profile_enable(0)
        ms = e0.elapsed_time(e1) / reps
        ks = _collect_kernels(lib, _lib)
        tot = sum(v for _, v in ks.values()) or 1.0
        res[prec] = y
        out[prec] = {"ms_per_tendency": ms, "member_tendencies_per_s": members * 1e3 / ms,
                     "kernel_share": {k: round(v / tot, 4)
                                      for k, (_, v) in sorted(ks.items(), key=lambda kv: -kv[1][1])}}
    model._plan.set_precision(_lib.PREC_FP64)
    d = res["split"] - res["fp64"]
    blk = lambda t, a, b: float(torch.linalg.vector_norm(t[:, a:b]))  # noqa: E731
    out["rel_l2_split_vs_fp64"] = {
        name: blk(d, a, b) / blk(res["fp64"], a, b)
        for name, a, b in (("zeta", 0, K), ("delta", K, 2 * K), ("temperature", 2 * K, 3 * K),
                           ("ln_ps", 3 * K, 3 * K + 1))}
    out["split_vs_fp64_speedup"] = out["fp64"]["ms_per_tendency"] / out["split"]["ms_per_tendency"]
    return out


# ------------------------------------------------------------ c1 / c2 full steps
DIRECT_CONFIGS = {"c1": dict(model="bve", nlat=32, nlon=64, lmax=21, dt=600.0),
                  "c2": dict(model="swe", nlat=128, nlon=256, lmax=85, dt=300.0)}


def direct_gpu_steps(dev, reps: int = 50):
    """One RK4 step of configs c1 (BVE, Gauss 32x64, l_max 21, dt 600 s) and
    c2 (SWE, Gauss 128x256, l_max 85, dt 300 s) for one member, on the same
    seeded inputs as the reference's directly timed steps: steps/s (CUDA
    events over `reps` steps from the same state) and the state after one
    step, FP64 (c1, c2) and split precision (c2)."""
    import torch
    import aeolus_gb300 as ae
    from aeolus_gb300 import _lib, workloads as W
    from aeolus_gb300.barotropic import BarotropicVorticity
    from aeolus_gb300.shallow_water import ShallowWaterModel

    out = {}
    for name, c in DIRECT_CONFIGS.items():
        for prec in (("fp64",) if c["model"] == "bve" else ("fp64", "split")):
            planet = ae.make_planet("latlon", nlat=c["nlat"], nlon=c["nlon"], l_max=c["lmax"], device=dev)
            if prec == "split":
                planet.so._product_space.sh.plan.set_precision(_lib.PREC_SPLIT_BF16)
            if c["model"] == "bve":
                model = BarotropicVorticity(planet, viscosity=0.0)
                y0 = torch.as_tensor(W.bve_vorticity(c["lmax"], 0), device=dev)[None]
                step = lambda y: model.rk4(y, c["dt"], 1)  # noqa: E731
            else:
                s0, depth = W.perturbed_williamson2(c["lmax"], seed=0)
                model = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth)
                y0 = torch.as_tensor(s0, device=dev)[None]
                step = lambda y: model.rk4(y, c["dt"], 1, check=False)  # noqa: E731
            for _ in range(3):
                y1 = step(y0)
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                y1 = step(y0)
            e1.record()
            torch.cuda.synchronize(dev)
            ms = e0.elapsed_time(e1) / reps
            out[f"{name}_{prec}"] = {"steps_per_s": 1000.0 / ms, "ms_per_step": ms,
                                     "state1": y1[0].cpu().numpy()}
    return out


def direct_reference_steps(reps_c1: int = 5, reps_c2: int = 1):
    """The reference's own RK4 steps at c1 and c2, timed directly (no
    scaling) on the host cores by baseline/reference_timing.py in a child
    process; None where the reference package is absent."""
    import tempfile
    if not (ROOT / "baseline" / "_ref" / "planetary_sandbox").is_dir():
        return None
    script = ROOT / "baseline" / "reference_timing.py"
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, reps in (("c1", reps_c1), ("c2", reps_c2)):
            npz = Path(tmp) / f"{name}.npz"
            r = subprocess.run([sys.executable, str(script), name, str(reps), str(npz)], capture_output=True,
                               text=True, env=env, timeout=900)
            if r.returncode != 0:
                print(f"reference {name} step unavailable: {r.stderr.strip().splitlines()[-1:]}", file=sys.stderr)
                continue
            d = json.loads(r.stdout.strip().splitlines()[-1])
            z = np.load(npz)
            d["state1"] = z["state1"]
            out[name] = d
    return out


def direct_steps_report(gpu, ref, cores: int):
    """c1 / c2: GPU steps/s beside the reference's directly timed CPU step on
    the same inputs, and the relative L2 between the two final states."""
    rep = {}
    for name, c in DIRECT_CONFIGS.items():
        r = (ref or {}).get(name)
        e = {"workload": f"{c['model']}_rk4_gauss{c['nlat']}x{c['nlon']}_lmax{c['lmax']}_dt{c['dt']:g}_1member"}
        if r is not None:
            e["reference_cpu"] = {"steps_per_s": 1.0 / r["seconds_per_step"], "seconds_per_step": r["seconds_per_step"],
                                  "reps": r["reps"], "cores": cores, "extrapolated": False,
                                  "code": "planetary_sandbox rk4_step (run/bve/runner.py:211-216)" if c["model"] == "bve"
                                  else "planetary_sandbox rk4_step_array over ShallowWaterModel.tendency "
                                       "(run/engine.py:406-431)"}
        for prec in ("fp64", "split"):
            g = gpu.get(f"{name}_{prec}")
            if g is None:
                continue
            e[f"gpu_{prec}"] = {"steps_per_s": g["steps_per_s"], "ms_per_step": g["ms_per_step"]}
            if r is not None:
                a, b = g["state1"], r["state1"]
                e[f"gpu_{prec}"]["rel_l2_vs_reference_step"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
                e[f"gpu_{prec}"]["speedup_vs_reference_cpu"] = g["steps_per_s"] * r["seconds_per_step"]
        rep[name] = e
    return rep


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
    extra = {"extrapolated": True, "measured_s_per_sample_tendency": t, "rows": rows,
             "scale": (NLAT / rows) * 4.0 * B}
    return 1.0 / (step_member * B), desc, t * reps, extra


def reference_own_sample(B: int, rows: int, reps: int = 1):
    """The reference's own SWE tendency (its package in baseline/_ref, run with
    the NumPy stand-in for CuPy in a child process by
    baseline/reference_timing.py) on `rows` of the 192 Gauss rows, scaled to
    the full grid, 4 stages and B members.  Returns (steps/s, description,
    seconds) or None when the reference package or its CPU-built basis
    kernel is not available on this host."""
    script = ROOT / "baseline" / "reference_timing.py"
    if not (ROOT / "baseline" / "_ref" / "planetary_sandbox").is_dir():
        return None
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
    t0 = time.perf_counter()
    r = subprocess.run([sys.executable, str(script), str(rows), str(reps)], capture_output=True, text=True,
                       env=env, timeout=900)
    if r.returncode != 0:
        print(f"reference CPU timing unavailable: {r.stderr.strip().splitlines()[-1:]}", file=sys.stderr)
        return None
    d = json.loads(r.stdout.strip().splitlines()[-1])
    t = d["seconds_per_tendency"]
    step_member = t * (NLAT / rows) * 4.0
    desc = (f"the reference's own ShallowWaterModel.tendency (planetary_sandbox, NumPy in place of CuPy, its "
            f"CUDA-C basis kernel built for the CPU) on {rows} of {NLAT} Gauss rows ({d['points']} points x "
            f"{d['modes']} modes), timed {reps}x, scaled x{NLAT / rows:g} rows x4 stages x{B} members")
    extra = {"extrapolated": True, "measured_s_per_sample_tendency": t, "rows": rows,
             "scale": (NLAT / rows) * 4.0 * B}
    return 1.0 / (step_member * B), desc, time.perf_counter() - t0, extra


def cpu_baseline_sample(B: int, rows: int, reps: int = 1):
    """(steps/s, description, seconds, extrapolation fields, kind): the
    reference's own code when it runs here ("reference"), else the oracle
    restatement ("port").  The step rate is extrapolated from a row sample:
    a full 64-member step of the reference takes hours on the host cores."""
    own = reference_own_sample(B, rows, reps)
    if own is not None:
        return own + ("reference",)
    return cpu_reference_sample(B, rows, reps) + ("port",)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    B = args.members
    cores = int(os.environ.get("OPENBLAS_NUM_THREADS", os.cpu_count() or 1))
    kind = "port"
    if args.warmup > 0:
        cpu_baseline_sample(B, max(2, args.cpu_rows // 4), 1)
    vals = []
    desc = ""
    extra = {}
    for _ in range(max(args.steps, 1)):
        v, desc, _, extra, kind = cpu_baseline_sample(B, args.cpu_rows, 1)
        vals.append(v)
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, B),
            "cpu_baseline": dict({"value": v, "unit": UNIT, "cores": cores, "kind": kind, "sample": desc}, **extra),
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------ clocks
class _Nvml:
    """Read-only NVML queries through ctypes (SM clock, max SM clock, clock
    event reasons), polled from a thread every few milliseconds so that a
    timed region of ~0.1 s still gets dozens of samples."""
    SW_POWER_CAP, HW_SLOWDOWN, SW_THERMAL, HW_THERMAL = 0x4, 0x8, 0x20, 0x40

    def __init__(self, torch_index: int):
        import ctypes
        self.ct = ctypes
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        import torch
        uuid = str(getattr(torch.cuda.get_device_properties(torch_index), "uuid", ""))
        ok = False
        if uuid:
            key = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
            ok = self.lib.nvmlDeviceGetHandleByUUID(key.encode(), ctypes.byref(self.h)) == 0
        if not ok and self.lib.nvmlDeviceGetHandleByIndex_v2(torch_index, ctypes.byref(self.h)) != 0:
            raise RuntimeError("no NVML handle")
        fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None)
        self.reasons_fn = fn or self.lib.nvmlDeviceGetCurrentClocksThrottleReasons

    def sample(self):
        ct = self.ct
        clk, mx, rs = ct.c_uint(), ct.c_uint(), ct.c_ulonglong()
        if self.lib.nvmlDeviceGetClockInfo(self.h, 1, ct.byref(clk)) != 0:
            return None
        self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, ct.byref(mx))
        self.reasons_fn(self.h, ct.byref(rs))
        return clk.value, mx.value, rs.value


class ClockSampler:
    """SM clock and clock-event reasons during the timed region: NVML polled
    every 2 ms when libnvidia-ml loads, else nvidia-smi at 200 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.nvml = None
        self.samples = []
        # the nvidia-smi fallback's raw samples (a directory chosen by the
        # caller, else the system temporary directory)
        import tempfile
        out = os.environ.get("AEOLUS_BENCH_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = Path(out) / f"aeolus_clocks_rank{index}.csv"

    def _poll(self):
        while not self._stop.is_set():
            v = self.nvml.sample()
            if v is not None:
                self.samples.append(v)
            self._stop.wait(0.002)

    def __enter__(self):
        import threading
        try:
            self.nvml = _Nvml(self.index)
        except Exception:
            self.nvml = None
        if self.nvml is not None:
            self._stop = threading.Event()
            self._thr = threading.Thread(target=self._poll, daemon=True)
            self._thr.start()
            return self
        try:
            self.path.parent.mkdir(parents=True, exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.nvml is not None:
            self._stop.set()
            self._thr.join(timeout=5)
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        names = {_Nvml.HW_SLOWDOWN: "hw_slowdown", _Nvml.HW_THERMAL: "hw_thermal_slowdown",
                 _Nvml.SW_THERMAL: "sw_thermal_slowdown", _Nvml.SW_POWER_CAP: "sw_power_cap"}
        if self.samples:
            reasons = sorted({nm for _, _, r in self.samples for bit, nm in names.items() if r & bit})
            return {"sm_mhz": statistics.median(c for c, _, _ in self.samples),
                    "sm_max_mhz": max(m for _, m, _ in self.samples), "reasons": reasons,
                    "samples": len(self.samples), "source": "nvml 2 ms"}
        if self.proc is None or not self.path.exists():
            return None
        sm, smax, reasons = [], None, set()
        order = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(order, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm), "source": "nvidia-smi 200 ms"}


# ------------------------------------------------------------ GPU arm
def _collect_kernels(lib, _lib):
    import ctypes
    buf = ctypes.create_string_buffer(1 << 16)
    _lib.check(lib.aeolus_profile_collect(buf, len(buf)))
    out = {}
    for line in buf.value.decode().splitlines():
        name, n, ms = line.split()
        out[name] = (int(n), float(ms))
    return out


PROF_STEPS = 2  # steps run with the per-kernel event profile after the timed ones


def _timed_steps(model, y0, steps, flush, stream, lib, _lib, prof_steps: int = PROF_STEPS):
    """K RK4 steps from y0, each bracketed by CUDA events on the launching
    stream, L2 flushed (outside the events) before each step; the library's
    per-kernel event profile is off while they run (its events would sit
    between the kernels) and is taken over `prof_steps` further steps from
    the same state, which do not count."""
    import torch
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    y = y0
    for i in range(steps):
        if flush is not None:
            flush.zero_()
        evs[i][0].record(stream)
        y = model.rk4(y, DT, 1, check=False)
        evs[i][1].record(stream)
    torch.cuda.synchronize()
    total = sum(a.elapsed_time(b) for a, b in evs)
    lib.aeolus_profile_reset()
    lib.aeolus_profile_enable(1)
    yp = y0
    for _ in range(prof_steps):
        if flush is not None:
            flush.zero_()
        yp = model.rk4(yp, DT, 1, check=False)
    torch.cuda.synchronize()
    lib.aeolus_profile_enable(0)
    kstats = _collect_kernels(lib, _lib)
    return total, kstats, y


def _rel_l2_fields(a, b):
    import torch
    d = (a - b).reshape(a.shape[0], 3, -1)
    r = b.reshape(b.shape[0], 3, -1)
    num = torch.linalg.vector_norm(d, dim=-1)
    den = torch.linalg.vector_norm(r, dim=-1).clamp_min(1e-300)
    worst = (num / den).amax(dim=0)
    return {name: float(v) for name, v in zip(("zeta", "delta", "phi"), worst)}


# DRAM bytes (read + write) per launch of the split-path kernels on this
# workload: dram__bytes_read.sum + dram__bytes_write.sum from one ncu capture
# of the first RK4 stage (cold L2).
NCU_TRAFFIC = {
    "split_synth_slice": 27.497728e6 + 86.54464e6,
    "tc_synth_bf16x6": 138.119424e6 + 174.368e6,
    "rows_fx_c2r_products_r2c": 226.578432e6 + 75.243008e6,
    "split_anal_slice": 100.69504e6 + 95.401472e6,
    "tc_anal_bf16x6": 230.352896e6 + 67.960576e6,
}


# Warp instructions per launch of the same kernels (smsp__inst_executed.sum
# of the same capture), for the instruction-issue roofline of the row stage.
NCU_WARP_INSTRUCTIONS = {
    "rows_fx_c2r_products_r2c": 294.58e6,
}
SM_COUNT, ISSUE_PER_SM_CLK = 152, 4  # GB300: 4 schedulers per SM, one warp instruction each per clock


def _roofline(kstats, B, peaks):
    """Roofline entry for every library kernel; the dominant one first."""
    ftx = 2.0 * NLAT * (LMAX + 1) * (LMAX + 2)  # flops of one real-field Legendre transform (no fold credit)
    hbm = peaks.get("hbm_gbs", 6800.0)
    tensor = peaks.get("bf16_tflops", 1900.0)
    entries = {}
    for name, (n, ms) in kstats.items():
        t = ms / n / 1000.0
        if name.startswith("tc_synth") or name.startswith("tc_anal"):
            # synthesis: the 7 contracted fields (the two longitude derivatives
            # the model also needs are formed in its epilogue, not contracted)
            fields = 7 if name.startswith("tc_synth") else 4
            useful = ftx * fields * B
            entries[name] = {"kernel": name, "bound": "tensor", "achieved": useful / t / 1e12, "peak": tensor,
                             "unit": "TFLOP/s", "frac": useful / t / 1e12 / tensor,
                             "traffic": NCU_TRAFFIC.get(name), "launch_ms": t * 1000.0,
                             "work_per_launch": f"{fields} fields x {B} members x 2*nlat*(L+1)(L+2) useful flops "
                                                "(the 21 bf16 digit-pair products are not counted)"}
        elif name.startswith("rows"):
            byt = B * NLAT * (9 + 4) * (LMAX + 1) * 16.0
            entries[name] = {"kernel": name, "bound": "hbm", "achieved": byt / t / 1e9, "peak": hbm, "unit": "GB/s",
                             "frac": byt / t / 1e9 / hbm, "traffic": NCU_TRAFFIC.get(name), "launch_ms": t * 1000.0,
                             "work_per_launch": f"{B} members x {NLAT} rows x 13 spectra x (L+1) x 16 B",
                             "note": "bound by integer issue and barrier latency of the fixed-point FFTs, not by HBM"}
            inst = NCU_WARP_INSTRUCTIONS.get(name)
            if inst is not None and B == 64:
                # instruction-issue roofline: warp instructions of one launch (ncu, same workload) over
                # its event-timed duration, against 4 issue slots per SM per clock at the sampled clock
                clk = peaks.get("_sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
                peak_issue = SM_COUNT * ISSUE_PER_SM_CLK * clk * 1e6
                entries[name]["issue"] = {"warp_instructions_per_launch": inst, "achieved_per_s": inst / t,
                                          "peak_per_s": peak_issue, "frac": inst / t / peak_issue,
                                          "clock_mhz": clk}
        elif name.endswith("_f64"):
            fields = 9 if "synth" in name else 4
            useful = ftx * fields * B
            entries[name] = {"kernel": name, "bound": "fp64", "achieved": useful / t / 1e12,
                             "peak": FP64_NOMINAL_GFLOPS / 1000.0, "unit": "TFLOP/s",
                             "frac": useful / t / 1e12 / (FP64_NOMINAL_GFLOPS / 1000.0), "traffic": None,
                             "launch_ms": t * 1000.0, "peak_source": "nominal (no FP64 figure measured)"}
    order = sorted(kstats, key=lambda k: -kstats[k][1])
    dom = next((entries[k] for k in order if k in entries), None)
    return dom, [entries[k] for k in order if k in entries]


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
    if args.side:
        if args.side == "geodesic":
            res = geodesic_measure(dev, res=args.geo_res, lmax=args.geo_lmax)
        else:
            res = {"ensemble": ensemble_measure, "adjoint": adjoint_measure, "pe": pe_measure}[args.side](dev)
        print(json.dumps({args.side: res}))
        return 0

    import aeolus_gb300 as ae
    from aeolus_gb300 import _lib, workloads as W
    from aeolus_gb300.shallow_water import ShallowWaterModel

    lib = _lib.load()
    B = args.members
    from aeolus_gb300.replicas import max_over_ranks, member_seed_base
    states, depth = W.member_states(LMAX, B, seed=member_seed_base(rank, B))

    def build(precision):
        planet = ae.make_planet("latlon", nlat=NLAT, nlon=NLON, l_max=LMAX, device=dev)
        if precision == "split":
            planet.so._product_space.sh.plan.set_precision(_lib.PREC_SPLIT_BF16)
        return ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth)

    model = build(args.precision)
    other = build("fp64") if args.precision == "split" else None
    y0 = torch.as_tensor(states, device=dev)
    flush = None if args.no_flush else torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    warm = max(args.warmup, 3)
    tuning = {}
    for name, m in (("split" if args.precision == "split" else "fp64", model), ("fp64", other)):
        if m is not None:
            y = y0
            if args.knobs and m is model:
                m._plan.set_tuning([int(x) for x in args.knobs.split(",")])
                tuning[name] = {"knobs_bc_synth_bc_anal_row_threads_slice_synth_anal": list(m._plan.tuning()),
                                "ms_per_step": None, "source": "--knobs"}
            for _ in range(warm):
                y = m.rk4(y, DT, 1, check=False)
            if args.knobs and m is model:
                continue
            tuned = m.autotune(y0, DT)   # launch shapes for this batch; results do not depend on them
            tuning[name] = {"knobs_bc_synth_bc_anal_row_threads_slice_synth_anal": list(tuned["chosen"]),
                            "ms_per_step": tuned["ms_per_step"]}
    barrier()

    with ClockSampler(local) as clk:
        barrier()
        total_ms, kstats, y_main = _timed_steps(model, y0, args.steps, flush, stream, lib, _lib)
        barrier()
    total_ms = max_over_ranks(total_ms, dev)
    value = world * args.steps / (total_ms / 1000.0)

    comparison = None
    if other is not None:
        ms64, k64, y64 = _timed_steps(other, y0, args.steps, flush, stream, lib, _lib)
        comparison = {"fp64_steps_per_s": args.steps / (ms64 / 1000.0),
                      "fp64_ms_per_step": ms64 / args.steps,
                      "speedup_split_vs_fp64": (ms64 / total_ms),
                      "rel_l2_split_vs_fp64_after_steps": _rel_l2_fields(y_main, y64),
                      "fp64_kernels": {k: {"launches": n, "ms": ms} for k, (n, ms) in k64.items()}}

    # end-to-end through the public API: pinned host state in, state out
    host_in = torch.as_tensor(states).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    for _ in range(warm):   # side streams and their workspaces exist before timing
        model.rk4_host(host_in, DT, 1, chunks=E2E_CHUNKS, out=host_out, check=True)
    torch.cuda.synchronize()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_wall = time.perf_counter()
    e0.record(stream)
    for _ in range(args.steps):
        # members in E2E_CHUNKS groups on streams of their own: copies of one
        # group overlap the steps of the others; status read back every step
        model.rk4_host(host_in, DT, 1, chunks=E2E_CHUNKS, out=host_out, check=True)
    e1.record(stream)
    barrier()
    e2e_ms = e0.elapsed_time(e1)
    e2e_wall_ms = (time.perf_counter() - t_wall) * 1000.0
    e2e_ms = max_over_ranks(e2e_ms, dev)
    bytes_state = host_in.numel() * host_in.element_size()

    peaks = json.loads(PEAKS_FILE.read_text()) if PEAKS_FILE.exists() else {}
    clock_summary = clk.summary()
    if isinstance(clock_summary, dict) and clock_summary.get("sm_mhz"):
        peaks["_sm_mhz"] = float(clock_summary["sm_mhz"])   # issue peak at the clock seen while timing
    roof, roof_all = _roofline(kstats, B, peaks)
    # library kernels launched in the timed region: the profiled steps run the
    # same launches per step as the timed ones
    launches = sum(n for n, _ in kstats.values()) * args.steps // PROF_STEPS

    extras = {}
    direct_gpu = None
    if rank == 0 and not args.no_extras:
        extras["ensemble"] = ensemble_measure(dev)
        extras["adjoint"] = adjoint_measure(dev)
        extras["geodesic"] = geodesic_measure(dev)
        extras["pe"] = pe_measure(dev)
        direct_gpu = direct_gpu_steps(dev)

    cores = int(os.environ.get("OPENBLAS_NUM_THREADS", "1"))
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, desc, _, extra, kind = cpu_baseline_sample(B, args.cpu_rows, 1)
        cpu = dict({"value": v, "unit": UNIT, "cores": cores, "kind": kind, "sample": desc}, **extra)
    direct = None
    if direct_gpu is not None:
        ref = None if args.no_cpu_baseline else direct_reference_steps()
        direct = direct_steps_report(direct_gpu, ref, cores)

    if rank == 0:
        # side measurements and per-kernel detail first, on a line of their
        # own; the headline line (with the split-vs-FP64 ratio) comes last
        side = {"side_measurements": dict(extras, direct_steps=direct, autotune=tuning,
                                          kernels={k: {"launches": n, "ms": ms} for k, (n, ms) in kstats.items()},
                                          roofline_all=roof_all,
                                          fp64_kernels=comparison.pop("fp64_kernels") if comparison else None)}
        print(json.dumps(side), flush=True)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": warm, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "bf16x6-digit/i64-fixed/f32x2/f64" if args.precision == "split" else "f64", "data": "synthetic",
                "config": dict(workload_config(args, B), l2="flushed between steps (256 MiB write)"
                               if flush is not None else "not flushed"),
                "member_steps_per_s": value * B,
                "e2e": {"value": world * args.steps / (e2e_ms / 1000.0), "unit": UNIT,
                        "h2d_bytes_per_step": bytes_state, "d2h_bytes_per_step": bytes_state + 4 * B,
                        "wall_ms": e2e_wall_ms},
                "gpu_launches": launches,
                "roofline": roof, "cpu_baseline": cpu, "clocks": clock_summary}
        if direct is not None:
            line["direct_steps_vs_reference"] = {
                k: {kk: {m: float(f"{x:.4g}") for m, x in vv.items()
                         if m in ("steps_per_s", "rel_l2_vs_reference_step")}
                    for kk, vv in v.items() if isinstance(vv, dict)} for k, v in direct.items()}
        line["split_vs_fp64"] = comparison
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
