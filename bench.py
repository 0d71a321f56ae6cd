"""Benchmark: RK4 site-updates/s of the fused GB300 level step.

Workload (native arm, N=1): uniform periodic 512^3 box, Moore mode (c0 = 2),
lambda0 = 2, radiation domination (a_inv = 2), dx = 0.5, dt = 0.1, seeded
Gaussian Fourier initial data with |n| < N/8 (k < 2 pi/(8 dx)), Pi = 0;
FP32 fields (the reference's default PRECISION=FLOAT), FP64 background.
One "step" = one classic-RK4 step of the whole box: one launch of the one-pass
fused step, or sweep A and sweep B, whichever tiling the autotuner picks.

Reported on one JSON line: whole-job site-updates/s (value), the FP64 path on
the same box, FP32-vs-FP64 energy / xi / string-count error after a short
evolution, the roofline of the dominant step kernel, an end-to-end number
through the C ABI with host buffers, the CPU oracle baseline and the SM
clocks sampled during the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl native|reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RK4 site-updates/s on 1 GB300, FP32 vs FP64 at <=1e-5 energy err; adjoint/fwd ratio"
UNIT = "site-updates/s"
N_DEFAULT = 512
DX, DT, TAU_I = 0.5, 0.1, 1.0
A_INV, C0, LAMBDA0 = 2.0, 2.0, 2.0
SEED = 20261203


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _config(n, extra=None):
    c = {"workload": f"uniform periodic {n}^3, Moore c0=2, lambda0=2, a_inv=2 (RD), dx=0.5, dt=0.1, "
                     f"seeded Gaussian IC |n|<N/8, FP32 fields + FP64 background",
         "grid": [n, n, n], "dx": DX, "dt": DT, "c0": C0, "lambda0": LAMBDA0, "a_inv": A_INV,
         "fields": "fp32", "l2": "inputs larger than L2 (state 2.2 GB + stage buffers 4.4 GB)",
         "parallelism": "replicas (one independent box per GPU)"}
    if extra:
        c.update(extra)
    return c


# ---------------------------------------------------------------- clocks
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 9:
                    rows.append(p)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for nm, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# ---------------------------------------------------------------- CPU baseline (oracle port)
def cpu_baseline(seconds: float = 10.0, n: int = N_DEFAULT):
    """The CPU restatement (oracle/, OpenMP over all host cores) on a bounded
    sample: FP32 RK4 steps of an n^3 box of the same workload until ~`seconds`."""
    import numpy as np
    from oracle import oracle as O
    O.lib()
    v = O.fourier_ic_state(n, O.strict_cutoff(n / 8), seed=SEED).astype(np.float32)
    fab = O.to_fab(v, 2)
    bg = O.background(a_inv=A_INV, c0=C0, lambda_scale=LAMBDA0)
    steps, t_total = 0, 0.0
    while t_total < seconds:
        t0 = time.perf_counter()
        O.rk4_advance(fab, 2, DX, bg, TAU_I, steps * DT, DT, 1)
        t_total += time.perf_counter() - t0
        steps += 1
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": steps * n ** 3 / t_total, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{steps} FP32 RK4 steps of a {n}^3 box of the same workload ({t_total:.1f} s)"}


# ---------------------------------------------------------------- reference arm
def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    import numpy as np
    from oracle import oracle as O
    O.build()
    n = args.ref_n
    v = O.fourier_ic_state(n, O.strict_cutoff(n / 8), seed=SEED).astype(np.float32)
    fab = O.to_fab(v, 2)
    bg = O.background(a_inv=A_INV, c0=C0, lambda_scale=LAMBDA0)
    for w in range(args.warmup):
        O.rk4_advance(fab, 2, DX, bg, TAU_I, w * DT, DT, 1)
    t0 = time.perf_counter()
    for s in range(args.steps):
        O.rk4_advance(fab, 2, DX, bg, TAU_I, (args.warmup + s) * DT, DT, 1)
    el = time.perf_counter() - t0
    value = args.steps * n ** 3 / el
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": _config(N_DEFAULT, {"reference_sample": f"each step = one FP32 RK4 step of a {n}^3 box"
                                                              + (" (the workload itself)" if n == N_DEFAULT else
                                                                 f" (bounded sample of the {N_DEFAULT}^3 workload)")}),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} FP32 RK4 steps of a {n}^3 box; CPU restatement of the "
                                       f"reference path (its AMReX build is not buildable here)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- CPU baseline table
def cpu_table():
    """The CPU oracle (OpenMP over all host cores) on the configurations of the
    reference's CPU baseline table: RK4 site-updates/s and one diagnostics pass
    (counts, 14 energy sums, velocity) per configuration, both precisions."""
    import numpy as np
    from oracle import oracle as O
    O.lib()
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    rows = []
    for n, c0, kdiv, prec, steps in ((64, 1.0, 4, "f64", 100), (64, 1.0, 4, "f32", 100), (512, 2.0, 8, "f32", 4),
                                     (512, 2.0, 8, "f64", 3)):
        v = O.fourier_ic_state(n, O.strict_cutoff(n / kdiv), seed=SEED)
        if prec == "f32":
            v = v.astype(np.float32)
        fab = O.to_fab(v, 2)
        del v
        bg = O.background(a_inv=A_INV, c0=c0, lambda_scale=LAMBDA0)
        O.rk4_advance(fab, 2, DX, bg, TAU_I, 0.0, DT, 1)
        t0 = time.perf_counter()
        O.rk4_advance(fab, 2, DX, bg, TAU_I, DT, DT, steps)
        el = time.perf_counter() - t0
        tau = TAU_I + (steps + 1) * DT
        co = O.background_eval(bg, tau)[0]
        R, lam = co[0], co[3]
        t1 = time.perf_counter()
        O.count_plaquettes(fab, 2)
        O.energy_sums(fab, 2, DX, R, lam, co[1] / R, O.MASK_A, 0.8)
        O.velocity(fab, 2, R, co[1] / R, float(np.sqrt(lam)))
        dg = time.perf_counter() - t1
        rows.append({"grid": n, "c0": c0, "precision": prec, "steps": steps, "cores": cores,
                     "site_updates_per_s": n ** 3 * steps / el, "diag_pass_ms": 1e3 * dg})
        del fab
    print(json.dumps({"cpu_table": rows, "host_cores": os.cpu_count()}), flush=True)


# ---------------------------------------------------------------- drop-in per-stage path
def dropin_report(A, ic, dev, n=512, steps=4, warmup=1):
    """The one-for-one replacement of specific_eval_rhs under a host RK driver
    (AxionStringsLevel.cpp:909-920, GRTeclyn's classic RK4): per step four
    ghost fills + axs_eval_rhs on AMReX-layout FABs, three axs_lincomb stage
    combinations and one axs_rk4_combine, in FP32 and FP64 on the headline
    box: ng = 2 (FP32 rows staged in 16-byte pieces) and, in FP32, ng = 3 (cell
    by cell). Algorithmic words per site and step: eval_rhs 8 (4 read, 4
    written) x 4, lincomb 12 x 3, rk4_combine 24: 92 (ghost fills excluded)."""
    import torch
    bg = A.Background.expanding(A_INV, C0, lambda0=LAMBDA0)
    out = {"words_per_site_step": 92, "kernels_per_step": ["fill_periodic x4", "eval_rhs x4", "lincomb x3",
                                                           "rk4_combine"]}
    s0 = ic.fourier_state(n, ic.strict_cutoff(n / 8), seed=SEED, dtype=torch.float64, device=dev)
    for name, dt_, ng in (("f32", torch.float32, 2), ("f32_ng3", torch.float32, 3), ("f64", torch.float64, 2)):
        u = A.new_fab((n, n, n), ng, dtype=dt_, device=dev)
        A.valid(u, ng).copy_(s0)
        uold, us = torch.empty_like(u), torch.empty_like(u)
        ks = [torch.empty_like(u) for _ in range(4)]
        def step(t):
            uold.copy_(u)
            for s_, (ts, cs) in enumerate(((t, 0.5 * DT), (t + 0.5 * DT, 0.5 * DT), (t + 0.5 * DT, DT), (t + DT, None))):
                src = uold if s_ == 0 else us
                A.fill_periodic_ghosts(src, ng)
                # specific_eval_rhs: the stage's coefficients, then the RHS kernel
                A.eval_rhs(src, ks[s_], ng, ng, DX, bg.rhs_coeffs(TAU_I + ts))
                if cs is not None:
                    A.lincomb(us, uold, cs, ks[s_], ng)
            A.rk4_combine(u, uold, *ks, ng, DT)
        for w in range(warmup):
            step(w * DT)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for s_ in range(steps):
            step((warmup + s_) * DT)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        es = 4 if dt_ == torch.float32 else 8
        out[name] = {"ms_per_step": ms, "value": n ** 3 / (ms * 1e-3), "unit": UNIT,
                     "achieved_gbs": 92 * es * n ** 3 / (ms * 1e-3) / 1e9}
        del u, uold, us, ks
        torch.cuda.empty_cache()
    return out


# ---------------------------------------------------------------- differentiation configuration
def differentiation_report(A, ic, dev, n=128, nsteps=200, ndir=16):
    import torch
    from axion_strings_adaptive_gb300.adjoint import EvolutionSpec, string_core_loss
    spec = EvolutionSpec(dx=DX, dt=DT, nsteps=nsteps, tau_i=TAU_I, a_inv=A_INV, c0=1.0, width=0.1,
                         checkpoint_every=20)
    s0 = ic.fourier_state(n, ic.strict_cutoff(n / 4), seed=SEED + 4, dtype=torch.float64, device=dev)
    res = {}
    for dt_, name in ((torch.float32, "fp32"), (torch.float64, "fp64")):
        x = s0.to(dt_).clone().requires_grad_(True)
        lam = torch.tensor(LAMBDA0, dtype=dt_, requires_grad=True)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        torch.cuda.synchronize()
        e0.record()
        loss = string_core_loss(x, lam, spec)
        e1.record()
        loss.backward()
        e2.record()
        torch.cuda.synchronize()
        res[name] = {"loss": float(loss), "grad": x.grad.double(), "lambda_grad": float(lam.grad),
                     "forward_ms": e0.elapsed_time(e1), "backward_ms": e1.elapsed_time(e2)}
    g32, g64 = res["fp32"]["grad"], res["fp64"]["grad"]
    lam64 = torch.tensor(LAMBDA0, dtype=torch.float64)
    gen = torch.Generator(device=dev).manual_seed(SEED + 5)
    eps = 1e-3
    dirs = []
    for _ in range(ndir):
        d = torch.zeros_like(s0)
        d[:2] = torch.randn(d[:2].shape, generator=gen, device=dev, dtype=torch.float64)
        d /= d.norm()
        fd = (float(string_core_loss(s0 + eps * d, lam64, spec)) -
              float(string_core_loss(s0 - eps * d, lam64, spec))) / (2 * eps)
        dirs.append({"fd": fd, "adjoint_fp32": float((g32 * d).sum()), "adjoint_fp64": float((g64 * d).sum())})
    fd_l = (float(string_core_loss(s0, lam64 + eps, spec)) - float(string_core_loss(s0, lam64 - eps, spec))) / (2 * eps)
    scale = float(g64[:2].norm())

    def rel(a, b, floor=0.0):
        return abs(a - b) / max(abs(b), floor, 1e-300)

    out = {"config": f"{n}^3 FP32, c0=1, lambda0=2, {nsteps} RK4 steps, dx=0.5, dt=0.1, checkpoint every 20, "
                     f"loss = sum exp(-|psi/R|^2/0.1) + <axion kinetic energy>, IC |n|<N/4, Pi=0",
           "loss": {k: v["loss"] for k, v in res.items()},
           "grad_psi_rel_err_fp32_vs_fp64": float((g32[:2] - g64[:2]).norm() / g64[:2].norm()),
           "lambda_grad": {"fp32": res["fp32"]["lambda_grad"], "fp64": res["fp64"]["lambda_grad"], "fd": fd_l},
           "lambda_grad_rel_err": {"fp32_vs_fd": rel(res["fp32"]["lambda_grad"], fd_l),
                                   "fp64_vs_fd": rel(res["fp64"]["lambda_grad"], fd_l)},
           "directions": len(dirs), "eps": eps,
           "max_rel_err_fp32_vs_fd": max(rel(d["adjoint_fp32"], d["fd"], 1e-3 * scale) for d in dirs),
           "max_rel_err_fp64_vs_fd": max(rel(d["adjoint_fp64"], d["fd"], 1e-3 * scale) for d in dirs),
           "rel_err_floor": "1e-3 x |grad_psi| (directional derivatives near zero)",
           "timing_ms": {k: {"forward": v["forward_ms"], "backward": v["backward_ms"],
                             "backward_over_forward": v["backward_ms"] / v["forward_ms"]} for k, v in res.items()},
           "directional": dirs}
    return out


# ---------------------------------------------------------------- batching configuration
def batching_report(A, ic, dev, hbm_peak, nboxes=64, nsteps=200, sizes=(32, 48, 64, 96, 128)):
    """64 seeded boxes of sizes drawn uniformly from `sizes`, FP32, c0 = 1,
    lambda0 = 2, IC |n| < N_box/4 (seed + box), 200 RK4 steps per box: the
    autotuned tiling over all boxes at once (the fused step: one persistent
    launch per RK4 step; a two-sweep tiling: one per sweep), the whole run plus
    per-box diagnostics captured as one CUDA graph; beside it the same boxes
    advanced one level at a time."""
    import numpy as np
    import torch
    rng = np.random.RandomState(SEED)
    ns = [int(v) for v in rng.choice(sizes, size=nboxes)]
    dims = [(n, n, n) for n in ns]
    bg = A.Background.expanding(A_INV, 1.0, lambda0=LAMBDA0)
    ens = A.Ensemble(dims, DX, dtype=torch.float32, device=dev)
    ics = []
    for b, n in enumerate(ns):
        s0 = ic.fourier_state(n, ic.strict_cutoff(n / 4), seed=SEED + b, dtype=torch.float64, device=dev).float()
        ens.set_box(b, s0)
        ics.append(s0)
    ens.fill_ghosts()
    tune = ens.autotune(bg, TAU_I, DT, steps=4, repeats=1)
    init = ens.state.clone()
    sites = ens.n_sites

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    ens.advance(bg, TAU_I, 0.0, DT, 3)  # warm
    ens.state.copy_(init)
    ms_eager = timed(lambda: ens.advance(bg, TAU_I, 0.0, DT, nsteps))
    ens.device_status()
    eager_final = ens.state.clone()
    ens.state.copy_(init)
    graph = ens.capture(bg, TAU_I, 0.0, DT, nsteps, diagnostics=True)
    graph.replay()  # warm replay
    ens.state.copy_(init)
    ms_graph = timed(graph.replay)
    ens.device_status()
    same = bool(torch.equal(ens.state, eager_final))
    tau_f = TAU_I + nsteps * DT
    res = ens.results(bg, tau_f)
    # the same graph with the diagnostics' per-cell terms in FP32 (FP64 accumulation)
    del graph
    ens.state.copy_(init)
    graph = ens.capture(bg, TAU_I, 0.0, DT, nsteps, diagnostics=True, per_cell_fp32=True)
    graph.replay()
    ens.state.copy_(init)
    ms_graph32 = timed(graph.replay)
    ens.device_status()
    res32 = ens.results(bg, tau_f)
    rho_rel32 = max(abs(a.energy["rho_tot_unscreened"] / b.energy["rho_tot_unscreened"] - 1.0)
                    for a, b in zip(res32, res))
    same_np32 = all(a.n_p_plain == b.n_p_plain for a, b in zip(res32, res))
    cfg_name = dict(ens.tile_configs()).get(ens.plan.tile_config, "default")
    plan = {"tile_config": cfg_name, "z_chunk": ens.plan.z_chunk or "auto", "work_items": ens.plan.n_items,
            "grid": [ens.plan.grid_a, ens.plan.grid_b]}
    del ens, graph, init, eager_final
    torch.cuda.empty_cache()

    # the same boxes, one level at a time (same kernels, one launch per box per sweep)
    levels = []
    for b, n in enumerate(ns):
        lv = A.PeriodicLevel(n, DX, dtype=torch.float32, device=dev, pierced_capacity=1)
        lv.set_state(ics[b])
        levels.append(lv)
    for lv in levels:
        lv.advance(bg, TAU_I, 0.0, DT, 1)
    for b, lv in enumerate(levels):
        lv.set_state(ics[b])

    def per_box():
        for s in range(nsteps):
            for lv in levels:
                lv.advance(bg, TAU_I, s * DT, DT, 1)

    ms_levels = timed(per_box)
    del levels
    torch.cuda.empty_cache()
    words = 28  # compulsory words per site per RK4 step (two sweeps of 4+8 and 12+4)
    return {"config": f"{nboxes} boxes, sizes uniform from {list(sizes)}^3 (seed {SEED}), FP32, c0=1, lambda0=2, "
                      f"IC |n|<N/4 seed+box, {nsteps} RK4 steps, per-box energy + winding diagnostics",
            "sizes": {str(k): ns.count(k) for k in sizes}, "sites": sites, "steps": nsteps,
            "graph_ms": ms_graph, "graph_site_updates_per_s": sites * nsteps / (ms_graph * 1e-3),
            "eager_ms": ms_eager, "eager_site_updates_per_s": sites * nsteps / (ms_eager * 1e-3),
            "graph_equals_eager": same,
            "graph_fp32_cells_ms": ms_graph32,
            "graph_fp32_cells_site_updates_per_s": sites * nsteps / (ms_graph32 * 1e-3),
            "fp32_cells_max_rho_rel_diff": rho_rel32, "fp32_cells_same_n_p": same_np32,
            "hbm_frac_of_measured": words * 4 * sites * nsteps / (ms_eager * 1e-3) / 1e9 / hbm_peak,
            "per_box_levels_ms": ms_levels, "speedup_vs_per_box_levels": ms_levels / ms_graph,
            "plan": plan, "autotune_ms_per_step": tune,
            "launches_per_step": 2, "graph_nodes": 2 * nsteps + 3 * nboxes,
            "n_p_total": sum(r.n_p_plain for r in res),
            "per_box": [{"n": n, "n_p": r.n_p_plain, "rho_tot": r.energy["rho_tot_unscreened"],
                         "xi": r.xi_plain} for n, r in zip(ns, res)][:8]}


# ---------------------------------------------------------------- replicas (one independent box per rank)
def replica_barrier(ws: int) -> None:
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def replica_max(x: float, ws: int, device) -> float:
    """Max of a per-rank scalar (the slowest rank's time) over all ranks."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seed(rank: int) -> int:
    """Each rank evolves its own seeded realisation (weak scaling, no data exchange)."""
    return SEED + rank


# ---------------------------------------------------------------- scale configuration (two-level refinement)
def scale_report(A, dev, hbm_peak, n=512, steps=20, block=16, kdiv=64, regrid_every=10, n_error_buf=4):
    """Physical mode (c0 = 0, lambda = 2) FP32 base level of n^3 plus 2x-refined
    patches on every block^3 block the tagger flags (pierced plaquettes grown
    by n_error_buf cells), `steps` coarse steps with two subcycled fine steps
    each, regridding every `regrid_every` coarse steps. Reports throughput in
    coarse + fine site-updates/s and the composite string-finder time."""
    import torch
    from axion_strings_adaptive_gb300 import ic
    from axion_strings_adaptive_gb300.amr import TwoLevel
    torch.cuda.empty_cache()  # earlier legs' cached blocks: the patch arenas want large free ranges
    bg = A.Background.expanding(A_INV, 0.0, lambda0=LAMBDA0)
    coarse = A.PeriodicLevel(n, DX, dtype=torch.float32, device=dev, pierced_capacity=1)
    coarse.set_state(ic.fourier_state(n, ic.strict_cutoff(n / kdiv), seed=SEED + 11, dtype=torch.float64,
                                      device=dev).float())
    two = TwoLevel(coarse, block)
    tags, n_tagged, _ = coarse.tag_cells(n_error_buf=n_error_buf)
    del tags
    two.regrid(n_error_buf=n_error_buf)
    torch.cuda.synchronize()
    fine_per_patch = (2 * block) ** 3
    regrid_ms, t_ms, site_updates = [], 0.0, 0
    patches = []
    for s0 in range(0, steps, regrid_every):
        if s0 > 0:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            two.regrid(n_error_buf=n_error_buf)
            e1.record()
            torch.cuda.synchronize()
            regrid_ms.append(e0.elapsed_time(e1))
        k = min(regrid_every, steps - s0)
        np_ = 0 if two.patches is None else two.patches.npatches
        patches.append(np_)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        two.advance(bg, TAU_I, s0 * DT, DT, k)
        e1.record()
        torch.cuda.synchronize()
        t_ms += e0.elapsed_time(e1)
        site_updates += k * (n ** 3 + 2 * np_ * fine_per_patch)
    two.device_status()
    tau = TAU_I + steps * DT

    def ev_ms(fn, reps=3):
        best = float("inf")
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record()
            r = fn()
            b.record()
            torch.cuda.synchronize()
            best = min(best, a.elapsed_time(b))
        return best, r

    diag_ms, d = ev_ms(lambda: two.diagnostics(bg, tau), reps=2)  # the first call sets up scratch and masks
    diag32_ms, d32 = ev_ms(lambda: two.diagnostics(bg, tau, per_cell_fp32=True), reps=2)
    finder_ms, dstr = ev_ms(lambda: two.diagnostics(bg, tau, strings_only=True))
    # one coarse step's parts, timed apart on the final patch set (best of 3)
    import ctypes as C
    from axion_strings_adaptive_gb300 import _lib as L
    p = two.patches
    parts = {}
    if p is not None:
        # as TwoLevel.advance takes it: one step into the spare buffer (the timing
        # leaves the new state there; the fills timed next only read it)
        parts["coarse_step"] = ev_ms(lambda: coarse.step_to(two.old_state, bg, TAU_I, tau, DT))[0]
        for name, theta in (("ring_fill_theta0", 0.0), ("ring_fill_theta_half", 0.5)):
            parts[name] = ev_ms(lambda: L.call("axs_patches_fill", C.byref(p.c), C.byref(two._map()),
                                               C.byref(two.old_c), C.byref(coarse.c), theta, DT, 0, None))[0]
        parts["fine_step"] = ev_ms(lambda: p.step(bg, TAU_I, tau, 0.5 * DT))[0]
        parts["ring_cells_per_fill"] = p.npatches * ((2 * block + 12) * (2 * block + 8) ** 2 - (2 * block) ** 3)
    # per site-update as the two sweeps move them on the coarse level (ghost-ring work excluded;
    # the fused patch step moves fewer)
    fine_words = 28
    out = {"config": f"{n}^3 FP32 base, physical mode c0=0, lambda=2, IC |n|<N/{kdiv}, 2x-refined "
                     f"{2 * block}^3-cell patches on tagged {block}^3 blocks (n_error_buf={n_error_buf}), {steps} "
                     f"coarse steps with 2 subcycled fine steps each, regrid every {regrid_every}",
           "coarse_sites": n ** 3, "patches_per_regrid": patches, "refined_block_fraction":
               patches[-1] / float((n // block) ** 3), "tagged_cell_fraction_at_start": n_tagged / n ** 3,
           "ms_per_coarse_step": t_ms / steps, "site_updates_per_s": site_updates / (t_ms * 1e-3),
           "algorithmic_hbm_gbs": fine_words * 4 * site_updates / (t_ms * 1e-3) / 1e9,
           "hbm_frac_of_measured": fine_words * 4 * site_updates / (t_ms * 1e-3) / 1e9 / hbm_peak,
           "regrid_ms": regrid_ms, "composite_diagnostics_ms": diag_ms,
           "composite_diagnostics_fp32_cells_ms": diag32_ms,
           "composite_rho_tot_rel_diff_fp32_cells": abs(d32.energy["rho_tot_unscreened"] /
                                                        d.energy["rho_tot_unscreened"] - 1.0),
           "string_finder_ms": finder_ms, "coarse_step_parts_ms": parts,
           "composite": {"n_p": d.n_p_plain, "n_p_finder_only": dstr.n_p_plain, "xi": d.xi_plain,
                         "rho_tot": d.energy["rho_tot_unscreened"]}}
    del two, coarse
    torch.cuda.empty_cache()
    return out


# ---------------------------------------------------------------- native arm
def run_native(args):
    import torch
    import torch.distributed as dist

    import axion_strings_adaptive_gb300 as A
    from axion_strings_adaptive_gb300 import ic

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=dev)
    A.build()
    A.lib()
    n = args.n
    bg = A.Background.expanding(A_INV, C0, lambda0=LAMBDA0)
    ic64 = ic.fourier_state(n, ic.strict_cutoff(n / 8), seed=replica_seed(rank), dtype=torch.float64, device=dev)

    def barrier():
        replica_barrier(ws)

    def allmax(x):
        return replica_max(x, ws, dev)

    def timed_run(level, steps, warmup, t_start=0.0, sample_clocks=False):
        """K RK4 steps of `level`, CUDA events on the launching stream around every
        kernel launch. Two-sweep tilings: sweep A and sweep B each step. The fused
        step (the fused launch and the padding launch), timed in pairs of steps:
        a pair returns the state to the level's state buffer; a single step runs
        as the two sweeps, so an odd K ends with one of those. Returns (total ms,
        {kernel: mean ms per launch}, clocks)."""
        fused = "fused" in level_config_name(level)
        for w in range(warmup):
            level.advance(bg, TAU_I, t_start + w * DT, DT, 1)
        t0 = t_start + warmup * DT
        ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
        e0, e1 = ev(), ev()
        sampler = ClockSampler(local) if sample_clocks else None
        if sampler:
            sampler.start()
            time.sleep(0.3)
        marks = []
        barrier()
        torch.cuda.synchronize()
        e0.record()
        if fused:
            s = 0
            while s < steps:
                k = 2 if s + 2 <= steps else 1
                a_, b_ = ev(), ev()
                a_.record()
                level.advance(bg, TAU_I, t0 + s * DT, DT, k)
                b_.record()
                marks.append((k, a_, b_))
                s += k
        else:
            for s in range(steps):
                t = t0 + s * DT
                ea, eb, ec = ev(), ev(), ev()
                ea.record()
                level.sweep(bg, TAU_I, t, DT, 0)
                eb.record()
                level.sweep(bg, TAU_I, t, DT, 1)
                ec.record()
                marks.append((ea, eb, ec))
        e1.record()
        torch.cuda.synchronize()
        barrier()
        clocks = sampler.stop() if sampler else None
        level.device_status()
        ms = e0.elapsed_time(e1)
        if fused:
            pairs = [x.elapsed_time(y) / 2 for k, x, y in marks if k == 2]
            per = {"rk4_fused_level": sum(pairs) / len(pairs)} if pairs else \
                {"rk4_fused_level": marks[0][1].elapsed_time(marks[0][2])}
        else:
            per = {"rk4_sweep_A": sum(a_.elapsed_time(b_) for a_, b_, c_ in marks) / steps,
                   "rk4_sweep_B": sum(b_.elapsed_time(c_) for a_, b_, c_ in marks) / steps}
        return ms, per, clocks

    def level_config_name(level):
        # tile_config 0 is the table's first entry (the default tiling)
        return A._lib.lib().axs_level_tile_config_name(A._lib.AXS_F32 if level.dtype == torch.float32
                                                       else A._lib.AXS_F64, level.tile_config).decode()

    # algorithmic words per site and launch (read + write, each compulsory word once)
    WORDS = {"rk4_sweep_A": 12, "rk4_sweep_B": 16, "rk4_fused_level": 8}

    # ---------------- FP32 (headline)
    lv32 = A.PeriodicLevel(n, DX, dtype=torch.float32, device=dev, pierced_capacity=1024)
    lv32.set_state(ic64.float())
    tune32 = None
    if args.tile_config:
        ids = {name: cid for cid, name in lv32.tile_configs()}
        if args.tile_config not in ids:
            raise SystemExit(f"unknown FP32 tile configuration {args.tile_config!r}; one of {sorted(ids)}")
        lv32.tile_config = ids[args.tile_config]
    elif not args.no_autotune:
        tune32 = lv32.autotune(bg, TAU_I, DT)
    cfg32 = level_config_name(lv32)
    ms, per32, clocks = timed_run(lv32, args.steps, args.warmup, sample_clocks=True)
    ms_max = allmax(ms)
    value = ws * n ** 3 * args.steps / (ms_max * 1e-3)
    es32 = 4
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    dom, dom_ms = max(per32.items(), key=lambda kv: kv[1])
    bytes_per_launch = WORDS[dom] * es32 * n ** 3
    achieved = bytes_per_launch / (dom_ms * 1e-3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "rk4_sweep_traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            t = json.load(f)
        key = {"rk4_sweep_A": "sweep_A_bytes_per_site_f32", "rk4_sweep_B": "sweep_B_bytes_per_site_f32",
               "rk4_fused_level": "fused_level_bytes_per_site_f32"}[dom]
        if key in t:
            traffic = t[key] * n ** 3
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                "traffic": traffic, "kernel": dom, "peak_source": peak_src,
                "algorithmic_bytes_per_launch": bytes_per_launch,
                "algorithmic_words_per_site": WORDS[dom],
                "kernel_ms": per32,
                "frac_of_nominal_8TBs": achieved / 8000.0}
    launches32 = 2 * args.steps  # fused + padding, or sweep A + sweep B, per step

    # ---------------- fused diagnostics pass (string finder + energies + velocities) on the FP32 box
    diag = None
    if not args.no_diag:
        tau_d = TAU_I + (args.warmup + args.steps) * DT
        bv = bg.values(tau_d)
        import ctypes as _C
        diag = {"fields": "fp32", "read_bytes_per_cell": 16}
        for mode, fp32 in (("per_cell_fp64", 0), ("per_cell_fp32", 1)):
            params = A._lib.DiagParams(DX, bv.R, bv.lambda_, bv.R_prime_over_R, bv.m_r, A._lib.MASK_A, 0.8,
                                       A._lib.BOUNDARY_PERIODIC, 1, 1, 1, fp32)
            t_ev = []
            for r in range(3):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                A._lib.call("axs_level_diagnostics", _C.byref(lv32.c), _C.byref(params), None,
                            lv32._result.data_ptr(), lv32._pierced.data_ptr(), lv32._pierced.numel(),
                            lv32._scratch.data_ptr(), lv32._scratch.numel(), torch.cuda.current_stream().cuda_stream)
                e1.record()
                e1.synchronize()
                t_ev.append(e0.elapsed_time(e1))
            ms_d = min(t_ev)
            res = A.level._result_from_bytes(lv32._result)
            diag[mode] = {"ms": ms_d, "read_gbps": 16 * n ** 3 / (ms_d * 1e-3) / 1e9, "n_p_plain": res.n_p_plain,
                          "n_near_tie": res.n_near_tie, "rho_tot_sum": res.energy_sums[0]}
        diag["rho_tot_rel_diff"] = abs(diag["per_cell_fp32"]["rho_tot_sum"] - diag["per_cell_fp64"]["rho_tot_sum"]) / \
            abs(diag["per_cell_fp64"]["rho_tot_sum"])
        # the string finder alone (windings, counts and the whole pierced list)
        params = A._lib.DiagParams(DX, bv.R, bv.lambda_, bv.R_prime_over_R, bv.m_r, A._lib.MASK_A, 0.8,
                                   A._lib.BOUNDARY_PERIODIC, 0, 1, 0, 0)
        full_list = torch.empty(n ** 3 // 4, dtype=torch.int64, device=dev)
        t_ev = []
        for r in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            A._lib.call("axs_level_diagnostics", _C.byref(lv32.c), _C.byref(params), None,
                        lv32._result.data_ptr(), full_list.data_ptr(), full_list.numel(),
                        lv32._scratch.data_ptr(), lv32._scratch.numel(), torch.cuda.current_stream().cuda_stream)
            e1.record()
            e1.synchronize()
            t_ev.append(e0.elapsed_time(e1))
        res = A.level._result_from_bytes(lv32._result)
        diag["string_finder_only"] = {"ms": min(t_ev), "n_p_plain": res.n_p_plain, "n_listed": res.n_listed,
                                      "read_gbps": 8 * n ** 3 / (min(t_ev) * 1e-3) / 1e9}
        del full_list
        tags, n_tagged, _ = lv32.tag_cells(n_error_buf=4, block=32)
        torch.cuda.synchronize()
        t_ev = []
        for r in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            lv32.tag_cells(n_error_buf=4, block=32)
            e1.record()
            e1.synchronize()
            t_ev.append(e0.elapsed_time(e1))
        diag["tagger"] = {"ms": min(t_ev), "n_error_buf": 4, "block": 32, "tagged_fraction": n_tagged / n ** 3}
        del tags

    # ---------------- adjoint step cost on the same FP32 box (recompute sweep A + adjoint sweeps B and A)
    adj = None
    if not args.no_adjoint:
        from axion_strings_adaptive_gb300 import adjoint as ADJ
        buf = ADJ.AdjointBuffers(lv32)
        stored = lv32.state.clone()
        tau_f = TAU_I + (args.warmup + args.steps) * DT
        ADJ.loss_and_seed(lv32, buf, bg.values(tau_f).R, 0.1)
        ka = max(3, args.steps // 4)
        t_end = (args.warmup + args.steps) * DT
        for w in range(2):
            ADJ.adjoint_step(lv32, stored, buf, bg, TAU_I, t_end - (w + 1) * DT, DT)
        torch.cuda.synchronize()
        ea0, ea1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ea0.record()
        for s in range(ka):
            ADJ.adjoint_step(lv32, stored, buf, bg, TAU_I, t_end - (s + 3) * DT, DT)
        ea1.record()
        torch.cuda.synchronize()
        lv32.device_status()
        ms_adj = allmax(ea0.elapsed_time(ea1)) / ka
        fwd_ms = ms_max / args.steps
        adj = {"ms_per_step": ms_adj, "forward_ms_per_step": fwd_ms, "adjoint_over_forward": ms_adj / fwd_ms,
               "steps": ka, "dtype": "f32", "algorithmic_bytes_per_site": 48 * es32,
               "achieved_gbs": 48 * es32 * n ** 3 / (ms_adj * 1e-3) / 1e9,
               "kernels_per_step": ["rk4_sweep_A (recompute u3,u4)", "adjoint_sweep_B", "adjoint_sweep_A",
                                    "lambda_bar_finalize"],
               "finite": bool(torch.isfinite(buf.abar).all())}
        del buf, stored
        torch.cuda.empty_cache()

    # ---------------- FP64 path on the same box
    fp64 = None
    if not args.no_fp64:
        del lv32
        torch.cuda.empty_cache()
        lv64 = A.PeriodicLevel(n, DX, dtype=torch.float64, device=dev, pierced_capacity=1024)
        lv64.set_state(ic64)
        tune64 = None if args.no_autotune else lv64.autotune(bg, TAU_I, DT, steps=2, repeats=1)
        k64 = max(2, args.steps // 4)
        ms64, per64, _ = timed_run(lv64, k64, 1)
        v64 = ws * n ** 3 * k64 / (allmax(ms64) * 1e-3)
        fp64 = {"value": v64, "ms_per_step": ms64 / k64, "steps": k64, "kernel_ms": per64,
                "tile_config": level_config_name(lv64),
                "autotune_ms_per_step": tune64}
        del lv64
        torch.cuda.empty_cache()

    # ---------------- precision: FP32 vs FP64 from the same IC, plus the FP64 evolution of the
    # FP32-rounded IC (how far an FP64 run moves when its input is perturbed at FP32 roundoff:
    # the conditioning floor of each observable)
    precision = None
    if not args.no_precision and args.precision_steps > 0:
        ps = args.precision_steps
        marks = sorted({min(40, ps), ps})
        # fp64_fp32_storage: FP64 arithmetic with the state rounded to FP32 after every step
        # (FP32 storage alone, without FP32 arithmetic); fp32_compensated: the FP32 step with
        # the FP32 remainders of its constants applied (AXS_LEVEL_COMPENSATED_FP32)
        legs = (("fp64", torch.float64, ic64, False, False), ("fp32", torch.float32, ic64.float(), False, False),
                ("fp32_compensated", torch.float32, ic64.float(), False, True),
                ("fp64_rounded_ic", torch.float64, ic64.float().double(), False, False),
                ("fp64_fp32_storage", torch.float64, ic64.float().double(), True, False))
        out, step_ms = {}, {}
        for name, dt_, s0, round_state, comp in legs:
            lv = A.PeriodicLevel(n, DX, dtype=dt_, device=dev, pierced_capacity=3 * n ** 3 // 8)
            lv.compensated = comp
            lv.set_state(s0.to(dt_))
            done, t_ms = 0, 0.0
            for mk in marks:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                if round_state:
                    for s_ in range(done, mk):
                        lv.advance(bg, TAU_I, s_ * DT, DT, 1)
                        lv.state.copy_(lv.state.float())
                else:
                    lv.advance(bg, TAU_I, done * DT, DT, mk - done)
                e1.record()
                torch.cuda.synchronize()
                t_ms += e0.elapsed_time(e1)
                done = mk
                lv.device_status()
                d = lv.diagnostics(bg, TAU_I + mk * DT, want_list=True)
                out[(name, mk)] = (d, torch.sort(d.pierced.to(torch.int64))[0])
            step_ms[name] = t_ms / done
            del lv
            torch.cuda.empty_cache()

        def compare(ref, oth):
            (a, la), (b, lb) = ref, oth
            errs = {k: abs(b.energy[k] - v) / abs(v) for k, v in a.energy.items() if k.startswith("rho_") and v != 0.0}
            only_a = int((~torch.isin(la, lb)).sum())
            only_b = int((~torch.isin(lb, la)).sum())
            return {"energy_rel_err": errs, "max_energy_rel_err": max(errs.values()),
                    "total_energy_rel_err": max(errs["rho_tot_unscreened"], errs["rho_tot_screened"]),
                    "xi_rel_err": abs(b.xi_plain - a.xi_plain) / max(a.xi_plain, 1e-300),
                    "n_p": [a.n_p_plain, b.n_p_plain], "pierced_only_in_fp64": only_a,
                    "pierced_only_in_other": only_b, "n_near_tie": [a.n_near_tie, b.n_near_tie]}

        precision = {"steps": ps, "workload": f"{n}^3 Moore c0=2 lambda0=2, same IC in both precisions",
                     "by_step": {}}
        for mk in marks:
            ref = out[("fp64", mk)]
            precision["by_step"][str(mk)] = {
                "tau": TAU_I + mk * DT, "xi_fp64": ref[0].xi_plain, "n_p_fp64": ref[0].n_p_plain,
                "fp32_vs_fp64": compare(ref, out[("fp32", mk)]),
                "fp32_compensated_vs_fp64": compare(ref, out[("fp32_compensated", mk)]),
                "fp64_rounded_ic_vs_fp64": compare(ref, out[("fp64_rounded_ic", mk)]),
                "fp64_fp32_storage_vs_fp64": compare(ref, out[("fp64_fp32_storage", mk)])}
        # step times of the legs (the 400-step advance, diagnostics excluded; FP32 levels on
        # the default tiling, odd first segments on its two-sweep fallback)
        precision["ms_per_step"] = {k: step_ms[k] for k in ("fp32", "fp32_compensated", "fp64")}
        fin = precision["by_step"][str(ps)]["fp32_vs_fp64"]
        precision["total_energy_rel_err"] = fin["total_energy_rel_err"]
        precision["max_energy_rel_err"] = fin["max_energy_rel_err"]
        del out

    # ---------------- differentiation: 128^3 FP32, c0 = 1, lambda0 = 2, 200 steps, checkpoint every 20;
    # gradients w.r.t. the initial psi and lambda0 against central differences (eps = 1e-3, FP64
    # evolution) on 16 unit-norm random directions in psi, and against the FP64 adjoint
    dropin = None
    if not args.no_dropin:
        dropin = dropin_report(A, ic, dev, n=args.n)

    differentiation = None
    if not args.no_differentiation:
        differentiation = differentiation_report(A, ic, dev, args.diff_n, args.diff_steps, args.diff_directions)

    # ---------------- batching: 64 uneven boxes advanced together, one CUDA graph
    batching = None
    if not args.no_batching:
        batching = batching_report(A, ic, dev, hbm_peak)

    # ---------------- scale: base level plus refined patches on tagged blocks, subcycled
    scale = None
    if not args.no_scale:
        scale = scale_report(A, dev, hbm_peak, n=args.scale_n, steps=args.scale_steps, kdiv=args.scale_kdiv)
    # the same at the full scale configuration: a 1024^3 base and 100 coarse steps.
    # IC |n| < N/76 tags 5.2 % of the cells (91 k -> 100 k patches of 32^3 in one
    # arena laid out for 1.25 x the first count).
    scale_1024 = None
    if not args.no_scale_1024:
        try:
            scale_1024 = scale_report(A, dev, hbm_peak, n=1024, steps=args.scale1024_steps,
                                      kdiv=args.scale1024_kdiv)
        except (A._lib.AxsError, torch.OutOfMemoryError) as e:
            scale_1024 = {"unavailable": f"{type(e).__name__}: {e}"}
            torch.cuda.empty_cache()

    # ---------------- end to end through the C ABI with host buffers: every step copies its input
    # state in from pinned host memory and its result back out; the copies of neighbouring steps
    # overlap the compute (HostStepPipeline), and the serial form is reported beside it
    e2e = None
    if not args.no_e2e:
        from axion_strings_adaptive_gb300.host_pipeline import HostStepPipeline
        lv = A.PeriodicLevel(n, DX, dtype=torch.float32, device=dev, pierced_capacity=1024)
        lv.tile_config = [cid for cid, name in lv.tile_configs() if name == cfg32][0] if cfg32 != "default" else 0
        hin = [ic64.float().cpu().pin_memory(), (ic64.float() * 0.999).cpu().pin_memory()]
        hout = [torch.empty_like(hin[0]).pin_memory() for _ in range(2)]
        steps_e = max(4, args.steps)
        pipe = HostStepPipeline(lv, depth=3)

        def run(k, serial):
            for s_ in range(k):
                pipe.submit(hin[s_ % 2], hout[s_ % 2], bg, TAU_I, s_ * DT, DT, 1)
                if serial:
                    pipe.join()
                    torch.cuda.current_stream().synchronize()
            pipe.join()

        def timed_e2e(serial):
            run(2, serial)
            torch.cuda.synchronize()
            barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            run(steps_e, serial)
            e1.record()
            torch.cuda.synchronize()
            barrier()
            return allmax(e0.elapsed_time(e1))

        ems_serial = timed_e2e(True)
        ems = timed_e2e(False)
        pipe.device_status()
        nbytes = hin[0].numel() * 4
        e2e = {"value": ws * n ** 3 * steps_e / (ems * 1e-3), "unit": UNIT,
               "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
               "steps": steps_e, "ms_per_step": ems / steps_e,
               "serial_value": ws * n ** 3 * steps_e / (ems_serial * 1e-3), "serial_ms_per_step": ems_serial / steps_e,
               "link_gbs_per_direction": nbytes / (ems / steps_e * 1e-3) / 1e9,
               "path": "pinned host state -> axs_level_upload (contiguous DMA into the level's work buffer, "
                       "scatter into the level layout) -> axs_level_rk4_advance(1 step) -> axs_level_download "
                       "(gather, contiguous DMA) -> pinned host result; upload, compute and download of "
                       "neighbouring steps overlap (HostStepPipeline: 3 levels, a compute stream and an upload and "
                       "a download stream per level)"}
        del lv, pipe, hin, hout

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(args.cpu_seconds)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": _config(n), "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clocks, "gpu_launches": launches32, "tile_config": cfg32,
                "autotune_ms_per_step": tune32, "diagnostics": diag, "fp64": fp64,
                "fp32_over_fp64": (value / fp64["value"]) if fp64 else None, "precision": precision,
                "adjoint": adj, "adjoint_over_forward": adj["adjoint_over_forward"] if adj else None,
                "differentiation": differentiation, "batching": batching, "scale": scale,
                "scale_1024": scale_1024, "dropin": dropin}
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["native", "reference"], default="native")
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--ref-n", type=int, default=N_DEFAULT)
    ap.add_argument("--precision-steps", type=int, default=400)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-precision", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tile-config", default=None,
                    help="run the FP32 headline with this tile configuration (by name) instead of autotuning")
    ap.add_argument("--no-diag", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-differentiation", action="store_true")
    ap.add_argument("--no-batching", action="store_true")
    ap.add_argument("--no-dropin", action="store_true")
    ap.add_argument("--cpu-table", action="store_true", help="time the CPU oracle for the baseline table and exit")
    ap.add_argument("--no-scale", action="store_true")
    ap.add_argument("--scale-n", type=int, default=512)
    ap.add_argument("--scale-steps", type=int, default=20)
    ap.add_argument("--scale-kdiv", type=int, default=64)
    ap.add_argument("--no-scale-1024", action="store_true")
    ap.add_argument("--scale1024-steps", type=int, default=100)
    ap.add_argument("--scale1024-kdiv", type=int, default=76)
    ap.add_argument("--diff-n", type=int, default=128)
    ap.add_argument("--diff-steps", type=int, default=200)
    ap.add_argument("--diff-directions", type=int, default=16)
    args = ap.parse_args()
    if args.cpu_table:
        cpu_table()
        return
    if args.warmup < 3 and args.impl == "native":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_native(args)


if __name__ == "__main__":
    main()
