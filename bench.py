"""Benchmark: RK4 site-updates/s of the fused GB300 level step.

Workload (native arm, N=1): uniform periodic 512^3 box, Moore mode (c0 = 2),
lambda0 = 2, radiation domination (a_inv = 2), dx = 0.5, dt = 0.1, seeded
Gaussian Fourier initial data with |n| < N/8 (k < 2 pi/(8 dx)), Pi = 0;
FP32 fields (the reference's default PRECISION=FLOAT), FP64 background.
One "step" = one classic-RK4 step of the whole box (two fused sweeps).

Reported on one JSON line: whole-job site-updates/s (value), the FP64 path on
the same box, FP32-vs-FP64 energy / xi / string-count error after a short
evolution, the roofline of the dominant sweep kernel, an end-to-end number
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
WORDS_PER_SITE = {"sweep_A": 12, "sweep_B": 12}  # compulsory words per site per launch (read + write)


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
def cpu_baseline(seconds: float = 10.0, n: int = 256):
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
            "config": _config(N_DEFAULT, {"reference_sample": f"each step = one FP32 RK4 step of a {n}^3 box "
                                                              f"(bounded sample of the {N_DEFAULT}^3 workload)"}),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} FP32 RK4 steps of a {n}^3 box; CPU restatement of the "
                                       f"reference path (its AMReX build is not buildable here)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


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
    ic64 = ic.fourier_state(n, ic.strict_cutoff(n / 8), seed=SEED + rank, dtype=torch.float64, device=dev)

    def barrier():
        if ws > 1:
            dist.barrier()

    def allmax(x):
        if ws == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def timed_run(level, steps, warmup, t_start=0.0, sample_clocks=False):
        for w in range(warmup):
            level.advance(bg, TAU_I, t_start + w * DT, DT, 1)
        t0 = t_start + warmup * DT
        evA = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        evB = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        sampler = ClockSampler(local) if sample_clocks else None
        if sampler:
            sampler.start()
            time.sleep(0.3)
        barrier()
        torch.cuda.synchronize()
        e0.record()
        for s in range(steps):
            t = t0 + s * DT
            evA[s][0].record()
            level.sweep(bg, TAU_I, t, DT, 0)
            evA[s][1].record()
            evB[s][0].record()
            level.sweep(bg, TAU_I, t, DT, 1)
            evB[s][1].record()
        e1.record()
        torch.cuda.synchronize()
        barrier()
        clocks = sampler.stop() if sampler else None
        level.device_status()
        ms = e0.elapsed_time(e1)
        a = sum(x.elapsed_time(y) for x, y in evA) / steps
        b = sum(x.elapsed_time(y) for x, y in evB) / steps
        return ms, a, b, clocks

    # ---------------- FP32 (headline)
    lv32 = A.PeriodicLevel(n, DX, dtype=torch.float32, device=dev, pierced_capacity=1024)
    lv32.set_state(ic64.float())
    tune32 = None
    if not args.no_autotune:
        tune32 = lv32.autotune(bg, TAU_I, DT)
    cfg32 = dict(lv32.tile_configs())[lv32.tile_config] if lv32.tile_config else "default"
    ms, msA, msB, clocks = timed_run(lv32, args.steps, args.warmup, sample_clocks=True)
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
    dom, dom_ms = ("rk4_sweep_A", msA) if msA >= msB else ("rk4_sweep_B", msB)
    bytes_per_launch = 12 * es32 * n ** 3
    achieved = bytes_per_launch / (dom_ms * 1e-3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "rk4_sweep_traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            t = json.load(f)
        key = "sweep_A_bytes_per_site_f32" if dom.endswith("A") else "sweep_B_bytes_per_site_f32"
        if key in t:
            traffic = t[key] * n ** 3
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                "traffic": traffic, "kernel": dom, "peak_source": peak_src,
                "algorithmic_bytes_per_launch": bytes_per_launch,
                "sweep_ms": {"A": msA, "B": msB},
                "frac_of_nominal_8TBs": achieved / 8000.0}

    # ---------------- fused diagnostics pass (string finder + energies + velocities) on the FP32 box
    diag = None
    if not args.no_diag:
        t_ev = []
        tau_d = TAU_I + (args.warmup + args.steps) * DT
        bv = bg.values(tau_d)
        params = A._lib.DiagParams(DX, bv.R, bv.lambda_, bv.R_prime_over_R, bv.m_r, A._lib.MASK_A, 0.8,
                                   A._lib.BOUNDARY_PERIODIC, 1, 1, 1)
        import ctypes as _C
        for r in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            A._lib.call("axs_level_diagnostics", _C.byref(lv32.c), _C.byref(params), None, lv32._result.data_ptr(),
                        lv32._pierced.data_ptr(), lv32._pierced.numel(), lv32._scratch.data_ptr(),
                        lv32._scratch.numel(), torch.cuda.current_stream().cuda_stream)
            e1.record()
            e1.synchronize()
            t_ev.append(e0.elapsed_time(e1))
        ms_d = min(t_ev)
        res = A.level._result_from_bytes(lv32._result)
        diag = {"ms": ms_d, "read_gbps": 16 * n ** 3 / (ms_d * 1e-3) / 1e9, "n_p_plain": res.n_p_plain,
                "n_near_tie": res.n_near_tie, "fields": "fp32", "per_cell_math": "fp64"}

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
        ms64, a64, b64, _ = timed_run(lv64, k64, 1)
        v64 = ws * n ** 3 * k64 / (allmax(ms64) * 1e-3)
        fp64 = {"value": v64, "ms_per_step": ms64 / k64, "steps": k64, "sweep_ms": {"A": a64, "B": b64},
                "tile_config": dict(lv64.tile_configs())[lv64.tile_config] if lv64.tile_config else "default",
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
        legs = (("fp64", torch.float64, ic64), ("fp32", torch.float32, ic64.float()),
                ("fp64_rounded_ic", torch.float64, ic64.float().double()))
        out = {}
        for name, dt_, s0 in legs:
            lv = A.PeriodicLevel(n, DX, dtype=dt_, device=dev, pierced_capacity=3 * n ** 3 // 8)
            lv.set_state(s0.to(dt_))
            done = 0
            for mk in marks:
                lv.advance(bg, TAU_I, done * DT, DT, mk - done)
                done = mk
                lv.device_status()
                d = lv.diagnostics(bg, TAU_I + mk * DT, want_list=True)
                out[(name, mk)] = (d, torch.sort(d.pierced.to(torch.int64))[0])
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
                "fp64_rounded_ic_vs_fp64": compare(ref, out[("fp64_rounded_ic", mk)])}
        fin = precision["by_step"][str(ps)]["fp32_vs_fp64"]
        precision["total_energy_rel_err"] = fin["total_energy_rel_err"]
        precision["max_energy_rel_err"] = fin["max_energy_rel_err"]
        del out

    # ---------------- end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        lv = A.PeriodicLevel(n, DX, dtype=torch.float32, device=dev, pierced_capacity=1024)
        host = ic64.float().cpu().pin_memory()
        staging = torch.empty((4, n, n, n), dtype=torch.float32, device=dev)
        back = torch.empty_like(host).pin_memory()
        steps_e = max(3, args.steps // 2)

        def one(t):
            staging.copy_(host, non_blocking=True)
            lv.import_fab(staging, 0)
            lv.advance(bg, TAU_I, t, DT, 1)
            lv.export_fab(staging, 0)
            back.copy_(staging, non_blocking=True)

        for w in range(2):
            one(w * DT)
        torch.cuda.synchronize()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for s in range(steps_e):
            one(s * DT)
        e1.record()
        torch.cuda.synchronize()
        barrier()
        ems = allmax(e0.elapsed_time(e1))
        e2e = {"value": ws * n ** 3 * steps_e / (ems * 1e-3), "unit": UNIT,
               "h2d_bytes_per_step": host.numel() * 4, "d2h_bytes_per_step": back.numel() * 4,
               "steps": steps_e, "ms_per_step": ems / steps_e,
               "path": "pinned host state -> H2D -> axs_level_import_fab -> axs_level_rk4_advance(1 step) -> "
                       "axs_level_export_fab -> D2H"}
        del lv, staging

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(args.cpu_seconds)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": _config(n), "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clocks, "gpu_launches": 2 * args.steps, "tile_config": cfg32,
                "autotune_ms_per_step": tune32, "diagnostics": diag, "fp64": fp64,
                "fp32_over_fp64": (value / fp64["value"]) if fp64 else None, "precision": precision,
                "adjoint": adj, "adjoint_over_forward": adj["adjoint_over_forward"] if adj else None}
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
    ap.add_argument("--ref-n", type=int, default=256)
    ap.add_argument("--precision-steps", type=int, default=400)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-precision", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-diag", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "native":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_native(args)


if __name__ == "__main__":
    main()
