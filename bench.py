#!/usr/bin/env python3
"""Benchmark of the GB300 ADER-DG element path.

Workload (default): Kelvin-Helmholtz, 2D compressible Euler, modal Legendre
p=3 (Np_s=10), single level 256x256 on periodic [0,1]^2, seeded noise,
FP64 -- the configuration the headline metric is quoted on.  A step is one
full ADER predictor-corrector step of every element plus the device-side
time-step reduction.  Metric: DOF-updates/s = (elements * Q * Np_s) per step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm's CPU restatement (the
oracle, C++/OpenMP on all host cores) on the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "ader-dg-amr_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

WORKLOADS = {
    "kh_p3_256": dict(D=2, P=3, n=(256, 256, 1), lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), periodic=(1, 1, 1),
                      ic="kh_noise", seed=12345, noise_amp=1e-3, c_dt=0.5),
    "vortex_p1_32": dict(D=2, P=1, n=(32, 32, 1), lo=(0.0, 0.0, 0.0), hi=(10.0, 10.0, 1.0), periodic=(1, 1, 1),
                         ic="vortex", u_inf=1.0, v_inf=1.0, c_dt=0.5),
    "blast3d_p2_64": dict(D=3, P=2, n=(64, 64, 64), lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), periodic=(0, 0, 0),
                          ic="blast3d", c_dt=0.5),
}
GPU_IC = {"kh_noise": "kh_noise", "vortex": "isentropic_vortex", "blast3d": "blast3d"}
METRIC = "DOF-updates/s at 1 GB300 (single-level plain FP64 ADER-DG)"


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        try:
            rows = [l.strip().split(",") for l in open(self.path) if l.strip()]
        except Exception:
            return out
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


def make_sim(G, w, E=0):
    s = G.AmrDG(P=w["P"], D=w["D"])
    s.setGeometrySettings(prob_lo=w["lo"], prob_hi=w["hi"], n_cell=w["n"], periodic=w["periodic"])
    s.settings(c_dt=w["c_dt"], elems_per_block=E)
    extra = {k: w[k] for k in ("seed", "noise_amp", "u_inf", "v_inf") if k in w}
    s.init(G.Compressible_Euler().settings(GPU_IC[w["ic"]], **extra))
    return s


def autotune(G, w, steps=3):
    """Pick elements-per-block of the predictor by timing each variant on this
    workload; the winner is cached per (D, P, cells) next to the library."""
    cache = os.path.join(ROOT, "ader-dg-amr_gb300", "_build", "autotune.json")
    key = f"D{w['D']}P{w['P']}_n{'x'.join(map(str, w['n'][:w['D']]))}"
    try:
        db = json.load(open(cache))
    except Exception:
        db = {}
    if key in db:
        return db[key]["E"], db[key]
    choices = [8, 16, 32] if w["D"] == 2 else [4, 8, 16]
    res = {}
    for E in choices:
        s = make_sim(G, w, E)
        s.advance(2, use_graph=False)
        res[E] = s.time_kernels(steps)["predictor"]
        s.close()
    best = min(res, key=res.get)
    db[key] = {"E": best, "predictor_ms": {str(k): v for k, v in res.items()}}
    try:
        os.makedirs(os.path.dirname(cache), exist_ok=True)
        json.dump(db, open(cache, "w"), indent=1)
    except Exception:
        pass
    return best, db[key]


def cpu_baseline(w, max_seconds=20.0, threads=None):
    """The oracle (C++/OpenMP restatement of the reference) on the host cores:
    a bounded sample of the same workload (whole grid, a few steps)."""
    import oracle_ffi as O

    threads = threads or os.cpu_count()
    O.set_threads(threads)
    cfg = O.make_cfg(D=w["D"], P=w["P"], n=w["n"], lo=w["lo"], hi=w["hi"], periodic=w["periodic"],
                     ic=w["ic"], c_dt=w["c_dt"], max_grid=128,
                     **{k: w[k] for k in ("seed", "noise_amp", "u_inf", "v_inf") if k in w})
    s = O.OracleSim(cfg)
    s.init()
    s.step()  # first step (page-in, allocation) not timed
    steps, t0 = 0, time.perf_counter()
    while True:
        s.step()
        steps += 1
        el = time.perf_counter() - t0
        if el > max_seconds or steps >= 50:
            break
    from math import comb
    dof = w["n"][0] * w["n"][1] * w["n"][2] * (w["D"] + 2) * comb(w["P"] + w["D"], w["D"])
    return {"value": dof * steps / el, "unit": "DOF-updates/s", "cores": threads, "kind": "port",
            "sample": f"{steps} steps of the full {'x'.join(map(str, w['n'][:w['D']]))} grid "
                      f"({el:.1f} s), CPU oracle (reference algorithm restated in C++/OpenMP)"}


def run_reference(args, w):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    per_step = []
    base = cpu_baseline(w, max_seconds=max(5.0, 60.0 / max(1, args.steps + args.warmup)))
    val = base["value"]
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "DOF-updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, **{k: v for k, v in w.items() if k != "lo"}},
            "cpu_baseline": base,
            "e2e": {"value": val, "unit": "DOF-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    from math import comb
    dof = w["n"][0] * w["n"][1] * w["n"][2] * (w["D"] + 2) * comb(w["P"] + w["D"], w["D"])
    line["ms_per_step"] = dof / val * 1e3
    print(json.dumps(line))
    return 0


def run_ours(args, w):
    rank, world, local = dist_env()
    import adg_gb300 as G

    G.set_device(local)
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist

        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
        dist = tdist

    def barrier_max(x):
        if dist is None:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64, device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    from math import comb
    n_elem = w["n"][0] * w["n"][1] * w["n"][2]
    Q = w["D"] + 2
    Nps = comb(w["P"] + w["D"], w["D"])
    dof = n_elem * Q * Nps

    E, tune = autotune(G, w)
    s = make_sim(G, w, E)
    s.advance(max(3, args.warmup), use_graph=True)  # warm-up (includes graph capture)
    s.Dt  # sync
    n0 = s.launch_count()
    with ClockSampler(local) as clk:
        if dist is not None:
            dist.barrier()
        ms = s.advance_timed(args.steps, use_graph=True)
    launches = s.launch_count() - n0
    ms = barrier_max(ms)
    value = dof * args.steps * world / (ms * 1e-3)
    status = s.status()

    # end to end through the C ABI with host buffers: H2D of the state from
    # page-locked memory, one step, D2H of the new state, every step.
    host = G.PinnedArray((n_elem, Q, Nps))
    host.array[:] = s.get_U_w()
    e2e_steps = max(5, min(args.steps, 50))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        s.set_U_w(host.array)
        s.time_integration()
        host.array[:] = s.get_U_w()
    e2e_s = barrier_max(time.perf_counter() - t0)
    e2e_val = dof * e2e_steps * world / e2e_s
    host.free()

    # roofline of the dominant kernel (predictor: Picard sweeps, corrector
    # volume term and face traces), CUDA events on the context's stream
    km = s.time_kernels(5)
    alg, issued = G.flops_per_element(w["D"], w["P"])
    Np_st = comb(w["P"] + w["D"] + 1, w["D"] + 1)
    qbd = (w["P"] + 1) ** w["D"]
    # algorithmic flops of the predictor kernel: the method's count minus the
    # corrector's face terms (2Q * 2D * Np_s * qMp_st_bd, done in k_corrector)
    alg_pred = alg - 2 * Q * 2 * w["D"] * Nps * qbd
    peak = G.fp64_peak_gflops() / 1e3  # TFLOP/s, measured now on this GPU
    achieved = alg_pred * n_elem / (km["predictor"] * 1e-3) / 1e12
    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": "DOF-updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "D": w["D"], "P": w["P"], "cells": list(w["n"][:w["D"]]),
                   "ic": w["ic"], "c_dt": w["c_dt"], "parallelism": "replicas" if world > 1 else "1 GPU",
                   "elems_per_block": E, "cuda_graph": True,
                   "l2": "working set per step (state, traces, face fluxes) exceeds the 129 MB L2"},
        "e2e": {"value": e2e_val, "unit": "DOF-updates/s", "h2d_bytes_per_step": dof * 8,
                "d2h_bytes_per_step": dof * 8},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": None,
                     "kernel": "k_predictor", "kernel_ms": km["predictor"],
                     "algorithmic_flops_per_element": alg_pred,
                     "issued_linear_fp64_per_element": issued,
                     "peak_source": "DFMA-chain probe on this GPU in this run (MEASURED_PEAKS.json has no FP64 figure)"},
        "kernel_ms": km,
        "gpu_launches": launches,
        "clocks": clocks,
        "status": status,
    }
    if rank == 0:
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(w, max_seconds=args.cpu_seconds)
        print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="kh_p3_256", choices=list(WORKLOADS))
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, w)
    return run_ours(args, w)


if __name__ == "__main__":
    sys.exit(main())
