"""Throughput benchmark of the GB300 MIDAS hot path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload W]

One *step* solves one particle at one frequency for all its incident directions
(each direction x 2 polarisations is one "solve", the unit of the metric), with
the fill, the factorisation and the refined solves inside the step.  The JSON
line follows the repository's benchmark contract: `value` is measured with
device-resident inputs (CUDA events on the library's stream), `e2e` through the
same C ABI with host buffers (copies inside the timed region).

--impl reference times the CPU restatement of the reference algorithm (the
Fortran reference cannot be built here) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "orientation-avg solves/s vs plain FP64 MoM on same GB300 at 1e-6 rel field err"
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def workload_mom_c1():
    """Plain MoM, homogeneous sphere x = 2, m = 1.5 + 0.01i, a/d = 10 (4,224 cells,
    12,672 unknowns), +z incidence (MIDAS angles theta = phi = 90 deg), V + H."""
    from midas_gb300 import geometry as G
    a, x, m = 1.0, 2.0, 1.5 + 0.01j
    k0 = x / a
    sc = a / 10.0
    xyz = G.sphere_cells(2 * a, sc)
    return {"name": "mom_c1_sphere_x2_m1.5+0.01i_4224cells", "xyz": xyz, "sc": sc,
            "eps": np.full(len(xyz), m * m), "k0": k0, "th": np.array([90.0]), "ph": np.array([90.0]),
            "method": "mom"}


WORKLOADS = {"mom_c1": workload_mom_c1}


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [v.strip() for v in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peaks():
    try:
        with open(PEAKS_PATH) as f:
            p = json.load(f)
        return {"hbm_gbs": p["hbm_gbs"], "bf16_tflops": p["bf16_tflops"], "src": "measured"}
    except (OSError, KeyError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "src": "fallback"}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allmax(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# reference arm: CPU restatement on the host cores
# ---------------------------------------------------------------------------
def run_reference(args, wl, world, rank, pg):
    if rank != 0:
        return 0
    from oracle import oracle as O
    O.build()
    cells = O.Cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
    times = []
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        if wl["method"] == "mom":
            O.mom_solve(cells, wl["th"], wl["ph"])
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
    per = float(np.mean(times))
    value = len(wl["th"]) / per
    cores = os.cpu_count()
    sample = f"full {wl['name']} solve per step (C fills with OpenMP + LAPACK zgesv via scipy)"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128 (fp64)", "data": "synthetic",
            "config": {"workload": wl["name"], "cells": int(len(wl["xyz"])), "directions": int(len(wl["th"]))},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args, wl, world, rank, local, pg):
    import torch
    from midas_gb300 import _lib
    from midas_gb300.solver import Context

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = len(wl["xyz"])
    ntr = len(wl["th"])
    N = 3 * n
    ctx = Context(device=local)
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=dev)
    # device-resident inputs
    xyz_d = torch.from_numpy(np.ascontiguousarray(wl["xyz"].T)).to(dev)
    sc_d = torch.full((n,), wl["sc"], dtype=torch.float64, device=dev)
    er_d = torch.from_numpy(np.ascontiguousarray(wl["eps"].real)).to(dev)
    ei_d = torch.from_numpy(np.ascontiguousarray(wl["eps"].imag)).to(dev)
    th_d = torch.from_numpy(wl["th"]).to(dev)
    ph_d = torch.from_numpy(wl["ph"]).to(dev)
    E_d = torch.zeros((2 * ntr, N, 2), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    L = ctx.L

    def step_resident():
        ctx._ck(L.midas_gpu_set_cells(ctx.h, n, xyz_d[0].data_ptr(), xyz_d[1].data_ptr(), xyz_d[2].data_ptr(),
                                      sc_d.data_ptr(), er_d.data_ptr(), ei_d.data_ptr(), float(wl["k0"])))
        ctx.n = n
        ctx._ck(L.midas_gpu_mom_solve(ctx.h, ntr, th_d.data_ptr(), ph_d.data_ptr(), E_d.data_ptr(),
                                      ctypes_byref(ctx.info)))

    # host buffers for the end-to-end leg
    xs = [np.ascontiguousarray(wl["xyz"][:, i]) for i in range(3)]
    sch = np.full(n, wl["sc"])
    erh, eih = np.ascontiguousarray(wl["eps"].real), np.ascontiguousarray(wl["eps"].imag)
    Eh = np.zeros((2 * ntr, N), np.complex128)

    def step_host():
        ctx._ck(L.midas_gpu_set_cells(ctx.h, n, xs[0].ctypes.data, xs[1].ctypes.data, xs[2].ctypes.data,
                                      sch.ctypes.data, erh.ctypes.data, eih.ctypes.data, float(wl["k0"])))
        ctx.n = n
        ctx._ck(L.midas_gpu_mom_solve(ctx.h, ntr, wl["th"].ctypes.data, wl["ph"].ctypes.data, Eh.ctypes.data,
                                      ctypes_byref(ctx.info)))

    for _ in range(args.warmup):
        step_resident()
    torch.cuda.synchronize()
    barrier(pg)
    l0 = ctx.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            step_resident()
        ev1.record(stream)
        ev1.synchronize()
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    launches = ctx.launch_count() - l0
    phases = ctx.info.as_dict()
    barrier(pg)
    ms = allmax(pg, ms)
    value = world * ntr * args.steps / (ms / 1e3)
    # end-to-end through the C ABI with host buffers
    for _ in range(max(1, args.warmup // 2)):
        step_host()
    barrier(pg)
    torch.cuda.synchronize()
    ev0.record(stream)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_host()
    ev1.record(stream)
    ev1.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_s = allmax(pg, e2e_s)
    e2e_value = world * ntr * args.steps / e2e_s
    h2d = 6 * 8 * n + 2 * 8 * ntr
    d2h = 16 * N * 2 * ntr

    # roofline of the dominant kernel (largest trailing update of the LU: M x 2M x 128)
    peaks = load_peaks()
    np_ = (N + 63) // 64 * 64
    M_ = np_ - 64
    gms = ctx.bench_gemm(M_, 2 * M_, 128, iters=10)
    flops = 2.0 * M_ * (2 * M_) * 128
    algo_bytes = 4.0 * (M_ * 128 + 2 * M_ * 128 + 2 * M_ * (2 * M_))
    tf_ach = flops / (gms * 1e-3) / 1e12
    gb_ach = algo_bytes / (gms * 1e-3) / 1e9
    tf_peak = peaks["bf16_tflops"] / 2.0
    hb_peak = peaks["hbm_gbs"]
    if gb_ach / hb_peak >= tf_ach / tf_peak:
        roof = {"bound": "hbm", "achieved": gb_ach, "peak": hb_peak, "unit": "GB/s", "frac": gb_ach / hb_peak,
                "traffic": None, "kernel": f"k_gemm_tc trailing update M={M_} N={2 * M_} K=128 (fp32/tf32)",
                "peak_src": peaks["src"], "tflops": tf_ach}
    else:
        roof = {"bound": "tensor", "achieved": tf_ach, "peak": tf_peak, "unit": "TFLOP/s", "frac": tf_ach / tf_peak,
                "traffic": None, "kernel": f"k_gemm_tc trailing update M={M_} N={2 * M_} K=128",
                "peak_src": peaks["src"] + " bf16 / 2 (tf32)", "gbs": gb_ach}

    # the plain FP64 MoM on the same GPU (cuSOLVER zgetrf), the metric's denominator
    fp64 = None
    if rank == 0 and not args.no_fp64:
        c64 = Context(device=local, solve_mode=_lib.SOLVE_FP64)
        c64.set_cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
        c64.mom_solve(wl["th"], wl["ph"])
        t0 = time.perf_counter()
        E64 = c64.mom_solve(wl["th"], wl["ph"])
        t64 = time.perf_counter() - t0
        E_mixed = E_d.cpu().numpy().view(np.complex128).reshape(2 * ntr, N).T
        relerr = float(np.linalg.norm(E_mixed - E64) / np.linalg.norm(E64))
        fp64 = {"value": ntr / t64, "unit": "solves/s", "impl": "cuSOLVER zgetrf/zgetrs FP64 + FP64 fill",
                "speedup": value / (ntr / t64), "field_rel_err_vs_fp64": relerr}
        c64.close()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        cells = O.Cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
        t0 = time.perf_counter()
        O.mom_solve(cells, wl["th"], wl["ph"])
        tc = time.perf_counter() - t0
        cpu = {"value": ntr / tc, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"one full {wl['name']} solve (C restatement with OpenMP + LAPACK zgesv)"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "c64 tf32-tensor LU + f64 refinement (FP64 fill)",
                "data": "synthetic (seeded voxelised scatterer, reference voxeliser)",
                "config": {"workload": wl["name"], "cells": n, "unknowns": N, "directions": ntr,
                           "polarisations": 2, "parallelism": f"replicas x{world}",
                           "l2": "inputs larger than L2 (FP64 + FP32 impedance matrices = "
                                 f"{(16 + 8) * np_ * np_ / 1e9:.1f} GB per step)"},
                "roofline": roof, "cpu_baseline": cpu,
                "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "gpu_launches": launches, "clocks": clk.summary(), "fp64_mom_gpu": fp64,
                "phases_ms": {k: phases[k] for k in ("t_fill_ms", "t_factor_ms", "t_solve_ms", "t_total_ms")},
                "ir": {"iters": phases["ir_iters"], "backward_error": phases["backward_error"]},
                "gemm_engine": ctx.gemm_selftest()}
        print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def ctypes_byref(x):
    import ctypes
    return ctypes.byref(x)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="mom_c1", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    world, rank, local, pg = dist_setup(args)
    wl = WORKLOADS[args.workload]()
    if args.impl == "reference":
        rc = run_reference(args, wl, world, rank, pg)
    else:
        rc = run_ours(args, wl, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
