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


from midas_gb300.workloads import WORKLOADS, mom_c1 as workload_mom_c1  # noqa: E402


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


# ncu counters of the kernel that leads the CBFM step: ncu --set full --clock-control none
# of the double-float CSR residual on the 15k-unknown extended block of the Gaussian sphere
# at a/d = 16 (113 M nonzeros, 380 right-hand sides, one lane: the regime of the benchmark
# scene's largest blocks).  Traffic is dram__bytes_read.sum + dram__bytes_write.sum per
# algorithmic byte of the launch (3.94 GB measured against 1.00 GB algorithmic: X rows come
# back from DRAM while the CSR values stream through L2).
NCU_COUNTERS = {
    "resid": {"kernel": "k_resid_csr_df32", "issue_active_pct": 79.4, "fma_pipe_pct": 71.3, "dram_pct": 0.85,
              "l2_hit_pct": 99.1, "instructions_per_complex_mac": 49, "note": "FP32-issue bound (double-float "
              "arithmetic on the CUDA cores: 44 FP32 operations per complex multiply-add, 32 FADD + 8 FFMA + 4 FMUL "
              "by the opcode counters, 90 % of the issued instructions); X rows served by L2"},
}
NCU_TRAFFIC_PER_ALG_BYTE = {"resid": 3.94}

# The CPU baseline of the CBFM scene is a bounded sample scaled to the full solve
# by each phase's order.  Full oracle solves of the same 40,992-cell scene check
# that model: (machine, cores, full solve measured, the model's prediction there).
CPU_MODEL_CHECKS = {
    "cbfm": [{"machine": "x86_64", "cores": 8, "full_solve_s": 827.9, "model_s": 826.1},
             {"machine": "aarch64", "cores": 16, "full_solve_s": 784.3, "model_s": 508.5,
              "note": "GB300 box host (Grace); the full solve shared the host with GPU jobs for part of its run, "
                      "the model is the benchmark's own sample on an idle host"}],
}


def cpu_model_calibration(method):
    """Full-solve / model ratio measured on this machine's architecture (1 when unknown)."""
    import platform
    for chk in CPU_MODEL_CHECKS.get(method, []):
        if chk["machine"] == platform.machine():
            return chk["full_solve_s"] / chk["model_s"], chk
    return 1.0, None


# The plain FP64 MoM (FP64 fill + cuSOLVER zgetrf / zgetrs) measured on GB300 at the
# largest size that fits a benchmark call: the 60,000-unknown inhomogeneous cube with
# 64 right-hand sides (bench.py --workload mom_c3 --fp64-measure).  Larger systems
# are scaled from this point: factorisation by N^3, fill by N^2.
FP64_MEASURED = {"workload": "mom_c3 (20,000 voxels, 60,000 unknowns, 64 right-hand sides)", "unknowns": 60000,
                 "seconds": 528.88, "fill_ms": 187.4, "factor_ms": 528688.4,
                 "mixed_solves_per_s_same_matrix": 31.42, "field_rel_err_mixed_vs_fp64": 3.6e-9}


def peaks_clock_mhz():
    """SM clock of the peak measurements (MEASURED_PEAKS.json), else GB300's maximum."""
    try:
        with open(PEAKS_PATH) as f:
            return float(json.load(f).get("sm_max_mhz", 2070.0))
    except (OSError, ValueError):
        return 2070.0


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
def cbfm_cpu_sample(wl):
    """Bounded CPU sample of the CBFM workload, extrapolated per phase.

    Times the oracle on (a) the CBF generation of the median-size extended block
    (SR threshold scan + thresholded fill, then the dense FP64 solve + SVD that
    stand in for PARDISO + GESVD), (b) the reduced-matrix assembly of one
    median-size block pair (FP64 fill + the two ZGEMMs) and (c) a reduced solve of
    the extrapolated K_total.  Each phase is scaled to the whole partition by its
    own order: block fills by s_b^2, block solves by s_b^3, pair fills by n_i n_j,
    pair products by n_i n_j K.  Returns (modelled seconds of the full solve, wall
    seconds of the sample, description).  The model is checked against full oracle
    runs of the same scene (CPU_MODEL_CHECKS)."""
    from oracle import oracle as O
    import scipy.linalg as sla
    O.build()
    cells = O.Cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
    offs = np.asarray(wl["offs"])
    nbk = np.diff(offs).astype(float)
    s = nbk + np.array([len(e) for e in wl["ext"]], float)
    part = O.Partition(offs, wl["ext"])
    b = int(np.argsort(s)[len(s) // 2])
    idx = part.extended(b)
    homog = int(wl.get("homog", 0))
    thr = O.cbf_threshold(cells)
    t0 = time.perf_counter()
    Eref = O.incident_c4(cells, wl["cth"], wl["cph"], idx=idx)
    fsr, _ = O.set_fsr(cells, idx, homog, O.RES_SR_DEFAULT)
    Zb = O.sr_dense(cells, idx, fsr, homog)[0]
    t1 = time.perf_counter()
    Ep = O._solve(Zb, Eref)
    U, S, _ = np.linalg.svd(Ep, full_matrices=False)
    K = int(np.count_nonzero(S / S[0] >= thr))
    t2 = time.perf_counter()
    del Zb
    order = np.argsort(nbk)
    i, j = int(order[len(order) // 2]), int(order[len(order) // 2 + 1])
    rng = np.random.default_rng(0)
    t3 = time.perf_counter()
    Zij = O.green_partial(cells, part.block(i), part.block(j))
    t4 = time.perf_counter()
    Ci = rng.standard_normal((Zij.shape[0], K)) + 1j * rng.standard_normal((Zij.shape[0], K))
    Cj = rng.standard_normal((Zij.shape[1], K)) + 1j * rng.standard_normal((Zij.shape[1], K))
    t4b = time.perf_counter()
    Zc_ij = (Ci.T @ Zij) @ Cj
    t5 = time.perf_counter()
    nblocks = len(nbk)
    kt = K * nblocks
    A = rng.standard_normal((kt, kt)) + 1j * rng.standard_normal((kt, kt))
    B = rng.standard_normal((kt, 2 * len(wl["th"]))) + 0j
    t6 = time.perf_counter()
    sla.solve(A, B, check_finite=False)
    t7 = time.perf_counter()
    del Zc_ij
    sb = s[b]
    pair = np.outer(nbk, nbk)
    scale_fill_b = float(np.sum((s / sb) ** 2))
    scale_solve_b = float(np.sum((s / sb) ** 3))
    scale_pair = float(pair.sum() / (nbk[i] * nbk[j]))
    T = ((t1 - t0) * scale_fill_b + (t2 - t1) * scale_solve_b + (t4 - t3) * scale_pair + (t5 - t4b) * scale_pair
         + (t7 - t6))
    wall = t7 - t0
    desc = (f"oracle (C + OpenMP fills, LAPACK via scipy) on block {b} (extended {int(sb)} cells, K={K}), pair "
            f"({i},{j}) and a {kt}-unknown reduced solve; {t2 - t0 + t4 - t3 + t5 - t4b + t7 - t6:.1f} s "
            f"measured, extrapolated x{scale_fill_b:.1f} (block fills, s^2), x{scale_solve_b:.1f} (block solves, "
            f"s^3), x{scale_pair:.0f} (pair fills and products, n_i n_j) to all {nblocks} blocks")
    return T, wall, desc


def mom_cpu_sample(wl, cells_sample=3000):
    """Bounded CPU sample of a large MoM solve: the oracle's FP64 fill and LAPACK solve
    on the first `cells_sample` cells, scaled to the full size by order (fill N^2,
    solve N^3).  Returns (seconds per step, description)."""
    from oracle import oracle as O
    import scipy.linalg as sla
    O.build()
    ns = min(cells_sample, len(wl["xyz"]))
    cells = O.Cells(wl["xyz"][:ns], wl["sc"], wl["eps"][:ns], wl["k0"])
    t0 = time.perf_counter()
    Z = O.mom_fill(cells)
    V = O.mom_rhs(cells, wl["th"], wl["ph"])
    t1 = time.perf_counter()
    sla.solve(Z, V, check_finite=False)
    t2 = time.perf_counter()
    r = len(wl["xyz"]) / ns
    T = (t1 - t0) * r ** 2 + (t2 - t1) * r ** 3
    desc = (f"oracle FP64 fill + LAPACK zgesv on the first {ns} cells ({3 * ns} unknowns): {t2 - t0:.1f} s measured, "
            f"fill x{r ** 2:.0f} (N^2) and solve x{r ** 3:.0f} (N^3) to {len(wl['xyz'])} cells")
    return T, t2 - t0, desc


def run_reference(args, wl, world, rank, pg):
    if rank != 0:
        return 0
    from oracle import oracle as O
    O.build()
    model, walls = [], []
    desc = None
    if wl["method"] == "batch":
        from midas_gb300.workloads import c4_instance
        c4cells = [c4_instance(wl, k) for k in range(len(wl["n_mono"]))]
        for it in range(args.warmup + args.steps):
            dt, tw, desc = c4_cpu_sample(wl, c4cells)
            if it >= args.warmup:
                model.append(dt / len(c4cells))   # per instance: the value below counts all instances
                walls.append(tw)
        wl = dict(wl, xyz=np.zeros((sum(len(x) for x, _ in c4cells), 3)))
    cells = None if wl["method"] == "batch" else O.Cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
    for it in range(0 if wl["method"] == "batch" else args.warmup + args.steps):
        t0 = time.perf_counter()
        if wl["method"] == "mom" and 3 * len(wl["xyz"]) > 20000:
            dt, _, desc = mom_cpu_sample(wl)
        elif wl["method"] == "mom":
            O.mom_solve(cells, wl["th"], wl["ph"])
            dt = time.perf_counter() - t0
        else:
            dt, _, desc = cbfm_cpu_sample(wl)
        if it >= args.warmup:
            model.append(dt)
            walls.append(time.perf_counter() - t0)
    per = float(np.mean(model))
    cal, chk = cpu_model_calibration("cbfm") if wl["method"] == "cbfm" else (1.0, None)
    per *= cal
    value = len(wl["th"]) / per
    wall = float(np.mean(walls))
    cores = os.cpu_count()
    sample = desc or f"full {wl['name']} solve per step (C fills with OpenMP + LAPACK zgesv via scipy)"
    # ms_per_step is the wall time of each step as run (the bounded sample); value is the
    # full solve's throughput the sample models (checked against full oracle runs)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128 (fp64)", "data": "synthetic",
            "config": {"workload": wl["name"], "cells": int(len(wl["xyz"])), "directions": int(len(wl["th"]))},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port", "sample": sample,
                             "modelled_full_solve_s": per, "calibration": cal, "calibrated_by": chk,
                             "sample_wall_s": wall},
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
    # FAST fill: dyads from the per-lattice-offset tables (voxel scatterers sit on one lattice)
    ctx = Context(device=local, fill_mode=_lib.FILL_FAST, ir_tol=wl.get("ir_tol", 1e-13))
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

    cbfm = wl["method"] == "cbfm"
    if cbfm:
        from midas_gb300 import _lib as LB
        from midas_gb300.workloads import cbfm_args
        bo, eo, ei = cbfm_args(wl)
        cth, cph = np.ascontiguousarray(wl["cth"]), np.ascontiguousarray(wl["cph"])
        flags = LB.CBFM_SR | (LB.CBFM_HOMOG if wl.get("homog") else 0) | (LB.CBFM_ACA if wl.get("aca") else 0)
        Kb = np.zeros(len(bo) - 1, np.int32)

    def solve(thp, php, Ep):
        if cbfm:
            ctx._ck(L.midas_gpu_cbfm_solve(ctx.h, len(bo) - 1, bo.ctypes.data, eo.ctypes.data, ei.ctypes.data,
                                           len(cth), cth.ctypes.data, cph.ctypes.data, 0.0, 0.0, flags,
                                           float(np.float32(1e-4)), 50, ntr, thp, php, Ep, Kb.ctypes.data,
                                           ctypes_byref(ctx.info)))
        else:
            ctx._ck(L.midas_gpu_mom_solve(ctx.h, ntr, thp, php, Ep, ctypes_byref(ctx.info)))

    def step_resident():
        ctx._ck(L.midas_gpu_set_cells(ctx.h, n, xyz_d[0].data_ptr(), xyz_d[1].data_ptr(), xyz_d[2].data_ptr(),
                                      sc_d.data_ptr(), er_d.data_ptr(), ei_d.data_ptr(), float(wl["k0"])))
        ctx.n = n
        solve(th_d.data_ptr(), ph_d.data_ptr(), E_d.data_ptr())

    # host buffers for the end-to-end leg, page-locked (pinned) so that the copies run
    # at the host link's DMA rate
    pinned_keep = []

    def pinned(a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        t = torch.empty(a.shape, dtype={np.float64: torch.float64, np.complex128: torch.complex128}[dtype],
                        pin_memory=True)
        v = t.numpy()
        v[...] = a
        pinned_keep.append(t)
        return v

    xs = [pinned(wl["xyz"][:, i], np.float64) for i in range(3)]
    sch = pinned(np.full(n, wl["sc"]), np.float64)
    erh, eih = pinned(wl["eps"].real, np.float64), pinned(wl["eps"].imag, np.float64)
    thh, phh = pinned(wl["th"], np.float64), pinned(wl["ph"], np.float64)
    Eh = pinned(np.zeros((2 * ntr, N)), np.complex128)

    def step_host():
        ctx._ck(L.midas_gpu_set_cells(ctx.h, n, xs[0].ctypes.data, xs[1].ctypes.data, xs[2].ctypes.data,
                                      sch.ctypes.data, erh.ctypes.data, eih.ctypes.data, float(wl["k0"])))
        ctx.n = n
        solve(thh.ctypes.data, phh.ctypes.data, Eh.ctypes.data)

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
    # up to three of the steps again with per-kernel-class CUDA events around every
    # launch (a second timed region: the events themselves cost a few % of the step)
    nprof = min(args.steps, 3)
    ctx.profile(True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(nprof):
        step_resident()
    ev1.record(stream)
    ev1.synchronize()
    ms_prof = ev0.elapsed_time(ev1)
    kprof = ctx.profile_query()
    ctx.profile(False)
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
    if cbfm:
        h2d += 4 * (bo.size + eo.size + ei.size) + 8 * (cth.size + cph.size)
    d2h = 16 * N * 2 * ntr + (4 * Kb.size if cbfm else 0)

    # Roofline of the largest kernel class of the step (CUDA events per launch in the
    # profiled pass): achieved = the class's algorithmic bytes (or flops) / its device
    # time, against the measured copy bandwidth or the measured dense-GEMM rate.
    # Classes on the CUDA cores (residuals, triangular applies, diagonal LUs, the
    # eigensolver) are reported against the HBM roof with their algorithmic bytes:
    # they are issue- or latency-bound, so their fraction is low by construction,
    # and the ncu counters of the same kernel say how busy the issue slots are.
    peaks = load_peaks()
    hb_peak = peaks["hbm_gbs"]
    # The roofline kernel is the class that holds the most SM-time: its device time
    # (one lane, so each event interval covers one kernel) times the fraction of the
    # SMs its launches occupy.  The diagonal-block LUs run one CTA per launch and the
    # eigensolver one CTA per block, so their long device times hold one SM each; every
    # other class fills the GPU.
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    sm_share = {"diag_lu": 1.0 / nsm, "eig": min(1.0, (len(bo) - 1 if cbfm else 1) / nsm)}
    top = max(kprof, key=lambda k: kprof[k]["ms"] * sm_share.get(k, 1.0))
    kp = kprof[top]
    sec = kp["ms"] * 1e-3
    gb_ach = kp["bytes"] / sec / 1e9 if sec > 0 else 0.0
    tf_ach = kp["flops"] / sec / 1e12 if sec > 0 else 0.0
    # the LU trailing update runs kind::f16 MMAs (the bf16 / fp16 rate); the other GEMM
    # classes are kind::tf32 (half of it)
    f16_class = top == "gemm_trail"
    tf_peak = peaks["bf16_tflops"] if f16_class else peaks["bf16_tflops"] / 2.0
    ridge = tf_peak * 1e12 / (hb_peak * 1e9)
    ai = kp["flops"] / kp["bytes"] if kp["bytes"] > 0 else float("inf")
    if top.startswith("gemm_") and ai >= ridge:
        roof = {"bound": "tensor", "achieved": tf_ach, "peak": tf_peak, "unit": "TFLOP/s", "frac": tf_ach / tf_peak,
                "peak_src": peaks["src"] + (" bf16_tflops (fp16 rate)" if f16_class else " bf16_tflops / 2 (tf32 rate)")}
    else:
        roof = {"bound": "hbm", "achieved": gb_ach, "peak": hb_peak, "unit": "GB/s", "frac": gb_ach / hb_peak,
                "peak_src": peaks["src"] + " hbm_gbs"}
    roof.update({"selection": "largest SM-time class (device time x share of the SMs its launches occupy)",
                 "traffic": NCU_TRAFFIC_PER_ALG_BYTE.get(top, None) and
                 NCU_TRAFFIC_PER_ALG_BYTE[top] * kp["bytes"] / max(1, kp["launches"]),
                 "kernel_class": top, "launches": kp["launches"],
                 "ms_per_launch": kp["ms"] / max(1, kp["launches"]),
                 "algorithmic_bytes_per_launch": kp["bytes"] / max(1, kp["launches"]),
                 "algorithmic_flops_per_launch": kp["flops"] / max(1, kp["launches"]),
                 "share_of_step": kp["ms"] / ms_prof if ms_prof > 0 else None, "tflops": tf_ach, "gbs": gb_ach,
                 "profiled_ms_per_step": ms_prof / nprof, "ncu": NCU_COUNTERS.get(top)})
    if top == "diag_lu":
        roof["note"] = ("the 64 x 64 diagonal-block LUs and their inverses: one CTA per block (1 of 152 SMs), "
                        "128 barrier-separated pivot phases -- latency-bound; in the timed seven-lane step their "
                        "launches overlap the other lanes' throughput-bound kernels")
    if top == "resid":
        # The double-float CSR residual is bound by FP32 instruction issue, not by HBM: its
        # arithmetic is 44 FP32 operations per complex multiply-add (four TwoProduct +
        # TwoSum updates), against one FP32 operation per lane per clock on every SM.
        props = torch.cuda.get_device_properties(local)
        mhz = clk.summary().get("sm_mhz") or peaks_clock_mhz()
        peak_ops = props.multi_processor_count * 128 * mhz * 1e6
        ops = kp["flops"] / 8.0 * 44.0 / sec if sec > 0 else 0.0
        roof["fp32_issue"] = {"achieved_ops_per_s": ops, "peak_ops_per_s": peak_ops, "frac": ops / peak_ops,
                              "ops_per_complex_mac": 44, "sm_mhz": mhz,
                              "peak_src": f"{props.multi_processor_count} SMs x 128 FP32 lanes x SM clock"}
    classes = {k: {"ms_per_step": v["ms"] / nprof, "launches_per_step": v["launches"] / nprof,
                   "gbs": v["bytes"] / (v["ms"] * 1e-3) / 1e9 if v["ms"] > 0 else None,
                   "tflops": v["flops"] / (v["ms"] * 1e-3) / 1e12 if v["ms"] > 0 else None}
               for k, v in kprof.items()}

    # the plain FP64 MoM on the same GPU (cuSOLVER zgetrf), the metric's denominator
    fp64 = None
    if rank == 0 and not args.no_fp64:
        if cbfm or (N > 20000 and not args.fp64_measure):
            # a full-size FP64 LU takes minutes (60k unknowns) to hours (123k unknowns)
            fp64 = fp64_mom_extrapolated(local, wl, value)
        else:
            c64 = Context(device=local, solve_mode=_lib.SOLVE_FP64)
            c64.set_cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
            if N <= 20000:
                c64.mom_solve(wl["th"], wl["ph"])   # warm-up (cuSOLVER workspace, module load)
            t0 = time.perf_counter()
            E64 = c64.mom_solve(wl["th"], wl["ph"])
            t64 = time.perf_counter() - t0
            inf64 = c64.info.as_dict()
            E_mixed = E_d.cpu().numpy().view(np.complex128).reshape(2 * ntr, N).T
            relerr = float(np.linalg.norm(E_mixed - E64) / np.linalg.norm(E64))
            fp64 = {"value": ntr / t64, "unit": "solves/s", "impl": "cuSOLVER zgetrf/zgetrs FP64 + FP64 fill",
                    "measured": True, "seconds": t64, "fill_ms": inf64["t_fill_ms"],
                    "factor_ms": inf64["t_factor_ms"], "speedup": value / (ntr / t64),
                    "field_rel_err_vs_fp64": relerr}
            c64.close()
    # the CBFM method against the dense MoM answer on a scene both solve: the metric's
    # "1e-6 rel field err" is parity with the reference's CBFM (the parity key); the
    # CBFM method itself approximates the MoM field to this error
    method_err = None
    if rank == 0 and cbfm and not args.no_fp64:
        method_err = cbfm_vs_mom(local)

    # the answer of the timed steps against the oracle's fixture of the same scene
    # (tests/golden/cfg_*.npz), outside the timed regions
    parity = None
    fx_name = {"cbfm_c2": "c2", "mom_c1": "c1", "mom_tiny": "c1_lit"}.get(args.workload)
    if rank == 0 and fx_name:
        parity = check_parity(ctx, wl, fx_name, E_d.cpu().numpy().view(np.complex128).reshape(2 * ntr, N).T,
                              Kb if cbfm else None)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        if cbfm:
            tc, tw, desc = cbfm_cpu_sample(wl)
            cal, chk = cpu_model_calibration("cbfm")
            cpu = {"value": ntr / (tc * cal), "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": desc, "modelled_full_solve_s": tc, "calibration": cal, "calibrated_by": chk,
                   "sample_wall_s": tw}
        elif N > 20000:
            tc, tw, desc = mom_cpu_sample(wl)
            cpu = {"value": ntr / tc, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port", "sample": desc,
                   "modelled_full_solve_s": tc, "sample_wall_s": tw}
        else:
            from oracle import oracle as O
            O.build()
            cells = O.Cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
            t0 = time.perf_counter()
            O.mom_solve(cells, wl["th"], wl["ph"])
            tc = time.perf_counter() - t0
            cpu = {"value": ntr / tc, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"one full {wl['name']} solve (C restatement with OpenMP + LAPACK zgesv)"}

    if rank == 0:
        cfg = {"workload": wl["name"], "cells": n, "unknowns": N, "directions": ntr, "polarisations": 2,
               "parallelism": f"replicas x{world}", "ir_tol": wl.get("ir_tol", 1e-13)}
        if cbfm:
            cfg.update({"blocks": len(bo) - 1, "cbf_excitations": int(2 * len(cth)), "K_total": int(Kb.sum()),
                        "K_min_max": [int(Kb.min()), int(Kb.max())], "flags": flags,
                        "l2": "inputs larger than L2 (per-block LU operands and reduced-matrix block columns of "
                              "several GB each step)"})
            dtype = "c64 tf32-tensor block LU + double-float refinement; split-tf32 reduced products; f64 reduced solve"
        else:
            np_ = (N + 63) // 64 * 64
            cfg["l2"] = ("inputs larger than L2 (FP64 + FP32 impedance matrices = "
                         f"{(16 + 8) * np_ * np_ / 1e9:.1f} GB per step)")
            dtype = "c64 tf32-tensor LU + f64 refinement (FP64 fill)"
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": dtype,
                "data": "synthetic (seeded voxelised scatterer)",
                "config": cfg, "roofline": roof, "cpu_baseline": cpu, "parity": parity,
                "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "gpu_launches": launches, "clocks": clk.summary(), "fp64_mom_gpu": fp64,
                "cbfm_vs_mom_field_err": method_err,
                "phases_ms": {k: phases[k] for k in ("t_fill_ms", "t_factor_ms", "t_solve_ms", "t_total_ms")},
                "kernel_classes": classes,
                "ir": {"iters": phases["ir_iters"], "backward_error": phases["backward_error"]},
                "gemm_engine": ctx.gemm_selftest()}
        print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def cbfm_vs_mom(local):
    """Relative L2 difference of the CBFM field and the MoM field (mixed solve
    refined to a 1e-13 backward error, i.e. the FP64 answer) on the benchmark
    scene's generator at a/d = 12 (7.6k cells, 22.8k unknowns), where both run."""
    from midas_gb300 import _lib
    from midas_gb300.solver import Context
    from midas_gb300.workloads import cbfm_c2_small
    wl = cbfm_c2_small()
    ctx = Context(device=local, fill_mode=_lib.FILL_FAST).set_cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
    Ec, _ = ctx.cbfm_solve(wl["offs"], wl["ext"], wl["cth"], wl["cph"], wl["th"], wl["ph"],
                           flags=_lib.CBFM_SR | (_lib.CBFM_HOMOG if wl.get("homog") else 0))
    Em = ctx.mom_solve(wl["th"], wl["ph"])
    berr = ctx.info.backward_error
    ctx.close()
    return {"scene": wl["name"], "cells": int(len(wl["xyz"])), "rel_l2": float(np.linalg.norm(Ec - Em) /
                                                                               np.linalg.norm(Em)),
            "mom_backward_error": berr}


def check_parity(ctx, wl, fx_name, E, K):
    """Compare a solved scene with the oracle's fixture: internal field (seeded row
    subset and column norms) <= 1e-6, Cext / Cabs <= 1e-6, S <= 1e-5 of max |S|,
    K per block identical.  E: (N, 2 ntr) complex."""
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import cfg_digest as D
    path = D.fixture_path(fx_name)
    if not os.path.exists(path):
        return {"fixture": os.path.relpath(path, ROOT), "ok": False, "error": "fixture missing"}
    fx = np.load(path)
    rx = "polar181" if fx_name.startswith("c1") else "grid37x2"
    ce, ca = ctx.cext_cabs(wl["th"], wl["ph"], E)
    S = ctx.smatrix(*D.receivers(rx), E)
    res = D.compare(fx, E, ce, ca, S, K)
    scene_ok = bool(np.array_equal(D.scene_signature(wl), fx["signature"]))
    ok = (scene_ok and res["E_rows_rel"] <= 1e-6 and res["colnorm_rel"] <= 1e-6 and res["cext_rel"] <= 1e-6
          and res["cabs_rel"] <= 1e-6 and res["S_rel"] <= 1e-5 and res.get("K_equal", True))
    return {"fixture": os.path.relpath(path, ROOT), "scene_matches": scene_ok, **res,
            "tolerances": {"E": 1e-6, "cext_cabs": 1e-6, "S": 1e-5}, "oracle_seconds": float(fx["seconds"]),
            "ok": bool(ok)}


def c4_cpu_sample(wl, cells):
    """Bounded CPU sample of the C4 batch: the oracle pipeline (C fill, LAPACK
    zgesv, S matrix, cross sections, list-rule averages) on the smallest and a
    median instance; per-instance time modelled as a N^2 + b N^3 (fill and
    averaging; the dense solve) through those two points and summed over all
    instances.  Returns (modelled seconds of the batch, sample wall seconds,
    description)."""
    from oracle import oracle as O
    O.build()
    th, ph, rth, rph = wl["th"], wl["ph"], wl["rx_th"], wl["rx_ph"]
    ntr = len(th)
    sizes = np.array([3 * len(x) for x, _ in cells], float)
    order = np.argsort(sizes)
    pick = [int(order[0]), int(order[len(order) // 2])]
    pts = []
    t_all = time.perf_counter()
    for k in pick:
        xyz, d = cells[k]
        c = O.Cells(xyz, d, wl["m"] ** 2, wl["k0"])
        t0 = time.perf_counter()
        r = O.mom_solve(c, th, ph, rth, rph)
        dm = 2.0 * (3.0 * len(xyz) * d ** 3 / (4.0 * math.pi)) ** (1.0 / 3.0)
        O.scattering_quantities("rf", "rf", (ntr, 1), (wl["nrx"], 1), th, ph, rth, rph, r["S"], r["cext"], r["cabs"],
                                dm, wl["k0"])
        pts.append((sizes[k], time.perf_counter() - t0))
    wall = time.perf_counter() - t_all
    (n0, t0), (n1, t1) = pts
    A = np.array([[n0 ** 2, n0 ** 3], [n1 ** 2, n1 ** 3]])
    a, b = np.linalg.solve(A, np.array([t0, t1]))
    a, b = max(a, 0.0), max(b, 0.0)
    T = float(np.sum(a * sizes ** 2 + b * sizes ** 3))
    desc = (f"oracle pipeline on instances of {int(n0)} and {int(n1)} unknowns ({t0:.2f} s, {t1:.2f} s), "
            f"per-instance time a N^2 + b N^3 through them, summed over all {len(sizes)} instances "
            f"({int(sizes.min())}-{int(sizes.max())} unknowns)")
    return T, wall, desc


def run_batch_bench(args, wl, world, rank, local, pg):
    """C4 line: all instances per step on concurrent lanes (contexts), through the
    library's public entry points.  The per-instance inputs (cell lists of at most
    a few hundred kB) are host arrays, so `value` already includes their copies;
    `e2e` is the same measurement."""
    import torch
    from midas_gb300 import _lib
    from midas_gb300.solver import Context
    from midas_gb300.workloads import batch_step, c4_instance
    torch.cuda.set_device(local)
    cells = [c4_instance(wl, k) for k in range(len(wl["n_mono"]))]
    ntr, n = len(wl["th"]), len(cells)
    ctx = Context(device=local, fill_mode=_lib.FILL_FAST, ir_tol=wl.get("ir_tol", 1e-13))
    contexts = [ctx] + [ctx.sibling() for _ in range(args.lanes - 1)]
    for _ in range(args.warmup):
        batch_step(contexts, wl, cells)
    torch.cuda.synchronize()
    barrier(pg)
    l0 = sum(c.launch_count() for c in contexts)
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            res = batch_step(contexts, wl, cells)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
    launches = sum(c.launch_count() for c in contexts) - l0
    dt = allmax(pg, dt)
    value = world * ntr * n * args.steps / dt
    # one more step with per-kernel-class CUDA events on every lane
    for c in contexts:
        c.profile(True)
    tp = time.perf_counter()
    batch_step(contexts, wl, cells)
    tp = time.perf_counter() - tp
    kprof = {}
    for c in contexts:
        for k, v in c.profile_query().items():
            e = kprof.setdefault(k, {"ms": 0.0, "flops": 0.0, "bytes": 0.0, "launches": 0})
            for f in e:
                e[f] += v[f]
        c.profile(False)
    peaks = load_peaks()
    top = max(kprof, key=lambda k: kprof[k]["ms"])
    kp = kprof[top]
    sec = kp["ms"] * 1e-3
    f16 = top == "gemm_trail"
    tf_peak = peaks["bf16_tflops"] if f16 else peaks["bf16_tflops"] / 2.0
    if top.startswith("gemm_"):
        ach = kp["flops"] / sec / 1e12
        roof = {"bound": "tensor", "achieved": ach, "peak": tf_peak, "unit": "TFLOP/s", "frac": ach / tf_peak}
    else:
        ach = kp["bytes"] / sec / 1e9
        roof = {"bound": "hbm", "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": ach / peaks["hbm_gbs"]}
    roof.update({"traffic": None, "kernel_class": top, "launches": kp["launches"], "peak_src": peaks["src"],
                 "note": "class time summed over the lanes (kernels of different lanes overlap)"})
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        tc, tw, desc = c4_cpu_sample(wl, cells)
        cpu = {"value": ntr * n / tc, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port", "sample": desc,
               "modelled_full_batch_s": tc, "sample_wall_s": tw}
    if rank == 0:
        sizes = [3 * len(x) for x, _ in cells]
        acc = sum(r[0] for r in res) / n
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "c64 tf32-tensor LU + double-float (or FP64 FFT) residual refinement",
                "data": "synthetic (seeded fractal aggregates)",
                "config": {"workload": wl["name"], "instances": n, "unknowns_min_max": [min(sizes), max(sizes)],
                           "directions": ntr, "polarisations": 2, "lanes": args.lanes,
                           "ir_tol": wl.get("ir_tol", 1e-13),
                           "parallelism": f"replicas x{world}",
                           "l2": "inputs larger than L2 (per-instance complex64 matrices up to 3.9 GB)"},
                "roofline": roof, "cpu_baseline": cpu,
                "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": int(sum(56 * len(x) for x, _ in cells)),
                        "d2h_bytes_per_step": int(sum(16 * 2 * ntr * s for s in sizes))},
                "gpu_launches": launches, "clocks": clk.summary(),
                "averages": {"Q_ext": float(acc[0]), "Q_abs": float(acc[1]), "Q_sca": float(acc[2]),
                             "g": float(acc[4])},
                "profiled_step_s": tp,
                "kernel_classes": {k: {"ms_per_step": v["ms"], "launches_per_step": v["launches"]}
                                   for k, v in kprof.items()}}
        print(json.dumps(line), flush=True)
    for c in contexts:
        c.close()
    return 0


def fp64_mom_extrapolated(local, wl, value):
    """Plain FP64 MoM (FP64 fill + cuSOLVER zgetrf/zgetrs) for a system too large to
    factor within the benchmark: scaled from the measured 60,000-unknown point
    (FP64_MEASURED) by N^3 (factorisation) and N^2 (fill).  A cross-check is timed
    here on the 12,672-unknown sphere and scaled the same way."""
    from midas_gb300 import _lib
    from midas_gb300.solver import Context
    n1 = 3 * len(wl["xyz"])
    r = n1 / FP64_MEASURED["unknowns"]
    t = FP64_MEASURED["factor_ms"] * 1e-3 * r ** 3 + FP64_MEASURED["fill_ms"] * 1e-3 * r ** 2
    ntr = len(wl["th"])
    ref = workload_mom_c1()
    c64 = Context(device=local, solve_mode=_lib.SOLVE_FP64)
    c64.set_cells(ref["xyz"], ref["sc"], ref["eps"], ref["k0"])
    th = np.asarray(wl["th"], float)
    ph = np.asarray(wl["ph"], float)
    c64.mom_solve(th, ph)
    c64.mom_solve(th, ph)
    inf = c64.info.as_dict()
    c64.close()
    n0 = 3 * len(ref["xyz"])
    t_c1 = inf["t_factor_ms"] * 1e-3 * (n1 / n0) ** 3 + inf["t_fill_ms"] * 1e-3 * (n1 / n0) ** 2
    return {"value": ntr / t, "unit": "solves/s", "impl": "cuSOLVER zgetrf/zgetrs FP64 + FP64 fill",
            "measured_on": FP64_MEASURED, "scaled_to_unknowns": n1, "scale_factor_n3": r ** 3, "seconds": t,
            "speedup": value / (ntr / t), "memory_gb_fp64_matrix": 16.0 * n1 * n1 / 1e9,
            "cross_check_from_12672_unknowns": {"factor_ms_measured": inf["t_factor_ms"], "scaled_s": t_c1}}


def ctypes_byref(x):
    import ctypes
    return ctypes.byref(x)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 10; 5 for the batch workloads, whose step is ~25 s)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cbfm_c2", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--lanes", type=int, default=4, help="concurrent contexts of a batch workload")
    ap.add_argument("--fp64-measure", action="store_true",
                    help="time the plain FP64 MoM (cuSOLVER) on the workload itself, whatever its size")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 5 if args.workload in ("c4", "c4_small") else 10
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    world, rank, local, pg = dist_setup(args)
    wl = WORKLOADS[args.workload]()
    if args.impl == "reference":
        rc = run_reference(args, wl, world, rank, pg)
    elif wl["method"] == "batch":
        rc = run_batch_bench(args, wl, world, rank, local, pg)
    else:
        rc = run_ours(args, wl, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
