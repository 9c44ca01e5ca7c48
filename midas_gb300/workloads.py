"""Benchmark scenes of the MIDAS hot path, and a runner that solves them
through the library without PyTorch (the command the profiler runs).

    python -m midas_gb300.workloads cbfm_c2_small --steps 1

Each scene is seeded synthetic input with the shapes of the reference's
configurations: the reference sphere voxeliser (src/Discretization.f90:246-310)
for the homogeneous sphere, a voxelised Gaussian random sphere for the CBFM
scene, a 3x3x3 bounding-box partition extended by 15 % of the block edge
(Extend_blocks, src/Extend_blocks.f90:46-151) and the 'un' CBF excitations
(getTransmitters_CBFM, src/getParameters_CBFM.f90:34-75).
"""
from __future__ import annotations

import argparse
import math
import time

import numpy as np


def mom_c1():
    """Plain MoM, homogeneous sphere x = 2, m = 1.5 + 0.01i, a/d = 10 (4,224 cells,
    12,672 unknowns), +z incidence (MIDAS angles theta = phi = 90 deg), V + H."""
    from . import geometry as G
    a, x, m = 1.0, 2.0, 1.5 + 0.01j
    k0 = x / a
    sc = a / 10.0
    xyz = G.sphere_cells(2 * a, sc)
    return {"name": "mom_c1_sphere_x2_m1.5+0.01i_4224cells", "xyz": xyz, "sc": sc,
            "eps": np.full(len(xyz), m * m), "k0": k0, "th": np.array([90.0]), "ph": np.array([90.0]),
            "method": "mom"}


def mom_c3(n_cells=20000, ndir=32, seed=5):
    """Mixed-precision dense solve on an inhomogeneous cube of side 2 lambda: a
    28^3 lattice truncated to n_cells voxels (20,000: 60k unknowns), per-voxel
    eps' ~ U[1.5, 3.5], eps'' ~ U[0, 0.2] (seeded), ndir seeded plane-wave
    directions x 2 polarisations (64 right-hand sides), refined to a 1e-8
    backward error."""
    from . import geometry as G
    side = 28
    d = 1.0 / side                      # cube side 1 = 2 lambda  ->  lambda = 0.5
    k0 = 2 * math.pi / 0.5
    rng = np.random.default_rng(seed)
    xyz = G.cube_cells(side, d, n_cells)
    eps = rng.uniform(1.5, 3.5, len(xyz)) + 1j * rng.uniform(0.0, 0.2, len(xyz))
    th, ph = G.random_directions(ndir, seed=seed + 1)
    return {"name": f"mom_c3_cube_2lambda_{len(xyz)}cells_{2 * ndir}rhs", "xyz": xyz, "sc": d, "eps": eps, "k0": k0,
            "th": th, "ph": ph, "method": "mom", "ir_tol": 1e-8}


def mom_c3_small():
    """The same cube truncated to 4,000 voxels (12k unknowns, 3.5 GB of matrices):
    the dense-solve kernels at a size a profiler captures in minutes."""
    return mom_c3(n_cells=4000)


def mom_tiny():
    """The reference's literal sphere case: x = 2, m = 1.5 + 0.01i, a/d = 4.775
    (489 cells), +z incidence, V + H -- small enough for CPU tests."""
    from . import geometry as G
    a, x, m = 1.0, 2.0, 1.5 + 0.01j
    sc = a / 4.775
    xyz = G.sphere_cells(2 * a, sc)
    return {"name": "mom_tiny_sphere_x2_ad4.775", "xyz": xyz, "sc": sc, "eps": np.full(len(xyz), m * m),
            "k0": x / a, "th": np.array([90.0]), "ph": np.array([90.0]), "method": "mom"}


def _gaussian_sphere_cbfm(name, x, a_over_d, ndir, nbox=3, seed=2026):
    from . import geometry as G
    a, m = 1.0, 1.55 + 0.005j
    k0 = x / a
    sc = a / a_over_d
    xyz = G.gaussian_sphere(a, 0.15, 20.0, sc, seed=seed)
    perm, offs = G.box_partition(xyz, nbox, nbox, nbox)
    xyz = np.ascontiguousarray(xyz[perm])
    box, sph = G.block_contours(xyz, offs)
    edge = float((box[:, 1] - box[:, 0]).max(axis=1).mean())
    ext = G.extend_blocks(xyz, offs, 0.15 * edge, sc)
    lam = 2 * math.pi / k0
    niws = G.init_nipws(float(sph[:, 3].max()) / (lam / abs(m)))
    cth, cph = G.transmitters_un(niws)
    th, ph = G.random_directions(ndir, seed=7)
    return {"name": name, "xyz": xyz, "sc": sc, "eps": np.full(len(xyz), m * m), "k0": k0, "th": th, "ph": ph,
            "method": "cbfm", "offs": offs, "ext": ext, "cth": cth, "cph": cph, "homog": 1, "niws": niws}


def cbfm_c2():
    """CBFM-E on a seeded Gaussian random sphere: x = 6, m = 1.55 + 0.005i, log-radius
    std 0.15, correlation angle 20 deg, voxel a/21.1 (~41k cells, ~123k unknowns),
    3x3x3 bounding-box blocks with a 15 % (of the block edge) extension, CBF
    excitations from the reference's Niws table ('un'), 24 seeded incident
    directions x 2 polarisations."""
    return _gaussian_sphere_cbfm("cbfm_c2_gaussian_sphere_x6_m1.55+0.005i", 6.0, 21.1, 24)


def cbfm_c2_small():
    """The same scene at a/d = 12 (~7.6k cells) in 2x2x2 blocks: the kernels of
    the full scene with a launch count a profiler lists in minutes.  (A 3x3x3
    split at this resolution leaves corner blocks of a few cells, fewer unknowns
    than CBFs, and a singular reduced system.)"""
    return _gaussian_sphere_cbfm("cbfm_c2_small_gaussian_sphere_x6_ad12_2x2x2", 6.0, 12.0, 24, nbox=2)


def cbfm_c2_mid():
    """The same scene at a/d = 16 (~18k cells) in 2x2x2 blocks: extended blocks of
    ~15k unknowns with tens of millions of CSR nonzeros, the regime of the full
    scene's large blocks, in a few GB (for full profiler captures)."""
    return _gaussian_sphere_cbfm("cbfm_c2_mid_gaussian_sphere_x6_ad16_2x2x2", 6.0, 16.0, 24, nbox=2)


def _post_scene(name, tr_grid, rx_grid, seed=3):
    """Orientation-averaging input: 'un' transmitter and receiver grids over theta
    0..180, phi 0..360 (the extra forward / backward receivers appended as
    get_trans_Receiv does), a seeded S matrix peaked in each forward direction,
    and cross sections -- the shapes of a scattering run, with synthetic values."""
    from . import geometry as G
    rng = np.random.default_rng(seed)
    tth, tph = G.uniform_directions(0.0, 180.0, tr_grid[0], 0.0, 360.0, tr_grid[1])
    rth, rph = G.uniform_directions(0.0, 180.0, rx_grid[0], 0.0, 360.0, rx_grid[1])
    rth, rph = G.receivers_with_extras(rth, rph, tth, tph)
    ntr = len(tth)
    r = np.radians
    cosang = (np.cos(r(rth))[:, None] * np.cos(r(tth))[None, :]
              + (np.sin(r(rth))[:, None] * np.sin(r(tth))[None, :]) * np.cos(r(rph[:, None] - tph[None, :])))
    amp = 0.3 + 2.0 * np.exp(2.0 * (cosang - 1.0))
    S = np.empty((len(rth), 4 * ntr), np.complex128, order="F")   # the C-ABI layout (column-major)
    for k, scale in enumerate((1.0, 0.1, 0.1, 1.0)):
        S[:, k::4] = scale * amp * np.exp(2j * np.pi * rng.random(amp.shape))
    return {"name": name, "method": "post", "tr_grid": tr_grid, "rx_grid": rx_grid, "tr_th": tth, "tr_ph": tph,
            "rx_th": rth, "rx_ph": rph, "S": S, "cext": rng.uniform(5, 7, ntr), "cabs": rng.uniform(0.2, 0.4, ntr),
            "dm": 2.0, "k0": 2.0}


def post_sphere():
    """Efficiencies of one incident direction over 181 x 25 receivers ('un'/'un'):
    the receiver layout of the reference's sphere example."""
    return _post_scene("post_un_1tr_181x25rx", (1, 1), (181, 25))


def post_avg():
    """Orientation average over a 19 x 37 'un' transmitter grid (703 incident
    directions) with 181 x 25 'un' receivers: 35k adaptive quadratures."""
    return _post_scene("post_un_19x37tr_181x25rx", (19, 37), (181, 25))


def c4_instance(wl, k):
    """Cells of aggregate k of a C4 workload: (xyz, edge)."""
    from . import geometry as G
    P = G.fractal_aggregate(int(wl["n_mono"][k]), a=wl["a"], df=wl["df"], kf=wl["kf"], seed=int(wl["seeds"][k]))
    return G.voxelise_spheres(P, wl["a"], wl["cells_per_diameter"])


def c4(n_instances=256, ndir=48, nrx=194, seed=11):
    """Batched uneven instances: n_instances seeded aggregates of 4-64 touching
    spheres of radius 0.8 lambda / 2 pi (k0 a = 0.8), m = 1.33 + 0.001i, grown by
    tunable particle-cluster aggregation (fractal dimension 1.8, prefactor 1.3) and
    voxelised at 6 cells per monomer diameter (113 cells per monomer: 1.4k-22k
    unknowns); ndir seeded incident directions x 2 polarisations each, and nrx
    seeded scattering directions with equal weights for Q_sca and g ('rf' rules,
    Compute_Scattering_Quantities_2).  Instances are built by c4_instance.  The
    mixed solves refine to a 1e-10 backward error: the averages need a field
    accurate to 1e-6, and the 1e-13 default costs a second double-float residual
    per instance."""
    from . import geometry as G
    rng = np.random.default_rng(seed)
    th, ph = G.random_directions(ndir, seed=seed + 1)
    rth, rph = G.random_directions(nrx, seed=seed + 2)
    rth, rph = G.list_receivers_with_extras(rth, rph, th, ph)
    return {"name": f"c4_{n_instances}_aggregates_df1.8_{ndir}dirs", "method": "batch", "a": 1.0, "k0": 0.8,
            "m": 1.33 + 0.001j, "df": 1.8, "kf": 1.3, "cells_per_diameter": 6,
            "n_mono": rng.integers(4, 65, n_instances), "seeds": rng.integers(1 << 30, size=n_instances),
            "th": th, "ph": ph, "rx_th": rth, "rx_ph": rph, "nrx": nrx, "ir_tol": 1e-10}


def c4_small():
    """Eight C4 aggregates: the batch path at a size that runs in seconds."""
    return c4(n_instances=8)


WORKLOADS = {"mom_c1": mom_c1, "mom_c3": mom_c3, "mom_c3_small": mom_c3_small, "mom_tiny": mom_tiny,
             "cbfm_c2": cbfm_c2, "cbfm_c2_small": cbfm_c2_small, "cbfm_c2_mid": cbfm_c2_mid,
             "post_sphere": post_sphere, "post_avg": post_avg, "c4": c4, "c4_small": c4_small}


def cbfm_args(wl):
    """Partition arrays of a CBFM scene in the C-ABI layout."""
    bo = np.ascontiguousarray(wl["offs"], np.int32)
    eo = np.ascontiguousarray(np.concatenate([[0], np.cumsum([len(e) for e in wl["ext"]])]), np.int32)
    ei = np.ascontiguousarray(np.concatenate(wl["ext"]), np.int32)
    return bo, eo, ei


def batch_instance(ctx, wl, xyz, d):
    """One C4 aggregate through the library: MoM solve for every direction, S
    matrix, cross sections and the list-rule orientation averages.  Returns
    (Q averages [5], far-field <Cext>, internal-field <Cabs>)."""
    th, ph, rth, rph = wl["th"], wl["ph"], wl["rx_th"], wl["rx_ph"]
    ntr = len(th)
    ctx.set_cells(xyz, d, wl["m"] ** 2, wl["k0"])
    E = ctx.mom_solve(th, ph)
    S = ctx.smatrix(rth, rph, E)
    ce, ca = ctx.cext_cabs(th, ph, E)
    dm = 2.0 * (3.0 * len(xyz) * d ** 3 / (4.0 * math.pi)) ** (1.0 / 3.0)   # volume-equivalent
    _, qa = ctx.scattering_quantities("rf", "rf", (ntr, 1), (wl["nrx"], 1), th, ph, rth, rph, S, ce, ca, dm,
                                      wl["k0"])
    return qa, float(qa[0]) * math.pi * (dm / 2.0) ** 2, float(np.mean(ca))


def batch_step(contexts, wl, cells):
    """Every instance once, largest first, pulled by len(contexts) concurrent lanes
    (one host thread and one context -- its own CUDA stream -- per lane).  Returns
    the per-instance results in instance order."""
    import threading
    order = sorted(range(len(cells)), key=lambda k: -len(cells[k][0]))
    out = [None] * len(cells)
    nxt = [0]
    lock = threading.Lock()
    err = []

    def lane(ctx):
        while True:
            with lock:
                if nxt[0] >= len(order) or err:
                    return
                k = order[nxt[0]]
                nxt[0] += 1
            try:
                out[k] = batch_instance(ctx, wl, *cells[k])
            except Exception as e:   # reported after the lanes join
                err.append(e)
                return

    ths = [threading.Thread(target=lane, args=(c,)) for c in contexts]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    if err:
        raise err[0]
    return out


def run_batch(ctx, wl, steps, lanes=4):
    """C4: every aggregate solved for all directions (fill, mixed LU, refinement),
    then its S matrix, Cext / Cabs and orientation averages; prints the
    orientation-averaged solves/s (directions x instances / wall time) and the
    averages over the instances.  <Cext> is the optical-theorem (far-field)
    extinction: the reference's internal-field cross sections sum the three field
    components before the products (Compute_ExtAbsCsec_fromIntField.f90:52-59),
    which holds only for axis-aligned incidence, and these directions are random.
    <Cabs> is the reference's internal-field value all the same (its Q_abs always
    is).  Instances run on `lanes` concurrent contexts."""
    cells = [c4_instance(wl, k) for k in range(len(wl["n_mono"]))]   # scene preparation, not timed
    ntr = len(wl["th"])
    unknowns = [3 * len(x) for x, _ in cells]
    contexts = [ctx] + [ctx.sibling() for _ in range(lanes - 1)]
    for step in range(steps):
        t0 = time.perf_counter()
        res = batch_step(contexts, wl, cells)
        dt = time.perf_counter() - t0
        n = len(cells)
        acc = sum(r[0] for r in res)
        cext = sum(r[1] for r in res)
        cabs = sum(r[2] for r in res)
        print(f"{wl['name']}: step {step} {dt:.3f} s, {ntr * n / dt:.2f} orientation-averaged solves/s "
              f"({n} instances, {min(unknowns)}-{max(unknowns)} unknowns, {lanes} lanes), <Cext> {cext / n:.5g}, "
              f"<Cabs> {cabs / n:.5g}, <g> {acc[4] / n:.4f}", flush=True)
    for c in contexts:
        c.close()
    return 0


def main(argv=None):
    from . import _lib
    from .solver import Context
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("workload", choices=sorted(WORKLOADS))
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--fill", default="fast", choices=["fast", "faithful"])
    ap.add_argument("--verbose", "-v", action="count", default=0,
                    help="library trace: -v refinement steps and CBFM lanes, -vv per-block detail")
    ap.add_argument("--lanes", type=int, default=4, help="concurrent contexts of the C4 batch")
    ap.add_argument("--aca", action="store_true", help="CBFM: off-diagonal reduced blocks from ACA factors")
    ap.add_argument("--classes", action="store_true",
                    help="after the steps, one more step with per-kernel-class CUDA-event timing (one lane)")
    args = ap.parse_args(argv)
    wl = WORKLOADS[args.workload]()
    ctx = Context(device=0, fill_mode=_lib.FILL_FAST if args.fill == "fast" else _lib.FILL_FAITHFUL,
                  ir_tol=wl.get("ir_tol", 1e-13), verbose=args.verbose)
    if wl["method"] == "post":
        for step in range(args.steps):
            ctx.profile(True)
            t0 = time.perf_counter()
            qd, qa = ctx.scattering_quantities("un", "un", wl["tr_grid"], wl["rx_grid"], wl["tr_th"], wl["tr_ph"],
                                               wl["rx_th"], wl["rx_ph"], wl["S"], wl["cext"], wl["cabs"], wl["dm"],
                                               wl["k0"])
            dt = time.perf_counter() - t0
            dev = ctx.profile_query().get("other", {}).get("ms", float("nan"))
            ctx.profile(False)
            print(f"{wl['name']}: step {step} {dt * 1e3:.2f} ms (kernels {dev:.2f} ms), "
                  f"<Q_ext, Q_abs, Q_sca, Q_bks, g> = {np.array2string(qa, precision=5)}", flush=True)
        ctx.close()
        return 0
    if wl["method"] == "batch":
        return run_batch(ctx, wl, args.steps, lanes=args.lanes)
    ctx.set_cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
    for step in range(args.steps):
        t0 = time.perf_counter()
        if wl["method"] == "cbfm":
            flags = _lib.CBFM_SR | (_lib.CBFM_HOMOG if wl.get("homog") else 0) | (_lib.CBFM_ACA if args.aca else 0)
            E, K = ctx.cbfm_solve(wl["offs"], wl["ext"], wl["cth"], wl["cph"], wl["th"], wl["ph"], flags=flags)
        else:
            E = ctx.mom_solve(wl["th"], wl["ph"])
        dt = time.perf_counter() - t0
        print(f"{wl['name']}: step {step} {dt:.3f} s, {ctx.launch_count()} launches so far", flush=True)
    if args.classes:
        ctx.profile(True)
        t0 = time.perf_counter()
        if wl["method"] == "cbfm":
            ctx.cbfm_solve(wl["offs"], wl["ext"], wl["cth"], wl["cph"], wl["th"], wl["ph"], flags=flags)
        else:
            ctx.mom_solve(wl["th"], wl["ph"])
        dt = time.perf_counter() - t0
        prof = ctx.profile_query()
        ctx.profile(False)
        print(f"{wl['name']}: profiled step {dt:.3f} s; kernel classes (ms, launches, TFLOP/s, GB/s):")
        for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"]):
            if v["launches"]:
                sec = v["ms"] * 1e-3
                print(f"  {k:11s} {v['ms']:9.2f} {v['launches']:7d} {v['flops'] / sec / 1e12:8.2f} "
                      f"{v['bytes'] / sec / 1e9:8.1f}", flush=True)
    ctx.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
