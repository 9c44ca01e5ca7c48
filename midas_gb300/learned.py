"""Learned initial guess for the Krylov solve of voxel scatterers.

    python -m midas_gb300.learned [--grid 32] [--train 2000] [--test 500] [--epochs 30]

Workflow (all arithmetic in the library: GMRES on the FFT lattice operator,
the network's forward, backward and Adam kernels; numpy only assembles arrays):

1. seeded scenes on a grid^3 voxel grid -- Gaussian random spheres and
   aggregates of touching spheres, per-voxel complex permittivity, size
   parameter 1..8, one incident direction (two polarisations);
2. training pairs from the solver itself: each scene's internal field from
   GMRES (midas_gpu_gmres_solve) to a 1e-6 true relative residual;
3. training of the network (midas_gpu_nn_train_step);
4. held-out scenes: GMRES from zero against GMRES from the network's
   prediction, both to the same FP64-checked residual, and the dense mixed
   solve (LU + refinement to a 1e-13 backward error, the reference's PZGESV
   answer) as the judge of the field error.

The reference (Compute_EFields_MoM, src/Compute_EFields_MoM.f90:153-198)
solves these systems densely; nothing here changes that answer -- the network
only chooses where the Krylov iteration starts.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import time

import numpy as np

from . import _lib
from . import geometry as G
from ._lib import addr

IN_CH, OUT_CH = 16, 6


class Net:
    """The library's network (midas_gpu_nn_*), on a grid^3 voxel grid."""

    def __init__(self, ctx, grid: int = 32, seed: int = 0):
        self.ctx, self.L, self.grid = ctx, ctx.L, grid
        h = ctypes.c_void_p()
        ctx._ck(self.L.midas_gpu_nn_create(ctx.h, grid, seed, ctypes.byref(h)))
        self.h = h
        self.n = int(self.L.midas_gpu_nn_param_count(h))

    def close(self):
        if self.h:
            self.L.midas_gpu_nn_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self, grads: bool = False) -> np.ndarray:
        buf = np.zeros(self.n, np.float32)
        self.ctx._ck(self.L.midas_gpu_nn_params(self.ctx.h, self.h, 0, addr(buf), int(grads)))
        return buf

    def set_params(self, theta):
        buf = np.ascontiguousarray(theta, np.float32)
        self.ctx._ck(self.L.midas_gpu_nn_params(self.ctx.h, self.h, 1, addr(buf), 0))

    def forward(self, inputs, mask):
        B = inputs.shape[0]
        E = np.zeros((B, self.grid ** 3, OUT_CH), np.float32)
        self.ctx._ck(self.L.midas_gpu_nn_forward(self.ctx.h, self.h, B, addr(_f32(inputs)), addr(_f32(mask)),
                                                 addr(E)))
        return E

    def gradients(self, inputs, mask, target) -> float:
        loss = ctypes.c_double()
        self.ctx._ck(self.L.midas_gpu_nn_gradients(self.ctx.h, self.h, inputs.shape[0], addr(_f32(inputs)),
                                                   addr(_f32(mask)), addr(_f32(target)), ctypes.byref(loss)))
        return loss.value

    def train_step(self, inputs, mask, target, lr: float) -> float:
        loss = ctypes.c_double()
        self.ctx._ck(self.L.midas_gpu_nn_train_step(self.ctx.h, self.h, inputs.shape[0], addr(_f32(inputs)),
                                                    addr(_f32(mask)), addr(_f32(target)), float(lr),
                                                    ctypes.byref(loss)))
        return loss.value


def _f32(a):
    if isinstance(a, np.ndarray):
        return np.ascontiguousarray(a, np.float32)
    return a   # a device tensor, already float32 and contiguous


# ---------------------------------------------------------------------------
# scenes on the voxel grid
# ---------------------------------------------------------------------------
def _centres(grid):
    g = np.arange(grid) - (grid - 1) / 2.0
    Z, Y, X = np.meshgrid(g, g, g, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)   # voxel order: x fastest


def shape_mask(rng, grid: int, kind: str) -> np.ndarray:
    """Boolean mask over the grid^3 voxels: a Gaussian random sphere or an aggregate."""
    p = _centres(grid)
    if kind == "gaussian":
        a = rng.uniform(0.28, 0.46) * grid
        sigma = rng.uniform(0.05, 0.2)
        coeffs = G._legendre_coeffs(rng.uniform(25.0, 60.0), 8)
        r = np.linalg.norm(p, axis=1)
        ct = np.where(r > 0, p[:, 2] / np.maximum(r, 1e-12), 1.0)
        ph = np.arctan2(p[:, 1], p[:, 0])
        s = np.zeros(len(p))
        for l in range(9):
            if coeffs[l] <= 0:
                continue
            sd = sigma * math.sqrt(coeffs[l] * 4 * math.pi / (2 * l + 1))
            for m in range(-l, l + 1):
                s += rng.normal(0.0, sd) * G._real_sph_harm(l, m, ct, ph)
        mask = r < a * np.exp(s - sigma ** 2 / 2.0)
    else:
        nmono = int(rng.integers(4, 17))
        cen = G.fractal_aggregate(nmono, a=1.0, seed=int(rng.integers(1 << 30)))
        ext = float(np.max(np.linalg.norm(cen, axis=1))) + 1.0
        am = 0.47 * grid / ext
        cen = cen * am
        mask = np.zeros(len(p), bool)
        for c in cen:
            mask |= np.sum((p - c) ** 2, axis=1) < am * am
    if mask.sum() < 8:
        mask[np.argsort(np.linalg.norm(p, axis=1))[:8]] = True
    return mask


def make_scene(rng, grid: int, kind: str) -> dict:
    """Cells, per-voxel permittivity, size parameter x in [1, 8] (capped so that
    the internal wavelength spans at least 2 pi voxels), one direction."""
    mask = shape_mask(rng, grid, kind)
    n = int(mask.sum())
    e1 = rng.uniform(1.5, 3.5) + rng.uniform(-0.2, 0.2, n)
    e2 = rng.uniform(0.0, 0.2, n)
    eps = e1 + 1j * e2
    a_eq = (3.0 * n / (4.0 * math.pi)) ** (1.0 / 3.0)           # equivalent radius, voxels
    m_max = float(np.max(np.sqrt(np.abs(eps))))
    x = float(rng.uniform(1.0, max(1.0, min(8.0, a_eq / m_max))))
    k0 = x / a_eq                                                # voxel edge d = 1
    th, ph = G.random_directions(1, seed=int(rng.integers(1 << 30)))
    xyz = np.ascontiguousarray(_centres(grid)[mask])
    return {"kind": kind, "grid": grid, "mask": mask, "xyz": xyz, "sc": 1.0, "eps": eps, "k0": k0, "x": x,
            "th": np.asarray(th, float), "ph": np.asarray(ph, float), "n": n}


def incident_grid(sc) -> np.ndarray:
    """Plane-wave incident field on every voxel, the MoM right-hand side's formula
    (Incident_Field_single_element, src/Compute_EFields_MoM.f90:529-598):
    [2 polarisations, grid^3, 3] complex."""
    p = _centres(sc["grid"])
    tr, pr = sc["th"][0] * G.REF_PI / 180.0, sc["ph"][0] * G.REF_PI / 180.0
    k = sc["k0"] * np.array([math.cos(tr), math.sin(tr) * math.cos(pr), math.sin(tr) * math.sin(pr)])
    e = np.exp(1j * (p @ k))
    st, ct, sp, cp = math.sin(tr), math.cos(tr), math.sin(pr), math.cos(pr)
    out = np.zeros((2, len(p), 3), complex)
    out[0] = np.stack([-e * st, e * ct * cp, e * ct * sp], axis=1)
    out[1] = np.stack([0 * e, -e * sp, e * cp], axis=1)
    return out


def grid_inputs(sc):
    """Network inputs [2, V, 16] and mask [2, V] (float32): chi = eps - 1 (0 outside),
    the incident field, chi times each incident component, the mask, 0."""
    V = sc["grid"] ** 3
    chi = np.zeros(V, complex)
    chi[sc["mask"]] = sc["eps"] - 1.0
    einc = incident_grid(sc)
    inp = np.zeros((2, V, IN_CH), np.float32)
    for pol in range(2):
        inp[pol, :, 0], inp[pol, :, 1] = chi.real, chi.imag
        for q in range(3):
            inp[pol, :, 2 + 2 * q] = einc[pol, :, q].real
            inp[pol, :, 3 + 2 * q] = einc[pol, :, q].imag
            prod = chi * einc[pol, :, q]
            inp[pol, :, 8 + 2 * q] = prod.real
            inp[pol, :, 9 + 2 * q] = prod.imag
        inp[pol, :, 14] = sc["mask"]
    mask = np.repeat(sc["mask"][None].astype(np.float32), 2, axis=0)
    return inp, mask


def cells_to_grid(sc, E) -> np.ndarray:
    """E (3n, 2) complex -> [2, V, 6] float32 (zero outside the scatterer)."""
    V = sc["grid"] ** 3
    out = np.zeros((2, V, OUT_CH), np.float32)
    idx = np.flatnonzero(sc["mask"])
    for pol in range(2):
        e = E[:, pol].reshape(-1, 3)
        for q in range(3):
            out[pol, idx, 2 * q] = e[:, q].real
            out[pol, idx, 2 * q + 1] = e[:, q].imag
    return out


def grid_to_cells(sc, Eg) -> np.ndarray:
    """[2, V, 6] -> E (3n, 2) complex."""
    idx = np.flatnonzero(sc["mask"])
    E = np.zeros((3 * sc["n"], 2), complex)
    for pol in range(2):
        v = Eg[pol][idx].astype(np.float64)
        E[:, pol] = (v[:, 0::2] + 1j * v[:, 1::2]).reshape(-1)
    return E


def scenes(seed: int, count: int, grid: int):
    rng = np.random.default_rng(seed)
    return [make_scene(rng, grid, "gaussian" if i % 2 == 0 else "aggregate") for i in range(count)]


# ---------------------------------------------------------------------------
# data, training, evaluation
# ---------------------------------------------------------------------------
def solve_gmres(ctx, sc, E0=None, tol=1e-6, maxit=3000, restart=50):
    ctx.set_cells(sc["xyz"], sc["sc"], sc["eps"], sc["k0"])
    t0 = time.perf_counter()
    E, it, rel = ctx.gmres_solve(sc["th"], sc["ph"], E0=E0, restart=restart, maxit=maxit, tol=tol, jacobi=True,
                                 check=False)
    return E, it, rel, time.perf_counter() - t0


def generate(ctx, scene_list, tol=1e-6, log=None):
    """Training pairs (inputs, mask, target) from GMRES solves of the scenes."""
    ins, masks, tgts, its = [], [], [], []
    for k, sc in enumerate(scene_list):
        E, it, rel, _ = solve_gmres(ctx, sc, tol=tol)
        if rel > tol:
            continue   # not converged within the cap: left out of the data
        inp, m = grid_inputs(sc)
        ins.append(inp)
        masks.append(m)
        tgts.append(cells_to_grid(sc, E))
        its.append(it)
        if log and (k + 1) % 100 == 0:
            log(f"  {k + 1}/{len(scene_list)} solves, mean GMRES iterations {np.mean(its):.0f}")
    return (np.concatenate(ins), np.concatenate(masks), np.concatenate(tgts)), its


def train(net, data, epochs=8, batch=8, lr=2e-3, seed=0, log=None):
    """Adam over shuffled batches; the learning rate falls as a cosine to 5 % of lr."""
    inputs, mask, target = data
    rng = np.random.default_rng(seed)
    hist = []
    nb = max(1, len(inputs) // batch)
    for ep in range(epochs):
        order = rng.permutation(len(inputs))
        losses = []
        lr_ep = lr * (0.05 + 0.95 * 0.5 * (1.0 + math.cos(math.pi * ep / max(1, epochs))))
        for b in range(nb):
            sel = order[b * batch:(b + 1) * batch]
            losses.append(net.train_step(inputs[sel], mask[sel], target[sel], lr_ep))
        hist.append(float(np.mean(losses)))
        if log:
            log(f"  epoch {ep}: mean relative squared error {hist[-1]:.4f}")
    return hist


def evaluate(ctx, net, scene_list, tol=1e-6, judge=0, log=None):
    """Per held-out scene: GMRES iterations and time from zero and from the
    network's guess (same tolerance), and for the first `judge` scenes the field
    error of both against the dense mixed solve."""
    rows = []
    for k, sc in enumerate(scene_list):
        inp, m = grid_inputs(sc)
        t0 = time.perf_counter()
        guess = grid_to_cells(sc, net.forward(inp, m))
        t_net = time.perf_counter() - t0
        E0, it0, rel0, t0s = solve_gmres(ctx, sc, tol=tol)
        _, iti, _, _ = solve_gmres(ctx, sc, E0=grid_to_cells(sc, inp[:, :, 2:8]), tol=tol)
        E1, it1, rel1, t1s = solve_gmres(ctx, sc, E0=guess, tol=tol)
        row = {"kind": sc["kind"], "unknowns": 3 * sc["n"], "x": sc["x"], "its_zero": it0, "its_inc": iti,
               "its_net": it1, "rel_zero": rel0, "rel_net": rel1, "t_zero": t0s, "t_net": t1s + t_net, "tol": tol}
        Et = ctx.mom_solve(sc["th"], sc["ph"]) if k < judge else None
        if Et is not None:
            nrm = np.linalg.norm(Et)
            row.update({"err_zero": float(np.linalg.norm(E0 - Et) / nrm), "err_net": float(np.linalg.norm(E1 - Et) / nrm),
                        "err_guess": float(np.linalg.norm(guess - Et) / nrm)})
        rows.append(row)
        if log and (k + 1) % 50 == 0:
            log(f"  {k + 1}/{len(scene_list)} held-out scenes")
    return rows


def summarise(rows):
    its0 = np.array([r["its_zero"] for r in rows], float)
    itsi = np.array([r["its_inc"] for r in rows], float)
    its1 = np.array([r["its_net"] for r in rows], float)
    t0 = sum(r["t_zero"] for r in rows)
    t1 = sum(r["t_net"] for r in rows)
    out = {"scenes": len(rows), "mean_its_zero": float(its0.mean()), "mean_its_incident_start": float(itsi.mean()),
           "mean_its_net": float(its1.mean()), "iteration_ratio": float(its1.sum() / its0.sum()),
           "solves_per_s_zero": len(rows) / t0, "solves_per_s_net": len(rows) / t1,
           "converged_zero": int(sum(r["rel_zero"] <= r["tol"] for r in rows)),
           "converged_net": int(sum(r["rel_net"] <= r["tol"] for r in rows))}
    judged = [r for r in rows if "err_net" in r]
    if judged:
        out.update({"judged": len(judged), "max_err_net_vs_dense": max(r["err_net"] for r in judged),
                    "max_err_zero_vs_dense": max(r["err_zero"] for r in judged),
                    "mean_err_guess_vs_dense": float(np.mean([r["err_guess"] for r in judged]))})
    return out


def main(argv=None):
    from .solver import Context
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--grid", type=int, default=32)
    ap.add_argument("--train", type=int, default=2000, help="training pairs (two per scene)")
    ap.add_argument("--test", type=int, default=500, help="held-out scenes")
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--judge", type=int, default=20, help="held-out scenes also solved densely")
    ap.add_argument("--tol", type=float, default=1e-6)
    args = ap.parse_args(argv)
    log = lambda s: print(s, flush=True)   # noqa: E731
    ctx = Context(fill_mode=_lib.FILL_FAST)
    t0 = time.perf_counter()
    train_scenes = scenes(11, args.train // 2, args.grid)
    data, its = generate(ctx, train_scenes, tol=args.tol, log=log)
    t_gen = time.perf_counter() - t0
    log(f"generated {len(data[0])} pairs in {t_gen:.1f} s (mean GMRES iterations {np.mean(its):.0f})")
    net = Net(ctx, args.grid, seed=1)
    t1 = time.perf_counter()
    hist = train(net, data, epochs=args.epochs, log=log)
    t_train = time.perf_counter() - t1
    rows = evaluate(ctx, net, scenes(12345, args.test, args.grid), tol=args.tol, judge=args.judge, log=log)
    summ = summarise(rows)
    summ.update({"grid": args.grid, "train_pairs": int(len(data[0])), "generate_s": t_gen, "train_s": t_train,
                 "epochs": args.epochs, "loss_history": hist, "params": net.n})
    print(json.dumps(summ), flush=True)
    net.close()
    ctx.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
