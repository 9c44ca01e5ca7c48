"""Learned initial guess and learned preconditioner for the Krylov solve of
voxel scatterers.

    python -m midas_gb300.learned [--grid 32] [--train 2000] [--prec-scenes 300] [--test 500]

Workflow (all arithmetic in the library: GMRES and flexible GMRES on the FFT
lattice operator, the network's forward, backward and Adam kernels; numpy only
assembles arrays):

1. seeded scenes on a grid^3 voxel grid -- Gaussian random spheres and
   aggregates of touching spheres, per-voxel complex permittivity, size
   parameter 1..8, one incident direction (two polarisations);
2. the initial-guess network: training pairs from the solver itself (each
   scene's internal field from GMRES, midas_gpu_gmres_solve, to a 1e-6 true
   relative residual), trained on (incident field, permittivity) -> field;
3. the preconditioner network: pairs (r = Z e, e) with e the Arnoldi vectors
   of the Jacobi-preconditioned operator (no solve needed), trained to map a
   Krylov vector to Z^-1 of it; it right-preconditions flexible GMRES
   (midas_gpu_fgmres_solve);
4. held-out scenes: GMRES from zero, from the incident field and from the
   guess, flexible GMRES with the preconditioner from zero and from the guess,
   all to the same FP64-checked true residual, with the dense mixed solve (LU
   + refinement to a 1e-13 backward error, the reference's PZGESV answer) as
   the judge of each field error.

The reference (Compute_EFields_MoM, src/Compute_EFields_MoM.f90:153-198)
solves these systems densely; nothing here changes that answer -- the
networks only choose where the Krylov iteration starts and which directions
it explores, and every answer is accepted on its FP64 true residual.
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

    def prec_grid(self, V, scale, out=None):
        """Preconditioner inputs [ncol, grid^3, 16] and mask [ncol, grid^3] of cell
        vectors V (3n, ncol) at scales scale[ncol] (midas_gpu_nn_prec_grid).  out =
        (inputs, mask) device tensors to write into, else host arrays."""
        V = np.ascontiguousarray(np.asarray(V, np.complex128).T)
        ncol = V.shape[0]
        sc = np.ascontiguousarray(scale, np.float64)
        if out is None:
            out = (np.zeros((ncol, self.grid ** 3, IN_CH), np.float32), np.zeros((ncol, self.grid ** 3), np.float32))
        self.ctx._ck(self.L.midas_gpu_nn_prec_grid(self.ctx.h, self.h, ncol, addr(V), addr(sc), addr(out[0]),
                                                   addr(out[1])))
        return out

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


def train(net, data, epochs=8, batch=8, lr=1e-3, seed=0, log=None):
    """Adam over shuffled batches; the learning rate falls as a cosine to 5 % of lr.
    (With He-initialised weights a rate of 3e-3 kills the ReLUs of this network on
    the 16^3 scenes within two epochs; 1e-3 trains.)"""
    inputs, mask, target = data
    rng = np.random.default_rng(seed)
    hist = []
    nb = max(1, len(inputs) // batch)
    for ep in range(epochs):
        order = rng.permutation(len(inputs))
        losses = []
        lr_ep = lr * (0.05 + 0.95 * 0.5 * (1.0 + math.cos(math.pi * ep / max(1, epochs))))
        for b in range(nb):
            sel = np.sort(order[b * batch:(b + 1) * batch])
            losses.append(net.train_step(inputs[sel], mask[sel], target[sel], lr_ep))
        hist.append(float(np.mean(losses)))
        if log:
            log(f"  epoch {ep}: mean relative squared error {hist[-1]:.4f}")
    return hist


def krylov_pairs(ctx, net, sc, nvec=16):
    """Training pairs of the preconditioner for one scene, with no solve: the
    Arnoldi basis e_1..e_nvec of the Jacobi-preconditioned MoM operator started
    from each polarisation's incident field (the directions GMRES explores), and
    r_j = Z e_j from the lattice operator.  The network input is r_j on the grid
    at scale s_j = sqrt(n) / |r_j| (midas_gpu_nn_prec_grid), the target s_j e_j
    (channels 8-13 of e_j's grid at the same scale): the network learns Z^-1 on
    Krylov-like vectors.  Returns float16 inputs, uint8 mask, float16 target."""
    ctx.set_cells(sc["xyz"], sc["sc"], sc["eps"], sc["k0"])
    b = ctx.mom_rhs(sc["th"], sc["ph"])                     # (3n, 2)
    D = np.repeat(1.0 - ctx.cell_params()["znnpp"], 3)
    V = [b / np.linalg.norm(b, axis=0)]
    for _ in range(nvec - 1):
        w = ctx.lattice_matvec(V[-1] / D[:, None])
        for _pass in range(2):                                # classical Gram-Schmidt, twice
            for v in V:
                w = w - v * np.sum(np.conj(v) * w, axis=0)
        V.append(w / np.linalg.norm(w, axis=0))
    E = np.concatenate(V, axis=1)                             # (3n, 2 nvec)
    R = ctx.lattice_matvec(E)
    s = math.sqrt(sc["n"]) / np.linalg.norm(R, axis=0)
    inp, mask = net.prec_grid(R, s)
    tg, _ = net.prec_grid(E, s)
    return inp.astype(np.float16), mask.astype(np.uint8), tg[:, :, 8:14].astype(np.float16)


class _Pairs:
    """Stored pairs, handed to train() batch by batch as float32."""

    def __init__(self, parts):
        self.a = [np.concatenate([p[q] for p in parts]) for q in range(3)]

    def __len__(self):
        return len(self.a[0])

    def view(self, q):
        arr = self.a[q]

        class _V:
            def __len__(self_v):
                return len(arr)

            def __getitem__(self_v, sel):
                return np.ascontiguousarray(arr[sel], np.float32)
        return _V()

    def as_data(self):
        return self.view(0), self.view(1), self.view(2)


def generate_prec(ctx, net, scene_list, nvec=16, log=None):
    parts = []
    for k, sc in enumerate(scene_list):
        parts.append(krylov_pairs(ctx, net, sc, nvec))
        if log and (k + 1) % 100 == 0:
            log(f"  {k + 1}/{len(scene_list)} scenes of preconditioner pairs")
    return _Pairs(parts)


def evaluate(ctx, scene_list, guess_net=None, prec_net=None, tol=1e-6, judge=0, log=None):
    """Per held-out scene, all to the same FP64-checked true residual: GMRES
    (Jacobi) from zero, from the incident field and from the guess network's
    prediction; flexible GMRES with the preconditioner network from zero and
    from the guess.  The first `judge` scenes are also solved densely (mixed LU +
    FP64-grade refinement) as the judge of each answer's field error."""
    rows = []
    for k, sc in enumerate(scene_list):
        inp, m = grid_inputs(sc)
        row = {"kind": sc["kind"], "unknowns": 3 * sc["n"], "x": sc["x"], "tol": tol}
        sols = {}
        E0, row["its_zero"], row["rel_zero"], row["t_zero"] = solve_gmres(ctx, sc, tol=tol)
        sols["zero"] = E0
        _, row["its_inc"], _, _ = solve_gmres(ctx, sc, E0=grid_to_cells(sc, inp[:, :, 2:8]), tol=tol)
        guess = None
        if guess_net is not None:
            t0 = time.perf_counter()
            guess = grid_to_cells(sc, guess_net.forward(inp, m))
            t_g = time.perf_counter() - t0
            sols["guess"], row["its_guess"], row["rel_guess"], t = solve_gmres(ctx, sc, E0=guess, tol=tol)
            row["t_guess"] = t + t_g
        if prec_net is not None:
            t0 = time.perf_counter()
            sols["prec"], row["its_prec"], row["rel_prec"] = ctx.fgmres_solve(prec_net, sc["th"], sc["ph"], tol=tol,
                                                                              maxit=3000, check=False)
            row["t_prec"] = time.perf_counter() - t0
            if guess is not None:
                t0 = time.perf_counter()
                sols["both"], row["its_both"], row["rel_both"] = ctx.fgmres_solve(prec_net, sc["th"], sc["ph"], E0=guess,
                                                                                  tol=tol, maxit=3000, check=False)
                row["t_both"] = time.perf_counter() - t0 + t_g
        if k < judge:
            Et = ctx.mom_solve(sc["th"], sc["ph"])
            nrm = np.linalg.norm(Et)
            for key, E in sols.items():
                row["err_" + key] = float(np.linalg.norm(E - Et) / nrm)
            if guess is not None:
                row["err_guess_start"] = float(np.linalg.norm(guess - Et) / nrm)
        rows.append(row)
        if log and (k + 1) % 50 == 0:
            log(f"  {k + 1}/{len(scene_list)} held-out scenes")
    return rows


def summarise(rows):
    out = {"scenes": len(rows)}
    its0 = sum(r["its_zero"] for r in rows)
    t0 = sum(r["t_zero"] for r in rows)
    out.update({"mean_its_zero": its0 / len(rows), "mean_its_incident_start": float(np.mean([r["its_inc"] for r in rows])),
                "solves_per_s_zero": len(rows) / t0,
                "converged_zero": int(sum(r["rel_zero"] <= r["tol"] for r in rows))})
    for key in ("guess", "prec", "both"):
        if "its_" + key not in rows[0]:
            continue
        its = sum(r["its_" + key] for r in rows)
        t = sum(r["t_" + key] for r in rows)
        out.update({f"mean_its_{key}": its / len(rows), f"iteration_ratio_{key}": its / its0,
                    f"solves_per_s_{key}": len(rows) / t,
                    f"converged_{key}": int(sum(r["rel_" + key] <= r["tol"] for r in rows))})
    judged = [r for r in rows if "err_zero" in r]
    if judged:
        out["judged"] = len(judged)
        for key in ("zero", "guess", "prec", "both"):
            if "err_" + key in judged[0]:
                out[f"max_err_{key}_vs_dense"] = max(r["err_" + key] for r in judged)
        if "err_guess_start" in judged[0]:
            out["mean_err_guess_start_vs_dense"] = float(np.mean([r["err_guess_start"] for r in judged]))
    return out


def main(argv=None):
    from .solver import Context
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--grid", type=int, default=32)
    ap.add_argument("--train", type=int, default=2000, help="training pairs of the guess network (two per scene)")
    ap.add_argument("--prec-scenes", type=int, default=300, help="scenes of preconditioner pairs")
    ap.add_argument("--nvec", type=int, default=8, help="Arnoldi vectors per polarisation and scene")
    ap.add_argument("--test", type=int, default=500, help="held-out scenes")
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--prec-epochs", type=int, default=20)
    ap.add_argument("--judge", type=int, default=20, help="held-out scenes also solved densely")
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--no-guess", action="store_true", help="preconditioner only")
    args = ap.parse_args(argv)
    log = lambda s: print(s, flush=True)   # noqa: E731
    ctx = Context(fill_mode=_lib.FILL_FAST)
    summ = {"grid": args.grid}
    guess_net = None
    if not args.no_guess:
        t0 = time.perf_counter()
        data, its = generate(ctx, scenes(11, args.train // 2, args.grid), tol=args.tol, log=log)
        t_gen = time.perf_counter() - t0
        log(f"guess: {len(data[0])} pairs in {t_gen:.1f} s (mean GMRES iterations {np.mean(its):.0f})")
        guess_net = Net(ctx, args.grid, seed=1)
        t1 = time.perf_counter()
        hist = train(guess_net, data, epochs=args.epochs, log=log)
        summ.update({"guess_pairs": int(len(data[0])), "guess_generate_s": t_gen, "guess_train_s": time.perf_counter() - t1,
                     "guess_loss_history": hist})
        del data
    prec_net = Net(ctx, args.grid, seed=2)
    t0 = time.perf_counter()
    pairs = generate_prec(ctx, prec_net, scenes(13, args.prec_scenes, args.grid), nvec=args.nvec, log=log)
    t_gen = time.perf_counter() - t0
    log(f"preconditioner: {len(pairs)} pairs in {t_gen:.1f} s")
    t1 = time.perf_counter()
    hist = train(prec_net, pairs.as_data(), epochs=args.prec_epochs, batch=16, log=log)
    summ.update({"prec_pairs": len(pairs), "prec_generate_s": t_gen, "prec_train_s": time.perf_counter() - t1,
                 "prec_loss_history": hist, "params": prec_net.n})
    del pairs
    rows = evaluate(ctx, scenes(12345, args.test, args.grid), guess_net, prec_net, tol=args.tol, judge=args.judge,
                    log=log)
    summ.update(summarise(rows))
    print(json.dumps(summ), flush=True)
    for nt in (guess_net, prec_net):
        if nt is not None:
            nt.close()
    ctx.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
