"""CPU oracle for the MIDAS VIE-MoM / CBFM hot path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module, and only as the checker.
The GPU product (``midas_gb300``) never imports it.

The element-level arithmetic (fills, incident fields, ACA, far field, cross
sections) lives in ``midas_oracle.c`` and the orientation averaging in
``midas_oracle_q.c`` (C restatements of the reference
Fortran, each routine citing its source).  This module binds it with ctypes and
restates the dense algebra of the reference drivers with LAPACK (numpy/scipy):

* ``mom_solve``   -- Compute_EFields_MoM (src/Compute_EFields_MoM.f90:1-427):
  FP64 fill, ``PZGESV`` -> ``zgesv``, then S-matrix and Cext/Cabs.
* ``cbfm_solve``  -- Compute_EFields_CBFME (src/Compute_EFields_CBFME.f90:1-1006)
  and, with ``use_aca``, Compute_EFields_CBFME_ACA
  (src/Compute_EFields_CBFME_ACA.f90:588-635).  PARDISO on the thresholded
  sparse block (src/pardiso_solver.f90) is replaced by a dense LAPACK solve of
  the same thresholded matrix; ``GESVD`` by ``numpy.linalg.svd``; ``ZGEMM`` by
  complex128 ``matmul``; the ScaLAPACK reduced solve by ``zgesv``.

Parity status: UNPINNED (the reference cannot be built here and ships no
golden outputs).  MKL's version is not pinned by the reference either.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libmidas_oracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build() -> str:
    """Compile the C restatement (idempotent)."""
    srcs = [os.path.join(_HERE, f) for f in ("midas_oracle.c", "midas_oracle_q.c", "Makefile")]
    if (not os.path.exists(_LIB_PATH)) or os.path.getmtime(_LIB_PATH) < max(map(os.path.getmtime, srcs)):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        i, d, l = ctypes.c_int, ctypes.c_double, ctypes.c_long
        sig = {
            "or_pi": (d, []),
            "or_set_cells_params": (None, [i, _dp, _dp, d, _dp, _dp, _dp, _dp]),
            "or_mom_fill": (None, [i, _dp, _dp, _dp, _dp, _dp, _dp, d, i, i, i, i, _dp]),
            "or_mom_rhs": (None, [i, _dp, _dp, _dp, d, i, _dp, _dp, _dp]),
            "or_incident_c4": (None, [i, _ip, _dp, _dp, _dp, d, _dp, _dp, i, i, _dp]),
            "or_incident_sph": (None, [i, _ip, _dp, _dp, _dp, d, _dp, _dp, i, i, _dp]),
            "or_green_partial": (None, [i, _ip, i, _ip, _dp, _dp, _dp, _dp, _dp, _dp, d, _dp]),
            "or_green_partial_fn": (d, [i, _ip, i, _ip, i, _dp, _dp, _dp, _dp, _dp, _dp, d]),
            "or_sr_dense": (l, [i, _ip, d, i, _dp, _dp, _dp, _dp, _dp, _dp, d, _dp, _dp]),
            "or_set_fsr": (d, [i, _ip, i, d, _dp, _dp, _dp, _dp, _dp, _dp, d, ctypes.POINTER(l)]),
            "or_transmitters_un": (i, [i, _dp, _dp]),
            "or_init_nipws": (i, [d, i, i]),
            "or_block_row": (None, [i, i, i, _dp, _dp, _dp, _dp, _dp, d, _dp]),
            "or_block_col": (None, [i, i, i, _dp, _dp, _dp, _dp, _dp, d, _dp]),
            "or_aca": (i, [i, i, i, i, d, i, _dp, _dp, _dp, _dp, _dp, d, _dp, _dp]),
            "or_smatrix": (None, [i, _dp, _dp, _dp, _dp, _dp, d, i, _dp, _dp, i, _dp, _dp]),
            "or_cext_cabs": (None, [i, _dp, _dp, _dp, _dp, _dp, d, i, _dp, _dp, _dp, _dp, _dp]),
            "or_sphere_cells": (i, [d, d, _dp, i]),
            "or_num_threads": (i, []),
            "or_qag_grid": (d, [_dp, i, d, d, _ip, _ip, _ip]),
            "or_scattering_quantities": (i, [i, i, i, i, i, i, i, d, d, i, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                             _dp, _dp, _dp, _dp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


# Reference literals that are single precision in the Fortran source.
RES_SR_DEFAULT = float(np.float32(1e-2))      # res_SR = 1e-2 (src/InOut_ReadWrite_Functions.f90:395)
EPS_ACA_DEFAULT = float(np.float32(1e-4))     # Epsilon_ACA = 1E-4 (:396)
THR_ACA_DRIVER = float(np.float32(1e-3))      # Threshold_CBFM = 1e-3 (src/Compute_EFields_CBFME_ACA.f90:124)
NB_IT_MAX_DEFAULT = 50                        # Nb_it_max = 50 (:396)


def ref_pi() -> float:
    return lib().or_pi()


@dataclass
class Cells:
    """Per-cell inputs (type Cell, src/Initialization.f90:22-26) + SetCellsParams."""

    xyz: np.ndarray          # (n, 3) centroids
    sc: np.ndarray           # (n,) cell edge
    eps: np.ndarray          # (n,) complex relative permittivity
    k0: float
    a_n: np.ndarray = field(init=False)
    che: np.ndarray = field(init=False)
    znnpp: np.ndarray = field(init=False)
    kappa: np.ndarray = field(init=False)

    def __post_init__(self):
        self.xyz = _f64(self.xyz).reshape(-1, 3)
        n = self.xyz.shape[0]
        self.sc = _f64(np.broadcast_to(self.sc, (n,)))
        self.eps = _c128(np.broadcast_to(self.eps, (n,)))
        self.x = _f64(self.xyz[:, 0])
        self.y = _f64(self.xyz[:, 1])
        self.z = _f64(self.xyz[:, 2])
        self.a_n = np.zeros(n)
        self.che = np.zeros(n, np.complex128)
        self.znnpp = np.zeros(n, np.complex128)
        self.kappa = np.zeros(n)
        lib().or_set_cells_params(n, _d(self.sc), _d(self.eps.view(np.float64)), self.k0,
                                  _d(self.a_n), _d(self.che.view(np.float64)),
                                  _d(self.znnpp.view(np.float64)), _d(self.kappa))

    @property
    def n(self) -> int:
        return self.xyz.shape[0]

    def geo(self):
        return (_d(self.x), _d(self.y), _d(self.z))

    def par(self):
        return (_d(self.kappa), _d(self.che.view(np.float64)), _d(self.znnpp.view(np.float64)))


# ---------------------------------------------------------------------------
# element-level wrappers
# ---------------------------------------------------------------------------
def mom_fill(c: Cells, r0: int = 0, nr: int | None = None, c0: int = 0, nc: int | None = None) -> np.ndarray:
    """compute_Green_s_tr_single_element over a sub-block (FP64)."""
    N = 3 * c.n
    nr = N - r0 if nr is None else nr
    nc = N - c0 if nc is None else nc
    Z = np.zeros((nc, nr), np.complex128)   # column-major storage of (nr x nc)
    lib().or_mom_fill(c.n, *c.geo(), *c.par(), c.k0, r0, nr, c0, nc, _d(Z.view(np.float64)))
    return Z.T


def mom_rhs(c: Cells, th, ph) -> np.ndarray:
    """Incident_Field_single_element for all unknowns: (3n, 2 NTr), FP64."""
    th, ph = _f64(th), _f64(ph)
    V = np.zeros((2 * len(th), 3 * c.n), np.complex128)
    lib().or_mom_rhs(c.n, *c.geo(), c.k0, len(th), _d(th), _d(ph), _d(V.view(np.float64)))
    return V.T


def incident_c4(c: Cells, th, ph, idx=None) -> np.ndarray:
    """Incident_Field with complex(4) locals: (3n_sel, 2 NTr)."""
    th, ph = _f64(th), _f64(ph)
    if idx is None:
        n, ip = c.n, None
    else:
        idx = _i32(idx)
        n, ip = len(idx), _i(idx)
    E = np.zeros((2 * len(th), 3 * n), np.complex128)
    lib().or_incident_c4(n, ip, *c.geo(), c.k0, _d(th), _d(ph), 0, len(th), _d(E.view(np.float64)))
    return E.T


def incident_sph(c: Cells, th, ph, idx=None) -> np.ndarray:
    """Incident_Field_Spherical (src/Incident_Field.f90:65-166) on the cells idx
    (all cells when None), complex(4) locals: (3n_sel, 2 NTr)."""
    th, ph = _f64(th), _f64(ph)
    if idx is None:
        n, ip = c.n, None
    else:
        idx = _i32(idx)
        n, ip = len(idx), _i(idx)
    E = np.zeros((2 * len(th), 3 * n), np.complex128)
    lib().or_incident_sph(n, ip, *c.geo(), c.k0, _d(th), _d(ph), 0, len(th), _d(E.view(np.float64)))
    return E.T


def green_partial(c: Cells, idx1, idx2) -> np.ndarray:
    """Green_s_tr_partial (complex(4) locals): (3 n1, 3 n2)."""
    idx1, idx2 = _i32(idx1), _i32(idx2)
    Z = np.zeros((3 * len(idx2), 3 * len(idx1)), np.complex128)
    lib().or_green_partial(len(idx1), _i(idx1), len(idx2), _i(idx2), *c.geo(), *c.par(), c.k0,
                           _d(Z.view(np.float64)))
    return Z.T


def green_partial_fn(c: Cells, idx1, idx2, homog: int) -> float:
    idx1, idx2 = _i32(idx1), _i32(idx2)
    return lib().or_green_partial_fn(len(idx1), _i(idx1), len(idx2), _i(idx2), homog, *c.geo(),
                                     *c.par(), c.k0)


def sr_dense(c: Cells, idx, fsr: float, homog: int, want_matrix: bool = True):
    """Dense equivalent of SR_Green_s_tr_partial's CSR block: (Z or None, nnz, fn)."""
    idx = _i32(idx)
    s = len(idx)
    fn = ctypes.c_double(0)
    Z = np.zeros((3 * s, 3 * s), np.complex128) if want_matrix else None
    nnz = lib().or_sr_dense(s, _i(idx), fsr, homog, *c.geo(), *c.par(), c.k0,
                            _d(Z.view(np.float64)) if want_matrix else None, ctypes.byref(fn))
    return (Z.T if want_matrix else None), int(nnz), fn.value


def set_fsr(c: Cells, idx, homog: int, res_sr: float = RES_SR_DEFAULT):
    idx = _i32(idx)
    nnz = ctypes.c_long(0)
    f = lib().or_set_fsr(len(idx), _i(idx), homog, res_sr, *c.geo(), *c.par(), c.k0, ctypes.byref(nnz))
    return f, int(nnz.value)


def transmitters_un(niws: int):
    cap = 2 * niws + 64
    th = np.zeros(cap)
    ph = np.zeros(cap)
    nt = lib().or_transmitters_un(niws, _d(th), _d(ph))
    return th[:nt].copy(), ph[:nt].copy()


def init_nipws(r_lambda: float, distr: int = 1, niws_input: int = 0) -> int:
    return lib().or_init_nipws(r_lambda, distr, niws_input)


def block_row(c: Cells, grow: int, col0: int, ncols: int) -> np.ndarray:
    out = np.zeros(ncols, np.complex128)
    lib().or_block_row(grow, col0, ncols, *c.geo(), _d(c.kappa), _d(c.che.view(np.float64)), c.k0,
                       _d(out.view(np.float64)))
    return out


def block_col(c: Cells, row0: int, nrows: int, gcol: int) -> np.ndarray:
    out = np.zeros(nrows, np.complex128)
    lib().or_block_col(row0, nrows, gcol, *c.geo(), _d(c.kappa), _d(c.che.view(np.float64)), c.k0,
                       _d(out.view(np.float64)))
    return out


def aca(c: Cells, row0: int, nrows: int, col0: int, ncols: int, eps: float = EPS_ACA_DEFAULT,
        itmax: int = NB_IT_MAX_DEFAULT):
    """Calcul_MatrixZij_ACA on the unknown block [row0, row0+nrows) x [col0, col0+ncols)."""
    U = np.zeros((itmax, nrows), np.complex128)
    V = np.zeros((ncols, itmax), np.complex128)
    k = lib().or_aca(row0, nrows, col0, ncols, eps, itmax, *c.geo(), _d(c.kappa),
                     _d(c.che.view(np.float64)), c.k0, _d(U.view(np.float64)), _d(V.view(np.float64)))
    return int(k), U.T, V.T


def smatrix(c: Cells, rth, rph, E: np.ndarray) -> np.ndarray:
    """S-matrix (NRx, 4 NTr): columns Vv, Vh, Hv, Hh per transmitter."""
    rth, rph = _f64(rth), _f64(rph)
    ntr = E.shape[1] // 2
    Ef = np.asfortranarray(E, dtype=np.complex128)
    S = np.zeros((4 * ntr, len(rth)), np.complex128)
    lib().or_smatrix(c.n, *c.geo(), _d(c.kappa), _d(c.che.view(np.float64)), c.k0, len(rth), _d(rth),
                     _d(rph), ntr, _d(Ef.T.view(np.float64).reshape(-1)), _d(S.view(np.float64)))
    return S.T


def cext_cabs(c: Cells, th, ph, E: np.ndarray):
    th, ph = _f64(th), _f64(ph)
    Ef = np.asfortranarray(E, dtype=np.complex128)
    cext = np.zeros(len(th))
    cabs = np.zeros(len(th))
    lib().or_cext_cabs(c.n, *c.geo(), _d(c.sc), _d(c.che.view(np.float64)), c.k0, len(th), _d(th),
                       _d(ph), _d(Ef.T.view(np.float64).reshape(-1)), _d(cext), _d(cabs))
    return cext, cabs


# Integration rules NumIntType_t / NumIntType_r (src/InOut_ReadWrite_Functions.f90:319).
QUAD = {"un": 0, "tr": 1, "gl": 2, "sd": 3, "lb": 4, "rf": 5}


def qag_grid(f, a0: float, b0: float):
    """getAdaptiveQuadPts2 on one sampled column: (result, neval, ier, bad_index)."""
    f = _f64(f)
    ne, ier, bad = (np.zeros(1, np.int32) for _ in range(3))
    r = lib().or_qag_grid(_d(f), len(f), a0, b0, _i(ne), _i(ier), _i(bad))
    return r, int(ne[0]), int(ier[0]), int(bad[0])


def scattering_quantities(quad_tr, quad_rx, tr_grid, rx_grid, tr_th, tr_ph, rx_th, rx_ph, S, cext, cabs,
                          dm, k0, cext_intfields=0, w_tr=None, w_rx=None):
    """Compute_Scattering_Quantities_1/_2: (status, q_dir (ntr, 5), q_avg (5)), columns
    Q_ext, Q_abs, Q_sca, Q_bks, g.  tr_grid / rx_grid = (n_theta, n_phi); S is
    (nrx_tot, 4 ntr) with the extra forward/backward receivers after the grid."""
    S = np.asfortranarray(S, dtype=np.complex128)
    ntr = tr_grid[0] * tr_grid[1]
    qd = np.zeros((ntr, 5))
    qa = np.zeros(5)
    wt = _f64(w_tr) if w_tr is not None else None
    wr = _f64(w_rx) if w_rx is not None else None
    st = lib().or_scattering_quantities(
        QUAD[quad_tr], QUAD[quad_rx], tr_grid[0], tr_grid[1], rx_grid[0], rx_grid[1], S.shape[0], dm, k0,
        cext_intfields, _d(_f64(tr_th)), _d(_f64(tr_ph)), _d(_f64(rx_th)), _d(_f64(rx_ph)),
        _d(S.T.view(np.float64).reshape(-1)), _d(_f64(cext)), _d(_f64(cabs)),
        _d(wt) if wt is not None else None, _d(wr) if wr is not None else None, _d(qd), _d(qa))
    return st, qd, qa


def sphere_cells(dm: float, sc: float) -> np.ndarray:
    n = lib().or_sphere_cells(dm, sc, None, 0)
    xyz = np.zeros((n, 3))
    lib().or_sphere_cells(dm, sc, _d(xyz), n)
    return xyz


# ---------------------------------------------------------------------------
# drivers
# ---------------------------------------------------------------------------
def _solve(A, B):
    import scipy.linalg as sla
    return sla.solve(A, B, check_finite=False)


def mom_solve(c: Cells, th, ph, rth=None, rph=None):
    """Compute_EFields_MoM: returns dict(E, S, cext, cabs)."""
    Z = mom_fill(c)
    V = mom_rhs(c, th, ph)
    E = _solve(Z, V)
    out = {"E": E}
    if rth is not None:
        out["S"] = smatrix(c, rth, rph, E)
    out["cext"], out["cabs"] = cext_cabs(c, th, ph, E)
    return out


def cbf_threshold(c: Cells) -> float:
    """Threshold_CBFM from max|m| (src/Compute_EFields_CBFME.f90:286-288)."""
    m_abs = np.sqrt(np.abs(c.eps))
    rel = math.ceil(float(np.max(m_abs))) - 2.0
    return max(10.0 ** (-3.0 - rel), float(np.float32(1e-10)))


@dataclass
class Partition:
    """Caller-supplied CBFM partition: cells ordered by block.

    blk_offsets[b]..blk_offsets[b+1] are the cells of block b (contiguous, as
    Division_blocks orders them); ext[b] lists the global indices of the
    extension cells of block b (CBFM_Blocks_Ext, src/Extend_blocks.f90:134).
    """

    blk_offsets: np.ndarray
    ext: list

    @property
    def nblocks(self) -> int:
        return len(self.blk_offsets) - 1

    def block(self, b):
        return np.arange(self.blk_offsets[b], self.blk_offsets[b + 1], dtype=np.int32)

    def extended(self, b):
        return np.concatenate([self.block(b), np.asarray(self.ext[b], dtype=np.int32)])


def cbf_generate(c: Cells, part: Partition, th_cbfm, ph_cbfm, thr: float, sr: int = 1, homog: int = 0,
                 res_sr: float = RES_SR_DEFAULT, keep=None, spherical: bool = False):
    """CBF generation loop (src/Compute_EFields_CBFME.f90:221-449).

    Returns the list of C_b (3 n_b x K_b) and K_b.  ``keep`` (dict) receives the
    per-block fSR, nnz and singular values when given.  ``spherical`` selects the
    spherical-wave excitations of type_iws = 2/3 (:363-368).
    """
    Cs, Ks = [], []
    for b in range(part.nblocks):
        ext = part.extended(b)
        nb = part.blk_offsets[b + 1] - part.blk_offsets[b]
        Eref = (incident_sph if spherical else incident_c4)(c, th_cbfm, ph_cbfm, idx=ext)
        if sr:
            fsr, nnz = set_fsr(c, ext, homog, res_sr)
            Zb, nnz2, _ = sr_dense(c, ext, fsr, homog)
        else:
            fsr, nnz = 0.0, 9 * len(ext) ** 2
            Zb = green_partial(c, ext, ext)
        Ep = _solve(Zb, Eref)
        U, S, _ = np.linalg.svd(Ep, full_matrices=False)
        rel = S / S[0]
        K = int(np.count_nonzero(rel >= thr))
        Cs.append(np.ascontiguousarray(U[: 3 * nb, :K]))
        Ks.append(K)
        if keep is not None:
            keep.setdefault("fsr", []).append(fsr)
            keep.setdefault("nnz", []).append(nnz)
            keep.setdefault("sv", []).append(S)
    return Cs, Ks


def reduced_matrix(c: Cells, part: Partition, Cs, use_aca=False, eps_aca=EPS_ACA_DEFAULT,
                   itmax=NB_IT_MAX_DEFAULT, stats=None):
    """Zc(i,j) = C_i^T Z_ij C_j (src/Compute_EFields_CBFME.f90:630-809), or the
    ACA form C_i^T (U (V C_j)) for i != j (src/Compute_EFields_CBFME_ACA.f90:588-635)."""
    Ks = [C.shape[1] for C in Cs]
    off = np.concatenate([[0], np.cumsum(Ks)]).astype(int)
    Zc = np.zeros((off[-1], off[-1]), np.complex128)
    for i in range(part.nblocks):
        bi = part.block(i)
        for j in range(part.nblocks):
            bj = part.block(j)
            if use_aca and i != j:
                k, U, V = aca(c, 3 * int(bi[0]), 3 * len(bi), 3 * int(bj[0]), 3 * len(bj), eps_aca, itmax)
                k = min(k, itmax)
                if stats is not None:
                    stats.setdefault("aca_rank", {})[(i, j)] = k
                if k < itmax:
                    Zc[off[i]:off[i + 1], off[j]:off[j + 1]] = Cs[i].T @ (U[:, :k] @ (V[:k, :] @ Cs[j]))
                    continue
            Zij = green_partial(c, bi, bj)
            Zc[off[i]:off[i + 1], off[j]:off[j + 1]] = (Cs[i].T @ Zij) @ Cs[j]
    return Zc, off


def cbfm_solve(c: Cells, part: Partition, th, ph, niws: int, use_aca: bool = False, sr: int = 1,
               homog: int = 0, thr: float | None = None, res_sr: float = RES_SR_DEFAULT,
               eps_aca: float = EPS_ACA_DEFAULT, itmax: int = NB_IT_MAX_DEFAULT, keep=None,
               spherical: bool = False):
    """Compute_EFields_CBFME (or _ACA): returns dict(E, K, Zc, Vc, alpha).
    ``spherical``: CBF excitations by Incident_Field_Spherical (type_iws = 2/3)."""
    th_c, ph_c = transmitters_un(niws)
    if thr is None:
        thr = THR_ACA_DRIVER if use_aca else cbf_threshold(c)
    Cs, Ks = cbf_generate(c, part, th_c, ph_c, thr, sr=sr, homog=homog, res_sr=res_sr, keep=keep,
                          spherical=spherical)
    Zc, off = reduced_matrix(c, part, Cs, use_aca=use_aca, eps_aca=eps_aca, itmax=itmax, stats=keep)
    ntr = len(th)
    Vc = np.zeros((off[-1], 2 * ntr), np.complex128)
    for b in range(part.nblocks):
        Einc = incident_c4(c, th, ph, idx=part.block(b))
        Vc[off[b]:off[b + 1]] = Cs[b].T @ Einc
    alpha = _solve(Zc, Vc)
    E = np.zeros((3 * c.n, 2 * ntr), np.complex128)
    for b in range(part.nblocks):
        r0, r1 = 3 * part.blk_offsets[b], 3 * part.blk_offsets[b + 1]
        E[r0:r1] = Cs[b] @ alpha[off[b]:off[b + 1]]
    return {"E": E, "K": np.array(Ks), "Zc": Zc, "Vc": Vc, "alpha": alpha, "C": Cs, "thr": thr,
            "ntr_cbfm": len(th_c)}
