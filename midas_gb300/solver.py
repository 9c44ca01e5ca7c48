"""Host-side mirror of the reference's solver interface, driving the GPU library.

``Context`` wraps one ``midas_gpu_ctx``.  Its methods follow the reference's
subroutines (same names, argument meaning and layout, reference file:line in
each docstring); arrays are numpy (host) or torch tensors (device) and are
passed to the C ABI by address.  Failures raise ``MidasError`` carrying the
MIDAS_* status -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import Info, MidasError, Opts, addr


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


@dataclass
class CellsIn:
    """type Cell inputs (src/Initialization.f90:22-26): centroids, edge, eps."""

    xyz: np.ndarray
    sc: np.ndarray
    eps: np.ndarray
    k0: float


class Context:
    def __init__(self, device: int = 0, solve_mode: int = _lib.SOLVE_MIXED, fill_mode: int = _lib.FILL_FAITHFUL,
                 index_base: int = 0, ir_tol: float = 1e-13, ir_max_iter: int = 30, verbose: int = 0):
        self.L = _lib.load()
        o = Opts()
        self.L.midas_gpu_default_opts(ctypes.byref(o))
        o.device, o.solve_mode, o.fill_mode, o.index_base = device, solve_mode, fill_mode, index_base
        o.ir_tol, o.ir_max_iter, o.verbose = ir_tol, ir_max_iter, verbose
        h = ctypes.c_void_p()
        st = self.L.midas_gpu_init(ctypes.byref(o), ctypes.byref(h))
        if st != 0:
            raise MidasError(st, "midas_gpu_init failed")
        self.h = h
        self.n = 0
        self.info = Info()
        self._keep = []
        self._opts = dict(device=device, solve_mode=solve_mode, fill_mode=fill_mode, index_base=index_base,
                          ir_tol=ir_tol, ir_max_iter=ir_max_iter, verbose=verbose)

    def sibling(self):
        """A new context with the same options (its own stream and scratch)."""
        return Context(**self._opts)

    def close(self):
        if self.h:
            self.L.midas_gpu_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, st):
        if st != 0:
            raise MidasError(st, self.L.midas_gpu_last_error(self.h).decode())

    # -- cells -------------------------------------------------------------
    def set_cells(self, xyz, sc, eps, k0: float):
        """SetCellsParams (src/SetCellsParams.f90:31-49) for the given cells."""
        xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
        n = xyz.shape[0]
        x, y, z = (_c(xyz[:, i], np.float64) for i in range(3))
        scv = _c(np.broadcast_to(sc, (n,)), np.float64)
        ev = np.broadcast_to(np.asarray(eps, dtype=np.complex128), (n,))
        er, ei = _c(ev.real, np.float64), _c(ev.imag, np.float64)
        self._ck(self.L.midas_gpu_set_cells(self.h, n, addr(x), addr(y), addr(z), addr(scv), addr(er), addr(ei),
                                            float(k0)))
        self.n = n
        return self

    def cell_params(self):
        n = self.n
        an, kap = np.zeros(n), np.zeros(n)
        che, zn = np.zeros(n, np.complex128), np.zeros(n, np.complex128)
        self._ck(self.L.midas_gpu_get_cell_params(self.h, addr(an), addr(che), addr(zn), addr(kap)))
        return {"a_n": an, "che": che, "znnpp": zn, "kappa": kap}

    # -- element-level entry points ----------------------------------------
    def mom_fill(self, r0=0, nr=None, c0=0, nc=None):
        """compute_Green_s_tr_single_element over a block (src/Compute_EFields_MoM.f90:433-523)."""
        N = 3 * self.n
        nr = N - r0 if nr is None else nr
        nc = N - c0 if nc is None else nc
        Z = np.zeros((nc, nr), np.complex128)
        self._ck(self.L.midas_gpu_mom_fill(self.h, r0, nr, c0, nc, addr(Z)))
        return Z.T

    def mom_rhs(self, th, ph):
        """Incident_Field_single_element (src/Compute_EFields_MoM.f90:529-598)."""
        th, ph = _c(th, np.float64), _c(ph, np.float64)
        V = np.zeros((2 * len(th), 3 * self.n), np.complex128)
        self._ck(self.L.midas_gpu_mom_rhs(self.h, len(th), addr(th), addr(ph), addr(V)))
        return V.T

    def incident_field(self, th, ph, idx=None):
        """Incident_Field with complex(4) locals (src/Incident_Field.f90:1-63)."""
        th, ph = _c(th, np.float64), _c(ph, np.float64)
        if idx is not None:
            idx = _c(idx, np.int32)
        nc = self.n if idx is None else len(idx)
        E = np.zeros((2 * len(th), 3 * nc), np.complex128)
        self._ck(self.L.midas_gpu_incident_field(self.h, nc, addr(idx), len(th), addr(th), addr(ph), addr(E)))
        return E.T

    def incident_field_spherical(self, th, ph, idx=None):
        """Incident_Field_Spherical with complex(4) locals (src/Incident_Field.f90:65-166):
        spherical waves from sources at 10 block radii around the cells' centroid."""
        th, ph = _c(th, np.float64), _c(ph, np.float64)
        if idx is not None:
            idx = _c(idx, np.int32)
        nc = self.n if idx is None else len(idx)
        E = np.zeros((2 * len(th), 3 * nc), np.complex128)
        self._ck(self.L.midas_gpu_incident_field_spherical(self.h, nc, addr(idx), len(th), addr(th), addr(ph),
                                                           addr(E)))
        return E.T

    def block_fill(self, idx1, idx2):
        """Green_s_tr_partial (src/Green_functions.f90:96-173)."""
        idx1, idx2 = _c(idx1, np.int32), _c(idx2, np.int32)
        Z = np.zeros((3 * len(idx2), 3 * len(idx1)), np.complex128)
        self._ck(self.L.midas_gpu_block_fill(self.h, len(idx1), addr(idx1), len(idx2), addr(idx2), addr(Z)))
        return Z.T

    def sr_fill(self, idx, fsr: float, homog: int, want_matrix=True):
        """SR_Green_s_tr_partial in dense form (src/Green_functions.f90:290-562)."""
        idx = _c(idx, np.int32)
        s = len(idx)
        Z = np.zeros((3 * s, 3 * s), np.complex128) if want_matrix else None
        nnz, fn = ctypes.c_longlong(0), ctypes.c_double(0)
        self._ck(self.L.midas_gpu_sr_fill(self.h, s, addr(idx), float(fsr), int(homog), addr(Z), ctypes.byref(nnz),
                                          ctypes.byref(fn)))
        return (Z.T if want_matrix else None), nnz.value, fn.value

    def set_fsr(self, idx, homog: int, res_sr: float = 0.0):
        """setfSR (src/getParameters_CBFM.f90:113-168)."""
        idx = _c(idx, np.int32)
        f, nnz = ctypes.c_double(0), ctypes.c_longlong(0)
        self._ck(self.L.midas_gpu_set_fsr(self.h, len(idx), addr(idx), int(homog), float(res_sr), ctypes.byref(f),
                                          ctypes.byref(nnz)))
        return f.value, nnz.value

    def aca(self, row0, nrows, col0, ncols, eps=float(np.float32(1e-4)), itmax=50):
        """Calcul_MatrixZij_ACA (src/Calcul_ACA_matrices.f90:6-219)."""
        U = np.zeros((itmax, nrows), np.complex128)
        V = np.zeros((ncols, itmax), np.complex128)
        k = ctypes.c_int(0)
        self._ck(self.L.midas_gpu_aca(self.h, row0, nrows, col0, ncols, float(eps), itmax, addr(U), addr(V),
                                      ctypes.byref(k)))
        return k.value, U.T, V.T

    # -- solves ------------------------------------------------------------
    def dense_solve(self, A, B):
        """PZGESV stand-in: solve A X = B (column-major complex)."""
        A = np.asfortranarray(A, dtype=np.complex128)
        X = np.array(B, dtype=np.complex128, order="F", copy=True)
        n, nrhs = X.shape
        self._ck(self.L.midas_gpu_dense_solve(self.h, n, nrhs, addr(A), addr(X), ctypes.byref(self.info)))
        return X

    def mom_solve(self, th, ph, out=None):
        """Field part of Compute_EFields_MoM (src/Compute_EFields_MoM.f90:66-229): E (3n x 2NTr)."""
        th, ph = _c(th, np.float64), _c(ph, np.float64)
        E = np.zeros((2 * len(th), 3 * self.n), np.complex128) if out is None else out
        self._ck(self.L.midas_gpu_mom_solve(self.h, len(th), addr(th), addr(ph), addr(E), ctypes.byref(self.info)))
        return E.T if out is None else E

    def lattice_matvec(self, X):
        """Y = Z X with the MoM matrix of compute_Green_s_tr_single_element
        (src/Compute_EFields_MoM.f90:433-523) applied as an FFT convolution on the
        cells' lattice.  X: (3n, nrhs) complex."""
        X = np.asarray(X, np.complex128)
        if X.ndim == 1:
            X = X[:, None]
        Xc = np.ascontiguousarray(X.T)   # column-major (3n, nrhs) = row-major (nrhs, 3n)
        Y = np.zeros_like(Xc)
        self._ck(self.L.midas_gpu_lattice_matvec(self.h, X.shape[1], addr(Xc), addr(Y)))
        return Y.T

    def gmres_solve(self, th, ph, E0=None, restart=50, maxit=2000, tol=1e-8, jacobi=False, check=True):
        """GMRES(restart) on the FFT lattice operator for the MoM system of
        Compute_EFields_MoM (src/Compute_EFields_MoM.f90:153-198): (E, iterations,
        true relative residual).  E0 (3n, 2ntr) is the initial guess.  With
        check=False a run that stops at maxit returns its last iterate instead
        of raising."""
        th, ph = _c(th, np.float64), _c(ph, np.float64)
        E = np.zeros((2 * len(th), 3 * self.n), np.complex128)
        e0 = None
        if E0 is not None:
            e0 = np.ascontiguousarray(np.asarray(E0, np.complex128).T)
        st = self.L.midas_gpu_gmres_solve(self.h, len(th), addr(th), addr(ph), addr(e0), int(restart), int(maxit),
                                          float(tol), _lib.GMRES_JACOBI if jacobi else 0, addr(E),
                                          ctypes.byref(self.info))
        if st != 0 and (check or st != 5):
            self._ck(st)
        return E.T, self.info.ir_iters, self.info.backward_error

    def fgmres_solve(self, net, th, ph, E0=None, restart=50, maxit=2000, tol=1e-8, check=True):
        """Flexible GMRES(restart) right-preconditioned by the learned network
        (midas_gpu_fgmres_solve): (E, iterations, true relative residual)."""
        th, ph = _c(th, np.float64), _c(ph, np.float64)
        E = np.zeros((2 * len(th), 3 * self.n), np.complex128)
        e0 = None if E0 is None else np.ascontiguousarray(np.asarray(E0, np.complex128).T)
        st = self.L.midas_gpu_fgmres_solve(self.h, net.h, len(th), addr(th), addr(ph), addr(e0), int(restart),
                                           int(maxit), float(tol), addr(E), ctypes.byref(self.info))
        if st != 0 and (check or st != 5):
            self._ck(st)
        return E.T, self.info.ir_iters, self.info.backward_error

    def cbfm_solve(self, blk_offsets, ext_lists, cbf_th, cbf_ph, th, ph, flags=_lib.CBFM_SR, thr_cbf=0.0,
                   res_sr=0.0, eps_aca=float(np.float32(1e-4)), aca_itmax=50, out=None):
        """Compute_EFields_CBFME(_ACA) (src/Compute_EFields_CBFME.f90:1-1006): (E, K)."""
        bo = _c(blk_offsets, np.int32)
        nb = len(bo) - 1
        eo = _c(np.concatenate([[0], np.cumsum([len(e) for e in ext_lists])]), np.int32)
        ei = _c(np.concatenate([np.asarray(e, np.int32) for e in ext_lists]) if eo[-1] > 0 else np.zeros(1),
                np.int32)
        cth, cph = _c(cbf_th, np.float64), _c(cbf_ph, np.float64)
        th, ph = _c(th, np.float64), _c(ph, np.float64)
        K = np.zeros(nb, np.int32)
        E = np.zeros((2 * len(th), 3 * self.n), np.complex128) if out is None else out
        self._ck(self.L.midas_gpu_cbfm_solve(self.h, nb, addr(bo), addr(eo), addr(ei), len(cth), addr(cth),
                                             addr(cph), float(thr_cbf), float(res_sr), int(flags), float(eps_aca),
                                             int(aca_itmax), len(th), addr(th), addr(ph), addr(E), addr(K),
                                             ctypes.byref(self.info)))
        return (E.T if out is None else E), K

    # -- scene preparation on the device --------------------------------------
    def voxelise_sphere(self, dm: float, sc: float) -> np.ndarray:
        """Discretization's sphere voxeliser (src/Discretization.f90:246-310): (n, 3) centroids."""
        n = ctypes.c_longlong(0)
        self._ck(self.L.midas_gpu_voxelise_sphere(self.h, float(dm), float(sc), 0, None, None, None, ctypes.byref(n)))
        xyz = np.zeros((3, n.value))
        self._ck(self.L.midas_gpu_voxelise_sphere(self.h, float(dm), float(sc), n.value, addr(xyz[0]), addr(xyz[1]),
                                                  addr(xyz[2]), ctypes.byref(n)))
        return np.ascontiguousarray(xyz.T)

    def voxelise_spheres(self, centres, a: float, cells_per_diameter: int = 6):
        """Cells inside a union of spheres: ((n, 3) centroids, edge)."""
        cen = _c(centres, np.float64).reshape(-1, 3)
        n, e = ctypes.c_longlong(0), ctypes.c_double(0)
        self._ck(self.L.midas_gpu_voxelise_spheres(self.h, len(cen), addr(cen), float(a), int(cells_per_diameter), 0,
                                                   None, None, None, ctypes.byref(n), ctypes.byref(e)))
        xyz = np.zeros((3, n.value))
        self._ck(self.L.midas_gpu_voxelise_spheres(self.h, len(cen), addr(cen), float(a), int(cells_per_diameter),
                                                   n.value, addr(xyz[0]), addr(xyz[1]), addr(xyz[2]), ctypes.byref(n),
                                                   ctypes.byref(e)))
        return np.ascontiguousarray(xyz.T), e.value

    def box_partition(self, xyz, nx: int, ny: int, nz: int):
        """Bounding-box blocks: (perm, blk_offsets) -- xyz[perm] is block-contiguous."""
        xyz = np.asarray(xyz, np.float64).reshape(-1, 3)
        x, y, z = (_c(xyz[:, i], np.float64) for i in range(3))
        perm = np.zeros(len(xyz), np.int32)
        offs = np.zeros(nx * ny * nz + 1, np.int32)
        nb = ctypes.c_int(0)
        self._ck(self.L.midas_gpu_box_partition(self.h, len(xyz), addr(x), addr(y), addr(z), nx, ny, nz, addr(perm),
                                                addr(offs), ctypes.byref(nb)))
        return perm, offs[: nb.value + 1].copy()

    def extend_blocks(self, xyz, blk_offsets, ext_length: float, sc: float):
        """Extend_blocks (src/Extend_blocks.f90:46-151): list of extension-cell index arrays."""
        xyz = np.asarray(xyz, np.float64).reshape(-1, 3)
        x, y, z = (_c(xyz[:, i], np.float64) for i in range(3))
        bo = _c(blk_offsets, np.int32)
        nb = len(bo) - 1
        eo = np.zeros(nb + 1, np.int32)
        tot = ctypes.c_longlong(0)
        self._ck(self.L.midas_gpu_extend_blocks(self.h, len(xyz), addr(x), addr(y), addr(z), nb, addr(bo),
                                                float(ext_length), float(sc), addr(eo), 0, None, ctypes.byref(tot)))
        ei = np.zeros(max(tot.value, 1), np.int32)
        self._ck(self.L.midas_gpu_extend_blocks(self.h, len(xyz), addr(x), addr(y), addr(z), nb, addr(bo),
                                                float(ext_length), float(sc), addr(eo), tot.value, addr(ei),
                                                ctypes.byref(tot)))
        return [ei[eo[b]:eo[b + 1]].copy() for b in range(nb)]

    # -- post-processing ---------------------------------------------------
    def cext_cabs(self, th, ph, E):
        """Compute_ExtAbsCsec_fromIntField (src/Compute_ExtAbsCsec_fromIntField.f90:45-64)."""
        th, ph = _c(th, np.float64), _c(ph, np.float64)
        Ef = np.asfortranarray(E, dtype=np.complex128)
        ce, ca = np.zeros(len(th)), np.zeros(len(th))
        self._ck(self.L.midas_gpu_cext_cabs(self.h, len(th), addr(th), addr(ph), addr(Ef), addr(ce), addr(ca)))
        return ce, ca

    def smatrix(self, rth, rph, E):
        """S matrix (src/Green_functions.f90:1399-1438, src/Compute_EFields_MoM.f90:306-369)."""
        rth, rph = _c(rth, np.float64), _c(rph, np.float64)
        Ef = np.asfortranarray(E, dtype=np.complex128)
        ntr = Ef.shape[1] // 2
        S = np.zeros((4 * ntr, len(rth)), np.complex128)
        self._ck(self.L.midas_gpu_smatrix(self.h, len(rth), addr(rth), addr(rph), ntr, addr(Ef), addr(S)))
        return S.T

    def scattering_quantities(self, quad_tr, quad_rx, tr_grid, rx_grid, tr_th, tr_ph, rx_th, rx_ph, S, cext, cabs,
                              dm, k0, cext_intfields=0, w_tr=None, w_rx=None):
        """Compute_Scattering_Quantities_1/_2 (src/Compute_Scattering_Quantities.f90:1-1012).

        quad_tr / quad_rx: 'un', 'tr', 'gl', 'sd', 'lb' or 'rf'; tr_grid / rx_grid:
        (n_theta, n_phi) of the transmitter and receiver sets (a list: (n, 1)); S
        (nrx_tot, 4 ntr) from smatrix over the receivers followed by the extra
        forward / backward ones; cext / cabs from cext_cabs; dm the scatterer's
        diameter.  Returns (q_dir (ntr, 5), q_avg (5)) with columns Q_ext, Q_abs,
        Q_sca, Q_bks, g."""
        S = np.asfortranarray(S, dtype=np.complex128)
        ntr = tr_grid[0] * tr_grid[1]
        arrs = [_c(a, np.float64) for a in (tr_th, tr_ph, rx_th, rx_ph, cext, cabs)]
        wt = _c(w_tr, np.float64) if w_tr is not None else None
        wr = _c(w_rx, np.float64) if w_rx is not None else None
        qd, qa = np.zeros((ntr, 5)), np.zeros(5)
        self._ck(self.L.midas_gpu_scattering_quantities(
            self.h, _lib.QUAD[quad_tr], _lib.QUAD[quad_rx], tr_grid[0], tr_grid[1], addr(arrs[0]), addr(arrs[1]),
            rx_grid[0], rx_grid[1], S.shape[0], addr(arrs[2]), addr(arrs[3]), addr(S), addr(arrs[4]),
            addr(arrs[5]), float(dm), float(k0), int(cext_intfields), addr(wt) if wt is not None else None,
            addr(wr) if wr is not None else None, addr(qd), addr(qa)))
        return qd, qa

    def launch_count(self) -> int:
        return int(self.L.midas_gpu_launch_count(self.h))

    def profile(self, enable: bool = True):
        """Start (clearing the totals) or stop per-kernel-class device timing."""
        self._ck(self.L.midas_gpu_profile(self.h, 1 if enable else 0))

    def profile_query(self) -> dict:
        """{class: {ms, flops, bytes, launches}} since profiling was enabled."""
        out = {}
        for k, name in enumerate(_lib.KCLASSES):
            ms, fl, by, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
            self._ck(self.L.midas_gpu_profile_query(self.h, k, ctypes.byref(ms), ctypes.byref(fl), ctypes.byref(by),
                                                    ctypes.byref(n)))
            if n.value:
                out[name] = {"ms": ms.value, "flops": fl.value, "bytes": by.value, "launches": n.value}
        return out

    def wait_event(self, event: int):
        """Order the context's later work after a caller's cudaEvent_t (an integer handle,
        e.g. torch.cuda.Event().cuda_event once recorded) without a host wait."""
        self._ck(self.L.midas_gpu_wait_event(self.h, ctypes.c_void_p(event)))

    def record_event(self, event: int):
        """Record a caller's cudaEvent_t on the context stream after the work issued so far."""
        self._ck(self.L.midas_gpu_record_event(self.h, ctypes.c_void_p(event)))

    def stream_handle(self) -> int:
        """cudaStream_t of the context (wrap with torch.cuda.ExternalStream to time on it)."""
        return int(self.L.midas_gpu_stream(self.h) or 0)

    def bench_gemm(self, M, N, K, iters=20, f16=False) -> float:
        """Average ms per launch of one tensor-core GEMM (CUDA events on the context stream);
        fp16 operands (the LU trailing-update path) when f16."""
        ms = ctypes.c_double(0)
        self._ck(self.L.midas_gpu_bench_gemm_ex(self.h, M, N, K, iters, int(bool(f16)), ctypes.byref(ms)))
        return ms.value

    def heev(self, A):
        """Hermitian eigen-decomposition on the device: (W descending, V columns)."""
        A = np.ascontiguousarray(A, dtype=np.complex128)
        m = A.shape[0]
        W = np.zeros(m)
        V = np.zeros((m, m), np.complex128)
        self._ck(self.L.midas_gpu_heev(self.h, m, addr(A), addr(W), addr(V)))
        return W, V

    def zgemm_x3(self, A, B):
        """FP32-grade complex product on the tensor cores (split TF32)."""
        A = np.ascontiguousarray(A, dtype=np.complex128)
        B = np.ascontiguousarray(B, dtype=np.complex128)
        D = np.zeros((A.shape[0], B.shape[1]), np.complex128)
        self._ck(self.L.midas_gpu_zgemm_x3(self.h, A.shape[0], B.shape[1], A.shape[1], addr(A), addr(B), addr(D)))
        return D

    def gemm_selftest(self):
        self._ck(self.L.midas_gpu_gemm_selftest(self.h))
        return self.L.midas_gpu_gemm_engine().decode()


def compute_efields_mom(ctx: Context, th, ph, rth, rph):
    """Compute_EFields_MoM (src/Compute_EFields_MoM.f90:1-427): returns
    (E_total, S_total, C_ext, C_abs) with the reference's layouts."""
    E = ctx.mom_solve(th, ph)
    S = ctx.smatrix(rth, rph, E)
    ce, ca = ctx.cext_cabs(th, ph, E)
    return E, S, ce, ca


def compute_efields_cbfme(ctx: Context, blk_offsets, ext_lists, cbf_th, cbf_ph, th, ph, **kw):
    """Compute_EFields_CBFME (src/Compute_EFields_CBFME.f90:1-1006): (E_total, K_patchs)."""
    return ctx.cbfm_solve(blk_offsets, ext_lists, cbf_th, cbf_ph, th, ph, **kw)
