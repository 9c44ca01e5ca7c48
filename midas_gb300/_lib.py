"""ctypes binding of libmidas_gpu.so (the C ABI declared in include/midas_gpu.h).

The GPU library is the only compute path: if it is missing this module raises,
it never substitutes a CPU implementation.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmidas_gpu.so")

MIDAS_OK = 0
STATUS = {0: "MIDAS_OK", 1: "MIDAS_ERR_ARG", 2: "MIDAS_ERR_CUDA", 3: "MIDAS_ERR_ALLOC", 4: "MIDAS_ERR_SINGULAR",
          5: "MIDAS_ERR_NOT_CONVERGED", 6: "MIDAS_ERR_STATE", 7: "MIDAS_ERR_DEVICE_TIMEOUT",
          8: "MIDAS_ERR_UNSUPPORTED"}
SOLVE_MIXED, SOLVE_FP64 = 0, 1
FILL_FAITHFUL, FILL_FAST = 0, 1
CBFM_SR, CBFM_HOMOG, CBFM_ACA, CBFM_FAST_CBF, CBFM_SPHERICAL = 1, 2, 4, 8, 16
GMRES_JACOBI = 1
# integration rules NumIntType_t / NumIntType_r (MIDAS_QUAD_* in the header)
QUAD = {"un": 0, "tr": 1, "gl": 2, "sd": 3, "lb": 4, "rf": 5}
# kernel classes of midas_gpu_profile_query (MIDAS_KC_* in the header)
KCLASSES = ["gemm_trail", "gemm_simt", "fill", "sr_scan", "diag_lu", "trsv", "resid", "zgemm64", "eig", "other",
            "gemm_panel", "gemm_solve", "gemm_prod", "split", "lattice", "nn", "resid32"]

# every symbol the header declares (checked by the CPU tests)
EXPORTS = [
    "midas_gpu_default_opts", "midas_gpu_init", "midas_gpu_free", "midas_gpu_last_error", "midas_gpu_set_cells",
    "midas_gpu_get_cell_params", "midas_gpu_mom_fill", "midas_gpu_mom_rhs", "midas_gpu_incident_field",
    "midas_gpu_incident_field_spherical", "midas_gpu_voxelise_sphere", "midas_gpu_voxelise_spheres",
    "midas_gpu_box_partition", "midas_gpu_extend_blocks",
    "midas_gpu_block_fill", "midas_gpu_sr_fill", "midas_gpu_set_fsr", "midas_gpu_aca", "midas_gpu_dense_solve",
    "midas_gpu_mom_solve", "midas_gpu_lattice_matvec", "midas_gpu_gmres_solve", "midas_gpu_nn_create", "midas_gpu_nn_free",
    "midas_gpu_nn_param_count", "midas_gpu_nn_params", "midas_gpu_nn_forward", "midas_gpu_nn_gradients",
    "midas_gpu_nn_train_step", "midas_gpu_nn_prec_grid", "midas_gpu_fgmres_solve", "midas_gpu_cbfm_solve", "midas_gpu_dense_solve_noalloc", "midas_gpu_cext_cabs", "midas_gpu_smatrix",
    "midas_gpu_scattering_quantities", "midas_gpu_wait_event", "midas_gpu_record_event",
    "midas_gpu_gemm_selftest", "midas_gpu_gemm_engine", "midas_gpu_wait_selftest", "midas_gpu_launch_count", "midas_gpu_stream",
    "midas_gpu_bench_gemm", "midas_gpu_bench_gemm_ex", "midas_gpu_heev", "midas_gpu_zgemm_x3", "midas_gpu_profile", "midas_gpu_profile_query",
]


class Opts(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_int), ("device", ctypes.c_int), ("index_base", ctypes.c_int),
                ("solve_mode", ctypes.c_int), ("fill_mode", ctypes.c_int), ("ir_max_iter", ctypes.c_int),
                ("ir_tol", ctypes.c_double), ("verbose", ctypes.c_int)]


class Info(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("ir_iters", ctypes.c_int), ("backward_error", ctypes.c_double),
                ("anorm", ctypes.c_double), ("k_total", ctypes.c_int), ("n_far_aca", ctypes.c_int),
                ("t_fill_ms", ctypes.c_double), ("t_factor_ms", ctypes.c_double), ("t_solve_ms", ctypes.c_double),
                ("t_total_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class MidasError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


_lib = None


def load(path: str = LIB_PATH):
    """Load the library (raises when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} not found: build it with `python -m midas_gb300.build`")
    L = ctypes.CDLL(path)
    vp, ip, dp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double
    P = ctypes.c_void_p   # array arguments are passed as raw addresses (host or device)
    sigs = {
        "midas_gpu_default_opts": (None, [ctypes.POINTER(Opts)]),
        "midas_gpu_init": (i, [ctypes.POINTER(Opts), ctypes.POINTER(vp)]),
        "midas_gpu_free": (i, [vp]),
        "midas_gpu_last_error": (ctypes.c_char_p, [vp]),
        "midas_gpu_set_cells": (i, [vp, i, P, P, P, P, P, P, d]),
        "midas_gpu_get_cell_params": (i, [vp, P, P, P, P]),
        "midas_gpu_mom_fill": (i, [vp, i, i, i, i, P]),
        "midas_gpu_mom_rhs": (i, [vp, i, P, P, P]),
        "midas_gpu_incident_field": (i, [vp, i, P, i, P, P, P]),
        "midas_gpu_incident_field_spherical": (i, [vp, i, P, i, P, P, P]),
        "midas_gpu_voxelise_sphere": (i, [vp, d, d, ctypes.c_longlong, P, P, P, ctypes.POINTER(ctypes.c_longlong)]),
        "midas_gpu_voxelise_spheres": (i, [vp, i, P, d, i, ctypes.c_longlong, P, P, P,
                                           ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_double)]),
        "midas_gpu_box_partition": (i, [vp, i, P, P, P, i, i, i, P, P, ctypes.POINTER(ctypes.c_int)]),
        "midas_gpu_extend_blocks": (i, [vp, i, P, P, P, i, P, d, d, P, ctypes.c_longlong, P,
                                        ctypes.POINTER(ctypes.c_longlong)]),
        "midas_gpu_block_fill": (i, [vp, i, P, i, P, P]),
        "midas_gpu_sr_fill": (i, [vp, i, P, d, i, P, ctypes.POINTER(ctypes.c_longlong),
                                  ctypes.POINTER(ctypes.c_double)]),
        "midas_gpu_set_fsr": (i, [vp, i, P, i, d, ctypes.POINTER(ctypes.c_double),
                                  ctypes.POINTER(ctypes.c_longlong)]),
        "midas_gpu_aca": (i, [vp, i, i, i, i, d, i, P, P, ctypes.POINTER(ctypes.c_int)]),
        "midas_gpu_dense_solve": (i, [vp, i, i, P, P, ctypes.POINTER(Info)]),
        "midas_gpu_mom_solve": (i, [vp, i, P, P, P, ctypes.POINTER(Info)]),
        "midas_gpu_lattice_matvec": (i, [vp, i, P, P]),
        "midas_gpu_gmres_solve": (i, [vp, i, P, P, P, i, i, d, i, P, ctypes.POINTER(Info)]),
        "midas_gpu_nn_create": (i, [vp, i, ctypes.c_ulonglong, ctypes.POINTER(vp)]),
        "midas_gpu_nn_free": (i, [vp]),
        "midas_gpu_nn_param_count": (ctypes.c_longlong, [vp]),
        "midas_gpu_nn_params": (i, [vp, vp, i, P, i]),
        "midas_gpu_nn_forward": (i, [vp, vp, i, P, P, P]),
        "midas_gpu_nn_prec_grid": (i, [vp, vp, i, P, P, P, P]),
        "midas_gpu_fgmres_solve": (i, [vp, vp, i, P, P, P, i, i, d, P, ctypes.POINTER(Info)]),
        "midas_gpu_nn_gradients": (i, [vp, vp, i, P, P, P, ctypes.POINTER(ctypes.c_double)]),
        "midas_gpu_nn_train_step": (i, [vp, vp, i, P, P, P, ctypes.c_float, ctypes.POINTER(ctypes.c_double)]),
        "midas_gpu_dense_solve_noalloc": (i, [i, vp, i, i, P, P, ctypes.POINTER(ctypes.c_double)]),
        "midas_gpu_cbfm_solve": (i, [vp, i, P, P, P, i, P, P, d, d, i, d, i, i, P, P, P, P, ctypes.POINTER(Info)]),
        "midas_gpu_cext_cabs": (i, [vp, i, P, P, P, P, P]),
        "midas_gpu_smatrix": (i, [vp, i, P, P, i, P, P]),
        "midas_gpu_scattering_quantities": (i, [vp, i, i, i, i, P, P, i, i, i, P, P, P, P, P, d, d, i, P, P, P, P]),
        "midas_gpu_gemm_selftest": (i, [vp]),
        "midas_gpu_gemm_engine": (ctypes.c_char_p, []),
        "midas_gpu_wait_selftest": (i, [vp, i, ctypes.POINTER(ctypes.c_int)]),
        "midas_gpu_launch_count": (ctypes.c_longlong, [vp]),
        "midas_gpu_stream": (ctypes.c_void_p, [vp]),
        "midas_gpu_wait_event": (i, [vp, vp]),
        "midas_gpu_record_event": (i, [vp, vp]),
        "midas_gpu_bench_gemm": (i, [vp, i, i, i, i, ctypes.POINTER(ctypes.c_double)]),
        "midas_gpu_bench_gemm_ex": (i, [vp, i, i, i, i, i, ctypes.POINTER(ctypes.c_double)]),
        "midas_gpu_profile": (i, [vp, i]),
        "midas_gpu_profile_query": (i, [vp, i, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)]),
        "midas_gpu_heev": (i, [vp, i, P, P, P]),
        "midas_gpu_zgemm_x3": (i, [vp, i, i, i, P, P, P]),
    }
    for name, (res, args) in sigs.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def exported_symbols(path: str = LIB_PATH):
    L = ctypes.CDLL(path)
    return [s for s in EXPORTS if hasattr(L, s)]


def addr(a) -> int | None:
    """Raw address of a numpy array or torch tensor (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()   # torch tensor
