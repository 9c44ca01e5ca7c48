"""The C-ABI library builds, loads and exports every symbol the header declares
(no GPU needed: nothing here launches a kernel)."""
import os
import re

from midas_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    h = open(os.path.join(ROOT, "include", "midas_gpu.h")).read()
    h = re.sub(r"/\*.*?\*/", "", h, flags=re.S)
    return sorted(set(re.findall(r"\b(midas_gpu_\w+)\s*\(", h)))


def test_library_exports_header(gpulib):
    syms = header_symbols()
    assert len(syms) >= 18
    missing = [s for s in syms if not hasattr(gpulib, s)]
    assert not missing, missing
    assert sorted(_lib.EXPORTS) == syms


def test_default_opts(gpulib):
    import ctypes
    o = _lib.Opts()
    gpulib.midas_gpu_default_opts(ctypes.byref(o))
    assert o.struct_size == ctypes.sizeof(_lib.Opts)
    assert o.solve_mode == _lib.SOLVE_MIXED and o.ir_max_iter == 30 and o.ir_tol == 1e-13


def test_init_rejects_bad_opts(gpulib):
    import ctypes
    o = _lib.Opts()
    gpulib.midas_gpu_default_opts(ctypes.byref(o))
    o.index_base = 7
    h = ctypes.c_void_p()
    assert gpulib.midas_gpu_init(ctypes.byref(o), ctypes.byref(h)) == 1   # MIDAS_ERR_ARG, before any device call
    assert gpulib.midas_gpu_free(None) == 0
    assert gpulib.midas_gpu_wait_event(None, None) == 1 and gpulib.midas_gpu_record_event(None, None) == 1
    assert gpulib.midas_gpu_last_error(None) == b"null context"
