"""GB300 (sm_103a) implementation of the MIDAS VIE-MoM / CBFM hot path.

``midas_gb300.solver.Context`` drives the CUDA library ``libmidas_gpu.so``
(C ABI in include/midas_gpu.h); ``midas_gb300.geometry`` prepares cells and
CBFM partitions.
"""
import os as _os

# The library's CBFM pipeline runs ~20 CUDA streams; the CUDA default of 8 hardware work
# queues makes streams share queues, so a long kernel on one holds up the others.  The
# setting must precede the process's first CUDA context (torch's included).
_os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from . import geometry  # noqa: E402,F401
