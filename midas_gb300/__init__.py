"""GB300 (sm_103a) implementation of the MIDAS VIE-MoM / CBFM hot path.

``midas_gb300.solver.Context`` drives the CUDA library ``libmidas_gpu.so``
(C ABI in include/midas_gpu.h); ``midas_gb300.geometry`` prepares cells and
CBFM partitions.
"""
from . import geometry  # noqa: F401
