"""snac_gb300 -- GB300 (sm_103a) implementation of SNaC's per-time-step hot path.

The compute runs in hand-written CUDA kernels inside libsnac_gb300.so, reached
through the C ABI of include/snac_gpu.h.  This package holds the Python view
of that ABI: ``capi`` (ctypes declarations), ``hotpath`` (the reference's
subroutine interfaces on numpy arrays), ``domain`` (all blocks resident on the
GPU, whole RK3 steps) and ``cases`` (the namelist inputs of the benchmark and
test cases).
"""
from . import cases  # noqa: F401

__all__ = ["cases", "capi", "hotpath", "domain", "build"]


def build(verbose: bool = False) -> str:
    """Compile libsnac_gb300.so for sm_103a in-tree and return its path."""
    from . import _build
    return _build.build(verbose=verbose)
