"""att_gb300 -- the ATT tensor-core sparse hot path on GB300 (sm_103a).

CSR -> row-window block conversion, blocked SpMM, and the GAT
SDDMM / edge-softmax / SpMM chain, as hand-written CUDA behind the C ABI in
include/att_gb300.h.  There is no CPU fallback.
"""
from . import _lib
from .ops import BlockFormat, block_convert, spmm, spmm_format, require_cuda

__all__ = ["BlockFormat", "block_convert", "spmm", "spmm_format", "require_cuda", "build"]


def build(verbose=False):
    from . import builder as _b
    return _b.build(verbose=verbose)
