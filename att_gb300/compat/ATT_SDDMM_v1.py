"""Drop-in for the reference extension ``ATT_SDDMM_v1`` (prebuilt only in the
reference).  Its functions have the same names, arguments and meaning as
``ATT_SDDMM_v3`` (the v1 callers, end2end_ori/gat_final/mgat_csr/mgat_conv.py,
call the same ops), so this module re-exports them."""
from att_gb300.compat.ATT_SDDMM_v3 import (  # noqa: F401
    att_fp16_h_nnz, att_tf32_h_nnz, attv2_fp16_h_nnz, attv2_tf32_h_nnz, sddmm_fp16_h_nnz,
    sddmm_fp16_ones_h_nnz, sddmm_tf32_h_nnz, sddmm_tf32_ones_h_nnz)
