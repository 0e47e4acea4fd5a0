"""Drop-in for the reference extension ``ATT_SpMM_v1`` (prebuilt only in the
reference).  Its functions have the same names, arguments and meaning as
``ATT_SpMM_v3`` (the v1 callers, end2end_ori/gat_final/mgat_csr/mgat_conv.py,
call the same ops), so this module re-exports them."""
from att_gb300.compat.ATT_SpMM_v3 import (  # noqa: F401
    spmm_fp16_h_m, spmm_fp16_h_m_rowsum, spmm_fp16_m_h, spmm_fp16_m_h_rowsum, spmm_tf32_h_m,
    spmm_tf32_h_m_rowsum, spmm_tf32_m_h, spmm_tf32_m_h_rowsum)
