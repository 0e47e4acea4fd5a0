"""Drop-in for the reference extension ``ATT_Block`` (GAT block format;
source absent from the reference: declared at Block/include/example.h:4-6,
built by setup.py:46; called as in
end2end_ori/gat_final/mgat_csr/mdataset_fp16.py:57-62 and
benchmark-v3/sddmm-benchmark/test/sddmm_fp16/test_sddmm_fp16.py:24).

``blockProcess_sddmm_balance_gnn(row, col, window, wide, partSize)`` returns
``[row_pointers, column_index, degrees, window, automic]``: the row-window
structure of the GCN conversion (empty windows emit no part) with
``degrees`` the slot -> CSR edge id map (-1 in empty slots, quad layout);
the ``_trans`` variant adds ``degrees_trans``, the edge id of the mirrored
edge (j, i) of each slot (i, j).  New CPU tensors, as the reference returns;
``device="cuda"`` keeps them on the GPU.
"""
from att_gb300.compat import _gat_common as _g


def blockProcess_sddmm_balance_gnn(row, col, window, wide, partSize, device=None):
    return _g.convert(row, col, window, wide, partSize, False, device)


def blockProcess_sddmm_balance_gnn_trans(row, col, window, wide, partSize, device=None):
    return _g.convert(row, col, window, wide, partSize, True, device)
