"""Drop-in for the reference extension ``ATT_Block_gpu`` (GPU preprocessing;
source absent: Block_gpu/setup.py:5-19 names DTCSpMM.cpp / DTCSpMM_kernel.cu).

``preprocess_gpu_fs(row, col, N, nnz, window, wide, partSize)`` as called at
end2end_overhead/gat_final/mgat_csr_ov/mdataset_fp16.py:53-58 returns
``[row_pointers, column_index, degrees, degrees_trans, window, automic, pre]``
with the format resident on the GPU and ``pre`` the conversion time in ms
(CUDA events around the conversion).
"""
import torch

from att_gb300.compat import _gat_common as _g


def preprocess_gpu_fs(row, col, N, nnz, window, wide, partSize):
    row = row.cuda()
    col = col.cuda()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    res = _g.convert(row, col, window, wide, partSize, True, device="cuda")
    t1.record()
    torch.cuda.synchronize()
    return res + [t0.elapsed_time(t1)]
