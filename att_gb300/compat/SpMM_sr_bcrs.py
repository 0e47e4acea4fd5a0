"""Drop-in for the reference extension ``SpMM_sr_bcrs``
(gcn/SpMM/src/benchmark.cpp, pybind11 module at :490-495; built by
gcn/setup.py:17).

``forward_{fp16,tf32}_gnn[_acc](row_offsets, col_indices, values, t_window_row,
t_atomic, rhs_matrix, dimM1, dimN, mOri)`` returns ``[Y]`` with Y a new fp32
CUDA tensor of shape [mOri, dimN] (benchmark.cpp:35-75), computed on tensor
cores with fp32 accumulation.  The format is the reference's: 8-row windows,
8-wide (fp16) or 4-wide (tf32) blocks.  The "_acc" variants accept any dimN
(spmmKernel.cu:2066-2330); here every variant does, by padding the feature
dimension to the kernel's granule on the device.
"""
import torch

from att_gb300 import ops


def _check(t, name):
    if not isinstance(t, torch.Tensor) or t.device.type != "cuda":
        raise TypeError("%s must be a CUDA tensor" % name)


def _forward(row_offsets, col_indices, values, t_window_row, t_atomic, rhs_matrix, dimN, mOri,
             x_dtype, wide, granule):
    for t, n in ((row_offsets, "row_offsets"), (col_indices, "col_indices"), (values, "values"),
                 (t_window_row, "t_window_row"), (t_atomic, "t_atomic"),
                 (rhs_matrix, "rhs_matrix")):
        _check(t, n)
    if rhs_matrix.dtype != x_dtype:
        raise TypeError("rhs_matrix must be %s" % x_dtype)
    dimN, mOri = int(dimN), int(mOri)
    X = rhs_matrix.reshape(-1, dimN)
    Fp = (dimN + granule - 1) // granule * granule
    if Fp != dimN:
        X = torch.nn.functional.pad(X, (0, Fp - dimN))
    Y = ops.spmm(row_offsets.contiguous(), col_indices.contiguous(), values.contiguous(),
                 t_window_row.contiguous(), t_atomic.contiguous(), X, mOri, window=8, wide=wide)
    if Fp != dimN:
        Y = Y[:, :dimN].contiguous()
    return [Y]


def forward_fp16_gnn(row_offsets, col_indices, values, t_window_row, t_atomic, rhs_matrix,
                     dimM1, dimN, mOri):
    """benchmark.cpp:35-75 -> spmmKernel.cu:1693-1727."""
    return _forward(row_offsets, col_indices, values, t_window_row, t_atomic, rhs_matrix, dimN,
                    mOri, torch.float16, 8, 8)


def forward_tf32_gnn(row_offsets, col_indices, values, t_window_row, t_atomic, rhs_matrix,
                     dimM1, dimN, mOri):
    """benchmark.cpp:91-130 -> spmmKernel.cu:1731-1765 (here 3xTF32)."""
    return _forward(row_offsets, col_indices, values, t_window_row, t_atomic, rhs_matrix, dimN,
                    mOri, torch.float32, 4, 4)


def forward_fp16_gnn_acc(row_offsets, col_indices, values, t_window_row, t_atomic, rhs_matrix,
                         dimM1, dimN, mOri):
    """benchmark.cpp:259-296 -> spmmKernel.cu:2175-2209."""
    return forward_fp16_gnn(row_offsets, col_indices, values, t_window_row, t_atomic,
                            rhs_matrix, dimM1, dimN, mOri)


def forward_tf32_gnn_acc(row_offsets, col_indices, values, t_window_row, t_atomic, rhs_matrix,
                         dimM1, dimN, mOri):
    """benchmark.cpp:305-335 -> spmmKernel.cu:2332-2366."""
    return forward_tf32_gnn(row_offsets, col_indices, values, t_window_row, t_atomic,
                            rhs_matrix, dimM1, dimN, mOri)
