"""Drop-in for the reference extension ``Block_sr_bcrs``
(gcn/Block_gcn/example.cpp, pybind11 module at :353-357; built by
gcn/setup.py:10).

Same functions, argument meaning and return value (a list of five new CPU
tensors ``[row_pointers, column_index, values, t_window_row, t_atomic]``),
computed by the GPU conversion and copied back.  ``device="cuda"`` keeps the
result resident on the GPU instead (a superset of the reference API).
"""
import torch

from att_gb300 import ops


def _convert(row1, column1, degree1, window1, wide1, partSize_t, emit_empty, device):
    if degree1.dim() != 1:
        raise ValueError("degree must be 1-D")
    fmt = ops.block_convert(row1, column1, degree1, window=int(window1), wide=int(wide1),
                            part=int(partSize_t), emit_empty=emit_empty)
    res = [fmt.rowptr, fmt.col, fmt.val, fmt.window_of_part, fmt.atomic]
    if device is not None and torch.device(device).type == "cuda":
        return res
    return [t.cpu() for t in res]


def blockProcess_fp16_balance(row1, column1, degree1, window1, wide1, partSize_t, device=None):
    """example.cpp:48-200: fp16 degrees -> fp16 values half(d_i*d_j);
    empty windows emit no part."""
    if degree1.dtype != torch.float16:
        raise TypeError("blockProcess_fp16_balance expects float16 degrees")
    return _convert(row1, column1, degree1, window1, wide1, partSize_t, False, device)


def blockProcess_tf32_balance(row1, column1, degree1, window1, wide1, partSize_t, device=None):
    """example.cpp:203-348: fp32 degrees -> fp32 values; an empty window
    emits a (0,0) part."""
    if degree1.dtype != torch.float32:
        raise TypeError("blockProcess_tf32_balance expects float32 degrees")
    return _convert(row1, column1, degree1, window1, wide1, partSize_t, True, device)
