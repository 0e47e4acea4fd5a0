"""ctypes binding of libattgb300.so (the C ABI declared in include/att_gb300.h).

There is no CPU fallback: if the library is missing or no CUDA device is
present, every op raises.
"""
import ctypes
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libattgb300.so")

# enum att_dtype
F32, F16, BF16, F8E4M3, I32, NONE = 0, 1, 2, 3, 4, -1
# enum att_status
OK = 0

_c_i64 = ctypes.c_int64
_c_int = ctypes.c_int
_c_vp = ctypes.c_void_p
_c_sz = ctypes.c_size_t

_SIGNATURES = {
    "att_status_string": (ctypes.c_char_p, [_c_int]),
    "att_last_error": (ctypes.c_char_p, []),
    "att_version": (_c_int, []),
    "att_set_option": (_c_int, [ctypes.c_char_p, _c_int]),
    "att_set_thread_option": (_c_int, [ctypes.c_char_p, _c_int]),
    "att_get_option": (_c_int, [ctypes.c_char_p, ctypes.POINTER(_c_int)]),
    "att_block_workspace_bytes": (_c_sz, [_c_i64, _c_i64, _c_i64, _c_int]),
    "att_block_plan": (_c_int, [_c_vp, _c_vp, _c_i64, _c_i64, _c_i64, _c_int, _c_int, _c_int,
                                _c_int, _c_vp, _c_sz, ctypes.POINTER(_c_i64),
                                ctypes.POINTER(_c_i64), _c_vp]),
    "att_block_plan_async": (_c_int, [_c_vp, _c_vp, _c_i64, _c_i64, _c_i64, _c_int, _c_int,
                                      _c_int, _c_int, _c_vp, _c_sz, _c_vp, _c_vp]),
    "att_block_plan_result": (_c_int, [_c_vp, _c_i64, _c_int, ctypes.POINTER(_c_i64),
                                       ctypes.POINTER(_c_i64)]),
    "att_block_fill": (_c_int, [_c_vp, _c_vp, _c_i64, _c_i64, _c_i64, _c_int, _c_int, _c_int,
                                _c_int, _c_vp, _c_int, _c_vp, _c_sz, _c_vp, _c_vp, _c_vp, _c_int,
                                _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "att_block_fill_async": (_c_int, [_c_vp, _c_vp, _c_i64, _c_i64, _c_i64, _c_int, _c_int,
                                      _c_int, _c_int, _c_vp, _c_int, _c_vp, _c_sz, _c_i64,
                                      _c_i64, _c_vp, _c_vp, _c_vp, _c_int, _c_vp, _c_vp, _c_vp,
                                      _c_vp, _c_vp, _c_vp, _c_vp]),
    "att_block_fill_result": (_c_int, [_c_vp, _c_int]),
    "att_block_convert_noalloc_max_scratch": (_c_sz, []),
    "att_block_convert_noalloc": (_c_int, [_c_vp, _c_vp, _c_i64, _c_i64, _c_i64, _c_int, _c_int,
                                           _c_int, _c_int, _c_vp, _c_int, _c_vp, _c_vp, _c_vp,
                                           _c_int, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_i64,
                                           _c_i64, ctypes.POINTER(_c_i64),
                                           ctypes.POINTER(_c_i64), _c_vp]),
    "att_spmm": (_c_int, [_c_vp, _c_vp, _c_vp, _c_int, _c_vp, _c_vp, _c_i64, _c_vp, _c_int,
                          _c_vp, _c_i64, _c_i64, _c_i64, _c_vp, _c_i64, _c_i64, _c_int, _c_int,
                          _c_vp, _c_vp]),
    "att_node_scores_pair": (_c_int, [_c_vp, _c_int, _c_i64, _c_i64, _c_i64, _c_i64, _c_i64,
                                      _c_vp, _c_vp, _c_i64, _c_vp, _c_vp, _c_i64, _c_vp]),
    "att_node_scores": (_c_int, [_c_vp, _c_int, _c_i64, _c_i64, _c_i64, _c_i64, _c_i64, _c_vp,
                                 _c_int, _c_i64, _c_vp, _c_i64, _c_vp]),
    "att_slot_edges": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_i64, _c_int, _c_int, _c_int,
                                _c_vp, _c_vp, _c_i64, _c_vp, _c_int, _c_i64, _c_i64, _c_i64,
                                _c_i64, _c_vp, _c_int, _c_i64, _c_i64, _c_vp]),
    "att_sddmm": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_i64, _c_int, _c_int, _c_vp, _c_vp,
                           _c_int, _c_i64, _c_i64, _c_i64, _c_i64, _c_i64, _c_i64, _c_i64,
                           _c_i64, _c_vp, _c_int, _c_i64, _c_i64, _c_vp, _c_vp]),
    "att_gather_slot_values": (_c_int, [_c_vp, _c_i64, _c_int, _c_int, _c_int, _c_vp, _c_int,
                                        _c_i64, _c_i64, _c_i64, _c_vp, _c_int, _c_i64, _c_vp]),
    "att_rowsum": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_i64, _c_int, _c_int, _c_vp, _c_int,
                            _c_i64, _c_i64, _c_i64, _c_vp, _c_i64, _c_i64, _c_i64, _c_vp]),
    "att_slot_mask": (_c_int, [_c_vp, _c_i64, _c_vp, _c_i64, _c_vp]),
    "att_edge_softmax": (_c_int, [_c_vp, _c_i64, _c_vp, _c_i64, _c_i64, ctypes.c_float, _c_int,
                                  _c_vp, _c_int, _c_i64, _c_vp, _c_vp, _c_vp]),
    "att_gat_grad_prepare": (_c_int, [_c_vp, _c_i64, _c_vp, _c_i64, _c_i64, _c_i64, _c_i64, _c_vp,
                                      _c_vp, _c_int, _c_i64, _c_vp, _c_vp]),
    "att_gat_grad_finish": (_c_int, [_c_vp, _c_i64, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_int,
                                     _c_i64, _c_i64, _c_i64, _c_i64, _c_vp, _c_i64, _c_vp, _c_vp,
                                     _c_vp]),
    "att_gat_forward": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_i64, _c_vp, _c_vp, _c_i64, _c_vp,
                                 _c_i64, _c_int, _c_int, _c_vp, _c_int, _c_i64, _c_i64, _c_i64,
                                 _c_i64, _c_int, _c_vp, _c_vp, ctypes.c_float, _c_vp, _c_i64,
                                 _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "att_gat_backward": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_i64, _c_int, _c_int, _c_vp,
                                  _c_vp, _c_vp, _c_int, _c_i64, _c_i64, _c_i64, _c_i64, _c_i64, _c_vp,
                                  _c_vp, _c_vp, _c_vp, _c_vp, ctypes.c_float, _c_vp, _c_i64,
                                  _c_vp, _c_vp, _c_vp, _c_vp]),
    "att_spmm_groups_scratch_bytes": (_c_sz, [_c_i64, _c_i64]),
    "att_spmm_groups": (_c_int, [_c_vp, _c_i64, _c_i64, _c_int, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                 _c_vp, _c_sz, _c_vp]),
    "att_host_device_pointer": (_c_int, [_c_vp, ctypes.POINTER(_c_vp)]),
    "att_spmm_batched_grid": (_c_sz, []),
    "att_spmm_batched": (_c_int, [_c_vp, _c_vp, _c_i64, _c_int, _c_int, _c_vp, _c_vp]),
}


class SpmmJob(ctypes.Structure):
    """Mirror of att_spmm_job (include/att_gb300.h)."""
    _fields_ = [("rowptr", _c_vp), ("col", _c_vp), ("val", _c_vp), ("window_of_part", _c_vp),
                ("n_parts", _c_i64), ("group_part", _c_vp), ("group_slot", _c_vp),
                ("red_first", _c_vp), ("empty_win", _c_vp), ("partial", _c_vp),
                ("n_groups", _c_i64), ("n_red", _c_i64), ("n_slots", _c_i64), ("n_empty", _c_i64),
                ("X", _c_vp), ("n_x", _c_i64), ("F", _c_i64), ("ldx", _c_i64), ("Y", _c_vp),
                ("m_out", _c_i64), ("ldy", _c_i64), ("item_begin", _c_i64),
                ("empty_begin", _c_i64), ("red_begin", _c_i64)]

_lib = None


class AttError(RuntimeError):
    """A C-ABI call returned a non-zero att_status."""

    def __init__(self, fn, status, msg):
        super().__init__("%s failed (status %d: %s): %s" % (fn, status, _status_name(status), msg))
        self.status = status


def _status_name(status):
    try:
        return lib().att_status_string(status).decode()
    except Exception:  # pragma: no cover - library unavailable
        return "?"


def declared_symbols():
    return sorted(_SIGNATURES)


def load(path=None):
    """Load the shared library (raises OSError if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise OSError("libattgb300.so not built (expected at %s); run "
                      "`python -c 'import __graft_entry__ as g; g.build()'`" % path)
    handle = ctypes.CDLL(path)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(handle, name)
        fn.restype = res
        fn.argtypes = args
    _lib = handle
    return _lib


def lib():
    return load()


def call(name, *args):
    """Call a C-ABI function; raise AttError on a non-zero status."""
    fn = getattr(lib(), name)
    status = fn(*args)
    if status != OK:
        raise AttError(name, status, lib().att_last_error().decode())
    return status
