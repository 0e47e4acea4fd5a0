"""The reference's own GCN SpMM kernel on the GPU: the "plain FP16 drop-in".

COMPARISON AND TEST INFRASTRUCTURE ONLY (the plain drop-in the bench times
beside the product).  ``oracle/build_ref.py`` compiles the reference's
``gcn/SpMM/src/spmmKernel.cu`` (unmodified, from the reference tree) into the
device-only fatbin ``oracle/_ref/ref_spmm.fatbin`` for sm_103a.
This module loads that fatbin through the CUDA driver API (ctypes over
libcuda) and launches its kernels exactly as the reference's binding and
launcher do:

* ``forward_fp16_gnn`` -- benchmark.cpp:35-75 (output ``torch.zeros`` fp32
  [mOri, dimN], parts = len(window)) and the launcher
  ``spmm_forward_cuda_fp16_balance_gnn`` spmmKernel.cu:1693-1727: dimN padded
  to a multiple of 16 (n1), grid (ceil(n1/64), splitk, parts/splitk + 1) with
  splitk = 8 below 500,000 parts else (parts/1,250,000 + 1) * 20, 128 threads,
  kernel ``spmm_forward_cuda_kernel_fp16_balance<64>`` (spmmKernel.cu:158-265),
  fp16 inputs passed as double pointers.
* ``forward_tf32_gnn`` -- benchmark.cpp:91-130 and spmmKernel.cu:1731-1765,
  kernel ``spmm_forward_cuda_kernel_tf32_balance<64>`` (spmmKernel.cu:959-1075).

The kernels launch on torch's current stream (the reference used the legacy
default stream).  Memory safety on the block format of this repository was
checked by reading the kernels: full 8-column steps touch only real columns,
the residue step zero-fills padding (-1) columns, feature reads stay below
dimN when dimN is a multiple of 16, and every output store is bounds-checked
against mOri and dimN.  The wrappers refuse any other dimN.

Nothing here is imported by the ``att_gb300`` package.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
FATBIN = os.path.join(HERE, "_ref", "ref_spmm.fatbin")
_KERNELS = {
    "fp16": "_Z37spmm_forward_cuda_kernel_fp16_balanceILi64EE",
    "tf32": "_Z37spmm_forward_cuda_kernel_tf32_balanceILi64EE",
}
_state = {}


def available():
    return os.path.isfile(FATBIN)


def _check(rc, what):
    if rc != 0:
        lib = _state.get("cuda")
        msg = ctypes.c_char_p()
        if lib is not None:
            lib.cuGetErrorString(rc, ctypes.byref(msg))
        raise RuntimeError("%s failed: %d %s" % (what, rc, msg.value.decode() if msg.value else ""))


def _load():
    """Load the fatbin into the current (torch primary) context and look up the
    two kernels by their mangled-name prefix."""
    if "funcs" in _state:
        return _state["funcs"]
    if not available():
        raise RuntimeError("reference SpMM fatbin not built: " + FATBIN)
    import torch
    torch.cuda.init()
    torch.zeros(1, device="cuda")  # makes torch's primary context current here
    lib = ctypes.CDLL("libcuda.so.1")
    _state["cuda"] = lib
    _check(lib.cuInit(0), "cuInit")
    ctx = ctypes.c_void_p()
    _check(lib.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
    if not ctx.value:
        raise RuntimeError("no current CUDA context")
    mod = ctypes.c_void_p()
    _check(lib.cuModuleLoad(ctypes.byref(mod), FATBIN.encode()), "cuModuleLoad")
    count = ctypes.c_uint()
    _check(lib.cuModuleGetFunctionCount(ctypes.byref(count), mod), "cuModuleGetFunctionCount")
    arr = (ctypes.c_void_p * count.value)()
    _check(lib.cuModuleEnumerateFunctions(arr, count, mod), "cuModuleEnumerateFunctions")
    funcs = {}
    for f in arr:
        name = ctypes.c_char_p()
        _check(lib.cuFuncGetName(ctypes.byref(name), ctypes.c_void_p(f)), "cuFuncGetName")
        for key, prefix in _KERNELS.items():
            if name.value and name.value.decode().startswith(prefix):
                funcs[key] = ctypes.c_void_p(f)
    missing = set(_KERNELS) - set(funcs)
    if missing:
        raise RuntimeError("kernels not found in the reference fatbin: %s" % sorted(missing))
    lib.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [
        ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
    _state["mod"] = mod
    _state["funcs"] = funcs
    return funcs


def _grid(n_parts, dimN):
    """The reference launcher's grid (spmmKernel.cu:1706-1715)."""
    n1 = dimN if dimN % 16 == 0 else (dimN // 16 + 1) * 16
    grid_x = n1 // 64 + (0 if n1 % 64 == 0 else 1)
    splitk = 8 if n_parts < 500_000 else (n_parts // 1_250_000 + 1) * 20
    return n1, (grid_x, splitk, n_parts // splitk + 1), splitk


def _launch(kind, rowptr, col, val, window, atomic, X, dimN, mOri, out):
    import torch
    funcs = _load()
    if dimN % 16:
        raise ValueError("the reference kernels read whole 16-feature groups: dimN % 16 must be 0")
    tensors = (rowptr, col, val, window, atomic, X)
    if any((not t.is_cuda) or (not t.is_contiguous()) for t in tensors):
        raise ValueError("inputs must be contiguous CUDA tensors")
    if X.shape[1] != dimN or out.shape != (mOri, dimN):
        raise ValueError("shape mismatch")
    n_parts = int(window.shape[0])
    n1, grid, splitk = _grid(n_parts, dimN)
    if grid[2] >= 65536:
        raise ValueError("grid.z beyond the launch limit")
    args = [ctypes.c_void_p(t.data_ptr()) for t in (rowptr, col, val, window, atomic, X, out)]
    args += [ctypes.c_int(n1), ctypes.c_int(n_parts), ctypes.c_long(dimN), ctypes.c_int(mOri),
             ctypes.c_int(splitk)]
    params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p)
                                            for a in args])
    stream = torch.cuda.current_stream().cuda_stream
    lib = _state["cuda"]
    _check(lib.cuLaunchKernel(funcs[kind], grid[0], grid[1], grid[2], 128, 1, 1, 0,
                              ctypes.c_void_p(stream), params, None), "cuLaunchKernel")
    return out


def forward_fp16_gnn(rowptr, col, val, window, atomic, X, dimM1, dimN, mOri):
    """SpMM_sr_bcrs.forward_fp16_gnn of the reference: [Y] with Y fp32 zeros
    [mOri, dimN] accumulated from the fp16 block format and fp16 X."""
    import torch
    if val.dtype != torch.float16 or X.dtype != torch.float16:
        raise ValueError("fp16 values and features expected")
    out = torch.zeros(mOri, dimN, device="cuda", dtype=torch.float32)
    return [_launch("fp16", rowptr, col, val, window, atomic, X, dimN, mOri, out)]


def forward_tf32_gnn(rowptr, col, val, window, atomic, X, dimM1, dimN, mOri):
    """SpMM_sr_bcrs.forward_tf32_gnn of the reference (fp32 values in 8x4
    blocks, fp32 X fed to TF32 tensor cores)."""
    import torch
    if val.dtype != torch.float32 or X.dtype != torch.float32:
        raise ValueError("fp32 values and features expected")
    out = torch.zeros(mOri, dimN, device="cuda", dtype=torch.float32)
    return [_launch("tf32", rowptr, col, val, window, atomic, X, dimN, mOri, out)]
