"""Recipe: compile the reference's own code for this path into ``oracle/_ref/``.

Test and baseline infrastructure only.  Two products, each compiled from the
reference tree where it lies (nothing is copied out of it), every build
product written under ``oracle/_ref/``:

* ``build()`` -- ``gcn/Block_gcn/example.cpp`` (``blockProcess_fp16_balance`` /
  ``blockProcess_tf32_balance``, example.cpp:48-348) as a torch CPU extension
  with OpenMP.  It pins the C restatement in ``oracle/block_oracle.c``, made
  the committed golden fixtures, and is the CPU conversion timed beside the
  GPU conversion.
* ``build_spmm()`` -- ``gcn/SpMM/src/spmmKernel.cu`` (the reference's GCN SpMM
  kernels, e.g. spmm_forward_cuda_kernel_fp16_balance, spmmKernel.cu:158-265)
  compiled by nvcc for sm_103a into a device-only fatbin,
  ``oracle/_ref/ref_spmm.fatbin``.  ``oracle/ref_spmm.py`` loads it with the
  CUDA driver API: it is the "plain FP16 drop-in" the GB300 kernels are
  measured and checked against.  A fatbin holds no host code, so it runs on
  any host architecture that drives the same GPU.

Neither runs on the product path.

Usage:  python oracle/build_ref.py [REFERENCE_ROOT]
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
DEFAULT_REF_ROOT = "/root/reference"


def ref_source(ref_root=DEFAULT_REF_ROOT):
    return os.path.join(ref_root, "gcn", "Block_gcn", "example.cpp")


def available(ref_root=DEFAULT_REF_ROOT):
    return os.path.isfile(ref_source(ref_root))


def build(ref_root=DEFAULT_REF_ROOT, verbose=False):
    """Build (or reuse) the reference conversion module; return it or None."""
    if not available(ref_root):
        return None
    from torch.utils.cpp_extension import load
    os.makedirs(REF_OUT, exist_ok=True)
    return load(
        name="Block_sr_bcrs_ref",
        sources=[ref_source(ref_root)],
        build_directory=REF_OUT,
        extra_cflags=["-O2", "-fopenmp"],
        extra_ldflags=["-fopenmp"],
        verbose=verbose,
    )


SPMM_FATBIN = os.path.join(REF_OUT, "ref_spmm.fatbin")


def spmm_source(ref_root=DEFAULT_REF_ROOT):
    return os.path.join(ref_root, "gcn", "SpMM", "src", "spmmKernel.cu")


def build_spmm(ref_root=DEFAULT_REF_ROOT, verbose=False):
    """nvcc the reference's SpMM kernels into a device-only sm_103a fatbin
    (rebuilt only when the source is newer); return its path or None."""
    import subprocess
    src = spmm_source(ref_root)
    if not os.path.isfile(src):
        return None
    if os.path.exists(SPMM_FATBIN) and os.path.getmtime(SPMM_FATBIN) >= os.path.getmtime(src):
        return SPMM_FATBIN
    from torch.utils.cpp_extension import include_paths
    os.makedirs(REF_OUT, exist_ok=True)
    nvcc = "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc"
    tmp = SPMM_FATBIN + ".tmp%d" % os.getpid()
    cmd = ([nvcc, "-fatbin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
            "-std=c++17", "-w"] + ["-I" + p for p in include_paths()] + ["-o", tmp, src])
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed on the reference SpMM:\n" + res.stdout[-4000:])
    os.replace(tmp, SPMM_FATBIN)
    if verbose:
        print("built", SPMM_FATBIN)
    return SPMM_FATBIN


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REF_ROOT
    mod = build(root, verbose=True)
    print("built" if mod is not None else "reference source not present", REF_OUT)
    print(build_spmm(root, verbose=True) or "reference SpMM source not present")
