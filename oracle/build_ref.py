"""Recipe: compile the reference's CPU block conversion into ``oracle/_ref/``.

Test infrastructure only.  It compiles ``gcn/Block_gcn/example.cpp`` of the
reference tree (``blockProcess_fp16_balance`` / ``blockProcess_tf32_balance``,
example.cpp:48-348) where it lies, as a torch CPU extension with OpenMP, and
writes every build product under ``oracle/_ref/``.  Nothing is copied out of
the reference tree.  The result is used only to pin the C restatement in
``oracle/block_oracle.c`` and to generate the committed golden fixtures; it
never runs on the product path.

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


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REF_ROOT
    mod = build(root, verbose=True)
    print("built" if mod is not None else "reference source not present", REF_OUT)
