"""Drop-in modules named like the reference's torch extensions.

``install()`` puts this directory on ``sys.path`` so that the reference's own
model code (``import Block_sr_bcrs``, ``import SpMM_sr_bcrs``,
``import ATT_Block_v3``, ``import ATT_SpMM_v1`` ...) runs unchanged on the
sm_103a kernels.
"""
import os
import sys

COMPAT_DIR = os.path.dirname(os.path.abspath(__file__))
MODULES = ("Block_sr_bcrs", "SpMM_sr_bcrs")


def install():
    if COMPAT_DIR not in sys.path:
        sys.path.insert(0, COMPAT_DIR)
    return COMPAT_DIR
