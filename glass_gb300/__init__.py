"""GB300-native resident light-stack hot path for GLASS.

The CUDA kernels and the C ABI live in ``libglass_gb300.so`` (sources in
``glass_gb300/csrc``, declarations in ``include/glass_gb300.h``).
``glass_gb300._glass_cuda_native`` is the ctypes module that stands in for
GLASS's ``_glass_cuda_native`` extension; ``install_drop_in()`` registers it
under that name so ``glass_cuda`` picks it up unchanged.
"""

from __future__ import annotations

import importlib
import sys

__all__ = ["install_drop_in", "native"]


def native():
    """Returns the drop-in module (loads libglass_gb300.so; raises if missing)."""
    return importlib.import_module("glass_gb300._glass_cuda_native")


def install_drop_in() -> None:
    """Makes ``import _glass_cuda_native`` resolve to this library."""
    sys.modules["_glass_cuda_native"] = native()
