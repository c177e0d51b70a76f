"""CPU checks of the C ABI boundary: the library builds, loads and exports
every function include/glass_gb300.h declares; the ctypes prototypes match the
header; the product package never reaches the oracle."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

from glass_gb300 import _lib

REPO = Path(__file__).resolve().parents[1]
HEADER = REPO / "include" / "glass_gb300.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*int\s+(gg_[a-z0-9_]+)\s*\(", text, flags=re.MULTILINE)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("gg_stack_create", "gg_stack_integrate", "gg_stack_calibrate_u16", "gg_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(built_library):
    lib = ctypes.CDLL(str(built_library))
    missing = [name for name in declared_functions() if not hasattr(lib, name)]
    assert not missing, f"not exported: {missing}"


def test_ctypes_prototypes_cover_the_header(built_library):
    declared = set(declared_functions())
    bound = set(_lib.PROTOTYPES)
    assert declared == bound, f"header-only: {declared - bound}; binding-only: {bound - declared}"


def test_struct_layouts_match_header():
    # Sizes follow from the C declarations (LP64): keep in sync with the header.
    assert ctypes.sizeof(_lib.CalibParams) == 16
    assert ctypes.sizeof(_lib.IntegrateParams) == 28
    assert ctypes.sizeof(_lib.FrameStats) == 32
    assert ctypes.sizeof(_lib.StackInfo) == 12 * 8 + 3 * 4 + 4
    assert ctypes.sizeof(_lib.StackDevicePtrs) == 9 * 8


def test_error_mapping_matches_reference_exceptions(built_library):
    _lib.load()
    import pytest

    # A null out-pointer is an argument error -> ValueError, no device needed.
    with pytest.raises(ValueError):
        _lib.call("gg_version", None)
    version = ctypes.c_int()
    _lib.call("gg_version", ctypes.byref(version))
    assert version.value >= 10000


def test_product_never_imports_the_oracle():
    for path in (REPO / "glass_gb300").rglob("*.py"):
        text = path.read_text()
        assert not re.search(r"^\s*(from|import)\s+oracle\b", text, flags=re.MULTILINE), path
