"""The C-ABI library loads and exports every entry point include/skity_cuda.h
declares (no GPU calls)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "skity_cuda.h")).read()
    return sorted(set(re.findall(r"SKITY_CUDA_API\s+[\w\s\*]+?\b(skity_cuda_\w+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared()
    assert "skity_cuda_canvas_draw_path" in names and len(names) >= 14


def test_library_exports_every_symbol():
    from skity_gb300 import build, _lib
    try:
        build.build()
    except RuntimeError as e:  # no nvcc in this environment
        pytest.skip(str(e))
    lib = _lib.load()
    for name in declared():
        assert hasattr(lib, name), name
    assert set(declared()) == set(_lib.SIGNATURES)
    assert lib.skity_cuda_version().startswith(b"skity-gb300")
