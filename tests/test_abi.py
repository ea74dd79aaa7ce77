"""The C-ABI library builds, loads and exports every symbol of include/gtgpu.h
(no compute calls: runs without a GPU)."""
import ctypes
import os
import re

from gtgpu import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "gtgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gt_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    path = _build.build()
    lib = ctypes.CDLL(path)
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_table_covers_header():
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared_symbols()) <= bound


def test_null_arguments_are_rejected_without_gpu():
    lib = _lib.load()
    assert lib.gt_ctx_create(0, None) == _lib.GT_ERR_INVALID
    assert lib.gt_ctx_destroy(None) == _lib.GT_ERR_INVALID
    assert lib.gt_matrix_destroy(None) == _lib.GT_ERR_INVALID
