"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/gms.h declares (no GPU needed: nothing is called but queries)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT, load_gms_module


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "gms.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gms_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    mod = load_gms_module()
    mod.build()
    return mod.load()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "gms_sort_i32" in names and "gms_merge_level_i32" in names and len(names) >= 25


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    mod = load_gms_module()
    assert set(declared_symbols()) <= set(mod.SIGNATURES), set(declared_symbols()) - set(mod.SIGNATURES)


def test_queries_without_gpu(lib):
    assert lib.gms_version() >= 100
    assert lib.gms_max_tile() == 512 * 17
    assert lib.gms_rounds(0, 0, 1 << 28) == 3
    assert lib.gms_base_tile(0, 0) == 8192  # keys-only: warp-shuffle base case
    assert lib.gms_base_tile(4, 0) == 4096  # 64-bit keys: 256 threads x 16 keys
    assert lib.gms_base_tile(0, 1) == 4352  # key/value: stable base case, 256 x 17
    assert lib.gms_rounds(0, 0, 8192) == 0
    assert lib.gms_rounds(0, 0, 8193) == 1
    assert lib.gms_workspace_bytes(0, 0, 1 << 28) < (1 << 28) * 4 // 4
    assert lib.gms_status_string(1) == b"GMS_ERR_INVALID"
