"""The C-ABI library without a GPU: it loads, exports every symbol that
include/ckm.h declares, and its host-only entry points behave (status
strings, scratch sizing, argument validation that fails before any device
work)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "ckm.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ckm_[a-z0-9_]+)\s*\(", text)))


def test_header_and_python_exports_agree(ckm):
    assert declared_symbols() == sorted(ckm.EXPORTS)


def test_library_exports_every_declared_symbol(ckm):
    L = ctypes.CDLL(ckm.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing


def test_status_strings_and_version(ckm):
    L = ckm.lib()
    assert L.ckm_status_string(0) == b"ok"
    assert L.ckm_status_string(-8) == b"unknown strategy"
    assert L.ckm_version() >= 10000


def test_scratch_layout(ckm):
    b = ckm.scratch_bytes(4, 16)
    assert b % 256 == 0 and b >= 4 * 16 * 8 + 16 * 8 + 8
    assert ckm.scratch_bytes(128, 1024) > ckm.scratch_bytes(4, 16)


def test_validation_before_device_work(ckm):
    L = ckm.lib()
    # d = 0 and k = 0 are rejected before any CUDA call
    assert L.ckm_fused_f32(0, 10, 4, None, None, None, None, None, None, 0, 1, None) == -1
    assert L.ckm_fused_f32(4, 10, 0, None, None, None, None, None, None, 0, 1, None) == -1
    assert L.ckm_labeling_f32(4, 10, 0, None, None, None, None) == -1
    # bad mode
    assert L.ckm_fused_f32(4, 10, 4, None, None, None, None, None, None, 0, 7, None) == -1
    # missing scratch
    assert L.ckm_fused_f32(4, 10, 4, None, None, None, None, None, None, 0, 1, None) == -1
    assert b"scratch" in L.ckm_last_error()
    # run config: unknown pipeline names fail with CKM_ERR_UNKNOWN_STRATEGY
    assert L.ckm_kmeans_run_f32(None, 1, 4, 10, 4, None, None, None, None, None) == -1


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    import importlib
    mod = importlib.import_module("cl-kmeans_gb300")
    monkeypatch.setattr(mod, "_lib", None)
    monkeypatch.setattr(mod, "LIB_PATH", str(tmp_path / "nope.so"))
    with pytest.raises(RuntimeError):
        mod.lib()
