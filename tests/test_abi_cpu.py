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


def test_documented_run_config_layout_and_name_checks(ckm):
    """The ctypes RunConfig layout a binding declares, over a plain CDLL handle: an
    unknown name in any field the pipeline uses is reported as
    CKM_ERR_UNKNOWN_STRATEGY naming it, before any device work (the
    reference's factories throw std::invalid_argument(strategy),
    fused_factory.hpp:83-85 and the three others); valid names get past the
    check to the device."""
    import ctypes
    import os
    import numpy as np
    ckm.lib()
    L = ctypes.CDLL(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                 "cl-kmeans_gb300", "lib", "libckm.so"))
    L.ckm_last_error.restype = ctypes.c_char_p

    class RunConfig(ctypes.Structure):
        _fields_ = [("pipeline", ctypes.c_char_p), ("fused_strategy", ctypes.c_char_p),
                    ("labeling_strategy", ctypes.c_char_p), ("mass_update_strategy", ctypes.c_char_p),
                    ("centroid_update_strategy", ctypes.c_char_p), ("device", ctypes.c_int),
                    ("device_budget_bytes", ctypes.c_uint64), ("chunk_bytes", ctypes.c_uint64),
                    ("converge", ctypes.c_int), ("tolerance", ctypes.c_double), ("spatial_order", ctypes.c_int)]

    n, d, k = 64, 4, 3
    P, C = np.zeros(n * d, np.float32), np.zeros(k * d, np.float32)
    M, lab = np.zeros(k, np.uint32), np.zeros(n, np.uint32)

    def run(**fields):
        cfg = RunConfig(b"single_stage", b"feature_sum", b"unroll_vector", b"part_local", b"feature_sum",
                        0, 0, 0, 0, 0.0, 0)
        for name, value in fields.items():
            setattr(cfg, name, value)
        rc = L.ckm_kmeans_run_f32(ctypes.byref(cfg), ctypes.c_uint32(2), ctypes.c_uint32(d), ctypes.c_uint64(n),
                                  ctypes.c_uint32(k), ctypes.c_void_p(P.ctypes.data), ctypes.c_void_p(C.ctypes.data),
                                  ctypes.c_void_p(M.ctypes.data), ctypes.c_void_p(lab.ctypes.data), None)
        return rc, L.ckm_last_error()

    cases = [dict(pipeline=b"nonsense"),
             dict(pipeline=b"single_stage", fused_strategy=b"bogus_fused"),
             dict(pipeline=b"single_stage_buffered", fused_strategy=b"bogus_fused"),
             dict(pipeline=b"three_stage", labeling_strategy=b"bogus_labeling"),
             dict(pipeline=b"three_stage", mass_update_strategy=b"bogus_mass"),
             dict(pipeline=b"three_stage_buffered", centroid_update_strategy=b"bogus_update")]
    for fields in cases:
        rc, msg = run(**fields)
        assert rc == -8, (fields, rc, msg)  # CKM_ERR_UNKNOWN_STRATEGY
        assert list(fields.values())[-1] in msg
    # a three-stage run does not read the fused strategy (as in the reference)
    rc, msg = run(pipeline=b"three_stage", fused_strategy=b"ignored")
    assert rc != -8, msg
