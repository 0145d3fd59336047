"""The C-ABI library builds for sm_103a, loads, and exports every symbol include/cctgpu.h
declares (no compute call: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

from cctpy_gb300 import _lib
from cctpy_gb300.build import build_library

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "cctgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|void)\s+\**(cct_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    build_library()
    return _lib.load()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "cct_field_f64" in names and "cct_track" in names and len(names) >= 10


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_host_only_calls(lib):
    assert lib.cct_version() >= 100
    assert lib.cct_f32c_tile() == 128
    off = (ctypes.c_int64 * 3)(0, 46080, 46081)
    n = lib.cct_f32c_packed_bytes(ctypes.cast(off, ctypes.c_void_p), 2)
    assert n == 256 + 256 + (360 + 1) * 4704
    assert lib.cct_track_scratch_bytes(1, 32) > 0
    # argument errors are reported without touching the GPU
    assert lib.cct_track_scratch_bytes(0, 32) == -1
    assert lib.cct_field_f64(None, None, -1, None, 0, None, 0, None, None) == _lib.CCT_ERR_ARG
    assert "negative" in _lib.last_error()
    bad = (ctypes.c_int64 * 2)(10, 5)
    assert lib.cct_f32c_packed_bytes(ctypes.cast(bad, ctypes.c_void_p), 1) == -1


def test_layer_records_checked_on_host(lib):
    import numpy as np
    from cctpy_gb300 import engine, workloads as W
    _, dipole = W.build_single_dipole()
    rec = np.ascontiguousarray(np.stack([engine.layer_record(dipole, 0), engine.layer_record(dipole, 46080)]))
    assert lib.cct_layer_segments(rec.ctypes.data_as(ctypes.c_void_p), 2) == 2 * 46080
    gap = rec.copy()
    gap[1, 30] = 50000                 # room for other current elements between the layers
    assert lib.cct_layer_segments(gap.ctypes.data_as(ctypes.c_void_p), 2) == 50000 + 46080
    bad = rec.copy()
    bad[1, 30] = 46079                  # overlapping layers
    assert lib.cct_layer_segments(bad.ctypes.data_as(ctypes.c_void_p), 2) == -1
    assert "overlap" in _lib.last_error()
    bad = rec.copy()
    bad[1, 21] = 9                      # more tilt angles than a record holds
    assert lib.cct_layer_segments(bad.ctypes.data_as(ctypes.c_void_p), 2) == -1
    assert "layer 1" in _lib.last_error()
    bad = rec.copy()
    bad[0, 19] = 2.5                    # fractional winding number
    assert lib.cct_layer_segments(bad.ctypes.data_as(ctypes.c_void_p), 2) == -1
