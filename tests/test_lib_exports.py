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
    return sorted(set(re.findall(r"^\s*(?:int|int32_t|int64_t|void|double)\s+\**(cct_\w+)\s*\(", text, flags=re.M)))


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


def test_tracking_arguments_checked_on_host(lib):
    """Argument errors of the tracking entry points are reported before any device work."""
    dummy = ctypes.c_void_p(256)   # never dereferenced: every call below fails its checks first
    args = dict(kls=None, p0s=None, seg_off=dummy, packed=None, qs=None, qs_off=dummy, n_designs=1,
                particles=dummy, n=4, distance=1.0, footstep=0.01, precision=0, scratch=dummy, nbytes=1 << 20)

    def track(**kw):
        a = dict(args, **kw)
        return lib.cct_track(a["kls"], a["p0s"], a["seg_off"], a["packed"], a["qs"], a["qs_off"], a["n_designs"],
                             a["particles"], a["n"], a["distance"], a["footstep"], a["precision"], a["scratch"],
                             a["nbytes"], None)

    assert track(n_designs=0) == _lib.CCT_ERR_ARG
    assert track(footstep=0.0) == _lib.CCT_ERR_ARG
    assert track(distance=float("nan")) == _lib.CCT_ERR_ARG
    assert track(precision=2) == _lib.CCT_ERR_ARG
    assert track(particles=None) == _lib.CCT_ERR_ARG
    assert track(precision=1, packed=None) == _lib.CCT_ERR_ARG
    assert "packed" in _lib.last_error()
    assert track(precision=1, packed=ctypes.c_void_p(300)) == _lib.CCT_ERR_ARG   # not 256-byte aligned
    assert track(n=0) == _lib.CCT_OK                                              # nothing to track
    assert lib.cct_track_async(None, None, dummy, None, None, dummy, 0, dummy, 4, 1.0, 0.01, 0, dummy,
                               1 << 20, None) == _lib.CCT_ERR_ARG
    assert lib.cct_track_async(None, None, dummy, None, None, dummy, 1, dummy, 4, 1.0, 0.01, 1, dummy,
                               1 << 20, None) == _lib.CCT_ERR_ARG                 # FP32c without packed set
    assert lib.cct_track_set_units_per_cta(65) == _lib.CCT_ERR_ARG
    assert lib.cct_track_set_units_per_cta(-1) == _lib.CCT_ERR_ARG


def test_every_exported_entry_point_is_declared(lib):
    """The reverse direction: no cct_* symbol leaves the library without a declaration in the
    header and a ctypes signature (dynamic symbol table, read with nm)."""
    import shutil
    import subprocess
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = sorted({line.split()[-1] for line in out.splitlines()
                       if line.split() and line.split()[-1].startswith("cct_")})
    assert exported, "no cct_ symbols exported"
    assert set(exported) == set(declared_functions())
    assert set(exported) == set(_lib.SIGNATURES)
