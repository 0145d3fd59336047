"""ctypes binding of libcctgpu.so (the C ABI declared in include/cctgpu.h).

There is no CPU fallback: if the library is missing or no CUDA device is
visible, every compute call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libcctgpu.so")

CCT_OK, CCT_ERR_ARG, CCT_ERR_CUDA, CCT_ERR_TIMEOUT, CCT_ERR_NONFINITE, CCT_ERR_UNSUPPORTED = range(6)

# exported symbol -> (restype, argtypes)
_i64, _i32, _d, _p = ctypes.c_int64, ctypes.c_int32, ctypes.c_double, ctypes.c_void_p
SIGNATURES = {
    "cct_version": (ctypes.c_int, []),
    "cct_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "cct_f32c_tile": (ctypes.c_int, []),
    "cct_field_f64": (ctypes.c_int, [_p, _p, _i64, _p, _i32, _p, _i64, _p, _p]),
    "cct_f32c_packed_bytes": (_i64, [_p, _i32]),
    "cct_f32c_pack": (ctypes.c_int, [_p, _p, _p, _i32, _p, _i64, _p]),
    "cct_field_f32c": (ctypes.c_int, [_p, _i32, _p, _i32, _p, _i64, _p, _p]),
    "cct_field_status": (ctypes.c_int, [_p]),
    "cct_field_host": (ctypes.c_int, [_p, _p, _i64, _p, _i32, _p, _i64, _p, _i32]),
    "cct_track_scratch_bytes": (_i64, [_i32, _i64]),
    "cct_track": (ctypes.c_int, [_p, _p, _p, _p, _p, _p, _i32, _p, _i64, _d, _d, _i32, _p, _i64, _p]),
    "cct_track_static_scratch_bytes": (_i64, []),
    "cct_track_static_scratch": (ctypes.c_int, [_p, _p, _p, _p, _p, _p, _i32, _p, _i64, _d, _d, _i32, _p]),
    "cct_track_async": (ctypes.c_int, [_p, _p, _p, _p, _p, _p, _i32, _p, _i64, _d, _d, _i32, _p, _i64, _p]),
    "cct_track_status": (ctypes.c_int, [_p, _p]),
    "cct_track_set_units_per_cta": (ctypes.c_int, [_i32]),
    "cct_track_units_per_cta": (_i32, []),
    "cct_track_set_particle_block": (ctypes.c_int, [_i32]),
    "cct_track_particle_block": (_i32, []),
    "cct_autotune_scratch_bytes": (_i64, [_i32, _i64]),
    "cct_autotune": (ctypes.c_int, [_p, _p, _p, _p, _p, _p, _i32, _p, _i64, _d, _i32, _i32, _p, _i64,
                                    ctypes.POINTER(ctypes.c_int32), _p]),
    "cct_adjoint_scratch_bytes": (_i64, [_i32, _i64, _i32, _i32]),
    "cct_track_adjoint": (ctypes.c_int, [_p, _p, _p, _p, _p, _p, _i32, _p, _i64, _d, _d, _i32, _p, _p, _p, _i32, _p,
                                         _i64, _p]),
    "cct_layer_segments": (_i64, [_p, _i32]),
    "cct_segments_build": (ctypes.c_int, [_p, _i32, _p, _p, _i64, _p]),
    "cct_segments_param_grad": (ctypes.c_int, [_p, _i32, _p, _i64, _p, _p]),
    "cct_beam_readout": (ctypes.c_int, [_p, _i32, _i64, _p, _p, _i32, _i32, _p, _p, _p]),
    "cct_probe_fma_peak": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "cct_test_set_barrier_fault": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "cct_test_set_flow_fault": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "cct_test_plan_units": (_i64, [_p, _i32, _i64, _i32, _i32, _i64, _p, _p, _p, ctypes.POINTER(ctypes.c_int32)]),
}

_lib = None
_lock = threading.Lock()


class CctTimeoutError(TimeoutError):
    """A bounded device-side wait gave up (CCT_ERR_TIMEOUT)."""


class CctNonFiniteError(FloatingPointError):
    """A particle state became NaN/Inf (CCT_ERR_NONFINITE)."""


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libcctgpu.so and declare its signatures.  Raises if it is missing."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise ImportError(
                    f"libcctgpu.so not found at {path}: build it with "
                    "`python -c 'import __graft_entry__ as g; g.build()'` (needs nvcc)")
            lib = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(lib, name)
                f.restype = res
                f.argtypes = args
            _lib = lib
    return _lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(512)
    load().cct_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(status: int, what: str) -> None:
    """Map a cct_status to the exception the reference raises for the same condition."""
    if status == CCT_OK:
        return
    msg = f"{what}: {last_error()}"
    if status == CCT_ERR_ARG:
        raise ValueError(msg)
    if status == CCT_ERR_TIMEOUT:
        raise CctTimeoutError(msg)
    if status == CCT_ERR_NONFINITE:
        raise CctNonFiniteError(msg)
    if status == CCT_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise RuntimeError(msg)
