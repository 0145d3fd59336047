"""The allocation-free tracking entry point, cct_track_static_scratch.

It exists for callers that may not allocate device memory while running -- a host
application that reserves its GPU memory at start-up and forbids cudaMalloc on its hot
path, or a plain C caller holding only the buffers it passes.  Its scratch is a fixed
device array inside the library, so these tests check that it tracks exactly like
cct_track (which takes a caller scratch buffer), on two calls in a row (the array keeps
the previous call's contents), and that problems larger than the array are refused with
a clear error instead of being run.

This file is collected last on purpose: a failure here leaves every other test already run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from cctpy_gb300 import HUST_SC_GANTRY, _lib, engine, workloads as W

POS_TOL = {"f64": 1e-9, "f32c": 1e-6}     # metres, the tracking tolerances of the other tests
PREC = {"f64": 0, "f32c": 1}


def static_track(ds, particles, length, footstep, precision):
    lib = _lib.load()
    p = torch.as_tensor(particles, dtype=torch.float64).cuda().contiguous()
    packed = ds.packed().data_ptr() if precision == "f32c" else 0
    rc = lib.cct_track_static_scratch(ds.kls.data_ptr(), ds.p0s.data_ptr(), ds.seg_off.data_ptr(), packed,
                                      ds.qs.data_ptr() if ds.qs.numel() else 0, ds.qs_off.data_ptr(), ds.n_designs,
                                      p.data_ptr(), p.shape[0], float(length), float(footstep), PREC[precision],
                                      torch.cuda.current_stream().cuda_stream)
    _lib.check(rc, "cct_track_static_scratch")
    return p.cpu().numpy()


@pytest.mark.parametrize("precision", ["f64", "f32c"])
def test_static_scratch_matches_caller_scratch_twice(precision):
    bl = HUST_SC_GANTRY().create_second_bending_part_beamline()
    ds = engine.design_of(bl)
    ps = W.beam_particles(bl, 37, seed=5, kinetic_MeV=215.0)      # a full and a ragged group of 32
    ref = engine.track(ds, ps, 0.6, 0.1, precision)[0]             # cct_track, caller scratch
    for call in range(2):
        out = static_track(ds, ps, 0.6, 0.1, precision)
        assert np.abs(out[:, :3] - ref[:, :3]).max() <= POS_TOL[precision], f"call {call}"
        np.testing.assert_allclose(out[:, 3:6], ref[:, 3:6], rtol=1e-9, atol=0)
        np.testing.assert_array_equal(out[:, 6:9], ref[:, 6:9])
        np.testing.assert_allclose(out[:, 9], ref[:, 9], rtol=1e-15)


def test_static_scratch_refuses_oversized_problems():
    """Every refused call is given buffers of the sizes it declares, so that even a
    regressed size check could not read or write past them."""
    lib = _lib.load()
    assert lib.cct_track_static_scratch_bytes() == 32 << 20
    _, cct = W.build_single_dipole()
    ds = engine.design_of(cct)
    stream = torch.cuda.current_stream().cuda_stream
    # 200 000 particles: their records take 16 MB, their RK4 state alone 38 MB, more than the
    # 32 MiB array holds -- refused before any launch, the records untouched
    n_big = 200_000
    big = torch.as_tensor(np.tile(W.single_dipole_particles(2, 0), (n_big // 2, 1))).cuda().contiguous()
    before = big.clone()
    rc = lib.cct_track_static_scratch(ds.kls.data_ptr(), ds.p0s.data_ptr(), ds.seg_off.data_ptr(), 0, 0,
                                      ds.qs_off.data_ptr(), 1, big.data_ptr(), n_big, 0.01, 0.001, 0, stream)
    assert rc == _lib.CCT_ERR_ARG
    assert "static scratch holds" in _lib.last_error()
    assert torch.equal(big, before)
    # 65 designs (one more than the entry point takes), with offsets and records for all of them
    n_d = 65
    seg_off = torch.zeros(n_d + 1, dtype=torch.int64, device="cuda")
    qs_off = torch.zeros(n_d + 1, dtype=torch.int64, device="cuda")
    many = torch.as_tensor(np.tile(W.single_dipole_particles(2, 0), (n_d, 1))).cuda().contiguous()
    rc = lib.cct_track_static_scratch(ds.kls.data_ptr(), ds.p0s.data_ptr(), seg_off.data_ptr(), 0, 0,
                                      qs_off.data_ptr(), n_d, many.data_ptr(), 2, 0.01, 0.001, 0, stream)
    assert rc == _lib.CCT_ERR_ARG
    # the refusals left the device usable
    out = static_track(ds, W.single_dipole_particles(2, 0), 0.01, 0.001, "f64")
    assert np.isfinite(out).all()


@pytest.mark.parametrize("precision", ["f64", "f32c"])
def test_static_scratch_call_takes_no_device_memory(precision):
    """The defining property: with its inputs in place, a call changes the device's free
    memory by nothing (no cudaMalloc, no library allocation behind it)."""
    lib = _lib.load()
    _, cct = W.build_single_dipole()
    ds = engine.design_of(cct)
    packed = ds.packed().data_ptr() if precision == "f32c" else 0
    p = torch.as_tensor(W.single_dipole_particles(64, 3)).cuda().contiguous()
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        rc = lib.cct_track_static_scratch(ds.kls.data_ptr(), ds.p0s.data_ptr(), ds.seg_off.data_ptr(), packed, 0,
                                          ds.qs_off.data_ptr(), 1, p.data_ptr(), p.shape[0], 0.02, 0.001,
                                          PREC[precision], stream)
        _lib.check(rc, "cct_track_static_scratch")

    call()                                  # first call: module, kernel and array already placed
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    call()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.isfinite(p).all()
