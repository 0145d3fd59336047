"""Asynchronous tracking (cct_track_async / cct_track_status), its capture in a CUDA graph,
and the work-split autotuner, against the synchronous cct_track."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from cctpy_gb300 import HUST_SC_GANTRY, engine, workloads as W


@pytest.fixture(scope="module")
def population():
    bls = [HUST_SC_GANTRY(**kw).create_second_bending_part_beamline()
           for kw in W.design_population(3, seed=5, part_per_winding=60)]
    ds = engine.design_set_of(bls, segments="device")
    ps = W.beam_particles(bls[0], 40, seed=9, kinetic_MeV=215.0)
    return ds, ps


@pytest.mark.parametrize("precision", ["f64", "f32c"])
def test_async_equals_sync(population, precision):
    ds, ps = population
    want = engine.track(ds, ps, 0.05, 0.01, precision)
    p = torch.as_tensor(np.broadcast_to(ps, (ds.n_designs,) + ps.shape).copy(), device="cuda")
    tl = engine.TrackLaunch(ds, p, 0.05, 0.01, precision)
    tl.launch()
    tl.status()
    np.testing.assert_array_equal(p.cpu().numpy(), want)


def test_graph_capture_and_replay(population):
    ds, ps = population
    bl0 = HUST_SC_GANTRY(**W.design_population(1, seed=5, part_per_winding=60)[0]).create_second_bending_part_beamline()
    starts = [ps, W.beam_particles(bl0, 40, seed=10, kinetic_MeV=215.0)]
    p = torch.as_tensor(np.broadcast_to(ps, (ds.n_designs,) + ps.shape).copy(), device="cuda")
    tl = engine.TrackLaunch(ds, p, 0.05, 0.01, "f32c")
    tl.launch()                      # first call outside the capture (occupancy query)
    tl.status()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        tl.launch()
    for start in starts:
        p.copy_(torch.as_tensor(np.broadcast_to(start, p.shape).copy(), device="cuda"))
        g.replay()
        tl.status()
        np.testing.assert_array_equal(p.cpu().numpy(), engine.track(ds, start, 0.05, 0.01, "f32c"))


def test_plan_rejects_mismatched_packed_set(population):
    ds, ps = population
    other = engine.design_set_of([W.build_single_dipole()[1]])
    p = torch.as_tensor(np.broadcast_to(ps, (ds.n_designs,) + ps.shape).copy(), device="cuda")
    before = p.clone()
    tl = engine.TrackLaunch(ds, p, 0.05, 0.01, "f32c")
    tl.packed = other.packed().data_ptr()          # a packed set of another design set
    tl.launch()
    with pytest.raises(ValueError, match="plan rejected"):
        tl.status()
    assert torch.equal(p, before)                  # nothing was tracked
    tl.packed = ds.packed().data_ptr()             # the context is still usable
    tl.launch()
    tl.status()


def test_autotune_picks_a_split_and_keeps_results(population):
    ds, ps = population
    base = engine.track(ds, ps, 0.05, 0.01, "f64")
    try:
        best = engine.autotune(ds, ps, 0.01, "f64", steps=2)
        assert best in (2, 4, 8, 16, 32)
        assert engine._lib.load().cct_track_units_per_cta() == best
        assert engine.particle_block() == 0            # FP64 keeps blocks of 32
        tuned = engine.track(ds, ps, 0.05, 0.01, "f64")
        assert np.abs(tuned[..., 0:3] - base[..., 0:3]).max() <= 1e-12
    finally:
        engine.set_units_per_cta(0)
    assert engine._lib.load().cct_track_units_per_cta() == 8


def test_autotune_particle_block_f32c(population):
    """FP32c: the autotuner also picks the particle block (40 protons a design: the automatic
    block of 64, or 16 or 32); every split it may keep gives the same tracks to FP32 rounding
    of a different chunk split (blocks of 16: three, the last ragged, on half-warp lanes)."""
    ds, ps = population
    base = engine.track(ds, ps, 0.05, 0.01, "f32c")
    try:
        best = engine.autotune(ds, ps, 0.01, "f32c", steps=2)
        assert best in (2, 4, 8, 16, 32)
        assert engine.particle_block() in (0, 16, 32, 64)
        tuned = engine.track(ds, ps, 0.05, 0.01, "f32c")
        assert np.abs(tuned[..., 0:3] - base[..., 0:3]).max() <= 1e-8
        for g in (16, 32, 64, 128):
            engine.set_particle_block(g)
            out = engine.track(ds, ps, 0.05, 0.01, "f32c")
            assert np.abs(out[..., 0:3] - base[..., 0:3]).max() <= 1e-8
            assert np.array_equal(out[..., 6:], base[..., 6:])
    finally:
        engine.set_units_per_cta(0)
        engine.set_particle_block(0)
    assert engine.particle_block() == 0
