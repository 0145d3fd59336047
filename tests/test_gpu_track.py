"""RK4 tracking parity on the GPU against particles tracked by the reference itself
(golden fixtures) and the CPU oracle, plus the accelerator API conventions and the
failure paths (bounded barrier wait, non-finite state)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from cctpy_gb300 import (GPU_ACCELERATOR, HUST_SC_GANTRY, ParticleRunner, RunningParticle, engine,
                         workloads as W, _lib)
from cctpy_gb300.particles import particles_to_array
from oracle import cct_oracle as O
from tests.conftest import oracle_records

POS_TOL_F64 = 1e-9      # m, FP64 GPU vs reference FP64 CPU after the whole track
VEL_RTOL_F64 = 1e-9
POS_TOL_F32C = 1e-6     # m (1 um), FP32-compensated vs reference FP64


def check(out, want, pos_tol, vel_rtol):
    assert np.abs(out[:, 0:3] - want[:, 0:3]).max() < pos_tol
    assert (np.abs(out[:, 3:6] - want[:, 3:6]).max() / np.abs(want[:, 3:6]).max()) < vel_rtol
    assert np.array_equal(out[:, 6:9], want[:, 6:9])
    np.testing.assert_allclose(out[:, 9], want[:, 9], rtol=1e-15)


@pytest.mark.parametrize("prec,ptol,vtol", [("f64", POS_TOL_F64, VEL_RTOL_F64), ("f32c", POS_TOL_F32C, 1e-6)])
def test_single_dipole_32_protons(golden, prec, ptol, vtol):
    _, cct = W.build_single_dipole()
    out = engine.track(engine.design_of(cct), golden["sd_particles_in"], W.single_dipole_track_length(), 0.001,
                       prec)[0]
    check(out, golden["sd_particles_out"], ptol, vtol)


@pytest.mark.parametrize("prec,ptol,vtol", [("f64", POS_TOL_F64, VEL_RTOL_F64), ("f32c", POS_TOL_F32C, 1e-6)])
def test_hust2_section_with_qs(golden, prec, ptol, vtol):
    bl = HUST_SC_GANTRY().create_second_bending_part_beamline()
    out = engine.track(engine.design_of(bl), golden["h2_particles_in"], float(golden["h2_length"][0]), 0.1,
                       prec)[0]
    check(out, golden["h2_particles_out"], ptol, vtol)


@pytest.mark.parametrize("prec,ptol,vtol", [("f64", POS_TOL_F64, VEL_RTOL_F64), ("f32c", POS_TOL_F32C, 1e-6)])
def test_hust1_section_with_three_qs(golden_hust1, prec, ptol, vtol):
    bl = HUST_SC_GANTRY().create_first_bending_part_beamline()
    out = engine.track(engine.design_of(bl), golden_hust1["h1_particles_in"], float(golden_hust1["h1_length"][0]),
                       0.1, prec)[0]
    check(out, golden_hust1["h1_particles_out"], ptol, vtol)


@pytest.mark.parametrize("prec,ptol,vtol", [("f64", POS_TOL_F64, VEL_RTOL_F64), ("f32c", POS_TOL_F32C, 1e-6)])
def test_gantry_section(golden, prec, ptol, vtol):
    bl = W.build_gantry_section()
    out = engine.track(engine.design_of(bl), golden["gs_particles_in"], 3.5, 0.05, prec)[0]
    check(out, golden["gs_particles_out"], ptol, vtol)


@pytest.mark.parametrize("prec,ptol,vtol", [("f64", POS_TOL_F64, VEL_RTOL_F64), ("f32c", POS_TOL_F32C, 1e-6)])
def test_design_population_one_launch(golden, prec, ptol, vtol):
    bls = [HUST_SC_GANTRY(**kw).create_second_bending_part_beamline() for kw in W.design_population(2, seed=3)]
    ds = engine.design_set_of(bls)
    L = float(golden["dp0_length"][0])
    assert abs(L - float(golden["dp1_length"][0])) < 1e-12
    parts = np.stack([golden["dp0_particles_in"], golden["dp1_particles_in"]])
    out = engine.track(ds, parts, L, 0.05, prec)
    for d in range(2):
        check(out[d], golden[f"dp{d}_particles_out"], ptol, vtol)


@pytest.mark.parametrize("prec,ptol,vtol,same", [("f64", POS_TOL_F64, VEL_RTOL_F64, 1e-12),
                                                 ("f32c", POS_TOL_F32C, 1e-6, 1e-8)])
def test_dataflow_schedule_matches_reference_and_barrier_schedule(golden, prec, ptol, vtol, same):
    """Eight copies of the gantry section in one launch are eight particle blocks, which the
    kernel runs on its dataflow schedule (per-block stage counters); one copy alone runs on
    grid barriers.  Every copy must give the reference's track.  Between the two launches the
    segment chunks differ (the planner sizes them for the whole batch) as well as the order of
    the chunk sums: FP64 tracks agree to 1e-12, FP32c ones to the FP32 rounding of a different
    chunk split (1e-8 m)."""
    bl = W.build_gantry_section()
    parts = golden["gs_particles_in"]
    one = engine.track(engine.design_of(bl), parts, 3.5, 0.05, prec)[0]
    many = engine.track(engine.design_set_of([bl] * 8), np.stack([parts] * 8), 3.5, 0.05, prec)
    for d in range(8):
        check(many[d], golden["gs_particles_out"], ptol, vtol)
        np.testing.assert_array_equal(many[d], many[0])     # same inputs, same chunks: same track
        assert np.abs(many[d][:, 0:3] - one[:, 0:3]).max() < same
        assert np.abs(many[d][:, 3:6] - one[:, 3:6]).max() / np.abs(one[:, 3:6]).max() < same
        assert np.array_equal(many[d][:, 6:], one[:, 6:])


def test_ragged_particle_counts_match_oracle(records_json):
    # 37 particles: one full group of 32 and a ragged group of 5; short track, oracle in seconds
    bl = HUST_SC_GANTRY().create_second_bending_part_beamline()
    ps = W.beam_particles(bl, 37, seed=5, kinetic_MeV=215.0)
    out = engine.track(engine.design_of(bl), ps, 0.6, 0.1, "f64")[0]
    ob = O.BeamlineOracle(oracle_records(records_json["hust2_default"]))
    for i in (0, 31, 32, 36):
        want = O.rk4_track(ps[i], ob.field_at, 0.6, 0.1)
        assert np.abs(out[i, :3] - want[:3]).max() < 1e-11


def test_accelerator_conventions(golden):
    bl = HUST_SC_GANTRY().create_second_bending_part_beamline()
    ps = [RunningParticle.from_numpy_array_data(r) for r in golden["h2_particles_in"]]
    L = float(golden["h2_length"][0])
    ga = GPU_ACCELERATOR(GPU_ACCELERATOR.FLOAT64, block_dim_x=512)
    before = particles_to_array(ps)
    res = ga.track_multi_particle_beamline_for_magnet_with_multi_qs([bl, bl], ps, L, 0.1)
    assert np.array_equal(particles_to_array(ps), before)          # inputs untouched
    assert len(res) == 2 and len(res[0]) == 4
    check(particles_to_array(res[1]), golden["h2_particles_out"], POS_TOL_F64, VEL_RTOL_F64)
    one = ps[0].copy()
    ga.track_one_particle_with_multi_qs(bl, one, L, 0.1)             # in place
    check(particles_to_array([one]), golden["h2_particles_out"][:1], POS_TOL_F64, VEL_RTOL_F64)
    many = [p.copy() for p in ps]
    ParticleRunner.run_only(many, bl, L, 0.1)
    check(particles_to_array(many), golden["h2_particles_out"], POS_TOL_F64, VEL_RTOL_F64)
    # the same beamline object given several times is built once and repeated on the device:
    # the results equal, bit for bit, those of a call of the same shape with a separately
    # built copy (calls of different shapes split the segment sums differently)
    bl2 = HUST_SC_GANTRY().create_second_bending_part_beamline()
    mixed = ga.track_multi_particle_beamline_for_magnet_with_multi_qs([bl, bl2, bl], ps, L, 0.1)
    same = ga.track_multi_particle_beamline_for_magnet_with_multi_qs([bl, bl, bl], ps, L, 0.1)
    for a, b in zip(mixed, same):
        np.testing.assert_array_equal(particles_to_array(a), particles_to_array(b))
        check(particles_to_array(a), golden["h2_particles_out"], POS_TOL_F64, VEL_RTOL_F64)
    d = engine.host_design(engine.magnet_list(bl))
    rep = engine.DesignSet([d, d, d])
    sep = engine.DesignSet([d, tuple(np.copy(a) for a in d), d])
    assert torch.equal(rep.kls, sep.kls) and torch.equal(rep.p0s, sep.p0s) and torch.equal(rep.qs, sep.qs)
    assert np.array_equal(rep.h_seg_off, sep.h_seg_off)
    with pytest.raises(ValueError):
        GPU_ACCELERATOR(block_dim_x=1000)
    with pytest.raises(ValueError):
        GPU_ACCELERATOR(GPU_ACCELERATOR.FLOAT32, max_current_element_number=1000).track_one_particle_with_multi_qs(
            bl, ps[0].copy(), L, 0.1)


def test_phase_ellipse_api():
    bl = HUST_SC_GANTRY().create_second_bending_part_beamline()
    ga = GPU_ACCELERATOR(GPU_ACCELERATOR.FLOAT32)
    res = ga.track_phase_ellipse_in_multi_beamline([bl], 3.5, 7.5, 3.5, 7.5, 0.0, 4, 215, length=1.0, footstep=0.05)
    assert len(res) == 1 and len(res[0][0]) == 4 and len(res[0][1]) == 4


def test_bounded_barrier_wait_reports_timeout(golden):
    """A barrier that can never complete (phantom CTAs that never arrive) gives up after
    the wait limit and reports CCT_ERR_TIMEOUT; the context stays usable afterwards."""
    _, cct = W.build_single_dipole()
    ds = engine.design_of(cct)
    lib = _lib.load()
    lib.cct_test_set_barrier_fault(1, 300)
    try:
        with pytest.raises(_lib.CctTimeoutError):
            engine.track(ds, golden["sd_particles_in"][:2], 0.01, 0.001, "f32c")
    finally:
        lib.cct_test_set_barrier_fault(0, 0)
    out = engine.track(ds, golden["sd_particles_in"][:2], 0.01, 0.001, "f64")
    assert np.isfinite(out).all()


@pytest.mark.parametrize("prec,same", [("f64", 1e-12), ("f32c", 1e-8)])
def test_dataflow_ragged_blocks_match_single_design_launches(prec, same):
    """Nine designs x 100 protons: nine ragged particle blocks of 128 (FP32c) or 36 blocks of 32
    (FP64, the last of each design ragged), run on the dataflow schedule; each design tracked
    alone is one (FP32c) or four (FP64) blocks, on grid barriers."""
    _, cct = W.build_single_dipole()
    parts = W.single_dipole_particles(100, seed=11)
    many = engine.track(engine.design_set_of([cct] * 9), np.stack([parts] * 9), 0.05, 0.001, prec)
    one = engine.track(engine.design_of(cct), parts, 0.05, 0.001, prec)[0]
    for d in range(9):
        np.testing.assert_array_equal(many[d], many[0])
        assert np.abs(many[d][:, 0:3] - one[:, 0:3]).max() < same
        assert np.abs(many[d][:, 3:6] - one[:, 3:6]).max() / np.abs(one[:, 3:6]).max() < same
        assert np.array_equal(many[d][:, 6:], one[:, 6:])


def test_bounded_dataflow_wait_reports_timeout(golden):
    """Eight designs run on the dataflow schedule; a wait for a particle block that never
    finishes its stage (the test hook asks one stage more than exists) gives up after the
    wait limit and reports CCT_ERR_TIMEOUT; the context stays usable afterwards."""
    _, cct = W.build_single_dipole()
    ds = engine.design_set_of([cct] * 8)
    parts = np.stack([golden["sd_particles_in"][:2]] * 8)
    lib = _lib.load()
    lib.cct_test_set_flow_fault(1, 300)
    try:
        with pytest.raises(_lib.CctTimeoutError):
            engine.track(ds, parts, 0.01, 0.001, "f32c")
    finally:
        lib.cct_test_set_flow_fault(0, 0)
    out = engine.track(ds, parts, 0.01, 0.001, "f32c")
    assert np.isfinite(out).all()


@pytest.mark.parametrize("prec", ["f64", "f32c"])
def test_nonfinite_particle_is_reported(golden, prec):
    """A NaN velocity (FP32c: a small batch, whose unit fields go through fixed-point
    accumulators; the NaN position that follows flags the particle there) is reported as
    CctNonFiniteError, and the other particles are tracked as alone."""
    _, cct = W.build_single_dipole()
    ps = golden["sd_particles_in"][:3].copy()
    ps[1, 3] = np.nan
    with pytest.raises(_lib.CctNonFiniteError):
        engine.track(engine.design_of(cct), ps, 0.01, 0.001, prec)
    good = engine.track(engine.design_of(cct), ps[[0, 2]], 0.01, 0.001, prec)[0]
    assert np.isfinite(good).all()
    with pytest.raises(ValueError):
        engine.track(engine.design_of(cct), ps, -1.0, 0.001, "f64")


@pytest.mark.parametrize("n_designs", [1, 5, 9])
def test_half_warp_blocks_of_16_protons(golden, n_designs):
    """FP32c designs of 16 protons run in blocks of 16 (lanes l and l + 16 of a warp hold
    proton l and sum different halves of each sub-block): one design on the small-batch
    schedule, five on grid barriers, nine on the dataflow schedule.  Every copy tracks the
    reference's 16 protons to 1 um, the same as alone to FP32 rounding, and the same as the
    FP64 kernel to 1 um."""
    _, cct = W.build_single_dipole()
    parts = golden["sd_particles_in"][:16]
    L = W.single_dipole_track_length()
    ds = engine.design_set_of([cct] * n_designs)
    out = engine.track(ds, np.stack([parts] * n_designs), L, 0.001, "f32c")
    one = engine.track(engine.design_of(cct), parts, L, 0.001, "f32c")[0]
    f64 = engine.track(engine.design_of(cct), parts, L, 0.001, "f64")[0]
    for d in range(n_designs):
        check(out[d], golden["sd_particles_out"][:16], POS_TOL_F32C, 1e-6)
        np.testing.assert_array_equal(out[d], out[0])
        assert np.abs(out[d][:, 0:3] - one[:, 0:3]).max() < 1e-8
        assert np.abs(out[d][:, 0:3] - f64[:, 0:3]).max() < POS_TOL_F32C


@pytest.mark.parametrize("n_designs", [1, 9])
def test_fp64_half_warp_blocks_of_16_protons(golden, n_designs):
    """FP64 designs of 16 protons run in blocks of 16 too (lanes l and l + 16 hold proton l
    and sum the two halves of every 32-segment group): one design on grid barriers, nine on
    the dataflow schedule.  Every copy tracks the reference's protons at the FP64 bar, and
    agrees with the same protons in a block of 32 (a 17th proton added) to rounding."""
    _, cct = W.build_single_dipole()
    parts = golden["sd_particles_in"][:16]
    L = W.single_dipole_track_length()
    ds = engine.design_set_of([cct] * n_designs)
    out = engine.track(ds, np.stack([parts] * n_designs), L, 0.001, "f64")
    blk32 = engine.track(engine.design_of(cct), golden["sd_particles_in"][:17], L, 0.001, "f64")[0][:16]
    for d in range(n_designs):
        check(out[d], golden["sd_particles_out"][:16], POS_TOL_F64, VEL_RTOL_F64)
        np.testing.assert_array_equal(out[d], out[0])
        assert np.abs(out[d][:, 0:3] - blk32[:, 0:3]).max() < 1e-12
        assert (np.abs(out[d][:, 3:6] - blk32[:, 3:6]) / np.abs(blk32[:, 3:6]).max()).max() < 1e-12


def test_bounded_small_batch_wait_reports_timeout(golden):
    """A small FP32c batch (the small-batch schedule: CTAs wait on unit counters between
    stages); the test hook makes every such wait ask for a stage more than exists: it gives
    up after the wait limit, reports CCT_ERR_TIMEOUT, and the context stays usable."""
    _, cct = W.build_single_dipole()
    ds = engine.design_of(cct)
    parts = golden["sd_particles_in"][:8]
    lib = _lib.load()
    lib.cct_test_set_flow_fault(1, 300)
    try:
        with pytest.raises(_lib.CctTimeoutError):
            engine.track(ds, parts, 0.01, 0.001, "f32c")
    finally:
        lib.cct_test_set_flow_fault(0, 0)
    out = engine.track(ds, parts, 0.01, 0.001, "f32c")
    assert np.isfinite(out).all()
