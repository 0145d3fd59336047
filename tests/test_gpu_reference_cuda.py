"""The engine beside cctpy's own CUDA tracking kernel on the same GPU and the same inputs.

cctpy's GPU path (final_code/packages/gpu_accelerator.py:100-1078, launched at :1931-2031) is
compiled for this device from cctpy's own source by ``oracle/ref_cuda_build.py`` (at build
time, where the cctpy sources are) and launched unmodified by ``oracle/ref_cuda.py``: one
block per beamline, particles one after another, every field a block-wide strided sum and
tree reduction.  Two beamlines of the reference's GPU speed test (the second with other
AG-CCT currents, so that a design mix-up shows) carry four 250 MeV protons through the
entrance of the AG-CCT.

* FP64: cctpy's FLOAT64 kernel and the engine's FP64 path agree to rounding: their field sums
  differ only in summation order.
* FP32: cctpy's FLOAT32 kernel (its speed-test configuration) is several orders of magnitude
  further from the FP64 track than the engine's FP32-compensated path.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

S0, LENGTH, STEP = 4.9, 1.2, 0.01      # m: from the end of the entrance drift into the AG-CCT
N_P = 4


def _setup():
    from oracle import ref_cuda
    if not ref_cuda.available():
        pytest.skip("cctpy's CUDA kernels were not built (oracle/ref_cuda_build.py needs cctpy's sources)")
    from cctpy_gb300 import engine, workloads as W
    from cctpy_gb300.particles import ParticleFactory, PhaseSpaceParticle, particles_to_array
    a = W.build_speed_test_beamline()
    b = W.build_speed_test_beamline(currents=(8000.0, 12000.0))
    ideal = ParticleFactory.create_proton_along(a, S0, 250.0)
    pss = W.gaussian_phase_space(N_P, seed=11)
    ps = particles_to_array(ParticleFactory.create_from_phase_space_particles(
        ideal, ideal.get_natural_coordinate_system(), [PhaseSpaceParticle(*map(float, r)) for r in pss]))
    designs = [engine.host_design(engine.magnet_list(bl)) for bl in (a, b)]
    return ref_cuda, engine, designs, ps


def test_fp64_matches_cctpy_cuda_kernel():
    ref_cuda, engine, designs, ps = _setup()
    ref = ref_cuda.ReferenceCudaTracker("f64")
    try:
        want, _, _ = ref.track(designs, ps, LENGTH, STEP)
    finally:
        ref.close()
    ds = engine.DesignSet(designs)
    got = engine.track(ds, ps, LENGTH, STEP, "f64")
    assert got.shape == want.shape == (2, N_P, 10)
    # the two designs really differ at this tolerance
    assert np.abs(want[0, :, :3] - want[1, :, :3]).max() > 1e-6
    pos = np.abs(got[:, :, :3] - want[:, :, :3]).max()
    vel = (np.abs(got[:, :, 3:6] - want[:, :, 3:6]) / np.abs(want[:, :, 3:6]).max()).max()
    assert pos < 1e-12, f"FP64 positions differ from cctpy's CUDA kernel by {pos:.3e} m"
    assert vel < 1e-12, f"FP64 velocities differ from cctpy's CUDA kernel by {vel:.3e} (relative)"


def test_fp32c_closer_to_fp64_than_cctpy_fp32_kernel():
    ref_cuda, engine, designs, ps = _setup()
    ds = engine.DesignSet(designs)
    truth = engine.track(ds, ps, LENGTH, STEP, "f64")
    ours = engine.track(ds, ps, LENGTH, STEP, "f32c")
    ref = ref_cuda.ReferenceCudaTracker("f32")
    try:
        theirs, _, _ = ref.track(designs, ps, LENGTH, STEP)
    finally:
        ref.close()
    err_ours = np.abs(ours[:, :, :3] - truth[:, :, :3]).max()
    err_ref = np.abs(theirs[:, :, :3] - truth[:, :, :3]).max()
    assert err_ours < 1e-6, f"FP32c position error {err_ours:.3e} m"
    assert err_ours * 10 < err_ref, f"FP32c {err_ours:.3e} m against cctpy's FLOAT32 kernel {err_ref:.3e} m"
    # the reference's FP32 kernel still tracks the same beam (its documented error: ~0.05 mm)
    assert err_ref < 1e-3


def test_gantry_designs_match_cctpy_cuda_kernel():
    """The workloads' own magnets through cctpy's kernels built with room for 700 000 current
    elements a beamline: the gantry section (597 600 segments + QS) and two designs of the
    population (their own, ragged segment counts: each block of cctpy's kernel reads its own
    padded slice), four 215 MeV protons each, 10 RK4 steps of the workloads' 1 mm from the
    start of the section.  FP64 agrees with cctpy's FLOAT64 kernel to rounding; FP32c is far
    closer to FP64 than cctpy's FLOAT32 kernel, which keeps positions in FP32."""
    ref_cuda, engine, _, _ = _setup()
    from cctpy_gb300 import HUST_SC_GANTRY, workloads as W
    g = W.build_gantry_section()
    pop = [HUST_SC_GANTRY(**kw).create_second_bending_part_beamline() for kw in W.design_population(2, seed=3)]
    designs = [engine.host_design(engine.magnet_list(b)) for b in [g] + pop]
    assert designs[0][0].shape[0] == 597600 and len({d[0].shape[0] for d in designs}) == 3
    ps = W.beam_particles(g, N_P, seed=2, kinetic_MeV=215.0)
    L, step = 0.01, 0.001
    ds = engine.DesignSet(designs)
    truth = engine.track(ds, ps, L, step, "f64")
    ours = engine.track(ds, ps, L, step, "f32c")
    got = {}
    for cfg in ("f64_700k", "f32_700k"):
        ref = ref_cuda.ReferenceCudaTracker(cfg)
        try:
            got[cfg] = ref.track(designs, ps, L, step)[0]
        finally:
            ref.close()
    want = got["f64_700k"]
    pos = np.abs(truth[:, :, :3] - want[:, :, :3]).max()
    vel = (np.abs(truth[:, :, 3:6] - want[:, :, 3:6]) / np.abs(want[:, :, 3:6]).max()).max()
    assert pos < 1e-12, f"FP64 positions differ from cctpy's CUDA kernel by {pos:.3e} m"
    assert vel < 1e-12, f"FP64 velocities differ from cctpy's CUDA kernel by {vel:.3e} (relative)"
    err_ours = np.abs(ours[:, :, :3] - truth[:, :, :3]).max()
    err_ref = np.abs(got["f32_700k"][:, :, :3] - truth[:, :, :3]).max()
    assert err_ours < 1e-8, f"FP32c position error {err_ours:.3e} m"
    assert err_ours * 10 < err_ref, f"FP32c {err_ours:.3e} m against cctpy's FLOAT32 kernel {err_ref:.3e} m"


def test_single_qs_calls_match_cctpy_single_qs_kernel():
    """cctpy's single-QS beamline kernel (track_multi_particle_beamline_for_magnet_with_single_qs,
    gpu_accelerator.py:1023-1041) gets one QS a beamline, the last one its host loop sees
    (gpu_accelerator.py:1834-1874).  The gantry's first bending section has three: the drop-in
    accelerator's single-QS call must agree with cctpy's kernel to rounding in FP64, and differ
    from the multi-QS call (which sums all three) by far more."""
    ref_cuda, engine, _, _ = _setup()
    from cctpy_gb300 import GPU_ACCELERATOR, HUST_SC_GANTRY, RunningParticle, workloads as W
    from cctpy_gb300.particles import particles_to_array
    bl = HUST_SC_GANTRY().create_first_bending_part_beamline()
    design = engine.host_design(engine.magnet_list(bl))
    assert design[2].shape[0] == 3
    ps = W.beam_particles(bl, N_P, seed=3, kinetic_MeV=215.0)
    L, step = bl.get_length(), 0.05
    ref = ref_cuda.ReferenceCudaTracker("f64", kernel="single_qs")
    try:
        want = ref.track([design, design], ps, L, step)[0]
    finally:
        ref.close()
    ga = GPU_ACCELERATOR(GPU_ACCELERATOR.FLOAT64, block_dim_x=512)
    rps = [RunningParticle.from_numpy_array_data(r) for r in ps]
    single = np.stack([particles_to_array(row) for row in
                       ga.track_multi_particle_beamline_for_magnet_with_single_qs([bl, bl], rps, L, step)])
    multi = np.stack([particles_to_array(row) for row in
                      ga.track_multi_particle_beamline_for_magnet_with_multi_qs([bl, bl], rps, L, step)])
    pos = np.abs(single[:, :, :3] - want[:, :, :3]).max()
    assert pos < 1e-12, f"single-QS FP64 positions differ from cctpy's single-QS kernel by {pos:.3e} m"
    assert np.abs(multi[:, :, :3] - want[:, :, :3]).max() > 1e-6
