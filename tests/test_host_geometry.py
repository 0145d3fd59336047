"""Host-side logic of the package against the reference fixtures (CPU only):
magnet placement, winding segments, particle set-up, phase-space read-out."""
import math

import numpy as np
import pytest

from cctpy_gb300 import (CCT, HUST_SC_GANTRY, QS, Beamline, LocalCoordinateSystem, P2, P3, ParticleFactory,
                         PhaseSpaceParticle, RunningParticle, Trajectory, workloads as W)
from cctpy_gb300 import engine
from cctpy_gb300.particles import particles_to_array


def frame(m):
    return m.local_coordinate_system.axes()


def params_match(m, r):
    if r["kind"] == "cct":
        assert isinstance(m, CCT)
        assert m.big_r == r["big_r"] and m.small_r == r["small_r"]
        assert m.tilt_angles == r["tilt_angles"] and m.winding_number == r["winding_number"]
        assert m.current == r["current"] and m.disperse_number_per_winding == r["dpw"]
        assert np.allclose(m.starting_point_in_ksi_phi_coordinate.to_list(), r["start"], rtol=1e-15, atol=1e-15)
        assert np.allclose(m.end_point_in_ksi_phi_coordinate.to_list(), r["end"], rtol=1e-15, atol=1e-15)
    else:
        assert isinstance(m, QS)
        assert (m.length, m.gradient, m.second_gradient, m.aperture_radius) == (
            r["length"], r["gradient"], r["second_gradient"], r["aperture_radius"])


def test_single_dipole_placement(records_json):
    _, cct = W.build_single_dipole()
    r = records_json["single_dipole"][0]
    params_match(cct, r)
    assert np.allclose(frame(cct), np.array(r["frame"]), rtol=0, atol=1e-14)


@pytest.mark.parametrize("case,kw", [("hust2_default", {}),
                                     ("gantry_section", dict(agcct345_tilt_angles=[90.0, 30.0, 90.0, 90.0],
                                                             agcct345_current=-7000.0, part_per_winding=600))])
def test_gantry_placement(records_json, case, kw):
    bl = HUST_SC_GANTRY(**kw).create_second_bending_part_beamline()
    recs = records_json[case]
    assert len(bl.magnets) == len(recs) == 17
    for m, r in zip(bl.magnets, recs):
        params_match(m, r)
        assert np.allclose(frame(m), np.array(r["frame"]), rtol=0, atol=1e-12)


def test_first_section_placement(golden_hust1):
    bl = HUST_SC_GANTRY().create_first_bending_part_beamline()
    recs = golden_hust1["records"]
    assert len(bl.magnets) == len(recs) == 15
    for m, r in zip(bl.magnets, recs):
        params_match(m, r)
        assert np.allclose(frame(m), np.array(r["frame"]), rtol=0, atol=1e-12)
    assert abs(bl.get_length() - float(golden_hust1["h1_length"][0])) < 1e-12


def test_total_gantry_placement(golden_hust1):
    bl = HUST_SC_GANTRY().create_total_beamline()
    recs = golden_hust1["records_total"]
    assert len(bl.magnets) == len(recs) == 32
    for m, r in zip(bl.magnets, recs):
        params_match(m, r)
        assert np.allclose(frame(m), np.array(r["frame"]), rtol=0, atol=1e-12)
    assert abs(bl.get_length() - float(golden_hust1["tot_length"][0])) < 1e-12


def test_design_population_placement(records_json):
    for d, kw in enumerate(W.design_population(2, seed=3)):
        bl = HUST_SC_GANTRY(**kw).create_second_bending_part_beamline()
        for m, r in zip(bl.magnets, records_json["design_population"][d]):
            params_match(m, r)
            assert np.allclose(frame(m), np.array(r["frame"]), rtol=0, atol=1e-12)


def test_single_dipole_segments(golden):
    _, cct = W.build_single_dipole()
    idx = golden["sd_idx"]
    assert cct.total_disperse_number == 46080
    np.testing.assert_allclose(cct.elementary_current[idx], golden["sd_kl_local"], rtol=1e-12, atol=1e-20)
    np.testing.assert_allclose(cct.elementary_current_position[idx], golden["sd_p0_local"], rtol=0, atol=1e-15)
    kl, p0 = cct.global_segments()
    np.testing.assert_allclose(kl[idx], golden["sd_kl_global"], rtol=1e-12, atol=1e-20)
    np.testing.assert_allclose(p0[idx], golden["sd_p0_global"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(kl.sum(0), golden["sd_kl_global_sum"], rtol=1e-9, atol=1e-16)
    flat_kl, flat_p0 = cct.global_current_elements_and_elementary_current_positions()
    assert flat_kl.shape == (3 * 46080,) and np.array_equal(flat_kl, kl.reshape(-1))


def test_segment_counts(golden):
    bl = W.build_gantry_section()
    kl, p0, qs = engine.host_design(engine.magnet_list(bl))
    assert kl.shape[0] == int(golden["gs_n_seg"][0]) == 597600
    assert qs.shape == (1, 16)
    for d, kw in enumerate(W.design_population(2, seed=3)):
        bl = HUST_SC_GANTRY(**kw).create_second_bending_part_beamline()
        assert engine.host_design(engine.magnet_list(bl))[0].shape[0] == int(golden[f"dp{d}_n_seg"][0])


def test_particle_setup(golden):
    np.testing.assert_allclose(W.single_dipole_particles(32, 0), golden["sd_particles_in"], rtol=1e-14, atol=1e-14)
    bl = W.build_gantry_section()
    np.testing.assert_allclose(W.beam_particles(bl, 2, 2, 215.0), golden["gs_particles_in"], rtol=1e-14, atol=1e-14)


def test_phase_space_readout(golden):
    ideal = RunningParticle.from_numpy_array_data(golden["sd_ideal_end"])
    fr = ideal.get_natural_coordinate_system()
    ps = [RunningParticle.from_numpy_array_data(r) for r in golden["sd_particles_out"]]
    got = np.array([p.to_list() for p in PhaseSpaceParticle.create_from_running_particles(ideal, fr, ps)])
    np.testing.assert_allclose(got, golden["sd_ps_out"], rtol=1e-12, atol=1e-15)


def test_errors_match_reference():
    lcs = LocalCoordinateSystem()
    with pytest.raises(ValueError):
        CCT(lcs, 1.0, 0.1, -10, [30], 10, 100, P2(), P2(1, 1))
    with pytest.raises(ValueError):
        CCT(lcs, 1.0, 1.1, 10, [30], 10, 100, P2(), P2(1, 1))
    bl = Beamline.set_start_point(P2()).first_drift(P2.x_direct(), 1.0)
    with pytest.raises(ValueError):
        bl.append_agcct(1.0, [0.1, 0.2, 0.3, 0.4], [10], [[30], [90, 30]], [[10], [5]], [100, 100])
    with pytest.raises(ValueError):
        engine.host_design([object()])
