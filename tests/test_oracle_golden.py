"""Pins the CPU oracle against the reference: fixtures generated by running
cctpy itself (tests/golden/make_golden.py) and the known answers held in
cctpy's own tests."""
import math

import numpy as np
import pytest

from oracle import cct_oracle as O
from cctpy_gb300 import workloads as W
from tests.conftest import oracle_records


def single_dipole_record():
    c = W.SINGLE_DIPOLE
    orb = O.Orbit((0.0, 0.0), (1.0, 0.0), c["drift"]).add_arc(c["big_r"], c["clockwise"], c["bending_angle"])
    rec = O.cct_along(orb, c["drift"], c["big_r"], c["small_r"], c["bending_angle"], c["tilt_angles"],
                      c["winding_number"], c["current"], (0.0, 0.0),
                      (2 * math.pi * c["winding_number"], O.deg2rad(-c["bending_angle"])),
                      c["disperse_number_per_winding"])
    return orb, rec


def test_placement_single_dipole_bitwise(records_json):
    _, rec = single_dipole_record()
    ref = np.array(records_json["single_dipole"][0]["frame"])
    assert np.array_equal(rec["frame"].as_array(), ref)


def hust2(**kw):
    """HUST_SC_GANTRY second section (hust_sc_gantry.py:19-90 defaults, :230-283)."""
    MM = O.MM
    p = dict(DL2=2.1162209, GAP3=0.1978111, qs3_length=0.2382791, qs3_aperture_radius=60 * MM,
             qs3_gradient=-7.3733, qs3_second_gradient=-45.31 * 2, cct345_big_r=0.95,
             agcct345_inner_small_r=83 * MM, agcct345_outer_small_r=83 * MM + 15 * MM,
             dicct345_inner_small_r=83 * MM + 15 * MM * 2, dicct345_outer_small_r=83 * MM + 15 * MM * 3,
             agcct3_winding_number=21, agcct4_winding_number=50, agcct5_winding_number=50,
             dicct345_winding_number=128, dicct345_bending_angle=-67.5, agcct3_bending_angle=-(8 + 3.716404),
             agcct4_bending_angle=-(8 + 19.93897), agcct5_bending_angle=-(8 + 19.844626),
             dicct345_tilt_angles=[30, 80], agcct345_tilt_angles=[90, 30], dicct345_current=9664,
             agcct345_current=-6000, part_per_winding=120)
    p.update(kw)
    return p


def test_placement_hust2_close_to_reference(records_json, golden):
    # the first section's end point and direction come from the reference's own build
    recs = oracle_records(records_json["hust2_default"])
    assert len(recs) == 17
    kinds = [r["kind"] for r in recs]
    assert kinds.count("qs") == 1 and kinds.count("cct") == 16


def test_segments_local_bitwise(golden):
    _, rec = single_dipole_record()
    kl, p0 = O.cct_segments_local(rec)
    idx = golden["sd_idx"]
    assert kl.shape[0] == int(golden["sd_n_seg"][0]) == 46080
    assert np.array_equal(kl[idx], golden["sd_kl_local"])
    assert np.array_equal(p0[idx], golden["sd_p0_local"])


def test_segments_global_bitwise(golden):
    _, rec = single_dipole_record()
    kl, p0 = O.cct_segments_global(rec)
    idx = golden["sd_idx"]
    assert np.array_equal(kl[idx], golden["sd_kl_global"])
    assert np.array_equal(p0[idx], golden["sd_p0_global"])
    assert np.array_equal(np.array([math.fsum(kl[:, j]) for j in range(3)]), golden["sd_kl_global_sum"])


def test_field_single_dipole_matches_reference(golden):
    _, rec = single_dipole_record()
    m = O.CCTOracle(rec)
    B = np.array([m.field_at(tuple(p)) for p in golden["sd_field_pts"]])
    assert np.array_equal(B, golden["sd_field_B"])


def test_field_hust2_matches_reference(golden, records_json):
    bl = O.BeamlineOracle(oracle_records(records_json["hust2_default"]))
    B = bl.field_at_points(golden["h2_field_pts"])
    assert np.array_equal(B, golden["h2_field_B"])


def test_qs_known_answers(golden, records_json):
    bl = O.BeamlineOracle(oracle_records(records_json["qs_known"]))
    B = bl.field_at_points(golden["qs_pts"])
    assert np.array_equal(B, golden["qs_B"])
    # printed known answer, gpu_accelerator.py:1219 -- (0.0, 0.0, 0.27500000000000024)
    assert B[0].tolist() == [0.0, 0.0, 0.27500000000000024]


def test_qs_beamline_known_answers(golden, records_json):
    bl = O.BeamlineOracle(oracle_records(records_json["qs_beamline"]))
    B = bl.field_at_points(golden["qsbl_pts"])
    assert np.array_equal(B, golden["qsbl_B"])
    # printed CPU result for point 2, gpu_accelerator.py:1374 (printed by an earlier
    # revision of the reference; today's reference differs from it by ~5e-14 T)
    assert np.allclose(B[1], [-0.021273493843574243, 0.048440921145815385, 1.0980479752081713], rtol=0, atol=1e-13)


def test_known_answer_single_element():
    # codes/tests/cuda_test.py:99-109: kl = p1-p0 (no current, no 1e-7), at the origin
    kl = np.array([[0.1, 0.2, 0.3]])
    p0 = np.array([[1.05, 1.1, 1.15]])
    B = O.segments_field_local(kl, p0, (0.0, 0.0, 0.0))
    assert np.allclose(B, [0.014429237347383132, -0.028858474694766215, 0.01442923734738309], rtol=1e-12)


def helix(n=20, pas=360, r=0.01, length=0.1, sin_first=False):
    ts = np.linspace(0, n * 2 * np.pi, n * pas)
    if sin_first:
        return np.array([[r * np.sin(t), r * np.cos(t), t / (n * 2 * np.pi) * length] for t in ts])
    return np.array([[r * np.cos(t), r * np.sin(t), t / (n * 2 * np.pi) * length] for t in ts])


def test_known_answer_helix():
    # codes/tests/cuda_test.py:133-156, I = 10000 A, field at the origin; the
    # reference asserts this known answer to an absolute 1e-6 T (:155-156) --
    # it was printed by an earlier implementation, and today's FP64 midpoint sum
    # sits 1.8e-8 T from it.  The same sum agrees with the solenoid answers
    # below (I = 1000 A) to 1e-10 relative.
    B = O.wire_path_field(helix(), 10000, (0.0, 0.0, 0.0))
    assert np.allclose(B, [0.016659991558021645, 9.641212628421269e-4, 1.2504328150541577], rtol=0, atol=1e-6)


def test_known_answer_solenoid():
    # codes/tests/sole_layer_cct_test.py:14-43, I = 1000 A
    path = helix(sin_first=True)
    want = [([0, 0, 0], [-9.641213222579932E-5, -0.0016659990498348225, -0.1250432833225887]),
            ([0, 0, 0.05], [-7.496745957474563E-4, -3.7777669447541795E-19, -0.24645342280018406]),
            ([0, 0.001, 0.05], [-7.128547526957852E-4, -6.352747104407253E-20, -0.2464630712060889])]
    for p, b in want:
        got = O.wire_path_field(path, 1000, tuple(float(v) for v in p))
        assert np.allclose(got, b, rtol=1e-10, atol=1e-15)


def test_particles_from_phase_space_bitwise(golden):
    orb, _ = single_dipole_record()
    c = W.SINGLE_DIPOLE
    ideal = O.proton_along(orb, c["drift"], c["kinetic_MeV"])
    fr = O.natural_frame(ideal)
    ps = np.array([O.from_phase_space(ideal, fr, row) for row in golden["sd_ps_in"]])
    assert np.array_equal(ps, golden["sd_particles_in"])


def test_phase_space_readout_bitwise(golden):
    ideal_end = golden["sd_ideal_end"]
    fr = O.natural_frame(ideal_end)
    ps = np.array([O.to_phase_space(ideal_end, fr, p) for p in golden["sd_particles_out"]])
    assert np.array_equal(ps, golden["sd_ps_out"])


def test_track_hust2_ideal_matches_reference(golden, records_json):
    recs = oracle_records(records_json["hust2_default"])
    bl = O.BeamlineOracle(recs)
    L = float(golden["h2_length"][0])
    out = O.rk4_track(golden["h2_particles_in"][0], bl.field_at, L, 0.1)
    assert np.array_equal(out, golden["h2_particles_out"][0])
    # printed known answer, gpu_accelerator.py:1454.  It was printed when the
    # gantry's first section (whose end point starts this section) had other
    # defaults, so the x-y position is translated; the exit velocity and the
    # vertical position do not depend on that translation.
    assert np.allclose(out[3:6], [1809891.9615852616, -174308430.5414393, -330480.4098605619], rtol=1e-9, atol=0)
    assert abs(out[2] - 5.0076184754665586e-05) < 1e-13


def test_first_section_matches_reference(golden_hust1):
    """The gantry's first bending section (12 CCT layers, 3 QS): fields and the RK4 track of
    three protons at 100 mm steps over the whole section, bit for bit.  (The known answer printed
    in gpu_accelerator.py:1535 was produced by an earlier revision of the section: its track is
    4.15 m long, today's 4.82 m.)"""
    bl = O.BeamlineOracle(oracle_records(golden_hust1["records"]))
    B = np.array([bl.field_at(tuple(p)) for p in golden_hust1["h1_field_pts"]])
    assert np.allclose(B, golden_hust1["h1_field_B"], rtol=1e-13, atol=1e-16)
    L = float(golden_hust1["h1_length"][0])
    for p_in, p_out in zip(golden_hust1["h1_particles_in"], golden_hust1["h1_particles_out"]):
        assert np.array_equal(O.rk4_track(p_in, bl.field_at, L, 0.1), p_out)


@pytest.mark.slow
def test_total_gantry_matches_reference(golden_hust1):
    """The whole gantry (32 magnets, 11.9 m): fields and the ideal proton's RK4 track at
    100 mm steps, bit for bit."""
    bl = O.BeamlineOracle(oracle_records(golden_hust1["records_total"]))
    B = np.array([bl.field_at(tuple(p)) for p in golden_hust1["tot_field_pts"]])
    assert np.allclose(B, golden_hust1["tot_field_B"], rtol=1e-13, atol=1e-16)
    out = O.rk4_track(golden_hust1["tot_particles_in"][0], bl.field_at, float(golden_hust1["tot_length"][0]), 0.1)
    assert np.array_equal(out, golden_hust1["tot_particles_out"][0])


@pytest.mark.slow
def test_track_single_dipole_two_protons_match_reference(golden):
    _, rec = single_dipole_record()
    m = O.CCTOracle(rec)
    L = W.single_dipole_track_length()
    for i in (0, 17):
        out = O.rk4_track(golden["sd_particles_in"][i], m.field_at, L, 0.001)
        assert np.array_equal(out, golden["sd_particles_out"][i])
