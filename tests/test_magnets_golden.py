"""Magnets beside the CCT and QS (Wire, AGCCT_CONNECTOR, Q, LocalUniformMagnet, UniformMagnet):
the oracle's fields and this package's construction against tests/golden/golden_magnets.npz
(generated from cctpy itself by tests/golden/make_golden_magnets.py)."""
import math
import os

import numpy as np
import pytest

from cctpy_gb300 import MM, P2, P3, Beamline, LocalCoordinateSystem
from cctpy_gb300.magnets import AGCCT_CONNECTOR, CCT, Wire
from cctpy_gb300.geometry import FunctionLine3
from oracle import cct_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gm():
    return np.load(os.path.join(HERE, "golden", "golden_magnets.npz"))


def frame_of(a):
    return O.Frame.from_axes(*[tuple(r) for r in a])


def test_oracle_fields_bitwise(gm):
    con = O.SegmentsOracle(gm["con_kl_local"], gm["con_p0_local"], float(gm["con_current"][0]), frame_of(gm["con_frame"]))
    np.testing.assert_array_equal(np.array([con.field_at(tuple(p)) for p in gm["con_pts"]]), gm["con_B"])
    for name in ("wcct", "whelix"):
        w = O.SegmentsOracle(gm[name + "_kl"], gm[name + "_p0"], 1.0)
        np.testing.assert_array_equal(np.array([w.field_at(tuple(p)) for p in gm[name + "_pts"]]), gm[name + "_B"])
    q = O.QSOracle({"frame": frame_of(gm["q_frame"]), "length": 0.2, "gradient": 5.0, "second_gradient": 0.0,
                    "aperture_radius": 30 * MM})
    np.testing.assert_array_equal(np.array([q.field_at(tuple(p)) for p in gm["ql_pts"]]), gm["q_B"])
    lum = O.LocalUniformOracle(frame_of(gm["lum_frame"]), 0.25, 40 * MM, 0.3)
    np.testing.assert_array_equal(np.array([lum.field_at(tuple(p)) for p in gm["ql_pts"]]), gm["lum_B"])
    assert np.count_nonzero(gm["q_B"].any(axis=1)) > 0 and np.count_nonzero(~gm["lum_B"].any(axis=1)) > 0


def agcct_beamline():
    R = 0.95
    return (Beamline.set_start_point(P2(R, -20 / 180.0 * math.pi * R))
            .first_drift(P2.y_direct(), 20 / 180.0 * math.pi * R)
            .append_agcct(big_r=R, small_rs=[128 * MM + 9.5 * MM, 113 * MM + 9.5 * MM, 98 * MM + 9.5 * MM,
                                             83 * MM + 9.5 * MM],
                          bending_angles=[17.05, 27.27, 23.18],
                          tilt_angles=[[30, 87.076, 91.829, 85.857], [101.317, 30, 75.725, 92.044]],
                          winding_numbers=[[128], [25, 40, 34]], currents=[9536.310, -6259.974],
                          disperse_number_per_winding=36)
            .append_drift(20 / 180.0 * math.pi * R))


def test_connector_construction_matches_reference(gm):
    bl = agcct_beamline()
    ac = AGCCT_CONNECTOR(bl.magnets[5], bl.magnets[7])
    np.testing.assert_allclose(ac.elementary_current, gm["con_kl_local"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(ac.elementary_current_position, gm["con_p0_local"], rtol=0, atol=1e-13)
    lcs = ac.local_coordinate_system
    np.testing.assert_allclose(np.array([lcs.location.to_list(), lcs.XI.to_list(), lcs.YI.to_list(),
                                         lcs.ZI.to_list()]), gm["con_frame"], rtol=0, atol=1e-12)


def test_wires_match_reference(gm):
    small = CCT(LocalCoordinateSystem(), 0.95, 83 * MM, 22.5, [30, 80, 90, 90], 4, 9000.0, P2(0, 0),
                P2(2 * math.pi * 4, 22.5 / 180.0 * math.pi), 36)
    w = Wire.create_by_cct(small)
    np.testing.assert_array_equal(w.elementary_current, gm["wcct_kl"])
    np.testing.assert_array_equal(w.elementary_current_position, gm["wcct_p0"])
    helix = Wire(FunctionLine3(lambda s: P3(0.02 * math.cos(s), 0.02 * math.sin(s), 0.001 * s), 0.0, 20 * math.pi),
                 current=100.0, delta_length=0.05)
    np.testing.assert_array_equal(helix.elementary_current, gm["whelix_kl"])
    np.testing.assert_array_equal(helix.elementary_current_position, gm["whelix_p0"])


def test_q_and_straight_dipole_placement(gm):
    bq = (Beamline.set_start_point(P2()).first_drift(P2.x_direct(), 0.2)
          .append_q(length=0.2, gradient=5.0, aperture_radius=30 * MM).append_drift(0.1)
          .append_straight_dipole_magnet(magnetic_field=0.3, length=0.25, aperture_radius=40 * MM)
          .append_drift(0.15))
    for m, key in zip(bq.magnets, ("q_frame", "lum_frame")):
        f = m.local_coordinate_system
        np.testing.assert_array_equal(np.array([f.location.to_list(), f.XI.to_list(), f.YI.to_list(),
                                                f.ZI.to_list()]), gm[key])
