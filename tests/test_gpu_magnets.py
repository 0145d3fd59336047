"""Wires, AG-CCT connectors, Q, straight dipoles and uniform fields on the GPU (field and
tracking) against the reference's own values (golden_magnets.npz)."""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from cctpy_gb300 import GPU_ACCELERATOR, MM, P2, P3, Beamline, LocalCoordinateSystem, engine, workloads as W
from cctpy_gb300.geometry import FunctionLine3
from cctpy_gb300.magnets import AGCCT_CONNECTOR, CCT, CombinedMagnet, UniformMagnet, Wire
from cctpy_gb300.particles import RunningParticle
from tests.test_magnets_golden import agcct_beamline

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gm():
    return np.load(os.path.join(HERE, "golden", "golden_magnets.npz"))


def close(b, ref, rtol, atol=1e-14):
    n = np.linalg.norm(ref, axis=1)
    return np.all(np.linalg.norm(b - ref, axis=1) <= rtol * n + atol)


# FP64: relative; FP32c: the FP32-compensated bound (1e-7 |B| + 2e-8 T: FP32 segment offsets
# limit it near a lone wire, a few mm from its elements)
TOL = {"f64": (1e-12, 1e-14), "f32c": (1e-7, 2e-8)}


class CctpyLikeConnector:
    """Stands for cctpy's own AGCCT_CONNECTOR object (duck typing on its attributes)."""

    def __init__(self, gm):
        f = gm["con_frame"]
        self.local_coordinate_system = LocalCoordinateSystem(P3(*f[0]), P3(*f[1]), P3(*f[3]))
        self.current = float(gm["con_current"][0])
        self.elementary_current = gm["con_kl_local"]
        self.elementary_current_position = gm["con_p0_local"]


def test_connector_fields(gm):
    bl = agcct_beamline()
    ours = AGCCT_CONNECTOR(bl.magnets[5], bl.magnets[7])
    for con in (ours, CctpyLikeConnector(gm)):
        for prec in ("f64", "f32c"):
            assert close(engine.field_at_points(engine.design_of(con), gm["con_pts"], prec),
                         gm["con_B"], *TOL[prec]), prec
    linked = CombinedMagnet(bl.magnets[5], ours, bl.magnets[7])
    assert close(engine.field_at_points(engine.design_of(linked), gm["con_pts"], "f64"), gm["con_linked_B"], 1e-11)


def test_wire_fields(gm):
    small = CCT(LocalCoordinateSystem(), 0.95, 83 * MM, 22.5, [30, 80, 90, 90], 4, 9000.0, P2(0, 0),
                P2(2 * math.pi * 4, 22.5 / 180.0 * math.pi), 36)
    helix = Wire(FunctionLine3(lambda s: P3(0.02 * math.cos(s), 0.02 * math.sin(s), 0.001 * s), 0.0, 20 * math.pi),
                 current=100.0, delta_length=0.05)
    for w, name in ((Wire.create_by_cct(small), "wcct"), (helix, "whelix")):
        for prec in ("f64", "f32c"):
            assert close(w.magnetic_field_at_points(gm[name + "_pts"], prec), gm[name + "_B"], *TOL[prec]), (name, prec)


def bq_beamline():
    return (Beamline.set_start_point(P2()).first_drift(P2.x_direct(), 0.2)
            .append_q(length=0.2, gradient=5.0, aperture_radius=30 * MM).append_drift(0.1)
            .append_straight_dipole_magnet(magnetic_field=0.3, length=0.25, aperture_radius=40 * MM)
            .append_drift(0.15))


def test_q_straight_dipole_uniform_fields_bitwise(gm):
    bq = bq_beamline()
    q, lum = bq.magnets
    for prec in ("f64", "f32c"):
        np.testing.assert_array_equal(q.magnetic_field_at_points(gm["ql_pts"], prec), gm["q_B"])
        np.testing.assert_array_equal(lum.magnetic_field_at_points(gm["ql_pts"], prec), gm["lum_B"])
        np.testing.assert_array_equal(bq.magnetic_field_at_points(gm["ql_pts"], prec), gm["bq_B"])
    uni = UniformMagnet(P3(0.1, -0.2, 0.3))
    np.testing.assert_allclose(uni.magnetic_field_at_points(gm["ql_pts"][:3]), gm["uni_B"], rtol=1e-15, atol=1e-16)


def test_track_through_q_and_straight_dipole(gm):
    bq = bq_beamline()
    L = float(gm["bq_length"][0])
    for prec in ("f64", "f32c"):
        out = engine.track(engine.design_of(bq), gm["bq_particles_in"], L, 5 * MM, prec)[0]
        assert np.abs(out[:, 0:3] - gm["bq_particles_out"][:, 0:3]).max() <= 1e-12
        np.testing.assert_allclose(out[:, 3:6], gm["bq_particles_out"][:, 3:6], rtol=1e-12, atol=1e-6)


def test_accelerator_keeps_reference_errors(gm):
    bq = bq_beamline()
    p = RunningParticle.from_numpy_array_data(gm["bq_particles_in"][0])
    with pytest.raises(ValueError):
        GPU_ACCELERATOR().track_one_particle_with_multi_qs(bq, p, 0.1, 0.01)


def test_device_design_set_with_wire(gm):
    bl = agcct_beamline()
    con = AGCCT_CONNECTOR(bl.magnets[5], bl.magnets[7])
    mags = CombinedMagnet(bl.magnets[5], con, bl.magnets[7])
    host = engine.design_set_of([mags], segments="host")
    dev = engine.design_set_of([mags], segments="device")
    assert host.n_segments == dev.n_segments
    bh = engine.field_at_points(host, gm["con_pts"], "f64")
    bd = engine.field_at_points(dev, gm["con_pts"], "f64")
    assert close(bd, bh, 1e-11)


def test_small_batch_with_a_design_without_segments(gm, golden):
    """One small FP32c launch (the small-batch schedule) over a design with no current
    elements (a quadrupole and a straight dipole) and the single CCT dipole: the first design
    tracks as cctpy does (analytic fields only), the second as it does alone."""
    bq = bq_beamline()
    _, cct = W.build_single_dipole()
    L = float(gm["bq_length"][0])
    parts = np.stack([gm["bq_particles_in"], golden["sd_particles_in"][:2]])
    out = engine.track(engine.design_set_of([bq, cct]), parts, L, 5 * MM, "f32c")
    assert np.abs(out[0][:, 0:3] - gm["bq_particles_out"][:, 0:3]).max() <= 1e-12
    alone = engine.track(engine.design_of(cct), golden["sd_particles_in"][:2], L, 5 * MM, "f32c")[0]
    assert np.abs(out[1][:, 0:3] - alone[:, 0:3]).max() <= 1e-8
