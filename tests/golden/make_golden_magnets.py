"""Golden fixture of the magnets beside the CCT and QS on the tracking path, generated from the
cctpy reference itself: Wire (cct.py:625-691, create_by_cct :814-832), AGCCT_CONNECTOR
(cct.py:835-994), Q (magnets.py:762-832), LocalUniformMagnet (magnets.py:440-536),
UniformMagnet (magnets.py:417-437), the Beamline builders append_q / append_straight_dipole_magnet
(beamline.py:420-505), and a CPU track through a Q and a straight dipole.

    python tests/golden/make_golden_magnets.py      # writes golden_magnets.npz

The connector joins layers 5 and 7 of the AG-CCT of the reference's own connector example
(final_code/工具集/AGCCT连接.py:20-45).
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import load_reference, particles_array  # noqa: E402


def fields(m, pts):
    from packages.point import P3
    return np.array([m.magnetic_field_at(P3(*map(float, p))).to_list() for p in pts])


def main():
    load_reference()
    from packages.base_utils import BaseUtils
    from packages.beamline import Beamline
    from packages.cct import AGCCT_CONNECTOR, CCT, Wire
    from packages.constants import MM
    from packages.line3s import FunctionLine3
    from packages.local_coordinate_system import LocalCoordinateSystem
    from packages.magnets import CombinedMagnet, UniformMagnet
    from packages.particles import ParticleFactory, ParticleRunner
    from packages.point import P2, P3

    out = {}
    rng = np.random.default_rng(17)

    # ------------------------------------------------ AG-CCT connector
    R = 0.95
    bl = (Beamline.set_start_point(start_point=P2(R, BaseUtils.angle_to_radian(-20) * R))
          .first_drift(P2.y_direct(), BaseUtils.angle_to_radian(20) * R)
          .append_agcct(big_r=R, small_rs=[128 * MM + 9.5 * MM, 113 * MM + 9.5 * MM, 98 * MM + 9.5 * MM,
                                           83 * MM + 9.5 * MM],
                        bending_angles=[17.05, 27.27, 23.18],
                        tilt_angles=[[30, 87.076, 91.829, 85.857], [101.317, 30, 75.725, 92.044]],
                        winding_numbers=[[128], [25, 40, 34]], currents=[9536.310, -6259.974],
                        disperse_number_per_winding=36)
          .append_drift(BaseUtils.angle_to_radian(20) * R))
    a3, a4 = bl.magnets[5], bl.magnets[7]
    ac = AGCCT_CONNECTOR(a3, a4)
    lcs = ac.local_coordinate_system
    out["con_frame"] = np.array([lcs.location.to_list(), lcs.XI.to_list(), lcs.YI.to_list(), lcs.ZI.to_list()])
    out["con_kl_local"] = ac.elementary_current
    out["con_p0_local"] = ac.elementary_current_position
    out["con_current"] = np.array([ac.current])
    end = a3.p3_function(a3.end_point_in_ksi_phi_coordinate.x)
    centre = lcs.point_to_global_coordinate(end)
    pts = np.array([[centre.x + d[0], centre.y + d[1], centre.z + d[2]] for d in rng.uniform(-0.05, 0.05, (8, 3))])
    out["con_pts"] = pts
    out["con_B"] = fields(ac, pts)
    out["con_linked_B"] = fields(CombinedMagnet(a3, ac, a4), pts)

    # ------------------------------------------------ wires
    small = CCT(LocalCoordinateSystem.global_coordinate_system(), 0.95, 83 * MM, 22.5, [30, 80, 90, 90], 4, 9000.0,
                P2(0, 0), P2(2 * math.pi * 4, BaseUtils.angle_to_radian(22.5)), 36)
    w = Wire.create_by_cct(small)
    out["wcct_kl"] = w.elementary_current
    out["wcct_p0"] = w.elementary_current_position
    wp = np.array([[0.95, 0.01, 0.0], [0.93, 0.1, 0.02], [0.9, 0.2, -0.03], [0.85, 0.3, 0.0]])
    out["wcct_pts"] = wp
    out["wcct_B"] = fields(w, wp)
    helix = Wire(FunctionLine3(lambda s: P3(0.02 * math.cos(s), 0.02 * math.sin(s), 0.001 * s), 0.0, 20 * math.pi),
                 current=100.0, delta_length=0.05)
    out["whelix_kl"] = helix.elementary_current
    out["whelix_p0"] = helix.elementary_current_position
    hp = np.array([[0.0, 0.0, 0.03], [0.005, -0.004, 0.01], [0.03, 0.0, 0.02]])
    out["whelix_pts"] = hp
    out["whelix_B"] = fields(helix, hp)

    # ------------------------------------------------ Q, straight dipole, uniform field; a CPU track
    bq = (Beamline.set_start_point(P2.origin()).first_drift(P2.x_direct(), 0.2)
          .append_q(length=0.2, gradient=5.0, aperture_radius=30 * MM)
          .append_drift(0.1)
          .append_straight_dipole_magnet(magnetic_field=0.3, length=0.25, aperture_radius=40 * MM)
          .append_drift(0.15))
    q, lum = bq.magnets[0], bq.magnets[1]
    for name, m in (("q", q), ("lum", lum)):
        f = m.local_coordinate_system
        out[name + "_frame"] = np.array([f.location.to_list(), f.XI.to_list(), f.YI.to_list(), f.ZI.to_list()])
    qp = []
    for s in np.linspace(0.15, 0.75, 13):
        p, d = bq.point_at(float(s)), bq.direct_at(float(s))
        n = d.rotate(math.pi / 2)
        for off, z in ((0.0, 0.0), (0.01, 0.005), (-0.025, -0.01), (0.05, 0.0)):
            qp.append([p.x + n.x * off, p.y + n.y * off, z])
    qp = np.array(qp)
    out["ql_pts"] = qp
    out["q_B"] = fields(q, qp)
    out["lum_B"] = fields(lum, qp)
    out["bq_B"] = fields(bq, qp)
    uni = UniformMagnet(P3(0.1, -0.2, 0.3))
    out["uni_B"] = fields(uni, qp[:3])
    ip = ParticleFactory.create_proton_along(bq, 0.0, 250)
    from packages.particles import PhaseSpaceParticle
    ps = ParticleFactory.create_from_phase_space_particles(
        ip, ip.get_natural_coordinate_system(),
        [PhaseSpaceParticle(3 * MM, 2 * MM, -2 * MM, 1 * MM, 0.0, 0.01), PhaseSpaceParticle(-1 * MM, 0, 1 * MM, -2 * MM, 0, -0.02)])
    out["bq_particles_in"] = particles_array(ps)
    ParticleRunner.run_only(ps, bq, bq.get_length(), footstep=5 * MM, concurrency_level=1, report=False)
    out["bq_particles_out"] = particles_array(ps)
    out["bq_length"] = np.array([bq.get_length()])
    np.savez_compressed(os.path.join(HERE, "golden_magnets.npz"), **out)
    print("wrote golden_magnets.npz:", {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
