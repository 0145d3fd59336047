"""Generate the golden fixtures of the parity tests from the cctpy reference itself.

Run where the cctpy sources are available, with ``CCTPY_REFERENCE`` set to the
directory that holds cctpy's ``final_code/``:

    CCTPY_REFERENCE=<cctpy checkout> python tests/golden/make_golden.py

The reference is imported unmodified with two harness-side shims:
matplotlib is stubbed (every package module imports pyplot at top level but
the tracking path never calls it) and ``P2.from_numpy_ndarry`` is given a
(2, 1) -> (2,) reshape, since numpy 2 rejects ``float()`` of a 1-element array
inside ``BaseUtils.circle_center_and_radius`` (base_utils.py:140-145).

Outputs (small, committed): ``golden.npz`` (arrays) and ``records.json``
(magnet placement and parameters, as the reference built them).
"""
from __future__ import annotations

import json
import math
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from cctpy_gb300 import workloads  # noqa: E402

REF = os.environ.get("CCTPY_REFERENCE", "")


def load_reference():
    if not REF or not os.path.isdir(os.path.join(REF, "final_code")):
        raise SystemExit("set CCTPY_REFERENCE to the directory holding cctpy's final_code/ "
                         f"(got {REF!r})")
    for name in ["matplotlib", "matplotlib.pyplot", "mpl_toolkits", "mpl_toolkits.mplot3d"]:
        sys.modules[name] = types.ModuleType(name)
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    sys.modules["mpl_toolkits"].mplot3d = sys.modules["mpl_toolkits.mplot3d"]

    class _Any:
        def __getattr__(self, k):
            return _Any()

        def __call__(self, *a, **k):
            return _Any()

    sys.modules["mpl_toolkits.mplot3d"].Axes3D = _Any
    sys.path.insert(0, os.path.join(REF, "final_code"))
    import packages.point as pt
    orig = pt.P2.from_numpy_ndarry

    def reshaped(nd):
        if isinstance(nd, np.ndarray) and nd.shape == (2, 1):
            nd = nd.reshape(2)
        return orig(nd)

    pt.P2.from_numpy_ndarry = staticmethod(reshaped)


def frame_of(lcs):
    return [lcs.location.to_list(), lcs.XI.to_list(), lcs.YI.to_list(), lcs.ZI.to_list()]


def record_of(m):
    from packages.cct import CCT
    from packages.magnets import QS
    if isinstance(m, CCT):
        return dict(kind="cct", frame=frame_of(m.local_coordinate_system), big_r=m.big_r, small_r=m.small_r,
                    bending_angle=m.bending_angle, tilt_angles=list(m.tilt_angles),
                    winding_number=m.winding_number, current=m.current,
                    start=m.starting_point_in_ksi_phi_coordinate.to_list(),
                    end=m.end_point_in_ksi_phi_coordinate.to_list(), dpw=m.disperse_number_per_winding)
    if isinstance(m, QS):
        return dict(kind="qs", frame=frame_of(m.local_coordinate_system), length=m.length,
                    gradient=m.gradient, second_gradient=m.second_gradient,
                    aperture_radius=m.aperture_radius)
    raise ValueError(m)


def particles_array(ps):
    return np.array([p.to_numpy_array_data(np.float64) for p in ps])


def make_particles(ideal, pss):
    from packages.particles import ParticleFactory, PhaseSpaceParticle
    frame = ideal.get_natural_coordinate_system()
    pps = [PhaseSpaceParticle(*[float(v) for v in row]) for row in pss]
    return ParticleFactory.create_from_phase_space_particles(ideal, frame, pps)


def phase_space_of(ideal_end, ps):
    from packages.particles import PhaseSpaceParticle
    out = PhaseSpaceParticle.create_from_running_particles(ideal_end, ideal_end.get_natural_coordinate_system(), ps)
    return np.array([[p.x, p.xp, p.y, p.yp, p.z, p.delta] for p in out])


def field_points(m, pts):
    from packages.point import P3
    return np.array([m.magnetic_field_at(P3(*p)).to_list() for p in pts])


def main():
    load_reference()
    from packages.point import P2, P3
    from packages.constants import MM
    from packages.base_utils import BaseUtils
    from packages.trajectory import Trajectory
    from packages.cct import CCT
    from packages.magnets import QS
    from packages.local_coordinate_system import LocalCoordinateSystem
    from packages.beamline import Beamline
    from packages.particles import ParticleFactory, ParticleRunner
    from hust_sc_gantry import HUST_SC_GANTRY

    arrays = {}
    records = {}
    t00 = time.time()

    # ---------------------------------------------------------------- single dipole (46 080 segments)
    c = workloads.SINGLE_DIPOLE
    traj = (Trajectory.set_start_point(P2.origin()).first_line(P2.x_direct(), c["drift"])
            .add_arc_line(c["big_r"], c["clockwise"], c["bending_angle"]))
    cct = CCT.create_cct_along(traj, c["drift"], c["big_r"], c["small_r"], c["bending_angle"], c["tilt_angles"],
                               c["winding_number"], c["current"], P2(0, 0),
                               P2(2 * math.pi * c["winding_number"],
                                  BaseUtils.angle_to_radian(-c["bending_angle"])),
                               c["disperse_number_per_winding"])
    records["single_dipole"] = [record_of(cct)]
    n = cct.total_disperse_number
    idx = np.arange(0, n, 997)
    kls, p0s = cct.global_current_elements_and_elementary_current_positions(np.float64)
    kls, p0s = kls.reshape(-1, 3), p0s.reshape(-1, 3)
    arrays["sd_idx"] = idx
    arrays["sd_kl_local"] = cct.elementary_current[idx]
    arrays["sd_p0_local"] = cct.elementary_current_position[idx]
    arrays["sd_kl_global"] = kls[idx]
    arrays["sd_p0_global"] = p0s[idx]
    arrays["sd_kl_global_sum"] = np.array([math.fsum(kls[:, j]) for j in range(3)])
    arrays["sd_p0_global_sum"] = np.array([math.fsum(p0s[:, j]) for j in range(3)])
    arrays["sd_n_seg"] = np.array([n])
    pts = workloads.field_map_points(64, seed=11)
    arrays["sd_field_pts"] = pts
    arrays["sd_field_B"] = field_points(cct, pts)
    L = workloads.single_dipole_track_length()
    ideal = ParticleFactory.create_proton_along(traj, c["drift"], c["kinetic_MeV"])
    ideal_end = ParticleFactory.create_proton_along(traj, c["drift"] + L, c["kinetic_MeV"])
    pss = workloads.uniform_ellipse_phase_space(32, seed=0)
    ps = make_particles(ideal, pss)
    arrays["sd_ps_in"] = pss
    arrays["sd_particles_in"] = particles_array(ps)
    arrays["sd_ideal_end"] = ideal_end.to_numpy_array_data(np.float64)
    t0 = time.time()
    ParticleRunner.run_only(ps, cct, L, footstep=c["footstep"], concurrency_level=os.cpu_count(), report=False)
    print(f"single dipole: tracked 32 protons in {time.time() - t0:.1f} s")
    arrays["sd_particles_out"] = particles_array(ps)
    arrays["sd_ps_out"] = phase_space_of(ideal_end, ps)

    # ---------------------------------------------------------------- HUST second section, default build
    g = HUST_SC_GANTRY()
    bl = g.create_second_bending_part_beamline()
    records["hust2_default"] = [record_of(m) for m in bl.magnets]
    s_pts = np.linspace(0.0, bl.get_length(), 16)
    pts = []
    for k, s in enumerate(s_pts):
        p = bl.point_at(s)
        d = bl.direct_at(s)
        off = d.rotate(math.pi / 2).change_length(((k % 5) - 2) * 10 * MM)
        pts.append([p.x + off.x, p.y + off.y, ((k % 3) - 1) * 8 * MM])
    pts = np.array(pts)
    arrays["h2_field_pts"] = pts
    arrays["h2_field_B"] = field_points(bl, pts)
    ideal = ParticleFactory.create_proton_along(bl, kinetic_MeV=215)
    ideal_end = ParticleFactory.create_proton_along(bl, bl.get_length(), kinetic_MeV=215)
    pss = workloads.gaussian_phase_space(3, seed=21)
    ps = [ideal.copy()] + make_particles(ideal, pss)
    arrays["h2_particles_in"] = particles_array(ps)
    arrays["h2_length"] = np.array([bl.get_length()])
    arrays["h2_ideal_end"] = ideal_end.to_numpy_array_data(np.float64)
    t0 = time.time()
    ParticleRunner.run_only(ps, bl, bl.get_length(), footstep=100 * MM, concurrency_level=4, report=False)
    print(f"hust2 default: tracked 4 protons in {time.time() - t0:.1f} s")
    arrays["h2_particles_out"] = particles_array(ps)

    # ---------------------------------------------------------------- gantry section workload (597 600 segments)
    gs = workloads.GANTRY_SECTION
    g = HUST_SC_GANTRY(agcct345_tilt_angles=gs["agcct345_tilt_angles"], agcct345_current=gs["agcct345_current"],
                       part_per_winding=gs["part_per_winding"])
    bl = g.create_second_bending_part_beamline()
    records["gantry_section"] = [record_of(m) for m in bl.magnets]
    arrays["gs_n_seg"] = np.array([sum(m.total_disperse_number for m in bl.magnets if isinstance(m, CCT))])
    pts = np.array([[bl.point_at(s).x, bl.point_at(s).y, 0.005] for s in np.linspace(0.5, 6.5, 6)])
    arrays["gs_field_pts"] = pts
    arrays["gs_field_B"] = field_points(bl, pts)
    ideal = ParticleFactory.create_proton_along(bl, kinetic_MeV=gs["kinetic_MeV"])
    pss = workloads.gaussian_phase_space(2, seed=2)
    ps = make_particles(ideal, pss)
    arrays["gs_ps_in"] = pss
    arrays["gs_particles_in"] = particles_array(ps)
    t0 = time.time()
    ParticleRunner.run_only(ps, bl, gs["track_length"], footstep=50 * MM, concurrency_level=2, report=False)
    print(f"gantry section: tracked 2 protons in {time.time() - t0:.1f} s")
    arrays["gs_particles_out"] = particles_array(ps)

    # ---------------------------------------------------------------- design population (two designs)
    designs = workloads.design_population(2, seed=3)
    records["design_population"] = []
    for d, kw in enumerate(designs):
        bl = HUST_SC_GANTRY(**kw).create_second_bending_part_beamline()
        records["design_population"].append([record_of(m) for m in bl.magnets])
        ideal = ParticleFactory.create_proton_along(bl, kinetic_MeV=215)
        ps = make_particles(ideal, workloads.gaussian_phase_space(2, seed=30 + d))
        arrays[f"dp{d}_particles_in"] = particles_array(ps)
        arrays[f"dp{d}_n_seg"] = np.array([sum(m.total_disperse_number for m in bl.magnets
                                               if isinstance(m, CCT))])
        ParticleRunner.run_only(ps, bl, 1.0 + bl.get_length() * 0.2, footstep=50 * MM, concurrency_level=2,
                                report=False)
        arrays[f"dp{d}_length"] = np.array([1.0 + bl.get_length() * 0.2])
        arrays[f"dp{d}_particles_out"] = particles_array(ps)

    # ---------------------------------------------------------------- QS known answers (gpu_accelerator.py:1198-1222)
    qs = QS(local_coordinate_system=LocalCoordinateSystem(location=P3(1, 0, 0), x_direction=-P3.x_direct(),
                                                          z_direction=P3.y_direct()),
            length=0.27, gradient=5, second_gradient=20, aperture_radius=100 * MM)
    records["qs_known"] = [record_of(qs)]
    qpts = np.array([[0.95, 0, 0], [1.02, 0.1, 0.03], [0.99, 0.2, -0.05], [1.0, 0.28, 0.0], [0.9, 0.1, 0.01]])
    arrays["qs_pts"] = qpts
    arrays["qs_B"] = field_points(qs, qpts)

    # beamline with one QS and a dipole CCT pair (gpu_accelerator.py:1349-1376)
    bl = (Beamline.set_start_point(P2.origin()).first_drift(direct=P2.x_direct(), length=1)
          .append_qs(length=0.27, gradient=5, second_gradient=20, aperture_radius=100 * MM)
          .append_drift(length=1)
          .append_dipole_cct(big_r=1, small_r_inner=100 * MM, small_r_outer=120 * MM, bending_angle=45,
                             tilt_angles=[30], winding_number=60, current=10000)
          .append_drift(length=1))
    records["qs_beamline"] = [record_of(m) for m in bl.magnets]
    bpts = np.array([[1.2, 50 * MM, 0], [2.3, 50 * MM, 0]])
    arrays["qsbl_pts"] = bpts
    arrays["qsbl_B"] = field_points(bl, bpts)

    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    with open(os.path.join(HERE, "records.json"), "w") as f:
        json.dump(records, f, indent=1)
    print(f"done in {time.time() - t00:.1f} s")


if __name__ == "__main__":
    main()
