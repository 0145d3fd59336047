"""Seeded synthetic inputs for the benchmark and parity workloads.

The workloads (sizes, seeds and distributions) are:

* ``single_dipole`` -- one CCT bending-dipole layer: bending radius 0.95 m,
  aperture radius 83 mm, 22.5 deg clockwise bend, tilt angles [30, 80, 90, 90]
  deg, 128 turns x 360 segments (46 080 segments), 9000 A, placed after a
  0.1 m drift along +x; 32 protons at 250 MeV with (x, xp) and (y, yp)
  uniform inside a 3.5 mm x 7.5 mrad ellipse and delta uniform in +-1 %,
  tracked 0.95 m x 22.5 deg (0.37306 m) at a 1 mm RK4 step (374 steps).
* ``field_map`` -- 2**20 field points uniform in a 60 mm-radius tube around the
  single-dipole design arc (uniform in arc length and in the disc).
* ``gantry_section`` -- the HUST gantry second bending section with AG-CCT tilt
  angles [90, 30, 90, 90], AG current -7000 A and 600 segments per turn
  (597 600 segments, 16 CCT layers + 1 QS); 4096 protons at 215 MeV with
  Gaussian sigma_x = 1 mm, sigma_xp = 2 mrad (same in y) and delta uniform in
  +-2 %, RK4 step 1 mm over 3.5 m.
* ``design_population`` -- 64 second-section designs with seeded tilt angles,
  currents and winding counts (uneven segment totals), 512 protons each.

Only numpy is used here; geometry is built by the package's beamline module.
"""
from __future__ import annotations

import math

import numpy as np

MM = 0.001

SINGLE_DIPOLE = dict(drift=0.1, big_r=0.95, small_r=83 * MM, bending_angle=22.5, clockwise=True,
                     tilt_angles=[30.0, 80.0, 90.0, 90.0], winding_number=128, current=9000.0,
                     disperse_number_per_winding=360, kinetic_MeV=250.0, footstep=1 * MM)


def single_dipole_track_length() -> float:
    return SINGLE_DIPOLE["big_r"] * math.radians(SINGLE_DIPOLE["bending_angle"])


def uniform_ellipse_phase_space(n: int, seed: int, x_max=3.5 * MM, xp_max=7.5 * MM, y_max=3.5 * MM,
                                yp_max=7.5 * MM, delta_max=0.01) -> np.ndarray:
    """(n, 6) phase-space tuples (x, xp, y, yp, z, delta): (x, xp) and (y, yp)
    uniform inside the ellipses, z = 0, delta uniform in +-delta_max."""
    rng = np.random.default_rng(seed)
    out = np.zeros((n, 6))
    for col, (a, b) in ((0, (x_max, xp_max)), (2, (y_max, yp_max))):
        r = np.sqrt(rng.random(n))
        t = rng.random(n) * 2 * math.pi
        out[:, col] = a * r * np.cos(t)
        out[:, col + 1] = b * r * np.sin(t)
    out[:, 5] = rng.uniform(-delta_max, delta_max, n)
    return out


def gaussian_phase_space(n: int, seed: int, sx=1 * MM, sxp=2 * MM, sy=1 * MM, syp=2 * MM,
                         delta_max=0.02) -> np.ndarray:
    """(n, 6) Gaussian transverse phase space, delta uniform in +-delta_max."""
    rng = np.random.default_rng(seed)
    out = np.zeros((n, 6))
    out[:, 0] = rng.normal(0.0, sx, n)
    out[:, 1] = rng.normal(0.0, sxp, n)
    out[:, 2] = rng.normal(0.0, sy, n)
    out[:, 3] = rng.normal(0.0, syp, n)
    out[:, 5] = rng.uniform(-delta_max, delta_max, n)
    return out


def field_map_points(n: int, seed: int = 1, tube_radius: float = 60 * MM) -> np.ndarray:
    """(n, 3) points uniform in a tube around the single-dipole design arc.

    The arc starts at (drift, 0, 0) heading +x and bends clockwise with radius R
    about the centre (drift, -R, 0)."""
    c = SINGLE_DIPOLE
    R, d0 = c["big_r"], c["drift"]
    L = single_dipole_track_length()
    rng = np.random.default_rng(seed)
    s = rng.random(n) * L
    rho = tube_radius * np.sqrt(rng.random(n))
    th = rng.random(n) * 2 * math.pi
    phi = math.pi / 2 - s / R
    radial = np.stack([np.cos(phi), np.sin(phi), np.zeros(n)], axis=1)
    base = np.stack([d0 + R * np.cos(phi), -R + R * np.sin(phi), np.zeros(n)], axis=1)
    return base + (rho * np.cos(th))[:, None] * radial + (rho * np.sin(th))[:, None] * np.array([0, 0, 1.0])


GANTRY_SECTION = dict(agcct345_tilt_angles=[90.0, 30.0, 90.0, 90.0], agcct345_current=-7000.0,
                      part_per_winding=600, kinetic_MeV=215.0, footstep=1 * MM, track_length=3.5)


def design_population(n: int, seed: int = 3, part_per_winding: int = 360):
    """Seeded second-section design parameters (keyword arguments of the
    HUST_SC_GANTRY builder): 4 dipole + 4 AG tilt angles uniform in [20, 160]
    deg, dipole and AG currents uniform in [-10000, 10000] A, dipole winding
    count uniform in [64, 160] and AG part winding counts uniform in [21, 100]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        t = rng.uniform(20.0, 160.0, 8)
        cur = rng.uniform(-10000.0, 10000.0, 2)
        wd = int(rng.integers(64, 161))
        wa = [int(w) for w in rng.integers(21, 101, 3)]
        out.append(dict(dicct345_tilt_angles=[float(x) for x in t[:4]],
                        agcct345_tilt_angles=[float(x) for x in t[4:]],
                        dicct345_current=float(cur[0]), agcct345_current=float(cur[1]),
                        dicct345_winding_number=wd, agcct3_winding_number=wa[0],
                        agcct4_winding_number=wa[1], agcct5_winding_number=wa[2],
                        part_per_winding=part_per_winding))
    return out


# ---------------------------------------------------------------- builders (this package's classes)
def build_single_dipole():
    """(trajectory, CCT) of the single-dipole workload."""
    from .geometry import P2, Trajectory
    from .magnets import CCT
    c = SINGLE_DIPOLE
    traj = (Trajectory.set_start_point(P2()).first_line(P2.x_direct(), c["drift"])
            .add_arc_line(c["big_r"], c["clockwise"], c["bending_angle"]))
    sign = -1.0 if c["clockwise"] else 1.0
    cct = CCT.create_cct_along(traj, c["drift"], c["big_r"], c["small_r"], c["bending_angle"], c["tilt_angles"],
                               c["winding_number"], c["current"], P2(0.0, 0.0),
                               P2(2 * math.pi * c["winding_number"], sign * c["bending_angle"] / 180.0 * math.pi),
                               c["disperse_number_per_winding"])
    return traj, cct


def single_dipole_particles(n: int = 32, seed: int = 0) -> np.ndarray:
    """(n, 10) proton records at the start of the single-dipole arc."""
    from .particles import ParticleFactory, PhaseSpaceParticle, particles_to_array
    c = SINGLE_DIPOLE
    traj, _ = build_single_dipole()
    ideal = ParticleFactory.create_proton_along(traj, c["drift"], c["kinetic_MeV"])
    pss = uniform_ellipse_phase_space(n, seed)
    ps = ParticleFactory.create_from_phase_space_particles(
        ideal, ideal.get_natural_coordinate_system(), [PhaseSpaceParticle(*map(float, r)) for r in pss])
    return particles_to_array(ps)


def build_gantry_section(**overrides):
    """HUST second bending section with the gantry-section workload's parameters."""
    from .beamline import HUST_SC_GANTRY
    g = GANTRY_SECTION
    kw = dict(agcct345_tilt_angles=g["agcct345_tilt_angles"], agcct345_current=g["agcct345_current"],
              part_per_winding=g["part_per_winding"])
    kw.update(overrides)
    return HUST_SC_GANTRY(**kw).create_second_bending_part_beamline()


def build_speed_test_beamline(currents=(10000.0, 10000.0)):
    """The beamline of cctpy's GPU speed test (final_code/work/小论文2回复/CPU和CPU代码速度测试.py:
    36-52): a 5 m drift, an AG-CCT (bending radius 1 m, aperture radii 200/180/160/140 mm,
    bends 10/10/15/15 deg, tilts [30] and [90, 30], 50 and 10/10/15/15 turns, 10 kA each),
    a 2 m drift, a 1 m QS of zero gradients (200 mm aperture) and a 2 m drift: 24 000
    segments, 10.8727 m.  ``currents``: the dipole and AG layers' currents (A)."""
    from .beamline import Beamline
    from .geometry import P2
    return (Beamline.set_start_point(P2.origin()).first_drift(direct=P2.x_direct(), length=5)
            .append_agcct(big_r=1.0, small_rs=[200 * MM, 180 * MM, 160 * MM, 140 * MM],
                          bending_angles=[10, 10, 15, 15], tilt_angles=[[30], [90, 30]],
                          winding_numbers=[[50], [10, 10, 15, 15]], currents=[float(c) for c in currents])
            .append_drift(2).append_qs(length=1, gradient=0, second_gradient=0, aperture_radius=200 * MM)
            .append_drift(2))


def beam_particles(bl, n: int, seed: int, kinetic_MeV: float, gaussian: bool = True) -> np.ndarray:
    """(n, 10) proton records at the start of beamline `bl`."""
    from .particles import ParticleFactory, PhaseSpaceParticle, particles_to_array
    ideal = ParticleFactory.create_proton_along(bl, 0.0, kinetic_MeV)
    pss = gaussian_phase_space(n, seed) if gaussian else uniform_ellipse_phase_space(n, seed)
    ps = ParticleFactory.create_from_phase_space_particles(
        ideal, ideal.get_natural_coordinate_system(), [PhaseSpaceParticle(*map(float, r)) for r in pss])
    return particles_to_array(ps)
