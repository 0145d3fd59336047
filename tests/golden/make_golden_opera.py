"""Fixture of the OPERA cross-check of the reference (final_code/demos/D04OperaTrack对比.py):
a 215 MeV proton through two single-tilt CCT layers (42 windings, -6192 A, 120 segments per
winding, global frame), tracked by OPERA-3D with brick conductors 3.2 mm x 11 mm
(final_code/data/track_verify_opera.txt: x, y, z, vx, vy, vz, t every 1 mm of path) and by
cctpy's own RK4 with the midpoint Biot-Savart field.

    python tests/golden/make_golden_opera.py      # writes golden_opera.npz

Kept: OPERA's positions every 50 mm of path, and cctpy's positions at the same path lengths
(ParticleRunner.run_only in 50 mm calls of 1 mm steps, which is the same RK4 as one call).
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import REF, load_reference, particles_array  # noqa: E402

CHUNK = 0.05
N_CHUNKS = 47


def main():
    load_reference()
    from packages.base_utils import BaseUtils
    from packages.cct import CCT
    from packages.constants import MM
    from packages.local_coordinate_system import LocalCoordinateSystem
    from packages.magnets import CombinedMagnet
    from packages.particles import ParticleFactory, ParticleRunner
    from packages.point import P2, P3

    def layer(small_r, tilt, sign):
        return CCT(local_coordinate_system=LocalCoordinateSystem.global_coordinate_system(), big_r=0.95,
                   small_r=small_r, bending_angle=22.5, tilt_angles=[tilt], winding_number=42, current=-6192,
                   starting_point_in_ksi_phi_coordinate=P2.zeros(),
                   end_point_in_ksi_phi_coordinate=P2(sign * 2 * math.pi * 42, BaseUtils.angle_to_radian(22.5)),
                   disperse_number_per_winding=120)

    magnet = CombinedMagnet(layer(104.5 * MM, -30, -1), layer(120.5 * MM, 30, 1))
    p = ParticleFactory.create_proton(position=P3(x=0.95, y=-1), direct=P3.y_direct(), kinetic_MeV=215)
    start = particles_array([p])[0]
    pos = []
    for k in range(N_CHUNKS):
        ParticleRunner.run_only(p, magnet, CHUNK, footstep=1 * MM, report=False)
        pos.append(p.position.to_list())
        print(f"{(k + 1) * CHUNK:.2f} m", p.position, flush=True)
    opera = np.loadtxt(os.path.join(REF, "final_code", "data", "track_verify_opera.txt"))
    s = CHUNK * np.arange(1, N_CHUNKS + 1)
    rows = np.rint(s / 0.001).astype(int) - 1            # row i holds the point at (i + 1) mm
    np.savez_compressed(os.path.join(HERE, "golden_opera.npz"), s=s, opera_pos=opera[rows, 0:3],
                        cctpy_pos=np.array(pos), particle_in=start)
    print("wrote golden_opera.npz")


if __name__ == "__main__":
    main()
