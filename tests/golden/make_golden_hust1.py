"""Fixture of the HUST gantry's first bending section, generated by the cctpy reference itself
(same loader and shims as make_golden.py):

    python tests/golden/make_golden_hust1.py

Outputs (small, committed): ``golden_hust1.npz`` (field points and fields, the ideal 215 MeV
proton plus two beam protons before and after the reference's own RK4 track over the whole
section at 100 mm steps; the same for the whole gantry with the ideal proton) and
``records_hust1.json`` (the magnets as the reference built them).
"""
from __future__ import annotations

import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import (field_points, load_reference, make_particles, particles_array,  # noqa: E402
                         record_of, workloads)


def main():
    t00 = time.time()
    load_reference()
    from hust_sc_gantry import HUST_SC_GANTRY
    from packages.particles import ParticleFactory, ParticleRunner
    from packages.constants import MM

    bl = HUST_SC_GANTRY().create_first_bending_part_beamline()
    records = {"hust1_default": [record_of(m) for m in bl.magnets]}
    arrays = {"h1_length": np.array([bl.get_length()])}
    pts = []
    for k, s in enumerate(np.linspace(0.0, bl.get_length(), 12)):
        p, d = bl.point_at(s), bl.direct_at(s)
        off = d.rotate(math.pi / 2).change_length(((k % 5) - 2) * 10 * MM)
        pts.append([p.x + off.x, p.y + off.y, ((k % 3) - 1) * 8 * MM])
    pts = np.array(pts)
    arrays["h1_field_pts"] = pts
    arrays["h1_field_B"] = field_points(bl, pts)
    ideal = ParticleFactory.create_proton_along(bl, kinetic_MeV=215)
    ps = [ideal.copy()] + make_particles(ideal, workloads.gaussian_phase_space(2, seed=31))
    arrays["h1_particles_in"] = particles_array(ps)
    t0 = time.time()
    ParticleRunner.run_only(ps, bl, bl.get_length(), footstep=100 * MM, concurrency_level=3, report=False)
    print(f"hust1 default: tracked 3 protons in {time.time() - t0:.1f} s")
    arrays["h1_particles_out"] = particles_array(ps)
    # the whole gantry (first section, the second section after it): placement, fields and
    # the ideal proton tracked over the whole length at 100 mm
    total = HUST_SC_GANTRY().create_total_beamline()
    records["total_default"] = [record_of(m) for m in total.magnets]
    arrays["tot_length"] = np.array([total.get_length()])
    pts = np.array([[total.point_at(s).x, total.point_at(s).y, 0.004] for s in np.linspace(0.3, total.get_length() - 0.3, 8)])
    arrays["tot_field_pts"] = pts
    arrays["tot_field_B"] = field_points(total, pts)
    tp = [ParticleFactory.create_proton_along(total, kinetic_MeV=215)]
    arrays["tot_particles_in"] = particles_array(tp)
    t0 = time.time()
    ParticleRunner.run_only(tp, total, total.get_length(), footstep=100 * MM, concurrency_level=1, report=False)
    print(f"total gantry: tracked the ideal proton in {time.time() - t0:.1f} s")
    arrays["tot_particles_out"] = particles_array(tp)
    np.savez_compressed(os.path.join(HERE, "golden_hust1.npz"), **arrays)
    with open(os.path.join(HERE, "records_hust1.json"), "w") as f:
        json.dump(records, f, indent=1)
    print(f"done in {time.time() - t00:.1f} s")


if __name__ == "__main__":
    main()
