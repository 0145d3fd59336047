"""Generate the fixtures of the 1 mm tracking parity tests and of the reference's own FP64
field known-answer test, from the cctpy reference itself.

    CCTPY_REFERENCE=<cctpy checkout> python tests/golden/make_golden_1mm.py

Contents (``golden_1mm.npz`` + ``records_1mm.json``, small, committed):

* ``f64k_*``: the FP64 known-answer test of cctpy's GPU module (cctpy3/ccpty_cuda.py:1149-1176,
  ``Test.test_cct``) restated on the final_code package: one CCT layer of the whole gantry
  (``magnets[15]``), the point 0.5 m past the second section's entrance drift on the design
  orbit plus (1e-3, 1e-4, 1e-5) m, and cctpy's CPU field there (``CCT.magnetic_field_at``,
  cct.py:249-285).  The reference asserts its FP64 GPU sum within 1e-14 T of that.
* ``gs1_*``: the gantry-section workload (597 600 segments, AG tilts [90, 30, 90, 90],
  -7000 A) with 8 protons of 215 MeV (seeded Gaussian phase space) started on the design orbit
  at s = 1.9 m and tracked by ``ParticleRunner.run_only`` (particles.py:562-632) over 1.0 m at
  the workload's 1 mm step, through the end of the entrance drift into the first dipole.
* ``dp1mm{d}_*``: two designs of the seeded population, 4 protons each, the same window.

Uses the same shims as make_golden.py (matplotlib stub, the numpy-2 reshape of
``P2.from_numpy_ndarry``).
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from make_golden import load_reference, make_particles, particles_array, record_of  # noqa: E402
from cctpy_gb300 import workloads  # noqa: E402

S0 = 1.9          # m, start of the tracked window on the design orbit
WINDOW = 1.0      # m, tracked length
STEP = 0.001      # m, the workloads' RK4 step


def main():
    load_reference()
    from packages.point import P3
    from packages.cct import CCT
    from packages.particles import ParticleFactory, ParticleRunner
    from hust_sc_gantry import HUST_SC_GANTRY

    arrays, records = {}, {}
    cores = os.cpu_count() or 1

    # ------------------------------------------------ the reference's FP64 known answer
    g = HUST_SC_GANTRY()
    total = g.create_total_beamline()
    cct = total.magnets[15]
    assert isinstance(cct, CCT), type(cct)
    s = g.create_first_bending_part_beamline().get_length() + g.DL2 + 0.5
    p = total.trajectory.point_at(s).to_p3() + P3(1e-3, 1e-4, 1e-5)
    records["f64_known"] = [record_of(cct)]
    arrays["f64k_pt"] = np.array(p.to_list())
    arrays["f64k_B"] = np.array(cct.magnetic_field_at(p).to_list())

    # ------------------------------------------------ gantry section at 1 mm
    gs = workloads.GANTRY_SECTION
    bl = HUST_SC_GANTRY(agcct345_tilt_angles=gs["agcct345_tilt_angles"], agcct345_current=gs["agcct345_current"],
                        part_per_winding=gs["part_per_winding"]).create_second_bending_part_beamline()
    records["gantry_section"] = [record_of(m) for m in bl.magnets]
    ideal = ParticleFactory.create_proton_along(bl, S0, gs["kinetic_MeV"])
    pss = workloads.gaussian_phase_space(8, seed=41)
    ps = make_particles(ideal, pss)
    arrays["gs1_ps_in"] = pss
    arrays["gs1_particles_in"] = particles_array(ps)
    t0 = time.time()
    ParticleRunner.run_only(ps, bl, WINDOW, footstep=STEP, concurrency_level=min(cores, 8), report=False)
    print(f"gantry section: 8 protons over {WINDOW} m at 1 mm in {time.time() - t0:.0f} s", flush=True)
    arrays["gs1_particles_out"] = particles_array(ps)

    # ------------------------------------------------ two population designs at 1 mm
    records["design_population"] = []
    for d, kw in enumerate(workloads.design_population(2, seed=3)):
        bl = HUST_SC_GANTRY(**kw).create_second_bending_part_beamline()
        records["design_population"].append([record_of(m) for m in bl.magnets])
        ideal = ParticleFactory.create_proton_along(bl, S0, 215.0)
        ps = make_particles(ideal, workloads.gaussian_phase_space(4, seed=50 + d))
        arrays[f"dp1mm{d}_particles_in"] = particles_array(ps)
        t0 = time.time()
        ParticleRunner.run_only(ps, bl, WINDOW, footstep=STEP, concurrency_level=min(cores, 4), report=False)
        print(f"design {d}: 4 protons in {time.time() - t0:.0f} s", flush=True)
        arrays[f"dp1mm{d}_particles_out"] = particles_array(ps)

    arrays["window"] = np.array([S0, WINDOW, STEP])
    np.savez_compressed(os.path.join(HERE, "golden_1mm.npz"), **arrays)
    with open(os.path.join(HERE, "records_1mm.json"), "w") as f:
        json.dump(records, f)
    print("wrote golden_1mm.npz, records_1mm.json")


if __name__ == "__main__":
    main()
