"""Golden fixture of the optimiser read-out, generated from the cctpy reference itself:
the phase space of tracked protons at the beamline exit (PhaseSpaceParticle.
create_from_running_particles, particles.py:1078-1138) and the eleven beam objectives that
the reference's optimiser run script computes from it for every gantry design
(final_code/work/optim/A05run.py:247-330, with BaseUtils.Statistic, base_utils.py:603-683).

    python tests/golden/make_golden_readout.py      # writes golden_readout.npz

The run script is a program, not a function, so its statistics sequence is restated below
with the reference's own Statistic class; the particles stand for tracked ones: the
script's beam (4 momentum spreads x 12 particles on the x-xp and the y-y' ellipse edges)
placed at the exit, with seeded offsets of position and velocity, and the record's speed
left as tracking leaves it (the script first resets it to |v|, A05run.py:265-267); they are
handed over as the reference's GPU tracking hands them over, rebuilt from the record array.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import load_reference, particles_array  # noqa: E402

DELTAS = [-0.05, -0.0167, 0.0167, 0.05]     # A05run.py:15
PER_PLANE = 12                              # A05run.py:17


def objectives_of(ip_end, ps):
    """A05run.py:247-330 for one design, with the reference's classes."""
    from packages.base_utils import BaseUtils
    from packages.constants import MM, MRAD
    from packages.particles import PhaseSpaceParticle
    sx, sy, sxp, syp = (BaseUtils.Statistic() for _ in range(4))
    sx_dp, sy_dp, swx, swy = (BaseUtils.Statistic() for _ in range(4))
    for p in ps:
        p.speed = p.velocity.length()
    pps = PhaseSpaceParticle.create_from_running_particles(ip_end, ip_end.get_natural_coordinate_system(), ps)
    for pid in range(0, len(pps), PER_PLANE):
        for pp in pps[pid:pid + PER_PLANE]:
            sx.add(pp.x / MM)
            sy.add(pp.y / MM)
            sxp.add(pp.xp / MRAD)
            syp.add(pp.yp / MRAD)
            sx_dp.add(pp.x / MM)
            sy_dp.add(pp.y / MM)
        swx.add(sx_dp.half_width())
        swy.add(sy_dp.half_width())
        sx_dp.clear()
        sy_dp.clear()
    wx, wxp, wy, wyp = sx.absolute_max(), sxp.absolute_max(), sy.absolute_max(), syp.absolute_max()
    obj = [wx, wxp, wy, wyp, abs(sx.average()), abs(sxp.average()), abs(sy.average()), abs(syp.average()),
           abs(wx - wy), swx.width(), swy.width()]
    ps_rows = [[pp.x, pp.xp, pp.y, pp.yp, pp.z, pp.delta] for pp in pps]
    return np.array(obj, dtype=np.float64), np.array(ps_rows)


def main():
    load_reference()
    from packages.constants import MM
    from packages.particles import ParticleFactory, PhaseSpaceParticle, RunningParticle
    from packages.point import P3
    from hust_sc_gantry import HUST_SC_GANTRY

    bl = HUST_SC_GANTRY().create_second_bending_part_beamline()
    ip_end = ParticleFactory.create_proton_along(bl, bl.get_length(), 215)
    cs = ip_end.get_natural_coordinate_system()
    pps = []
    for dp in DELTAS:
        pps.extend(PhaseSpaceParticle.phase_space_particles_along_positive_ellipse_in_xxp_plane(
            xMax=3.5 * MM, xpMax=7.5 * MM, delta=dp, number=PER_PLANE))
        pps.extend(PhaseSpaceParticle.phase_space_particles_along_positive_ellipse_in_yyp_plane(
            yMax=3.5 * MM, ypMax=7.5 * MM, delta=dp, number=PER_PLANE))
    rng = np.random.default_rng(5)
    finals, objs, rows = [], [], []
    for d in range(3):
        ps = ParticleFactory.create_from_phase_space_particles(ip_end, cs, pps)
        for p in ps:
            dx = rng.normal(0.0, 2e-3, 3)
            dv = rng.normal(0.0, 2e-3 * p.speed, 3)
            p.position = p.position + P3(*[float(v) for v in dx])
            p.velocity = p.velocity + P3(*[float(v) for v in dv])
        arr = particles_array(ps)
        finals.append(arr)
        # as the reference's GPU tracking returns them (gpu_accelerator.py:1899-1910): rebuilt
        # from the FP64 record array (P3 stores Python floats, point.py:322-325, so the
        # builtin sum in Statistic.average is CPython's compensated float sum on 3.12+)
        o, r = objectives_of(ip_end, [RunningParticle.from_numpy_array_data(a) for a in arr])
        objs.append(o)
        rows.append(r)
    np.savez_compressed(os.path.join(HERE, "golden_readout.npz"),
                        ps_in=np.array([[p.x, p.xp, p.y, p.yp, p.z, p.delta] for p in pps]),
                        finals=np.stack(finals), ideal_end=ip_end.to_numpy_array_data(np.float64),
                        frame=np.array([cs.XI.to_list(), cs.YI.to_list(), cs.ZI.to_list()]),
                        phase_space=np.stack(rows), objectives=np.stack(objs),
                        group=np.array([PER_PLANE]))
    print("wrote golden_readout.npz:", np.stack(objs))


if __name__ == "__main__":
    main()
