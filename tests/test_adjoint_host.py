"""Host side of the adjoint (CPU only): the complex-step Jacobian of segment generation
against central differences of CCT.global_segments, and the design-parameter mapping."""
import numpy as np

from cctpy_gb300 import CCT, workloads as W
from cctpy_gb300.adjoint import GantryDesign, ROLE_CURRENT, ROLE_TILTS, layer_gradient


def clone(c, tilts=None, current=None, big_r=None):
    return CCT(c.local_coordinate_system, c.big_r if big_r is None else big_r, c.small_r, c.bending_angle,
               c.tilt_angles if tilts is None else tilts, c.winding_number,
               c.current if current is None else current, c.starting_point_in_ksi_phi_coordinate,
               c.end_point_in_ksi_phi_coordinate, c.disperse_number_per_winding)


def test_segment_jacobian_matches_central_differences():
    _, c = W.build_single_dipole()
    c = CCT(c.local_coordinate_system, c.big_r, c.small_r, c.bending_angle, c.tilt_angles, 8, c.current,
            c.starting_point_in_ksi_phi_coordinate, c.end_point_in_ksi_phi_coordinate, 36)
    rng = np.random.default_rng(0)
    G = rng.normal(size=(c.total_disperse_number, 6))
    lg = layer_gradient(c, G)

    def J(m):
        kl, p0 = m.global_segments()
        return float(np.sum(G[:, :3] * kl) + np.sum(G[:, 3:] * p0))

    for i, t in enumerate(c.tilt_angles):
        h = 1e-5 * abs(t)
        tp, tm = list(c.tilt_angles), list(c.tilt_angles)
        tp[i] += h
        tm[i] -= h
        fd = (J(clone(c, tilts=tp)) - J(clone(c, tilts=tm))) / (2 * h)
        assert abs(lg["tilt"][i] - fd) <= 1e-7 * abs(fd) + 1e-12
    h = 1e-5 * abs(c.current)
    fd = (J(clone(c, current=c.current + h)) - J(clone(c, current=c.current - h))) / (2 * h)
    assert abs(lg["current"] - fd) <= 1e-7 * abs(fd)   # J is linear in I: FD error is rounding only
    h = 1e-6 * c.big_r
    fd = (J(clone(c, big_r=c.big_r + h)) - J(clone(c, big_r=c.big_r - h))) / (2 * h)
    assert abs(lg["big_r"] - fd) <= 1e-6 * abs(fd)


def test_gantry_design_layers():
    kw = W.design_population(1, seed=3)[0]
    theta = np.array(kw["dicct345_tilt_angles"] + kw["agcct345_tilt_angles"] + [1000.0, 2000.0, 3000.0, 4000.0, 0.96])
    d = GantryDesign(theta, part_per_winding=36)
    ccts = [m for m in d.beamline.magnets if isinstance(m, CCT)]
    assert len(ccts) == 16
    for m in ccts:
        first, sign = ROLE_TILTS[m.role]
        assert m.tilt_angles == [sign * t for t in theta[first:first + 4]]
        assert m.current == theta[ROLE_CURRENT[m.role]]
        assert m.big_r == 0.96
    assert sorted({m.role for m in ccts}) == ["ag_inner", "ag_outer", "dipole_inner", "dipole_outer"]
