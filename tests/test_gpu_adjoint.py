"""Adjoint gradients (cct_track_adjoint + the complex-step segment Jacobian) against
central finite differences, h = 1e-4 relative: of the GPU FP64 forward, of the CPU
oracle (reduced magnet), and of the 13-parameter gantry design."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from cctpy_gb300 import CCT, engine, workloads as W
from cctpy_gb300.adjoint import (BeamObjective, GantryDesign, design_gradients, exit_frame, layer_gradient,
                                 objective_host, segment_gradient)
from oracle import cct_oracle as O

H_REL = 1e-4
GRAD_RTOL = 1e-5


def clone(c: CCT, tilts=None, current=None, big_r=None, dpw=None, winding=None) -> CCT:
    return CCT(c.local_coordinate_system, c.big_r if big_r is None else big_r, c.small_r, c.bending_angle,
               c.tilt_angles if tilts is None else tilts, c.winding_number if winding is None else winding,
               c.current if current is None else current, c.starting_point_in_ksi_phi_coordinate,
               c.end_point_in_ksi_phi_coordinate, c.disperse_number_per_winding if dpw is None else dpw)


def params_of(c: CCT):
    return list(c.tilt_angles) + [c.current, c.big_r]


def with_params(c: CCT, v):
    return clone(c, tilts=list(v[:-2]), current=v[-2], big_r=v[-1])


def flat(lg):
    return np.array(list(lg["tilt"]) + [lg["current"], lg["big_r"]])


def check_close(g_adj, g_fd):
    scale = np.abs(g_fd).max()
    err = np.abs(g_adj - g_fd)
    assert np.all(err <= GRAD_RTOL * np.abs(g_fd) + 1e-7 * scale), (g_adj, g_fd, err / np.maximum(np.abs(g_fd), 1e-300))


def test_adjoint_matches_gpu_central_differences():
    traj, base = W.build_single_dipole()
    c0 = W.SINGLE_DIPOLE
    ps = W.single_dipole_particles(16, seed=4)
    L, step = 0.1, 0.002
    frame = exit_frame(traj, c0["drift"] + L, c0["kinetic_MeV"])
    J, seg, final = segment_gradient(engine.design_of(base), ps, L, step, frame[None, :], checkpoint=16)
    J_fwd = objective_host(engine.track(engine.design_of(base), ps, L, step, "f64")[0], frame)
    assert abs(J[0] - J_fwd) <= 1e-12 * J_fwd
    g_adj = flat(layer_gradient(base, seg))
    v0 = params_of(base)
    g_fd = np.zeros(len(v0))
    for k in range(len(v0)):
        h = H_REL * abs(v0[k])
        Jk = []
        for sgn in (1, -1):
            v = list(v0)
            v[k] += sgn * h
            m = with_params(base, v)
            Jk.append(objective_host(engine.track(engine.design_of(m), ps, L, step, "f64")[0], frame))
        g_fd[k] = (Jk[0] - Jk[1]) / (2 * h)
    check_close(g_adj, g_fd)


def test_adjoint_matches_oracle_central_differences():
    traj, base = W.build_single_dipole()
    # 32 turns x 36 segments (1152): the oracle finishes in seconds, and central differences
    # at h = 1e-4 sit within 1e-6 of their h -> 0 limit (with 8 turns J(big_r) is so curved
    # that they are 1 % off it)
    small = clone(base, winding=32, dpw=36)
    c0 = W.SINGLE_DIPOLE
    ps = W.single_dipole_particles(8, seed=6)
    L, step = 0.04, 0.004
    frame = exit_frame(traj, c0["drift"] + L, c0["kinetic_MeV"])
    _, seg, _ = segment_gradient(engine.design_of(small), ps, L, step, frame[None, :], checkpoint=4)
    g_adj = flat(layer_gradient(small, seg))

    def oracle_J(m: CCT) -> float:
        lcs = m.local_coordinate_system
        fr = O.Frame.from_axes(*[tuple(r) for r in lcs.axes()])
        rec = O.cct_record(fr, m.big_r, m.small_r, m.bending_angle, m.tilt_angles, m.winding_number, m.current,
                           (m.starting_point_in_ksi_phi_coordinate.x, m.starting_point_in_ksi_phi_coordinate.y),
                           (m.end_point_in_ksi_phi_coordinate.x, m.end_point_in_ksi_phi_coordinate.y),
                           m.disperse_number_per_winding)
        mo = O.CCTOracle(rec)
        return objective_host(np.array([O.rk4_track(p, mo.field_at, L, step) for p in ps]), frame)

    v0 = params_of(small)
    g_fd = np.zeros(len(v0))
    for k in range(len(v0)):
        h = H_REL * abs(v0[k])
        vp, vm = list(v0), list(v0)
        vp[k] += h
        vm[k] -= h
        g_fd[k] = (oracle_J(with_params(small, vp)) - oracle_J(with_params(small, vm))) / (2 * h)
    check_close(g_adj, g_fd)


@pytest.mark.parametrize("precision", ["f64", "f32c"])
def test_gantry_design_gradient_matches_central_differences(precision):
    """All 13 parameters of a gantry design (4 dipole tilts, 4 AG tilts, 4 currents, the
    winding radius), from the FP64 adjoint and from the FP32-compensated one (the form the
    design-gradient rate is measured on; forward and reverse sweeps in packed FP32 with
    compensation), against central differences (h = 1e-4 relative) of the FP64 forward.
    Measured on GB300: FP32c within 1.3e-7 of the differences on the largest component and
    within 2.2e-8 of it on the others; the FP64 adjoint within 2.1e-7 and 2.2e-8."""
    kw = W.design_population(1, seed=3)[0]
    theta = np.array(kw["dicct345_tilt_angles"] + kw["agcct345_tilt_angles"]
                     + [kw["dicct345_current"], kw["dicct345_current"], kw["agcct345_current"],
                        kw["agcct345_current"], 0.95])
    dpw = 60
    base = GantryDesign(theta, part_per_winding=dpw)
    ps = W.beam_particles(base.beamline, 8, seed=7, kinetic_MeV=215.0)
    L, step = 0.3, 0.01
    J, g = design_gradients([base], ps, L, step, 215.0, checkpoint=8, precision=precision)
    frame = exit_frame(base.beamline.trajectory, L, 215.0)
    fd = np.zeros(len(theta))
    for k in range(len(theta)):
        h = H_REL * abs(theta[k])
        Jk = []
        for sgn in (1, -1):
            t = theta.copy()
            t[k] += sgn * h
            d = GantryDesign(t, part_per_winding=dpw)
            Jk.append(objective_host(engine.track(engine.design_of(d.beamline), ps, L, step, "f64")[0], frame))
        fd[k] = (Jk[0] - Jk[1]) / (2 * h)
    check_close(g[0], fd)


def test_autograd_function_and_batched_designs():
    designs = W.design_population(2, seed=3)
    theta = torch.tensor([kw["dicct345_tilt_angles"] + kw["agcct345_tilt_angles"]
                          + [kw["dicct345_current"], kw["dicct345_current"], kw["agcct345_current"],
                             kw["agcct345_current"], 0.95] for kw in designs], dtype=torch.float64,
                         requires_grad=True)
    bl0 = GantryDesign(theta[0].detach().numpy(), part_per_winding=60).beamline
    ps = W.beam_particles(bl0, 4, seed=8, kinetic_MeV=215.0)
    J = BeamObjective.apply(theta, ps, 0.1, 0.01, 215.0, 60)
    J.sum().backward()
    J2, g2 = design_gradients([GantryDesign(t, part_per_winding=60) for t in theta.detach().numpy()], ps, 0.1,
                              0.01, 215.0)
    np.testing.assert_allclose(J.detach().numpy(), J2, rtol=1e-14)
    np.testing.assert_allclose(theta.grad.numpy(), g2, rtol=1e-12)
    # each design's gradient equals the one of a single-design run
    _, g0 = design_gradients([GantryDesign(theta[0].detach().numpy(), part_per_winding=60)], ps, 0.1, 0.01, 215.0)
    np.testing.assert_allclose(g2[0], g0[0], rtol=1e-12, atol=0)


def test_f32c_adjoint_matches_f64_adjoint_and_differences():
    kw = W.design_population(1, seed=3)[0]
    theta = np.array(kw["dicct345_tilt_angles"] + kw["agcct345_tilt_angles"]
                     + [kw["dicct345_current"], kw["dicct345_current"], kw["agcct345_current"],
                        kw["agcct345_current"], 0.95])
    base = GantryDesign(theta, part_per_winding=60)
    ps = W.beam_particles(base.beamline, 96, seed=7, kinetic_MeV=215.0)   # 96: a ragged block of 128
    L, step = 0.3, 0.01
    J64, g64 = design_gradients([base], ps, L, step, 215.0, checkpoint=8, precision="f64")
    J32, g32 = design_gradients([base], ps, L, step, 215.0, checkpoint=8, precision="f32c")
    assert abs(J32[0] - J64[0]) <= 1e-6 * J64[0]
    scale = np.abs(g64[0]).max()
    assert np.all(np.abs(g32[0] - g64[0]) <= 1e-4 * np.abs(g64[0]) + 1e-6 * scale), (g32, g64)


@pytest.mark.parametrize("precision", ["f64", "f32c"])
def test_checkpoint_segments_on_dataflow_schedule(precision):
    """Eight designs x 40 protons are eight particle blocks or more (FP32c: one block of 64 a
    design, FP64: two of 32), so the forward runs on the dataflow schedule.  Twenty RK4 steps
    taken as five checkpoint segments of four (each segment's forward recomputed from its
    checkpoint before its reverse sweep) give the objectives and gradients of one segment of
    twenty (the whole forward recorded as it runs).  The forwards are the same to rounding; the
    segment gradient is summed per checkpoint segment, so FP32c gradients (compensated FP32
    sums) agree to FP32 accumulation order: within 1e-6 of the largest component (measured
    3.6e-8), ten times inside the 1e-5 bar against central differences."""
    kws = W.design_population(8, seed=5, part_per_winding=60)
    thetas = [np.array(kw["dicct345_tilt_angles"] + kw["agcct345_tilt_angles"]
                       + [kw["dicct345_current"], kw["dicct345_current"], kw["agcct345_current"],
                          kw["agcct345_current"], 0.95]) for kw in kws]
    designs = [GantryDesign(t, part_per_winding=60) for t in thetas]
    ps = W.beam_particles(designs[0].beamline, 40, seed=12, kinetic_MeV=215.0)
    L, step = 0.2, 0.01
    J1, g1 = design_gradients(designs, ps, L, step, 215.0, checkpoint=20, precision=precision)
    J5, g5 = design_gradients(designs, ps, L, step, 215.0, checkpoint=4, precision=precision)
    np.testing.assert_allclose(J5, J1, rtol=1e-13, atol=0)
    gtol = 1e-12 if precision == "f64" else 1e-6
    np.testing.assert_allclose(g5, g1, rtol=0, atol=gtol * np.abs(g1).max())
