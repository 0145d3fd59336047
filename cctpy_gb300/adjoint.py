"""Gradients of a beam objective with respect to CCT design parameters.

The GPU (libcctgpu ``cct_track_adjoint``) returns, for every design, the objective

    J = mean_i (x_i^2 + y_i^2)        (x, y: final positions in the ideal particle's exit frame)

-- the RMS spot size squared plus the centroid squared in both planes -- and its gradient
with respect to every current element (kl_i, p0_i), by the discrete adjoint of the FP64
RK4 track with checkpointing.  This module maps those segment gradients to design
parameters through the Jacobian of segment generation (``CCT.path_local``): on the GPU by
forward-mode derivatives of the generation formulas (``cct_segments_param_grad``, the
default), or on the host by the complex-step method (the winding path evaluated once per
parameter with that parameter perturbed by i*1e-30, exact to rounding with no subtractive
cancellation), which the tests use as the check.  The magnet frames are held fixed (they
come from the design orbit).

Per CCT layer the parameters are its tilt angles (degrees), its current and its winding
torus radius big_r.  ``GantryDesign`` groups the layers of the HUST second bending section
into the 13 parameters of a design: 4 dipole tilt angles, 4 AG tilt angles, 4 currents
(dipole outer / dipole inner / AG inner / AG outer layers) and the winding radius.
``BeamObjective`` exposes the whole computation as a torch.autograd.Function.
"""
from __future__ import annotations

import math
from typing import Dict, List, Sequence, Tuple

import numpy as np
import torch

from . import _lib, engine
from .beamline import HUST_SC_GANTRY
from .geometry import P3
from .magnets import CCT
from .particles import ParticleFactory

_H = 1e-30   # complex-step size


def exit_frame(trajectory, s: float, kinetic_MeV: float) -> np.ndarray:
    """(9,) origin, XI, YI of the ideal particle's natural frame at arc length s
    (RunningParticle.get_natural_coordinate_system, y = global z)."""
    ip = ParticleFactory.create_proton_along(trajectory, s, kinetic_MeV)
    f = ip.get_natural_coordinate_system()
    return np.array(ip.position.to_list() + f.XI.to_list() + f.YI.to_list())


def objective_host(final: np.ndarray, frame: np.ndarray) -> float:
    """J of (n, 10) final records for one design (host FP64; the same formula as the GPU)."""
    d = final[:, 0:3] - frame[0:3]
    x = d @ frame[3:6]
    y = d @ frame[6:9]
    return float(np.mean(x * x + y * y))


def auto_checkpoint(n_records: int, max_steps: int) -> int:
    """Checkpoint interval (RK4 steps) for `n_records` tracked particles: the whole track in
    one segment when its stage records (4 x 96 bytes per particle and step) fit in a quarter
    of the free device memory (at most 64 GiB) -- the forward then records as it goes and
    nothing is recomputed --, else as many steps per segment as that budget holds."""
    free, _ = torch.cuda.mem_get_info()
    budget = min(free // 4, 64 << 30)
    per_step = 4 * 96 * int(n_records)
    if per_step * max_steps <= budget:
        return int(max_steps)
    return int(max(16, budget // per_step))


def segment_gradient(ds: engine.DesignSet, particles, distance: float, footstep: float, frames: np.ndarray,
                     checkpoint: int = None, precision: str = "f64", on_device: bool = False):
    """(J (D,), dJ/d(kl, p0) (N_seg, 6), final records (D, n, 10)) for the designs of `ds`;
    precision "f64" or "f32c" (forward and adjoint sweeps); checkpoint: RK4 steps per
    checkpoint segment (None: auto_checkpoint).  on_device=True returns the segment gradient
    as a CUDA tensor (for DesignSet.param_grad)."""
    lib = _lib.load()
    dev = ds.kls.device
    p = torch.as_tensor(np.asarray(particles, dtype=np.float64), device=dev)
    if p.ndim == 2:
        p = p.unsqueeze(0).expand(ds.n_designs, -1, -1)
    p = p.contiguous().clone()
    n_p = p.shape[1]
    speeds = p[..., 8].min().item()
    max_steps = int(math.ceil(distance / footstep * (1 + 1e-9))) + 1
    if not (speeds > 0):
        raise ValueError("particle speeds must be positive")
    fr = torch.as_tensor(np.asarray(frames, dtype=np.float64).reshape(ds.n_designs, 9), device=dev).contiguous()
    J = torch.empty(ds.n_designs, dtype=torch.float64, device=dev)
    grad = torch.empty((max(ds.n_segments, 1), 6), dtype=torch.float64, device=dev)
    if checkpoint is None:
        checkpoint = auto_checkpoint(ds.n_designs * n_p, max_steps)
    nbytes = lib.cct_adjoint_scratch_bytes(ds.n_designs, n_p, max_steps, checkpoint)
    _lib.check(0 if nbytes >= 0 else _lib.CCT_ERR_ARG, "cct_adjoint_scratch_bytes")
    prec = {"f64": 0, "f32c": 1}.get(precision)
    if prec is None:
        raise ValueError(f"precision must be 'f64' or 'f32c', not {precision!r}")
    packed = ds.packed().data_ptr() if prec == 1 else 0
    with engine._scratch_lock:
        sc = engine.scratch(nbytes, dev)
        rc = lib.cct_track_adjoint(engine._ptr(ds.kls), engine._ptr(ds.p0s), engine._ptr(ds.seg_off), packed,
                                   engine._ptr(ds.qs), engine._ptr(ds.qs_off), ds.n_designs, p.data_ptr(), n_p,
                                   float(distance), float(footstep), prec, fr.data_ptr(), J.data_ptr(),
                                   grad.data_ptr(), int(checkpoint), sc.data_ptr(), int(nbytes), engine._stream())
    _lib.check(rc, "cct_track_adjoint")
    g = grad[:ds.n_segments]
    return J.cpu().numpy(), (g if on_device else g.cpu().numpy()), p.cpu().numpy()


# ---------------------------------------------------------------- segment-generation Jacobian
def _path_local_complex(c: CCT, tilts: Sequence[complex], big_r: complex) -> np.ndarray:
    """Winding path of CCT `c` (local frame) with complex tilt angles / big_r: the formula of
    CCT.path_local with every tilt term kept (the 90-degree skip does not change values)."""
    ksi = c.ksi_samples()
    x1, y1 = c.starting_point_in_ksi_phi_coordinate.x, c.starting_point_in_ksi_phi_coordinate.y
    x2, y2 = c.end_point_in_ksi_phi_coordinate.x, c.end_point_in_ksi_phi_coordinate.y
    k = (y2 - y1) / (x2 - x1)
    b = -k * x1 + y1
    a = np.sqrt(big_r ** 2 - c.small_r ** 2 + 0j)
    eta = 0.5 * np.log((big_r + a) / (big_r - a))
    sh, ch = np.sinh(eta), np.cosh(eta)
    phi = (k * ksi + b).astype(np.complex128)
    for i, t in enumerate(tilts):
        phi = phi + (1 / np.tan(t / 180.0 * math.pi)) / ((i + 1) * sh) * np.sin((i + 1) * ksi)
    temp = a / (ch - np.cos(ksi))
    return np.stack([temp * sh * np.cos(phi), temp * sh * np.sin(phi), temp * np.sin(ksi)], 1)


def layer_gradient(c: CCT, seg_grad: np.ndarray) -> Dict[str, object]:
    """dJ/d(tilt angles, current, big_r) of one CCT layer from its slice of the segment
    gradient ((N, 6): dJ/dkl, dJ/dp0)."""
    R = c.local_coordinate_system.axes()[1:4]          # rows XI, YI, ZI
    gk, gp = seg_grad[:, 0:3], seg_grad[:, 3:6]

    def contract(dw_local: np.ndarray) -> float:
        dw = dw_local @ R                                # local -> global (rotation only)
        dkl = 1e-7 * c.current * (dw[1:] - dw[:-1])
        dp0 = 0.5 * (dw[1:] + dw[:-1])
        return float(np.sum(gk * dkl) + np.sum(gp * dp0))

    base_t = [complex(t) for t in c.tilt_angles]
    out = {"tilt": []}
    for i in range(len(base_t)):
        t = list(base_t)
        t[i] += 1j * _H
        out["tilt"].append(contract(_path_local_complex(c, t, complex(c.big_r)).imag / _H))
    out["big_r"] = contract(_path_local_complex(c, base_t, c.big_r + 1j * _H).imag / _H)
    w = c.path_local()
    out["current"] = float(np.sum(gk * (1e-7 * (w[1:] - w[:-1]) @ R)))
    return out


def layer_gradients(magnets: Sequence, seg_grad: np.ndarray) -> List[Dict[str, object]]:
    """Per CCT layer gradients (None for QS), slicing the design's segment gradient in the
    order engine.host_design concatenates the layers."""
    out, at = [], 0
    for m in magnets:
        if engine._classify(m) != "cct":
            out.append(None)
            continue
        if abs(float(m.current)) <= 1e-6:
            out.append(None)
            continue
        n = m.total_disperse_number
        out.append(layer_gradient(m, seg_grad[at:at + n]))
        at += n
    return out


# ---------------------------------------------------------------- 13-parameter gantry design
ROLE_CURRENT = {"dipole_outer": 8, "dipole_inner": 9, "ag_inner": 10, "ag_outer": 11}
ROLE_TILTS = {"dipole_outer": (0, -1.0), "dipole_inner": (0, 1.0), "ag_inner": (4, -1.0), "ag_outer": (4, 1.0)}
PARAM_NAMES = (["dipole_tilt_%d" % i for i in range(4)] + ["ag_tilt_%d" % i for i in range(4)]
               + ["I_dipole_outer", "I_dipole_inner", "I_ag_inner", "I_ag_outer", "winding_big_r"])


class GantryDesign:
    """The HUST second bending section as a 13-parameter design:
    theta = (4 dipole tilt angles, 4 AG tilt angles [deg], currents of the dipole-outer,
    dipole-inner, AG-inner and AG-outer layers [A], winding torus radius [m]).  The design
    orbit (and so every magnet frame) keeps the builder's 0.95 m bending radius; the
    winding radius moves the windings on their torus."""

    def __init__(self, theta: Sequence[float], part_per_winding: int = 360, **builder):
        self.theta = np.asarray(theta, dtype=np.float64)
        if self.theta.shape != (13,):
            raise ValueError("a gantry design has 13 parameters")
        t = self.theta
        g = HUST_SC_GANTRY(dicct345_tilt_angles=list(t[0:4]), agcct345_tilt_angles=list(t[4:8]),
                           dicct345_current=float(t[8]), agcct345_current=float(t[10]),
                           part_per_winding=part_per_winding, **builder)
        self.beamline = g.create_second_bending_part_beamline()
        mags = []
        for m in self.beamline.magnets:
            if isinstance(m, CCT):
                role = m.role
                c = CCT(m.local_coordinate_system, float(t[12]), m.small_r, m.bending_angle, m.tilt_angles,
                        m.winding_number, float(t[ROLE_CURRENT[role]]), m.starting_point_in_ksi_phi_coordinate,
                        m.end_point_in_ksi_phi_coordinate, m.disperse_number_per_winding)
                c.role = role
                mags.append(c)
            else:
                mags.append(m)
        self.beamline.magnets = mags
        self.beamline._changed()

    def gradient(self, layer_grads: Sequence) -> np.ndarray:
        g = np.zeros(13)
        for m, lg in zip(self.beamline.magnets, layer_grads):
            if lg is None:
                continue
            first, sign = ROLE_TILTS[m.role]
            for i, v in enumerate(lg["tilt"][:4]):
                g[first + i] += sign * v
            g[ROLE_CURRENT[m.role]] += lg["current"]
            g[12] += lg["big_r"]
        return g


def layer_grads_from_rows(magnets: Sequence, rows: np.ndarray) -> List[Dict[str, object]]:
    """Per-magnet gradient dicts (None for QS and zero-current layers) from the rows of
    DesignSet.param_grad, which follow engine.device_layers' layer order."""
    out, k = [], 0
    for m in magnets:
        if engine._classify(m) != "cct" or abs(float(m.current)) <= 1e-6:
            out.append(None)
            continue
        r = rows[k]
        k += 1
        out.append({"tilt": [float(v) for v in r[:len(m.tilt_angles)]], "current": float(r[8]),
                    "big_r": float(r[9])})
    return out


def design_gradients(designs: Sequence[GantryDesign], particles: np.ndarray, distance: float, footstep: float,
                     kinetic_MeV: float, checkpoint: int = None, precision: str = "f64",
                     jacobian: str = "device") -> Tuple[np.ndarray, np.ndarray]:
    """J (D,) and dJ/dtheta (D, 13) of every design, all tracked in one adjoint run.  The
    designs share the design orbit: particles start at s = 0 and the objective is read in
    the ideal particle's frame at s = distance.  jacobian="device" generates the segments
    and contracts the segment gradient with the segment-generation Jacobian on the GPU
    (forward mode, cct_segments_param_grad); "host" builds segments with numpy and takes
    the Jacobian by complex step."""
    if jacobian not in ("device", "host"):
        raise ValueError(f"jacobian must be 'device' or 'host', not {jacobian!r}")
    ds = engine.design_set_of([d.beamline for d in designs], segments=jacobian)
    frame = exit_frame(designs[0].beamline.trajectory, distance, kinetic_MeV)
    J, seg, _ = segment_gradient(ds, particles, distance, footstep, np.tile(frame, (len(designs), 1)), checkpoint,
                                 precision, on_device=(jacobian == "device"))
    grads = np.zeros((len(designs), 13))
    if jacobian == "device":
        rows = ds.param_grad(seg)
        for d, des in enumerate(designs):
            grads[d] = des.gradient(layer_grads_from_rows(des.beamline.magnets, rows[ds.layer_design == d]))
        return J, grads
    for d, des in enumerate(designs):
        a, b = int(ds.h_seg_off[d]), int(ds.h_seg_off[d + 1])
        grads[d] = des.gradient(layer_gradients(des.beamline.magnets, seg[a:b]))
    return J, grads


class BeamObjective(torch.autograd.Function):
    """J(theta) for a batch of gantry designs (theta: (D, 13) float64 tensor) with the
    adjoint gradient as its backward: forward runs the GPU adjoint once and keeps dJ/dtheta."""

    @staticmethod
    def forward(ctx, theta: torch.Tensor, particles: np.ndarray, distance: float, footstep: float,
                kinetic_MeV: float, part_per_winding: int = 360):
        th = theta.detach().cpu().numpy().reshape(-1, 13)
        designs = [GantryDesign(t, part_per_winding=part_per_winding) for t in th]
        J, g = design_gradients(designs, particles, distance, footstep, kinetic_MeV)
        ctx.save_for_backward(torch.as_tensor(g, dtype=theta.dtype, device=theta.device))
        return torch.as_tensor(J, dtype=theta.dtype, device=theta.device)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return grad_out.reshape(-1, 1) * g, None, None, None, None, None
