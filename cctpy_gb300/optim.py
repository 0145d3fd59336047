"""The optimiser's caller loop on the GPU: one generation of gantry designs evaluated as
device work, with the phase-space read-out and the beam objectives computed on the device.

The reference's optimiser run script (final_code/work/optim/A05run.py:218-330) builds every
design's beamline on the host, tracks all designs in one GPU call, then loops in Python over
every design's protons: phase space at the exit (PhaseSpaceParticle.
create_from_running_particles, particles.py:1078-1138) and eleven statistics
(BaseUtils.Statistic, base_utils.py:603-683).  Here a generation is: layer records on the
host, segments generated on the device (cct_segments_build), FP32c tiles (cct_f32c_pack),
one tracking launch for all designs (cct_track), and the read-out (cct_beam_readout); only
the (designs x 11) objectives come back to the host.
"""
from __future__ import annotations

import ctypes
from typing import Callable, List, Sequence, Tuple

import numpy as np
import torch

from . import _lib, engine
from .geometry import MM
from .particles import ParticleFactory, PhaseSpaceParticle, RunningParticle, particles_to_array

OBJECTIVE_NAMES = ("width_max_x", "width_max_xp", "width_max_y", "width_max_yp", "center_x", "center_xp",
                   "center_y", "center_yp", "diff_xy", "fluct_x", "fluct_y")
A05_DELTAS = (-0.05, -0.0167, 0.0167, 0.05)      # A05run.py:15
A05_PER_PLANE = 12                                # A05run.py:17


def a05_phase_space(deltas: Sequence[float] = A05_DELTAS, per_plane: int = A05_PER_PLANE, xMax: float = 3.5 * MM,
                    xpMax: float = 7.5 * MM, yMax: float = 3.5 * MM, ypMax: float = 7.5 * MM) -> List[PhaseSpaceParticle]:
    """The optimiser's beam (A05run.py:199-208): per momentum spread, `per_plane` particles
    on the edge of the x-x' ellipse, then `per_plane` on the edge of the y-y' ellipse."""
    out = []
    for dp in deltas:
        out.extend(PhaseSpaceParticle.phase_space_particles_along_positive_ellipse_in_xxp_plane(xMax, xpMax, dp,
                                                                                               per_plane))
        out.extend(PhaseSpaceParticle.phase_space_particles_along_positive_ellipse_in_yyp_plane(yMax, ypMax, dp,
                                                                                               per_plane))
    return out


def _record(p) -> np.ndarray:
    if isinstance(p, np.ndarray):
        return np.asarray(p, dtype=np.float64).reshape(10)
    return np.asarray(p.to_numpy_array_data(np.float64), dtype=np.float64)


def _frame9(ideal) -> np.ndarray:
    if isinstance(ideal, np.ndarray):
        ideal = RunningParticle.from_numpy_array_data(ideal)
    cs = ideal.get_natural_coordinate_system()
    return np.array([cs.XI.x, cs.XI.y, cs.XI.z, cs.YI.x, cs.YI.y, cs.YI.z, cs.ZI.x, cs.ZI.y, cs.ZI.z])


def beam_readout(final, ideal_end, group: int = A05_PER_PLANE, speed_from_velocity: bool = True,
                 frame: np.ndarray = None) -> Tuple[object, object]:
    """(phase space (D, n, 6), objectives (D, 11)) of tracked records `final` ((D, n, 10) or
    (n, 10); numpy -> numpy results, CUDA tensor -> CUDA tensors) against the ideal particle
    at the exit (RunningParticle or its 10-double record) and its natural frame (`frame`,
    9 doubles XI, YI, ZI; computed from the ideal particle when omitted)."""
    lib = _lib.load()
    as_numpy = not isinstance(final, torch.Tensor)
    dev = engine._device()
    f = torch.as_tensor(np.asarray(final, dtype=np.float64) if as_numpy else final, dtype=torch.float64, device=dev)
    if f.ndim == 2:
        f = f.unsqueeze(0)
    if f.ndim != 3 or f.shape[2] != 10:
        raise ValueError(f"tracked records must be (designs, n, 10) or (n, 10), not {tuple(f.shape)}")
    f = f.contiguous()
    D, n = f.shape[0], f.shape[1]
    ideal = np.ascontiguousarray(_record(ideal_end))
    fr = np.ascontiguousarray(_frame9(ideal_end) if frame is None else np.asarray(frame, dtype=np.float64).reshape(9))
    ps = torch.empty((D, n, 6), dtype=torch.float64, device=dev)
    obj = torch.empty((D, len(OBJECTIVE_NAMES)), dtype=torch.float64, device=dev)
    rc = lib.cct_beam_readout(f.data_ptr(), D, n, ideal.ctypes.data_as(ctypes.c_void_p),
                              fr.ctypes.data_as(ctypes.c_void_p), int(group), int(bool(speed_from_velocity)),
                              ps.data_ptr(), obj.data_ptr(), engine._stream())
    _lib.check(rc, "cct_beam_readout")
    if as_numpy:
        return ps.cpu().numpy(), obj.cpu().numpy()
    return ps, obj


class GenerationEvaluator:
    """Objectives of one generation of designs, computed on the GPU.

    make_beamline(params_row) -> beamline (CCT and QS magnets); `particles`: the beam at the
    start ((n, 10) records, or RunningParticles), tracked `distance` metres with `footstep`
    RK4 steps; `ideal_end`: the ideal particle at the exit.  Calling the evaluator with a
    (G, k) parameter array returns the (G, 11) objectives (OBJECTIVE_NAMES)."""

    def __init__(self, make_beamline: Callable[[np.ndarray], object], particles, distance: float, footstep: float,
                 ideal_end, precision: str = "f32c", group: int = A05_PER_PLANE, speed_from_velocity: bool = True):
        self.make_beamline = make_beamline
        arr = particles if isinstance(particles, np.ndarray) else particles_to_array(particles)
        self.particles = torch.as_tensor(np.asarray(arr, dtype=np.float64), device=engine._device())
        self.distance, self.footstep = float(distance), float(footstep)
        self.ideal_end = ideal_end
        self.frame = _frame9(ideal_end)
        self.precision, self.group, self.speed_from_velocity = precision, int(group), bool(speed_from_velocity)
        self.last_design_set = None

    def __call__(self, params) -> np.ndarray:
        bls = [self.make_beamline(np.asarray(row)) for row in np.atleast_2d(np.asarray(params))]
        ds = engine.design_set_of(bls, segments="device")
        self.last_design_set = ds
        final = engine.track(ds, self.particles, self.distance, self.footstep, self.precision)
        _, obj = beam_readout(final, self.ideal_end, self.group, self.speed_from_velocity, self.frame)
        return obj.cpu().numpy()
