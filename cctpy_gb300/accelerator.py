"""GPU_ACCELERATOR: drop-in for cctpy's accelerator class (final_code/packages/gpu_accelerator.py:46-2152).

Same constructor arguments and method names, argument meaning, return
conventions and errors:

* ``track_one_*`` and ``track_multi_particle_for_*`` update the given particles in
  place (RunningParticle.populate semantics);
* ``track_multi_particle_beamline_*`` return new ``[design][particle]`` lists and
  leave the inputs untouched;
* a magnet other than CCT / QS raises ValueError.

Differences, by design of this engine:

* FLOAT32 selects the FP32-compensated kernels (<= 1e-7 relative field error),
  FLOAT64 the plain FP64 kernels; nothing is JIT-compiled per call; a beamline object
  given several times in one call has its segments built and copied to the device once
  (every call still builds them afresh, as the reference does, so that changes to the
  magnets between calls are seen; ``cctpy_gb300.engine`` keeps design sets resident);
* every design of a population runs in one persistent launch (no block-per-design
  serial particle loop), so ``block_dim_x`` only keeps its validation;
* segment counts are not padded to ``max_current_element_number``; exceeding it still
  raises ValueError as the reference's padding copy would;
* ``distance`` of tracked particles grows by the tracked length (as the reference's CPU
  path and its CPU mode do), rather than being overwritten;
* there is no CPU mode: ``cpu_mode=True`` raises NotImplementedError.
"""
from __future__ import annotations

from typing import List, Optional, Tuple

import numpy as np

from . import engine
from .geometry import MM, MRAD, P2, P3, as_xyz
from .particles import (ParticleFactory, PhaseSpaceParticle, RunningParticle, particles_to_array)


class GPU_ACCELERATOR:
    FLOAT32: str = "FLOAT32"
    FLOAT64: str = "FLOAT64"
    QS_DATA_LENGTH = 16

    def __init__(self, float_number_type: str = FLOAT32, block_dim_x: int = 1024,
                 max_current_element_number: int = 2000 * 120, max_qs_datas_length: int = 10000,
                 cpu_mode: bool = False) -> None:
        if cpu_mode:
            raise NotImplementedError("cctpy_gb300 runs on the GPU only; there is no CPU mode")
        if block_dim_x > 1024 or block_dim_x < 0:
            raise ValueError(f"block_dim_x must be in [1, 1024], not {block_dim_x}")
        if block_dim_x & (block_dim_x - 1) != 0:
            raise ValueError(f"block_dim_x must be a power of 2, not {block_dim_x}")
        if float_number_type == self.FLOAT32:
            self.precision, self.numpy_dtype = "f32c", np.float32
        elif float_number_type == self.FLOAT64:
            self.precision, self.numpy_dtype = "f64", np.float64
        else:
            raise ValueError("float_number_type must be GPU_ACCELERATOR.FLOAT32 or GPU_ACCELERATOR.FLOAT64")
        self.float_number_type = float_number_type
        self.block_dim_x = int(block_dim_x)
        self.max_current_element_number = int(max_current_element_number)
        self.max_qs_datas_length = int(max_qs_datas_length)
        self.cpu_mode = False

    # ------------------------------------------------------------------ helpers
    def _design(self, magnets: list, single_qs: bool = False):
        for m in magnets:
            if engine._classify(m) not in ("cct", "qs"):
                # the reference accelerator takes CCT and QS only (gpu_accelerator.py:1417, :1970)
                raise ValueError(f"GPU_ACCELERATOR evaluates CCT and QS magnets only, not {m}; use "
                                 "cctpy_gb300.engine for Q, LocalUniformMagnet, UniformMagnet, Wire and connectors")
        kl, p0, qs = engine.host_design(magnets)
        if single_qs and qs.shape[0] > 1:
            qs = qs[-1:]      # the single-QS kernels of the reference keep the last QS
        if kl.shape[0] > self.max_current_element_number:
            raise ValueError(f"{kl.shape[0]} current elements exceed max_current_element_number "
                             f"({self.max_current_element_number})")
        if qs.shape[0] > self.max_qs_datas_length:
            raise ValueError(f"{qs.shape[0]} QS magnets exceed max_qs_datas_length ({self.max_qs_datas_length})")
        return kl, p0, qs

    def _field(self, design, point: P3) -> P3:
        ds = engine.DesignSet([design])
        B = engine.field_at_points(ds, as_xyz(point)[None, :], self.precision)[0]
        return P3(B[0], B[1], B[2])

    def _track(self, designs, ps: List[RunningParticle], distance: float, footstep: float) -> np.ndarray:
        ds = engine.DesignSet(designs)
        return engine.track(ds, particles_to_array(ps), distance, footstep, self.precision)

    # ------------------------------------------------------------------ field calls
    def current_element_B(self, kls: np.ndarray, p0s: np.ndarray, number: int, p: P3) -> P3:
        """Field of `number` raw current elements (flat kls / p0s, global frame) at p
        (gpu_accelerator.py:1147-1196)."""
        kl = np.asarray(kls, dtype=np.float64).reshape(-1, 3)[:number]
        p0 = np.asarray(p0s, dtype=np.float64).reshape(-1, 3)[:number]
        return self._field((kl, p0, np.zeros((0, 16))), p)

    def magnet_at_qs(self, qs_data, p3: P3) -> P3:
        """One QS record (16 numbers) at p (gpu_accelerator.py:1198-1259)."""
        return self._field((np.zeros((0, 3)), np.zeros((0, 3)), np.asarray(qs_data, np.float64).reshape(1, 16)), p3)

    magnet_at_qs_date = magnet_at_qs

    def magnet_at_qs_dates(self, qss: list, p: P3) -> P3:
        """Sum of several QS magnets at p (gpu_accelerator.py:1306-1347)."""
        rec = np.stack([engine.qs_record(q) for q in qss]) if qss else np.zeros((0, 16))
        return self._field((np.zeros((0, 3)), np.zeros((0, 3)), rec), p)

    def magnet_at_beamline_with_single_qs(self, bl, p: P3) -> P3:
        """Beamline field at p, CCTs plus one QS (gpu_accelerator.py:1349-1432)."""
        return self._field(self._design(engine.magnet_list(bl), single_qs=True), p)

    # ------------------------------------------------------------------ tracking
    def track_one_particle_with_single_qs(self, bl, p: RunningParticle, distance: float, footstep: float):
        out = self._track([self._design(engine.magnet_list(bl), single_qs=True)], [p], distance, footstep)[0, 0]
        p.populate(RunningParticle.from_numpy_array_data(out))

    def track_one_particle_with_multi_qs(self, bl, p: RunningParticle, distance: float, footstep: float):
        out = self._track([self._design(engine.magnet_list(bl))], [p], distance, footstep)[0, 0]
        p.populate(RunningParticle.from_numpy_array_data(out))

    def track_multi_particle_for_magnet_with_single_qs(self, bl, ps: List[RunningParticle], distance: float,
                                                       footstep: float):
        out = self._track([self._design(engine.magnet_list(bl), single_qs=True)], ps, distance, footstep)[0]
        for p, r in zip(ps, out):
            p.populate(RunningParticle.from_numpy_array_data(r))

    def track_multi_particle_for_magnet_with_multi_qs(self, bl, ps: List[RunningParticle], distance: float,
                                                      footstep: float):
        out = self._track([self._design(engine.magnet_list(bl))], ps, distance, footstep)[0]
        for p, r in zip(ps, out):
            p.populate(RunningParticle.from_numpy_array_data(r))

    def _multi_beamline(self, bls, ps, distance, footstep, single_qs):
        if not bls:
            return []
        built = {}
        for b in bls:      # the same beamline object several times: one design, repeated on the device
            if id(b) not in built:
                built[id(b)] = self._design(engine.magnet_list(b), single_qs)
        out = self._track([built[id(b)] for b in bls], ps, distance, footstep)
        return [[RunningParticle.from_numpy_array_data(r) for r in row] for row in out]

    def track_multi_particle_beamline_for_magnet_with_single_qs(self, bls: list, ps: List[RunningParticle],
                                                                distance: float,
                                                                footstep: float) -> List[List[RunningParticle]]:
        return self._multi_beamline(bls, ps, distance, footstep, True)

    def track_multi_particle_beamline_for_magnet_with_multi_qs(self, bls: list, ps: List[RunningParticle],
                                                               distance: float,
                                                               footstep: float) -> List[List[RunningParticle]]:
        return self._multi_beamline(bls, ps, distance, footstep, False)

    def track_phase_ellipse_in_multi_beamline(self, beamlines: list, x_sigma_mm: float, xp_sigma_mrad: float,
                                              y_sigma_mm: float, yp_sigma_mrad, delta: float, particle_number: int,
                                              kinetic_MeV: float, s: float = 0.0, length: Optional[float] = None,
                                              footstep: float = 10 * MM,
                                              report: bool = True) -> List[Tuple[List[P2], List[P2]]]:
        """Track x-xp and y-yp phase ellipses through every beamline (which share one design
        orbit); returns per beamline the (x, xp) and (y, yp) end points in mm / mrad
        (gpu_accelerator.py:2047-2152)."""
        traj = beamlines[0].trajectory
        if length is None:
            length = traj.get_length() - s
        ip_start = ParticleFactory.create_proton_along(traj, s, kinetic_MeV)
        ip_end = ParticleFactory.create_proton_along(traj, s + length, kinetic_MeV)
        pp_x = PhaseSpaceParticle.phase_space_particles_along_positive_ellipse_in_xxp_plane(
            x_sigma_mm * MM, xp_sigma_mrad * MRAD, delta, particle_number)
        pp_y = PhaseSpaceParticle.phase_space_particles_along_positive_ellipse_in_yyp_plane(
            y_sigma_mm * MM, yp_sigma_mrad * MRAD, delta, particle_number)
        frame = ip_start.get_natural_coordinate_system()
        rp = (ParticleFactory.create_from_phase_space_particles(ip_start, frame, pp_x)
              + ParticleFactory.create_from_phase_space_particles(ip_start, frame, pp_y))
        ends = self.track_multi_particle_beamline_for_magnet_with_multi_qs(beamlines, rp, length, footstep)
        end_frame = ip_end.get_natural_coordinate_system()
        ret = []
        for row in ends:
            for p in row:
                p.speed = p.velocity.length()
            pps = PhaseSpaceParticle.create_from_running_particles(ip_end, end_frame, row)
            xs = PhaseSpaceParticle.phase_space_particles_project_to_xxp_plane(pps[:particle_number], True)
            ys = PhaseSpaceParticle.phase_space_particles_project_to_yyp_plane(pps[particle_number:], True)
            ret.append((xs, ys))
        return ret
