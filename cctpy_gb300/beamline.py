"""Beamline assembly: a design orbit with magnets placed along it, and the HUST
superconducting gantry builder.

Same builder names, arguments and layer conventions as cctpy
(final_code/packages/beamline.py:33-793, final_code/hust_sc_gantry.py:18-385):
a dipole CCT is an inner layer (tilts as given, xi from 0 to +2 pi W) and an
outer layer (tilts negated, xi to -2 pi W); an AG-CCT adds, after the outer and
inner dipole layers, an inner/outer pair per alternating-gradient part, whose
xi-phi start points continue from the previous part's end shifted by one
winding's phi advance.
"""
from __future__ import annotations

import math
from typing import List, Optional, Tuple

from .geometry import MM, P2, P3, Line2, Trajectory
from .magnets import CCT, QS, LocalUniformMagnet, Magnet, Q


def _rad(d: float) -> float:
    return d / 180.0 * math.pi


class Beamline(Line2, Magnet):
    """Design orbit + magnets (cctpy beamline.py:33-53); also a Magnet whose field is the sum."""

    def __init__(self, trajectory: Trajectory):
        self.magnets: List[Magnet] = []
        self.trajectory = trajectory
        self.elements: List[Tuple[float, Optional[Magnet], float]] = []

    class _Builder:
        def __init__(self, start_point: P2):
            self.start_point = start_point

        def first_drift(self, direct: P2 = None, length: float = 1.0) -> "Beamline":
            bl = Beamline(Trajectory.set_start_point(self.start_point).first_line(
                P2.x_direct() if direct is None else direct, length))
            bl.elements.append((0, None, length))
            return bl

    @staticmethod
    def set_start_point(start_point: P2 = None) -> "Beamline._Builder":
        return Beamline._Builder(P2() if start_point is None else start_point)

    # ---- Line2
    def get_length(self) -> float:
        return self.trajectory.get_length()

    def point_at(self, s: float) -> P2:
        return self.trajectory.point_at(s)

    def direct_at(self, s: float) -> P2:
        return self.trajectory.direct_at(s)

    def get_magnets(self) -> List[Magnet]:
        return self.magnets

    def get_trajectory(self) -> Trajectory:
        return self.trajectory

    def magnets_for_gpu(self) -> List[Magnet]:
        out = []
        for m in self.magnets:
            out.extend(m.magnets_for_gpu())
        return out

    def _changed(self) -> "Beamline":
        self.__dict__.pop("_cctgpu_design", None)
        return self

    # ---- builders
    def append_drift(self, length: float) -> "Beamline":
        old = self.trajectory.get_length()
        self.trajectory.add_strait_line(length=length)
        self.elements.append((old, None, length))
        return self

    def append_qs(self, length: float, gradient: float, second_gradient: float, aperture_radius: float) -> "Beamline":
        old = self.trajectory.get_length()
        self.trajectory.add_strait_line(length=length)
        qs = QS.create_qs_along(self.trajectory, old, length, gradient, second_gradient, aperture_radius)
        self.magnets.append(qs)
        self.elements.append((old, qs, length))
        return self._changed()

    def append_q(self, length: float, gradient: float, aperture_radius: float) -> "Beamline":
        """A hard-edge quadrupole along the orbit (beamline.py:478-505)."""
        old = self.trajectory.get_length()
        self.trajectory.add_strait_line(length=length)
        q = Q.create_q_along(self.trajectory, old, length, gradient, aperture_radius)
        self.magnets.append(q)
        self.elements.append((old, q, length))
        return self._changed()

    def append_straight_dipole_magnet(self, magnetic_field: float, length: float,
                                      aperture_radius: float) -> "Beamline":
        """A straight dipole (LocalUniformMagnet) along the orbit (beamline.py:420-444)."""
        old = self.trajectory.get_length()
        self.trajectory.add_strait_line(length=length)
        lum = LocalUniformMagnet.create_local_uniform_magnet_along(self.trajectory, old, magnetic_field, length,
                                                                   aperture_radius)
        self.magnets.append(lum)
        self.elements.append((old, lum, length))
        return self._changed()

    def append_dipole_cct(self, big_r: float, small_r_inner: float, small_r_outer: float, bending_angle: float,
                          tilt_angles: List[float], winding_number: int, current: float,
                          disperse_number_per_winding: int = 120) -> "Beamline":
        old = self.trajectory.get_length()
        length = big_r * abs(_rad(bending_angle))
        self.trajectory.add_arc_line(radius=big_r, clockwise=bending_angle < 0, angle_deg=abs(bending_angle))
        end_phi = _rad(bending_angle)
        for role, small_r, tilts, ksi_end in (
                ("dipole_inner", small_r_inner, tilt_angles, 2 * math.pi * winding_number),
                ("dipole_outer", small_r_outer, [t * -1 for t in tilt_angles], -2 * math.pi * winding_number)):
            c = CCT.create_cct_along(self.trajectory, old, big_r, small_r, abs(bending_angle), tilts, winding_number,
                                     current, P2.origin(), P2(ksi_end, end_phi), disperse_number_per_winding)
            c.role = role
            self.magnets.append(c)
            self.elements.append((old, c, length))
        return self._changed()

    def append_agcct(self, big_r: float, small_rs: List[float], bending_angles: List[float],
                     tilt_angles: List[List[float]], winding_numbers: List[List[int]], currents: List[float],
                     disperse_number_per_winding: int = 120) -> "Beamline":
        if len(small_rs) != 4:
            raise ValueError(f"small_rs({small_rs}) must hold 4 radii: dipole outer, dipole inner, AG outer, "
                             "AG inner")
        if any(small_rs[i] < small_rs[i + 1] for i in range(3)):
            raise ValueError(f"small_rs({small_rs}) must be sorted from largest to smallest")
        dpw = disperse_number_per_winding
        total = sum(bending_angles)
        old = self.trajectory.get_length()
        length = big_r * abs(_rad(total))
        self.trajectory.add_arc_line(radius=big_r, clockwise=total < 0, angle_deg=abs(total))
        wd = winding_numbers[0][0]
        for role, small_r, tilts, sign in (("dipole_outer", small_rs[0], [t * -1 for t in tilt_angles[0]], -1),
                                           ("dipole_inner", small_rs[1], tilt_angles[0], 1)):
            c = CCT.create_cct_along(self.trajectory, old, big_r, small_r, abs(total), tilts, wd, currents[0],
                                     P2.origin(), P2(sign * 2 * math.pi * wd, _rad(total)), dpw)
            c.role = role
            self.magnets.append(c)
            self.elements.append((old, c, length))
        ag_tilt, ag_cur, wn = tilt_angles[1], currents[1], winding_numbers[1]
        rad = [_rad(a) for a in bending_angles]
        start_in, start_out = P2.origin(), P2.origin()
        end_in = end_out = None
        s_part = old
        for k in range(len(bending_angles)):
            if k > 0:
                shift = P2(0, rad[k - 1] / wn[k - 1])
                start_in, start_out = end_in + shift, end_out + shift
            sgn = (-1.0) ** k
            end_in = start_in + P2(sgn * 2 * math.pi * wn[k], rad[k])
            end_out = start_out + P2(-sgn * 2 * math.pi * wn[k], rad[k])
            part_len = big_r * _rad(abs(bending_angles[k]))
            for role, small_r, tilts, a, b in (("ag_inner", small_rs[3], [t * -1 for t in ag_tilt], start_in, end_in),
                                               ("ag_outer", small_rs[2], ag_tilt, start_out, end_out)):
                c = CCT.create_cct_along(self.trajectory, old, big_r, small_r, abs(bending_angles[k]), tilts, wn[k],
                                         ag_cur, a, b, dpw)
                c.role = role
                self.magnets.append(c)
                self.elements.append((s_part, c, part_len))
            s_part += part_len
        return self._changed()

    def __repr__(self) -> str:
        return f"beamline(magnet_size={len(self.magnets)}, traj_len={self.trajectory.get_length()})"


class HUST_SC_GANTRY:
    """HUST superconducting proton gantry (cctpy final_code/hust_sc_gantry.py:18-385):
    first bending section (two AG-CCT blocks around a QS triplet) and second
    bending section (two AG-CCT blocks around one QS)."""

    DEFAULTS = dict(
        DL1=0.9007765, GAP1=0.4301517, GAP2=0.370816,
        qs1_length=0.2340128, qs1_aperture_radius=60 * MM, qs1_gradient=3.1, qs1_second_gradient=7.9,
        qs2_length=0.200139, qs2_aperture_radius=60 * MM, qs2_gradient=3.8, qs2_second_gradient=-34.5,
        cct12_big_r=0.95, agcct12_inner_small_r=72.5 * MM, agcct12_outer_small_r=88.5 * MM,
        dicct12_inner_small_r=104.5 * MM, dicct12_outer_small_r=120.5 * MM,
        agcct1_winding_number=21, agcct2_winding_number=21, dicct12_winding_number=42,
        dicct12_bending_angle=22.5, agcct1_bending_angle=22.5 / 2, agcct2_bending_angle=22.5 / 2,
        dicct12_tilt_angles=[30, 102.8, 95.6, 87.3], agcct12_tilt_angles=[93.5, 30, 78.3, 97.5],
        dicct12_current=-9780.7, agcct12_current=9736.8,
        DL2=2.1162209, GAP3=0.1978111,
        qs3_length=0.2382791, qs3_aperture_radius=60 * MM, qs3_gradient=-7.3733, qs3_second_gradient=-45.31 * 2,
        cct345_big_r=0.95, agcct345_inner_small_r=83 * MM, agcct345_outer_small_r=83 * MM + 15 * MM,
        dicct345_inner_small_r=83 * MM + 15 * MM * 2, dicct345_outer_small_r=83 * MM + 15 * MM * 3,
        agcct3_winding_number=21, agcct4_winding_number=50, agcct5_winding_number=50, dicct345_winding_number=128,
        dicct345_bending_angle=-67.5, agcct3_bending_angle=-(8 + 3.716404), agcct4_bending_angle=-(8 + 19.93897),
        agcct5_bending_angle=-(8 + 19.844626), dicct345_tilt_angles=[30, 80], agcct345_tilt_angles=[90, 30],
        dicct345_current=9664, agcct345_current=-6000, part_per_winding=120)

    def __init__(self, **kwargs):
        unknown = set(kwargs) - set(self.DEFAULTS)
        if unknown:
            raise TypeError(f"unknown HUST_SC_GANTRY arguments: {sorted(unknown)}")
        for k, v in self.DEFAULTS.items():
            setattr(self, k, kwargs.get(k, v))
        self._first = None
        self._second = None
        self._total = None

    def _first_section(self, bl: Beamline) -> Beamline:
        ag = lambda angles, windings: dict(
            big_r=self.cct12_big_r,
            small_rs=[self.dicct12_outer_small_r, self.dicct12_inner_small_r, self.agcct12_outer_small_r,
                      self.agcct12_inner_small_r],
            bending_angles=angles, tilt_angles=[self.dicct12_tilt_angles, self.agcct12_tilt_angles],
            winding_numbers=[[self.dicct12_winding_number], windings],
            currents=[self.dicct12_current, self.agcct12_current], disperse_number_per_winding=self.part_per_winding)
        q1 = dict(length=self.qs1_length, gradient=self.qs1_gradient, second_gradient=self.qs1_second_gradient,
                  aperture_radius=self.qs1_aperture_radius)
        q2 = dict(length=self.qs2_length, gradient=self.qs2_gradient, second_gradient=self.qs2_second_gradient,
                  aperture_radius=self.qs2_aperture_radius)
        return (bl.append_agcct(**ag([self.agcct1_bending_angle, self.agcct2_bending_angle],
                                     [self.agcct1_winding_number, self.agcct2_winding_number]))
                .append_drift(self.GAP1).append_qs(**q1).append_drift(self.GAP2).append_qs(**q2)
                .append_drift(self.GAP2).append_qs(**q1).append_drift(self.GAP1)
                .append_agcct(**ag([self.agcct2_bending_angle, self.agcct1_bending_angle],
                                   [self.agcct2_winding_number, self.agcct1_winding_number]))
                .append_drift(self.DL1))

    def _second_section(self, bl: Beamline) -> Beamline:
        ag = lambda angles, windings: dict(
            big_r=self.cct345_big_r,
            small_rs=[self.dicct345_outer_small_r, self.dicct345_inner_small_r, self.agcct345_outer_small_r,
                      self.agcct345_inner_small_r],
            bending_angles=angles, tilt_angles=[self.dicct345_tilt_angles, self.agcct345_tilt_angles],
            winding_numbers=[[self.dicct345_winding_number], windings],
            currents=[self.dicct345_current, self.agcct345_current],
            disperse_number_per_winding=self.part_per_winding)
        return (bl.append_agcct(**ag([self.agcct3_bending_angle, self.agcct4_bending_angle, self.agcct5_bending_angle],
                                     [self.agcct3_winding_number, self.agcct4_winding_number,
                                      self.agcct5_winding_number]))
                .append_drift(self.GAP3)
                .append_qs(length=self.qs3_length, gradient=self.qs3_gradient,
                           second_gradient=self.qs3_second_gradient, aperture_radius=self.qs3_aperture_radius)
                .append_drift(self.GAP3)
                .append_agcct(**ag([self.agcct5_bending_angle, self.agcct4_bending_angle, self.agcct3_bending_angle],
                                   [self.agcct5_winding_number, self.agcct4_winding_number,
                                    self.agcct3_winding_number]))
                .append_drift(self.DL2))

    def create_first_bending_part_beamline(self) -> Beamline:
        if self._first is None:
            self._first = self._first_section(Beamline.set_start_point(P2.origin()).first_drift(P2.x_direct(),
                                                                                                  self.DL1))
        return self._first

    def create_second_bending_part_beamline(self) -> Beamline:
        if self._second is None:
            first = self.create_first_bending_part_beamline()
            bl = Beamline.set_start_point(first.point_at_end()).first_drift(first.direct_at_end(), self.DL2)
            self._second = self._second_section(bl)
        return self._second

    def create_total_beamline(self) -> Beamline:
        if self._total is None:
            bl = Beamline.set_start_point(P2.origin()).first_drift(P2.x_direct(), self.DL1)
            bl = self._first_section(bl).append_drift(self.DL2)
            self._total = self._second_section(bl)
        return self._total
