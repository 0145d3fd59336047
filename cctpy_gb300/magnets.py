"""Magnets on the tracking path: the Magnet interface, CCT layers, QS magnets.

Same names, arguments and errors as cctpy (final_code/packages/magnets.py:57,
:539-586, :589-748 and cct.py:31-457).  Field evaluation always runs on the
GPU through libcctgpu (see ``engine``); segment generation is host-side,
vectorised numpy in FP64.
"""
from __future__ import annotations

import math
from typing import Iterable, List, Optional, Tuple

import numpy as np

from .geometry import (MM, FunctionLine3, P2, P3, LocalCoordinateSystem, StraightLine2, Trajectory, approx_equal,
                       as_xyz, circle_center_and_radius, derivative, linspace)


def _deg2rad(d: float) -> float:
    return d / 180.0 * math.pi


def _is_90(t: float) -> bool:
    return t == 90.0 or abs(t - 90.0) <= 1e-6 or ((t + 90.0 != 0.0) and 2 * abs((t - 90.0) / (t + 90.0)) <= 1e-6)


class Magnet:
    """Anything with a magnetic field (cctpy magnets.py:48-67)."""

    def magnetic_field_at(self, point: P3) -> P3:
        """Field at one global point, evaluated on the GPU in FP64."""
        B = self.magnetic_field_at_points(as_xyz(point)[None, :])[0]
        return P3(B[0], B[1], B[2])

    def magnetic_field_at_points(self, points: np.ndarray, precision: str = "f64") -> np.ndarray:
        """Field at an (n, 3) array of global points -> (n, 3) tesla (batched GPU call).

        precision: "f64" (plain FP64) or "f32c" (FP32 with FP64 tile origins and
        compensated sums, <= 1e-7 relative)."""
        from . import engine
        return engine.field_at_points(engine.design_of(self), points, precision)

    def magnets_for_gpu(self) -> List["Magnet"]:
        """The CCT / QS magnets whose fields sum to this magnet's field."""
        return [self]


class CombinedMagnet(Magnet):
    """Sum of several magnets (cctpy magnets.py:539-586)."""

    def __init__(self, *magnets):
        for m in magnets:
            if not isinstance(m, Magnet):
                raise ValueError(f"{m} is not a magnet")
        self._magnets: List[Magnet] = list(magnets)

    def add(self, m: Magnet) -> "CombinedMagnet":
        self._magnets.append(m)
        self.__dict__.pop("_cctgpu_design", None)
        return self

    def add_all(self, ms: Iterable[Magnet]) -> "CombinedMagnet":
        self._magnets.extend(ms)
        self.__dict__.pop("_cctgpu_design", None)
        return self

    def get_magnets(self) -> List[Magnet]:
        return self._magnets

    def remove(self, m: Magnet) -> "CombinedMagnet":
        self._magnets.remove(m)
        self.__dict__.pop("_cctgpu_design", None)
        return self

    def magnets_for_gpu(self) -> List[Magnet]:
        out = []
        for m in self._magnets:
            out.extend(m.magnets_for_gpu())
        return out


class QS(Magnet):
    """Hard-edge quadrupole + sextupole (cctpy magnets.py:589-748)."""

    def __init__(self, local_coordinate_system: LocalCoordinateSystem, length: float, gradient: float,
                 second_gradient: float, aperture_radius: float):
        self.local_coordinate_system = local_coordinate_system
        self.length = float(length)
        self.gradient = float(gradient)
        self.second_gradient = float(second_gradient)
        self.aperture_radius = float(aperture_radius)

    def to_numpy_array(self, numpy_dtype=np.float64) -> np.ndarray:
        """16 numbers: origin, XI, YI, ZI, length, gradient, second gradient, aperture radius."""
        lcs = self.local_coordinate_system
        return np.array(lcs.location.to_list() + lcs.XI.to_list() + lcs.YI.to_list() + lcs.ZI.to_list()
                        + [self.length, self.gradient, self.second_gradient, self.aperture_radius],
                        dtype=numpy_dtype)

    def is_out_of_aperture(self, point: P3) -> bool:
        lp = self.local_coordinate_system.point_to_local_coordinate(point)
        if 0 <= lp.z <= self.length:
            return (lp.x ** 2 + lp.y ** 2) > self.aperture_radius ** 2
        return False

    @staticmethod
    def create_qs_along(trajectory, s: float, length: float, gradient: float, second_gradient: float,
                        aperture_radius: float) -> "QS":
        origin = trajectory.point_at(s)
        z = trajectory.direct_at(s)
        x = z.rotate(_deg2rad(90))
        return QS(LocalCoordinateSystem(origin.to_p3(), x.to_p3(), z.to_p3()), length, gradient, second_gradient,
                  aperture_radius)

    @staticmethod
    def as_qs(anything) -> "QS":
        return anything

    def __repr__(self) -> str:
        return (f"QS:local_coordinate_system={self.local_coordinate_system}, length={self.length}, "
                f"gradient={self.gradient}, second_gradient={self.second_gradient}, "
                f"aperture_radius={self.aperture_radius}")


class CCT(Magnet):
    """One layer of a bent CCT winding (cctpy cct.py:31-457).

    The winding is the curve xi -> (xi, phi(xi)) in bipolar-toroidal coordinates,
    phi(xi) = k xi + b + sum_i cot(tilt_i) / ((i+1) sinh eta) sin((i+1) xi) over
    the tilt angles that are not 90 deg, mapped to xyz with
    a / (cosh eta - cos xi) * (sinh eta cos phi, sinh eta sin phi, sin xi),
    a = sqrt(R^2 - r^2), eta = ln((R + a)/(R - a)) / 2; it is cut at
    W * n + 1 equally spaced xi into W * n straight current elements.
    """

    def __init__(self, local_coordinate_system: LocalCoordinateSystem, big_r: float, small_r: float,
                 bending_angle: float, tilt_angles: List[float], winding_number: int, current: float,
                 starting_point_in_ksi_phi_coordinate: P2, end_point_in_ksi_phi_coordinate: P2,
                 disperse_number_per_winding: int = 120):
        if bending_angle < 0:
            raise ValueError(f"CCT bending angle must be positive, not {bending_angle}; reverse the bend "
                             "through the xi-phi start and end points")
        if big_r < 0:
            raise ValueError(f"big_r = {big_r} is negative")
        if small_r < 0:
            raise ValueError(f"small_r = {small_r} is negative")
        if small_r >= big_r:
            raise ValueError(f"small_r {small_r} >= big_r {big_r}")
        self.local_coordinate_system = local_coordinate_system
        self.big_r = float(big_r)
        self.small_r = float(small_r)
        self.bending_angle = float(bending_angle)
        self.tilt_angles = [float(t) for t in tilt_angles]
        self.winding_number = int(winding_number)
        self.current = float(current)
        self.starting_point_in_ksi_phi_coordinate = starting_point_in_ksi_phi_coordinate
        self.end_point_in_ksi_phi_coordinate = end_point_in_ksi_phi_coordinate
        self.disperse_number_per_winding = int(disperse_number_per_winding)
        self.bending_radian = _deg2rad(self.bending_angle)
        self.tilt_radians = [_deg2rad(t) for t in self.tilt_angles]
        self.phi0 = self.bending_radian / self.winding_number
        self.a = math.sqrt(self.big_r ** 2 - self.small_r ** 2)
        self.eta = 0.5 * math.log((self.big_r + self.a) / (self.big_r - self.a))
        self.total_disperse_number = self.winding_number * self.disperse_number_per_winding
        self._path_local = None

    # ---- winding path
    def phi_ksi_function(self, ksi):
        x1, y1 = self.starting_point_in_ksi_phi_coordinate.x, self.starting_point_in_ksi_phi_coordinate.y
        x2, y2 = self.end_point_in_ksi_phi_coordinate.x, self.end_point_in_ksi_phi_coordinate.y
        k = (y2 - y1) / (x2 - x1)
        b = -k * x1 + y1
        phi = k * ksi + b
        sh = math.sinh(self.eta)
        for i, t in enumerate(self.tilt_angles):
            if not _is_90(t):
                phi = phi + ((1 / math.tan(self.tilt_radians[i])) / ((i + 1) * sh)) * np.sin((i + 1) * ksi)
        return phi

    def phi_at(self, ksi: float) -> float:
        """phi(xi) for one xi with the math module, term by term as cct.py:166-188."""
        x1, y1 = self.starting_point_in_ksi_phi_coordinate.x, self.starting_point_in_ksi_phi_coordinate.y
        x2, y2 = self.end_point_in_ksi_phi_coordinate.x, self.end_point_in_ksi_phi_coordinate.y
        k = (y2 - y1) / (x2 - x1)
        b = -k * x1 + y1
        phi = k * ksi + b
        for i, t in enumerate(self.tilt_angles):
            if not _is_90(t):
                phi += (1 / math.tan(self.tilt_radians[i])) / ((i + 1) * math.sinh(self.eta)) * math.sin((i + 1) * ksi)
        return phi

    def p2_function(self, ksi: float) -> P2:
        """(xi, phi(xi)) (cct.py:459-465)."""
        return P2(ksi, self.phi_at(ksi))

    def p3_function(self, ksi: float) -> P3:
        """Winding point at xi in the local frame (cct.py:467-473 with the bipolar-toroidal
        conversion of :213-224)."""
        phi = self.phi_at(ksi)
        temp = self.a / (math.cosh(self.eta) - math.cos(ksi))
        return P3(temp * math.sinh(self.eta) * math.cos(phi), temp * math.sinh(self.eta) * math.sin(phi),
                  temp * math.sin(ksi))

    def ksi_samples(self) -> np.ndarray:
        x1, x2 = self.starting_point_in_ksi_phi_coordinate.x, self.end_point_in_ksi_phi_coordinate.x
        n = self.total_disperse_number
        d = (x2 - x1) * (1 / n)
        return x1 + d * np.arange(n + 1, dtype=np.float64)

    def path_local(self) -> np.ndarray:
        """(W*n+1, 3) winding points in the CCT's local frame."""
        if self._path_local is None:
            ksi = self.ksi_samples()
            phi = self.phi_ksi_function(ksi)
            temp = self.a / (math.cosh(self.eta) - np.cos(ksi))
            sh = math.sinh(self.eta)
            self._path_local = np.stack([temp * sh * np.cos(phi), temp * sh * np.sin(phi), temp * np.sin(ksi)], 1)
        return self._path_local

    @property
    def dispersed_path3(self) -> np.ndarray:
        return self.path_local()

    @property
    def elementary_current(self) -> np.ndarray:
        p = self.path_local()
        return 1e-7 * self.current * (p[1:] - p[:-1])

    @property
    def elementary_current_position(self) -> np.ndarray:
        p = self.path_local()
        return 0.5 * (p[1:] + p[:-1])

    def global_segments(self) -> Tuple[np.ndarray, np.ndarray]:
        """(kl, p0) in the global frame, (N, 3) FP64 each."""
        g = self.local_coordinate_system.points_to_global(self.path_local())
        return 1e-7 * self.current * (g[1:] - g[:-1]), 0.5 * (g[1:] + g[:-1])

    def global_current_elements_and_elementary_current_positions(self, numpy_dtype=np.float64):
        """Flat (3N,) arrays as cctpy returns them (cct.py:434-457)."""
        kl, p0 = self.global_segments()
        return kl.astype(numpy_dtype).reshape(-1), p0.astype(numpy_dtype).reshape(-1)

    def is_out_of_aperture(self, point: P3) -> bool:
        lp = self.local_coordinate_system.point_to_local_coordinate(point)
        r2 = P2(lp.x, lp.y)
        clockwise = self.end_point_in_ksi_phi_coordinate.y < 0
        phi = r2.angle_to_x_axis()
        inside = phi > (2 * math.pi - self.bending_radian) if clockwise else phi < self.bending_radian
        if not inside:
            return False
        return (abs(lp.z) > self.small_r or r2.length() > self.big_r + self.small_r
                or r2.length() < self.big_r - self.small_r)

    @staticmethod
    def create_cct_along(trajectory, s: float, big_r: float, small_r: float, bending_angle: float,
                         tilt_angles: List[float], winding_number: int, current: float,
                         starting_point_in_ksi_phi_coordinate: P2, end_point_in_ksi_phi_coordinate: P2,
                         disperse_number_per_winding: int = 120) -> "CCT":
        """Place a CCT on the orbit at arc length s (cct.py:341-421): the frame's origin is
        the centre of the orbit arc it spans (mean of the circles through the start and
        third points and through the third points and the end), z is global z, y is the
        start direction (counter-clockwise bend) or its reverse (clockwise bend)."""
        L = big_r * _deg2rad(bending_angle)
        sp, ep = trajectory.point_at(s), trajectory.point_at(s + L)
        m0, m1 = trajectory.point_at(s + L / 3 * 1), trajectory.point_at(s + L / 3 * 2)
        c1, _ = circle_center_and_radius(sp, m0, m1)
        c2, _ = circle_center_and_radius(m0, m1, ep)
        center = (c1 + c2) * 0.5
        sd = trajectory.direct_at(s)
        side = StraightLine2(1.0, sd, sp).side_of(center)
        if side == 0:
            raise ValueError(f"CCT centre {center} lies on the design orbit {trajectory}")
        y = -sd.to_p3() if side == 1 else sd.to_p3()
        lcs = LocalCoordinateSystem.create_by_y_and_z_direction(center.to_p3(), y, P3.z_direct())
        return CCT(lcs, big_r, small_r, bending_angle, tilt_angles, winding_number, current,
                   starting_point_in_ksi_phi_coordinate, end_point_in_ksi_phi_coordinate,
                   disperse_number_per_winding)

    @staticmethod
    def as_cct(anything) -> "CCT":
        return anything

    def __repr__(self) -> str:
        return (f"CCT: local_coordinate_system({self.local_coordinate_system})big_r({self.big_r})"
                f"small_r({self.small_r})bending_angle({self.bending_angle})tilt_angles({self.tilt_angles})"
                f"winding_number({self.winding_number})current({self.current})"
                f"disperse_number_per_winding({self.disperse_number_per_winding})")



class Q(Magnet):
    """Hard-edge quadrupole: a QS without the sextupole term (magnets.py:762-832)."""

    def __init__(self, local_coordinate_system: LocalCoordinateSystem, length: float, gradient: float,
                 aperture_radius: float):
        self.local_coordinate_system = local_coordinate_system
        self.length = float(length)
        self.gradient = float(gradient)
        self.aperture_radius = float(aperture_radius)
        self.qs = QS(local_coordinate_system, length, gradient, 0.0, aperture_radius)

    def is_out_of_aperture(self, point: P3) -> bool:
        return self.qs.is_out_of_aperture(point)

    @staticmethod
    def create_q_along(trajectory, s: float, length: float, gradient: float, aperture_radius: float) -> "Q":
        origin = trajectory.point_at(s)
        z = trajectory.direct_at(s)
        x = z.rotate(_deg2rad(90))
        return Q(LocalCoordinateSystem(origin.to_p3(), x.to_p3(), z.to_p3()), length, gradient, aperture_radius)

    @staticmethod
    def as_q(anything) -> "Q":
        return anything

    def __repr__(self) -> str:
        return (f"Q:local_coordinate_system={self.local_coordinate_system}, length={self.length}, "
                f"gradient={self.gradient}, aperture_radius={self.aperture_radius}")


class LocalUniformMagnet(Magnet):
    """Uniform field `magnetic_field` (tesla) along the frame's YI inside the cylinder of radius
    aperture_radius around ZI for 0 <= z <= length, zero outside: a straight dipole
    (magnets.py:440-536)."""

    def __init__(self, local_coordinate_system: LocalCoordinateSystem, length: float, aperture_radius: float,
                 magnetic_field: float):
        self.local_coordinate_system = local_coordinate_system
        self.length = float(length)
        self.aperture_radius = float(aperture_radius)
        self.magnetic_field = float(magnetic_field)
        self.magnetic_field_vector = local_coordinate_system.YI * self.magnetic_field

    def is_out_of_aperture(self, point: P3) -> bool:
        lp = self.local_coordinate_system.point_to_local_coordinate(point)
        if lp.z < 0 or lp.z > self.length:
            return True
        a = self.aperture_radius
        return abs(lp.x) > a or abs(lp.y) > a or math.sqrt(lp.x ** 2 + lp.y ** 2) > a

    @staticmethod
    def create_local_uniform_magnet_along(trajectory, s: float, magnetic_field: float, length: float,
                                          aperture_radius: float) -> "LocalUniformMagnet":
        origin = trajectory.point_at(s)
        z = trajectory.direct_at(s)
        x = z.rotate(_deg2rad(90))
        return LocalUniformMagnet(LocalCoordinateSystem(origin.to_p3(), x.to_p3(), z.to_p3()), length,
                                  aperture_radius, magnetic_field)


class UniformMagnet(Magnet):
    """The same field everywhere (magnets.py:417-437)."""

    def __init__(self, magnetic_field: P3 = None):
        self.magnetic_field = P3() if magnetic_field is None else magnetic_field


class Wire(Magnet):
    """A wire along a 3-D curve in the global frame, cut into straight current elements of
    about delta_length in the curve's parameter (cct.py:625-691)."""

    def __init__(self, function_line3: FunctionLine3, current: float, delta_length: float = 1 * MM):
        self.function_line3 = function_line3
        self.current = current
        self.start = function_line3.get_start()
        self.end = function_line3.get_end()
        part_number = int(math.ceil((self.end - self.start) / delta_length))
        if part_number < 1:
            raise ValueError(f"a wire from {self.start} to {self.end} has no current element (the curve parameter "
                             "must increase)")
        self.dispersed_s = np.array(linspace(self.start, self.end, part_number + 1))
        self.dispersed_path3 = np.array([function_line3.point_at_p3_function(t).to_numpy_ndarry3()
                                         for t in self.dispersed_s])
        p = self.dispersed_path3
        self.elementary_current = 1e-7 * self.current * (p[1:] - p[:-1])
        self.elementary_current_position = 0.5 * (p[1:] + p[:-1])

    @staticmethod
    def create_by_cct(cct: "CCT") -> "Wire":
        """The CCT's winding as a wire (cct.py:814-832; the path is the CCT's local one)."""
        return Wire(FunctionLine3(cct.p3_function, cct.starting_point_in_ksi_phi_coordinate.x,
                                  cct.end_point_in_ksi_phi_coordinate.x),
                    cct.current, cct.small_r * _deg2rad(360 / cct.winding_number))


class AGCCT_CONNECTOR(Magnet):
    """The winding joining two consecutive AG-CCT layers of one frame (cct.py:835-994): in the
    plane (z, Xi) = (phi R, xi r) a straight run and a half circle from the first layer's end
    to the second layer's start, along the tangents of the two windings there, cut into
    `step` pieces and mapped back to the torus.  Current elements in the layers' local frame."""

    def __init__(self, agcct1: "CCT", agcct2: "CCT", step: float = 1 * MM):
        lcs1, lcs2 = agcct1.local_coordinate_system, agcct2.local_coordinate_system
        if not (lcs1.location == lcs2.location and lcs1.XI == lcs2.XI and lcs1.YI == lcs2.YI
                and lcs1.ZI == lcs2.ZI):
            raise ValueError(f"the CCTs to connect are not in one frame: {agcct1}, {agcct2}")
        for what, u, v in (("big_r", agcct1.big_r, agcct2.big_r), ("small_r", agcct1.small_r, agcct2.small_r),
                           ("current", agcct1.current, agcct2.current)):
            if not approx_equal(u, v):
                raise ValueError(f"the CCTs to connect differ in {what}: {u} != {v}")
        pre_end, next_start = agcct1.end_point_in_ksi_phi_coordinate, agcct2.starting_point_in_ksi_phi_coordinate
        if not approx_equal(pre_end.x, next_start.x):
            raise ValueError(f"the first CCT ends at xi = {pre_end.x}, the second starts at xi = {next_start.x}")
        self.current = agcct1.current
        self.local_coordinate_system = lcs1
        a = P2(x=pre_end.y * agcct1.big_r, y=0.0)
        b = P2(x=next_start.y * agcct2.big_r, y=0.0)

        def tangent(c):
            sign = -1 if c.starting_point_in_ksi_phi_coordinate.x > c.end_point_in_ksi_phi_coordinate.x else 1
            f = derivative(lambda ksi: P2(x=c.p2_function(ksi).y * c.big_r, y=c.p2_function(ksi).x * c.small_r))
            return f, sign

        fa, sa = tangent(agcct1)
        fb, sb = tangent(agcct2)
        va = fa(pre_end.x) * sa
        vb = fb(next_start.x) * sb
        ip, ka, kb = StraightLine2.intersecting_point(pa=a, va=va.copy().rotate(_deg2rad(90)), pb=b, vb=vb)
        if kb > 0:
            ip, ka, kb = StraightLine2.intersecting_point(pa=a, va=va, pb=b, vb=vb.copy().rotate(_deg2rad(90)))
            if ka < 0:
                raise ValueError("AGCCT_CONNECTOR: the tangents of the two windings do not meet ahead")
            ca = a + ka * va
            line = (Trajectory.set_start_point(a).first_line(direct=va, length=abs(ka * va.length()))
                    .add_arc_line(radius=(ca - b).length() / 2,
                                  clockwise=StraightLine2.is_on_right(ca, va, b) == 1, angle_deg=180.0))
        else:
            cb = b + kb * vb
            line = (Trajectory.set_start_point(a).first_line(direct=va, length=0.0)
                    .add_arc_line(radius=(a - cb).length() / 2, clockwise=StraightLine2.is_on_right(a, va, b) == 1,
                                  angle_deg=180.0)
                    .add_strait_line(length=abs(kb * vb.length())))
        self.connector_line_in_z_Θ = line
        self.length_in_z_Θ = line.get_length()
        r, R = agcct1.small_r, agcct1.big_r
        pts = []
        for p2 in line.disperse2d(step=step):
            ksi, phi = p2.y / r, p2.x / R
            temp = agcct1.a / (math.cosh(agcct1.eta) - math.cos(ksi))
            pts.append([temp * math.sinh(agcct1.eta) * math.cos(phi), temp * math.sinh(agcct1.eta) * math.sin(phi),
                        temp * math.sin(ksi)])
        self.dispersed_path3 = np.array(pts)
        p = self.dispersed_path3
        self.elementary_current = 1e-7 * self.current * (p[1:] - p[:-1])
        self.elementary_current_position = 0.5 * (p[1:] + p[:-1])
