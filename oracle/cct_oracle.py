"""CPU oracle (FP64) for the CCT Biot-Savart sum and the RK4 proton push.

TEST INFRASTRUCTURE.  This module restates, in plain Python scalars and numpy,
the algorithm of madokast/cctpy's CPU code for the tracking hot path.  It is
the checker for the CUDA kernels and the timed CPU reference in ``bench.py``;
the product package never imports it.

Every function names the reference lines it follows (paths relative to the
cctpy project root).  Scalar steps keep the reference's operation order, so
that segment generation and magnet placement agree bit for bit with the
reference and the field sum agrees to the last few ulps.  The restatement is
pinned against fixtures produced by the reference itself
(``tests/golden/make_golden.py``) and against the known answers held in the
reference's own tests.

Vectors are plain 3-tuples / 2-tuples of Python floats.
"""
from __future__ import annotations

import math
from typing import Callable, Dict, List, Sequence, Tuple

import numpy

V2 = Tuple[float, float]
V3 = Tuple[float, float, float]

# constants: final_code/packages/constants.py:12-19, particles.py:35-47
MM = 0.001
MRAD = 1.0 * MM * 1.0          # constants.py:14-15 (RAD = 1)
LIGHT_SPEED = 299792458.0
PROTON_STATIC_MASS_KG = 1.672621898e-27
PROTON_STATIC_ENERGY_MEV = 938.2720813
PROTON_CHARGE = 1.6021766208e-19


# ---------------------------------------------------------------- scalars
def approx_equal(a: float, b: float, err: float = 1e-6) -> bool:
    """final_code/packages/base_utils.py:35-58 (numeric branch)."""
    return a == b or abs(a - b) <= err or ((a + b != 0.0) and (2 * abs((a - b) / (a + b))) <= err)


def deg2rad(d: float) -> float:
    """base_utils.py:92-104: ``deg / 180.0 * math.pi``."""
    return d / 180.0 * math.pi


def linspace(start: float, end: float, number: int) -> List[float]:
    """base_utils.py:79-90: ``d = (end-start)*(1/(number-1)); start + d*float(i)``."""
    d = (end - start) * (1 / (number - 1))
    return [start + d * float(i) for i in range(number)]


# ---------------------------------------------------------------- 2-D / 3-D vectors (point.py)
def v2_len(a: V2) -> float:
    return math.sqrt(a[0] ** 2 + a[1] ** 2)          # point.py:31-35


def v2_scale(a: V2, s: float) -> V2:
    return (a[0] * s, a[1] * s)                      # point.py:121-127


def v2_norm(a: V2) -> V2:
    return v2_scale(a, 1 / v2_len(a))                 # point.py:37-41


def v2_change_length(a: V2, n: float) -> V2:
    return v2_scale(v2_norm(a), float(n))             # point.py:43-47


def v2_add(a: V2, b: V2) -> V2:
    return (a[0] + b[0], a[1] + b[1])


def v2_sub(a: V2, b: V2) -> V2:
    return (a[0] + (-b[0]), a[1] + (-b[1]))           # point.py:67-71 (add of negation)


def v2_dot(a: V2, b: V2) -> float:
    return a[0] * b[0] + a[1] * b[1]


def v2_rotate(a: V2, phi: float) -> V2:
    """point.py:89-112: rotation-matrix product."""
    c, s = math.cos(phi), math.sin(phi)
    return (c * a[0] + (-s) * a[1], s * a[0] + c * a[1])


def v2_angle_to_x_axis(a: V2) -> float:
    """point.py:114-119."""
    t = float(math.atan2(a[1], a[0]))
    return t if t >= 0 else math.pi * 2 + t


def v2_eq(a: V2, b: V2, err: float = 1e-6) -> bool:
    return abs(a[0] - b[0]) <= err and abs(a[1] - b[1]) <= err   # point.py:179-190


def v3_len(a: V3) -> float:
    return math.sqrt(a[0] ** 2 + a[1] ** 2 + a[2] ** 2)           # point.py:329-333


def v3_scale(a: V3, s: float) -> V3:
    return (a[0] * s, a[1] * s, a[2] * s)


def v3_norm(a: V3) -> V3:
    return v3_scale(a, 1 / v3_len(a))


def v3_change_length(a: V3, n: float) -> V3:
    return v3_scale(v3_norm(a), n)                    # point.py:341-345


def v3_add(a: V3, b: V3) -> V3:
    return (a[0] + b[0], a[1] + b[1], a[2] + b[2])


def v3_sub(a: V3, b: V3) -> V3:
    return (a[0] + (-b[0]), a[1] + (-b[1]), a[2] + (-b[2]))     # point.py:359-363


def v3_dot(a: V3, b: V3) -> float:
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def v3_cross(a: V3, b: V3) -> V3:
    """point.py:402-410: ``(ay*bz - az*by, -ax*bz + az*bx, ax*by - ay*bx)``."""
    return (a[1] * b[2] - a[2] * b[1], -a[0] * b[2] + a[2] * b[0], a[0] * b[1] - a[1] * b[0])


# ---------------------------------------------------------------- local frames
class Frame:
    """LocalCoordinateSystem, final_code/packages/local_coordinate_system.py:32-125."""

    def __init__(self, location: V3, x_direction: V3, z_direction: V3):
        self.location = tuple(location)
        self.ZI = v3_norm(z_direction)
        self.XI = v3_norm(x_direction)
        self.YI = v3_cross(self.ZI, self.XI)

    @staticmethod
    def from_y_z(location: V3, y_direction: V3, z_direction: V3) -> "Frame":
        """local_coordinate_system.py:152-177."""
        return Frame(location, v3_cross(y_direction, z_direction), z_direction)

    @staticmethod
    def from_axes(location, XI, YI, ZI) -> "Frame":
        f = Frame.__new__(Frame)
        f.location, f.XI, f.YI, f.ZI = tuple(location), tuple(XI), tuple(YI), tuple(ZI)
        return f

    def point_to_local(self, p: V3) -> V3:           # :60-74
        d = v3_sub(p, self.location)
        return (v3_dot(self.XI, d), v3_dot(self.YI, d), v3_dot(self.ZI, d))

    def point_to_global(self, p: V3) -> V3:          # :76-92
        return v3_add(self.location, v3_add(v3_add(v3_scale(self.XI, p[0]), v3_scale(self.YI, p[1])),
                                            v3_scale(self.ZI, p[2])))

    def vector_to_global(self, v: V3) -> V3:         # :109-125
        return v3_add(v3_add(v3_scale(self.XI, v[0]), v3_scale(self.YI, v[1])), v3_scale(self.ZI, v[2]))

    def as_array(self) -> numpy.ndarray:
        return numpy.array([self.location, self.XI, self.YI, self.ZI], dtype=numpy.float64)


# ---------------------------------------------------------------- design orbit (line2s.py, trajectory.py)
class Straight:
    """StraightLine2, final_code/packages/line2s.py:257-283."""

    def __init__(self, length: float, direct: V2, start: V2):
        self.length = float(length)
        self.direct = v2_norm(direct)
        self.start = start

    def point_at(self, s: float) -> V2:
        return v2_add(self.start, v2_change_length(self.direct, s))

    def direct_at(self, s: float) -> V2:
        return self.direct

    def position_of(self, p: V2) -> int:
        """line2s.py:291-328: 1 right, -1 left, 0 on the line."""
        d = self.direct
        p0p = v2_sub(p, self.start)
        k = v2_dot(d, p0p)
        vert = v2_sub(p0p, v2_scale(d, k))
        if v2_eq(vert, (0.0, 0.0)):
            return 0
        vert = v2_norm(vert)
        right = v2_norm(v2_rotate(d, deg2rad(-90)))
        return 1 if v2_eq(vert, right) else -1


class Arc:
    """ArcLine2, line2s.py:461-565."""

    def __init__(self, start: V2, start_direct: V2, radius: float, clockwise: bool, total_deg: float):
        self.center = v2_add(start, v2_change_length(
            v2_rotate(start_direct, -math.pi / 2 if clockwise else math.pi / 2), radius))
        self.starting_phi = v2_angle_to_x_axis(v2_sub(start, self.center))
        self.radius = radius
        self.total_phi = deg2rad(total_deg)
        self.clockwise = clockwise
        self.length = radius * self.total_phi

    def _phi(self, s: float) -> float:
        phi = s / self.radius
        return self.starting_phi - phi if self.clockwise else self.starting_phi + phi

    def point_at(self, s: float) -> V2:
        c = self._phi(s)
        return v2_add(v2_change_length((math.cos(c), math.sin(c)), self.radius), self.center)

    def direct_at(self, s: float) -> V2:
        c = self._phi(s)
        return v2_rotate((math.cos(c), math.sin(c)), -math.pi / 2 if self.clockwise else math.pi / 2)


class Orbit:
    """Trajectory, final_code/packages/trajectory.py:30-160 (lines and arcs)."""

    def __init__(self, start: V2, direct: V2, length: float):
        self.lines = [Straight(length, direct, start)]
        self.length = self.lines[0].length

    def _end(self):
        last = self.lines[-1]
        return last.point_at(last.length), last.direct_at(last.length)

    def add_straight(self, length: float) -> "Orbit":
        sp, sd = self._end()
        self.lines.append(Straight(length, sd, sp))
        self.length += length
        return self

    def add_arc(self, radius: float, clockwise: bool, angle_deg: float) -> "Orbit":
        sp, sd = self._end()
        a = Arc(sp, sd, radius, clockwise, angle_deg)
        self.lines.append(a)
        self.length += a.length
        return self

    def _locate(self, s: float):
        for ln in self.lines:
            if s <= ln.length:
                return ln, s
            s -= ln.length
        return self.lines[-1], self.lines[-1].length if abs(s) <= 1e-8 else s + self.lines[-1].length

    def point_at(self, s: float) -> V2:
        ln, t = self._locate(s)
        return ln.point_at(t)

    def direct_at(self, s: float) -> V2:
        ln, t = self._locate(s)
        return ln.direct_at(t)


def circle_center_and_radius(p1: V2, p2: V2, p3: V2) -> Tuple[V2, float]:
    """base_utils.py:124-151: least-squares centre through three points."""
    x1, y1 = p1
    x2, y2 = p2
    x3, y3 = p3
    z1 = x2 ** 2 + y2 ** 2 - x1 ** 2 - y1 ** 2
    z2 = x3 ** 2 + y3 ** 2 - x1 ** 2 - y1 ** 2
    z3 = x3 ** 2 + y3 ** 2 - x2 ** 2 - y2 ** 2
    A = numpy.array([[(x2 - x1), (y2 - y1)], [(x3 - x1), (y3 - y1)], [(x3 - x2), (y3 - y2)]])
    B = 0.5 * numpy.array([[z1], [z2], [z3]])
    c = numpy.linalg.inv(A.T @ A) @ A.T @ B
    cx, cy = float(c[0, 0]), float(c[1, 0])
    r1 = math.sqrt((cx - x1) ** 2 + (cy - y1) ** 2)
    r2 = math.sqrt((cx - x2) ** 2 + (cy - y2) ** 2)
    r3 = math.sqrt((cx - x3) ** 2 + (cy - y3) ** 2)
    return (cx, cy), (r1 + r2 + r3) / 3


# ---------------------------------------------------------------- magnets
def cct_record(frame: Frame, big_r, small_r, bending_angle, tilt_angles, winding_number, current,
               start_ksi_phi: V2, end_ksi_phi: V2, disperse_number_per_winding: int) -> Dict:
    """Parameter record of one CCT layer (the constructor arguments of cct.py:36-57)."""
    return dict(kind="cct", frame=frame, big_r=float(big_r), small_r=float(small_r),
                bending_angle=float(bending_angle), tilt_angles=[float(t) for t in tilt_angles],
                winding_number=int(winding_number), current=float(current),
                start=(float(start_ksi_phi[0]), float(start_ksi_phi[1])),
                end=(float(end_ksi_phi[0]), float(end_ksi_phi[1])),
                dpw=int(disperse_number_per_winding))


def qs_record(frame: Frame, length, gradient, second_gradient, aperture_radius) -> Dict:
    """Parameter record of one QS magnet (magnets.py:614-628)."""
    return dict(kind="qs", frame=frame, length=float(length), gradient=float(gradient),
                second_gradient=float(second_gradient), aperture_radius=float(aperture_radius))


def cct_path_local(c: Dict) -> numpy.ndarray:
    """Winding path points in the CCT's local frame, shape (W*n+1, 3).

    cct.py:87-145 (constants a, eta; linspace over xi), phi_ksi_function
    cct.py:166-188, BipolarToroidalCoordinateSystem.convert cct.py:213-224.
    """
    big_r, small_r = c["big_r"], c["small_r"]
    a = math.sqrt(big_r ** 2 - small_r ** 2)
    eta = 0.5 * math.log((big_r + a) / (big_r - a))
    tilt_rad = [deg2rad(t) for t in c["tilt_angles"]]
    x1, y1 = c["start"]
    x2, y2 = c["end"]
    k = (y2 - y1) / (x2 - x1)
    b = -k * x1 + y1
    terms = []
    for i, t in enumerate(c["tilt_angles"]):
        if approx_equal(t, 90.0):
            continue
        terms.append((i, (1 / math.tan(tilt_rad[i])) / ((i + 1) * math.sinh(eta))))
    ch, sh = math.cosh(eta), math.sinh(eta)
    n = c["winding_number"] * c["dpw"]
    out = numpy.empty((n + 1, 3))
    for j, ksi in enumerate(linspace(x1, x2, n + 1)):
        phi = k * ksi + b
        for i, coef in terms:
            phi += coef * math.sin((i + 1) * ksi)
        temp = a / (ch - math.cos(ksi))
        out[j, 0] = temp * sh * math.cos(phi)
        out[j, 1] = temp * sh * math.sin(phi)
        out[j, 2] = temp * math.sin(ksi)
    return out


def cct_segments_local(c: Dict) -> Tuple[numpy.ndarray, numpy.ndarray]:
    """(kl, p0) in the local frame: cct.py:157-164."""
    path = cct_path_local(c)
    kl = 1e-7 * c["current"] * (path[1:] - path[:-1])
    p0 = 0.5 * (path[1:] + path[:-1])
    return kl, p0


def cct_segments_global(c: Dict) -> Tuple[numpy.ndarray, numpy.ndarray]:
    """(kl, p0) in the global frame, shape (N, 3) each: cct.py:423-457."""
    path = cct_path_local(c)
    f = c["frame"]
    g = numpy.array([f.point_to_global((p[0], p[1], p[2])) for p in path], dtype=numpy.float64)
    kl = 1e-7 * c["current"] * (g[1:] - g[:-1])
    p0 = 0.5 * (g[1:] + g[:-1])
    return kl, p0


def segments_field_local(kl: numpy.ndarray, p0: numpy.ndarray, p: V3) -> V3:
    """Midpoint Biot-Savart sum at a local-frame point: cct.py:257-276."""
    r = numpy.array(p) - p0
    rr = (numpy.linalg.norm(r, ord=2, axis=1) ** (-3)).reshape((r.shape[0], 1))
    dB = numpy.cross(kl, r) * rr
    B = numpy.sum(dB, axis=0)
    return (float(B[0]), float(B[1]), float(B[2]))


class CCTOracle:
    """CCT field evaluator: cct.py:249-285 (local frame, rotated back to global)."""

    def __init__(self, rec: Dict):
        self.rec = rec
        self.frame = rec["frame"]
        self.kl, self.p0 = cct_segments_local(rec)

    def field_at(self, point: V3) -> V3:
        if approx_equal(self.rec["current"], 0, err=1e-6):
            return (0.0, 0.0, 0.0)
        B = segments_field_local(self.kl, self.p0, self.frame.point_to_local(point))
        return self.frame.vector_to_global(B)


class QSOracle:
    """Hard-edge quadrupole + sextupole: magnets.py:637-668."""

    def __init__(self, rec: Dict):
        self.rec = rec
        self.frame = rec["frame"]

    def field_at(self, point: V3) -> V3:
        x, y, z = self.frame.point_to_local(point)
        r = self.rec
        if z < 0 or z > r["length"]:
            return (0.0, 0.0, 0.0)
        a = r["aperture_radius"]
        if abs(x) > a or abs(y) > a or math.sqrt(x ** 2 + y ** 2) > a:
            return (0.0, 0.0, 0.0)
        g, s = r["gradient"], r["second_gradient"]
        bx = g * y + s * (x * y)
        by = g * x + 0.5 * s * (x ** 2 - y ** 2)
        return v3_add(v3_scale(self.frame.XI, bx), v3_scale(self.frame.YI, by))

    def to_array(self) -> numpy.ndarray:
        """magnets.py:726-748: origin, XI, YI, ZI, length, g, s, aperture."""
        f, r = self.frame, self.rec
        return numpy.array(list(f.location) + list(f.XI) + list(f.YI) + list(f.ZI)
                           + [r["length"], r["gradient"], r["second_gradient"], r["aperture_radius"]])


class LocalUniformOracle:
    """LocalUniformMagnet.magnetic_field_at, magnets.py:469-481: YI * B inside the cylinder."""

    def __init__(self, frame: Frame, length: float, aperture_radius: float, field: float):
        self.frame, self.length, self.a, self.b = frame, length, aperture_radius, field
        self.vector = v3_scale(frame.YI, field)

    def field_at(self, point: V3) -> V3:
        x, y, z = self.frame.point_to_local(point)
        if z < 0 or z > self.length:
            return (0.0, 0.0, 0.0)
        if abs(x) > self.a or abs(y) > self.a or math.sqrt(x ** 2 + y ** 2) > self.a:
            return (0.0, 0.0, 0.0)
        return self.vector


class SegmentsOracle:
    """Current elements (kl, p0): a Wire in the global frame (cct.py:668-698) or an
    AGCCT_CONNECTOR in its frame, rotated back to global (cct.py:962-994)."""

    def __init__(self, kl: numpy.ndarray, p0: numpy.ndarray, current: float, frame: Frame = None):
        self.kl, self.p0, self.current, self.frame = kl, p0, current, frame

    def field_at(self, point: V3) -> V3:
        if approx_equal(self.current, 0, err=1e-6):
            return (0.0, 0.0, 0.0)
        if self.frame is None:
            return segments_field_local(self.kl, self.p0, point)
        return self.frame.vector_to_global(segments_field_local(self.kl, self.p0, self.frame.point_to_local(point)))


class BeamlineOracle:
    """Magnet list with Beamline.magnetic_field_at (beamline.py:46-53)."""

    def __init__(self, records: Sequence[Dict]):
        self.magnets = [CCTOracle(r) if r["kind"] == "cct" else QSOracle(r) for r in records]

    def field_at(self, point: V3) -> V3:
        b = (0.0, 0.0, 0.0)
        for m in self.magnets:
            b = v3_add(b, m.field_at(point))
        return b

    def field_at_points(self, pts: numpy.ndarray) -> numpy.ndarray:
        return numpy.array([self.field_at((float(p[0]), float(p[1]), float(p[2]))) for p in pts])


def wire_path_field(path: numpy.ndarray, current: float, p: V3) -> V3:
    """Field of a polyline wire with the midpoint rule, ``x 1e-7`` applied last
    (codes/cctpy/cct.py:25-57, the SoleLayerCct form used by the known-answer tests)."""
    kl = current * (path[1:] - path[:-1])
    p0 = 0.5 * (path[1:] + path[:-1])
    B = segments_field_local(kl, p0, p)
    return (B[0] * 1e-7, B[1] * 1e-7, B[2] * 1e-7)


# ---------------------------------------------------------------- placement (cct.py, magnets.py, beamline.py)
def cct_along(orbit: Orbit, s, big_r, small_r, bending_angle, tilt_angles, winding_number, current,
              start_ksi_phi: V2, end_ksi_phi: V2, dpw: int) -> Dict:
    """CCT.create_cct_along, cct.py:341-421."""
    sp = orbit.point_at(s)
    arc_length = big_r * deg2rad(bending_angle)
    ep = orbit.point_at(s + arc_length)
    m0 = orbit.point_at(s + arc_length / 3 * 1)
    m1 = orbit.point_at(s + arc_length / 3 * 2)
    c1, _ = circle_center_and_radius(sp, m0, m1)
    c2, _ = circle_center_and_radius(m0, m1, ep)
    center = v2_scale(v2_add(c1, c2), 0.5)
    sd = orbit.direct_at(s)
    pos = Straight(1.0, sd, sp).position_of(center)
    if pos == 0:
        raise ValueError("centre on the design orbit")
    # pos == 1: centre on the right of the start direction (clockwise), y = -start direction
    ydir = (-sd[0], -sd[1], -0.0) if pos == 1 else (sd[0], sd[1], 0.0)
    frame = Frame.from_y_z((center[0], center[1], 0.0), ydir, (0.0, 0.0, 1.0))
    return cct_record(frame, big_r, small_r, bending_angle, tilt_angles, winding_number, current,
                      start_ksi_phi, end_ksi_phi, dpw)


def qs_along(orbit: Orbit, s, length, gradient, second_gradient, aperture_radius) -> Dict:
    """QS.create_qs_along, magnets.py:683-724."""
    o = orbit.point_at(s)
    zd = orbit.direct_at(s)
    xd = v2_rotate(zd, deg2rad(90))
    frame = Frame((o[0], o[1], 0.0), (xd[0], xd[1], 0.0), (zd[0], zd[1], 0.0))
    return qs_record(frame, length, gradient, second_gradient, aperture_radius)


class LineBuilder:
    """Beamline assembly: beamline.py:379-574 (drift, QS, dipole CCT) and :576-793 (AG-CCT)."""

    def __init__(self, start: V2, direct: V2, first_drift: float):
        self.orbit = Orbit(start, direct, first_drift)
        self.records: List[Dict] = []

    def drift(self, length):
        self.orbit.add_straight(length)
        return self

    def qs(self, length, gradient, second_gradient, aperture_radius):
        old = self.orbit.length
        self.orbit.add_straight(length)
        self.records.append(qs_along(self.orbit, old, length, gradient, second_gradient, aperture_radius))
        return self

    def dipole_cct(self, big_r, small_r_inner, small_r_outer, bending_angle, tilt_angles,
                   winding_number, current, dpw=120):
        """beamline.py:507-574."""
        old = self.orbit.length
        self.orbit.add_arc(big_r, bending_angle < 0, abs(bending_angle))
        end_phi = deg2rad(bending_angle)
        self.records.append(cct_along(self.orbit, old, big_r, small_r_inner, abs(bending_angle), tilt_angles,
                                      winding_number, current, (0.0, 0.0),
                                      (2 * math.pi * winding_number, end_phi), dpw))
        self.records.append(cct_along(self.orbit, old, big_r, small_r_outer, abs(bending_angle),
                                      [t * -1 for t in tilt_angles], winding_number, current, (0.0, 0.0),
                                      (-2 * math.pi * winding_number, end_phi), dpw))
        return self

    def agcct(self, big_r, small_rs, bending_angles, tilt_angles, winding_numbers, currents, dpw=120):
        """beamline.py:576-793: outer dipole, inner dipole, then inner/outer AG layers per part."""
        total = sum(bending_angles)
        old = self.orbit.length
        self.orbit.add_arc(big_r, total < 0, abs(total))
        tot_rad = deg2rad(total)
        wd = winding_numbers[0][0]
        self.records.append(cct_along(self.orbit, old, big_r, small_rs[0], abs(total),
                                      [t * -1 for t in tilt_angles[0]], wd, currents[0], (0.0, 0.0),
                                      (-2 * math.pi * wd, tot_rad), dpw))
        self.records.append(cct_along(self.orbit, old, big_r, small_rs[1], abs(total), tilt_angles[0], wd,
                                      currents[0], (0.0, 0.0), (2 * math.pi * wd, tot_rad), dpw))
        wn = winding_numbers[1]
        ang_rad = [deg2rad(a) for a in bending_angles]
        ag_tilt = tilt_angles[1]
        cur = currents[1]
        start_in = (0.0, 0.0)
        start_out = (0.0, 0.0)
        end_in = (((-1.0) ** 0) * 2 * math.pi * wn[0], ang_rad[0])
        end_out = (((-1.0) ** 1) * 2 * math.pi * wn[0], ang_rad[0])
        self.records.append(cct_along(self.orbit, old, big_r, small_rs[3], abs(bending_angles[0]),
                                      [t * -1 for t in ag_tilt], wn[0], cur, start_in, end_in, dpw))
        self.records.append(cct_along(self.orbit, old, big_r, small_rs[2], abs(bending_angles[0]),
                                      ag_tilt, wn[0], cur, start_out, end_out, dpw))
        for idx in range(1, len(bending_angles)):
            step = ang_rad[idx - 1] / wn[idx - 1]
            start_in = v2_add(end_in, (0, step))
            start_out = v2_add(end_out, (0, step))
            end_in = v2_add(start_in, (((-1) ** idx) * 2 * math.pi * wn[idx], ang_rad[idx]))
            end_out = v2_add(start_out, (((-1) ** (idx + 1)) * 2 * math.pi * wn[idx], ang_rad[idx]))
            self.records.append(cct_along(self.orbit, old, big_r, small_rs[3], abs(bending_angles[idx]),
                                          [t * -1 for t in ag_tilt], wn[idx], cur, start_in, end_in, dpw))
            self.records.append(cct_along(self.orbit, old, big_r, small_rs[2], abs(bending_angles[idx]),
                                          ag_tilt, wn[idx], cur, start_out, end_out, dpw))
        return self


# ---------------------------------------------------------------- particles (particles.py)
def proton(position: V3, direct: V3, kinetic_mev: float) -> numpy.ndarray:
    """ParticleFactory.create_proton, particles.py:1325-1352; 10-float record :443-457."""
    speed = LIGHT_SPEED * math.sqrt(
        1.0 - (PROTON_STATIC_ENERGY_MEV / (PROTON_STATIC_ENERGY_MEV + kinetic_mev)) ** 2)
    rm = PROTON_STATIC_MASS_KG / math.sqrt(1.0 - (speed ** 2) / (LIGHT_SPEED ** 2))
    v = v3_change_length(direct, speed)
    return numpy.array(list(position) + list(v) + [rm, PROTON_CHARGE, speed, 0.0])


def proton_along(orbit: Orbit, s: float, kinetic_mev: float) -> numpy.ndarray:
    """particles.py:1378-1395."""
    p = orbit.point_at(s)
    d = orbit.direct_at(s)
    return proton((p[0], p[1], 0.0), (d[0], d[1], 0.0), kinetic_mev)


def natural_frame(ideal: numpy.ndarray) -> Frame:
    """RunningParticle.get_natural_coordinate_system, particles.py:405-416 (y = global z)."""
    return Frame.from_y_z(tuple(ideal[0:3]), (0.0, 0.0, 1.0), tuple(ideal[3:6]))


def from_phase_space(ideal: numpy.ndarray, frame: Frame, ps: Sequence[float]) -> numpy.ndarray:
    """ParticleFactory.create_from_phase_space_particle, particles.py:1398-1438."""
    x, xp, y, yp, z, delta = [float(t) for t in ps]
    pos = tuple(ideal[0:3])
    vel = tuple(ideal[3:6])
    rm, e, speed, dist = float(ideal[6]), float(ideal[7]), float(ideal[8]), float(ideal[9])
    pos = v3_add(pos, v3_scale(frame.XI, x))
    pos = v3_add(pos, v3_scale(frame.YI, y))
    pos = v3_add(pos, v3_scale(frame.ZI, z))
    if delta != 0.0:
        # RunningParticle.change_scalar_momentum, particles.py:375-403
        pm = speed * rm * (1.0 + delta)
        m0 = rm * math.sqrt(1 - (speed ** 2) / (LIGHT_SPEED ** 2))
        new_speed = pm / math.sqrt(m0 ** 2 + (pm / LIGHT_SPEED) ** 2)
        rm = m0 / math.sqrt(1 - (new_speed / LIGHT_SPEED) ** 2)
        speed = new_speed
        vel = v3_change_length(vel, new_speed)
    vel = v3_add(vel, v3_scale(frame.XI, xp * speed))
    vel = v3_add(vel, v3_scale(frame.YI, yp * speed))
    vel = v3_change_length(vel, speed)
    return numpy.array(list(pos) + list(vel) + [rm, e, speed, dist])


def to_phase_space(ideal: numpy.ndarray, frame: Frame, p: numpy.ndarray) -> Tuple[float, ...]:
    """PhaseSpaceParticle.create_from_running_particle, particles.py:1078-1121."""
    rel_p = v3_sub(tuple(p[0:3]), tuple(ideal[0:3]))
    x, y, z = v3_dot(frame.XI, rel_p), v3_dot(frame.YI, rel_p), v3_dot(frame.ZI, rel_p)
    rel_v = v3_sub(tuple(p[3:6]), tuple(ideal[3:6]))
    sp = float(p[8])
    xv, yv = v3_dot(frame.XI, rel_v), v3_dot(frame.YI, rel_v)
    xp = xv / math.sqrt(sp ** 2 - xv ** 2)
    yp = yv / math.sqrt(sp ** 2 - yv ** 2)
    rmom = sp * float(p[6])
    imom = float(ideal[8]) * float(ideal[6])
    return (x, xp, y, yp, z, (rmom - imom) / imom)


# ---------------------------------------------------------------- optimiser read-out
A05_OBJECTIVES = ("width_max_x", "width_max_xp", "width_max_y", "width_max_yp", "center_x", "center_xp",
                  "center_y", "center_yp", "diff_xy", "fluct_x", "fluct_y")


def beam_objectives(ideal: numpy.ndarray, frame: Frame, finals: numpy.ndarray, group: int = 12,
                    speed_from_velocity: bool = True) -> Tuple[List[float], List[Tuple[float, ...]]]:
    """The eleven objectives of one gantry design in the reference's optimiser run script
    (final_code/work/optim/A05run.py:247-330): speeds reset to |v| (:265-267,
    P3.length, point.py:327-331), phase space at the exit (to_phase_space), then with the
    semantics of BaseUtils.Statistic (base_utils.py:603-683; average = sum / len in list
    order, width = max - min, half_width = width / 2): the largest |x|, |x'|, |y|, |y'| (mm,
    mrad), |mean| of each, |max|x| - max|y||, and the spread (width) of the half widths in
    x and in y of consecutive groups of `group` particles."""
    rows = []
    for p in finals:
        q = numpy.array(p, dtype=numpy.float64)
        if speed_from_velocity:
            q[8] = math.sqrt(q[3] ** 2 + q[4] ** 2 + q[5] ** 2)
        rows.append(to_phase_space(ideal, frame, q))
    xs = [r[0] / MM for r in rows]
    xps = [r[1] / MRAD for r in rows]
    ys = [r[2] / MM for r in rows]
    yps = [r[3] / MRAD for r in rows]

    def average(v):
        # Statistic.average is sum(data) / len(data) over Python floats (P3 stores floats,
        # point.py:322-325): on CPython >= 3.12 the builtin sum of floats is Neumaier's
        # compensated sum, which the GPU read-out restates
        return sum(float(t) for t in v) / len(v)

    def absolute_max(v):
        return max(abs(t) for t in v)

    hx, hy = [], []
    for g in range(0, len(rows), group):
        gx, gy = xs[g:g + group], ys[g:g + group]
        hx.append((max(gx) - min(gx)) / 2)
        hy.append((max(gy) - min(gy)) / 2)
    wx, wxp, wy, wyp = absolute_max(xs), absolute_max(xps), absolute_max(ys), absolute_max(yps)
    obj = [wx, wxp, wy, wyp, abs(average(xs)), abs(average(xps)), abs(average(ys)), abs(average(yps)),
           abs(wx - wy), max(hx) - min(hx), max(hy) - min(hy)]
    return obj, rows


# ---------------------------------------------------------------- RK4 push (base_utils.py, particles.py)
def rk4_track(particle: numpy.ndarray, field: Callable[[V3], V3], length: float, footstep: float) -> numpy.ndarray:
    """ParticleRunner.run_only for one particle (particles.py:562-596) with the RK4
    of BaseUtils.runge_kutta4 (base_utils.py:264-311) and the callback
    ``Y' = [v, (e/rm) v x B(p)]`` of particles.py:515-537."""
    p = numpy.array(particle, dtype=numpy.float64)
    speed = float(p[8])
    k = float(p[7]) / float(p[6])
    dt = footstep / speed
    t_end = length / speed
    t0 = 0.0
    number = math.ceil((t_end - t0) / dt)
    dt = (t_end - t0) / float(number)

    def f(Y):
        pos = (Y[0, 0], Y[0, 1], Y[0, 2])
        vel = (Y[1, 0], Y[1, 1], Y[1, 2])
        B = field((float(pos[0]), float(pos[1]), float(pos[2])))
        a = v3_cross(vel, B)
        return numpy.array([vel, (a[0] * k, a[1] * k, a[2] * k)])

    Y0 = numpy.array([p[0:3], p[3:6]])
    for _ in range(number):
        k1 = f(Y0)
        k2 = f(Y0 + dt / 2 * k1)
        k3 = f(Y0 + dt / 2 * k2)
        k4 = f(Y0 + dt * k3)
        t0 += dt
        Y0 = Y0 + (dt / 6) * (k1 + 2 * k2 + 2 * k3 + k4)
    out = p.copy()
    out[0:3] = Y0[0]
    out[3:6] = Y0[1]
    out[9] = p[9] + length
    return out


def rk4_steps(length: float, footstep: float, speed: float) -> Tuple[int, float]:
    """Step count and time step of base_utils.py:284-285 as driven by particles.py:586-588."""
    dt = footstep / speed
    t_end = length / speed
    number = math.ceil(t_end / dt)
    return number, t_end / float(number)


def _track_worker(args):
    records, particle, length, footstep = args
    bl = BeamlineOracle(records)
    return rk4_track(particle, bl.field_at, length, footstep)


def track_many(records: Sequence[Dict], particles: numpy.ndarray, length: float, footstep: float,
               processes: int = 1) -> numpy.ndarray:
    """ParticleRunner.run_only over a particle list (particles.py:598-632); with
    ``processes > 1`` a spawn-started process pool plays the role of
    BaseUtils.submit_process_task (base_utils.py:370-444)."""
    work = [(list(records), numpy.array(p), length, footstep) for p in particles]
    if processes <= 1:
        return numpy.array([_track_worker(w) for w in work])
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(processes) as pool:
        return numpy.array(pool.map(_track_worker, work))


def _field_worker(args):
    records, pts = args
    return BeamlineOracle(records).field_at_points(pts)


def field_many(records: Sequence[Dict], pts: numpy.ndarray, processes: int = 1) -> numpy.ndarray:
    """Beamline field at many points, optionally over a spawn-started process pool."""
    if processes <= 1:
        return _field_worker((list(records), pts))
    import multiprocessing as mp
    chunks = numpy.array_split(pts, processes * 4)
    ctx = mp.get_context("spawn")
    with ctx.Pool(processes) as pool:
        parts = pool.map(_field_worker, [(list(records), c) for c in chunks if len(c)])
    return numpy.concatenate(parts)


# ---------------------------------------------------------------- persistent worker pool (timed CPU baselines)
_POOL_LINE = None


def _pool_init(records):
    global _POOL_LINE
    _POOL_LINE = BeamlineOracle(records)


def _pool_field(pts):
    return _POOL_LINE.field_at_points(pts)


def _pool_track(args):
    particle, length, footstep = args
    return rk4_track(particle, _POOL_LINE.field_at, length, footstep)


class OraclePool:
    """A spawn-started process pool whose workers each build the beamline once, at start-up,
    and then evaluate fields or track particles on request -- BaseUtils.submit_process_task
    (base_utils.py:370-444) kept alive between calls, so that a timed CPU baseline measures
    the field sums and not pool start-up or segment generation."""

    def __init__(self, records: Sequence[Dict], processes: int):
        import multiprocessing as mp
        self.processes = max(1, int(processes))
        self._pool = mp.get_context("spawn").Pool(self.processes, initializer=_pool_init,
                                                  initargs=(list(records),))

    def field(self, pts: numpy.ndarray) -> numpy.ndarray:
        chunks = [c for c in numpy.array_split(pts, self.processes * 4) if len(c)]
        return numpy.concatenate(self._pool.map(_pool_field, chunks))

    def track(self, particles: numpy.ndarray, length: float, footstep: float) -> numpy.ndarray:
        return numpy.array(self._pool.map(_pool_track, [(numpy.array(p), length, footstep) for p in particles],
                                          chunksize=1))

    def close(self) -> None:
        self._pool.close()
        self._pool.join()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
