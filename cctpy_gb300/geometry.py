"""2-D / 3-D vectors, local frames and design orbits (lines and arcs).

Same names and meaning as cctpy's final_code/packages/point.py (P2, P3),
local_coordinate_system.py (LocalCoordinateSystem), line2s.py
(StraightLine2, ArcLine2) and trajectory.py (Trajectory), written for this
package.  Points are plain Python floats; the frame also offers vectorised
numpy transforms for segment sets.
"""
from __future__ import annotations

import math
from typing import Callable, List, Optional, Tuple, Union

import numpy as np

MM = 0.001
M = 1.0
LIGHT_SPEED = 299792458.0
MRAD = 1.0 * MM


class P2:
    """2-D point / vector (cctpy point.py:22-250)."""

    __slots__ = ("x", "y")

    def __init__(self, x: float = 0.0, y: float = 0.0):
        self.x = float(x)
        self.y = float(y)

    def length(self) -> float:
        return math.sqrt(self.x ** 2 + self.y ** 2)

    def normalize(self) -> "P2":
        return self * (1 / self.length())

    def change_length(self, new_length: float) -> "P2":
        return self.normalize() * float(new_length)

    def copy(self) -> "P2":
        return P2(self.x, self.y)

    def __add__(self, o: "P2") -> "P2":
        return P2(self.x + o.x, self.y + o.y)

    def __neg__(self) -> "P2":
        return P2(-self.x, -self.y)

    def __sub__(self, o: "P2") -> "P2":
        return P2(self.x + (-o.x), self.y + (-o.y))

    def __mul__(self, o):
        if isinstance(o, P2):
            return self.x * o.x + self.y * o.y
        return P2(self.x * o, self.y * o)

    __rmul__ = __mul__

    def __truediv__(self, n: float) -> "P2":
        if n == 0:
            raise ValueError(f"{self}/{n}: division by zero")
        return self * (1 / n)

    def rotate(self, phi: float) -> "P2":
        c, s = math.cos(phi), math.sin(phi)
        return P2(c * self.x + (-s) * self.y, s * self.x + c * self.y)

    def angle_to_x_axis(self) -> float:
        a = float(math.atan2(self.y, self.x))
        return a if a >= 0 else math.pi * 2 + a

    def to_p3(self, transformation=None) -> "P3":
        return transformation(self) if transformation else P3(self.x, self.y, 0.0)

    def to_list(self) -> List[float]:
        return [self.x, self.y]

    def __eq__(self, o: "P2", err: float = 1e-6, msg: Optional[str] = None) -> bool:
        ok = abs(self.x - o.x) <= err and abs(self.y - o.y) <= err
        if not ok and msg is not None:
            raise AssertionError(msg)
        return ok

    __hash__ = None

    def __repr__(self) -> str:
        return f"({self.x}, {self.y})"

    @staticmethod
    def origin() -> "P2":
        return P2()

    zeros = origin

    @staticmethod
    def x_direct(x: float = 1.0) -> "P2":
        return P2(x, 0.0)

    @staticmethod
    def y_direct(y: float = 1.0) -> "P2":
        return P2(0.0, y)


class P3:
    """3-D point / vector (cctpy point.py:318-540); ``@`` is the cross product."""

    __slots__ = ("x", "y", "z")

    def __init__(self, x: float = 0.0, y: float = 0.0, z: float = 0.0):
        self.x = float(x)
        self.y = float(y)
        self.z = float(z)

    def length(self) -> float:
        return math.sqrt(self.x ** 2 + self.y ** 2 + self.z ** 2)

    def normalize(self) -> "P3":
        return self * (1 / self.length())

    def change_length(self, new_length: float) -> "P3":
        return self.normalize() * new_length

    def copy(self) -> "P3":
        return P3(self.x, self.y, self.z)

    def __add__(self, o: "P3") -> "P3":
        return P3(self.x + o.x, self.y + o.y, self.z + o.z)

    def __neg__(self) -> "P3":
        return P3(-self.x, -self.y, -self.z)

    def __sub__(self, o: "P3") -> "P3":
        return P3(self.x + (-o.x), self.y + (-o.y), self.z + (-o.z))

    def __iadd__(self, o: "P3") -> "P3":
        self.x += o.x
        self.y += o.y
        self.z += o.z
        return self

    def __isub__(self, o: "P3") -> "P3":
        self.x -= o.x
        self.y -= o.y
        self.z -= o.z
        return self

    def __mul__(self, o):
        if isinstance(o, P3):
            return self.x * o.x + self.y * o.y + self.z * o.z
        if isinstance(o, (int, float)):
            return P3(self.x * o, self.y * o, self.z * o)
        raise ValueError(f"{self} * {o}: unsupported operand")

    __rmul__ = __mul__

    def __truediv__(self, n: float) -> "P3":
        if n == 0:
            raise ValueError(f"{self}/{n}: division by zero")
        return self * (1 / n)

    def __matmul__(self, o: "P3") -> "P3":
        return P3(self.y * o.z - self.z * o.y, -self.x * o.z + self.z * o.x, self.x * o.y - self.y * o.x)

    def __eq__(self, o: "P3", err: float = 1e-6, msg: Optional[str] = None) -> bool:
        if not isinstance(o, P3):
            raise ValueError(f"{o} is not a P3")
        ok = abs(self.x - o.x) <= err and abs(self.y - o.y) <= err and abs(self.z - o.z) <= err
        if not ok and msg is not None:
            raise AssertionError(msg)
        return ok

    __hash__ = None

    def __repr__(self) -> str:
        return f"({self.x}, {self.y}, {self.z})"

    def to_list(self) -> List[float]:
        return [self.x, self.y, self.z]

    def to_p2(self, transformation=None) -> P2:
        return transformation(self) if transformation else P2(self.x, self.y)

    def to_numpy_ndarry3(self, numpy_dtype=np.float64) -> np.ndarray:
        return np.array(self.to_list(), dtype=numpy_dtype)

    def populate(self, o: "P3") -> None:
        self.x, self.y, self.z = o.x, o.y, o.z

    @staticmethod
    def from_numpy_ndarry(a: np.ndarray) -> Union["P3", List["P3"]]:
        a = np.asarray(a)
        if a.ndim == 1:
            if a.shape[0] != 3:
                raise ValueError(f"cannot convert shape {a.shape} to P3")
            return P3(a[0], a[1], a[2])
        return [P3.from_numpy_ndarry(r) for r in a]

    @staticmethod
    def origin() -> "P3":
        return P3()

    zeros = origin

    @staticmethod
    def x_direct(x: float = 1.0) -> "P3":
        return P3(x, 0.0, 0.0)

    @staticmethod
    def y_direct(y: float = 1.0) -> "P3":
        return P3(0.0, y, 0.0)

    @staticmethod
    def z_direct(z: float = 1.0) -> "P3":
        return P3(0.0, 0.0, z)


def as_xyz(p) -> np.ndarray:
    """Any object with x, y, z attributes (this package's or cctpy's P3) -> float64[3]."""
    return np.array([float(p.x), float(p.y), float(p.z)])


class LocalCoordinateSystem:
    """Magnet frame: origin + orthonormal axes (cctpy local_coordinate_system.py:25-199)."""

    def __init__(self, location: P3 = None, x_direction: P3 = None, z_direction: P3 = None):
        location = P3() if location is None else location
        x_direction = P3.x_direct() if x_direction is None else x_direction
        z_direction = P3.z_direct() if z_direction is None else z_direction
        if abs(x_direction.copy().normalize() * z_direction.copy().normalize()) > 1e-4:
            raise AssertionError(f"x_direction {x_direction} and z_direction {z_direction} are not orthogonal")
        self.location = location.copy()
        self.ZI = z_direction.copy().normalize()
        self.XI = x_direction.copy().normalize()
        self.YI = self.ZI @ self.XI

    @staticmethod
    def create_by_y_and_z_direction(location: P3, y_direction: P3, z_direction: P3) -> "LocalCoordinateSystem":
        if abs(y_direction * z_direction) > 1e-6:
            raise AssertionError(f"y_direction {y_direction} and z_direction {z_direction} are not orthogonal")
        return LocalCoordinateSystem(location, y_direction @ z_direction, z_direction)

    @staticmethod
    def global_coordinate_system() -> "LocalCoordinateSystem":
        return LocalCoordinateSystem()

    def point_to_local_coordinate(self, p: P3) -> P3:
        d = p - self.location
        return P3(self.XI * d, self.YI * d, self.ZI * d)

    def point_to_global_coordinate(self, p: P3) -> P3:
        return self.location + (self.XI * p.x + self.YI * p.y + self.ZI * p.z)

    def vector_to_local_coordinate(self, v: P3) -> P3:
        return P3(self.XI * v, self.YI * v, self.ZI * v)

    def vector_to_global_coordinate(self, v: P3) -> P3:
        return self.XI * v.x + self.YI * v.y + self.ZI * v.z

    def axes(self) -> np.ndarray:
        """(4, 3): location, XI, YI, ZI."""
        return np.array([self.location.to_list(), self.XI.to_list(), self.YI.to_list(), self.ZI.to_list()])

    def points_to_global(self, pts: np.ndarray) -> np.ndarray:
        """Vectorised point_to_global_coordinate of an (n, 3) array, same rounding per element."""
        A = self.axes()
        out = np.empty_like(pts)
        for c in range(3):
            out[:, c] = A[0, c] + ((A[1, c] * pts[:, 0] + A[2, c] * pts[:, 1]) + A[3, c] * pts[:, 2])
        return out

    def copy(self) -> "LocalCoordinateSystem":
        return LocalCoordinateSystem(self.location.copy(), self.XI.copy(), self.ZI.copy())

    def __repr__(self) -> str:
        return f"LOCATION={self.location}, xi={self.XI}, yi={self.YI}, zi={self.ZI}"


class Line2:
    """Directed planar curve with a length (cctpy line2s.py:26-160)."""

    def get_length(self) -> float:
        raise NotImplementedError

    def point_at(self, s: float) -> P2:
        raise NotImplementedError

    def direct_at(self, s: float) -> P2:
        raise NotImplementedError

    def point_at_start(self) -> P2:
        return self.point_at(0.0)

    def point_at_end(self) -> P2:
        return self.point_at(self.get_length())

    def direct_at_start(self) -> P2:
        return self.direct_at(0.0)

    def direct_at_end(self) -> P2:
        return self.direct_at(self.get_length())

    def disperse2d(self, step: float = 1.0 * MM) -> List[P2]:
        """Points at ceil(length / step) + 1 equally spaced arc lengths (line2s.py:190-205)."""
        number = int(math.ceil(self.get_length() / step)) + 1
        return [self.point_at(s) for s in linspace(0, self.get_length(), number)]


def approx_equal(a: float, b: float, err: float = 1e-6) -> bool:
    """BaseUtils.equal for numbers (base_utils.py:35-58)."""
    return a == b or abs(a - b) <= err or ((a + b != 0.0) and 2 * abs((a - b) / (a + b)) <= err)


def linspace(start, end, number: int) -> list:
    """BaseUtils.linspace (base_utils.py:81-90): d = (end - start) * (1 / (number - 1)),
    start + d * float(i)."""
    d = (end - start) * (1 / (number - 1))
    return [start + d * float(i) for i in range(number)]


def derivative(func: Callable, delta: float = 1e-7) -> Callable:
    """BaseUtils.derivative (base_utils.py:194-203): central difference of step delta."""
    def d(x):
        return (func(x + delta / 2) - func(x - delta / 2)) / delta
    return d


class StraightLine2(Line2):
    def __init__(self, length: float, direct: P2, start_point: P2):
        self.length = float(length)
        self.direct = direct.normalize()
        self.start_point = start_point

    def get_length(self) -> float:
        return self.length

    def point_at(self, s: float) -> P2:
        return self.start_point + self.direct.copy().change_length(s)

    def direct_at(self, s: float) -> P2:
        return self.direct

    def straight_line_equation(self) -> Tuple[float, float, float]:
        """A, B, C of A x + B y + C = 0 through the start and start + direct
        (line2s.py:330-365)."""
        if approx_equal(self.direct.length(), 0, err=1e-10):
            raise ValueError("straight_line_equation: the direction has zero length")
        x1, y1 = self.start_point.x, self.start_point.y
        e = self.direct + self.start_point
        x2, y2 = e.x, e.y
        if approx_equal(x1, x2, err=1e-10):
            return 1.0, 0.0, -x1
        if approx_equal(y1, y2, err=1e-10):
            return 0.0, 1.0, -y1
        return (y2 - y1), (x1 - x2), (x2 * y1 - x1 * y2)

    @staticmethod
    def intersecting_point(pa: P2, va: P2, pb: P2, vb: P2) -> Tuple[P2, float, float]:
        """Intersection cp of the lines pa + ka va and pb + kb vb, with ka and kb
        (line2s.py:368-412)."""
        if approx_equal(va.length(), 0.0, err=1e-10) or approx_equal(vb.length(), 0.0, err=1e-10):
            raise ValueError(f"intersecting_point: a direction has zero length (va={va}, vb={vb})")
        A1, B1, C1 = StraightLine2(1.0, va, pa).straight_line_equation()
        A2, B2, C2 = StraightLine2(1.0, vb, pb).straight_line_equation()
        cpy = (A1 * C2 - A2 * C1) / (A2 * B1 - A1 * B2)
        cpx = -(B1 * cpy + C1) / A1 if A1 != 0 else -(B2 * cpy + C2) / A2
        cp = P2(cpx, cpy)
        ka = (cp.x - pa.x) / va.x if va.x != 0 else (cp.y - pa.y) / va.y
        kb = (cp.x - pb.x) / vb.x if vb.x != 0 else (cp.y - pb.y) / vb.y
        return cp, ka, kb

    @staticmethod
    def is_on_right(view_point: P2, view_direct: P2, viewed_point: P2) -> int:
        """1 if viewed_point is on the right of the view direction, -1 left, 0 ahead or
        behind (line2s.py:414-434)."""
        right = view_direct.copy().rotate(-90 / 180.0 * math.pi)
        k = right * (viewed_point - view_point)
        return 1 if k > 0 else (-1 if k < 0 else 0)

    def side_of(self, p: P2) -> int:
        """+1 if p lies on the right of the directed line, -1 on the left, 0 on it (1e-6)."""
        d = self.direct
        w = p - self.start_point
        cross = d.x * w.y - d.y * w.x
        if abs(cross) <= 1e-6 * max(1.0, w.length()):
            return 0
        return 1 if cross < 0 else -1


class ArcLine2(Line2):
    def __init__(self, starting_phi: float, center: P2, radius: float, total_phi: float, clockwise: bool):
        self.starting_phi = starting_phi
        self.center = center
        self.radius = radius
        self.total_phi = total_phi
        self.clockwise = clockwise
        self.length = radius * total_phi

    def get_length(self) -> float:
        return self.length

    def _phi(self, s: float) -> float:
        t = s / self.radius
        return self.starting_phi - t if self.clockwise else self.starting_phi + t

    def point_at(self, s: float) -> P2:
        c = self._phi(s)
        return P2(math.cos(c), math.sin(c)).change_length(self.radius) + self.center

    def direct_at(self, s: float) -> P2:
        c = self._phi(s)
        return P2(math.cos(c), math.sin(c)).rotate(-math.pi / 2 if self.clockwise else math.pi / 2)

    @staticmethod
    def create(start_point: P2, start_direct: P2, radius: float, clockwise: bool, total_deg: float) -> "ArcLine2":
        center = start_point + start_direct.copy().rotate(-math.pi / 2 if clockwise else math.pi / 2).change_length(
            radius)
        return ArcLine2((start_point - center).angle_to_x_axis(), center, radius, total_deg / 180.0 * math.pi,
                        clockwise)


class Trajectory(Line2):
    """Design orbit made of straight lines and arcs (cctpy trajectory.py:30-160)."""

    def __init__(self, first_line: Line2):
        self._lines: List[Line2] = [first_line]
        self._length = first_line.get_length()

    class _Builder:
        def __init__(self, start_point: P2):
            self.start_point = start_point

        def first_line(self, direct: P2 = None, length: float = 1.0) -> "Trajectory":
            return Trajectory(StraightLine2(length, P2.x_direct() if direct is None else direct, self.start_point))

    @staticmethod
    def set_start_point(start_point: P2 = None) -> "Trajectory._Builder":
        return Trajectory._Builder(P2() if start_point is None else start_point)

    def add_strait_line(self, length: float) -> "Trajectory":
        last = self._lines[-1]
        self._lines.append(StraightLine2(length, last.direct_at_end(), last.point_at_end()))
        self._length += length
        return self

    def add_arc_line(self, radius: float, clockwise: bool, angle_deg: float) -> "Trajectory":
        last = self._lines[-1]
        arc = ArcLine2.create(last.point_at_end(), last.direct_at_end(), radius, clockwise, angle_deg)
        self._lines.append(arc)
        self._length += arc.get_length()
        return self

    def get_length(self) -> float:
        return self._length

    def _locate(self, s: float):
        for ln in self._lines:
            if s <= ln.get_length():
                return ln, s
            s -= ln.get_length()
        last = self._lines[-1]
        return last, (last.get_length() if abs(s) <= 1e-8 else last.get_length() + s)

    def point_at(self, s: float) -> P2:
        ln, t = self._locate(s)
        return ln.point_at(t)

    def direct_at(self, s: float) -> P2:
        ln, t = self._locate(s)
        return ln.direct_at(t)

    def get_line2_list(self) -> List[Line2]:
        return self._lines


def circle_center_and_radius(p1: P2, p2: P2, p3: P2):
    """Centre and radius of the circle through three points, as the least-squares
    solution of the chord-bisector equations (x_j - x_i) cx + (y_j - y_i) cy =
    (|p_j|^2 - |p_i|^2) / 2 over the three chords, solved through the normal
    equations -- the same steps as cctpy's BaseUtils.circle_center_and_radius
    (base_utils.py:124-151), so that magnets land where the reference puts them."""
    xs, ys = (p1.x, p2.x, p3.x), (p1.y, p2.y, p3.y)
    pairs = ((0, 1), (0, 2), (1, 2))
    A = np.array([[xs[j] - xs[i], ys[j] - ys[i]] for i, j in pairs])
    rhs = 0.5 * np.array([[xs[j] ** 2 + ys[j] ** 2 - xs[i] ** 2 - ys[i] ** 2] for i, j in pairs])
    c = np.linalg.inv(A.T @ A) @ A.T @ rhs
    cx, cy = float(c[0, 0]), float(c[1, 0])
    r = sum(math.sqrt((cx - x) ** 2 + (cy - y) ** 2) for x, y in zip(xs, ys)) / 3
    return P2(cx, cy), r


class FunctionLine3:
    """A 3-D curve p = f(s), s from start to end (cctpy line3s.py:166-264)."""

    def __init__(self, p3_function: Callable[[float], P3], start: float, end: float,
                 direct_function: Optional[Callable[[float], P3]] = None, delta_for_disperse: float = 1 * MM,
                 delta_for_compute_direct_function: float = 0.1 * MM):
        self._f = p3_function
        self._start, self._end = start, end
        if direct_function is None:
            def direct_function(t):
                return (self._f(t + delta_for_compute_direct_function) - self._f(t)) / delta_for_compute_direct_function
        self._direct = direct_function

    def point_at_p3_function(self, s: float) -> P3:
        return self._f(s)

    def direct_at_p3_function(self, s: float) -> P3:
        return self._direct(s)

    def get_start(self) -> float:
        return self._start

    def get_end(self) -> float:
        return self._end

    def get_p3_function(self) -> Callable[[float], P3]:
        return self._f
