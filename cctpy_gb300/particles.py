"""Protons, phase space and the RK4 particle runner (on the GPU).

Same names, record layout and arithmetic as cctpy final_code/packages/particles.py
(Protons :28-47, RunningParticle :286-506, ParticleRunner :509-632,
PhaseSpaceParticle :873-1138, ParticleFactory :1318-1454) and the ellipse
edge sampler of base_utils.py (Ellipse :470-600).  ParticleRunner.run_only
tracks on the GPU; there is no CPU path.
"""
from __future__ import annotations

import math
from typing import List, Sequence, Union

import numpy as np

from .geometry import LIGHT_SPEED, MM, P2, P3, LocalCoordinateSystem


class Protons:
    STATIC_MASS_KG = 1.672621898e-27
    STATIC_ENERGY_MeV = 938.2720813
    CHARGE_QUANTITY = 1.6021766208e-19

    @classmethod
    def get_total_energy_MeV(cls, kinetic_energy_MeV: float) -> float:
        return cls.STATIC_ENERGY_MeV + kinetic_energy_MeV


class RunningParticle:
    """A particle in the global frame: position, velocity, relativistic mass, charge,
    speed, distance travelled."""

    def __init__(self, position: P3, velocity: P3, relativistic_mass: float, e: float, speed: float,
                 distance: float = 0.0):
        self.position = position
        self.velocity = velocity
        self.relativistic_mass = relativistic_mass
        self.e = e
        self.speed = speed
        self.distance = distance

    def copy(self) -> "RunningParticle":
        return RunningParticle(self.position.copy(), self.velocity.copy(), self.relativistic_mass, self.e,
                               self.speed, self.distance)

    def compute_scalar_momentum(self) -> float:
        return self.speed * self.relativistic_mass

    def change_scalar_momentum(self, scalar_momentum: float) -> None:
        m0 = self.relativistic_mass * math.sqrt(1 - (self.speed ** 2) / (LIGHT_SPEED ** 2))
        new_speed = scalar_momentum / math.sqrt(m0 ** 2 + (scalar_momentum / LIGHT_SPEED) ** 2)
        self.relativistic_mass = m0 / math.sqrt(1 - (new_speed / LIGHT_SPEED) ** 2)
        self.speed = new_speed
        self.velocity = self.velocity.change_length(new_speed)

    def get_natural_coordinate_system(self, y_direction: P3 = None) -> LocalCoordinateSystem:
        return LocalCoordinateSystem.create_by_y_and_z_direction(
            self.position, P3.z_direct() if y_direction is None else y_direction, self.velocity)

    def to_numpy_array_data(self, numpy_dtype=np.float64) -> np.ndarray:
        return np.array(self.position.to_list() + self.velocity.to_list()
                        + [self.relativistic_mass, self.e, self.speed, self.distance], dtype=numpy_dtype)

    @staticmethod
    def from_numpy_array_data(a) -> "RunningParticle":
        return RunningParticle(P3(a[0], a[1], a[2]), P3(a[3], a[4], a[5]), float(a[6]), float(a[7]), float(a[8]),
                               float(a[9]))

    def populate(self, other: "RunningParticle") -> None:
        self.position.populate(other.position)
        self.velocity.populate(other.velocity)
        self.relativistic_mass = other.relativistic_mass
        self.e = other.e
        self.speed = other.speed
        self.distance = other.distance

    def __sub__(self, o: "RunningParticle") -> "RunningParticle":
        return RunningParticle(self.position - o.position, self.velocity - o.velocity,
                               self.relativistic_mass - o.relativistic_mass, self.e - o.e, self.speed - o.speed,
                               self.distance - o.distance)

    def detailed_info(self) -> str:
        return (f"Particle[p={self.position}, v={self.velocity}], rm={self.relativistic_mass}, e={self.e}, "
                f"speed={self.speed}, distance={self.distance}]")

    def __repr__(self) -> str:
        return f"p={self.position},v={self.velocity},v0={self.speed}"


def particles_to_array(ps: Sequence) -> np.ndarray:
    return np.array([[p.position.x, p.position.y, p.position.z, p.velocity.x, p.velocity.y, p.velocity.z,
                      p.relativistic_mass, p.e, p.speed, p.distance] for p in ps], dtype=np.float64).reshape(-1, 10)


class ParticleRunner:
    """RK4 tracking (cctpy particles.py:509-632), on the GPU."""

    @staticmethod
    def run_only(p: Union[RunningParticle, List[RunningParticle]], m, length: float, footstep: float = 20 * MM,
                 concurrency_level: int = 1, report: bool = True, precision: str = "f64"):
        """Move particle(s) `length` metres through magnet `m` (fixed-step RK4 in time:
        dt = footstep/speed, steps = ceil(t_end/dt), Y' = [v, (e/m) v x B]).  The particles
        are updated in place and returned.  `concurrency_level` and `report` are accepted
        for compatibility; the GPU runs every particle at once."""
        from . import engine
        single = isinstance(p, RunningParticle)
        ps = [p] if single else list(p)
        if not ps:
            return p
        for q in ps:
            if q.speed == 0:
                raise ZeroDivisionError("particle speed is zero")
        if length == 0 or footstep == 0:
            raise ZeroDivisionError("length and footstep must be non-zero")
        out = engine.track(engine.design_of(m), particles_to_array(ps), length, footstep, precision)[0]
        for q, r in zip(ps, out):
            q.position = P3(r[0], r[1], r[2])
            q.velocity = P3(r[3], r[4], r[5])
            q.distance = float(r[9])
        return p


class Ellipse:
    """Ellipse A x^2 + B x y + C y^2 = D (cctpy base_utils.py:470-600).  Points along the
    edge are found as the reference does: a ray from the origin meets the ellipse at
    polar angle theta; arc length is walked in 0.05 deg chords; the circumference is
    the sum of 14 400 chords."""

    def __init__(self, A: float, B: float, C: float, D: float):
        self.A, self.B, self.C, self.D = float(A), float(B), float(C), float(D)

    @staticmethod
    def _eq(a, b, err=1e-6):
        return a == b or abs(a - b) <= err or ((a + b != 0.0) and (2 * abs((a - b) / (a + b))) <= err)

    def point_at(self, theta: float) -> P2:
        x = y = 0.0
        while theta < 0:
            theta += 2 * math.pi
        while theta > 2 * math.pi:
            theta -= 2 * math.pi
        if self._eq(theta, 0) or self._eq(theta, 2 * math.pi):
            x, y = math.sqrt(self.D / self.A), 0.0
        if self._eq(theta, math.pi):
            x, y = -math.sqrt(self.D / self.A), 0.0
        if 0 < theta < math.pi:
            t = 1 / math.tan(theta)
            y = math.sqrt(self.D / (self.A * t * t + self.B * t + self.C))
            x = t * y
        if math.pi < theta < 2 * math.pi:
            t = 1 / math.tan(theta - math.pi)
            y = -math.sqrt(self.D / (self.A * t * t + self.B * t + self.C))
            x = t * y
        return P2(x, y)

    @property
    def circumference(self) -> float:
        num = 3600 * 4
        c = 0.0
        prev = self.point_at(0.0)
        for i in range(num):
            cur = self.point_at(2.0 * math.pi / float(num) * (i + 1))
            c += (cur - prev).length()
            prev = cur
        return c

    def point_after(self, length: float) -> P2:
        step = 0.05 / 180.0 * math.pi
        theta = 0.0
        while length > 0.0:
            length -= (self.point_at(theta + step) - self.point_at(theta)).length()
            theta += step
        return self.point_at(theta)

    def uniform_distribution_points_along_edge(self, num: int) -> List[P2]:
        c = self.circumference
        return [self.point_after(c / num * i) for i in range(num)]


class PhaseSpaceParticle:
    """Phase-space coordinates (x, xp, y, yp, z, delta) relative to an ideal particle."""

    XXP_PLANE = 1
    YYP_PLANE = 2

    def __init__(self, x=0.0, xp=0.0, y=0.0, yp=0.0, z=0.0, delta=0.0):
        self.x, self.xp, self.y, self.yp, self.z, self.delta = x, xp, y, yp, z, delta

    def project_to_xxp_plane(self, convert_to_mm: bool = False) -> P2:
        f = 1000 if convert_to_mm else 1
        return P2(self.x * f, self.xp * f)

    def project_to_yyp_plane(self, convert_to_mm: bool = False) -> P2:
        f = 1000 if convert_to_mm else 1
        return P2(self.y * f, self.yp * f)

    def project_to_plane(self, plane_id: int, convert_to_mm: bool = False) -> P2:
        if plane_id == self.XXP_PLANE:
            return self.project_to_xxp_plane(convert_to_mm)
        if plane_id == self.YYP_PLANE:
            return self.project_to_yyp_plane(convert_to_mm)
        raise ValueError(f"no plane {plane_id}")

    def to_list(self) -> List[float]:
        return [self.x, self.xp, self.y, self.yp, self.z, self.delta]

    @staticmethod
    def phase_space_particles_along_positive_ellipse_in_xxp_plane(xMax, xpMax, delta, number):
        e = Ellipse(1 / (xMax ** 2), 0, 1 / (xpMax ** 2), 1)
        return [PhaseSpaceParticle(p.x, p.y, 0, 0, 0, delta) for p in e.uniform_distribution_points_along_edge(number)]

    @staticmethod
    def phase_space_particles_along_positive_ellipse_in_yyp_plane(yMax, ypMax, delta, number):
        e = Ellipse(1 / (yMax ** 2), 0, 1 / (ypMax ** 2), 1)
        return [PhaseSpaceParticle(0, 0, p.x, p.y, 0, delta) for p in e.uniform_distribution_points_along_edge(number)]

    @staticmethod
    def phase_space_particles_project_to_xxp_plane(pss, convert_to_mm: bool = False) -> List[P2]:
        return [p.project_to_xxp_plane(convert_to_mm) for p in pss]

    @staticmethod
    def phase_space_particles_project_to_yyp_plane(pss, convert_to_mm: bool = False) -> List[P2]:
        return [p.project_to_yyp_plane(convert_to_mm) for p in pss]

    @staticmethod
    def create_from_running_particle(ideal_particle: RunningParticle, coordinate_system: LocalCoordinateSystem,
                                     running_particle: RunningParticle) -> "PhaseSpaceParticle":
        rel = running_particle.position - ideal_particle.position
        x, y, z = coordinate_system.XI * rel, coordinate_system.YI * rel, coordinate_system.ZI * rel
        relv = running_particle.velocity - ideal_particle.velocity
        xv, yv = coordinate_system.XI * relv, coordinate_system.YI * relv
        sp = running_particle.speed
        xp = xv / math.sqrt(sp ** 2 - xv ** 2)
        yp = yv / math.sqrt(sp ** 2 - yv ** 2)
        rm = running_particle.compute_scalar_momentum()
        im = ideal_particle.compute_scalar_momentum()
        return PhaseSpaceParticle(x, xp, y, yp, z, (rm - im) / im)

    @staticmethod
    def create_from_running_particles(ideal_particle, coordinate_system, running_particles):
        return [PhaseSpaceParticle.create_from_running_particle(ideal_particle, coordinate_system, p)
                for p in running_particles]


class ParticleFactory:
    @staticmethod
    def create_proton(position: P3, direct: P3, kinetic_MeV: float = 250) -> RunningParticle:
        e0 = Protons.STATIC_ENERGY_MeV
        speed = LIGHT_SPEED * math.sqrt(1.0 - (e0 / (e0 + kinetic_MeV)) ** 2)
        rm = Protons.STATIC_MASS_KG / math.sqrt(1.0 - (speed ** 2) / (LIGHT_SPEED ** 2))
        return RunningParticle(position, direct.copy().change_length(speed), rm, Protons.CHARGE_QUANTITY, speed)

    @staticmethod
    def create_proton_by_position_and_velocity(position: P3, velocity: P3) -> RunningParticle:
        speed = velocity.length()
        rm = Protons.STATIC_MASS_KG / math.sqrt(1.0 - (speed ** 2) / (LIGHT_SPEED ** 2))
        return RunningParticle(position, velocity, rm, Protons.CHARGE_QUANTITY, speed)

    @staticmethod
    def create_proton_along(trajectory, s: float = 0.0, kinetic_MeV: float = 250) -> RunningParticle:
        return ParticleFactory.create_proton(trajectory.point_at(s).to_p3(), trajectory.direct_at(s).to_p3(),
                                             kinetic_MeV)

    @staticmethod
    def create_from_phase_space_particle(ideal_particle: RunningParticle, coordinate_system: LocalCoordinateSystem,
                                         phase_space_particle: PhaseSpaceParticle) -> RunningParticle:
        ps = phase_space_particle
        p = ideal_particle.copy()
        p.position += coordinate_system.XI * ps.x
        p.position += coordinate_system.YI * ps.y
        p.position += coordinate_system.ZI * ps.z
        if ps.delta != 0.0:
            p.change_scalar_momentum(p.compute_scalar_momentum() * (1.0 + ps.delta))
        p.velocity += coordinate_system.XI * (ps.xp * p.speed)
        p.velocity += coordinate_system.YI * (ps.yp * p.speed)
        p.velocity = p.velocity.change_length(p.speed)
        return p

    @staticmethod
    def create_from_phase_space_particles(ideal_particle, coordinate_system, phase_space_particles):
        return [ParticleFactory.create_from_phase_space_particle(ideal_particle, coordinate_system, p)
                for p in phase_space_particles]
