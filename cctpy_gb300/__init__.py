"""cctpy_gb300 -- GB300-native (sm_103a) engine for cctpy's tracking hot path.

The Biot-Savart sum over discretised CCT winding segments, evaluated at every
field point of a 4th-order Runge-Kutta proton push through a gantry beamline,
behind cctpy's own Python API:

    from cctpy_gb300 import (P2, P3, LocalCoordinateSystem, Trajectory, CCT, QS,
                             CombinedMagnet, Beamline, HUST_SC_GANTRY, RunningParticle,
                             ParticleFactory, PhaseSpaceParticle, ParticleRunner,
                             GPU_ACCELERATOR)

Compute runs in libcctgpu.so (C ABI, include/cctgpu.h); there is no CPU path.
"""
from .geometry import (LIGHT_SPEED, MM, MRAD, ArcLine2, FunctionLine3, Line2, LocalCoordinateSystem, P2, P3,
                       StraightLine2, Trajectory)
from .magnets import (AGCCT_CONNECTOR, CCT, QS, CombinedMagnet, LocalUniformMagnet, Magnet, Q, UniformMagnet,
                      Wire)
from .beamline import HUST_SC_GANTRY, Beamline
from .particles import (Ellipse, ParticleFactory, ParticleRunner, PhaseSpaceParticle, Protons, RunningParticle)
from .accelerator import GPU_ACCELERATOR

__all__ = ["LIGHT_SPEED", "MM", "MRAD", "ArcLine2", "Line2", "LocalCoordinateSystem", "P2", "P3", "StraightLine2",
           "Trajectory", "FunctionLine3", "CCT", "QS", "Q", "LocalUniformMagnet", "UniformMagnet", "Wire",
           "AGCCT_CONNECTOR", "CombinedMagnet", "Magnet", "HUST_SC_GANTRY", "Beamline", "Ellipse",
           "ParticleFactory", "ParticleRunner", "PhaseSpaceParticle", "Protons", "RunningParticle",
           "GPU_ACCELERATOR"]
