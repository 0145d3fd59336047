"""OPERA cross-check (the reference's final_code/demos/D04OperaTrack对比.py): a 215 MeV
proton through two single-tilt CCT layers, tracked on the GPU, against cctpy's own CPU track
(parity) and OPERA-3D's track with brick conductors (physical agreement); fixture from
tests/golden/make_golden_opera.py."""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from cctpy_gb300 import MM, P2, LocalCoordinateSystem, engine
from cctpy_gb300.magnets import CCT, CombinedMagnet

HERE = os.path.dirname(os.path.abspath(__file__))


def magnet():
    def layer(small_r, tilt, sign):
        return CCT(LocalCoordinateSystem(), 0.95, small_r, 22.5, [tilt], 42, -6192.0, P2(0, 0),
                   P2(sign * 2 * math.pi * 42, 22.5 / 180.0 * math.pi), 120)
    return CombinedMagnet(layer(104.5 * MM, -30, -1), layer(120.5 * MM, 30, 1))


@pytest.mark.parametrize("precision,tol", [("f64", 1e-9), ("f32c", 1e-6)])
def test_track_vs_cctpy_and_opera(precision, tol):
    g = np.load(os.path.join(HERE, "golden", "golden_opera.npz"))
    ds = engine.design_of(magnet())
    p = g["particle_in"][None, :]
    pos = []
    for _ in range(len(g["s"])):
        p = engine.track(ds, p, 0.05, 1 * MM, precision)[0]
        pos.append(p[0, 0:3])
    pos = np.array(pos)
    assert np.abs(pos - g["cctpy_pos"]).max() <= tol                   # parity with cctpy
    dev = np.linalg.norm(pos - g["opera_pos"], axis=1)
    ref_dev = np.linalg.norm(g["cctpy_pos"] - g["opera_pos"], axis=1)
    assert np.abs(dev - ref_dev).max() <= 2 * tol                       # the same agreement as cctpy's
    assert dev.max() < 0.2e-3                                           # within 0.2 mm of OPERA over 2.35 m
