"""Parity at the workloads' full sizes, through properties that hold whatever the size.

* Field map (2^20 points x 46 080 segments): FP32c within 1e-7 relative of the FP64 drop-in
  at every point; both kernels exactly linear in the currents (a power-of-two scale is exact
  in every rounding, so doubling every kl doubles every field bit for bit); superposition
  over a ragged split of the windings (two designs of one set).
* Gantry section (597 600 segments + QS, 4096 protons, 3.5 m at 1 mm: 3500 RK4 steps, the
  dataflow schedule): tracking the particles in reverse order gives the reversed result bit
  for bit (a particle's sums do not depend on its slot or on which CTA ran which unit), and
  32 of them tracked alone (one particle block: grid barriers, other chunks) land within
  1 um of the same particles in the full batch.

The file sorts last: its cases are the longest of the GPU suite (about a minute).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from cctpy_gb300 import engine, workloads as W

N_POINTS = 1 << 20


@pytest.fixture(scope="module")
def field_map():
    _, cct = W.build_single_dipole()
    kl, p0, qs = engine.host_design(engine.magnet_list(cct))
    assert kl.shape[0] == 46080 and qs.shape[0] == 0
    pts = torch.from_numpy(W.field_map_points(N_POINTS, seed=1)).cuda()
    ds = engine.DesignSet([(kl, p0, qs)])
    return kl, p0, qs, pts, ds, engine.field_at_points(ds, pts, "f64")


def test_field_map_f32c_within_1e7_of_f64(field_map):
    kl, p0, qs, pts, ds, b64 = field_map
    b32 = engine.field_at_points(ds, pts, "f32c")
    rel = torch.linalg.norm(b32 - b64, dim=1) / torch.linalg.norm(b64, dim=1)
    assert bool(torch.isfinite(b32).all())
    assert float(rel.max()) <= 1e-7


@pytest.mark.parametrize("prec", ["f64", "f32c"])
def test_field_map_exactly_linear_in_current(field_map, prec):
    kl, p0, qs, pts, _, _ = field_map
    ds = engine.DesignSet([(kl, p0, qs), (2.0 * kl, p0, qs)])
    b1 = engine.field_at_points(ds, pts, prec, design=0)
    b2 = engine.field_at_points(ds, pts, prec, design=1)
    assert torch.equal(b2, 2.0 * b1)


@pytest.mark.parametrize("prec,tol", [("f64", 1e-11), ("f32c", 1e-6)])
def test_field_map_superposition(field_map, prec, tol):
    kl, p0, qs, pts, _, b = field_map
    h = 23001                                   # not a tile boundary: both designs end in a ragged tile
    parts = engine.DesignSet([(kl[:h], p0[:h], qs), (kl[h:], p0[h:], qs)])
    s = engine.field_at_points(parts, pts, prec, design=0) + engine.field_at_points(parts, pts, prec, design=1)
    bmax = float(torch.linalg.norm(b, dim=1).max())
    assert float((s - b).abs().max()) <= tol * bmax


def test_gantry_section_full_track_order_and_schedule_independent():
    g = W.GANTRY_SECTION
    bl = W.build_gantry_section()
    ds = engine.design_of(bl)
    assert ds.n_segments == 597600
    ps = W.beam_particles(bl, 4096, seed=2, kinetic_MeV=g["kinetic_MeV"])
    L, step = g["track_length"], g["footstep"]
    out = engine.track(ds, ps, L, step, "f32c")[0]
    assert np.isfinite(out).all()
    assert np.allclose(out[:, 9], ps[:, 9] + L, rtol=0, atol=1e-12)
    rev = engine.track(ds, np.ascontiguousarray(ps[::-1]), L, step, "f32c")[0]
    assert np.array_equal(rev[::-1], out)
    alone = engine.track(ds, ps[:32], L, step, "f32c")[0]
    assert np.abs(alone[:, 0:3] - out[:32, 0:3]).max() < 1e-6
    assert np.abs(alone[:, 3:6] - out[:32, 3:6]).max() < 1e-6 * np.abs(out[:32, 3:6]).max()
