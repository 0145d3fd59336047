"""FP32 emulation of the field kernels' two pair forms (CPU, numpy float32), checking the
precision argument behind the moment form:

  direct   B_tile = sum_i kl_i x (q - p_i) |r_i|^-3                 (FP32 cross per pair)
  moment   B_sub  = A x (q - o) - M,  A = sum kl_i |r_i|^-3,  M = sum (kl_i x (p_i - o)) |r_i|^-3

with q and p_i taken from the tile's double-float origin, o the centroid of each 32-segment
sub-block.  |r|^-3 is rsqrt(|r|^2) cubed (two multiplies), or rsqrt(|r|^2) x rcp(|r|^2): one
multiply fewer on the FMA pipe for a second MUFU operation, at the same precision.  Against an FP64 sum of the same segments: in the aperture both forms stay far
below 1e-7; 3-8 mm from the windings the moment form about sub-block origins stays within a
small factor of the direct form, while the same form about the tile origin does not.
(The kernels round rsqrt on the MUFU unit; here it is correctly rounded.)"""
import numpy as np

from cctpy_gb300 import workloads as W

f32, f64 = np.float32, np.float64
TILE, SUB = 128, 32


def _fma(a, b, c):
    return (a.astype(f64) * b.astype(f64) + c.astype(f64)).astype(f32)


def _cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
                     a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], axis=-1)


def _segments():
    _, cct = W.build_single_dipole()
    kl, p0 = cct.global_segments()
    n = kl.shape[0] // TILE * TILE
    return kl[:n], p0[:n]


def _points(n, r1, r2, seed):
    c = W.SINGLE_DIPOLE
    R, d0, L = c["big_r"], c["drift"], W.single_dipole_track_length()
    rng = np.random.default_rng(seed)
    s = rng.random(n) * L
    rho = rng.uniform(r1, r2, n)
    th = rng.random(n) * 2 * np.pi
    phi = np.pi / 2 - s / R
    radial = np.stack([np.cos(phi), np.sin(phi), np.zeros(n)], axis=1)
    base = np.stack([d0 + R * np.cos(phi), -R + R * np.sin(phi), np.zeros(n)], axis=1)
    return base + (rho * np.cos(th))[:, None] * radial + (rho * np.sin(th))[:, None] * np.array([0, 0, 1.0])


def _emulate(kl, p0, pts, form, inv3_form="cube"):
    nt = kl.shape[0] // TILE
    klt, p0t = kl.reshape(nt, TILE, 3), p0.reshape(nt, TILE, 3)
    cen = p0t.mean(1)
    ohi = cen.astype(f32)
    olo = (cen - ohi).astype(f32)
    o = ohi.astype(f64) + olo
    off = p0t - o[:, None, :]                                   # FP64 offsets from the represented origin
    kf, pf = klt.astype(f32), off.astype(f32)
    sub = off.reshape(nt, TILE // SUB, SUB, 3).mean(2).astype(f32) if form == "moment_sub" else \
        np.zeros((nt, TILE // SUB, 3), f32)
    e = off - np.repeat(sub.astype(f64), SUB, axis=1)
    mf = _cross(klt, e).astype(f32)
    ph = pts.astype(f32)
    pl = (pts - ph).astype(f32)
    q = ((ph[:, None, :] - ohi[None]).astype(f32) + (pl[:, None, :] - olo[None]).astype(f32)).astype(f32)  # (P, nt, 3)
    r = (q[:, :, None, :] - pf[None]).astype(f32)                                                     # (P, nt, T, 3)
    r2 = _fma(r[..., 0], r[..., 0], _fma(r[..., 1], r[..., 1], (r[..., 2] * r[..., 2]).astype(f32)))
    inv = (1.0 / np.sqrt(r2.astype(f64))).astype(f32)
    if inv3_form == "cube":
        inv3 = ((inv * inv).astype(f32) * inv).astype(f32)
    else:
        inv3 = (inv * (1.0 / r2.astype(f64)).astype(f32)).astype(f32)
    P = pts.shape[0]
    if form == "direct":
        c = _cross(kf[None], r).astype(f32)
        terms = (c * inv3[..., None]).astype(f32).reshape(P, nt, TILE // SUB, SUB, 3)
        blocks = terms.sum(3, dtype=f32)                                                              # FP32 sub-block sums
    else:
        A = (kf[None] * inv3[..., None]).astype(f32).reshape(P, nt, TILE // SUB, SUB, 3).sum(3, dtype=f32)
        M = (mf[None] * inv3[..., None]).astype(f32).reshape(P, nt, TILE // SUB, SUB, 3).sum(3, dtype=f32)
        w = (q[:, :, None, :] - sub[None]).astype(f32)
        blocks = (_cross(A.astype(f64), w.astype(f64)).astype(f32) - M).astype(f32)
    return blocks.astype(f64).sum((1, 2))                                                         # compensated across


def _exact(kl, p0, pts):
    r = pts[:, None, :] - p0[None]
    inv3 = np.sum(r * r, -1) ** -1.5
    return (_cross(kl[None], r) * inv3[..., None]).sum(1)


def _rel(b, ref):
    return np.linalg.norm(b - ref, axis=1) / np.linalg.norm(ref, axis=1)


def test_moment_form_precision():
    kl, p0 = _segments()
    for (r1, r2, n, seed) in ((0.0, 0.06, 24, 3), (0.075, 0.080, 24, 4)):
        pts = _points(n, r1, r2, seed)
        ref = _exact(kl, p0, pts)
        err = {form: _rel(_emulate(kl, p0, pts, form), ref).max() for form in ("direct", "moment_sub", "moment_tile")}
        err["moment_sub_rcp"] = _rel(_emulate(kl, p0, pts, "moment_sub", "rsqrt_rcp"), ref).max()
        assert err["moment_sub_rcp"] < 1.25 * err["moment_sub"], err
        if r2 <= 0.06:     # in the aperture
            assert err["direct"] < 1e-7 and err["moment_sub"] < 1e-7, err
        else:              # 3-8 mm from the windings
            assert err["moment_sub"] < 2.5 * err["direct"], err
            assert err["moment_tile"] > err["moment_sub"], err
