"""Device-side segment generation (cct_segments_build) against the host construction, and
the device segment-to-parameter Jacobian (cct_segments_param_grad) against the host
complex-step Jacobian."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from cctpy_gb300 import HUST_SC_GANTRY, _lib, engine, workloads as W
from cctpy_gb300.adjoint import GantryDesign, design_gradients, layer_gradient

POINT_ATOL = 2e-14  # metres: device and host trigonometric functions round differently
P0_ATOL = 1e-13     # metres
JAC_RTOL = 1e-9     # forward mode on the GPU vs complex step on the host


def designs():
    _, dipole = W.build_single_dipole()
    pop = [HUST_SC_GANTRY(**kw).create_second_bending_part_beamline() for kw in W.design_population(3, seed=3)]
    return [dipole, W.build_gantry_section()] + pop


def test_device_segments_match_host():
    objs = designs()
    host = engine.design_set_of(objs, segments="host")
    dev = engine.design_set_of(objs, segments="device")
    np.testing.assert_array_equal(host.h_seg_off, dev.h_seg_off)
    np.testing.assert_array_equal(host.h_qs_off, dev.h_qs_off)
    assert torch.equal(host.qs, dev.qs)
    kh, kd = host.kls.cpu().numpy(), dev.kls.cpu().numpy()
    ph, pd = host.p0s.cpu().numpy(), dev.p0s.cpu().numpy()
    for d in range(len(objs)):
        a, b = host.h_seg_off[d], host.h_seg_off[d + 1]
        # kl = 1e-7 I (w[i+1] - w[i]): bound by the winding points' displacement
        i_max = np.abs(dev.h_layers[dev.layer_design == d, 14]).max()
        assert np.abs(kd[a:b] - kh[a:b]).max() <= 1e-7 * i_max * 2 * POINT_ATOL, d
        assert np.abs(pd[a:b] - ph[a:b]).max() <= P0_ATOL, d


def test_fields_of_device_built_set():
    objs = designs()[:2]
    host = engine.design_set_of(objs, segments="host")
    dev = engine.design_set_of(objs, segments="device")
    pts = W.field_map_points(4096, seed=5)
    for d in range(2):
        bh = engine.field_at_points(host, pts, "f64", design=d)
        bd = engine.field_at_points(dev, pts, "f64", design=d)
        assert (np.linalg.norm(bd - bh, axis=1) <= 1e-11 * np.linalg.norm(bh, axis=1) + 1e-15).all()


def test_param_grad_matches_complex_step():
    objs = designs()[:3]
    ds = engine.design_set_of(objs, segments="device")
    rng = np.random.default_rng(11)
    g = rng.standard_normal((ds.n_segments, 6))
    # segment gradients of a real objective are smooth along the winding: add a smooth part
    g += np.cos(np.arange(ds.n_segments) * 1e-3)[:, None]
    rows = ds.param_grad(torch.as_tensor(g, device=ds.kls.device))
    assert rows.shape == (len(ds.layer_magnets), 10)
    at = 0
    for l, m in enumerate(ds.layer_magnets):
        n = m.total_disperse_number
        ref = layer_gradient(m, g[at:at + n])
        at += n
        got = rows[l]
        want = np.array(list(ref["tilt"]) + [ref["current"], ref["big_r"]])
        have = np.array(list(got[:len(m.tilt_angles)]) + [got[8], got[9]])
        scale = np.abs(want).max()
        assert np.all(np.abs(have - want) <= JAC_RTOL * np.abs(want) + 1e-12 * scale), (l, have, want)
        assert np.all(got[len(m.tilt_angles):8] == 0)
    assert at == ds.n_segments


def test_design_gradients_device_equals_host():
    kw = W.design_population(2, seed=3)
    theta = [np.array(k["dicct345_tilt_angles"] + k["agcct345_tilt_angles"]
                      + [k["dicct345_current"], k["dicct345_current"], k["agcct345_current"],
                         k["agcct345_current"], 0.95]) for k in kw]
    des = [GantryDesign(t, part_per_winding=60) for t in theta]
    ps = W.beam_particles(des[0].beamline, 8, seed=7, kinetic_MeV=215.0)
    Jh, gh = design_gradients(des, ps, 0.1, 0.01, 215.0, checkpoint=4, jacobian="host")
    Jd, gd = design_gradients(des, ps, 0.1, 0.01, 215.0, checkpoint=4, jacobian="device")
    np.testing.assert_allclose(Jd, Jh, rtol=1e-11)
    for d in range(2):
        assert np.all(np.abs(gd[d] - gh[d]) <= 1e-8 * np.abs(gh[d]) + 1e-12 * np.abs(gh[d]).max()), (gd[d], gh[d])


def test_bad_records_are_argument_errors():
    _, dipole = W.build_single_dipole()
    rec = engine.layer_record(dipole)
    dev = engine._device()
    kls = torch.empty((dipole.total_disperse_number, 3), dtype=torch.float64, device=dev)
    p0s = torch.empty_like(kls)
    lib = _lib.load()
    bad = rec.copy()
    bad[13] = bad[12] + 0.1          # small_r >= big_r
    t = torch.as_tensor(bad, device=dev)
    assert lib.cct_segments_build(t.data_ptr(), 1, kls.data_ptr(), p0s.data_ptr(), kls.shape[0],
                                  engine._stream()) == _lib.CCT_ERR_ARG
    assert "small_r" in _lib.last_error()
    t = torch.as_tensor(rec, device=dev)
    assert lib.cct_segments_build(t.data_ptr(), 1, kls.data_ptr(), p0s.data_ptr(), kls.shape[0] - 1,
                                  engine._stream()) == _lib.CCT_ERR_ARG
    assert "segments" in _lib.last_error()
    # the context is still usable
    assert lib.cct_segments_build(t.data_ptr(), 1, kls.data_ptr(), p0s.data_ptr(), kls.shape[0],
                                  engine._stream()) == _lib.CCT_OK
