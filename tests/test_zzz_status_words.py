"""The status word of the FP32c field kernels (cct_field_status): clear after good calls; a
buffer that is not a packed set, or a design index the set does not hold, gives NaN fields
and CCT_ERR_ARG once, after which the status is clear again.  Neither case issues a tile copy:
the kernel reads the set's 16-byte header, finds no match and writes NaN."""
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from cctpy_gb300 import _lib, engine, workloads as W


def test_field_status_reports_foreign_buffers_once():
    lib = _lib.load()
    _, cct = W.build_single_dipole()
    ds = engine.design_of(cct)
    pts = torch.from_numpy(W.field_map_points(1000, seed=5)).cuda()
    lib.cct_field_status(engine._stream())          # start clear
    b = engine.field_at_points(ds, pts, "f32c")
    assert bool(torch.isfinite(b).all())
    engine.field_status()

    foreign = torch.zeros(1 << 12, dtype=torch.uint8, device=pts.device)
    assert foreign.data_ptr() % 256 == 0
    for packed, design in ((foreign, 0), (ds.packed(), 1)):
        out = torch.zeros_like(pts)
        rc = lib.cct_field_f32c(packed.data_ptr(), design, None, 0, pts.data_ptr(), pts.shape[0], out.data_ptr(),
                                engine._stream())
        assert rc == _lib.CCT_OK                     # asynchronous: the kernel finds out
        with pytest.raises(ValueError, match="not a packed segment set"):
            engine.field_status()
        assert bool(torch.isnan(out).all())
        engine.field_status()                        # read once, then clear
