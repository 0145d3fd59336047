"""The beamline of cctpy's GPU speed test as this package builds it
(`workloads.build_speed_test_beamline`) against cctpy's own construction of it
(`tests/golden/golden_speedtest.npz`, made by `tests/golden/make_golden_speedtest.py` from
cctpy itself): the workload on which the engine is compared with cctpy's own CUDA kernel must
be cctpy's geometry.  Track length, segment count of every CCT layer, every 97th segment (kl
and midpoint, as cctpy exports them to its kernel), the sums of all segments and the QS
record agree to 1e-12 (bit for bit on x86; the tolerance covers the BLAS of other hosts in the
least-squares circle fit that places magnets)."""
import os

import numpy as np

from cctpy_gb300 import engine, workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))


def test_speed_test_beamline_matches_cctpy():
    g = np.load(os.path.join(HERE, "golden", "golden_speedtest.npz"))
    bl = W.build_speed_test_beamline()
    assert abs(bl.get_length() - g["length"][0]) < 1e-12
    mags = engine.magnet_list(bl)
    layers = [engine.cct_global_segments(m)[0].shape[0] for m in mags if engine._classify(m) == "cct"]
    assert layers == [int(c) for c in g["layer_counts"]]
    kl, p0, qs = engine.host_design(mags)
    assert kl.shape[0] == sum(layers) == 24000
    scale = np.abs(g["kl"]).max()
    np.testing.assert_allclose(kl[g["idx"]], g["kl"], rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(p0[g["idx"]], g["p0"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(kl.sum(axis=0), g["kl_sum"], rtol=0, atol=1e-12 * scale * kl.shape[0])
    np.testing.assert_allclose(p0.sum(axis=0), g["p0_sum"], rtol=0, atol=1e-12 * p0.shape[0])
    np.testing.assert_allclose(qs, g["qs"], rtol=0, atol=1e-12)
    # the other currents of the same builder scale kl only
    bl2 = W.build_speed_test_beamline(currents=(5000.0, 20000.0))
    kl2, p02, _ = engine.host_design(engine.magnet_list(bl2))
    np.testing.assert_array_equal(p02, p0)
    np.testing.assert_allclose(kl2[:12000], 0.5 * kl[:12000], rtol=1e-14)
    np.testing.assert_allclose(kl2[12000:], 2.0 * kl[12000:], rtol=1e-14)
