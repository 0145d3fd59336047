"""Golden fixture of the beamline of cctpy's GPU speed test, generated from the cctpy reference
itself (final_code/work/小论文2回复/CPU和CPU代码速度测试.py:36-52, the AG-CCT builder
beamline.py:576-793, the QS builder and its record magnets.py:726-748), so that the
workload the same-GPU comparison with cctpy's own kernel runs is pinned to cctpy's geometry:
the track length, the segment count of every CCT layer, every 97th segment (kl and midpoint,
global frame) and the QS record, all as cctpy exports them to its GPU kernel
(`global_current_elements_and_elementary_current_positions`, cct.py:434-457).

    CCTPY_REFERENCE=<cctpy checkout> python tests/golden/make_golden_speedtest.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import load_reference  # noqa: E402

STRIDE = 97


def main():
    load_reference()
    from packages.beamline import Beamline
    from packages.cct import CCT
    from packages.constants import MM
    from packages.magnets import QS
    from packages.point import P2

    bl = (Beamline.set_start_point(P2.origin()).first_drift(direct=P2.x_direct(), length=5)
          .append_agcct(big_r=1.0, small_rs=[200 * MM, 180 * MM, 160 * MM, 140 * MM],
                        bending_angles=[10, 10, 15, 15], tilt_angles=[[30], [90, 30]],
                        winding_numbers=[[50], [10, 10, 15, 15]], currents=[10000, 10000])
          .append_drift(2).append_qs(length=1, gradient=0, second_gradient=0, aperture_radius=200 * MM)
          .append_drift(2))
    kls, p0s, counts, qs = [], [], [], []
    for m in bl.magnets:
        if isinstance(m, CCT):
            kl, p0 = m.global_current_elements_and_elementary_current_positions(np.float64)
            kls.append(np.asarray(kl).reshape(-1, 3))
            p0s.append(np.asarray(p0).reshape(-1, 3))
            counts.append(kls[-1].shape[0])
        elif isinstance(m, QS):
            qs.append(np.asarray(m.to_numpy_array(np.float64)))
    kl = np.concatenate(kls)
    p0 = np.concatenate(p0s)
    idx = np.arange(0, kl.shape[0], STRIDE)
    np.savez_compressed(os.path.join(HERE, "golden_speedtest.npz"), length=np.array([bl.get_length()]),
                        layer_counts=np.array(counts), idx=idx, kl=kl[idx], p0=p0[idx], qs=np.stack(qs),
                        kl_sum=kl.sum(axis=0), p0_sum=p0.sum(axis=0))
    print(f"length {bl.get_length()}, layers {counts}, {kl.shape[0]} segments, {len(qs)} QS")


if __name__ == "__main__":
    main()
