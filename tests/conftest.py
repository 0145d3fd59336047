import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libcctgpu")
    config.addinivalue_line("markers", "slow: CPU oracle runs of tens of seconds")


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(os.path.join(GOLDEN, "golden.npz")))


@pytest.fixture(scope="session")
def golden_hust1():
    """The gantry's first bending section and the whole gantry from the reference
    (make_golden_hust1.py)."""
    g = dict(np.load(os.path.join(GOLDEN, "golden_hust1.npz")))
    with open(os.path.join(GOLDEN, "records_hust1.json")) as f:
        recs = json.load(f)
    g["records"] = recs["hust1_default"]
    g["records_total"] = recs["total_default"]
    return g


@pytest.fixture(scope="session")
def records_json():
    with open(os.path.join(GOLDEN, "records.json")) as f:
        return json.load(f)


def oracle_records(recs):
    """Reference-built magnet records (records.json) as oracle records."""
    from oracle import cct_oracle as O
    out = []
    for r in recs:
        fr = O.Frame.from_axes(*[tuple(v) for v in r["frame"]])
        if r["kind"] == "cct":
            out.append(O.cct_record(fr, r["big_r"], r["small_r"], r["bending_angle"], r["tilt_angles"],
                                    r["winding_number"], r["current"], tuple(r["start"]), tuple(r["end"]),
                                    r["dpw"]))
        else:
            out.append(O.qs_record(fr, r["length"], r["gradient"], r["second_gradient"], r["aperture_radius"]))
    return out


def reference_design(recs):
    """(kls (N, 3), p0s (N, 3), analytic records (M, 16)) of a magnet list as cctpy itself
    places it: the oracle's segment generation (a plain-float restatement of cct.py:87-164,
    :423-457, bitwise equal to the reference) from the frames cctpy recorded.  These arrays do
    not depend on the host's BLAS, unlike the package's own placement, whose least-squares
    circle fit (numpy, as cctpy's base_utils.py:124-151) lands frames a few 1e-13 m apart on
    different CPUs."""
    from oracle import cct_oracle as O
    kls, p0s, qs = [], [], []
    for r in oracle_records(recs):
        if r["kind"] == "cct":
            k, p = O.cct_segments_global(r)
            kls.append(k)
            p0s.append(p)
        else:
            qs.append(O.QSOracle(r).to_array())
    return (np.ascontiguousarray(np.concatenate(kls)), np.ascontiguousarray(np.concatenate(p0s)),
            np.ascontiguousarray(np.array(qs).reshape(-1, 16)))
