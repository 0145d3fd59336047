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
