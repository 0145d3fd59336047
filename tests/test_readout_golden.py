"""Optimiser read-out pinned to the reference: the oracle's phase space and beam
objectives, and this package's beam set-up, against tests/golden/golden_readout.npz
(generated from cctpy itself by tests/golden/make_golden_readout.py)."""
import os

import numpy as np
import pytest

from oracle import cct_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gr():
    return np.load(os.path.join(HERE, "golden", "golden_readout.npz"))


def test_oracle_readout_bitwise(gr):
    fr = O.Frame.from_axes((0.0, 0.0, 0.0), *[tuple(r) for r in gr["frame"]])
    for d in range(gr["finals"].shape[0]):
        obj, rows = O.beam_objectives(gr["ideal_end"], fr, gr["finals"][d], int(gr["group"][0]))
        np.testing.assert_array_equal(np.array(rows), gr["phase_space"][d])
        np.testing.assert_array_equal(np.array(obj), gr["objectives"][d])


def test_oracle_readout_plants_are_caught(gr):
    """A planted change in the statistics (plain instead of compensated mean) is visible."""
    fr = O.Frame.from_axes((0.0, 0.0, 0.0), *[tuple(r) for r in gr["frame"]])
    obj, rows = O.beam_objectives(gr["ideal_end"], fr, gr["finals"][0], int(gr["group"][0]))
    xs = [r[0] / O.MM for r in rows]
    s = 0.0
    for t in xs:
        s = s + t
    plain = abs(s / len(xs))
    assert plain != gr["objectives"][0][4] and obj[4] == gr["objectives"][0][4]


def test_a05_beam_matches_reference(gr):
    from cctpy_gb300.optim import a05_phase_space
    rows = np.array([p.to_list() for p in a05_phase_space()])
    np.testing.assert_array_equal(rows, gr["ps_in"])
