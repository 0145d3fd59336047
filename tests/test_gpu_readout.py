"""Optimiser read-out on the GPU (cct_beam_readout) against the reference's own values
(golden_readout.npz), and one generation evaluated on the device against the oracle's
read-out of the same tracked protons."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from cctpy_gb300 import HUST_SC_GANTRY, ParticleFactory, engine, workloads as W
from cctpy_gb300.optim import GenerationEvaluator, a05_phase_space, beam_readout
from cctpy_gb300.particles import particles_to_array
from oracle import cct_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gr():
    return np.load(os.path.join(HERE, "golden", "golden_readout.npz"))


def test_readout_bitwise_vs_reference(gr):
    ps, obj = beam_readout(gr["finals"], gr["ideal_end"], int(gr["group"][0]), frame=gr["frame"].reshape(-1))
    np.testing.assert_array_equal(ps, gr["phase_space"])
    np.testing.assert_array_equal(obj, gr["objectives"])


def test_readout_with_own_frame_and_device_tensors(gr):
    f = torch.as_tensor(gr["finals"], device="cuda")
    ps, obj = beam_readout(f, gr["ideal_end"], int(gr["group"][0]))
    assert ps.is_cuda and obj.is_cuda
    np.testing.assert_allclose(obj.cpu().numpy(), gr["objectives"], rtol=1e-12, atol=1e-12)


def test_readout_ragged_group_and_no_speed_reset(gr):
    fr = O.Frame.from_axes((0.0, 0.0, 0.0), *[tuple(r) for r in gr["frame"]])
    finals = gr["finals"][:, :91]                       # 91 = 7 groups of 12 + a group of 7
    _, obj = beam_readout(finals, gr["ideal_end"], 12, speed_from_velocity=False, frame=gr["frame"].reshape(-1))
    for d in range(finals.shape[0]):
        want, _ = O.beam_objectives(gr["ideal_end"], fr, finals[d], 12, speed_from_velocity=False)
        np.testing.assert_array_equal(obj[d], np.array(want))


def test_generation_on_device_matches_oracle_readout():
    kws = W.design_population(2, seed=3, part_per_winding=60)
    params = np.arange(2)[:, None]

    def make(row):
        return HUST_SC_GANTRY(**kws[int(row[0])]).create_second_bending_part_beamline()

    bl0 = make(params[0])
    ip = ParticleFactory.create_proton_along(bl0, 0.0, 215.0)
    beam = ParticleFactory.create_from_phase_space_particles(ip, ip.get_natural_coordinate_system(), a05_phase_space())
    L, step = 0.2, 0.05
    ip_end = ParticleFactory.create_proton_along(bl0, L, 215.0)
    ev = GenerationEvaluator(make, beam, L, step, ip_end, precision="f64")
    obj = ev(params)
    assert obj.shape == (2, 11)
    final = engine.track(ev.last_design_set, particles_to_array(beam), L, step, "f64")
    rec = ip_end.to_numpy_array_data()
    cs = ip_end.get_natural_coordinate_system()
    fr = O.Frame.from_axes(tuple(rec[0:3]), tuple(cs.XI.to_list()), tuple(cs.YI.to_list()), tuple(cs.ZI.to_list()))
    for d in range(2):
        want, _ = O.beam_objectives(rec, fr, final[d], 12)
        np.testing.assert_array_equal(obj[d], np.array(want))
    # the FP32-compensated generation agrees to the tracking tolerance (1 um, ~1e-6 mrad)
    obj32 = GenerationEvaluator(make, beam, L, step, ip_end, precision="f32c")(params)
    np.testing.assert_allclose(obj32, obj, rtol=1e-5, atol=1e-5)
