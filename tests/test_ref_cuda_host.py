"""The checker side of the same-GPU comparison with cctpy's own CUDA kernel, on the host.

The recipe (``oracle/ref_cuda_build.py``) compiles both of cctpy's configurations for sm_103a
with register counts that fit their block sizes and leaves no kernel source in the repository;
the packing follows cctpy's GPU layout (gpu_accelerator.py:1953-2016: per beamline, segment
arrays padded to the compiled capacity, QS records likewise, the same particles for every
beamline) and refuses what those capacities cannot hold.
"""
import os

import numpy as np
import pytest

import __graft_entry__ as G
from oracle import ref_cuda, ref_cuda_build


def test_recipe_builds_every_configuration():
    if not os.path.isdir(os.path.join(G.REFERENCE_TREE, "final_code")):
        pytest.skip("cctpy's sources are not on this machine")
    meta = ref_cuda_build.build(G.REFERENCE_TREE)
    assert meta["kernel"] == "track_multi_particle_beamline_for_magnet_with_multi_qs"
    assert set(meta["configs"]) == {"f32", "f64", "f32_700k", "f64_700k"}
    for name, block, width, cap in (("f32", 1024, 4, 240000), ("f64", 512, 8, 240000), ("f32_700k", 1024, 4, 700000),
                                    ("f64_700k", 512, 8, 700000)):
        c = meta["configs"][name]
        assert c["block"] == block and c["float_bytes"] == width
        assert c["registers"] is not None and c["registers"] * block <= 65536
        assert c["max_current_element_number"] == cap and c["max_qs_datas_length"] == 10000
        assert os.path.getsize(os.path.join(ref_cuda.REF_DIR, c["cubin"])) > 0
    assert not [f for f in os.listdir(ref_cuda.REF_DIR) if f.endswith((".cu", ".cuh", ".py", ".c"))]
    assert ref_cuda.available()
    assert ref_cuda_build.build(G.REFERENCE_TREE) == meta      # cached: the same source is not rebuilt


def test_packing_follows_cctpys_layout():
    rng = np.random.default_rng(0)
    designs = [(rng.normal(size=(5, 3)), rng.normal(size=(5, 3)), rng.normal(size=(1, 16))),
               (rng.normal(size=(3, 3)), rng.normal(size=(3, 3)), np.zeros((0, 16)))]
    parts = rng.normal(size=(4, 10))
    h = ref_cuda.pack(designs, parts, 8, 2, np.float32)
    assert h["kls"].shape == h["p0s"].shape == (2, 24) and h["qs"].shape == (2, 32)
    assert all(h[k].dtype == np.float32 for k in ("kls", "p0s", "qs", "particles"))
    assert list(h["n_ce"]) == [5, 3] and list(h["n_qs"]) == [1, 0] and list(h["n_p"]) == [4]
    for d, (k, p, q) in enumerate(designs):
        n = k.size
        np.testing.assert_array_equal(h["kls"][d, :n], k.reshape(-1).astype(np.float32))
        np.testing.assert_array_equal(h["p0s"][d, :n], p.reshape(-1).astype(np.float32))
        assert not h["kls"][d, n:].any() and not h["p0s"][d, n:].any()
        np.testing.assert_array_equal(h["qs"][d, :q.size], q.reshape(-1).astype(np.float32))
        assert not h["qs"][d, q.size:].any()
    np.testing.assert_array_equal(h["particles"].reshape(2, 4, 10), np.stack([parts, parts]).astype(np.float32))
    h64 = ref_cuda.pack(designs, parts, 5, 1, np.float64)       # exactly at the capacities
    np.testing.assert_array_equal(h64["particles"][:4], parts)


def test_packing_refuses_what_the_kernel_cannot_hold():
    rng = np.random.default_rng(1)
    parts = rng.normal(size=(2, 10))
    seg = lambda n: (rng.normal(size=(n, 3)), rng.normal(size=(n, 3)), np.zeros((0, 16)))
    with pytest.raises(ValueError, match="capacities"):
        ref_cuda.pack([seg(9)], parts, 8, 2, np.float64)
    with pytest.raises(ValueError, match="capacities"):
        ref_cuda.pack([(*seg(2)[:2], np.zeros((3, 16)))], parts, 8, 2, np.float64)
    with pytest.raises(ValueError):
        ref_cuda.pack([], parts, 8, 2, np.float64)
    with pytest.raises(ValueError):
        ref_cuda.pack([seg(2)], np.zeros((0, 10)), 8, 2, np.float64)
    with pytest.raises(ValueError):
        ref_cuda.pack([(np.zeros((2, 3)), np.zeros((3, 3)), np.zeros((0, 16)))], parts, 8, 2, np.float64)


def test_single_qs_packing_keeps_each_beamlines_last_qs():
    rng = np.random.default_rng(2)
    parts = rng.normal(size=(3, 10))
    q3, q1 = rng.normal(size=(3, 16)), rng.normal(size=(1, 16))
    designs = [(rng.normal(size=(4, 3)), rng.normal(size=(4, 3)), q3),
               (rng.normal(size=(2, 3)), rng.normal(size=(2, 3)), q1)]
    h = ref_cuda.pack(designs, parts, 8, 4, np.float64, single_qs=True)
    assert h["qs"].shape == (2, 16)
    np.testing.assert_array_equal(h["qs"][0], q3[2])
    np.testing.assert_array_equal(h["qs"][1], q1[0])
    np.testing.assert_array_equal(h["kls"][0, :12], designs[0][0].reshape(-1))
    with pytest.raises(ValueError, match="single-QS"):
        ref_cuda.pack([(designs[0][0], designs[0][1], np.zeros((0, 16)))], parts, 8, 4, np.float64, single_qs=True)
    assert set(ref_cuda.KERNELS) == {"multi_qs", "single_qs"}
    assert len(ref_cuda.KERNELS["single_qs"][1]) == 8 and len(ref_cuda.KERNELS["multi_qs"][1]) == 9
