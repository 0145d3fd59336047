"""The tracking work split (cct_track's planner), checked on the host without a device.

A unit is (design, particle block of G, chunk of ct tiles of 128 segments).  The planner
must cover every tile of every design exactly once with one chunk size for the whole
population, keep each (design, block) within 4096 chunks and the unit count within the
scratch bound, and give every CTA work when there is enough of it.
"""
import ctypes

import numpy as np
import pytest

from cctpy_gb300 import _lib

TILE = 128
MAX_CHUNKS = 4096
MIN_CHUNK_TILES = 32
UNITS_PER_CTA = 8


@pytest.fixture(scope="module")
def lib():
    try:
        return _lib.load()
    except ImportError as e:
        pytest.skip(str(e))


def plan(lib, seg_counts, n_p, precision, grid, max_units=0):
    off = np.concatenate([[0], np.cumsum(seg_counts)]).astype(np.int64)
    n = len(seg_counts)
    unit_off = np.zeros(n + 1, np.int64)
    chunks = np.zeros(n, np.int64)
    ct = np.zeros(n, np.int64)
    g = ctypes.c_int32(0)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    units = lib.cct_test_plan_units(p(off), n, n_p, precision, grid, max_units, p(unit_off), p(chunks), p(ct),
                                    ctypes.byref(g))
    return units, unit_off, chunks, ct, g.value


def expected_group(precision, n_p):
    if n_p <= 16:              # half-warp blocks for designs of at most 16 particles
        return 16
    if precision == 0:
        return 32
    best, slots = 256, -(-n_p // 256) * 256
    for G in (128, 64, 32):
        s = -(-n_p // G) * G
        if s < slots:
            best, slots = G, s
    return best


def check_plan(lib, seg_counts, n_p, precision, grid):
    units, unit_off, chunks, ct, G = plan(lib, seg_counts, n_p, precision, grid)
    assert G == expected_group(precision, n_p)
    blocks = -(-n_p // G)
    nts = [-(-s // TILE) for s in seg_counts]
    bound = UNITS_PER_CTA * grid + len(seg_counts) * blocks
    assert 0 < units <= bound
    assert unit_off[0] == 0 and unit_off[-1] == units
    sizes = {int(c) for c, nt in zip(ct, nts) if nt > 0}
    assert len(sizes) <= 1, "one chunk size for every design"
    for d, nt in enumerate(nts):
        assert unit_off[d + 1] - unit_off[d] == blocks * chunks[d]
        assert 1 <= chunks[d] <= MAX_CHUNKS
        if nt == 0:
            assert chunks[d] == 1 and ct[d] == 1
        else:
            assert chunks[d] * ct[d] >= nt, "every tile covered"
            assert (chunks[d] - 1) * ct[d] < nt, "no empty chunk"
    work = blocks * sum(max(nt, 1) for nt in nts)
    target = max(grid, min(UNITS_PER_CTA * grid, -(-work // MIN_CHUNK_TILES)))
    # one chunk size: at most the target plus one short chunk per (design, block)
    assert units <= target + len(seg_counts) * blocks
    # every CTA gets work when there is enough of it
    assert units >= min(target, work) // 2
    return units, int(max(ct))


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("grid", [1, 152, 456, 4096])
def test_random_populations(lib, precision, grid):
    rng = np.random.default_rng(7 + grid + precision)
    for _ in range(60):
        n = int(rng.integers(1, 70))
        kind = rng.integers(0, 4)
        if kind == 0:      # uneven optimisation population
            segs = rng.integers(200_000, 700_000, n)
        elif kind == 1:    # small and ragged, with empty designs
            segs = rng.integers(0, 3 * TILE, n)
        elif kind == 2:    # whole tiles
            segs = TILE * rng.integers(1, 400, n)
        else:              # a single segment each
            segs = np.ones(n, np.int64)
        n_p = int(rng.choice([1, 31, 32, 33, 96, 100, 257, 512, 1024, 4096, 5000]))
        check_plan(lib, [int(s) for s in segs], n_p, precision, grid)


def test_headline_workloads(lib):
    # gantry section: one design of 597 600 segments, 4096 protons, FP32c, 456 CTAs
    units, ct = check_plan(lib, [597_600], 4096, 1, 456)
    assert ct >= MIN_CHUNK_TILES and units >= 456
    # single dipole: 46 080 segments (360 tiles), 32 protons, fewer tiles than CTAs: a tile a unit
    units, ct = check_plan(lib, [46_080], 32, 1, 456)
    assert units == 360 and ct == 1
    # a design population with an empty design among them
    check_plan(lib, [358_560, 0, 119_520, 1], 512, 1, 456)


def test_one_chunk_per_block_is_the_floor(lib):
    segs, n_p, grid = [50_000, 20_000, 5], 1000, 456
    G = expected_group(1, n_p)
    least = len(segs) * -(-n_p // G)
    units, unit_off, chunks, ct, _ = plan(lib, segs, n_p, 1, grid, max_units=least)
    assert units == least and list(chunks) == [1, 1, 1]
    assert plan(lib, segs, n_p, 1, grid, max_units=least - 1)[0] == -1
    # a tighter cap than the default is kept
    cap = least + 10
    assert least <= plan(lib, segs, n_p, 1, grid, max_units=cap)[0] <= cap


def test_units_per_cta_setting(lib):
    try:
        _lib.check(lib.cct_track_set_units_per_cta(2), "set")
        u2 = plan(lib, [597_600], 4096, 1, 456)[0]
        _lib.check(lib.cct_track_set_units_per_cta(32), "set")
        u32 = plan(lib, [597_600], 4096, 1, 456)[0]
        assert u2 < u32 <= 32 * 456 + 16
        assert lib.cct_track_set_units_per_cta(65) == _lib.CCT_ERR_ARG
    finally:
        lib.cct_track_set_units_per_cta(0)
    assert lib.cct_track_units_per_cta() == UNITS_PER_CTA


def test_bad_arguments(lib):
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    t = np.zeros(8, np.int64)
    g = ctypes.c_int32(0)
    dec = np.array([0, 10, 5], np.int64)
    assert lib.cct_test_plan_units(p(dec), 2, 10, 1, 456, 0, p(t), p(t), p(t), ctypes.byref(g)) == -2
    assert "decrease" in _lib.last_error()
    ok = np.array([0, 10], np.int64)
    assert lib.cct_test_plan_units(p(ok), 1, 10, 2, 456, 0, p(t), p(t), p(t), ctypes.byref(g)) == -2
    assert lib.cct_test_plan_units(p(ok), 1, 0, 1, 456, 0, p(t), p(t), p(t), ctypes.byref(g)) == -2
    assert lib.cct_test_plan_units(p(ok), 1, 10, 1, 0, 0, p(t), p(t), p(t), ctypes.byref(g)) == -2


def test_particle_block_setting(lib):
    """The FP32c particle block set by hand (or by cct_autotune) is the one the planner uses;
    FP64 keeps blocks of 32; 0 restores the automatic choice; other sizes are refused."""
    try:
        assert lib.cct_track_particle_block() == 0
        assert plan(lib, [46080], 4096, 1, 456)[4] == 256
        for g in (16, 32, 64, 128, 256):
            assert lib.cct_track_set_particle_block(g) == _lib.CCT_OK
            assert lib.cct_track_particle_block() == g
            units, unit_off, chunks, ct, got = plan(lib, [46080, 12345], 4096, 1, 456)
            assert got == g
            assert units == unit_off[-1] and np.all(unit_off[1:] - unit_off[:-1] == (4096 // g) * chunks)
            assert plan(lib, [46080], 4096, 0, 456)[4] == 32
        for bad in (-1, 8, 48, 512):
            assert lib.cct_track_set_particle_block(bad) == _lib.CCT_ERR_ARG
        assert lib.cct_track_particle_block() == 256          # a refused value leaves the setting alone
        # every split the autotuner tries fits the scratch it asks for
        need = lib.cct_autotune_scratch_bytes(1, 4096)
        for g in (16, 32, 64, 128, 256):
            lib.cct_track_set_particle_block(g)
            assert need >= lib.cct_track_scratch_bytes(1, 4096) + 80 * 4096
    finally:
        lib.cct_track_set_particle_block(0)
    assert lib.cct_track_particle_block() == 0
    assert plan(lib, [46080], 100, 1, 456)[4] == 128


def test_adjoint_scratch_ignores_the_particle_block_setting(lib):
    """cct_track_adjoint plans with the automatic particle block whatever the forward entry
    points are set to, so its scratch query must not follow the setting (a query made after
    cct_autotune once returned too little)."""
    want = lib.cct_adjoint_scratch_bytes(16, 1024, 3, 2)
    try:
        for g in (32, 64, 128, 256):
            lib.cct_track_set_particle_block(g)
            assert lib.cct_adjoint_scratch_bytes(16, 1024, 3, 2) == want
    finally:
        lib.cct_track_set_particle_block(0)


def test_small_fp32c_batches_plan_one_unit_per_cta(lib):
    """FP32c batches of at most 64 particles in fewer than eight particle blocks run the
    small-batch schedule, in which every CTA keeps one unit for the whole launch: the planner
    gives them at most one unit a CTA, covering every tile; FP64 and larger batches keep the
    usual split (here: more units than CTAs)."""
    grid = 100
    for seg_counts, n_p in (([597600], 32), ([46080], 32), ([119520, 200000], 16), ([46080] * 4, 16)):
        units, unit_off, chunks, ct, g = plan(lib, seg_counts, n_p, 1, grid)
        assert 0 < units <= grid, (seg_counts, n_p, units)
        for d, n in enumerate(seg_counts):
            tiles = -(-n // TILE)
            assert chunks[d] * ct[d] >= tiles and (chunks[d] - 1) * ct[d] < tiles
    assert plan(lib, [597600], 32, 0, grid)[0] > grid          # FP64: not the small-batch schedule
    assert plan(lib, [597600], 65, 1, grid)[0] > grid          # more than 64 particles


def test_half_warp_blocks_for_designs_of_up_to_16_particles(lib):
    """Designs of at most 16 particles get blocks of 16 in both precisions (a particle per
    half-warp lane, so that no lane idles); 17 particles keep blocks of 32."""
    for n_p in (1, 5, 16):
        assert plan(lib, [24000] * 100, n_p, 1, 456)[4] == 16
        assert plan(lib, [24000] * 100, n_p, 0, 456)[4] == 16
    assert plan(lib, [24000] * 100, 17, 1, 456)[4] == 32
    assert plan(lib, [24000] * 100, 17, 0, 456)[4] == 32
    units, unit_off, chunks, ct, g = plan(lib, [24000] * 100, 16, 1, 456)
    assert units == unit_off[-1] and np.all(unit_off[1:] - unit_off[:-1] == chunks)
