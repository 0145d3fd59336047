"""Benchmark: Biot-Savart Gpairs/s on the field-map workload, FP32-compensated vs FP64.

Workload (one step): the field of the single CCT bending dipole (46 080 winding
segments: R 0.95 m, r 83 mm, 22.5 deg, tilts [30, 80, 90, 90], 128 turns x 360,
9000 A) at 2**20 seeded points uniform in a 60 mm tube around its design arc:
2**20 x 46 080 = 4.832e10 pairs per step.  Synthetic inputs stand in for
measured data (there is none in the reference for this path).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  `value` = FP32c Gpairs/s with inputs resident in HBM
(device-timed; L2 flushed between steps); `e2e` = the same metric through the
package's public call with pinned host points and a host result (copies inside
the timed region); `fp64` = the plain FP64 drop-in on the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

N_POINTS = 1 << 20
N_SEG = 46080
FLOPS_PER_PAIR = 26
# DRAM bytes (read + write) of one field_f32c_kernel launch on the field map, from an ncu
# capture of this bench's field-map run (dram__bytes.sum.per_second x gpu__time_duration.sum):
# the 25 MB of points and 1.7 MB of tiles read; the 25 MB of fields written are still in L2
# when the kernel ends.
FIELD_MAP_TRAFFIC_BYTES = 26.96e6
METRIC = "Biot-Savart Gpairs/s & design-grads/s, 1 GB300: FP32+comp vs FP64 @1e-7 rel"
WORKLOAD = "field_map: 2^20 points x 46080-segment single CCT dipole"


def rank_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9 and f[1].replace(".", "").isdigit():
                    rows.append(f)
        except OSError:
            pass
        finally:
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"], "samples": 0}
        sm = [float(r[1]) for r in rows]
        mx = max(float(r[2]) for r in rows)
        busy = [s for s in sm if s > 0.5 * mx] or sm
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())}


# ---------------------------------------------------------------- CPU oracle (reference arm / cpu_baseline)
def oracle_single_dipole():
    """The oracle's record of the single dipole (the field-map and C0 magnet)."""
    from oracle import cct_oracle as O
    from cctpy_gb300 import workloads as W
    c = W.SINGLE_DIPOLE
    orb = O.Orbit((0.0, 0.0), (1.0, 0.0), c["drift"]).add_arc(c["big_r"], c["clockwise"], c["bending_angle"])
    return O.cct_along(orb, c["drift"], c["big_r"], c["small_r"], c["bending_angle"], c["tilt_angles"],
                       c["winding_number"], c["current"], (0.0, 0.0),
                       (2 * math.pi * c["winding_number"], O.deg2rad(-c["bending_angle"])),
                       c["disperse_number_per_winding"])


def oracle_pool(processes: int):
    """Spawn-started pool of oracle workers holding the single dipole, built once: the timed
    CPU legs then measure field sums and RK4 steps, not pool start-up."""
    from oracle import cct_oracle as O
    return O.OraclePool([oracle_single_dipole()], processes)


def oracle_field_sample(pool, n_points: int, seed: int):
    """Time the CPU oracle (numpy restatement of cctpy's CCT.magnetic_field_at) over the pool on
    n_points points of the field-map workload.  Returns (pairs/s, seconds, points, fields)."""
    from cctpy_gb300 import workloads as W
    pts = W.field_map_points(n_points, seed=seed)
    t0 = time.perf_counter()
    B = pool.field(pts)
    dt = time.perf_counter() - t0
    return n_points * N_SEG / dt, dt, pts, B


def oracle_track_sample(pool, n_protons: int):
    """Time the oracle's RK4 track (cctpy's ParticleRunner.run_only path: particles.py:562-596
    with the RK4 of base_utils.py:264-311) of n_protons C0 protons through the whole single-dipole
    arc at 1 mm, one proton per worker.  Returns (particle-steps/s, seconds, steps, inputs, outputs)."""
    from cctpy_gb300 import workloads as W
    ps = W.single_dipole_particles(n_protons, seed=0)
    L = W.single_dipole_track_length()
    steps = int(np.ceil(L / 0.001))
    t0 = time.perf_counter()
    out = pool.track(ps, L, 0.001)
    dt = time.perf_counter() - t0
    return n_protons * steps / dt, dt, steps, ps, out


def run_reference(args):
    rank, world, _ = rank_info()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    n = args.ref_points
    with oracle_pool(cores) as pool:
        for k in range(max(args.warmup, 0)):   # untimed: workers page in numpy and the segments
            oracle_field_sample(pool, max(cores * 4, 64), seed=100 + k)
        times = []
        for k in range(args.steps):
            times.append(oracle_field_sample(pool, n, seed=200 + k)[1])
    value = (n * N_SEG * args.steps) / sum(times) / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Gpairs/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "n_points_per_step": n, "n_segments": N_SEG,
                       "sample": f"{n} of the 2^20 field points per step"},
            "cpu_baseline": {"value": value, "unit": "Gpairs/s", "cores": cores, "kind": "port",
                             "sample": f"{n} points x {N_SEG} segments per step, {args.steps} steps, over a "
                                       f"{cores}-process pool started and warmed before the timed steps"},
            "e2e": {"value": value, "unit": "Gpairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- tracking (beside the headline)
def measure_tracking(args, dev, rank):
    """RK4 tracking throughput, FP32c vs FP64, over equal windows (same steps, same
    repetitions, best of them): C0 whole, and slices of C2 (the gantry section: 597 600
    segments, 4096 protons, 1 mm steps) and C3 (64 second-section designs of uneven segment
    counts, 512 protons each, one launch; also through cct_track_async captured once in a CUDA
    graph and replayed).  The cost of a step does not depend on the track length, so a few
    steps stand for the 3.5 m track.  Returns a dict of particle-steps/s and Gpairs/s."""
    import torch
    from cctpy_gb300 import HUST_SC_GANTRY, engine, workloads as W

    def timed(ds, ps, steps, prec, reps):
        engine.track(ds, ps, 0.002, 0.001, prec)          # warm-up (2 steps)
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(reps):
            t0 = time.perf_counter()
            engine.track(ds, ps, steps * 0.001, 0.001, prec)
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        return best

    def tuned(ds_, ps_, steps, n_p, reps):
        """The same FP32c slice after cct_autotune picked the work split for this problem."""
        best = engine.autotune(ds_, ps_, 0.001, "f32c", steps=2)
        block = engine.particle_block()
        try:
            t = timed(ds_, ps_, steps, "f32c", reps)
        finally:
            engine.set_units_per_cta(0)
            engine.set_particle_block(0)
        r = ds_.n_designs * n_p * steps / t
        return {"units_per_cta": best, "particle_block": block or "automatic", "seconds": t,
                "particle_steps_per_s": r, "gpairs_per_s": n_p * steps * 4 * ds_.n_segments / t / 1e9}

    out = {"windows": "FP32c and FP64 timed over the same RK4 steps and repetitions (best of them), "
                      "each call with its host copies of the particle records"}
    # C0: the reference's CPU-runnable case, whole track (32 protons, 374 steps of 1 mm)
    _, dip = W.build_single_dipole()
    dsd = engine.design_of(dip)
    dsd.packed()
    p32 = W.single_dipole_particles(32, seed=0)
    L0 = W.single_dipole_track_length()
    n0 = int(np.ceil(L0 / 0.001))
    c0 = {}
    for prec in ("f32c", "f64"):
        engine.track(dsd, p32, 0.002, 0.001, prec)
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(2):
            t0 = time.perf_counter()
            engine.track(dsd, p32, L0, 0.001, prec)
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        c0[prec] = {"seconds": best, "steps": n0, "us_per_stage": best / (4 * n0) * 1e6,
                    "particle_steps_per_s": 32 * n0 / best, "gpairs_per_s": 32 * n0 * 4 * dsd.n_segments / best / 1e9}
    out["single_dipole"] = dict(
        workload=f"single CCT dipole, {dsd.n_segments} segments; 32 protons 250 MeV through the whole "
                 f"{L0:.4f} m arc at 1 mm ({n0} RK4 steps), one call, best of 2 (latency-bound: one particle block)",
        speedup_f32c_vs_f64=c0["f64"]["seconds"] / c0["f32c"]["seconds"], **c0)
    bl = W.build_gantry_section()
    ds = engine.design_of(bl)
    ds.packed()
    ps = W.beam_particles(bl, 4096, seed=2 + rank, kinetic_MeV=215.0)
    n_seg = ds.n_segments
    steps, reps = args.track_steps, 2
    res = {}
    for prec in ("f32c", "f64"):
        t = timed(ds, ps, steps, prec, reps)
        r = 4096 * steps / t
        res[prec] = {"steps": steps, "reps": reps, "seconds": t, "particle_steps_per_s": r,
                     "gpairs_per_s": r * 4 * n_seg / 1e9}
    out["gantry_section"] = dict(
        workload=f"HUST second section, AG tilts [90,30,90,90], -7000 A, {n_seg} segments + 1 QS; 4096 protons "
                 "215 MeV, 1 mm RK4 steps (one cooperative launch per call, host copies included)",
        speedup_f32c_vs_f64=res["f32c"]["particle_steps_per_s"] / res["f64"]["particle_steps_per_s"], **res)
    out["gantry_section"]["f32c_autotuned"] = tuned(ds, ps, steps, 4096, reps)
    if not args.no_population:
        bls = [HUST_SC_GANTRY(**kw).create_second_bending_part_beamline() for kw in W.design_population(64, seed=3)]
        dsp = engine.design_set_of(bls)
        dsp.packed()
        pp = W.beam_particles(bls[0], 512, seed=2 + rank, kinetic_MeV=215.0)
        psteps, preps = args.population_steps, 1     # one repetition each: FP64 takes ~20 s a call
        res = {}
        for prec in ("f32c", "f64"):
            t = timed(dsp, pp, psteps, prec, preps)
            r = 64 * 512 * psteps / t
            res[prec] = {"steps": psteps, "reps": preps, "seconds": t, "particle_steps_per_s": r,
                         "gpairs_per_s": 512 * psteps * 4 * dsp.n_segments / t / 1e9}
        segs = [dsp.segments_of(d) for d in range(64)]
        out["design_population"] = dict(
            workload=f"64 designs ({min(segs)}..{max(segs)} segments, {dsp.n_segments} total), 512 protons each, "
                     "one launch",
            speedup_f32c_vs_f64=res["f32c"]["particle_steps_per_s"] / res["f64"]["particle_steps_per_s"], **res)
        out["design_population"]["f32c_graph_replay"] = measure_graph_replay(dsp, pp, psteps)
        out["design_population"]["f32c_autotuned"] = tuned(dsp, pp, psteps, 512, preps)
    if not args.no_speed_test:
        out["reference_speed_test"] = measure_speed_test(rank)
    if not args.no_adjoint:
        out["design_gradients"] = measure_design_grads(args, rank)
    if not args.no_generation:
        out["optimiser_generation"] = measure_generation(args, rank)
    return out


def measure_population_shard(args, rank, world, dist):
    """The multi-GPU split of the tracking path: a C3-style population of 64 second-section
    designs per rank (weak scaling) cut into contiguous shards balanced by segment count
    (shard.shard_by_cost), each rank tracking its shard (FP32c, 512 protons a design, one
    launch) and reading out the eleven optimiser objectives, then one gather of the objective
    rows (shard.gather_rows) -- no collective on the data path.  Timed from a barrier to the
    gathered rows, max over ranks; design sets are built before the timed region.  With one
    GPU the same steps run without the gather."""
    import torch
    from cctpy_gb300 import HUST_SC_GANTRY, ParticleFactory, engine, workloads as W
    from cctpy_gb300.optim import beam_readout
    from cctpy_gb300.shard import gather_rows, max_over_ranks, shard_by_cost
    n = 64 * world
    kws = W.design_population(n, seed=3)
    bls_all = [HUST_SC_GANTRY(**kw).create_second_bending_part_beamline() for kw in kws]
    costs = [sum(m.total_disperse_number for m in engine.magnet_list(bl) if hasattr(m, "total_disperse_number"))
             for bl in bls_all]
    a, b = shard_by_cost(costs, world, rank) if world > 1 else (0, n)
    steps = args.population_steps
    ps = W.beam_particles(bls_all[0], 512, seed=2, kinetic_MeV=215.0)
    ip_end = ParticleFactory.create_proton_along(bls_all[0], steps * 0.001, 215.0)
    ds = engine.design_set_of(bls_all[a:b], segments="device") if b > a else None
    p0 = torch.as_tensor(np.broadcast_to(ps, (b - a,) + ps.shape).copy(), device="cuda") if b > a else None

    def step():
        if ds is None:
            local = np.zeros((0,))
        else:
            final = engine.track(ds, p0, steps * 0.001, 0.001, "f32c")
            local = beam_readout(final, ip_end, group=512)[1].cpu().numpy()
        return gather_rows(local) if world > 1 else local

    if ds is not None:
        ds.packed()
    step()                                        # warm-up
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rows = step()
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    if world > 1:
        t = max_over_ranks(t)
    return {"workload": f"{n} second-section designs (64 a GPU), 512 protons each, {steps} RK4 steps of 1 mm, FP32c, "
                        "objectives per design gathered",
            "scaling": "weak", "ranks": world, "designs_this_rank": b - a,
            "segments_this_rank": int(sum(costs[a:b])), "segments_total": int(sum(costs)),
            "seconds": t, "particle_steps_per_s": n * 512 * steps / t, "rows_gathered": int(rows.shape[0]),
            "split": "contiguous shards balanced by segment count, one all-gather of the objective rows"}


def measure_graph_replay(ds, ps, steps, replays=5):
    """C3 as configured: the population's FP32c tracking enqueued by cct_track_async (plan kernel
    + cooperative tracking launch, no host read-back), captured once in a CUDA graph and
    replayed; each replay first restores the start records (device copy, in the graph).  Timed
    with CUDA events over the replays, beside the same launch enqueued directly; both
    device-resident (the synchronous engine.track line above includes its host copies)."""
    import torch
    from cctpy_gb300 import engine
    n_p = ps.shape[0]
    start = torch.as_tensor(np.broadcast_to(ps, (ds.n_designs,) + ps.shape).copy(), device="cuda")
    p = start.clone()
    tl = engine.TrackLaunch(ds, p, steps * 0.001, 0.001, "f32c")
    tl.launch()                       # first call outside any capture (occupancy query)
    tl.status()
    direct = None
    for _ in range(2):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(replays):
            p.copy_(start)
            tl.launch()
        e1.record()
        tl.status()
        direct = e0.elapsed_time(e1) / replays / 1e3
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        p.copy_(start)
        tl.launch()
    g.replay()
    tl.status()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(replays):
        g.replay()
    e1.record()
    tl.status()
    t = e0.elapsed_time(e1) / replays / 1e3
    r = ds.n_designs * n_p * steps / t
    return {"steps": steps, "replays": replays, "seconds_per_replay": t, "particle_steps_per_s": r,
            "gpairs_per_s": n_p * steps * 4 * ds.n_segments / t / 1e9, "seconds_per_direct_launch": direct,
            "call": "engine.TrackLaunch (cct_track_async) captured by torch.cuda.graph, device-resident"}


def measure_speed_test(rank):
    """The reference's own GPU speed test (final_code/work/小论文2回复/CPU和CPU代码速度测试.py:36-198):
    100 copies of a 24 000-segment AG-CCT beamline (5 m drift, AG-CCT, 2 m drift, QS, 2 m drift;
    10.8727 m), 16 copies of the ideal 250 MeV proton each, tracked over the whole length at its
    20 mm and 2 mm steps, FP32c.  The reference reports 20 s and 68.39 s for this with 100
    blocks x 1024 threads in FP32 (its hardware unstated; including its per-call kernel
    compilation and host packing).  Timed here: the tracking call (host particle records in and
    out), the same with the design set built (host segments of 100 separately built beamlines,
    upload, FP32c packing), and the reference's own call through the drop-in accelerator
    (GPU_ACCELERATOR(FLOAT32).track_multi_particle_beamline_for_magnet_with_multi_qs with the
    speed test's arguments: one beamline object 100 times, 16 RunningParticle objects)."""
    import torch
    from cctpy_gb300 import Beamline, MM, ParticleFactory, engine
    from cctpy_gb300.geometry import P2
    from cctpy_gb300.particles import particles_to_array

    def beamline():
        return (Beamline.set_start_point(P2.origin()).first_drift(direct=P2.x_direct(), length=5)
                .append_agcct(big_r=1.0, small_rs=[200 * MM, 180 * MM, 160 * MM, 140 * MM],
                              bending_angles=[10, 10, 15, 15], tilt_angles=[[30], [90, 30]],
                              winding_numbers=[[50], [10, 10, 15, 15]], currents=[10000, 10000])
                .append_drift(2).append_qs(length=1, gradient=0, second_gradient=0, aperture_radius=200 * MM)
                .append_drift(2))

    bl = beamline()
    L = bl.get_length()
    ps = particles_to_array([ParticleFactory.create_proton_along(bl)] * 16)
    warm = engine.design_set_of([bl] * 100)
    engine.track(warm, ps, 0.04, 0.02, "f32c")
    torch.cuda.synchronize()
    out = {"workload": f"100 designs x {warm.segments_of(0)} segments (AG-CCT beamline, {L:.4f} m), 16 protons "
                       "each, whole length, FP32c (the reference's GPU speed test)"}
    from cctpy_gb300 import GPU_ACCELERATOR
    ga = GPU_ACCELERATOR(GPU_ACCELERATOR.FLOAT32)
    rps = [ParticleFactory.create_proton_along(bl) for _ in range(16)]
    ga.track_multi_particle_beamline_for_magnet_with_multi_qs([bl] * 100, rps, 0.04, 0.02)     # warm
    for step, published in ((0.02, 20.0), (0.002, 68.39)):
        n_steps = int(np.ceil(L / step))
        pairs = 100 * 16 * n_steps * 4 * warm.segments_of(0)
        t0 = time.perf_counter()
        engine.track(warm, ps, L, step, "f32c")
        torch.cuda.synchronize()
        t_track = time.perf_counter() - t0
        t0 = time.perf_counter()
        ds = engine.design_set_of([beamline() for _ in range(100)])
        ds.packed()
        engine.track(ds, ps, L, step, "f32c")
        torch.cuda.synchronize()
        t_all = time.perf_counter() - t0
        t0 = time.perf_counter()
        ga.track_multi_particle_beamline_for_magnet_with_multi_qs([bl] * 100, rps, L, step)
        torch.cuda.synchronize()
        t_call = time.perf_counter() - t0
        out[f"step_{int(round(step * 1000))}mm"] = {
            "steps": n_steps, "seconds": t_track, "gpairs_per_s": pairs / t_track / 1e9,
            "seconds_with_design_set": t_all, "accelerator_call_seconds": t_call,
            "reference_published_seconds": published, "reference_published_over_ours": published / t_all,
            "reference_published_over_accelerator_call": published / t_call}
    best = engine.autotune(warm, ps, 0.02, "f32c", steps=8)
    try:
        n_steps = int(np.ceil(L / 0.02))
        t0 = time.perf_counter()
        engine.track(warm, ps, L, 0.02, "f32c")
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
    finally:
        block = engine.particle_block()
        engine.set_units_per_cta(0)
        engine.set_particle_block(0)
    out["step_20mm"]["autotuned"] = {"units_per_cta": best, "particle_block": block or "automatic", "seconds": t,
                                     "gpairs_per_s": 100 * 16 * n_steps * 4 * warm.segments_of(0) / t / 1e9}
    return out


def measure_generation(args, rank):
    """One optimiser generation (the caller loop of the reference's NSGA run script): 64
    second-section designs, the script's beam (96 protons on the x-x' and y-y' ellipse edges
    at 4 momentum spreads), tracked through the whole section at the script's 50 mm step,
    then phase space and the eleven objectives per design.  Timed apart: host beamline build
    (layer records), device segment generation, FP32c packing, tracking, read-out."""
    import torch
    from cctpy_gb300 import HUST_SC_GANTRY, ParticleFactory, engine, workloads as W
    from cctpy_gb300.optim import a05_phase_space, beam_readout

    kws = W.design_population(64, seed=3 + rank)
    t0 = time.perf_counter()
    bls = [HUST_SC_GANTRY(**kw).create_second_bending_part_beamline() for kw in kws]
    t_host = time.perf_counter() - t0
    L = bls[0].get_length()
    ip = ParticleFactory.create_proton_along(bls[0], 0.0, 215.0)
    beam = ParticleFactory.create_from_phase_space_particles(ip, ip.get_natural_coordinate_system(), a05_phase_space())
    ip_end = ParticleFactory.create_proton_along(bls[0], L, 215.0)
    p0 = torch.as_tensor(np.array([b.to_numpy_array_data() for b in beam]), device="cuda")
    engine.design_set_of(bls[:1], segments="device")          # warm-up
    torch.cuda.synchronize()
    t = {}
    t0 = time.perf_counter()
    ds = engine.design_set_of(bls, segments="device")
    torch.cuda.synchronize()
    t["segments"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    ds.packed()
    torch.cuda.synchronize()
    t["pack"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    final = engine.track(ds, p0, L, 0.05, "f32c")
    torch.cuda.synchronize()
    t["track"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    _, obj = beam_readout(final, ip_end)
    obj = obj.cpu().numpy()
    t["readout"] = time.perf_counter() - t0
    steps = int(np.ceil(L / 0.05))
    gpu = sum(t.values())
    return {"workload": f"64 second-section designs ({ds.n_segments} segments), 96 protons each, {L:.3f} m at 50 mm "
                        f"({steps} RK4 steps), FP32c; objectives per design as the reference's optimiser script",
            "host_beamline_seconds": t_host, "device_seconds": t, "generation_seconds_device": gpu,
            "generations_per_s_device": 1.0 / gpu, "track_gpairs_per_s": 96 * steps * 4 * ds.n_segments / t["track"] / 1e9,
            "objectives_design0": [float(v) for v in obj[0]]}


def measure_design_grads(args, rank):
    """C4: 13-parameter gradients of J = <x^2> + <y^2> at the exit for 16 gantry designs x 1024
    protons in one adjoint run (1 mm RK4 steps), with the configuration's RK4 checkpointing
    every 64 steps and recompute: the forward keeps a checkpoint every 64 steps, and each
    segment is recomputed (its stage records written) before its reverse sweep.  FP32c
    (forward and adjoint sweeps in packed FP32 with compensation) on args.adjoint_steps steps,
    the FP64 adjoint on args.adjoint_steps_f64 of them.  Timed apart: the design set (segments
    generated on the GPU from layer records), the adjoint (cct_track_adjoint) and the parameter
    Jacobian (forward-mode contraction on the GPU, cct_segments_param_grad, plus the
    13-parameter grouping).  A design-grad-step is one RK4 step of one design's gradient; a
    whole C4 gradient over the 3.5 m track at 1 mm is 3500 of them."""
    import torch
    from cctpy_gb300 import engine, workloads as W
    from cctpy_gb300.adjoint import GantryDesign, exit_frame, layer_grads_from_rows, segment_gradient

    kws = W.design_population(16, seed=3)
    thetas = [np.array(kw["dicct345_tilt_angles"] + kw["agcct345_tilt_angles"]
                       + [kw["dicct345_current"], kw["dicct345_current"], kw["agcct345_current"],
                          kw["agcct345_current"], 0.95]) for kw in kws]
    designs = [GantryDesign(t, part_per_winding=360) for t in thetas]
    ps = W.beam_particles(designs[0].beamline, 1024, seed=4 + rank, kinetic_MeV=215.0)
    engine.design_set_of([designs[0].beamline], segments="device")          # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ds = engine.design_set_of([d.beamline for d in designs], segments="device")
    ds.packed()
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    n_seg = ds.n_segments
    full_steps = 3500
    out = {"workload": f"16 second-section designs ({n_seg} segments total), 1024 protons each, 13 parameters "
                       "(8 tilts, 4 layer currents, winding radius), J = <x^2>+<y^2> at the exit; 1 mm RK4 steps, "
                       "checkpoint every 64 steps with recompute",
           "design_set_seconds": t_setup, "full_track_steps": full_steps}
    for prec, steps in (("f32c", args.adjoint_steps), ("f64", args.adjoint_steps_f64)):
        L = steps * 0.001
        ck = min(64, steps)
        frames = np.tile(exit_frame(designs[0].beamline.trajectory, L, 215.0), (16, 1))
        segment_gradient(ds, ps, 0.002, 0.001, frames, 2, prec)        # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        J, seg, _ = segment_gradient(ds, ps, L, 0.001, frames, ck, prec, on_device=True)
        torch.cuda.synchronize()
        t_gpu = time.perf_counter() - t0
        t0 = time.perf_counter()
        rows = ds.param_grad(seg)
        g = [d.gradient(layer_grads_from_rows(d.beamline.magnets, rows[ds.layer_design == i]))
             for i, d in enumerate(designs)]
        t_jac = time.perf_counter() - t0
        fwd_pairs = 1024 * steps * 4 * n_seg          # each design's protons x its own segments
        rate = 16 * steps / (t_gpu + t_jac)
        out[prec] = {"steps": steps, "checkpoint_steps": ck, "checkpoint_segments": -(-steps // ck),
                     "adjoint_seconds": t_gpu, "jacobian_seconds": t_jac,
                     "design_grad_steps_per_s": rate,
                     "design_grad_steps_per_s_adjoint": 16 * steps / t_gpu,
                     "full_track_design_grads_per_s": rate / full_steps,
                     "seconds_per_16_full_track_gradients": 16 * full_steps / rate,
                     "forward_equivalent_gpairs_per_s": fwd_pairs / t_gpu / 1e9,
                     "gradient_norm_design0": float(np.linalg.norm(g[0]))}
    out["speedup_f32c_vs_f64"] = out["f32c"]["design_grad_steps_per_s"] / out["f64"]["design_grad_steps_per_s"]
    return out


def add_pipe_fractions(node, peak32: float, peak64: float, prec: str = None):
    """Beside every Gpairs/s figure of the tracking block, its fraction of this run's measured
    FMA-pipe peak at 26 flop a pair: FP32 for FP32c lines, FP64 for FP64 lines (the adjoint's
    forward-equivalent rate included)."""
    if isinstance(node, dict):
        for k, v in list(node.items()):
            p = prec
            if k.startswith("f32c") or k in ("reference_speed_test", "optimiser_generation"):   # FP32c only
                p = "f32c"
            elif k.startswith("f64"):
                p = "f64"
            if isinstance(v, dict):
                add_pipe_fractions(v, peak32, peak64, p)
            elif isinstance(v, (int, float)) and p and k.endswith("gpairs_per_s"):
                peak = peak32 if p == "f32c" else peak64
                node[k.replace("gpairs_per_s", "frac_of_") + ("fp32_pipe" if p == "f32c" else "fp64_pipe")] = \
                    FLOPS_PER_PAIR * v * 1e9 / peak


# ---------------------------------------------------------------- CPU baselines beside the GPU arm
def measure_cpu_baselines(args, ds):
    """The oracle on the machine's host cores (rank 0, one GPU): field sums on args.cpu_points of the
    field-map points, and the C0 track (as many 250 MeV protons as cores, the whole 374-step
    arc at 1 mm).  Both GPU forms are compared with the oracle on the same inputs (C1's
    "max and RMS relative |B| error vs the FP64 CPU oracle"; final positions of C0)."""
    import torch
    from cctpy_gb300 import engine, workloads as W
    cores = os.cpu_count() or 1
    with oracle_pool(cores) as pool:
        oracle_field_sample(pool, cores * 4, seed=299)                    # workers ready (untimed)
        rate, dt, pts, B_cpu = oracle_field_sample(pool, args.cpu_points, seed=300)
        cpu = {"value": rate / 1e9, "unit": "Gpairs/s", "cores": cores, "kind": "port",
               "sample": f"{args.cpu_points} of the 2^20 points x {N_SEG} segments ({dt:.1f} s, numpy oracle over a "
                         f"{cores}-process pool started and warmed before the timed call)"}
        acc = {"points": int(args.cpu_points)}
        for prec in ("f64", "f32c"):
            B = engine.field_at_points(ds, pts, prec)
            rel = np.linalg.norm(B - B_cpu, axis=1) / np.linalg.norm(B_cpu, axis=1)
            acc[f"max_rel_{prec}_vs_oracle"] = float(rel.max())
            acc[f"rms_rel_{prec}_vs_oracle"] = float(np.sqrt(np.mean(rel ** 2)))
        cpu_track = None
        if not args.no_tracking:
            trate, tdt, steps, p_in, p_out = oracle_track_sample(pool, cores)
            L = W.single_dipole_track_length()
            dev = {}
            for prec in ("f64", "f32c"):
                got = engine.track(ds, p_in, L, 0.001, prec)[0]
                dev[f"max_pos_diff_m_{prec}"] = float(np.abs(got[:, 0:3] - p_out[:, 0:3]).max())
            torch.cuda.synchronize()
            cpu_track = {"value": trate, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{cores} C0 protons (250 MeV, one per process) through the whole {L:.4f} m "
                                   f"single-dipole arc at 1 mm ({steps} RK4 steps, {N_SEG} segments): {tdt:.1f} s",
                         "gpairs_per_s": trate * 4 * N_SEG / 1e9, "gpu_vs_cpu_final_position": dev}
    return cpu, cpu_track, acc


def measure_reference_gpu_baseline(steps_f32: int = 0, steps_f64: int = 0, tracking=None):
    """cctpy's own CUDA tracking kernel on this GPU, beside the engine on the same inputs: the
    workload of cctpy's GPU speed test (100 copies of its 24 000-segment AG-CCT beamline, 16
    copies of the ideal 250 MeV proton each, 20 mm RK4 step).  FLOAT32 (1024 threads a block,
    the speed test's configuration) over the whole 10.87 m; FLOAT64 (512 threads) over 1/32 of
    it (0.34 m) from 4.9 m on the design orbit, into the AG-CCT.  With `tracking`, also C0 (the
    single dipole's 32 protons: FLOAT32 over the whole arc, FLOAT64 over 8 steps, cctpy's
    default build).  steps_f32 / steps_f64 > 0
    shorten the two legs to that many 20 mm steps (small cases for profiling).  With
    `tracking` (this run's tracking block) also the gantry workloads, through cctpy's FLOAT32 x
    1024 kernel sized for 700 000 current elements a beamline: cctpy runs a design's particles
    one after another in one block, so its rate per pair does not depend on the particle count
    and a bounded sample (64 protons, 2 steps of 1 mm) gives it; the engine is timed on the
    same sample and its full-configuration rate is taken from `tracking`.  cctpy's kernel source (final_code/packages/gpu_accelerator.py:100-1078)
    is compiled for sm_103a from cctpy's tree at build time (oracle/ref_cuda_build.py) and
    launched as cctpy's host code does (gpu_accelerator.py:1931-2031; oracle/ref_cuda.py);
    its per-call JIT compile is left out.  "call" times include cctpy's array packing (segment
    arrays padded to its capacities) and its copies; ours are engine.track with the same host
    particle records in and out."""
    import torch
    from oracle import ref_cuda
    if not ref_cuda.available():
        return {"unavailable": "cctpy's CUDA kernels were not built (oracle/ref_cuda_build.py needs cctpy's "
                               "sources at build time)"}
    from cctpy_gb300 import engine, workloads as W
    from cctpy_gb300.particles import ParticleFactory, particles_to_array
    bl = W.build_speed_test_beamline()
    L = bl.get_length()
    design = engine.host_design(engine.magnet_list(bl))
    n_seg = design[0].shape[0]
    starts = {"f32": 0.0, "f64": 4.9}
    designs = [design] * 100
    ds = engine.DesignSet(designs)
    out = {"kernel": "cctpy track_multi_particle_beamline_for_magnet_with_multi_qs, compiled from its source "
                     "for sm_103a, one block per beamline",
           "workload": f"100 beamlines x {n_seg} segments (cctpy's GPU speed test), 16 protons each, 20 mm step"}
    for prec, ours_prec, frac, n_steps in (("f32", "f32c", 1.0, steps_f32), ("f64", "f64", 1.0 / 32, steps_f64)):
        ps = particles_to_array([ParticleFactory.create_proton_along(bl, starts[prec])] * 16)
        ref = ref_cuda.ReferenceCudaTracker(prec)
        try:
            ref.track(designs[:2], ps, 0.04, 0.02)                              # module loaded, warm
            dist = 0.02 * n_steps if n_steps > 0 else L * frac
            theirs, k_s, call_s = ref.track(designs, ps, dist, 0.02)
        finally:
            ref.close()
        engine.track(ds, ps, 0.04, 0.02, ours_prec)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mine = engine.track(ds, ps, dist, 0.02, ours_prec)
        torch.cuda.synchronize()
        ours_s = time.perf_counter() - t0
        steps = int(np.ceil(dist / 0.02))
        pairs = 100 * 16 * steps * 4 * n_seg
        out[prec] = {"start_m": starts[prec], "length_m": dist, "steps": steps, "block": ref.block,
                     "kernel_seconds": k_s,
                     "call_seconds": call_s, "gpairs_per_s": pairs / k_s / 1e9,
                     f"ours_{ours_prec}_seconds": ours_s, "ours_gpairs_per_s": pairs / ours_s / 1e9,
                     "ours_over_reference_kernel": k_s / ours_s, "ours_over_reference_call": call_s / ours_s,
                     f"max_pos_diff_m_vs_ours_{ours_prec}": float(np.abs(theirs[:, :, :3] - mine[:, :, :3]).max())}
    if tracking is None:
        return out
    # C0: the single dipole's 32 protons through cctpy's kernel (one beamline: one block),
    # FLOAT32 over the whole arc, FLOAT64 over its first 8 steps
    _, cct = W.build_single_dipole()
    d0 = engine.host_design(engine.magnet_list(cct))
    p32 = W.single_dipole_particles(32, seed=0)
    L0 = W.single_dipole_track_length()
    ds0 = engine.design_of(cct)
    c0 = {"workload": f"C0: {d0[0].shape[0]} segments, 32 protons of 250 MeV, 1 mm steps"}
    for cfg, ours_prec, steps0 in (("f32", "f32c", 0), ("f64", "f64", 8)):
        dist = L0 if steps0 == 0 else steps0 * 0.001
        ref = ref_cuda.ReferenceCudaTracker(cfg)
        try:
            ref.track([d0], p32[:2], 0.002, 0.001)                               # warm
            theirs, k_s, call_s = ref.track([d0], p32, dist, 0.001)
        finally:
            ref.close()
        engine.track(ds0, p32, 0.002, 0.001, ours_prec)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mine = engine.track(ds0, p32, dist, 0.001, ours_prec)
        torch.cuda.synchronize()
        ours_s = time.perf_counter() - t0
        steps = int(np.ceil(dist / 0.001 - 1e-9))
        pairs = 32 * steps * 4 * d0[0].shape[0]
        c0[cfg] = {"steps": steps, "kernel_seconds": k_s, "call_seconds": call_s, "gpairs_per_s": pairs / k_s / 1e9,
                   f"ours_{ours_prec}_seconds": ours_s, "ours_over_reference_kernel": k_s / ours_s,
                   f"max_pos_diff_m_vs_ours_{ours_prec}": float(np.abs(theirs[:, :, :3] - mine[:, :, :3]).max())}
    out["single_dipole"] = c0
    from cctpy_gb300 import HUST_SC_GANTRY
    g = W.build_gantry_section()
    samples = {
        "gantry_section": ([engine.host_design(engine.magnet_list(g))],
                           W.beam_particles(g, 4096, seed=2, kinetic_MeV=215.0)[:64],
                           tracking.get("gantry_section", {}).get("f32c", {}).get("gpairs_per_s")),
    }
    if "design_population" in tracking:
        bls = [HUST_SC_GANTRY(**kw).create_second_bending_part_beamline() for kw in W.design_population(64, seed=3)]
        samples["design_population"] = ([engine.host_design(engine.magnet_list(b)) for b in bls],
                                        W.beam_particles(bls[0], 512, seed=2, kinetic_MeV=215.0)[:64],
                                        tracking["design_population"].get("f32c", {}).get("gpairs_per_s"))
    ref = ref_cuda.ReferenceCudaTracker("f32_700k")
    try:
        for name, (designs_g, ps_g, ours_full) in samples.items():
            steps, step = 2, 0.001
            ref.track(designs_g[:1], ps_g[:2], step, step)                         # warm
            theirs, k_s, call_s = ref.track(designs_g, ps_g, steps * step, step)
            half = len(ps_g) // 2     # half the protons: cctpy's per-pair rate should not change
            _, k_half, _ = ref.track(designs_g, ps_g[:half], steps * step, step)
            ds_g = engine.DesignSet(designs_g)
            engine.track(ds_g, ps_g, step, step, "f32c")
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            mine = engine.track(ds_g, ps_g, steps * step, step, "f32c")
            torch.cuda.synchronize()
            ours_s = time.perf_counter() - t0
            pairs = len(ps_g) * steps * 4 * sum(d[0].shape[0] for d in designs_g)
            rate = pairs / k_s / 1e9
            out[name] = {"sample": f"{len(designs_g)} design(s), {sum(d[0].shape[0] for d in designs_g)} segments, "
                                   f"{len(ps_g)} protons each, {steps} steps of 1 mm",
                         "block": ref.block, "max_current_element_number": ref.max_ce, "kernel_seconds": k_s,
                         "call_seconds": call_s, "gpairs_per_s": rate,
                         f"gpairs_per_s_with_{half}_protons": pairs * half / len(ps_g) / k_half / 1e9,
                         "ours_f32c_same_sample_seconds": ours_s,
                         "ours_f32c_full_configuration_gpairs_per_s": ours_full,
                         "ours_full_configuration_over_reference_kernel": ours_full / rate if ours_full else None,
                         "max_pos_diff_m_vs_ours_f32c": float(np.abs(theirs[:, :, :3] - mine[:, :, :3]).max())}
    finally:
        ref.close()
    return out


# ---------------------------------------------------------------- GPU arm
def run_ours(args):
    import torch
    N_POINTS = args.points
    PAIRS = N_POINTS * N_SEG
    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from cctpy_gb300 import _lib, engine, workloads as W
    import ctypes

    lib = _lib.load()
    dev = torch.device("cuda", local)
    _, cct = W.build_single_dipole()
    ds = engine.design_of(cct)
    assert ds.n_segments == N_SEG
    packed = ds.packed()
    pts_np = W.field_map_points(N_POINTS, seed=1 + rank)
    pts = torch.from_numpy(pts_np).to(dev)
    out = torch.empty_like(pts)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)   # > 129 MB L2
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    def f32c_step():
        rc = lib.cct_field_f32c(packed.data_ptr(), 0, None, 0, pts.data_ptr(), N_POINTS, out.data_ptr(), sptr)
        if rc:
            _lib.check(rc, "cct_field_f32c")

    def f64_step():
        rc = lib.cct_field_f64(ds.kls.data_ptr(), ds.p0s.data_ptr(), N_SEG, None, 0, pts.data_ptr(), N_POINTS,
                               out.data_ptr(), sptr)
        if rc:
            _lib.check(rc, "cct_field_f64")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- accuracy of the timed kernel on the full workload (FP32c vs FP64, same points)
    f64_step()
    torch.cuda.synchronize()
    b64 = out.clone()
    f32c_step()
    torch.cuda.synchronize()
    rel = (torch.linalg.norm(out - b64, dim=1) / torch.linalg.norm(b64, dim=1))
    acc = {"max_rel_f32c_vs_f64": float(rel.max()), "rms_rel_f32c_vs_f64": float(torch.sqrt((rel ** 2).mean()))}

    # ---- FP32c, device-resident, K timed steps with per-step kernel events
    for _ in range(args.warmup):
        flush.zero_()
        f32c_step()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier()
    with ClockSampler(local) as clk:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record()
            f32c_step()
            ev[k][1].record()
        t1.record()
        barrier()
    total_ms = t0.elapsed_time(t1)
    kern_ms = [a.elapsed_time(b) for a, b in ev]
    clocks = clk.summary()
    if dist is not None:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t)
    value = world * PAIRS * args.steps / (total_ms * 1e-3) / 1e9
    kernel_ms = statistics.mean(kern_ms)

    # ---- roofline: FP32 FMA pipe, measured live
    peak = ctypes.c_double()
    _lib.check(lib.cct_probe_fma_peak(0, ctypes.byref(peak)), "cct_probe_fma_peak")
    peak32_scalar = peak.value / 1e12
    _lib.check(lib.cct_probe_fma_peak(2, ctypes.byref(peak)), "cct_probe_fma_peak")
    peak32_packed = peak.value / 1e12
    peak32 = max(peak32_scalar, peak32_packed)
    _lib.check(lib.cct_probe_fma_peak(1, ctypes.byref(peak)), "cct_probe_fma_peak")
    peak64 = peak.value / 1e12
    achieved = FLOPS_PER_PAIR * PAIRS / (kernel_ms * 1e-3) / 1e12

    # ---- FP64 drop-in on the same workload
    f64_steps = max(1, args.fp64_steps)
    f64_step()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(f64_steps):
        flush.zero_()
        f64_step()
    e1.record()
    barrier()
    f64_ms = e0.elapsed_time(e1) / f64_steps
    f64_value = PAIRS / (f64_ms * 1e-3) / 1e9
    f64_achieved = FLOPS_PER_PAIR * PAIRS / (f64_ms * 1e-3) / 1e12

    # ---- end to end through the public call: pinned host points in, host field out
    h_pts = torch.from_numpy(pts_np).pin_memory()
    h_out = torch.empty_like(h_pts).pin_memory()
    for _ in range(2):
        engine.field_at_points(ds, h_pts, "f32c", out_host=h_out)
    barrier()
    w0 = time.perf_counter()
    for _ in range(args.steps):
        engine.field_at_points(ds, h_pts, "f32c", out_host=h_out)
    barrier()
    e2e_s = time.perf_counter() - w0
    if dist is not None:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t)
    e2e = world * PAIRS * args.steps / e2e_s / 1e9

    tracking = None if args.no_tracking else measure_tracking(args, dev, rank)
    if tracking is not None:
        add_pipe_fractions(tracking, peak32 * 1e12, peak64 * 1e12)
    shard = None
    if not (args.no_tracking or args.no_population):
        try:
            shard = measure_population_shard(args, rank, world, dist)
        except Exception as e:   # the headline line is printed whatever happens to this leg
            shard = {"error": f"{type(e).__name__}: {e}"[:300]}

    line = None
    if rank == 0:
        cpu = cpu_track = acc_oracle = ref_gpu = None
        if world == 1 and not args.no_cpu_baseline:
            cpu, cpu_track, acc_oracle = measure_cpu_baselines(args, ds)
            if not (args.no_tracking or args.no_speed_test):
                try:
                    ref_gpu = measure_reference_gpu_baseline(tracking=tracking)
                except Exception as e:   # the headline line is printed whatever happens to this leg
                    ref_gpu = {"error": f"{type(e).__name__}: {e}"[:300]}
        line = {
            "metric": METRIC, "value": value, "unit": "Gpairs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+comp (f64 origins/accumulation)",
            "data": "synthetic (seeded points in a 60 mm tube around the dipole arc)",
            "config": {"workload": WORKLOAD if N_POINTS == 1 << 20 else f"field_map: {N_POINTS} points x 46080 "
                                   "segments (reduced case)", "n_points": N_POINTS, "n_segments": N_SEG, "pairs_per_step": PAIRS,
                       "precision": "f32c", "l2": "256 MiB buffer written between timed steps",
                       "parallelism": (f"field map: replicas x{world} (independent points); population: designs "
                                       f"sharded over {world} ranks by segment count" if world > 1 else "single GPU")},
            "e2e": {"value": e2e, "unit": "Gpairs/s", "h2d_bytes_per_step": N_POINTS * 24,
                    "d2h_bytes_per_step": N_POINTS * 24,
                    "call": "engine.field_at_points(design, pinned host points, 'f32c', out_host=pinned)"},
            "roofline": {"bound": "fp32-pipe", "achieved": achieved, "peak": peak32, "unit": "TFLOP/s",
                         "frac": achieved / peak32,
                         "traffic": args.traffic if args.traffic is not None else
                         (FIELD_MAP_TRAFFIC_BYTES if N_POINTS == 1 << 20 else None),
                         "traffic_unit": "bytes per launch (dram read + write, from an ncu capture of this kernel "
                                         "on this workload)",
                         "peak_source": "measured in this run: best of scalar FFMA and packed FP32x2 FMA "
                                        "chains (cct_probe_fma_peak); the driver's measured peaks hold no FP32 or "
                                        "FP64 CUDA-core figure, and its bf16 tensor and HBM peaks do not bound "
                                        "this non-contraction",
                         "frac_of": "measured FP32 FMA-pipe peak (this run's probe)",
                         "peak_scalar_ffma": peak32_scalar, "peak_packed_ffma2": peak32_packed,
                         "flops_per_pair": FLOPS_PER_PAIR, "kernel": "field_f32c_kernel",
                         "kernel_ms": kernel_ms},
            "fp64": {"value": f64_value, "unit": "Gpairs/s", "ms_per_step": f64_ms, "steps": f64_steps,
                     "roofline": {"bound": "fp64-pipe", "achieved": f64_achieved, "peak": peak64,
                                  "unit": "TFLOP/s", "frac": f64_achieved / peak64,
                                  "peak_source": "measured in this run: FP64 DFMA-chain probe"},
                     "speedup_f32c_vs_f64": value / f64_value},
            "accuracy": dict(acc, vs_oracle=acc_oracle),
            "tracking": tracking,
            "population_shard": shard,
            "cpu_baseline_tracking": cpu_track,
            "reference_gpu_baseline": ref_gpu,
            "gpu_launches": args.steps,
            "clocks": clocks,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--points", type=int, default=N_POINTS, help="field points per step (2^20 = the workload)")
    ap.add_argument("--cpu-points", type=int, default=65536)
    ap.add_argument("--ref-points", type=int, default=4096)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tracking", action="store_true")
    ap.add_argument("--no-population", action="store_true")
    ap.add_argument("--track-steps", type=int, default=20,
                    help="timed RK4 steps of the C2 tracking slice (both precisions)")
    ap.add_argument("--population-steps", type=int, default=10,
                    help="timed RK4 steps of the C3 population slice (both precisions)")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-generation", action="store_true")
    ap.add_argument("--no-speed-test", action="store_true", help="skip the reference's own GPU speed-test slice")
    ap.add_argument("--adjoint-steps", type=int, default=256,
                    help="RK4 steps of the FP32c design-gradient slice (checkpoint every 64)")
    ap.add_argument("--adjoint-steps-f64", type=int, default=4, help="RK4 steps of the FP64 design-gradient slice")
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per launch of the timed kernel from an ncu capture (default: the committed "
                         "capture of the field-map launch)")
    ap.add_argument("--only", choices=["speed-test"], default=None,
                    help="speed-test: only cctpy's speed-test shape, the engine beside cctpy's own CUDA kernel "
                         "(reference_gpu_baseline), over --speed-test-steps steps; for profiling")
    ap.add_argument("--speed-test-steps", type=int, default=8)
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.only == "speed-test":
        import torch
        torch.cuda.set_device(0)
        n = args.speed_test_steps
        print(json.dumps({"only": "speed-test", "reference_gpu_baseline": measure_reference_gpu_baseline(n, n)}))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
