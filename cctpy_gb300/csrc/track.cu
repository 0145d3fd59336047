// Batched RK4 proton tracking through CCT beamlines: one cooperative persistent launch.
//
// Reference semantics (cctpy): ParticleRunner.run_only particles.py:562-596, RK4
// BaseUtils.runge_kutta4 base_utils.py:264-311, callback Y' = [v, (e/rm) v x B(p)]
// particles.py:515-537, beamline field beamline.py:46-53.
//
// Work decomposition.  Each design's particles are cut into blocks of G particles and its
// segments into tiles of 128, the tiles into chunks.  A unit is (design, block, chunk).
// Every RK4 stage has two parts:
//   A. field sums: a CTA takes a unit and computes the chunk's field at the stage positions
//      of the block's particles, one partial per (unit, particle):
//        FP32c: the chunk's packed tiles stream into a shared-memory ring by TMA bulk copies;
//               every warp reads every tile; a warp owns 32*PPT particles and a 128/S-segment
//               slice of each tile (S = warps * 32 * PPT / G), lanes hold particles;
//        FP64:  G = 32, the CTA's warps split the chunk's tiles, lane = particle, segments
//               are read with warp-uniform loads;
//   C. particle update: the chunk partials of a particle are summed in fixed order, the
//      analytic QS fields added and the RK4 bookkeeping advanced.
// Three schedules:
//   * small batches (FP32c, at most 64 particles in fewer than 8 particle blocks): CTA b owns
//     unit b for the whole launch (its tiles stay in shared memory when they fit the ring) and
//     keeps its own copy of every particle's RK4 state in shared memory; each unit adds its
//     field into fixed-point int64 accumulators (exact integer sums: no order dependence) and
//     counts itself done; every CTA waits for the stage's count, reads the accumulators and
//     advances its copy of the particles.  No grid barrier per stage (latency-bound batches:
//     C0's 32 protons at 9 us a stage against 18 us on grid barriers);
//   * dataflow (8 or more particle blocks): one sequence of units over all stages, handed
//     out by a global counter.  Before a unit a CTA waits until the unit's block has finished
//     the previous stage (per-block stage counter); after it, it counts the unit done on the
//     block; the CTA that completes a block's stage runs part C for that block and marks it
//     ready.  Blocks of different stages overlap, so no CTA waits at a stage's end.
//   * grid barriers (fewer blocks): part A with units taken from a per-stage counter, a grid
//     barrier, part C on every CTA at once (a warp per particle), a grid barrier; for a small
//     batch part C is shortest this way.
// Grid barriers and dataflow waits count on global words and have a wall-clock limit after
// which the kernel records CCT_ERR_TIMEOUT and returns; TMA waits are bounded too.  No wait
// is unbounded.
#include <cstdlib>
#include <mutex>
#include <vector>

#include <algorithm>

#include "track_common.cuh"

namespace cctgpu {

// Dataflow schedule, FP32c: the CTA walks the launch's unit sequence; before a unit it waits
// until the unit's particle block has finished the previous stage, after it counts the unit
// done, and the CTA that finishes a block's stage runs that block's particle update.
// Returns false if a wait gave up (CCT_ERR_TIMEOUT recorded, ring drained).
template <int PPT, bool HALF = false>
static __device__ bool flow_f32c(const TrackParams &P, TrackSmem &sm, uint32_t &kt, int64_t n_units, int64_t n_seq) {
    int64_t s = first_unit();
    if (s < n_seq) unit_prefetch(P, s % n_units, sm, kt);
    while (s < n_seq) {
        const int k = (int)(s / n_units);
        const int64_t u = s % n_units;
        const UnitRef U = locate_unit(P, u);
        const int64_t blk = (int64_t)U.d * P.blocks + U.b;
        if (!flow_wait(P, sm, blk, k)) {
            if (threadIdx.x == 0) ring_drain(sm);   // the unit's first tiles are in flight
            __syncthreads();
            return false;
        }
        if (unit_sum_f32c<PPT, false, true, false, HALF>(P, stage_points(P), u, sm, kt, k, n_units, n_seq) < 0)
            return false;
        if (flow_complete(P, sm, blk, k, P.chunks[U.d])) block_update(P, U.d, U.b, k);
        s = claim_seq(P, sm);
        if (s < n_seq) unit_prefetch(P, s % n_units, sm, kt);
    }
    return true;
}

// The same for FP64 units (no tile ring).
template <bool HALF = false>
static __device__ bool flow_f64(const TrackParams &P, TrackSmem &sm, int64_t n_units, int64_t n_seq) {
    for (int64_t s = first_unit(); s < n_seq; s = claim_seq(P, sm)) {
        const int k = (int)(s / n_units);
        const int64_t u = s % n_units;
        const UnitRef U = locate_unit(P, u);
        const int64_t blk = (int64_t)U.d * P.blocks + U.b;
        if (!flow_wait(P, sm, blk, k)) return false;
        unit_field_f64<HALF>(P, u, sm);
        if (flow_complete(P, sm, blk, k, P.chunks[U.d])) block_update(P, U.d, U.b, k);
    }
    return true;
}

// Small-batch schedule (P.tiny): CTA b runs unit b in every stage (units <= CTAs), keeps its
// tiles in the ring when they fit and its own copy of every particle's state in shared memory;
// a stage ends when every group's unit counter reaches the stage's count (one warp polls the
// groups' counters, a lane each).  CTA 0 writes its copy of the final state back.  Returns
// false if a wait gave up (CCT_ERR_TIMEOUT recorded).
template <int PPT, bool HALF = false>
static __device__ bool tiny_track(const TrackParams &P, TrackSmem &sm, uint32_t &kt, int step_end, int64_t n_units) {
    const int64_t total = (int64_t)P.n_designs * P.n_p;
    const int tid = threadIdx.x, lane = tid & 31;
    for (int64_t i = tid; i < total * kStateD; i += blockDim.x) sm.tiny_state[i] = P.state[i];
    for (int i = tid; i < 2 * kTinyMax * 4; i += blockDim.x) sm.tiny_prev[i] = 0;
    for (int64_t pi = tid; pi < total; pi += blockDim.x) {
        const int64_t d = pi / P.n_p;
        sm.tiny_qs[pi][0] = P.qs_off[d];
        sm.tiny_qs[pi][1] = P.qs_off[d + 1];
    }
    __syncthreads();
    for (int64_t pi = tid; pi < total; pi += blockDim.x)   // positions as double-float pairs
#pragma unroll
        for (int c = 0; c < 3; ++c)
            split_df(sm.tiny_state[pi * kStateD + ST_YS + c], sm.tiny_pts[pi][c], sm.tiny_pts[pi][3 + c]);
    __syncthreads();
    const int64_t u = blockIdx.x;
    if (u >= n_units) return true;   // no unit: nothing to do until the final barrier (CTA 0 has unit 0)
    const UnitRef U = locate_unit(P, u);
    const bool fits = U.t_end - U.t_beg <= kRing;
    // unit groups: units [g * gsz, (g + 1) * gsz) count on group g's line
    const int64_t gsz = (n_units + kTinyGroups - 1) / kTinyGroups;
    const int64_t n_groups = (n_units + gsz - 1) / gsz;
    unsigned long long *counts = reinterpret_cast<unsigned long long *>(P.ctrl + kCtrlTinyCount);
    unsigned long long *mine = counts + (u / gsz) * (kCtrlLineWords / 2);
    const int64_t lane_units = lane < n_groups ? hd_min(gsz, n_units - lane * gsz) : 0;
    const PointSrc src{sm.tiny_state + ST_YS, kStateD, nullptr, 0};
    int phase = 0;
    for (int step = P.step_begin; step < step_end; ++step) {
        for (int stage = 0; stage < 4; ++stage, ++phase) {
            const bool resident = fits && phase > 0;
            if (!resident) unit_prefetch(P, u, sm, kt);
            if (unit_sum_f32c<PPT, false, true, true, HALF>(P, src, u, sm, kt, phase, n_units, 0, resident, &U) < 0)
                return false;
            if (tid < 32) {
                if (tid == 0) {
                    __threadfence();                   // this unit's accumulator additions first
                    atomicAdd(mine, 1ull);
                }
                __syncwarp();
                // (test hook: flow_skew more stages than exist, so that the wait runs out)
                const unsigned long long want =
                    (unsigned long long)(phase + 1 + P.flow_skew) * (unsigned long long)lane_units;
                const volatile unsigned long long *c = counts + lane * (kCtrlLineWords / 2);
                volatile int *err = reinterpret_cast<volatile int *>(P.ctrl + CW_ERR);
                int ok = 1;
                const unsigned long long t0 = global_ns();
                unsigned polls = 0;
                while (!__all_sync(0xffffffffu, lane >= n_groups || *c >= want)) {
                    if ((++polls & 63u) == 0) {
                        const int give_up = *err == CCT_ERR_TIMEOUT || global_ns() - t0 > P.wait_ns;
                        if (__any_sync(0xffffffffu, give_up)) {
                            if (lane == 0) set_timeout(P);
                            ok = 0;
                            break;
                        }
                    }
                    __nanosleep(32);
                }
                if (lane == 0) {
                    __threadfence();
                    sm.verdict = ok;
                }
            }
            __syncthreads();
            if (!sm.verdict) return false;
            tiny_advance(P, sm, step, stage, phase);
            __syncthreads();
        }
    }
    if (blockIdx.x == 0)
        for (int64_t i = tid; i < total * kStateD; i += blockDim.x) P.state[i] = sm.tiny_state[i];
    return true;
}

// Start of every tracking launch: state from the particle records with the step count and dt
// as the CPU reference computes them (init_from_records), the small-batch accumulators
// cleared, the unit counters reset; ends at the first grid barrier.  Returns false if the
// device-side plan rejected the inputs or the barrier gave up; else the launch's last step.
static __device__ bool track_begin(const TrackParams &P, TrackSmem &sm, int &step_end) {
    const int64_t total = (int64_t)P.n_designs * P.n_p;
    const int64_t tstride = (int64_t)gridDim.x * blockDim.x;
    if (*(volatile unsigned *)(P.ctrl + CW_ERR) != 0) return false;   // the device-side plan rejected the inputs
    if (threadIdx.x == 0) ring_init(sm);
    for (int64_t pi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; P.init_from_records && pi < total;
         pi += tstride) {
        const double *r = P.particles + pi * 10;
        double *S = P.state + pi * kStateD;
        for (int c = 0; c < 6; ++c) S[ST_Y0 + c] = S[ST_YS + c] = r[c];
        const double speed = r[8];
        const double dt0 = P.footstep / speed;
        const double t_end = P.distance / speed;
        const double steps = ceil(t_end / dt0);
        S[ST_KQ] = r[7] / r[6];
        // at most 5e8 steps, so that 4 stages a step stay within the int stage counters
        const bool ok = isfinite(steps) && steps >= 1.0 && steps < 5.0e8;
        S[ST_NSTEPS] = ok ? steps : 0.0;
        S[ST_DT] = ok ? t_end / steps : 0.0;
        if (!ok) atomicExch(P.ctrl + CW_NONFINITE, 1u);
        else atomicMax(P.ctrl + CW_MAXSTEPS, (unsigned)steps);
        if (P.tiny) {   // every copy of both stage parities' accumulators starts at zero
            for (int q = 0; q < 2 * P.tiny_copies; ++q) {
                for (int c = 0; c < 3; ++c) P.tiny_acc[(q * total + pi) * 3 + c] = 0;
                P.tiny_bad[q * total + pi] = 0u;
            }
        }
    }
    clear_unit_counters(P);
    if (!grid_barrier(P, sm)) return false;
    const int max_steps = P.init_from_records ? (int)*(volatile unsigned *)(P.ctrl + CW_MAXSTEPS) : P.step_end;
    step_end = min(max_steps, P.step_end);
    return true;
}

// End of a tracking launch: the final state into the particle records (write_back).
static __device__ void track_end(const TrackParams &P) {
    const int64_t total = (int64_t)P.n_designs * P.n_p;
    const int64_t tstride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t pi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; P.write_back && pi < total; pi += tstride) {
        double *r = P.particles + pi * 10;
        const double *S = P.state + pi * kStateD;
        for (int c = 0; c < 6; ++c) r[c] = S[ST_Y0 + c];
        if (S[ST_NSTEPS] > 0.0) r[9] = r[9] + P.distance;
    }
}

// The dataflow and grid-barrier schedules.
__global__ void __launch_bounds__(kTrackBlock, kTrackMinBlocks) track_kernel(TrackParams P) {
    __shared__ __align__(128) TrackSmem sm;
    const int64_t total = (int64_t)P.n_designs * P.n_p;
    int step_end = 0;
    if (!track_begin(P, sm, step_end)) return;
    uint32_t kt = 0;   // tiles consumed through the ring by this CTA
    const int64_t n_units = P.unit_off[P.n_designs];
    const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;

    if (P.use_flow) {
        const int64_t n_seq = step_end > P.step_begin ? (int64_t)(step_end - P.step_begin) * 4 * n_units : 0;
        if (P.precision == 0 && P.G == kHalfGroup) (void)flow_f64<true>(P, sm, n_units, n_seq);
        else if (P.precision == 0) (void)flow_f64(P, sm, n_units, n_seq);
        else if (P.G == kHalfGroup) (void)flow_f32c<1, true>(P, sm, kt, n_units, n_seq);
        else if (P.ppt == 2) (void)flow_f32c<2>(P, sm, kt, n_units, n_seq);
        else (void)flow_f32c<1>(P, sm, kt, n_units, n_seq);
        if (!grid_barrier(P, sm)) return;   // every stage of every block is done (or a wait gave up)
    }
    int phase = 0;
    for (int step = P.step_begin; !P.use_flow && step < step_end; ++step) {
        for (int stage = 0; stage < 4; ++stage, ++phase) {
            if (P.precision == 0) {
                for (int64_t u = first_unit(); u < n_units; u = next_unit(P, sm, phase)) {
                    if (P.G == kHalfGroup) unit_field_f64<true>(P, u, sm);
                    else unit_field_f64(P, u, sm);
                }
            } else if (P.G == kHalfGroup) {
                units_f32c<1, false, true>(P, stage_points(P), sm, kt, phase, n_units);
            } else if (P.ppt == 2) {
                units_f32c<2, false>(P, stage_points(P), sm, kt, phase, n_units);
            } else {
                units_f32c<1, false>(P, stage_points(P), sm, kt, phase, n_units);
            }
            if (!grid_barrier(P, sm)) return;   // a TMA timeout is recorded in CW_ERR and ends here
            reset_next_unit(P, phase);
            if (total <= (int64_t)gridDim.x) {   // few particles: a CTA per particle
                for (int64_t pi = blockIdx.x; pi < total; pi += gridDim.x) {
                    if (!particle_active(P, pi, step)) continue;
                    double B[3];
                    cta_sum_partials(P, pi, B, sm);
                    if (threadIdx.x == 0) particle_update(P, pi, step, stage, B);
                }
            } else {
                for (int64_t pi = gwarp; pi < total; pi += nwarps) {   // a warp per particle
                    if (!particle_active(P, pi, step)) continue;
                    double B[3];
                    warp_sum_partials(P, pi, B);
                    if ((threadIdx.x & 31) == 0) particle_update(P, pi, step, stage, B);
                }
            }
            if (!grid_barrier(P, sm)) return;
        }
    }

    track_end(P);
}

// The small-batch schedule, a kernel of its own so that its code does not weigh on the other
// schedules' register allocation.
__global__ void __launch_bounds__(kTrackBlock, kTrackMinBlocks) track_tiny_kernel(TrackParams P) {
    __shared__ __align__(128) TrackSmem sm;
    int step_end = 0;
    if (!track_begin(P, sm, step_end)) return;
    uint32_t kt = 0;
    const int64_t n_units = P.unit_off[P.n_designs];
    if (P.G == kHalfGroup) (void)tiny_track<1, true>(P, sm, kt, step_end, n_units);
    else if (P.ppt == 2) (void)tiny_track<2>(P, sm, kt, step_end, n_units);
    else (void)tiny_track<1>(P, sm, kt, step_end, n_units);
    if (!grid_barrier(P, sm)) return;   // CTA 0's copy of the state is in P.state (or a wait gave up)
    track_end(P);
}

// ---------------------------------------------------------------- host side
cudaError_t launch_track_kernel(TrackParams &P, int grid, cudaStream_t st) {
    void *args[] = {&P};
    const void *fn = P.tiny ? (const void *)track_tiny_kernel : (const void *)track_kernel;
    return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kTrackBlock), args, 0, st);
}

int g_test_phantom_blocks = 0;
int g_test_flow_skew = 0;
long long g_wait_ms = 60000;

TrackScratchLayout track_scratch_layout(int n_designs, int64_t n_particles, int64_t n_units, int group) {
    TrackScratchLayout L;
    auto up = [](int64_t b) { return (b + 255) / 256 * 256; };
    const int64_t tables = up(8 * (int64_t)(3 * n_designs + 1));
    L.ctrl_off = 0;
    L.state_off = kCtrlBytes + tables;
    L.partial_off = L.state_off + up(8 * kStateD * (int64_t)n_designs * n_particles);
    L.flow_off = L.partial_off + up(24 * (int64_t)group * n_units);
    L.total = L.flow_off + up(kFlowBytesPerBlock * (int64_t)n_designs * ((n_particles + group - 1) / group));
    return L;
}

// Particles per unit: FP64 keeps 32 (warps split the tiles); FP32c takes the block size that
// needs the fewest particle slots (blocks x G), the largest of those: e.g. 100 particles run as
// one block of 128 rather than two of 64 (the same slots), 96 as three blocks of 32.
// min_group 16 (the forward tracking, both precisions) also allows half-warp blocks of 16, for
// designs of at most 16 particles.
int group_size(int precision, int64_t n_p, int min_group) {
    if (min_group <= kHalfGroup && n_p <= kHalfGroup) return kHalfGroup;
    if (precision == 0) return 32;
    int best = kMaxGroup;
    int64_t best_slots = (n_p + best - 1) / best * best;
    for (int G = kMaxGroup / 2; G >= 32; G /= 2) {
        const int64_t slots = (n_p + G - 1) / G * G;
        if (slots < best_slots) {
            best = G;
            best_slots = slots;
        }
    }
    return best;
}

int g_particle_block = 0;   // FP32c particle block set by hand or by cct_autotune (0: group_size's choice)

// Particle block of the forward tracking entry points: the process-wide setting for FP32c if
// one is made, else group_size's.  (The adjoint keeps group_size's, which its scratch query
// assumes.)
int track_group(int precision, int64_t n_p) {
    if (precision == 1 && g_particle_block != 0) return g_particle_block;
    return group_size(precision, n_p, kHalfGroup);
}

int track_grid(int *grid_out) {
    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    CCT_TRY_CUDA(cudaGetDevice(&dev));
    CCT_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CCT_TRY_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return set_error(CCT_ERR_UNSUPPORTED, "device %d has no cooperative launch", dev);
    // both tracking kernels are launched with this grid: the smaller of their occupancies
    int per_sm_tiny = 0;
    CCT_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, track_kernel, kTrackBlock, 0));
    CCT_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_tiny, track_tiny_kernel, kTrackBlock, 0));
    per_sm = std::min(per_sm, per_sm_tiny);
    if (per_sm < 1) return set_error(CCT_ERR_UNSUPPORTED, "tracking kernel does not fit on an SM");
    *grid_out = sms * per_sm;
    return CCT_OK;
}

int g_units_per_cta = kUnitsPerCta;

// Dataflow schedule for batches of at least kFlowMinBlocks particle blocks (their stage
// particle updates overlap other blocks' field sums); smaller batches keep the two grid
// barriers per stage, whose particle update runs on every CTA at once.
void set_flow(TrackParams &P, unsigned char *flow) {
    P.blocks = (P.n_p + P.G - 1) / P.G;
    P.use_flow = (int64_t)P.n_designs * P.blocks >= kFlowMinBlocks ? 1 : 0;
    P.flow_skew = g_test_flow_skew;
    P.flow_done = reinterpret_cast<unsigned long long *>(flow);
    P.flow_ready = reinterpret_cast<unsigned *>(flow + 8 * (int64_t)P.n_designs * P.blocks);
}

// Small-batch schedule: FP32c, at most kTinyMax particles in fewer than kFlowMinBlocks particle
// blocks.  Its units are planned for at most one a CTA.
bool tiny_eligible(int precision, int n_designs, int64_t n_p, int G) {
    const int64_t blocks = (n_p + G - 1) / G;
    return precision == 1 && (int64_t)n_designs * n_p <= kTinyMax && (int64_t)n_designs * blocks < kFlowMinBlocks;
}

// Its fixed-point accumulators (copies x 2 x particles x 3 int64) and flag counts (copies x 2 x
// particles) take the start of the partial-sum region, which it does not otherwise use;
// `partial_units` is what that region holds, and sets how many copies (up to kTinyCopies) fit.
void set_tiny(TrackParams &P, bool eligible, int64_t partial_units) {
    const int64_t total = (int64_t)P.n_designs * P.n_p;
    const int64_t room = 24 * (int64_t)P.G * partial_units;
    const int64_t copies = std::min<int64_t>(kTinyCopies, total > 0 ? room / (56 * total) : 0);
    P.tiny = (eligible && !P.use_flow && copies >= 1) ? 1 : 0;
    P.tiny_copies = P.tiny ? (int)copies : 1;
    P.tiny_acc = reinterpret_cast<long long *>(P.partial);
    P.tiny_bad = reinterpret_cast<unsigned *>(P.partial + 6 * total * P.tiny_copies);
}

int64_t plan_units(const int64_t *hoff, int n_designs, int64_t n_p, int G, int grid, int64_t max_units,
                   int64_t *unit_off, int64_t *chunks, int64_t *chunk_tiles) {
    return plan_units_hd(hoff, n_designs, n_p, G, (int64_t)g_units_per_cta * grid, grid, max_units, unit_off, chunks,
                         chunk_tiles);
}

// Units the planner may use: g_units_per_cta per CTA plus one remainder chunk per (design, block).
int64_t units_bound(int n_designs, int64_t n_p, int G, int grid) {
    return (int64_t)g_units_per_cta * grid + (int64_t)n_designs * ((n_p + G - 1) / G);
}

int64_t track_scratch_bound(int n_designs, int64_t n_particles, bool block_setting) {
    int grid = 0;
    if (track_grid(&grid) != CCT_OK) {
        clear_error();
        grid = 4096;   // no device visible: a bound for any current GPU
    }
    int64_t best = 0;
    for (int prec = 0; prec < 2; ++prec) {
        const int G = block_setting ? track_group(prec, n_particles) : group_size(prec, n_particles);
        const int64_t t = track_scratch_layout(n_designs, n_particles, units_bound(n_designs, n_particles, G, grid), G).total;
        if (t > best) best = t;
    }
    return best;
}

// Largest unit count whose partial sums fit in `bytes` of scratch next to the fixed parts.
static int64_t units_fitting(int n_designs, int64_t n_p, int G, int64_t bytes) {
    const int64_t fixed = track_scratch_layout(n_designs, n_p, 0, G).total;
    return bytes > fixed + 256 ? (bytes - fixed - 256) / (24 * (int64_t)G) : 0;
}

// Shared by both entry points: validate, plan, write the tables, launch, read the status.
// hoff / tables are caller storage of n_designs+1 and 3*n_designs+1 int64.
static int run_track(const double *kls, const double *p0s, const int64_t *seg_off, const void *packed,
                     const double *qs, const int64_t *qs_off, int n_designs, double *particles, int64_t n_particles,
                     double distance, double footstep, int precision, unsigned char *sc, int64_t scratch_bytes,
                     const char *scratch_name, const char *hint, int64_t *hoff, int64_t *tables,
                     cudaStream_t st) {
    CCT_TRY_CUDA(cudaMemcpyAsync(hoff, seg_off, 8 * (n_designs + 1), cudaMemcpyDeviceToHost, st));
    CCT_TRY_CUDA(cudaStreamSynchronize(st));
    for (int d = 0; d < n_designs; ++d)
        if (hoff[d + 1] < hoff[d]) return set_error(CCT_ERR_ARG, "segment offsets decrease at design %d", d);
    if (precision == 0 && hoff[n_designs] > hoff[0] && (!kls || !p0s))
        return set_error(CCT_ERR_ARG, "FP64 tracking of %lld segments needs d_kls and d_p0s",
                         (long long)(hoff[n_designs] - hoff[0]));
    const unsigned char *tiles = nullptr;
    const int64_t *tile_off = nullptr;
    if (precision == 1) {
        int64_t ph[3];
        CCT_TRY_CUDA(cudaMemcpyAsync(ph, packed, sizeof ph, cudaMemcpyDeviceToHost, st));
        CCT_TRY_CUDA(cudaStreamSynchronize(st));
        int64_t tiles_total = 0;
        for (int d = 0; d < n_designs; ++d) tiles_total += (hoff[d + 1] - hoff[d] + kTile - 1) / kTile;
        if (ph[0] != kPackedMagic || ph[1] != n_designs || ph[2] != tiles_total)
            return set_error(CCT_ERR_ARG,
                             "packed segments do not match the %d designs' segment offsets (built by "
                             "cct_f32c_pack with the same offsets?)", n_designs);
        tile_off = reinterpret_cast<const int64_t *>(static_cast<const unsigned char *>(packed) + kPackedHeaderBytes);
        tiles = static_cast<const unsigned char *>(packed) + kPackedHeaderBytes + packed_index_bytes(n_designs);
    }
    int grid = 0;
    const int rc = track_grid(&grid);
    if (rc != CCT_OK) return rc;
    const int G = track_group(precision, n_particles);
    int64_t *unit_off = tables, *chunks = unit_off + n_designs + 1, *chunk_tiles = chunks + n_designs;
    const bool tiny = tiny_eligible(precision, n_designs, n_particles, G);
    const int64_t fitting = units_fitting(n_designs, n_particles, G, scratch_bytes);
    const int64_t n_units =
        tiny ? plan_units_hd(hoff, n_designs, n_particles, G, grid, grid, std::min<int64_t>(grid, fitting), unit_off,
                             chunks, chunk_tiles)
             : plan_units(hoff, n_designs, n_particles, G, grid, fitting, unit_off, chunks, chunk_tiles);
    const int64_t blocks = (n_particles + G - 1) / G;
    const int64_t least = track_scratch_layout(n_designs, n_particles, (int64_t)n_designs * blocks, G).total;
    if (n_units < 0)
        return set_error(CCT_ERR_ARG,
                         "%d designs x %lld particles need %lld bytes of tracking scratch; the %s holds %lld%s",
                         n_designs, (long long)n_particles, (long long)least, scratch_name, (long long)scratch_bytes,
                         hint);
    const TrackScratchLayout L = track_scratch_layout(n_designs, n_particles, n_units, G);
    if (reinterpret_cast<uintptr_t>(sc) % 256) return set_error(CCT_ERR_ARG, "tracking scratch must be 256-byte aligned");
    // the scratch keeps a previous call's contents: clear the control words, rewrite the tables
    CCT_TRY_CUDA(cudaMemsetAsync(sc, 0, kCtrlBytes, st));
    CCT_TRY_CUDA(cudaMemcpyAsync(sc + kCtrlBytes, tables, 8 * (3 * n_designs + 1), cudaMemcpyHostToDevice, st));

    TrackParams P;
    P.kls = kls;
    P.p0s = p0s;
    P.seg_off = seg_off;
    P.tiles = tiles;
    P.tile_off = tile_off;
    P.qs = qs;
    P.qs_off = qs_off;
    P.n_designs = n_designs;
    P.G = G;
    P.ppt = G >= 64 ? 2 : 1;
    P.n_p = n_particles;
    P.particles = particles;
    P.distance = distance;
    P.footstep = footstep;
    P.state = reinterpret_cast<double *>(sc + L.state_off);
    P.partial = reinterpret_cast<double *>(sc + L.partial_off);
    P.ctrl = reinterpret_cast<unsigned *>(sc);
    P.unit_off = reinterpret_cast<const int64_t *>(sc + kCtrlBytes);
    P.chunks = P.unit_off + n_designs + 1;
    P.chunk_tiles = P.chunks + n_designs;
    P.precision = precision;
    P.barrier_blocks = (unsigned)(grid + g_test_phantom_blocks);
    P.wait_ns = (unsigned long long)g_wait_ms * 1000000ull;
    P.init_from_records = 1;
    P.write_back = 1;
    P.step_begin = 0;
    P.step_end = 0x7fffffff;
    P.record = nullptr;
    set_flow(P, sc + L.flow_off);
    set_tiny(P, tiny, n_units);
    CCT_TRY_CUDA(launch_track_kernel(P, grid, st));

    unsigned ctrl[8];
    CCT_TRY_CUDA(cudaMemcpyAsync(ctrl, sc, sizeof ctrl, cudaMemcpyDeviceToHost, st));
    CCT_TRY_CUDA(cudaStreamSynchronize(st));
    if ((int)ctrl[CW_ERR] == CCT_ERR_TIMEOUT)
        return set_error(CCT_ERR_TIMEOUT, "a tracking grid barrier or tile copy waited longer than its limit (%lld ms)",
                         g_wait_ms);
    if (ctrl[CW_NONFINITE]) return set_error(CCT_ERR_NONFINITE, "a particle state or step count was not finite");
    return CCT_OK;
}

int launch_track(const double *kls, const double *p0s, const int64_t *seg_off, const void *packed, const double *qs,
                 const int64_t *qs_off, int n_designs, double *particles, int64_t n_particles, double distance,
                 double footstep, int precision, void *scratch, int64_t scratch_bytes, cudaStream_t st) {
    if (n_designs <= 0 || n_particles <= 0) return CCT_OK;
    std::vector<int64_t> hoff(n_designs + 1), tables(3 * n_designs + 1);
    return run_track(kls, p0s, seg_off, packed, qs, qs_off, n_designs, particles, n_particles, distance, footstep,
                     precision, static_cast<unsigned char *>(scratch), scratch_bytes, "caller's scratch buffer", "",
                     hoff.data(), tables.data(), st);
}

// ---------------------------------------------------------------- asynchronous form
// cct_track_async: nothing is read back to the host, so the call can be captured in a CUDA
// graph.  A one-thread kernel checks the offsets (and the packed set) and plans the units
// on the device; the tracking kernel is launched cooperatively through cudaLaunchKernelEx;
// the status stays in the scratch's control words for cct_track_status.
__global__ void plan_kernel(TrackParams P, const unsigned char *packed, int64_t target_units, int64_t min_units,
                            int64_t max_units,
                            int64_t *tables) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned *err = P.ctrl + CW_ERR;
    int64_t tiles_total = 0;
    for (int d = 0; d < P.n_designs; ++d) {
        if (P.seg_off[d + 1] < P.seg_off[d]) {
            atomicExch(err, (unsigned)CCT_ERR_ARG);
            return;
        }
        tiles_total += tiles_of(P.seg_off, d);
    }
    if (P.precision == 0 && P.seg_off[P.n_designs] > P.seg_off[0] && (!P.kls || !P.p0s)) {
        atomicExch(err, (unsigned)CCT_ERR_ARG);
        return;
    }
    if (P.precision == 1) {
        const int64_t *h = reinterpret_cast<const int64_t *>(packed);
        if (h[0] != kPackedMagic || h[1] != P.n_designs || h[2] != tiles_total) {
            atomicExch(err, (unsigned)CCT_ERR_ARG);
            return;
        }
    }
    int64_t *unit_off = tables, *chunks = unit_off + P.n_designs + 1, *chunk_tiles = chunks + P.n_designs;
    if (plan_units_hd(P.seg_off, P.n_designs, P.n_p, P.G, target_units, min_units, max_units, unit_off, chunks,
                      chunk_tiles) < 0)
        atomicExch(err, (unsigned)CCT_ERR_ARG);
}

static int g_async_grid[64];   // cached cooperative grid per device (occupancy queries stay out of captures)

int launch_track_async(const double *kls, const double *p0s, const int64_t *seg_off, const void *packed,
                       const double *qs, const int64_t *qs_off, int n_designs, double *particles, int64_t n_p,
                       double distance, double footstep, int precision, void *scratch, int64_t scratch_bytes,
                       cudaStream_t st) {
    int dev = 0;
    CCT_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_error(CCT_ERR_UNSUPPORTED, "device index %d", dev);
    if (!g_async_grid[dev]) {
        int grid = 0;
        const int rc = track_grid(&grid);
        if (rc != CCT_OK) return rc;
        g_async_grid[dev] = grid;
    }
    const int grid = g_async_grid[dev];
    unsigned char *sc = static_cast<unsigned char *>(scratch);
    if (reinterpret_cast<uintptr_t>(sc) % 256) return set_error(CCT_ERR_ARG, "tracking scratch must be 256-byte aligned");
    const int G = track_group(precision, n_p);
    const int64_t max_units = units_fitting(n_designs, n_p, G, scratch_bytes);
    if (max_units < (int64_t)n_designs * ((n_p + G - 1) / G))
        return set_error(CCT_ERR_ARG, "%d designs x %lld particles need at least %lld bytes of tracking scratch, %lld given",
                         n_designs, (long long)n_p,
                         (long long)track_scratch_layout(n_designs, n_p, (int64_t)n_designs * ((n_p + G - 1) / G), G).total,
                         (long long)scratch_bytes);
    const TrackScratchLayout L = track_scratch_layout(n_designs, n_p, max_units, G);
    TrackParams P;
    P.kls = kls;
    P.p0s = p0s;
    P.seg_off = seg_off;
    P.tiles = precision == 1 ? static_cast<const unsigned char *>(packed) + kPackedHeaderBytes +
                                   packed_index_bytes(n_designs)
                             : nullptr;
    P.tile_off = precision == 1
                     ? reinterpret_cast<const int64_t *>(static_cast<const unsigned char *>(packed) + kPackedHeaderBytes)
                     : nullptr;
    P.qs = qs;
    P.qs_off = qs_off;
    P.n_designs = n_designs;
    P.G = G;
    P.ppt = G >= 64 ? 2 : 1;
    P.n_p = n_p;
    P.particles = particles;
    P.distance = distance;
    P.footstep = footstep;
    P.state = reinterpret_cast<double *>(sc + L.state_off);
    P.partial = reinterpret_cast<double *>(sc + L.partial_off);
    P.ctrl = reinterpret_cast<unsigned *>(sc);
    P.unit_off = reinterpret_cast<const int64_t *>(sc + kCtrlBytes);
    P.chunks = P.unit_off + n_designs + 1;
    P.chunk_tiles = P.chunks + n_designs;
    P.precision = precision;
    P.barrier_blocks = (unsigned)(grid + g_test_phantom_blocks);
    P.wait_ns = (unsigned long long)g_wait_ms * 1000000ull;
    P.init_from_records = 1;
    P.write_back = 1;
    P.step_begin = 0;
    P.step_end = 0x7fffffff;
    P.record = nullptr;
    set_flow(P, sc + L.flow_off);
    const bool tiny = tiny_eligible(precision, n_designs, n_p, G);
    set_tiny(P, tiny, max_units);
    CCT_TRY_CUDA(cudaMemsetAsync(sc, 0, kCtrlBytes, st));
    plan_kernel<<<1, 32, 0, st>>>(P, static_cast<const unsigned char *>(packed),
                                  tiny ? (int64_t)grid : (int64_t)g_units_per_cta * grid, grid,
                                  tiny ? std::min<int64_t>(grid, max_units) : max_units,
                                  reinterpret_cast<int64_t *>(sc + kCtrlBytes));
    CCT_TRY_CUDA(cudaGetLastError());
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kTrackBlock);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    CCT_TRY_CUDA(cudaLaunchKernelEx(&cfg, P.tiny ? track_tiny_kernel : track_kernel, P));
    return CCT_OK;
}

int track_status(const void *scratch, cudaStream_t st) {
    unsigned ctrl[8];
    CCT_TRY_CUDA(cudaMemcpyAsync(ctrl, scratch, sizeof ctrl, cudaMemcpyDeviceToHost, st));
    CCT_TRY_CUDA(cudaStreamSynchronize(st));
    if ((int)ctrl[CW_ERR] == CCT_ERR_TIMEOUT)
        return set_error(CCT_ERR_TIMEOUT, "a tracking grid barrier or tile copy waited longer than its limit (%lld ms)",
                         g_wait_ms);
    if ((int)ctrl[CW_ERR] == CCT_ERR_ARG)
        return set_error(CCT_ERR_ARG, "the tracking plan rejected its inputs: segment offsets decrease, the packed set "
                                      "does not match them, or the scratch is too small");
    if (ctrl[CW_NONFINITE]) return set_error(CCT_ERR_NONFINITE, "a particle state or step count was not finite");
    return CCT_OK;
}

}  // namespace cctgpu

extern "C" int cct_test_set_flow_fault(int stages_ahead, int wait_ms) {
    // Test hook: dataflow waits require `stages_ahead` more finished stages than they need
    // (so that they run out), and the wait limit is shortened.
    cctgpu::g_test_flow_skew = stages_ahead < 0 ? 0 : stages_ahead;
    cctgpu::g_wait_ms = wait_ms > 0 ? wait_ms : 60000;
    return CCT_OK;
}

extern "C" int cct_test_set_barrier_fault(int phantom_blocks, int wait_ms) {
    // Test hook: count `phantom_blocks` CTAs that never arrive, and shorten the wait limit,
    // so that a test can make every barrier wait run out and check CCT_ERR_TIMEOUT.
    cctgpu::g_test_phantom_blocks = phantom_blocks < 0 ? 0 : phantom_blocks;
    cctgpu::g_wait_ms = wait_ms > 0 ? wait_ms : 60000;
    return CCT_OK;
}

extern "C" int64_t cct_test_plan_units(const int64_t *seg_off, int32_t n_designs, int64_t n_particles,
                                       int32_t precision, int32_t grid, int64_t max_units, int64_t *unit_off,
                                       int64_t *chunks, int64_t *chunk_tiles, int32_t *group) {
    // Test hook: the planner cct_track runs on the host, for a grid given by the caller.
    using namespace cctgpu;
    clear_error();
    if (n_designs <= 0 || n_particles <= 0 || grid <= 0 || (precision != 0 && precision != 1)) {
        set_error(CCT_ERR_ARG, "need designs, particles, a grid and precision 0 or 1");
        return -2;
    }
    if (!seg_off || !unit_off || !chunks || !chunk_tiles || !group) {
        set_error(CCT_ERR_ARG, "null offsets or tables");
        return -2;
    }
    for (int d = 0; d < n_designs; ++d)
        if (seg_off[d + 1] < seg_off[d]) {
            set_error(CCT_ERR_ARG, "segment offsets decrease at design %d", d);
            return -2;
        }
    const int G = track_group(precision, n_particles);
    *group = G;
    if (max_units <= 0) max_units = units_bound(n_designs, n_particles, G, grid);
    if (tiny_eligible(precision, n_designs, n_particles, G))   // small batches: at most one unit a CTA
        return plan_units_hd(seg_off, n_designs, n_particles, G, grid, grid, std::min<int64_t>(grid, max_units),
                             unit_off, chunks, chunk_tiles);
    return plan_units(seg_off, n_designs, n_particles, G, grid, max_units, unit_off, chunks, chunk_tiles);
}

// ---------------------------------------------------------------- asynchronous form, tuning
extern "C" int cct_track_async(const double *d_kls, const double *d_p0s, const int64_t *d_seg_off,
                               const void *d_packed, const double *d_qs, const int64_t *d_qs_off, int32_t n_designs,
                               double *d_particles, int64_t n_particles, double distance, double footstep,
                               int32_t precision, void *d_scratch, int64_t scratch_bytes, void *stream) {
    using namespace cctgpu;
    clear_error();
    if (n_designs <= 0 || n_particles <= 0) return set_error(CCT_ERR_ARG, "need at least one design and particle");
    if (!d_seg_off || !d_particles || !d_scratch) return set_error(CCT_ERR_ARG, "null offsets, particles or scratch");
    if (precision != 0 && precision != 1) return set_error(CCT_ERR_ARG, "precision must be 0 (FP64) or 1 (FP32c)");
    if (precision == 1 && !d_packed) return set_error(CCT_ERR_ARG, "FP32c tracking needs the packed segments");
    if (!(distance >= 0.0) || !(footstep > 0.0)) return set_error(CCT_ERR_ARG, "distance >= 0 and footstep > 0 needed");
    return launch_track_async(d_kls, d_p0s, d_seg_off, d_packed, d_qs, d_qs_off, n_designs, d_particles, n_particles,
                              distance, footstep, precision, d_scratch, scratch_bytes,
                              static_cast<cudaStream_t>(stream));
}

extern "C" int cct_track_status(const void *d_scratch, void *stream) {
    cctgpu::clear_error();
    if (!d_scratch) return cctgpu::set_error(CCT_ERR_ARG, "null scratch");
    return cctgpu::track_status(d_scratch, static_cast<cudaStream_t>(stream));
}

extern "C" int cct_track_set_units_per_cta(int32_t units_per_cta) {
    cctgpu::clear_error();
    if (units_per_cta < 0 || units_per_cta > 64)
        return cctgpu::set_error(CCT_ERR_ARG, "units per CTA %d (1..64, 0 = default)", units_per_cta);
    cctgpu::g_units_per_cta = units_per_cta == 0 ? cctgpu::kUnitsPerCta : units_per_cta;
    return CCT_OK;
}

extern "C" int32_t cct_track_units_per_cta(void) { return cctgpu::g_units_per_cta; }

extern "C" int cct_track_set_particle_block(int32_t particles) {
    cctgpu::clear_error();
    if (particles != 0 && particles != 16 && particles != 32 && particles != 64 && particles != 128 && particles != 256)
        return cctgpu::set_error(CCT_ERR_ARG, "particle block %d (16, 32, 64, 128 or 256; 0 = automatic)", particles);
    cctgpu::g_particle_block = particles;
    return CCT_OK;
}

extern "C" int32_t cct_track_particle_block(void) { return cctgpu::g_particle_block; }

namespace cctgpu {
static const int kTuneUnits[] = {2, 4, 8, 16, 32};
static const int kTuneBlocks[] = {16, 32, 64, 128, 256};
constexpr int kNumTuneUnits = (int)(sizeof kTuneUnits / sizeof kTuneUnits[0]);
constexpr int kNumTuneBlocks = (int)(sizeof kTuneBlocks / sizeof kTuneBlocks[0]);
static int64_t up256(int64_t b) { return (b + 255) / 256 * 256; }

// Particle blocks worth timing for n_p particles of one design: the automatic choice, and every
// block size up to the smallest that holds all n_p (a larger one only adds idle lanes).
static int tune_blocks(int precision, int64_t n_p, int *out) {
    if (precision == 0) {
        out[0] = 0;
        return 1;
    }
    int n = 0;
    out[n++] = 0;
    for (int i = 0; i < kNumTuneBlocks; ++i) {
        out[n++] = kTuneBlocks[i];
        if (kTuneBlocks[i] >= n_p) break;
    }
    return n;
}

// Scratch of the largest candidate split (tracking scratch of every candidate, plus a copy of
// the particle records).
static int64_t autotune_bytes(int n_designs, int64_t n_p) {
    const int saved_u = g_units_per_cta, saved_g = g_particle_block;
    int blocks[kNumTuneBlocks + 1];
    int64_t best = 0;
    for (int prec = 0; prec < 2; ++prec) {
        const int nb = tune_blocks(prec, n_p, blocks);
        for (int i = 0; i < nb; ++i) {
            g_particle_block = blocks[i];
            g_units_per_cta = kTuneUnits[kNumTuneUnits - 1];
            best = std::max(best, track_scratch_bound(n_designs, n_p));
        }
    }
    g_units_per_cta = saved_u;
    g_particle_block = saved_g;
    return up256(80 * (int64_t)n_designs * n_p) + best;
}
}  // namespace cctgpu

extern "C" int64_t cct_autotune_scratch_bytes(int32_t n_designs, int64_t n_particles) {
    using namespace cctgpu;
    clear_error();
    if (n_designs <= 0 || n_particles <= 0) {
        set_error(CCT_ERR_ARG, "need at least one design and particle");
        return -1;
    }
    return autotune_bytes(n_designs, n_particles);
}

extern "C" int cct_autotune(const double *d_kls, const double *d_p0s, const int64_t *d_seg_off, const void *d_packed,
                            const double *d_qs, const int64_t *d_qs_off, int32_t n_designs,
                            const double *d_particles, int64_t n_particles, double footstep, int32_t precision,
                            int32_t steps, void *d_scratch, int64_t scratch_bytes, int32_t *units_per_cta_out,
                            void *stream) {
    using namespace cctgpu;
    clear_error();
    if (n_designs <= 0 || n_particles <= 0 || steps < 1 || !(footstep > 0.0))
        return set_error(CCT_ERR_ARG, "need designs, particles, steps >= 1 and footstep > 0");
    if (precision != 0 && precision != 1) return set_error(CCT_ERR_ARG, "precision must be 0 (FP64) or 1 (FP32c)");
    if (!d_particles || !d_scratch || !units_per_cta_out) return set_error(CCT_ERR_ARG, "null particles, scratch or output");
    const int64_t need = autotune_bytes(n_designs, n_particles);
    if (scratch_bytes < need)
        return set_error(CCT_ERR_ARG, "autotune needs %lld bytes of scratch, %lld given", (long long)need,
                         (long long)scratch_bytes);
    const int64_t copy = up256(80 * (int64_t)n_designs * n_particles);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned char *sc = static_cast<unsigned char *>(d_scratch);
    double *work = reinterpret_cast<double *>(sc);
    const int saved_u = g_units_per_cta, saved_g = g_particle_block;
    int blocks[kNumTuneBlocks + 1];
    const int nb = tune_blocks(precision, n_particles, blocks);
    cudaEvent_t a = nullptr, b = nullptr;
    CCT_TRY_CUDA(cudaEventCreate(&a));
    CCT_TRY_CUDA(cudaEventCreate(&b));
    float best_ms = 3.4e38f;
    int best_u = saved_u, best_g = saved_g, rc = CCT_OK;
    // candidate -1: warm-up with the current setting; then every (particle block, units per CTA)
    for (int c = -1; c < nb * kNumTuneUnits && rc == CCT_OK; ++c) {
        g_units_per_cta = c < 0 ? saved_u : kTuneUnits[c % kNumTuneUnits];
        g_particle_block = c < 0 ? saved_g : blocks[c / kNumTuneUnits];
        cudaError_t e = cudaMemcpyAsync(work, d_particles, 80 * (size_t)n_designs * n_particles,
                                        cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaEventRecord(a, st);
        if (e != cudaSuccess) {
            rc = check_cuda(e, "autotune copy");
            break;
        }
        rc = launch_track(d_kls, d_p0s, d_seg_off, d_packed, d_qs, d_qs_off, n_designs, work, n_particles,
                          steps * footstep, footstep, precision, sc + copy, scratch_bytes - copy, st);
        if (rc != CCT_OK) break;
        e = cudaEventRecord(b, st);
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
        if (e != cudaSuccess) {
            rc = check_cuda(e, "autotune timing");
            break;
        }
        if (c >= 0 && ms < best_ms) {
            best_ms = ms;
            best_u = g_units_per_cta;
            best_g = g_particle_block;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    g_units_per_cta = rc == CCT_OK ? best_u : saved_u;
    g_particle_block = rc == CCT_OK ? best_g : saved_g;
    if (rc == CCT_OK) *units_per_cta_out = best_u;
    return rc;
}

// ============================================================================
// Tracking without device allocation.
//
// Some callers cannot allocate device memory once they are running: a treatment-planning
// or optimisation host that reserves its GPU memory at start-up and forbids cudaMalloc on
// its hot path (an allocation there can fail mid-run or stall the device), or a plain C
// caller that owns only the buffers it was handed.  cct_track_static_scratch gives them
// the tracking kernel with its scratch in a fixed, file-scope device array instead of a
// caller-provided buffer.  The array takes its device memory when this file's CUDA module is
// loaded on a device -- under lazy module loading, its first use there -- and keeps it until
// the process exits; cct_track_static_scratch_bytes() looks the array up on the current
// device so that a start-up call places it before the caller reserves its memory.  Its size
// bounds the problem (see cctgpu.h).  All calls share it, so calls whose kernels overlap on
// the GPU race on it; each call rewrites every word it reads before the kernel starts.
// ============================================================================
namespace cctgpu {

constexpr int64_t kStaticScratchBytes = 32LL << 20;   // 32 MiB
constexpr int kStaticMaxDesigns = 64;
constexpr int kStaticMaxDevices = 64;

static __device__ __align__(256) unsigned char g_track_static_scratch[kStaticScratchBytes];
static void *g_static_scratch_addr[kStaticMaxDevices];
static std::mutex g_static_scratch_mutex;

// Device address of the static scratch on the current device.  The first call on a
// device looks the symbol up (cudaGetSymbolAddress) with that device current and keeps the
// address for the life of the process (a cudaDeviceReset of that device would make it stale).
static int static_scratch_address(void **out) {
    int dev = 0;
    CCT_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kStaticMaxDevices)
        return set_error(CCT_ERR_UNSUPPORTED, "device ordinal %d beyond %d", dev, kStaticMaxDevices);
    std::lock_guard<std::mutex> lock(g_static_scratch_mutex);
    if (!g_static_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_track_static_scratch);
        if (e != cudaSuccess) return check_cuda(e, "cudaGetSymbolAddress(static tracking scratch)");
        g_static_scratch_addr[dev] = p;
    }
    *out = g_static_scratch_addr[dev];
    return CCT_OK;
}

static int launch_track_static(const double *kls, const double *p0s, const int64_t *seg_off, const void *packed,
                               const double *qs, const int64_t *qs_off, int n_designs, double *particles,
                               int64_t n_particles, double distance, double footstep, int precision,
                               cudaStream_t st) {
    if (n_designs > kStaticMaxDesigns)
        return set_error(CCT_ERR_ARG, "%d designs exceed the %d the static-scratch entry point takes", n_designs,
                         kStaticMaxDesigns);
    void *scratch = nullptr;
    const int rc = static_scratch_address(&scratch);
    if (rc != CCT_OK) return rc;
    int64_t hoff[kStaticMaxDesigns + 1];
    int64_t tables[3 * kStaticMaxDesigns + 1];
    return run_track(kls, p0s, seg_off, packed, qs, qs_off, n_designs, particles, n_particles, distance, footstep,
                     precision, static_cast<unsigned char *>(scratch), kStaticScratchBytes, "static scratch",
                     " (use cct_track with a caller buffer)", hoff, tables, st);
}

}  // namespace cctgpu

extern "C" int64_t cct_track_static_scratch_bytes(void) {
    // With a device visible, also look the array up on the current device: that loads this
    // file's module there and so commits the array, letting a start-up call place it before
    // the application reserves its memory.  Without a device only the size is returned.
    int n = 0;
    if (cudaGetDeviceCount(&n) == cudaSuccess && n > 0) {
        void *p = nullptr;
        if (cctgpu::static_scratch_address(&p) != CCT_OK) cctgpu::clear_error();
    } else {
        (void)cudaGetLastError();
    }
    return cctgpu::kStaticScratchBytes;
}

extern "C" int cct_track_static_scratch(const double *d_kls, const double *d_p0s, const int64_t *d_seg_off,
                                        const void *d_packed, const double *d_qs, const int64_t *d_qs_off,
                                        int32_t n_designs, double *d_particles, int64_t n_particles, double distance,
                                        double footstep, int32_t precision, void *stream) {
    using namespace cctgpu;
    clear_error();
    if (n_designs <= 0 || n_particles < 0) return set_error(CCT_ERR_ARG, "need at least one design");
    if (n_particles == 0) return CCT_OK;
    if (!(distance > 0.0) || !(footstep > 0.0))
        return set_error(CCT_ERR_ARG, "distance (%g) and footstep (%g) must be positive", distance, footstep);
    if (precision != 0 && precision != 1) return set_error(CCT_ERR_ARG, "precision must be 0 or 1");
    if (!d_seg_off || !d_qs_off || !d_particles) return set_error(CCT_ERR_ARG, "null pointer");
    if (precision == 1 && (!d_packed || reinterpret_cast<uintptr_t>(d_packed) % 256))
        return set_error(CCT_ERR_ARG, "FP32c tracking needs a 256-byte aligned packed buffer");
    return launch_track_static(d_kls, d_p0s, d_seg_off, d_packed, d_qs, d_qs_off, n_designs, d_particles,
                               n_particles, distance, footstep, precision, static_cast<cudaStream_t>(stream));
}
