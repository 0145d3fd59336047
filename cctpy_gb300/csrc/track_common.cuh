// Device-side pieces of the tracking kernels shared by track.cu (forward RK4) and
// adjoint.cu (checkpointed reverse sweep): parameters, shared memory, bounded grid barrier,
// unit decomposition, the phase-A field sums and the phase-C RK4 bookkeeping.
#pragma once

#include "cctgpu_internal.cuh"
#include "qs.cuh"
#include "tile.cuh"

namespace cctgpu {

// 4 warps per CTA, 3 CTAs per SM (up to 168 registers a thread): measured faster than 8 CTAs
// of 2 warps capped at 128 registers (gantry section 1890 -> 1950 Gpairs/s)
constexpr int kTrackBlock = 128;
constexpr int kTrackMinBlocks = 3;
constexpr int kTrackWarps = kTrackBlock / 32;
static_assert((kTile / kTrackWarps) % kSub == 0, "tile slices hold whole FP32c sub-blocks");
constexpr int kMaxGroup = 64 * kTrackWarps;   // particles per unit: 2 per lane in every warp
constexpr int kHalfGroup = 16;                 // smallest FP32c particle block: a particle per half-warp lane
constexpr int kStateD = 24;          // doubles of RK4 state per particle
constexpr int kMaxChunks = 4096;     // chunks per (design, block)
constexpr int kUnitsPerCta = 8;      // default target units per CTA and stage (dynamic load balance)
constexpr int kMinChunkTiles = 32;   // smallest chunk (tiles) a unit covers, given enough units for every CTA
constexpr int kRing = 4;             // TMA ring depth (tiles)
constexpr int kTrackUnroll = 8;      // unroll of the 4-segment loop of a sub-block (8: fully)
constexpr int kGradUnroll = 4;       // the same in the adjoint's gradient sums
constexpr bool kTrackRcp = false;     // |r|^-3 as rsqrt x rcp in the tracking field sums (tile.cuh inv_r3)
constexpr int kRedDoubles = kMaxGroup * 3;   // per-CTA reduction buffer: S slices x G particles x 3
constexpr uint32_t kTmaPolls = 1u << 22;

// control words (CW_SEQ: a 64-bit counter in words 8-9)
enum { CW_COUNT = 0, CW_GEN = 1, CW_ERR = 2, CW_NONFINITE = 3, CW_MAXSTEPS = 4, CW_NEXT0 = 5, CW_NEXT1 = 6, CW_SEQ = 8 };

// Control block at the start of the scratch: the words above in its first 128-byte line, then
// one line per group of units of the small-batch schedule (a 64-bit count of finished units
// each, on its own line so that the groups' additions do not queue on one L2 line).  The unit
// tables follow it.
constexpr int kCtrlBytes = 4096;
constexpr int kCtrlLineWords = 32;
constexpr int kTinyGroups = kCtrlBytes / 128 - 1;      // lines 1..31
constexpr int kCtrlTinyCount = kCtrlLineWords;          // word index of the first group's counter

// Small batches (FP32c, at most kTinyMax particles in fewer than kFlowMinBlocks particle
// blocks): every CTA owns at most one unit for the whole launch and keeps its own copy of every
// particle's RK4 state in shared memory.  A unit adds its chunk's field into per-particle
// fixed-point accumulators (int64, kTinyScale units a tesla; two stage parities; never cleared:
// a stage's field is the difference from the previous reading of the same parity, exact in
// integers, so it does not depend on the order the units arrive in) and counts itself done;
// every CTA waits for the stage's count, reads the accumulators and advances its copy of every
// particle (all copies identical: same integers, same arithmetic).  No grid barrier and no
// serial section per stage; a unit whose tiles fit the ring keeps them in shared memory.  The
// accumulators come in up to kTinyCopies copies (unit u adds into copy u % copies), so that the
// units' atomic additions spread over more addresses; readers add the copies up.
constexpr int kTinyMax = 64;
constexpr int kTinyCopies = 8;    // measured on C0 (32 protons): 2 -> 12.5, 4 -> 10.0, 8 -> 9.1, 12 -> 9.9, 16 -> 10.1 us a stage
constexpr int kTinyShift = 44;                          // fixed point: 2^-44 T, 5.7e-14 T resolution
constexpr double kTinyScale = 17592186044416.0;        // 2^kTinyShift
constexpr int kTinyRange = 18;                          // unit fields below 2^18 T: far inside int64
static_assert(kTinyShift + kTinyRange + 1 <= 63, "fixed-point fields (< 2^62) and their differences fit int64");

// Dataflow schedule (batches of at least kFlowMinBlocks particle blocks): per particle block a
// 64-bit count of finished chunk units and a 32-bit count of finished stages.
constexpr int kFlowMinBlocks = 8;
constexpr int kFlowBytesPerBlock = 16;

// state layout per particle
enum { ST_Y0 = 0, ST_YS = 6, ST_KSUM = 12, ST_DT = 18, ST_KQ = 19, ST_NSTEPS = 20 };

struct TrackParams {
    const double *kls, *p0s;
    const int64_t *seg_off;
    const unsigned char *tiles;    // FP32c tiles base (precision 1)
    const int64_t *tile_off;       // FP32c per-design first tile (precision 1)
    const double *qs;
    const int64_t *qs_off;
    int n_designs;
    int G;                         // particles per unit
    int ppt;                       // particles per lane in FP32c phase A (1 or 2)
    int64_t n_p;
    double *particles;
    double distance, footstep;
    double *state, *partial;
    unsigned *ctrl;
    const int64_t *unit_off;       // [n_designs+1] first unit of each design
    const int64_t *chunks;         // [n_designs] chunks per block
    const int64_t *chunk_tiles;    // [n_designs] tiles per chunk
    int precision;
    unsigned barrier_blocks;       // CTAs expected at each barrier
    unsigned long long wait_ns;    // barrier wait limit
    // step range and I/O of one launch (the adjoint runs the track in checkpoint segments)
    int init_from_records;         // 1: state from the particle records (and step count)
    int write_back;                // 1: write the final state into the particle records
    int step_begin, step_end;      // steps [step_begin, min(step_end, step count)) run here
    double *record;                // null, or per (step, stage, particle): stage state + field
    // small-batch schedule (tiny = 1): fixed-point field accumulators and, per particle, a count
    // of unit fields that were non-finite or out of range
    int tiny;
    int tiny_copies;               // copies of the accumulators (1..kTinyCopies)
    long long *tiny_acc;           // [copies][2][particles][3]
    unsigned *tiny_bad;            // [copies][2][particles]
    // dataflow schedule (use_flow = 1): per particle block (design d, block b at d * blocks + b)
    int use_flow;
    int flow_skew;                 // test hook: extra stages every wait requires (0 in use)
    int64_t blocks;                // particle blocks per design
    unsigned long long *flow_done; // units finished, all stages of this launch
    unsigned *flow_ready;          // stages whose particle update is complete
};

// record entry of one (step, stage, particle): stage Y (6), B at the stage position (3),
// adjoint weight a = kq (lambda_v x v) written by the reverse sweep (3)
constexpr int kRec = 12;

struct TrackSmem {
    unsigned char ring[kRing][kTileBytes];
    uint64_t full[kRing];
    uint32_t last_issued[kRing];   // ring tile index last copied into each slot (kNone: none)
    int released[kRing];           // warps done with the slot's current tile
    double red[kRedDoubles];
    int64_t unit;                  // unit handed to this CTA (dynamic schedule)
    int verdict;
    // small-batch schedule: this CTA's copy of every particle's RK4 state, its last reading of
    // each stage parity's accumulators (3 components and the flag count) per particle, and each
    // particle's design's QS record range
    double tiny_state[kTinyMax * kStateD];
    long long tiny_prev[2 * kTinyMax * 4];
    int64_t tiny_qs[kTinyMax][2];
    float tiny_pts[kTinyMax][6];   // each particle's stage position as double-float (hi xyz, lo xyz)
};
constexpr uint32_t kNone = 0xffffffffu;

// Ring set-up by thread 0 at kernel start (made visible by the kernel's first barrier).
static __device__ __forceinline__ void ring_init(TrackSmem &sm) {
    for (int s = 0; s < kRing; ++s) {
        cctdev::mbar_init(&sm.full[s], 1);
        sm.last_issued[s] = kNone;
        sm.released[s] = 0;
    }
    cctdev::mbar_fence_init();
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void set_timeout(const TrackParams &P) {
    atomicCAS(reinterpret_cast<int *>(P.ctrl + CW_ERR), 0, (int)CCT_ERR_TIMEOUT);
}

// Grid-wide barrier with a wall-clock limit; every thread of the CTA returns the same
// verdict (false = some CTA timed out, stop).
static __device__ bool grid_barrier(const TrackParams &P, TrackSmem &sm) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *gen = P.ctrl + CW_GEN;
        volatile int *err = reinterpret_cast<volatile int *>(P.ctrl + CW_ERR);
        const unsigned g = *gen;
        __threadfence();
        const unsigned prev = atomicAdd(P.ctrl + CW_COUNT, 1u);
        if (prev == P.barrier_blocks - 1) {
            atomicExch(P.ctrl + CW_COUNT, 0u);
            __threadfence();
            atomicAdd(P.ctrl + CW_GEN, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            unsigned polls = 0;
            while (*gen == g) {
                if (*err == CCT_ERR_TIMEOUT) break;
                if ((++polls & 255u) == 0 && global_ns() - t0 > P.wait_ns) {
                    set_timeout(P);
                    break;
                }
                __nanosleep(128);
            }
        }
        __threadfence();
        sm.verdict = (*err == CCT_ERR_TIMEOUT) ? 0 : 1;
    }
    __syncthreads();
    return sm.verdict != 0;
}

// Unit schedule.  In every phase CTA b first takes unit b; further units come from counter
// CW_NEXT0 + (k & 1) of phase k, offset by the grid size (so a phase with no more units than
// CTAs costs no atomic at all).  The other counter is cleared during the phase's particle
// step (reset_next_unit, after the grid barrier that ends the unit phase), so it is zero
// again when phase k + 1 starts.  Every unit writes its partial sums to its own slots, so
// which CTA takes which unit does not change any result.
static __device__ __forceinline__ int64_t first_unit() { return (int64_t)blockIdx.x; }
static __device__ __forceinline__ int64_t next_unit(const TrackParams &P, TrackSmem &sm, int phase) {
    __syncthreads();   // the previous value has been read by every thread
    if (threadIdx.x == 0) sm.unit = (int64_t)gridDim.x + (int64_t)atomicAdd(P.ctrl + CW_NEXT0 + (phase & 1), 1u);
    __syncthreads();
    return sm.unit;
}
// Dataflow schedule: one sequence over all stages of the launch, unit u of stage k at
// k * n_units + u.  CTA b first takes b, further entries come from the 64-bit counter CW_SEQ.
static __device__ __forceinline__ int64_t claim_seq(const TrackParams &P, TrackSmem &sm) {
    __syncthreads();
    if (threadIdx.x == 0)
        sm.unit = (int64_t)gridDim.x +
                  (int64_t)atomicAdd(reinterpret_cast<unsigned long long *>(P.ctrl + CW_SEQ), 1ull);
    __syncthreads();
    return sm.unit;
}
static __device__ __forceinline__ void reset_next_unit(const TrackParams &P, int phase) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(P.ctrl + CW_NEXT0 + ((phase + 1) & 1), 0u);
}
// At kernel start, before the first grid barrier.
static __device__ __forceinline__ void clear_unit_counters(const TrackParams &P) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicExch(P.ctrl + CW_NEXT0, 0u);
        atomicExch(P.ctrl + CW_NEXT1, 0u);
        atomicExch(reinterpret_cast<unsigned long long *>(P.ctrl + CW_SEQ), 0ull);
    }
    if (P.use_flow) {
        const int64_t n_blk = (int64_t)P.n_designs * P.blocks;
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_blk; i += (int64_t)gridDim.x * blockDim.x) {
            P.flow_done[i] = 0ull;
            P.flow_ready[i] = 0u;
        }
    }
}

// Thread 0, after a wait gave up: let the last copy into every ring slot land before the
// CTA's shared memory is given up (earlier copies into a slot were consumed before its refill).
static __device__ void ring_drain(TrackSmem &sm) {
    for (int s = 0; s < kRing; ++s)
        if (sm.last_issued[s] != kNone)
            (void)cctdev::mbar_wait_bounded(&sm.full[s], (sm.last_issued[s] / kRing) & 1u, kTmaPolls);
}

// Dataflow: wait (thread 0 polls, wall-clock limit) until particle block `blk` has finished
// `k` stages, i.e. its stage-k positions are written.  CTA-uniform verdict; false = stop.
static __device__ bool flow_wait(const TrackParams &P, TrackSmem &sm, int64_t blk, int k) {
    if (threadIdx.x == 0) {
        volatile unsigned *ready = P.flow_ready + blk;
        volatile int *err = reinterpret_cast<volatile int *>(P.ctrl + CW_ERR);
        int ok = *err == CCT_ERR_TIMEOUT ? 0 : 1;
        k += P.flow_skew;
        if (ok && (int)*ready < k) {
            // back off (64 ns doubling to 4 us): many CTAs polling a few hot words would
            // otherwise load the L2 slices that also serve the running units' tiles
            const unsigned long long t0 = global_ns();
            unsigned polls = 0, nap = 64;
            while ((int)*ready < k) {
                if ((++polls & 15u) == 0) {
                    if (*err == CCT_ERR_TIMEOUT) {
                        ok = 0;
                        break;
                    }
                    if (global_ns() - t0 > P.wait_ns) {
                        set_timeout(P);
                        ok = 0;
                        break;
                    }
                }
                __nanosleep(nap);
                if (nap < 4096) nap *= 2;
            }
        }
        __threadfence();
        sm.verdict = ok;
    }
    __syncthreads();
    return sm.verdict != 0;
}

// Dataflow: the calling CTA has written the partial sums of one unit of block `blk` at stage
// k; true (CTA-uniform) if it was the block's last unit of that stage (cd units per stage).
static __device__ bool flow_complete(const TrackParams &P, TrackSmem &sm, int64_t blk, int k, int64_t cd) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned long long prev = atomicAdd(P.flow_done + blk, 1ull);
        const bool last = (long long)prev + 1 == (long long)(k + 1) * cd;
        if (last) __threadfence();
        sm.verdict = last;
    }
    __syncthreads();
    return sm.verdict != 0;
}

// cross product with the reference's component formula (point.py:402-410), unfused
__device__ __forceinline__ void cross_rn(double ax, double ay, double az, double bx, double by, double bz,
                                         double &cx, double &cy, double &cz) {
    cx = __dadd_rn(__dmul_rn(ay, bz), -__dmul_rn(az, by));
    cy = __dadd_rn(-__dmul_rn(ax, bz), __dmul_rn(az, bx));
    cz = __dadd_rn(__dmul_rn(ax, by), -__dmul_rn(ay, bx));
}

struct UnitRef {
    int d;
    int64_t b, c, t_beg, t_end;
};

__device__ __forceinline__ UnitRef locate_unit(const TrackParams &P, int64_t u) {
    int lo = 0, hi = P.n_designs - 1;   // last d with unit_off[d] <= u
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (P.unit_off[mid] <= u) lo = mid; else hi = mid - 1;
    }
    UnitRef r;
    r.d = lo;
    const int64_t cd = P.chunks[lo], local = u - P.unit_off[lo];
    r.b = local / cd;
    r.c = local % cd;
    const int64_t nt = (P.seg_off[lo + 1] - P.seg_off[lo] + kTile - 1) / kTile;
    const int64_t ct = P.chunk_tiles[lo];
    r.t_beg = r.c * ct;
    r.t_end = min(nt, (r.c + 1) * ct);
    return r;
}

// Phase A, FP64: G = 32, warps split the chunk's tiles, lane = particle.  A warp takes a
// tile's segments 32 at a time: lane l loads segment l of the group and forms its moment
// m = kl x (p0 - o) about the tile's first midpoint o, then the group's segments are broadcast
// lane to lane and every lane sums A = sum kl |r|^-3, M = sum m |r|^-3 for its particle; the
// tile's field is A x (p - o) - M (the moment form of the field kernel, in FP64).
// HALF: blocks of kHalfGroup particles: lanes l and l + 16 hold particle l and sum the first
// and the second 16 segments of each group of 32 (an FP64 warp instruction costs the same
// with half its lanes idle, so designs of at most 16 particles would otherwise run at half
// rate); the halves are added lane l + 16 into lane l before the CTA reduction.
template <bool HALF = false>
static __device__ void unit_field_f64(const TrackParams &P, int64_t u, TrackSmem &sm) {
    const UnitRef U = locate_unit(P, u);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int G = HALF ? kHalfGroup : 32;
    constexpr int KN = HALF ? 16 : 32;                 // segments of a group summed by a lane
    const int pl = HALF ? (lane & 15) : lane, k0 = HALF ? (lane & 16) : 0;
    int64_t j = U.b * G + pl;
    if (j >= P.n_p) j = P.n_p - 1;
    const double *Ys = P.state + ((int64_t)U.d * P.n_p + j) * kStateD + ST_YS;
    const double px = Ys[0], py = Ys[1], pz = Ys[2];
    double bx = 0.0, by = 0.0, bz = 0.0;
    const int64_t s_beg = P.seg_off[U.d], s_end = P.seg_off[U.d + 1];
    for (int64_t t = U.t_beg + warp; t < U.t_end; t += kTrackWarps) {
        const int64_t a = s_beg + t * kTile, e = min(s_end, a + kTile);
        const double ox = __ldg(P.p0s + 3 * a), oy = __ldg(P.p0s + 3 * a + 1), oz = __ldg(P.p0s + 3 * a + 2);
        const double wx = px - ox, wy = py - oy, wz = pz - oz;
        double Ax = 0.0, Ay = 0.0, Az = 0.0, Mx = 0.0, My = 0.0, Mz = 0.0;
        for (int64_t g = a; g < e; g += 32) {
            const int64_t s = g + lane;
            double kx = 0.0, ky = 0.0, kz = 0.0, qx = 1.0e18, qy = 1.0e18, qz = 1.0e18;
            if (s < e) {
                kx = __ldg(P.kls + 3 * s);
                ky = __ldg(P.kls + 3 * s + 1);
                kz = __ldg(P.kls + 3 * s + 2);
                qx = __ldg(P.p0s + 3 * s) - ox;
                qy = __ldg(P.p0s + 3 * s + 1) - oy;
                qz = __ldg(P.p0s + 3 * s + 2) - oz;
            }
            const double mx = ky * qz - kz * qy, my = kz * qx - kx * qz, mz = kx * qy - ky * qx;
            // past the tile's end a lane holds kl = 0 far away, whose terms are exactly zero:
            // half-warps run all 16 of theirs (a warp-uniform count for the shuffles)
            const int n = HALF ? KN : (int)min((int64_t)32, e - g);
            for (int kk = 0; kk < n; ++kk) {
                const int k = k0 + kk;
                const double skx = __shfl_sync(0xffffffffu, kx, k), sky = __shfl_sync(0xffffffffu, ky, k),
                             skz = __shfl_sync(0xffffffffu, kz, k);
                const double sqx = __shfl_sync(0xffffffffu, qx, k), sqy = __shfl_sync(0xffffffffu, qy, k),
                             sqz = __shfl_sync(0xffffffffu, qz, k);
                const double smx = __shfl_sync(0xffffffffu, mx, k), smy = __shfl_sync(0xffffffffu, my, k),
                             smz = __shfl_sync(0xffffffffu, mz, k);
                const double rx = wx - sqx, ry = wy - sqy, rz = wz - sqz;
                const double inv = rsqrt(rx * rx + ry * ry + rz * rz);
                const double inv3 = inv * inv * inv;
                Ax += skx * inv3;
                Ay += sky * inv3;
                Az += skz * inv3;
                Mx += smx * inv3;
                My += smy * inv3;
                Mz += smz * inv3;
            }
        }
        bx += (Ay * wz - Az * wy) - Mx;
        by += (Az * wx - Ax * wz) - My;
        bz += (Ax * wy - Ay * wx) - Mz;
    }
    if (HALF) {
        bx += __shfl_down_sync(0xffffffffu, bx, 16);
        by += __shfl_down_sync(0xffffffffu, by, 16);
        bz += __shfl_down_sync(0xffffffffu, bz, 16);
    }
    double *red = sm.red + (warp * G + pl) * 3;
    if (lane < G) {
        red[0] = bx;
        red[1] = by;
        red[2] = bz;
    }
    __syncthreads();
    if (warp == 0 && lane < G) {
        double sx = 0.0, sy = 0.0, sz = 0.0;
        for (int w = 0; w < kTrackWarps; ++w) {
            const double *r = sm.red + (w * G + lane) * 3;
            sx += r[0];
            sy += r[1];
            sz += r[2];
        }
        double *out = P.partial + (u * G + lane) * 3;
        out[0] = sx;
        out[1] = sy;
        out[2] = sz;
    }
    __syncthreads();
}

// Where phase A reads its points: the position of particle pi is at pos + pi * pos_stride;
// for the adjoint's gradient sums the per-point weight a is at w + pi * w_stride.
struct PointSrc {
    const double *pos;
    int64_t pos_stride;
    const double *w;
    int64_t w_stride;
};

__device__ __forceinline__ PointSrc stage_points(const TrackParams &P) {
    return PointSrc{P.state + ST_YS, kStateD, nullptr, 0};
}

// Issue the first ring tiles of unit u (thread 0 only; the ring is idle: every tile of the
// previous unit has been consumed and no refill past a unit's end is ever issued).
static __device__ __forceinline__ void unit_prefetch(const TrackParams &P, int64_t u, TrackSmem &sm, uint32_t kt) {
    if (threadIdx.x != 0) return;
    const UnitRef U = locate_unit(P, u);
    const unsigned char *tiles = P.tiles + (P.tile_off[U.d] + U.t_beg) * (int64_t)kTileBytes;
    const int64_t nt = U.t_end - U.t_beg;
    for (int64_t t = 0; t < kRing && t < nt; ++t) {
        const int s = (int)((kt + t) % kRing);
        sm.last_issued[s] = kt + (uint32_t)t;
        cctdev::fence_proxy_async();
        cctdev::mbar_arrive_expect_tx(&sm.full[s], kTileBytes);
        cctdev::bulk_g2s(sm.ring[s], tiles + t * (int64_t)kTileBytes, kTileBytes, &sm.full[s]);
    }
}

// Phase A, FP32c, for unit u whose first tiles unit_prefetch has issued: the unit's tiles
// stream through the shared-memory ring (TMA).  GRAD = false: field sums B at the points;
// GRAD = true: gradient sums grad_p (a . B) with the per-point weights of `src`.  `kt` counts
// the tiles this CTA has consumed (ring slot and phase parity).  Once the tiles are done it
// claims the CTA's next unit of the phase and issues that unit's first tiles, so that their
// copies overlap this unit's reduction.  Returns the next unit (>= n_units: none), or -1 if a
// TMA wait gave up (CCT_ERR_TIMEOUT recorded).
// round(x * 2^kTinyShift) of an FP32 value by integer operations (no FP64 or 64-bit
// conversion: both run at GB300's low FP64 rate), halves rounded away from zero; kTinyBad for
// |x| >= 2^kTinyRange T, infinities and NaN.
constexpr long long kTinyBad = (long long)0x8000000000000000ull;
__device__ __forceinline__ long long fixed44(float x) {
    const unsigned b = __float_as_uint(x);
    const int e = (int)((b >> 23) & 0xffu);
    if (e >= 127 + kTinyRange) return kTinyBad;
    if (e == 0) return 0;                                   // zero, or below 2^-126
    const long long m = (long long)((b & 0x7fffffu) | 0x800000u);
    const int sh = e - (127 + 23 - kTinyShift);            // x 2^44 = m 2^(e - 127 - 23 + 44)
    long long v = 0;
    if (sh >= 0) v = m << sh;                               // < 2^24 2^38 = 2^62
    else if (sh >= -24) v = (m + (1ll << (-sh - 1))) >> (-sh);
    return (b >> 31) ? -v : v;
}

// A compensated FP32 pair (S, C) as fixed point: fixed44(S) - fixed44(C), or kTinyBad.
__device__ __forceinline__ long long fixed44_pair(float S, float C) {
    const long long a = fixed44(S), c = fixed44(C);
    if (a == kTinyBad || c == kTinyBad) return kTinyBad;
    return a - c;                                           // |a|, |c| < 2^62
}

// Small-batch schedule: unit u adds its field at particle pi, in fixed point, into its copy of
// the accumulators of stage parity `parity` (kTinyBad components count on the particle's flag).
static __device__ __forceinline__ void tiny_add_fixed(const TrackParams &P, int64_t u, int parity, int64_t pi,
                                                      const long long (&v)[3]) {
    const int64_t total = (int64_t)P.n_designs * P.n_p;
    const int64_t slot = ((u % P.tiny_copies) * 2 + parity) * total + pi;
    unsigned long long *acc = reinterpret_cast<unsigned long long *>(P.tiny_acc + slot * 3);
    bool bad = false;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (v[c] != kTinyBad) atomicAdd(acc + c, (unsigned long long)v[c]);
        else bad = true;
    }
    if (bad) atomicAdd(P.tiny_bad + slot, 1u);
}

// (TINY: the unit's reduced field goes to the small-batch accumulators; resident: the unit's
// nt <= kRing tiles already sit in ring slots 0..nt-1 from an earlier stage of this CTA's only
// unit; known: the unit's description, if the caller has it.)
// HALF: blocks of kHalfGroup particles (PPT 1): lanes l and l + 16 of a warp hold particle l.
// A tile is shared by a pair of warps (warps 0-1 take the even tiles, 2-3 the odd ones), each
// half-warp summing one whole 32-segment sub-block of it, so that the per-tile work of a
// thread (offsets from the tile origin, the sub-block epilogue, the compensated add) covers
// 32 segments rather than 16.
template <int PPT, bool GRAD, bool FLOW = false, bool TINY = false, bool HALF = false>
static __device__ int64_t unit_sum_f32c(const TrackParams &P, const PointSrc &src, int64_t u, TrackSmem &sm,
                                        uint32_t &kt, int phase, int64_t n_units, int64_t n_seq = 0,
                                        bool resident = false, const UnitRef *known = nullptr) {
    static_assert(!HALF || (PPT == 1 && !GRAD), "half-warp blocks: one particle a lane, forward sums only");
    const UnitRef U = known ? *known : locate_unit(P, u);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int G = P.G;
    const int NB = HALF ? 1 : G / (32 * PPT);                      // particle sub-blocks
    const int S = HALF ? 2 * kTrackWarps : kTrackWarps / NB;       // slices of each tile
    const int sb = HALF ? 0 : warp % NB;
    const int sl = HALF ? 2 * warp + (lane >> 4) : warp / NB;
    const int pl0 = HALF ? (lane & 15) : sb * 32 * PPT + lane;       // this lane's first particle slot
    constexpr int TW = HALF ? kTrackWarps / 2 : 1;                  // tiles in flight across the warps
    constexpr int WPT = kTrackWarps / TW;                            // warps consuming each tile
    static_assert(!HALF || 2 * WPT * kSub == kTile, "HALF: a warp pair's four half-warps cover a tile");
    static_assert(kRing % TW == 0, "a ring slot holds tiles of one warp pair");
    const int g0 = HALF ? (2 * (warp % WPT) + (lane >> 4)) * (kSub / 4) : sl * (kTile / 4 / S);
    const int g1 = HALF ? g0 + kSub / 4 : g0 + kTile / 4 / S;

    float ph[PPT][3], pl[PPT][3], a[PPT][3];
#pragma unroll
    for (int i = 0; i < PPT; ++i) {
        int64_t j = U.b * G + pl0 + i * 32;
        if (j >= P.n_p) j = P.n_p - 1;
        const int64_t pi = (int64_t)U.d * P.n_p + j;
        if (TINY) {   // the CTA's own double-float copy of the position
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                ph[i][c] = sm.tiny_pts[pi][c];
                pl[i][c] = sm.tiny_pts[pi][3 + c];
            }
        } else {
            const double *Ys = src.pos + pi * src.pos_stride;
#pragma unroll
            for (int c = 0; c < 3; ++c) split_df(Ys[c], ph[i][c], pl[i][c]);
        }
        if (GRAD) {
#pragma unroll
            for (int c = 0; c < 3; ++c) a[i][c] = (float)src.w[pi * src.w_stride + c];
        }
    }
    F32cAcc<PPT> acc;
    acc.zero();

    const int64_t nt = U.t_end - U.t_beg;
    // Warps run through the ring independently: a warp waits only for its next tile to
    // land; the last warp done with a slot refills it with the tile kRing further on (HALF:
    // a slot holds tiles of one parity, kRing being even, and so one warp pair's).
    bool ok_all = true;
    for (int64_t t = HALF ? warp / WPT : 0; t < nt; t += TW) {
        const uint32_t k = kt + (uint32_t)t;
        const int s = resident ? (int)t : (int)(k % kRing);
        if (!resident) {
            const bool ok = cctdev::mbar_wait_bounded(&sm.full[s], (k / kRing) & 1u, kTmaPolls);
            if (!__all_sync(0xffffffffu, ok)) {
                ok_all = false;
                break;
            }
        }
        if (GRAD) tile_grad_f32c<PPT, kGradUnroll>(sm.ring[s], ph, pl, a, acc, g0, g1);
        else tile_f32c<PPT, kTrackUnroll, kTrackRcp>(sm.ring[s], ph, pl, acc, g0, g1);
        if (resident) continue;
        if (cctdev::ring_release_last(&sm.released[s], WPT) && t + kRing < nt) {
            const unsigned char *tiles = P.tiles + (P.tile_off[U.d] + U.t_beg) * (int64_t)kTileBytes;
            sm.last_issued[s] = k + kRing;
            cctdev::fence_proxy_async();
            cctdev::mbar_arrive_expect_tx(&sm.full[s], kTileBytes);
            cctdev::bulk_g2s(sm.ring[s], tiles + (t + kRing) * (int64_t)kTileBytes, kTileBytes, &sm.full[s]);
        }
    }
    if (__syncthreads_or(!ok_all)) {
        if (tid == 0) {
            set_timeout(P);
            ring_drain(sm);
        }
        __syncthreads();
        return -1;
    }
    if (!resident) kt += (uint32_t)nt;
    // all warps are past their last tile: claim the next unit and start its copies, so that
    // they overlap this unit's reduction (FLOW: the caller claims after the unit is counted,
    // so that a CTA that then runs a block update holds no claimed unit meanwhile)
    int64_t next = 0;
    if (!FLOW) {
        next = next_unit(P, sm, phase);
        if (next < n_units) unit_prefetch(P, next, sm, kt);
    }

    if (TINY) {   // small batches: the slices' fields in fixed point, summed in integers
        long long *ri = reinterpret_cast<long long *>(sm.red);
#pragma unroll
        for (int i = 0; i < PPT; ++i)
#pragma unroll
            for (int c = 0; c < 3; ++c) ri[((size_t)sl * G + pl0 + i * 32) * 3 + c] = fixed44_pair(acc.S[i][c], acc.C[i][c]);
        __syncthreads();
        for (int slot = tid; slot < G; slot += kTrackBlock) {
            long long v[3] = {0, 0, 0};
            for (int q = 0; q < S; ++q)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const long long t = ri[((size_t)q * G + slot) * 3 + c];
                    v[c] = (v[c] == kTinyBad || t == kTinyBad)
                               ? kTinyBad
                               : (long long)((unsigned long long)v[c] + (unsigned long long)t);
                }
            const int64_t j = U.b * G + slot;
            if (j < P.n_p) tiny_add_fixed(P, u, phase & 1, (int64_t)U.d * P.n_p + j, v);
        }
    } else {   // reduce the S slices of every particle in fixed order
#pragma unroll
        for (int i = 0; i < PPT; ++i) {
            double *r = sm.red + ((size_t)sl * G + pl0 + i * 32) * 3;
            r[0] = acc.total(i, 0);
            r[1] = acc.total(i, 1);
            r[2] = acc.total(i, 2);
        }
        __syncthreads();
        for (int slot = tid; slot < G; slot += kTrackBlock) {
            double sx = 0.0, sy = 0.0, sz = 0.0;
            for (int q = 0; q < S; ++q) {
                const double *r = sm.red + ((size_t)q * G + slot) * 3;
                sx += r[0];
                sy += r[1];
                sz += r[2];
            }
            double *out = P.partial + (u * G + slot) * 3;
            out[0] = sx;
            out[1] = sy;
            out[2] = sz;
        }
    }
    __syncthreads();
    return next;
}

// All FP32c units of one phase handed to this CTA.  Returns false if a TMA wait gave up.
template <int PPT, bool GRAD, bool HALF = false>
static __device__ bool units_f32c(const TrackParams &P, const PointSrc &src, TrackSmem &sm, uint32_t &kt, int phase,
                                  int64_t n_units) {
    int64_t u = first_unit();
    if (u < n_units) unit_prefetch(P, u, sm, kt);
    while (u < n_units) {
        u = unit_sum_f32c<PPT, GRAD, false, false, HALF>(P, src, u, sm, kt, phase, n_units);
        if (u < 0) return false;
    }
    return true;
}

// Sum of the chunk partials of particle pi by the calling warp (all 32 lanes, converged):
// lane l adds chunks l, l + 32, ... into four accumulators in a fixed pattern, then a fixed
// shuffle tree; lane 0 gets the total.  A fixed order (deterministic), and the chunk loads of one particle are spread
// over the warp instead of one thread walking them in sequence.
static __device__ __forceinline__ void warp_sum_partials(const TrackParams &P, int64_t pi, double out[3]) {
    const int lane = threadIdx.x & 31;
    const int d = (int)(pi / P.n_p);
    const int64_t j = pi % P.n_p;
    const int64_t b = j / P.G, slot = j % P.G;
    const int64_t cd = P.chunks[d];
    const int64_t u0 = P.unit_off[d] + b * cd;
    // four independent accumulators, so that a lane has up to 12 loads in flight
    double a[4][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
    int64_t c = lane;
    for (; c + 96 < cd; c += 128) {
        double v[4][3];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const double *p = P.partial + ((u0 + c + 32 * k) * P.G + slot) * 3;
            v[k][0] = p[0];
            v[k][1] = p[1];
            v[k][2] = p[2];
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int q = 0; q < 3; ++q) a[k][q] += v[k][q];
    }
    for (; c < cd; c += 32) {
        const double *p = P.partial + ((u0 + c) * P.G + slot) * 3;
        a[0][0] += p[0];
        a[0][1] += p[1];
        a[0][2] += p[2];
    }
    double x = (a[0][0] + a[1][0]) + (a[2][0] + a[3][0]);
    double y = (a[0][1] + a[1][1]) + (a[2][1] + a[3][1]);
    double z = (a[0][2] + a[1][2]) + (a[2][2] + a[3][2]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        x += __shfl_down_sync(0xffffffffu, x, o);
        y += __shfl_down_sync(0xffffffffu, y, o);
        z += __shfl_down_sync(0xffffffffu, z, o);
    }
    out[0] = x;
    out[1] = y;
    out[2] = z;
}

// The same sum by the whole CTA (for batches with no more particles than CTAs, where the
// particle update is the latency of the stage): thread t adds chunks t, t + blockDim, ... into
// four accumulators in a fixed pattern, then a fixed-order tree in shared memory; all threads
// get the total.
static __device__ void cta_sum_partials(const TrackParams &P, int64_t pi, double out[3], TrackSmem &sm) {
    const int tid = threadIdx.x;
    const int d = (int)(pi / P.n_p);
    const int64_t j = pi % P.n_p;
    const int64_t b = j / P.G, slot = j % P.G;
    const int64_t cd = P.chunks[d];
    const int64_t u0 = P.unit_off[d] + b * cd;
    double a[4][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
    int64_t c = tid;
    for (; c + 3 * kTrackBlock < cd; c += 4 * kTrackBlock) {
        double v[4][3];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const double *p = P.partial + ((u0 + c + k * kTrackBlock) * P.G + slot) * 3;
            v[k][0] = p[0];
            v[k][1] = p[1];
            v[k][2] = p[2];
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int q = 0; q < 3; ++q) a[k][q] += v[k][q];
    }
    for (; c < cd; c += kTrackBlock) {
        const double *p = P.partial + ((u0 + c) * P.G + slot) * 3;
        a[0][0] += p[0];
        a[0][1] += p[1];
        a[0][2] += p[2];
    }
    double *red = sm.red;   // kRedDoubles >= 3 * kTrackBlock
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 3; ++q) red[3 * tid + q] = (a[0][q] + a[1][q]) + (a[2][q] + a[3][q]);
    __syncthreads();
    for (int w = kTrackBlock / 2; w > 0; w >>= 1) {
        if (tid < w) {
#pragma unroll
            for (int q = 0; q < 3; ++q) red[3 * tid + q] += red[3 * (tid + w) + q];
        }
        __syncthreads();
    }
    out[0] = red[0];
    out[1] = red[1];
    out[2] = red[2];
    __syncthreads();
}
static_assert(kRedDoubles >= 3 * kTrackBlock, "CTA partial-sum buffer");

// True while particle pi still has RK4 steps at `step`.
__device__ __forceinline__ bool particle_active(const TrackParams &P, int64_t pi, int step) {
    return (double)step < P.state[pi * kStateD + ST_NSTEPS];
}

// Phase C for one particle at RK4 stage `stage` (0..3) of step `step`, given the CCT field
// B (sum of the chunk partials; QS are added here).
static __device__ void particle_update_at(const TrackParams &P, double *S, int64_t pi, int step, int stage,
                                          const double Bc[3], int64_t q0, int64_t q1) {
    if ((double)step >= S[ST_NSTEPS]) return;
    double B[3] = {Bc[0], Bc[1], Bc[2]};
    const double *Ys = S + ST_YS;
    for (int64_t q = q0; q < q1; ++q)
        qs_field_add(P.qs + kQsRecord * q, Ys[0], Ys[1], Ys[2], B[0], B[1], B[2]);
    if (P.record) {
        double *rec = P.record + (((int64_t)(step - P.step_begin) * 4 + stage) * ((int64_t)P.n_designs * P.n_p) + pi) * kRec;
        for (int c = 0; c < 6; ++c) rec[c] = Ys[c];
        rec[6] = B[0];
        rec[7] = B[1];
        rec[8] = B[2];
    }

    // k = [v_s, kq * (v_s x B)]
    double k[6];
    k[0] = Ys[3];
    k[1] = Ys[4];
    k[2] = Ys[5];
    double ax, ay, az;
    cross_rn(Ys[3], Ys[4], Ys[5], B[0], B[1], B[2], ax, ay, az);
    const double kq = S[ST_KQ];
    k[3] = __dmul_rn(ax, kq);
    k[4] = __dmul_rn(ay, kq);
    k[5] = __dmul_rn(az, kq);

    const double dt = S[ST_DT];
    double *Y0 = S + ST_Y0, *Yn = S + ST_YS, *ks = S + ST_KSUM;
    if (stage == 0) {
        const double h = dt / 2;
        for (int c = 0; c < 6; ++c) {
            ks[c] = k[c];
            Yn[c] = __dadd_rn(Y0[c], __dmul_rn(h, k[c]));
        }
    } else if (stage == 1 || stage == 2) {
        const double h = stage == 1 ? dt / 2 : dt;
        for (int c = 0; c < 6; ++c) {
            ks[c] = __dadd_rn(ks[c], __dmul_rn(2.0, k[c]));
            Yn[c] = __dadd_rn(Y0[c], __dmul_rn(h, k[c]));
        }
    } else {
        const double h = dt / 6;
        bool finite = true;
        for (int c = 0; c < 6; ++c) {
            ks[c] = __dadd_rn(ks[c], k[c]);
            Y0[c] = __dadd_rn(Y0[c], __dmul_rn(h, ks[c]));
            Yn[c] = Y0[c];
            finite = finite && isfinite(Y0[c]);
        }
        if (!finite) atomicExch(P.ctrl + CW_NONFINITE, 1u);
    }
}

// The same for the particle's state in P.state, with its design's QS records.
static __device__ __forceinline__ void particle_update(const TrackParams &P, int64_t pi, int step, int stage,
                                                       const double Bc[3]) {
    const int d = (int)(pi / P.n_p);
    particle_update_at(P, P.state + pi * kStateD, pi, step, stage, Bc, P.qs_off[d], P.qs_off[d + 1]);
}

// Small-batch schedule: after stage `phase` is complete, every particle's field for it from the
// accumulators of its parity (all copies, read from L2; integer sums, exact in any order) minus
// this CTA's previous reading of them, and this CTA's copy of the particle advanced.  A thread
// a particle: the particles' FP64 updates then share as few warps as possible (an FP64 warp
// instruction costs the FP64 pipe about the same with few lanes active as with all).
static __device__ void tiny_advance(const TrackParams &P, TrackSmem &sm, int step, int stage, int phase) {
    const int64_t total = (int64_t)P.n_designs * P.n_p;
    const int par = phase & 1;
    for (int64_t pi = threadIdx.x; pi < total; pi += blockDim.x) {
        unsigned long long a[3] = {0ull, 0ull, 0ull};
        unsigned bad = 0u;
        for (int r = 0; r < P.tiny_copies; ++r) {
            const int64_t slot = ((int64_t)r * 2 + par) * total + pi;
            const unsigned long long *acc = reinterpret_cast<const unsigned long long *>(P.tiny_acc + slot * 3);
#pragma unroll
            for (int c = 0; c < 3; ++c) a[c] += __ldcg(acc + c);
            bad += __ldcg(P.tiny_bad + slot);
        }
        long long *prev = sm.tiny_prev + ((int64_t)par * kTinyMax + pi) * 4;
        const bool nonfinite = (long long)bad != prev[3];
        double B[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const long long f = (long long)(a[c] - (unsigned long long)prev[c]);
            B[c] = nonfinite ? __longlong_as_double(0x7ff8000000000000LL) : __ll2double_rn(f) * (1.0 / kTinyScale);
            prev[c] = (long long)a[c];
        }
        prev[3] = (long long)bad;
        double *S = sm.tiny_state + pi * kStateD;
        if ((double)step < S[ST_NSTEPS]) {
            particle_update_at(P, S, pi, step, stage, B, sm.tiny_qs[pi][0], sm.tiny_qs[pi][1]);
#pragma unroll
            for (int c = 0; c < 3; ++c) split_df(S[ST_YS + c], sm.tiny_pts[pi][c], sm.tiny_pts[pi][3 + c]);
        }
    }
}

// Dataflow: block (d, b) has finished stage k of its field sums.  Sums each of its particles'
// chunk partials, calls fn(pi, B) for it (the thread that summed it), and marks the block
// ready for stage k + 1.  A thread takes up to kMaxGroup / kTrackBlock particles at once and
// sums their partials in chunk order (four accumulators per particle, combined in a fixed
// pattern: deterministic); neighbouring threads read neighbouring particles' partials, and
// each thread keeps 12 loads per particle in flight.
template <typename Fn>
static __device__ void block_finish(const TrackParams &P, int d, int64_t b, int k, Fn fn) {
    constexpr int R = kMaxGroup / kTrackBlock;   // particles per thread
    const int G = P.G;
    const int64_t cd = P.chunks[d];
    const int64_t stride = (int64_t)G * 3;       // doubles between a particle's chunk partials
    const double *base = P.partial + (P.unit_off[d] + b * cd) * stride;
    double a[R][4][3];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) a[r][q][0] = a[r][q][1] = a[r][q][2] = 0.0;
    int64_t c = 0;
    for (; c + 4 <= cd; c += 4) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int slot = threadIdx.x + r * kTrackBlock;
            if (slot >= G) break;
            double v[4][3];
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int x = 0; x < 3; ++x) v[q][x] = base[(c + q) * stride + slot * 3 + x];
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int x = 0; x < 3; ++x) a[r][q][x] += v[q][x];
        }
    }
    for (; c < cd; ++c) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int slot = threadIdx.x + r * kTrackBlock;
            if (slot >= G) break;
#pragma unroll
            for (int x = 0; x < 3; ++x) a[r][0][x] += base[c * stride + slot * 3 + x];
        }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int slot = threadIdx.x + r * kTrackBlock;
        const int64_t j = b * G + slot;
        if (slot >= G || j >= P.n_p) continue;
        double B[3];
#pragma unroll
        for (int x = 0; x < 3; ++x) B[x] = (a[r][0][x] + a[r][1][x]) + (a[r][2][x] + a[r][3][x]);
        fn((int64_t)d * P.n_p + j, B);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicExch(P.flow_ready + (int64_t)d * P.blocks + b, (unsigned)(k + 1));
    }
}

// Forward tracking: stage k of the launch is stage k % 4 of step step_begin + k / 4.
static __device__ void block_update(const TrackParams &P, int d, int64_t b, int k) {
    const int step = P.step_begin + k / 4, stage = k % 4;
    block_finish(P, d, b, k, [&](int64_t pi, const double *B) {
        if (particle_active(P, pi, step)) particle_update(P, pi, step, stage, B);
    });
}

// ---------------------------------------------------------------- unit planner (host and device)
__host__ __device__ inline int64_t hd_max(int64_t a, int64_t b) { return a > b ? a : b; }
__host__ __device__ inline int64_t hd_min(int64_t a, int64_t b) { return a < b ? a : b; }
__host__ __device__ inline int64_t tiles_of(const int64_t *seg_off, int d) {
    return (seg_off[d + 1] - seg_off[d] + kTile - 1) / kTile;
}

// Units are (design, particle block of G, chunk of ct tiles).  Every chunk of every design
// spans the same ct tiles (the last one of a design fewer), with ct chosen for about
// target_units units -- fewer if the chunks would then cover less than kMinChunkTiles tiles,
// but not fewer than min_units (the CTAs) -- and at most max_units.  Fills unit_off[n+1], chunks[n], chunk_tiles[n];
// returns the unit count, or -1 if one chunk per (design, block) is already more than
// max_units.  The host plans cct_track's units with it, a one-thread kernel those of
// cct_track_async.
__host__ __device__ inline int64_t plan_units_hd(const int64_t *seg_off, int n_designs, int64_t n_p, int G,
                                                 int64_t target_units, int64_t min_units, int64_t max_units,
                                                 int64_t *unit_off, int64_t *chunks, int64_t *chunk_tiles) {
    const int64_t blocks = (n_p + G - 1) / G;
    int64_t work = 0, max_nt = 1;
    for (int d = 0; d < n_designs; ++d) {
        const int64_t nt = hd_max(tiles_of(seg_off, d), 1);
        work += blocks * nt;
        max_nt = hd_max(max_nt, nt);
    }
    // no smaller chunks than kMinChunkTiles tiles, unless that leaves fewer units than min_units
    const int64_t by_size = (work + kMinChunkTiles - 1) / kMinChunkTiles;
    const int64_t target = hd_max(1, hd_min(hd_max(min_units, hd_min(target_units, by_size)), max_units));
    int64_t ct = hd_max(hd_max((work + target - 1) / target, (max_nt + kMaxChunks - 1) / kMaxChunks), 1);
    for (;;) {
        int64_t units = 0;
        for (int d = 0; d < n_designs; ++d) {
            const int64_t nt = tiles_of(seg_off, d);
            units += blocks * (nt > 0 ? (nt + ct - 1) / ct : 1);
        }
        if (units <= max_units) break;
        if (ct >= max_nt) return -1;
        ct = hd_min(max_nt, ct + hd_max(1, ct / 8));
    }
    unit_off[0] = 0;
    for (int d = 0; d < n_designs; ++d) {
        const int64_t nt = tiles_of(seg_off, d);
        const int64_t cd = nt > 0 ? (nt + ct - 1) / ct : 1;
        chunks[d] = cd;
        chunk_tiles[d] = nt > 0 ? ct : 1;
        unit_off[d + 1] = unit_off[d] + blocks * cd;
    }
    return unit_off[n_designs];
}

// ---------------------------------------------------------------- host helpers (track.cu)
extern int g_units_per_cta;
extern int g_test_phantom_blocks;
extern int g_test_flow_skew;
extern long long g_wait_ms;
extern int g_particle_block;
int group_size(int precision, int64_t n_p, int min_group = 32);
int track_group(int precision, int64_t n_p);
int track_grid(int *grid_out);
int64_t plan_units(const int64_t *hoff, int n_designs, int64_t n_p, int G, int grid, int64_t max_units, int64_t *unit_off,
                   int64_t *chunks, int64_t *chunk_tiles);
int64_t units_bound(int n_designs, int64_t n_p, int G, int grid);
cudaError_t launch_track_kernel(TrackParams &P, int grid, cudaStream_t st);
void set_flow(TrackParams &P, unsigned char *flow);
bool tiny_eligible(int precision, int n_designs, int64_t n_p, int G);
void set_tiny(TrackParams &P, bool eligible, int64_t partial_units);

}  // namespace cctgpu
