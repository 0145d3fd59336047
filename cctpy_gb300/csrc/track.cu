// Batched RK4 proton tracking through CCT beamlines: one cooperative persistent launch.
//
// Reference semantics (cctpy): ParticleRunner.run_only particles.py:562-596, RK4
// BaseUtils.runge_kutta4 base_utils.py:264-311, callback Y' = [v, (e/rm) v x B(p)]
// particles.py:515-537, beamline field beamline.py:46-53.
//
// Work decomposition.  Each design's particles are cut into blocks of G particles and its
// segments into tiles of 128, the tiles into chunks.  A unit is (design, block, chunk).
// Every RK4 stage runs two phases separated by grid barriers:
//   A. each CTA takes units (u = blockIdx.x, += gridDim.x) and computes the chunk's field at
//      the stage positions of the block's particles:
//        FP32c: the chunk's packed tiles stream into a shared-memory ring by TMA bulk copies;
//               every warp reads every tile; a warp owns 32*PPT particles and a 128/S-segment
//               slice of each tile (S = 8 * 32 * PPT / G), lanes hold particles;
//        FP64:  G = 32, the 8 warps split the chunk's tiles, lane = particle, segments are
//               read with warp-uniform loads;
//      the S slices are reduced in fixed order and one partial per (unit, particle) is stored;
//   C. each thread takes particles, sums the chunk partials of its particle in fixed order,
//      adds the analytic QS fields and advances the RK4 bookkeeping.
// Grid barriers count on a global word and have a wall-clock limit after which the kernel
// records CCT_ERR_TIMEOUT and returns; TMA waits are bounded too.  No wait is unbounded.
#include <cstdlib>
#include <mutex>
#include <vector>

#include "cctgpu_internal.cuh"
#include "qs.cuh"
#include "tile.cuh"

namespace cctgpu {

constexpr int kTrackBlock = 256;
constexpr int kTrackWarps = kTrackBlock / 32;
constexpr int kStateD = 24;          // doubles of RK4 state per particle
constexpr int kMaxChunks = 4096;     // chunks per (design, block)
constexpr int kUnitsPerCta = 4;      // target units per CTA and stage (load balance)
constexpr int kRing = 4;             // TMA ring depth (tiles)
constexpr int kRedDoubles = 512 * 3; // per-CTA reduction buffer: S slices x G particles x 3
constexpr uint32_t kTmaPolls = 1u << 22;

// control words
enum { CW_COUNT = 0, CW_GEN = 1, CW_ERR = 2, CW_NONFINITE = 3, CW_MAXSTEPS = 4 };

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
};

struct TrackSmem {
    unsigned char ring[kRing][kTileBytes];
    uint64_t full[kRing];
    double red[kRedDoubles];
    int verdict;
};

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
__device__ bool grid_barrier(const TrackParams &P, TrackSmem &sm) {
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

// Phase A, FP64: G = 32, warps split the chunk's tiles, lane = particle.
__device__ void unit_field_f64(const TrackParams &P, int64_t u, TrackSmem &sm) {
    const UnitRef U = locate_unit(P, u);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t j = U.b * 32 + lane;
    if (j >= P.n_p) j = P.n_p - 1;
    const double *Ys = P.state + ((int64_t)U.d * P.n_p + j) * kStateD + ST_YS;
    const double px = Ys[0], py = Ys[1], pz = Ys[2];
    double bx = 0.0, by = 0.0, bz = 0.0;
    const int64_t s_beg = P.seg_off[U.d], s_end = P.seg_off[U.d + 1];
    for (int64_t t = U.t_beg + warp; t < U.t_end; t += kTrackWarps) {
        const int64_t a = s_beg + t * kTile, e = min(s_end, a + kTile);
        double tx = 0.0, ty = 0.0, tz = 0.0;
        for (int64_t s = a; s < e; ++s) {
            const double kx = __ldg(P.kls + 3 * s), ky = __ldg(P.kls + 3 * s + 1), kz = __ldg(P.kls + 3 * s + 2);
            const double rx = px - __ldg(P.p0s + 3 * s), ry = py - __ldg(P.p0s + 3 * s + 1),
                         rz = pz - __ldg(P.p0s + 3 * s + 2);
            const double inv = rsqrt(rx * rx + ry * ry + rz * rz);
            const double inv3 = inv * inv * inv;
            tx += (ky * rz - kz * ry) * inv3;
            ty += (kz * rx - kx * rz) * inv3;
            tz += (kx * ry - ky * rx) * inv3;
        }
        bx += tx;
        by += ty;
        bz += tz;
    }
    double *red = sm.red + (warp * 32 + lane) * 3;
    red[0] = bx;
    red[1] = by;
    red[2] = bz;
    __syncthreads();
    if (warp == 0) {
        double sx = 0.0, sy = 0.0, sz = 0.0;
        for (int w = 0; w < kTrackWarps; ++w) {
            const double *r = sm.red + (w * 32 + lane) * 3;
            sx += r[0];
            sy += r[1];
            sz += r[2];
        }
        double *out = P.partial + (u * 32 + lane) * 3;
        out[0] = sx;
        out[1] = sy;
        out[2] = sz;
    }
    __syncthreads();
}

// Phase A, FP32c: the chunk's tiles stream through the shared-memory ring (TMA).
// `kt` counts the tiles this CTA has consumed so far (ring slot and phase parity).
// Returns false if a TMA wait gave up (CCT_ERR_TIMEOUT recorded).
template <int PPT>
__device__ bool unit_field_f32c(const TrackParams &P, int64_t u, TrackSmem &sm, uint32_t &kt) {
    const UnitRef U = locate_unit(P, u);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int G = P.G;
    const int NB = G / (32 * PPT);                 // particle sub-blocks
    const int S = kTrackWarps / NB;                // slices of each tile
    const int sb = warp % NB, sl = warp / NB;
    const int g0 = sl * (kTile / 4 / S), g1 = g0 + kTile / 4 / S;

    float ph[PPT][3], pl[PPT][3];
#pragma unroll
    for (int i = 0; i < PPT; ++i) {
        int64_t j = U.b * G + sb * 32 * PPT + i * 32 + lane;
        if (j >= P.n_p) j = P.n_p - 1;
        const double *Ys = P.state + ((int64_t)U.d * P.n_p + j) * kStateD + ST_YS;
#pragma unroll
        for (int c = 0; c < 3; ++c) split_df(Ys[c], ph[i][c], pl[i][c]);
    }
    F32cAcc<PPT> acc;
    acc.zero();

    const unsigned char *tiles = P.tiles + (P.tile_off[U.d] + U.t_beg) * (int64_t)kTileBytes;
    const int64_t nt = U.t_end - U.t_beg;
    if (tid == 0) {
        for (int64_t t = 0; t < kRing && t < nt; ++t) {
            const int s = (int)((kt + t) % kRing);
            cctdev::fence_proxy_async();
            cctdev::mbar_arrive_expect_tx(&sm.full[s], kTileBytes);
            cctdev::bulk_g2s(sm.ring[s], tiles + t * (int64_t)kTileBytes, kTileBytes, &sm.full[s]);
        }
    }
    bool ok_all = true;
    for (int64_t t = 0; t < nt; ++t) {
        const uint32_t k = kt + (uint32_t)t;
        const int s = (int)(k % kRing);
        const bool ok = cctdev::mbar_wait_bounded(&sm.full[s], (k / kRing) & 1u, kTmaPolls);
        if (__syncthreads_or(!ok)) {   // also: all threads are done with tile t-1
            ok_all = false;
            break;
        }
        if (tid == 0 && t >= 1 && t - 1 + kRing < nt) {
            const int sp = (int)((k - 1) % kRing);
            cctdev::fence_proxy_async();
            cctdev::mbar_arrive_expect_tx(&sm.full[sp], kTileBytes);
            cctdev::bulk_g2s(sm.ring[sp], tiles + (t - 1 + kRing) * (int64_t)kTileBytes, kTileBytes, &sm.full[sp]);
        }
        tile_f32c<PPT>(sm.ring[s], ph, pl, acc, g0, g1);
    }
    if (!ok_all) {
        if (tid == 0) {
            set_timeout(P);
            for (int s = 0; s < kRing; ++s) (void)cctdev::mbar_wait_bounded(&sm.full[s], 0, 1024);
        }
        __syncthreads();
        return false;
    }
    kt += (uint32_t)nt;

    // reduce the S slices of every particle in fixed order
#pragma unroll
    for (int i = 0; i < PPT; ++i) {
        double *r = sm.red + ((size_t)sl * G + sb * 32 * PPT + i * 32 + lane) * 3;
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
    __syncthreads();
    return true;
}

// Phase C for one particle at RK4 stage `stage` (0..3) of step `step`.
__device__ void particle_update(const TrackParams &P, int64_t pi, int step, int stage) {
    double *S = P.state + pi * kStateD;
    if ((double)step >= S[ST_NSTEPS]) return;
    const int d = (int)(pi / P.n_p);
    const int64_t j = pi % P.n_p;
    const int64_t b = j / P.G, slot = j % P.G;
    const int64_t cd = P.chunks[d];
    const int64_t u0 = P.unit_off[d] + b * cd;
    double B[3] = {0.0, 0.0, 0.0};
    for (int64_t c = 0; c < cd; ++c) {
        const double *p = P.partial + ((u0 + c) * P.G + slot) * 3;
        B[0] += p[0];
        B[1] += p[1];
        B[2] += p[2];
    }
    const double *Ys = S + ST_YS;
    for (int64_t q = P.qs_off[d]; q < P.qs_off[d + 1]; ++q)
        qs_field_add(P.qs + kQsRecord * q, Ys[0], Ys[1], Ys[2], B[0], B[1], B[2]);

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

__global__ void __launch_bounds__(kTrackBlock) track_kernel(TrackParams P) {
    __shared__ __align__(128) TrackSmem sm;
    const int64_t total = (int64_t)P.n_designs * P.n_p;
    const int64_t tstride = (int64_t)gridDim.x * blockDim.x;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kRing; ++s) cctdev::mbar_init(&sm.full[s], 1);
        cctdev::mbar_fence_init();
    }
    uint32_t kt = 0;   // tiles consumed through the ring by this CTA

    // init: state from the particle records; step count and dt as the CPU reference computes them
    for (int64_t pi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pi < total; pi += tstride) {
        const double *r = P.particles + pi * 10;
        double *S = P.state + pi * kStateD;
        for (int c = 0; c < 6; ++c) S[ST_Y0 + c] = S[ST_YS + c] = r[c];
        const double speed = r[8];
        const double dt0 = P.footstep / speed;
        const double t_end = P.distance / speed;
        const double steps = ceil(t_end / dt0);
        S[ST_KQ] = r[7] / r[6];
        const bool ok = isfinite(steps) && steps >= 1.0 && steps < 1.0e9;
        S[ST_NSTEPS] = ok ? steps : 0.0;
        S[ST_DT] = ok ? t_end / steps : 0.0;
        if (!ok) atomicExch(P.ctrl + CW_NONFINITE, 1u);
        else atomicMax(P.ctrl + CW_MAXSTEPS, (unsigned)steps);
    }
    if (!grid_barrier(P, sm)) return;
    const int max_steps = (int)*(volatile unsigned *)(P.ctrl + CW_MAXSTEPS);
    const int64_t n_units = P.unit_off[P.n_designs];

    for (int step = 0; step < max_steps; ++step) {
        for (int stage = 0; stage < 4; ++stage) {
            bool ok = true;
            for (int64_t u = blockIdx.x; u < n_units && ok; u += gridDim.x) {
                if (P.precision == 0) unit_field_f64(P, u, sm);
                else if (P.ppt == 2) ok = unit_field_f32c<2>(P, u, sm, kt);
                else ok = unit_field_f32c<1>(P, u, sm, kt);
            }
            if (!grid_barrier(P, sm)) return;
            for (int64_t pi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pi < total; pi += tstride)
                particle_update(P, pi, step, stage);
            if (!grid_barrier(P, sm)) return;
        }
    }

    for (int64_t pi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pi < total; pi += tstride) {
        double *r = P.particles + pi * 10;
        const double *S = P.state + pi * kStateD;
        for (int c = 0; c < 6; ++c) r[c] = S[ST_Y0 + c];
        if (S[ST_NSTEPS] > 0.0) r[9] = r[9] + P.distance;
    }
}

// ---------------------------------------------------------------- host side
static int g_test_phantom_blocks = 0;
static long long g_wait_ms = 60000;

TrackScratchLayout track_scratch_layout(int n_designs, int64_t n_particles, int64_t n_units, int group) {
    TrackScratchLayout L;
    auto up = [](int64_t b) { return (b + 255) / 256 * 256; };
    const int64_t tables = up(8 * (int64_t)(3 * n_designs + 1));
    L.ctrl_off = 0;
    L.state_off = 256 + tables;
    L.partial_off = L.state_off + up(8 * kStateD * (int64_t)n_designs * n_particles);
    L.total = L.partial_off + up(24 * (int64_t)group * n_units);
    return L;
}

// Particles per unit: FP64 keeps 32 (warps split the tiles); FP32c takes the largest block
// the batch fills, so that every warp reads every staged tile.
static int group_size(int precision, int64_t n_p) {
    if (precision == 0) return 32;
    int G = 512;
    while (G > 32 && n_p < G) G /= 2;
    return G;
}

static int track_grid(int *grid_out) {
    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    CCT_TRY_CUDA(cudaGetDevice(&dev));
    CCT_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CCT_TRY_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return set_error(CCT_ERR_UNSUPPORTED, "device %d has no cooperative launch", dev);
    CCT_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, track_kernel, kTrackBlock, 0));
    if (per_sm < 1) return set_error(CCT_ERR_UNSUPPORTED, "tracking kernel does not fit on an SM");
    *grid_out = sms * per_sm;
    return CCT_OK;
}

static int64_t chunks_wanted(int grid, int n_designs, int64_t blocks) {
    const int64_t target = (int64_t)kUnitsPerCta * grid;
    int64_t want = (target + (int64_t)n_designs * blocks - 1) / ((int64_t)n_designs * blocks);
    return want < 1 ? 1 : (want > kMaxChunks ? kMaxChunks : want);
}

// Fills unit_off[n+1], chunks[n], chunk_tiles[n] (caller storage); returns the unit count.
static int64_t plan_units(const int64_t *hoff, int n_designs, int64_t n_p, int G, int grid, int64_t *unit_off,
                          int64_t *chunks, int64_t *chunk_tiles) {
    const int64_t blocks = (n_p + G - 1) / G;
    const int64_t want = chunks_wanted(grid, n_designs, blocks);
    unit_off[0] = 0;
    for (int d = 0; d < n_designs; ++d) {
        const int64_t nt = (hoff[d + 1] - hoff[d] + kTile - 1) / kTile;
        const int64_t ct = nt > 0 ? (nt + want - 1) / want : 1;
        const int64_t cd = nt > 0 ? (nt + ct - 1) / ct : 1;
        chunks[d] = cd;
        chunk_tiles[d] = ct;
        unit_off[d + 1] = unit_off[d] + blocks * cd;
    }
    return unit_off[n_designs];
}

int64_t track_scratch_bound(int n_designs, int64_t n_particles) {
    int grid = 0;
    if (track_grid(&grid) != CCT_OK) {
        clear_error();
        grid = 4096;   // no device visible: a bound for any current GPU
    }
    int64_t best = 0;
    for (int prec = 0; prec < 2; ++prec) {
        const int G = group_size(prec, n_particles);
        const int64_t blocks = (n_particles + G - 1) / G;
        const int64_t units = (int64_t)n_designs * blocks * chunks_wanted(grid, n_designs, blocks);
        const int64_t t = track_scratch_layout(n_designs, n_particles, units, G).total;
        if (t > best) best = t;
    }
    return best;
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
    const int G = group_size(precision, n_particles);
    int64_t *unit_off = tables, *chunks = unit_off + n_designs + 1, *chunk_tiles = chunks + n_designs;
    const int64_t n_units = plan_units(hoff, n_designs, n_particles, G, grid, unit_off, chunks, chunk_tiles);
    const TrackScratchLayout L = track_scratch_layout(n_designs, n_particles, n_units, G);
    if (scratch_bytes < L.total)
        return set_error(CCT_ERR_ARG,
                         "%d designs x %lld particles need %lld bytes of tracking scratch; the %s holds %lld%s",
                         n_designs, (long long)n_particles, (long long)L.total, scratch_name, (long long)scratch_bytes,
                         hint);
    if (reinterpret_cast<uintptr_t>(sc) % 256) return set_error(CCT_ERR_ARG, "tracking scratch must be 256-byte aligned");
    // the scratch keeps a previous call's contents: clear the control words, rewrite the tables
    CCT_TRY_CUDA(cudaMemsetAsync(sc, 0, 256, st));
    CCT_TRY_CUDA(cudaMemcpyAsync(sc + 256, tables, 8 * (3 * n_designs + 1), cudaMemcpyHostToDevice, st));

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
    P.unit_off = reinterpret_cast<const int64_t *>(sc + 256);
    P.chunks = P.unit_off + n_designs + 1;
    P.chunk_tiles = P.chunks + n_designs;
    P.precision = precision;
    P.barrier_blocks = (unsigned)(grid + g_test_phantom_blocks);
    P.wait_ns = (unsigned long long)g_wait_ms * 1000000ull;
    void *args[] = {&P};
    CCT_TRY_CUDA(cudaLaunchCooperativeKernel((const void *)track_kernel, dim3(grid), dim3(kTrackBlock), args, 0, st));

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

}  // namespace cctgpu

extern "C" int cct_test_set_barrier_fault(int phantom_blocks, int wait_ms) {
    // Test hook: count `phantom_blocks` CTAs that never arrive, and shorten the wait limit,
    // so that a test can make every barrier wait run out and check CCT_ERR_TIMEOUT.
    cctgpu::g_test_phantom_blocks = phantom_blocks < 0 ? 0 : phantom_blocks;
    cctgpu::g_wait_ms = wait_ms > 0 ? wait_ms : 60000;
    return CCT_OK;
}

// ============================================================================
// Tracking without device allocation.
//
// Some callers cannot allocate device memory once they are running: a treatment-planning
// or optimisation host that reserves its GPU memory at start-up and forbids cudaMalloc on
// its hot path (an allocation there can fail mid-run or stall the device), or a plain C
// caller that owns only the buffers it was handed.  cct_track_static_scratch gives them
// the tracking kernel with its scratch in a fixed, file-scope device array instead of a
// caller-provided buffer.  The array is created when the library is loaded, on every GPU
// the process uses, and stays allocated until the process exits; its size bounds the
// problem (see cctgpu.h).  All calls share it, so calls whose kernels overlap on the GPU
// race on it; each call rewrites every word it reads before the kernel starts.
// ============================================================================
namespace cctgpu {

constexpr int64_t kStaticScratchBytes = 32LL << 20;   // 32 MiB
constexpr int kStaticMaxDesigns = 64;
constexpr int kStaticMaxDevices = 64;

static __device__ __align__(256) unsigned char g_track_static_scratch[kStaticScratchBytes];
static void *g_static_scratch_addr[kStaticMaxDevices];
static std::mutex g_static_scratch_mutex;

// Device address of the static scratch on the current device.  The first call on a
// device looks the symbol up (cudaGetSymbolAddress) with that device current.
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

extern "C" int64_t cct_track_static_scratch_bytes(void) { return cctgpu::kStaticScratchBytes; }

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
    if (precision == 0 && (!d_kls || !d_p0s)) return set_error(CCT_ERR_ARG, "FP64 tracking needs segments");
    if (precision == 1 && (!d_packed || reinterpret_cast<uintptr_t>(d_packed) % 256))
        return set_error(CCT_ERR_ARG, "FP32c tracking needs a 256-byte aligned packed buffer");
    return launch_track_static(d_kls, d_p0s, d_seg_off, d_packed, d_qs, d_qs_off, n_designs, d_particles,
                               n_particles, distance, footstep, precision, static_cast<cudaStream_t>(stream));
}
