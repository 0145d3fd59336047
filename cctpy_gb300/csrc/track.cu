// Batched RK4 proton tracking through CCT beamlines: one cooperative persistent launch.
//
// Reference semantics (cctpy): ParticleRunner.run_only particles.py:562-596, RK4
// BaseUtils.runge_kutta4 base_utils.py:264-311, callback Y' = [v, (e/rm) v x B(p)]
// particles.py:515-537, beamline field beamline.py:46-53.
//
// Work decomposition.  Particles of every design are cut into groups of 32 (one per lane);
// each design's segments are cut into tiles of 128 and the tiles into chunks.  A unit is
// (design, group, chunk).  Every RK4 stage runs two phases separated by grid barriers:
//   A. each CTA takes units (u = blockIdx.x, += gridDim.x); its 8 warps split the unit's
//      tiles; lane j accumulates the field of the chunk at particle j's stage position;
//      the CTA reduces its warps in fixed order and stores one partial per unit;
//   C. each thread takes particles, sums the chunk partials of its particle in fixed order,
//      adds the analytic QS fields and advances the RK4 bookkeeping.
// Barriers are sense-counting on a global word, with a wall-clock limit after which the
// kernel records CCT_ERR_TIMEOUT and returns; no wait is unbounded.
#include <cstdlib>
#include <vector>

#include "cctgpu_internal.cuh"
#include "qs.cuh"
#include "tile.cuh"

namespace cctgpu {

constexpr int kTrackBlock = 256;
constexpr int kTrackWarps = kTrackBlock / 32;
constexpr int kStateD = 24;        // doubles of RK4 state per particle
constexpr int kMaxChunks = 64;     // chunks per (design, group)
constexpr int kCtrlWords = 64;     // uint32 control words at the start of the scratch

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
    int groups;                    // particle groups per design
    int64_t n_p;
    double *particles;
    double distance, footstep;
    double *state, *partial;
    unsigned *ctrl;
    const int64_t *unit_off;       // [n_designs+1] first unit of each design
    const int64_t *chunks;         // [n_designs] chunks per group
    const int64_t *chunk_tiles;    // [n_designs] tiles per chunk
    int precision;
    unsigned barrier_blocks;       // CTAs expected at each barrier
    unsigned long long wait_ns;    // barrier wait limit
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier with a wall-clock limit; every thread of the CTA returns the same
// verdict (false = some CTA timed out, stop).
__device__ bool grid_barrier(const TrackParams &P) {
    __shared__ int verdict;
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
                    atomicCAS(reinterpret_cast<int *>(P.ctrl + CW_ERR), 0, (int)CCT_ERR_TIMEOUT);
                    break;
                }
                __nanosleep(128);
            }
        }
        __threadfence();
        verdict = (*err == CCT_ERR_TIMEOUT) ? 0 : 1;
    }
    __syncthreads();
    return verdict != 0;
}

// cross product with the reference's component formula (point.py:402-410), unfused
__device__ __forceinline__ void cross_rn(double ax, double ay, double az, double bx, double by, double bz,
                                         double &cx, double &cy, double &cz) {
    cx = __dadd_rn(__dmul_rn(ay, bz), -__dmul_rn(az, by));
    cy = __dadd_rn(-__dmul_rn(ax, bz), __dmul_rn(az, bx));
    cz = __dadd_rn(__dmul_rn(ax, by), -__dmul_rn(ay, bx));
}

// Phase A for one unit: partial field of the chunk at the 32 stage positions of the group.
__device__ void unit_field(const TrackParams &P, int64_t u, double (*red)[32][3]) {
    // locate the design: last d with unit_off[d] <= u
    int lo = 0, hi = P.n_designs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (P.unit_off[mid] <= u) lo = mid; else hi = mid - 1;
    }
    const int d = lo;
    const int64_t cd = P.chunks[d];
    const int64_t local = u - P.unit_off[d];
    const int64_t g = local / cd, c = local % cd;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t j = g * 32 + lane;
    if (j >= P.n_p) j = P.n_p - 1;
    const double *Ys = P.state + ((int64_t)d * P.n_p + j) * kStateD + ST_YS;
    double px[1] = {Ys[0]}, py[1] = {Ys[1]}, pz[1] = {Ys[2]};
    double bx[1] = {0.0}, by[1] = {0.0}, bz[1] = {0.0};

    const int64_t s_beg = P.seg_off[d], s_end = P.seg_off[d + 1];
    const int64_t nt = (s_end - s_beg + kTile - 1) / kTile;
    const int64_t ct = P.chunk_tiles[d];
    const int64_t t_beg = c * ct, t_end = min(nt, (c + 1) * ct);
    if (P.precision == 1) {
        const unsigned char *tiles = P.tiles + P.tile_off[d] * (int64_t)kTileBytes;
        float ph[1][3], pl[1][3];
        split_df(px[0], ph[0][0], pl[0][0]);
        split_df(py[0], ph[0][1], pl[0][1]);
        split_df(pz[0], ph[0][2], pl[0][2]);
        F32cAcc<1> acc;
        acc.zero();
        for (int64_t t = t_beg + warp; t < t_end; t += kTrackWarps)
            tile_f32c<1>(tiles + t * (int64_t)kTileBytes, ph, pl, acc);
        bx[0] = acc.total(0, 0);
        by[0] = acc.total(0, 1);
        bz[0] = acc.total(0, 2);
    } else {
        for (int64_t t = t_beg + warp; t < t_end; t += kTrackWarps) {
            const int64_t a = s_beg + t * kTile, b = min(s_end, a + kTile);
            double tx = 0.0, ty = 0.0, tz = 0.0;
            for (int64_t s = a; s < b; ++s) {
                const double kx = __ldg(P.kls + 3 * s), ky = __ldg(P.kls + 3 * s + 1), kz = __ldg(P.kls + 3 * s + 2);
                const double rx = px[0] - __ldg(P.p0s + 3 * s), ry = py[0] - __ldg(P.p0s + 3 * s + 1),
                             rz = pz[0] - __ldg(P.p0s + 3 * s + 2);
                const double inv = rsqrt(rx * rx + ry * ry + rz * rz);
                const double inv3 = inv * inv * inv;
                tx += (ky * rz - kz * ry) * inv3;
                ty += (kz * rx - kx * rz) * inv3;
                tz += (kx * ry - ky * rx) * inv3;
            }
            bx[0] += tx;
            by[0] += ty;
            bz[0] += tz;
        }
    }
    red[warp][lane][0] = bx[0];
    red[warp][lane][1] = by[0];
    red[warp][lane][2] = bz[0];
    __syncthreads();
    if (warp == 0) {
        double sx = 0.0, sy = 0.0, sz = 0.0;
        for (int w = 0; w < kTrackWarps; ++w) {
            sx += red[w][lane][0];
            sy += red[w][lane][1];
            sz += red[w][lane][2];
        }
        double *out = P.partial + (u * 32 + lane) * 3;
        out[0] = sx;
        out[1] = sy;
        out[2] = sz;
    }
    __syncthreads();
}

// Phase C for one particle at RK4 stage `stage` (0..3) of step `step`.
__device__ void particle_update(const TrackParams &P, int64_t pi, int step, int stage) {
    double *S = P.state + pi * kStateD;
    if ((double)step >= S[ST_NSTEPS]) return;
    const int d = (int)(pi / P.n_p);
    const int64_t j = pi % P.n_p;
    const int64_t g = j / 32, lane = j % 32;
    const int64_t cd = P.chunks[d];
    const int64_t u0 = P.unit_off[d] + g * cd;
    double B[3] = {0.0, 0.0, 0.0};
    for (int64_t c = 0; c < cd; ++c) {
        const double *p = P.partial + ((u0 + c) * 32 + lane) * 3;
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
    __shared__ double red[kTrackWarps][32][3];
    const int64_t total = (int64_t)P.n_designs * P.n_p;
    const int64_t tstride = (int64_t)gridDim.x * blockDim.x;

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
        bool ok = isfinite(steps) && steps >= 1.0 && steps < 1.0e9;
        S[ST_NSTEPS] = ok ? steps : 0.0;
        S[ST_DT] = ok ? t_end / steps : 0.0;
        if (!ok) atomicExch(P.ctrl + CW_NONFINITE, 1u);
        else atomicMax(P.ctrl + CW_MAXSTEPS, (unsigned)steps);
    }
    if (!grid_barrier(P)) return;
    const int max_steps = (int)*(volatile unsigned *)(P.ctrl + CW_MAXSTEPS);
    const int64_t n_units = P.unit_off[P.n_designs];

    for (int step = 0; step < max_steps; ++step) {
        for (int stage = 0; stage < 4; ++stage) {
            for (int64_t u = blockIdx.x; u < n_units; u += gridDim.x) unit_field(P, u, red);
            if (!grid_barrier(P)) return;
            for (int64_t pi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pi < total; pi += tstride)
                particle_update(P, pi, step, stage);
            if (!grid_barrier(P)) return;
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

TrackScratchLayout track_scratch_layout(int n_designs, int64_t n_particles, int64_t n_units) {
    TrackScratchLayout L;
    auto up = [](int64_t b) { return (b + 255) / 256 * 256; };
    const int64_t tables = up(8 * (int64_t)(3 * n_designs + 1));
    L.ctrl_off = 0;
    L.state_off = 256 + tables;
    L.partial_off = L.state_off + up(8 * kStateD * (int64_t)n_designs * n_particles);
    L.total = L.partial_off + up(8 * 96 * n_units);
    return L;
}

int64_t track_max_units(int n_designs, int64_t n_particles) {
    const int64_t groups = (n_particles + 31) / 32;
    return (int64_t)n_designs * groups * kMaxChunks;
}

int launch_track(const double *kls, const double *p0s, const int64_t *seg_off, const void *packed, const double *qs,
                 const int64_t *qs_off, int n_designs, double *particles, int64_t n_particles, double distance,
                 double footstep, int precision, void *scratch, int64_t scratch_bytes, cudaStream_t st) {
    if (n_designs <= 0 || n_particles <= 0) return CCT_OK;
    std::vector<int64_t> hoff(n_designs + 1);
    CCT_TRY_CUDA(cudaMemcpyAsync(hoff.data(), seg_off, 8 * (n_designs + 1), cudaMemcpyDeviceToHost, st));
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

    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    CCT_TRY_CUDA(cudaGetDevice(&dev));
    CCT_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CCT_TRY_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return set_error(CCT_ERR_UNSUPPORTED, "device %d has no cooperative launch", dev);
    CCT_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, track_kernel, kTrackBlock, 0));
    if (per_sm < 1) return set_error(CCT_ERR_UNSUPPORTED, "tracking kernel does not fit on an SM");
    const int grid = sms * per_sm;

    // units: chunks per (design, group) so that there are ~8 units per CTA
    const int64_t groups = (n_particles + 31) / 32;
    std::vector<int64_t> tables(3 * n_designs + 1);
    int64_t *unit_off = tables.data(), *chunks = unit_off + n_designs + 1, *chunk_tiles = chunks + n_designs;
    const int64_t target = 8LL * grid;
    int64_t want = (target + (int64_t)n_designs * groups - 1) / ((int64_t)n_designs * groups);
    if (want < 1) want = 1;
    if (want > kMaxChunks) want = kMaxChunks;
    unit_off[0] = 0;
    for (int d = 0; d < n_designs; ++d) {
        const int64_t nt = (hoff[d + 1] - hoff[d] + kTile - 1) / kTile;
        int64_t ct = nt > 0 ? (nt + want - 1) / want : 1;
        int64_t cd = nt > 0 ? (nt + ct - 1) / ct : 1;
        chunks[d] = cd;
        chunk_tiles[d] = ct;
        unit_off[d + 1] = unit_off[d] + groups * cd;
    }
    const int64_t n_units = unit_off[n_designs];
    const TrackScratchLayout L = track_scratch_layout(n_designs, n_particles, n_units);
    if (scratch_bytes < L.total)
        return set_error(CCT_ERR_ARG, "tracking scratch holds %lld bytes, needs %lld", (long long)scratch_bytes,
                         (long long)L.total);
    if (reinterpret_cast<uintptr_t>(scratch) % 256)
        return set_error(CCT_ERR_ARG, "tracking scratch must be 256-byte aligned");
    unsigned char *sc = static_cast<unsigned char *>(scratch);
    CCT_TRY_CUDA(cudaMemsetAsync(sc, 0, 256, st));
    CCT_TRY_CUDA(cudaMemcpyAsync(sc + 256, tables.data(), 8 * tables.size(), cudaMemcpyHostToDevice, st));

    TrackParams P;
    P.kls = kls;
    P.p0s = p0s;
    P.seg_off = seg_off;
    P.tiles = tiles;
    P.tile_off = tile_off;
    P.qs = qs;
    P.qs_off = qs_off;
    P.n_designs = n_designs;
    P.groups = (int)groups;
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
        return set_error(CCT_ERR_TIMEOUT, "a tracking grid barrier waited longer than %lld ms", g_wait_ms);
    if (ctrl[CW_NONFINITE])
        return set_error(CCT_ERR_NONFINITE, "a particle state or step count was not finite");
    return CCT_OK;
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
#include <mutex>

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
    int rc = static_scratch_address(&scratch);
    if (rc != CCT_OK) return rc;

    int64_t hoff[kStaticMaxDesigns + 1];
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

    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    CCT_TRY_CUDA(cudaGetDevice(&dev));
    CCT_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CCT_TRY_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return set_error(CCT_ERR_UNSUPPORTED, "device %d has no cooperative launch", dev);
    CCT_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, track_kernel, kTrackBlock, 0));
    if (per_sm < 1) return set_error(CCT_ERR_UNSUPPORTED, "tracking kernel does not fit on an SM");
    const int grid = sms * per_sm;

    const int64_t groups = (n_particles + 31) / 32;
    int64_t tables[3 * kStaticMaxDesigns + 1];
    int64_t *unit_off = tables, *chunks = unit_off + n_designs + 1, *chunk_tiles = chunks + n_designs;
    const int64_t target = 8LL * grid;
    int64_t want = (target + (int64_t)n_designs * groups - 1) / ((int64_t)n_designs * groups);
    if (want < 1) want = 1;
    if (want > kMaxChunks) want = kMaxChunks;
    unit_off[0] = 0;
    for (int d = 0; d < n_designs; ++d) {
        const int64_t nt = (hoff[d + 1] - hoff[d] + kTile - 1) / kTile;
        const int64_t ct = nt > 0 ? (nt + want - 1) / want : 1;
        const int64_t cd = nt > 0 ? (nt + ct - 1) / ct : 1;
        chunks[d] = cd;
        chunk_tiles[d] = ct;
        unit_off[d + 1] = unit_off[d] + groups * cd;
    }
    const TrackScratchLayout L = track_scratch_layout(n_designs, n_particles, unit_off[n_designs]);
    if (L.total > kStaticScratchBytes)
        return set_error(CCT_ERR_ARG,
                         "%d designs x %lld particles need %lld bytes of tracking scratch; the static scratch holds "
                         "%lld (use cct_track with a caller buffer)", n_designs, (long long)n_particles,
                         (long long)L.total, (long long)kStaticScratchBytes);
    unsigned char *sc = static_cast<unsigned char *>(scratch);
    // the array keeps the previous call's contents: clear the control words, rewrite the tables
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
    P.groups = (int)groups;
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
        return set_error(CCT_ERR_TIMEOUT, "a tracking grid barrier waited longer than %lld ms", g_wait_ms);
    if (ctrl[CW_NONFINITE])
        return set_error(CCT_ERR_NONFINITE, "a particle state or step count was not finite");
    return CCT_OK;
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
