// Discrete adjoint of the batched RK4 track: gradient of a beam objective at the exit with
// respect to every current element (kl, p0) of every design.
//
// Objective per design (over its N particles, positions p_i after the track, exit frame
// (o, XI, YI) of the ideal particle): J = (1/N) sum_i (x_i^2 + y_i^2), x_i = XI.(p_i - o),
// y_i = YI.(p_i - o) -- the RMS spot size squared plus the centroid squared in both planes.
//
// The adjoint is that of the exact discrete map the forward kernel applies (the reference's
// RK4, base_utils.py:264-311, with f(Y) = [v, kq v x B(p)], particles.py:515-537), so it
// agrees with finite differences of the forward up to their truncation error.  For one step,
// with lambda' the adjoint after the step and J_f(Y)^T l = ((dB/dp)^T a, l_p + kq B x l_v),
// a = kq (l_v x v):
//   lk4 = h/6 l', mu4 = J_f(Y4)^T lk4;  lk3 = h/3 l' + h mu4,   mu3 = J_f(Y3)^T lk3;
//   lk2 = h/3 l' + h/2 mu3, mu2 = ...;  lk1 = h/6 l' + h/2 mu2, mu1 = ...;
//   l = l' + mu1 + mu2 + mu3 + mu4,
// and every stage adds a . dB/d(segment) to the segment gradient:
//   dJ/dkl_i += (r x a) / |r|^3,  dJ/dp0_i += -grad_p(a . B_i) = -(c/|r|^3 - 3 (c.r) r/|r|^5),
//   r = p - p0_i, c = a x kl_i.
//
// Schedule (host, one stream, no synchronisation but the step count): initialise the state,
// run the forward in segments of K steps keeping a checkpoint of the state before each,
// evaluate J and dJ/dY at the exit, then for each checkpoint segment in reverse: restore,
// re-run its K steps recording every stage's (Y, B), sweep its steps backwards
// (adjoint_kernel: phase A' sums (dB/dp)^T a over segment chunks per particle block, as the
// forward's phase A sums B; phase C' advances the lambdas), and accumulate the segment
// gradient from the recorded (p, a) pairs (seg_adjoint_kernel, one thread per segment).
// The sweeps run in the forward's precision: FP64, or FP32c (packed FP32 pair terms on the
// tile-local frames, Kahan-compensated, as the forward field sums).
#include <algorithm>
#include <vector>

#include "track_common.cuh"

namespace cctgpu {

constexpr int kAdjD = 24;   // per particle: LP (6), LY (6), LK (6), a (3), pad
enum { AD_LP = 0, AD_LY = 6, AD_LK = 12, AD_A = 18 };

struct AdjParams {
    TrackParams T;              // the forward's parameters (plan, partials, state, record)
    double *adj;                // per particle adjoint state
    const double *exit_frame;   // per design: o (3), XI (3), YI (3)
    double *J;                  // per design objective
    int step_begin, step_end;   // the checkpoint segment swept here (in reverse)
};

// ---------------------------------------------------------------- objective and dJ/dY
// One CTA per design: J_d and the adjoint of the final state (LY).
__global__ void __launch_bounds__(256) objective_kernel(AdjParams A) {
    const TrackParams &P = A.T;
    const int d = blockIdx.x;
    const double *f = A.exit_frame + 9 * d;
    __shared__ double red[256];
    double s = 0.0;
    const double inv_n = 1.0 / (double)P.n_p;
    for (int64_t j = threadIdx.x; j < P.n_p; j += blockDim.x) {
        const int64_t pi = (int64_t)d * P.n_p + j;
        const double *Y = P.state + pi * kStateD + ST_Y0;
        const double dx = Y[0] - f[0], dy = Y[1] - f[1], dz = Y[2] - f[2];
        const double x = f[3] * dx + f[4] * dy + f[5] * dz;
        const double y = f[6] * dx + f[7] * dy + f[8] * dz;
        s += x * x + y * y;
        double *ad = A.adj + pi * kAdjD;
        for (int c = 0; c < 3; ++c) {
            ad[AD_LY + c] = 2.0 * inv_n * (x * f[3 + c] + y * f[6 + c]);
            ad[AD_LY + 3 + c] = 0.0;
        }
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {   // fixed-order tree: deterministic
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) A.J[d] = red[0] * inv_n;
}

// ---------------------------------------------------------------- reverse sweep
__device__ __forceinline__ double *rec_at(const TrackParams &P, int step, int stage, int64_t pi) {
    return P.record + (((int64_t)(step - P.step_begin) * 4 + stage) * ((int64_t)P.n_designs * P.n_p) + pi) * kRec;
}

// Phase A': for the 32 particles of a unit's block, sum over the chunk's segments
// grad_p (a . B_i) = c/|r|^3 - 3 (c.r) r / |r|^5, c = a x kl_i (FP64; G = 32, warps split tiles).
__device__ void unit_grad_f64(const AdjParams &A, int64_t u, int step, int stage, TrackSmem &sm) {
    const TrackParams &P = A.T;
    const UnitRef U = locate_unit(P, u);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t j = U.b * 32 + lane;
    if (j >= P.n_p) j = P.n_p - 1;
    const int64_t pi = (int64_t)U.d * P.n_p + j;
    const double *rec = rec_at(P, step, stage, pi);
    const double px = rec[0], py = rec[1], pz = rec[2];
    const double *a = A.adj + pi * kAdjD + AD_A;
    const double ax = a[0], ay = a[1], az = a[2];
    double gx = 0.0, gy = 0.0, gz = 0.0;
    const int64_t s_beg = P.seg_off[U.d], s_end = P.seg_off[U.d + 1];
    for (int64_t t = U.t_beg + warp; t < U.t_end; t += kTrackWarps) {
        const int64_t b0 = s_beg + t * kTile, e = min(s_end, b0 + kTile);
        double tx = 0.0, ty = 0.0, tz = 0.0;
        for (int64_t s = b0; s < e; ++s) {
            const double kx = __ldg(P.kls + 3 * s), ky = __ldg(P.kls + 3 * s + 1), kz = __ldg(P.kls + 3 * s + 2);
            const double rx = px - __ldg(P.p0s + 3 * s), ry = py - __ldg(P.p0s + 3 * s + 1),
                         rz = pz - __ldg(P.p0s + 3 * s + 2);
            const double inv = rsqrt(rx * rx + ry * ry + rz * rz);
            const double inv3 = inv * inv * inv, inv5 = inv3 * inv * inv;
            const double cx = ay * kz - az * ky, cy = az * kx - ax * kz, cz = ax * ky - ay * kx;
            const double q = 3.0 * (cx * rx + cy * ry + cz * rz) * inv5;
            tx += cx * inv3 - q * rx;
            ty += cy * inv3 - q * ry;
            tz += cz * inv3 - q * rz;
        }
        gx += tx;
        gy += ty;
        gz += tz;
    }
    double *red = sm.red + (warp * 32 + lane) * 3;
    red[0] = gx;
    red[1] = gy;
    red[2] = gz;
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

// grad_p (a . B_qs) of one QS magnet (magnets.py:637-668: bx = g y + s x y,
// by = g x + s (x^2 - y^2) / 2 in the local frame, zero outside); added to g.
__device__ __forceinline__ void qs_grad_add(const double *q, const double *p, const double *a, double *g) {
    if (q[12] < 0.0) return;   // straight dipole / uniform field: piecewise constant, no gradient
    const double dx = p[0] - q[0], dy = p[1] - q[1], dz = p[2] - q[2];
    const double x = q[3] * dx + q[4] * dy + q[5] * dz;
    const double y = q[6] * dx + q[7] * dy + q[8] * dz;
    const double z = q[9] * dx + q[10] * dy + q[11] * dz;
    if (z < 0.0 || z > q[12]) return;
    const double ap = q[15];
    if (fabs(x) > ap || fabs(y) > ap || sqrt(x * x + y * y) > ap) return;
    const double gr = q[13], s = q[14];
    const double al = a[0] * q[3] + a[1] * q[4] + a[2] * q[5];   // a . XI
    const double be = a[0] * q[6] + a[1] * q[7] + a[2] * q[8];   // a . YI
    const double dfx = al * s * y + be * (gr + s * x);            // d(a.B)/dx
    const double dfy = al * (gr + s * x) - be * s * y;            // d(a.B)/dy
    for (int c = 0; c < 3; ++c) g[c] += q[3 + c] * dfx + q[6 + c] * dfy;
}

// a = kq (l_v x v) for the stage `stage` (0-based) of `step`; written to the particle's
// adjoint state and to the record (for the segment gradient).
__device__ __forceinline__ void set_weight(const AdjParams &A, int64_t pi, int step, int stage, const double *lk) {
    const TrackParams &P = A.T;
    double *rec = rec_at(P, step, stage, pi);
    const double kq = P.state[pi * kStateD + ST_KQ];
    const double *v = rec + 3;
    double *a = A.adj + pi * kAdjD + AD_A;
    a[0] = kq * (lk[4] * v[2] - lk[5] * v[1]);
    a[1] = kq * (lk[5] * v[0] - lk[3] * v[2]);
    a[2] = kq * (lk[3] * v[1] - lk[4] * v[0]);
    rec[9] = a[0];
    rec[10] = a[1];
    rec[11] = a[2];
}

__device__ __forceinline__ void clear_weight(const AdjParams &A, int64_t pi, int step, int stage) {
    double *rec = rec_at(A.T, step, stage, pi);
    double *a = A.adj + pi * kAdjD + AD_A;
    a[0] = a[1] = a[2] = rec[9] = rec[10] = rec[11] = 0.0;
}

// Start of a step in reverse: l' = LY, lk4 = h/6 l', weight of stage 4.
__device__ void begin_step(const AdjParams &A, int64_t pi, int step) {
    const TrackParams &P = A.T;
    const double *S = P.state + pi * kStateD;
    if ((double)step >= S[ST_NSTEPS]) {
        for (int s = 0; s < 4; ++s) clear_weight(A, pi, step, s);
        return;
    }
    double *ad = A.adj + pi * kAdjD;
    const double h = S[ST_DT];
    for (int c = 0; c < 6; ++c) {
        ad[AD_LP + c] = ad[AD_LY + c];
        ad[AD_LK + c] = h / 6 * ad[AD_LP + c];
    }
    set_weight(A, pi, step, 3, ad + AD_LK);
}

// Phase C' of stage `stage` (3..0): mu = J_f^T lk, LY += mu, next lk and weight; g = the
// CCT part of grad_p (a . B) (sum of the chunk partials).
__device__ void end_stage(const AdjParams &A, int64_t pi, int step, int stage, const double g[3]) {
    const TrackParams &P = A.T;
    const double *S = P.state + pi * kStateD;
    if ((double)step >= S[ST_NSTEPS]) return;
    const int d = (int)(pi / P.n_p);
    double mu[6] = {g[0], g[1], g[2], 0.0, 0.0, 0.0};
    const double *rec = rec_at(P, step, stage, pi);
    double *ad = A.adj + pi * kAdjD;
    for (int64_t q = P.qs_off[d]; q < P.qs_off[d + 1]; ++q) qs_grad_add(P.qs + kQsRecord * q, rec, ad + AD_A, mu);
    const double kq = S[ST_KQ];
    const double *B = rec + 6, *lk = ad + AD_LK;
    mu[3] = lk[0] + kq * (B[1] * lk[5] - B[2] * lk[4]);
    mu[4] = lk[1] + kq * (B[2] * lk[3] - B[0] * lk[5]);
    mu[5] = lk[2] + kq * (B[0] * lk[4] - B[1] * lk[3]);
    for (int c = 0; c < 6; ++c) ad[AD_LY + c] += mu[c];
    if (stage > 0) {
        const double h = S[ST_DT];
        const double cl = stage == 1 ? h / 6 : h / 3;    // coefficient of l' in lk(stage-1)
        const double cm = stage == 3 ? h : h / 2;        // coefficient of mu in lk(stage-1)
        double nk[6];
        for (int c = 0; c < 6; ++c) nk[c] = cl * ad[AD_LP + c] + cm * mu[c];
        for (int c = 0; c < 6; ++c) ad[AD_LK + c] = nk[c];
        set_weight(A, pi, step, stage - 1, nk);
    }
}

__global__ void __launch_bounds__(kTrackBlock, kTrackMinBlocks) adjoint_kernel(AdjParams A) {
    __shared__ __align__(128) TrackSmem sm;
    const TrackParams &P = A.T;
    const int64_t total = (int64_t)P.n_designs * P.n_p;
    const int64_t tstride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n_units = P.unit_off[P.n_designs];
    const int64_t first = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t gwarp = first >> 5, nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    if (A.step_end <= A.step_begin) return;
    if (threadIdx.x == 0) ring_init(sm);
    for (int64_t pi = first; pi < total; pi += tstride) begin_step(A, pi, A.step_end - 1);
    clear_unit_counters(P);
    if (!grid_barrier(P, sm)) return;
    uint32_t kt = 0;   // tiles consumed through the TMA ring by this CTA (FP32c)
    int phase = 0;
    for (int step = A.step_end - 1; step >= A.step_begin; --step) {
        for (int stage = 3; stage >= 0; --stage, ++phase) {
            const PointSrc src{rec_at(P, step, stage, 0), kRec, A.adj + AD_A, kAdjD};
            if (P.precision == 0) {
                for (int64_t u = first_unit(); u < n_units; u = next_unit(P, sm, phase))
                    unit_grad_f64(A, u, step, stage, sm);
            } else if (P.ppt == 2) {
                units_f32c<2, true>(P, src, sm, kt, phase, n_units);
            } else {
                units_f32c<1, true>(P, src, sm, kt, phase, n_units);
            }
            if (!grid_barrier(P, sm)) return;   // a TMA timeout is recorded in CW_ERR and ends here
            reset_next_unit(P, phase);
            for (int64_t pi = gwarp; pi < total; pi += nwarps) {   // a warp per particle
                double g[3] = {0.0, 0.0, 0.0};
                if (particle_active(P, pi, step)) warp_sum_partials(P, pi, g);
                if ((threadIdx.x & 31) == 0) {
                    end_stage(A, pi, step, stage, g);
                    if (stage == 0 && step > A.step_begin) begin_step(A, pi, step - 1);
                }
            }
            if (!grid_barrier(P, sm)) return;
        }
    }
}

// ---------------------------------------------------------------- segment gradient
// One thread per segment of design blockIdx.y; the design's recorded (p, a) pairs of the
// segment of steps stream through shared memory.  Adds into grad[seg][6] (dJ/dkl, dJ/dp0).
constexpr int kSegBlock = 256;

__global__ void __launch_bounds__(kSegBlock) seg_adjoint_kernel(TrackParams P, int n_steps, double *grad) {
    __shared__ double pts[kSegBlock][6];
    const int d = blockIdx.y;
    const int64_t s_beg = P.seg_off[d], s_end = P.seg_off[d + 1];
    const int64_t s = s_beg + (int64_t)blockIdx.x * kSegBlock + threadIdx.x;
    if (s_beg + (int64_t)blockIdx.x * kSegBlock >= s_end) return;   // whole CTA beyond this design
    const bool mine = s < s_end;
    double kx = 0, ky = 0, kz = 0, qx = 0, qy = 0, qz = 0;
    if (mine) {
        kx = P.kls[3 * s];
        ky = P.kls[3 * s + 1];
        kz = P.kls[3 * s + 2];
        qx = P.p0s[3 * s];
        qy = P.p0s[3 * s + 1];
        qz = P.p0s[3 * s + 2];
    }
    double gk[3] = {0, 0, 0}, gp[3] = {0, 0, 0};
    const int64_t total = (int64_t)P.n_designs * P.n_p;
    const int64_t n_pts = (int64_t)n_steps * 4 * P.n_p;   // this design's (step, stage, particle)
    for (int64_t base = 0; base < n_pts; base += kSegBlock) {
        __syncthreads();
        const int64_t e = base + threadIdx.x;
        if (e < n_pts) {
            const int64_t ss = e / P.n_p, j = e % P.n_p;
            const double *r = P.record + (ss * total + (int64_t)d * P.n_p + j) * kRec;
            pts[threadIdx.x][0] = r[0];
            pts[threadIdx.x][1] = r[1];
            pts[threadIdx.x][2] = r[2];
            pts[threadIdx.x][3] = r[9];
            pts[threadIdx.x][4] = r[10];
            pts[threadIdx.x][5] = r[11];
        } else {
            for (int c = 0; c < 6; ++c) pts[threadIdx.x][c] = 0.0;
        }
        __syncthreads();
        const int cnt = (int)min((int64_t)kSegBlock, n_pts - base);
        double tk[3] = {0, 0, 0}, tp[3] = {0, 0, 0};
        for (int i = 0; i < cnt; ++i) {
            const double ax = pts[i][3], ay = pts[i][4], az = pts[i][5];
            if (ax == 0.0 && ay == 0.0 && az == 0.0) continue;      // inactive stage (uniform)
            const double rx = pts[i][0] - qx, ry = pts[i][1] - qy, rz = pts[i][2] - qz;
            const double inv = rsqrt(rx * rx + ry * ry + rz * rz);
            const double inv3 = inv * inv * inv, inv5 = inv3 * inv * inv;
            tk[0] += (ry * az - rz * ay) * inv3;
            tk[1] += (rz * ax - rx * az) * inv3;
            tk[2] += (rx * ay - ry * ax) * inv3;
            const double cx = ay * kz - az * ky, cy = az * kx - ax * kz, cz = ax * ky - ay * kx;
            const double q = 3.0 * (cx * rx + cy * ry + cz * rz) * inv5;
            tp[0] -= cx * inv3 - q * rx;
            tp[1] -= cy * inv3 - q * ry;
            tp[2] -= cz * inv3 - q * rz;
        }
        for (int c = 0; c < 3; ++c) {
            gk[c] += tk[c];
            gp[c] += tp[c];
        }
    }
    if (mine) {
        for (int c = 0; c < 3; ++c) {
            grad[6 * s + c] += gk[c];
            grad[6 * s + 3 + c] += gp[c];
        }
    }
}

// FP32c segment gradient.  seg_prep_kernel converts every recorded stage point once: its
// position as a double-float pair (hi, lo) and its weight a in FP32, three float4 per point
// {hx, hy, hz, ax}, {lx, ly, lz, ay}, {az, 0, 0, 0}.  seg_adjoint_f32c_kernel then runs one
// warp per packed tile, four segments per thread (two packed pairs, whose chains interleave
// and share each staged point's loads); the design's
// points are staged in shared memory 128 at a time in the tile's local frame (point minus
// tile origin in double-float FP32, no FP64 work per tile) together with n = q x a, and the
// sums are taken in moment form: with r = q - p,
//   dJ/dkl  = sum (r x a) |r|^-3            = V - p x W,
//   grad_p  = sum (a x kl) |r|^-3 + t r     = W x kl + U - p T,
//   V = sum n |r|^-3, W = sum a |r|^-3, t = -3 (kl.n + a.(p x kl)) |r|^-5, U = sum t q, T = sum t,
// 27 FMA-pipe operations per pair instead of 35.  Each chunk's result is Kahan-added per
// segment.
constexpr int kSegPts = 128;
constexpr int kSegThreads = 32;     // one warp per tile, two packed segment pairs per thread
constexpr int kSegUnroll = 4;
constexpr int kSegMinBlocks = 8;   // CTAs per SM the register budget allows for (184 registers used)

__global__ void seg_prep_kernel(const double *__restrict__ record, int64_t n_rec, float4 *__restrict__ out) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n_rec; e += (int64_t)gridDim.x * blockDim.x) {
        const double *r = record + e * kRec;
        float h[3], l[3];
        for (int c = 0; c < 3; ++c) split_df(r[c], h[c], l[c]);
        out[3 * e] = make_float4(h[0], h[1], h[2], (float)r[9]);
        out[3 * e + 1] = make_float4(l[0], l[1], l[2], (float)r[10]);
        out[3 * e + 2] = make_float4((float)r[11], 0.0f, 0.0f, 0.0f);
    }
}

__global__ void __launch_bounds__(kSegThreads, kSegMinBlocks) seg_adjoint_f32c_kernel(TrackParams P, int n_steps,
                                                                          const float4 *__restrict__ pts_df,
                                                                          double *grad) {
    // per point, as packed pairs (v, v): a x3, q x3, n x3 with n = q x a, pad (80 B: five 16-byte loads)
    __shared__ __align__(16) f2 pts[kSegPts][10];
    constexpr int R = kTile / 2 / kSegThreads;      // packed segment pairs per thread
    const int64_t t = blockIdx.x;
    int lo = 0, hi = P.n_designs - 1;               // design of tile t: last d with tile_off[d] <= t
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (P.tile_off[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const int d = lo;
    const unsigned char *tile = P.tiles + t * (int64_t)kTileBytes;
    const TileHeader *h = reinterpret_cast<const TileHeader *>(tile);
    const f2 *v = reinterpret_cast<const f2 *>(tile + kTileHeaderBytes);
    constexpr int Q2 = kTile / 2;                   // packed pairs per component array
    const int tid = threadIdx.x;
    const int cnt = h->count;
    const int64_t s0 = P.seg_off[d] + (t - P.tile_off[d]) * kTile;
    // pair r of this thread: packed index tid + r * kSegThreads (segments 2 * that and + 1)
    f2 kx[R], ky[R], kz[R], px[R], py[R], pz[R], hx[R], hy[R], hz[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int e = tid + r * kSegThreads;
        kx[r] = v[0 * Q2 + e];
        ky[r] = v[1 * Q2 + e];
        kz[r] = v[2 * Q2 + e];
        px[r] = v[6 * Q2 + e];
        py[r] = v[7 * Q2 + e];
        pz[r] = v[8 * Q2 + e];
        // h = p x kl
        hx[r] = f2_fma(py[r], kz[r], f2_mul(f2_neg(pz[r]), ky[r]));
        hy[r] = f2_fma(pz[r], kx[r], f2_mul(f2_neg(px[r]), kz[r]));
        hz[r] = f2_fma(px[r], ky[r], f2_mul(f2_neg(py[r]), kx[r]));
    }
    float S[2 * R][6], C[2 * R][6];
#pragma unroll
    for (int m = 0; m < 2 * R; ++m)
#pragma unroll
        for (int c = 0; c < 6; ++c) S[m][c] = C[m][c] = 0.0f;
    const f2 m3 = f2_pack(-3.0f, -3.0f);
    const int64_t total = (int64_t)P.n_designs * P.n_p;
    const int64_t n_pts = (int64_t)n_steps * 4 * P.n_p;
    for (int64_t base = 0; base < n_pts; base += kSegPts) {
        __syncthreads();
        for (int k = tid; k < kSegPts; k += kSegThreads) {
            const int64_t e = base + k;
            float q[3] = {0.f, 0.f, 0.f}, a[3] = {0.f, 0.f, 0.f};
            if (e < n_pts) {
                const float4 *rp = pts_df + 3 * ((e / P.n_p) * total + (int64_t)d * P.n_p + e % P.n_p);
                const float4 u = rp[0], w = rp[1], z = rp[2];
                q[0] = __fadd_rn(__fsub_rn(u.x, h->o_hi[0]), __fsub_rn(w.x, h->o_lo[0]));
                q[1] = __fadd_rn(__fsub_rn(u.y, h->o_hi[1]), __fsub_rn(w.y, h->o_lo[1]));
                q[2] = __fadd_rn(__fsub_rn(u.z, h->o_hi[2]), __fsub_rn(w.z, h->o_lo[2]));
                a[0] = u.w;
                a[1] = w.w;
                a[2] = z.x;
            }
            if (a[0] == 0.0f && a[1] == 0.0f && a[2] == 0.0f) {
                // no weight (an inactive stage, or past the last point): park the point far
                // away (opposite the padding segments), so that its terms are exactly zero
                // and the pair loop needs no branch
                q[0] = q[1] = q[2] = -kPadOffset;
            }
            const float n[3] = {__fmaf_rn(q[1], a[2], -q[2] * a[1]), __fmaf_rn(q[2], a[0], -q[0] * a[2]),
                                __fmaf_rn(q[0], a[1], -q[1] * a[0])};
            for (int c = 0; c < 3; ++c) {
                pts[k][c] = f2_pack(a[c], a[c]);
                pts[k][3 + c] = f2_pack(q[c], q[c]);
                pts[k][6 + c] = f2_pack(n[c], n[c]);
            }
            pts[k][9] = 0ull;
        }
        __syncthreads();
        f2 V[R][3], W[R][3], U[R][3], T[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            T[r] = 0ull;
#pragma unroll
            for (int c = 0; c < 3; ++c) V[r][c] = W[r][c] = U[r][c] = 0ull;
        }
        const int np = (int)min((int64_t)kSegPts, n_pts - base);
#pragma unroll kSegUnroll
        for (int i = 0; i < np; ++i) {
            const ulonglong2 *row = reinterpret_cast<const ulonglong2 *>(pts[i]);
            const ulonglong2 v0 = row[0], v1 = row[1], v2 = row[2], v3 = row[3], v4 = row[4];
            const f2 Ax = v0.x, Ay = v0.y, Az = v1.x;
            const f2 Qx = v1.y, Qy = v2.x, Qz = v2.y;
            const f2 Nx = v3.x, Ny = v3.y, Nz = v4.x;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const f2 rx = f2_sub(Qx, px[r]), ry = f2_sub(Qy, py[r]), rz = f2_sub(Qz, pz[r]);
                const f2 r2 = f2_fma(rx, rx, f2_fma(ry, ry, f2_mul(rz, rz)));
                float l0, l1;
                f2_unpack(r2, l0, l1);
                const f2 inv = f2_pack(rsqrt_mufu(l0), rsqrt_mufu(l1));
                const f2 inv2 = f2_mul(inv, inv);
                const f2 inv3 = f2_mul(inv2, inv);
                const f2 m3inv5 = f2_mul(f2_mul(inv3, inv2), m3);
                V[r][0] = f2_fma(Nx, inv3, V[r][0]);
                V[r][1] = f2_fma(Ny, inv3, V[r][1]);
                V[r][2] = f2_fma(Nz, inv3, V[r][2]);
                W[r][0] = f2_fma(Ax, inv3, W[r][0]);
                W[r][1] = f2_fma(Ay, inv3, W[r][1]);
                W[r][2] = f2_fma(Az, inv3, W[r][2]);
                // kl.n + a.h = (a x kl).r
                const f2 cr = f2_fma(kx[r], Nx, f2_fma(ky[r], Ny, f2_fma(kz[r], Nz,
                              f2_fma(hx[r], Ax, f2_fma(hy[r], Ay, f2_mul(hz[r], Az))))));
                const f2 tt = f2_mul(cr, m3inv5);
                U[r][0] = f2_fma(tt, Qx, U[r][0]);
                U[r][1] = f2_fma(tt, Qy, U[r][1]);
                U[r][2] = f2_fma(tt, Qz, U[r][2]);
                T[r] = f2_add(T[r], tt);
            }
        }
        // per segment: dJ/dkl = V - p x W, grad_p = W x kl + U - p T
#pragma unroll
        for (int r = 0; r < R; ++r) {
            float v_[3][2], w_[3][2], u_[3][2], t_[2], p_[3][2], k_[3][2];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                f2_unpack(V[r][c], v_[c][0], v_[c][1]);
                f2_unpack(W[r][c], w_[c][0], w_[c][1]);
                f2_unpack(U[r][c], u_[c][0], u_[c][1]);
            }
            f2_unpack(T[r], t_[0], t_[1]);
            f2_unpack(px[r], p_[0][0], p_[0][1]);
            f2_unpack(py[r], p_[1][0], p_[1][1]);
            f2_unpack(pz[r], p_[2][0], p_[2][1]);
            f2_unpack(kx[r], k_[0][0], k_[0][1]);
            f2_unpack(ky[r], k_[1][0], k_[1][1]);
            f2_unpack(kz[r], k_[2][0], k_[2][1]);
#pragma unroll
            for (int m = 0; m < 2; ++m) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
                    const float dk = v_[c][m] - __fmaf_rn(p_[c1][m], w_[c2][m], -p_[c2][m] * w_[c1][m]);
                    const float gp = __fmaf_rn(w_[c1][m], k_[c2][m], -w_[c2][m] * k_[c1][m]) +
                                     __fmaf_rn(-p_[c][m], t_[m], u_[c][m]);
                    kahan_add(S[2 * r + m][c], C[2 * r + m][c], dk);
                    kahan_add(S[2 * r + m][3 + c], C[2 * r + m][3 + c], gp);
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            const int j = 2 * (tid + r * kSegThreads) + m;
            if (j >= cnt) continue;
            double *g = grad + 6 * (s0 + j);
            for (int c = 0; c < 3; ++c) g[c] += (double)S[2 * r + m][c] - (double)C[2 * r + m][c];
            for (int c = 0; c < 3; ++c)   // dJ/dp0 = -grad_p
                g[3 + c] -= (double)S[2 * r + m][3 + c] - (double)C[2 * r + m][3 + c];
        }
}

// ---------------------------------------------------------------- host side
struct AdjLayout {
    int64_t track_total, ckpt_off, record_off, adj_off, pts_off, total;
};

static AdjLayout adj_layout(const TrackScratchLayout &L, int n_designs, int64_t n_p, int n_ckpt, int K) {
    auto up = [](int64_t b) { return (b + 255) / 256 * 256; };
    const int64_t tot = (int64_t)n_designs * n_p;
    AdjLayout A;
    A.track_total = L.total;
    A.ckpt_off = up(L.total);
    A.record_off = A.ckpt_off + up(8 * kStateD * tot * (int64_t)n_ckpt);
    A.adj_off = A.record_off + up(8 * (int64_t)kRec * 4 * K * tot);
    A.pts_off = A.adj_off + up(8 * kAdjD * tot);                   // FP32c: converted stage points
    A.total = A.pts_off + up(48 * (int64_t)4 * K * tot);
    return A;
}

static int adjoint_grid(int *grid_out) {
    int dev = 0, sms = 0, per_sm = 0;
    CCT_TRY_CUDA(cudaGetDevice(&dev));
    CCT_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CCT_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, adjoint_kernel, kTrackBlock, 0));
    if (per_sm < 1) return set_error(CCT_ERR_UNSUPPORTED, "adjoint kernel does not fit on an SM");
    *grid_out = sms * per_sm;
    return CCT_OK;
}

static int64_t adjoint_scratch_bound(int n_designs, int64_t n_p, int max_steps, int K) {
    const int64_t track = track_scratch_bound(n_designs, n_p, false);   // the adjoint's own particle block
    TrackScratchLayout L{0, 0, 0, 0, track};
    const int n_ckpt = (max_steps + K - 1) / K;
    return adj_layout(L, n_designs, n_p, n_ckpt, K).total;
}

static int launch_adjoint(const double *kls, const double *p0s, const int64_t *seg_off, const void *packed,
                          const double *qs, const int64_t *qs_off, int n_designs, double *particles, int64_t n_p,
                          double distance, double footstep, int precision, const double *exit_frame, double *J,
                          double *seg_grad, int K, void *scratch, int64_t scratch_bytes, cudaStream_t st) {
    std::vector<int64_t> hoff(n_designs + 1), tables(3 * n_designs + 1);
    CCT_TRY_CUDA(cudaMemcpyAsync(hoff.data(), seg_off, 8 * (n_designs + 1), cudaMemcpyDeviceToHost, st));
    CCT_TRY_CUDA(cudaStreamSynchronize(st));
    for (int d = 0; d < n_designs; ++d)
        if (hoff[d + 1] < hoff[d]) return set_error(CCT_ERR_ARG, "segment offsets decrease at design %d", d);
    const unsigned char *tiles = nullptr;
    const int64_t *tile_off = nullptr;
    int64_t tiles_total = 0;
    for (int d = 0; d < n_designs; ++d) tiles_total += (hoff[d + 1] - hoff[d] + kTile - 1) / kTile;
    if (precision == 1) {
        int64_t ph[3];
        CCT_TRY_CUDA(cudaMemcpyAsync(ph, packed, sizeof ph, cudaMemcpyDeviceToHost, st));
        CCT_TRY_CUDA(cudaStreamSynchronize(st));
        if (ph[0] != kPackedMagic || ph[1] != n_designs || ph[2] != tiles_total)
            return set_error(CCT_ERR_ARG, "packed segments do not match the %d designs' segment offsets", n_designs);
        tile_off = reinterpret_cast<const int64_t *>(static_cast<const unsigned char *>(packed) + kPackedHeaderBytes);
        tiles = static_cast<const unsigned char *>(packed) + kPackedHeaderBytes + packed_index_bytes(n_designs);
    }
    int grid = 0, agrid = 0;
    int rc = track_grid(&grid);
    if (rc == CCT_OK) rc = adjoint_grid(&agrid);
    if (rc != CCT_OK) return rc;
    const int G = group_size(precision, n_p);
    int64_t *unit_off = tables.data(), *chunks = unit_off + n_designs + 1, *chunk_tiles = chunks + n_designs;
    const int64_t n_units = plan_units(hoff.data(), n_designs, n_p, G, grid, units_bound(n_designs, n_p, G, grid),
                                       unit_off, chunks, chunk_tiles);
    const TrackScratchLayout L = track_scratch_layout(n_designs, n_p, n_units, G);
    if (reinterpret_cast<uintptr_t>(scratch) % 256) return set_error(CCT_ERR_ARG, "adjoint scratch must be 256-byte aligned");
    if (scratch_bytes < L.total) return set_error(CCT_ERR_ARG, "adjoint scratch too small (%lld bytes)", (long long)scratch_bytes);
    unsigned char *sc = static_cast<unsigned char *>(scratch);
    const int64_t tot = (int64_t)n_designs * n_p;

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
    P.record = nullptr;
    P.tiny = 0;                     // the adjoint's forward keeps the chunk partial sums
    P.tiny_copies = 1;
    P.tiny_acc = nullptr;
    P.tiny_bad = nullptr;
    set_flow(P, sc + L.flow_off);   // the forward launches (the reverse sweep keeps its barriers)

    // 1. state from the records; learn the step count
    CCT_TRY_CUDA(cudaMemsetAsync(sc, 0, kCtrlBytes, st));
    CCT_TRY_CUDA(cudaMemcpyAsync(sc + kCtrlBytes, tables.data(), 8 * tables.size(), cudaMemcpyHostToDevice, st));
    P.init_from_records = 1;
    P.write_back = 0;
    P.step_begin = 0;
    P.step_end = 0;
    CCT_TRY_CUDA(launch_track_kernel(P, grid, st));
    unsigned ctrl[8];
    CCT_TRY_CUDA(cudaMemcpyAsync(ctrl, sc, sizeof ctrl, cudaMemcpyDeviceToHost, st));
    CCT_TRY_CUDA(cudaStreamSynchronize(st));
    if ((int)ctrl[CW_ERR] == CCT_ERR_TIMEOUT) return set_error(CCT_ERR_TIMEOUT, "adjoint: initialisation timed out");
    if (ctrl[CW_NONFINITE]) return set_error(CCT_ERR_NONFINITE, "adjoint: a particle step count was not finite");
    const int steps = (int)ctrl[CW_MAXSTEPS];
    if (K < 1) K = 64;
    const int n_ckpt = (steps + K - 1) / K;
    const AdjLayout AL = adj_layout(L, n_designs, n_p, n_ckpt, K);
    if (scratch_bytes < AL.total)
        return set_error(CCT_ERR_ARG, "adjoint needs %lld bytes of scratch for %d steps (K = %d), %lld given",
                         (long long)AL.total, steps, K, (long long)scratch_bytes);
    double *ckpt = reinterpret_cast<double *>(sc + AL.ckpt_off);
    double *record = reinterpret_cast<double *>(sc + AL.record_off);
    const size_t state_bytes = 8 * (size_t)kStateD * tot;

    // 2. forward in checkpoint segments; the last one records its stages right away, so the
    //    reverse sweep starts without recomputing it (with one segment: no recompute at all)
    P.init_from_records = 0;
    for (int c = 0; c < n_ckpt; ++c) {
        CCT_TRY_CUDA(cudaMemcpyAsync(ckpt + (int64_t)c * kStateD * tot, P.state, state_bytes, cudaMemcpyDeviceToDevice,
                                     st));
        P.step_begin = c * K;
        P.step_end = std::min(steps, (c + 1) * K);
        P.write_back = c == n_ckpt - 1;
        P.record = c == n_ckpt - 1 ? record : nullptr;
        CCT_TRY_CUDA(launch_track_kernel(P, grid, st));
    }
    P.record = nullptr;

    // 3. objective and the adjoint of the final state
    AdjParams A;
    A.T = P;
    A.adj = reinterpret_cast<double *>(sc + AL.adj_off);
    A.exit_frame = exit_frame;
    A.J = J;
    objective_kernel<<<n_designs, 256, 0, st>>>(A);
    CCT_TRY_CUDA(cudaGetLastError());
    CCT_TRY_CUDA(cudaMemsetAsync(seg_grad, 0, 48 * (size_t)hoff[n_designs], st));

    // 4. reverse over the checkpoint segments
    int64_t max_seg = 0;
    for (int d = 0; d < n_designs; ++d) max_seg = std::max(max_seg, hoff[d + 1] - hoff[d]);
    for (int c = n_ckpt - 1; c >= 0; --c) {
        P.step_begin = c * K;
        P.step_end = std::min(steps, (c + 1) * K);
        P.write_back = 0;
        P.record = record;
        if (c < n_ckpt - 1) {   // recompute this segment from its checkpoint, recording its stages
            CCT_TRY_CUDA(cudaMemcpyAsync(P.state, ckpt + (int64_t)c * kStateD * tot, state_bytes,
                                         cudaMemcpyDeviceToDevice, st));
            CCT_TRY_CUDA(launch_track_kernel(P, grid, st));
        }
        A.T = P;
        A.T.barrier_blocks = (unsigned)(agrid + g_test_phantom_blocks);
        // The reverse sweep stays on grid barriers: measured on the dataflow schedule it was
        // no faster with 3 CTAs of 4 warps per SM, and slower with 8 CTAs of 2 warps (the warp
        // scheduler favoured some CTAs of an SM, the others' units ran up to 20x longer, and
        // their blocks' late stages held back the next stage).
        A.T.use_flow = 0;
        A.step_begin = P.step_begin;
        A.step_end = P.step_end;
        void *args[] = {&A};
        CCT_TRY_CUDA(cudaLaunchCooperativeKernel((const void *)adjoint_kernel, dim3(agrid), dim3(kTrackBlock), args,
                                                 0, st));
        if (precision == 1 && tiles_total > 0) {
            const int64_t n_rec = (int64_t)(P.step_end - P.step_begin) * 4 * tot;
            float4 *pts_df = reinterpret_cast<float4 *>(sc + AL.pts_off);
            const int64_t prep_blocks = std::min<int64_t>((n_rec + 255) / 256, 65536);
            seg_prep_kernel<<<(unsigned)std::max<int64_t>(prep_blocks, 1), 256, 0, st>>>(record, n_rec, pts_df);
            CCT_TRY_CUDA(cudaGetLastError());
            seg_adjoint_f32c_kernel<<<(unsigned)tiles_total, kSegThreads, 0, st>>>(P, P.step_end - P.step_begin,
                                                                                   pts_df, seg_grad);
            CCT_TRY_CUDA(cudaGetLastError());
        } else if (precision == 0 && max_seg > 0) {
            const dim3 sg((unsigned)((max_seg + kSegBlock - 1) / kSegBlock), (unsigned)n_designs);
            seg_adjoint_kernel<<<sg, kSegBlock, 0, st>>>(P, P.step_end - P.step_begin, seg_grad);
            CCT_TRY_CUDA(cudaGetLastError());
        }
        P.record = nullptr;
    }
    CCT_TRY_CUDA(cudaMemcpyAsync(ctrl, sc, sizeof ctrl, cudaMemcpyDeviceToHost, st));
    CCT_TRY_CUDA(cudaStreamSynchronize(st));
    if ((int)ctrl[CW_ERR] == CCT_ERR_TIMEOUT)
        return set_error(CCT_ERR_TIMEOUT, "adjoint: a grid barrier or tile copy waited longer than its limit");
    if (ctrl[CW_NONFINITE]) return set_error(CCT_ERR_NONFINITE, "adjoint: a particle state was not finite");
    return CCT_OK;
}

}  // namespace cctgpu

extern "C" int64_t cct_adjoint_scratch_bytes(int32_t n_designs, int64_t n_particles, int32_t max_steps,
                                             int32_t checkpoint_steps) {
    using namespace cctgpu;
    clear_error();
    if (n_designs <= 0 || n_particles <= 0 || max_steps <= 0) {
        set_error(CCT_ERR_ARG, "need at least one design, one particle and one step");
        return -1;
    }
    return adjoint_scratch_bound(n_designs, n_particles, max_steps, checkpoint_steps > 0 ? checkpoint_steps : 64);
}

extern "C" int cct_track_adjoint(const double *d_kls, const double *d_p0s, const int64_t *d_seg_off,
                                 const void *d_packed, const double *d_qs, const int64_t *d_qs_off, int32_t n_designs,
                                 double *d_particles, int64_t n_particles, double distance, double footstep,
                                 int32_t precision, const double *d_exit_frame, double *d_J, double *d_seg_grad,
                                 int32_t checkpoint_steps, void *d_scratch, int64_t scratch_bytes, void *stream) {
    using namespace cctgpu;
    clear_error();
    if (n_designs <= 0 || n_particles <= 0) return set_error(CCT_ERR_ARG, "need at least one design and particle");
    if (!(distance > 0.0) || !(footstep > 0.0))
        return set_error(CCT_ERR_ARG, "distance (%g) and footstep (%g) must be positive", distance, footstep);
    if (precision != 0 && precision != 1) return set_error(CCT_ERR_ARG, "precision must be 0 or 1");
    if (!d_kls || !d_p0s || !d_seg_off || !d_qs_off || !d_particles || !d_exit_frame || !d_J || !d_seg_grad ||
        !d_scratch)
        return set_error(CCT_ERR_ARG, "null pointer");
    if (precision == 1 && (!d_packed || reinterpret_cast<uintptr_t>(d_packed) % 256))
        return set_error(CCT_ERR_ARG, "FP32c adjoint needs a 256-byte aligned packed buffer");
    return launch_adjoint(d_kls, d_p0s, d_seg_off, d_packed, d_qs, d_qs_off, n_designs, d_particles, n_particles,
                          distance, footstep, precision, d_exit_frame, d_J, d_seg_grad, checkpoint_steps, d_scratch,
                          scratch_bytes, static_cast<cudaStream_t>(stream));
}
