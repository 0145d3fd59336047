// Device-side CCT segment generation and the segment-to-parameter Jacobian contraction.
//
// A CCT layer is the curve xi -> (xi, phi(xi)) in bipolar-toroidal coordinates
// (cctpy final_code/packages/cct.py:87-164, :166-188, :213-224):
//   phi(xi) = k xi + b + sum_i cot(tilt_i) / ((i+1) sinh eta) sin((i+1) xi)   (tilt_i != 90 deg)
//   w(xi)   = a / (cosh eta - cos xi) * (sinh eta cos phi, sinh eta sin phi, sin xi)
//   a = sqrt(R^2 - r^2), eta = ln((R + a)/(R - a)) / 2,
// cut at W*n + 1 equally spaced xi into W*n straight elements, moved to the global frame
// (g = O + x XI + y YI + z ZI, local_coordinate_system.py:84-93) and turned into
// kl = 1e-7 I (g[i+1] - g[i]), p0 = (g[i+1] + g[i]) / 2 (cct.py:434-457).
//
// segments_build_kernel writes kl/p0 of every layer of a design set in HBM (the host
// never builds or copies segment arrays).  param_grad_kernel maps a segment gradient
// dJ/d(kl_i, p0_i) to dJ/d(tilt angles, current, big_r) of each layer by forward-mode
// differentiation of the same formulas, one CTA per layer with a fixed-order reduction.
#include <algorithm>
#include <cmath>
#include <utility>
#include <vector>

#include "cctgpu_internal.cuh"

namespace cctgpu {

constexpr int kLayerDoubles = CCT_LAYER_DOUBLES;
constexpr int kMaxTilts = CCT_LAYER_MAX_TILTS;
constexpr int kLayerParams = CCT_LAYER_PARAMS;

// Layer record fields (doubles).
enum : int {
    LR_ORIGIN = 0, LR_XI = 3, LR_YI = 6, LR_ZI = 9, LR_BIG_R = 12, LR_SMALL_R = 13, LR_CURRENT = 14,
    LR_KSI0 = 15, LR_PHI0 = 16, LR_KSI1 = 17, LR_PHI1 = 18, LR_WINDINGS = 19, LR_PER_WINDING = 20,
    LR_NTILT = 21, LR_TILT = 22, LR_FIRST = 30
};

struct LayerGeom {
    double A[12];              // origin, XI, YI, ZI
    double k, b, a, sh, ch, x1, d, c_kl;
    double coef[kMaxTilts];    // cot(tilt_i) / ((i+1) sinh eta); 0 where the tilt is 90 deg
    double coef_all[kMaxTilts];  // the same without the 90-degree skip (derivative in big_r)
    double dcoef[kMaxTilts];   // d coef_i / d tilt_i, per degree
    double da, dsh, dch;       // d a, d sinh eta, d cosh eta per unit big_r
    int64_t n;
    int n_tilt;
};

__device__ __forceinline__ bool is_90(double t) {
    return t == 90.0 || fabs(t - 90.0) <= 1e-6 || ((t + 90.0 != 0.0) && 2.0 * fabs((t - 90.0) / (t + 90.0)) <= 1e-6);
}

__device__ void layer_geom(const double *__restrict__ rec, LayerGeom &G) {
    for (int i = 0; i < 12; ++i) G.A[i] = rec[i];
    const double R = rec[LR_BIG_R], r = rec[LR_SMALL_R];
    const double x1 = rec[LR_KSI0], y1 = rec[LR_PHI0], x2 = rec[LR_KSI1], y2 = rec[LR_PHI1];
    G.k = __ddiv_rn(__dsub_rn(y2, y1), __dsub_rn(x2, x1));
    G.b = __dadd_rn(-__dmul_rn(G.k, x1), y1);
    G.a = __dsqrt_rn(__dsub_rn(__dmul_rn(R, R), __dmul_rn(r, r)));
    const double eta = __dmul_rn(0.5, log(__ddiv_rn(__dadd_rn(R, G.a), __dsub_rn(R, G.a))));
    G.sh = sinh(eta);
    G.ch = cosh(eta);
    G.n = (int64_t)rec[LR_WINDINGS] * (int64_t)rec[LR_PER_WINDING];
    G.x1 = x1;
    G.d = __dmul_rn(__dsub_rn(x2, x1), __ddiv_rn(1.0, (double)G.n));
    G.c_kl = __dmul_rn(1e-7, rec[LR_CURRENT]);
    G.n_tilt = (int)rec[LR_NTILT];
    const double deg = 3.141592653589793 / 180.0;
    for (int i = 0; i < kMaxTilts; ++i) {
        G.coef[i] = G.coef_all[i] = G.dcoef[i] = 0.0;
        if (i >= G.n_tilt) continue;
        const double t = rec[LR_TILT + i];
        const double rad = __dmul_rn(__ddiv_rn(t, 180.0), 3.141592653589793);
        const double c = __ddiv_rn(__ddiv_rn(1.0, tan(rad)), __dmul_rn((double)(i + 1), G.sh));
        G.coef_all[i] = c;
        if (!is_90(t)) G.coef[i] = c;
        const double s = sin(rad);
        G.dcoef[i] = -deg / (s * s) / ((double)(i + 1) * G.sh);
    }
    // cosh eta = R / r and sinh eta = a / r, so d eta / dR = 1 / a
    G.da = R / G.a;
    G.dsh = G.ch / G.a;
    G.dch = G.sh / G.a;
}

// Winding point j of a layer in its local frame, in the reference's operation order.
__device__ __forceinline__ void layer_point(const LayerGeom &G, int64_t j, double &ksi, double &phi, double &x,
                                            double &y, double &z) {
    ksi = __dadd_rn(G.x1, __dmul_rn(G.d, (double)j));
    phi = __dadd_rn(__dmul_rn(G.k, ksi), G.b);
    for (int i = 0; i < G.n_tilt; ++i)
        if (G.coef[i] != 0.0) phi = __dadd_rn(phi, __dmul_rn(G.coef[i], sin(__dmul_rn((double)(i + 1), ksi))));
    const double temp = __ddiv_rn(G.a, __dsub_rn(G.ch, cos(ksi)));
    const double ts = __dmul_rn(temp, G.sh);
    double s, c;
    sincos(phi, &s, &c);
    x = __dmul_rn(ts, c);
    y = __dmul_rn(ts, s);
    z = __dmul_rn(temp, sin(ksi));
}

__device__ __forceinline__ void to_global(const LayerGeom &G, double x, double y, double z, double g[3]) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
        g[c] = __dadd_rn(G.A[c], __dadd_rn(__dadd_rn(__dmul_rn(G.A[3 + c], x), __dmul_rn(G.A[6 + c], y)),
                                           __dmul_rn(G.A[9 + c], z)));
}

// First segment of layer l in the segment arrays (record field 30).
__device__ __forceinline__ int64_t layer_first_segment(const double *__restrict__ layers, int l) {
    return (int64_t)layers[(int64_t)l * kLayerDoubles + LR_FIRST];
}

constexpr int kBuildBlock = 256;

__global__ void __launch_bounds__(kBuildBlock) segments_build_kernel(const double *__restrict__ layers,
                                                                     double *__restrict__ kls,
                                                                     double *__restrict__ p0s) {
    __shared__ LayerGeom G;
    __shared__ int64_t first;
    const int l = blockIdx.y;
    if (threadIdx.x == 0) {
        layer_geom(layers + (int64_t)l * kLayerDoubles, G);
        first = layer_first_segment(layers, l);
    }
    __syncthreads();
    for (int64_t s = (int64_t)blockIdx.x * kBuildBlock + threadIdx.x; s < G.n; s += (int64_t)gridDim.x * kBuildBlock) {
        double ksi, phi, x, y, z, g0[3], g1[3];
        layer_point(G, s, ksi, phi, x, y, z);
        to_global(G, x, y, z, g0);
        layer_point(G, s + 1, ksi, phi, x, y, z);
        to_global(G, x, y, z, g1);
        const int64_t o = 3 * (first + s);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            kls[o + c] = __dmul_rn(G.c_kl, __dsub_rn(g1[c], g0[c]));
            p0s[o + c] = __dmul_rn(0.5, __dadd_rn(g1[c], g0[c]));
        }
    }
}

constexpr int kGradBlock = 512;

// One CTA per layer.  The segment gradient (gk_i = dJ/dkl_i, gp_i = dJ/dp0_i, global) is
// regrouped per winding point j:  sum_i gk_i.dkl_i + gp_i.dp0_i = sum_j dg_j . V_j with
// V_j = c (gk_{j-1} - gk_j) + (gp_{j-1} + gp_j)/2 (zero beyond the ends), and dg_j = R^T dw_j,
// so each point contributes (R V_j) . dw_j/dtheta.  dJ/dI = sum_j w_j . R (1e-7 (gk_{j-1} - gk_j)).
__global__ void __launch_bounds__(kGradBlock) param_grad_kernel(const double *__restrict__ layers,
                                                                const double *__restrict__ seg_grad,
                                                                double *__restrict__ out) {
    __shared__ LayerGeom G;
    __shared__ int64_t first;
    __shared__ double red[kLayerParams][kGradBlock / 32];
    const int l = blockIdx.x;
    if (threadIdx.x == 0) {
        layer_geom(layers + (int64_t)l * kLayerDoubles, G);
        first = layer_first_segment(layers, l);
    }
    __syncthreads();
    double acc[kLayerParams];
#pragma unroll
    for (int p = 0; p < kLayerParams; ++p) acc[p] = 0.0;
    const double *R = G.A + 3;   // rows XI, YI, ZI
    for (int64_t j = threadIdx.x; j <= G.n; j += kGradBlock) {
        double gkp[3] = {0, 0, 0}, gkc[3] = {0, 0, 0}, gpp[3] = {0, 0, 0}, gpc[3] = {0, 0, 0};
        if (j > 0) {
            const double *q = seg_grad + 6 * (first + j - 1);
            for (int c = 0; c < 3; ++c) { gkp[c] = q[c]; gpp[c] = q[3 + c]; }
        }
        if (j < G.n) {
            const double *q = seg_grad + 6 * (first + j);
            for (int c = 0; c < 3; ++c) { gkc[c] = q[c]; gpc[c] = q[3 + c]; }
        }
        double V[3], Wc[3], U[3], Uc[3];
        for (int c = 0; c < 3; ++c) {
            V[c] = G.c_kl * (gkp[c] - gkc[c]) + 0.5 * (gpp[c] + gpc[c]);
            Wc[c] = 1e-7 * (gkp[c] - gkc[c]);
        }
        for (int m = 0; m < 3; ++m) {
            U[m] = R[3 * m] * V[0] + R[3 * m + 1] * V[1] + R[3 * m + 2] * V[2];
            Uc[m] = R[3 * m] * Wc[0] + R[3 * m + 1] * Wc[1] + R[3 * m + 2] * Wc[2];
        }
        double ksi, phi, x, y, z;
        layer_point(G, j, ksi, phi, x, y, z);
        double sp, cp, sk, ck;
        sincos(phi, &sp, &cp);
        sincos(ksi, &sk, &ck);
        const double den = G.ch - ck;
        const double temp = G.a / den;
        const double ts = temp * G.sh;
        // d w / d phi = ts (-sin phi, cos phi, 0)
        const double gphi = ts * (U[1] * cp - U[0] * sp);
        double tilt_sum = 0.0;
        for (int i = 0; i < G.n_tilt; ++i) {
            const double si = sin((double)(i + 1) * ksi);
            acc[i] += gphi * G.dcoef[i] * si;
            tilt_sum += G.coef_all[i] * si;
        }
        acc[kMaxTilts] += Uc[0] * x + Uc[1] * y + Uc[2] * z;
        // big_r: a, sinh eta, cosh eta move; phi moves through 1/sinh eta
        const double dphi = -(G.dsh / G.sh) * tilt_sum;
        const double dtemp = (G.da - temp * G.dch) / den;
        const double dts = dtemp * G.sh + temp * G.dsh;
        const double dx = dts * cp - ts * sp * dphi;
        const double dy = dts * sp + ts * cp * dphi;
        const double dz = dtemp * sk;
        acc[kMaxTilts + 1] += U[0] * dx + U[1] * dy + U[2] * dz;
    }
    // fixed-order reduction: warp shuffle tree, then warp 0 over the warps
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int p = 0; p < kLayerParams; ++p) {
        double v = acc[p];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[p][warp] = v;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int p = 0; p < kLayerParams; ++p) {
            double v = lane < kGradBlock / 32 ? red[p][lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) out[(int64_t)l * kLayerParams + p] = v;
        }
    }
}

// ------------------------------------------------------------------ host side
static int check_layers(const double *h, int n_layers, int64_t *total) {
    std::vector<std::pair<int64_t, int64_t>> ranges;
    ranges.reserve(n_layers);
    for (int l = 0; l < n_layers; ++l) {
        const double *r = h + (int64_t)l * kLayerDoubles;
        for (int i = 0; i < kLayerDoubles; ++i)
            if (!std::isfinite(r[i])) return set_error(CCT_ERR_ARG, "layer %d: field %d is not finite", l, i);
        const double W = r[LR_WINDINGS], n = r[LR_PER_WINDING], nt = r[LR_NTILT], f = r[LR_FIRST];
        if (W < 1 || W != std::floor(W) || n < 1 || n != std::floor(n) || W * n > 1e10)
            return set_error(CCT_ERR_ARG, "layer %d: winding number %g and segments per winding %g must be "
                                          "positive integers", l, W, n);
        if (nt < 0 || nt > kMaxTilts || nt != std::floor(nt))
            return set_error(CCT_ERR_ARG, "layer %d: %g tilt angles (0..%d supported)", l, nt, kMaxTilts);
        if (r[LR_BIG_R] < 0 || r[LR_SMALL_R] < 0 || r[LR_SMALL_R] >= r[LR_BIG_R])
            return set_error(CCT_ERR_ARG, "layer %d: need 0 <= small_r (%g) < big_r (%g)", l, r[LR_SMALL_R],
                             r[LR_BIG_R]);
        if (r[LR_KSI1] == r[LR_KSI0]) return set_error(CCT_ERR_ARG, "layer %d: xi start equals xi end", l);
        if (f < 0 || f != std::floor(f) || f > 9e15)
            return set_error(CCT_ERR_ARG, "layer %d: first segment %g must be a non-negative integer", l, f);
        ranges.emplace_back((int64_t)f, (int64_t)f + (int64_t)W * (int64_t)n);
    }
    std::vector<std::pair<int64_t, int64_t>> sorted = ranges;
    std::sort(sorted.begin(), sorted.end());
    for (size_t i = 1; i < sorted.size(); ++i)
        if (sorted[i].first < sorted[i - 1].second)
            return set_error(CCT_ERR_ARG, "layers overlap in the segment arrays (segments %lld..%lld and %lld..%lld)",
                             (long long)sorted[i - 1].first, (long long)sorted[i - 1].second,
                             (long long)sorted[i].first, (long long)sorted[i].second);
    *total = sorted.empty() ? 0 : sorted.back().second;
    return CCT_OK;
}

static int fetch_and_check(const double *d_layers, int n_layers, int64_t n_seg, cudaStream_t st) {
    if (n_layers <= 0 || n_layers > 65535) return set_error(CCT_ERR_ARG, "n_layers = %d (1..65535)", n_layers);
    if (!d_layers) return set_error(CCT_ERR_ARG, "null layer records");
    std::vector<double> h((size_t)n_layers * kLayerDoubles);
    CCT_TRY_CUDA(cudaMemcpyAsync(h.data(), d_layers, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    CCT_TRY_CUDA(cudaStreamSynchronize(st));
    int64_t total = 0;
    int rc = check_layers(h.data(), n_layers, &total);
    if (rc != CCT_OK) return rc;
    if (total > n_seg)
        return set_error(CCT_ERR_ARG, "the layers reach segment %lld, the buffers hold %lld segments",
                         (long long)total, (long long)n_seg);
    return CCT_OK;
}

}  // namespace cctgpu

using namespace cctgpu;

extern "C" {

int64_t cct_layer_segments(const double *h_layers, int32_t n_layers) {
    clear_error();
    if (n_layers <= 0 || !h_layers) {
        set_error(CCT_ERR_ARG, "need at least one layer record");
        return -1;
    }
    int64_t total = 0;
    if (check_layers(h_layers, n_layers, &total) != CCT_OK) return -1;
    return total;
}

int cct_segments_build(const double *d_layers, int32_t n_layers, double *d_kls, double *d_p0s, int64_t n_seg,
                       void *stream) {
    clear_error();
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (!d_kls || !d_p0s) return set_error(CCT_ERR_ARG, "null segment arrays");
    int rc = fetch_and_check(d_layers, n_layers, n_seg, st);
    if (rc != CCT_OK) return rc;
    int sms = 0, dev = 0;
    CCT_TRY_CUDA(cudaGetDevice(&dev));
    CCT_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t per_layer = (std::max<int64_t>(n_seg / n_layers, 1) + kBuildBlock - 1) / kBuildBlock;
    const int gx = (int)std::max<int64_t>(1, std::min<int64_t>(per_layer, 8 * (int64_t)sms));
    segments_build_kernel<<<dim3(gx, n_layers), kBuildBlock, 0, st>>>(d_layers, d_kls, d_p0s);
    CCT_TRY_CUDA(cudaGetLastError());
    CCT_TRY_CUDA(cudaStreamSynchronize(st));
    return CCT_OK;
}

int cct_segments_param_grad(const double *d_layers, int32_t n_layers, const double *d_seg_grad, int64_t n_seg,
                            double *d_param_grad, void *stream) {
    clear_error();
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (!d_seg_grad || !d_param_grad) return set_error(CCT_ERR_ARG, "null gradient arrays");
    int rc = fetch_and_check(d_layers, n_layers, n_seg, st);
    if (rc != CCT_OK) return rc;
    param_grad_kernel<<<n_layers, kGradBlock, 0, st>>>(d_layers, d_seg_grad, d_param_grad);
    CCT_TRY_CUDA(cudaGetLastError());
    CCT_TRY_CUDA(cudaStreamSynchronize(st));
    return CCT_OK;
}

}  // extern "C"
