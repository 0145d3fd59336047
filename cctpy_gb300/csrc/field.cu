// Biot-Savart field of CCT winding segments (+ analytic QS magnets) at field points.
//
//   B(p) = sum_i kl_i x r_i / |r_i|^3,  r_i = p - p0_i,  kl_i = 1e-7 I (w[i+1]-w[i]),
//   p0_i = (w[i+1]+w[i])/2            -- cctpy final_code/packages/cct.py:157-164, :249-285
//
// Two forms:
//  * field_f64_kernel   plain FP64, one thread per field point (x2), segment tiles staged in
//                       shared memory by the CTA, pair sums in moment form about each tile's
//                       first midpoint; the drop-in for CCT.magnetic_field_at.
//  * field_f32c_kernel  FP32 arithmetic on per-tile local offsets: each tile of 128 segments
//                       carries a double-float origin, point-minus-origin is taken in
//                       double-float, the pair terms run as packed FP32x2 (two segments
//                       per instruction; rsqrt on the MUFU pipe) in the moment form
//                       (sums of kl |r|^-3 and (kl x p0) |r|^-3 per 32-segment
//                       sub-block, crossed with the point once per sub-block), summed into
//                       a Kahan-compensated (S, C) pair resolved in FP64 at the end
//                       (tile.cuh).  Tiles are streamed into
//                       shared memory by the TMA bulk-copy engine through a 4-deep
//                       mbarrier ring.
#include <cstdarg>
#include <cstdio>
#include <vector>

#include "cctgpu_internal.cuh"
#include "qs.cuh"
#include "tile.cuh"

namespace cctgpu {

// ===================================================================== FP64
constexpr int kF64Block = 256;
constexpr int kF64Ppt = 2;

__global__ void __launch_bounds__(kF64Block) field_f64_kernel(const double *__restrict__ kls,
                                                              const double *__restrict__ p0s, int64_t n_seg,
                                                              const double *__restrict__ qs, int n_qs,
                                                              const double *__restrict__ pts, int64_t n,
                                                              double *__restrict__ B) {
    // staged per segment, about the tile's first midpoint o: kl, p0 - o and the moment
    // m = kl x (p0 - o); per tile and point the sums A = sum kl |r|^-3 and M = sum m |r|^-3
    // give the tile's field A x (p - o) - M (the moment form: 23 instead of 26 FP64 operations
    // per pair; the cancellation in it costs |p - o| / |r| ulps)
    __shared__ double sk[3][kF64Block];
    __shared__ double sp[3][kF64Block];
    __shared__ double sm[3][kF64Block];
    const int tid = threadIdx.x;
    const int64_t base = (int64_t)blockIdx.x * kF64Block * kF64Ppt;

    double px[kF64Ppt], py[kF64Ppt], pz[kF64Ppt], bx[kF64Ppt], by[kF64Ppt], bz[kF64Ppt];
#pragma unroll
    for (int i = 0; i < kF64Ppt; ++i) {
        int64_t idx = base + tid + (int64_t)i * kF64Block;
        if (idx >= n) idx = n - 1;
        px[i] = pts[3 * idx];
        py[i] = pts[3 * idx + 1];
        pz[i] = pts[3 * idx + 2];
        bx[i] = by[i] = bz[i] = 0.0;
    }

    for (int64_t t0 = 0; t0 < n_seg; t0 += kF64Block) {
        const int64_t s = t0 + tid;
        const double ox = p0s[3 * t0], oy = p0s[3 * t0 + 1], oz = p0s[3 * t0 + 2];
        __syncthreads();
        if (s < n_seg) {
            const double kx = kls[3 * s], ky = kls[3 * s + 1], kz = kls[3 * s + 2];
            const double qx = p0s[3 * s] - ox, qy = p0s[3 * s + 1] - oy, qz = p0s[3 * s + 2] - oz;
            sk[0][tid] = kx;
            sk[1][tid] = ky;
            sk[2][tid] = kz;
            sp[0][tid] = qx;
            sp[1][tid] = qy;
            sp[2][tid] = qz;
            sm[0][tid] = ky * qz - kz * qy;
            sm[1][tid] = kz * qx - kx * qz;
            sm[2][tid] = kx * qy - ky * qx;
        }
        __syncthreads();
        const int cnt = (int)min((int64_t)kF64Block, n_seg - t0);
        double ax[kF64Ppt], ay[kF64Ppt], az[kF64Ppt], mx[kF64Ppt], my[kF64Ppt], mz[kF64Ppt];
        double wx[kF64Ppt], wy[kF64Ppt], wz[kF64Ppt];
#pragma unroll
        for (int i = 0; i < kF64Ppt; ++i) {
            ax[i] = ay[i] = az[i] = mx[i] = my[i] = mz[i] = 0.0;
            wx[i] = px[i] - ox;
            wy[i] = py[i] - oy;
            wz[i] = pz[i] - oz;
        }
#pragma unroll 2
        for (int j = 0; j < cnt; ++j) {
            const double kx = sk[0][j], ky = sk[1][j], kz = sk[2][j];
            const double qx = sp[0][j], qy = sp[1][j], qz = sp[2][j];
            const double nx = sm[0][j], ny = sm[1][j], nz = sm[2][j];
#pragma unroll
            for (int i = 0; i < kF64Ppt; ++i) {
                const double rx = wx[i] - qx, ry = wy[i] - qy, rz = wz[i] - qz;
                const double inv = rsqrt(rx * rx + ry * ry + rz * rz);
                const double inv3 = inv * inv * inv;
                ax[i] += kx * inv3;
                ay[i] += ky * inv3;
                az[i] += kz * inv3;
                mx[i] += nx * inv3;
                my[i] += ny * inv3;
                mz[i] += nz * inv3;
            }
        }
#pragma unroll
        for (int i = 0; i < kF64Ppt; ++i) {   // A x (p - o) - M
            bx[i] += (ay[i] * wz[i] - az[i] * wy[i]) - mx[i];
            by[i] += (az[i] * wx[i] - ax[i] * wz[i]) - my[i];
            bz[i] += (ax[i] * wy[i] - ay[i] * wx[i]) - mz[i];
        }
    }

#pragma unroll
    for (int i = 0; i < kF64Ppt; ++i) {
        const int64_t idx = base + tid + (int64_t)i * kF64Block;
        if (idx >= n) continue;
        for (int q = 0; q < n_qs; ++q) qs_field_add(qs + kQsRecord * q, px[i], py[i], pz[i], bx[i], by[i], bz[i]);
        B[3 * idx] = bx[i];
        B[3 * idx + 1] = by[i];
        B[3 * idx + 2] = bz[i];
    }
}

int launch_field_f64(const double *kls, const double *p0s, int64_t n_seg, const double *qs, int n_qs,
                     const double *pts, int64_t n, double *B, cudaStream_t st) {
    if (n == 0) return CCT_OK;
    const int64_t per = (int64_t)kF64Block * kF64Ppt;
    const int64_t grid = (n + per - 1) / per;
    if (grid > 0x7fffffff) return set_error(CCT_ERR_ARG, "too many field points (%lld)", (long long)n);
    field_f64_kernel<<<(unsigned)grid, kF64Block, 0, st>>>(kls, p0s, n_seg, qs, n_qs, pts, n, B);
    CCT_TRY_CUDA(cudaGetLastError());
    return CCT_OK;
}

// ===================================================================== FP32c pack
// Packs FP64 segments into FP32c tiles (layout in tile.cuh).  The tile origin is the
// centroid of the tile's midpoints rounded to a double-float (hi, lo) pair; offsets are
// taken from that represented origin, so point - origin needs no FP64 in the kernels.  Each
// 32-segment sub-block gets its own FP32 origin (centroid of its offsets), about which the
// moments kl x (p0 - origin - sub-block origin) are formed in FP64 and rounded once.
__global__ void __launch_bounds__(kTile) pack_f32c_kernel(const double *__restrict__ kls,
                                                          const double *__restrict__ p0s,
                                                          unsigned char *__restrict__ packed) {
    const int64_t n_designs = reinterpret_cast<const int64_t *>(packed)[1];
    const int64_t *tile_off = reinterpret_cast<const int64_t *>(packed + kPackedHeaderBytes);
    const int64_t *seg_off = tile_off + (n_designs + 1);
    unsigned char *tiles = packed + kPackedHeaderBytes + packed_index_bytes((int)n_designs);
    const int64_t t = blockIdx.x;
    // design holding tile t: last d with tile_off[d] <= t
    int64_t lo = 0, hi = n_designs - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) / 2;
        if (tile_off[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const int64_t d = lo;
    const int64_t s0 = seg_off[d] + (t - tile_off[d]) * kTile;
    const int cnt = (int)min((int64_t)kTile, seg_off[d + 1] - s0);
    const int i = threadIdx.x;

    __shared__ double red[3][kTile];
    double k[3] = {0.0, 0.0, 0.0}, p[3] = {0.0, 0.0, 0.0};
    if (i < cnt) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            k[c] = kls[3 * (s0 + i) + c];
            p[c] = p0s[3 * (s0 + i) + c];
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) red[c][i] = p[c];
    __syncthreads();
    for (int w = kTile / 2; w > 0; w >>= 1) {   // fixed-order tree: deterministic origin
        if (i < w) {
#pragma unroll
            for (int c = 0; c < 3; ++c) red[c][i] += red[c][i + w];
        }
        __syncthreads();
    }
    float ohi[3], olo[3];
    double o[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        split_df(cnt > 0 ? red[c][0] / cnt : 0.0, ohi[c], olo[c]);
        o[c] = (double)ohi[c] + (double)olo[c];
    }
    // sub-block origins: FP32 centroid of the sub-block's offsets from the tile origin
    double off[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) off[c] = p[c] - o[c];
    __syncthreads();                              // everyone has read red[c][0]
#pragma unroll
    for (int c = 0; c < 3; ++c) red[c][i] = i < cnt ? off[c] : 0.0;
    __syncthreads();
    for (int w = kSub / 2; w > 0; w >>= 1) {      // fixed-order tree within each sub-block
        if (i % kSub < w) {
#pragma unroll
            for (int c = 0; c < 3; ++c) red[c][i] += red[c][i + w];
        }
        __syncthreads();
    }
    const int sbk = i / kSub;
    const int cnt_sb = min(max(cnt - sbk * kSub, 0), kSub);
    float so[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) so[c] = cnt_sb > 0 ? (float)(red[c][sbk * kSub] / cnt_sb) : 0.0f;

    unsigned char *tile = tiles + t * (int64_t)kTileBytes;
    TileHeader *hdr = reinterpret_cast<TileHeader *>(tile);
    float *f = reinterpret_cast<float *>(tile + kTileHeaderBytes);
    if (i == 0) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            hdr->o_hi[c] = ohi[c];
            hdr->o_lo[c] = olo[c];
        }
        hdr->count = cnt;
        hdr->pad = 0;
#pragma unroll
        for (int c = 0; c < 4; ++c) hdr->pad2[c] = 0.0f;
    }
    if (i % kSub == 0) {
#pragma unroll
        for (int c = 0; c < 3; ++c) hdr->sub_o[sbk][c] = so[c];
    }
    if (i < cnt) {
        // kl x (p0 - origin - sub-block origin), in FP64, rounded once
        const double e[3] = {off[0] - (double)so[0], off[1] - (double)so[1], off[2] - (double)so[2]};
        const double m[3] = {k[1] * e[2] - k[2] * e[1], k[2] * e[0] - k[0] * e[2], k[0] * e[1] - k[1] * e[0]};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            f[c * kTile + i] = (float)k[c];
            f[(3 + c) * kTile + i] = (float)m[c];
            f[(6 + c) * kTile + i] = (float)off[c];
        }
    } else {   // padding: zero current element far away (contributes exactly 0)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            f[c * kTile + i] = 0.0f;
            f[(3 + c) * kTile + i] = 0.0f;
            f[(6 + c) * kTile + i] = kPadOffset;
        }
    }
}

int launch_pack_f32c(const double *kls, const double *p0s, const int64_t *h_seg_off, int n_designs,
                     void *packed, int64_t packed_bytes, cudaStream_t st) {
    std::vector<int64_t> hdr(kPackedHeaderBytes / 8 + 2 * (n_designs + 1), 0);
    int64_t *tile_off = hdr.data() + kPackedHeaderBytes / 8;
    int64_t *seg_off = tile_off + (n_designs + 1);
    tile_off[0] = 0;
    for (int d = 0; d < n_designs; ++d) {
        const int64_t ns = h_seg_off[d + 1] - h_seg_off[d];
        tile_off[d + 1] = tile_off[d] + (ns + kTile - 1) / kTile;
    }
    for (int d = 0; d <= n_designs; ++d) seg_off[d] = h_seg_off[d];
    hdr[0] = kPackedMagic;
    hdr[1] = n_designs;
    hdr[2] = tile_off[n_designs];
    const int64_t need = kPackedHeaderBytes + packed_index_bytes(n_designs) + tile_off[n_designs] * kTileBytes;
    if (packed_bytes < need)
        return set_error(CCT_ERR_ARG, "packed buffer holds %lld bytes, needs %lld", (long long)packed_bytes,
                         (long long)need);
    CCT_TRY_CUDA(cudaMemcpyAsync(packed, hdr.data(), hdr.size() * 8, cudaMemcpyHostToDevice, st));
    if (tile_off[n_designs] > 0) {
        pack_f32c_kernel<<<(unsigned)tile_off[n_designs], kTile, 0, st>>>(kls, p0s,
                                                                         static_cast<unsigned char *>(packed));
        CCT_TRY_CUDA(cudaGetLastError());
    }
    // the header copy reads a host vector that goes out of scope here
    CCT_TRY_CUDA(cudaStreamSynchronize(st));
    return CCT_OK;
}

// ===================================================================== FP32c field
// Launch shape from a sweep of (threads, points per thread, CTAs per SM, unroll, ring depth)
// on the 2^20-point field map: 3 points per thread, 3 CTAs of 4 warps per SM (146 registers),
// the sub-block's 8-iteration segment loop fully unrolled.  CTAs of 3 or 6 warps were 20 %
// slower (their warps leave one SM sub-partition idle).
constexpr int kF32Block = 128;
constexpr int kF32Ppt = 3;
constexpr int kF32Blocks = 3;
constexpr int kF32Unroll = 8;
constexpr int kStages = 3;
constexpr bool kF32Rcp = false;   // |r|^-3 as rsqrt x rcp (tile.cuh inv_r3)
constexpr uint32_t kWaitPolls = 1u << 22;

__device__ int g_field_status;   // last non-OK status seen by a field kernel (sticky)

__global__ void __launch_bounds__(kF32Block, kF32Blocks) field_f32c_kernel(const unsigned char *__restrict__ packed,
                                                                  int design, const double *__restrict__ qs,
                                                                  int n_qs, const double *__restrict__ pts,
                                                                  int64_t n, double *__restrict__ B) {
    __shared__ __align__(128) unsigned char buf[kStages][kTileBytes];
    __shared__ __align__(8) uint64_t full[kStages];
    __shared__ int64_t last_issued[kStages];   // tile index last copied into each slot (-1: none)
    __shared__ int released[kStages];          // warps done with the slot's current tile
    constexpr int kWarps = kF32Block / 32;
    const int tid = threadIdx.x, lane = tid & 31;
    const int64_t magic = reinterpret_cast<const int64_t *>(packed)[0];
    const int64_t n_designs = reinterpret_cast<const int64_t *>(packed)[1];
    const int64_t base = (int64_t)blockIdx.x * kF32Block * kF32Ppt;
    if (magic != kPackedMagic || design >= n_designs) {   // not a packed set, or no such design
        if (tid == 0 && blockIdx.x == 0) atomicExch(&g_field_status, (int)CCT_ERR_ARG);
        for (int i = 0; i < kF32Ppt; ++i) {
            const int64_t idx = base + tid + (int64_t)i * kF32Block;
            if (idx < n) B[3 * idx] = B[3 * idx + 1] = B[3 * idx + 2] = __longlong_as_double(0x7ff8000000000000LL);
        }
        return;
    }
    const int64_t *tile_off = reinterpret_cast<const int64_t *>(packed + kPackedHeaderBytes);
    const unsigned char *tiles = packed + kPackedHeaderBytes + packed_index_bytes((int)n_designs) +
                                 tile_off[design] * (int64_t)kTileBytes;
    const int64_t nt = tile_off[design + 1] - tile_off[design];

    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            cctdev::mbar_init(&full[s], 1);
            released[s] = 0;
            last_issued[s] = -1;
        }
        cctdev::mbar_fence_init();
    }
    __syncthreads();
    if (tid == 0) {
        for (int s = 0; s < kStages && s < nt; ++s) {
            last_issued[s] = s;
            cctdev::mbar_arrive_expect_tx(&full[s], kTileBytes);
            cctdev::bulk_g2s(buf[s], tiles + (int64_t)s * kTileBytes, kTileBytes, &full[s]);
        }
    }

    // each thread's points as double-float pairs in shared memory (only that thread reads them):
    // spt[c][i][tid], c = hi x, y, z, lo x, y, z
    __shared__ float spt[6][kF32Ppt][kF32Block];
#pragma unroll
    for (int i = 0; i < kF32Ppt; ++i) {
        int64_t idx = base + tid + (int64_t)i * kF32Block;
        if (idx >= n) idx = n - 1;
#pragma unroll
        for (int c = 0; c < 3; ++c) split_df(pts[3 * idx + c], spt[c][i][tid], spt[3 + c][i][tid]);
    }
    F32cAcc<kF32Ppt> acc;
    acc.zero();

    // Warps run through the ring independently: a warp waits only for its next tile to land;
    // the last warp done with a slot refills it with the tile kStages further on.
    bool failed = false;
    for (int64_t t = 0; t < nt; ++t) {
        const int s = (int)(t % kStages);
        const bool ok = cctdev::mbar_wait_bounded(&full[s], (uint32_t)((t / kStages) & 1), kWaitPolls);
        if (!__all_sync(0xffffffffu, ok)) {
            failed = true;
            break;
        }
        tile_f32c_smem<kF32Ppt, kF32Unroll, kF32Rcp>(buf[s], &spt[0][0][tid], kF32Ppt * kF32Block, kF32Block, acc);
        if (cctdev::ring_release_last(&released[s], kWarps) && t + kStages < nt) {
            last_issued[s] = t + kStages;
            cctdev::fence_proxy_async();
            cctdev::mbar_arrive_expect_tx(&full[s], kTileBytes);
            cctdev::bulk_g2s(buf[s], tiles + (t + kStages) * (int64_t)kTileBytes, kTileBytes, &full[s]);
        }
    }
    failed = __syncthreads_or(failed);
    if (failed && tid == 0) {
        // a warp gave up: let the last copy into every slot land before the CTA's shared
        // memory is released (earlier copies into a slot were consumed before its refill)
        for (int s = 0; s < kStages; ++s)
            if (last_issued[s] >= 0)
                (void)cctdev::mbar_wait_bounded(&full[s], (uint32_t)((last_issued[s] / kStages) & 1), kWaitPolls);
        atomicExch(&g_field_status, (int)CCT_ERR_TIMEOUT);
    }
    (void)lane;

#pragma unroll
    for (int i = 0; i < kF32Ppt; ++i) {
        const int64_t idx = base + tid + (int64_t)i * kF32Block;
        if (idx >= n) continue;
        if (failed) {
            B[3 * idx] = B[3 * idx + 1] = B[3 * idx + 2] = __longlong_as_double(0x7ff8000000000000LL);
            continue;
        }
        double bx = acc.total(i, 0), by = acc.total(i, 1), bz = acc.total(i, 2);
        for (int q = 0; q < n_qs; ++q)
            qs_field_add(qs + kQsRecord * q, pts[3 * idx], pts[3 * idx + 1], pts[3 * idx + 2], bx, by, bz);
        B[3 * idx] = bx;
        B[3 * idx + 1] = by;
        B[3 * idx + 2] = bz;
    }
}

__device__ int g_field_status_taken;   // g_field_status as field_status_take_kernel last found it

__global__ void field_status_take_kernel() { g_field_status_taken = atomicExch(&g_field_status, 0); }

int take_field_status(cudaStream_t st, int *status) {
    field_status_take_kernel<<<1, 1, 0, st>>>();
    CCT_TRY_CUDA(cudaGetLastError());
    CCT_TRY_CUDA(cudaMemcpyFromSymbolAsync(status, g_field_status_taken, sizeof(int), 0, cudaMemcpyDeviceToHost, st));
    CCT_TRY_CUDA(cudaStreamSynchronize(st));
    return CCT_OK;
}

int launch_field_f32c(const void *packed, int design, const double *qs, int n_qs, const double *pts, int64_t n,
                      double *B, cudaStream_t st) {
    if (n == 0) return CCT_OK;
    const int64_t per = (int64_t)kF32Block * kF32Ppt;
    const int64_t grid = (n + per - 1) / per;
    if (grid > 0x7fffffff) return set_error(CCT_ERR_ARG, "too many field points (%lld)", (long long)n);
    field_f32c_kernel<<<(unsigned)grid, kF32Block, 0, st>>>(static_cast<const unsigned char *>(packed), design, qs,
                                                            n_qs, pts, n, B);
    CCT_TRY_CUDA(cudaGetLastError());
    return CCT_OK;
}

}  // namespace cctgpu
