// One FP32-compensated tile of the packed segment form, shared by the field-map and
// tracking kernels.
#pragma once

#include "cctgpu_internal.cuh"

namespace cctgpu {

// Kahan-compensated accumulation of one 128-segment tile for PPT points; adds the tile
// partial to the FP64 accumulators.  `tile` may point to shared or global memory.
template <int PPT>
__device__ __forceinline__ void tile_f32c(const unsigned char *tile, const double (&px)[PPT],
                                          const double (&py)[PPT], const double (&pz)[PPT], double (&bx)[PPT],
                                          double (&by)[PPT], double (&bz)[PPT]) {
    const double *hdr = reinterpret_cast<const double *>(tile);
    const float4 *f4 = reinterpret_cast<const float4 *>(tile + kTileHeaderBytes);
    const double ox = hdr[0], oy = hdr[1], oz = hdr[2];
    float qx[PPT], qy[PPT], qz[PPT];
    float Sx[PPT], Sy[PPT], Sz[PPT], Cx[PPT], Cy[PPT], Cz[PPT];
#pragma unroll
    for (int i = 0; i < PPT; ++i) {
        qx[i] = (float)(px[i] - ox);
        qy[i] = (float)(py[i] - oy);
        qz[i] = (float)(pz[i] - oz);
        Sx[i] = Sy[i] = Sz[i] = Cx[i] = Cy[i] = Cz[i] = 0.0f;
    }
#pragma unroll 1
    for (int sb = 0; sb < kTile / 32; ++sb) {
        float sx[PPT], sy[PPT], sz[PPT];
#pragma unroll
        for (int i = 0; i < PPT; ++i) sx[i] = sy[i] = sz[i] = 0.0f;
#pragma unroll 2
        for (int j4 = sb * 8; j4 < sb * 8 + 8; ++j4) {
            const float4 KX = f4[0 * (kTile / 4) + j4], KY = f4[1 * (kTile / 4) + j4], KZ = f4[2 * (kTile / 4) + j4];
            const float4 PX = f4[3 * (kTile / 4) + j4], PY = f4[4 * (kTile / 4) + j4], PZ = f4[5 * (kTile / 4) + j4];
            const float kx[4] = {KX.x, KX.y, KX.z, KX.w}, ky[4] = {KY.x, KY.y, KY.z, KY.w};
            const float kz[4] = {KZ.x, KZ.y, KZ.z, KZ.w}, ox4[4] = {PX.x, PX.y, PX.z, PX.w};
            const float oy4[4] = {PY.x, PY.y, PY.z, PY.w}, oz4[4] = {PZ.x, PZ.y, PZ.z, PZ.w};
#pragma unroll
            for (int u = 0; u < 4; ++u) {
#pragma unroll
                for (int i = 0; i < PPT; ++i) {
                    const float rx = qx[i] - ox4[u], ry = qy[i] - oy4[u], rz = qz[i] - oz4[u];
                    const float inv = rsqrtf(fmaf(rx, rx, fmaf(ry, ry, rz * rz)));
                    const float inv3 = inv * inv * inv;
                    sx[i] = fmaf(fmaf(ky[u], rz, -kz[u] * ry), inv3, sx[i]);
                    sy[i] = fmaf(fmaf(kz[u], rx, -kx[u] * rz), inv3, sy[i]);
                    sz[i] = fmaf(fmaf(kx[u], ry, -ky[u] * rx), inv3, sz[i]);
                }
            }
        }
#pragma unroll
        for (int i = 0; i < PPT; ++i) {   // Kahan step: S += s with compensation C
            float y, t;
            y = __fsub_rn(sx[i], Cx[i]); t = __fadd_rn(Sx[i], y); Cx[i] = __fsub_rn(__fsub_rn(t, Sx[i]), y); Sx[i] = t;
            y = __fsub_rn(sy[i], Cy[i]); t = __fadd_rn(Sy[i], y); Cy[i] = __fsub_rn(__fsub_rn(t, Sy[i]), y); Sy[i] = t;
            y = __fsub_rn(sz[i], Cz[i]); t = __fadd_rn(Sz[i], y); Cz[i] = __fsub_rn(__fsub_rn(t, Sz[i]), y); Sz[i] = t;
        }
    }
#pragma unroll
    for (int i = 0; i < PPT; ++i) {
        bx[i] += (double)Sx[i] - (double)Cx[i];
        by[i] += (double)Sy[i] - (double)Cy[i];
        bz[i] += (double)Sz[i] - (double)Cz[i];
    }
}

}  // namespace cctgpu
