// One FP32-compensated tile of the packed segment form, shared by the field-map and
// tracking kernels.
//
// Tile (kTileBytes = 4704 = 16 * 294):
//   float o_hi[3], o_lo[3];  int count; int pad;      origin = o_hi + o_lo (double-float)
//   float sub_o[4][3]; float pad2[4];                 origin of each 32-segment sub-block,
//                                                     relative to the tile origin
//   float kx[128], ky[128], kz[128];                   kl
//   float mx[128], my[128], mz[128];                   kl x (p0 - origin - sub_o)
//   float px[128], py[128], pz[128];                   p0 - origin
// Arithmetic ("moment form"): over a sub-block with origin o,
//   sum_i kl_i x (q - p_i) |r_i|^-3 = A x (q - o) - M,  A = sum_i kl_i |r_i|^-3,
//                                                        M = sum_i (kl_i x (p_i - o)) |r_i|^-3,
// so a pair costs r = q - p_i, |r|^2, rsqrt, |r|^-3 and the six multiply-adds into A and M
// (14 FMA-pipe operations instead of 17 for kl x r scaled and summed); the cross product with
// q - o is taken once per sub-block.  The sub-block origin keeps |q - o| within the
// sub-block's extent of |r|, so the cancellation in A x (q - o) - M adds little to the
// rounding of r itself (measured by an FP32 emulation: at points 3-8 mm from the windings
// 1.3x the error of the direct form with 32-segment sub-blocks, 1.85x with 64).  Pair terms
// run as packed FP32 pairs (PTX f32x2, two segments per instruction), rsqrt on the MUFU pipe;
// each half accumulates A over the 16 segments of a sub-block and M over the whole call (a
// tile or a slice of it) in FP32; the call's field sum(A x w) - M is added to a
// Kahan-compensated (S, C) pair, and S - C is taken in FP64 at the end.
#pragma once

#include <stdint.h>

#include "cctgpu_internal.cuh"

namespace cctgpu {

typedef uint64_t f2;   // two packed FP32 values (low half = even segment)

__device__ __forceinline__ f2 f2_pack(float lo, float hi) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2 v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) {
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// sign flip of both halves (integer XOR, off the FMA pipe)
__device__ __forceinline__ f2 f2_neg(f2 a) { return a ^ 0x8000000080000000ull; }
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ float rsqrt_mufu(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_mufu(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// |r|^-3 of two packed squared distances.  RCP = false: rsqrt cubed (MUFU rsqrt, two FMA-pipe
// multiplies); RCP = true: rsqrt(r^2) x rcp(r^2) (two MUFU operations, one multiply), which
// moves one of the pair's FMA-pipe operations to the MUFU pipe.
template <bool RCP>
__device__ __forceinline__ f2 inv_r3(f2 r2) {
    float a, b;
    f2_unpack(r2, a, b);
    const f2 inv = f2_pack(rsqrt_mufu(a), rsqrt_mufu(b));
    if (RCP) return f2_mul(inv, f2_pack(rcp_mufu(a), rcp_mufu(b)));
    return f2_mul(f2_mul(inv, inv), inv);
}

// Kahan step: (S, C) += s
__device__ __forceinline__ void kahan_add(float &S, float &C, float s) {
    const float y = __fsub_rn(s, C);
    const float t = __fadd_rn(S, y);
    C = __fsub_rn(__fsub_rn(t, S), y);
    S = t;
}

struct TileHeader {
    float o_hi[3], o_lo[3];
    int count, pad;
    float sub_o[kTile / kSub][3];
    float pad2[4];
};
static_assert(sizeof(TileHeader) == kTileHeaderBytes, "tile header layout");
static_assert(kTile == 4 * kSub, "four sub-blocks per tile");

// Per-point state of the compensated sum.
template <int PPT>
struct F32cAcc {
    float S[PPT][3], C[PPT][3];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int i = 0; i < PPT; ++i)
#pragma unroll
            for (int c = 0; c < 3; ++c) S[i][c] = C[i][c] = 0.0f;
    }
    __device__ __forceinline__ double total(int i, int c) const { return (double)S[i][c] - (double)C[i][c]; }
};

// Accumulate segments [4*g0, 4*g1) of one tile (default: all 128) for PPT points given as
// double-float (hi, lo) coordinates.  JU: unroll of the 4-segment loop (2 keeps more
// independent pair terms in flight where registers allow).
// The point offsets from the tile origin, q = (p_hi - o_hi) + (p_lo - o_lo) in FP32, packed.
template <int PPT>
__device__ __forceinline__ void tile_offsets(const TileHeader *h, const float (&ph)[PPT][3], const float (&pl)[PPT][3],
                                             f2 (&q)[PPT][3]) {
#pragma unroll
    for (int i = 0; i < PPT; ++i)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float d = __fadd_rn(__fsub_rn(ph[i][c], h->o_hi[c]), __fsub_rn(pl[i][c], h->o_lo[c]));
            q[i][c] = f2_pack(d, d);
        }
}

// g0 and g1 are multiples of kSub / 4 (whole sub-blocks).
template <int PPT, int JU, bool RCP>
__device__ __forceinline__ void tile_pairs(const unsigned char *tile, const f2 (&q)[PPT][3], F32cAcc<PPT> &acc,
                                           int g0, int g1);

template <int PPT, int JU = 1, bool RCP = false>
__device__ __forceinline__ void tile_f32c(const unsigned char *tile, const float (&ph)[PPT][3],
                                          const float (&pl)[PPT][3], F32cAcc<PPT> &acc, int g0 = 0,
                                          int g1 = kTile / 4) {
    f2 q[PPT][3];
    tile_offsets<PPT>(reinterpret_cast<const TileHeader *>(tile), ph, pl, q);
    tile_pairs<PPT, JU, RCP>(tile, q, acc, g0, g1);
}

// The same with the point's double-float coordinates kept in shared memory: component c
// (hi x, y, z, lo x, y, z) of point i at sp[c * c_stride + i * i_stride], so that they hold
// no registers during the segment loop.
template <int PPT, int JU = 1, bool RCP = false>
__device__ __forceinline__ void tile_f32c_smem(const unsigned char *tile, const float *sp, int c_stride, int i_stride,
                                               F32cAcc<PPT> &acc, int g0 = 0, int g1 = kTile / 4) {
    float ph[PPT][3], pl[PPT][3];
#pragma unroll
    for (int i = 0; i < PPT; ++i)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            ph[i][c] = sp[c * c_stride + i * i_stride];
            pl[i][c] = sp[(3 + c) * c_stride + i * i_stride];
        }
    f2 q[PPT][3];
    tile_offsets<PPT>(reinterpret_cast<const TileHeader *>(tile), ph, pl, q);
    tile_pairs<PPT, JU, RCP>(tile, q, acc, g0, g1);
}

template <int PPT, int JU, bool RCP>
__device__ __forceinline__ void tile_pairs(const unsigned char *tile, const f2 (&q)[PPT][3], F32cAcc<PPT> &acc,
                                           int g0, int g1) {
    const TileHeader *h = reinterpret_cast<const TileHeader *>(tile);
    const ulonglong2 *v = reinterpret_cast<const ulonglong2 *>(tile + kTileHeaderBytes);
    constexpr int Q = kTile / 4;          // ulonglong2 (4 floats) per component array
    constexpr int SG = kSub / 4;          // 4-segment groups per sub-block
    // g0 and g1 are multiples of SG (whole sub-blocks).  T collects the sub-blocks' A x w
    // (A summed over a sub-block, w = q - that sub-block's origin); the moments M of the call are summed
    // together and subtracted once.
    float T[PPT][3];
    f2 M[PPT][3];
#pragma unroll
    for (int i = 0; i < PPT; ++i)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            T[i][c] = 0.0f;
            M[i][c] = 0ull;
        }
#pragma unroll 1
    for (int sb = g0; sb < g1; sb += SG) {
        f2 A[PPT][3];
#pragma unroll
        for (int i = 0; i < PPT; ++i) A[i][0] = A[i][1] = A[i][2] = 0ull;
#pragma unroll JU
        for (int j = sb; j < sb + SG; ++j) {                     // 4 segments per iteration
            const ulonglong2 KX = v[0 * Q + j], KY = v[1 * Q + j], KZ = v[2 * Q + j];
            const ulonglong2 MX = v[3 * Q + j], MY = v[4 * Q + j], MZ = v[5 * Q + j];
            const ulonglong2 PX = v[6 * Q + j], PY = v[7 * Q + j], PZ = v[8 * Q + j];
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const f2 kx = hh ? KX.y : KX.x, ky = hh ? KY.y : KY.x, kz = hh ? KZ.y : KZ.x;
                const f2 mx = hh ? MX.y : MX.x, my = hh ? MY.y : MY.x, mz = hh ? MZ.y : MZ.x;
                const f2 px = hh ? PX.y : PX.x, py = hh ? PY.y : PY.x, pz = hh ? PZ.y : PZ.x;
#pragma unroll
                for (int i = 0; i < PPT; ++i) {
                    const f2 rx = f2_sub(q[i][0], px), ry = f2_sub(q[i][1], py), rz = f2_sub(q[i][2], pz);
                    const f2 r2 = f2_fma(rx, rx, f2_fma(ry, ry, f2_mul(rz, rz)));
                    const f2 inv3 = inv_r3<RCP>(r2);
                    A[i][0] = f2_fma(kx, inv3, A[i][0]);
                    A[i][1] = f2_fma(ky, inv3, A[i][1]);
                    A[i][2] = f2_fma(kz, inv3, A[i][2]);
                    M[i][0] = f2_fma(mx, inv3, M[i][0]);
                    M[i][1] = f2_fma(my, inv3, M[i][1]);
                    M[i][2] = f2_fma(mz, inv3, M[i][2]);
                }
            }
        }
        const float *o = h->sub_o[sb / SG];
#pragma unroll
        for (int i = 0; i < PPT; ++i) {
            float a[3], w[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float lo, hi;
                f2_unpack(A[i][c], lo, hi);
                a[c] = __fadd_rn(lo, hi);
                f2_unpack(q[i][c], lo, hi);
                w[c] = __fsub_rn(lo, o[c]);
            }
            // T += A x w
            T[i][0] = __fmaf_rn(a[1], w[2], __fmaf_rn(-a[2], w[1], T[i][0]));
            T[i][1] = __fmaf_rn(a[2], w[0], __fmaf_rn(-a[0], w[2], T[i][1]));
            T[i][2] = __fmaf_rn(a[0], w[1], __fmaf_rn(-a[1], w[0], T[i][2]));
        }
    }
#pragma unroll
    for (int i = 0; i < PPT; ++i)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            float lo, hi;
            f2_unpack(M[i][c], lo, hi);
            kahan_add(acc.S[i][c], acc.C[i][c], __fsub_rn(T[i][c], __fadd_rn(lo, hi)));
        }
}

// Split an FP64 coordinate into a double-float (hi, lo) pair.
__device__ __forceinline__ void split_df(double x, float &hi, float &lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

}  // namespace cctgpu

namespace cctgpu {

// Adjoint counterpart of tile_f32c: for PPT points with weights a (per point), accumulate
// grad_p (a . B_i) = c |r|^-3 - 3 (c.r) r |r|^-5, c = a x kl_i, over segments [4*g0, 4*g1)
// of one tile, with the same compensation (FP32 sums over 32-segment sub-blocks, Kahan (S, C)).
template <int PPT, int JU = 1>
__device__ __forceinline__ void tile_grad_f32c(const unsigned char *tile, const float (&ph)[PPT][3],
                                               const float (&pl)[PPT][3], const float (&a)[PPT][3],
                                               F32cAcc<PPT> &acc, int g0 = 0, int g1 = kTile / 4) {
    const TileHeader *h = reinterpret_cast<const TileHeader *>(tile);
    const ulonglong2 *v = reinterpret_cast<const ulonglong2 *>(tile + kTileHeaderBytes);
    constexpr int Q = kTile / 4;
    f2 q[PPT][3], A[PPT][3], NA[PPT][3];
#pragma unroll
    for (int i = 0; i < PPT; ++i)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float d = __fadd_rn(__fsub_rn(ph[i][c], h->o_hi[c]), __fsub_rn(pl[i][c], h->o_lo[c]));
            q[i][c] = f2_pack(d, d);
            A[i][c] = f2_pack(a[i][c], a[i][c]);
            NA[i][c] = f2_pack(-a[i][c], -a[i][c]);
        }
    const f2 m3 = f2_pack(-3.0f, -3.0f);
    constexpr int SG = kSub / 4;          // 4-segment groups per FP32 sub-sum
    // g0 and g1 are multiples of SG (a slice of a tile holds whole sub-blocks)
#pragma unroll 1
    for (int sb = g0; sb < g1; sb += SG) {
        f2 G[PPT][3];
#pragma unroll
        for (int i = 0; i < PPT; ++i) G[i][0] = G[i][1] = G[i][2] = 0ull;
#pragma unroll JU
        for (int j = sb; j < sb + SG; ++j) {
            const ulonglong2 KX = v[0 * Q + j], KY = v[1 * Q + j], KZ = v[2 * Q + j];
            const ulonglong2 PX = v[6 * Q + j], PY = v[7 * Q + j], PZ = v[8 * Q + j];
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const f2 kx = hh ? KX.y : KX.x, ky = hh ? KY.y : KY.x, kz = hh ? KZ.y : KZ.x;
                const f2 px = hh ? PX.y : PX.x, py = hh ? PY.y : PY.x, pz = hh ? PZ.y : PZ.x;
#pragma unroll
                for (int i = 0; i < PPT; ++i) {
                    const f2 rx = f2_sub(q[i][0], px), ry = f2_sub(q[i][1], py), rz = f2_sub(q[i][2], pz);
                    const f2 r2 = f2_fma(rx, rx, f2_fma(ry, ry, f2_mul(rz, rz)));
                    float lo, hi;
                    f2_unpack(r2, lo, hi);
                    const f2 inv = f2_pack(rsqrt_mufu(lo), rsqrt_mufu(hi));
                    const f2 inv2 = f2_mul(inv, inv);
                    const f2 inv3 = f2_mul(inv2, inv);
                    const f2 m3inv5 = f2_mul(f2_mul(inv3, inv2), m3);
                    // c = a x kl = (ay kz - az ky, az kx - ax kz, ax ky - ay kx)
                    const f2 cx = f2_fma(A[i][1], kz, f2_mul(NA[i][2], ky));
                    const f2 cy = f2_fma(A[i][2], kx, f2_mul(NA[i][0], kz));
                    const f2 cz = f2_fma(A[i][0], ky, f2_mul(NA[i][1], kx));
                    const f2 cr = f2_fma(cx, rx, f2_fma(cy, ry, f2_mul(cz, rz)));
                    const f2 nq = f2_mul(cr, m3inv5);
                    G[i][0] = f2_fma(nq, rx, f2_fma(cx, inv3, G[i][0]));
                    G[i][1] = f2_fma(nq, ry, f2_fma(cy, inv3, G[i][1]));
                    G[i][2] = f2_fma(nq, rz, f2_fma(cz, inv3, G[i][2]));
                }
            }
        }
#pragma unroll
        for (int i = 0; i < PPT; ++i)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float lo, hi;
                f2_unpack(G[i][c], lo, hi);
                kahan_add(acc.S[i][c], acc.C[i][c], __fadd_rn(lo, hi));
            }
    }
}

}  // namespace cctgpu
