// Internal declarations shared by the CUDA translation units of libcctgpu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/cctgpu.h"

namespace cctgpu {

// ---------------------------------------------------------------- constants
constexpr int kTile = 128;                   // segments per FP32c tile
constexpr int kSub = 32;                     // segments per FP32c sub-block (own moment origin)
constexpr int kTileHeaderBytes = 96;         // double-float origin, count, pad, sub-block origins
constexpr int kTileBytes = kTileHeaderBytes + 9 * kTile * 4;   // 4704, a multiple of 16
constexpr int kPackedHeaderBytes = 256;      // magic, n_designs, n_tiles
constexpr int64_t kPackedMagic = 0x4343543332434332LL;          // "CCT32CC2"
constexpr float kPadOffset = 1.0e18f;        // padding segment: kl = 0, far away
constexpr int kQsRecord = 16;                // doubles per QS record

// Packed buffer: [header 256 B][int64 tile_off[n+1], int64 seg_off[n+1], padded to 256][tiles]
__host__ __device__ inline int64_t packed_index_bytes(int n_designs) {
    int64_t b = 16 * (int64_t)(n_designs + 1);
    return (b + 255) / 256 * 256;
}

// ---------------------------------------------------------------- error state (host)
int set_error(int status, const char *fmt, ...);
int check_cuda(cudaError_t e, const char *what);
int clear_error();

#define CCT_TRY_CUDA(expr)                                        \
    do {                                                          \
        cudaError_t _e = (expr);                                  \
        if (_e != cudaSuccess) return check_cuda(_e, #expr);      \
    } while (0)

// ---------------------------------------------------------------- launchers (host, defined in the .cu files)
int launch_field_f64(const double *kls, const double *p0s, int64_t n_seg, const double *qs, int n_qs,
                     const double *pts, int64_t n, double *B, cudaStream_t st);
int launch_pack_f32c(const double *kls, const double *p0s, const int64_t *h_seg_off, int n_designs,
                     void *packed, int64_t packed_bytes, cudaStream_t st);
int launch_field_f32c(const void *packed, int design, const double *qs, int n_qs, const double *pts,
                      int64_t n, double *B, cudaStream_t st);
// Reads and clears the status the FP32c field kernels recorded on the current device; waits for st.
int take_field_status(cudaStream_t st, int *status);

struct TrackScratchLayout {
    int64_t state_off, partial_off, ctrl_off, flow_off, total;
};
// Scratch layout for n_units units of `group` particles each.
TrackScratchLayout track_scratch_layout(int n_designs, int64_t n_particles, int64_t n_units, int group);
// Upper bound of the scratch any precision needs on the current device (or a generous
// device-independent bound when no device is visible), with the particle block the forward
// entry points use (block_setting: the process-wide setting if made) or group_size's (the
// adjoint's).
int64_t track_scratch_bound(int n_designs, int64_t n_particles, bool block_setting = true);
int launch_track_async(const double *kls, const double *p0s, const int64_t *seg_off, const void *packed,
                       const double *qs, const int64_t *qs_off, int n_designs, double *particles, int64_t n_p,
                       double distance, double footstep, int precision, void *scratch, int64_t scratch_bytes,
                       cudaStream_t st);
int track_status(const void *scratch, cudaStream_t st);
int launch_track(const double *kls, const double *p0s, const int64_t *seg_off, const void *packed,
                 const double *qs, const int64_t *qs_off, int n_designs, double *particles, int64_t n_particles,
                 double distance, double footstep, int precision, void *scratch, int64_t scratch_bytes,
                 cudaStream_t st);

}  // namespace cctgpu

// ---------------------------------------------------------------- device helpers
namespace cctdev {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// One-dimensional bulk copy global -> shared (TMA engine), completion counted on `bar`.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase; returns false after `limit` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if (i > 64) __nanosleep(64);
    }
    return false;
}

// Release of a ring slot without a CTA-wide barrier.  Every warp of the CTA calls this (all
// lanes, converged) after its last read of the slot; lane 0 of the last of `n_warps` warps
// to arrive gets true and refills the slot.  The counter's fences order every warp's shared
// reads of the slot before the refill (the refilling lane then issues fence.proxy.async
// before the bulk copy); the counter is reset for the slot's next round.
__device__ __forceinline__ bool ring_release_last(int *cnt, int n_warps) {
    __syncwarp();
    bool last = false;
    if ((threadIdx.x & 31) == 0) {
        __threadfence_block();
        last = atomicAdd(cnt, 1) == n_warps - 1;
        if (last) {
            __threadfence_block();
            atomicExch(cnt, 0);
        }
    }
    return last;
}

}  // namespace cctdev
