// extern "C" entry points of libcctgpu (declared in include/cctgpu.h).
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "cctgpu_internal.cuh"

namespace cctgpu {

static thread_local std::string g_err;
static thread_local int g_status = CCT_OK;

int set_error(int status, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    g_status = status;
    return status;
}

int check_cuda(cudaError_t e, const char *what) {
    return set_error(CCT_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

int clear_error() {
    g_err.clear();
    g_status = CCT_OK;
    return CCT_OK;
}

static bool aligned(const void *p, size_t a) { return reinterpret_cast<uintptr_t>(p) % a == 0; }

}  // namespace cctgpu

using namespace cctgpu;

extern "C" {

int cct_version(void) { return 100; }

int cct_last_error(char *buf, size_t n) {
    if (buf && n) {
        std::strncpy(buf, g_err.c_str(), n - 1);
        buf[n - 1] = 0;
    }
    return g_status;
}

int cct_f32c_tile(void) { return kTile; }

int cct_field_f64(const double *d_kls, const double *d_p0s, int64_t n_seg, const double *d_qs, int32_t n_qs,
                  const double *d_points, int64_t n_points, double *d_B, void *stream) {
    clear_error();
    if (n_seg < 0 || n_qs < 0 || n_points < 0) return set_error(CCT_ERR_ARG, "negative size");
    if (n_points > 0 && (!d_points || !d_B)) return set_error(CCT_ERR_ARG, "null points or output");
    if (n_seg > 0 && (!d_kls || !d_p0s)) return set_error(CCT_ERR_ARG, "null segment arrays");
    if (n_qs > 0 && !d_qs) return set_error(CCT_ERR_ARG, "null QS records");
    return launch_field_f64(d_kls, d_p0s, n_seg, d_qs, n_qs, d_points, n_points, d_B,
                            static_cast<cudaStream_t>(stream));
}

int64_t cct_f32c_packed_bytes(const int64_t *h_seg_off, int32_t n_designs) {
    clear_error();
    if (n_designs <= 0 || !h_seg_off) {
        set_error(CCT_ERR_ARG, "need at least one design");
        return -1;
    }
    int64_t tiles = 0;
    for (int d = 0; d < n_designs; ++d) {
        const int64_t ns = h_seg_off[d + 1] - h_seg_off[d];
        if (ns < 0) {
            set_error(CCT_ERR_ARG, "segment offsets decrease at design %d", d);
            return -1;
        }
        tiles += (ns + kTile - 1) / kTile;
    }
    return kPackedHeaderBytes + packed_index_bytes(n_designs) + tiles * kTileBytes;
}

int cct_f32c_pack(const double *d_kls, const double *d_p0s, const int64_t *h_seg_off, int32_t n_designs,
                  void *d_packed, int64_t packed_bytes, void *stream) {
    const int64_t need = cct_f32c_packed_bytes(h_seg_off, n_designs);
    if (need < 0) return g_status;
    if (!d_packed || !aligned(d_packed, 256)) return set_error(CCT_ERR_ARG, "packed buffer must be 256-byte aligned");
    if (h_seg_off[n_designs] > h_seg_off[0] && (!d_kls || !d_p0s)) return set_error(CCT_ERR_ARG, "null segments");
    return launch_pack_f32c(d_kls, d_p0s, h_seg_off, n_designs, d_packed, packed_bytes,
                            static_cast<cudaStream_t>(stream));
}

int cct_field_f32c(const void *d_packed, int32_t design, const double *d_qs, int32_t n_qs, const double *d_points,
                   int64_t n_points, double *d_B, void *stream) {
    clear_error();
    if (!d_packed || !aligned(d_packed, 256)) return set_error(CCT_ERR_ARG, "packed buffer must be 256-byte aligned");
    if (design < 0 || n_qs < 0 || n_points < 0) return set_error(CCT_ERR_ARG, "negative design index or size");
    if (n_points > 0 && (!d_points || !d_B)) return set_error(CCT_ERR_ARG, "null points or output");
    if (n_qs > 0 && !d_qs) return set_error(CCT_ERR_ARG, "null QS records");
    return launch_field_f32c(d_packed, design, d_qs, n_qs, d_points, n_points, d_B, static_cast<cudaStream_t>(stream));
}

int cct_field_status(void *stream) {
    clear_error();
    int s = CCT_OK;
    const int rc = take_field_status(static_cast<cudaStream_t>(stream), &s);
    if (rc != CCT_OK) return rc;
    if (s == CCT_ERR_ARG)
        return set_error(CCT_ERR_ARG, "an FP32c field call was given a buffer that is not a packed segment set, or a "
                                      "design index the set does not hold (its fields are NaN)");
    if (s == CCT_ERR_TIMEOUT)
        return set_error(CCT_ERR_TIMEOUT, "an FP32c field call's tile copy did not land within the wait limit (its "
                                          "fields are NaN)");
    return s == CCT_OK ? CCT_OK : set_error(s, "field kernel status %d", s);
}

int cct_field_host(const double *h_kls, const double *h_p0s, int64_t n_seg, const double *h_qs, int32_t n_qs,
                   const double *h_points, int64_t n_points, double *h_B, int32_t precision) {
    clear_error();
    if (n_seg < 0 || n_qs < 0 || n_points < 0) return set_error(CCT_ERR_ARG, "negative size");
    if (precision != 0 && precision != 1) return set_error(CCT_ERR_ARG, "precision must be 0 or 1");
    if (n_points == 0) return CCT_OK;
    cudaStream_t st = nullptr;
    const int64_t seg_off[2] = {0, n_seg};
    const int64_t pk = precision == 1 ? cct_f32c_packed_bytes(seg_off, 1) : 0;
    const size_t seg_b = 24 * (size_t)n_seg, pts_b = 24 * (size_t)n_points, qs_b = 8 * kQsRecord * (size_t)n_qs;
    unsigned char *mem = nullptr;
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t total = 2 * up(seg_b) + 2 * up(pts_b) + up(qs_b) + up((size_t)pk);
    CCT_TRY_CUDA(cudaMalloc(&mem, total));
    double *kls = reinterpret_cast<double *>(mem);
    double *p0s = reinterpret_cast<double *>(mem + up(seg_b));
    double *pts = reinterpret_cast<double *>(mem + 2 * up(seg_b));
    double *B = reinterpret_cast<double *>(mem + 2 * up(seg_b) + up(pts_b));
    double *qs = reinterpret_cast<double *>(mem + 2 * up(seg_b) + 2 * up(pts_b));
    void *packed = mem + 2 * up(seg_b) + 2 * up(pts_b) + up(qs_b);
    int rc = CCT_OK;
    cudaError_t e = cudaSuccess;
    if (seg_b) e = cudaMemcpyAsync(kls, h_kls, seg_b, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && seg_b) e = cudaMemcpyAsync(p0s, h_p0s, seg_b, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && qs_b) e = cudaMemcpyAsync(qs, h_qs, qs_b, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(pts, h_points, pts_b, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) rc = check_cuda(e, "cudaMemcpyAsync (inputs)");
    if (rc == CCT_OK) {
        if (precision == 0) {
            rc = launch_field_f64(kls, p0s, n_seg, qs, n_qs, pts, n_points, B, st);
        } else {
            rc = launch_pack_f32c(kls, p0s, seg_off, 1, packed, pk, st);
            if (rc == CCT_OK) rc = launch_field_f32c(packed, 0, qs, n_qs, pts, n_points, B, st);
        }
    }
    if (rc == CCT_OK) {
        e = cudaMemcpyAsync(h_B, B, pts_b, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = check_cuda(e, "cudaMemcpyAsync (field)");
    }
    cudaFree(mem);
    return rc;
}

int64_t cct_track_scratch_bytes(int32_t n_designs, int64_t n_particles) {
    clear_error();
    if (n_designs <= 0 || n_particles <= 0) {
        set_error(CCT_ERR_ARG, "need at least one design and one particle");
        return -1;
    }
    return track_scratch_bound(n_designs, n_particles);
}

int cct_track(const double *d_kls, const double *d_p0s, const int64_t *d_seg_off, const void *d_packed,
              const double *d_qs, const int64_t *d_qs_off, int32_t n_designs, double *d_particles,
              int64_t n_particles, double distance, double footstep, int32_t precision, void *d_scratch,
              int64_t scratch_bytes, void *stream) {
    clear_error();
    if (n_designs <= 0 || n_particles < 0) return set_error(CCT_ERR_ARG, "need at least one design");
    if (n_particles == 0) return CCT_OK;
    if (!(distance > 0.0) || !(footstep > 0.0))
        return set_error(CCT_ERR_ARG, "distance (%g) and footstep (%g) must be positive", distance, footstep);
    if (precision != 0 && precision != 1) return set_error(CCT_ERR_ARG, "precision must be 0 or 1");
    if (!d_seg_off || !d_qs_off || !d_particles || !d_scratch) return set_error(CCT_ERR_ARG, "null pointer");
    if (precision == 1 && (!d_packed || !aligned(d_packed, 256)))
        return set_error(CCT_ERR_ARG, "FP32c tracking needs a 256-byte aligned packed buffer");
    return launch_track(d_kls, d_p0s, d_seg_off, d_packed, d_qs, d_qs_off, n_designs, d_particles, n_particles,
                        distance, footstep, precision, d_scratch, scratch_bytes, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
