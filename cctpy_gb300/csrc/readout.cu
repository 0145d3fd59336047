// Optimiser read-out: phase space of tracked protons at the beamline exit and the beam
// objectives the reference's optimiser run script computes from it for every design
// (cctpy final_code/work/optim/A05run.py:247-330), one CTA per design.
//
// Phase space (PhaseSpaceParticle.create_from_running_particle, particles.py:1078-1121),
// unfused FP64 in the reference's operation order, so the values are bit-identical:
//   x, y, z   = XI.(p - p_ideal), YI.(...), ZI.(...)
//   x', y'    = XI.dv / sqrt(speed^2 - (XI.dv)^2), dv = v - v_ideal (likewise y')
//   delta     = (speed m - speed_ideal m_ideal) / (speed_ideal m_ideal)
// with speed reset to |v| first where the script does so (A05run.py:265-267).
// Objectives (BaseUtils.Statistic, base_utils.py:603-683), x, y in mm and x', y' in mrad:
//   max |x|, max |x'|, max |y|, max |y'|, |mean x|, |mean x'|, |mean y|, |mean y'|,
//   |max|x| - max|y||, and the width (max - min) of the half widths (max - min)/2 in x and
//   in y of consecutive groups of `group` particles.
// The means restate the float sum the reference's Statistic.average gets from CPython 3.12+
// (Neumaier's compensated sum: Neumaier 1974, ZAMM 54:39-51), summed in list order.
#include "cctgpu_internal.cuh"

namespace cctgpu {

struct ReadoutParams {
    double ideal[10];
    double XI[3], YI[3], ZI[3];
    int group;
    int speed_from_velocity;
};

constexpr int kReadBlock = 128;
constexpr double kMM = 0.001;     // constants.py:12
constexpr double kMRAD = 0.001;   // constants.py:15, 1.0 * MM * RAD with RAD = 1

__device__ __forceinline__ double dot_rn(const double *a, double x, double y, double z) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a[0], x), __dmul_rn(a[1], y)), __dmul_rn(a[2], z));
}

// NaN-propagating max / min (numpy.max / numpy.min semantics)
__device__ __forceinline__ double nmax(double m, double v) { return (isnan(v) || v > m) ? v : m; }
__device__ __forceinline__ double nmin(double m, double v) { return (isnan(v) || v < m) ? v : m; }

struct NeumaierSum {
    double f = 0.0, c = 0.0;
    __device__ void add(double x) {
        const double t = __dadd_rn(f, x);
        if (fabs(f) >= fabs(x)) c = __dadd_rn(c, __dadd_rn(__dsub_rn(f, t), x));
        else c = __dadd_rn(c, __dadd_rn(__dsub_rn(x, t), f));
        f = t;
    }
    __device__ double total() const { return (c != 0.0 && isfinite(c)) ? __dadd_rn(f, c) : f; }
};

__global__ void __launch_bounds__(kReadBlock) readout_kernel(const double *__restrict__ particles, int64_t n_p,
                                                            ReadoutParams R, double *__restrict__ ps,
                                                            double *__restrict__ obj) {
    const int64_t d = blockIdx.x;
    const double *rec = particles + d * n_p * 10;
    double *out = ps + d * n_p * 6;
    const double *I = R.ideal;
    const double im = __dmul_rn(I[8], I[6]);
    for (int64_t j = threadIdx.x; j < n_p; j += kReadBlock) {
        const double *p = rec + j * 10;
        const double rx = __dsub_rn(p[0], I[0]), ry = __dsub_rn(p[1], I[1]), rz = __dsub_rn(p[2], I[2]);
        const double vx = __dsub_rn(p[3], I[3]), vy = __dsub_rn(p[4], I[4]), vz = __dsub_rn(p[5], I[5]);
        const double sp = R.speed_from_velocity
                              ? __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(p[3], p[3]), __dmul_rn(p[4], p[4])),
                                                     __dmul_rn(p[5], p[5])))
                              : p[8];
        const double xv = dot_rn(R.XI, vx, vy, vz), yv = dot_rn(R.YI, vx, vy, vz);
        const double sp2 = __dmul_rn(sp, sp);
        double *o = out + j * 6;
        o[0] = dot_rn(R.XI, rx, ry, rz);
        o[1] = __ddiv_rn(xv, __dsqrt_rn(__dsub_rn(sp2, __dmul_rn(xv, xv))));
        o[2] = dot_rn(R.YI, rx, ry, rz);
        o[3] = __ddiv_rn(yv, __dsqrt_rn(__dsub_rn(sp2, __dmul_rn(yv, yv))));
        o[4] = dot_rn(R.ZI, rx, ry, rz);
        o[5] = __ddiv_rn(__dsub_rn(__dmul_rn(sp, p[6]), im), im);
    }
    if (!obj) return;
    __syncthreads();
    if (threadIdx.x != 0) return;
    // the statistics in list order, one thread (max / min are order-free; the sums are not)
    double wx = 0.0, wxp = 0.0, wy = 0.0, wyp = 0.0;
    NeumaierSum sx, sxp, sy, syp;
    double hx_max = 0.0, hx_min = 0.0, hy_max = 0.0, hy_min = 0.0;
    for (int64_t g = 0; g < n_p; g += R.group) {
        const int64_t e = min(n_p, g + (int64_t)R.group);
        double gx_max = 0.0, gx_min = 0.0, gy_max = 0.0, gy_min = 0.0;
        for (int64_t j = g; j < e; ++j) {
            const double *o = out + j * 6;
            const double x = __ddiv_rn(o[0], kMM), xp = __ddiv_rn(o[1], kMRAD);
            const double y = __ddiv_rn(o[2], kMM), yp = __ddiv_rn(o[3], kMRAD);
            if (j == 0) {
                wx = fabs(x), wxp = fabs(xp), wy = fabs(y), wyp = fabs(yp);
            } else {
                wx = nmax(wx, fabs(x)), wxp = nmax(wxp, fabs(xp)), wy = nmax(wy, fabs(y)), wyp = nmax(wyp, fabs(yp));
            }
            sx.add(x), sxp.add(xp), sy.add(y), syp.add(yp);
            if (j == g) {
                gx_max = gx_min = x, gy_max = gy_min = y;
            } else {
                gx_max = nmax(gx_max, x), gx_min = nmin(gx_min, x), gy_max = nmax(gy_max, y), gy_min = nmin(gy_min, y);
            }
        }
        const double hx = __ddiv_rn(__dsub_rn(gx_max, gx_min), 2.0), hy = __ddiv_rn(__dsub_rn(gy_max, gy_min), 2.0);
        if (g == 0) {
            hx_max = hx_min = hx, hy_max = hy_min = hy;
        } else {
            hx_max = nmax(hx_max, hx), hx_min = nmin(hx_min, hx), hy_max = nmax(hy_max, hy), hy_min = nmin(hy_min, hy);
        }
    }
    const double n = (double)n_p;
    double *ob = obj + d * CCT_BEAM_OBJECTIVES;
    ob[0] = wx;
    ob[1] = wxp;
    ob[2] = wy;
    ob[3] = wyp;
    ob[4] = fabs(__ddiv_rn(sx.total(), n));
    ob[5] = fabs(__ddiv_rn(sxp.total(), n));
    ob[6] = fabs(__ddiv_rn(sy.total(), n));
    ob[7] = fabs(__ddiv_rn(syp.total(), n));
    ob[8] = fabs(__dsub_rn(wx, wy));
    ob[9] = __dsub_rn(hx_max, hx_min);
    ob[10] = __dsub_rn(hy_max, hy_min);
}

}  // namespace cctgpu

using namespace cctgpu;

extern "C" int cct_beam_readout(const double *d_particles, int32_t n_designs, int64_t n_particles,
                                const double *h_ideal, const double *h_frame, int32_t group,
                                int32_t speed_from_velocity, double *d_phase_space, double *d_objectives,
                                void *stream) {
    clear_error();
    if (n_designs <= 0 || n_particles <= 0) return set_error(CCT_ERR_ARG, "need at least one design and particle");
    if (n_designs > 0x7fffffff / 2) return set_error(CCT_ERR_ARG, "too many designs (%d)", n_designs);
    if (!d_particles || !d_phase_space || !h_ideal || !h_frame)
        return set_error(CCT_ERR_ARG, "null particles, phase-space buffer, ideal particle or frame");
    if (d_objectives && group < 1) return set_error(CCT_ERR_ARG, "group size %d (must be >= 1)", group);
    ReadoutParams R;
    for (int i = 0; i < 10; ++i) R.ideal[i] = h_ideal[i];
    for (int i = 0; i < 3; ++i) {
        R.XI[i] = h_frame[i];
        R.YI[i] = h_frame[3 + i];
        R.ZI[i] = h_frame[6 + i];
    }
    R.group = group < 1 ? 1 : group;
    R.speed_from_velocity = speed_from_velocity != 0;
    readout_kernel<<<n_designs, kReadBlock, 0, static_cast<cudaStream_t>(stream)>>>(d_particles, n_particles, R,
                                                                                    d_phase_space, d_objectives);
    CCT_TRY_CUDA(cudaGetLastError());
    return CCT_OK;
}
