/*
 * cctgpu.h -- C ABI of the GB300 (sm_103a) Biot-Savart / RK4 tracking engine
 * for CCT (canted-cosine-theta) magnet beamlines.
 *
 * Every entry point takes plain pointers and sizes, returns a cct_status, and
 * records a message retrievable with cct_last_error().  Pointers named d_* are
 * device pointers (any allocator: cudaMalloc, torch, ...); pointers named h_*
 * are host pointers.  `stream` is a cudaStream_t passed as void* (NULL = the
 * legacy default stream).  Calls are asynchronous on `stream` unless stated.
 *
 * Data layouts (all little-endian, C order):
 *   segments   d_kls[n_seg*3], d_p0s[n_seg*3]  -- per straight current element,
 *              kl = 1e-7 * I * (p[i+1]-p[i]) and p0 = (p[i+1]+p[i])/2 in the
 *              GLOBAL frame, FP64, xyz interleaved: exactly the two flat arrays
 *              of CCT.global_current_elements_and_elementary_current_positions
 *              (cctpy final_code/packages/cct.py:434-457).  Several designs
 *              are concatenated; d_seg_off[n_designs+1] (int64, device) gives
 *              each design's first segment.
 *   QS         d_qs[n_qs*16], FP64: origin, XI, YI, ZI, length, gradient,
 *              second gradient, aperture radius -- QS.to_numpy_array
 *              (cctpy final_code/packages/magnets.py:726-748); a Q is a QS
 *              without second gradient.  The same records also carry the
 *              straight dipole (LocalUniformMagnet, magnets.py:440-481) as
 *              origin, XI, YI, ZI, -length, field (T, along YI), 0, aperture
 *              radius -- a negative length marks it -- and the uniform field
 *              (UniformMagnet, :417-437) as length -inf with the field along
 *              YI.  Per design ranges in d_qs_off[n_designs+1].  Wires and
 *              AG-CCT connectors (cct.py:625-994) are current elements: their
 *              kl/p0 go into the segment arrays like a CCT's.
 *   points     d_points[n*3] FP64 global xyz; fields d_B[n*3] FP64 tesla.
 *   particles  d_particles[n_designs*n_particles*10] FP64 records
 *              (px,py,pz,vx,vy,vz,relativistic mass,charge,speed,distance),
 *              RunningParticle.to_numpy_array_data (cctpy particles.py:443-457).
 */
#ifndef CCTGPU_H
#define CCTGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    CCT_OK = 0,
    CCT_ERR_ARG = 1,         /* bad size, pointer or alignment (ValueError in Python) */
    CCT_ERR_CUDA = 2,        /* a CUDA runtime call or launch failed */
    CCT_ERR_TIMEOUT = 3,     /* a bounded device-side wait gave up */
    CCT_ERR_NONFINITE = 4,   /* a particle state became NaN/Inf */
    CCT_ERR_UNSUPPORTED = 5  /* device or configuration not supported */
} cct_status;

/* Library version (major*10000 + minor*100 + patch). */
int cct_version(void);

/* Copies the last error message of the calling thread into buf (NUL
 * terminated, truncated to n bytes).  Returns the last status code. */
int cct_last_error(char *buf, size_t n);

/* Tile length (segments) of the FP32-compensated packed form. */
int cct_f32c_tile(void);

/* ---------------------------------------------------------------------------
 * Field at points.
 * Replaces the per-point CPU sum CCT.magnetic_field_at (cct.py:249-285) summed
 * over a beamline (Beamline.magnetic_field_at, beamline.py:46-53) and the
 * block-per-point CUDA kernels current_element_B / magnet_with_multi_qs
 * (gpu_accelerator.py:363-383, :512-526).  B = sum over segments of
 * kl x r / |r|^3 (r = point - p0) plus the analytic QS field of every QS.
 * ------------------------------------------------------------------------- */

/* Plain FP64 form (the drop-in). */
int cct_field_f64(const double *d_kls, const double *d_p0s, int64_t n_seg,
                  const double *d_qs, int32_t n_qs,
                  const double *d_points, int64_t n_points, double *d_B,
                  void *stream);

/* FP32-compensated form: segments re-packed once into tiles of
 * cct_f32c_tile() segments, each with a double-float origin and FP32 offsets;
 * point - origin is taken in double-float, the pair terms run in packed FP32,
 * and the sum is Kahan-compensated in FP32 and resolved in FP64 (<= 1e-7
 * relative inside the magnets).  `packed` must be 256-byte aligned and hold
 * cct_f32c_packed_bytes() bytes. */
int64_t cct_f32c_packed_bytes(const int64_t *h_seg_off, int32_t n_designs);
int cct_f32c_pack(const double *d_kls, const double *d_p0s,
                  const int64_t *h_seg_off, int32_t n_designs,
                  void *d_packed, int64_t packed_bytes, void *stream);
int cct_field_f32c(const void *d_packed, int32_t design,
                   const double *d_qs, int32_t n_qs,
                   const double *d_points, int64_t n_points, double *d_B,
                   void *stream);

/* Status the cct_field_f32c kernels of the current device (every stream) have
 * recorded since the last call, which clears it: CCT_OK; CCT_ERR_ARG if a
 * call was given a buffer that is not a packed set, or a design index the set
 * does not hold; CCT_ERR_TIMEOUT if a tile copy did not land within the wait
 * limit.  The fields of such a call are NaN.  Waits for `stream`.  No
 * counterpart in the reference (its kernels have no such failure). */
int cct_field_status(void *stream);

/* Host-buffer convenience form of cct_field_f64 / cct_field_f32c used as the
 * end-to-end call: copies h_kls/h_p0s/h_points to the device, evaluates, and
 * copies B back; synchronous.  precision: 0 = FP64, 1 = FP32-compensated.
 * Allocates device memory internally. */
int cct_field_host(const double *h_kls, const double *h_p0s, int64_t n_seg,
                   const double *h_qs, int32_t n_qs,
                   const double *h_points, int64_t n_points, double *h_B,
                   int32_t precision);

/* ---------------------------------------------------------------------------
 * Batched RK4 tracking of n_particles protons through each of n_designs
 * beamlines (particles of design d at d_particles + d*n_particles*10; updated
 * in place).  Replaces ParticleRunner.run_only (particles.py:562-632, RK4 of
 * base_utils.py:264-311) and the GPU tracking kernels
 * track_multi_particle_beamline_for_magnet_with_multi_qs
 * (gpu_accelerator.py:1044-1063, host wrapper :1912-2044).  Step semantics
 * follow the CPU reference: dt = footstep/speed, t_end = distance/speed,
 * steps = ceil(t_end/dt), dt := t_end/steps, Y' = [v, (e/m) v x B(p)],
 * distance += `distance`.
 *
 * One cooperative persistent launch; CTAs take (design, particle block,
 * segment chunk) units from a work counter.  With 8 or more particle blocks
 * each block advances stage by stage as soon as its own units are done
 * (bounded waits on per-block counters); FP32c batches of at most 64
 * particles in fewer blocks keep one unit per CTA and a copy of every
 * particle's state in each CTA, summing fields in fixed-point integers and
 * waiting (bounded) on per-group unit counters between stages; other smaller
 * batches meet at bounded grid barriers between RK4 stages.  Results do not
 * depend on which CTA ran which unit.  Needs caller-provided device scratch of
 * cct_track_scratch_bytes() bytes (256-byte aligned); a smaller buffer is
 * accepted down to the particle state plus one chunk per (design, particle
 * block), the work then being cut into fewer, larger units.  Returns
 * CCT_ERR_TIMEOUT if a wait gives up and CCT_ERR_NONFINITE if a particle
 * state became non-finite or needs 5e8 or more steps (those particles are
 * still written).
 * Synchronous (reads the device status word before returning).
 * precision: 0 = FP64 (d_kls/d_p0s used), 1 = FP32-compensated (d_packed
 * used, built by cct_f32c_pack with the same design offsets).
 * ------------------------------------------------------------------------- */
int64_t cct_track_scratch_bytes(int32_t n_designs, int64_t n_particles);
int cct_track(const double *d_kls, const double *d_p0s, const int64_t *d_seg_off,
              const void *d_packed,
              const double *d_qs, const int64_t *d_qs_off, int32_t n_designs,
              double *d_particles, int64_t n_particles,
              double distance, double footstep, int32_t precision,
              void *d_scratch, int64_t scratch_bytes, void *stream);

/* Asynchronous form of cct_track, for pipelines and CUDA-graph capture: the
 * same arguments and results, but nothing is read back to the host.  A
 * one-thread kernel checks the segment offsets and the packed set and plans
 * the units on the device, then the tracking kernel is launched cooperatively
 * (cudaLaunchKernelEx); both are ordinary stream work, so the call can be
 * captured into a graph and replayed (the inputs are read at replay time).
 * The status stays in the scratch: cct_track_status(d_scratch, stream)
 * synchronises `stream` and returns CCT_OK, CCT_ERR_ARG (inputs rejected by
 * the plan), CCT_ERR_TIMEOUT or CCT_ERR_NONFINITE.  The first call on a
 * device queries its occupancy; make it before any capture.  No counterpart in
 * the reference, whose GPU calls are synchronous. */
int cct_track_async(const double *d_kls, const double *d_p0s,
                    const int64_t *d_seg_off, const void *d_packed,
                    const double *d_qs, const int64_t *d_qs_off,
                    int32_t n_designs, double *d_particles, int64_t n_particles,
                    double distance, double footstep, int32_t precision,
                    void *d_scratch, int64_t scratch_bytes, void *stream);
int cct_track_status(const void *d_scratch, void *stream);

/* Work split of the tracking kernels, process-wide:
 *  - units of (design, particle block, segment chunk) per CTA and RK4 stage
 *    (default 8; 1..64, 0 restores the default);
 *  - the FP32c particle block: particles whose field sums a unit computes
 *    together (16, 32, 64, 128 or 256; 0 = automatic: 16 for designs of at most
 *    16 particles, else the power of two from 32 that needs the fewest particle
 *    slots, the largest of those).  FP64 tracking uses blocks of 16 for designs
 *    of at most 16 particles and blocks of 32 otherwise, whatever the setting,
 *    and cct_track_adjoint the automatic choice from 32 up.
 * cct_autotune times a few RK4 steps of the caller's problem (`steps` steps of
 * `footstep`, on a copy of d_particles, which is not modified) for every
 * particle block from the automatic one up to the first that holds all of a
 * design's particles (FP32c) and 2, 4, 8, 16 and 32 units per CTA, keeps the
 * fastest pair as the process-wide setting and returns its units per CTA
 * (cct_track_particle_block() then gives its particle block); it needs
 * cct_autotune_scratch_bytes() of scratch.  Stands in for the reference's
 * block_dim_x choice (GPU_ACCELERATOR(block_dim_x=...),
 * gpu_accelerator.py:54-96), which the caller sets by hand.  Synchronous. */
int cct_track_set_units_per_cta(int32_t units_per_cta);
int32_t cct_track_units_per_cta(void);
int cct_track_set_particle_block(int32_t particles);
int32_t cct_track_particle_block(void);
int64_t cct_autotune_scratch_bytes(int32_t n_designs, int64_t n_particles);
int cct_autotune(const double *d_kls, const double *d_p0s,
                 const int64_t *d_seg_off, const void *d_packed,
                 const double *d_qs, const int64_t *d_qs_off,
                 int32_t n_designs, const double *d_particles,
                 int64_t n_particles, double footstep, int32_t precision,
                 int32_t steps, void *d_scratch, int64_t scratch_bytes,
                 int32_t *units_per_cta_out, void *stream);

/* ---------------------------------------------------------------------------
 * Adjoint (gradients): no counterpart in the reference, which has no
 * derivatives; it differentiates cct_track's FP64 forward (the reference's RK4
 * with the midpoint Biot-Savart field, particles.py:515-596, cct.py:249-285).
 * Objective per design d over its particles' final positions p_i, with the
 * exit frame d_exit_frame[9*d..] = (o, XI, YI) of the ideal particle:
 *   J_d = mean_i (x_i^2 + y_i^2),  x_i = XI.(p_i - o),  y_i = YI.(p_i - o)
 * (RMS spot size squared plus centroid squared, both planes).  Writes J_d to
 * d_J[d] and dJ_d/d(kl_i) (3), dJ_d/d(p0_i) (3) of every segment i of design d
 * to d_seg_grad[6*i..] (the caller maps them to design parameters through the
 * segment-generation Jacobian).  Discrete adjoint of the exact RK4 map, with
 * the state checkpointed every `checkpoint_steps` steps and each segment of
 * steps recomputed once.  Particles are tracked as by cct_track with the
 * same precision (0 = FP64 with d_kls/d_p0s, 1 = FP32-compensated with
 * d_packed; the adjoint sweeps run in that precision) and their final records
 * are written to d_particles.  Scratch: at least
 * cct_adjoint_scratch_bytes(n_designs, n_particles, steps, checkpoint_steps)
 * bytes, `steps` an upper bound of any particle's step count.  Synchronous. */
int64_t cct_adjoint_scratch_bytes(int32_t n_designs, int64_t n_particles,
                                  int32_t max_steps, int32_t checkpoint_steps);
int cct_track_adjoint(const double *d_kls, const double *d_p0s,
                      const int64_t *d_seg_off, const void *d_packed,
                      const double *d_qs, const int64_t *d_qs_off,
                      int32_t n_designs, double *d_particles,
                      int64_t n_particles, double distance, double footstep,
                      int32_t precision, const double *d_exit_frame, double *d_J,
                      double *d_seg_grad, int32_t checkpoint_steps,
                      void *d_scratch, int64_t scratch_bytes, void *stream);

/* cct_track without any device allocation, for callers that may not allocate
 * device memory once running (memory reserved up front by a host application;
 * a C caller that owns only the buffers it passes).  No counterpart in the
 * reference: cctpy's GPU path allocates and copies on every call.  The scratch
 * is a fixed device array inside the library, held on each GPU until the
 * process exits; its size, cct_track_static_scratch_bytes() = 32 MiB, bounds
 * the problem (for example 64 designs x 512 protons, or one design x 100 000
 * protons), and at most 64 designs are taken.  Larger problems return
 * CCT_ERR_ARG with the size they need; use cct_track with a caller buffer for
 * them.
 * The array takes its device memory when the CUDA module holding it is loaded
 * on a device, which under lazy module loading (the CUDA default) is its first
 * use there, not the loading of the library.  Place it at start-up, before the
 * application reserves its memory: call cct_track_static_scratch_bytes() with
 * each device current once (with a device visible it looks the array up on the
 * current device, which loads the module), or make the first
 * cct_track_static_scratch call on each device then.  That first lookup on a
 * device records the array's address for the life of the process; make it
 * before any stream capture, and do not use this entry point on a device
 * after cudaDeviceReset on it.  Every call shares the array: calls whose
 * kernels overlap on the GPU (other streams, other host threads) race and must
 * be serialised by the caller.  Synchronous: like cct_track it reads the
 * segment offsets back and waits for `stream` before returning.  Same
 * arguments, results and status codes as cct_track otherwise; no
 * cudaMalloc/cudaFree is made. */
int64_t cct_track_static_scratch_bytes(void);
int cct_track_static_scratch(const double *d_kls, const double *d_p0s,
                             const int64_t *d_seg_off, const void *d_packed,
                             const double *d_qs, const int64_t *d_qs_off,
                             int32_t n_designs, double *d_particles,
                             int64_t n_particles, double distance, double footstep,
                             int32_t precision, void *stream);

/* ---------------------------------------------------------------------------
 * Device-side segment generation.  Replaces the host loop of the CCT
 * constructor and its global export (cct.py:87-164 with phi_ksi_function
 * :166-188 and BipolarToroidalCoordinateSystem.convert :213-224; export
 * :423-457), which the reference runs in Python for every design on every GPU
 * call.  A layer is described by one record of CCT_LAYER_DOUBLES doubles:
 *   [0..2]  origin, [3..5] XI, [6..8] YI, [9..11] ZI of its local frame
 *   [12] big_r  [13] small_r  [14] current (A)
 *   [15] xi start  [16] phi start  [17] xi end  [18] phi end
 *        (starting/end_point_in_ksi_phi_coordinate)
 *   [19] winding number  [20] segments per winding
 *   [21] number of tilt angles (0..CCT_LAYER_MAX_TILTS)
 *   [22..29] tilt angles in degrees
 *   [30] index of the layer's first segment in d_kls / d_p0s  [31] unused (0)
 * Layer l owns winding_number * segments_per_winding segments from its first
 * one on; layers must not overlap, and segments no layer covers (a wire's or a
 * connector's current elements, filled by the caller) are left untouched.
 * Values agree with the host construction to rounding of the trigonometric
 * functions (winding points within about 2e-14 m).  Both calls read the records
 * back to check them (CCT_ERR_ARG on a bad record, overlapping layers, or a
 * layer reaching past n_seg) and are synchronous.
 * ------------------------------------------------------------------------- */
#define CCT_LAYER_DOUBLES 32
#define CCT_LAYER_MAX_TILTS 8
#define CCT_LAYER_PARAMS 10

/* End (one past the last segment) of the furthest of the host layer records;
 * -1 and an error on a bad record or overlapping layers. */
int64_t cct_layer_segments(const double *h_layers, int32_t n_layers);

/* Writes d_kls[n_seg*3], d_p0s[n_seg*3] (global frame, FP64) of the layers in
 * d_layers[n_layers*CCT_LAYER_DOUBLES]. */
int cct_segments_build(const double *d_layers, int32_t n_layers, double *d_kls,
                       double *d_p0s, int64_t n_seg, void *stream);

/* Maps a segment gradient d_seg_grad[n_seg*6] (dJ/dkl, dJ/dp0 as written by
 * cct_track_adjoint) to d_param_grad[n_layers*CCT_LAYER_PARAMS] =
 * dJ/d(tilt angle 0..7 [per degree], current [per A], big_r [per m]) of every
 * layer (tilts past the layer's count are 0), by forward-mode derivatives of
 * the segment construction; the frame, small_r and xi/phi ends are held fixed.
 * No counterpart in the reference (it has no derivatives). */
int cct_segments_param_grad(const double *d_layers, int32_t n_layers,
                            const double *d_seg_grad, int64_t n_seg,
                            double *d_param_grad, void *stream);

/* ---------------------------------------------------------------------------
 * Optimiser read-out.  Replaces the host loop of the reference's optimiser run
 * script over every design's tracked protons (final_code/work/optim/
 * A05run.py:247-330): PhaseSpaceParticle.create_from_running_particles
 * (particles.py:1078-1138) and the BaseUtils.Statistic objectives
 * (base_utils.py:603-683).  d_particles[n_designs*n_particles*10] are tracked
 * records (as cct_track leaves them); h_ideal[10] is the ideal particle at the
 * exit and h_frame[9] its natural frame (XI, YI, ZI).  Writes the phase space
 * (x, x', y, y', z, delta) of every particle to d_phase_space[...*6]
 * (required) and, if d_objectives is not NULL, CCT_BEAM_OBJECTIVES values per
 * design: max|x|, max|x'|, max|y|, max|y'| (mm, mrad), |mean| of the same four,
 * |max|x| - max|y||, and the spread (max - min) of the half widths in x and in
 * y of consecutive groups of `group` particles.  speed_from_velocity != 0
 * first sets each speed to |v| (A05run.py:265-267).  Values are bit-identical
 * to the reference's (means: CPython 3.12+'s compensated float sum, in list
 * order).  Asynchronous on `stream`. */
#define CCT_BEAM_OBJECTIVES 11
int cct_beam_readout(const double *d_particles, int32_t n_designs,
                     int64_t n_particles, const double *h_ideal,
                     const double *h_frame, int32_t group,
                     int32_t speed_from_velocity, double *d_phase_space,
                     double *d_objectives, void *stream);

/* Measures the device's fused multiply-add pipe peak (flop/s, 2 per FMA) with
 * independent FMA chains on every SM: kind 0 = scalar FP32, 1 = FP64, 2 = packed
 * FP32x2.  These are the roofline denominators of the field kernels.
 * Synchronous. */
int cct_probe_fma_peak(int kind, double *flops_per_s);

/* Test hook for failure detection without a GPU fault: makes every tracking
 * grid barrier expect `phantom_blocks` extra CTAs that never arrive, and sets
 * the barrier wait limit to `wait_ms` (<= 0 restores the 60 s default).  A
 * tracking call then returns CCT_ERR_TIMEOUT after about wait_ms and the
 * context stays usable.  Process-wide; not for production use. */
int cct_test_set_barrier_fault(int phantom_blocks, int wait_ms);

/* Test hook for the dataflow schedule (batches of 8 or more particle blocks)
 * and the small-batch schedule (FP32c, at most 64 particles): every wait of a
 * unit for its particle block, or of a CTA for a stage's unit count, then
 * requires `stages_ahead` more finished stages than it needs, so with
 * stages_ahead >= 1 the first waits never end; the wait limit becomes
 * `wait_ms` (<= 0 restores the 60 s default).  A tracking call then returns CCT_ERR_TIMEOUT after about
 * wait_ms and the context stays usable.  No counterpart in the reference.
 * Process-wide; not for production use. */
int cct_test_set_flow_fault(int stages_ahead, int wait_ms);

/* Test hook: the work split cct_track plans, computed on the host for a grid
 * of `grid` CTAs (no device needed).  Writes the particle block size to
 * *group and, per design d, unit_off[d] (first unit; unit_off[n_designs] =
 * total), chunks[d] (segment chunks per particle block) and chunk_tiles[d]
 * (tiles of 128 segments per chunk).  max_units <= 0 takes the bound that
 * cct_track_scratch_bytes sizes for (units per CTA x grid, plus one chunk
 * per design and particle block).  Returns the unit count, -1 if one chunk
 * per (design, block) is more than max_units, -2 on bad arguments.  No
 * counterpart in the reference. */
int64_t cct_test_plan_units(const int64_t *seg_off, int32_t n_designs,
                            int64_t n_particles, int32_t precision,
                            int32_t grid, int64_t max_units,
                            int64_t *unit_off, int64_t *chunks,
                            int64_t *chunk_tiles, int32_t *group);

#ifdef __cplusplus
}
#endif
#endif /* CCTGPU_H */
