/*
 * seisfat2d.h - C ABI of the GB300 first-arrival traveltime engine.
 *
 * A drop-in for the fast-sweeping eikonal path of phbastosa/SeisFAT2D:
 * every entry point names the reference interface it replaces. Plain C: plain
 * pointers and sizes, int status codes, no exceptions cross the boundary.
 *
 * Grid conventions (the reference's, src/modeling/modeling.cu:3-36):
 *   model   nz x nx samples, z fastest: model[i + j*nz]
 *   padded  nzz = nz + 2*nb rows, nxx = nx + 2*nb columns, nb = 3,
 *           z fastest: T[i + j*nzz]; the pad replicates the edge samples
 *   shots   source (sx, sz) in metres from the model origin
 *
 * Threading: one context per host thread; contexts are independent.
 * Streams: `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 * Calls that take SF_MEM_HOST buffers synchronise the stream before returning.
 */
#ifndef SEISFAT2D_H
#define SEISFAT2D_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define SF_OK 0
#define SF_ERR_ARG 1     /* bad argument (null pointer, size, layout)        */
#define SF_ERR_CUDA 2    /* a CUDA runtime call or kernel launch failed      */
#define SF_ERR_TIMEOUT 3 /* a bounded in-kernel wait gave up (results void)  */
#define SF_ERR_RANGE 4   /* source or window outside the grid                */
#define SF_ERR_STATE 5   /* call out of order (e.g. adjoint without a tape)  */
#define SF_ERR_NOMEM 6   /* device allocation failed                          */

/* memory kinds for buffer arguments */
#define SF_MEM_HOST 0
#define SF_MEM_DEVICE 1

/* slowness layouts */
#define SF_LAYOUT_MODEL 0  /* nz x nx, expanded to the padded grid on device */
#define SF_LAYOUT_PADDED 1 /* nzz x nxx, taken as is                          */

/* arithmetic of the FP32 sweeps (sf_set_arithmetic) */
#define SF_ARITH_REFERENCE 0 /* the reference build's: FP32 init, nvcc's FMAs (default) */
#define SF_ARITH_IEEE 1      /* every operation rounded once, FP64 3x3 initialisation */
#define SF_ARITH_COMPENSATED 2 /* traveltimes carried as FP32 pairs hi + lo (see sf_set_arithmetic) */

/* strip-loop forms (sf_set_strip_loop) */
#define SF_LOOP_AUTO -1    /* interior-block body when all shots run at once, one window width, a warp per strip */
#define SF_LOOP_GENERAL 0  /* one loop body with bounds tests in every block            */
#define SF_LOOP_INTERIOR 1 /* blocks inside the window run a body without bounds tests   */

/* sf_batch_forward flags */
#define SF_KEEP_TAPE 1   /* record the update tape for sf_batch_adjoint      */
#define SF_KEEP_TABLES 2 /* keep every shot's traveltime window on device   */

typedef struct sf_ctx sf_ctx;

/* One shot of a batch. The solve runs on padded columns [c0, c0+ncols)
 * (ncols <= 0: the whole width), with that window's first and last columns
 * held fixed like the grid's outer ring. */
typedef struct {
    float sx, sz;
    int c0, ncols;
} sf_shot;

const char* sf_status_string(int status);
const char* sf_ctx_last_error(const sf_ctx* ctx);

/* Modeling::set_parameters (modeling.cu:3-36) + set_eikonal (:62-102):
 * grid sizes, spacing and device buffers. nb is fixed at 3. */
int sf_ctx_create(sf_ctx** out, int nx, int nz, float dx, float dz, int device);
int sf_ctx_destroy(sf_ctx* ctx);
int sf_ctx_dims(const sf_ctx* ctx, int* nxx, int* nzz, int* nb);

/* Modeling::set_properties + expand_boundary (modeling.cu:47-60, :204-232)
 * and copy_slowness_to_device (:281-284). */
int sf_set_slowness(sf_ctx* ctx, const float* s, int layout, int mem);
/* padded slowness back (nzz x nxx) */
int sf_get_slowness(sf_ctx* ctx, float* out, int mem);

/* Eikonal_ANI::set_conditions / set_stiffness_element (eikonal_ani.cu:3-31)
 * with Modeling::compression (modeling.cu:264-279): six nz x nx fields
 * C11,C13,C15,C33,C35,C55, padded and quantised to uint16 with a
 * deterministic min/max. */
int sf_set_stiffness(sf_ctx* ctx, const float* const cij[6], int mem);
/* Same with already quantised padded codes (nzz x nxx each) and their
 * (min, max) pairs, for inputs quantised elsewhere. */
int sf_set_stiffness_codes(sf_ctx* ctx, const uint16_t* const codes[6], const float minmax[12],
                           int mem);

/* Eikonal_ISO::time_propagation / Eikonal_ANI::time_propagation
 * (eikonal_iso.cu:9-12, eikonal_ani.cu:33-45): initialization() +
 * eikonal_solver() [+ get_quasi_slowness + second solve] for one source on
 * the whole padded grid. T receives nzz x nxx traveltimes. One CTA. */
int sf_time_propagation(sf_ctx* ctx, int ani, float sx, float sz, float* T, int T_mem,
                        void* stream);

/* Modeling::compute_seismogram (modeling.cu:161-194): 4x4 Catmull-Rom picks
 * of a padded traveltime field (device pointer, nzz x nxx) at nrec receivers
 * (host coordinates). Receivers whose stencil leaves the grid give NaN. */
int sf_compute_seismogram(sf_ctx* ctx, const float* T_dev, const float* rx, const float* rz,
                          int nrec, float* picks, int picks_mem, void* stream);

/* Batched forward: the shot loop of modeling_main.cpp:21-29 (and the
 * traveltime-table loops of migration.cu:116-171) in one persistent launch.
 * shots/rx/rz are host arrays; picks is nshots x nrec (shot-major).
 * ani = 1: three launches (eikonal_ani.cu:33-45): the solve of every shot on
 * S, the qP pass over every shot's window, the solve of every shot on its
 * qP slowness. Every shot then keeps its traveltime window and its qP
 * slowness window on the device (nzz x ncols floats each, a second
 * traveltime window in the compensated arithmetic, three factor windows
 * with SF_KEEP_TAPE), so device memory grows with the batch: split batches
 * whose windows exceed it (SF_ERR_CUDA when an allocation fails). */
int sf_batch_forward(sf_ctx* ctx, int ani, const sf_shot* shots, int nshots, const float* rx,
                     const float* rz, int nrec, float* picks, int picks_mem, int flags,
                     void* stream);

/* Traveltime window of shot `shot` of the last batch run with
 * SF_KEEP_TABLES: nzz x ncols values, z fastest. */
int sf_batch_table(sf_ctx* ctx, int shot, float* T, int mem, void* stream);

/* Adjoint-state gradient (no counterpart in the reference, whose tomography
 * traced rays on the host: inversion.cpp:95-177). Needs the last batch run
 * with SF_KEEP_TAPE. pick_grad: dJ/dpicks, nshots x nrec (NaN picks are
 * ignored); grad receives dJ/dS on the padded grid (nzz x nxx, overwritten). */
int sf_batch_adjoint(sf_ctx* ctx, const float* pick_grad, int pg_mem, float* grad, int grad_mem,
                     void* stream);

/* Branch codes of shot `shot` (caller order) of the last SF_KEEP_TAPE batch:
 * 4 x ncols x nzz bytes, [sweep][window column][row], one code per node and
 * sweep (bits 0-2: candidate 0 none/kept, 1 t1d1, 2 t1d2, 3 2D, 4 and 5 the
 * edge updates; bits 3-4: the slowness cell (i-1+b3, j-1+b4) that candidate
 * read). No counterpart in the reference: it lets a checker evaluate the same
 * branch pattern in FP64. Synchronises the stream. */
int sf_batch_tape_codes(sf_ctx* ctx, int shot, uint8_t* codes, int mem, void* stream);

/* Anisotropic batches (sf_batch_forward with ani = 1 and SF_KEEP_TAPE) tape
 * the second, qP solve. Their adjoint (sf_batch_adjoint or
 * sf_batch_misfit_gradient) multiplies each shot's gradient with respect to
 * its own qP slowness field by that field's derivatives, with the
 * propagation direction of the first solve held fixed (the first solve sees
 * S only, so the stiffness derivatives are exact): grad is then dJ/dS, and
 * sf_batch_stiffness_gradient gives dJ/dC11 and dJ/dC13 (padded grid, nzz x
 * nxx, z fastest) of the same adjoint. These are the three sensitivities
 * Tomography_VTI::set_sensitivity_matrix builds from rays
 * (src/inversion/tomography_vti.cpp:24-109) in the parameters the stiffness
 * enters through (dC11/depsilon = 2 C33; dC13/ddelta = C33 (C33 - C55) /
 * (C13 + C55) for VTI). SF_ERR_STATE unless the last adjoint was of an
 * anisotropic batch. */
int sf_batch_stiffness_gradient(sf_ctx* ctx, float* grad_c11, float* grad_c13, int mem, void* stream);

/* Misfit J = 1/2 sum (pick - t_obs)^2 over valid picks (FP64) and its
 * gradient dJ/dS, from the last SF_KEEP_TAPE batch. Replaces
 * Inversion::check_convergence + optimization (inversion.cpp:179-345). */
int sf_batch_misfit_gradient(sf_ctx* ctx, const float* t_obs, int obs_mem, double* misfit,
                             float* grad, int grad_mem, void* stream);

/* Waits for `stream` and reports in-kernel failures (SF_ERR_TIMEOUT). */
int sf_synchronize(sf_ctx* ctx, void* stream);

/* Failure detection (no counterpart in the reference, which checks no CUDA
 * errors). Every in-kernel wait (a strip waiting for the strip above it, a
 * gang barrier, a gather tile waiting for its shots) gives up after
 * `seconds` (0: the default of about 2 s; at most 60), raises the launch's
 * error flag and lets every other wait of the launch return at once, so the
 * kernel always finishes; the call that reads the flag returns
 * SF_ERR_TIMEOUT, the launch's results are void, and the context stays
 * usable. Applies to launches configured after the call. */
int sf_set_wait_limit(sf_ctx* ctx, double seconds);
/* Test of that path: in the next sf_batch_forward / sf_time_propagation
 * launch only, every strip waits for a handoff tag that no strip writes, so
 * each wait runs into the limit. Nothing else changes; later launches are
 * unaffected. */
int sf_test_stall_next_batch(sf_ctx* ctx);

/* FP32 arithmetic of the solves. SF_ARITH_REFERENCE reproduces the
 * reference build of inner_sweep/time_init (modeling.cu:293-357 compiled by
 * nvcc with its default FMA contraction): FP32 initialisation and fused
 * multiply-adds for t1d1, t1d2, the 2D numerator and the discriminant.
 * SF_ARITH_IEEE rounds every operation once and evaluates the 3x3
 * initialisation in FP64. SF_ARITH_COMPENSATED (no counterpart in the
 * reference) solves the same scheme with every traveltime carried as an
 * unevaluated FP32 pair hi + lo: the update's branch tests and increments
 * are formed from differences of the pairs and the winning candidate is
 * added to its base time with TwoSum, so rounding no longer accumulates
 * along a sweep (the FP32 field stays within about 1e-7 of an FP64 solve,
 * where the other two drift to about 1e-5, and the adjoint's coefficients,
 * which depend on differences of neighbouring times, follow). The
 * traveltimes callers see are the hi parts; tapes, picks and gradients keep
 * their formats. At most 8 warps per CTA (sf_set_launch). */
int sf_set_arithmetic(sf_ctx* ctx, int mode);
int sf_get_arithmetic(const sf_ctx* ctx, int* mode);

/* Per-shot solve that allocates nothing. No counterpart in the reference.
 * For callers that may not allocate device memory inside a call (hosts that
 * own all device memory through their own pool and forbid cudaMalloc/cudaFree
 * in plugin calls, latency-critical loops). Same result as
 * sf_time_propagation in the default (reference) arithmetic, isotropic.
 * S: padded slowness on the current device (nzz x nxx, nzz = nz+6, nxx =
 * nx+6); T: output on the current device (nzz x nxx). Scratch lives in one
 * static device array of about 8 MiB that every GPU loading the library
 * holds until exit: grids with ceil(nzz/32) * nxx > 262144 are rejected with
 * SF_ERR_RANGE. The first call on a device sets that device up (looks up the
 * array's device address, sets the kernel's shared-memory limit). The first
 * call with new cell sizes (dx, dz) on
 * a device also checks the node update's fast division for them, in the
 * array, and waits for that check. Calls share the array: calls that
 * overlap on the GPU (other streams, other threads) race and must be
 * serialised by the caller. Synchronises `stream`; returns SF_ERR_TIMEOUT
 * if an in-kernel wait gave up. */
int sf_time_propagation_noalloc(const float* S, int nx, int nz, float dx, float dz, float sx, float sz,
                                float* T, void* stream);

/* Launch shape. A shot is solved by a gang of CTAs whose warps each run
 * every k-th 32-row strip. warps: warps per CTA (1..16; 0 keeps the current
 * value, default 1); gang_warps: warps per shot (0: chosen per batch so that
 * all shots of the batch are resident at once when possible). */
int sf_set_launch(sf_ctx* ctx, int warps, int gang_warps);
int sf_get_launch(const sf_ctx* ctx, int* warps, int* gang_warps);

/* Form of the strip loops of the forward and reverse sweeps (no counterpart
 * in the reference). Both forms compute the same bits; the interior-block
 * form runs fewer instructions per step but is larger code, which measured
 * faster for a batch whose shots all run at once with one window width and
 * one warp per strip, slower for uneven windows or several strips per warp.
 * SF_LOOP_AUTO (default) chooses per batch (taped batches with more than 8
 * warps per CTA always run the general form);
 * sf_plan_autotune times both. last_interior: whether the last batch's
 * forward used the interior-block form (the reverse sweeps follow it). */
int sf_set_strip_loop(sf_ctx* ctx, int mode);
int sf_get_strip_loop(const sf_ctx* ctx, int* mode, int* last_interior);

/* Gradient gather inside the reverse-sweep launch (no counterpart in the
 * reference; default on). With 2 or 4 warps per CTA and an isotropic batch,
 * and when the device holds every reverse-sweep CTA plus gather CTAs at
 * once, one launch runs both: each gather tile starts as soon as every shot's
 * last reverse sweep has finished its columns in the tile's strip and the
 * next, instead of after the whole reverse pass. Same bits either way.
 * last_fused: whether the last adjoint ran fused. */
int sf_set_fused_gather(sf_ctx* ctx, int enable);
int sf_get_fused_gather(const sf_ctx* ctx, int* enable, int* last_fused);

/* ---- planned batches, CUDA graphs, autotuner (no counterpart in the
 * reference, which solves one shot per call: inversion.cpp:52-67 and
 * migration.cu:116-171 loop over time_propagation) ----
 *
 * sf_plan_batch fixes a batch on the context: isotropic shots (windows as in
 * sf_batch_forward) and receivers are uploaded once and every buffer a
 * forward + adjoint iteration needs is reserved, so that sf_plan_iteration
 * only enqueues device work on `stream` (no allocation, no host copy, no
 * synchronisation); it zeroes the handoff buffers of its two persistent
 * kernels first, so it may be captured into a CUDA graph by the caller and
 * replayed any number of times.
 * Synchronises `stream` once. Any other batch call on the context (or
 * sf_time_propagation) ends the plan; sf_set_launch / sf_set_arithmetic make
 * the next iteration reconfigure it (outside a capture).
 *
 * One iteration, device pointers only: the taped forward of every shot with
 * its picks (picks, nshots x nrec, caller order); then, when t_obs is not
 * null, the residuals picks - t_obs (NaN = no pick), the misfit
 * 1/2 sum r^2 in FP64 (misfit: one device double, may be null), the reverse
 * sweeps and the deterministic gather of dJ/dS into grad (padded nxx x nzz,
 * overwritten). Errors of in-kernel waits surface at sf_synchronize. */
int sf_plan_batch(sf_ctx* ctx, const sf_shot* shots, int nshots, const float* rx, const float* rz,
                  int nrec, void* stream);
int sf_plan_iteration(sf_ctx* ctx, const float* t_obs, float* picks, double* misfit, float* grad,
                      void* stream);
/* The same iteration from a CUDA graph the context owns: captured on first use
 * (and again when the pointers or the plan's launch shape change), then
 * replayed with cudaGraphLaunch on `stream`. */
int sf_plan_graph_launch(sf_ctx* ctx, const float* t_obs, float* picks, double* misfit, float* grad,
                         void* stream);
/* Autotuner: times `reps` iterations of the plan for each candidate launch
 * shape (1, 2, 4 warps per CTA x automatic, all, 1/2, 1/3, 1/4 of the strips
 * per gang; under SF_LOOP_AUTO also both strip-loop forms), keeps the fastest
 * (as sf_set_launch and sf_set_strip_loop would) and reports its launch
 * shape. Every shape computes the same bits. Synchronises `stream`. */
int sf_plan_autotune(sf_ctx* ctx, const float* t_obs, float* picks, double* misfit, float* grad, int reps,
                     void* stream, int* best_warps, int* best_gang_warps, float* best_ms);

/* Per-kernel device times: with timing on, CUDA events are recorded around
 * each launch of the batched kernels on the call's stream (not inside graph
 * captures). sf_kernel_times writes, for the latest launch of each kernel
 * since the previous query, its time in ms (-1: not launched), waiting for
 * it: ms[0] forward (k_shots), ms[1] pick residuals, ms[2] reverse sweeps
 * (k_adjoint), ms[3] gradient gather. */
int sf_set_kernel_timing(sf_ctx* ctx, int enable);
int sf_kernel_times(sf_ctx* ctx, float* ms, int n);

/* ---- tomography model update (src/inversion/inversion.cpp:347-447,
 * src/inversion/tomography_iso.cpp:77-92) ----
 *
 * sf_smooth_model: the reference's Inversion::model_smoothing of a model-sized
 * field (nz x nx, z fastest; in and out host or device per `mem`, distinct):
 * zero padding of `samples` cells, normalised Gaussian taps 1/(pi stdv)
 * exp(-r^2/(2 stdv^2)) over samples x samples cells (stdv 0: identity),
 * FP32 products summed in the reference's tap order. samples must be odd
 * (the reference indexes past its kernel for even counts); with host memory
 * the call synchronises `stream`.
 *
 * sf_update_slowness: Tomography_ISO::model_update on the context's slowness:
 * dS = scale * grad over the model interior of a padded gradient (as from
 * sf_batch_misfit_gradient; grad_mem says where it is), smoothed as above
 * unless samples is 0, then S += dS on the interior (the pad ring keeps its
 * values, as in the reference). dS (model-sized, may be null) receives the
 * applied update. Synchronises `stream`. */
int sf_smooth_model(sf_ctx* ctx, const float* in, float* out, float stdv, int samples, int mem, void* stream);
int sf_update_slowness(sf_ctx* ctx, const float* grad, int grad_mem, float scale, float stdv, int samples,
                       float* dS, int dS_mem, void* stream);

/* ---- Kirchhoff depth migration, image domain (src/migration/KDM.cu:3-55,
 * IDKDM.cu:19-22, migration.cu:54-71, :173-228, :398-483) ----
 *
 * sf_adjoint_convolution: Migration::adjoint_convolution of ntr traces of nt
 * samples (trace-major, host or device per `mem`): cross-correlation with the
 * reference's wavelet for max_frequency fmax (Migration::set_wavelet), as
 * its FFTW product A*conj(B) and unnormalised inverse give it (scaled by the
 * FFT length), shifted by nw/2 + nw/10 samples; earlier samples are 0.
 * Computed directly in FP64 and rounded once to FP32.
 *
 * sf_kirchhoff_image: the image (nz x nx, z fastest; host or device per
 * image_mem) = sum over sources s and receivers r with |xsrc[s] - xrec[r]| <
 * max_offset, in that order, of the reference's image-domain weight times
 * the correlated trace sample at t = Ts + Tr (data: nsrc x nrec x nt, host or
 * device per data_mem). Ts and Tr are device arrays of nsrc and nrec padded
 * traveltime tables (nzz x nxx each, as sf_batch_table writes them); the
 * context's slowness is the model. The reference sums the traces with one
 * launch and one atomicAdd per trace; this is one launch that sums each
 * cell's terms in the same order. Host outputs synchronise `stream`. */
int sf_adjoint_convolution(sf_ctx* ctx, const float* traces, float* out, int ntr, int nt, float dt, float fmax,
                           int mem, void* stream);
int sf_kirchhoff_image(sf_ctx* ctx, const float* Ts, const float* Tr, int nsrc, int nrec, const float* xsrc,
                       const float* xrec, const float* data, int data_mem, int nt, float dt, float aperture,
                       float max_offset, float* image, int image_mem, void* stream);

/* Angle-domain Kirchhoff migration (the reference's ADKDM: KDM.cu:3-55 with
 * angle_domain_adjoint_kernel, migration.cu:572-663; bins of
 * Migration::set_gathers, migration.cu:73-97): gathers (nz x nang x ncmp,
 * z fastest, then angle, then CMP bin) of the same trace terms as
 * sf_kirchhoff_image, each added to the bin of its trace's midpoint
 * ((xsrc + xrec)/2 from the smallest midpoint in steps of half the smaller
 * first source / receiver spacing) and of its reflection angle (steps of
 * da up to max_angle). The reference adds with atomics from all columns at
 * once; here each (depth, CMP) bin sums its traces in trace order and each
 * trace's cells left to right, so bins agree with the reference to rounding.
 * With gathers null the call only reports nang and ncmp. At most 256 angle
 * bins. Host outputs synchronise `stream`. */
int sf_kirchhoff_angle_gathers(sf_ctx* ctx, const float* Ts, const float* Tr, int nsrc, int nrec,
                               const float* xsrc, const float* xrec, const float* data, int data_mem, int nt,
                               float dt, float aperture, float max_offset, float max_angle, float da,
                               float* gathers, int gathers_mem, int* nang, int* ncmp, void* stream);

/* ---- Least-squares Kirchhoff migration's operators (the reference's IDLSKDM
 * and ADLSKDM: LSKDM.cu:3-245 driving IDLSKDM.cu:24-37 / ADLSKDM.cu:43-59;
 * kernels image_domain_forward_kernel, migration.cu:485-570, and
 * angle_domain_forward_kernel, :665-756; Migration::forward_convolution,
 * :230-261). The adjoints are sf_kirchhoff_image and
 * sf_kirchhoff_angle_gathers with sf_adjoint_convolution. ----
 *
 * sf_forward_convolution: convolution of ntr traces of nt samples with the
 * reference's wavelet for fmax, as its FFTW product A*B and unnormalised
 * inverse give it (scaled by the FFT length), output sample t taken from
 * t + nw/2 + nw/10. Computed directly in FP64 and rounded once to FP32.
 *
 * sf_kirchhoff_image_forward: traces (nsrc x nrec x nt, host or device per
 * data_mem) from an image (nz x nx, z fastest, per image_mem): for each pair
 * with |xsrc - xrec| < max_offset, each image cell adds its image-domain
 * weight times its value to sample floor((Ts + Tr)/dt) when that is below nt;
 * the other traces are 0. The reference adds with one atomicAdd per cell and
 * launch; here each trace's terms are summed in a fixed order that depends on
 * the sizes only, so results agree with the reference to rounding and repeat
 * bit for bit. Tables as for sf_kirchhoff_image. At most about 51,000 time
 * samples (SF_ERR_RANGE beyond).
 *
 * sf_kirchhoff_angle_forward: the same from angle gathers (nz x nang x ncmp,
 * bins as sf_kirchhoff_angle_gathers): each cell reads the gather of its
 * trace's CMP bin at its depth and reflection-angle bin.
 *
 * Host outputs synchronise `stream`. */
int sf_forward_convolution(sf_ctx* ctx, const float* traces, float* out, int ntr, int nt, float dt, float fmax,
                           int mem, void* stream);
int sf_kirchhoff_image_forward(sf_ctx* ctx, const float* Ts, const float* Tr, int nsrc, int nrec, const float* xsrc,
                               const float* xrec, const float* image, int image_mem, int nt, float dt,
                               float aperture, float max_offset, float* data, int data_mem, void* stream);
int sf_kirchhoff_angle_forward(sf_ctx* ctx, const float* Ts, const float* Tr, int nsrc, int nrec, const float* xsrc,
                               const float* xrec, const float* gathers, int gathers_mem, int nt, float dt,
                               float aperture, float max_offset, float max_angle, float da, float* data,
                               int data_mem, void* stream);

#ifdef __cplusplus
}
#endif
#endif
