/*
 * CPU oracle for the SeisFAT2D fast-sweeping eikonal path.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker: tests/, the smoke entry and the
 * bench's CPU-baseline leg call it; the product path never does.
 *
 * It restates the reference's arithmetic (phbastosa/SeisFAT2D):
 *   src/modeling/modeling.cu:204-232  expand_boundary (edge-replicated pad)
 *   src/modeling/modeling.cu:104-121  source index and initialisation
 *   src/modeling/modeling.cu:123-159  eikonal_solver launch schedule (4 sweeps)
 *   src/modeling/modeling.cu:286-357  time_set / time_init / inner_sweep
 *   src/modeling/modeling.cu:264-279  compression (uint16 Cij quantisation)
 *   src/modeling/eikonal_ani.cu:33-111 two-pass anisotropic solve, qP slowness
 *   src/modeling/modeling.cu:161-194 + src/admin/admin.cpp:121-133  picks
 *
 * FP32 mode evaluates every operation with one IEEE rounding in the order the
 * reference source writes it (the library builds this file with
 * -ffp-contract=off). The 3x3 near-source initialisation is evaluated in FP64
 * and rounded once to FP32, in every mode.
 */
#ifndef SF_EIKONAL_ORACLE_H
#define SF_EIKONAL_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Pad an nz x nx (z fastest) field by nb cells on every side, replicating edges. */
void orc_expand_boundary(const float* in, int nx, int nz, int nb, float* out);
void orc_reduce_boundary(const float* in, int nx, int nz, int nb, float* out);

/* Interior cells the reference launch schedule never updates, per sweep
 * (-1 when none). Depends only on the grid shape and the 256-thread blocks. */
void orc_skip_cells(int ncols, int nzz, int skip_i[4], int skip_j[4]);

/* Source node (padded indices) by the reference's round-half-up rule. */
void orc_source_index(float sx, float sz, float dx, float dz, int nb, int* sIdx, int* sIdz);

/* 3x3 initial times around the source node, FP64 arithmetic. S is the padded
 * model (column stride nzz); node (zi, xi) gets S[zi + xi*nzz] * distance.
 * vals[a + 3*b] is node (sIdz - 1 + a, sIdx - 1 + b). */
void orc_init_block_f64(const float* S, int nzz, float sx, float sz, float dx, float dz,
                        int nb, int sIdx, int sIdz, double vals[9]);

/* The same in the reference build's FP32 arithmetic (orc_set_arith(1)). */
void orc_init_block_f32(const float* S, int nzz, float sx, float sz, float dx, float dz, int nb,
                        int sIdx, int sIdz, float vals[9]);

/* One solve on a window of the padded grid: nzz rows x ncols columns.
 * S: slowness of the window, column stride ldS. T: output, column stride nzz.
 * sIdz / sIdx_loc: source node inside the window; init: 9 FP32 values.
 * passes: number of 4-sweep passes (the reference runs exactly 1).
 * order: 0 = anti-diagonal levels exactly as the reference launches them,
 *        1 = nested column/row loops (same dependency order, same bits). */
void orc_solve_f32(int nzz, int ncols, const float* S, int ldS, float dx, float dz,
                   int sIdz, int sIdx_loc, const float init[9], float* T, int passes, int order);

/* FP64 twin. passes > 0: that many passes; passes <= 0: iterate until the
 * largest change of a pass is <= tol (at most max_passes); returns passes run. */
int orc_solve_f64(int nzz, int ncols, const float* S, int ldS, double dx, double dz,
                  int sIdz, int sIdx_loc, const double init[9], double* T, int passes,
                  double tol, int max_passes);

/* Deterministic min/max quantisation of n values to uint16 (reference rule). */
void orc_compress(const float* in, int n, uint16_t* out, float* vmax, float* vmin);

/* qP slowness pass (eikonal_ani.cu:47-111) on a window: writes Sout for the
 * interior cells (rows/cols in [nb, n-nb)) except the source node, copies
 * Sin elsewhere. codes[6]: C11,C13,C15,C33,C35,C55 (window base, stride ldS),
 * mm[12]: (min,max) pairs in the same order. */
void orc_qslowness_f32(int nzz, int ncols, int nb, const float* T, const float* Sin, int ldS,
                       float dx, float dz, int sIdz, int sIdx_loc,
                       const uint16_t* const codes[6], const float mm[12], float* Sout);

/* FP64 twins of the anisotropic path: the qP pass (FP64 traveltimes in,
 * FP64 slowness out, codes decoded in FP64) and the whole two-pass shot in
 * FP64 (T: nzz x ncols doubles; returns -1 for a source outside). */
void orc_qslowness_f64(int nzz, int ncols, int nb, const double* T, const float* Sin, int ldS, double dx,
                       double dz, int sIdz, int sIdx_loc, const uint16_t* const codes[6], const float mm[12],
                       double* Sout);
int orc_shot_ani_f64(int nzz, int nxx, int nb, const float* S, float dx, float dz, int c0, int ncols, float sx,
                     float sz, const uint16_t* const codes[6], const float mm[12], double* T);

/* Receiver picks by the reference's 4x4 Catmull-Rom rule on a window whose
 * first padded column is c0. Receivers whose stencil leaves the window's
 * columns [1, ncols-2] or rows [1, nzz-2] give NaN. */
void orc_picks_f32(const float* T, int nzz, int ncols, int c0, float dx, float dz, int nb,
                   const float* rx, const float* rz, int nrec, float* out);

/* Full shot (init + 1 or 2 solves + picks), FP32, as the C-ABI runs it.
 * ani != 0 uses codes/mm for the two-pass qP solve. T (nzz x ncols) and picks
 * are outputs; either may be NULL. Returns 0, or -1 for a source outside. */
int orc_shot_f32(int nzz, int nxx, int nb, const float* S, float dx, float dz, int c0, int ncols,
                 float sx, float sz, int ani, const uint16_t* const codes[6], const float mm[12],
                 float* T, const float* rx, const float* rz, int nrec, float* picks);

/* Many shots on the host cores (OpenMP over shots): the CPU baseline.
 * Shots b use windows [c0[b], c0[b]+ncols[b]); T_all may be NULL, picks is
 * nshots x nrec. Returns the number of OpenMP threads used. */
int orc_batch_f32(int nzz, int nxx, int nb, const float* S, float dx, float dz, int nshots,
                  const float* sx, const float* sz, const int* c0, const int* ncols, int ani,
                  const uint16_t* const codes[6], const float mm[12],
                  const float* rx, const float* rz, int nrec, float* picks, int nthreads);

/* ------------------------------------------------------------------------
 * Adjoint (no counterpart in the reference; it replaces the ray tracing and
 * LSCG gradient of src/inversion/inversion.cpp:95-177, :200-345).
 *
 * Tape: per node and sweep one code byte and two coefficients:
 *   code bits 0-2: active candidate 0 = none (old value kept or node not
 *                  updated), 1 = t1d1, 2 = t1d2, 3 = t1 (2D), 4 = t2, 5 = t3
 *   code bits 3-4: slowness cell that candidate read, (dr, dc): cell
 *                  (i-1+dr, j-1+dc)
 *   c1: t1 -> dT/dtv (dT/dte = -c1, dT/dtev = 1); t2 -> dT/dtev
 *       (dT/dte = 1 - c1); t3 -> dT/dtev (dT/dtv = 1 - c1)
 *   c2: dT/dS of the cell named by bits 3-4
 * tape index for node (i,j), sweep k: (k*ncols + j)*nzz + i.
 * ------------------------------------------------------------------------ */
void orc_solve_tape_f32(int nzz, int ncols, const float* S, int ldS, float dx, float dz,
                        int sIdz, int sIdx_loc, const float init[9], float* T,
                        uint8_t* code, float* c1, float* c2);
void orc_solve_tape_f64(int nzz, int ncols, const float* S, int ldS, double dx, double dz,
                        int sIdz, int sIdx_loc, const double init[9], double* T,
                        uint8_t* code, double* c1, double* c2);

/* FP64 solve that follows a given branch pattern: every node takes the
 * candidate and slowness cell named by code_in (tape layout above, e.g. the
 * codes of an FP32 taped solve) instead of choosing its own, and records the
 * FP64 coefficients of that candidate. With orc_adjoint_f64 over code_in it
 * gives the FP64 adjoint of the same discrete scheme as the FP32 tape. */
void orc_solve_follow_f64(int nzz, int ncols, const float* S, int ldS, double dx, double dz, int sIdz,
                          int sIdx_loc, const double init[9], const uint8_t* code_in, double* T, double* c1,
                          double* c2);

/* FP64 picks of an FP64 window field (weights of orc_pick_weights_f64). */
void orc_picks_f64(const double* T, int nzz, int ncols, int c0, float dx, float dz, int nb, const float* rx,
                   const float* rz, int nrec, double* out);

/* FP64 misfit 0.5 sum (p - tobs)^2 of a batch of shot windows (tobs nshots x
 * nrec, NaN entries skipped), p from the FP64 1-pass solve choosing its own
 * branches; and its central finite differences on a list of padded cells
 * (the slowness s replaced by RN32(s(1 +- rel)), returned in sp / sm). */
double orc_misfit_f64(int nzz, int nxx, int nb, const float* S, float dx, float dz, int nshots, const float* sx,
                      const float* sz, const int* c0, const int* ncols, const float* rx, const float* rz, int nrec,
                      const double* tobs);
int orc_fd_misfit_f64(int nzz, int nxx, int nb, const float* S, float dx, float dz, int nshots, const float* sx,
                      const float* sz, const int* c0, const int* ncols, const float* rx, const float* rz, int nrec,
                      const double* tobs, int ncells, const int* ci, const int* cj, double rel, float* sp,
                      float* sm, double* Jp, double* Jm, int nthreads);

/* Reverse sweeps over a tape. lam: adjoint of the final T (nzz x ncols), in
 * place; on return it holds the adjoint of the initial field. grad (nzz x
 * ncols, column stride nzz) receives += dJ/dS for the window, including the
 * 3x3 initialisation term (dist[9] = node distances). Per node of a sweep
 * with signs (sz, sx): mu = (lam + (pv(i+sz, j) + pev(i+sz, j+sx))) +
 * pe(i, j+sx), missing neighbours contributing 0. */
void orc_adjoint_f32(int nzz, int ncols, int sIdz, int sIdx_loc, const uint8_t* code,
                     const float* c1, const float* c2, const float dist[9], float* lam, float* grad);
void orc_adjoint_f64(int nzz, int ncols, int sIdz, int sIdx_loc, const uint8_t* code,
                     const double* c1, const double* c2, const double dist[9], double* lam,
                     double* grad);

/* Adjoint seed of one shot window from pick gradients pg[nrec] (NaN = no
 * pick), receivers in order, 16 taps each: lam[node] += pg * w, w the
 * Catmull-Rom weight product (FP64 weights, t^2 = t*t, t^3 = t^2*t, rounded
 * once to FP32 in the _f32 variant). lam is zeroed first. */
void orc_seed_lambda_f32(int nzz, int ncols, int c0, float dx, float dz, int nb, const float* rx,
                         const float* rz, int nrec, const float* pg, float* lam);
void orc_seed_lambda_f64(int nzz, int ncols, int c0, float dx, float dz, int nb, const float* rx,
                         const float* rz, int nrec, const double* pg, double* lam);

/* FP32 oracle of sf_batch_misfit_gradient for a batch of shot windows, one
 * shot per thread: taped solve, picks, pick residual r = pick - tobs (NaN:
 * no pick), seed, reverse sweeps into the shot's window gradient (FP32); the
 * window gradients are then summed onto grad (nxx x nzz) in FP64 in caller
 * order and rounded once. misfit = sum 0.5 r^2 in FP64 over (shot, receiver)
 * in order, r the FP32 residual. Returns the number of threads used, or -1 if a source lies
 * outside its window. */
int orc_batch_gradient_f32(int nzz, int nxx, int nb, const float* S, float dx, float dz, int nshots,
                           const float* sx, const float* sz, const int* c0, const int* ncols,
                           const float* rx, const float* rz, int nrec, const float* tobs,
                           float* picks, double* misfit, float* grad, int nthreads, int ani,
                           const uint16_t* const codes[6], const float mm[12], float* grad_c11,
                           float* grad_c13);
void orc_qp_factors(int nzz, int ncols, int nb, const float* T, const float* Sin, int ldS, float dx, float dz,
                    int sIdz, int sIdx_loc, const uint16_t* const codes[6], const float mm[12], float* fS,
                    float* f11, float* f13);

/* Tomography update (inversion.cpp:347-447, tomography_iso.cpp:77-92):
 * the Gaussian kernel of smooth_matrix (n x n, x major), model_smoothing of a
 * model-sized field (nz x nx, z fastest) and the slowness update of a padded
 * model (see the definitions for the arithmetic). */
void orc_smooth_kernel(float stdv, int n, float* k);
void orc_model_smoothing(const float* model, int nx, int nz, float stdv, int samples, float* out);
void orc_update_slowness(float* S, const float* grad, int nx, int nz, int nb, float scale, float stdv,
                         int samples, float* dS);

/* Kirchhoff image-domain migration (src/migration/migration.cu:54-71,
 * :197-228, :398-483, KDM.cu:3-55): the wavelet (returns its length, or
 * minus it when wmax is too small), the trace cross-correlation, and the
 * image (nz x nx) from padded tables Ts (nsrc) and Tr (nrec). */
int orc_kirchhoff_wavelet(float fmax, float dt, float* w, int wmax);
void orc_adjoint_convolution(const float* in, float* out, int ntr, int nt, const float* w, int nw);
void orc_kirchhoff_image(int nxx, int nzz, int nb, const float* S, const float* Ts, const float* Tr, int nsrc,
                         int nrec, const float* xsrc, const float* xrec, const float* data, int nt, float dt,
                         float dx, float dz, float aperture, float max_offset, float* image);
void orc_kirchhoff_forward(int nxx, int nzz, int nb, const float* S, const float* Ts, const float* Tr, int nsrc,
                           int nrec, const float* xsrc, const float* xrec, const float* model, int nt, float dt,
                           float dx, float dz, float aperture, float max_offset, int nang, float da, float mincmp,
                           float dcmp, float* data);
void orc_forward_convolution(const float* in, float* out, int ntr, int nt, const float* w, int nw);

/* Arithmetic of the FP32 solvers: 0 = every operation rounded once and the
 * 3x3 initialisation in FP64 (default); 1 = the reference build's arithmetic:
 * FP32 initialisation and fused multiply-adds where nvcc forms them in
 * inner_sweep (t1d1, t1d2, the 2D numerator and discriminant, Sref^2 - q^2 and
 * the two edge updates) and get_quasi_slowness (|grad T|^2, the Christoffel
 * sums). */
void orc_set_arith(int mode);

/* Catmull-Rom weights of the pick rule: w[16], node (i-1+b, j-1+a) -> w[a*4+b]
 * (a along x, b along z); i, j padded node of the receiver; returns 0 when the
 * stencil is inside the window (same test as orc_picks_f32), else -1. */
int orc_pick_weights_f64(float x, float z, float dx, float dz, int nb, int nzz, int ncols, int c0,
                         int* i, int* j, double w[16]);

#ifdef __cplusplus
}
#endif
#endif
