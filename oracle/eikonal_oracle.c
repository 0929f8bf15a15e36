/*
 * CPU oracle for the SeisFAT2D fast-sweeping eikonal path (test infrastructure;
 * see eikonal_oracle.h for what each function restates). Build with
 * -ffp-contract=off so that every FP32 operation rounds once, in source order.
 *
 * Pinned to the reference itself: the solver (isotropic and anisotropic)
 * against the reference's own kernels, compiled from its sources and run on
 * a GB300 (the npz files of tests/golden, tests/test_gpu_reference.py); the padding,
 * Cij quantisation, picks, smoothing and Kirchhoff wavelet against the
 * reference's own host methods, compiled from its sources by
 * oracle/build_ref.py (tests/test_oracle.py). The adjoint has no counterpart
 * in the reference; it is checked against finite differences.
 */
#include "eikonal_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define SF_BIG 1e6f

static int g_arith = 0; /* see orc_set_arith */
void orc_set_arith(int mode) { g_arith = mode; }
#define NTHREADS_REF 256 /* modeling.cuh:11 */

/* ---------------------------------------------------------------- padding */

/* modeling.cu:204-232 */
void orc_expand_boundary(const float* in, int nx, int nz, int nb, float* out)
{
    int nxx = nx + 2 * nb, nzz = nz + 2 * nb;
    for (int j = 0; j < nx; j++)
        for (int i = 0; i < nz; i++) out[(i + nb) + (j + nb) * nzz] = in[i + j * nz];
    for (int i = 0; i < nb; i++)
        for (int j = nb; j < nxx - nb; j++) {
            out[i + j * nzz] = out[nb + j * nzz];
            out[(nzz - i - 1) + j * nzz] = out[(nzz - nb - 1) + j * nzz];
        }
    for (int i = 0; i < nzz; i++)
        for (int j = 0; j < nb; j++) {
            out[i + j * nzz] = out[i + nb * nzz];
            out[i + (nxx - j - 1) * nzz] = out[i + (nxx - nb - 1) * nzz];
        }
}

/* modeling.cu:234-244 */
void orc_reduce_boundary(const float* in, int nx, int nz, int nb, float* out)
{
    int nzz = nz + 2 * nb;
    for (int j = 0; j < nx; j++)
        for (int i = 0; i < nz; i++) out[i + j * nz] = in[(i + nb) + (j + nb) * nzz];
}

/* ------------------------------------------------ reference launch schedule */

/* The per-level offsets of modeling.cu:137-148, restated. */
static void level_offsets(int sweep, int level, int nxx, int nzz, int* zo, int* xo)
{
    switch (sweep) {
    case 0:
        *zo = (level < nxx) ? 0 : level - nxx + 1;
        *xo = (level < nxx) ? level : nxx - 1;
        break;
    case 1:
        *zo = (level < nzz) ? nzz - level - 1 : 0;
        *xo = (level < nzz) ? 0 : level - nzz + 1;
        break;
    case 2:
        *zo = (level < nzz) ? level : nzz - 1;
        *xo = (level < nzz) ? nxx - 1 : nxx - 1 - (level - nzz + 1);
        break;
    default:
        *zo = (level < nxx) ? nzz - 1 : nzz - 1 - (level - nxx + 1);
        *xo = (level < nxx) ? nxx - level - 1 : 0;
        break;
    }
}

/* modeling.cu:150-154: threads launched for a level (the middle-band count is
 * level-2, which can fall one short of the diagonal; the bound check at
 * modeling.cu:319 hides the excess). */
static int level_threads(int level, int nxx, int nzz)
{
    int total = nxx + nzz - 2, mn = nxx < nzz ? nxx : nzz, mx = nxx < nzz ? nzz : nxx;
    int n = (level < mn) ? level + 1 : (level >= mx) ? total - level : total - mn - mx + level;
    int nblk = (n + NTHREADS_REF - 1) / NTHREADS_REF;
    return nblk * NTHREADS_REF;
}

static void sweep_dirs(int sweep, int* zd, int* xd)
{
    *zd = (sweep == 2 || sweep == 3) ? -1 : 1; /* modeling.cu:132-133 */
    *xd = (sweep == 0 || sweep == 2) ? -1 : 1;
}

static int imax(int a, int b) { return a > b ? a : b; }
static int imin(int a, int b) { return a < b ? a : b; }

void orc_skip_cells(int ncols, int nzz, int skip_i[4], int skip_j[4])
{
    int nxx = ncols, total = nxx + nzz - 2;
    for (int s = 0; s < 4; s++) {
        skip_i[s] = -1;
        skip_j[s] = -1;
        int zd, xd;
        sweep_dirs(s, &zd, &xd);
        for (int level = 0; level < total; level++) {
            int zo, xo;
            level_offsets(s, level, nxx, nzz, &zo, &xo);
            /* element range e >= 0 whose node is interior */
            int lo = 0, hi = 1 << 30;
            if (zd > 0) { lo = imax(lo, 1 - zo); hi = imin(hi, nzz - 2 - zo); }
            else        { lo = imax(lo, zo - (nzz - 2)); hi = imin(hi, zo - 1); }
            if (xd > 0) { lo = imax(lo, 1 - xo); hi = imin(hi, nxx - 2 - xo); }
            else        { lo = imax(lo, xo - (nxx - 2)); hi = imin(hi, xo - 1); }
            int nl = level_threads(level, nxx, nzz);
            for (int e = imax(lo, nl); e <= hi; e++) {
                /* at most one per sweep for any shape (checked by the tests) */
                skip_i[s] = zo + zd * e;
                skip_j[s] = xo + xd * e;
            }
        }
    }
}

/* ----------------------------------------------------------- source / init */

/* modeling.cu:112-113 */
void orc_source_index(float sx, float sz, float dx, float dz, int nb, int* sIdx, int* sIdz)
{
    *sIdx = (int)((sx + 0.5f * dx) / dx) + nb;
    *sIdz = (int)((sz + 0.5f * dz) / dz) + nb;
}

/* modeling.cu:293-306, evaluated in FP64. */
void orc_init_block_f64(const float* S, int nzz, float sx, float sz, float dx, float dz,
                        int nb, int sIdx, int sIdz, double vals[9])
{
    for (int b = 0; b < 3; b++)
        for (int a = 0; a < 3; a++) {
            int zi = sIdz + a - 1, xi = sIdx + b - 1;
            double ddx = (double)(xi - nb) * (double)dx - (double)sx;
            double ddz = (double)(zi - nb) * (double)dz - (double)sz;
            vals[a + 3 * b] = (double)S[zi + (size_t)xi * nzz] * sqrt(ddx * ddx + ddz * ddz);
        }
}

/* modeling.cu:293-306 in the reference build's FP32 arithmetic: nvcc fuses
 * (xi-nb)*dx - sx into one FMA. The reference squares with CUDA's powf(v,
 * 2.0f), which this restatement cannot reproduce bit for bit; v*v (correctly
 * rounded) is used, which differs from CUDA's powf by an ulp for about 3% of
 * arguments. Exact for sources whose offsets X, Z are exact small values. */
void orc_init_block_f32(const float* S, int nzz, float sx, float sz, float dx, float dz, int nb,
                           int sIdx, int sIdz, float vals[9])
{
    for (int b = 0; b < 3; b++)
        for (int a = 0; a < 3; a++) {
            int zi = sIdz + a - 1, xi = sIdx + b - 1;
            float X = fmaf((float)(xi - nb), dx, -sx);
            float Z = fmaf((float)(zi - nb), dz, -sz);
            vals[a + 3 * b] = S[zi + (size_t)xi * nzz] * sqrtf(X * X + Z * Z);
        }
}

static void init_dist_f64(int nb, float sx, float sz, float dx, float dz, int sIdx, int sIdz,
                          double dist[9])
{
    for (int b = 0; b < 3; b++)
        for (int a = 0; a < 3; a++) {
            int zi = sIdz + a - 1, xi = sIdx + b - 1;
            double ddx = (double)(xi - nb) * (double)dx - (double)sx;
            double ddz = (double)(zi - nb) * (double)dz - (double)sz;
            dist[a + 3 * b] = sqrt(ddx * ddx + ddz * ddz);
        }
}

/* ------------------------------------------------------------- the update */

typedef struct {
    float dx, dz, dx2i, dz2i, hyp;
} k32;

typedef struct {
    double dx, dz, dx2i, dz2i, hyp;
} k64;

static k32 make_k32(float dx, float dz)
{
    k32 k;
    k.dx = dx;
    k.dz = dz;
    k.dz2i = 1.0f / (dz * dz); /* modeling.cu:64-65 */
    k.dx2i = 1.0f / (dx * dx);
    k.hyp = sqrtf(dx * dx + dz * dz);
    return k;
}

static k64 make_k64(double dx, double dz)
{
    k64 k;
    k.dx = dx;
    k.dz = dz;
    k.dz2i = 1.0 / (dz * dz);
    k.dx2i = 1.0 / (dx * dx);
    k.hyp = sqrt(dx * dx + dz * dz);
    return k;
}

/* Tape record of one node update. */
typedef struct {
    int code;
    double c1, c2;
} rec_t;

/*
 * inner_sweep's per-node arithmetic (modeling.cu:319-356). s1a/s1b are the two
 * cells of the vertical upwind edge (row i1, columns max(j-1,1) and j), s2a/s2b
 * of the horizontal one (rows max(i-1,1) and i, column j1), sref = S[i1][j1].
 * dc1a: column offset code (0 -> j-1, 1 -> j) of s1a, dr2a: row code of s2a;
 * dr1 / dc2: row code of the vertical edge's cells / column code of the
 * horizontal edge's cells; those describe where a candidate read its slowness.
 */
static float upd32(float told, float tv, float te, float tev, float s1a, float s1b, float s2a,
                   float s2b, float sref, const k32* k, int dr1, int dc1a, int dc2, int dr2a,
                   rec_t* rec)
{
    float m1 = fminf(s1a, s1b);
    float m2 = fminf(s2a, s2b);
    const int ref = g_arith == 1;
    float t1d1 = ref ? fmaf(k->dz, m1, tv) : tv + k->dz * m1;
    float t1d2 = ref ? fmaf(k->dx, m2, te) : te + k->dx * m2;
    float t1D = fminf(t1d1, t1d2);
    float t1 = SF_BIG, t2 = SF_BIG, t3 = SF_BIG;
    int br = 0;
    float rr = 0.0f, dd = 0.0f, q = 0.0f, qq = 0.0f;
    if ((tv <= te + k->dx * sref) && (te <= tv + k->dz * sref) && (te - tev >= 0.0f) &&
        (tv - tev >= 0.0f)) {
        float ta = tev + te - tv;
        float tb = tev - te + tv;
        dd = ta - tb;
        if (ref) {
            float kd = k->dz2i * k->dx2i * dd;
            rr = sqrtf(fmaf(4.0f * sref * sref, (k->dz2i + k->dx2i), -(kd * dd)));
            t1 = (fmaf(tb, k->dz2i, ta * k->dx2i) + rr) / (k->dz2i + k->dx2i);
        } else {
            rr = sqrtf(4.0f * sref * sref * (k->dz2i + k->dx2i) - k->dz2i * k->dx2i * dd * dd);
            t1 = ((tb * k->dz2i + ta * k->dx2i) + rr) / (k->dz2i + k->dx2i);
        }
        br = 3;
    } else if ((te - tev <= sref * k->dz * k->dz / k->hyp) && (te - tev > 0.0f)) {
        q = (te - tev) / k->dz;
        qq = sqrtf(ref ? fmaf(-q, q, sref * sref) : sref * sref - q * q);
        t2 = ref ? fmaf(k->dx, qq, te) : te + k->dx * qq;
        br = 4;
    } else if ((tv - tev <= sref * k->dx * k->dx / k->hyp) && (tv - tev > 0.0f)) {
        q = (tv - tev) / k->dx;
        qq = sqrtf(ref ? fmaf(-q, q, sref * sref) : sref * sref - q * q);
        t3 = ref ? fmaf(k->dz, qq, tv) : tv + k->dz * qq;
        br = 5;
    }
    float t2D = fminf(t1, fminf(t2, t3));
    float cand = fminf(t1D, t2D);
    float tnew = fminf(told, cand);
    if (rec) {
        rec->code = 0;
        rec->c1 = 0.0;
        rec->c2 = 0.0;
        if (cand < told) {
            if (t1D <= t2D) {
                if (t1d1 <= t1d2) {
                    int dc = (s1a <= s1b) ? dc1a : 1;
                    rec->code = 1 | (dr1 << 3) | (dc << 4);
                    rec->c2 = k->dz;
                } else {
                    int dr = (s2a <= s2b) ? dr2a : 1;
                    rec->code = 2 | (dr << 3) | (dc2 << 4);
                    rec->c2 = k->dx;
                }
            } else if (br != 0) {
                int pos = (dr1 << 3) | (dc2 << 4); /* Sref = S[i1][j1] */
                rec->code = br | pos;
                if (br == 3) {
                    float D = k->dz2i + k->dx2i;
                    float kA = k->dz2i - k->dx2i;
                    float k2K = 2.0f * (k->dz2i * k->dx2i);
                    if (rr > 0.0f) {
                        rec->c1 = (kA + (k2K * dd) / rr) / D;
                        rec->c2 = (4.0f * sref) / rr;
                    } else {
                        rec->c1 = kA / D;
                        rec->c2 = 0.0f;
                    }
                } else {
                    float hx = (br == 4) ? k->dx : k->dz; /* multiplies the sqrt */
                    float hq = (br == 4) ? k->dz : k->dx; /* divides the difference */
                    if (qq > 0.0f) {
                        rec->c1 = (hx * q) / (hq * qq);
                        rec->c2 = (hx * sref) / qq;
                    } else {
                        rec->c1 = 0.0f;
                        rec->c2 = 0.0f;
                    }
                }
            }
        }
    }
    return tnew;
}

static double upd64(double told, double tv, double te, double tev, double s1a, double s1b,
                    double s2a, double s2b, double sref, const k64* k, int dr1, int dc1a, int dc2,
                    int dr2a, rec_t* rec)
{
    double m1 = fmin(s1a, s1b);
    double m2 = fmin(s2a, s2b);
    double t1d1 = tv + k->dz * m1;
    double t1d2 = te + k->dx * m2;
    double t1D = fmin(t1d1, t1d2);
    double t1 = 1e6, t2 = 1e6, t3 = 1e6;
    int br = 0;
    double rr = 0.0, dd = 0.0, q = 0.0, qq = 0.0;
    if ((tv <= te + k->dx * sref) && (te <= tv + k->dz * sref) && (te - tev >= 0.0) &&
        (tv - tev >= 0.0)) {
        double ta = tev + te - tv;
        double tb = tev - te + tv;
        dd = ta - tb;
        rr = sqrt(4.0 * sref * sref * (k->dz2i + k->dx2i) - k->dz2i * k->dx2i * dd * dd);
        t1 = ((tb * k->dz2i + ta * k->dx2i) + rr) / (k->dz2i + k->dx2i);
        br = 3;
    } else if ((te - tev <= sref * k->dz * k->dz / k->hyp) && (te - tev > 0.0)) {
        q = (te - tev) / k->dz;
        qq = sqrt(sref * sref - q * q);
        t2 = te + k->dx * qq;
        br = 4;
    } else if ((tv - tev <= sref * k->dx * k->dx / k->hyp) && (tv - tev > 0.0)) {
        q = (tv - tev) / k->dx;
        qq = sqrt(sref * sref - q * q);
        t3 = tv + k->dz * qq;
        br = 5;
    }
    double t2D = fmin(t1, fmin(t2, t3));
    double cand = fmin(t1D, t2D);
    double tnew = fmin(told, cand);
    if (rec) {
        rec->code = 0;
        rec->c1 = 0.0;
        rec->c2 = 0.0;
        if (cand < told) {
            if (t1D <= t2D) {
                if (t1d1 <= t1d2) {
                    int dc = (s1a <= s1b) ? dc1a : 1;
                    rec->code = 1 | (dr1 << 3) | (dc << 4);
                    rec->c2 = k->dz;
                } else {
                    int dr = (s2a <= s2b) ? dr2a : 1;
                    rec->code = 2 | (dr << 3) | (dc2 << 4);
                    rec->c2 = k->dx;
                }
            } else if (br != 0) {
                rec->code = br | (dr1 << 3) | (dc2 << 4);
                if (br == 3) {
                    double D = k->dz2i + k->dx2i;
                    if (rr > 0.0) {
                        rec->c1 = ((k->dz2i - k->dx2i) + 2.0 * k->dz2i * k->dx2i * dd / rr) / D;
                        rec->c2 = 4.0 * sref / rr;
                    } else {
                        rec->c1 = (k->dz2i - k->dx2i) / D;
                    }
                } else {
                    double hx = (br == 4) ? k->dx : k->dz;
                    double hq = (br == 4) ? k->dz : k->dx;
                    if (qq > 0.0) {
                        rec->c1 = hx * q / (hq * qq);
                        rec->c2 = hx * sref / qq;
                    }
                }
            }
        }
    }
    return tnew;
}

/* ------------------------------------------------------------- the solvers */

#define SAT(i, j) S[(size_t)(i) + (size_t)(j) * ldS]
#define TAT(i, j) T[(size_t)(i) + (size_t)(j) * nzz]

static void sweep_signs(int sweep, int* sz, int* sx)
{
    /* sgnt of modeling.cu:68: {1,1},{-1,1},{1,-1},{-1,-1} (z, x) */
    *sz = (sweep == 1 || sweep == 3) ? -1 : 1;
    *sx = (sweep >= 2) ? -1 : 1;
}

/* Node (i, j) of sweep `sweep` in FP32; returns the new value. */
static float node32(int sweep, int i, int j, int nzz, int ncols, const float* S, int ldS,
                    const float* T, const k32* k, rec_t* rec)
{
    int sz, sx;
    sweep_signs(sweep, &sz, &sx);
    int i1 = (sz > 0) ? i - 1 : i; /* i - sgnv[sgni] */
    int j1 = (sx > 0) ? j - 1 : j;
    float tv = TAT(i - sz, j);
    float te = TAT(i, j - sx);
    float tev = TAT(i - sz, j - sx);
    float s1a = SAT(i1, imax(j - 1, 1)), s1b = SAT(i1, imin(j, ncols - 1));
    float s2a = SAT(imax(i - 1, 1), j1), s2b = SAT(imin(i, nzz - 1), j1);
    float sref = SAT(i1, j1);
    int dr1 = (sz > 0) ? 0 : 1, dc2 = (sx > 0) ? 0 : 1;
    int dc1a = (j - 1 >= 1) ? 0 : 1, dr2a = (i - 1 >= 1) ? 0 : 1;
    return upd32(TAT(i, j), tv, te, tev, s1a, s1b, s2a, s2b, sref, k, dr1, dc1a, dc2, dr2a, rec);
}

/* S or, when Sd is given, the FP64 slowness Sd (same layout) */
#define SAT64(i, j) (Sd ? Sd[(size_t)(i) + (size_t)(j) * ldS] : (double)SAT(i, j))

static double node64(int sweep, int i, int j, int nzz, int ncols, const float* S, const double* Sd, int ldS,
                     const double* T, const k64* k, rec_t* rec)
{
    int sz, sx;
    sweep_signs(sweep, &sz, &sx);
    int i1 = (sz > 0) ? i - 1 : i;
    int j1 = (sx > 0) ? j - 1 : j;
    double tv = TAT(i - sz, j);
    double te = TAT(i, j - sx);
    double tev = TAT(i - sz, j - sx);
    double s1a = SAT64(i1, imax(j - 1, 1)), s1b = SAT64(i1, imin(j, ncols - 1));
    double s2a = SAT64(imax(i - 1, 1), j1), s2b = SAT64(imin(i, nzz - 1), j1);
    double sref = SAT64(i1, j1);
    int dr1 = (sz > 0) ? 0 : 1, dc2 = (sx > 0) ? 0 : 1;
    int dc1a = (j - 1 >= 1) ? 0 : 1, dr2a = (i - 1 >= 1) ? 0 : 1;
    return upd64(TAT(i, j), tv, te, tev, s1a, s1b, s2a, s2b, sref, k, dr1, dc1a, dc2, dr2a, rec);
}

#define TP(k, i, j) (((size_t)(k) * ncols + (size_t)(j)) * nzz + (size_t)(i))

static int is_skip(int s, int i, int j, const int si[4], const int sj[4])
{
    return i == si[s] && j == sj[s];
}

/*
 * Compensated FP32 update (orc_set_arith(2); no counterpart in the reference).
 * A traveltime is an unevaluated sum hi + lo of two FP32 values. All the
 * update's decisions and increments depend on differences of the upwind
 * times only, so they are formed from the pairs, (a.h - b.h) + (a.l - b.l),
 * and the candidates are compared in FP32 next to a nearby finite time (the
 * two 1D ones next to te, the 1D and the 2D or edge winner next to tev, the
 * winner and the old value next to the winner's base), never next to the
 * 1e6 sentinel; the winner is its base time plus its FP32 increment, added
 * with Knuth's TwoSum and
 * renormalised with Dekker's Fast2Sum (D. E. Knuth, TAOCP vol. 2, 4.2.2;
 * T. J. Dekker, Numer. Math. 18, 1971). The rounding error of each node is
 * then relative to its increment instead of its time, so it no longer
 * accumulates along the sweep. Same candidates, branch tests and tape
 * coefficients as upd32 (IEEE operations, no contraction); hi is the
 * traveltime that callers see.
 */
typedef struct {
    float h, l;
} ff_t;

static ff_t ff_add(ff_t a, float b)
{
    const float s = a.h + b, bb = s - a.h;
    const float e = (a.h - (s - bb)) + (b - bb);
    const float l = e + a.l, h = s + l;
    ff_t r = {h, l - (h - s)};
    return r;
}

static float ff_diff(ff_t a, ff_t b) { return (a.h - b.h) + (a.l - b.l); }

static ff_t updc(ff_t told, ff_t tv, ff_t te, ff_t tev, float s1a, float s1b, float s2a, float s2b, float sref,
                 const k32* k, int dr1, int dc1a, int dc2, int dr2a, rec_t* rec)
{
    const float dte = ff_diff(te, tev), dtv = ff_diff(tv, tev), dvt = ff_diff(tv, te);
    const float m1 = fminf(s1a, s1b), m2 = fminf(s2a, s2b);
    const float i1 = k->dz * m1, i2 = k->dx * m2;   /* t1d1 = tv + i1, t1d2 = te + i2 */
    const int w11 = (dvt + i1) <= i2;                /* t1d1 <= t1d2, compared next to te */
    const float o1D = w11 ? dtv + i1 : dte + i2;     /* the 1D winner's offset to tev */
    float o3 = SF_BIG, o4 = SF_BIG, o5 = SF_BIG, inc = 0.0f;
    int br = 0;
    float rr = 0.0f, dd = 0.0f, q = 0.0f, qq = 0.0f;
    const float D = k->dz2i + k->dx2i;
    if ((dvt <= k->dx * sref) && (-dvt <= k->dz * sref) && (dte >= 0.0f) && (dtv >= 0.0f)) {
        dd = -2.0f * dvt; /* ta - tb = 2 (te - tv) */
        rr = sqrtf(4.0f * sref * sref * D - k->dz2i * k->dx2i * dd * dd);
        o3 = (rr - dvt * (k->dx2i - k->dz2i)) / D; /* t1 = tev + o3 */
        br = 3;
    } else if ((dte <= sref * k->dz * k->dz / k->hyp) && (dte > 0.0f)) {
        q = dte / k->dz;
        qq = sqrtf(sref * sref - q * q);
        inc = k->dx * qq; /* t2 = te + inc */
        o4 = dte + inc;
        br = 4;
    } else if ((dtv <= sref * k->dx * k->dx / k->hyp) && (dtv > 0.0f)) {
        q = dtv / k->dx;
        qq = sqrtf(sref * sref - q * q);
        inc = k->dz * qq; /* t3 = tv + inc */
        o5 = dtv + inc;
        br = 5;
    }
    /* a 2D or edge candidate needs tev close to its base, so both winners'
     * offsets to tev are exact enough to compare */
    const float o2D = fminf(o3, fminf(o4, o5));
    const int w1 = o1D <= o2D;
    ff_t base;
    float bi;
    if (w1) {
        base = w11 ? tv : te;
        bi = w11 ? i1 : i2;
    } else {
        base = (br == 3) ? tev : (br == 4 ? te : tv);
        bi = (br == 3) ? o3 : inc;
    }
    if (rec) {
        rec->code = 0;
        rec->c1 = 0.0;
        rec->c2 = 0.0;
    }
    /* the candidate replaces told when it is smaller, compared next to its base */
    if (!(bi < ff_diff(told, base))) return told;
    if (rec) {
        if (w1) {
            if (w11) {
                int dc = (s1a <= s1b) ? dc1a : 1;
                rec->code = 1 | (dr1 << 3) | (dc << 4);
                rec->c2 = k->dz;
            } else {
                int dr = (s2a <= s2b) ? dr2a : 1;
                rec->code = 2 | (dr << 3) | (dc2 << 4);
                rec->c2 = k->dx;
            }
        } else {
            rec->code = br | (dr1 << 3) | (dc2 << 4);
            if (br == 3) {
                float kA = k->dz2i - k->dx2i;
                float k2K = 2.0f * (k->dz2i * k->dx2i);
                if (rr > 0.0f) {
                    rec->c1 = (kA + (k2K * dd) / rr) / D;
                    rec->c2 = (4.0f * sref) / rr;
                } else {
                    rec->c1 = kA / D;
                }
            } else {
                float hx = (br == 4) ? k->dx : k->dz, hq = (br == 4) ? k->dz : k->dx;
                if (qq > 0.0f) {
                    rec->c1 = (hx * q) / (hq * qq);
                    rec->c2 = (hx * sref) / qq;
                }
            }
        }
    }
    return ff_add(base, bi);
}

/* One compensated solve (1 pass, any DAG order gives the same bits): T gets
 * the hi parts; the initial 3x3 values enter with lo = 0. */
static void solve_comp(int nzz, int ncols, const float* S, int ldS, float dx, float dz, int sIdz, int sIdx_loc,
                       const float init[9], float* T, float* Lout, uint8_t* code, float* c1, float* c2)
{
    k32 k = make_k32(dx, dz);
    int si[4], sj[4];
    orc_skip_cells(ncols, nzz, si, sj);
    float* L = Lout ? Lout : (float*)calloc((size_t)nzz * ncols, sizeof(float));
    if (Lout) memset(L, 0, sizeof(float) * (size_t)nzz * ncols);
    for (size_t n = 0; n < (size_t)nzz * ncols; n++) T[n] = SF_BIG;
    for (int b = 0; b < 3; b++)
        for (int a = 0; a < 3; a++) TAT(sIdz + a - 1, sIdx_loc + b - 1) = init[a + 3 * b];
    if (code) {
        memset(code, 0, (size_t)4 * ncols * nzz);
        for (size_t n = 0; n < (size_t)4 * ncols * nzz; n++) c1[n] = c2[n] = 0.0f;
    }
#define PAIR(i, j) ((ff_t){TAT(i, j), L[(size_t)(i) + (size_t)(j) * nzz]})
    for (int s = 0; s < 4; s++) {
        int sz, sx;
        sweep_signs(s, &sz, &sx);
        for (int jj = 1; jj <= ncols - 2; jj++) {
            int j = (sx > 0) ? jj : ncols - 1 - jj;
            for (int ii = 1; ii <= nzz - 2; ii++) {
                int i = (sz > 0) ? ii : nzz - 1 - ii;
                if (is_skip(s, i, j, si, sj)) continue;
                int i1 = (sz > 0) ? i - 1 : i, j1 = (sx > 0) ? j - 1 : j;
                float s1a = SAT(i1, imax(j - 1, 1)), s1b = SAT(i1, imin(j, ncols - 1));
                float s2a = SAT(imax(i - 1, 1), j1), s2b = SAT(imin(i, nzz - 1), j1);
                int dr1 = (sz > 0) ? 0 : 1, dc2 = (sx > 0) ? 0 : 1;
                int dc1a = (j - 1 >= 1) ? 0 : 1, dr2a = (i - 1 >= 1) ? 0 : 1;
                rec_t r;
                ff_t v = updc(PAIR(i, j), PAIR(i - sz, j), PAIR(i, j - sx), PAIR(i - sz, j - sx), s1a, s1b, s2a,
                              s2b, SAT(i1, j1), &k, dr1, dc1a, dc2, dr2a, code ? &r : NULL);
                TAT(i, j) = v.h;
                L[(size_t)i + (size_t)j * nzz] = v.l;
                if (code) {
                    code[TP(s, i, j)] = (uint8_t)r.code;
                    c1[TP(s, i, j)] = (float)r.c1;
                    c2[TP(s, i, j)] = (float)r.c2;
                }
            }
        }
    }
#undef PAIR
    if (!Lout) free(L);
}

static void init_field_f32(float* T, int nzz, int ncols, int sIdz, int sIdx_loc, const float init[9])
{
    for (size_t n = 0; n < (size_t)nzz * ncols; n++) T[n] = SF_BIG; /* time_set */
    for (int b = 0; b < 3; b++)
        for (int a = 0; a < 3; a++) TAT(sIdz + a - 1, sIdx_loc + b - 1) = init[a + 3 * b];
}

static void init_field_f64(double* T, int nzz, int ncols, int sIdz, int sIdx_loc, const double init[9])
{
    for (size_t n = 0; n < (size_t)nzz * ncols; n++) T[n] = 1e6;
    for (int b = 0; b < 3; b++)
        for (int a = 0; a < 3; a++) TAT(sIdz + a - 1, sIdx_loc + b - 1) = init[a + 3 * b];
}


void orc_solve_f32(int nzz, int ncols, const float* S, int ldS, float dx, float dz, int sIdz,
                   int sIdx_loc, const float init[9], float* T, int passes, int order)
{
    if (g_arith == 2) {
        solve_comp(nzz, ncols, S, ldS, dx, dz, sIdz, sIdx_loc, init, T, NULL, NULL, NULL, NULL);
        return;
    }
    k32 k = make_k32(dx, dz);
    int si[4], sj[4];
    orc_skip_cells(ncols, nzz, si, sj);
    init_field_f32(T, nzz, ncols, sIdz, sIdx_loc, init);
    int nxx = ncols, total = nxx + nzz - 2;
    for (int p = 0; p < passes; p++)
        for (int s = 0; s < 4; s++) {
            if (order == 0) {
                int zd, xd;
                sweep_dirs(s, &zd, &xd);
                for (int level = 0; level < total; level++) {
                    int zo, xo;
                    level_offsets(s, level, nxx, nzz, &zo, &xo);
                    int nl = level_threads(level, nxx, nzz);
                    /* cells of one level are independent: update in place */
                    for (int e = 0; e < nl; e++) {
                        int i = zo + zd * e, j = xo + xd * e;
                        if (i > 0 && i < nzz - 1 && j > 0 && j < nxx - 1)
                            TAT(i, j) = node32(s, i, j, nzz, ncols, S, ldS, T, &k, NULL);
                    }
                }
            } else {
                int sz, sx;
                sweep_signs(s, &sz, &sx);
                for (int jj = 1; jj <= ncols - 2; jj++) {
                    int j = (sx > 0) ? jj : ncols - 1 - jj;
                    for (int ii = 1; ii <= nzz - 2; ii++) {
                        int i = (sz > 0) ? ii : nzz - 1 - ii;
                        if (is_skip(s, i, j, si, sj)) continue;
                        TAT(i, j) = node32(s, i, j, nzz, ncols, S, ldS, T, &k, NULL);
                    }
                }
            }
        }
}

static int solve_f64_any(int nzz, int ncols, const float* S, const double* Sd, int ldS, double dx, double dz,
                         int sIdz, int sIdx_loc, const double init[9], double* T, int passes, double tol,
                         int max_passes);

int orc_solve_f64(int nzz, int ncols, const float* S, int ldS, double dx, double dz, int sIdz,
                  int sIdx_loc, const double init[9], double* T, int passes, double tol,
                  int max_passes)
{
    return solve_f64_any(nzz, ncols, S, NULL, ldS, dx, dz, sIdz, sIdx_loc, init, T, passes, tol, max_passes);
}

static int solve_f64_any(int nzz, int ncols, const float* S, const double* Sd, int ldS, double dx, double dz,
                         int sIdz, int sIdx_loc, const double init[9], double* T, int passes, double tol,
                         int max_passes)
{
    k64 k = make_k64(dx, dz);
    int si[4], sj[4];
    orc_skip_cells(ncols, nzz, si, sj);
    init_field_f64(T, nzz, ncols, sIdz, sIdx_loc, init);
    int npass = passes > 0 ? passes : max_passes;
    int run = 0;
    for (int p = 0; p < npass; p++) {
        double change = 0.0;
        for (int s = 0; s < 4; s++) {
            int sz, sx;
            sweep_signs(s, &sz, &sx);
            for (int jj = 1; jj <= ncols - 2; jj++) {
                int j = (sx > 0) ? jj : ncols - 1 - jj;
                for (int ii = 1; ii <= nzz - 2; ii++) {
                    int i = (sz > 0) ? ii : nzz - 1 - ii;
                    if (is_skip(s, i, j, si, sj)) continue;
                    double old = TAT(i, j);
                    double nv = node64(s, i, j, nzz, ncols, S, Sd, ldS, T, &k, NULL);
                    TAT(i, j) = nv;
                    if (old < 1e6 && old - nv > change) change = old - nv;
                    if (old >= 1e6 && nv < 1e6) change = 1e30;
                }
            }
        }
        run++;
        if (passes <= 0 && change <= tol) break;
    }
    return run;
}

/* ------------------------------------------------------------- anisotropy */

/* modeling.cu:264-279 with a deterministic min/max (the reference's OpenMP
 * loop races on min_value/max_value). max == min gives code 1 (decodes to min
 * exactly, as the reference's NaN-derived code does). */
void orc_compress(const float* in, int n, uint16_t* out, float* vmax, float* vmin)
{
    float mx = -1e20f, mn = 1e20f;
    for (int i = 0; i < n; i++) {
        mn = fminf(in[i], mn);
        mx = fmaxf(in[i], mx);
    }
    *vmax = mx;
    *vmin = mn;
    for (int i = 0; i < n; i++) {
        if (mx == mn) {
            out[i] = 1;
            continue;
        }
        float v = 1.0f + (float)(65535 - 1) * (in[i] - mn) / (mx - mn);
        out[i] = (uint16_t)v;
    }
}

static float decode_c(uint16_t c, float mn, float mx)
{
    /* eikonal_ani.cu:76-83 */
    return (mn + ((float)c - 1.0f) * (mx - mn) / (float)(65535 - 1));
}

/* eikonal_ani.cu:47-111 */
/* Central differences T(i+1) - T(i-1) and T(j+1) - T(j-1) at window index
 * it; of the pairs (T, L) in the compensated arithmetic (L not NULL). */
static void central_diffs(const float* T, const float* L, size_t it, int nzz, float* dzr, float* dxr)
{
    if (L) {
        *dzr = (T[it + 1] - T[it - 1]) + (L[it + 1] - L[it - 1]);
        *dxr = (T[it + nzz] - T[it - nzz]) + (L[it + nzz] - L[it - nzz]);
    } else {
        *dzr = T[it + 1] - T[it - 1];
        *dxr = T[it + nzz] - T[it - nzz];
    }
}

static void qslowness_f32(int nzz, int ncols, int nb, const float* T, const float* L, const float* Sin, int ldS,
                          float dx, float dz, int sIdz, int sIdx_loc, const uint16_t* const codes[6],
                          const float mm[12], float* Sout);

void orc_qslowness_f32(int nzz, int ncols, int nb, const float* T, const float* Sin, int ldS,
                       float dx, float dz, int sIdz, int sIdx_loc,
                       const uint16_t* const codes[6], const float mm[12], float* Sout)
{
    qslowness_f32(nzz, ncols, nb, T, NULL, Sin, ldS, dx, dz, sIdz, sIdx_loc, codes, mm, Sout);
}

static void qslowness_f32(int nzz, int ncols, int nb, const float* T, const float* L, const float* Sin, int ldS,
                          float dx, float dz, int sIdz, int sIdx_loc, const uint16_t* const codes[6],
                          const float mm[12], float* Sout)
{
    for (int j = 0; j < ncols; j++)
        for (int i = 0; i < nzz; i++) {
            size_t is = (size_t)i + (size_t)j * ldS;
            size_t it = (size_t)i + (size_t)j * nzz;
            float s = Sin[is];
            Sout[it] = s;
            if (!((i >= nb) && (i < nzz - nb) && (j >= nb) && (j < ncols - nb))) continue;
            if ((i == sIdz) && (j == sIdx_loc)) continue;
            float dzr, dxr;
            central_diffs(T, L, it, nzz, &dzr, &dxr);
            float dTz = 0.5f * dzr / dz;
            float dTx = 0.5f * dxr / dx;
            const int ref = g_arith == 1;
            float norm = sqrtf(ref ? fmaf(dTz, dTz, dTx * dTx) : dTx * dTx + dTz * dTz);
            float p0 = dTx / norm, p1 = dTz / norm;
            float c11 = decode_c(codes[0][is], mm[0], mm[1]);
            float c13 = decode_c(codes[1][is], mm[2], mm[3]);
            float c15 = decode_c(codes[2][is], mm[4], mm[5]);
            float c33 = decode_c(codes[3][is], mm[6], mm[7]);
            float c35 = decode_c(codes[4][is], mm[8], mm[9]);
            float c55 = decode_c(codes[5][is], mm[10], mm[11]);
            float C[9];
            C[0] = c11; C[3] = c13; C[6] = c15;
            C[1] = c13; C[4] = c33; C[7] = c35;
            C[2] = c15; C[5] = c35; C[8] = c55;
            float Ro = c33 * s * s;
            for (int q = 0; q < 9; q++) C[q] = C[q] / Ro / Ro;
            float Gxx, Gzz, Gxz;
            if (ref) { /* nvcc's FMAs: ((a p0) p0 + (b p1) p1) + (c p0) p1 -> fma(c p0, p1, fma(a p0, p0, (b p1) p1)) */
                Gxx = fmaf(2.0f * C[6] * p0, p1, fmaf(C[0] * p0, p0, C[8] * p1 * p1));
                Gzz = fmaf(2.0f * C[7] * p0, p1, fmaf(C[8] * p0, p0, C[4] * p1 * p1));
                Gxz = fmaf((C[3] + C[8]) * p0, p1, fmaf(C[6] * p0, p0, C[7] * p1 * p1));
            } else {
                Gxx = C[0] * p0 * p0 + C[8] * p1 * p1 + 2.0f * C[6] * p0 * p1;
                Gzz = C[8] * p0 * p0 + C[4] * p1 * p1 + 2.0f * C[7] * p0 * p1;
                Gxz = C[6] * p0 * p0 + C[7] * p1 * p1 + (C[3] + C[8]) * p0 * p1;
            }
            float coeff1 = Gxx + Gzz;
            float coeff2 = Gxx - Gzz;
            float det = sqrtf((coeff2 * coeff2) / 4.0f + Gxz * Gxz);
            /* coeff1 / 2.0 is a double expression in the reference */
            float g0 = (float)((double)coeff1 / 2.0 + (double)det);
            float g1 = (float)((double)coeff1 / 2.0 - (double)det);
            if (g0 < g1) g0 = g1;
            Sout[it] = 1.0f / sqrtf(g0 * Ro);
        }
}

/* FP64 twin of orc_qslowness_f32 (eikonal_ani.cu:47-111 evaluated in FP64,
 * the uint16 codes decoded in FP64): Sout (FP64) gets the qP slowness of the
 * interior cells except the source node and Sin elsewhere. */
void orc_qslowness_f64(int nzz, int ncols, int nb, const double* T, const float* Sin, int ldS, double dx,
                       double dz, int sIdz, int sIdx_loc, const uint16_t* const codes[6], const float mm[12],
                       double* Sout)
{
    for (int j = 0; j < ncols; j++)
        for (int i = 0; i < nzz; i++) {
            size_t is = (size_t)i + (size_t)j * ldS;
            size_t it = (size_t)i + (size_t)j * nzz;
            double s = Sin[is];
            Sout[it] = s;
            if (!((i >= nb) && (i < nzz - nb) && (j >= nb) && (j < ncols - nb))) continue;
            if ((i == sIdz) && (j == sIdx_loc)) continue;
            double dTz = 0.5 * (T[it + 1] - T[it - 1]) / dz;
            double dTx = 0.5 * (T[it + nzz] - T[it - nzz]) / dx;
            double norm = sqrt(dTx * dTx + dTz * dTz);
            double p0 = dTx / norm, p1 = dTz / norm;
            double c[6];
            for (int q = 0; q < 6; q++)
                c[q] = (double)mm[2 * q] + ((double)codes[q][is] - 1.0) * ((double)mm[2 * q + 1] - (double)mm[2 * q]) /
                                           65534.0;
            /* c11, c13, c15, c33, c35, c55 */
            double Ro = c[3] * s * s;
            double C0 = c[0] / Ro / Ro, C3 = c[1] / Ro / Ro, C6 = c[2] / Ro / Ro;
            double C4 = c[3] / Ro / Ro, C7 = c[4] / Ro / Ro, C8 = c[5] / Ro / Ro;
            double Gxx = C0 * p0 * p0 + C8 * p1 * p1 + 2.0 * C6 * p0 * p1;
            double Gzz = C8 * p0 * p0 + C4 * p1 * p1 + 2.0 * C7 * p0 * p1;
            double Gxz = C6 * p0 * p0 + C7 * p1 * p1 + (C3 + C8) * p0 * p1;
            double coeff1 = Gxx + Gzz, coeff2 = Gxx - Gzz;
            double det = sqrt(coeff2 * coeff2 / 4.0 + Gxz * Gxz);
            double g0 = coeff1 / 2.0 + det, g1 = coeff1 / 2.0 - det;
            if (g0 < g1) g0 = g1;
            Sout[it] = 1.0 / sqrt(g0 * Ro);
        }
}

/* The whole two-pass anisotropic shot (eikonal_ani.cu:33-45) in FP64: FP64
 * initialisation and solve, FP64 qP field from the FP64 traveltimes, FP64
 * initialisation from it and the second FP64 solve. T: nzz x ncols (FP64).
 * Returns 0, or -1 for a source outside its window. */
int orc_shot_ani_f64(int nzz, int nxx, int nb, const float* S, float dx, float dz, int c0, int ncols, float sx,
                     float sz, const uint16_t* const codes[6], const float mm[12], double* T)
{
    int sIdx, sIdz;
    orc_source_index(sx, sz, dx, dz, nb, &sIdx, &sIdz);
    const int sloc = sIdx - c0;
    if (sIdz < 1 || sIdz > nzz - 2 || sloc < 1 || sloc > ncols - 2 || c0 < 0 || c0 + ncols > nxx) return -1;
    const size_t n = (size_t)nzz * ncols;
    const float* Sw = S + (size_t)c0 * nzz;
    double init[9], dist[9];
    orc_init_block_f64(S, nzz, sx, sz, dx, dz, nb, sIdx, sIdz, init);
    solve_f64_any(nzz, ncols, Sw, NULL, nzz, dx, dz, sIdz, sloc, init, T, 1, 0.0, 1);
    double* Sq = (double*)malloc(n * sizeof(double));
    const uint16_t* cw[6];
    for (int q = 0; q < 6; q++) cw[q] = codes[q] + (size_t)c0 * nzz;
    orc_qslowness_f64(nzz, ncols, nb, T, Sw, nzz, dx, dz, sIdz, sloc, cw, mm, Sq);
    init_dist_f64(nb, sx, sz, dx, dz, sIdx, sIdz, dist);
    for (int b = 0; b < 3; b++)
        for (int a = 0; a < 3; a++) init[a + 3 * b] = Sq[(size_t)(sIdz + a - 1) + (size_t)(sloc + b - 1) * nzz] * dist[a + 3 * b];
    solve_f64_any(nzz, ncols, NULL, Sq, nzz, dx, dz, sIdz, sloc, init, T, 1, 0.0, 1);
    free(Sq);
    return 0;
}

/* Derivatives of one node's qP slowness with the direction p = grad T /
 * |grad T| of the first solve held fixed: Sq = S sqrt(c33 / lambda), lambda the
 * larger eigenvalue of the Christoffel matrix along p, v its unit eigenvector;
 * dSq/dS = sqrt(c33/lambda), dSq/dC11 = -Sq px^2 vx^2 / (2 lambda),
 * dSq/dC13 = -Sq px pz vx vz / lambda. FP32, each operation rounded once, in
 * this order (the engine's qp_factors in sf_device.cuh); (1, 0, 0) for a zero
 * gradient or a non-positive eigenvalue. */
static void qp_factors_f32(float dzr, float dxr, float s, float dx, float dz, float c11, float c13, float c15,
                           float c33, float c35, float c55, float* fS, float* f11, float* f13)
{
    float dTz = (0.5f * dzr) / dz;
    float dTx = (0.5f * dxr) / dx;
    float nrm = sqrtf(dTx * dTx + dTz * dTz);
    *fS = 1.0f;
    *f11 = 0.0f;
    *f13 = 0.0f;
    if (!(nrm > 0.0f)) return;
    float px = dTx / nrm, pz = dTz / nrm;
    float Gxx = c11 * px * px + c55 * pz * pz + 2.0f * c15 * px * pz;
    float Gzz = c55 * px * px + c33 * pz * pz + 2.0f * c35 * px * pz;
    float Gxz = c15 * px * px + c35 * pz * pz + (c13 + c55) * px * pz;
    float h = 0.5f * (Gxx - Gzz);
    float r = sqrtf(h * h + Gxz * Gxz);
    float lam = 0.5f * (Gxx + Gzz) + r;
    if (!(lam > 0.0f)) return;
    float vx, vz;
    if (h >= 0.0f) { vx = h + r; vz = Gxz; }
    else           { vx = Gxz; vz = r - h; }
    float nv = sqrtf(vx * vx + vz * vz);
    if (nv > 0.0f) { vx = vx / nv; vz = vz / nv; }
    else           { vx = px; vz = pz; }
    float fs = sqrtf(c33 / lam);
    float sq = s * fs;
    *fS = fs;
    *f11 = (-0.5f * sq * (px * px) * (vx * vx)) / lam;
    *f13 = (-sq * (px * pz) * (vx * vz)) / lam;
}

/* The factors over a window, as the qP pass runs (interior nodes except the
 * source; the others keep S: (1, 0, 0)). */
static void qp_factors_all(int nzz, int ncols, int nb, const float* T, const float* L, const float* Sin, int ldS,
                           float dx, float dz, int sIdz, int sIdx_loc, const uint16_t* const codes[6],
                           const float mm[12], float* fS, float* f11, float* f13);

void orc_qp_factors(int nzz, int ncols, int nb, const float* T, const float* Sin, int ldS, float dx, float dz,
                    int sIdz, int sIdx_loc, const uint16_t* const codes[6], const float mm[12], float* fS,
                    float* f11, float* f13)
{
    qp_factors_all(nzz, ncols, nb, T, NULL, Sin, ldS, dx, dz, sIdz, sIdx_loc, codes, mm, fS, f11, f13);
}

static void qp_factors_all(int nzz, int ncols, int nb, const float* T, const float* L, const float* Sin, int ldS,
                           float dx, float dz, int sIdz, int sIdx_loc, const uint16_t* const codes[6],
                           const float mm[12], float* fS, float* f11, float* f13)
{
    for (int j = 0; j < ncols; j++)
        for (int i = 0; i < nzz; i++) {
            size_t is = (size_t)i + (size_t)j * ldS;
            size_t it = (size_t)i + (size_t)j * nzz;
            fS[it] = 1.0f;
            f11[it] = 0.0f;
            f13[it] = 0.0f;
            if (!((i >= nb) && (i < nzz - nb) && (j >= nb) && (j < ncols - nb))) continue;
            if ((i == sIdz) && (j == sIdx_loc)) continue;
            float dzr, dxr;
            central_diffs(T, L, it, nzz, &dzr, &dxr);
            qp_factors_f32(dzr, dxr, Sin[is], dx, dz,
                           decode_c(codes[0][is], mm[0], mm[1]), decode_c(codes[1][is], mm[2], mm[3]),
                           decode_c(codes[2][is], mm[4], mm[5]), decode_c(codes[3][is], mm[6], mm[7]),
                           decode_c(codes[4][is], mm[8], mm[9]), decode_c(codes[5][is], mm[10], mm[11]),
                           &fS[it], &f11[it], &f13[it]);
        }
}

/* ------------------------------------------------------------------ picks */

/* admin.cpp:121-133 */
static float cubic1d(const float P[4], float t)
{
    return P[1] + 0.5f * t *
                      (P[2] - P[0] +
                       t * (2.0f * P[0] - 5.0f * P[1] + 4.0f * P[2] - P[3] +
                            t * (3.0f * (P[1] - P[2]) + P[3] - P[0])));
}

static int pick_geom(float x, float z, float dx, float dz, int nb, int nzz, int ncols, int c0,
                     int* pi, int* pj, float* pxd, float* pzd)
{
    /* modeling.cu:170-181 */
    float x0 = floorf((x + 0.5f * dx) / dx) * dx;
    float z0 = floorf((z + 0.5f * dz) / dz) * dz;
    float x1 = floorf((x + 0.5f * dx) / dx) * dx + dx;
    float z1 = floorf((z + 0.5f * dz) / dz) * dz + dz;
    *pxd = (x - x0) / (x1 - x0);
    *pzd = (z - z0) / (z1 - z0);
    int i = (int)((z + 0.5f * dz) / dz) + nb;
    int j = (int)((x + 0.5f * dx) / dx) + nb - c0;
    *pi = i;
    *pj = j;
    if (i - 1 < 1 || i + 2 > nzz - 2 || j - 1 < 1 || j + 2 > ncols - 2) return -1;
    return 0;
}

void orc_picks_f32(const float* T, int nzz, int ncols, int c0, float dx, float dz, int nb,
                   const float* rx, const float* rz, int nrec, float* out)
{
    for (int r = 0; r < nrec; r++) {
        int i, j;
        float xd, zd;
        if (pick_geom(rx[r], rz[r], dx, dz, nb, nzz, ncols, c0, &i, &j, &xd, &zd)) {
            out[r] = NAN;
            continue;
        }
        float P[4][4], p[4];
        for (int a = 0; a < 4; a++)
            for (int b = 0; b < 4; b++) P[a][b] = TAT(i + b - 1, j + a - 1);
        for (int a = 0; a < 4; a++) p[a] = cubic1d(P[a], zd);
        out[r] = cubic1d(p, xd);
    }
}

static void cubic_w(double t, double w[4])
{
    /* cubic1d is linear in P: coefficients of P[0..3] */
    w[0] = -0.5 * t + t * t - 0.5 * t * t * t;
    w[1] = 1.0 - 2.5 * t * t + 1.5 * t * t * t;
    w[2] = 0.5 * t + 2.0 * t * t - 1.5 * t * t * t;
    w[3] = -0.5 * t * t + 0.5 * t * t * t;
}

int orc_pick_weights_f64(float x, float z, float dx, float dz, int nb, int nzz, int ncols, int c0,
                         int* i, int* j, double w[16])
{
    float xd, zd;
    if (pick_geom(x, z, dx, dz, nb, nzz, ncols, c0, i, j, &xd, &zd)) return -1;
    double wx[4], wz[4];
    cubic_w(xd, wx);
    cubic_w(zd, wz);
    for (int a = 0; a < 4; a++)
        for (int b = 0; b < 4; b++) w[a * 4 + b] = wx[a] * wz[b];
    return 0;
}

static void cubic_w_ops(double t, double w[4])
{
    double t2 = t * t, t3 = t2 * t;
    w[0] = (-0.5 * t + t2) - 0.5 * t3;
    w[1] = (1.0 - 2.5 * t2) + 1.5 * t3;
    w[2] = (0.5 * t + 2.0 * t2) - 1.5 * t3;
    w[3] = -0.5 * t2 + 0.5 * t3;
}

void orc_seed_lambda_f32(int nzz, int ncols, int c0, float dx, float dz, int nb, const float* rx,
                         const float* rz, int nrec, const float* pg, float* lam)
{
    memset(lam, 0, sizeof(float) * (size_t)nzz * ncols);
    for (int r = 0; r < nrec; r++) {
        int i, j;
        float xd, zd;
        float g = pg[r];
        if (pick_geom(rx[r], rz[r], dx, dz, nb, nzz, ncols, c0, &i, &j, &xd, &zd) || g != g) continue;
        double wx[4], wz[4];
        cubic_w_ops((double)xd, wx);
        cubic_w_ops((double)zd, wz);
        for (int a = 0; a < 4; a++)
            for (int b = 0; b < 4; b++) {
                float w = (float)(wx[a] * wz[b]);
                float* at = lam + (size_t)(i + b - 1) + (size_t)(j + a - 1) * nzz;
                *at = *at + g * w;
            }
    }
}

void orc_seed_lambda_f64(int nzz, int ncols, int c0, float dx, float dz, int nb, const float* rx,
                         const float* rz, int nrec, const double* pg, double* lam)
{
    memset(lam, 0, sizeof(double) * (size_t)nzz * ncols);
    for (int r = 0; r < nrec; r++) {
        int i, j;
        float xd, zd;
        double g = pg[r];
        if (pick_geom(rx[r], rz[r], dx, dz, nb, nzz, ncols, c0, &i, &j, &xd, &zd) || g != g) continue;
        double wx[4], wz[4];
        cubic_w_ops((double)xd, wx);
        cubic_w_ops((double)zd, wz);
        for (int a = 0; a < 4; a++)
            for (int b = 0; b < 4; b++)
                lam[(size_t)(i + b - 1) + (size_t)(j + a - 1) * nzz] += g * (wx[a] * wz[b]);
    }
}

/* FP64 picks of one FP64 window field: the 16 FP64 Catmull-Rom weights of
 * orc_pick_weights_f64 times the nodes, NaN where the stencil leaves the
 * window. */
void orc_picks_f64(const double* T, int nzz, int ncols, int c0, float dx, float dz, int nb, const float* rx,
                   const float* rz, int nrec, double* out)
{
    for (int r = 0; r < nrec; r++) {
        int i, j;
        double w[16];
        if (orc_pick_weights_f64(rx[r], rz[r], dx, dz, nb, nzz, ncols, c0, &i, &j, w)) {
            out[r] = NAN;
            continue;
        }
        double acc = 0.0;
        for (int a = 0; a < 4; a++)
            for (int b = 0; b < 4; b++) acc += w[a * 4 + b] * TAT(i + b - 1, j + a - 1);
        out[r] = acc;
    }
}

/* FP64 misfit of a batch on the padded slowness S: 0.5 sum over shots and
 * receivers (in order) of (p - tobs)^2, p the FP64 picks of the FP64 1-pass
 * solve with its own branches and the FP64 initialisation; receivers
 * without a pick or NaN tobs are left out. T is nzz x max(ncols) scratch. */
static double misfit_f64(int nzz, int nb, const float* S, float dx, float dz, int nshots, const float* sx,
                         const float* sz, const int* c0, const int* ncols, const float* rx, const float* rz,
                         int nrec, const double* tobs, double* T, double* pk)
{
    double J = 0.0;
    for (int b = 0; b < nshots; b++) {
        int sIdx, sIdz;
        orc_source_index(sx[b], sz[b], dx, dz, nb, &sIdx, &sIdz);
        double init[9];
        orc_init_block_f64(S, nzz, sx[b], sz[b], dx, dz, nb, sIdx, sIdz, init);
        const float* Sw = S + (size_t)c0[b] * nzz;
        orc_solve_f64(nzz, ncols[b], Sw, nzz, dx, dz, sIdz, sIdx - c0[b], init, T, 1, 0.0, 1);
        orc_picks_f64(T, nzz, ncols[b], c0[b], dx, dz, nb, rx, rz, nrec, pk);
        for (int r = 0; r < nrec; r++) {
            const double d = pk[r] - tobs[(size_t)b * nrec + r];
            if (d == d) J += 0.5 * d * d;
        }
    }
    return J;
}

double orc_misfit_f64(int nzz, int nxx, int nb, const float* S, float dx, float dz, int nshots, const float* sx,
                      const float* sz, const int* c0, const int* ncols, const float* rx, const float* rz, int nrec,
                      const double* tobs)
{
    (void)nxx;
    int mc = 1;
    for (int b = 0; b < nshots; b++) mc = ncols[b] > mc ? ncols[b] : mc;
    double* T = (double*)malloc(sizeof(double) * (size_t)nzz * mc);
    double* pk = (double*)malloc(sizeof(double) * (nrec > 0 ? nrec : 1));
    const double J = misfit_f64(nzz, nb, S, dx, dz, nshots, sx, sz, c0, ncols, rx, rz, nrec, tobs, T, pk);
    free(T);
    free(pk);
    return J;
}

/* Central finite differences of orc_misfit_f64: for each cell (ci[q], cj[q])
 * of the padded grid, the misfit with that slowness replaced by sp[q] =
 * RN32(s (1 + rel)) and by sm[q] = RN32(s (1 - rel)) (both FP32 values, so
 * the step sp - sm is exact), one (cell, sign) per thread. Returns the
 * threads used. */
int orc_fd_misfit_f64(int nzz, int nxx, int nb, const float* S, float dx, float dz, int nshots, const float* sx,
                      const float* sz, const int* c0, const int* ncols, const float* rx, const float* rz, int nrec,
                      const double* tobs, int ncells, const int* ci, const int* cj, double rel, float* sp,
                      float* sm, double* Jp, double* Jm, int nthreads)
{
    int used = 1;
    int mc = 1;
    for (int b = 0; b < nshots; b++) mc = ncols[b] > mc ? ncols[b] : mc;
    const size_t npad = (size_t)nzz * nxx;
    for (int q = 0; q < ncells; q++) {
        const double s = S[(size_t)ci[q] + (size_t)cj[q] * nzz];
        sp[q] = (float)(s * (1.0 + rel));
        sm[q] = (float)(s * (1.0 - rel));
    }
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    used = nthreads;
#pragma omp parallel num_threads(nthreads)
#endif
    {
        float* Sc = (float*)malloc(sizeof(float) * npad);
        double* T = (double*)malloc(sizeof(double) * (size_t)nzz * mc);
        double* pk = (double*)malloc(sizeof(double) * (nrec > 0 ? nrec : 1));
        memcpy(Sc, S, sizeof(float) * npad);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int t = 0; t < 2 * ncells; t++) {
            const int q = t >> 1;
            const size_t at = (size_t)ci[q] + (size_t)cj[q] * nzz;
            Sc[at] = (t & 1) ? sm[q] : sp[q];
            const double J = misfit_f64(nzz, nb, Sc, dx, dz, nshots, sx, sz, c0, ncols, rx, rz, nrec, tobs, T, pk);
            if (t & 1) Jm[q] = J;
            else Jp[q] = J;
            Sc[at] = S[at];
        }
        free(Sc);
        free(T);
        free(pk);
    }
    return used;
}

/* -------------------------------------------------------------- full shot */

int orc_shot_f32(int nzz, int nxx, int nb, const float* S, float dx, float dz, int c0, int ncols,
                 float sx, float sz, int ani, const uint16_t* const codes[6], const float mm[12],
                 float* T, const float* rx, const float* rz, int nrec, float* picks)
{
    int sIdx, sIdz;
    orc_source_index(sx, sz, dx, dz, nb, &sIdx, &sIdz);
    int sloc = sIdx - c0;
    if (sIdz < 1 || sIdz > nzz - 2 || sloc < 1 || sloc > ncols - 2 || c0 < 0 || c0 + ncols > nxx)
        return -1;
    size_t n = (size_t)nzz * ncols;
    float* Tw = T ? T : (float*)malloc(n * sizeof(float));
    const float* Sw = S + (size_t)c0 * nzz;
    double iv[9];
    float init[9];
    if (g_arith == 1) {
        orc_init_block_f32(S, nzz, sx, sz, dx, dz, nb, sIdx, sIdz, init);
    } else {
        orc_init_block_f64(S, nzz, sx, sz, dx, dz, nb, sIdx, sIdz, iv);
        for (int q = 0; q < 9; q++) init[q] = (float)iv[q];
    }
    /* compensated: the qP pass reads the lo parts of the first solve too */
    float* L = (ani && g_arith == 2) ? (float*)malloc(n * sizeof(float)) : NULL;
    if (L) solve_comp(nzz, ncols, Sw, nzz, dx, dz, sIdz, sloc, init, Tw, L, NULL, NULL, NULL);
    else orc_solve_f32(nzz, ncols, Sw, nzz, dx, dz, sIdz, sloc, init, Tw, 1, 1);
    if (ani) {
        float* Sq = (float*)malloc(n * sizeof(float));
        const uint16_t* cw[6];
        for (int c = 0; c < 6; c++) cw[c] = codes[c] + (size_t)c0 * nzz;
        qslowness_f32(nzz, ncols, nb, Tw, L, Sw, nzz, dx, dz, sIdz, sloc, cw, mm, Sq);
        free(L);
        /* second initialisation reads the qP slowness (eikonal_ani.cu:40-41) */
        for (int b = 0; b < 3; b++)
            for (int a = 0; a < 3; a++) {
                int zi = sIdz + a - 1, xl = sloc + b - 1;
                if (g_arith == 1) {
                    float X = fmaf((float)(xl + c0 - nb), dx, -sx);
                    float Z = fmaf((float)(zi - nb), dz, -sz);
                    init[a + 3 * b] = Sq[zi + (size_t)xl * nzz] * sqrtf(X * X + Z * Z);
                } else {
                    double ddx = (double)(xl + c0 - nb) * (double)dx - (double)sx;
                    double ddz = (double)(zi - nb) * (double)dz - (double)sz;
                    init[a + 3 * b] = (float)((double)Sq[zi + (size_t)xl * nzz] * sqrt(ddx * ddx + ddz * ddz));
                }
            }
        orc_solve_f32(nzz, ncols, Sq, nzz, dx, dz, sIdz, sloc, init, Tw, 1, 1);
        free(Sq);
    }
    if (picks) orc_picks_f32(Tw, nzz, ncols, c0, dx, dz, nb, rx, rz, nrec, picks);
    if (!T) free(Tw);
    return 0;
}

int orc_batch_f32(int nzz, int nxx, int nb, const float* S, float dx, float dz, int nshots,
                  const float* sx, const float* sz, const int* c0, const int* ncols, int ani,
                  const uint16_t* const codes[6], const float mm[12], const float* rx,
                  const float* rz, int nrec, float* picks, int nthreads)
{
    int used = 1;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (int b = 0; b < nshots; b++) {
        orc_shot_f32(nzz, nxx, nb, S, dx, dz, c0[b], ncols[b], sx[b], sz[b], ani, codes, mm, NULL,
                     rx, rz, nrec, picks + (size_t)b * nrec);
    }
#ifdef _OPENMP
    used = nthreads;
#endif
    return used;
}

/* ---------------------------------------------------------------- adjoint */

void orc_solve_tape_f32(int nzz, int ncols, const float* S, int ldS, float dx, float dz, int sIdz,
                        int sIdx_loc, const float init[9], float* T, uint8_t* code, float* c1,
                        float* c2)
{
    if (g_arith == 2) {
        solve_comp(nzz, ncols, S, ldS, dx, dz, sIdz, sIdx_loc, init, T, NULL, code, c1, c2);
        return;
    }
    k32 k = make_k32(dx, dz);
    int si[4], sj[4];
    orc_skip_cells(ncols, nzz, si, sj);
    init_field_f32(T, nzz, ncols, sIdz, sIdx_loc, init);
    memset(code, 0, (size_t)4 * ncols * nzz);
    for (size_t n = 0; n < (size_t)4 * ncols * nzz; n++) c1[n] = c2[n] = 0.0f;
    for (int s = 0; s < 4; s++) {
        int sz, sx;
        sweep_signs(s, &sz, &sx);
        for (int jj = 1; jj <= ncols - 2; jj++) {
            int j = (sx > 0) ? jj : ncols - 1 - jj;
            for (int ii = 1; ii <= nzz - 2; ii++) {
                int i = (sz > 0) ? ii : nzz - 1 - ii;
                if (is_skip(s, i, j, si, sj)) continue;
                rec_t r;
                TAT(i, j) = node32(s, i, j, nzz, ncols, S, ldS, T, &k, &r);
                code[TP(s, i, j)] = (uint8_t)r.code;
                c1[TP(s, i, j)] = (float)r.c1;
                c2[TP(s, i, j)] = (float)r.c2;
            }
        }
    }
}

void orc_solve_tape_f64(int nzz, int ncols, const float* S, int ldS, double dx, double dz, int sIdz,
                        int sIdx_loc, const double init[9], double* T, uint8_t* code, double* c1,
                        double* c2)
{
    k64 k = make_k64(dx, dz);
    int si[4], sj[4];
    orc_skip_cells(ncols, nzz, si, sj);
    init_field_f64(T, nzz, ncols, sIdz, sIdx_loc, init);
    memset(code, 0, (size_t)4 * ncols * nzz);
    for (size_t n = 0; n < (size_t)4 * ncols * nzz; n++) c1[n] = c2[n] = 0.0;
    for (int s = 0; s < 4; s++) {
        int sz, sx;
        sweep_signs(s, &sz, &sx);
        for (int jj = 1; jj <= ncols - 2; jj++) {
            int j = (sx > 0) ? jj : ncols - 1 - jj;
            for (int ii = 1; ii <= nzz - 2; ii++) {
                int i = (sz > 0) ? ii : nzz - 1 - ii;
                if (is_skip(s, i, j, si, sj)) continue;
                rec_t r;
                TAT(i, j) = node64(s, i, j, nzz, ncols, S, NULL, ldS, T, &k, &r);
                code[TP(s, i, j)] = (uint8_t)r.code;
                c1[TP(s, i, j)] = r.c1;
                c2[TP(s, i, j)] = r.c2;
            }
        }
    }
}

/*
 * The FP64 evaluation of a given branch pattern: node (i, j) of sweep s takes
 * the candidate and the slowness cell that code_in names (an FP32 tape's
 * codes), with upd64's formulas; code 0 keeps the old value. The recorded
 * coefficients are upd64's for that candidate. This is the same discrete
 * scheme as the FP32 solve that wrote code_in, evaluated in FP64: its
 * adjoint (orc_adjoint_f64 with code_in) differs from the FP32 adjoint only
 * by FP32 rounding, while an FP64 solve that chooses its own branches also
 * differs wherever near-tied candidates fall the other way. A radicand that
 * rounding has pushed below zero counts as zero.
 */
static double follow64(int cd, double told, double tv, double te, double tev, const float* S, int ldS,
                       int i, int j, const k64* k, double* c1, double* c2)
{
    const int br = cd & 7;
    *c1 = 0.0;
    *c2 = 0.0;
    if (br == 0) return told;
    const double s = SAT(i - 1 + ((cd >> 3) & 1), j - 1 + ((cd >> 4) & 1));
    switch (br) {
    case 1: *c2 = k->dz; return tv + k->dz * s;
    case 2: *c2 = k->dx; return te + k->dx * s;
    case 3: {
        const double D = k->dz2i + k->dx2i;
        const double ta = tev + te - tv, tb = tev - te + tv, dd = ta - tb;
        const double disc = 4.0 * s * s * D - k->dz2i * k->dx2i * dd * dd;
        const double rr = disc > 0.0 ? sqrt(disc) : 0.0;
        if (rr > 0.0) {
            *c1 = ((k->dz2i - k->dx2i) + 2.0 * k->dz2i * k->dx2i * dd / rr) / D;
            *c2 = 4.0 * s / rr;
        } else {
            *c1 = (k->dz2i - k->dx2i) / D;
        }
        return ((tb * k->dz2i + ta * k->dx2i) + rr) / D;
    }
    default: {
        const double hx = (br == 4) ? k->dx : k->dz, hq = (br == 4) ? k->dz : k->dx;
        const double base = (br == 4) ? te : tv;
        const double q = (base - tev) / hq;
        const double arg = s * s - q * q;
        const double qq = arg > 0.0 ? sqrt(arg) : 0.0;
        if (qq > 0.0) {
            *c1 = hx * q / (hq * qq);
            *c2 = hx * s / qq;
        }
        return base + hx * qq;
    }
    }
}

void orc_solve_follow_f64(int nzz, int ncols, const float* S, int ldS, double dx, double dz, int sIdz,
                          int sIdx_loc, const double init[9], const uint8_t* code_in, double* T, double* c1,
                          double* c2)
{
    k64 k = make_k64(dx, dz);
    init_field_f64(T, nzz, ncols, sIdz, sIdx_loc, init);
    for (size_t n = 0; n < (size_t)4 * ncols * nzz; n++) c1[n] = c2[n] = 0.0;
    for (int s = 0; s < 4; s++) {
        int sz, sx;
        sweep_signs(s, &sz, &sx);
        for (int jj = 1; jj <= ncols - 2; jj++) {
            int j = (sx > 0) ? jj : ncols - 1 - jj;
            for (int ii = 1; ii <= nzz - 2; ii++) {
                int i = (sz > 0) ? ii : nzz - 1 - ii;
                const size_t t = TP(s, i, j);
                TAT(i, j) = follow64(code_in[t], TAT(i, j), TAT(i - sz, j), TAT(i, j - sx), TAT(i - sz, j - sx), S,
                                     ldS, i, j, &k, &c1[t], &c2[t]);
            }
        }
    }
}

/*
 * Reverse sweeps in pull form: for sweep k (signs sz, sx), node n = (i, j)
 *   mu(n) = ((lam(n) + pv(i+sz, j)) + pe(i, j+sx)) + pev(i+sz, j+sx)
 * where pv/pe/pev(d) = mu(d) * dT(d)/d{tv,te,tev}; then lam(n) = mu(n) if the
 * node kept its old value (code 0), else 0, and the node's slowness term
 * v = mu(n) * c2 goes to the cell named by the code. Cells gather their terms
 * in the order sweep 0..3, corner (dr,dc) = (0,0),(0,1),(1,0),(1,1), then the
 * 3x3 initialisation term lam_init * dist.
 */
#define ADJ_BODY(REAL)                                                                          \
    size_t npl = (size_t)nzz * ncols;                                                           \
    REAL* pv = (REAL*)calloc(npl, sizeof(REAL));                                                \
    REAL* pe = (REAL*)calloc(npl, sizeof(REAL));                                                \
    REAL* pev = (REAL*)calloc(npl, sizeof(REAL));                                               \
    REAL* vr = (REAL*)calloc(4 * npl, sizeof(REAL));                                            \
    for (int s = 3; s >= 0; s--) {                                                              \
        int sz, sx;                                                                             \
        sweep_signs(s, &sz, &sx);                                                               \
        memset(pv, 0, npl * sizeof(REAL));                                                      \
        memset(pe, 0, npl * sizeof(REAL));                                                      \
        memset(pev, 0, npl * sizeof(REAL));                                                     \
        for (int jj = ncols - 1; jj >= 0; jj--) {                                               \
            int j = (sx > 0) ? jj : ncols - 1 - jj;                                             \
            for (int ii = nzz - 1; ii >= 0; ii--) {                                             \
                int i = (sz > 0) ? ii : nzz - 1 - ii;                                           \
                int id = i + sz, jd = j + sx;                                                   \
                int iok = id >= 0 && id < nzz, jok = jd >= 0 && jd < ncols;                     \
                REAL tpv = iok ? pv[(size_t)id + (size_t)j * nzz] : (REAL)0;                    \
                REAL tpev = (iok && jok) ? pev[(size_t)id + (size_t)jd * nzz] : (REAL)0;        \
                REAL tpe = jok ? pe[(size_t)i + (size_t)jd * nzz] : (REAL)0;                    \
                /* the upwind row's two pushes are summed first (one value per row) */         \
                REAL mu = (lam[(size_t)i + (size_t)j * nzz] + (tpv + tpev)) + tpe;              \
                int cd = code[TP(s, i, j)];                                                     \
                int br = cd & 7;                                                                \
                size_t here = (size_t)i + (size_t)j * nzz;                                      \
                if (br == 0) {                                                                  \
                    lam[here] = mu;                                                             \
                    continue;                                                                   \
                }                                                                               \
                lam[here] = 0;                                                                  \
                REAL a = c1[TP(s, i, j)];                                                       \
                REAL one = 1;                                                                   \
                switch (br) {                                                                   \
                case 1: pv[here] = mu; break;                                                   \
                case 2: pe[here] = mu; break;                                                   \
                case 3: pv[here] = mu * a; pe[here] = mu * (-a); pev[here] = mu; break;         \
                case 4: pe[here] = mu * (one - a); pev[here] = mu * a; break;                   \
                default: pv[here] = mu * (one - a); pev[here] = mu * a; break;                  \
                }                                                                               \
                vr[(size_t)s * npl + here] = mu * c2[TP(s, i, j)];                              \
            }                                                                                   \
        }                                                                                       \
    }                                                                                           \
    for (int b = 0; b < ncols; b++)                                                             \
        for (int a = 0; a < nzz; a++) {                                                         \
            REAL g = grad[(size_t)a + (size_t)b * nzz];                                         \
            for (int s = 0; s < 4; s++)                                                         \
                for (int dr = 0; dr < 2; dr++)                                                  \
                    for (int dc = 0; dc < 2; dc++) {                                            \
                        int i = a + 1 - dr, j = b + 1 - dc;                                     \
                        if (i >= nzz || j >= ncols) continue;                                   \
                        int cd = code[TP(s, i, j)];                                             \
                        if ((cd & 7) && ((cd >> 3) & 1) == dr && ((cd >> 4) & 1) == dc)         \
                            g = g + vr[(size_t)s * npl + (size_t)i + (size_t)j * nzz];          \
                    }                                                                           \
            grad[(size_t)a + (size_t)b * nzz] = g;                                              \
        }                                                                                       \
    for (int b = 0; b < 3; b++)                                                                 \
        for (int a = 0; a < 3; a++) {                                                           \
            size_t n = (size_t)(sIdz + a - 1) + (size_t)(sIdx_loc + b - 1) * nzz;               \
            grad[n] = grad[n] + lam[n] * (REAL)dist[a + 3 * b];                                 \
        }                                                                                       \
    free(pv);                                                                                   \
    free(pe);                                                                                   \
    free(pev);                                                                                  \
    free(vr);

void orc_adjoint_f32(int nzz, int ncols, int sIdz, int sIdx_loc, const uint8_t* code,
                     const float* c1, const float* c2, const float dist[9], float* lam, float* grad)
{
    ADJ_BODY(float)
}

void orc_adjoint_f64(int nzz, int ncols, int sIdz, int sIdx_loc, const uint8_t* code,
                     const double* c1, const double* c2, const double dist[9], double* lam,
                     double* grad)
{
    ADJ_BODY(double)
}

/* ------------------------------------------------- batch misfit gradient */

int orc_batch_gradient_f32(int nzz, int nxx, int nb, const float* S, float dx, float dz, int nshots,
                           const float* sx, const float* sz, const int* c0, const int* ncols,
                           const float* rx, const float* rz, int nrec, const float* tobs,
                           float* picks, double* misfit, float* grad, int nthreads, int ani,
                           const uint16_t* const codes[6], const float mm[12], float* grad_c11,
                           float* grad_c13)
{
    int used = 1;
    size_t* off = (size_t*)malloc(sizeof(size_t) * ((size_t)nshots + 1));
    off[0] = 0;
    for (int b = 0; b < nshots; b++) off[b + 1] = off[b] + (size_t)nzz * ncols[b];
    float* gw = (float*)calloc(off[nshots] ? off[nshots] : 1, sizeof(float));
    /* anisotropic: each shot's dSq/dS, dSq/dC11, dSq/dC13 */
    float* fq = ani ? (float*)malloc(3 * (off[nshots] ? off[nshots] : 1) * sizeof(float)) : NULL;
    int bad = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(| : bad)
#endif
    for (int b = 0; b < nshots; b++) {
        const int nc = ncols[b];
        int sIdx, sIdz;
        orc_source_index(sx[b], sz[b], dx, dz, nb, &sIdx, &sIdz);
        const int sloc = sIdx - c0[b];
        if (sIdz < 1 || sIdz > nzz - 2 || sloc < 1 || sloc > nc - 2 || c0[b] < 0 || c0[b] + nc > nxx) {
            bad |= 1;
            continue;
        }
        const size_t n = (size_t)nzz * nc;
        const float* Sw = S + (size_t)c0[b] * nzz;
        float init[9];
        double iv[9], dist[9];
        if (g_arith == 1) {
            orc_init_block_f32(S, nzz, sx[b], sz[b], dx, dz, nb, sIdx, sIdz, init);
        } else {
            orc_init_block_f64(S, nzz, sx[b], sz[b], dx, dz, nb, sIdx, sIdz, iv);
            for (int q = 0; q < 9; q++) init[q] = (float)iv[q];
        }
        init_dist_f64(nb, sx[b], sz[b], dx, dz, sIdx, sIdz, dist);
        float df[9];
        for (int q = 0; q < 9; q++) df[q] = (float)dist[q];
        float* T = (float*)malloc(n * sizeof(float));
        uint8_t* code = (uint8_t*)malloc(4 * n);
        float* c1 = (float*)malloc(4 * n * sizeof(float));
        float* c2 = (float*)malloc(4 * n * sizeof(float));
        float* lam = (float*)malloc(n * sizeof(float));
        float* pg = (float*)malloc(sizeof(float) * (nrec > 0 ? nrec : 1));
        if (ani) {
            /* first solve untaped, qP pass and its derivative factors, then the
             * second (qP) solve taped; its initial values read the qP field */
            float* fS = fq + off[b];
            float* Sq = (float*)malloc(n * sizeof(float));
            const uint16_t* cw[6];
            for (int q = 0; q < 6; q++) cw[q] = codes[q] + (size_t)c0[b] * nzz;
            float* L = (g_arith == 2) ? (float*)malloc(n * sizeof(float)) : NULL;
            if (L) solve_comp(nzz, nc, Sw, nzz, dx, dz, sIdz, sloc, init, T, L, NULL, NULL, NULL);
            else orc_solve_f32(nzz, nc, Sw, nzz, dx, dz, sIdz, sloc, init, T, 1, 1);
            qslowness_f32(nzz, nc, nb, T, L, Sw, nzz, dx, dz, sIdz, sloc, cw, mm, Sq);
            qp_factors_all(nzz, nc, nb, T, L, Sw, nzz, dx, dz, sIdz, sloc, cw, mm, fS, fS + off[nshots],
                           fS + 2 * off[nshots]);
            free(L);
            for (int bb = 0; bb < 3; bb++)
                for (int a = 0; a < 3; a++) {
                    int zi = sIdz + a - 1, xl = sloc + bb - 1;
                    if (g_arith == 1) {
                        float X = fmaf((float)(xl + c0[b] - nb), dx, -sx[b]);
                        float Z = fmaf((float)(zi - nb), dz, -sz[b]);
                        init[a + 3 * bb] = Sq[zi + (size_t)xl * nzz] * sqrtf(X * X + Z * Z);
                    } else {
                        init[a + 3 * bb] = (float)((double)Sq[zi + (size_t)xl * nzz] * dist[a + 3 * bb]);
                    }
                }
            orc_solve_tape_f32(nzz, nc, Sq, nzz, dx, dz, sIdz, sloc, init, T, code, c1, c2);
            free(Sq);
        } else {
            orc_solve_tape_f32(nzz, nc, Sw, nzz, dx, dz, sIdz, sloc, init, T, code, c1, c2);
        }
        float* pk = picks + (size_t)b * nrec;
        orc_picks_f32(T, nzz, nc, c0[b], dx, dz, nb, rx, rz, nrec, pk);
        for (int r = 0; r < nrec; r++) pg[r] = pk[r] - tobs[(size_t)b * nrec + r]; /* NaN: no pick */
        orc_seed_lambda_f32(nzz, nc, c0[b], dx, dz, nb, rx, rz, nrec, pg, lam);
        orc_adjoint_f32(nzz, nc, sIdz, sloc, code, c1, c2, df, lam, gw + off[b]);
        free(T); free(code); free(c1); free(c2); free(lam); free(pg);
    }
#ifdef _OPENMP
    used = nthreads;
#endif
    /* shot gradients summed in FP64 in caller order; misfit over (shot, receiver) */
    double* acc = (double*)calloc((size_t)nzz * nxx * (ani ? 3 : 1), sizeof(double));
    double J = 0.0;
    for (int b = 0; b < nshots; b++) {
        const size_t base = (size_t)c0[b] * nzz;
        const size_t npad = (size_t)nzz * nxx;
        for (size_t q = 0; q < off[b + 1] - off[b]; q++) {
            if (ani) {
                /* the shot's gradient with respect to its qP field times the factors */
                const double gq = (double)gw[off[b] + q];
                acc[base + q] += gq * (double)fq[off[b] + q];
                acc[npad + base + q] += gq * (double)fq[off[nshots] + off[b] + q];
                acc[2 * npad + base + q] += gq * (double)fq[2 * off[nshots] + off[b] + q];
            } else {
                acc[base + q] += (double)gw[off[b] + q];
            }
        }
        for (int r = 0; r < nrec; r++) {
            /* the residual is the FP32 pick gradient; its square is summed in FP64 */
            double d = (double)(picks[(size_t)b * nrec + r] - tobs[(size_t)b * nrec + r]);
            if (d == d) J += 0.5 * d * d;
        }
    }
    for (size_t q = 0; q < (size_t)nzz * nxx; q++) grad[q] = (float)acc[q];
    if (ani)
        for (size_t q = 0; q < (size_t)nzz * nxx; q++) {
            grad_c11[q] = (float)acc[(size_t)nzz * nxx + q];
            grad_c13[q] = (float)acc[2 * (size_t)nzz * nxx + q];
        }
    if (misfit) *misfit = J;
    free(acc);
    free(fq);
    free(gw);
    free(off);
    return bad ? -1 : used;
}

/* ---------------------------------------------------- tomography update */

#define ORC_PI 3.14159265358979323846 /* M_PI of the reference's math.h */

/* Inversion::smooth_matrix's kernel (src/inversion/inversion.cpp:387-418):
 * the prefactor 1/(M_PI*stdv) in double, expf of a float argument, the
 * product rounded once to float; FP32 sum (x outer, z inner); division by it. */
void orc_smooth_kernel(float stdv, int n, float* k)
{
    int mid = n / 2;
    for (int q = 0; q < n * n; q++) k[q] = 0.0f;
    k[mid + mid * n] = 1.0f;
    if (stdv == 0.0f) return;
    float sum = 0.0f;
    for (int x = -mid; x <= mid; x++)
        for (int z = -mid; z <= mid; z++) {
            int index = (z + mid) + (x + mid) * n;
            float r = sqrtf((float)(x * x + z * z));
            k[index] = (float)(1.0f / (ORC_PI * stdv) * (double)expf(-((r * r) / (2.0f * stdv * stdv))));
            sum += k[index];
        }
    for (int q = 0; q < n * n; q++) k[q] /= sum;
}

/* Inversion::model_smoothing + smooth_matrix (inversion.cpp:347-447) as
 * written: the model (nz x nx) copied into a zero grid padded by `samples`
 * cells, the padded grid smoothed where the kernel fits (FP32, xk outer, zk
 * inner, product then sum), the model window copied back. */
void orc_model_smoothing(const float* model, int nx, int nz, float stdv, int samples, float* out)
{
    int anx = nx + 2 * samples, anz = nz + 2 * samples;
    size_t an = (size_t)anx * anz;
    float* aux = (float*)calloc(an, sizeof(float));
    float* sm = (float*)calloc(an, sizeof(float));
    float* k = (float*)malloc(sizeof(float) * (size_t)samples * samples);
    for (int j = 0; j < nx; j++)
        for (int i = 0; i < nz; i++) aux[(i + samples) + (size_t)(j + samples) * anz] = model[i + (size_t)j * nz];
    orc_smooth_kernel(stdv, samples, k);
    for (size_t q = 0; q < an; q++) sm[q] = aux[q];
    int mid = samples / 2;
    for (int j = mid; j < anx - mid; j++)
        for (int i = mid; i < anz - mid; i++) {
            float accum = 0.0f;
            for (int xk = 0; xk < samples; xk++)
                for (int zk = 0; zk < samples; zk++) {
                    float prod = aux[(i - mid + zk) + (size_t)(j - mid + xk) * anz] * k[zk + xk * samples];
                    accum = accum + prod;
                }
            sm[i + (size_t)j * anz] = accum;
        }
    for (int j = 0; j < nx; j++)
        for (int i = 0; i < nz; i++) out[i + (size_t)j * nz] = sm[(i + samples) + (size_t)(j + samples) * anz];
    free(aux);
    free(sm);
    free(k);
}

/* Tomography_ISO::model_update (tomography_iso.cpp:77-92) on a padded
 * slowness S (nzz x nxx): dS = scale * grad over the model interior,
 * smoothed unless samples == 0, added to the interior; dS returned. */
void orc_update_slowness(float* S, const float* grad, int nx, int nz, int nb, float scale, float stdv,
                         int samples, float* dS)
{
    int nzz = nz + 2 * nb;
    float* d = (float*)malloc(sizeof(float) * (size_t)nx * nz);
    for (int j = 0; j < nx; j++)
        for (int i = 0; i < nz; i++) d[i + (size_t)j * nz] = scale * grad[(i + nb) + (size_t)(j + nb) * nzz];
    if (samples != 0) orc_model_smoothing(d, nx, nz, stdv, samples, dS);
    else memcpy(dS, d, sizeof(float) * (size_t)nx * nz);
    for (int j = 0; j < nx; j++)
        for (int i = 0; i < nz; i++) S[(i + nb) + (size_t)(j + nb) * nzz] += dS[i + (size_t)j * nz];
    free(d);
}

/* ------------------------------------------------------------- Kirchhoff */

/* Migration::set_wavelet (src/migration/migration.cu:54-71) as written: the
 * offsets and the centre frequency in float, the phase term in double, expf
 * of it rounded to float. Returns nw; w must hold it (nw <= wmax). */
int orc_kirchhoff_wavelet(float fmax, float dt, float* w, int wmax)
{
    float t0 = 2.0f * sqrtf((float)ORC_PI) / fmax;
    float fc = fmax / (3.0f * sqrtf((float)ORC_PI));
    int nw = 2 * ((int)((t0 - 0.5f * dt) / dt));
    if (nw > wmax) return -nw;
    for (int k = 0; k < nw; k++) {
        float td = k * dt - t0;
        float arg = (float)(ORC_PI * ORC_PI * ORC_PI * fc * fc * td * td);
        w[k] = (1.0f - 2.0f * arg) * expf(-arg);
    }
    return nw;
}

/* Migration::adjoint_convolution (migration.cu:197-228) without the FFT: the
 * product A conj(B) of the zero-padded spectra and FFTW's unnormalised
 * inverse are the linear cross-correlation times nfft (nfft >= nt + nw - 1),
 * summed here directly in FP64; out[t] for t >= nw/2 + nw/10, else 0. */
void orc_adjoint_convolution(const float* in, float* out, int ntr, int nt, const float* w, int nw)
{
    int nfft = 1;
    while (nfft < nt + nw - 1) nfft <<= 1;
    int shift = nw / 2 + nw / 10;
    for (int q = 0; q < ntr; q++) {
        const float* a = in + (size_t)q * nt;
        float* o = out + (size_t)q * nt;
        for (int t = 0; t < nt; t++) {
            if (t < shift) {
                o[t] = 0.0f;
                continue;
            }
            int l = t - shift;
            double acc = 0.0;
            for (int m = 0; m < nw && l + m < nt; m++) acc += (double)a[l + m] * (double)w[m];
            o[t] = (float)(acc * (double)nfft);
        }
    }
}

/* The reference accumulates with a float atomicAdd, which flushes subnormal
 * operands and results to zero (sign kept). */
static float ftz(float x) { return fabsf(x) < FLT_MIN ? copysignf(0.0f, x) : x; }

/* One cell's Kirchhoff weight and reflection angle (degrees), as the
 * reference's four kernels compute them (migration.cu:418-466, :505-553,
 * :592-645, :685-738), FP32 with libm functions (the GPU uses CUDA's;
 * agreement is to rounding). */
static float orc_kweight(const float* S, const float* ts, const float* tr, int i, int j, int nzz, int nb, float dx,
                         float dz, float aperture, float cmp, float* ang_deg)
{
    const float EPSK = 1e-6f;
    size_t index = (size_t)i + (size_t)j * nzz;
    float z = (float)(i - nb) * dz, x = (float)(j - nb) * dx;
#define ORC_D(A)                                                                                      \
    float A##_dz = 0.5f * (A[(i + 1) + j * nzz] - A[(i - 1) + j * nzz]) / dz;                        \
    float A##_dx = 0.5f * (A[i + (j + 1) * nzz] - A[i + (j - 1) * nzz]) / dx;                        \
    float A##_dz2 = (A[(i + 1) + j * nzz] - 2.0f * A[i + j * nzz] + A[(i - 1) + j * nzz]) / (dz * dz); \
    float A##_dx2 = (A[i + (j + 1) * nzz] - 2.0f * A[i + j * nzz] + A[i + (j - 1) * nzz]) / (dx * dx); \
    float A##_dxdz = (A[(i + 1) + (j + 1) * nzz] - A[(i - 1) + (j + 1) * nzz] - A[(i + 1) + (j - 1) * nzz] + \
                      A[(i - 1) + (j - 1) * nzz]) / (4.0f * dx * dz);
    ORC_D(ts)
    ORC_D(tr)
#undef ORC_D
    float norm_s = sqrtf(ts_dx * ts_dx + ts_dz * ts_dz) + EPSK;
    float norm_r = sqrtf(tr_dx * tr_dx + tr_dz * tr_dz) + EPSK;
    float detHs = fabsf(ts_dx2 * ts_dz2 - ts_dxdz * ts_dxdz) + EPSK;
    float detHr = fabsf(tr_dx2 * tr_dz2 - tr_dxdz * tr_dxdz) + EPSK;
    float Jterm = sqrtf(detHs * detHr) * S[index] / (norm_s * norm_r);
    float ux_s = ts_dx / norm_s, uz_s = ts_dz / norm_s;
    float ux_r = tr_dx / norm_r, uz_r = tr_dz / norm_r;
    float nxn = 0.0f, nzn = -1.0f;
    float cos_s = fabsf(ux_s * nxn + uz_s * nzn);
    float cos_r = fabsf(ux_r * nxn + uz_r * nzn);
    float obl = sqrtf(fmaxf(0.0f, cos_s) * fmaxf(0.0f, cos_r));
    float R_s = fmaxf(ts[index] / S[index], EPSK);
    float R_r = fmaxf(tr[index] / S[index], EPSK);
    float G = 1.0f / sqrtf(R_s * R_r);
    float th_s = acosf(fminf(1.0f, fmaxf(-1.0f, ux_s * nxn + uz_s * nzn)));
    float th_r = acosf(fminf(1.0f, fmaxf(-1.0f, ux_r * nxn + uz_r * nzn)));
    float R = 1.0f + 0.2f * cosf(0.5f * (th_s + th_r));
    float scale_const = (float)(1.0f / (2.0f * ORC_PI));
    float sigma = tanf((float)(aperture * ORC_PI / 180.0f)) * z;
    float u = (x - cmp) / (sigma + EPSK);
    float taper = expf(-0.5f * u * u);
    if (ang_deg) {
        float refl = 0.5f * acosf((ts_dx * tr_dx + ts_dz * tr_dz) / (norm_s * norm_r));
        *ang_deg = (float)(180.0f * refl / ORC_PI);
    }
    return scale_const * Jterm * obl * G * R * taper;
}

/* KDM::kirchhoff_depth_migration + image_domain_adjoint_kernel
 * (KDM.cu:3-55, migration.cu:398-483): for every source, every receiver
 * within max_offset (in that order), every model cell with T = Ts + Tr below
 * nt*dt: image += weight * trace[floor(T/dt)], FP32. */
void orc_kirchhoff_image(int nxx, int nzz, int nb, const float* S, const float* Ts, const float* Tr, int nsrc,
                         int nrec, const float* xsrc, const float* xrec, const float* data, int nt, float dt,
                         float dx, float dz, float aperture, float max_offset, float* image)
{
    size_t matsize = (size_t)nxx * nzz;
    int nz = nzz - 2 * nb, nx = nxx - 2 * nb;
    for (size_t q = 0; q < (size_t)nx * nz; q++) image[q] = 0.0f;
    for (int s = 0; s < nsrc; s++)
        for (int r = 0; r < nrec; r++) {
            float offset = fabsf(xsrc[s] - xrec[r]);
            if (!(offset < max_offset)) continue;
            float cmp = 0.5f * (xsrc[s] + xrec[r]);
            const float* ts = Ts + matsize * s;
            const float* tr = Tr + matsize * r;
            const float* trace = data + ((size_t)s * nrec + r) * nt;
            for (int j = nb; j < nxx - nb; j++)
                for (int i = nb; i < nzz - nb; i++) {
                    size_t index = (size_t)i + (size_t)j * nzz;
                    float T = ts[index] + tr[index];
                    int tId = (int)floorf(T / dt);
                    if (tId >= nt) continue;
                    float wgt = orc_kweight(S, ts, tr, i, j, nzz, nb, dx, dz, aperture, cmp, NULL);
                    size_t mId = (size_t)(i - nb) + (size_t)(j - nb) * nz;
                    image[mId] = ftz(ftz(image[mId]) + ftz(wgt * trace[tId]));
                }
        }
}

/* The least-squares variants' forward operators (image_domain_forward_kernel,
 * migration.cu:485-570, nang = 0; angle_domain_forward_kernel, :665-756,
 * nang > 0 with model = gathers nz x nang x ncmp): for every source, every
 * receiver within max_offset, every cell with floor((Ts + Tr)/dt) in
 * [0, nt) (and its reflection-angle bin in [0, nang)), trace sample += the
 * FP32 product weight * model value. The reference adds with atomics in no
 * fixed order; here each sample's terms are summed in FP64 and rounded once,
 * an order-free value every FP32 summation order approximates. */
void orc_kirchhoff_forward(int nxx, int nzz, int nb, const float* S, const float* Ts, const float* Tr, int nsrc,
                           int nrec, const float* xsrc, const float* xrec, const float* model, int nt, float dt,
                           float dx, float dz, float aperture, float max_offset, int nang, float da, float mincmp,
                           float dcmp, float* data)
{
    size_t matsize = (size_t)nxx * nzz;
    int nz = nzz - 2 * nb;
    double* acc = (double*)malloc(sizeof(double) * (size_t)(nt > 0 ? nt : 1));
    for (int s = 0; s < nsrc; s++)
        for (int r = 0; r < nrec; r++) {
            float* out = data + ((size_t)s * nrec + r) * nt;
            for (int t = 0; t < nt; t++) out[t] = 0.0f;
            float offset = fabsf(xsrc[s] - xrec[r]);
            if (!(offset < max_offset)) continue;
            float cmp = 0.5f * (xsrc[s] + xrec[r]);
            int cmpId = nang > 0 ? (int)((cmp - mincmp) / dcmp) : 0;
            const float* ts = Ts + matsize * s;
            const float* tr = Tr + matsize * r;
            for (int t = 0; t < nt; t++) acc[t] = 0.0;
            for (int j = nb; j < nxx - nb; j++)
                for (int i = nb; i < nzz - nb; i++) {
                    size_t index = (size_t)i + (size_t)j * nzz;
                    float T = ts[index] + tr[index];
                    int tId = (int)floorf(T / dt);
                    if (tId < 0 || tId >= nt) continue;
                    float ang = 0.0f;
                    float wgt = orc_kweight(S, ts, tr, i, j, nzz, nb, dx, dz, aperture, cmp, nang > 0 ? &ang : NULL);
                    size_t mId = (size_t)(i - nb) + (size_t)(j - nb) * nz;
                    if (nang > 0) {
                        int aId = (int)floorf(ang / da);
                        if (aId < 0 || aId >= nang) continue;
                        mId = (size_t)(i - nb) + (size_t)aId * nz + (size_t)cmpId * nang * nz;
                    }
                    acc[tId] += (double)ftz(wgt * model[mId]);
                }
            for (int t = 0; t < nt; t++) out[t] = (float)acc[t];
        }
    free(acc);
}

/* Migration::forward_convolution (migration.cu:230-261) without the FFT: the
 * product A B of the zero-padded spectra and FFTW's unnormalised inverse are
 * the linear convolution times nfft; out[t] = that at t + nw/2 + nw/10,
 * summed directly in FP64 (m ascending). */
void orc_forward_convolution(const float* in, float* out, int ntr, int nt, const float* w, int nw)
{
    int nfft = 1;
    while (nfft < nt + nw - 1) nfft <<= 1;
    int shift = nw / 2 + nw / 10;
    for (int q = 0; q < ntr; q++) {
        const float* a = in + (size_t)q * nt;
        float* o = out + (size_t)q * nt;
        for (int t = 0; t < nt; t++) {
            int c = t + shift;
            double acc = 0.0;
            for (int m = (c - nt + 1 > 0 ? c - nt + 1 : 0); m < nw && m <= c; m++)
                acc += (double)a[c - m] * (double)w[m];
            o[t] = (float)(acc * (double)nfft);
        }
    }
}
