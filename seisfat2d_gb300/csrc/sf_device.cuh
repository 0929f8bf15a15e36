// Device-side building blocks of the GB300 eikonal engine: the per-node
// fast-sweeping update, the anisotropic qP slowness, the receiver rule and the
// FP64 near-source initialisation.
//
// Every FP32 operation is written with an explicit round-to-nearest intrinsic
// (__fadd_rn, __fmul_rn, ...). Those are never contracted into FMAs, so the
// result of each node is exactly the IEEE evaluation of the reference source
// expression in source order (src/modeling/modeling.cu:319-356), independent
// of compiler flags and identical to the CPU oracle built with
// -ffp-contract=off.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sf {

constexpr float kBig = 1e6f;  // time_set sentinel (modeling.cu:290)

struct Consts {
    float dx, dz;
    float dx2i, dz2i;  // 1/(dx*dx), 1/(dz*dz) rounded as modeling.cu:64-65
    float hyp;         // sqrtf(dx*dx + dz*dz)
    float D;           // dz2i + dx2i
    float K;           // dz2i * dx2i
    float kA;          // dz2i - dx2i      (tape coefficient)
    float kB;          // dx2i - dz2i      (compensated 2D increment)
    float k2K;         // 2 * (dz2i*dx2i)  (tape coefficient)
    // correctly rounded reciprocals of the four divisors and, per divisor, whether
    // Markstein's correction step has been verified to equal IEEE division for
    // every finite dividend (bit 0 dx, 1 dz, 2 hyp, 3 D)
    float rdx, rdz, rhyp, rD;
    int mflags;
};

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

// a / b for one of the context's constant divisors b with reciprocal rb =
// RN(1/b): Markstein's correction step (P. Markstein, IBM J. Res. Dev. 34,
// 1990): q = RN(a rb), r = a - b q exactly (one FMA), q' = RN(q + r rb).
// Every step scales exactly with a by powers of two while all values stay
// normal, so checking the 2^23 dividends of [1, 2) against IEEE division
// (done per divisor when a context is created) covers every dividend of
// magnitude in [2^-100, 2^100]. EXACT (or an unverified divisor) divides.
// Otherwise a dividend outside that range (or NaN) sets `bad`, and the
// caller recomputes the node with EXACT: the check stays a compare, and the
// rare exact path is one warp-uniform branch per step instead of a branch
// per division.
template <bool EXACT>
__device__ __forceinline__ float fdiv_k(float a, float b, float rb, bool verified, bool& bad)
{
    if (EXACT) return __fdiv_rn(a, b);
    bad |= !verified || (__float_as_uint(a) & 0x7f800000u) - 0x0d800000u > 0x64000000u;  // exponent not in [27, 227]
    const float q = __fmul_rn(a, rb);
    const float r = __fmaf_rn(-q, b, a);
    return __fmaf_rn(r, rb, q);
}

// Tape record of one node (adjoint bookkeeping; see the tape description in
// include/seisfat2d.h). code bits 0-2 candidate, 3 row code, 4 column code.
struct Rec {
    uint8_t code;
    float c1, c2;
};

// One node update. REF selects the reference build's arithmetic: nvcc
// contracts seven multiply-adds of inner_sweep into FMAs (t1d1, t1d2, the 2D
// numerator tb*dz2i + ta*dx2i, the discriminant 4 Sref^2 D - K dd^2, and in
// the edge updates Sref^2 - q^2 and te/tv + h*sqrt(..)); with REF false every
// operation rounds once. s1a/s1b: cells of the vertical upwind edge (row i1,
// columns max(j-1,1) and j); s2a/s2b: cells of the horizontal edge (rows
// max(i-1,1) and i, column j1); sref = S[i1][j1]. dr1/dc2 locate i1/j1 in the
// 2x2 block around the node, dc1a/dr2a locate the clamped first cells.
// SQ: square cells (dx and dz equal as floats). Then the two edge
// thresholds are one quotient and the step constants need no per-node
// selection; every value is the one the general form computes.
template <bool TAPE, bool REF, bool EXACT = false, bool SQ = false>
__device__ __forceinline__ float node_update(float told, float tv, float te, float tev, float s1a,
                                             float s1b, float s2a, float s2b, float sref,
                                             const Consts& k, int dr1, int dc1a, int dc2, int dr2a,
                                             Rec& rec, bool& bad)
{
    float m1 = fminf(s1a, s1b);
    float m2 = fminf(s2a, s2b);
    float t1d1 = REF ? __fmaf_rn(k.dz, m1, tv) : fadd(tv, fmul(k.dz, m1));
    float t1d2 = REF ? __fmaf_rn(k.dx, m2, te) : fadd(te, fmul(k.dx, m2));
    float t1D = fminf(t1d1, t1d2);
    const float dte = fsub(te, tev);
    const float dtv = fsub(tv, tev);
    // The 2D candidate (modeling.cu:328-339) and the edge candidates (:342-353)
    // through one code path, so that the lanes of a warp do not diverge: the
    // edge update divides first, then takes a root; the 2D one takes a root,
    // then divides. Each lane selects the operands of the candidate the
    // reference's branches would take (same operations, same bits); the
    // operations of the other candidate get operands that keep them on their
    // fast paths.
    const float dxs = fmul(k.dx, sref);
    const float dzs = SQ ? dxs : fmul(k.dz, sref);
    const bool c2d = (tv <= fadd(te, dxs)) && (te <= fadd(tv, dzs)) && (dte >= 0.0f) && (dtv >= 0.0f);
    const float thz = fdiv_k<EXACT>(fmul(fmul(sref, k.dz), k.dz), k.hyp, k.rhyp, k.mflags & 4, bad);
    const float thx = SQ ? thz : fdiv_k<EXACT>(fmul(fmul(sref, k.dx), k.dx), k.hyp, k.rhyp, k.mflags & 4, bad);
    const bool c2 = !c2d && (dte <= thz) && (dte > 0.0f);        // t2: from te, step dz
    const bool c3 = !c2d && !c2 && (dtv <= thx) && (dtv > 0.0f);  // t3: from tv, step dx
    const bool ce = c2 || c3;
    const float hq = SQ ? k.dz : (c2 ? k.dz : k.dx);  // step the difference is divided by
    const float rq = SQ ? k.rdz : (c2 ? k.rdz : k.rdx);
    const bool vq = SQ ? (k.mflags & 2) : (c2 ? (k.mflags & 2) : (k.mflags & 1));
    const float hx = SQ ? k.dz : (c2 ? k.dx : k.dz);  // step that multiplies the root
    const float bs = c2 ? te : tv;
    const float qe = fdiv_k<EXACT>(ce ? (c2 ? dte : dtv) : hq, hq, rq, vq, bad);
    const float ta = fsub(fadd(tev, te), tv);
    const float tb = fadd(fsub(tev, te), tv);
    const float dde = fsub(ta, tb);
    float disc, earg, num0;
    if (REF) {
        disc = __fmaf_rn(fmul(fmul(4.0f, sref), sref), k.D, -fmul(fmul(k.K, dde), dde));
        earg = __fmaf_rn(-qe, qe, fmul(sref, sref));
        num0 = __fmaf_rn(tb, k.dz2i, fmul(ta, k.dx2i));
    } else {
        disc = fsub(fmul(fmul(fmul(4.0f, sref), sref), k.D), fmul(fmul(k.K, dde), dde));
        earg = fsub(fmul(sref, sref), fmul(qe, qe));
        num0 = fadd(fmul(tb, k.dz2i), fmul(ta, k.dx2i));
    }
    const float root = fsqrt(c2d ? disc : (ce ? earg : 1.0f));
    const float t1v = fdiv_k<EXACT>(c2d ? fadd(num0, root) : k.D, k.D, k.rD, k.mflags & 8, bad);
    const float tq = REF ? __fmaf_rn(hx, root, bs) : fadd(bs, fmul(hx, root));
    const float t1 = c2d ? t1v : kBig;
    const float t2 = c2 ? tq : kBig;
    const float t3 = c3 ? tq : kBig;
    const int br = c2d ? 3 : (c2 ? 4 : (c3 ? 5 : 0));
    const float rr = c2d ? root : 0.0f, dd = c2d ? dde : 0.0f;
    const float q = ce ? qe : 0.0f, qq = ce ? root : 0.0f;
    float t2D = fminf(t1, fminf(t2, t3));
    float cand = fminf(t1D, t2D);
    float tnew = fminf(told, cand);
    if (TAPE) {
        rec.code = 0;
        rec.c1 = 0.0f;
        rec.c2 = 0.0f;
        if (cand < told) {
            if (t1D <= t2D) {
                if (t1d1 <= t1d2) {
                    int dc = (s1a <= s1b) ? dc1a : 1;
                    rec.code = (uint8_t)(1 | (dr1 << 3) | (dc << 4));
                    rec.c2 = k.dz;
                } else {
                    int dr = (s2a <= s2b) ? dr2a : 1;
                    rec.code = (uint8_t)(2 | (dr << 3) | (dc2 << 4));
                    rec.c2 = k.dx;
                }
            } else if (br != 0) {
                rec.code = (uint8_t)(br | (dr1 << 3) | (dc2 << 4));
                if (br == 3) {
                    if (rr > 0.0f) {
                        rec.c1 = fdiv_k<EXACT>(fadd(k.kA, fdiv(fmul(k.k2K, dd), rr)), k.D, k.rD, k.mflags & 8, bad);
                        rec.c2 = fdiv(fmul(4.0f, sref), rr);
                    } else {
                        rec.c1 = fdiv_k<EXACT>(k.kA, k.D, k.rD, k.mflags & 8, bad);
                    }
                } else {
                    float hx = SQ ? k.dz : ((br == 4) ? k.dx : k.dz);
                    float hq = SQ ? k.dz : ((br == 4) ? k.dz : k.dx);
                    if (qq > 0.0f) {
                        rec.c1 = fdiv(fmul(hx, q), fmul(hq, qq));
                        rec.c2 = fdiv(fmul(hx, sref), qq);
                    }
                }
            }
        }
    }
    return tnew;
}

// Compensated update (SF_ARITH_COMPENSATED; no counterpart in the
// reference). Traveltimes are unevaluated sums hi + lo of two FP32 values.
// Every decision and increment of the update depends only on differences of
// the upwind times, so these are formed from the pairs, (a.h - b.h) + (a.l -
// b.l), and the candidates are compared in FP32 next to a nearby finite time
// (the two 1D ones next to te, the 1D and the 2D or edge winner next to tev,
// the winner and the old value next to the winner's base), never next to
// the 1e6 sentinel; the winner is its base time plus its FP32 increment,
// added with Knuth's TwoSum and renormalised with Dekker's Fast2Sum. A node's rounding error is then
// relative to its increment instead of its time and does not accumulate
// along the sweep. Same candidates, branch tests, tape codes and coefficient
// formulas as node_update; each operation rounded once, in the order of the
// oracle's restatement (updc in oracle/eikonal_oracle.c).
__device__ __forceinline__ void ff_add(float ah, float al, float b, float& h, float& l)
{
    const float s = fadd(ah, b), bb = fsub(s, ah);
    const float e = fadd(fsub(ah, fsub(s, bb)), fsub(b, bb));
    const float t = fadd(e, al);
    h = fadd(s, t);
    l = fsub(t, fsub(h, s));
}
__device__ __forceinline__ float ff_diff(float ah, float al, float bh, float bl)
{
    return fadd(fsub(ah, bh), fsub(al, bl));
}

template <bool TAPE, bool EXACT = false, bool SQ = false>
__device__ __forceinline__ void node_update_comp(float toh, float tol, float tvh, float tvl, float teh, float tel,
                                                 float tevh, float tevl, float s1a, float s1b, float s2a, float s2b,
                                                 float sref, const Consts& k, int dr1, int dc1a, int dc2, int dr2a,
                                                 float& oh, float& ol, Rec& rec, bool& bad)
{
    const float dte = ff_diff(teh, tel, tevh, tevl);
    const float dtv = ff_diff(tvh, tvl, tevh, tevl);
    const float dvt = ff_diff(tvh, tvl, teh, tel);
    const float m1 = fminf(s1a, s1b), m2 = fminf(s2a, s2b);
    const float i1 = fmul(k.dz, m1), i2 = fmul(k.dx, m2);  // t1d1 = tv + i1, t1d2 = te + i2
    const bool w11 = fadd(dvt, i1) <= i2;                  // t1d1 <= t1d2, compared next to te
    const float o1D = w11 ? fadd(dtv, i1) : fadd(dte, i2); // the 1D winner's offset to tev
    const float dxs = fmul(k.dx, sref);
    const float dzs = SQ ? dxs : fmul(k.dz, sref);
    const bool c2d = (dvt <= dxs) && (-dvt <= dzs) && (dte >= 0.0f) && (dtv >= 0.0f);
    const float thz = fdiv_k<EXACT>(fmul(fmul(sref, k.dz), k.dz), k.hyp, k.rhyp, k.mflags & 4, bad);
    const float thx = SQ ? thz : fdiv_k<EXACT>(fmul(fmul(sref, k.dx), k.dx), k.hyp, k.rhyp, k.mflags & 4, bad);
    const bool c2 = !c2d && (dte <= thz) && (dte > 0.0f);        // t2: from te, step dz
    const bool c3 = !c2d && !c2 && (dtv <= thx) && (dtv > 0.0f);  // t3: from tv, step dx
    const bool ce = c2 || c3;
    // one root for the 2D and the edge candidates (operands selected per lane)
    const float hq = SQ ? k.dz : (c2 ? k.dz : k.dx);
    const float rq = SQ ? k.rdz : (c2 ? k.rdz : k.rdx);
    const bool vq = SQ ? (k.mflags & 2) : (c2 ? (k.mflags & 2) : (k.mflags & 1));
    const float hx = SQ ? k.dz : (c2 ? k.dx : k.dz);
    const float dq = c2 ? dte : dtv;
    const float qe = fdiv_k<EXACT>(ce ? dq : hq, hq, rq, vq, bad);
    const float dd = fmul(-2.0f, dvt);  // ta - tb = 2 (te - tv)
    const float disc = fsub(fmul(fmul(fmul(4.0f, sref), sref), k.D), fmul(fmul(k.K, dd), dd));
    const float earg = fsub(fmul(sref, sref), fmul(qe, qe));
    const float root = fsqrt(c2d ? disc : (ce ? earg : 1.0f));
    const float o3v = fdiv_k<EXACT>(c2d ? fsub(root, fmul(dvt, k.kB)) : k.D, k.D, k.rD, k.mflags & 8, bad);
    const float inc = ce ? fmul(hx, root) : 0.0f;
    const float o3 = c2d ? o3v : kBig;
    const float oq = fadd(dq, inc);
    const float o4 = c2 ? oq : kBig;
    const float o5 = c3 ? oq : kBig;
    // a 2D or edge candidate needs tev close to its base, so both winners'
    // offsets to tev are exact enough to compare
    const float o2D = fminf(o3, fminf(o4, o5));
    const int br = c2d ? 3 : (c2 ? 4 : (c3 ? 5 : 0));
    // the winner's base and increment
    const bool w1 = o1D <= o2D;
    float bh, bl, bi;
    if (w1) {
        bh = w11 ? tvh : teh;
        bl = w11 ? tvl : tel;
        bi = w11 ? i1 : i2;
    } else {
        bh = (br == 3) ? tevh : (br == 4 ? teh : tvh);
        bl = (br == 3) ? tevl : (br == 4 ? tel : tvl);
        bi = (br == 3) ? o3v : inc;
    }
    // the candidate replaces told when it is smaller, compared next to its base
    const bool upd = bi < ff_diff(toh, tol, bh, bl);
    float nh, nl;
    ff_add(bh, bl, bi, nh, nl);
    oh = upd ? nh : toh;
    ol = upd ? nl : tol;
    if (TAPE) {
        rec.code = 0;
        rec.c1 = 0.0f;
        rec.c2 = 0.0f;
        if (upd) {
            if (w1) {
                if (w11) {
                    int dc = (s1a <= s1b) ? dc1a : 1;
                    rec.code = (uint8_t)(1 | (dr1 << 3) | (dc << 4));
                    rec.c2 = k.dz;
                } else {
                    int dr = (s2a <= s2b) ? dr2a : 1;
                    rec.code = (uint8_t)(2 | (dr << 3) | (dc2 << 4));
                    rec.c2 = k.dx;
                }
            } else if (br != 0) {
                rec.code = (uint8_t)(br | (dr1 << 3) | (dc2 << 4));
                if (br == 3) {
                    if (root > 0.0f) {
                        rec.c1 = fdiv_k<EXACT>(fadd(k.kA, fdiv(fmul(k.k2K, dd), root)), k.D, k.rD, k.mflags & 8, bad);
                        rec.c2 = fdiv(fmul(4.0f, sref), root);
                    } else {
                        rec.c1 = fdiv_k<EXACT>(k.kA, k.D, k.rD, k.mflags & 8, bad);
                    }
                } else {
                    const float hq2 = SQ ? k.dz : ((br == 4) ? k.dz : k.dx);
                    if (root > 0.0f) {
                        rec.c1 = fdiv(fmul(hx, qe), fmul(hq2, root));
                        rec.c2 = fdiv(fmul(hx, sref), root);
                    }
                }
            }
        }
    }
}

// Near-source value of node (zi, xi) in the reference build's FP32
// arithmetic (time_init, modeling.cu:293-306): X = (xi-nb)*dx - sx fused into
// one FMA by nvcc, then S * sqrtf(powf(X, 2) + powf(Z, 2)) with CUDA's powf.
__device__ __forceinline__ float src_value_f32(float s, int zi, int xi, int nb, float dx, float dz,
                                               float sx, float sz)
{
    const float X = __fmaf_rn((float)(xi - nb), dx, -sx);
    const float Z = __fmaf_rn((float)(zi - nb), dz, -sz);
    return fmul(s, fsqrt(fadd(powf(X, 2.0f), powf(Z, 2.0f))));
}

// Near-source value of node (zi, xi) (global padded indices), FP64 then one
// rounding: S * |x_node - x_src| (modeling.cu:293-306).
__device__ __forceinline__ double src_dist(int zi, int xi, int nb, float dx, float dz, float sx,
                                           float sz)
{
    double ddx = __dsub_rn(__dmul_rn((double)(xi - nb), (double)dx), (double)sx);
    double ddz = __dsub_rn(__dmul_rn((double)(zi - nb), (double)dz), (double)sz);
    return __dsqrt_rn(__dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddz, ddz)));
}

// Catmull-Rom 1D rule of admin.cpp:121-124, each operation rounded once.
__device__ __forceinline__ float cubic1d(float p0, float p1, float p2, float p3, float t)
{
    float inner = fsub(fadd(fmul(3.0f, fsub(p1, p2)), p3), p0);
    float mid = fadd(fsub(fadd(fsub(fmul(2.0f, p0), fmul(5.0f, p1)), fmul(4.0f, p2)), p3),
                     fmul(t, inner));
    float outer = fadd(fsub(p2, p0), fmul(t, mid));
    return fadd(p1, fmul(fmul(0.5f, t), outer));
}

// Receiver stencil geometry (modeling.cu:170-181). Returns false when the
// 4x4 stencil leaves rows [1, nzz-2] or window columns [1, ncols-2].
__device__ __forceinline__ bool pick_geom(float x, float z, float dx, float dz, int nb, int nzz,
                                          int ncols, int c0, int& i, int& j, float& xd, float& zd)
{
    float ax = fdiv(fadd(x, fmul(0.5f, dx)), dx);
    float az = fdiv(fadd(z, fmul(0.5f, dz)), dz);
    float x0 = fmul(floorf(ax), dx);
    float z0 = fmul(floorf(az), dz);
    float x1 = fadd(fmul(floorf(ax), dx), dx);
    float z1 = fadd(fmul(floorf(az), dz), dz);
    xd = fdiv(fsub(x, x0), fsub(x1, x0));
    zd = fdiv(fsub(z, z0), fsub(z1, z0));
    i = __float2int_rz(az) + nb;
    j = __float2int_rz(ax) + nb - c0;
    return !(i - 1 < 1 || i + 2 > nzz - 2 || j - 1 < 1 || j + 2 > ncols - 2);
}

// cubic2d of admin.cpp:126-133 over the padded window T (column stride nzz).
__device__ __forceinline__ float pick_value(const float* T, int nzz, int i, int j, float xd,
                                            float zd)
{
    float p[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const float* col = T + (size_t)(j + a - 1) * nzz + (i - 1);
        p[a] = cubic1d(col[0], col[1], col[2], col[3], zd);
    }
    return cubic1d(p[0], p[1], p[2], p[3], xd);
}

// Cij decompression (eikonal_ani.cu:76-83).
__device__ __forceinline__ float decode_c(uint16_t c, float mn, float mx)
{
    return fadd(mn, fdiv(fmul(fsub((float)c, 1.0f), fsub(mx, mn)), 65534.0f));
}

// qP phase slowness of one node (eikonal_ani.cu:59-108); codes already
// decoded. dzr, dxr: the central differences T(i+1) - T(i-1) and T(j+1) -
// T(j-1) (of the pairs, in the compensated arithmetic). REF: the reference
// build's FMAs (|grad T|^2 and the three Christoffel sums).
template <bool REF>
__device__ __forceinline__ float qp_slowness(float dzr, float dxr, float s, float dx, float dz, float c11,
                                             float c13, float c15, float c33, float c35, float c55)
{
    float dTz = fdiv(fmul(0.5f, dzr), dz);
    float dTx = fdiv(fmul(0.5f, dxr), dx);
    float norm = fsqrt(REF ? __fmaf_rn(dTz, dTz, fmul(dTx, dTx)) : fadd(fmul(dTx, dTx), fmul(dTz, dTz)));
    float p0 = fdiv(dTx, norm), p1 = fdiv(dTz, norm);
    float Ro = fmul(fmul(c33, s), s);
    // C[q] / Ro / Ro
    float C0 = fdiv(fdiv(c11, Ro), Ro);   // c11
    float C3 = fdiv(fdiv(c13, Ro), Ro);   // c13
    float C6 = fdiv(fdiv(c15, Ro), Ro);   // c15
    float C4 = fdiv(fdiv(c33, Ro), Ro);   // c33
    float C7 = fdiv(fdiv(c35, Ro), Ro);   // c35
    float C8 = fdiv(fdiv(c55, Ro), Ro);   // c55
    float Gxx, Gzz, Gxz;
    if (REF) {
        Gxx = __fmaf_rn(fmul(fmul(2.0f, C6), p0), p1, __fmaf_rn(fmul(C0, p0), p0, fmul(fmul(C8, p1), p1)));
        Gzz = __fmaf_rn(fmul(fmul(2.0f, C7), p0), p1, __fmaf_rn(fmul(C8, p0), p0, fmul(fmul(C4, p1), p1)));
        Gxz = __fmaf_rn(fmul(fadd(C3, C8), p0), p1, __fmaf_rn(fmul(C6, p0), p0, fmul(fmul(C7, p1), p1)));
    } else {
        Gxx = fadd(fadd(fmul(fmul(C0, p0), p0), fmul(fmul(C8, p1), p1)), fmul(fmul(fmul(2.0f, C6), p0), p1));
        Gzz = fadd(fadd(fmul(fmul(C8, p0), p0), fmul(fmul(C4, p1), p1)), fmul(fmul(fmul(2.0f, C7), p0), p1));
        Gxz = fadd(fadd(fmul(fmul(C6, p0), p0), fmul(fmul(C7, p1), p1)), fmul(fmul(fadd(C3, C8), p0), p1));
    }
    float coeff1 = fadd(Gxx, Gzz);
    float coeff2 = fsub(Gxx, Gzz);
    // x / 4 and x * 0.25 have the same exact value, hence the same rounding
    float det = fsqrt(fadd(fmul(fmul(coeff2, coeff2), 0.25f), fmul(Gxz, Gxz)));
    // The reference evaluates coeff1 / 2.0 +- det in double and rounds to
    // float. The halving is exact, and rounding a sum of two 24-bit values
    // first to binary64 and then to binary32 gives the binary32 rounding of
    // the exact sum (double rounding is innocuous for addition when the
    // wider format has at least 2p + 1 bits, 53 >= 49; S. A. Figueroa, "When
    // is double rounding innocuous?", ACM SIGNUM Newsletter 30(3), 1995). So
    // one FP32 FMA gives the same bits, without the GPU's slow FP64 pipe.
    float g0 = __fmaf_rn(coeff1, 0.5f, det);
    float g1 = __fmaf_rn(coeff1, 0.5f, -det);
    if (g0 < g1) g0 = g1;
    return fdiv(1.0f, fsqrt(fmul(g0, Ro)));
}

// Derivatives of the qP slowness of one node (eikonal_ani.cu:59-108) with the
// propagation direction p = grad T / |grad T| of the first solve held fixed
// (the first solve sees S only, so for the stiffnesses this is exact):
// Sq = S sqrt(c33 / lambda), lambda the larger eigenvalue of the Christoffel
// matrix Gamma(C, p) and v its unit eigenvector, so
//   dSq/dS   = sqrt(c33 / lambda)
//   dSq/dC11 = -Sq / (2 lambda) * px^2 vx^2          (dGamma_xx/dC11 = px^2)
//   dSq/dC13 = -Sq / lambda * px pz vx vz            (dGamma_xz/dC13 = px pz)
// In FP32 with each operation rounded once (no contraction), so a C
// restatement gives the same bits; FP32 keeps the pass off the GPU's slow
// FP64 pipe. A zero gradient or a non-positive eigenvalue gives (1, 0, 0).
__device__ __forceinline__ void qp_factors(float dzr, float dxr, float s, float dx, float dz, float c11,
                                           float c13, float c15, float c33, float c35, float c55, float& fS,
                                           float& f11, float& f13)
{
    const float dTz = fdiv(fmul(0.5f, dzr), dz);
    const float dTx = fdiv(fmul(0.5f, dxr), dx);
    const float nrm = fsqrt(fadd(fmul(dTx, dTx), fmul(dTz, dTz)));
    fS = 1.0f;
    f11 = 0.0f;
    f13 = 0.0f;
    if (!(nrm > 0.0f)) return;
    const float px = fdiv(dTx, nrm), pz = fdiv(dTz, nrm);
    const float Gxx = fadd(fadd(fmul(fmul(c11, px), px), fmul(fmul(c55, pz), pz)), fmul(fmul(fmul(2.0f, c15), px), pz));
    const float Gzz = fadd(fadd(fmul(fmul(c55, px), px), fmul(fmul(c33, pz), pz)), fmul(fmul(fmul(2.0f, c35), px), pz));
    const float Gxz = fadd(fadd(fmul(fmul(c15, px), px), fmul(fmul(c35, pz), pz)), fmul(fmul(fadd(c13, c55), px), pz));
    const float h = fmul(0.5f, fsub(Gxx, Gzz));
    const float r = fsqrt(fadd(fmul(h, h), fmul(Gxz, Gxz)));
    const float lam = fadd(fmul(0.5f, fadd(Gxx, Gzz)), r);
    if (!(lam > 0.0f)) return;
    float vx, vz;
    if (h >= 0.0f) { vx = fadd(h, r); vz = Gxz; }
    else           { vx = Gxz; vz = fsub(r, h); }
    const float nv = fsqrt(fadd(fmul(vx, vx), fmul(vz, vz)));
    if (nv > 0.0f) { vx = fdiv(vx, nv); vz = fdiv(vz, nv); }
    else           { vx = px; vz = pz; }
    const float fs = fsqrt(fdiv(c33, lam));
    const float sq = fmul(s, fs);
    fS = fs;
    f11 = fdiv(fmul(fmul(fmul(-0.5f, sq), fmul(px, px)), fmul(vx, vx)), lam);
    f13 = fdiv(fmul(fmul(-sq, fmul(px, pz)), fmul(vx, vz)), lam);
}

}  // namespace sf
