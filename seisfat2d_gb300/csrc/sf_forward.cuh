// Whole-shot forward kernel: one CTA solves one shot window at a time (init,
// 4 sweeps, optional qP pass + second solve, receiver picks) and pulls the
// next shot from a device work counter. The same kernel with one shot and one
// CTA is the per-shot drop-in solver.
#pragma once
#include "sf_sweep.cuh"

namespace sf {

// Device description of one shot (host computes it once per batch).
struct ShotDev {
    int c0, ncols;        // window: padded columns [c0, c0+ncols)
    int sIdx, sIdz;       // source node, global padded indices
    float sx, sz;         // source position (m)
    int skip_i[4];        // cells the reference schedule never updates
    int skip_j[4];        // (window coordinates, -1 = none), per sweep
    int orig;             // index of the shot in the caller's order
    int pad_;
    long long t_off;      // traveltime window offset (floats) when tables are kept
    long long tape_off;   // tape offset (entries)
};

struct FwdParams {
    const float* S;       // padded slowness, column stride nzz
    int nzz, nxx, nb;
    Consts kc;
    const ShotDev* shots;
    int nshots;
    float* Tpool;
    long long t_per_cta;  // > 0: each CTA reuses Tpool + blockIdx.x * t_per_cta
    int* counter;
    int* err;
    float* hand;          // strip handoff buffer, hand + blockIdx.x * hand_per_cta
    long long hand_per_cta;  // >= nstrips * widest window
    // anisotropy
    int ani;
    const uint16_t* cij[6];
    float mm[12];
    float* Sq;            // qP slowness scratch, Sq + blockIdx.x * sq_per_cta
    long long sq_per_cta;
    // tape
    uint8_t* tcode;
    float* tc1;
    float* tc2;
    // receivers
    const float* rx;
    const float* rz;
    int nrec;
    float* picks;         // nshots x nrec, caller order
};

// 3x3 initial values of one solve into shared memory (modeling.cu:293-306):
// FP32 as the reference build computes them (REF) or in FP64, rounded once.
template <bool REF>
__device__ __forceinline__ void init_block(const FwdParams& p, const ShotDev& sh, const float* Sw,
                                           float* out)
{
    const int tid = threadIdx.x;
    if (tid < 9) {
        const int a = tid % 3, bb = tid / 3;
        const int zi = sh.sIdz + a - 1, xl = sh.sIdx - sh.c0 + bb - 1;
        const float s = Sw[zi + (size_t)xl * p.nzz];
        if (REF)
            out[tid] = src_value_f32(s, zi, xl + sh.c0, p.nb, p.kc.dx, p.kc.dz, sh.sx, sh.sz);
        else
            out[tid] = __double2float_rn(
                __dmul_rn((double)s, src_dist(zi, xl + sh.c0, p.nb, p.kc.dx, p.kc.dz, sh.sx, sh.sz)));
    }
}

__device__ __forceinline__ size_t tape_strip_base(long long tape_off, int sweep, int k, int nstrips,
                                                  int ncols)
{
    return (size_t)tape_off + ((size_t)sweep * nstrips + k) * (size_t)(ncols + 31) * 32;
}

// Position of strip p (p >= 1) among the strips fed through handoff channel
// p % W: channel 0 carries W, 2W, ..., channel w > 0 carries w, w+W, ...
__device__ __forceinline__ int chan_entry(int p, int W) { return p / W - ((p % W == 0) ? 1 : 0); }

// The four sweeps of one solve on the window held by this CTA.
template <bool TAPE, bool REF>
__device__ void solve_window(const FwdParams& p, const ShotDev& sh, const float* Sw, int ldS,
                             float* T, CtaShared* cs, WarpRing* rings)
{
    const int W = blockDim.x >> 5, warp = threadIdx.x >> 5;
    const int nzz = p.nzz, ncols = sh.ncols;
    const int nstrips = (nzz + 31) >> 5;
    StripArgs a;
    a.S = Sw;
    a.ldS = ldS;
    a.T = T;
    a.nzz = nzz;
    a.ncols = ncols;
    a.nstrips = nstrips;
    a.sIdz = sh.sIdz;
    a.sIdx = sh.sIdx - sh.c0;
    a.kc = p.kc;
    a.init = cs->init;
    a.ring = rings + warp;
    a.sh = cs;
    a.err = p.err;
    a.tcode = nullptr;
    a.tc1 = nullptr;
    a.tc2 = nullptr;
    float* hb = p.hand + (size_t)blockIdx.x * p.hand_per_cta;
#pragma unroll 1
    for (int sw = 0; sw < 4; sw++) {
        if (threadIdx.x < kMaxWarps) cs->prod[threadIdx.x] = 0;
        __syncthreads();
        const bool szpos = !(sw == 1 || sw == 3);
        a.skip_i = sh.skip_i[sw];
        a.skip_j = sh.skip_j[sw];
#pragma unroll 1
        for (int pidx = warp; pidx < nstrips; pidx += W) {
            a.k = szpos ? pidx : nstrips - 1 - pidx;
            // channel w carries strips p = w, w+W, ... (p >= 1) back to back
            a.w_in = (pidx > 0) ? warp : -1;
            a.e_in = chan_entry(pidx, W) * ncols;
            a.w_out = (pidx < nstrips - 1) ? (pidx + 1) % W : -1;
            a.e_out = chan_entry(pidx + 1, W) * ncols;
            a.h_in = hb + (size_t)pidx * ncols;
            a.h_out = hb + (size_t)(pidx + 1) * ncols;
            if (TAPE) {
                size_t base = tape_strip_base(sh.tape_off, sw, a.k, nstrips, ncols);
                a.tcode = p.tcode + base;
                a.tc1 = p.tc1 + base;
                a.tc2 = p.tc2 + base;
            }
            switch (sw) {
            case 0: run_strip<1, 1, true, TAPE, REF>(a); break;
            case 1: run_strip<-1, 1, false, TAPE, REF>(a); break;
            case 2: run_strip<1, -1, false, TAPE, REF>(a); break;
            default: run_strip<-1, -1, false, TAPE, REF>(a); break;
            }
        }
        __syncthreads();
    }
}

template <bool TAPE, bool REF>
__global__ void __launch_bounds__(kMaxWarps * 32) k_shots(FwdParams p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CtaShared* cs = reinterpret_cast<CtaShared*>(smem_raw);
    WarpRing* rings = reinterpret_cast<WarpRing*>(smem_raw + ((sizeof(CtaShared) + 15) & ~size_t(15)));
    const int tid = threadIdx.x;
    if (tid == 0) cs->abort_flag = 0;
    __syncthreads();
#pragma unroll 1
    for (;;) {
        if (tid == 0) cs->item = atomicAdd(p.counter, 1);
        __syncthreads();
        const int b = cs->item;
        __syncthreads();
        if (b >= p.nshots) break;
        const ShotDev sh = p.shots[b];
        const int nzz = p.nzz, ncols = sh.ncols;
        float* T = (p.t_per_cta > 0) ? p.Tpool + (size_t)blockIdx.x * p.t_per_cta
                                     : p.Tpool + sh.t_off;
        const float* Sw = p.S + (size_t)sh.c0 * nzz;
        init_block<REF>(p, sh, Sw, cs->init);
        __syncthreads();
        solve_window<TAPE, REF>(p, sh, Sw, nzz, T, cs, rings);
        if (p.ani) {
            // get_quasi_slowness (eikonal_ani.cu:47-111) on the window
            float* Sq = p.Sq + (size_t)blockIdx.x * p.sq_per_cta;
            const int sloc = sh.sIdx - sh.c0, nb = p.nb;
            const size_t n = (size_t)nzz * ncols;
            for (size_t idx = tid; idx < n; idx += blockDim.x) {
                const int i = (int)(idx % nzz), j = (int)(idx / nzz);
                const size_t g = (size_t)i + (size_t)(sh.c0 + j) * nzz;
                float s = p.S[g];
                float out = s;
                if (i >= nb && i < nzz - nb && j >= nb && j < ncols - nb && !(i == sh.sIdz && j == sloc)) {
                    const float* Tc = T + idx;
                    out = qp_slowness<REF>(Tc[1], Tc[-1], Tc[nzz], Tc[-(long)nzz], s, p.kc.dx, p.kc.dz,
                                      decode_c(p.cij[0][g], p.mm[0], p.mm[1]),
                                      decode_c(p.cij[1][g], p.mm[2], p.mm[3]),
                                      decode_c(p.cij[2][g], p.mm[4], p.mm[5]),
                                      decode_c(p.cij[3][g], p.mm[6], p.mm[7]),
                                      decode_c(p.cij[4][g], p.mm[8], p.mm[9]),
                                      decode_c(p.cij[5][g], p.mm[10], p.mm[11]));
                }
                Sq[idx] = out;
            }
            __syncthreads();
            {
                // second time_init reads the qP field (window-local columns)
                if (tid < 9) {
                    const int a = tid % 3, bb = tid / 3;
                    const int zi = sh.sIdz + a - 1, xl = sloc + bb - 1;
                    const float s = Sq[zi + (size_t)xl * nzz];
                    if (REF)
                        cs->init[tid] = src_value_f32(s, zi, xl + sh.c0, p.nb, p.kc.dx, p.kc.dz, sh.sx, sh.sz);
                    else
                        cs->init[tid] = __double2float_rn(__dmul_rn(
                            (double)s, src_dist(zi, xl + sh.c0, p.nb, p.kc.dx, p.kc.dz, sh.sx, sh.sz)));
                }
            }
            __syncthreads();
            solve_window<false, REF>(p, sh, Sq, nzz, T, cs, rings);
        }
        // receivers (modeling.cu:161-194)
        if (p.nrec > 0 && p.picks) {
            for (int r = tid; r < p.nrec; r += blockDim.x) {
                int i, j;
                float xd, zd;
                float v = __int_as_float(0x7fc00000);
                if (pick_geom(p.rx[r], p.rz[r], p.kc.dx, p.kc.dz, p.nb, nzz, ncols, sh.c0, i, j, xd, zd))
                    v = pick_value(T, nzz, i, j, xd, zd);
                p.picks[(size_t)sh.orig * p.nrec + r] = v;
            }
        }
        __syncthreads();
    }
}

}  // namespace sf
