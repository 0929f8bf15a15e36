// Whole-shot forward kernel: a gang of CTAs solves one shot window at a time
// (init, 4 sweeps, receiver picks) and takes the shots k, k+NG, ... of its
// gang. The same kernel with one shot and one CTA is the per-shot drop-in
// solver. An anisotropic batch (eikonal_ani.cu:33-45) is three launches: the
// solve of every shot on S, the qP pass over every shot's window (k_qp, a
// map over cells), and the solve of every shot on its own qP slowness.
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
    long long q_off;      // window cells of the shots before it (qP slowness and derivative factors)
};

struct FwdParams {
    const float* S;       // padded slowness, column stride nzz
    const float* Sshots;  // per-shot slowness windows at q_off (column stride nzz) instead of S, or nullptr
    int nzz, nxx, nb;
    Consts kc;
    const ShotDev* shots;
    int nshots;
    int G;                // CTAs per gang (one gang solves one shot at a time)
    int NG;               // gangs; gang k solves shots k, k+NG, ...
    int maxcols;          // widest window of the batch
    float* Tpool;
    float* Tlpool;        // compensated: lo parts of the traveltimes, same layout as Tpool
    long long t_per_gang; // > 0: each gang reuses Tpool + gang * t_per_gang
    int* err;
    unsigned long long* hand;  // tagged strip handoff pairs: per gang [4 sweeps][nstrips][maxcols] (x2 compensated)
    unsigned* bar;        // per gang barrier counter
    unsigned epoch;       // launch number (tags: epoch << 10 | shot-solve number)
    unsigned long long wait_ns;  // time limit of the bounded waits
    int stall_handoff;    // test of the timeout path: consumers wait for a tag no producer writes
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

// Where a gang's warps sit: warp w of CTA g of the gang is slot w*G + g.
// Strip k belongs to slot k mod slots in every sweep, so consecutive strips
// run on different CTAs and SMs and a warp only rereads rows it wrote.
struct GangPos {
    int gang, g, warp, slot, slots;
};

__device__ __forceinline__ GangPos gang_pos(int G)
{
    GangPos q;
    q.gang = blockIdx.x / G;
    q.g = blockIdx.x % G;
    q.warp = threadIdx.x >> 5;
    q.slots = G * (blockDim.x >> 5);
    q.slot = q.warp * G + q.g;
    return q;
}

// The four sweeps of one solve of the current shot; every warp of the gang
// runs the strips of its slot. No barrier between sweeps: consecutive sweeps
// run the rows in opposite directions, a warp rereads only rows it wrote
// itself, and the handoff chain orders everything else. Square cells (dx and
// dz equal) run the strip loops' square-cell form. COMP: compensated
// arithmetic, lo parts in Tl, two handoff pairs per column.
template <bool TAPE, bool REF, bool INTERIOR, bool COMP>
__device__ void solve_window(const FwdParams& p, const ShotDev& sh, const GangPos& gp, const float* Sw,
                             int ldS, float* T, float* Tl, unsigned tag, CtaShared* cs, unsigned char* rings)
{
    const int nzz = p.nzz, ncols = sh.ncols;
    const int nstrips = (nzz + 31) >> 5;
    constexpr size_t HS = COMP ? 2 : 1;
    unsigned long long* hb = p.hand + (size_t)gp.gang * 4 * nstrips * p.maxcols * HS;
    StripArgs a;
    a.S = Sw;
    a.ldS = ldS;
    a.T = T;
    a.Tl = Tl;
    a.nzz = nzz;
    a.ncols = ncols;
    a.nstrips = nstrips;
    a.sIdz = sh.sIdz;
    a.sIdx = sh.sIdx - sh.c0;
    a.kc = p.kc;
    a.init = cs->init;
    a.ring = rings + (size_t)gp.warp * ring_bytes<COMP>(FwdBlock<TAPE>::RING);
    a.sh = cs;
    a.err = p.err;
    a.tcode = nullptr;
    a.tc1 = nullptr;
    a.tc2 = nullptr;
    a.tag = tag;
    a.tag_in = p.stall_handoff ? 1u : tag;  // epoch 0 is never used, zeroed pairs carry tag 0
#pragma unroll 1
    for (int sw = 0; sw < 4; sw++) {
        const bool szpos = !(sw == 1 || sw == 3);
        a.skip_i = sh.skip_i[sw];
        a.skip_j = sh.skip_j[sw];
        unsigned long long* hs = hb + (size_t)sw * nstrips * p.maxcols * HS;
        const int first = szpos ? gp.slot : ((nstrips - 1 - gp.slot) % gp.slots + gp.slots) % gp.slots;
#pragma unroll 1
        for (int pidx = first; pidx < nstrips; pidx += gp.slots) {
            a.k = szpos ? pidx : nstrips - 1 - pidx;
            a.h_in = (pidx > 0) ? hs + (size_t)pidx * p.maxcols * HS : nullptr;
            a.h_out = (pidx < nstrips - 1) ? hs + (size_t)(pidx + 1) * p.maxcols * HS : nullptr;
            if (TAPE) {
                size_t base = tape_strip_base(sh.tape_off, sw, a.k, nstrips, ncols);
                a.tcode = p.tcode + base;
                a.tc1 = p.tc1 + base;
                a.tc2 = p.tc2 + base;
            }
            if (p.kc.dx == p.kc.dz) {
                switch (sw) {
                case 0: run_strip<1, 1, true, TAPE, REF, INTERIOR, true, COMP>(a); break;
                case 1: run_strip<-1, 1, false, TAPE, REF, INTERIOR, true, COMP>(a); break;
                case 2: run_strip<1, -1, false, TAPE, REF, INTERIOR, true, COMP>(a); break;
                default: run_strip<-1, -1, false, TAPE, REF, INTERIOR, true, COMP>(a); break;
                }
            } else {
                switch (sw) {
                case 0: run_strip<1, 1, true, TAPE, REF, INTERIOR, false, COMP>(a); break;
                case 1: run_strip<-1, 1, false, TAPE, REF, INTERIOR, false, COMP>(a); break;
                case 2: run_strip<1, -1, false, TAPE, REF, INTERIOR, false, COMP>(a); break;
                default: run_strip<-1, -1, false, TAPE, REF, INTERIOR, false, COMP>(a); break;
                }
            }
        }
    }
}

// Persistent gangs of G CTAs: gang k solves shots k, k+NG, ... (shots are
// sorted widest window first). The grid never exceeds what the device can
// hold at once, so every gang's CTAs are resident together. INTERIOR: the
// strip loops' bounds-test-free body for interior blocks (see run_strip).
// COMP: compensated arithmetic (node_update_comp; the 3x3 initial values are
// the FP64 ones rounded once).
template <bool TAPE, bool REF, bool INTERIOR, bool COMP = false>
// (kMaxWarps * 32, 1): with the block size alone as the bound ptxas caps the
// kernel at 64 registers and spills the strip loop's state to local memory.
__global__ void __launch_bounds__((COMP ? kMaxWarpsComp : ((TAPE && INTERIOR) ? kMaxWarpsTapedInterior : kMaxWarps)) * 32, 1)
    k_shots(FwdParams p)
{
    static_assert(!(COMP && REF), "the compensated arithmetic has no reference-build variant");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CtaShared* cs = reinterpret_cast<CtaShared*>(smem_raw);
    unsigned char* rings = smem_raw + ((sizeof(CtaShared) + 15) & ~size_t(15));
    const int tid = threadIdx.x;
    const GangPos gp = gang_pos(p.G);
    const int nzz = p.nzz;
    unsigned* bar = p.bar + gp.gang;
    unsigned nbar = 0;
    if (tid == 0) {
        cs->abort_flag = 0;
        cs->wait_ns = p.wait_ns ? p.wait_ns : kSpinNs;
    }
    __syncthreads();
    int it = 0;
#pragma unroll 1
    for (int b = gp.gang; b < p.nshots; b += p.NG, it++) {
        const ShotDev sh = p.shots[b];
        float* T = (p.t_per_gang > 0) ? p.Tpool + (size_t)gp.gang * p.t_per_gang : p.Tpool + sh.t_off;
        float* Tl = !COMP ? nullptr
                          : (p.t_per_gang > 0) ? p.Tlpool + (size_t)gp.gang * p.t_per_gang : p.Tlpool + sh.t_off;
        // the shot's slowness window: columns c0.. of S, or its own qP slowness
        const float* Sw = p.Sshots ? p.Sshots + sh.q_off : p.S + (size_t)sh.c0 * nzz;
        const unsigned tag = (p.epoch << 10) | (unsigned)(it & 1023);
        init_block<REF>(p, sh, Sw, cs->init);
        __syncthreads();
        solve_window<TAPE, REF, INTERIOR, COMP>(p, sh, gp, Sw, nzz, T, Tl, tag, cs, rings);
        // receivers (modeling.cu:161-194), spread over the gang once the field is final
        if (p.nrec > 0 && p.picks) {
            gang_barrier(bar, (++nbar) * p.G, cs, p.err);
            for (int r = (gp.g * (blockDim.x >> 5) + gp.warp) * 32 + (tid & 31); r < p.nrec; r += gp.slots * 32) {
                int i, j;
                float xd, zd;
                float v = __int_as_float(0x7fc00000);
                if (pick_geom(p.rx[r], p.rz[r], p.kc.dx, p.kc.dz, p.nb, nzz, sh.ncols, sh.c0, i, j, xd, zd))
                    v = pick_value(T, nzz, i, j, xd, zd);
                p.picks[(size_t)sh.orig * p.nrec + r] = v;
            }
        }
        // the gang's buffers are reused by its next shot
        gang_barrier(bar, (++nbar) * p.G, cs, p.err);
    }
}

// The qP pass of an anisotropic batch, get_quasi_slowness
// (eikonal_ani.cu:47-111), on every shot's window once the first solves are
// done: the qP slowness of each window cell from the central differences of
// the window's traveltimes (of their pairs in the compensated arithmetic)
// and the decoded stiffness; the window's edge cells (nb of them) and the
// source node keep S. FACT (taped batches): also the derivative factors dSq/dS,
// dSq/dC11, dSq/dC13 of each cell. A map over cells: blockIdx.y strides over
// the shots, blockIdx.x over a window's columns, 128 threads over a column's
// rows (coalesced, z fastest; four rows per thread unrolled measured 1.5%
// faster on the VTI batch than 256 threads one row at a time).
struct QpParams {
    const float* S;       // padded slowness, column stride nzz
    int nzz, nb;
    Consts kc;
    const ShotDev* shots;
    int nshots;
    const float* Tpool;   // per-shot traveltime windows at t_off
    const float* Tlpool;  // their lo parts (compensated)
    const uint16_t* cij[6];
    float mm[12];
    float* Sq;            // per-shot qP slowness windows at q_off
    float* vfac;          // FACT: dSq/dS, dSq/dC11, dSq/dC13 per window cell (3 x vfac_total)
    long long vfac_total;
};

template <bool REF, bool COMP, bool FACT>
__global__ void __launch_bounds__(128) k_qp(QpParams p)
{
    const int nzz = p.nzz, nb = p.nb;
#pragma unroll 1
    for (int b = blockIdx.y; b < p.nshots; b += gridDim.y) {
        const ShotDev sh = p.shots[b];
        const int ncols = sh.ncols, sloc = sh.sIdx - sh.c0;
        const float* T = p.Tpool + sh.t_off;
        const float* Tl = COMP ? p.Tlpool + sh.t_off : nullptr;
        float* Sq = p.Sq + sh.q_off;
#pragma unroll 1
        for (int j = blockIdx.x; j < ncols; j += gridDim.x)
#pragma unroll 4
        for (int i = threadIdx.x; i < nzz; i += blockDim.x) {
            const size_t idx = (size_t)i + (size_t)j * nzz;
            const size_t g = (size_t)i + (size_t)(sh.c0 + j) * nzz;
            const float s = p.S[g];
            float out = s;
            float fS = 1.0f, f11 = 0.0f, f13 = 0.0f;
            if (i >= nb && i < nzz - nb && j >= nb && j < ncols - nb && !(i == sh.sIdz && j == sloc)) {
                const float* Tc = T + idx;
                const float c11 = decode_c(p.cij[0][g], p.mm[0], p.mm[1]);
                const float c13 = decode_c(p.cij[1][g], p.mm[2], p.mm[3]);
                const float c15 = decode_c(p.cij[2][g], p.mm[4], p.mm[5]);
                const float c33 = decode_c(p.cij[3][g], p.mm[6], p.mm[7]);
                const float c35 = decode_c(p.cij[4][g], p.mm[8], p.mm[9]);
                const float c55 = decode_c(p.cij[5][g], p.mm[10], p.mm[11]);
                // central differences; of the pairs in the compensated arithmetic
                float dzr, dxr;
                if (COMP) {
                    const float* Lc = Tl + idx;
                    dzr = ff_diff(Tc[1], Lc[1], Tc[-1], Lc[-1]);
                    dxr = ff_diff(Tc[nzz], Lc[nzz], Tc[-(long)nzz], Lc[-(long)nzz]);
                } else {
                    dzr = fsub(Tc[1], Tc[-1]);
                    dxr = fsub(Tc[nzz], Tc[-(long)nzz]);
                }
                out = qp_slowness<REF>(dzr, dxr, s, p.kc.dx, p.kc.dz, c11, c13, c15, c33, c35, c55);
                if (FACT) qp_factors(dzr, dxr, s, p.kc.dx, p.kc.dz, c11, c13, c15, c33, c35, c55, fS, f11, f13);
            }
            Sq[idx] = out;
            if (FACT) {
                float* f = p.vfac + sh.q_off + idx;
                f[0] = fS;
                f[p.vfac_total] = f11;
                f[2 * p.vfac_total] = f13;
            }
        }
    }
}

}  // namespace sf
