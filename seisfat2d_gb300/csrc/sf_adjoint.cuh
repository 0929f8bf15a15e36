// Adjoint-state gradient: reverse sweeps over the forward tape.
//
// The forward pass (k_shots<true>) records, for every node of every sweep,
// which candidate set the node (code bits 0-2), which slowness cell that
// candidate read (bits 3-4) and two derivative coefficients c1, c2 (see
// include/seisfat2d.h). The discrete adjoint of one sweep is then the linear
// recurrence, in pull form, for node n = (i, j) of a sweep with signs (sz, sx):
//
//   mu(n)  = ((lam(n) + pv(i+sz, j)) + pe(i, j+sx)) + pev(i+sz, j+sx)
//   lam(n) <- mu(n) if the node kept its value (code 0), else 0
//   pv/pe/pev(n) = mu(n) * dT(n)/d{tv, te, tev}   (pushed to the upwind nodes)
//   v(n)   = mu(n) * c2                           (term of the node's slowness cell)
//
// swept in the reverse order. It is the forward's dependency pattern with the
// march reversed, so the same strip-systolic schedule runs it: lane l owns a
// row, the lane above supplies pv/pev of the previous step by shfl, the lane's
// own previous pe is kept in a register. The tape was written in the forward
// strip's skewed step order, which makes the reverse read of one step 32
// consecutive entries (lane l of the reverse march is lane 31-l of the
// forward one).
#pragma once
#include "sf_adjoint_params.cuh"
#include "sf_forward.cuh"

namespace sf {

constexpr int kLP = 36;    // lambda slot pitch: 32 rows, then the {pv,tag},{pev,tag} handoff pairs
constexpr int kTR = 16;    // tape ring slots (>= kLook + 2)
constexpr int kTPitch = 72;  // c1[32], c2[32], code bytes (8 words)

struct AdjRing {
    float L[kRing * kLP];
    float TP[kTR * kTPitch];
};

struct AdjStripArgs {
    float* lam;        // window adjoint field (column stride nzz), in place
    int nzz, ncols, k;
    const uint8_t* tcode;  // tape of this (sweep, strip): entries [fstep*32 + flane]
    const float* tc1;
    float* tc2;            // overwritten with v = mu * c2
    AdjRing* ring;
    CtaShared* sh;
    const unsigned long long* h_in;  // {pv,tag},{pev,tag} of the upwind strip's row (nullptr: first strip)
    unsigned long long* h_out;       // pairs this strip feeds to the next one (nullptr: last strip)
    unsigned tag;
    int* err;
};

// SZ, SX: signs of the forward sweep being reversed.
template <int SZ, int SX>
__device__ __forceinline__ void adj_strip(const AdjStripArgs& a)
{
    const int lane = threadIdx.x & 31;
    const int nzz = a.nzz, ncols = a.ncols;
    const int rb = 32 * a.k;
    // reverse march: rows along -SZ, columns along -SX
    const int r = (SZ < 0) ? rb + lane : rb + 31 - lane;
    const bool vrow = r < nzz;
    const int tix = r - rb;
    const int flane = 31 - lane;  // this row's lane in the forward strip
    float* Lr = a.ring->L;
    float* TPr = a.ring->TP;
    float* lamg = a.lam;
    const bool lt_ok = (rb + lane) < nzz;
    CtaShared* sh = a.sh;
    const bool consumer = (lane == 0) && (a.h_in != nullptr);
    const int nsteps = ncols + 31;
    auto col_of = [&](int m) { return (SX < 0) ? m : ncols - 1 - m; };
    // running source addresses of march q (q advances by one per call): the
    // lambda column, the handoff pairs, and forward tape step ncols+30-q
    const long long dL = (SX < 0) ? (long long)nzz : -(long long)nzz;
    const float* pL = lamg + (size_t)(rb + lane) + (long long)col_of(0) * (long long)nzz;
    const unsigned long long* pH = a.h_in;
    const size_t fs0 = (size_t)(ncols + 30) * 32;
    const float* pT1 = a.tc1 + fs0 + lane;
    const float* pT2 = a.tc2 + fs0 + lane;
    const uint8_t* pTc = a.tcode + fs0 + 4 * lane;
    auto prefetch = [&](int q, int lslot, int tslot) {
        if (q < ncols) {
            if (lt_ok) cp_async4(&Lr[lslot * kLP + lane], pL);
            if (consumer) cp_async16(&Lr[lslot * kLP + 32], pH);
        }
        if (q < nsteps) {
            cp_async4(&TPr[tslot * kTPitch + lane], pT1);
            cp_async4(&TPr[tslot * kTPitch + 32 + lane], pT2);
            if (lane < 8) cp_async4(&TPr[tslot * kTPitch + 64 + lane], pTc);
        }
        cp_commit();
        pL += dL;
        pH += 2;
        pT1 -= 32;
        pT2 -= 32;
        pTc -= 32;
    };

    // let the previous strip get kLook+4 columns ahead before the first prefetches
    if (consumer) wait_pair(a.h_in + 2 * (size_t)min(kLook + 4, ncols - 1) + 1, a.tag, sh, a.err);
    __syncwarp();
#pragma unroll 1
    for (int q = 0; q < kLook; q++) prefetch(q, q, q % kTR);

    // running destinations: the term v of forward tape step ncols+30-s, and
    // the write-back of march column s-31 (row r)
    float* pV = a.tc2 + fs0 + flane;
    float* pW = lamg + (size_t)r + (long long)col_of(0) * (long long)nzz;

    int pf_slot = kLook, pf_tslot = kLook % kTR;
    int m_slot = (kRing - lane) % kRing;
    int wb_slot = (kRing - 31) % kRing;
    int t_slot = 0;
    float my_pv = 0.0f, my_pe = 0.0f, my_pev = 0.0f, pev_hold = 0.0f;

#pragma unroll 1
    for (int s = 0; s < nsteps; s++) {
        prefetch(s + kLook, pf_slot, pf_tslot);
        cp_wait<kLook - 1>();
        __syncwarp();

        const int m = s - lane;
        const bool act = vrow && (m >= 0) && (m < ncols);
        float pv_in = __shfl_up_sync(0xffffffffu, my_pv, 1);
        float pev_in = __shfl_up_sync(0xffffffffu, my_pev, 1);
        if (lane == 0) {  // upwind row of the strip: the previous strip, or outside the grid
            pv_in = 0.0f;
            pev_in = 0.0f;
            if (consumer && s < ncols) {
                const unsigned long long* e = reinterpret_cast<const unsigned long long*>(&Lr[m_slot * kLP + 32]);
                const unsigned long long e0 = e[0], e1 = e[1];
                if (tag_of(e0) == a.tag && tag_of(e1) == a.tag) {
                    pv_in = val_of(e0);
                    pev_in = val_of(e1);
                } else {
                    pv_in = wait_pair(a.h_in + 2 * (size_t)s, a.tag, sh, a.err);
                    pev_in = wait_pair(a.h_in + 2 * (size_t)s + 1, a.tag, sh, a.err);
                    wait_pair(a.h_in + 2 * (size_t)min(s + kLook + 4, ncols - 1) + 1, a.tag, sh, a.err);
                }
            }
        }
        const float lam_in = Lr[m_slot * kLP + tix];
        const float c1 = TPr[t_slot * kTPitch + flane];
        const float c2 = TPr[t_slot * kTPitch + 32 + flane];
        const int code = reinterpret_cast<const uint8_t*>(&TPr[t_slot * kTPitch + 64])[flane];

        float mu = fadd(fadd(fadd(lam_in, pv_in), my_pe), pev_hold);
        pev_hold = pev_in;
        float npv = 0.0f, npe = 0.0f, npev = 0.0f;
        if (act) {
            const int br = code & 7;
            float lo = mu, v = 0.0f;
            if (br != 0) {
                lo = 0.0f;
                v = fmul(mu, c2);
                switch (br) {
                case 1: npv = mu; break;
                case 2: npe = mu; break;
                case 3: npv = fmul(mu, c1); npe = fmul(mu, -c1); npev = mu; break;
                case 4: npe = fmul(mu, fsub(1.0f, c1)); npev = fmul(mu, c1); break;
                default: npv = fmul(mu, fsub(1.0f, c1)); npev = fmul(mu, c1); break;
                }
            }
            Lr[m_slot * kLP + tix] = lo;
            *pV = v;
            if (lane == 31 && a.h_out != nullptr) {
                st_u64(a.h_out + 2 * (size_t)m, pack_tag(npv, a.tag));
                st_u64(a.h_out + 2 * (size_t)m + 1, pack_tag(npev, a.tag));
            }
        }
        my_pv = npv;
        my_pe = npe;
        my_pev = npev;

        pV -= 32;
        if (s >= 31) {
            if (vrow) *pW = Lr[wb_slot * kLP + tix];
            pW += dL;
        }

        if (++pf_slot == kRing) pf_slot = 0;
        if (++pf_tslot == kTR) pf_tslot = 0;
        if (++m_slot == kRing) m_slot = 0;
        if (++wb_slot == kRing) wb_slot = 0;
        if (++t_slot == kTR) t_slot = 0;
    }
    cp_wait<0>();
    __syncwarp();
}

// Cubic weights of the pick rule (the rule is linear in the 16 nodes):
// P -> P1 + 0.5 t (P2 - P0 + t (2P0 - 5P1 + 4P2 - P3 + t (3(P1 - P2) + P3 - P0)))
// (every FP64 operation rounded once, left to right, as written)
__device__ __forceinline__ void cubic_weights(double t, double w[4])
{
    const double t2 = __dmul_rn(t, t), t3 = __dmul_rn(t2, t);
    w[0] = __dsub_rn(__dadd_rn(__dmul_rn(-0.5, t), t2), __dmul_rn(0.5, t3));
    w[1] = __dadd_rn(__dsub_rn(1.0, __dmul_rn(2.5, t2)), __dmul_rn(1.5, t3));
    w[2] = __dsub_rn(__dadd_rn(__dmul_rn(0.5, t), __dmul_rn(2.0, t2)), __dmul_rn(1.5, t3));
    w[3] = __dadd_rn(__dmul_rn(-0.5, t2), __dmul_rn(0.5, t3));
}

// (kMaxWarps * 32, 1): the block size alone as the bound caps the kernel at
// 64 registers and spills the strip loop's state.
__global__ void __launch_bounds__(kMaxWarps * 32, 1) k_adjoint(AdjParams p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CtaShared* cs = reinterpret_cast<CtaShared*>(smem_raw);
    AdjRing* rings = reinterpret_cast<AdjRing*>(smem_raw + ((sizeof(CtaShared) + 15) & ~size_t(15)));
    const int tid = threadIdx.x, lane = tid & 31;
    const GangPos gp = gang_pos(p.G);
    const int nzz = p.nzz, nstrips = p.nstrips;
    float* lam = p.lam + (size_t)gp.gang * p.lam_per_gang;
    unsigned long long* hb = p.hand + (size_t)gp.gang * 4 * nstrips * 2 * p.maxcols;
    unsigned* bar = p.bar + gp.gang;
    unsigned nbar = 0;
    if (tid == 0) cs->abort_flag = 0;
    __syncthreads();
    int it = 0;
#pragma unroll 1
    for (int b = gp.gang; b < p.nshots; b += p.NG, it++) {
        const ShotDev sh = p.shots[b];
        const int ncols = sh.ncols;
        const unsigned tag = (p.epoch << 10) | (unsigned)(it & 1023);
        // seed: adjoint of the final field from the pick gradients
        for (int k = gp.slot; k < nstrips; k += gp.slots) {
            const int i = 32 * k + lane;
            if (i < nzz)
                for (int j = 0; j < ncols; j++) lam[(size_t)i + (size_t)j * nzz] = 0.0f;
        }
        gang_barrier(bar, (++nbar) * p.G, cs, p.err);
        if (gp.g == 0 && gp.warp == 0) {
            const float* pg = p.pick_grad + (size_t)sh.orig * p.nrec;
            for (int rr = 0; rr < p.nrec; rr++) {
                const float g = pg[rr];
                int i, j;
                float xd, zd;
                const bool ok = pick_geom(p.rx[rr], p.rz[rr], p.dx, p.dz, p.nb, nzz, ncols, sh.c0, i, j, xd, zd);
                if (ok && g == g && lane < 16) {
                    double wx[4], wz[4];
                    cubic_weights((double)xd, wx);
                    cubic_weights((double)zd, wz);
                    const int aa = lane >> 2, bb = lane & 3;
                    const float w = __double2float_rn(__dmul_rn(wx[aa], wz[bb]));
                    float* at = lam + (size_t)(i + bb - 1) + (size_t)(j + aa - 1) * nzz;
                    *at = fadd(*at, fmul(g, w));
                }
                __syncwarp();
            }
        }
        gang_barrier(bar, (++nbar) * p.G, cs, p.err);
        // reverse sweeps 3, 2, 1, 0 (consecutive ones run the rows in opposite
        // directions: no barrier between them, as in the forward)
        AdjStripArgs a;
        a.lam = lam;
        a.nzz = nzz;
        a.ncols = ncols;
        a.ring = rings + gp.warp;
        a.sh = cs;
        a.err = p.err;
        a.tag = tag;
#pragma unroll 1
        for (int sw = 3; sw >= 0; sw--) {
            const bool fz_pos = !(sw == 1 || sw == 3);  // forward SZ > 0: reverse march goes up
            unsigned long long* hs = hb + (size_t)sw * nstrips * 2 * p.maxcols;
            // strips have a fixed owner (strip k -> slot k mod slots) in every sweep;
            // processing index pidx runs along the reverse march
            const int first = fz_pos ? ((nstrips - 1 - gp.slot) % gp.slots + gp.slots) % gp.slots : gp.slot;
#pragma unroll 1
            for (int pidx = first; pidx < nstrips; pidx += gp.slots) {
                a.k = fz_pos ? nstrips - 1 - pidx : pidx;
                a.h_in = (pidx > 0) ? hs + 2 * (size_t)pidx * p.maxcols : nullptr;
                a.h_out = (pidx < nstrips - 1) ? hs + 2 * (size_t)(pidx + 1) * p.maxcols : nullptr;
                const size_t tb = tape_strip_base(sh.tape_off, sw, a.k, nstrips, ncols);
                a.tcode = p.tcode + tb;
                a.tc1 = p.tc1 + tb;
                a.tc2 = p.tc2 + tb;
                switch (sw) {
                case 0: adj_strip<1, 1>(a); break;
                case 1: adj_strip<-1, 1>(a); break;
                case 2: adj_strip<1, -1>(a); break;
                default: adj_strip<-1, -1>(a); break;
                }
            }
        }
        gang_barrier(bar, (++nbar) * p.G, cs, p.err);
        if (gp.g == 0 && tid < 9) {
            const int aa = tid % 3, bb = tid / 3;
            const int zi = sh.sIdz + aa - 1, xl = sh.sIdx - sh.c0 + bb - 1;
            p.lam_init[(size_t)sh.orig * 9 + tid] = lam[(size_t)zi + (size_t)xl * nzz];
        }
        gang_barrier(bar, (++nbar) * p.G, cs, p.err);
    }
}

// Tape index of node (i, j) (window coordinates) in forward sweep sw.
__device__ __forceinline__ size_t tape_index(const ShotDev& sh, int sw, int i, int j, int nstrips, int nzz)
{
    const int k = i >> 5;
    const bool szpos = !(sw == 1 || sw == 3);
    const bool sxpos = sw < 2;
    const int flane = szpos ? (i - 32 * k) : (32 * k + 31 - i);
    const int fm = sxpos ? j : sh.ncols - 1 - j;
    return tape_strip_base(sh.tape_off, sw, k, nstrips, sh.ncols) + (size_t)(fm + flane) * 32 + flane;
}

// g(a, b) = sum over shots (caller order, FP64) of the shot's FP32 sum over
// sweeps 0..3 and corners (dr, dc) = (0,0),(0,1),(1,0),(1,1) of the matching
// node terms, plus the 3x3 initialisation term lam_init * dist.
__global__ void k_gather(GatherParams p)
{
    const size_t ncell = (size_t)p.nzz * p.nxx;
    for (size_t cell = blockIdx.x * (size_t)blockDim.x + threadIdx.x; cell < ncell;
         cell += (size_t)gridDim.x * blockDim.x) {
        const int a = (int)(cell % p.nzz), bcol = (int)(cell / p.nzz);
        double total = 0.0;
        for (int q = p.colptr[bcol]; q < p.colptr[bcol + 1]; q++) {
            const int orig = p.colshots[q];
            const ShotDev sh = p.shots[p.shot_of_orig[orig]];
            const int b = bcol - sh.c0;
            float g = 0.0f;
            for (int sw = 0; sw < 4; sw++)
                for (int dr = 0; dr < 2; dr++)
                    for (int dc = 0; dc < 2; dc++) {
                        const int i = a + 1 - dr, j = b + 1 - dc;
                        if (i >= p.nzz || j >= sh.ncols) continue;
                        const size_t t = tape_index(sh, sw, i, j, p.nstrips, p.nzz);
                        const int cd = p.tcode[t];
                        if ((cd & 7) && ((cd >> 3) & 1) == dr && ((cd >> 4) & 1) == dc) g = fadd(g, p.vrec[t]);
                    }
            const int da = a - sh.sIdz + 1, db = bcol - sh.sIdx + 1;
            if (da >= 0 && da < 3 && db >= 0 && db < 3) {
                const double d = src_dist(a, bcol, p.nb, p.dx, p.dz, sh.sx, sh.sz);
                g = fadd(g, fmul(p.lam_init[(size_t)orig * 9 + da + 3 * db], __double2float_rn(d)));
            }
            total += (double)g;
        }
        p.grad[cell] = __double2float_rn(total);
    }
}

// Residuals r = pick - t_obs (NaN picks or observations contribute nothing)
// and the misfit 1/2 sum r^2 in FP64 by one CTA in a fixed order.
__global__ void k_residual(const float* picks, const float* tobs, size_t n, float* res, double* misfit)
{
    __shared__ double part[1024];
    double acc = 0.0;
    for (size_t k = threadIdx.x; k < n; k += blockDim.x) {
        const float pk = picks[k], ob = tobs[k];
        float r = fsub(pk, ob);
        if (!(r == r)) r = __int_as_float(0x7fc00000);
        res[k] = r;
        if (r == r) acc += 0.5 * (double)r * (double)r;
    }
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *misfit = part[0];
}

}  // namespace sf
