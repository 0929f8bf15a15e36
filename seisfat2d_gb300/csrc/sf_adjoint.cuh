// Adjoint-state gradient: reverse sweeps over the forward tape.
//
// The forward pass (k_shots<true>) records, for every node of every sweep,
// which candidate set the node (code bits 0-2), which slowness cell that
// candidate read (bits 3-4) and two derivative coefficients c1, c2 (see
// include/seisfat2d.h). The discrete adjoint of one sweep is then the linear
// recurrence, in pull form, for node n = (i, j) of a sweep with signs (sz, sx):
//
//   mu(n)  = (lam(n) + (pv(i+sz, j) + pev(i+sz, j+sx))) + pe(i, j+sx)
//   lam(n) <- mu(n) if the node kept its value (code 0), else 0
//   pv/pe/pev(n) = mu(n) * dT(n)/d{tv, te, tev}   (pushed to the upwind nodes)
//   v(n)   = mu(n) * c2                           (term of the node's slowness cell)
//
// swept in the reverse order. It is the forward's dependency pattern with the
// march reversed, so the same strip-systolic schedule runs it: lane l owns a
// row, the lane above supplies the sum of its pv of the previous step and its
// pev of the step before by one shfl (the two pushes of the upwind row are
// summed by their sender), the lane's own previous pe is kept in a register.
// The tape was written in the forward strip's skewed step order, which makes
// the reverse read of one step 32 consecutive entries (lane l of the reverse
// march is lane 31-l of the forward one).
//
// The node terms v overwrite the tape's c2; the gradient gather (gather_tile)
// sums them per slowness cell, either in its own launch (k_gather) or inside
// the reverse-sweep launch (k_adjoint_gather), where each tile starts as soon
// as the last reverse sweep of every shot has finished it.
#pragma once
#include "sf_adjoint_params.cuh"
#include "sf_forward.cuh"

namespace sf {

constexpr int kGT = 32;    // gather tile columns (the column blocks of the gradient gather)
constexpr int kLP = 36;    // lambda slot pitch: 32 rows, then the {pv,tag},{pev,tag} handoff pairs
// The reverse sweeps stage 4 columns ahead (one block): their tape rows come
// from DRAM, but a shorter lead keeps consecutive strips closer together,
// which measured faster than 8 or 12.
constexpr int kLookA = 4;
constexpr int kAheadA = kLookA + kU;  // a consumer's fall-back distance after a stall
constexpr int kTR = 12;    // tape ring slots (a multiple of kU, > kLookA + kU)
constexpr int kTPitch = 72;  // c1[32], c2[32], code bytes (8 words)
// the prefetch slots b0 + kLookA + u and tb0 + kLookA + u are wrapped once:
// blocks must tile the lead and both rings
static_assert(kLookA % kU == 0 && kRing % kU == 0 && kTR % kU == 0, "ring slots of a block would wrap twice");
static_assert(kTR >= kLookA + kU && kRing >= 32 + kLookA + kU, "ring too small for the lead");

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
    // last reverse sweep inside a fused launch: count each column block of
    // kGT padded columns once all lanes have finished its columns
    unsigned* ready;   // this strip's row of counters (nullptr: no counting)
    int c0;            // the window's first padded column
};

// SZ, SX: signs of the forward sweep being reversed. INTERIOR: blocks whose
// marches all lie inside the window run a body without bounds tests.
template <int SZ, int SX, bool INTERIOR>
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
    // march q reads lambda column col_of(q), the pairs of march q and forward
    // tape step ncols+30-q; the pointers below stand at the block's first
    // march and move once per block, the steps inside a block are offsets
    const long long dL = (SX < 0) ? (long long)nzz : -(long long)nzz;
    const float* pL = lamg + (size_t)(rb + lane) + (long long)col_of(0) * (long long)nzz;
    const unsigned long long* pH = a.h_in;
    const size_t fs0 = (size_t)(ncols + 30) * 32;
    const float* pT1 = a.tc1 + fs0 + lane;
    const float* pT2 = a.tc2 + fs0 + lane;
    const uint8_t* pTc = a.tcode + fs0 + 4 * lane;
    // FAST: every march of the call is inside the window (no bounds tests)
    auto prefetch = [&](int q, int u, int lslot, int tslot, auto fast_tag) {
        constexpr bool FAST = decltype(fast_tag)::value;
        if (FAST || q < ncols) {
            if (lt_ok) cp_async4(&Lr[lslot * kLP + lane], pL + u * dL);
            if (consumer) cp_async16(&Lr[lslot * kLP + 32], pH + 2 * u);
        }
        if (FAST || q < nsteps) {
            cp_async4(&TPr[tslot * kTPitch + lane], pT1 - 32 * u);
            cp_async4(&TPr[tslot * kTPitch + 32 + lane], pT2 - 32 * u);
            if (lane < 8) cp_async4(&TPr[tslot * kTPitch + 64 + lane], pTc - 32 * u);
        }
        cp_commit();
    };
    auto advance = [&](int n) {
        pL += n * dL;
        pH += 2 * n;
        pT1 -= 32 * n;
        pT2 -= 32 * n;
        pTc -= 32 * n;
    };

    // let the previous strip get kAheadA columns ahead before the first prefetches
    if (consumer) wait_pair(a.h_in + 2 * (size_t)min(kAheadA, ncols - 1) + 1, a.tag, sh, a.err);
    __syncwarp();
#pragma unroll 1
    for (int q = 0; q < kLookA; q++) {
        prefetch(q, 0, q, q % kTR, std::false_type{});
        advance(1);
    }

    // running destinations: the term v of forward tape step ncols+30-s, and
    // the write-back of march column s-31 (row r)
    float* pV = a.tc2 + fs0 + flane;
    float* pW = lamg + (size_t)r + (long long)col_of(0) * (long long)nzz;

    float my_x = 0.0f, my_pe = 0.0f, my_pev = 0.0f, pev_hold = 0.0f;
    int b0 = 0, tb0 = 0;  // ring slots of march s0 (lambda, tape)

    // Blocks of kU steps, as in the forward: one wait per block, the block's
    // ring reads, its kU linear updates (the only serial chain), its stores.
    auto block = [&](int s0, auto fast_tag) {
        constexpr bool FAST = decltype(fast_tag)::value;
        {
            int pf0 = b0 + kLookA;
            if (pf0 >= kRing) pf0 -= kRing;
            int tf0 = tb0 + kLookA;
            if (tf0 >= kTR) tf0 -= kTR;
#pragma unroll
            for (int u = 0; u < kU; u++) prefetch(s0 + kLookA + u, u, pf0 + u, tf0 + u, fast_tag);
            advance(kU);
        }
        cp_wait<kLookA>();
        __syncwarp();

        int ml = b0 - lane;  // slot of march s0 - lane
        if (ml < 0) ml += kRing;
        int msl[kU], code[kU];
        float lam_in[kU], c1[kU], c2[kU];
        unsigned long long e0[kU], e1[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) {
            int ms = ml + u;
            if (ms >= kRing) ms -= kRing;
            msl[u] = ms;
            lam_in[u] = Lr[ms * kLP + tix];
            const int ts = tb0 + u;
            c1[u] = TPr[ts * kTPitch + flane];
            c2[u] = TPr[ts * kTPitch + 32 + flane];
            code[u] = reinterpret_cast<const uint8_t*>(&TPr[ts * kTPitch + 64])[flane];
            if (consumer) {
                const unsigned long long* e = reinterpret_cast<const unsigned long long*>(&Lr[ms * kLP + 32]);
                e0[u] = e[0];
                e1[u] = e[1];
            } else {
                e0[u] = e1[u] = 0ull;
            }
        }
        if (consumer) {
            // pairs the previous strip had not written when they were prefetched:
            // wait for them, then fall kAheadA columns behind so later prefetches hit
#pragma unroll
            for (int u = 0; u < kU; u++) {
                const int s = s0 + u;
                if ((FAST || s < ncols) && (tag_of(e0[u]) != a.tag || tag_of(e1[u]) != a.tag)) {
                    e0[u] = pack_tag(wait_pair(a.h_in + 2 * (size_t)s, a.tag, sh, a.err), a.tag);
                    e1[u] = pack_tag(wait_pair(a.h_in + 2 * (size_t)s + 1, a.tag, sh, a.err), a.tag);
                    wait_pair(a.h_in + 2 * (size_t)min(s + kAheadA, ncols - 1) + 1, a.tag, sh, a.err);
                }
            }
        }

        float lo[kU], vv[kU], opv[kU], opev[kU];
        bool actv[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) {
            const int s = s0 + u;
            const int m = s - lane;
            const bool act = FAST ? vrow : (vrow && (m >= 0) && (m < ncols));
            // pv of the upwind row's node in this column plus pev of its node in
            // the previous column, summed by the lane above
            float x_in = __shfl_up_sync(0xffffffffu, my_x, 1);
            if (lane == 0) {  // upwind row of the strip: the previous strip, or outside the grid
                const bool have = consumer && (FAST || s < ncols);
                x_in = fadd(have ? val_of(e0[u]) : 0.0f, pev_hold);
                pev_hold = have ? val_of(e1[u]) : 0.0f;
            }
            const float mu = fadd(fadd(lam_in[u], x_in), my_pe);
            float npv = 0.0f, npe = 0.0f, npev = 0.0f, l = mu, v = 0.0f;
            const int br = code[u] & 7;
            if (act && br != 0) {
                l = 0.0f;
                v = fmul(mu, c2[u]);
                const float cc = c1[u];
                switch (br) {
                case 1: npv = mu; break;
                case 2: npe = mu; break;
                case 3: npv = fmul(mu, cc); npe = fmul(mu, -cc); npev = mu; break;
                case 4: npe = fmul(mu, fsub(1.0f, cc)); npev = fmul(mu, cc); break;
                default: npv = fmul(mu, fsub(1.0f, cc)); npev = fmul(mu, cc); break;
                }
            }
            lo[u] = l;
            vv[u] = v;
            opv[u] = npv;
            opev[u] = npev;
            actv[u] = act;
            my_x = fadd(npv, my_pev);  // this node's pv + the previous node's pev
            my_pe = npe;
            my_pev = npev;
        }

#pragma unroll
        for (int u = 0; u < kU; u++) {
            const int s = s0 + u;
            if (actv[u]) {
                Lr[msl[u] * kLP + tix] = lo[u];
                pV[-32 * u] = vv[u];
                if (lane == 31 && a.h_out != nullptr) {
                    const int m = s - 31;
                    st_u64(a.h_out + 2 * (size_t)m, pack_tag(opv[u], a.tag));
                    st_u64(a.h_out + 2 * (size_t)m + 1, pack_tag(opev[u], a.tag));
                }
            }
        }
        pV -= 32 * kU;
        int wb = b0 + (kRing - 31);  // slot of march s0 - 31
        if (wb >= kRing) wb -= kRing;
#pragma unroll
        for (int u = 0; u < kU; u++) {
            const int s = s0 + u;
            if (FAST || (s >= 31 && s < nsteps)) {
                int ws = wb + u;
                if (ws >= kRing) ws -= kRing;
                if (vrow) *pW = Lr[ws * kLP + tix];
                pW += dL;
            }
        }
        b0 += kU;
        if (b0 >= kRing) b0 -= kRing;
        tb0 += kU;
        if (tb0 >= kTR) tb0 -= kTR;
    };
    // column blocks in the order the march finishes them: the counted sweep
    // is the reverse of sweep 0 (SX > 0), which marches down the columns, so
    // block b is done once lane 31 has passed its first window column (the
    // tile's extra node column, the next block's first, came earlier)
    const int blo = a.c0 / kGT, bhi = (a.c0 + ncols - 1) / kGT;
    int next_b = bhi;
    auto count_done = [&](int s_end) {
        while (SX > 0 && next_b >= blo) {
            const int wcol = max(next_b * kGT, a.c0) - a.c0;
            const int m = ncols - 1 - wcol;  // march of that column
            if (m + 31 > s_end) break;
            __threadfence();  // this lane's terms before the count
            __syncwarp();
            if (lane == 0) atomicAdd(a.ready + next_b, 1u);
            next_b--;
        }
    };
#pragma unroll 1
    for (int s0 = 0; s0 < nsteps; s0 += kU) {
        if constexpr (INTERIOR) {
            if (s0 >= 31 && s0 + kLookA + kU <= ncols)
                block(s0, std::true_type{});
            else
                block(s0, std::false_type{});
        } else {
            block(s0, std::false_type{});
        }
        if (a.ready) count_done(s0 + kU - 1);
    }
    cp_wait<0>();
    __syncwarp();
}

// (kMaxWarps * 32, 1): the block size alone as the bound caps the kernel at
// 64 registers and spills the strip loop's state.
// The reverse sweeps of every shot (persistent gangs, as the forward). f:
// inside a fused launch, count finished column blocks in the last reverse
// sweep and flag each shot's initialisation term.
template <bool INTERIOR>
__device__ void adjoint_body(const AdjParams& p, const FuseParams* f)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CtaShared* cs = reinterpret_cast<CtaShared*>(smem_raw);
    AdjRing* rings = reinterpret_cast<AdjRing*>(smem_raw + ((sizeof(CtaShared) + 15) & ~size_t(15)));
    const int tid = threadIdx.x;
    const GangPos gp = gang_pos(p.G);
    const int nzz = p.nzz, nstrips = p.nstrips;
    float* lam = p.lam + (size_t)gp.gang * p.lam_per_gang;
    unsigned long long* hb = p.hand + (size_t)gp.gang * 4 * nstrips * 2 * p.maxcols;
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
        const int ncols = sh.ncols;
        const unsigned tag = (p.epoch << 10) | (unsigned)(it & 1023);
        // seed: adjoint of the final field from the pick gradients. The window
        // is zeroed by the whole gang, then each seeded node sums its
        // receivers' terms in receiver order (the order of a receiver-by-
        // receiver accumulation, hence the same bits).
        {
            const int gt = gp.g * blockDim.x + tid, gn = p.G * blockDim.x;
            const size_t nw = (size_t)nzz * ncols;
#pragma unroll 4
            for (size_t q = gt; q < nw; q += gn) lam[q] = 0.0f;
            gang_barrier(bar, (++nbar) * p.G, cs, p.err);
            const float* pg = p.pick_grad + (size_t)sh.orig * p.nrec;
            for (int n = gt; n < p.nseed; n += gn) {
                const int col = p.seed_col[n] - sh.c0;
                if (col < 0 || col >= ncols) continue;
                float acc = 0.0f;
                bool any = false;
                for (int e = p.seed_ptr[n]; e < p.seed_ptr[n + 1]; e++) {
                    const int rr = p.seed_rec[e];
                    const int jl = p.rec_jg[rr] - sh.c0;
                    const float g = pg[rr];
                    if (jl - 1 < 1 || jl + 2 > ncols - 2 || !(g == g)) continue;
                    acc = fadd(acc, fmul(g, p.seed_w[e]));
                    any = true;
                }
                if (any) lam[(size_t)p.seed_row[n] + (size_t)col * nzz] = acc;
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
                a.ready = (f && sw == 0) ? f->ready + (size_t)a.k * f->nblk : nullptr;
                a.c0 = sh.c0;
                switch (sw) {
                case 0: adj_strip<1, 1, INTERIOR>(a); break;
                case 1: adj_strip<-1, 1, INTERIOR>(a); break;
                case 2: adj_strip<1, -1, INTERIOR>(a); break;
                default: adj_strip<-1, -1, INTERIOR>(a); break;
                }
            }
        }
        gang_barrier(bar, (++nbar) * p.G, cs, p.err);
        if (gp.g == 0 && tid < 9) {
            const int aa = tid % 3, bb = tid / 3;
            const int zi = sh.sIdz + aa - 1, xl = sh.sIdx - sh.c0 + bb - 1;
            p.lam_init[(size_t)sh.orig * 9 + tid] = lam[(size_t)zi + (size_t)xl * nzz];
        }
        if (f && gp.g == 0) {
            __threadfence();
            __syncthreads();
            if (tid == 0) st_release_gpu(f->shot_done + sh.orig, f->done_tag);
        }
        gang_barrier(bar, (++nbar) * p.G, cs, p.err);
    }
}

template <bool INTERIOR>
__global__ void __launch_bounds__(kMaxWarps * 32, 1) k_adjoint(AdjParams p)
{
    adjoint_body<INTERIOR>(p, nullptr);
}

// g(a, b) = sum over shots (caller order, FP64) of the shot's FP32 sum over
// sweeps 0..3 and corners (dr, dc) = (0,0),(0,1),(1,0),(1,1) of the matching
// node terms, plus the 3x3 initialisation term lam_init * dist.
//
// One CTA per tile of 32 rows (one strip) x kGT columns. The terms of node
// (i, j) in a sweep sit in the tape in the forward strip's skewed step order,
// so the nodes a tile reads (its rows and the first row of the next strip,
// its columns and one more) are, per shot and sweep, one contiguous run of
// kGT + 32 tape steps of the strip plus kGT + 1 entries of the next strip.
// These runs stream through kGStages shared-memory stages (cp.async) while
// the threads sum their cells' terms in the order above. The shots covering
// the tile's columns come from a per-column-block list built on the host,
// staged in shared memory kGChunk at a time.
constexpr int kGSteps = kGT + 32;   // tape steps a tile's strip spans per sweep
constexpr int kGStages = 3;
constexpr int kGChunk = 128;

struct __align__(16) GatherStage {
    float v[kGSteps * 32];
    uint32_t code[kGSteps * 8];      // code bytes
    float v2[kGT + 1];               // next strip, first row
    uint32_t code2[kGT + 1];         // the aligned words holding its code bytes
};

struct GatherSmem {
    GatherStage stg[kGStages];
    GatherShot shots[kGChunk];
};

// One stage's node terms for the thread's NQ = 32 / W cells (columns W
// apart) when the tile lies inside the shot's window and is not the last
// strip: the same terms and order as the general loop of gather_tile (cells q,
// corners (0,0),(0,1),(1,0),(1,1)), with the node slots one base plus offsets
// fixed by the sweep's directions.
template <int W, bool SZPOS, bool SXPOS>
__device__ __forceinline__ void gather_interior(const GatherStage& S, float* g, int a, int rb, int bl0, int ncols,
                                                int fmlo, bool last_row)
{
    constexpr int NQ = 32 / W;
    const unsigned char* cbytes = reinterpret_cast<const unsigned char*>(S.code);
    // node (ni, nj) = (a + 1 - dr, bl + 1 - dc) of cell (a, bl), bl = bl0 + W q
    const int fl0 = SZPOS ? a + 1 - rb : rb + 31 - (a + 1);
    const int fm0 = SXPOS ? bl0 + 1 : ncols - 1 - (bl0 + 1);
    const int base = (fm0 + fl0 - fmlo) * 32 + fl0;
    constexpr int DR = SZPOS ? -33 : 33;            // ni - 1: fl -/+ 1
    constexpr int DC = SXPOS ? -32 : 32;            // nj - 1: fm -/+ 1
    constexpr int DQ = SXPOS ? 32 * W : -32 * W;    // nj + W: fm +/- W
#pragma unroll
    for (int q = 0; q < NQ; q++)
#pragma unroll
        for (int dr = 0; dr < 2; dr++)
#pragma unroll
            for (int dc = 0; dc < 2; dc++) {
                int cd;
                float v;
                if (dr == 0 && last_row) {  // node row a + 1: the next strip's first row
                    const int q2 = (SXPOS ? bl0 + W * q + 1 - dc : ncols - 1 - (bl0 + W * q + 1 - dc)) - fmlo;
                    cd = (S.code2[q2] >> (SZPOS ? 0 : 24)) & 0xff;
                    v = S.v2[q2];
                } else {
                    const int idx = base + q * DQ + dr * DR + dc * DC;
                    cd = cbytes[idx];
                    v = S.v[idx];
                }
                if ((cd & 7) && (cd & 0x18) == ((dr << 3) | (dc << 4))) g[q] = fadd(g[q], v);
            }
}

__device__ __forceinline__ void cp_async16_cg(void* smem, const void* gmem)
{
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}

// Bounded wait of one thread until *p >= target (acquire); false after the
// limit, with the error flag set.
__device__ __forceinline__ bool wait_count(const unsigned* p, unsigned target, int* err, unsigned long long wait_ns)
{
    if (ld_acquire_gpu(p) >= target) return true;
    const unsigned long long t0 = global_ns();
    const unsigned long long lim = wait_ns ? wait_ns : kSpinNs;
    long long n = 0;
    while (ld_acquire_gpu(p) < target) {
        if (*(volatile int*)err) return false;
        __nanosleep(256);
        if (++n > kSpinLimit || ((n & 255) == 0 && global_ns() - t0 > lim)) {
            atomicExch(err, 2);
            return false;
        }
    }
    return true;
}

// g(a, b) of one tile (strip k, column block cb) by 32 W threads: thread
// (warp w, lane l) owns cells (32 k + l, 32 cb + w + W q), q < 32 / W.
// VTI: the batch was anisotropic; each shot's summed terms (its gradient with
// respect to its own qP slowness) are multiplied by the shot's derivative
// factors of the qP slowness before the FP64 sum over shots, giving dJ/dS,
// dJ/dC11 and dJ/dC13. FUSED: the tile runs inside the reverse-sweep launch
// while other shots may still be writing terms; it reads the tape through L2
// only (cp.async.cg, ld.global.cg) and waits for a shot's flag before using
// its initialisation term. Returns false when a wait gave up.
template <int W, bool VTI, bool FUSED>
__device__ bool gather_tile(const GatherParams& p, GatherSmem& sm, int k, int cb)
{
    constexpr int NQ = 32 / W;
    const int tid = threadIdx.x;
    const int c = cb * kGT;
    const int rb = 32 * k;
    const bool next_strip = k + 1 < p.nstrips;
    const int a = rb + (tid & 31);   // the thread's cells: row a, columns c + (tid>>5) + W q
    const int cq = tid >> 5;

    // node-column range of stage (shot entry e, sweep sw) in march order
    auto fm_range = [&](const GatherShot& t, int sw, int& fmlo, int& fmhi) {
        const int jlo = max(c - t.c0, 0);
        const int jhi = min(c + kGT - t.c0, t.ncols - 1);   // covered cells' columns and one more
        fmlo = (sw < 2) ? jlo : t.ncols - 1 - jhi;
        fmhi = (sw < 2) ? jhi : t.ncols - 1 - jlo;
    };
    auto issue = [&](const GatherShot& t, int sw, GatherStage& S) {
        int fmlo, fmhi;
        fm_range(t, sw, fmlo, fmhi);
        const int nst = t.ncols + 31;
        const size_t base = tape_strip_base(t.tape_off, sw, k, p.nstrips, t.ncols);
        for (int q = tid; q < kGSteps * 8; q += blockDim.x) {
            const int st = fmlo + (q >> 3);
            if (st < nst) {
                if (FUSED) cp_async16_cg(&S.v[q * 4], p.vrec + base + (size_t)st * 32 + (q & 7) * 4);
                else cp_async16(&S.v[q * 4], p.vrec + base + (size_t)st * 32 + (q & 7) * 4);
            }
        }
        for (int q = tid; q < kGSteps * 2; q += blockDim.x) {
            const int st = fmlo + (q >> 1);
            if (st < nst) cp_async16(&S.code[q * 4], p.tcode + base + (size_t)st * 32 + (q & 1) * 16);
        }
        if (next_strip) {
            const size_t base2 = tape_strip_base(t.tape_off, sw, k + 1, p.nstrips, t.ncols);
            const int fl2 = (sw == 1 || sw == 3) ? 31 : 0;
            for (int q = tid; q <= fmhi - fmlo; q += blockDim.x) {
                const size_t e = base2 + (size_t)(fmlo + q + fl2) * 32 + fl2;
                if (FUSED) {
                    S.v2[q] = __ldcg(p.vrec + e);
                } else {
                    cp_async4(&S.v2[q], p.vrec + e);
                }
                cp_async4(&S.code2[q], p.tcode + (e & ~(size_t)3));
            }
        }
        cp_commit();
    };

    double total[NQ], t11[VTI ? NQ : 1], t13[VTI ? NQ : 1];
    float g[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        total[q] = 0.0;
        g[q] = 0.0f;
        if (VTI) t11[q] = t13[q] = 0.0;
    }
    bool ok = true;
    const int e_end = p.blk_ptr[cb + 1];
#pragma unroll 1
    for (int e0 = p.blk_ptr[cb]; e0 < e_end; e0 += kGChunk) {
        const int n = min(kGChunk, e_end - e0);
        __syncthreads();  // the previous chunk's list and stages are no longer read
        for (int q = tid; q < n; q += blockDim.x) sm.shots[q] = p.blk_shots[e0 + q];
        __syncthreads();
        const int nst = 4 * n;  // stages (entry, sweep) of the chunk
        for (int i = 0; i < kGStages - 1 && i < nst; i++) issue(sm.shots[i >> 2], i & 3, sm.stg[i]);
#pragma unroll 1
        for (int i = 0; i < nst; i++) {
            const int ahead = min(kGStages - 1, nst - 1 - i);  // stages issued after stage i
            if (i + kGStages - 1 < nst) {
                const int j = i + kGStages - 1;
                issue(sm.shots[j >> 2], j & 3, sm.stg[j % kGStages]);
                cp_wait<kGStages - 1>();
            } else if (ahead == 1) {
                cp_wait<1>();
            } else {
                cp_wait<0>();
            }
            const GatherShot& t = sm.shots[i >> 2];
            const int sw = i & 3;
            if (FUSED && sw == 3 && tid == 0) {
                // the shot's initialisation term is written when its reverse sweeps end
                const bool src = t.sIdz + 1 >= rb && t.sIdz - 1 < rb + 32 && t.sIdx + 1 >= c && t.sIdx - 1 < c + kGT;
                if (src && !wait_count(p.shot_done + t.orig, p.done_tag, p.err, p.wait_ns)) ok = false;
            }
            __syncthreads();
            const bool szpos = !(sw == 1 || sw == 3), sxpos = sw < 2;
            int fmlo, fmhi;
            fm_range(t, sw, fmlo, fmhi);
            const GatherStage& S = sm.stg[i % kGStages];
            const unsigned char* cbytes = reinterpret_cast<const unsigned char*>(S.code);
            // the tile's cells and their nodes all inside the window, rows below the last strip
            const bool interior = (c >= t.c0) && (c + kGT - t.c0 <= t.ncols - 1) && (rb + 33 <= p.nzz);
            if (interior) {
                const int bl0 = c + cq - t.c0;
                const bool last_row = a == rb + 31;
                switch (sw) {
                case 0: gather_interior<W, true, true>(S, g, a, rb, bl0, t.ncols, fmlo, last_row); break;
                case 1: gather_interior<W, false, true>(S, g, a, rb, bl0, t.ncols, fmlo, last_row); break;
                case 2: gather_interior<W, true, false>(S, g, a, rb, bl0, t.ncols, fmlo, last_row); break;
                default: gather_interior<W, false, false>(S, g, a, rb, bl0, t.ncols, fmlo, last_row); break;
                }
            }
#pragma unroll
            for (int q = 0; q < NQ; q++) {
                const int bc = c + cq + W * q;
                const int bl = bc - t.c0;
                if (a >= p.nzz || bc >= p.nxx || bl < 0 || bl >= t.ncols) continue;
                if (!interior)
                for (int dr = 0; dr < 2; dr++)
                    for (int dc = 0; dc < 2; dc++) {
                        const int ni = a + 1 - dr, nj = bl + 1 - dc;
                        if (ni >= p.nzz || nj >= t.ncols) continue;
                        const int fm = sxpos ? nj : t.ncols - 1 - nj;
                        int cd;
                        float v;
                        if (ni < rb + 32) {
                            const int fl = szpos ? ni - rb : rb + 31 - ni;
                            const int idx = (fm + fl - fmlo) * 32 + fl;
                            cd = cbytes[idx];
                            v = S.v[idx];
                        } else {
                            const int q2 = fm - fmlo;
                            cd = (S.code2[q2] >> (szpos ? 0 : 24)) & 0xff;
                            v = S.v2[q2];
                        }
                        if ((cd & 7) && ((cd >> 3) & 1) == dr && ((cd >> 4) & 1) == dc) g[q] = fadd(g[q], v);
                    }
                if (sw == 3) {
                    const int da = a - t.sIdz + 1, db = bc - t.sIdx + 1;
                    if (da >= 0 && da < 3 && db >= 0 && db < 3) {
                        const double d = src_dist(a, bc, p.nb, p.dx, p.dz, t.sx, t.sz);
                        const float li = FUSED ? __ldcg(p.lam_init + (size_t)t.orig * 9 + da + 3 * db)
                                               : p.lam_init[(size_t)t.orig * 9 + da + 3 * db];
                        g[q] = fadd(g[q], fmul(li, __double2float_rn(d)));
                    }
                    if (VTI) {
                        const float* f = p.vfac + t.q_off + (size_t)a + (size_t)bl * p.nzz;
                        total[q] += (double)g[q] * (double)f[0];
                        t11[q] += (double)g[q] * (double)f[p.vfac_total];
                        t13[q] += (double)g[q] * (double)f[2 * p.vfac_total];
                    } else {
                        total[q] += (double)g[q];
                    }
                    g[q] = 0.0f;
                }
            }
            __syncthreads();  // stage i's buffer is refilled by stage i + kGStages
        }
    }
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        const int bc = c + cq + W * q;
        if (a < p.nzz && bc < p.nxx) {
            p.grad[(size_t)a + (size_t)bc * p.nzz] = __double2float_rn(total[q]);
            if (VTI) {
                p.grad_c11[(size_t)a + (size_t)bc * p.nzz] = __double2float_rn(t11[q]);
                p.grad_c13[(size_t)a + (size_t)bc * p.nzz] = __double2float_rn(t13[q]);
            }
        }
    }
    return ok;
}

// The gather as its own launch: one CTA of 8 warps per tile.
template <bool VTI>
__global__ void __launch_bounds__(256) k_gather(GatherParams p)
{
    extern __shared__ __align__(16) unsigned char gsm_raw[];
    GatherSmem& sm = *reinterpret_cast<GatherSmem*>(gsm_raw);
    const int ntx = (p.nxx + kGT - 1) / kGT;
    gather_tile<8, VTI, false>(p, sm, blockIdx.x / ntx, blockIdx.x % ntx);
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

namespace sf {

// Reverse sweeps and gather in one launch of 32 W-thread CTAs (see
// FuseParams). Every CTA of the launch is resident at once (the host sizes
// the grid to the device), the reverse sweeps never wait on the gather, and
// every gather wait is bounded.
template <bool INTERIOR, int W>
__global__ void __launch_bounds__(kMaxWarps * 32, 1) k_adjoint_gather(AdjParams p, GatherParams g, FuseParams f)
{
    if ((int)blockIdx.x < f.nadj) {
        adjoint_body<INTERIOR>(p, &f);
        return;
    }
    extern __shared__ __align__(16) unsigned char fsm_raw[];
    GatherSmem& sm = *reinterpret_cast<GatherSmem*>(fsm_raw);
    __shared__ int tile_s, ok_s;
    const int ntiles = p.nstrips * f.nblk;
#pragma unroll 1
    while (true) {
        if (threadIdx.x == 0) {
            const int t = (int)atomicAdd(f.tile_ctr, 1u);
            int ok = 1;
            if (t < ntiles) {
                // bottom strips first, columns right to left: the order the last
                // reverse sweep finishes them
                const int k = p.nstrips - 1 - t / f.nblk, cb = f.nblk - 1 - t % f.nblk;
                const unsigned cover = (unsigned)(g.blk_ptr[cb + 1] - g.blk_ptr[cb]);
                ok = wait_count(f.ready + (size_t)k * f.nblk + cb, cover, g.err, g.wait_ns);
                if (ok && k + 1 < p.nstrips) ok = wait_count(f.ready + (size_t)(k + 1) * f.nblk + cb, cover, g.err, g.wait_ns);
            }
            tile_s = t;
            ok_s = ok;
        }
        __syncthreads();
        const int t = tile_s, ok = ok_s;
        __syncthreads();
        if (t >= ntiles || !ok) break;
        if (!gather_tile<W, false, true>(g, sm, p.nstrips - 1 - t / f.nblk, f.nblk - 1 - t % f.nblk)) break;
    }
}

}  // namespace sf
