// Strip-systolic fast sweeping (GB300, sm_103a).
//
// A shot window of nzz rows x ncols columns is cut into 32-row strips; a warp
// sweeps a strip with lane l owning one row and marching across the columns,
// lane l running l steps behind lane 0. At step s lane l updates node (row(l),
// column of march index s-l), so the three upwind values of the reference
// update (modeling.cu:324-326) are: the lane above's result of the previous
// step (shfl), the lane's own previous result, and the lane's own previous
// upwind value. Consecutive strips (usually on other SMs) are chained through
// global memory without fences: the last lane of strip p writes each value of
// its row together with a tag (launch epoch and shot number) as one 64-bit
// store; lane 0 of strip p+1 prefetches the pair through the same cp.async
// pipeline as its own columns and checks the tag. A stale pair (the producer
// has not got there yet) sends lane 0 into a bounded spin on the pair itself,
// after which it waits until the producer is some columns further on, so
// later prefetches find their data. Producers never wait on consumers, so
// every wait points to a lower strip and the schedule cannot deadlock however
// strips are spread over warps and CTAs.
//
// Column chunks are staged into a per-warp shared-memory ring by cp.async,
// a few march columns ahead (32 consecutive rows = one coalesced 128-byte
// request per field), and lane l reads its own row of column s-l from the
// ring. With slot pitches of 32 (T) and 36 (S, with the halo row and the
// handoff pair) floats both the coalesced fill and the skewed read are
// bank-conflict free. Finished columns go back to global memory through the
// same ring, coalesced. The march runs in blocks of a few steps: one wait for
// the staged columns per block, the block's ring reads, its node updates
// (the only serial chain), then its stores.
//
// Any order of node updates that respects the sweep's dependency DAG gives the
// same bits as the reference's anti-diagonal launches, so this schedule is a
// bit-exact replacement of eikonal_solver (modeling.cu:123-159).
#pragma once
#include <type_traits>

#include "sf_device.cuh"

namespace sf {

constexpr int kU = 4;       // march steps per block of the reverse sweeps' strip loop
constexpr int kRing = 48;   // column slots per warp ring of the reverse sweeps and the plain forward

// Block size, staging lead (march columns, a multiple of the block) and ring
// length of a forward strip loop: 4, 8 and 48 slots for the plain solve; 2,
// 4 and 40 for the taped one, which keeps a tape record per step of the
// block in registers (measured 19% faster than 4 and 8 there). After a stall
// a consumer lets its producer get `lead` columns ahead (lead + block
// measured 1% slower). The ring holds the 32 marches the lanes work on, the
// lead and two blocks, so a block's prefetches never refill a slot that the
// block before it still read: RING >= 31 + LOOK + 2 U.
template <bool TAPE>
struct FwdBlock {
    static constexpr int U = TAPE ? 2 : 4;
    static constexpr int LOOK = TAPE ? 4 : 8;
    static constexpr int AHEAD = LOOK;
    static constexpr int RING = TAPE ? 40 : 48;
    static_assert(LOOK % U == 0 && RING % U == 0 && RING >= 31 + LOOK + 2 * U, "ring too small");
};
constexpr int kSP = 36;     // S slot pitch: rows rb-1 .. rb+31 at 0..32, handoff pair at 34..35
constexpr int kSPc = 40;    // compensated: S slot pitch, handoff pairs {hi,tag},{lo,tag} at 36..39
constexpr int kTP = 32;     // T slot pitch
constexpr int kMaxWarps = 16;
// compensated kernels keep a second traveltime ring (the lo parts): at most
// 8 warps per CTA fit in shared memory
constexpr int kMaxWarpsComp = 8;
// the taped interior-block forward kernels bound their CTAs to 8 warps, which
// lets them keep more of the block's state in registers (measured 2.6%
// faster on the headline batch; the other kernels measured slower that way)
constexpr int kMaxWarpsTapedInterior = 8;
constexpr long long kSpinLimit = 1ll << 30;          // iterations
constexpr unsigned long long kSpinNs = 2000000000ull;  // and at most ~2 s (default; sf_set_wait_limit)

// A warp's forward ring of R column slots: S (slot pitch kSP; compensated
// kSPc, with the two handoff pairs of the hi and the lo parts), T, and in the
// compensated arithmetic L (the lo parts of the traveltimes), one after the
// other. Every size is a multiple of 16 bytes.
template <bool COMP>
constexpr size_t ring_bytes(int R)
{
    return sizeof(float) * (size_t)R * ((COMP ? kSPc : kSP) + (COMP ? 2 : 1) * kTP);
}

// Per-CTA shared state (static part), followed by the CTA's warp rings in
// dynamic shared memory.
struct CtaShared {
    int abort_flag;
    int item;
    unsigned long long wait_ns;  // time limit of every bounded wait of the CTA
    float init[9];
};

__device__ __forceinline__ void cp_async4(void* smem, const void* gmem)
{
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem)
{
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__device__ __forceinline__ int ld_volatile(const int* p) { return *(const volatile int*)p; }
__device__ __forceinline__ void st_volatile(int* p, int v) { *(volatile int*)p = v; }
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_u64(unsigned long long* p, unsigned long long v)
{
    asm volatile("st.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long pack_tag(float v, unsigned tag)
{
    return ((unsigned long long)tag << 32) | (unsigned long long)__float_as_uint(v);
}
__device__ __forceinline__ unsigned tag_of(unsigned long long e) { return (unsigned)(e >> 32); }
__device__ __forceinline__ float val_of(unsigned long long e) { return __uint_as_float((unsigned)e); }

// Everything one warp needs for one strip of one sweep.
struct StripArgs {
    const float* S;   // slowness of the window, column stride ldS
    int ldS;
    float* T;         // traveltimes of the window, column stride nzz
    float* Tl;        // compensated: their lo parts, same layout
    int nzz, ncols;
    int k;            // strip index: rows [32k, 32k+32)
    int nstrips;
    int sIdz, sIdx;   // source node (window coordinates)
    int skip_i, skip_j;
    Consts kc;
    const float* init;  // 9 values in shared memory
    unsigned char* ring;  // this warp's ring (ring_bytes<COMP>(FwdBlock<TAPE>::RING) bytes at least)
    CtaShared* sh;
    const unsigned long long* h_in;  // {value, tag} of the upwind strip's row by march column (nullptr: first strip)
    unsigned long long* h_out;       // pairs this strip feeds to the next one (nullptr: last strip)
    unsigned tag;                    // tag of this shot's pairs
    unsigned tag_in;                 // tag a consumer waits for (= tag; 1, which no launch writes, to test the timeout path)
    // tape (TAPE only): base of this sweep/strip, entries [step*32 + lane]
    uint8_t* tcode;
    float* tc1;
    float* tc2;
    int* err;
};

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait until the pair at p carries `tag`; returns its value. On
// timeout it behaves like wait_counter.
__device__ __forceinline__ float wait_pair(const unsigned long long* p, unsigned tag, CtaShared* sh, int* err)
{
    unsigned long long e = ld_relaxed_u64(p);
    if (tag_of(e) == tag) return val_of(e);
    const unsigned long long t0 = global_ns();
    long long n = 0;
    while (tag_of(e = ld_relaxed_u64(p)) != tag) {
        if (ld_volatile(&sh->abort_flag) || *(volatile int*)err) return 0.0f;
        __nanosleep(32);
        if (++n > kSpinLimit || ((n & 255) == 0 && global_ns() - t0 > sh->wait_ns)) {
            st_volatile(&sh->abort_flag, 1);
            atomicExch(err, 2);
            return 0.0f;
        }
    }
    return val_of(e);
}

// Bounded wait until the counter at p reaches `target` (acquire); returns
// the value seen. On timeout it raises the CTA's abort flag and the launch's
// error flag and returns `target`, and every later wait of the CTA (or of any
// CTA once the launch's flag is up) returns at once, so the kernel always
// finishes (its results are then void and the host reports SF_ERR_TIMEOUT).
__device__ __forceinline__ unsigned wait_counter(const unsigned* p, unsigned target, CtaShared* sh, int* err)
{
    unsigned v = ld_acquire_gpu(p);
    if (v >= target) return v;
    const unsigned long long t0 = global_ns();
    long long n = 0;
    while ((v = ld_acquire_gpu(p)) < target) {
        if (ld_volatile(&sh->abort_flag) || *(volatile int*)err) return target;
        __nanosleep(64);
        if (++n > kSpinLimit || ((n & 255) == 0 && global_ns() - t0 > sh->wait_ns)) {
            st_volatile(&sh->abort_flag, 1);
            atomicExch(err, 2);
            return target;
        }
    }
    return v;
}

// INTERIOR: blocks whose marches all lie inside the window run a body without
// bounds tests (fewer instructions per step, more code); otherwise every block
// runs the general body. SQ: square cells (node_update). All forms give the
// same bits. COMP: compensated arithmetic (node_update_comp): every
// traveltime the loop carries, stages, hands on and writes back is a pair
// (hi, lo); the second handoff pair of a column carries lo.
template <int SZ, int SX, bool SW0, bool TAPE, bool REF, bool INTERIOR, bool SQ, bool COMP = false>
__device__ __forceinline__ void run_strip(const StripArgs& a)
{
    constexpr int kU = FwdBlock<TAPE>::U, kLook = FwdBlock<TAPE>::LOOK, kAhead = FwdBlock<TAPE>::AHEAD;
    constexpr int kRing = FwdBlock<TAPE>::RING;
    const int lane = threadIdx.x & 31;
    const int nzz = a.nzz, ncols = a.ncols;
    const int rb = 32 * a.k;
    const int r = (SZ > 0) ? rb + lane : rb + 31 - lane;
    const bool vrow = r < nzz;
    const bool irow = (r >= 1) && (r <= nzz - 2);
    const int tix = r - rb;    // T slot index of row r; S slot index of row r-1
    const int six = tix + 1;   // S slot index of row r
    const int dr1 = (SZ > 0) ? 0 : 1;
    const int dc2 = (SX > 0) ? 0 : 1;
    const int dr2a = (r - 1 >= 1) ? 0 : 1;

    constexpr int SP = COMP ? kSPc : kSP;    // S slot pitch
    constexpr int PQ = COMP ? 36 : 34;       // first handoff pair in an S slot
    float* Sring = reinterpret_cast<float*>(a.ring);
    float* Tring = Sring + kRing * SP;
    float* Lring = COMP ? Tring + kRing * kTP : nullptr;
    constexpr int HS = COMP ? 2 : 1;         // handoff pairs per column

    // global rows this lane stages
    const int ls_row = rb - 1 + lane;
    const bool ls_ok = (ls_row >= 0) && (ls_row < nzz);
    const bool lx_ok = (lane == 0) && (rb + 31 < nzz);
    const bool lt_ok = (rb + lane) < nzz;
    const float* Sg = a.S;
    float* Tg = a.T;
    const int ldS = a.ldS;

    CtaShared* sh = a.sh;
    const bool consumer = (lane == 0) && (a.h_in != nullptr);
    // the strip holds rows of the source's 3x3 block (first sweep only)
    const bool src_rows = SW0 && (a.sIdz + 1 >= rb) && (a.sIdz - 1 <= rb + 31);
    auto col_of = [&](int m) { return (SX > 0) ? m : ncols - 1 - m; };
    // running source addresses of march column q (q advances by one per call)
    const long long dcol = (SX > 0) ? 1 : -1;
    const float* pS = Sg + (size_t)ls_row + (long long)col_of(0) * (long long)ldS;
    const float* pX = Sg + (size_t)(rb + 31) + (long long)col_of(0) * (long long)ldS;
    const float* pT = Tg + (size_t)(rb + lane) + (long long)col_of(0) * (long long)nzz;
    const float* pTl = COMP ? a.Tl + (size_t)(rb + lane) + (long long)col_of(0) * (long long)nzz : nullptr;
    const long long dS = dcol * (long long)ldS, dT = dcol * (long long)nzz;
    // FAST: every march the call touches lies inside the window (no bounds tests)
    auto prefetch = [&](int q, int slot, auto fast_tag) {
        constexpr bool FAST = decltype(fast_tag)::value;
        if (FAST || q < ncols) {
            if (ls_ok) cp_async4(&Sring[slot * SP + lane], pS);
            if (lx_ok) cp_async4(&Sring[slot * SP + 32], pX);
            if (!SW0 && lt_ok) {
                cp_async4(&Tring[slot * kTP + lane], pT);
                if (COMP) cp_async4(&Lring[slot * kTP + lane], pTl);
            }
            // upwind-row pair(s) of march q
            if (consumer) {
                if (COMP) cp_async16(&Sring[slot * SP + PQ], a.h_in + 2 * q);
                else cp_async8(&Sring[slot * SP + PQ], a.h_in + q);
            }
        }
        cp_commit();
        pS += dS;
        pX += dS;
        pT += dT;
        if (COMP) pTl += dT;
    };

    // let the previous strip get kAhead columns ahead before the first
    // prefetches of its values
    if (consumer) wait_pair(a.h_in + HS * min(kAhead, ncols - 1), a.tag_in, sh, a.err);
    __syncwarp();

    // prologue: march columns 0 .. kLook-1
#pragma unroll 1
    for (int q = 0; q < kLook; q++) prefetch(q, q, std::false_type{});

    // running destinations: write-back of march column s-31 (row r), tape entry s*32+lane
    float* pW = Tg + (size_t)r + (long long)col_of(0) * (long long)nzz;
    float* pWl = COMP ? a.Tl + (size_t)r + (long long)col_of(0) * (long long)nzz : nullptr;
    uint8_t* pcode = TAPE ? a.tcode + lane : nullptr;
    float* pc1 = TAPE ? a.tc1 + lane : nullptr;
    float* pc2 = TAPE ? a.tc2 + lane : nullptr;

    float tn = 0.0f, tvp = 0.0f;                          // own last result, last upwind value
    float tnl = 0.0f, tvpl = 0.0f;                        // their lo parts (compensated)
    float cU = 0.0f, cI = 0.0f;                           // carried S of rows r-1, r
    const int nsteps = ncols + 31;
    int b0 = 0;                                           // ring slot of march s0

    // Blocks of kU steps: one wait for the staged columns per block, then the
    // block's ring reads, its kU node updates, and its stores. Within a block
    // the node updates are the only serial chain; the loads before and the
    // stores after it are independent of it.
    auto block = [&](int s0, auto fast_tag) {
        constexpr bool FAST = decltype(fast_tag)::value;
        {
            int pf0 = b0 + kLook;
            if (pf0 >= kRing) pf0 -= kRing;
#pragma unroll
            for (int u = 0; u < kU; u++) prefetch(s0 + kLook + u, pf0 + u, fast_tag);
        }
        // march columns <= s0+kU are staged (SX < 0 reads one column ahead)
        cp_wait<kLook - 1>();
        __syncwarp();

        int ml = b0 - lane;                               // slot of march s0 - lane
        if (ml < 0) ml += kRing;
        int msl[kU];
        float nU[kU], nI[kU], told[kU], toldl[kU];
        unsigned long long pr[kU], prl[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) {
            int ms = ml + u;
            if (ms >= kRing) ms -= kRing;
            msl[u] = ms;
            // S of the new column: march m (SX>0) or m+1 (SX<0)
            const int ns = (SX > 0) ? ms : (ms + 1 == kRing ? 0 : ms + 1);
            nU[u] = Sring[ns * SP + tix];
            nI[u] = Sring[ns * SP + six];
            told[u] = SW0 ? kBig : Tring[ms * kTP + tix];
            toldl[u] = (COMP && !SW0) ? Lring[ms * kTP + tix] : 0.0f;
            pr[u] = consumer ? *reinterpret_cast<const unsigned long long*>(&Sring[ms * SP + PQ]) : 0ull;
            prl[u] = (COMP && consumer) ? *reinterpret_cast<const unsigned long long*>(&Sring[ms * SP + PQ + 2]) : 0ull;
        }
        if (consumer) {
            // a pair the previous strip had not written when it was prefetched:
            // wait for it, then fall kAhead columns behind so later prefetches hit
#pragma unroll
            for (int u = 0; u < kU; u++) {
                const int s = s0 + u;
                if ((FAST || s < ncols) && (tag_of(pr[u]) != a.tag_in || (COMP && tag_of(prl[u]) != a.tag_in))) {
                    pr[u] = pack_tag(wait_pair(a.h_in + HS * s, a.tag_in, sh, a.err), a.tag_in);
                    if (COMP) prl[u] = pack_tag(wait_pair(a.h_in + HS * s + 1, a.tag_in, sh, a.err), a.tag_in);
                    wait_pair(a.h_in + HS * min(s + kAhead, ncols - 1), a.tag_in, sh, a.err);
                }
            }
        }

        float tnw[kU], tnwl[kU];
        bool actv[kU];
        Rec rec[kU];
        // the block's kU node updates; EXACT divides with IEEE division
        auto updates = [&](auto exact_tag) -> bool {
        constexpr bool EXACT = decltype(exact_tag)::value;
        bool bad = false;
#pragma unroll
        for (int u = 0; u < kU; u++) {
            const int s = s0 + u;
            const int m = s - lane;
            const bool act = FAST ? vrow : (vrow && (m >= 0) && (m < ncols));
            const int j = col_of(m);
            // upwind value from the lane above (or the previous strip)
            float tv = __shfl_up_sync(0xffffffffu, tn, 1);
            float tvl = COMP ? __shfl_up_sync(0xffffffffu, tnl, 1) : 0.0f;
            if (consumer && (FAST || s < ncols)) {
                tv = val_of(pr[u]);
                if (COMP) tvl = val_of(prl[u]);
            }
            const float te = tn, tev = tvp;
            const float tel = tnl, tevl = tvpl;

            float to = told[u], tol = toldl[u];
            if (SW0 && src_rows) {
                const int da = r - a.sIdz + 1, db = j - a.sIdx + 1;
                if (da >= 0 && da < 3 && db >= 0 && db < 3) {
                    to = a.init[da + 3 * db];
                    tol = 0.0f;
                }
            }
            float U_j, I_j, U_jm, I_jm;
            if (SX > 0) { U_j = nU[u]; I_j = nI[u]; U_jm = cU; I_jm = cI; }
            else        { U_j = cU; I_j = cI; U_jm = nU[u]; I_jm = nI[u]; }

            float tnew = to, tnewl = tol;
            rec[u].code = 0; rec[u].c1 = 0.0f; rec[u].c2 = 0.0f;
            const bool inner = act && irow && (FAST || ((j >= 1) && (j <= ncols - 2))) &&
                               !(r == a.skip_i && j == a.skip_j);
            // rows: i1 (SZ>0: r-1, else r); columns: j-1 (clamped to 1), j
            const float Si1_j = (SZ > 0) ? U_j : I_j;
            const float Si1_jm = (SZ > 0) ? U_jm : I_jm;
            const float s1a = (j == 1) ? Si1_j : Si1_jm;   // S[i1][max(j-1,1)]
            const float s1b = Si1_j;                       // S[i1][j]
            const float Sa_j1 = (SX > 0) ? ((r == 1) ? I_jm : U_jm) : ((r == 1) ? I_j : U_j);
            const float s2a = Sa_j1;                       // S[max(i-1,1)][j1]
            const float s2b = (SX > 0) ? I_jm : I_j;       // S[i][j1]
            const float sref = (SX > 0) ? Si1_jm : Si1_j;  // S[i1][j1]
            const int dc1a = (j - 1 >= 1) ? 0 : 1;
            bool bad_u = false;
            if (inner) {
                if constexpr (COMP)
                    node_update_comp<TAPE, EXACT, SQ>(to, tol, tv, tvl, te, tel, tev, tevl, s1a, s1b, s2a, s2b, sref,
                                                      a.kc, dr1, dc1a, dc2, dr2a, tnew, tnewl, rec[u], bad_u);
                else
                    tnew = node_update<TAPE, REF, EXACT, SQ>(to, tv, te, tev, s1a, s1b, s2a, s2b, sref, a.kc,
                                                             dr1, dc1a, dc2, dr2a, rec[u], bad_u);
            }
            bad |= bad_u;
            tnw[u] = tnew;
            tnwl[u] = tnewl;
            actv[u] = act;
            // carry state
            if (act) {
                tn = tnew;
                tnl = tnewl;
            }
            tvp = tv;
            tvpl = tvl;
            cU = nU[u];
            cI = nI[u];
        }
        return bad;
        };
        {
            const float tn0 = tn, tvp0 = tvp, cU0 = cU, cI0 = cI, tnl0 = tnl, tvpl0 = tvpl;
            // a quotient outside the range the fast division was verified on
            // (one vote per block): the block again with IEEE division
            if (__any_sync(0xffffffffu, updates(std::false_type{}))) {
                tn = tn0;
                tvp = tvp0;
                tnl = tnl0;
                tvpl = tvpl0;
                cU = cU0;
                cI = cI0;
                updates(std::true_type{});
            }
        }

#pragma unroll
        for (int u = 0; u < kU; u++) {
            const int s = s0 + u;
            if (actv[u]) {
                Tring[msl[u] * kTP + tix] = tnw[u];
                if (COMP) Lring[msl[u] * kTP + tix] = tnwl[u];
            }
            if (TAPE && (FAST || s < nsteps)) {
                pcode[32 * u] = actv[u] ? rec[u].code : (uint8_t)0;
                pc1[32 * u] = rec[u].c1;
                pc2[32 * u] = rec[u].c2;
            }
            // feed the next strip: lane 31 just finished march s-31
            if (lane == 31 && a.h_out != nullptr && actv[u]) {
                st_u64(a.h_out + HS * (s - 31), pack_tag(tnw[u], a.tag));
                if (COMP) st_u64(a.h_out + HS * (s - 31) + 1, pack_tag(tnwl[u], a.tag));
            }
        }
        if (TAPE) {
            pcode += 32 * kU;
            pc1 += 32 * kU;
            pc2 += 32 * kU;
        }
        // write back the columns every lane has finished (march s-31)
        int wb = b0 + (kRing - 31);
        if (wb >= kRing) wb -= kRing;
#pragma unroll
        for (int u = 0; u < kU; u++) {
            const int s = s0 + u;
            if (FAST || (s >= 31 && s < nsteps)) {
                int ws = wb + u;
                if (ws >= kRing) ws -= kRing;
                if (vrow) {
                    *pW = Tring[ws * kTP + tix];
                    if (COMP) *pWl = Lring[ws * kTP + tix];
                }
                pW += dT;
                if (COMP) pWl += dT;
            }
        }
        b0 += kU;
        if (b0 >= kRing) b0 -= kRing;
    };
#pragma unroll 1
    for (int s0 = 0; s0 < nsteps; s0 += kU) {
        if constexpr (INTERIOR) {
            if (s0 >= 32 && s0 + kLook + kU <= ncols - 1)
                block(s0, std::true_type{});
            else
                block(s0, std::false_type{});
        } else {
            block(s0, std::false_type{});
        }
    }
    cp_wait<0>();
    __syncwarp();
}

// Gang-wide barrier: every CTA of the gang arrives once per barrier instance;
// `target` = (instance + 1) * gang size. Bounded like every wait.
__device__ __forceinline__ void gang_barrier(unsigned* ctr, unsigned target, CtaShared* sh, int* err)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(ctr, 1u);
        wait_counter(ctr, target, sh, err);
        __threadfence();
    }
    __syncthreads();
}

}  // namespace sf
