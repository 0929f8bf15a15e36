// Strip-systolic fast sweeping on one CTA (GB300, sm_103a).
//
// One CTA owns one shot window of nzz rows x ncols columns. The rows are cut
// into 32-row strips; a warp sweeps a strip with lane l owning one row and
// marching across the columns, lane l running l steps behind lane 0. At step s
// lane l updates node (row(l), column of march index s-l), so the three upwind
// values of the reference update (modeling.cu:324-326) are: the lane above's
// result of the previous step (shfl), the lane's own previous result, and the
// lane's own previous upwind value. Consecutive strips are chained through a
// per-CTA global buffer: the last lane of strip p writes its row, column by
// column, and publishes a counter in shared memory; lane 0 of strip p+1
// prefetches those values through the same cp.async pipeline as its own
// columns (bounded spin on the counter). Producers never wait on consumers, so
// every wait points to a lower strip and the schedule cannot deadlock however
// many strips share a warp.
//
// Column chunks are staged into a per-warp shared-memory ring by cp.async:
// at step s the warp fetches march column s+LOOK (32 consecutive rows = one
// coalesced 128-byte request per field), and lane l reads its own row of
// column s-l from the ring. With a slot pitch of 32 (T) and 34 (S) floats both
// the coalesced fill and the skewed read are bank-conflict free. Finished
// columns go back to global memory through the same ring, coalesced.
//
// Any order of node updates that respects the sweep's dependency DAG gives the
// same bits as the reference's anti-diagonal launches, so this schedule is a
// bit-exact replacement of eikonal_solver (modeling.cu:123-159).
#pragma once
#include "sf_device.cuh"

namespace sf {

constexpr int kRing = 48;   // column slots per warp ring (>= 32 + kLook + 1)
constexpr int kLook = 12;   // prefetch distance in march columns
constexpr int kSP = 34;     // S slot pitch: rows rb-1 .. rb+31 at 0..32, handoff at 33
constexpr int kTP = 32;     // T slot pitch
constexpr int kMaxWarps = 16;
constexpr long long kSpinLimit = 1ll << 30;          // iterations
constexpr unsigned long long kSpinNs = 2000000000ull;  // and at most ~2 s

struct WarpRing {
    float S[kRing * kSP];
    float T[kRing * kTP];
};

// Per-CTA shared state (static part), followed by kMaxWarps WarpRing blocks in
// dynamic shared memory (only the CTA's warps are used).
struct CtaShared {
    int prod[kMaxWarps];             // handoff entries published on channel w
    int abort_flag;
    int item;
    float init[9];
};

__device__ __forceinline__ void cp_async4(void* smem, const void* gmem)
{
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__device__ __forceinline__ int ld_volatile(const int* p) { return *(const volatile int*)p; }
__device__ __forceinline__ void st_volatile(int* p, int v) { *(volatile int*)p = v; }

// Everything one warp needs for one strip of one sweep.
struct StripArgs {
    const float* S;   // slowness of the window, column stride ldS
    int ldS;
    float* T;         // traveltimes of the window, column stride nzz
    int nzz, ncols;
    int k;            // strip index: rows [32k, 32k+32)
    int nstrips;
    int sIdz, sIdx;   // source node (window coordinates)
    int skip_i, skip_j;
    Consts kc;
    const float* init;  // 9 values in shared memory
    WarpRing* ring;
    CtaShared* sh;
    int w_in, e_in;     // consumer side: channel and entry base (-1: first strip)
    int w_out, e_out;   // producer side (-1: last strip)
    const float* h_in;  // handoff values of this strip's upwind row, by march column
    float* h_out;       // handoff values this strip feeds to the next one
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

// Bounded wait for *p >= target. On timeout it raises the CTA's abort flag and
// the launch's error flag, and every later wait returns at once, so the
// kernel always finishes (its results are then void and the host reports
// SF_ERR_TIMEOUT).
__device__ __forceinline__ bool spin_until(const int* p, int target, CtaShared* sh, int* err)
{
    if (ld_volatile(p) >= target) {
        __threadfence_block();
        return true;
    }
    const unsigned long long t0 = global_ns();
    long long n = 0;
    while (ld_volatile(p) < target) {
        if (ld_volatile(&sh->abort_flag)) return false;
        if (++n > kSpinLimit || ((n & 1023) == 0 && global_ns() - t0 > kSpinNs)) {
            st_volatile(&sh->abort_flag, 1);
            atomicExch(err, 2);
            return false;
        }
    }
    __threadfence_block();
    return true;
}

template <int SZ, int SX, bool SW0, bool TAPE, bool REF>
__device__ __forceinline__ void run_strip(const StripArgs& a)
{
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

    float* Sring = a.ring->S;
    float* Tring = a.ring->T;

    // global rows this lane stages
    const int ls_row = rb - 1 + lane;
    const bool ls_ok = (ls_row >= 0) && (ls_row < nzz);
    const bool lx_ok = (lane == 0) && (rb + 31 < nzz);
    const bool lt_ok = (rb + lane) < nzz;
    const float* Sg = a.S;
    float* Tg = a.T;
    const size_t ldS = (size_t)a.ldS;

    CtaShared* sh = a.sh;
    const bool consumer = (lane == 0) && (a.w_in >= 0);
    auto col_of = [&](int m) { return (SX > 0) ? m : ncols - 1 - m; };
    auto prefetch = [&](int q, int slot) {
        if (q < ncols) {
            const int jq = col_of(q);
            if (ls_ok) cp_async4(&Sring[slot * kSP + lane], Sg + (size_t)ls_row + (size_t)jq * ldS);
            if (lx_ok) cp_async4(&Sring[slot * kSP + 32], Sg + (size_t)(rb + 31) + (size_t)jq * ldS);
            if (!SW0 && lt_ok)
                cp_async4(&Tring[slot * kTP + lane], Tg + (size_t)(rb + lane) + (size_t)jq * nzz);
            if (consumer) {
                // upwind-row value of march q, once the previous strip has published it
                spin_until(&sh->prod[a.w_in], a.e_in + q + 1, sh, a.err);
                cp_async4(&Sring[slot * kSP + 33], a.h_in + q);
            }
        }
        cp_commit();
    };

    // prologue: march columns 0 .. kLook-1
#pragma unroll 1
    for (int q = 0; q < kLook; q++) prefetch(q, q);

    int pf_slot = kLook;                                  // slot of march s+kLook
    int m_slot = (kRing - lane) % kRing;                  // slot of march s-lane
    int wb_slot = (kRing - 31) % kRing;                   // slot of march s-31
    float tn = 0.0f, tvp = 0.0f;                          // own last result, last upwind value
    float cU = 0.0f, cI = 0.0f;                           // carried S of rows r-1, r
    const int nsteps = ncols + 31;

#pragma unroll 1
    for (int s = 0; s < nsteps; s++) {
        prefetch(s + kLook, pf_slot);
        cp_wait<kLook - 1>();
        __syncwarp();

        const int m = s - lane;
        const bool act = vrow && (m >= 0) && (m < ncols);
        const int j = col_of(m);
        // S of the new column: march m (SX>0) or m+1 (SX<0)
        int n_slot = (SX > 0) ? m_slot : (m_slot + 1 == kRing ? 0 : m_slot + 1);
        float nU = Sring[n_slot * kSP + tix];
        float nI = Sring[n_slot * kSP + six];

        // upwind value from the lane above (or the previous strip)
        float tv = __shfl_up_sync(0xffffffffu, tn, 1);
        if (consumer) tv = Sring[m_slot * kSP + 33];
        const float te = tn, tev = tvp;

        float told;
        if (SW0) {
            told = kBig;
            const int da = r - a.sIdz + 1, db = j - a.sIdx + 1;
            if (da >= 0 && da < 3 && db >= 0 && db < 3) told = a.init[da + 3 * db];
        } else {
            told = Tring[m_slot * kTP + tix];
        }

        float U_j, I_j, U_jm, I_jm;
        if (SX > 0) { U_j = nU; I_j = nI; U_jm = cU; I_jm = cI; }
        else        { U_j = cU; I_j = cI; U_jm = nU; I_jm = nI; }

        float tnew = told;
        Rec rec;
        rec.code = 0; rec.c1 = 0.0f; rec.c2 = 0.0f;
        const bool inner = act && irow && (j >= 1) && (j <= ncols - 2) &&
                           !(r == a.skip_i && j == a.skip_j);
        if (inner) {
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
            tnew = node_update<TAPE, REF>(told, tv, te, tev, s1a, s1b, s2a, s2b, sref, a.kc, dr1,
                                     dc1a, dc2, dr2a, rec);
        }
        if (act) Tring[m_slot * kTP + tix] = tnew;
        if (TAPE) {
            const size_t t = (size_t)s * 32 + lane;
            a.tcode[t] = act ? rec.code : (uint8_t)0;
            a.tc1[t] = rec.c1;
            a.tc2[t] = rec.c2;
        }

        // feed the next strip: lane 31 just finished march s-31
        if (lane == 31 && a.w_out >= 0 && act) {
            a.h_out[m] = tnew;
            __threadfence_block();
            st_volatile(&sh->prod[a.w_out], a.e_out + m + 1);
        }

        // write back the column every lane has finished
        const int mw = s - 31;
        if (mw >= 0 && vrow) {
            Tg[(size_t)r + (size_t)col_of(mw) * nzz] = Tring[wb_slot * kTP + tix];
        }

        // carry state
        if (act) tn = tnew;
        tvp = tv;
        cU = nU;
        cI = nI;
        if (++pf_slot == kRing) pf_slot = 0;
        if (++m_slot == kRing) m_slot = 0;
        if (++wb_slot == kRing) wb_slot = 0;
    }
    cp_wait<0>();
    __syncwarp();
}

}  // namespace sf
