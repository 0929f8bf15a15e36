// C ABI of the GB300 eikonal engine (include/seisfat2d.h): context, buffers,
// launches of the forward kernels. Compiled for sm_103a only.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/seisfat2d.h"
#include "sf_engine.h"

using namespace sf;

// ------------------------------------------------------------------ helpers

const char* sf_status_string(int s)
{
    switch (s) {
    case SF_OK: return "ok";
    case SF_ERR_ARG: return "invalid argument";
    case SF_ERR_CUDA: return "CUDA error";
    case SF_ERR_TIMEOUT: return "in-kernel wait timed out";
    case SF_ERR_RANGE: return "source or window outside the grid";
    case SF_ERR_STATE: return "call out of order";
    case SF_ERR_NOMEM: return "device allocation failed";
    default: return "unknown status";
    }
}

int sf_fail(sf_ctx* c, int status, const std::string& msg)
{
    if (c) c->err = msg;
    return status;
}

int sf_cuda_check(sf_ctx* c, cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return SF_OK;
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return sf_fail(c, SF_ERR_NOMEM, m);
    return sf_fail(c, SF_ERR_CUDA, m);
}

#define CK(call)                                                          \
    do {                                                                  \
        int _st = sf_cuda_check(c, (call), #call);                        \
        if (_st != SF_OK) return _st;                                     \
    } while (0)

int sf_dev_reserve(sf_ctx* c, void** p, size_t* cap, size_t bytes)
{
    if (bytes <= *cap && *p) return SF_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMalloc(p, want);
    if (e != cudaSuccess) {
        *p = nullptr;
        return sf_cuda_check(c, e, "cudaMalloc");
    }
    *cap = want;
    return SF_OK;
}

int sf_dev_reserve_zero(sf_ctx* c, void** p, size_t* cap, size_t bytes)
{
    const bool grow = !(bytes <= *cap && *p);
    int rc = sf_dev_reserve(c, p, cap, bytes);
    if (rc || !grow) return rc;
    return sf_cuda_check(c, cudaMemset(*p, 0, *cap), "cudaMemset");
}

unsigned sf_next_epoch(sf_ctx* c)
{
    // after a wrap an epoch's tags could meet pairs an earlier cycle left in
    // the handoff buffers: the next forward and adjoint launches clear them
    if (c->epoch == (1u << 22) - 1) c->hand_stale_f = c->hand_stale_a = true;
    c->epoch = (c->epoch % ((1u << 22) - 1)) + 1;
    return c->epoch;
}

// ------------------------------------------------------------------ kernels

namespace {

// expand_boundary (modeling.cu:204-232): clamp-to-edge copy of the model.
__global__ void k_expand(const float* __restrict__ in, int nx, int nz, int nb, float* __restrict__ out)
{
    const int nzz = nz + 2 * nb, nxx = nx + 2 * nb;
    const size_t n = (size_t)nzz * nxx;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        int i = (int)(idx % nzz), j = (int)(idx / nzz);
        int si = min(max(i - nb, 0), nz - 1), sj = min(max(j - nb, 0), nx - 1);
        out[idx] = in[si + (size_t)sj * nz];
    }
}

// Checks fdiv_k against __fdiv_rn for b = divs[w] over all dividends of [1, 2)
// (both signs follow by symmetry); rbs[w] = RN(1/b), bad bit w set on any
// difference.
__global__ void k_verify_div(const float* divs, int n, float* rbs, int* bad)
{
    const unsigned total = (unsigned)n << 23;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const int w = t >> 23;
        const float b = divs[w], rb = __frcp_rn(b);
        if ((t & 0x7fffffu) == 0) rbs[w] = rb;
        const float a = __uint_as_float(0x3f800000u | (t & 0x7fffffu));
        bool out_of_range = false;
        if (__float_as_uint(fdiv_k<false>(a, b, rb, true, out_of_range)) != __float_as_uint(__fdiv_rn(a, b)))
            atomicOr(bad, 1 << w);
    }
}

// compute_seismogram on a device field (modeling.cu:161-194).
__global__ void k_picks(const float* __restrict__ T, int nzz, int ncols, int c0, int nb, float dx,
                        float dz, const float* __restrict__ rx, const float* __restrict__ rz,
                        int nrec, float* __restrict__ out)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    int i, j;
    float xd, zd;
    float v = __int_as_float(0x7fc00000);
    if (pick_geom(rx[r], rz[r], dx, dz, nb, nzz, ncols, c0, i, j, xd, zd))
        v = pick_value(T, nzz, i, j, xd, zd);
    out[r] = v;
}

}  // namespace

size_t sf_fwd_smem_bytes(int warps, bool comp, bool tape)
{
    const int slots = tape ? FwdBlock<true>::RING : FwdBlock<false>::RING;
    return ((sizeof(CtaShared) + 15) & ~size_t(15)) + (size_t)warps * (comp ? ring_bytes<true>(slots) : ring_bytes<false>(slots));
}

// ------------------------------------------------------------------ context

extern "C" const char* sf_ctx_last_error(const sf_ctx* c) { return c ? c->err.c_str() : "null context"; }

extern "C" int sf_ctx_create(sf_ctx** out, int nx, int nz, float dx, float dz, int device)
{
    if (!out) return SF_ERR_ARG;
    *out = nullptr;
    if (nx < 2 || nz < 2 || !(dx > 0.0f) || !(dz > 0.0f)) return SF_ERR_ARG;
    sf_ctx* c = new sf_ctx();
    c->dev = device;
    c->nx = nx;
    c->nz = nz;
    c->nb = 3;
    c->nxx = nx + 2 * c->nb;
    c->nzz = nz + 2 * c->nb;
    c->dx = dx;
    c->dz = dz;
    Consts& k = c->kc;
    k.dx = dx;
    k.dz = dz;
    k.dz2i = 1.0f / (dz * dz);  // modeling.cu:64-65 (host, no contraction)
    k.dx2i = 1.0f / (dx * dx);
    k.hyp = sqrtf(dx * dx + dz * dz);
    k.D = k.dz2i + k.dx2i;
    k.K = k.dz2i * k.dx2i;
    k.kA = k.dz2i - k.dx2i;
    k.kB = k.dx2i - k.dz2i;
    k.k2K = 2.0f * k.K;
    int st = sf_cuda_check(c, cudaSetDevice(device), "cudaSetDevice");
    if (st == SF_OK) {
        cudaDeviceProp prop;
        st = sf_cuda_check(c, cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
        if (st == SF_OK) c->sms = prop.multiProcessorCount;
    }
    if (st == SF_OK) st = sf_verify_divisors(c);
    size_t cap = 0;
    if (st == SF_OK) st = sf_dev_reserve(c, (void**)&c->d_S, &cap, sizeof(float) * (size_t)c->nxx * c->nzz);
    cap = 0;
    if (st == SF_OK) st = sf_dev_reserve(c, (void**)&c->d_flags, &cap, 256);
    if (st == SF_OK) st = sf_cuda_check(c, cudaMemset(c->d_flags, 0, 256), "cudaMemset");
    if (st == SF_OK) st = sf_fwd_setup(c);
    if (st != SF_OK) {
        sf_ctx_destroy(c);
        return st;
    }
    *out = c;
    return SF_OK;
}

extern "C" int sf_ctx_destroy(sf_ctx* c)
{
    if (!c) return SF_OK;
    cudaSetDevice(c->dev);
    sf_plan_release(c);
    sf_adjoint_release(c);
    void* bufs[] = {c->d_S, c->d_flags, c->d_shots, c->d_T, c->d_rx, c->d_rz, c->d_picks, c->d_Sq,
                    c->d_tcode, c->d_tc1, c->d_tc2, c->d_model, c->d_cij_all, c->d_hand, c->d_ctr,
                    c->d_skern, c->d_upd, c->d_wav, c->d_mig, c->d_kgeo, c->d_kint, c->d_kpart,
                    c->d_vfac, c->d_gcij, c->d_fuse, c->d_Tl};
    for (void* b : bufs)
        if (b) cudaFree(b);
    delete c;
    return SF_OK;
}

extern "C" int sf_ctx_dims(const sf_ctx* c, int* nxx, int* nzz, int* nb)
{
    if (!c) return SF_ERR_ARG;
    if (nxx) *nxx = c->nxx;
    if (nzz) *nzz = c->nzz;
    if (nb) *nb = c->nb;
    return SF_OK;
}

extern "C" int sf_set_launch(sf_ctx* c, int warps, int gang_warps)
{
    if (!c) return SF_ERR_ARG;
    if (warps < 0 || warps > kMaxWarps) return sf_fail(c, SF_ERR_ARG, "warps per CTA must be 1..16");
    if (gang_warps < 0 || gang_warps > 1024) return sf_fail(c, SF_ERR_ARG, "gang warps must be 0..1024");
    if (warps) c->warps = warps;
    c->gang_warps = gang_warps;
    c->plan_dirty = true;  // a planned batch is reconfigured before its next iteration
    return SF_OK;
}

extern "C" int sf_set_wait_limit(sf_ctx* c, double seconds)
{
    if (!c) return SF_ERR_ARG;
    if (!(seconds >= 0.0 && seconds <= 60.0)) return sf_fail(c, SF_ERR_ARG, "wait limit must be in [0, 60] s");
    c->wait_ns = (unsigned long long)(seconds * 1e9);  // 0: the default of about 2 s
    c->plan_dirty = true;
    return SF_OK;
}

extern "C" int sf_test_stall_next_batch(sf_ctx* c)
{
    if (!c) return SF_ERR_ARG;
    c->stall_next = true;
    return SF_OK;
}

extern "C" int sf_set_arithmetic(sf_ctx* c, int mode)
{
    if (!c) return SF_ERR_ARG;
    if (mode != SF_ARITH_REFERENCE && mode != SF_ARITH_IEEE && mode != SF_ARITH_COMPENSATED)
        return sf_fail(c, SF_ERR_ARG, "unknown arithmetic");
    c->arith = mode;
    c->plan_dirty = true;
    return SF_OK;
}

extern "C" int sf_get_arithmetic(const sf_ctx* c, int* mode)
{
    if (!c || !mode) return SF_ERR_ARG;
    *mode = c->arith;
    return SF_OK;
}

extern "C" int sf_set_strip_loop(sf_ctx* c, int mode)
{
    if (!c) return SF_ERR_ARG;
    if (mode != SF_LOOP_AUTO && mode != SF_LOOP_GENERAL && mode != SF_LOOP_INTERIOR)
        return sf_fail(c, SF_ERR_ARG, "unknown strip-loop mode");
    c->strip_loop = mode;
    c->plan_dirty = true;
    return SF_OK;
}

extern "C" int sf_get_strip_loop(const sf_ctx* c, int* mode, int* last_interior)
{
    if (!c) return SF_ERR_ARG;
    if (mode) *mode = c->strip_loop;
    if (last_interior) *last_interior = c->batch_interior ? 1 : 0;
    return SF_OK;
}

extern "C" int sf_get_launch(const sf_ctx* c, int* warps, int* gang_warps)
{
    if (!c) return SF_ERR_ARG;
    if (warps) *warps = c->warps;
    if (gang_warps) *gang_warps = c->gang_warps;
    return SF_OK;
}

// Warps per shot ("slots"): all strips of a shot on their own warp when the
// device can hold every shot that way, else the largest divisor of the strip
// count that keeps all shots resident at once (at least 1).
int sf_gang_shape(sf_ctx* c, const void* kernel, size_t smem, int nshots, int nstrips, int gang_warps, int* G,
                  int* NG)
{
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, c->warps * 32, smem));
    if (per_sm < 1) return sf_fail(c, SF_ERR_CUDA, "kernel does not fit on an SM");
    const long long cap_ctas = (long long)per_sm * c->sms;
    int slots = gang_warps;
    if (slots <= 0) {
        const long long cap_warps = cap_ctas * c->warps;
        slots = 1;
        for (int d = 1; d <= nstrips; d++)
            if (nstrips % d == 0 && (long long)d * nshots <= cap_warps) slots = d;
        if ((long long)nstrips * std::max(1, nshots) <= cap_warps) slots = nstrips;
    }
    int g = std::max(1, (slots + c->warps - 1) / c->warps);
    if (g > cap_ctas) g = (int)cap_ctas;
    *G = g;
    *NG = (int)std::max(1LL, std::min<long long>(nshots, cap_ctas / g));
    return SF_OK;
}

// Reciprocals of the four constant divisors and whether the fast division
// equals IEEE division for them (see fdiv_k).
int sf_verify_divisors(sf_ctx* c)
{
    Consts& k = c->kc;
    float h_div[4] = {k.dx, k.dz, k.hyp, k.D}, h_rb[4] = {0, 0, 0, 0};
    int h_bad = 0;
    float* d_div = nullptr;
    int* d_bad = nullptr;
    CK(cudaMalloc(&d_div, 8 * sizeof(float) + sizeof(int)));
    d_bad = reinterpret_cast<int*>(d_div + 8);
    cudaError_t e = cudaMemcpy(d_div, h_div, sizeof(h_div), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d_bad, 0, sizeof(int));
    if (e == cudaSuccess) {
        k_verify_div<<<c->sms * 8, 256>>>(d_div, 4, d_div + 4, d_bad);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(h_rb, d_div + 4, sizeof(h_rb), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&h_bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d_div);
    CK(e);
    k.rdx = h_rb[0];
    k.rdz = h_rb[1];
    k.rhyp = h_rb[2];
    k.rD = h_rb[3];
    k.mflags = (~h_bad) & 0xf;
    return SF_OK;
}

namespace sf {
// accessors of the k_shots instantiations: tape, reference arithmetic,
// interior-block body, compensated arithmetic
const void* sf_kshots_0000();
const void* sf_kshots_0010();
const void* sf_kshots_0100();
const void* sf_kshots_0110();
const void* sf_kshots_1000();
const void* sf_kshots_1010();
const void* sf_kshots_1100();
const void* sf_kshots_1110();
const void* sf_kshots_0001();
const void* sf_kshots_0011();
const void* sf_kshots_1001();
const void* sf_kshots_1011();
}  // namespace sf

// The compensated arithmetic has no reference-build variant.
const void* sf_kshots_kernel(bool tape, bool ref, bool interior, bool comp)
{
    if (comp) ref = false;
    switch (((int)tape << 3) | ((int)ref << 2) | ((int)interior << 1) | (int)comp) {
    case 0x0: return sf::sf_kshots_0000();
    case 0x2: return sf::sf_kshots_0010();
    case 0x4: return sf::sf_kshots_0100();
    case 0x6: return sf::sf_kshots_0110();
    case 0x8: return sf::sf_kshots_1000();
    case 0xa: return sf::sf_kshots_1010();
    case 0xc: return sf::sf_kshots_1100();
    case 0xe: return sf::sf_kshots_1110();
    case 0x1: return sf::sf_kshots_0001();
    case 0x3: return sf::sf_kshots_0011();
    case 0x9: return sf::sf_kshots_1001();
    case 0xb: return sf::sf_kshots_1011();
    default: return nullptr;
    }
}

// The qP pass kernels: arithmetic (reference / IEEE / compensated) x
// derivative factors (taped batches).
const void* sf_kqp_kernel(bool ref, bool comp, bool fact)
{
    if (comp) return fact ? (const void*)k_qp<false, true, true> : (const void*)k_qp<false, true, false>;
    if (ref) return fact ? (const void*)k_qp<true, false, true> : (const void*)k_qp<true, false, false>;
    return fact ? (const void*)k_qp<false, false, true> : (const void*)k_qp<false, false, false>;
}

// The interior-block body saves instructions per step but adds code. It
// measured faster for 100 equal windows of 1707 x 357 with every shot at once
// and one warp per strip (forward 3.93 -> 3.58 ms, reverse sweeps 6.66 ->
// 5.46 ms), and slower for 1000 windows of 2-8 km with four strips per warp
// (forward 46 -> 55 ms, reverse 46 -> 67 ms) and for 200 equal windows with
// two strips per warp (9.39 -> 9.67 ms). SF_LOOP_AUTO takes it only when all
// three conditions of the first case hold.
bool sf_interior_loops(sf_ctx* c, const void* kernel, size_t smem, int G)
{
    if (c->strip_loop == SF_LOOP_GENERAL) return false;
    if (c->strip_loop == SF_LOOP_INTERIOR) return true;
    const int ns = (int)c->hshots.size();
    if (ns == 0) return false;
    if (c->hshots.front().ncols != c->hshots.back().ncols) return false;  // sorted widest first
    if ((long long)G * c->warps < (c->nzz + 31) / 32) return false;       // a warp per strip
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, c->warps * 32, smem) != cudaSuccess)
        return false;
    return (long long)ns * G <= (long long)per_sm * c->sms;
}

int sf_fwd_setup(sf_ctx* c)
{
    for (int k = 0; k < 16; k++) {
        const bool tape = k & 8, comp = k & 1;
        const size_t mx = sf_fwd_smem_bytes(comp ? kMaxWarpsComp : kMaxWarps, comp, tape);
        const void* f = sf_kshots_kernel(tape, k & 4, k & 2, comp);
        if (f) CK(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mx));
    }
    return sf_adj_setup(c);
}

// ------------------------------------------------------------------ models

extern "C" int sf_set_slowness(sf_ctx* c, const float* s, int layout, int mem)
{
    if (!c || !s) return SF_ERR_ARG;
    CK(cudaSetDevice(c->dev));
    const size_t npad = (size_t)c->nxx * c->nzz;
    if (layout == SF_LAYOUT_PADDED) {
        CK(cudaMemcpy(c->d_S, s, npad * sizeof(float),
                      mem == SF_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
        return SF_OK;
    }
    if (layout != SF_LAYOUT_MODEL) return sf_fail(c, SF_ERR_ARG, "unknown layout");
    const size_t nm = (size_t)c->nx * c->nz;
    int st = sf_dev_reserve(c, (void**)&c->d_model, &c->cap_model, nm * sizeof(float));
    if (st) return st;
    CK(cudaMemcpy(c->d_model, s, nm * sizeof(float),
                  mem == SF_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
    k_expand<<<std::min<size_t>((npad + 255) / 256, 4096), 256>>>(c->d_model, c->nx, c->nz, c->nb, c->d_S);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    return SF_OK;
}

extern "C" int sf_get_slowness(sf_ctx* c, float* out, int mem)
{
    if (!c || !out) return SF_ERR_ARG;
    CK(cudaSetDevice(c->dev));
    CK(cudaMemcpy(out, c->d_S, sizeof(float) * (size_t)c->nxx * c->nzz,
                  mem == SF_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost));
    return SF_OK;
}

// Deterministic quantisation of one padded field (modeling.cu:264-279).
static void compress_field(const float* in, size_t n, uint16_t* out, float* vmax, float* vmin)
{
    float mx = -1e20f, mn = 1e20f;
    for (size_t i = 0; i < n; i++) {
        mn = std::fmin(in[i], mn);
        mx = std::fmax(in[i], mx);
    }
    *vmax = mx;
    *vmin = mn;
    for (size_t i = 0; i < n; i++) {
        if (mx == mn) {
            out[i] = 1;
            continue;
        }
        float v = 1.0f + (float)(65535 - 1) * (in[i] - mn) / (mx - mn);
        out[i] = (uint16_t)v;
    }
}

static int upload_codes(sf_ctx* c, const uint16_t* const codes[6], int mem)
{
    const size_t npad = (size_t)c->nxx * c->nzz;
    int st = sf_dev_reserve(c, (void**)&c->d_cij_all, &c->cap_cij, 6 * npad * sizeof(uint16_t));
    if (st) return st;
    for (int q = 0; q < 6; q++) {
        CK(cudaMemcpy(c->d_cij_all + q * npad, codes[q], npad * sizeof(uint16_t),
                      mem == SF_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
    }
    c->have_cij = true;
    return SF_OK;
}

extern "C" int sf_set_stiffness(sf_ctx* c, const float* const cij[6], int mem)
{
    if (!c || !cij) return SF_ERR_ARG;
    for (int q = 0; q < 6; q++)
        if (!cij[q]) return SF_ERR_ARG;
    CK(cudaSetDevice(c->dev));
    const int nx = c->nx, nz = c->nz, nb = c->nb, nzz = c->nzz, nxx = c->nxx;
    const size_t nm = (size_t)nx * nz, npad = (size_t)nxx * nzz;
    std::vector<float> model(nm), padded(npad);
    std::vector<std::vector<uint16_t>> codes(6, std::vector<uint16_t>(npad));
    for (int q = 0; q < 6; q++) {
        if (mem == SF_MEM_DEVICE) CK(cudaMemcpy(model.data(), cij[q], nm * sizeof(float), cudaMemcpyDeviceToHost));
        else std::memcpy(model.data(), cij[q], nm * sizeof(float));
        for (int j = 0; j < nxx; j++)
            for (int i = 0; i < nzz; i++) {
                int si = std::min(std::max(i - nb, 0), nz - 1), sj = std::min(std::max(j - nb, 0), nx - 1);
                padded[i + (size_t)j * nzz] = model[si + (size_t)sj * nz];
            }
        compress_field(padded.data(), npad, codes[q].data(), &c->mm[2 * q + 1], &c->mm[2 * q]);
    }
    const uint16_t* ptrs[6];
    for (int q = 0; q < 6; q++) ptrs[q] = codes[q].data();
    return upload_codes(c, ptrs, SF_MEM_HOST);
}

extern "C" int sf_set_stiffness_codes(sf_ctx* c, const uint16_t* const codes[6], const float mm[12], int mem)
{
    if (!c || !codes || !mm) return SF_ERR_ARG;
    for (int q = 0; q < 6; q++)
        if (!codes[q]) return SF_ERR_ARG;
    CK(cudaSetDevice(c->dev));
    std::memcpy(c->mm, mm, sizeof(c->mm));
    return upload_codes(c, codes, mem);
}

// ------------------------------------------------------------------ shots

// Interior cells the reference's launch schedule (modeling.cu:123-159) never
// updates, for a grid of nzz x ncols, per sweep: the middle-band thread count
// (level-2) can fall one short of the diagonal when min(n)-2 is a multiple of
// the 256-thread block.
void sf_skip_cells(int ncols, int nzz, int si[4], int sj[4])
{
    const int nxx = ncols, total = nxx + nzz - 2, mn = std::min(nxx, nzz), mxl = std::max(nxx, nzz);
    for (int s = 0; s < 4; s++) {
        si[s] = sj[s] = -1;
        const int zd = (s == 2 || s == 3) ? -1 : 1;
        const int xd = (s == 0 || s == 2) ? -1 : 1;
        for (int level = 0; level < total; level++) {
            int zo, xo;
            switch (s) {
            case 0: zo = (level < nxx) ? 0 : level - nxx + 1; xo = (level < nxx) ? level : nxx - 1; break;
            case 1: zo = (level < nzz) ? nzz - level - 1 : 0; xo = (level < nzz) ? 0 : level - nzz + 1; break;
            case 2: zo = (level < nzz) ? level : nzz - 1; xo = (level < nzz) ? nxx - 1 : nxx - 1 - (level - nzz + 1); break;
            default: zo = (level < nxx) ? nzz - 1 : nzz - 1 - (level - nxx + 1); xo = (level < nxx) ? nxx - level - 1 : 0; break;
            }
            int n = (level < mn) ? level + 1 : (level >= mxl) ? total - level : total - mn - mxl + level;
            int nl = ((n + 255) / 256) * 256;
            int lo = 0, hi = 1 << 30;
            if (zd > 0) { lo = std::max(lo, 1 - zo); hi = std::min(hi, nzz - 2 - zo); }
            else { lo = std::max(lo, zo - (nzz - 2)); hi = std::min(hi, zo - 1); }
            if (xd > 0) { lo = std::max(lo, 1 - xo); hi = std::min(hi, nxx - 2 - xo); }
            else { lo = std::max(lo, xo - (nxx - 2)); hi = std::min(hi, xo - 1); }
            for (int e = std::max(lo, nl); e <= hi; e++) {
                si[s] = zo + zd * e;
                sj[s] = xo + xd * e;
            }
        }
    }
}

// Builds the device shot table (sorted widest window first for the work
// queue). Returns SF_ERR_RANGE for a source outside its window.
int sf_prepare_shots(sf_ctx* c, const sf_shot* shots, int nshots, bool tape)
{
    c->plan_valid = false;  // the planned batch's tables are replaced
    // a new generation unless the table comes out the same as before (an
    // early error return leaves it new)
    const std::vector<ShotDev> prev = c->hshots;
    const unsigned long long prev_gen = c->shots_gen++;
    c->hshots.resize(nshots);
    long long toff = 0, tape_off = 0, q_off = 0;
    const int nstrips = (c->nzz + 31) / 32;
    int maxcols = 0;
    for (int b = 0; b < nshots; b++) {
        const sf_shot& s = shots[b];
        ShotDev d;
        std::memset(&d, 0, sizeof(d));
        d.c0 = s.c0;
        d.ncols = (s.ncols <= 0) ? c->nxx - s.c0 : s.ncols;
        if (d.c0 < 0 || d.ncols < 3 || d.c0 + d.ncols > c->nxx)
            return sf_fail(c, SF_ERR_RANGE, "shot " + std::to_string(b) + ": window outside the grid");
        // modeling.cu:112-113 (host float arithmetic, no contraction)
        float fx = (s.sx + 0.5f * c->dx) / c->dx;
        float fz = (s.sz + 0.5f * c->dz) / c->dz;
        if (!(fx > -1e9f && fx < 1e9f && fz > -1e9f && fz < 1e9f))
            return sf_fail(c, SF_ERR_RANGE, "shot " + std::to_string(b) + ": source not finite");
        d.sIdx = (int)fx + c->nb;
        d.sIdz = (int)fz + c->nb;
        d.sx = s.sx;
        d.sz = s.sz;
        const int sloc = d.sIdx - d.c0;
        if (d.sIdz < 1 || d.sIdz > c->nzz - 2 || sloc < 1 || sloc > d.ncols - 2)
            return sf_fail(c, SF_ERR_RANGE, "shot " + std::to_string(b) + ": source outside its window");
        // the skipped cells depend on the window width alone (nzz is the
        // context's): computed once per width for the context's lifetime
        auto it = c->skip_cache.find(d.ncols);
        if (it == c->skip_cache.end()) {
            std::array<int, 8> v;
            sf_skip_cells(d.ncols, c->nzz, v.data(), v.data() + 4);
            it = c->skip_cache.emplace(d.ncols, v).first;
        }
        for (int q = 0; q < 4; q++) { d.skip_i[q] = it->second[q]; d.skip_j[q] = it->second[4 + q]; }
        d.orig = b;
        d.t_off = toff;  // per-shot traveltime windows (tables, anisotropic batches)
        toff += (long long)c->nzz * d.ncols;
        d.tape_off = tape_off;
        if (tape) tape_off += 4LL * nstrips * (d.ncols + 31) * 32;
        d.q_off = q_off;
        q_off += (long long)c->nzz * d.ncols;
        maxcols = std::max(maxcols, d.ncols);
        c->hshots[b] = d;
    }
    std::stable_sort(c->hshots.begin(), c->hshots.end(),
                     [](const ShotDev& a, const ShotDev& b) { return a.ncols > b.ncols; });
    c->batch_T_floats = toff;
    c->batch_tape_entries = tape_off;
    c->batch_q_cells = q_off;
    c->batch_maxcols = maxcols;
    c->tables_index.assign(nshots, 0);
    for (int q = 0; q < nshots; q++) c->tables_index[c->hshots[q].orig] = q;
    if (prev.size() == c->hshots.size() &&
        std::memcmp(prev.data(), c->hshots.data(), prev.size() * sizeof(ShotDev)) == 0)
        c->shots_gen = prev_gen;
    return SF_OK;
}

// One solve of every shot of the prepared batch: kernel, gang shape,
// buffers, parameters. per_shot_T: every shot keeps its own traveltime window
// (tables, anisotropic batches) instead of one window per gang. Sshots: the
// shots' own slowness windows (the qP slowness of an anisotropic batch's
// second solve), or nullptr for S.
int sf_fwd_configure(sf_ctx* c, int nrec, bool per_shot_T, bool tape, int gang_warps, cudaStream_t st,
                     FwdLaunch* L, const float* Sshots)
{
    const int nshots = (int)c->hshots.size();
    const size_t nzz = c->nzz;
    const int nstrips = (c->nzz + 31) / 32;
    const bool comp = c->arith == SF_ARITH_COMPENSATED;
    if (comp && c->warps > kMaxWarpsComp)
        return sf_fail(c, SF_ERR_ARG, "the compensated arithmetic runs at most 8 warps per CTA (sf_set_launch)");
    const bool ref = c->arith == SF_ARITH_REFERENCE;
    const size_t smem = sf_fwd_smem_bytes(c->warps, comp, tape);
    const void* kern = sf_kshots_kernel(tape, ref, false, comp);
    int G, NG;
    int rc = sf_gang_shape(c, kern, smem, nshots, nstrips, gang_warps, &G, &NG);
    if (rc) return rc;
    // the interior-block kernels of taped batches are built for at most
    // kMaxWarpsTapedInterior warps per CTA; the gang shape must come from the
    // kernel that runs (every CTA of a gang resident at once)
    c->batch_interior = !(tape && c->warps > kMaxWarpsTapedInterior) && sf_interior_loops(c, kern, smem, G);
    if (c->batch_interior) {
        const void* ik = sf_kshots_kernel(tape, ref, true, comp);
        int Gi, NGi;
        rc = sf_gang_shape(c, ik, smem, nshots, nstrips, gang_warps, &Gi, &NGi);
        if (rc) return rc;
        if (c->strip_loop == SF_LOOP_INTERIOR || sf_interior_loops(c, ik, smem, Gi)) {
            kern = ik;
            G = Gi;
            NG = NGi;
        } else {
            c->batch_interior = false;
        }
    }
    if ((long long)(nshots + NG - 1) / NG > 1023)
        return sf_fail(c, SF_ERR_ARG, "too many shots per gang for one launch; split the batch");
    c->last_G = G;
    c->last_NG = NG;
    rc = sf_dev_reserve(c, (void**)&c->d_shots, &c->cap_shots, nshots * sizeof(ShotDev));
    if (rc) return rc;
    CK(cudaMemcpyAsync(c->d_shots, c->hshots.data(), nshots * sizeof(ShotDev), cudaMemcpyHostToDevice, st));
    const long long t_per_gang = per_shot_T ? 0 : (long long)nzz * c->batch_maxcols;
    const size_t tfloats = per_shot_T ? (size_t)c->batch_T_floats : (size_t)NG * t_per_gang;
    rc = sf_dev_reserve(c, (void**)&c->d_T, &c->cap_T, tfloats * sizeof(float));
    if (rc) return rc;
    if (comp) {
        rc = sf_dev_reserve(c, (void**)&c->d_Tl, &c->cap_Tl, tfloats * sizeof(float));
        if (rc) return rc;
    }
    const size_t hand_bytes =
        (size_t)NG * 4 * nstrips * c->batch_maxcols * sizeof(unsigned long long) * (comp ? 2 : 1);
    rc = sf_dev_reserve_zero(c, (void**)&c->d_hand, &c->cap_hand, hand_bytes);
    if (rc) return rc;
    const size_t nctr = (size_t)NG;
    rc = sf_dev_reserve(c, (void**)&c->d_ctr, &c->cap_ctr, nctr * sizeof(unsigned));
    if (rc) return rc;
    if (tape) {
        size_t n = (size_t)c->batch_tape_entries;
        rc = sf_dev_reserve(c, (void**)&c->d_tcode, &c->cap_tcode, n);
        if (!rc) rc = sf_dev_reserve(c, (void**)&c->d_tc1, &c->cap_tc1, n * sizeof(float));
        if (!rc) rc = sf_dev_reserve(c, (void**)&c->d_tc2, &c->cap_tc2, n * sizeof(float));
        if (rc) return rc;
    }
    FwdParams& p = L->p;
    std::memset(&p, 0, sizeof(p));
    p.S = c->d_S;
    p.Sshots = Sshots;
    p.nzz = c->nzz;
    p.nxx = c->nxx;
    p.nb = c->nb;
    p.kc = c->kc;
    p.shots = c->d_shots;
    p.nshots = nshots;
    p.G = G;
    p.NG = NG;
    p.maxcols = c->batch_maxcols;
    p.Tpool = c->d_T;
    p.Tlpool = comp ? c->d_Tl : nullptr;
    p.t_per_gang = t_per_gang;
    p.err = c->d_flags + 1;          // flags[1]: error flag
    p.wait_ns = c->wait_ns;
    p.hand = c->d_hand;
    p.bar = c->d_ctr;
    if (tape) {
        p.tcode = c->d_tcode;
        p.tc1 = c->d_tc1;
        p.tc2 = c->d_tc2;
    }
    p.rx = c->d_rx;
    p.rz = c->d_rz;
    p.nrec = nrec;
    L->kern = kern;
    L->grid = dim3(NG * G);
    L->block = dim3(c->warps * 32);
    L->smem = smem;
    L->nctr = nctr;
    L->hand_bytes = hand_bytes;
    return SF_OK;
}

int sf_kt_begin(sf_ctx* c, int k, cudaStream_t st)
{
    if (!c->timing) return SF_OK;
    c->kt_rec[k] = true;
    CK(cudaEventRecord(c->kt_ev[k][0], st));
    return SF_OK;
}

int sf_kt_end(sf_ctx* c, int k, cudaStream_t st)
{
    if (!c->timing) return SF_OK;
    CK(cudaEventRecord(c->kt_ev[k][1], st));
    return SF_OK;
}

// One forward launch (counters zeroed first), without the kernel timing.
int sf_fwd_launch(sf_ctx* c, FwdLaunch& L, float* d_picks, unsigned epoch, cudaStream_t st)
{
    L.p.picks = d_picks;
    L.p.epoch = epoch;
    CK(cudaMemsetAsync(L.p.bar, 0, L.nctr * sizeof(unsigned), st));
    if (c->hand_stale_f) {
        CK(cudaMemsetAsync(c->d_hand, 0, c->cap_hand, st));
        c->hand_stale_f = false;
    }
    void* args[] = {&L.p};
    CK(cudaLaunchKernel(L.kern, L.grid, L.block, args, L.smem, st));
    return SF_OK;
}

int sf_fwd_enqueue(sf_ctx* c, FwdLaunch& L, float* d_picks, unsigned epoch, cudaStream_t st)
{
    int rc = sf_kt_begin(c, SF_KT_FORWARD, st);
    if (!rc) rc = sf_fwd_launch(c, L, d_picks, epoch, st);
    if (rc) return rc;
    return sf_kt_end(c, SF_KT_FORWARD, st);
}

// The qP pass of the prepared anisotropic batch (k_qp) over the traveltime
// windows of the first solves: the qP slowness windows into d_Sq, and with
// `fact` the derivative factors into d_vfac.
int sf_qp_launch(sf_ctx* c, bool fact, cudaStream_t st)
{
    QpParams q;
    std::memset(&q, 0, sizeof(q));
    q.S = c->d_S;
    q.nzz = c->nzz;
    q.nb = c->nb;
    q.kc = c->kc;
    q.shots = c->d_shots;
    q.nshots = (int)c->hshots.size();
    q.Tpool = c->d_T;
    q.Tlpool = c->d_Tl;
    const size_t npad = (size_t)c->nxx * c->nzz;
    for (int k = 0; k < 6; k++) q.cij[k] = c->d_cij_all + k * npad;
    std::memcpy(q.mm, c->mm, sizeof(q.mm));
    q.Sq = c->d_Sq;
    q.vfac = fact ? c->d_vfac : nullptr;
    q.vfac_total = c->batch_q_cells;
    const bool comp = c->arith == SF_ARITH_COMPENSATED, ref = c->arith == SF_ARITH_REFERENCE;
    // x: the widest window's columns (grid-strided past 2048); y: the shots
    const unsigned gx = (unsigned)std::min(c->batch_maxcols, 2048);
    const unsigned gy = (unsigned)std::min(q.nshots, 65535);
    void* args[] = {&q};
    CK(cudaLaunchKernel(sf_kqp_kernel(ref, comp, fact), dim3(gx, gy), dim3(128), args, 0, st));
    return SF_OK;
}

int sf_launch_shots(sf_ctx* c, int ani, int nrec, float* d_picks, bool keep_tables, bool tape, int gang_warps,
                    cudaStream_t st)
{
    const bool stall = c->stall_next;  // sf_test_stall_next_batch
    c->stall_next = false;
    int rc;
    if (!ani) {
        FwdLaunch L;
        rc = sf_fwd_configure(c, nrec, keep_tables, tape, gang_warps, st, &L, nullptr);
        L.p.stall_handoff = stall ? 1 : 0;
        if (!rc) rc = sf_fwd_enqueue(c, L, d_picks, sf_next_epoch(c), st);
    } else {
        // eikonal_ani.cu:33-45: solve on S, qP pass, solve on the qP slowness;
        // every shot keeps its window between the launches
        rc = sf_dev_reserve(c, (void**)&c->d_Sq, &c->cap_Sq, (size_t)c->batch_q_cells * sizeof(float));
        if (!rc && tape)
            rc = sf_dev_reserve(c, (void**)&c->d_vfac, &c->cap_vfac, 3 * (size_t)c->batch_q_cells * sizeof(float));
        FwdLaunch L1, L2;
        if (!rc) rc = sf_fwd_configure(c, 0, true, false, gang_warps, st, &L1, nullptr);
        if (!rc) rc = sf_fwd_configure(c, nrec, true, tape, gang_warps, st, &L2, c->d_Sq);
        if (rc) return rc;
        // the second configuration may have grown the shared buffers
        L1.p.shots = c->d_shots;
        L1.p.Tpool = c->d_T;
        L1.p.Tlpool = L2.p.Tlpool;
        L1.p.hand = c->d_hand;
        L1.p.bar = c->d_ctr;
        L1.p.stall_handoff = L2.p.stall_handoff = stall ? 1 : 0;
        rc = sf_kt_begin(c, SF_KT_FORWARD, st);
        if (!rc) rc = sf_fwd_launch(c, L1, nullptr, sf_next_epoch(c), st);
        if (!rc) rc = sf_qp_launch(c, tape, st);
        if (!rc) rc = sf_fwd_launch(c, L2, d_picks, sf_next_epoch(c), st);
        if (!rc) rc = sf_kt_end(c, SF_KT_FORWARD, st);
    }
    if (rc) return rc;
    c->tables_valid = keep_tables;
    c->tape_valid = tape;
    c->batch_nrec = nrec;
    c->batch_ani = ani;
    c->gcij_valid = false;
    return SF_OK;
}

int sf_upload_receivers(sf_ctx* c, const float* rx, const float* rz, int nrec, cudaStream_t st)
{
    if (nrec <= 0) return SF_OK;
    int rc = sf_dev_reserve(c, (void**)&c->d_rx, &c->cap_rx, nrec * sizeof(float));
    if (!rc) rc = sf_dev_reserve(c, (void**)&c->d_rz, &c->cap_rz, nrec * sizeof(float));
    if (rc) return rc;
    if (c->h_rx.size() == (size_t)nrec && std::equal(rx, rx + nrec, c->h_rx.begin()) &&
        std::equal(rz, rz + nrec, c->h_rz.begin()))
        return SF_OK;  // unchanged receivers stay on the device
    c->h_rx.assign(rx, rx + nrec);
    c->h_rz.assign(rz, rz + nrec);
    c->recv_gen++;
    CK(cudaMemcpyAsync(c->d_rx, c->h_rx.data(), nrec * sizeof(float), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->d_rz, c->h_rz.data(), nrec * sizeof(float), cudaMemcpyHostToDevice, st));
    return SF_OK;
}

int sf_check_flags(sf_ctx* c, cudaStream_t st)
{
    CK(cudaStreamSynchronize(st));
    int err = 0;
    CK(cudaMemcpy(&err, c->d_flags + 1, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
        cudaMemset(c->d_flags + 1, 0, sizeof(int));
        return sf_fail(c, SF_ERR_TIMEOUT, "an in-kernel wait gave up; results of the launch are void");
    }
    return SF_OK;
}

extern "C" int sf_synchronize(sf_ctx* c, void* stream)
{
    if (!c) return SF_ERR_ARG;
    CK(cudaSetDevice(c->dev));
    return sf_check_flags(c, (cudaStream_t)stream);
}

extern "C" int sf_batch_forward(sf_ctx* c, int ani, const sf_shot* shots, int nshots, const float* rx,
                                const float* rz, int nrec, float* picks, int picks_mem, int flags,
                                void* stream)
{
    if (!c || !shots || nshots <= 0 || nrec < 0 || (nrec > 0 && (!rx || !rz || !picks)))
        return sf_fail(c, SF_ERR_ARG, "bad batch arguments");
    if (ani && !c->have_cij) return sf_fail(c, SF_ERR_STATE, "anisotropic solve needs sf_set_stiffness");
    const bool tape = (flags & SF_KEEP_TAPE) != 0, tables = (flags & SF_KEEP_TABLES) != 0;
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    c->tape_valid = false;
    c->tables_valid = false;
    int rc = sf_prepare_shots(c, shots, nshots, tape);
    if (rc) return rc;
    rc = sf_upload_receivers(c, rx, rz, nrec, st);
    if (rc) return rc;
    float* dp = nullptr;
    if (nrec > 0) {
        if (picks_mem == SF_MEM_DEVICE) dp = picks;
        else {
            rc = sf_dev_reserve(c, (void**)&c->d_picks, &c->cap_picks, (size_t)nshots * nrec * sizeof(float));
            if (rc) return rc;
            dp = c->d_picks;
        }
    }
    rc = sf_launch_shots(c, ani, nrec, dp, tables, tape, c->gang_warps, st);
    if (rc) return rc;
    c->batch_nshots = nshots;
    c->batch_picks = dp;
    if (nrec > 0 && picks_mem == SF_MEM_HOST) {
        CK(cudaMemcpyAsync(picks, dp, (size_t)nshots * nrec * sizeof(float), cudaMemcpyDeviceToHost, st));
        return sf_check_flags(c, st);
    }
    return SF_OK;
}

extern "C" int sf_batch_table(sf_ctx* c, int shot, float* T, int mem, void* stream)
{
    if (!c || !T) return SF_ERR_ARG;
    if (!c->tables_valid) return sf_fail(c, SF_ERR_STATE, "last batch did not keep tables");
    if (shot < 0 || shot >= (int)c->hshots.size()) return sf_fail(c, SF_ERR_ARG, "shot out of range");
    CK(cudaSetDevice(c->dev));
    const ShotDev& d = c->hshots[c->tables_index[shot]];
    cudaStream_t st = (cudaStream_t)stream;
    CK(cudaMemcpyAsync(T, c->d_T + d.t_off, sizeof(float) * (size_t)c->nzz * d.ncols,
                       mem == SF_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    if (mem == SF_MEM_HOST) return sf_check_flags(c, st);
    return SF_OK;
}

// The tape is kept per (sweep, strip) in the strip's skewed step order: entry
// [step * 32 + lane] is the node of row 32k + lane (rows downward, sweeps 0
// and 2) or 32k + 31 - lane (upward, sweeps 1 and 3) and window column of
// march step - lane (columns rightward, sweeps 0 and 1, else leftward).
// This entry point unskews one shot's codes into [sweep][column][row].
extern "C" int sf_batch_tape_codes(sf_ctx* c, int shot, uint8_t* codes, int mem, void* stream)
{
    if (!c || !codes) return SF_ERR_ARG;
    if (!c->tape_valid) return sf_fail(c, SF_ERR_STATE, "last batch did not keep a tape");
    if (shot < 0 || shot >= (int)c->hshots.size()) return sf_fail(c, SF_ERR_ARG, "shot out of range");
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    const ShotDev& d = c->hshots[c->tables_index[shot]];
    const int nzz = c->nzz, ncols = d.ncols, nstrips = (nzz + 31) / 32;
    const size_t per_strip = (size_t)(ncols + 31) * 32;
    std::vector<uint8_t> raw(4 * (size_t)nstrips * per_strip), out(4 * (size_t)ncols * nzz, 0);
    CK(cudaMemcpyAsync(raw.data(), c->d_tcode + d.tape_off, raw.size(), cudaMemcpyDeviceToHost, st));
    int rc = sf_check_flags(c, st);
    if (rc) return rc;
    for (int sw = 0; sw < 4; sw++) {
        const bool zdown = (sw == 0 || sw == 2), xright = (sw == 0 || sw == 1);
        for (int k = 0; k < nstrips; k++) {
            const uint8_t* blk = raw.data() + ((size_t)sw * nstrips + k) * per_strip;
            for (int step = 0; step < ncols + 31; step++)
                for (int lane = 0; lane < 32; lane++) {
                    const int r = zdown ? 32 * k + lane : 32 * k + 31 - lane, m = step - lane;
                    if (r >= nzz || m < 0 || m >= ncols) continue;
                    const int j = xright ? m : ncols - 1 - m;
                    out[((size_t)sw * ncols + j) * nzz + r] = blk[(size_t)step * 32 + lane];
                }
        }
    }
    CK(cudaMemcpyAsync(codes, out.data(), out.size(),
                       mem == SF_MEM_DEVICE ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost, st));
    CK(cudaStreamSynchronize(st));
    return SF_OK;
}

extern "C" int sf_time_propagation(sf_ctx* c, int ani, float sx, float sz, float* T, int T_mem, void* stream)
{
    if (!c || !T) return sf_fail(c, SF_ERR_ARG, "null argument");
    if (ani && !c->have_cij) return sf_fail(c, SF_ERR_STATE, "anisotropic solve needs sf_set_stiffness");
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    sf_shot s{sx, sz, 0, c->nxx};
    int rc = sf_prepare_shots(c, &s, 1, false);
    if (rc) return rc;
    const size_t npad = (size_t)c->nxx * c->nzz;
    // the whole-grid table is written straight into the caller's device buffer
    float* keepT = c->d_T;
    size_t keepcap = c->cap_T;
    if (T_mem == SF_MEM_DEVICE) {
        c->d_T = T;
        c->cap_T = npad * sizeof(float);
    }
    rc = sf_launch_shots(c, ani, 0, nullptr, true, false, c->gang_warps, st);
    if (T_mem == SF_MEM_DEVICE) {
        c->d_T = keepT;
        c->cap_T = keepcap;
        c->tables_valid = false;
    }
    if (rc) return rc;
    if (T_mem == SF_MEM_HOST) {
        CK(cudaMemcpyAsync(T, c->d_T, npad * sizeof(float), cudaMemcpyDeviceToHost, st));
        return sf_check_flags(c, st);
    }
    return SF_OK;
}

extern "C" int sf_compute_seismogram(sf_ctx* c, const float* T_dev, const float* rx, const float* rz,
                                     int nrec, float* picks, int picks_mem, void* stream)
{
    if (!c || !T_dev || nrec < 0 || (nrec > 0 && (!rx || !rz || !picks))) return SF_ERR_ARG;
    if (nrec == 0) return SF_OK;
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    int rc = sf_upload_receivers(c, rx, rz, nrec, st);
    if (rc) return rc;
    float* dp = picks;
    if (picks_mem == SF_MEM_HOST) {
        rc = sf_dev_reserve(c, (void**)&c->d_picks, &c->cap_picks, (size_t)nrec * sizeof(float));
        if (rc) return rc;
        dp = c->d_picks;
    }
    k_picks<<<(nrec + 127) / 128, 128, 0, st>>>(T_dev, c->nzz, c->nxx, 0, c->nb, c->dx, c->dz, c->d_rx,
                                                c->d_rz, nrec, dp);
    CK(cudaGetLastError());
    if (picks_mem == SF_MEM_HOST) {
        CK(cudaMemcpyAsync(picks, dp, (size_t)nrec * sizeof(float), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    return SF_OK;
}

// The allocation-free per-shot entry point shares this translation unit's
// instantiation of k_shots.
#include "sf_noalloc.cu"
