// Kirchhoff depth migration in the image domain (the reference's IDKDM,
// src/migration/KDM.cu:3-55 + IDKDM.cu:19-22) on traveltime tables kept on the
// device, and the wavelet cross-correlation of its input traces
// (Migration::set_wavelet + adjoint_convolution, migration.cu:54-71,
// :173-228).
//
// The reference launches image_domain_adjoint_kernel (migration.cu:398-483)
// once per source-receiver trace over the whole grid and adds each trace's
// term with atomicAdd; a cell is touched by one thread per launch, so the
// image is the FP32 sum of the traces' terms in trace order (source outer,
// receiver inner). Here one thread owns an image cell and walks every trace
// in that order: the same sum, one launch, no atomics, and the source-table
// derivatives computed once per source instead of once per trace.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "sf_engine.h"

using namespace sf;

#define CK(call)                                                          \
    do {                                                                  \
        int _st = sf_cuda_check(c, (call), #call);                        \
        if (_st != SF_OK) return _st;                                     \
    } while (0)

namespace {

constexpr float kEps = 1e-6f;  // EPS of migration.cuh:7

// The reference adds each term with a global float atomicAdd, which flushes
// subnormal operands and results to zero; the gather adds the same way.
__device__ __forceinline__ float add_ftz(float a, float b)
{
    float r;
    asm("add.rn.ftz.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}

struct KirchParams {
    const float* S;     // padded slowness
    const float* Ts;    // nsrc padded tables
    const float* Tr;    // nrec padded tables
    const float* xs;    // nsrc
    const float* xr;    // nrec
    const float* data;  // nsrc x nrec x nt correlated traces
    float* image;       // nz x nx
    int nsrc, nrec, nt, nxx, nzz, nb;
    float dt, dx, dz, aperture, max_offset;
};

// The geometric terms of one table at padded node (i, j): centred first and
// second differences, gradient norm, unit direction (migration.cu:418-450).
struct TableTerms {
    float dx1, dz1, norm, detH;
};

__device__ __forceinline__ TableTerms table_terms(const float* T, int i, int j, int nzz, float dx, float dz)
{
    TableTerms t;
    const float c = T[i + j * nzz];
    const float zp = T[(i + 1) + j * nzz], zm = T[(i - 1) + j * nzz];
    const float xp = T[i + (j + 1) * nzz], xm = T[i + (j - 1) * nzz];
    float d_dz = 0.5f * (zp - zm) / dz;
    float d_dx = 0.5f * (xp - xm) / dx;
    float d2_dz2 = (zp - 2.0f * c + zm) / (dz * dz);
    float d2_dx2 = (xp - 2.0f * c + xm) / (dx * dx);
    float d2_dxdz = (T[(i + 1) + (j + 1) * nzz] - T[(i - 1) + (j + 1) * nzz] -
                     T[(i + 1) + (j - 1) * nzz] + T[(i - 1) + (j - 1) * nzz]) / (4.0f * dx * dz);
    t.dz1 = d_dz;
    t.dx1 = d_dx;
    t.norm = sqrtf(d_dx * d_dx + d_dz * d_dz) + kEps;
    float a = d2_dx2, b = d2_dxdz, cc = d2_dz2;
    float det = a * cc - b * b;
    t.detH = fabsf(det) + kEps;
    return t;
}

__global__ void k_kirchhoff_image(KirchParams p)
{
    const int nz = p.nzz - 2 * p.nb, nx = p.nxx - 2 * p.nb;
    const size_t ncell = (size_t)nz * nx;
    for (size_t m = blockIdx.x * (size_t)blockDim.x + threadIdx.x; m < ncell; m += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(m % nz) + p.nb, j = (int)(m / nz) + p.nb;
        const size_t index = (size_t)i + (size_t)j * p.nzz;
        const size_t matsize = (size_t)p.nzz * p.nxx;
        const float z = __int2float_rd(i - p.nb) * p.dz;
        const float x = __int2float_rd(j - p.nb) * p.dx;
        const float Sc = p.S[index];
        const float scale_const = 1.0f / (2.0f * M_PI);
        const float sigma = tanf(p.aperture * M_PI / 180.0f) * z;
        float acc = 0.0f;
        for (int s = 0; s < p.nsrc; s++) {
            const float* Ts = p.Ts + matsize * s;
            const TableTerms ts = table_terms(Ts, i, j, p.nzz, p.dx, p.dz);
            const float Tsc = Ts[index];
            const float ux_s = ts.dx1 / ts.norm, uz_s = ts.dz1 / ts.norm;
            const float nx_norm = 0.0f, nz_norm = -1.0f;
            const float cos_s = fabs(ux_s * nx_norm + uz_s * nz_norm);
            const float R_s = max(Tsc / Sc, kEps);
            const float theta_s = acosf(min(1.0f, max(-1.0f, ux_s * nx_norm + uz_s * nz_norm)));
            const float xs = p.xs[s];
            for (int r = 0; r < p.nrec; r++) {
                const float offset = fabsf((xs - p.xr[r]));
                if (!(offset < p.max_offset)) continue;
                const float cmp = 0.5f * (xs + p.xr[r]);
                const float* Tr = p.Tr + matsize * r;
                const float T = Tsc + Tr[index];
                const int tId = __float2int_rd(T / p.dt);
                if (tId >= p.nt) continue;
                const TableTerms tr = table_terms(Tr, i, j, p.nzz, p.dx, p.dz);
                const float Jterm = sqrtf(ts.detH * tr.detH) * Sc / (ts.norm * tr.norm);
                const float ux_r = tr.dx1 / tr.norm, uz_r = tr.dz1 / tr.norm;
                const float cos_r = fabs(ux_r * nx_norm + uz_r * nz_norm);
                const float obliquity = sqrt(max(0.0f, cos_s) * max(0.0f, cos_r));
                const float R_r = max(Tr[index] / Sc, kEps);
                const float G = 1.0f / sqrt(R_s * R_r);
                const float theta_r = acosf(min(1.0f, max(-1.0f, ux_r * nx_norm + uz_r * nz_norm)));
                const float theta = 0.5f * (theta_s + theta_r);
                const float R = 1.0f + 0.2f * cosf(theta);
                const float taper = expf(-0.5f * ((x - cmp) / (sigma + kEps)) * ((x - cmp) / (sigma + kEps)));
                const float weights = scale_const * Jterm * obliquity * G * R * taper;
                acc = add_ftz(acc, __fmul_rn(weights, p.data[((size_t)s * p.nrec + r) * p.nt + tId]));
            }
        }
        p.image[m] = acc;
    }
}

// Cross-correlation of each trace with the wavelet as the reference's FFT
// product A conj(B) with FFTW's unnormalised inverse gives it: for output
// sample t >= shift, nfft * sum_m trace[t - shift + m] * w[m] in FP64 (the
// zero padding to nfft >= nt + nw - 1 makes the circular sum a linear one),
// rounded once to FP32 (each FP64 operation rounded once, in the order of
// the sum); samples before the shift are 0.
__global__ void k_correlate(const float* __restrict__ in, float* __restrict__ out, int ntr, int nt,
                            const double* __restrict__ w, int nw, int shift, double nfft)
{
    const size_t n = (size_t)ntr * nt;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const int t = (int)(q % nt);
        const float* a = in + (q - t);
        float v = 0.0f;
        if (t >= shift) {
            const int l = t - shift;
            double acc = 0.0;
            for (int m = 0; m < nw && l + m < nt; m++) acc = __dadd_rn(acc, __dmul_rn((double)a[l + m], w[m]));
            v = __double2float_rn(__dmul_rn(acc, nfft));
        }
        out[q] = v;
    }
}

constexpr int kMaxAngles = 256;

struct AngleParams {
    const float* S;
    const float* Ts;
    const float* Tr;
    const float* xs;
    const float* xr;
    const float* data;      // nsrc x nrec x nt correlated traces
    const int* cmp_ptr;     // traces of CMP bin b: [cmp_ptr[b], cmp_ptr[b+1]) of cmp_tr
    const int* cmp_tr;      // trace s * nrec + r, trace order within a bin
    float* gathers;         // nz x nang x ncmp
    int nsrc, nrec, nt, nxx, nzz, nb, nang, ncmp;
    float dt, dx, dz, da, aperture;
};

// ADKDM's angle_domain_adjoint_kernel (migration.cu:572-663) as a gather: one
// thread per (depth row, CMP bin) walks the bin's traces in trace order and,
// for each, the row's cells left to right, adding each term to its
// reflection-angle bin. The reference adds with atomics from all columns of a
// launch at once, so its order within a bin is not fixed; the terms are the
// same.
__global__ void k_kirchhoff_angles(AngleParams p)
{
    const int nz = p.nzz - 2 * p.nb;
    const size_t nthr = (size_t)nz * p.ncmp;
    float acc[kMaxAngles];
    for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < nthr; w += (size_t)gridDim.x * blockDim.x) {
        const int iz = (int)(w % nz), b = (int)(w / nz);
        const int i = iz + p.nb;
        for (int a = 0; a < p.nang; a++) acc[a] = 0.0f;
        const size_t matsize = (size_t)p.nzz * p.nxx;
        const float z = __int2float_rd(i - p.nb) * p.dz;
        const float scale_const = 1.0f / (2.0f * M_PI);
        const float sigma = tanf(p.aperture * M_PI / 180.0f) * z;
        for (int e = p.cmp_ptr[b]; e < p.cmp_ptr[b + 1]; e++) {
            const int tr_id = p.cmp_tr[e];
            const int s = tr_id / p.nrec, r = tr_id % p.nrec;
            const float cmp = 0.5f * (p.xs[s] + p.xr[r]);
            const float* Ts = p.Ts + matsize * s;
            const float* Tr = p.Tr + matsize * r;
            const float* trace = p.data + (size_t)tr_id * p.nt;
            for (int j = p.nb; j < p.nxx - p.nb; j++) {
                const size_t index = (size_t)i + (size_t)j * p.nzz;
                const float x = __int2float_rd(j - p.nb) * p.dx;
                const float T = Ts[index] + Tr[index];
                const int tId = __float2int_rd(T / p.dt);
                if (tId >= p.nt) continue;
                const TableTerms ts = table_terms(Ts, i, j, p.nzz, p.dx, p.dz);
                const TableTerms tr = table_terms(Tr, i, j, p.nzz, p.dx, p.dz);
                const float Sc = p.S[index];
                const float Jterm = sqrtf(ts.detH * tr.detH) * Sc / (ts.norm * tr.norm);
                const float ux_s = ts.dx1 / ts.norm, uz_s = ts.dz1 / ts.norm;
                const float ux_r = tr.dx1 / tr.norm, uz_r = tr.dz1 / tr.norm;
                const float nx_norm = 0.0f, nz_norm = -1.0f;
                const float cos_s = fabs(ux_s * nx_norm + uz_s * nz_norm);
                const float cos_r = fabs(ux_r * nx_norm + uz_r * nz_norm);
                const float obliquity = sqrt(max(0.0f, cos_s) * max(0.0f, cos_r));
                const float R_s = max(Ts[index] / Sc, kEps);
                const float R_r = max(Tr[index] / Sc, kEps);
                const float G = 1.0f / sqrt(R_s * R_r);
                const float theta_s = acosf(min(1.0f, max(-1.0f, ux_s * nx_norm + uz_s * nz_norm)));
                const float theta_r = acosf(min(1.0f, max(-1.0f, ux_r * nx_norm + uz_r * nz_norm)));
                const float theta = 0.5f * (theta_s + theta_r);
                const float R = 1.0f + 0.2f * cosf(theta);
                const float taper = expf(-0.5f * ((x - cmp) / (sigma + kEps)) * ((x - cmp) / (sigma + kEps)));
                const float weights = scale_const * Jterm * obliquity * G * R * taper;
                const float reflection_angle = 0.5f * acos((ts.dx1 * tr.dx1 + ts.dz1 * tr.dz1) / (ts.norm * tr.norm));
                const float ang = 180.0f * reflection_angle / M_PI;
                const int aId = __float2int_rd(ang / p.da);
                if (aId >= 0 && aId < p.nang) acc[aId] = add_ftz(acc[aId], __fmul_rn(weights, trace[tId]));
            }
        }
        for (int a = 0; a < p.nang; a++) p.gathers[(size_t)iz + (size_t)a * nz + (size_t)b * p.nang * nz] = acc[a];
    }
}

// The trace-independent part of one cell's weight, as the reference's four
// Kirchhoff kernels compute it (migration.cu:418-466, :505-553, :592-640,
// :685-733), from both tables' terms at the cell; sigma = tan(aperture) z.
__device__ __forceinline__ float kirchhoff_weight(const TableTerms& ts, const TableTerms& tr, float Tsc, float Trc,
                                                  float Sc, float x, float cmp, float sigma)
{
    const float Jterm = sqrtf(ts.detH * tr.detH) * Sc / (ts.norm * tr.norm);
    const float ux_s = ts.dx1 / ts.norm, uz_s = ts.dz1 / ts.norm;
    const float ux_r = tr.dx1 / tr.norm, uz_r = tr.dz1 / tr.norm;
    const float nx_norm = 0.0f, nz_norm = -1.0f;
    const float cos_s = fabs(ux_s * nx_norm + uz_s * nz_norm);
    const float cos_r = fabs(ux_r * nx_norm + uz_r * nz_norm);
    const float obliquity = sqrt(max(0.0f, cos_s) * max(0.0f, cos_r));
    const float R_s = max(Tsc / Sc, kEps);
    const float R_r = max(Trc / Sc, kEps);
    const float G = 1.0f / sqrt(R_s * R_r);
    const float theta_s = acosf(min(1.0f, max(-1.0f, ux_s * nx_norm + uz_s * nz_norm)));
    const float theta_r = acosf(min(1.0f, max(-1.0f, ux_r * nx_norm + uz_r * nz_norm)));
    const float theta = 0.5f * (theta_s + theta_r);
    const float R = 1.0f + 0.2f * cosf(theta);
    const float scale_const = 1.0f / (2.0f * M_PI);
    const float taper = expf(-0.5f * ((x - cmp) / (sigma + kEps)) * ((x - cmp) / (sigma + kEps)));
    return scale_const * Jterm * obliquity * G * R * taper;
}

struct KirchFwdParams {
    const float* S;
    const float* Ts;
    const float* Tr;
    const float* xs;
    const float* xr;
    const float* model;  // image (nz x nx) or angle gathers (nz x nang x ncmp)
    const int* trace;    // work trace e -> s * nrec + r, in trace order
    const int* cmp;      // work trace e -> CMP bin (angle domain)
    float* part;         // ntrace x nchunk x nt partial traces (nchunk > 1)
    float* data;         // nsrc x nrec x nt
    int nchunk, chunk, nrec, nt, nxx, nzz, nb, nang, warps;
    float dt, dx, dz, da, aperture;
};

// The forward (demigration) operator of the least-squares variants:
// image_domain_forward_kernel / angle_domain_forward_kernel
// (migration.cu:485-570, :665-756) add weight * model[cell] to sample
// floor((Ts + Tr)/dt) of the trace with a global atomicAdd per cell, in no
// fixed order. Here one CTA takes one chunk of one trace's cells. Each warp
// walks 32 consecutive cells (z fastest) at a time; lanes that hit the same
// sample are summed in lane order and the sum is added to the warp's own
// histogram of the trace in shared memory (one adder per sample, no
// atomics). The warps' histograms are summed in warp order, the chunks in
// chunk order: a fixed order that depends only on the sizes, so the traces
// are reproducible bit for bit.
template <bool ANGLE>
__global__ void k_kirchhoff_forward(KirchFwdParams p)
{
    extern __shared__ float smem[];
    const int W = p.warps, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* hist = smem + (size_t)warp * p.nt;
    int* st_t = reinterpret_cast<int*>(smem + (size_t)W * p.nt) + warp * 32;
    float* st_v = smem + (size_t)W * p.nt + W * 32 + warp * 32;
    for (int q = threadIdx.x; q < W * p.nt; q += blockDim.x) smem[q] = 0.0f;
    __syncthreads();
    const int e = blockIdx.x / p.nchunk, ck = blockIdx.x % p.nchunk;
    const int tid = p.trace[e], s = tid / p.nrec, r = tid % p.nrec;
    const float cmp = 0.5f * (p.xs[s] + p.xr[r]);
    const int cmpId = ANGLE ? p.cmp[e] : 0;
    const size_t matsize = (size_t)p.nzz * p.nxx;
    const float* Ts = p.Ts + matsize * s;
    const float* Tr = p.Tr + matsize * r;
    const int nz = p.nzz - 2 * p.nb;
    const long ncell = (long)nz * (p.nxx - 2 * p.nb);
    const long m0 = (long)ck * p.chunk, m1 = min(m0 + (long)p.chunk, ncell);
    for (long g = m0 + 32L * warp; g < m1; g += 32L * W) {
        const long m = g + lane;
        int tq = -1;
        float v = 0.0f;
        if (m < m1) {
            const int i = (int)(m % nz) + p.nb, j = (int)(m / nz) + p.nb;
            const size_t index = (size_t)i + (size_t)j * p.nzz;
            const float T = Ts[index] + Tr[index];
            const int tId = __float2int_rd(T / p.dt);
            if (tId >= 0 && tId < p.nt) {
                const float z = __int2float_rd(i - p.nb) * p.dz;
                const float x = __int2float_rd(j - p.nb) * p.dx;
                const float sigma = tanf(p.aperture * M_PI / 180.0f) * z;
                const TableTerms ts = table_terms(Ts, i, j, p.nzz, p.dx, p.dz);
                const TableTerms tr = table_terms(Tr, i, j, p.nzz, p.dx, p.dz);
                const float weights = kirchhoff_weight(ts, tr, Ts[index], Tr[index], p.S[index], x, cmp, sigma);
                if (ANGLE) {
                    const float reflection_angle =
                        0.5f * acos((ts.dx1 * tr.dx1 + ts.dz1 * tr.dz1) / (ts.norm * tr.norm));
                    const float ang = 180.0f * reflection_angle / M_PI;
                    const int aId = __float2int_rd(ang / p.da);
                    if (aId >= 0 && aId < p.nang) {
                        const size_t mId = (size_t)(i - p.nb) + (size_t)aId * nz + (size_t)cmpId * p.nang * nz;
                        v = __fmul_rn(weights, p.model[mId]);
                        tq = tId;
                    }
                } else {
                    v = __fmul_rn(weights, p.model[m]);
                    tq = tId;
                }
            }
        }
        st_t[lane] = tq;
        st_v[lane] = v;
        __syncwarp();
        const unsigned grp = __match_any_sync(0xffffffffu, tq);
        if (tq >= 0 && lane == __ffs(grp) - 1) {
            float sum = v;
            for (unsigned rest = grp & (grp - 1); rest; rest &= rest - 1) sum = add_ftz(sum, st_v[__ffs(rest) - 1]);
            hist[tq] = add_ftz(hist[tq], sum);
        }
        __syncwarp();
    }
    __syncthreads();
    float* out = (p.nchunk == 1) ? p.data + (size_t)tid * p.nt : p.part + ((size_t)e * p.nchunk + ck) * p.nt;
    for (int t = threadIdx.x; t < p.nt; t += blockDim.x) {
        float a = smem[t];
        for (int w = 1; w < W; w++) a = add_ftz(a, smem[(size_t)w * p.nt + t]);
        out[t] = a;
    }
}

// Chunk partials of each work trace summed in chunk order.
__global__ void k_sum_chunks(const float* __restrict__ part, const int* __restrict__ trace, float* __restrict__ data,
                             int ntrace, int nchunk, int nt)
{
    const size_t n = (size_t)ntrace * nt;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const int e = (int)(q / nt), t = (int)(q % nt);
        const float* pp = part + (size_t)e * nchunk * nt + t;
        float a = pp[0];
        for (int c = 1; c < nchunk; c++) a = add_ftz(a, pp[(size_t)c * nt]);
        data[(size_t)trace[e] * nt + t] = a;
    }
}

// Convolution of each trace with the wavelet as the reference's FFT product
// A B with FFTW's unnormalised inverse gives it (Migration::
// forward_convolution, migration.cu:230-261): for output sample t,
// nfft * sum_m trace[t + shift - m] * w[m] over the samples inside the trace,
// in FP64 (m ascending), rounded once to FP32.
__global__ void k_convolve(const float* __restrict__ in, float* __restrict__ out, int ntr, int nt,
                           const double* __restrict__ w, int nw, int shift, double nfft)
{
    const size_t n = (size_t)ntr * nt;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const int t = (int)(q % nt);
        const float* a = in + (q - t);
        const int c = t + shift;
        double acc = 0.0;
        for (int m = max(0, c - nt + 1); m < nw && m <= c; m++) acc = __dadd_rn(acc, __dmul_rn((double)a[c - m], w[m]));
        out[q] = __double2float_rn(__dmul_rn(acc, nfft));
    }
}

}  // namespace

// Migration::set_wavelet (migration.cu:54-71) as its source computes it.
void sf_kirchhoff_wavelet(float fmax, float dt, std::vector<float>& w)
{
    const float t0 = 2.0f * sqrtf(M_PI) / fmax;
    const float fc = fmax / (3.0f * sqrtf(M_PI));
    const int nw = 2 * ((int)((t0 - 0.5f * dt) / dt));
    w.assign(std::max(nw, 0), 0.0f);
    for (int k = 0; k < nw; k++) {
        const float td = k * dt - t0;
        const float arg = M_PI * M_PI * M_PI * fc * fc * td * td;
        w[k] = (1.0f - 2.0f * arg) * expf(-arg);
    }
}

static int next_pow2(int n)
{
    int p = 1;
    while (p < n) p <<= 1;
    return p;
}

// The wavelet correlation (forward = false) or convolution (forward = true)
// of ntr traces, as Migration::adjoint_convolution / forward_convolution.
static int wavelet_filter(sf_ctx* c, const float* traces, float* out, int ntr, int nt, float dt, float fmax, int mem,
                          void* stream, bool forward)
{
    if (!c || !traces || !out || ntr < 0 || nt < 1 || !(dt > 0.0f) || !(fmax > 0.0f))
        return sf_fail(c, SF_ERR_ARG, "bad convolution arguments");
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<float> wf;
    sf_kirchhoff_wavelet(fmax, dt, wf);
    const int nw = (int)wf.size();
    if (nw < 1) return sf_fail(c, SF_ERR_ARG, "wavelet shorter than one sample (fmax too high for dt)");
    c->h_wav.assign(wf.begin(), wf.end());  // FP64 copy of the FP32 samples
    const size_t nb = (size_t)ntr * nt * sizeof(float);
    int rc = sf_dev_reserve(c, (void**)&c->d_wav, &c->cap_wav, c->h_wav.size() * sizeof(double));
    if (!rc && mem == SF_MEM_HOST) rc = sf_dev_reserve(c, (void**)&c->d_mig, &c->cap_mig, 2 * nb + 16);
    if (rc) return rc;
    CK(cudaMemcpyAsync(c->d_wav, c->h_wav.data(), c->h_wav.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    const float* din = traces;
    float* dout = out;
    if (mem == SF_MEM_HOST) {
        CK(cudaMemcpyAsync(c->d_mig, traces, nb, cudaMemcpyHostToDevice, st));
        din = c->d_mig;
        dout = c->d_mig + (size_t)ntr * nt;
    }
    const size_t n = (size_t)ntr * nt;
    if (n) {
        const unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)c->sms * 16);
        const double nfft = (double)next_pow2(nt + nw - 1);
        if (forward)
            k_convolve<<<grid, 256, 0, st>>>(din, dout, ntr, nt, c->d_wav, nw, nw / 2 + nw / 10, nfft);
        else
            k_correlate<<<grid, 256, 0, st>>>(din, dout, ntr, nt, c->d_wav, nw, nw / 2 + nw / 10, nfft);
        CK(cudaGetLastError());
    }
    if (mem == SF_MEM_HOST) {
        CK(cudaMemcpyAsync(out, dout, nb, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    return SF_OK;
}

extern "C" int sf_adjoint_convolution(sf_ctx* c, const float* traces, float* out, int ntr, int nt, float dt,
                                      float fmax, int mem, void* stream)
{
    return wavelet_filter(c, traces, out, ntr, nt, dt, fmax, mem, stream, false);
}

extern "C" int sf_forward_convolution(sf_ctx* c, const float* traces, float* out, int ntr, int nt, float dt,
                                      float fmax, int mem, void* stream)
{
    return wavelet_filter(c, traces, out, ntr, nt, dt, fmax, mem, stream, true);
}

extern "C" int sf_kirchhoff_image(sf_ctx* c, const float* Ts, const float* Tr, int nsrc, int nrec, const float* xsrc,
                                  const float* xrec, const float* data, int data_mem, int nt, float dt,
                                  float aperture, float max_offset, float* image, int image_mem, void* stream)
{
    if (!c || !Ts || !Tr || !xsrc || !xrec || !data || !image || nsrc < 1 || nrec < 1 || nt < 1 || !(dt > 0.0f))
        return sf_fail(c, SF_ERR_ARG, "bad Kirchhoff arguments");
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t nd = (size_t)nsrc * nrec * nt, ni = (size_t)c->nx * c->nz;
    int rc = sf_dev_reserve(c, (void**)&c->d_kgeo, &c->cap_kgeo, (size_t)(nsrc + nrec) * sizeof(float));
    if (!rc && (data_mem == SF_MEM_HOST || image_mem == SF_MEM_HOST))
        rc = sf_dev_reserve(c, (void**)&c->d_mig, &c->cap_mig, (nd + ni) * sizeof(float));
    if (rc) return rc;
    c->h_kgeo.assign(xsrc, xsrc + nsrc);
    c->h_kgeo.insert(c->h_kgeo.end(), xrec, xrec + nrec);
    CK(cudaMemcpyAsync(c->d_kgeo, c->h_kgeo.data(), c->h_kgeo.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    const float* dd = data;
    float* di = image;
    if (data_mem == SF_MEM_HOST) {
        CK(cudaMemcpyAsync(c->d_mig, data, nd * sizeof(float), cudaMemcpyHostToDevice, st));
        dd = c->d_mig;
    }
    if (image_mem == SF_MEM_HOST) di = c->d_mig + nd;
    KirchParams p;
    p.S = c->d_S;
    p.Ts = Ts;
    p.Tr = Tr;
    p.xs = c->d_kgeo;
    p.xr = c->d_kgeo + nsrc;
    p.data = dd;
    p.image = di;
    p.nsrc = nsrc;
    p.nrec = nrec;
    p.nt = nt;
    p.nxx = c->nxx;
    p.nzz = c->nzz;
    p.nb = c->nb;
    p.dt = dt;
    p.dx = c->dx;
    p.dz = c->dz;
    p.aperture = aperture;
    p.max_offset = max_offset;
    k_kirchhoff_image<<<(unsigned)std::min<size_t>((ni + 127) / 128, (size_t)c->sms * 32), 128, 0, st>>>(p);
    CK(cudaGetLastError());
    if (image_mem == SF_MEM_HOST) {
        CK(cudaMemcpyAsync(image, di, ni * sizeof(float), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    return SF_OK;
}

// Migration::set_gathers (migration.cu:73-97): CMP spacing half the smaller of
// the first source and receiver spacings, bins from the smallest CMP of all
// pairs. The reference starts the largest CMP from an uninitialised value
// (it assigns minCMP twice); here it starts from the first pair's CMP.
static int angle_dims(const float* xsrc, int nsrc, const float* xrec, int nrec, float max_angle, float da,
                      int* nang, int* ncmp, float* mincmp, float* dcmp)
{
    if (nsrc < 2 || nrec < 2 || !(da > 0.0f)) return SF_ERR_ARG;
    const float ds = xsrc[1] - xsrc[0], dr = xrec[1] - xrec[0];
    const float d = 0.5f * std::min(ds, dr);
    if (!(d > 0.0f)) return SF_ERR_ARG;
    float mn = 1e6f, mx = 0.5f * (xsrc[0] + xrec[0]);
    for (int s = 0; s < nsrc; s++)
        for (int r = 0; r < nrec; r++) {
            const float cmp = 0.5f * (xsrc[s] + xrec[r]);
            mn = (cmp < mn) ? cmp : mn;
            mx = (cmp > mx) ? cmp : mx;
        }
    *nang = (int)(max_angle / da) + 1;
    *ncmp = (int)((mx - mn) / d) + 1;
    *mincmp = mn;
    *dcmp = d;
    return SF_OK;
}

extern "C" int sf_kirchhoff_angle_gathers(sf_ctx* c, const float* Ts, const float* Tr, int nsrc, int nrec,
                                          const float* xsrc, const float* xrec, const float* data, int data_mem, int nt,
                                          float dt, float aperture, float max_offset, float max_angle, float da,
                                          float* gathers, int gathers_mem, int* nang_out, int* ncmp_out, void* stream)
{
    if (!c || !xsrc || !xrec) return sf_fail(c, SF_ERR_ARG, "null argument");
    int nang, ncmp;
    float mincmp, dcmp;
    if (angle_dims(xsrc, nsrc, xrec, nrec, max_angle, da, &nang, &ncmp, &mincmp, &dcmp))
        return sf_fail(c, SF_ERR_ARG, "angle gathers need two sources, two receivers, increasing positions, da > 0");
    if (nang > kMaxAngles) return sf_fail(c, SF_ERR_RANGE, "more than 256 angle bins");
    if (nang_out) *nang_out = nang;
    if (ncmp_out) *ncmp_out = ncmp;
    if (!gathers) return SF_OK;  // dimensions only
    if (!Ts || !Tr || !data || nt < 1 || !(dt > 0.0f)) return sf_fail(c, SF_ERR_ARG, "bad Kirchhoff arguments");
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    // traces by CMP bin, trace order kept (KDM.cu:28-53)
    std::vector<int> cnt(ncmp + 1, 0), ids;
    std::vector<std::pair<int, int>> tr;
    for (int s = 0; s < nsrc; s++)
        for (int r = 0; r < nrec; r++) {
            if (!(fabsf(xsrc[s] - xrec[r]) < max_offset)) continue;
            const float cmp = 0.5f * (xsrc[s] + xrec[r]);
            const int b = (int)((cmp - mincmp) / dcmp);
            if (b < 0 || b >= ncmp) continue;
            tr.push_back({b, s * nrec + r});
            cnt[b + 1]++;
        }
    for (int b = 0; b < ncmp; b++) cnt[b + 1] += cnt[b];
    ids.resize(tr.size());
    {
        std::vector<int> fill(cnt.begin(), cnt.end() - 1);
        for (auto& t : tr) ids[fill[t.first]++] = t.second;
    }
    const size_t nd = (size_t)nsrc * nrec * nt, ng = (size_t)(c->nzz - 2 * c->nb) * nang * ncmp;
    c->h_kgeo.assign(xsrc, xsrc + nsrc);
    c->h_kgeo.insert(c->h_kgeo.end(), xrec, xrec + nrec);
    c->h_kint.assign(cnt.begin(), cnt.end());
    c->h_kint.insert(c->h_kint.end(), ids.begin(), ids.end());
    int rc = sf_dev_reserve(c, (void**)&c->d_kgeo, &c->cap_kgeo, c->h_kgeo.size() * sizeof(float));
    if (!rc) rc = sf_dev_reserve(c, (void**)&c->d_kint, &c->cap_kint, c->h_kint.size() * sizeof(int));
    if (!rc && (data_mem == SF_MEM_HOST || gathers_mem == SF_MEM_HOST))
        rc = sf_dev_reserve(c, (void**)&c->d_mig, &c->cap_mig, (nd + ng) * sizeof(float));
    if (rc) return rc;
    CK(cudaMemcpyAsync(c->d_kgeo, c->h_kgeo.data(), c->h_kgeo.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->d_kint, c->h_kint.data(), c->h_kint.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    const float* dd = data;
    float* dg = gathers;
    if (data_mem == SF_MEM_HOST) {
        CK(cudaMemcpyAsync(c->d_mig, data, nd * sizeof(float), cudaMemcpyHostToDevice, st));
        dd = c->d_mig;
    }
    if (gathers_mem == SF_MEM_HOST) dg = c->d_mig + nd;
    AngleParams p;
    p.S = c->d_S;
    p.Ts = Ts;
    p.Tr = Tr;
    p.xs = c->d_kgeo;
    p.xr = c->d_kgeo + nsrc;
    p.data = dd;
    p.cmp_ptr = c->d_kint;
    p.cmp_tr = c->d_kint + ncmp + 1;
    p.gathers = dg;
    p.nsrc = nsrc;
    p.nrec = nrec;
    p.nt = nt;
    p.nxx = c->nxx;
    p.nzz = c->nzz;
    p.nb = c->nb;
    p.nang = nang;
    p.ncmp = ncmp;
    p.dt = dt;
    p.dx = c->dx;
    p.dz = c->dz;
    p.da = da;
    p.aperture = aperture;
    const size_t nthr = (size_t)(c->nzz - 2 * c->nb) * ncmp;
    k_kirchhoff_angles<<<(unsigned)std::min<size_t>((nthr + 127) / 128, (size_t)c->sms * 64), 128, 0, st>>>(p);
    CK(cudaGetLastError());
    if (gathers_mem == SF_MEM_HOST) {
        CK(cudaMemcpyAsync(gathers, dg, ng * sizeof(float), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    return SF_OK;
}

// Shared memory of one forward CTA: per warp a histogram of nt samples and 32
// staged (sample, term) pairs.
constexpr size_t kFwdSmem = 200 * 1024;
// Work traces times chunks the forward aims at when traces are few; a fixed
// number, so the summation order depends on the sizes only.
constexpr long kFwdCtas = 2432;

// The forward operator over the pairs LSKDM::compute_gradient and
// compute_stepLength visit (LSKDM.cu:52-90, :168-201): every source, every
// receiver with |xsrc - xrec| < max_offset, in that order; the other traces
// of data are zero.
static int kirchhoff_forward(sf_ctx* c, bool angle, const float* Ts, const float* Tr, int nsrc, int nrec,
                             const float* xsrc, const float* xrec, const float* model, int model_mem, size_t nmodel,
                             int nt, float dt, float aperture, float max_offset, int nang, int ncmp, float mincmp,
                             float dcmp, float da, float* data, int data_mem, void* stream)
{
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<int> ids, bins;
    for (int s = 0; s < nsrc; s++)
        for (int r = 0; r < nrec; r++) {
            if (!(fabsf(xsrc[s] - xrec[r]) < max_offset)) continue;
            if (angle) {
                const float cmp = 0.5f * (xsrc[s] + xrec[r]);
                const int b = (int)((cmp - mincmp) / dcmp);
                if (b < 0 || b >= ncmp) continue;
                bins.push_back(b);
            }
            ids.push_back(s * nrec + r);
        }
    const int ntrace = (int)ids.size();
    const size_t per_warp = (size_t)nt * sizeof(float) + 64 * sizeof(float);
    const int W = (int)std::min<size_t>(8, kFwdSmem / per_warp);
    if (W < 1) return sf_fail(c, SF_ERR_RANGE, "too many time samples for the forward operator");
    const int nz = c->nzz - 2 * c->nb;
    const long ncell = (long)nz * (c->nxx - 2 * c->nb);
    const int nchunk = (int)std::max<long>(
        1, std::min<long>((kFwdCtas + std::max(ntrace, 1) - 1) / std::max(ntrace, 1), (ncell + 4095) / 4096));
    const int chunk = (int)((ncell + nchunk - 1) / nchunk);
    const size_t nd = (size_t)nsrc * nrec * nt;
    c->h_kgeo.assign(xsrc, xsrc + nsrc);
    c->h_kgeo.insert(c->h_kgeo.end(), xrec, xrec + nrec);
    c->h_kint.assign(ids.begin(), ids.end());
    c->h_kint.insert(c->h_kint.end(), bins.begin(), bins.end());
    int rc = sf_dev_reserve(c, (void**)&c->d_kgeo, &c->cap_kgeo, c->h_kgeo.size() * sizeof(float));
    if (!rc) rc = sf_dev_reserve(c, (void**)&c->d_kint, &c->cap_kint, std::max<size_t>(1, c->h_kint.size()) * sizeof(int));
    if (!rc && (model_mem == SF_MEM_HOST || data_mem == SF_MEM_HOST))
        rc = sf_dev_reserve(c, (void**)&c->d_mig, &c->cap_mig, (nd + nmodel) * sizeof(float));
    if (!rc && nchunk > 1)
        rc = sf_dev_reserve(c, (void**)&c->d_kpart, &c->cap_kpart, (size_t)ntrace * nchunk * nt * sizeof(float));
    if (rc) return rc;
    CK(cudaMemcpyAsync(c->d_kgeo, c->h_kgeo.data(), c->h_kgeo.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    if (!c->h_kint.empty())
        CK(cudaMemcpyAsync(c->d_kint, c->h_kint.data(), c->h_kint.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    const float* dm = model;
    float* dd = data;
    if (model_mem == SF_MEM_HOST) {
        CK(cudaMemcpyAsync(c->d_mig + nd, model, nmodel * sizeof(float), cudaMemcpyHostToDevice, st));
        dm = c->d_mig + nd;
    }
    if (data_mem == SF_MEM_HOST) dd = c->d_mig;
    CK(cudaMemsetAsync(dd, 0, nd * sizeof(float), st));
    if (ntrace > 0) {
        KirchFwdParams p;
        p.S = c->d_S;
        p.Ts = Ts;
        p.Tr = Tr;
        p.xs = c->d_kgeo;
        p.xr = c->d_kgeo + nsrc;
        p.model = dm;
        p.trace = c->d_kint;
        p.cmp = c->d_kint + ntrace;
        p.part = c->d_kpart;
        p.data = dd;
        p.nchunk = nchunk;
        p.chunk = chunk;
        p.nrec = nrec;
        p.nt = nt;
        p.nxx = c->nxx;
        p.nzz = c->nzz;
        p.nb = c->nb;
        p.nang = nang;
        p.warps = W;
        p.dt = dt;
        p.dx = c->dx;
        p.dz = c->dz;
        p.da = da;
        p.aperture = aperture;
        const size_t smem = (size_t)W * per_warp;
        const unsigned grid = (unsigned)((long)ntrace * nchunk);
        if (angle) {
            CK(cudaFuncSetAttribute(k_kirchhoff_forward<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k_kirchhoff_forward<true><<<grid, 32 * W, smem, st>>>(p);
        } else {
            CK(cudaFuncSetAttribute(k_kirchhoff_forward<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
            k_kirchhoff_forward<false><<<grid, 32 * W, smem, st>>>(p);
        }
        CK(cudaGetLastError());
        if (nchunk > 1) {
            const size_t n = (size_t)ntrace * nt;
            k_sum_chunks<<<(unsigned)std::min<size_t>((n + 255) / 256, (size_t)c->sms * 16), 256, 0, st>>>(
                c->d_kpart, c->d_kint, dd, ntrace, nchunk, nt);
            CK(cudaGetLastError());
        }
    }
    if (data_mem == SF_MEM_HOST) {
        CK(cudaMemcpyAsync(data, dd, nd * sizeof(float), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    return SF_OK;
}

extern "C" int sf_kirchhoff_image_forward(sf_ctx* c, const float* Ts, const float* Tr, int nsrc, int nrec,
                                          const float* xsrc, const float* xrec, const float* image, int image_mem,
                                          int nt, float dt, float aperture, float max_offset, float* data,
                                          int data_mem, void* stream)
{
    if (!c || !Ts || !Tr || !xsrc || !xrec || !image || !data || nsrc < 1 || nrec < 1 || nt < 1 || !(dt > 0.0f))
        return sf_fail(c, SF_ERR_ARG, "bad Kirchhoff arguments");
    return kirchhoff_forward(c, false, Ts, Tr, nsrc, nrec, xsrc, xrec, image, image_mem, (size_t)c->nx * c->nz, nt,
                             dt, aperture, max_offset, 0, 0, 0.0f, 1.0f, 1.0f, data, data_mem, stream);
}

extern "C" int sf_kirchhoff_angle_forward(sf_ctx* c, const float* Ts, const float* Tr, int nsrc, int nrec,
                                          const float* xsrc, const float* xrec, const float* gathers,
                                          int gathers_mem, int nt, float dt, float aperture, float max_offset,
                                          float max_angle, float da, float* data, int data_mem, void* stream)
{
    if (!c || !xsrc || !xrec) return sf_fail(c, SF_ERR_ARG, "null argument");
    int nang, ncmp;
    float mincmp, dcmp;
    if (angle_dims(xsrc, nsrc, xrec, nrec, max_angle, da, &nang, &ncmp, &mincmp, &dcmp))
        return sf_fail(c, SF_ERR_ARG, "angle gathers need two sources, two receivers, increasing positions, da > 0");
    if (!Ts || !Tr || !gathers || !data || nt < 1 || !(dt > 0.0f))
        return sf_fail(c, SF_ERR_ARG, "bad Kirchhoff arguments");
    const size_t ng = (size_t)(c->nzz - 2 * c->nb) * nang * ncmp;
    return kirchhoff_forward(c, true, Ts, Tr, nsrc, nrec, xsrc, xrec, gathers, gathers_mem, ng, nt, dt, aperture,
                             max_offset, nang, ncmp, mincmp, dcmp, da, data, data_mem, stream);
}
