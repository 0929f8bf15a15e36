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

extern "C" int sf_adjoint_convolution(sf_ctx* c, const float* traces, float* out, int ntr, int nt, float dt,
                                      float fmax, int mem, void* stream)
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
        k_correlate<<<(unsigned)std::min<size_t>((n + 255) / 256, (size_t)c->sms * 16), 256, 0, st>>>(
            din, dout, ntr, nt, c->d_wav, nw, nw / 2 + nw / 10, (double)next_pow2(nt + nw - 1));
        CK(cudaGetLastError());
    }
    if (mem == SF_MEM_HOST) {
        CK(cudaMemcpyAsync(out, dout, nb, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    return SF_OK;
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
