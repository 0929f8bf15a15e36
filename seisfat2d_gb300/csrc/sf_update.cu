// Tomography model update on the device: the Gaussian smoothing of
// Inversion::model_smoothing / smooth_matrix (src/inversion/inversion.cpp:
// 347-447) and the slowness update of Tomography_ISO::model_update
// (src/inversion/tomography_iso.cpp:77-92), with the reference's arithmetic.
#include <cuda_runtime.h>

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

// Output cell (i, j) of the model (nz x nx, z fastest): the reference pads the
// model with `samples` zero cells on every side, then sums samples x samples taps
// (tap (zk, xk) of the kernel on cell (i - mid + zk, j - mid + xk) of the padded
// grid) in FP32, xk outer, zk inner, product then sum. Every model cell lies
// at least mid = samples/2 cells inside the padded grid, so every model cell
// is smoothed.
__global__ void k_smooth(const float* __restrict__ in, int nx, int nz, int n, const float* __restrict__ K,
                         float* __restrict__ out)
{
    const size_t np = (size_t)nx * nz;
    const int mid = n / 2;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < np;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx % nz), j = (int)(idx / nz);
        float acc = 0.0f;
        for (int xk = 0; xk < n; xk++) {
            const int mj = j - mid + xk;          // model column of the tap
            for (int zk = 0; zk < n; zk++) {
                const int mi = i - mid + zk;      // model row of the tap
                const float v = (mi >= 0 && mi < nz && mj >= 0 && mj < nx) ? in[mi + (size_t)mj * nz] : 0.0f;
                acc = __fadd_rn(acc, __fmul_rn(v, K[zk + xk * n]));
            }
        }
        out[idx] = acc;
    }
}

// dS = scale * grad over the model interior of the padded gradient.
__global__ void k_scale_interior(const float* __restrict__ g, int nx, int nz, int nb, int nzz, float scale,
                                 float* __restrict__ dS)
{
    const size_t np = (size_t)nx * nz;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < np;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx % nz), j = (int)(idx / nz);
        dS[idx] = __fmul_rn(scale, g[(i + nb) + (size_t)(j + nb) * nzz]);
    }
}

// S += dS on the model interior of the padded slowness (the pad ring keeps its
// values, as in the reference).
__global__ void k_add_interior(float* __restrict__ S, int nx, int nz, int nb, int nzz, const float* __restrict__ dS)
{
    const size_t np = (size_t)nx * nz;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < np;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx % nz), j = (int)(idx / nz);
        float* p = S + (i + nb) + (size_t)(j + nb) * nzz;
        *p = __fadd_rn(*p, dS[idx]);
    }
}

}  // namespace

// The reference's normalised Gaussian: weight 1/(pi stdv) exp(-r^2/(2 stdv^2))
// computed as its source does (the prefactor in double, expf in float, the
// product rounded once to float), summed in FP32 (x outer, z inner) and
// divided by the sum; stdv == 0 gives the unit tap at the centre.
void sf_smooth_kernel(float stdv, int n, std::vector<float>& k)
{
    k.assign((size_t)n * n, 0.0f);
    const int mid = n / 2;
    k[mid + (size_t)mid * n] = 1.0f;
    if (stdv == 0.0f) return;
    float sum = 0.0f;
    for (int x = -mid; x <= mid; x++)
        for (int z = -mid; z <= mid; z++) {
            const int index = (z + mid) + (x + mid) * n;
            const float r = std::sqrt((float)(x * x + z * z));
            k[index] = (float)(1.0f / (M_PI * stdv) * (double)std::exp(-((r * r) / (2.0f * stdv * stdv))));
            sum += k[index];
        }
    for (auto& v : k) v /= sum;
}

static int smooth_on_device(sf_ctx* c, const float* d_in, float* d_out, float stdv, int samples, cudaStream_t st)
{
    std::vector<float> k;
    sf_smooth_kernel(stdv, samples, k);
    int rc = sf_dev_reserve(c, (void**)&c->d_skern, &c->cap_skern, k.size() * sizeof(float));
    if (rc) return rc;
    c->h_skern.swap(k);
    CK(cudaMemcpyAsync(c->d_skern, c->h_skern.data(), c->h_skern.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    const size_t np = (size_t)c->nx * c->nz;
    k_smooth<<<(unsigned)std::min<size_t>((np + 255) / 256, (size_t)c->sms * 8), 256, 0, st>>>(
        d_in, c->nx, c->nz, samples, c->d_skern, d_out);
    CK(cudaGetLastError());
    return SF_OK;
}

static int check_samples(sf_ctx* c, int samples)
{
    if (samples < 1 || samples % 2 == 0 || samples > 1001)
        return sf_fail(c, SF_ERR_ARG, "gaussian_filter_samples must be an odd number in 1..1001");
    return SF_OK;
}

extern "C" int sf_smooth_model(sf_ctx* c, const float* in, float* out, float stdv, int samples, int mem,
                               void* stream)
{
    if (!c || !in || !out) return sf_fail(c, SF_ERR_ARG, "null argument");
    int rc = check_samples(c, samples);
    if (rc) return rc;
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t nb = (size_t)c->nx * c->nz * sizeof(float);
    const float* d_in = in;
    float* d_out = out;
    if (mem == SF_MEM_HOST) {
        rc = sf_dev_reserve(c, (void**)&c->d_upd, &c->cap_upd, 2 * nb);
        if (rc) return rc;
        CK(cudaMemcpyAsync(c->d_upd, in, nb, cudaMemcpyHostToDevice, st));
        d_in = c->d_upd;
        d_out = c->d_upd + (size_t)c->nx * c->nz;
    }
    rc = smooth_on_device(c, d_in, d_out, stdv, samples, st);
    if (rc) return rc;
    if (mem == SF_MEM_HOST) {
        CK(cudaMemcpyAsync(out, d_out, nb, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    return SF_OK;
}

extern "C" int sf_update_slowness(sf_ctx* c, const float* grad, int grad_mem, float scale, float stdv, int samples,
                                  float* dS, int dS_mem, void* stream)
{
    if (!c || !grad) return sf_fail(c, SF_ERR_ARG, "null argument");
    if (samples != 0) {
        int rc = check_samples(c, samples);
        if (rc) return rc;
    }
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t np = (size_t)c->nx * c->nz, npad = (size_t)c->nxx * c->nzz;
    int rc = sf_dev_reserve(c, (void**)&c->d_upd, &c->cap_upd, (2 * np + npad) * sizeof(float));
    if (rc) return rc;
    float* d_a = c->d_upd;
    float* d_b = c->d_upd + np;
    const float* d_g = grad;
    if (grad_mem == SF_MEM_HOST) {
        CK(cudaMemcpyAsync(c->d_upd + 2 * np, grad, npad * sizeof(float), cudaMemcpyHostToDevice, st));
        d_g = c->d_upd + 2 * np;
    }
    const unsigned grid = (unsigned)std::min<size_t>((np + 255) / 256, (size_t)c->sms * 8);
    k_scale_interior<<<grid, 256, 0, st>>>(d_g, c->nx, c->nz, c->nb, c->nzz, scale, d_a);
    CK(cudaGetLastError());
    float* d_dS = d_a;
    if (samples != 0) {
        rc = smooth_on_device(c, d_a, d_b, stdv, samples, st);
        if (rc) return rc;
        d_dS = d_b;
    }
    k_add_interior<<<grid, 256, 0, st>>>(c->d_S, c->nx, c->nz, c->nb, c->nzz, d_dS);
    CK(cudaGetLastError());
    if (dS) CK(cudaMemcpyAsync(dS, d_dS, np * sizeof(float),
                               dS_mem == SF_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));  // the slowness is read by calls on any stream
    return SF_OK;
}
