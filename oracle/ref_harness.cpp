// Runs the reference's own modeling kernels (compiled from the reference
// sources into cubins by build_ref.py) through the CUDA driver API, replaying
// the reference's host launch sequence. TEST INFRASTRUCTURE ONLY: it is the
// checker that pins the oracle and the engine to the reference's arithmetic.
//
// Host sequence restated from phbastosa/SeisFAT2D:
//   Modeling::set_eikonal        src/modeling/modeling.cu:62-102 (sign tables)
//   Modeling::initialization     src/modeling/modeling.cu:110-121
//   Modeling::eikonal_solver     src/modeling/modeling.cu:123-159
//   Eikonal_ANI::time_propagation src/modeling/eikonal_ani.cu:33-45
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {
CUmodule g_mod = nullptr, g_ani = nullptr, g_mig = nullptr;
CUfunction f_img = nullptr;
CUfunction f_set = nullptr, f_init = nullptr, f_sweep = nullptr, f_qs = nullptr;
CUcontext g_ctx = nullptr;
CUdevice g_dev = 0;

#define DR(call)                                       \
    do {                                               \
        CUresult _r = (call);                          \
        if (_r != CUDA_SUCCESS) {                      \
            const char* s = nullptr;                   \
            cuGetErrorString(_r, &s);                  \
            fprintf(stderr, "%s: %s\n", #call, s ? s : "?"); \
            return -(int)_r - 1000;                    \
        }                                              \
    } while (0)

CUresult get_fn(CUmodule m, const char* const* names, CUfunction* f)
{
    CUresult r = CUDA_ERROR_NOT_FOUND;
    for (int k = 0; names[k]; k++) {
        r = cuModuleGetFunction(f, m, names[k]);
        if (r == CUDA_SUCCESS) return r;
    }
    return r;
}
}  // namespace

extern "C" int ref_open(const char* modeling_cubin, const char* ani_cubin, int device)
{
    DR(cuInit(0));
    DR(cuDeviceGet(&g_dev, device));
    DR(cuDevicePrimaryCtxRetain(&g_ctx, g_dev));
    DR(cuCtxSetCurrent(g_ctx));
    DR(cuModuleLoad(&g_mod, modeling_cubin));
    DR(cuModuleLoad(&g_ani, ani_cubin));
    const char* n_set[] = {"_Z8time_setPfi", nullptr};
    const char* n_init[] = {"_Z9time_initPfS_ffffiiii", nullptr};
    const char* n_sweep[] = {"_Z11inner_sweepPfS_PiS0_iiiiiiiiffff", nullptr};
    const char* n_qs[] = {"_Z18get_quasi_slownessPfS_ffiiiiiPtS0_S0_S0_S0_S0_ffffffffffff", nullptr};
    DR(get_fn(g_mod, n_set, &f_set));
    DR(get_fn(g_mod, n_init, &f_init));
    DR(get_fn(g_mod, n_sweep, &f_sweep));
    DR(get_fn(g_ani, n_qs, &f_qs));
    return 0;
}

extern "C" int ref_close()
{
    if (g_mod) cuModuleUnload(g_mod);
    if (g_ani) cuModuleUnload(g_ani);
    if (g_mig) cuModuleUnload(g_mig);
    g_mod = g_ani = g_mig = nullptr;
    if (g_ctx) cuDevicePrimaryCtxRelease(g_dev);
    g_ctx = nullptr;
    return 0;
}

namespace {
int initialization(CUdeviceptr dT, CUdeviceptr dS, int matsize, int nzz, int nb, float sx, float sz,
                   float dx, float dz, int* sIdx_out, int* sIdz_out)
{
    int sIdx = (int)((sx + 0.5f * dx) / dx) + nb;
    int sIdz = (int)((sz + 0.5f * dz) / dz) + nb;
    *sIdx_out = sIdx;
    *sIdz_out = sIdz;
    int nBlocks = (matsize + 256 - 1) / 256;
    void* a1[] = {&dT, &matsize};
    DR(cuLaunchKernel(f_set, nBlocks, 1, 1, 256, 1, 1, 0, 0, a1, nullptr));
    void* a2[] = {&dT, &dS, &sx, &sz, &dx, &dz, &sIdx, &sIdz, &nzz, &nb};
    DR(cuLaunchKernel(f_init, 1, 1, 1, 3, 3, 1, 0, 0, a2, nullptr));
    return 0;
}

int eikonal_solver(CUdeviceptr dT, CUdeviceptr dS, CUdeviceptr dsgnv, CUdeviceptr dsgnt, int nxx, int nzz,
                   float dx, float dz)
{
    float dz2i = 1.0f / (dz * dz);
    float dx2i = 1.0f / (dx * dx);
    int total_levels = (nxx - 1) + (nzz - 1);
    int min_level = std::min(nxx, nzz), max_level = std::max(nxx, nzz);
    for (int sweep = 0; sweep < 4; sweep++) {
        int zd = (sweep == 2 || sweep == 3) ? -1 : 1;
        int xd = (sweep == 0 || sweep == 2) ? -1 : 1;
        int sgni = sweep + 0 * 4;
        int sgnj = sweep + 1 * 4;
        for (int level = 0; level < total_levels; level++) {
            int z_offset = (sweep == 0) ? ((level < nxx) ? 0 : level - nxx + 1)
                         : (sweep == 1) ? ((level < nzz) ? nzz - level - 1 : 0)
                         : (sweep == 2) ? ((level < nzz) ? level : nzz - 1)
                                        : ((level < nxx) ? nzz - 1 : nzz - 1 - (level - nxx + 1));
            int x_offset = (sweep == 0) ? ((level < nxx) ? level : nxx - 1)
                         : (sweep == 1) ? ((level < nzz) ? 0 : level - nzz + 1)
                         : (sweep == 2) ? ((level < nzz) ? nxx - 1 : nxx - 1 - (level - nzz + 1))
                                        : ((level < nxx) ? nxx - level - 1 : 0);
            int n_elements = (level < min_level) ? level + 1
                           : (level >= max_level) ? total_levels - level
                                                  : total_levels - min_level - max_level + level;
            int nblk = (n_elements + 256 - 1) / 256;
            void* a[] = {&dT, &dS, &dsgnv, &dsgnt, &sgni, &sgnj, &x_offset, &z_offset, &xd, &zd,
                         &nxx, &nzz, &dx, &dz, &dx2i, &dz2i};
            DR(cuLaunchKernel(f_sweep, nblk, 1, 1, 256, 1, 1, 0, 0, a, nullptr));
        }
    }
    return 0;
}
}  // namespace

// One shot on the padded grid (host buffers). ani != 0 runs the two-pass
// anisotropic solve with the quantised codes. ms_out: GPU time of the
// time_propagation sequence (CUDA events), excluding the copies.
extern "C" int ref_solve(int nxx, int nzz, int nb, const float* S, float dx, float dz, float sx, float sz,
                         int ani, const uint16_t* const* codes, const float* mm, float* T_out, double* ms_out,
                         int repeats)
{
    DR(cuCtxSetCurrent(g_ctx));
    const int matsize = nxx * nzz;
    CUdeviceptr dT, dS, dsgnv, dsgnt;
    CUdeviceptr dC[6] = {0, 0, 0, 0, 0, 0};
    DR(cuMemAlloc(&dT, sizeof(float) * matsize));
    DR(cuMemAlloc(&dS, sizeof(float) * matsize));
    DR(cuMemAlloc(&dsgnv, sizeof(int) * 8));
    DR(cuMemAlloc(&dsgnt, sizeof(int) * 8));
    // modeling.cu:69-82: sgnv = {{1,1},{0,1},{1,0},{0,0}}, sgnt = {{1,1},{-1,1},{1,-1},{-1,-1}}
    const int sgnv[4][2] = {{1, 1}, {0, 1}, {1, 0}, {0, 0}};
    const int sgnt[4][2] = {{1, 1}, {-1, 1}, {1, -1}, {-1, -1}};
    int hv[8], ht[8];
    for (int index = 0; index < 8; index++) {
        int j = index / 4, i = index % 4;
        hv[i + j * 4] = sgnv[i][j];
        ht[i + j * 4] = sgnt[i][j];
    }
    DR(cuMemcpyHtoD(dsgnv, hv, sizeof(hv)));
    DR(cuMemcpyHtoD(dsgnt, ht, sizeof(ht)));
    if (ani) {
        for (int q = 0; q < 6; q++) {
            DR(cuMemAlloc(&dC[q], sizeof(uint16_t) * matsize));
            DR(cuMemcpyHtoD(dC[q], codes[q], sizeof(uint16_t) * matsize));
        }
    }
    CUevent e0, e1;
    DR(cuEventCreate(&e0, CU_EVENT_DEFAULT));
    DR(cuEventCreate(&e1, CU_EVENT_DEFAULT));
    double best = 1e30;
    if (repeats < 1) repeats = 1;
    for (int rep = 0; rep < repeats; rep++) {
        DR(cuMemcpyHtoD(dS, S, sizeof(float) * matsize));
        DR(cuCtxSynchronize());
        DR(cuEventRecord(e0, 0));
        int sIdx, sIdz, rc;
        if ((rc = initialization(dT, dS, matsize, nzz, nb, sx, sz, dx, dz, &sIdx, &sIdz))) return rc;
        if ((rc = eikonal_solver(dT, dS, dsgnv, dsgnt, nxx, nzz, dx, dz))) return rc;
        if (ani) {
            int nBlocks = (matsize + 256 - 1) / 256;
            float m[12];
            std::memcpy(m, mm, sizeof(m));  // (min, max) pairs C11..C55
            void* a[] = {&dT, &dS, &dx, &dz, &sIdx, &sIdz, &nxx, &nzz, &nb,
                         &dC[0], &dC[1], &dC[2], &dC[3], &dC[4], &dC[5],
                         &m[0], &m[1], &m[2], &m[3], &m[4], &m[5], &m[6], &m[7], &m[8], &m[9], &m[10], &m[11]};
            DR(cuLaunchKernel(f_qs, nBlocks, 1, 1, 256, 1, 1, 0, 0, a, nullptr));
            if ((rc = initialization(dT, dS, matsize, nzz, nb, sx, sz, dx, dz, &sIdx, &sIdz))) return rc;
            if ((rc = eikonal_solver(dT, dS, dsgnv, dsgnt, nxx, nzz, dx, dz))) return rc;
        }
        DR(cuEventRecord(e1, 0));
        DR(cuEventSynchronize(e1));
        float ms = 0.0f;
        DR(cuEventElapsedTime(&ms, e0, e1));
        best = std::min(best, (double)ms);
    }
    DR(cuMemcpyDtoH(T_out, dT, sizeof(float) * matsize));
    if (ms_out) *ms_out = best;
    cuEventDestroy(e0);
    cuEventDestroy(e1);
    cuMemFree(dT);
    cuMemFree(dS);
    cuMemFree(dsgnv);
    cuMemFree(dsgnt);
    for (int q = 0; q < 6; q++)
        if (dC[q]) cuMemFree(dC[q]);
    return 0;
}

// time_set + time_init only (modeling.cu:110-121): the reference's initial
// field for one source, to pin the near-source arithmetic.
extern "C" int ref_init(int nxx, int nzz, int nb, const float* S, float dx, float dz, float sx, float sz,
                        float* T_out)
{
    DR(cuCtxSetCurrent(g_ctx));
    const int matsize = nxx * nzz;
    CUdeviceptr dT, dS;
    DR(cuMemAlloc(&dT, sizeof(float) * matsize));
    DR(cuMemAlloc(&dS, sizeof(float) * matsize));
    DR(cuMemcpyHtoD(dS, S, sizeof(float) * matsize));
    int sIdx, sIdz, rc;
    if ((rc = initialization(dT, dS, matsize, nzz, nb, sx, sz, dx, dz, &sIdx, &sIdz))) return rc;
    DR(cuCtxSynchronize());
    DR(cuMemcpyDtoH(T_out, dT, sizeof(float) * matsize));
    cuMemFree(dT);
    cuMemFree(dS);
    return 0;
}

// ---------------------------------------------------------------- Kirchhoff
//
// KDM::kirchhoff_depth_migration (src/migration/KDM.cu:3-55) with the image-
// domain kernel (IDKDM::perform_adjoint, src/migration/IDKDM.cu:19-22): for
// every source, for every receiver within max_offset, one launch of
// image_domain_adjoint_kernel over the padded grid with that pair's tables and
// (already correlated) trace, CMP = (sx + rx) / 2. Tables are padded nzz x nxx
// fields, z fastest; data is nsrc x nrec x nt.
extern "C" int ref_kirchhoff_open(const char* migration_cubin)
{
    if (!g_ctx) return -1;
    DR(cuCtxSetCurrent(g_ctx));
    if (!g_mig) {
        DR(cuModuleLoad(&g_mig, migration_cubin));
        const char* n_img[] = {"_Z27image_domain_adjoint_kernelPfS_S_S_S_fiffiiiff", nullptr};
        DR(get_fn(g_mig, n_img, &f_img));
    }
    return 0;
}

extern "C" int ref_kirchhoff_adjoint(int nxx, int nzz, int nb, const float* S, const float* Ts, const float* Tr,
                                     int nsrc, int nrec, const float* xsrc, const float* xrec, const float* data,
                                     int nt, float dt, float dx, float dz, float aperture, float max_offset,
                                     float* image)
{
    DR(cuCtxSetCurrent(g_ctx));
    const size_t matsize = (size_t)nxx * nzz;
    const int nx = nxx - 2 * nb, nz = nzz - 2 * nb;
    CUdeviceptr dS, dTs, dTr, dd, dm;
    DR(cuMemAlloc(&dS, sizeof(float) * matsize));
    DR(cuMemAlloc(&dTs, sizeof(float) * matsize * nsrc));
    DR(cuMemAlloc(&dTr, sizeof(float) * matsize * nrec));
    DR(cuMemAlloc(&dd, sizeof(float) * (size_t)nsrc * nrec * nt));
    DR(cuMemAlloc(&dm, sizeof(float) * (size_t)nx * nz));
    DR(cuMemcpyHtoD(dS, S, sizeof(float) * matsize));
    DR(cuMemcpyHtoD(dTs, Ts, sizeof(float) * matsize * nsrc));
    DR(cuMemcpyHtoD(dTr, Tr, sizeof(float) * matsize * nrec));
    DR(cuMemcpyHtoD(dd, data, sizeof(float) * (size_t)nsrc * nrec * nt));
    DR(cuMemsetD32(dm, 0, (size_t)nx * nz));
    const unsigned nblocks = (unsigned)((matsize + 255) / 256);
    for (int s = 0; s < nsrc; s++)
        for (int r = 0; r < nrec; r++) {
            const float offset = fabsf(xsrc[s] - xrec[r]);
            if (!(offset < max_offset)) continue;
            float cmp = 0.5f * (xsrc[s] + xrec[r]);
            CUdeviceptr ts = dTs + sizeof(float) * matsize * s, tr = dTr + sizeof(float) * matsize * r;
            CUdeviceptr tdat = dd + sizeof(float) * ((size_t)s * nrec + r) * nt;
            void* args[] = {&dS, &ts, &tr, &tdat, &dm, &dt, &nt, &dx, &dz, &nxx, &nzz, &nb, &aperture, &cmp};
            DR(cuLaunchKernel(f_img, nblocks, 1, 1, 256, 1, 1, 0, nullptr, args, nullptr));
        }
    DR(cuCtxSynchronize());
    DR(cuMemcpyDtoH(image, dm, sizeof(float) * (size_t)nx * nz));
    cuMemFree(dS);
    cuMemFree(dTs);
    cuMemFree(dTr);
    cuMemFree(dd);
    cuMemFree(dm);
    return 0;
}

// ADKDM (src/migration/ADKDM.cu:17-20 in the KDM.cu:3-55 loop): one launch of
// angle_domain_adjoint_kernel per trace within max_offset, with that trace's
// CMP and CMP bin (cmpId = (int)((CMP - minCMP) / dCMP)).
extern "C" int ref_kirchhoff_angles(int nxx, int nzz, int nb, const float* S, const float* Ts, const float* Tr,
                                    int nsrc, int nrec, const float* xsrc, const float* xrec, const float* data,
                                    int nt, float dt, float dx, float dz, float aperture, float max_offset, float da,
                                    int na, int ncmp, float mincmp, float dcmp, float* gathers)
{
    DR(cuCtxSetCurrent(g_ctx));
    static CUfunction f_ang = nullptr;
    if (!f_ang) {
        const char* n_ang[] = {"_Z27angle_domain_adjoint_kernelPfS_S_S_S_ffffiiiiiffi", nullptr};
        DR(get_fn(g_mig, n_ang, &f_ang));
    }
    const size_t matsize = (size_t)nxx * nzz;
    const int nz = nzz - 2 * nb;
    const size_t ng = (size_t)nz * na * ncmp;
    CUdeviceptr dS, dTs, dTr, dd, dm;
    DR(cuMemAlloc(&dS, sizeof(float) * matsize));
    DR(cuMemAlloc(&dTs, sizeof(float) * matsize * nsrc));
    DR(cuMemAlloc(&dTr, sizeof(float) * matsize * nrec));
    DR(cuMemAlloc(&dd, sizeof(float) * (size_t)nsrc * nrec * nt));
    DR(cuMemAlloc(&dm, sizeof(float) * ng));
    DR(cuMemcpyHtoD(dS, S, sizeof(float) * matsize));
    DR(cuMemcpyHtoD(dTs, Ts, sizeof(float) * matsize * nsrc));
    DR(cuMemcpyHtoD(dTr, Tr, sizeof(float) * matsize * nrec));
    DR(cuMemcpyHtoD(dd, data, sizeof(float) * (size_t)nsrc * nrec * nt));
    DR(cuMemsetD32(dm, 0, ng));
    const unsigned nblocks = (unsigned)((matsize + 255) / 256);
    for (int s = 0; s < nsrc; s++)
        for (int r = 0; r < nrec; r++) {
            if (!(fabsf(xsrc[s] - xrec[r]) < max_offset)) continue;
            float cmp = 0.5f * (xsrc[s] + xrec[r]);
            int cmpId = (int)((cmp - mincmp) / dcmp);
            CUdeviceptr ts = dTs + sizeof(float) * matsize * s, tr = dTr + sizeof(float) * matsize * r;
            CUdeviceptr tdat = dd + sizeof(float) * ((size_t)s * nrec + r) * nt;
            void* args[] = {&dS, &ts, &tr, &tdat, &dm, &dx, &dz, &dt, &da, &nxx, &nzz, &nt, &na, &nb, &aperture, &cmp,
                            &cmpId};
            DR(cuLaunchKernel(f_ang, nblocks, 1, 1, 256, 1, 1, 0, nullptr, args, nullptr));
        }
    DR(cuCtxSynchronize());
    DR(cuMemcpyDtoH(gathers, dm, sizeof(float) * ng));
    cuMemFree(dS);
    cuMemFree(dTs);
    cuMemFree(dTr);
    cuMemFree(dd);
    cuMemFree(dm);
    return 0;
}

// The least-squares variants' forward operators as LSKDM::compute_gradient
// runs them (LSKDM.cu:52-90): per source, per receiver within max_offset, the
// trace buffer zeroed, then one launch of image_domain_forward_kernel
// (migration.cu:485-570; angle = 0, model nz x nx) or
// angle_domain_forward_kernel (:665-756; angle = 1, model nz x na x ncmp,
// cmpId = (cmp - mincmp) / dcmp). data (nsrc x nrec x nt) gets the raw
// (unconvolved) traces; the other traces are 0.
extern "C" int ref_kirchhoff_forward(int angle, int nxx, int nzz, int nb, const float* S, const float* Ts,
                                     const float* Tr, int nsrc, int nrec, const float* xsrc, const float* xrec,
                                     const float* model, size_t nmodel, int nt, float dt, float dx, float dz,
                                     float aperture, float max_offset, float da, int na, float mincmp, float dcmp,
                                     float* data)
{
    DR(cuCtxSetCurrent(g_ctx));
    static CUfunction f_fimg = nullptr, f_fang = nullptr;
    if (!f_fimg) {
        const char* n1[] = {"_Z27image_domain_forward_kernelPfS_S_S_S_fiffiiiff", nullptr};
        const char* n2[] = {"_Z27angle_domain_forward_kernelPfS_S_S_S_ffffiiiiiffi", nullptr};
        DR(get_fn(g_mig, n1, &f_fimg));
        DR(get_fn(g_mig, n2, &f_fang));
    }
    const size_t matsize = (size_t)nxx * nzz;
    CUdeviceptr dS, dTs, dTr, dd, dm;
    DR(cuMemAlloc(&dS, sizeof(float) * matsize));
    DR(cuMemAlloc(&dTs, sizeof(float) * matsize * nsrc));
    DR(cuMemAlloc(&dTr, sizeof(float) * matsize * nrec));
    DR(cuMemAlloc(&dd, sizeof(float) * (size_t)nt));
    DR(cuMemAlloc(&dm, sizeof(float) * nmodel));
    DR(cuMemcpyHtoD(dS, S, sizeof(float) * matsize));
    DR(cuMemcpyHtoD(dTs, Ts, sizeof(float) * matsize * nsrc));
    DR(cuMemcpyHtoD(dTr, Tr, sizeof(float) * matsize * nrec));
    DR(cuMemcpyHtoD(dm, model, sizeof(float) * nmodel));
    const unsigned nblocks = (unsigned)((matsize + 255) / 256);
    for (int s = 0; s < nsrc; s++)
        for (int r = 0; r < nrec; r++) {
            float* out = data + ((size_t)s * nrec + r) * nt;
            for (int t = 0; t < nt; t++) out[t] = 0.0f;
            if (!(fabsf(xsrc[s] - xrec[r]) < max_offset)) continue;
            float cmp = 0.5f * (xsrc[s] + xrec[r]);
            CUdeviceptr ts = dTs + sizeof(float) * matsize * s, tr = dTr + sizeof(float) * matsize * r;
            DR(cuMemsetD32(dd, 0, (size_t)nt));
            if (angle) {
                int cmpId = (int)((cmp - mincmp) / dcmp);
                void* args[] = {&dS, &ts, &tr, &dd, &dm, &dx, &dz, &dt, &da, &nxx, &nzz, &nt, &na, &nb, &aperture, &cmp,
                                &cmpId};
                DR(cuLaunchKernel(f_fang, nblocks, 1, 1, 256, 1, 1, 0, nullptr, args, nullptr));
            } else {
                void* args[] = {&dS, &ts, &tr, &dd, &dm, &dt, &nt, &dx, &dz, &nxx, &nzz, &nb, &aperture, &cmp};
                DR(cuLaunchKernel(f_fimg, nblocks, 1, 1, 256, 1, 1, 0, nullptr, args, nullptr));
            }
            DR(cuCtxSynchronize());
            DR(cuMemcpyDtoH(out, dd, sizeof(float) * (size_t)nt));
        }
    cuMemFree(dS);
    cuMemFree(dTs);
    cuMemFree(dTr);
    cuMemFree(dd);
    cuMemFree(dm);
    return 0;
}
