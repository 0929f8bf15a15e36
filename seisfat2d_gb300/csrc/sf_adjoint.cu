// Adjoint-state gradient of the pick misfit: C ABI entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "sf_adjoint.cuh"
#include "sf_engine.h"

using namespace sf;

#define CK(call)                                                          \
    do {                                                                  \
        int _st = sf_cuda_check(c, (call), #call);                        \
        if (_st != SF_OK) return _st;                                     \
    } while (0)

void sf_adjoint_release(sf_ctx* c)
{
    void* bufs[] = {c->d_lam, c->d_vrec, c->d_gshot, c->d_pg, c->d_misfit, c->d_colptr,
                    c->d_lam_init, c->d_hand2, c->d_ctr2, c->d_seed_i, c->d_seed_w, c->d_gshots};
    for (void* b : bufs)
        if (b) cudaFree(b);
}

size_t sf_adj_smem_bytes(int warps)
{
    return ((sizeof(CtaShared) + 15) & ~size_t(15)) + (size_t)warps * sizeof(AdjRing);
}

int sf_adj_setup(sf_ctx* c)
{
    CK(cudaFuncSetAttribute(k_adjoint<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)sf_adj_smem_bytes(kMaxWarps)));
    CK(cudaFuncSetAttribute(k_adjoint<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)sf_adj_smem_bytes(kMaxWarps)));
    const int fs = (int)std::max(sf_adj_smem_bytes(kMaxWarps), sizeof(GatherSmem));
    for (const void* f : {(const void*)k_adjoint_gather<false, 2>, (const void*)k_adjoint_gather<true, 2>,
                          (const void*)k_adjoint_gather<false, 4>, (const void*)k_adjoint_gather<true, 4>})
        CK(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, fs));
    return SF_OK;
}

// Catmull-Rom weights of the pick rule for offset t (the rule is linear in
// its 16 nodes): P -> P1 + 0.5 t (P2 - P0 + t (2P0 - 5P1 + 4P2 - P3 + t (3(P1 -
// P2) + P3 - P0))), every FP64 operation rounded once, left to right.
static void cubic_weights(double t, double w[4])
{
    const double t2 = t * t, t3 = t2 * t;
    w[0] = ((-0.5 * t) + t2) - (0.5 * t3);
    w[1] = (1.0 - (2.5 * t2)) + (1.5 * t3);
    w[2] = ((0.5 * t) + (2.0 * t2)) - (1.5 * t3);
    w[3] = (-0.5 * t2) + (0.5 * t3);
}

// Seed table of the batch's receivers for the adjoint (host, once per batch):
// the receiver's node and offsets as the pick rule computes them in FP32
// (modeling.cu:161-194: the same operations as pick_geom on the device), its
// 16 weights in FP64 rounded once to FP32, and per padded node the list of
// (receiver, weight) in receiver order. Whether a receiver's stencil lies in
// a shot's window is decided per shot from its padded column.
static int prepare_seed(sf_ctx* c, cudaStream_t st)
{
    if (c->seed_gen == c->recv_gen && c->seed_nrec == c->batch_nrec) return SF_OK;  // same receivers
    const int nrec = c->batch_nrec, nzz = c->nzz, nb = c->nb;
    const float dx = c->dx, dz = c->dz;
    std::vector<int> rec_jg(std::max(nrec, 1), -1000000);
    std::vector<std::pair<long long, std::pair<int, float>>> ent;  // (node key, (receiver, weight))
    for (int r = 0; r < nrec; r++) {
        const float x = c->h_rx[r], z = c->h_rz[r];
        const float ax = (x + 0.5f * dx) / dx, az = (z + 0.5f * dz) / dz;
        const float x0 = std::floor(ax) * dx, z0 = std::floor(az) * dz;
        const float x1 = std::floor(ax) * dx + dx, z1 = std::floor(az) * dz + dz;
        const float xd = (x - x0) / (x1 - x0), zd = (z - z0) / (z1 - z0);
        if (!(ax > -1e9f && ax < 1e9f && az > -1e9f && az < 1e9f)) continue;
        const int i = (int)az + nb, jg = (int)ax + nb;
        if (i - 1 < 1 || i + 2 > nzz - 2) continue;  // rows outside the grid: never picked
        if (jg - 1 < 1 || jg + 2 > c->nxx - 2) continue;  // no window can hold the stencil
        rec_jg[r] = jg;
        double wx[4], wz[4];
        cubic_weights((double)xd, wx);
        cubic_weights((double)zd, wz);
        for (int aa = 0; aa < 4; aa++)
            for (int bb = 0; bb < 4; bb++) {
                const long long key = (long long)(jg + aa - 1) * nzz + (i + bb - 1);
                ent.push_back({key, {r, (float)(wx[aa] * wz[bb])}});
            }
    }
    std::stable_sort(ent.begin(), ent.end(),
                     [](const auto& a, const auto& b) { return a.first < b.first; });  // receiver order kept
    std::vector<int> ptr(1, 0), row, col, rec;
    std::vector<float> w;
    for (size_t e = 0; e < ent.size(); e++) {
        if (e == 0 || ent[e].first != ent[e - 1].first) {
            if (e) ptr.push_back((int)e);
            row.push_back((int)(ent[e].first % nzz));
            col.push_back((int)(ent[e].first / nzz));
        }
        rec.push_back(ent[e].second.first);
        w.push_back(ent[e].second.second);
    }
    ptr.push_back((int)ent.size());
    if (ent.empty()) ptr.assign(1, 0);
    const int nn = (int)row.size(), ne = (int)rec.size();
    std::vector<int> pack;
    pack.reserve(ptr.size() + 2 * nn + ne + rec_jg.size());
    pack.insert(pack.end(), ptr.begin(), ptr.end());
    pack.insert(pack.end(), row.begin(), row.end());
    pack.insert(pack.end(), col.begin(), col.end());
    pack.insert(pack.end(), rec.begin(), rec.end());
    pack.insert(pack.end(), rec_jg.begin(), rec_jg.end());
    int rc = sf_dev_reserve(c, (void**)&c->d_seed_i, &c->cap_seed_i, pack.size() * sizeof(int));
    if (!rc) rc = sf_dev_reserve(c, (void**)&c->d_seed_w, &c->cap_seed_w, std::max<size_t>(w.size(), 1) * sizeof(float));
    if (rc) return rc;
    c->h_seed_pack.swap(pack);
    c->h_seed_w.swap(w);
    CK(cudaMemcpyAsync(c->d_seed_i, c->h_seed_pack.data(), c->h_seed_pack.size() * sizeof(int),
                       cudaMemcpyHostToDevice, st));
    if (!c->h_seed_w.empty())
        CK(cudaMemcpyAsync(c->d_seed_w, c->h_seed_w.data(), c->h_seed_w.size() * sizeof(float),
                           cudaMemcpyHostToDevice, st));
    c->seed_nodes = nn;
    c->seed_entries = ne;
    c->seed_gen = c->recv_gen;
    c->seed_nrec = nrec;
    return SF_OK;
}

// The gather's shot lists (host, once per batch): for each block of kGT
// padded columns, the shots whose window covers any of its columns, in caller
// order, with what the gather needs of each.
static int prepare_gather(sf_ctx* c, cudaStream_t st)
{
    if (c->gather_gen == c->shots_gen) return SF_OK;  // same shot table

    const int ns = (int)c->hshots.size();
    const int nblk = (c->nxx + kGT - 1) / kGT;
    std::vector<int> ptr(nblk + 1, 0);
    std::vector<GatherShot> ent;
    for (int cb = 0; cb < nblk; cb++) {
        const int col = cb * kGT;
        for (int o = 0; o < ns; o++) {
            const ShotDev& d = c->hshots[c->tables_index[o]];
            if (d.c0 < col + kGT && d.c0 + d.ncols > col) {
                GatherShot g;
                std::memset(&g, 0, sizeof(g));
                g.tape_off = d.tape_off;
                g.c0 = d.c0;
                g.ncols = d.ncols;
                g.sIdx = d.sIdx;
                g.sIdz = d.sIdz;
                g.sx = d.sx;
                g.sz = d.sz;
                g.orig = o;
                g.q_off = d.q_off;
                ent.push_back(g);
            }
        }
        ptr[cb + 1] = (int)ent.size();
    }
    int rc = sf_dev_reserve(c, (void**)&c->d_colptr, &c->cap_colptr, ptr.size() * sizeof(int));
    if (!rc) rc = sf_dev_reserve(c, (void**)&c->d_gshots, &c->cap_gshots, std::max<size_t>(ent.size(), 1) * sizeof(GatherShot));
    if (rc) return rc;
    c->h_colptr.swap(ptr);
    c->h_gshots.swap(ent);
    CK(cudaMemcpyAsync(c->d_colptr, c->h_colptr.data(), c->h_colptr.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    if (!c->h_gshots.empty())
        CK(cudaMemcpyAsync(c->d_gshots, c->h_gshots.data(), c->h_gshots.size() * sizeof(GatherShot),
                           cudaMemcpyHostToDevice, st));
    c->gather_gen = c->shots_gen;
    return SF_OK;
}

int sf_adj_configure(sf_ctx* c, cudaStream_t st, AdjLaunch* A)
{
    const int ns = (int)c->hshots.size();
    const int nstrips = (c->nzz + 31) / 32;
    const size_t smem = sf_adj_smem_bytes(c->warps);
    int G, NG;
    // the reverse sweeps take the loop form of the taped forward they reverse
    const void* akern = c->batch_interior ? (const void*)k_adjoint<true> : (const void*)k_adjoint<false>;
    int rc = sf_gang_shape(c, akern, smem, ns, nstrips, c->gang_warps, &G, &NG);
    if (rc) return rc;
    rc = sf_dev_reserve(c, (void**)&c->d_lam, &c->cap_lam, (size_t)NG * c->nzz * c->batch_maxcols * sizeof(float));
    if (!rc) rc = sf_dev_reserve_zero(c, (void**)&c->d_hand2, &c->cap_hand2,
                                      (size_t)NG * 4 * nstrips * c->batch_maxcols * 2 * sizeof(unsigned long long));
    if (!rc) rc = sf_dev_reserve(c, (void**)&c->d_lam_init, &c->cap_lam_init, (size_t)ns * 9 * sizeof(float));
    const size_t nctr = (size_t)NG;
    if (!rc) rc = sf_dev_reserve(c, (void**)&c->d_ctr2, &c->cap_ctr2, nctr * sizeof(unsigned));
    if (rc) return rc;
    rc = prepare_gather(c, st);
    if (!rc) rc = prepare_seed(c, st);
    if (rc) return rc;
    AdjParams& p = A->p;
    std::memset(&p, 0, sizeof(p));
    p.nzz = c->nzz;
    p.nxx = c->nxx;
    p.nb = c->nb;
    p.dx = c->dx;
    p.dz = c->dz;
    p.shots = c->d_shots;
    p.nshots = ns;
    p.nstrips = nstrips;
    p.G = G;
    p.NG = NG;
    p.maxcols = c->batch_maxcols;
    p.lam = c->d_lam;
    p.lam_per_gang = (long long)c->nzz * c->batch_maxcols;
    p.hand = c->d_hand2;
    p.bar = c->d_ctr2;
    p.tcode = c->d_tcode;
    p.tc1 = c->d_tc1;
    p.tc2 = c->d_tc2;
    p.rx = c->d_rx;
    p.rz = c->d_rz;
    p.nrec = c->batch_nrec;
    p.lam_init = c->d_lam_init;
    p.err = c->d_flags + 1;
    p.wait_ns = c->wait_ns;
    {
        const int nn = c->seed_nodes, ne = c->seed_entries;
        p.nseed = nn;
        p.seed_ptr = c->d_seed_i;
        p.seed_row = c->d_seed_i + nn + 1;
        p.seed_col = c->d_seed_i + 2 * nn + 1;
        p.seed_rec = c->d_seed_i + 3 * nn + 1;
        p.rec_jg = c->d_seed_i + 3 * nn + 1 + ne;
        p.seed_w = c->d_seed_w;
    }
    GatherParams& g = A->g;
    std::memset(&g, 0, sizeof(g));
    g.nzz = c->nzz;
    g.nxx = c->nxx;
    g.nb = c->nb;
    g.nstrips = nstrips;
    g.nshots = ns;
    g.dx = c->dx;
    g.dz = c->dz;
    g.blk_ptr = c->d_colptr;
    g.blk_shots = c->d_gshots;
    g.tcode = c->d_tcode;
    g.vrec = c->d_tc2;
    g.lam_init = c->d_lam_init;
    g.wait_ns = c->wait_ns;
    if (c->batch_ani) {
        const size_t npad = (size_t)c->nzz * c->nxx;
        rc = sf_dev_reserve(c, (void**)&c->d_gcij, &c->cap_gcij, 2 * npad * sizeof(float));
        if (rc) return rc;
        g.vfac = c->d_vfac;
        g.vfac_total = c->batch_q_cells;
        g.grad_c11 = c->d_gcij;
        g.grad_c13 = c->d_gcij + npad;
    }
    A->kern = akern;
    A->gkern = c->batch_ani ? (const void*)k_gather<true> : (const void*)k_gather<false>;
    A->grid = dim3(NG * G);
    A->block = dim3(c->warps * 32);
    A->smem = smem;
    A->nctr = nctr;
    A->hand_bytes = (size_t)NG * 4 * nstrips * c->batch_maxcols * 2 * sizeof(unsigned long long);
    A->ggrid = dim3((unsigned)(nstrips * ((c->nxx + kGT - 1) / kGT)));
    A->gblock = dim3(256);
    // The gather inside the reverse-sweep launch (isotropic batches, 2 or 4
    // warps per CTA) when the device holds every reverse-sweep CTA and at
    // least one gather CTA at once.
    A->fused = false;
    if (c->fuse_gather && !c->batch_ani && (c->warps == 2 || c->warps == 4)) {
        const bool in = c->batch_interior;
        const void* fk = (c->warps == 2) ? (in ? (const void*)k_adjoint_gather<true, 2> : (const void*)k_adjoint_gather<false, 2>)
                                         : (in ? (const void*)k_adjoint_gather<true, 4> : (const void*)k_adjoint_gather<false, 4>);
        const size_t fsmem = std::max(smem, sizeof(GatherSmem));
        int per_sm = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fk, c->warps * 32, fsmem));
        const long long cap = (long long)per_sm * c->sms, nadj = (long long)NG * G;
        const int nblk = (c->nxx + kGT - 1) / kGT, ntiles = nstrips * nblk;
        const long long nga = std::min<long long>(cap - nadj, ntiles);
        if (nga >= 1) {
            const size_t nz = (size_t)ntiles + 1 + (size_t)ns;  // ready counters, tile counter, shot flags
            rc = sf_dev_reserve(c, (void**)&c->d_fuse, &c->cap_fuse, nz * sizeof(unsigned));
            if (rc) return rc;
            A->fused = true;
            A->fkern = fk;
            A->fsmem = fsmem;
            A->fgrid = dim3((unsigned)(nadj + nga));
            A->fzero_bytes = nz * sizeof(unsigned);
            A->f.nadj = (int)nadj;
            A->f.nblk = nblk;
            A->f.ready = c->d_fuse;
            A->f.tile_ctr = c->d_fuse + ntiles;
            A->f.shot_done = c->d_fuse + ntiles + 1;
            A->f.done_tag = 1u;
            g.shot_done = A->f.shot_done;
            g.done_tag = 1u;
            g.err = c->d_flags + 1;
        }
    }
    return SF_OK;
}

int sf_adj_enqueue(sf_ctx* c, AdjLaunch& A, const float* d_pg, float* d_grad, unsigned epoch, cudaStream_t st)
{
    A.p.pick_grad = d_pg;
    A.p.epoch = epoch;
    A.g.grad = d_grad;
    CK(cudaMemsetAsync(A.p.bar, 0, A.nctr * sizeof(unsigned), st));
    if (c->hand_stale_a) {  // the epoch wrapped (sf_next_epoch)
        CK(cudaMemsetAsync(c->d_hand2, 0, c->cap_hand2, st));
        c->hand_stale_a = false;
    }
    c->last_fused = A.fused;
    if (A.fused) {
        // one launch: the gather's tiles start as the last reverse sweep finishes them
        CK(cudaMemsetAsync(A.f.ready, 0, A.fzero_bytes, st));
        int rc = sf_kt_begin(c, SF_KT_ADJOINT, st);
        if (rc) return rc;
        void* fargs[] = {&A.p, &A.g, &A.f};
        CK(cudaLaunchKernel(A.fkern, A.fgrid, A.block, fargs, A.fsmem, st));
        return sf_kt_end(c, SF_KT_ADJOINT, st);
    }
    int rc = sf_kt_begin(c, SF_KT_ADJOINT, st);
    if (rc) return rc;
    void* args[] = {&A.p};
    CK(cudaLaunchKernel(A.kern, A.grid, A.block, args, A.smem, st));
    rc = sf_kt_end(c, SF_KT_ADJOINT, st);
    if (!rc) rc = sf_kt_begin(c, SF_KT_GATHER, st);
    if (rc) return rc;
    void* gargs[] = {&A.g};
    CK(cudaLaunchKernel(A.gkern, A.ggrid, A.gblock, gargs, sizeof(GatherSmem), st));
    return sf_kt_end(c, SF_KT_GATHER, st);
}

int sf_residual_enqueue(sf_ctx* c, const float* d_picks, const float* d_obs, float* d_pg, double* d_misfit,
                        cudaStream_t st)
{
    const size_t npk = (size_t)c->batch_nshots * c->batch_nrec;
    int rc = sf_kt_begin(c, SF_KT_RESIDUAL, st);
    if (rc) return rc;
    k_residual<<<1, 1024, 0, st>>>(d_picks, d_obs, npk, d_pg, d_misfit);
    CK(cudaGetLastError());
    return sf_kt_end(c, SF_KT_RESIDUAL, st);
}

// Runs the reverse sweeps and the gather for pick gradients already on the
// device (d_pg, nshots x nrec, caller order); grad is a device pointer.
int sf_adjoint_device(sf_ctx* c, const float* d_pg, float* d_grad, cudaStream_t st)
{
    AdjLaunch A;
    int rc = sf_adj_configure(c, st, &A);
    if (!rc) rc = sf_adj_enqueue(c, A, d_pg, d_grad, sf_next_epoch(c), st);
    if (rc) return rc;
    c->tape_valid = false;  // the reverse sweeps overwrite the tape's c2 with their terms
    c->gcij_valid = c->batch_ani != 0;
    return SF_OK;
}

static int grad_target(sf_ctx* c, float* grad, int grad_mem, float** dg)
{
    if (grad_mem == SF_MEM_DEVICE) {
        *dg = grad;
        return SF_OK;
    }
    int rc = sf_dev_reserve(c, (void**)&c->d_gshot, &c->cap_gshot, (size_t)c->nzz * c->nxx * sizeof(float));
    *dg = c->d_gshot;
    return rc;
}

extern "C" int sf_batch_adjoint(sf_ctx* c, const float* pick_grad, int pg_mem, float* grad, int grad_mem,
                                void* stream)
{
    if (!c) return SF_ERR_ARG;
    if (!c->tape_valid) return sf_fail(c, SF_ERR_STATE, "no taped forward batch to differentiate");
    if (!grad || (c->batch_nrec > 0 && !pick_grad)) return sf_fail(c, SF_ERR_ARG, "null argument");
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t npk = (size_t)c->batch_nshots * c->batch_nrec;
    const float* d_pg = pick_grad;
    int rc;
    if (pg_mem == SF_MEM_HOST) {
        rc = sf_dev_reserve(c, (void**)&c->d_pg, &c->cap_pg, std::max<size_t>(npk, 1) * sizeof(float));
        if (rc) return rc;
        CK(cudaMemcpyAsync(c->d_pg, pick_grad, npk * sizeof(float), cudaMemcpyHostToDevice, st));
        d_pg = c->d_pg;
    }
    float* dg;
    rc = grad_target(c, grad, grad_mem, &dg);
    if (rc) return rc;
    rc = sf_adjoint_device(c, d_pg, dg, st);
    if (rc) return rc;
    if (grad_mem == SF_MEM_HOST) {
        CK(cudaMemcpyAsync(grad, dg, (size_t)c->nzz * c->nxx * sizeof(float), cudaMemcpyDeviceToHost, st));
        return sf_check_flags(c, st);
    }
    return SF_OK;
}

extern "C" int sf_batch_misfit_gradient(sf_ctx* c, const float* t_obs, int obs_mem, double* misfit, float* grad,
                                        int grad_mem, void* stream)
{
    if (!c) return SF_ERR_ARG;
    if (!c->tape_valid) return sf_fail(c, SF_ERR_STATE, "no taped forward batch to differentiate");
    if (!t_obs || !grad) return sf_fail(c, SF_ERR_ARG, "null argument");
    if (!c->batch_picks) return sf_fail(c, SF_ERR_STATE, "the taped batch computed no picks");
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t npk = (size_t)c->batch_nshots * c->batch_nrec;
    int rc = sf_dev_reserve(c, (void**)&c->d_pg, &c->cap_pg, std::max<size_t>(2 * npk, 2) * sizeof(float));
    if (!rc) rc = sf_dev_reserve(c, (void**)&c->d_misfit, &c->cap_misfit, sizeof(double));
    if (rc) return rc;
    const float* d_obs = t_obs;
    if (obs_mem == SF_MEM_HOST) {
        CK(cudaMemcpyAsync(c->d_pg + npk, t_obs, npk * sizeof(float), cudaMemcpyHostToDevice, st));
        d_obs = c->d_pg + npk;
    }
    rc = sf_residual_enqueue(c, c->batch_picks, d_obs, c->d_pg, c->d_misfit, st);
    if (rc) return rc;
    float* dg;
    rc = grad_target(c, grad, grad_mem, &dg);
    if (rc) return rc;
    rc = sf_adjoint_device(c, c->d_pg, dg, st);
    if (rc) return rc;
    if (misfit) CK(cudaMemcpyAsync(misfit, c->d_misfit, sizeof(double), cudaMemcpyDeviceToHost, st));
    if (grad_mem == SF_MEM_HOST)
        CK(cudaMemcpyAsync(grad, dg, (size_t)c->nzz * c->nxx * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (misfit || grad_mem == SF_MEM_HOST) return sf_check_flags(c, st);
    return SF_OK;
}

extern "C" int sf_batch_stiffness_gradient(sf_ctx* c, float* grad_c11, float* grad_c13, int mem, void* stream)
{
    if (!c) return SF_ERR_ARG;
    if (!c->gcij_valid) return sf_fail(c, SF_ERR_STATE, "no adjoint of an anisotropic taped batch");
    if (!grad_c11 || !grad_c13) return sf_fail(c, SF_ERR_ARG, "null argument");
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t npad = (size_t)c->nzz * c->nxx;
    const cudaMemcpyKind kind = (mem == SF_MEM_HOST) ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    CK(cudaMemcpyAsync(grad_c11, c->d_gcij, npad * sizeof(float), kind, st));
    CK(cudaMemcpyAsync(grad_c13, c->d_gcij + npad, npad * sizeof(float), kind, st));
    if (mem == SF_MEM_HOST) return sf_check_flags(c, st);
    return SF_OK;
}

extern "C" int sf_set_fused_gather(sf_ctx* c, int enable)
{
    if (!c) return SF_ERR_ARG;
    c->fuse_gather = enable != 0;
    c->plan_dirty = true;
    return SF_OK;
}

extern "C" int sf_get_fused_gather(const sf_ctx* c, int* enable, int* last_fused)
{
    if (!c) return SF_ERR_ARG;
    if (enable) *enable = c->fuse_gather ? 1 : 0;
    if (last_fused) *last_fused = c->last_fused ? 1 : 0;
    return SF_OK;
}
