// Planned batches (sf_plan_*): a fixed set of shots and receivers whose
// forward + adjoint iteration enqueues device work only, so that it can run
// eagerly or be replayed from a CUDA graph; the launch-shape autotuner; and
// per-kernel timing with CUDA events.
//
// A graph replays its kernels with the handoff-tag epoch of the capture, so a
// consumer could take a pair left by the previous replay for one of this
// replay's. A planned iteration therefore zeroes the handoff pairs of both
// persistent kernels before launching them (32 B per gang, strip and column
// for the forward, 64 B for the adjoint: 0.2 GB for 100 gangs on a 1707 x 357
// grid, a few tens of microseconds), which makes it safe to replay from any
// graph, the context's own or one the caller captured.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "sf_engine.h"

using namespace sf;

#define CK(call)                                                          \
    do {                                                                  \
        int _st = sf_cuda_check(c, (call), #call);                        \
        if (_st != SF_OK) return _st;                                     \
    } while (0)

static void graph_release(sf_ctx* c)
{
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    if (c->graph) cudaGraphDestroy(c->graph);
    c->graph_exec = nullptr;
    c->graph = nullptr;
}

void sf_plan_release(sf_ctx* c)
{
    graph_release(c);
    if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
    c->cap_stream = nullptr;
    for (int k = 0; k < SF_KT_N; k++)
        for (int e = 0; e < 2; e++)
            if (c->kt_ev[k][e]) cudaEventDestroy(c->kt_ev[k][e]);
}

// ------------------------------------------------------------ kernel timing

extern "C" int sf_set_kernel_timing(sf_ctx* c, int enable)
{
    if (!c) return SF_ERR_ARG;
    CK(cudaSetDevice(c->dev));
    if (enable && !c->kt_ev[0][0])
        for (int k = 0; k < SF_KT_N; k++)
            for (int e = 0; e < 2; e++) CK(cudaEventCreate(&c->kt_ev[k][e]));
    c->timing = enable != 0;
    std::fill(c->kt_rec, c->kt_rec + SF_KT_N, false);
    return SF_OK;
}

extern "C" int sf_kernel_times(sf_ctx* c, float* ms, int n)
{
    if (!c || !ms || n < 0) return SF_ERR_ARG;
    CK(cudaSetDevice(c->dev));
    for (int k = 0; k < n; k++) {
        ms[k] = -1.0f;
        if (k >= SF_KT_N || !c->kt_rec[k]) continue;
        CK(cudaEventSynchronize(c->kt_ev[k][1]));
        CK(cudaEventElapsedTime(&ms[k], c->kt_ev[k][0], c->kt_ev[k][1]));
    }
    std::fill(c->kt_rec, c->kt_rec + SF_KT_N, false);
    return SF_OK;
}

// ------------------------------------------------------------------ plans

static int plan_configure(sf_ctx* c, cudaStream_t st)
{
    int rc = sf_fwd_configure(c, c->plan_nrec, false, true, c->gang_warps, st, &c->plan_f, nullptr);
    if (!rc) rc = sf_adj_configure(c, st, &c->plan_a);
    if (rc) {
        c->plan_valid = false;
        return rc;
    }
    c->plan_gen++;
    c->plan_dirty = false;
    return SF_OK;
}

extern "C" int sf_plan_batch(sf_ctx* c, const sf_shot* shots, int nshots, const float* rx, const float* rz,
                             int nrec, void* stream)
{
    if (!c || !shots || nshots <= 0 || nrec <= 0 || !rx || !rz)
        return sf_fail(c, SF_ERR_ARG, "bad plan arguments");
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    c->tape_valid = false;
    c->tables_valid = false;
    c->batch_ani = 0;
    int rc = sf_prepare_shots(c, shots, nshots, true);
    if (!rc) rc = sf_upload_receivers(c, rx, rz, nrec, st);
    if (rc) return rc;
    c->batch_nshots = nshots;
    c->batch_nrec = nrec;
    c->plan_nrec = nrec;
    const size_t npk = (size_t)nshots * nrec;
    rc = sf_dev_reserve(c, (void**)&c->d_pg, &c->cap_pg, std::max<size_t>(2 * npk, 2) * sizeof(float));
    if (!rc) rc = sf_dev_reserve(c, (void**)&c->d_misfit, &c->cap_misfit, sizeof(double));
    if (!rc) rc = plan_configure(c, st);
    if (rc) return rc;
    CK(cudaStreamSynchronize(st));  // uploads read host tables that later calls replace
    c->plan_valid = true;
    return SF_OK;
}

static int plan_check(sf_ctx* c, const float* t_obs, float* picks, float* grad)
{
    if (!c) return SF_ERR_ARG;
    if (!c->plan_valid) return sf_fail(c, SF_ERR_STATE, "no planned batch (sf_plan_batch)");
    if (!picks || (t_obs && !grad)) return sf_fail(c, SF_ERR_ARG, "null argument");
    return SF_OK;
}

static int plan_enqueue(sf_ctx* c, const float* t_obs, float* picks, double* misfit, float* grad, unsigned ef,
                        unsigned ea, cudaStream_t st)
{
    CK(cudaMemsetAsync(c->plan_f.p.hand, 0, c->plan_f.hand_bytes, st));
    int rc = sf_fwd_enqueue(c, c->plan_f, picks, ef, st);
    if (rc || !t_obs) return rc;
    rc = sf_residual_enqueue(c, picks, t_obs, c->d_pg, misfit ? misfit : c->d_misfit, st);
    if (rc) return rc;
    CK(cudaMemsetAsync(c->plan_a.p.hand, 0, c->plan_a.hand_bytes, st));
    return sf_adj_enqueue(c, c->plan_a, c->d_pg, grad, ea, st);
}

static void plan_done(sf_ctx* c, const float* t_obs, float* picks)
{
    c->batch_picks = picks;
    c->batch_nshots = (int)c->hshots.size();
    c->batch_nrec = c->plan_nrec;
    c->tape_valid = (t_obs == nullptr);  // the reverse sweeps consume the tape
    c->batch_ani = 0;
    c->gcij_valid = false;
}

extern "C" int sf_plan_iteration(sf_ctx* c, const float* t_obs, float* picks, double* misfit, float* grad,
                                 void* stream)
{
    int rc = plan_check(c, t_obs, picks, grad);
    if (rc) return rc;
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    if (c->plan_dirty) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        CK(cudaStreamIsCapturing(st, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            return sf_fail(c, SF_ERR_STATE, "launch shape changed: run the plan once before capturing it");
        rc = plan_configure(c, st);
        if (rc) return rc;
    }
    const unsigned ef = sf_next_epoch(c), ea = sf_next_epoch(c);
    rc = plan_enqueue(c, t_obs, picks, misfit, grad, ef, ea, st);
    if (rc) return rc;
    plan_done(c, t_obs, picks);
    return SF_OK;
}

static int graph_capture(sf_ctx* c, const float* t_obs, float* picks, double* misfit, float* grad)
{
    graph_release(c);
    if (!c->cap_stream) CK(cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking));
    const bool timing = c->timing;
    c->timing = false;  // no event records inside the graph
    CK(cudaStreamBeginCapture(c->cap_stream, cudaStreamCaptureModeThreadLocal));
    int rc = plan_enqueue(c, t_obs, picks, misfit, grad, 1, 1, c->cap_stream);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->cap_stream, &g);
    c->timing = timing;
    if (rc || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return rc ? rc : sf_cuda_check(c, e, "cudaStreamEndCapture");
    }
    c->graph = g;
    CK(cudaGraphInstantiate(&c->graph_exec, c->graph, 0));
    c->graph_gen = c->plan_gen;
    c->graph_ptrs[0] = t_obs;
    c->graph_ptrs[1] = picks;
    c->graph_ptrs[2] = misfit;
    c->graph_ptrs[3] = grad;
    return SF_OK;
}

extern "C" int sf_plan_graph_launch(sf_ctx* c, const float* t_obs, float* picks, double* misfit, float* grad,
                                    void* stream)
{
    int rc = plan_check(c, t_obs, picks, grad);
    if (rc) return rc;
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    if (c->plan_dirty) {
        rc = plan_configure(c, st);
        if (rc) return rc;
    }
    const void* ptrs[4] = {t_obs, picks, misfit, grad};
    if (!c->graph_exec || c->graph_gen != c->plan_gen || std::memcmp(ptrs, c->graph_ptrs, sizeof(ptrs)) != 0) {
        rc = graph_capture(c, t_obs, picks, misfit, grad);
        if (rc) return rc;
    }
    CK(cudaGraphLaunch(c->graph_exec, st));
    plan_done(c, t_obs, picks);
    return SF_OK;
}

// Times `reps` planned iterations for each candidate launch shape (warps per
// CTA x warps per shot) and keeps the fastest. Every shape computes the same
// bits; only the schedule of strips on warps and SMs differs.
extern "C" int sf_plan_autotune(sf_ctx* c, const float* t_obs, float* picks, double* misfit, float* grad,
                                int reps, void* stream, int* best_warps, int* best_gang, float* best_ms)
{
    int rc = plan_check(c, t_obs, picks, grad);
    if (rc) return rc;
    if (reps < 1) return sf_fail(c, SF_ERR_ARG, "reps must be >= 1");
    CK(cudaSetDevice(c->dev));
    cudaStream_t st = (cudaStream_t)stream;
    const int nstrips = (c->nzz + 31) / 32;
    std::vector<int> gangs = {0, nstrips};
    for (int d = 2; d <= 4; d++)
        if ((nstrips + d - 1) / d >= 1) gangs.push_back((nstrips + d - 1) / d);
    std::sort(gangs.begin(), gangs.end());
    gangs.erase(std::unique(gangs.begin(), gangs.end()), gangs.end());
    const int warps_c[] = {1, 2, 4};
    const int w0 = c->warps, g0 = c->gang_warps, l0 = c->strip_loop;
    // both strip-loop forms unless the caller fixed one
    std::vector<int> loops;
    if (l0 == SF_LOOP_AUTO) loops = {SF_LOOP_GENERAL, SF_LOOP_INTERIOR};
    else loops = {l0};
    int bw = w0, bg = g0, bl = l0;
    float bms = -1.0f;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    for (int lp : loops)
    for (int w : warps_c) {
        for (int g : gangs) {
            c->warps = w;
            c->gang_warps = g;
            c->strip_loop = lp;
            rc = plan_configure(c, st);
            if (!rc) rc = plan_enqueue(c, t_obs, picks, misfit, grad, sf_next_epoch(c), sf_next_epoch(c), st);
            if (!rc) rc = sf_cuda_check(c, cudaEventRecord(e0, st), "cudaEventRecord");
            for (int r = 0; r < reps && !rc; r++)
                rc = plan_enqueue(c, t_obs, picks, misfit, grad, sf_next_epoch(c), sf_next_epoch(c), st);
            if (!rc) rc = sf_cuda_check(c, cudaEventRecord(e1, st), "cudaEventRecord");
            if (!rc) rc = sf_cuda_check(c, cudaEventSynchronize(e1), "cudaEventSynchronize");
            float ms = 0.0f;
            if (!rc) rc = sf_cuda_check(c, cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
            if (!rc) rc = sf_check_flags(c, st);
            if (rc) break;
            ms /= reps;
            if (bms < 0.0f || ms < bms) {
                bms = ms;
                bw = w;
                bg = g;
                bl = lp;
            }
        }
        if (rc) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->warps = rc ? w0 : bw;
    c->gang_warps = rc ? g0 : bg;
    c->strip_loop = rc ? l0 : bl;
    int rc2 = plan_configure(c, st);
    if (rc) return rc;
    if (rc2) return rc2;
    plan_done(c, t_obs, picks);
    if (best_warps) *best_warps = bw;
    if (best_gang) *best_gang = bg;
    if (best_ms) *best_ms = bms;
    return SF_OK;
}
