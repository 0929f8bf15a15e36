// Internal state of an engine context (not part of the public ABI).
#pragma once
#include <array>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/seisfat2d.h"
#include "sf_adjoint_params.cuh"
#include "sf_forward.cuh"

// One configured launch of the batched forward: parameters fixed except the
// handoff-tag epoch and the picks pointer, which every enqueue sets.
struct FwdLaunch {
    sf::FwdParams p{};
    const void* kern = nullptr;  // the k_shots instantiation
    dim3 grid, block;
    size_t smem = 0;
    size_t nctr = 0;             // gang barrier counters zeroed before the launch
    size_t hand_bytes = 0;       // handoff pairs of the launch's gangs
};

// One configured adjoint (reverse sweeps + gather); the pick gradients, the
// gradient target and the epoch are set by every enqueue.
struct AdjLaunch {
    sf::AdjParams p{};
    sf::GatherParams g{};
    const void* kern = nullptr;   // k_adjoint
    const void* gkern = nullptr;  // k_gather (when not fused)
    dim3 grid, block, ggrid, gblock;
    size_t smem = 0;
    size_t nctr = 0;
    size_t hand_bytes = 0;
    // reverse sweeps and gather in one launch (k_adjoint_gather)
    bool fused = false;
    const void* fkern = nullptr;
    sf::FuseParams f{};
    dim3 fgrid;
    size_t fsmem = 0;
    size_t fzero_bytes = 0;  // counters zeroed before each launch (f.ready ...)
};

// Kernels timed by sf_kernel_times (events around each launch when enabled).
enum { SF_KT_FORWARD = 0, SF_KT_RESIDUAL = 1, SF_KT_ADJOINT = 2, SF_KT_GATHER = 3, SF_KT_N = 4 };

struct sf_ctx {
    int dev = 0;
    int nx = 0, nz = 0, nb = 3, nxx = 0, nzz = 0;
    float dx = 0.0f, dz = 0.0f;
    sf::Consts kc{};
    int sms = 1;
    int warps = 1;        // warps per CTA
    int gang_warps = 0;   // warps solving one shot (0: chosen per batch)
    int strip_loop = -1;  // strip loops: SF_LOOP_* (sf_set_strip_loop)
    bool fuse_gather = true;  // gather inside the reverse-sweep launch when it fits (sf_set_fused_gather)
    bool last_fused = false;  // the last adjoint ran fused
    unsigned* d_fuse = nullptr; size_t cap_fuse = 0;
    bool batch_interior = false;  // the last batch's forward ran the interior-block body
    int arith = SF_ARITH_REFERENCE;
    unsigned long long wait_ns = 0;  // limit of the in-kernel waits (0: default, about 2 s)
    bool stall_next = false;          // sf_test_stall_next_batch
    std::string err;

    float* d_S = nullptr;       // padded slowness
    int* d_flags = nullptr;     // [0] work counter, [1] error flag, [2..] adjoint counters
    float* d_model = nullptr;
    size_t cap_model = 0;
    uint16_t* d_cij_all = nullptr;  // six padded code fields
    size_t cap_cij = 0;
    float mm[12] = {};
    bool have_cij = false;

    // batch state
    std::vector<sf::ShotDev> hshots;  // sorted widest first
    std::unordered_map<int, std::array<int, 8>> skip_cache;  // window width -> skipped cells (sf_skip_cells)
    std::vector<int> tables_index;    // caller index -> hshots index
    long long batch_T_floats = 0, batch_tape_entries = 0;
    long long batch_q_cells = 0;      // window cells of all shots (qP derivative factors)
    int batch_maxcols = 0, batch_nshots = 0, batch_nrec = 0;
    int batch_ani = 0;                // the last batch solved the anisotropic two-pass scheme
    float* batch_picks = nullptr;
    bool tables_valid = false, tape_valid = false;
    std::vector<float> h_rx, h_rz;

    sf::ShotDev* d_shots = nullptr; size_t cap_shots = 0;
    float* d_T = nullptr; size_t cap_T = 0;
    float* d_Tl = nullptr; size_t cap_Tl = 0;  // lo parts of the traveltimes (compensated arithmetic)
    float* d_rx = nullptr; size_t cap_rx = 0;
    float* d_rz = nullptr; size_t cap_rz = 0;
    float* d_picks = nullptr; size_t cap_picks = 0;
    float* d_Sq = nullptr; size_t cap_Sq = 0;
    unsigned long long* d_hand = nullptr; size_t cap_hand = 0;
    unsigned* d_ctr = nullptr; size_t cap_ctr = 0;
    unsigned epoch = 0;  // launches so far (handoff tags)
    bool hand_stale_f = false, hand_stale_a = false;  // the epoch wrapped: clear the handoff buffers
    int last_G = 1, last_NG = 1;
    uint8_t* d_tcode = nullptr; size_t cap_tcode = 0;
    float* d_tc1 = nullptr; size_t cap_tc1 = 0;
    float* d_tc2 = nullptr; size_t cap_tc2 = 0;

    // adjoint state
    float* d_lam = nullptr; size_t cap_lam = 0;
    float* d_vrec = nullptr; size_t cap_vrec = 0;
    float* d_gshot = nullptr; size_t cap_gshot = 0;
    float* d_pg = nullptr; size_t cap_pg = 0;
    double* d_misfit = nullptr; size_t cap_misfit = 0;
    int* d_colptr = nullptr; size_t cap_colptr = 0;
    float* d_lam_init = nullptr; size_t cap_lam_init = 0;
    unsigned long long* d_hand2 = nullptr; size_t cap_hand2 = 0;
    unsigned* d_ctr2 = nullptr; size_t cap_ctr2 = 0;
    std::vector<int> h_colptr;
    sf::GatherShot* d_gshots = nullptr; size_t cap_gshots = 0;
    std::vector<sf::GatherShot> h_gshots;
    // adjoint seed table (receivers of the batch): seeded nodes, CSR of
    // their (receiver, weight) entries in receiver order
    int* d_seed_i = nullptr; size_t cap_seed_i = 0;    // [ptr nn+1][row nn][gcol nn][rec ne][rec_jg nrec]
    float* d_seed_w = nullptr; size_t cap_seed_w = 0;
    int seed_nodes = 0, seed_entries = 0;
    std::vector<int> h_seed_pack;
    std::vector<float> h_seed_w;
    // the gather's shot lists and the seed table are rebuilt only when the
    // batch's shots or receivers changed (generations of each)
    unsigned long long shots_gen = 1, recv_gen = 1;
    unsigned long long gather_gen = 0, seed_gen = 0;
    int seed_nrec = -1;

    // model update (sf_smooth_model, sf_update_slowness)
    float* d_skern = nullptr; size_t cap_skern = 0;
    float* d_upd = nullptr; size_t cap_upd = 0;
    std::vector<float> h_skern;

    // Kirchhoff migration (sf_kirchhoff_image, sf_adjoint_convolution)
    double* d_wav = nullptr; size_t cap_wav = 0;
    float* d_mig = nullptr; size_t cap_mig = 0;
    float* d_kgeo = nullptr; size_t cap_kgeo = 0;
    int* d_kint = nullptr; size_t cap_kint = 0;
    float* d_kpart = nullptr; size_t cap_kpart = 0;  // forward operator chunk partials

    // anisotropic adjoint: per-shot dSq/d{S, C11, C13} factors and the
    // stiffness gradients of the last adjoint (sf_batch_stiffness_gradient)
    float* d_vfac = nullptr; size_t cap_vfac = 0;
    float* d_gcij = nullptr; size_t cap_gcij = 0;
    bool gcij_valid = false;
    std::vector<int> h_kint;
    std::vector<double> h_wav;
    std::vector<float> h_kgeo;

    // per-kernel timing (sf_set_kernel_timing)
    bool timing = false;
    cudaEvent_t kt_ev[SF_KT_N][2] = {};
    bool kt_rec[SF_KT_N] = {};

    // planned batch (sf_plan_batch) and its CUDA graph
    bool plan_valid = false;
    bool plan_dirty = false;     // launch shape or arithmetic changed since configuring
    unsigned plan_gen = 0;        // bumped whenever the plan's launches change
    FwdLaunch plan_f;
    AdjLaunch plan_a;
    int plan_nrec = 0;
    cudaStream_t cap_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    unsigned graph_gen = 0;
    const void* graph_ptrs[4] = {};   // t_obs, picks, misfit, grad of the capture
};

int sf_fail(sf_ctx* c, int status, const std::string& msg);
int sf_cuda_check(sf_ctx* c, cudaError_t e, const char* what);
int sf_dev_reserve(sf_ctx* c, void** p, size_t* cap, size_t bytes);
// Same, zero-filled whenever it (re)allocates.
int sf_dev_reserve_zero(sf_ctx* c, void** p, size_t* cap, size_t bytes);
// Next handoff-tag epoch (never 0; wraps within 22 bits).
unsigned sf_next_epoch(sf_ctx* c);
int sf_check_flags(sf_ctx* c, cudaStream_t st);
int sf_fwd_setup(sf_ctx* c);
int sf_verify_divisors(sf_ctx* c);
size_t sf_fwd_smem_bytes(int warps, bool comp, bool tape);
// k_shots instantiation (one object file each, sf_shots_inst.cu)
const void* sf_kshots_kernel(bool tape, bool ref, bool interior, bool comp);
const void* sf_kqp_kernel(bool ref, bool comp, bool fact);
// whether the batch of hshots, G CTAs per shot, runs the interior-block body
bool sf_interior_loops(sf_ctx* c, const void* kernel, size_t smem, int G);
void sf_skip_cells(int ncols, int nzz, int si[4], int sj[4]);
int sf_prepare_shots(sf_ctx* c, const sf_shot* shots, int nshots, bool tape);
int sf_launch_shots(sf_ctx* c, int ani, int nrec, float* d_picks, bool keep_tables, bool tape, int gang_warps,
                    cudaStream_t st);
// The two halves of sf_launch_shots: configure (gang shape, buffers, shot
// table upload; host work and allocation) and enqueue (counter reset and the
// launch; stream work only, capturable).
int sf_fwd_configure(sf_ctx* c, int nrec, bool per_shot_T, bool tape, int gang_warps, cudaStream_t st,
                     FwdLaunch* L, const float* Sshots);
int sf_fwd_enqueue(sf_ctx* c, FwdLaunch& L, float* d_picks, unsigned epoch, cudaStream_t st);
int sf_fwd_launch(sf_ctx* c, FwdLaunch& L, float* d_picks, unsigned epoch, cudaStream_t st);
int sf_qp_launch(sf_ctx* c, bool fact, cudaStream_t st);
int sf_adj_configure(sf_ctx* c, cudaStream_t st, AdjLaunch* A);
int sf_adj_enqueue(sf_ctx* c, AdjLaunch& A, const float* d_pg, float* d_grad, unsigned epoch, cudaStream_t st);
int sf_residual_enqueue(sf_ctx* c, const float* d_picks, const float* d_obs, float* d_pg, double* d_misfit,
                        cudaStream_t st);
int sf_upload_receivers(sf_ctx* c, const float* rx, const float* rz, int nrec, cudaStream_t st);
// Event pair around one launch when kernel timing is on.
int sf_kt_begin(sf_ctx* c, int k, cudaStream_t st);
int sf_kt_end(sf_ctx* c, int k, cudaStream_t st);
void sf_plan_release(sf_ctx* c);
// Normalised Gaussian taps of the reference's smooth_matrix (n x n, x major).
void sf_smooth_kernel(float stdv, int n, std::vector<float>& k);
// The reference's Ricker-type wavelet of Migration::set_wavelet.
void sf_kirchhoff_wavelet(float fmax, float dt, std::vector<float>& w);
// Gang shape for nshots shots of nstrips strips: CTAs per gang and gangs, so
// that every gang of the grid is resident at once.
int sf_gang_shape(sf_ctx* c, const void* kernel, size_t smem, int nshots, int nstrips, int gang_warps, int* G,
                  int* NG);
void sf_adjoint_release(sf_ctx* c);
int sf_adj_setup(sf_ctx* c);
int sf_adjoint_device(sf_ctx* c, const float* d_pg, float* d_grad, cudaStream_t st);
