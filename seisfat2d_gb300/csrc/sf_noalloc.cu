// Per-shot solve that allocates nothing (sf_time_propagation_noalloc).
//
// For callers that may not allocate device memory during a call: hosts that
// own all device memory through their own pool and forbid cudaMalloc/cudaFree
// inside plugin calls (both can synchronise the device and fragment the
// host's pool), or latency-critical loops that cannot afford an allocation.
// The caller passes the padded slowness and the output traveltimes; every
// other buffer the solve needs (the strip-handoff values, the launch's
// counters and error flag, the shot descriptor, the check of the fast
// division for the call's cell sizes) lives in one file-scope static device
// array of fixed size, which every GPU that loads this library holds until
// the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "sf_engine.h"

using namespace sf;

namespace {

// Scratch capacity: the tagged strip-handoff pairs of the four sweeps for
// grids with ceil(nzz/32) * nxx <= kNoAllocCells (4 x 8 bytes each: 8 MiB),
// plus a 256-byte header with the launch's error flag, barrier counter,
// epoch and shot descriptor.
constexpr size_t kNoAllocCells = 262144;
constexpr size_t kNoAllocHeader = 256;

struct NoAllocHeader {
    int err;           // in-kernel wait timeout flag (must start at 0)
    unsigned bar;      // gang barrier counter (must start at 0)
    unsigned epoch;    // handoff tag epoch of the last call (host copy below)
    int div_bad;       // k_verify_div: bit w set when divisor w failed (must start at 0)
    float divs[4];     // the four constant divisors (dx, dz, hyp, D) being verified
    float rdivs[4];    // their reciprocals, written by k_verify_div
    ShotDev shot;      // the one shot of the call
};
static_assert(sizeof(NoAllocHeader) <= 256, "header too large");

// Shared by every call on a device; keeps the last call's contents.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocHeader + 4 * kNoAllocCells * sizeof(unsigned long long)];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_addr[kMaxDevices] = {};  // device address of the array, per device
unsigned g_epoch[kMaxDevices] = {};               // handoff tag epoch per device
int g_sms[kMaxDevices] = {};                      // multiprocessors per device
// the cell sizes whose divisors were last verified on each device, and the result
float g_vdx[kMaxDevices] = {}, g_vdz[kMaxDevices] = {};
float g_rdiv[kMaxDevices][4] = {};
int g_mflags[kMaxDevices] = {};
bool g_verified[kMaxDevices] = {};

// Once per device, with that device current: the device address of the
// scratch array (host code only knows a stand-in for the symbol) and the
// kernel's shared-memory limit.
int noalloc_setup(int dev, unsigned char** addr)
{
    if (dev < 0 || dev >= kMaxDevices) return SF_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return SF_ERR_CUDA;
        if (cudaFuncSetAttribute(sf_kshots_kernel(false, true, true, false), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sf_fwd_smem_bytes(kMaxWarps, false, false)) != cudaSuccess)
            return SF_ERR_CUDA;
        // the tagged pairs must not start with a valid-looking tag
        if (cudaMemset(p, 0, sizeof(g_noalloc_scratch)) != cudaSuccess) return SF_ERR_CUDA;
        if (cudaDeviceSynchronize() != cudaSuccess) return SF_ERR_CUDA;
        if (cudaDeviceGetAttribute(&g_sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return SF_ERR_CUDA;
        g_scratch_addr[dev] = static_cast<unsigned char*>(p);
    }
    *addr = g_scratch_addr[dev];
    return SF_OK;
}

}  // namespace

extern "C" int sf_time_propagation_noalloc(const float* S, int nx, int nz, float dx, float dz, float sx, float sz,
                                           float* T, void* stream)
{
    if (!S || !T || nx < 2 || nz < 2 || !(dx > 0.0f) || !(dz > 0.0f)) return SF_ERR_ARG;
    const int nb = 3, nxx = nx + 2 * nb, nzz = nz + 2 * nb;
    const size_t nstrips = (size_t)(nzz + 31) / 32;
    if (nstrips * (size_t)nxx > kNoAllocCells) return SF_ERR_RANGE;  // grid beyond the scratch capacity
    // source node (modeling.cu:112-113)
    const float fx = (sx + 0.5f * dx) / dx, fz = (sz + 0.5f * dz) / dz;
    if (!(fx > -1e9f && fx < 1e9f && fz > -1e9f && fz < 1e9f)) return SF_ERR_RANGE;
    ShotDev sh{};
    sh.c0 = 0;
    sh.ncols = nxx;
    sh.sIdx = (int)fx + nb;
    sh.sIdz = (int)fz + nb;
    sh.sx = sx;
    sh.sz = sz;
    if (sh.sIdz < 1 || sh.sIdz > nzz - 2 || sh.sIdx < 1 || sh.sIdx > nxx - 2) return SF_ERR_RANGE;
    sf_skip_cells(nxx, nzz, sh.skip_i, sh.skip_j);
    sh.orig = 0;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SF_ERR_CUDA;
    unsigned char* base = nullptr;
    int rc = noalloc_setup(dev, &base);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned epoch;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        g_epoch[dev] = (g_epoch[dev] % ((1u << 22) - 1)) + 1;
        epoch = g_epoch[dev];
    }
    Consts k;
    k.dx = dx;
    k.dz = dz;
    k.dz2i = 1.0f / (dz * dz);
    k.dx2i = 1.0f / (dx * dx);
    k.hyp = sqrtf(dx * dx + dz * dz);
    k.D = k.dz2i + k.dx2i;
    k.K = k.dz2i * k.dx2i;
    k.kA = k.dz2i - k.dx2i;
    k.kB = k.dx2i - k.dz2i;
    k.k2K = 2.0f * k.K;
    NoAllocHeader hdr{};
    hdr.shot = sh;  // err, the barrier counter and the division check start at zero
    hdr.epoch = epoch;
    hdr.divs[0] = k.dx;
    hdr.divs[1] = k.dz;
    hdr.divs[2] = k.hyp;
    hdr.divs[3] = k.D;
    if (cudaMemcpyAsync(base, &hdr, sizeof(hdr), cudaMemcpyHostToDevice, st) != cudaSuccess) return SF_ERR_CUDA;
    NoAllocHeader* dh = reinterpret_cast<NoAllocHeader*>(base);
    // a wrapped epoch could meet pairs an earlier cycle of calls left with the
    // same tag: clear the handoff region first (every 2^22 - 1 calls)
    if (epoch == 1 &&
        cudaMemsetAsync(base + kNoAllocHeader, 0, sizeof(g_noalloc_scratch) - kNoAllocHeader, st) != cudaSuccess)
        return SF_ERR_CUDA;
    // the fast division of the node update, checked once per device and cell
    // sizes against IEEE division (as a context does at creation); blocks with
    // an unverified divisor would run twice
    bool have = false;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (g_verified[dev] && g_vdx[dev] == dx && g_vdz[dev] == dz) {
            k.rdx = g_rdiv[dev][0];
            k.rdz = g_rdiv[dev][1];
            k.rhyp = g_rdiv[dev][2];
            k.rD = g_rdiv[dev][3];
            k.mflags = g_mflags[dev];
            have = true;
        }
    }
    if (!have) {
        k_verify_div<<<g_sms[dev] * 8, 256, 0, st>>>(dh->divs, 4, dh->rdivs, &dh->div_bad);
        if (cudaGetLastError() != cudaSuccess) return SF_ERR_CUDA;
        float rd[4];
        int bad = 0;
        if (cudaMemcpyAsync(rd, dh->rdivs, sizeof(rd), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(&bad, &dh->div_bad, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return SF_ERR_CUDA;
        k.rdx = rd[0];
        k.rdz = rd[1];
        k.rhyp = rd[2];
        k.rD = rd[3];
        k.mflags = (~bad) & 0xf;
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        g_vdx[dev] = dx;
        g_vdz[dev] = dz;
        for (int q = 0; q < 4; q++) g_rdiv[dev][q] = rd[q];
        g_mflags[dev] = k.mflags;
        g_verified[dev] = true;
    }
    FwdParams p{};
    p.S = S;
    p.nzz = nzz;
    p.nxx = nxx;
    p.nb = nb;
    p.kc = k;
    p.shots = &dh->shot;
    p.nshots = 1;
    p.G = 1;  // one CTA of 8 warps solves the shot
    p.NG = 1;
    p.maxcols = nxx;
    p.Tpool = T;
    p.t_per_gang = 0;
    p.err = &dh->err;
    p.hand = reinterpret_cast<unsigned long long*>(base + kNoAllocHeader);
    p.bar = &dh->bar;
    p.epoch = epoch;
    const int warps = 8;
    void* args[] = {&p};
    if (cudaLaunchKernel(sf_kshots_kernel(false, true, true, false), dim3(1), dim3(warps * 32), args,
                         sf_fwd_smem_bytes(warps, false, false), st) != cudaSuccess)
        return SF_ERR_CUDA;
    int err = 0;
    if (cudaMemcpyAsync(&err, &dh->err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return SF_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return SF_ERR_CUDA;
    return err ? SF_ERR_TIMEOUT : SF_OK;
}
