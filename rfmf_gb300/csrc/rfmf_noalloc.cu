// rfmf_noalloc.cu -- rfmf_anneal_noalloc: the annealing kernel with all of
// its scratch in a fixed, file-scope device array, for callers that cannot
// allocate device memory.
//
// Who needs this: hosts that own every byte of device memory themselves (a
// framework allocator or memory pool that forbids third-party cudaMalloc),
// code that must not allocate in the middle of its own work (allocation
// synchronises the device and can fail at the worst moment), and embedders
// that hand the library pre-sized buffers only.  Such a caller passes its
// inputs and outputs as device buffers; everything else the kernel needs
// (chain records, work items, the work-queue head and the error word) lives
// in g_noallocScratch below, which every GPU that loads this library holds
// until the process exits.
//
// Set-up: the first call on a device, with that device current, looks up
// the array's device address (cudaGetSymbolAddress) and caches it; make that
// first call before any stream capture.  The array is shared by every call
// and keeps the last call's contents; each call rewrites the records and
// clears the queue head and error word before its launch.  Calls whose
// launches overlap on the GPU (different streams, or different host threads
// on one device) race on the array: serialise them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/rfmf.h"
#include "rfmf_device.h"

namespace rfmf {
int set_last_error(int code, const char* msg);
const void* kernel_ptr(int dbytes, int fmt, bool s64);
cudaError_t launch_anneal(const DevLaunch& L, int dbytes, int fmt, bool s64, int grid,
                          int threads, size_t smem, cudaStream_t stream);
}  // namespace rfmf

using namespace rfmf;

namespace {

// Fixed limits of the no-allocation path.
constexpr int64_t kNoAllocMaxChains = 4096;
constexpr int64_t kNoAllocMaxPhases = 64;

// Scratch layout (bytes): control words, one graph record, one schedule,
// phases, chain records, work items, work order.
constexpr size_t kOffCtl = 0;                                    // queue, error, errorItem
constexpr size_t kOffGraph = 256;
constexpr size_t kOffSched = kOffGraph + 256;
constexpr size_t kOffPhaseP = kOffSched + 256;
constexpr size_t kOffPhaseIters = kOffPhaseP + kNoAllocMaxPhases * sizeof(uint32_t);
constexpr size_t kOffChains = (kOffPhaseIters + kNoAllocMaxPhases * sizeof(uint64_t) + 255) & ~size_t(255);
constexpr size_t kOffItems = (kOffChains + kNoAllocMaxChains * sizeof(DevChain) + 255) & ~size_t(255);
constexpr size_t kOffOrder = (kOffItems + kNoAllocMaxChains * sizeof(DevItem) + 255) & ~size_t(255);
constexpr size_t kNoAllocScratchBytes =
    (kOffOrder + kNoAllocMaxChains * sizeof(int32_t) + 255) & ~size_t(255);
static_assert(sizeof(DevGraph) <= 256 && sizeof(DevSchedule) <= 256, "record slots too small");
static_assert(kNoAllocScratchBytes <= 640 * 1024, "no-alloc scratch larger than stated");

// The scratch itself: file-scope, statically sized, one per device.
static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocScratchBytes];

// Reports through rfmf_last_error() like every other entry point.
int nerr(int code, const char* msg) { return set_last_error(code, msg); }

// Per-device cache of the array's device address (host code may not use the
// symbol's name as an address).
std::mutex g_mu;
std::vector<unsigned char*> g_scratchAddr;

int scratch_address(int device, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (static_cast<int>(g_scratchAddr.size()) <= device) g_scratchAddr.resize(device + 1, nullptr);
    if (!g_scratchAddr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess || !p) return nerr(RFMF_ERR_CUDA, cudaGetErrorString(e));
        g_scratchAddr[device] = static_cast<unsigned char*>(p);
    }
    *out = g_scratchAddr[device];
    return RFMF_OK;
}

}  // namespace

namespace {

// One-block reduction of the weight column of the 8-byte entries into *out
// (the sum of weights over directed entries), used by the set-up below.
__global__ void wsum_kernel(const int32_t* edges, int64_t m2, int64_t* out) {
    __shared__ long long part[32];
    long long acc = 0;
    for (int64_t i = threadIdx.x; i < m2; i += blockDim.x) acc += edges[2 * i + 1];
    for (int m = 16; m > 0; m >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, m);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) t += part[w];
        *out = t;
    }
}
cudaError_t noalloc_wsum(const int32_t* edges, int64_t m2, int64_t* out, cudaStream_t stream) {
    wsum_kernel<<<1, 1024, 0, stream>>>(edges, m2, out);
    return cudaGetLastError();
}

}  // namespace

static int rfmf_anneal_noalloc_impl(int device, void* stream, int64_t n,
                                   const uint32_t* d_offsets, const int32_t* d_edges,
                                   int64_t max_weighted_deg, int64_t C, const double* t0s,
                                   const uint64_t* solver_seeds, int64_t nphases,
                                   const uint64_t* phases, const uint64_t* iters,
                                   const int64_t* d_beta_end, const int32_t* d_beta_val,
                                   const int64_t* chain_beta_off, const int64_t* chain_beta_runs,
                                   uint32_t* d_spin_bits, uint32_t* d_best_bits,
                                   int64_t* d_cur, int64_t* d_best) {
    if (n <= 0 || n >= (int64_t(1) << 31)) return nerr(RFMF_ERR_INVALID, "n out of range");
    if (C <= 0 || C > kNoAllocMaxChains)
        return nerr(RFMF_ERR_CAPACITY, "no-alloc path: chains must be 1..4096");
    if (nphases < 0 || nphases > kNoAllocMaxPhases)
        return nerr(RFMF_ERR_CAPACITY, "no-alloc path: at most 64 phases");
    if (!d_offsets || !d_edges || !t0s || !solver_seeds || !d_beta_end || !d_beta_val ||
        !chain_beta_off || !chain_beta_runs || !d_spin_bits || !d_best_bits || !d_cur || !d_best ||
        (nphases && (!phases || !iters)))
        return nerr(RFMF_ERR_INVALID, "NULL argument");
    if (max_weighted_deg < 0 || max_weighted_deg > std::numeric_limits<int32_t>::max())
        return nerr(RFMF_ERR_INVALID, "max_weighted_deg out of range");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaSetDevice(device) != cudaSuccess) return nerr(RFMF_ERR_CUDA, "cudaSetDevice failed");
    unsigned char* base = nullptr;
    if (int rc = scratch_address(device, &base)) return rc;

    uint64_t total = 0, maxP = 1;
    for (int64_t p = 0; p < nphases; ++p) {
        if (phases[p] > 0x7FFFFFFFull) return nerr(RFMF_ERR_CAPACITY, "phase P too large");
        if (phases[p]) { total += iters[p]; maxP = std::max<uint64_t>(maxP, phases[p]); }
    }
    for (int64_t c = 0; c < C; ++c)
        if (!(t0s[c] > 0.0)) return nerr(RFMF_ERR_INVALID, "t0 must be > 0");

    // Launch plan: CSR walked in HBM (the caller's buffers), one warp per
    // chain, int8 gains when B <= 127, compact int32 keys when the range
    // allows (else the int64 score path), K chains per CTA from occupancy.
    const int W = 1, T = 32;
    const int dbytes = (max_weighted_deg <= 127) ? 1 : 4;
    int kb = 4;
    while ((int64_t(1) << kb) < ((n + 7) / 8 + T - 1) / T) ++kb;
    bool s64 = false;
    for (int64_t c = 0; c < C && !s64; ++c) {
        const double bmax = std::round(std::log(1.0 + static_cast<double>(std::max<uint64_t>(total, 1))) /
                                       t0s[c] * 1048576.0);
        if (!((bmax * static_cast<double>(max_weighted_deg) + 3617614.0) * std::ldexp(1.0, kb) <
              2147483647.0))
            s64 = true;
    }
    const int words = static_cast<int>((n + 31) / 32);
    const int pmax = static_cast<int>(std::min<uint64_t>(maxP, static_cast<uint64_t>(n)));
    const uint32_t chainBytes = chain_layout(static_cast<int>(n), words, pmax, W, dbytes).total;
    int dev = device, sms = 0, optin = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        return nerr(RFMF_ERR_CUDA, "device attribute query failed");
    const void* kern = kernel_ptr(dbytes, kCsrGlobal, s64);
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess) return nerr(RFMF_ERR_CUDA, "kernel attributes");
    const int dynMax = optin - static_cast<int>(fa.sharedSizeBytes);
    const int64_t room = static_cast<int64_t>(dynMax) - kSmemHeader;
    const int Kmax = static_cast<int>(
        std::min<int64_t>(std::min(16, fa.maxThreadsPerBlock / (32 * W)), room / chainBytes));
    if (Kmax < 1) return nerr(RFMF_ERR_CAPACITY, "chain state does not fit shared memory");
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, dynMax) != cudaSuccess)
        return nerr(RFMF_ERR_CUDA, "kernel attribute");
    int K = Kmax, occ = 0;
    for (int k = 1; k <= Kmax; ++k) {
        int o = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &o, kern, 32 * W * k, kSmemHeader + static_cast<size_t>(k) * chainBytes) != cudaSuccess ||
            o <= 0) {
            cudaGetLastError();
            continue;
        }
        K = k;
        occ = o;
        if ((C + k - 1) / k <= static_cast<int64_t>(o) * sms) break;
    }
    if (occ <= 0) return nerr(RFMF_ERR_CAPACITY, "no resident launch configuration");
    const int nitems = static_cast<int>((C + K - 1) / K);
    const size_t smem = kSmemHeader + static_cast<size_t>(K) * chainBytes;

    // Records into the scratch array (plain copies; nothing is allocated on
    // the device; the host staging below is ordinary host memory).
    DevGraph g{};
    g.offsets = d_offsets;
    g.edges = reinterpret_cast<const Edge*>(d_edges);
    g.compact = nullptr;
    g.n = static_cast<int32_t>(n);
    g.words = words;
    g.offBytes = 0;
    g.entBytes = 0;
    // wsum2 (sum of weights over directed entries) is not known without the
    // host CSR: chains start fresh, so the kernel's cut check is not used and
    // the cut is derived from D and wsum2 -- compute wsum2 on the device.
    DevSchedule sch{reinterpret_cast<const uint32_t*>(base + kOffPhaseP),
                    reinterpret_cast<const uint64_t*>(base + kOffPhaseIters),
                    static_cast<int32_t>(nphases), 0};
    std::vector<uint32_t> hp(kNoAllocMaxPhases, 0);
    std::vector<uint64_t> hi(kNoAllocMaxPhases, 0);
    for (int64_t p = 0; p < nphases; ++p) { hp[p] = static_cast<uint32_t>(phases[p]); hi[p] = iters[p]; }
    std::vector<DevChain> ch(C);
    for (int64_t c = 0; c < C; ++c) {
        DevChain& d = ch[c];
        d.graph = 0;
        d.sched = 0;
        d.solverSeed = solver_seeds[c];
        d.betaEnd = d_beta_end + chain_beta_off[c];
        d.betaVal = d_beta_val + chain_beta_off[c];
        d.betaRuns = chain_beta_runs[c];
        d.spinBits = d_spin_bits + c * words;
        d.bestBits = d_best_bits + c * words;
        d.cur = kUnsetCut;
        d.best = kUnsetCut;
        d.sweepsDone = 0;
        d.sweepsTotal = total;
        d.improvedSweeps = 0;
    }
    std::vector<DevItem> items(nitems);
    std::vector<int32_t> order(C);
    for (int64_t c = 0; c < C; ++c) order[c] = static_cast<int32_t>(c);
    for (int i = 0; i < nitems; ++i)
        items[i] = DevItem{0, static_cast<int32_t>(i * K),
                           static_cast<int32_t>(std::min<int64_t>(K, C - static_cast<int64_t>(i) * K)), 0};

    // wsum2 on the device: the sum of the weight column, reduced by a
    // one-block kernel into the graph record (no temporary buffers).
    cudaError_t e = cudaSuccess;
    auto cp = [&](size_t off, const void* src, size_t bytes) {
        if (e == cudaSuccess) e = cudaMemcpyAsync(base + off, src, bytes, cudaMemcpyHostToDevice, st);
    };
    cp(kOffSched, &sch, sizeof sch);
    cp(kOffPhaseP, hp.data(), hp.size() * sizeof(uint32_t));
    cp(kOffPhaseIters, hi.data(), hi.size() * sizeof(uint64_t));
    cp(kOffChains, ch.data(), C * sizeof(DevChain));
    cp(kOffItems, items.data(), nitems * sizeof(DevItem));
    cp(kOffOrder, order.data(), C * sizeof(int32_t));
    cp(kOffGraph, &g, sizeof g);
    // m2 from the device offsets array (one 4-byte read).
    uint32_t m2 = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&m2, d_offsets + n, sizeof m2, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess)
        e = noalloc_wsum(d_edges, m2, reinterpret_cast<int64_t*>(base + kOffGraph +
                                                                        offsetof(DevGraph, wsum2)), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(base + kOffCtl, 0, 16, st);
    if (e != cudaSuccess) return nerr(RFMF_ERR_CUDA, cudaGetErrorString(e));

    DevLaunch L{};
    L.graphs = reinterpret_cast<const DevGraph*>(base + kOffGraph);
    L.scheds = reinterpret_cast<const DevSchedule*>(base + kOffSched);
    L.chains = reinterpret_cast<DevChain*>(base + kOffChains);
    L.items = reinterpret_cast<const DevItem*>(base + kOffItems);
    L.order = reinterpret_cast<const int32_t*>(base + kOffOrder);
    L.nitems = nitems;
    L.ngraphs = 1;
    L.nscheds = 1;
    L.warpsPerChain = W;
    L.chainsPerCta = K;
    L.maxN = static_cast<int32_t>(n);
    L.maxWords = words;
    L.pmax = pmax;
    L.csrBytes = 0;
    L.chainBytes = chainBytes;
    L.queue = reinterpret_cast<int32_t*>(base + kOffCtl);
    L.error = reinterpret_cast<int32_t*>(base + kOffCtl) + 1;
    L.errorItem = reinterpret_cast<int32_t*>(base + kOffCtl) + 2;
    L.itemNs = nullptr;
    L.window = total;
    for (int i = 0; i < 16; ++i)
        L.lut[i] = static_cast<int32_t>(std::lround(-std::log(-std::log((2.0 * i + 1.0) / 32.0)) * 1048576.0));
    const int grid = static_cast<int>(std::min<int64_t>(nitems, static_cast<int64_t>(occ) * sms));
    e = launch_anneal(L, dbytes, kCsrGlobal, s64, grid, 32 * W * K, smem, st);
    // Cut values out: the int64 fields of the chain records, strided.
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(d_cur, sizeof(int64_t), base + kOffChains + offsetof(DevChain, cur),
                              sizeof(DevChain), sizeof(int64_t), C, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(d_best, sizeof(int64_t), base + kOffChains + offsetof(DevChain, best),
                              sizeof(DevChain), sizeof(int64_t), C, cudaMemcpyDeviceToDevice, st);
    int32_t ctl[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctl, base + kOffCtl, sizeof ctl, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return nerr(RFMF_ERR_CUDA, cudaGetErrorString(e));
    if (ctl[1] != kDevOk) return nerr(RFMF_ERR_DEVICE, "device-side error during the anneal");
    return RFMF_OK;
}

// C ABI entry points: no C++ exception crosses the boundary.
extern "C" int rfmf_anneal_noalloc(int device, void* stream, int64_t n,
                                   const uint32_t* d_offsets, const int32_t* d_edges,
                                   int64_t max_weighted_deg, int64_t C, const double* t0s,
                                   const uint64_t* solver_seeds, int64_t nphases,
                                   const uint64_t* phases, const uint64_t* iters,
                                   const int64_t* d_beta_end, const int32_t* d_beta_val,
                                   const int64_t* chain_beta_off, const int64_t* chain_beta_runs,
                                   uint32_t* d_spin_bits, uint32_t* d_best_bits,
                                   int64_t* d_cur, int64_t* d_best) {
    try {
        return rfmf_anneal_noalloc_impl(device, stream, n, d_offsets, d_edges, max_weighted_deg, C,
                                        t0s, solver_seeds, nphases, phases, iters, d_beta_end,
                                        d_beta_val, chain_beta_off, chain_beta_runs, d_spin_bits,
                                        d_best_bits, d_cur, d_best);
    } catch (const std::bad_alloc&) {
        return rfmf::set_last_error(RFMF_ERR_NOMEM, "host allocation failed in rfmf_anneal_noalloc");
    } catch (...) {
        return rfmf::set_last_error(RFMF_ERR_INVALID, "unexpected host exception in rfmf_anneal_noalloc");
    }
}
