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
// (graph and schedule records, chain records, work items, the work-queue head
// and the error word) lives in g_noallocScratch below, a fixed 476,672-byte
// array that every GPU that loads this library holds until the process exits.
//
// Set-up: the first call on a device, with that device current, looks up
// the array's device address (cudaGetSymbolAddress) and caches it.  The
// array is shared by every call and keeps the last call's contents; each
// call rewrites the records and clears the queue head and error word before
// its launches.  Calls whose
// launches overlap on the GPU (different streams, or different host threads
// on one device) race on the array: serialise them.
//
// The caller's CSR is checked on the device before the anneal (the host
// never sees it): offsets start at 0 and never decrease, every neighbour id
// is in range and not the row itself, rows are strictly ascending, every
// entry has a twin of equal weight, and no row's sum of |w| exceeds the
// caller's max_weighted_deg (which picks the gain width and the score path,
// so an understated bound would overflow them).  A CSR that fails sets the
// error word and moves the work-queue head past every work item, so the
// anneal launch that follows takes no work; the call then returns
// RFMF_ERR_INVALID.  The only host synchronisation is the read of the error
// word at the end of the call.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
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
int fail(int code, const char* fmt, ...);
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
static_assert(kNoAllocScratchBytes == 476672, "the no-alloc scratch size is stated in rfmf.h");

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

// Records a failed check: the first code wins, and the queue head moves past
// any work-item count so the anneal launch that follows takes no work.
__device__ __forceinline__ void reject(int32_t* ctl) {
    atomicCAS(ctl + 1, 0, static_cast<int32_t>(kDevBadInput));
    atomicExch(ctl, 1 << 30);
}

// Checks the caller's CSR (one thread per row, grid-stride; every read stays
// inside [0, offsets[n]) once the row bounds are checked) and adds the sum of
// the weights over directed entries into the graph record's wsum2, which the
// kernel uses to derive each fresh chain's cut.
__global__ void check_csr_kernel(const uint32_t* __restrict__ off, const int2* __restrict__ edges,
                                 int n, long long maxB, long long* wsum2, int32_t* ctl) {
    const uint32_t m2 = off[n];
    if (blockIdx.x == 0 && threadIdx.x == 0 && off[0] != 0) reject(ctl);
    long long wsum = 0;
    bool bad = false;
    const int stride = gridDim.x * blockDim.x;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n && !bad; v += stride) {
        const uint32_t lo = off[v], hi = off[v + 1];
        if (hi < lo || hi > m2) { bad = true; break; }
        long long absSum = 0;
        int prev = -1;
        for (uint32_t i = lo; i < hi; ++i) {
            const int2 e = edges[i];
            if (e.x < 0 || e.x >= n || e.x == v || e.x <= prev) { bad = true; break; }
            prev = e.x;
            absSum += (e.y < 0) ? -static_cast<long long>(e.y) : static_cast<long long>(e.y);
            wsum += e.y;
            // The twin (e.x, v) with the same weight, by bisection of row e.x.
            const uint32_t rowEnd = off[e.x + 1];
            uint32_t a = off[e.x], b = rowEnd;
            if (b < a || b > m2) { bad = true; break; }
            while (a < b) {
                const uint32_t mid = a + (b - a) / 2;
                if (edges[mid].x < v) a = mid + 1; else b = mid;
            }
            if (a >= rowEnd || edges[a].x != v || edges[a].y != e.y) { bad = true; break; }
        }
        if (absSum > maxB) bad = true;
    }
    if (bad) reject(ctl);
    for (int m = 16; m > 0; m >>= 1) wsum += __shfl_xor_sync(0xFFFFFFFFu, wsum, m);
    if ((threadIdx.x & 31) == 0 && wsum != 0)
        atomicAdd(reinterpret_cast<unsigned long long*>(wsum2), static_cast<unsigned long long>(wsum));
}

bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

}  // namespace

static int rfmf_anneal_noalloc_impl(int device, void* stream, int64_t n,
                                   const uint32_t* d_offsets, const int32_t* d_edges,
                                   int64_t max_weighted_deg, int64_t C, const double* t0s,
                                   const uint64_t* solver_seeds, int64_t nphases,
                                   const uint64_t* phases, const uint64_t* iters,
                                   const int64_t* d_beta_end, const int32_t* d_beta_val,
                                   int64_t beta_runs, const int64_t* chain_beta_off,
                                   const int64_t* chain_beta_runs, uint32_t* d_spin_bits,
                                   uint32_t* d_best_bits, int64_t* d_cur, int64_t* d_best) {
    if (n <= 0 || n >= (int64_t(1) << 31)) return nerr(RFMF_ERR_INVALID, "n out of range");
    if (C <= 0 || C > kNoAllocMaxChains)
        return nerr(RFMF_ERR_CAPACITY, "no-alloc path: chains must be 1..4096");
    if (nphases < 0 || nphases > kNoAllocMaxPhases)
        return nerr(RFMF_ERR_CAPACITY, "no-alloc path: at most 64 phases");
    if (!d_offsets || !d_edges || !t0s || !solver_seeds || !d_beta_end || !d_beta_val ||
        !chain_beta_off || !chain_beta_runs || !d_spin_bits || !d_best_bits || !d_cur || !d_best ||
        (nphases && (!phases || !iters)))
        return nerr(RFMF_ERR_INVALID, "NULL argument");
    // The kernel reads offsets and spin words as 4-byte words, CSR entries as
    // 8-byte {col, weight} pairs and beta run ends and cut values as 8-byte
    // words: a pointer off those boundaries is refused here, before any
    // device work.
    if (!aligned(d_offsets, 4) || !aligned(d_edges, 8) || !aligned(d_beta_end, 8) ||
        !aligned(d_beta_val, 4) || !aligned(d_spin_bits, 4) || !aligned(d_best_bits, 4) ||
        !aligned(d_cur, 8) || !aligned(d_best, 8))
        return nerr(RFMF_ERR_INVALID,
                    "misaligned device pointer (offsets, beta_val, spin and best bits need 4 "
                    "bytes; edges, beta_end and the cut outputs 8)");
    if (max_weighted_deg < 0 || max_weighted_deg > std::numeric_limits<int32_t>::max())
        return nerr(RFMF_ERR_INVALID, "max_weighted_deg out of range");
    if (beta_runs < 1) return nerr(RFMF_ERR_INVALID, "beta_runs must be >= 1");
    for (int64_t c = 0; c < C; ++c) {
        if (chain_beta_off[c] < 0 || chain_beta_runs[c] < 1 ||
            chain_beta_runs[c] > beta_runs - chain_beta_off[c])
            return rfmf::fail(RFMF_ERR_INVALID, "chain %lld: beta runs outside the %lld-run table",
                              static_cast<long long>(c), static_cast<long long>(beta_runs));
        if (!(t0s[c] > 0.0)) return nerr(RFMF_ERR_INVALID, "t0 must be > 0");
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaSetDevice(device) != cudaSuccess) return nerr(RFMF_ERR_CUDA, "cudaSetDevice failed");
    unsigned char* base = nullptr;
    if (int rc = scratch_address(device, &base)) return rc;

    uint64_t total = 0, maxP = 1;
    for (int64_t p = 0; p < nphases; ++p) {
        if (phases[p] > 0x7FFFFFFFull) return nerr(RFMF_ERR_CAPACITY, "phase P too large");
        if (phases[p]) { total += iters[p]; maxP = std::max<uint64_t>(maxP, phases[p]); }
    }

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
    int sms = 0, optin = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess)
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
    // the device; the host staging below is ordinary host memory).  wsum2
    // starts at 0 and the check kernel adds the weights into it.
    DevGraph g{};
    g.offsets = d_offsets;
    g.edges = reinterpret_cast<const Edge*>(d_edges);
    g.compact = nullptr;
    g.n = static_cast<int32_t>(n);
    g.words = words;
    g.wsum2 = 0;
    g.offBytes = 0;
    g.entBytes = 0;
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

    cudaError_t e = cudaSuccess;
    auto cp = [&](size_t off, const void* src, size_t bytes) {
        if (e == cudaSuccess) e = cudaMemcpyAsync(base + off, src, bytes, cudaMemcpyHostToDevice, st);
    };
    cp(kOffGraph, &g, sizeof g);
    cp(kOffSched, &sch, sizeof sch);
    cp(kOffPhaseP, hp.data(), hp.size() * sizeof(uint32_t));
    cp(kOffPhaseIters, hi.data(), hi.size() * sizeof(uint64_t));
    cp(kOffChains, ch.data(), C * sizeof(DevChain));
    cp(kOffItems, items.data(), nitems * sizeof(DevItem));
    cp(kOffOrder, order.data(), C * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(base + kOffCtl, 0, 16, st);
    int32_t* ctl = reinterpret_cast<int32_t*>(base + kOffCtl);
    if (e == cudaSuccess) {
        const int threads = 256;
        const int blocks = static_cast<int>(std::min<int64_t>((n + threads - 1) / threads, 8 * static_cast<int64_t>(sms)));
        check_csr_kernel<<<blocks, threads, 0, st>>>(
            d_offsets, reinterpret_cast<const int2*>(d_edges), static_cast<int>(n),
            static_cast<long long>(max_weighted_deg),
            reinterpret_cast<long long*>(base + kOffGraph + offsetof(DevGraph, wsum2)), ctl);
        e = cudaGetLastError();
    }
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
    L.queue = ctl;
    L.error = ctl + 1;
    L.errorItem = ctl + 2;
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
    int32_t hctl[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(hctl, ctl, sizeof hctl, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return nerr(RFMF_ERR_CUDA, cudaGetErrorString(e));
    if (hctl[1] == kDevBadInput)
        return nerr(RFMF_ERR_INVALID,
                    "device CSR rejected: offsets must start at 0 and never decrease, ids lie in "
                    "[0, n) without self loops, rows strictly ascending, every entry has a twin of "
                    "equal weight, and no row's sum of |w| may exceed max_weighted_deg");
    if (hctl[1] != kDevOk) return nerr(RFMF_ERR_DEVICE, "device-side error during the anneal");
    return RFMF_OK;
}

// C ABI entry points: no C++ exception crosses the boundary.
extern "C" int rfmf_anneal_noalloc(int device, void* stream, int64_t n,
                                   const uint32_t* d_offsets, const int32_t* d_edges,
                                   int64_t max_weighted_deg, int64_t C, const double* t0s,
                                   const uint64_t* solver_seeds, int64_t nphases,
                                   const uint64_t* phases, const uint64_t* iters,
                                   const int64_t* d_beta_end, const int32_t* d_beta_val,
                                   int64_t beta_runs, const int64_t* chain_beta_off,
                                   const int64_t* chain_beta_runs, uint32_t* d_spin_bits,
                                   uint32_t* d_best_bits, int64_t* d_cur, int64_t* d_best) {
    try {
        return rfmf_anneal_noalloc_impl(device, stream, n, d_offsets, d_edges, max_weighted_deg, C,
                                        t0s, solver_seeds, nphases, phases, iters, d_beta_end,
                                        d_beta_val, beta_runs, chain_beta_off, chain_beta_runs,
                                        d_spin_bits, d_best_bits, d_cur, d_best);
    } catch (const std::bad_alloc&) {
        return rfmf::set_last_error(RFMF_ERR_NOMEM, "host allocation failed in rfmf_anneal_noalloc");
    } catch (...) {
        return rfmf::set_last_error(RFMF_ERR_INVALID, "unexpected host exception in rfmf_anneal_noalloc");
    }
}
