// rfmf_device.h -- structures shared by the host driver and the sm_103a
// kernels.  Plain C++ (no CUDA headers) so the host .cpp can include it.
#ifndef RFMF_DEVICE_H
#define RFMF_DEVICE_H

#include <climits>
#include <cstdint>

namespace rfmf {

// One directed CSR entry: neighbour id and weight, loaded as one 8-byte word.
struct alignas(8) Edge {
    int32_t col;
    int32_t w;
};

// How a launch reads the CSR.  The compact formats are copied once per CTA
// into shared memory (bulk async copy) and walked there; the HBM formats walk
// the graph's own arrays through L1/L2 (graphs too large for shared memory
// beside their chains), with the most compact entries the graph allows.
enum CsrFormat : int32_t {
    kCsrUnit16 = 0,    // uint16 entry = (col << 1) | (w < 0); |w| == 1, n <= 32768
    kCsrPacked32 = 1,  // uint32 entry = (w << 16) | col;  |w| < 2^15, n <= 65536
    kCsrGlobal = 2,    // Edge {col, w} in HBM
    kCsrGlobal16 = 3,  // the unit16 entries, in HBM
    kCsrGlobal32 = 4,  // the packed32 entries, in HBM
};

#if defined(__CUDACC__)
#define RFMF_CHD __host__ __device__ constexpr
#else
#define RFMF_CHD constexpr
#endif
// Formats walked in HBM (no shared-memory copy of the CSR).
RFMF_CHD bool csr_in_hbm(int fmt) { return fmt == kCsrGlobal || fmt == kCsrGlobal16 || fmt == kCsrGlobal32; }

// One CSR graph in HBM, read-only, shared by every chain that anneals it.
// Rows are sorted ascending by neighbour (the reference's AnnealCsr order,
// src/immutable_graph.hpp:83-101); each undirected edge is stored twice.
struct DevGraph {
    const uint32_t* offsets;   // n + 1 (padded to 16 B)
    const Edge*     edges;     // 2m  {col, weight}
    const void*     compact;   // 2m compact entries of the launch's format (padded to 16 B)
    int32_t         n;
    int32_t         words;     // ceil(n / 32): spin bit-words per chain
    int64_t         wsum2;     // sum of weight over directed entries (2 * sum over edges)
    uint32_t        offBytes;  // bytes of offsets, multiple of 16
    uint32_t        entBytes;  // bytes of compact entries, multiple of 16
};

// One schedule: phases (group counts P) and sweeps per phase, shared by the
// chains that reference it.  Phases with P == 0 are skipped without
// advancing the sweep counter (src/anneal_kernels.cu:272).
struct DevSchedule {
    const uint32_t* phaseP;
    const uint64_t* phaseIters;
    int32_t         nphases;
    int32_t         pad;
};

// One chain.  Its state (spin bits, best-spin bits, current and best cut,
// progress) lives in HBM between launches and in shared memory while a
// warp group runs it.
struct DevChain {
    int32_t         graph;        // index into the graph table
    int32_t         sched;        // index into the schedule table
    uint64_t        solverSeed;   // Philox key (seed + kSolverSeedOffset)
    const int64_t*  betaEnd;      // run-length beta table, 0-based exclusive ends
    const int32_t*  betaVal;      //   (one table per distinct t0)
    int64_t         betaRuns;
    uint32_t*       spinBits;     // words(graph) words, bit v = (spin[v] > 0)
    uint32_t*       bestBits;     // words(graph) words
    int64_t         cur;          // in/out: cut value of spinBits
    int64_t         best;         // in/out: cut value of bestBits
    uint64_t        sweepsDone;   // executed sweeps so far (in/out)
    uint64_t        sweepsTotal;  // executed sweeps of the whole schedule
    uint64_t        improvedSweeps;  // sweeps that raised the best cut (statistic)
};

// One work item of the persistent kernel: up to K chains of ONE graph, run
// side by side by the K warp groups of a CTA on one shared-memory copy of
// the graph.  The chains are order[first .. first + count).
struct DevItem {
    int32_t graph;
    int32_t first;
    int32_t count;
    int32_t pad;
};

// Error word written by the kernel (0 = ok).  The kernel never traps: it
// records the first problem it sees and lets the CTA finish.
enum DevError : int32_t {
    kDevOk = 0,
    kDevCutMismatch = 1,     // carried cut value disagrees with the spins
    kDevBetaTable = 2,       // beta table shorter than the window
    kDevBadItem = 3,         // graph/schedule index out of range
    kDevCopyTimeout = 4,     // bulk copy of the CSR did not complete in time
    kDevBadInput = 5,        // a caller's device CSR failed the on-device check
};

// Launch-wide parameters.
struct DevLaunch {
    const DevGraph*    graphs;
    const DevSchedule* scheds;
    DevChain*          chains;
    const DevItem*     items;
    const int32_t*     order;       // chain indices grouped by item
    int32_t            nitems;
    int32_t            ngraphs;
    int32_t            nscheds;
    int32_t            warpsPerChain;   // W: threads per chain = 32 W
    int32_t            chainsPerCta;    // K: warp groups per CTA
    int32_t            maxN;            // largest n (sizes the per-chain gain array)
    int32_t            maxWords;        // largest spin word count
    int32_t            pmax;            // group slots per chain: min(max P, max n)
    uint32_t           csrBytes;        // shared-memory CSR region (0 for kCsrGlobal)
    uint32_t           chainBytes;      // shared-memory bytes per chain
    int32_t*           queue;       // work-queue head (zeroed before the launch)
    int32_t*           error;       // first device error (DevError)
    int32_t*           errorItem;   // chain/item that raised it
    uint64_t*          itemNs;      // per item: device time the CTA spent on it (ns)
    uint64_t           window;      // sweeps each chain advances in this launch
    int32_t            lut[16];     // Q20 Gumbel quantile table
};

// cur == kUnsetCut on input: the kernel derives the cut of spinBits itself
// and starts bestBits/best from it (a fresh chain).
constexpr int64_t kUnsetCut = INT64_MIN;

// Shared-memory header in front of the CSR region: Gumbel table (64 B),
// bulk-copy mbarrier, work-item slot, chain pacing state (bytes 160..227).
constexpr uint32_t kSmemHeader = 256;

#if defined(__CUDACC__)
#define RFMF_HD __host__ __device__ __forceinline__
#else
#define RFMF_HD inline
#endif

RFMF_HD uint32_t align16(uint32_t x) { return (x + 15u) & ~15u; }

// Per-chain shared-memory region, in order: gains D (nPad * dbytes), spin
// bits, best-spin bits, spins as bytes (0/1, for one-load neighbour lookups
// in FLIP), group key slots (8 B), ids (4 B), winners (4 B),
// reduction partials (8 B per warp).
// Host and kernel both carve with this.
struct ChainLayout {
    uint32_t d, bits, best, sb, slots, ids, win, red, total;
};

RFMF_HD ChainLayout chain_layout(int maxN, int maxWords, int pmax, int warps, int dbytes) {
    ChainLayout c;
    const uint32_t nPad = (static_cast<uint32_t>(maxN) + 7u) & ~7u;
    uint32_t o = 0;
    c.d = o;     o = align16(o + nPad * static_cast<uint32_t>(dbytes));
    c.bits = o;  o = align16(o + static_cast<uint32_t>(maxWords) * 4u);
    c.best = o;  o = align16(o + static_cast<uint32_t>(maxWords) * 4u);
    c.sb = o;    o = align16(o + nPad);
    c.slots = o; o = align16(o + static_cast<uint32_t>(pmax) * 8u);
    c.ids = o;   o = align16(o + static_cast<uint32_t>(pmax) * 4u);
    c.win = o;   o = align16(o + static_cast<uint32_t>(pmax) * 4u);
    c.red = o;   o = align16(o + static_cast<uint32_t>(warps) * 8u);
    c.total = o;
    return c;
}

}  // namespace rfmf

#endif  // RFMF_DEVICE_H
