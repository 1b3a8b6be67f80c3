// rfmf_device.h -- structures shared by the host driver and the sm_103a
// kernels.  Plain C++ (no CUDA headers) so the host .cpp can include it.
#ifndef RFMF_DEVICE_H
#define RFMF_DEVICE_H

#include <cstdint>
#include <climits>

namespace rfmf {

// One directed CSR entry: neighbour id and weight, loaded as one 8-byte word.
struct alignas(8) Edge {
    int32_t col;
    int32_t w;
};

// One CSR graph in HBM, read-only, shared by every chain that anneals it.
// Rows are sorted ascending by neighbour (the reference's AnnealCsr order,
// src/immutable_graph.hpp:83-101); each undirected edge is stored twice.
// An edge is one 8-byte word {col, weight} so a neighbour walk issues one
// load per entry.
struct DevGraph {
    const uint32_t* offsets;   // n + 1
    const Edge*     edges;     // 2m  {col, weight}
    int32_t         n;
    int32_t         words;     // ceil(n / 32): spin bit-words per chain
    int64_t         wsum2;     // sum of weight over directed entries (2 * sum over edges)
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

// One chain = one work item of the persistent kernel.  The chain's state
// (spin bits, best-spin bits, current and best cut) lives in HBM between
// launches and in shared memory while a CTA runs it.
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

// Error word written by the kernel (0 = ok).  The kernel never traps: it
// records the first problem it sees and lets the CTA finish.
enum DevError : int32_t {
    kDevOk = 0,
    kDevCutMismatch = 1,     // carried cut value disagrees with the spins
    kDevBetaTable = 2,       // beta table shorter than the window
    kDevBadItem = 3,         // graph/schedule index out of range
};

// Launch-wide parameters.
struct DevLaunch {
    const DevGraph*    graphs;
    const DevSchedule* scheds;
    DevChain*          chains;
    const int32_t*     order;       // work-queue order (chain indices)
    int32_t            nchains;
    int32_t            ngraphs;
    int32_t            nscheds;
    int32_t            maxP;        // largest phase P in any schedule of the launch
    int32_t            maxWords;    // largest spin word count of any graph
    int32_t            maxN;        // largest n
    int32_t*           queue;       // work-queue head (zeroed before the launch)
    int32_t*           error;       // first device error (DevError)
    int32_t*           errorItem;   // chain that raised it
    uint64_t           window;      // sweeps each chain advances in this launch
    int32_t            lut[16];     // Q20 Gumbel quantile table
};

// cur == kUnsetCut on input: the kernel derives the cut of spinBits itself
// and starts bestBits/best from it (a fresh chain).
constexpr int64_t kUnsetCut = INT64_MIN;

}  // namespace rfmf

#endif  // RFMF_DEVICE_H
