// rfmf_batch.cpp -- batches: chains over many graphs with device-resident
// state, advanced window by window in persistent launches; and rfmf_anneal,
// the annealGpu drop-in, as a one-batch special case.
//
// Replaces the reference's host driver for the path (src/anneal_kernels.cu:
// 498-884, runDispatch/runMC/annealGpu): one graph per launch, V100 tuning
// constants (src/tuning.hpp), state allocated and freed per call.  Here:
//   * graphs of a batch fall into LAUNCH CLASSES -- gain width (int8 when
//     B <= 127), CSR format (the most compact shared-memory format whose copy
//     fits beside one chain, else HBM walks), warps per chain and score path
//     -- so that small graphs do not inherit the layout a large one needs;
//   * each class is planned by the autotuner (chains per CTA from the
//     occupancy API, the smallest that keeps every work item resident) and
//     runs as its own persistent launch; classes of one window go out on
//     separate streams and share the GPU;
//   * in a class of several graphs, each graph's chains per work item are
//     sized per phase from item costs by scheduler level (learned from the
//     %globaltimer item timings of earlier launches, else a shape model),
//     and a window is cut at phase boundaries so each piece runs with the
//     items of its phase.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <string>
#include <memory>
#include <new>
#include <queue>
#include <tuple>
#include <vector>

#include "../../include/rfmf_testing.h"
#include "rfmf_host.h"

using namespace rfmf;

namespace {

constexpr uint64_t kMinLearnSweeps = 256;

// Chains whose graphs share a kernel variant and a CTA layout.
struct BatchClass {
    bool score64 = false;
    int dbytes = 1, fmt = kCsrGlobal, warps = 1;
    int baseWarps = 1;           // the planner's width; `warps` may double per phase
    int K = 1, threads = 32, grid = 0, occ = 1, nitems = 0, pmax = 1;
    size_t smem = 0;
    std::vector<int> graphs;                      // batch graph indices
    std::vector<std::vector<int32_t>> chainsOf;   // per class graph: chain ids
    std::vector<int> Kg;                          // per class graph: chains per item
    std::vector<DevItem> items;
    std::vector<int32_t> order;
    bool balanced = false;       // items sized from graph costs (learned or modelled)
    uint64_t pendingSweeps = 0;  // sweeps of the last launch, whose item times are unread
    uint32_t pendingP = 0;       // its phase P (0: it spanned several phases)
    DevBuf dItems, dOrder, dItemNs, dCtl;
    DevLaunch L{};
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
};

}  // namespace

struct rfmf_batch {
    rfmf::CtxHold ctxHold;   // first member: released last
    rfmf::GraphHolds graphHolds;   // released after the device buffers
    rfmf_context* ctx = nullptr;
    int64_t C = 0;
    uint64_t total = 0;
    std::vector<int64_t> chainN, chainWordOff;   // per chain
    std::vector<int64_t> graphOfChain;
    int64_t words = 0;                           // total spin words over chains
    std::vector<const rfmf_graph*> glist;
    std::vector<uint32_t> phaseP;                // the schedule, host copy
    std::vector<uint64_t> phaseIters;
    DevBuf dGraphs, dScheds, dChains, dPhaseP, dPhaseIters, dBits, dBest;
    std::vector<DevBetaRef> betaRefs;            // the context's shared beta tables in use
    std::vector<BatchClass> cls;
    cudaEvent_t fork = nullptr;
    uint64_t hostDone = 0;       // sweeps every chain has been advanced by
    cudaGraphExec_t graphExec = nullptr;
    uint64_t graphSweeps = 0;
    int graphLaunches = 0;
    int64_t launches = 0;        // kernel launches enqueued (captured ones when replayed)
    rfmf_launch_config cfg{};    // the creation config (re-planning per phase)
    bool phaseWarps = false;     // the one class's width follows the phase
    ~rfmf_batch() {
        if (graphExec) cudaGraphExecDestroy(graphExec);
        for (BatchClass& k : cls) {
            if (k.done) cudaEventDestroy(k.done);
            if (k.stream) cudaStreamDestroy(k.stream);
        }
        if (fork) cudaEventDestroy(fork);
    }
};

namespace {

uint32_t csr_bytes(const rfmf_graph* g, int fmt) {
    if (fmt == kCsrUnit16) return g->offBytes + g->u16Bytes;
    if (fmt == kCsrPacked32) return g->offBytes + g->p32Bytes;
    return 0;
}

int64_t dyn_smem_max(const rfmf_context* ctx, const void* kern, cudaFuncAttributes& fa) {
    if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess) return -1;
    return static_cast<int64_t>(ctx->smemOptin) - static_cast<int64_t>(fa.sharedSizeBytes);
}

// Plan one class: chains per CTA K, CTA shape, grid.  `exact` sizes the CTA
// to the chosen K (several classes share SMs); otherwise the CTA keeps the
// largest K that fits as headroom for per-graph item sizes.
int plan_class(rfmf_batch& b, BatchClass& k, const rfmf_launch_config& c, bool exact) {
    const int sms = b.ctx->sms;
    int maxN = 0, maxWords = 0;
    uint32_t csrB = 0;
    std::vector<int64_t> perGraph;
    for (size_t q = 0; q < k.graphs.size(); ++q) {
        const rfmf_graph* g = b.glist[k.graphs[q]];
        maxN = std::max<int>(maxN, static_cast<int>(g->n));
        maxWords = std::max<int>(maxWords, static_cast<int>((g->n + 31) / 32));
        csrB = std::max(csrB, csr_bytes(g, k.fmt));
        perGraph.push_back(static_cast<int64_t>(k.chainsOf[q].size()));
    }
    k.pmax = std::max(1, std::min(k.pmax, maxN));
    const void* kern = kernel_ptr(k.dbytes, k.fmt, k.score64);
    cudaFuncAttributes fa{};
    const int64_t dynMax = dyn_smem_max(b.ctx, kern, fa);
    if (dynMax < 0) return fail(RFMF_ERR_CUDA, "kernel attributes unavailable");
    const uint32_t chainB = chain_layout(maxN, maxWords, k.pmax, k.warps, k.dbytes).total;
    // Warp groups per CTA: named barriers 1..15, and the variant's register
    // budget bounds the CTA's threads.
    const int W = k.warps;
    const int kCap = std::min(std::min(16 / W, W > 1 ? 15 : 16), fa.maxThreadsPerBlock / (32 * W));
    if (kCap < 1) return fail(RFMF_ERR_CAPACITY, "a %d-thread chain exceeds the kernel's CTA limit", 32 * W);
    const int64_t room = dynMax - kSmemHeader - csrB;
    int Kmax = room > 0 ? static_cast<int>(std::min<int64_t>(kCap, room / chainB)) : 0;
    if (c.chains_per_cta) {
        if (c.chains_per_cta < 1 || c.chains_per_cta > kCap)
            return fail(RFMF_ERR_INVALID, "chains_per_cta must be 0 or 1..%d", kCap);
        Kmax = std::min(Kmax, c.chains_per_cta);
    }
    if (Kmax < 1)
        return fail(RFMF_ERR_CAPACITY,
                    "one chain needs %u B of shared memory beside a %u B CSR, but a CTA has %lld B",
                    chainB, csrB, static_cast<long long>(dynMax));
    CU(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(dynMax)));
    CU(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                            cudaSharedmemCarveoutMaxShared));
    auto items_for = [&](int K) {
        int64_t it = 0;
        for (int64_t cg : perGraph) it += (cg + K - 1) / K;
        return it;
    };
    auto occ_for = [&](int K) {
        int occ = 0;
        const size_t smem = kSmemHeader + csrB + static_cast<size_t>(K) * chainB;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32 * W * K, smem) != cudaSuccess) {
            cudaGetLastError();
            occ = 0;
        }
        return occ;
    };
    int Kshape = Kmax, occ = 0;
    for (; Kshape >= 1; --Kshape)
        if ((occ = occ_for(Kshape)) > 0) break;
    if (Kshape < 1)
        return fail(RFMF_ERR_CAPACITY, "no resident configuration for %u B CSR + %u B per chain", csrB, chainB);
    // Smallest uniform K whose items all fit the resident CTA slots.
    int Kuni = c.chains_per_cta ? Kshape : 1;
    if (exact) {
        for (; Kuni < Kshape; ++Kuni) {
            const int o = occ_for(Kuni);
            if (o > 0 && items_for(Kuni) <= static_cast<int64_t>(o) * sms) break;
        }
        Kshape = Kuni;
        occ = occ_for(Kshape);
    } else {
        const int64_t slots = static_cast<int64_t>(occ) * sms;
        while (Kuni < Kshape && items_for(Kuni) > slots) ++Kuni;
    }
    k.occ = std::max(occ, 1);
    k.K = Kshape;
    k.threads = 32 * W * Kshape;
    k.smem = kSmemHeader + csrB + static_cast<size_t>(Kshape) * chainB;
    k.Kg.assign(k.graphs.size(), Kuni);
    k.L.warpsPerChain = W;
    k.L.chainsPerCta = Kshape;
    k.L.maxN = maxN;
    k.L.maxWords = maxWords;
    k.L.pmax = k.pmax;
    k.L.csrBytes = csrB;
    k.L.chainBytes = chainB;
    return RFMF_OK;
}

// Per-graph chains per item: graph q may use item sizes cand[q] (chain
// count, item time per sweep; ascending in both, each the largest count of
// its scheduler level), over `slots` resident CTAs that take items from the
// queue in order, longest first.
//
// When every item fits one round of the slots, the smallest makespan tau
// wins, each graph taking its largest size whose time is <= tau.  When even
// the largest sizes need more than one round, the makespan is that of the
// queue's longest-first list schedule, and sizes are lowered one graph and
// one level at a time while that shortens it (GB300, large sparse shapes,
// 768 chains of four warps on 152 CTAs: 7.85e7 -> 8.33e7 chain-steps/s).
// That model holds for a class alone on the GPU; classes that share the SMs
// (`rounds` false) keep their sizes instead (the 512-graph mix in six
// classes lost 5% under it).  False (kg untouched) when nothing is planned.
struct ItemCand {
    int K;
    double ns;
};

// The list-schedule makespan of sizes idx[q] (indices into cand[q]): items
// of the chosen size plus one remainder item per graph, longest first, each
// to the slot that frees first.
double list_makespan(const std::vector<std::vector<ItemCand>>& cand, const std::vector<int64_t>& chains,
                     const std::vector<size_t>& idx, int64_t slots) {
    std::vector<double> items;
    for (size_t q = 0; q < cand.size(); ++q) {
        const ItemCand& c = cand[q][idx[q]];
        const int64_t full = chains[q] / c.K, rest = chains[q] % c.K;
        items.insert(items.end(), static_cast<size_t>(full), c.ns);
        if (rest) {
            size_t r = 0;
            while (cand[q][r].K < rest) ++r;   // the level of a partial item
            items.push_back(cand[q][r].ns);
        }
    }
    std::sort(items.begin(), items.end(), std::greater<double>());
    const size_t S = static_cast<size_t>(std::max<int64_t>(1, std::min<int64_t>(slots, static_cast<int64_t>(items.size()))));
    std::priority_queue<double, std::vector<double>, std::greater<double>> freeAt;
    for (size_t i = 0; i < S; ++i) freeAt.push(0.0);
    double span = 0.0;
    for (double t : items) {
        const double f = freeAt.top() + t;
        freeAt.pop();
        freeAt.push(f);
        span = std::max(span, f);
    }
    return span;
}

bool balance_items(const std::vector<std::vector<ItemCand>>& cand, const std::vector<int64_t>& chains,
                   int64_t slots, std::vector<int>& kg, bool rounds = true) {
    const size_t G = cand.size();
    if (G == 0) return false;
    std::vector<double> taus;
    for (const auto& cq : cand)
        for (const ItemCand& c : cq) taus.push_back(c.ns);
    std::sort(taus.begin(), taus.end());
    auto pick = [&](double tau, std::vector<int>& out) {
        int64_t items = 0;
        for (size_t q = 0; q < G; ++q) {
            int K = 0;
            for (const ItemCand& c : cand[q])
                if (c.ns <= tau) K = c.K;
            if (!K) return false;
            out[q] = K;
            items += (chains[q] + K - 1) / K;
        }
        return items <= slots;
    };
    std::vector<int> trial(G, 0);
    size_t lo = 0, hi = taus.size();   // first feasible index in [lo, hi)
    while (lo < hi) {
        const size_t mid = (lo + hi) / 2;
        if (pick(taus[mid], trial)) hi = mid; else lo = mid + 1;
    }
    if (lo < taus.size() && pick(taus[lo], trial)) {
        kg = trial;
        return true;
    }
    if (!rounds) return false;
    // More than one round: descend from the largest sizes (at most 2000
    // schedule evaluations, a few hundred ms for the largest classes).
    std::vector<size_t> idx(G);
    for (size_t q = 0; q < G; ++q) idx[q] = cand[q].size() - 1;
    double best = list_makespan(cand, chains, idx, slots);
    int evals = 1;
    for (bool improved = true; improved && evals < 2000;) {
        improved = false;
        size_t bestQ = G;
        for (size_t q = 0; q < G && evals < 2000; ++q) {
            if (idx[q] == 0) continue;
            --idx[q];
            const double m = list_makespan(cand, chains, idx, slots);
            ++evals;
            ++idx[q];
            if (m < best * (1.0 - 1e-9)) { best = m; bestQ = q; }
        }
        if (bestQ < G) {
            --idx[bestQ];
            improved = true;
        }
    }
    kg.assign(G, 0);
    for (size_t q = 0; q < G; ++q) kg[q] = cand[q][idx[q]].K;
    return true;
}

// Whether every graph of class k has a cost learned at phase P.
bool class_learned(const rfmf_batch& b, const BatchClass& k, uint32_t P) {
    bool learned = true;
    for (int gi : k.graphs) learned = learned && b.glist[gi]->learned_at(k.warps, k.fmt, P);
    return learned;
}

// An item's time per sweep for graph q of class k at level L: learned, or
// modelled (for all graphs of the class alike).
double item_cost(const rfmf_batch& b, const BatchClass& k, size_t q, uint32_t P, int L, bool learned) {
    const rfmf_graph* g = b.glist[k.graphs[q]];
    return learned ? g->cost(k.warps, k.fmt, P, L) : g->model_cost(k.warps, P, L);
}

// Per-graph chains per item within a class, for phases of group count P.
// An item's time per sweep depends on its graph and its scheduler level
// (sched_level), so each graph's candidates are the largest chain count of
// each level up to the class's K, timed by the graphs' costs learned at P
// when every graph has some, else all by the shape model (learned and
// modelled costs are not on one scale: a cost learned in another batch
// shape, extrapolated to this one's levels, beside a modelled one, misled
// the split).
bool plan_balanced(const rfmf_batch& b, const BatchClass& k, uint32_t P, std::vector<int>& kg) {
    const size_t G = k.graphs.size();
    const bool alone = b.cls.size() == 1;
    const int64_t slots = static_cast<int64_t>(k.occ) * b.ctx->sms;
    // One graph: its uniform items are right unless even full ones need
    // more than one round (then the list schedule decides, as below).
    if (G == 0 || (G == 1 && !(alone && (static_cast<int64_t>(k.chainsOf[0].size()) + k.K - 1) / k.K > slots)))
        return false;
    const bool learned = class_learned(b, k, P);
    std::vector<std::vector<ItemCand>> cand(G);
    std::vector<int64_t> chains(G);
    for (size_t q = 0; q < G; ++q) {
        chains[q] = static_cast<int64_t>(k.chainsOf[q].size());
        for (int K = 1; K <= k.K; ++K) {
            if (K < k.K && sched_level(K + 1, k.warps) == sched_level(K, k.warps)) continue;
            cand[q].push_back({K, item_cost(b, k, q, P, sched_level(K, k.warps), learned)});
        }
    }
    return balance_items(cand, chains, slots, kg, alone);
}

// Items: graphs in decreasing per-item cost, each graph's chains in groups of
// its K_g (item.graph is the batch graph index).
void build_items(const rfmf_batch& b, BatchClass& k, uint32_t P) {
    const size_t G = k.graphs.size();
    std::vector<int> gorder(G);
    for (size_t q = 0; q < G; ++q) gorder[q] = static_cast<int>(q);
    const bool learned = class_learned(b, k, P);
    auto itemCost = [&](int q) {
        return item_cost(b, k, static_cast<size_t>(q), P, sched_level(k.Kg[q], k.warps), learned);
    };
    std::stable_sort(gorder.begin(), gorder.end(), [&](int a, int z) { return itemCost(a) > itemCost(z); });
    k.items.clear();
    k.order.clear();
    for (int q : gorder) {
        const auto& cl = k.chainsOf[q];
        const size_t K = static_cast<size_t>(k.Kg[q]);
        for (size_t s = 0; s < cl.size(); s += K) {
            DevItem it{};
            it.graph = k.graphs[q];
            it.first = static_cast<int32_t>(k.order.size());
            it.count = static_cast<int32_t>(std::min(K, cl.size() - s));
            for (int t = 0; t < it.count; ++t) k.order.push_back(cl[s + t]);
            k.items.push_back(it);
        }
    }
    k.nitems = static_cast<int>(k.items.size());
    k.grid = static_cast<int>(std::min<int64_t>(k.nitems, static_cast<int64_t>(k.occ) * b.ctx->sms));
    k.L.nitems = k.nitems;
}

int upload_items(rfmf_batch& b, BatchClass& k) {
    cudaStream_t st = b.ctx->stream;
    CU(cudaMemcpyAsync(k.dItems.p, k.items.data(), k.items.size() * sizeof(DevItem), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(k.dOrder.p, k.order.data(), k.order.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    CU(cudaMemsetAsync(k.dItemNs.p, 0, std::max<size_t>(k.items.size(), 1) * sizeof(uint64_t), st));
    return RFMF_OK;
}

// Fold the item timings of completed launches into the graphs' costs.
// Launches shorter than kMinLearnSweeps teach nothing: an item's time also
// holds its CSR staging and its chains' state load and gain set-up, which
// would dominate a short window and differ by graph.
int harvest_item_times(rfmf_batch& b, BatchClass& k) {
    if (!k.pendingSweeps || !k.pendingP || k.items.empty()) return RFMF_OK;
    const uint64_t sweeps = k.pendingSweeps;
    const uint32_t P = k.pendingP;
    k.pendingSweeps = 0;
    k.pendingP = 0;
    std::vector<uint64_t> ns(k.items.size());
    CU(cudaMemcpy(ns.data(), k.dItemNs.p, ns.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost));
    if (sweeps < kMinLearnSweeps) return RFMF_OK;
    for (size_t i = 0; i < k.items.size(); ++i) {
        const DevItem& it = k.items[i];
        if (ns[i] == 0 || it.count <= 0) continue;
        const double w = static_cast<double>(sweeps);
        const rfmf_graph* g = b.glist[it.graph];
        g->learn(k.warps, k.fmt, P, sched_level(std::min(it.count, k.K), k.warps), static_cast<double>(ns[i]) / w, w);
    }
    return RFMF_OK;
}

// The group count P of the phase that sweep `sweep` (0-based) falls in, and
// the end of that phase (phases with P = 0 are skipped, as the kernel skips
// them); past the schedule's end, the last phase with P > 0 and no end.
uint32_t phase_at(const rfmf_batch& b, uint64_t sweep, uint64_t* end) {
    uint64_t at = 0;
    uint32_t last = 1;
    for (size_t p = 0; p < b.phaseP.size(); ++p) {
        if (!b.phaseP[p]) continue;
        last = b.phaseP[p];
        at += b.phaseIters[p];
        if (sweep < at) {
            *end = at;
            return last;
        }
    }
    *end = UINT64_MAX;
    return last;
}

// Size the work items of classes for phases of group count P (multi-graph
// classes, and a lone class whose items need more than one round) from the
// costs learned so far (re-planned before every launch: costs keep
// arriving, and planning is a few microseconds per graph); uploaded only
// when the per-graph item sizes change (stream-ordered after older
// launches).  *changed (optional) tells whether any class's items did.
int rebalance(rfmf_batch* b, uint32_t P, bool* changed = nullptr) {
    if (changed) *changed = false;
    for (BatchClass& k : b->cls) {
        std::vector<int> kg;
        if (!plan_balanced(*b, k, P, kg)) continue;
        const bool differ = !k.balanced || kg != k.Kg;
        k.Kg = kg;
        k.balanced = true;
        if (differ) {
            build_items(*b, k, P);
            if (int rc = upload_items(*b, k)) return rc;
            if (changed) *changed = true;
        }
    }
    return RFMF_OK;
}

// Warps per chain for phases of group count P in a batch whose width
// follows the phase (one class, one graph, the rule's width W, every chain
// resident at 2W): 2W while the winners' rows hold at least half as many
// entries as the graph has vertices (P >= 64), W otherwise.  GB300, us per
// sweep at W / 2W: 1024 chains of ER n = 2000 d = 19 (W = 1) P = 128
// 10.0 / 8.08, P = 64 6.11 / 5.43, P = 32 4.14 / 4.60, P = 1 2.41 / 2.88;
// 32 chains of ER n = 800 d = 48 (W = 4) P = 128 5.56 / 4.39, P = 64
// 3.92 / 3.49, P = 1 1.72 / 1.78; the 50x60 torus (512 row entries at
// P = 128) is faster at one warp in every phase.
bool wide_phase(const rfmf_graph* g, uint32_t P) {
    const double n = static_cast<double>(g->n);
    const double rows = std::min(static_cast<double>(P), n);
    return P >= 64 && 2.0 * rows * (2.0 * static_cast<double>(g->m) / n) >= n;
}

int phase_warps(const rfmf_batch& b, const BatchClass& k, uint32_t P) {
    if (!b.phaseWarps) return k.warps;
    return wide_phase(b.glist[k.graphs[0]], P) ? 2 * k.baseWarps : k.baseWarps;
}

// Re-plans class k at `warps` per chain (CTA shape, items) for phase P.  A
// width that does not plan keeps the current one.
int set_warps(rfmf_batch* b, BatchClass& k, int warps, uint32_t P, bool* changed) {
    const int old = k.warps;
    k.warps = warps;
    if (plan_class(*b, k, b->cfg, false) != RFMF_OK) {
        k.warps = old;
        return plan_class(*b, k, b->cfg, false);
    }
    build_items(*b, k, P);
    if (int rc = upload_items(*b, k)) return rc;
    if (changed) *changed = true;
    return RFMF_OK;
}

// Everything that depends on the phase, before a launch in phase P: the
// width of a batch whose width follows the phase, then the item sizes of
// multi-graph classes.  *changed (optional) tells whether any launch shape
// or item list changed.
int prepare_phase(rfmf_batch* b, uint32_t P, bool* changed = nullptr) {
    bool any = false;
    if (b->phaseWarps) {
        BatchClass& k = b->cls[0];
        const int W = phase_warps(*b, k, P);
        if (W != k.warps)
            if (int rc = set_warps(b, k, W, P, &any)) return rc;
    }
    bool reb = false;
    if (int rc = rebalance(b, P, &reb)) return rc;
    if (changed) *changed = any || reb;
    return RFMF_OK;
}

// One launch per class over `sweeps` sweeps.  A single class goes out on
// the context's stream; several are forked onto their own streams and
// joined back, so run_timed events and graph capture see the whole window.
int launch_window(rfmf_batch* b, uint64_t sweeps) {
    cudaStream_t main = b->ctx->stream;
    const bool fork = b->cls.size() > 1;
    if (fork) CU(cudaEventRecord(b->fork, main));
    for (BatchClass& k : b->cls) {
        cudaStream_t st = fork ? k.stream : main;
        if (fork) CU(cudaStreamWaitEvent(st, b->fork, 0));
        DevLaunch L = k.L;
        L.window = sweeps;
        CU(cudaMemsetAsync(L.queue, 0, sizeof(int32_t), st));
        CU(launch_anneal(L, k.dbytes, k.fmt, k.score64, k.grid, k.threads, k.smem, st));
        if (fork) {
            CU(cudaEventRecord(k.done, st));
            CU(cudaStreamWaitEvent(main, k.done, 0));
        }
    }
    return RFMF_OK;
}

// One window of `sweeps` sweeps.  When a class holds several graphs, whose
// relative costs change with P, the window is cut at phase boundaries and
// each piece runs with items sized for its phase; results do not depend on
// the cut (a chain's sweeps are a function of its sweep index alone).
int enqueue_run(rfmf_batch* b, uint64_t sweeps, bool capturing = false) {
    if (capturing) return launch_window(b, sweeps);
    const int64_t perWindow = static_cast<int64_t>(b->cls.size());
    uint64_t left = std::min<uint64_t>(sweeps, b->total - std::min(b->total, b->hostDone));
    bool split = b->phaseWarps;
    for (const BatchClass& k : b->cls) split = split || k.graphs.size() > 1;
    uint64_t end = 0;
    const uint32_t P0 = phase_at(*b, b->hostDone, &end);
    if (!split || left == 0 || left <= end - b->hostDone) {
        if (int rc = prepare_phase(b, P0)) return rc;
        const bool onePhase = left > 0 && left <= end - b->hostDone;
        b->hostDone += left;
        for (BatchClass& k : b->cls) {
            k.pendingSweeps = left;
            k.pendingP = onePhase ? P0 : 0;
        }
        b->launches += perWindow;
        return launch_window(b, sweeps);
    }
    while (left) {
        const uint32_t P = phase_at(*b, b->hostDone, &end);
        const uint64_t piece = std::min<uint64_t>(left, end - b->hostDone);
        if (int rc = prepare_phase(b, P)) return rc;
        b->hostDone += piece;
        left -= piece;
        for (BatchClass& k : b->cls) {
            k.pendingSweeps = piece;
            k.pendingP = P;
        }
        b->launches += perWindow;
        if (int rc = launch_window(b, piece)) return rc;
    }
    return RFMF_OK;
}

}  // namespace

// Saved chain state a batch starts from (rfmf_batch_restore).
struct Resume {
    const int8_t* best_spins;
    const int64_t* cur_vals;
    const int64_t* best_vals;
    const uint64_t* sweeps_done;
};

// rfmf_batch_create, and with `resume` set rfmf_batch_restore (initial_spins
// are then the saved end spins).
static int rfmf_batch_create_impl(rfmf_context* ctx, int64_t C, const rfmf_graph* const* graphs,
                                 const double* t0s, const uint64_t* solver_seeds,
                                 const int8_t* initial_spins, int64_t nphases,
                                 const uint64_t* phases, const uint64_t* iters,
                                 const rfmf_launch_config* cfg, rfmf_batch** out,
                                 const Resume* resume = nullptr) {
    if (!ctx || !out) return fail(RFMF_ERR_INVALID, "ctx/out is NULL");
    *out = nullptr;
    host_alloc_point();
    if (C <= 0 || C > (int64_t(1) << 30)) return fail(RFMF_ERR_INVALID, "nchains=%lld", (long long)C);
    if (!graphs || !t0s || !solver_seeds || !initial_spins)
        return fail(RFMF_ERR_INVALID, "NULL per-chain array");
    if (nphases < 0 || (nphases > 0 && (!phases || !iters)))
        return fail(RFMF_ERR_INVALID, "bad phases/iters");
    rfmf_launch_config dflt{};
    const rfmf_launch_config& c = cfg ? *cfg : dflt;
    if (c.threads_per_chain && c.threads_per_chain != 32 && c.threads_per_chain != 64 &&
        c.threads_per_chain != 128 && c.threads_per_chain != 256)
        return fail(RFMF_ERR_INVALID, "threads_per_chain must be 0, 32, 64, 128 or 256");
    if (c.gain_width != 0 && c.gain_width != 1 && c.gain_width != 4)
        return fail(RFMF_ERR_INVALID, "gain_width must be 0, 1 or 4");
    if (c.csr_format < 0 || c.csr_format > 4) return fail(RFMF_ERR_INVALID, "csr_format must be 0..4");
    if (c.score_path < 0 || c.score_path > 2) return fail(RFMF_ERR_INVALID, "score_path must be 0..2");
    const int64_t totalAll = rfmf_total_steps(nphases, iters);   // src/host_common.cpp:196-210
    if (totalAll < 0) return fail(RFMF_ERR_CAPACITY, "iters total more than 10^12 sweeps");
    uint64_t total = 0, maxP = 0;
    for (int64_t p = 0; p < nphases; ++p) {
        if (phases[p] > 0x7FFFFFFFull) return fail(RFMF_ERR_CAPACITY, "phase P too large");
        if (phases[p]) { total += iters[p]; maxP = std::max<uint64_t>(maxP, phases[p]); }
    }
    for (int64_t i = 0; i < C; ++i) {
        if (!graphs[i] || graphs[i]->ctx != ctx) return fail(RFMF_ERR_INVALID, "graph %lld invalid", (long long)i);
        if (graphs[i]->n == 0) return fail(RFMF_ERR_INVALID, "chain %lld: graph has no vertices", (long long)i);
        if (!(t0s[i] > 0.0)) return fail(RFMF_ERR_INVALID, "t0s[%lld] must be > 0", (long long)i);
    }
    CU(cudaSetDevice(ctx->device));

    auto b = std::unique_ptr<rfmf_batch>(new (std::nothrow) rfmf_batch());
    if (!b) return fail(RFMF_ERR_NOMEM, "host allocation failed");
    b->ctxHold.set(ctx);
    b->ctx = ctx;
    b->C = C;
    b->total = total;
    b->phaseP.assign(static_cast<size_t>(nphases), 0u);
    b->phaseIters.assign(iters, iters + nphases);
    for (int64_t p = 0; p < nphases; ++p) b->phaseP[p] = static_cast<uint32_t>(phases[p]);

    // Graph table (distinct graphs in first-use order).
    std::map<const rfmf_graph*, int> gidx;
    b->graphOfChain.resize(C);
    for (int64_t i = 0; i < C; ++i) {
        auto it = gidx.find(graphs[i]);
        if (it == gidx.end()) {
            it = gidx.emplace(graphs[i], static_cast<int>(b->glist.size())).first;
            b->glist.push_back(graphs[i]);
            b->graphHolds.add(graphs[i]);
        }
        b->graphOfChain[i] = it->second;
    }
    const size_t G = b->glist.size();
    std::vector<std::vector<int32_t>> chainsOfGraph(G);
    for (int64_t i = 0; i < C; ++i) chainsOfGraph[b->graphOfChain[i]].push_back(static_cast<int32_t>(i));

    // Launch class of every graph.  Score path: the int32 kernel path packs
    // each score with its block iteration into one int (compact key), so it
    // needs (betaMax * B + max|gum| + 1) * 2^kb < 2^31 at every chain's
    // (t0, B, n); otherwise the exact int64 path (the reference's two-pass
    // route, src/anneal_kernels.cu:348-378).  Either way the winners are the
    // reference's.
    using Key = std::tuple<int, int, int, int>;   // dbytes, fmt, W, s64
    std::map<Key, int> classOf;
    std::vector<int> graphClass(G);
    for (size_t gi = 0; gi < G; ++gi) {
        const rfmf_graph* g = b->glist[gi];
        const int dbytes = c.gain_width ? c.gain_width : (g->B <= 127 ? 1 : 4);
        if (dbytes == 1 && g->B > 127)
            return fail(RFMF_ERR_INVALID, "int8 gains need max weighted degree <= 127 (B=%lld)", (long long)g->B);
        const int pmaxG = static_cast<int>(std::max<uint64_t>(1, std::min<uint64_t>(maxP, static_cast<uint64_t>(g->n))));
        const int64_t perSm = (b->C + ctx->sms - 1) / std::max(ctx->sms, 1);
        // Kernel variant, CSR format and chains resident per SM of this graph
        // at Wc warps per chain.
        struct Pick {
            bool s64 = false;
            int fmt = kCsrGlobal;
            int64_t resident = 0;
        };
        auto pick = [&](int Wc, Pick& pk) -> int {
            pk = Pick{};
            pk.s64 = (c.score_path == 2);
            if (!pk.s64) {
                for (int32_t ch : chainsOfGraph[gi])
                    if (!compact_key_safe(static_cast<int64_t>(total), t0s[ch], g->B, key_bits(g->n, 32 * Wc))) {
                        pk.s64 = true;
                        break;
                    }
                if (pk.s64 && c.score_path == 1)
                    return fail(RFMF_ERR_INVALID, "int32 scores would overflow for this (t0, B, sweeps)");
            }
            const int64_t chainB = chain_layout(static_cast<int>(g->n), static_cast<int>((g->n + 31) / 32), pmaxG,
                                                Wc, dbytes).total;
            // A shared-memory CSR pays only while it leaves room for the chains
            // a CTA should hold: about 8 warps, fewer when the graph has fewer
            // chains or the batch fewer than that per SM.  Otherwise its rows
            // are walked in HBM (L2-resident) and the CTA holds more chains.
            const int64_t kWant = std::max<int64_t>(
                1, std::min<int64_t>({static_cast<int64_t>(chainsOfGraph[gi].size()),
                                      static_cast<int64_t>(std::max(1, 8 / Wc)), perSm}));
            auto fits = [&](int f) {
                cudaFuncAttributes fa{};
                const int64_t dynMax = dyn_smem_max(ctx, kernel_ptr(dbytes, f, pk.s64), fa);
                return dynMax > 0 &&
                       static_cast<int64_t>(kSmemHeader) + csr_bytes(g, f) + kWant * chainB <= dynMax;
            };
            if (c.csr_format == 1) {
                if (!g->unit16) return fail(RFMF_ERR_INVALID, "unit16 CSR needs |w| == 1 and n <= 32768");
                pk.fmt = kCsrUnit16;
            } else if (c.csr_format == 2) {
                if (!g->packed32) return fail(RFMF_ERR_INVALID, "packed32 CSR needs |w| < 2^15 and n <= 65536");
                pk.fmt = kCsrPacked32;
            } else if (c.csr_format == 0) {
                if (g->unit16 && fits(kCsrUnit16)) pk.fmt = kCsrUnit16;
                else if (g->packed32 && fits(kCsrPacked32)) pk.fmt = kCsrPacked32;
            }
            // Walked in HBM: the most compact entries the graph has, unless
            // the 8-byte pairs are asked for.
            if (pk.fmt == kCsrGlobal && c.csr_format != 4) pk.fmt = hbm_format(g);
            cudaFuncAttributes fa{};
            const int64_t dynMax = dyn_smem_max(ctx, kernel_ptr(dbytes, pk.fmt, pk.s64), fa);
            const int64_t room = dynMax - static_cast<int64_t>(kSmemHeader) -
                                 (csr_in_hbm(pk.fmt) ? 0 : static_cast<int64_t>(csr_bytes(g, pk.fmt)));
            const int64_t warpCap = std::min(16 / Wc, Wc > 1 ? 15 : 16);
            pk.resident = std::max<int64_t>(0, std::min<int64_t>({perSm, warpCap, room / chainB}));
            return RFMF_OK;
        };
        int W = choose_warps(static_cast<int>(g->n), c, b->C, ctx->sms);
        Pick pk;
        if (int rc = pick(W, pk)) return rc;
        // When shared memory (not the chain count) keeps an SM's chains from
        // all being resident, wider chains fill the idle warp slots: widen
        // while that raises the warps resident per SM (GB300, 2432 chains:
        // ER n = 5000 d = 5 169 -> 216 M chain-steps/s at two warps, random
        // tree n = 10000 106 -> 112 at four).  Only within about two waves of
        // one-warp chains per SM: deeper queues keep every warp slot busy
        // anyway and one warp per chain does more per slot (512 graphs x 64
        // chains: 1.52e8 -> 1.44e8 when widened).
        if (c.threads_per_chain == 0 && perSm <= 32) {
            while (W < kMaxAutoWarps && pk.resident < perSm) {
                Pick wider;
                if (int rc = pick(2 * W, wider)) return rc;
                if (2 * W * wider.resident <= W * pk.resident) break;
                W *= 2;
                pk = wider;
            }
        }
        const bool s64 = pk.s64;
        const int fmt = pk.fmt;
        const Key key{dbytes, fmt, W, s64 ? 1 : 0};
        auto it = classOf.find(key);
        if (it == classOf.end()) {
            it = classOf.emplace(key, static_cast<int>(b->cls.size())).first;
            b->cls.emplace_back();
            BatchClass& k = b->cls.back();
            k.dbytes = dbytes;
            k.fmt = fmt;
            k.warps = W;
            k.score64 = s64;
            k.pmax = static_cast<int>(std::max<uint64_t>(1, maxP));
        }
        graphClass[gi] = it->second;
        BatchClass& k = b->cls[it->second];
        k.graphs.push_back(static_cast<int>(gi));
        k.chainsOf.push_back(chainsOfGraph[gi]);
    }
    // A shared-memory class's CTA holds the class's largest CSR beside K
    // chains sized for its largest graph.  While that leaves room for fewer
    // chains than a CTA should hold (as above, over the class), the graph
    // demanding the most moves to the HBM class of the same key, so that a
    // few large graphs do not shrink every CTA of the class.
    if (c.csr_format == 0) {
        const int64_t perSm = (b->C + ctx->sms - 1) / std::max(ctx->sms, 1);
        for (size_t ci = 0; ci < b->cls.size(); ++ci) {
            if (csr_in_hbm(b->cls[ci].fmt)) continue;
            cudaFuncAttributes fa{};
            const int64_t dynMax =
                dyn_smem_max(ctx, kernel_ptr(b->cls[ci].dbytes, b->cls[ci].fmt, b->cls[ci].score64), fa);
            while (!b->cls[ci].graphs.empty()) {
                BatchClass& k = b->cls[ci];
                auto chainOf = [&](int64_t n) {
                    const int ni = static_cast<int>(n);
                    return static_cast<int64_t>(
                        chain_layout(ni, (ni + 31) / 32, std::max(1, std::min(k.pmax, ni)), k.warps, k.dbytes).total);
                };
                int64_t maxN = 0, maxCsr = 0, maxCh = 0;
                for (size_t q = 0; q < k.graphs.size(); ++q) {
                    const rfmf_graph* g = b->glist[k.graphs[q]];
                    maxN = std::max(maxN, g->n);
                    maxCsr = std::max<int64_t>(maxCsr, csr_bytes(g, k.fmt));
                    maxCh = std::max<int64_t>(maxCh, static_cast<int64_t>(k.chainsOf[q].size()));
                }
                const int64_t kWant =
                    std::max<int64_t>(1, std::min<int64_t>({maxCh, static_cast<int64_t>(std::max(1, 8 / k.warps)), perSm}));
                if (dynMax > 0 && static_cast<int64_t>(kSmemHeader) + maxCsr + kWant * chainOf(maxN) <= dynMax) break;
                size_t worst = 0;
                int64_t worstD = -1;
                for (size_t q = 0; q < k.graphs.size(); ++q) {
                    const rfmf_graph* g = b->glist[k.graphs[q]];
                    const int64_t d = static_cast<int64_t>(csr_bytes(g, k.fmt)) + kWant * chainOf(g->n);
                    if (d > worstD) { worstD = d; worst = q; }
                }
                const int gi = k.graphs[worst];
                std::vector<int32_t> chains = std::move(k.chainsOf[worst]);
                k.graphs.erase(k.graphs.begin() + static_cast<std::ptrdiff_t>(worst));
                k.chainsOf.erase(k.chainsOf.begin() + static_cast<std::ptrdiff_t>(worst));
                const int dbytes = k.dbytes, W = k.warps, pmax = k.pmax;
                const bool s64 = k.score64;
                const int hf = hbm_format(b->glist[gi]);
                const Key gk{dbytes, hf, W, s64 ? 1 : 0};
                auto it = classOf.find(gk);
                if (it == classOf.end()) {
                    it = classOf.emplace(gk, static_cast<int>(b->cls.size())).first;
                    b->cls.emplace_back();     // invalidates k
                    BatchClass& h = b->cls.back();
                    h.dbytes = dbytes;
                    h.fmt = hf;
                    h.warps = W;
                    h.score64 = s64;
                    h.pmax = pmax;
                }
                b->cls[it->second].graphs.push_back(gi);
                b->cls[it->second].chainsOf.push_back(std::move(chains));
                graphClass[gi] = it->second;
            }
        }
        // Drop classes emptied by the moves and renumber.
        std::vector<int> remap(b->cls.size(), -1);
        std::vector<BatchClass> kept;
        for (size_t ci = 0; ci < b->cls.size(); ++ci) {
            if (b->cls[ci].graphs.empty()) continue;
            remap[ci] = static_cast<int>(kept.size());
            kept.push_back(std::move(b->cls[ci]));
        }
        b->cls = std::move(kept);
        for (size_t gi = 0; gi < G; ++gi) graphClass[gi] = remap[graphClass[gi]];
    }
    const bool exact = b->cls.size() > 1;
    for (BatchClass& k : b->cls) {
        int rc = plan_class(*b, k, c, exact);
        if (rc == RFMF_ERR_CAPACITY && !csr_in_hbm(k.fmt) && c.csr_format == 0) {
            // The class's largest CSR and largest n together do not fit: its
            // graphs (all of them 16-bit or all 32-bit capable) walk HBM.
            k.fmt = (k.fmt == kCsrUnit16) ? kCsrGlobal16 : kCsrGlobal32;
            rc = plan_class(*b, k, c, exact);
        }
        if (rc) return rc;
    }
    b->cfg = c;
    for (BatchClass& k : b->cls) k.baseWarps = k.warps;
    if (b->cls.size() == 1 && b->cls[0].graphs.size() == 1 && c.threads_per_chain == 0 &&
        2 * b->cls[0].warps <= kMaxLatencyWarps && b->C * 2 * b->cls[0].warps <= int64_t(16) * ctx->sms) {
        for (uint32_t P : b->phaseP)
            b->phaseWarps = b->phaseWarps || (P && wide_phase(b->glist[b->cls[0].graphs[0]], P));
    }
    {
        uint64_t end = 0;
        const uint32_t P0 = phase_at(*b, 0, &end);
        for (BatchClass& k : b->cls) build_items(*b, k, P0);
    }

    // Beta tables over the executed sweeps: the context's device copies,
    // shared with every other batch, call and request at the same (t0, sweeps).
    ChainBeta cb;
    int rc = acquire_beta(ctx, t0s, C, static_cast<int64_t>(total), cb);
    if (rc) return rc;
    b->betaRefs = cb.refs;

    std::vector<DevGraph> hg(G);
    for (size_t gi = 0; gi < G; ++gi) {
        const rfmf_graph* g = b->glist[gi];
        const int fmt = b->cls[graphClass[gi]].fmt;
        hg[gi].offsets = g->offsets.as<uint32_t>();
        hg[gi].edges = g->edges.as<Edge>();
        hg[gi].compact = compact_entries(g, fmt);
        hg[gi].n = static_cast<int32_t>(g->n);
        hg[gi].words = static_cast<int32_t>((g->n + 31) / 32);
        hg[gi].wsum2 = g->wsum2;
        hg[gi].offBytes = g->offBytes;
        hg[gi].entBytes = csr_bytes(g, fmt) ? csr_bytes(g, fmt) - g->offBytes : 0;
    }

    // Per-chain spin words and initial state.
    b->chainN.resize(C);
    b->chainWordOff.resize(C + 1);
    b->chainWordOff[0] = 0;
    for (int64_t i = 0; i < C; ++i) {
        b->chainN[i] = graphs[i]->n;
        b->chainWordOff[i + 1] = b->chainWordOff[i] + (graphs[i]->n + 31) / 32;
    }
    b->words = b->chainWordOff[C];
    std::vector<uint32_t> bits(static_cast<size_t>(std::max<int64_t>(b->words, 1)), 0u);
    std::vector<uint32_t> bestBits;
    {
        size_t sp = 0;
        for (int64_t i = 0; i < C; ++i) {
            pack_spins(initial_spins + sp, b->chainN[i], bits.data() + b->chainWordOff[i]);
            sp += static_cast<size_t>(b->chainN[i]);
        }
    }
    if (resume) {
        bestBits.assign(bits.size(), 0u);
        size_t sp = 0;
        uint64_t least = total;
        for (int64_t i = 0; i < C; ++i) {
            if (resume->sweeps_done[i] > total)
                return fail(RFMF_ERR_INVALID, "chain %lld: %llu sweeps done, the schedule has %llu", (long long)i,
                            (unsigned long long)resume->sweeps_done[i], (unsigned long long)total);
            least = std::min<uint64_t>(least, resume->sweeps_done[i]);
            pack_spins(resume->best_spins + sp, b->chainN[i], bestBits.data() + b->chainWordOff[i]);
            sp += static_cast<size_t>(b->chainN[i]);
        }
        b->hostDone = least;
    }

    // Device buffers.
    if ((rc = b->dGraphs.alloc(hg.size() * sizeof(DevGraph)))) return rc;
    if ((rc = b->dScheds.alloc(sizeof(DevSchedule)))) return rc;
    if ((rc = b->dChains.alloc(C * sizeof(DevChain)))) return rc;
    if ((rc = b->dPhaseP.alloc(std::max<int64_t>(nphases, 1) * sizeof(uint32_t)))) return rc;
    if ((rc = b->dPhaseIters.alloc(std::max<int64_t>(nphases, 1) * sizeof(uint64_t)))) return rc;
    if ((rc = b->dBits.alloc(bits.size() * sizeof(uint32_t)))) return rc;
    if ((rc = b->dBest.alloc(bits.size() * sizeof(uint32_t)))) return rc;
    for (BatchClass& k : b->cls) {
        const int64_t kc = static_cast<int64_t>(k.order.size());
        if ((rc = k.dItems.alloc(kc * sizeof(DevItem))) || (rc = k.dOrder.alloc(kc * sizeof(int32_t))) ||
            (rc = k.dItemNs.alloc(kc * sizeof(uint64_t))) || (rc = k.dCtl.alloc(4 * sizeof(int32_t))))
            return rc;
    }
    if (b->cls.size() > 1) {
        CU(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
        for (BatchClass& k : b->cls) {
            CU(cudaStreamCreateWithFlags(&k.stream, cudaStreamNonBlocking));
            CU(cudaEventCreateWithFlags(&k.done, cudaEventDisableTiming));
        }
    }

    std::vector<uint32_t> hp(std::max<int64_t>(nphases, 1), 0);
    std::vector<uint64_t> hi(std::max<int64_t>(nphases, 1), 0);
    for (int64_t p = 0; p < nphases; ++p) { hp[p] = static_cast<uint32_t>(phases[p]); hi[p] = iters[p]; }
    DevSchedule hs{b->dPhaseP.as<uint32_t>(), b->dPhaseIters.as<uint64_t>(), static_cast<int32_t>(nphases), 0};
    std::vector<DevChain> hc(C);
    for (int64_t i = 0; i < C; ++i) {
        DevChain& d = hc[i];
        d.graph = static_cast<int32_t>(b->graphOfChain[i]);
        d.sched = 0;
        d.solverSeed = solver_seeds[i];
        d.betaEnd = cb.end[i];
        d.betaVal = cb.val[i];
        d.betaRuns = cb.runs[i];
        d.spinBits = b->dBits.as<uint32_t>() + b->chainWordOff[i];
        d.bestBits = b->dBest.as<uint32_t>() + b->chainWordOff[i];
        d.cur = resume ? resume->cur_vals[i] : kUnsetCut;
        d.best = resume ? resume->best_vals[i] : kUnsetCut;
        d.sweepsDone = resume ? resume->sweeps_done[i] : 0;
        d.sweepsTotal = total;
        d.improvedSweeps = 0;
    }

    cudaStream_t st = ctx->stream;
    CU(cudaMemcpyAsync(b->dGraphs.p, hg.data(), hg.size() * sizeof(DevGraph), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(b->dScheds.p, &hs, sizeof hs, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(b->dChains.p, hc.data(), C * sizeof(DevChain), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(b->dPhaseP.p, hp.data(), hp.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(b->dPhaseIters.p, hi.data(), hi.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(b->dBits.p, bits.data(), bits.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(b->dBest.p, resume ? bestBits.data() : bits.data(), bits.size() * sizeof(uint32_t),
                       cudaMemcpyHostToDevice, st));
    for (BatchClass& k : b->cls) {
        if ((rc = upload_items(*b, k))) return rc;
        CU(cudaMemsetAsync(k.dCtl.p, 0, 4 * sizeof(int32_t), st));
        DevLaunch& L = k.L;
        L.graphs = b->dGraphs.as<DevGraph>();
        L.scheds = b->dScheds.as<DevSchedule>();
        L.chains = b->dChains.as<DevChain>();
        L.items = k.dItems.as<DevItem>();
        L.order = k.dOrder.as<int32_t>();
        L.nitems = k.nitems;
        L.itemNs = k.dItemNs.as<uint64_t>();
        L.ngraphs = static_cast<int32_t>(G);
        L.nscheds = 1;
        L.queue = k.dCtl.as<int32_t>();
        L.error = k.dCtl.as<int32_t>() + 1;
        L.errorItem = k.dCtl.as<int32_t>() + 2;
        L.window = 0;
        std::memcpy(L.lut, ctx->lut, sizeof L.lut);
    }
    CU(cudaStreamSynchronize(st));
    if (resume) {
        // The checkpoint's cut values against its spins, recomputed on the
        // device (cutValueCsr, src/max_cut.cpp:5-15).
        DevBuf d;
        if ((rc = d.alloc(static_cast<size_t>(2 * C) * sizeof(int64_t)))) return rc;
        CU(launch_chain_cuts(b->dChains.as<DevChain>(), b->dGraphs.as<DevGraph>(), static_cast<int>(C), 0,
                             d.as<int64_t>(), st));
        CU(launch_chain_cuts(b->dChains.as<DevChain>(), b->dGraphs.as<DevGraph>(), static_cast<int>(C), 1,
                             d.as<int64_t>() + C, st));
        std::vector<int64_t> cuts(static_cast<size_t>(2 * C));
        CU(cudaMemcpyAsync(cuts.data(), d.p, cuts.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        for (int64_t i = 0; i < C; ++i)
            if (cuts[i] != resume->cur_vals[i] || cuts[C + i] != resume->best_vals[i])
                return fail(RFMF_ERR_INVALID,
                            "checkpoint of chain %lld: cut values %lld / %lld, its spins give %lld / %lld",
                            (long long)i, (long long)resume->cur_vals[i], (long long)resume->best_vals[i],
                            (long long)cuts[i], (long long)cuts[C + i]);
    }
    *out = b.release();
    return RFMF_OK;
}

static int rfmf_batch_run_impl(rfmf_batch* b, uint64_t sweeps) {
    if (!b) return fail(RFMF_ERR_INVALID, "batch is NULL");
    CU(cudaSetDevice(b->ctx->device));
    return enqueue_run(b, sweeps);
}

// Captures `launches` windows of `sweeps` sweeps as one CUDA graph and
// replays it.  Work items are sized for the phase the batch is in before
// each replay; when that changes them (a new phase), the graph is captured
// again (the launches' item counts are part of it).
static int rfmf_batch_run_graph_impl(rfmf_batch* b, uint64_t sweeps, int launches, int replays) {
    if (!b || launches <= 0 || replays < 0) return fail(RFMF_ERR_INVALID, "bad arguments");
    CU(cudaSetDevice(b->ctx->device));
    auto capture = [&]() -> int {
        if (b->graphExec) { cudaGraphExecDestroy(b->graphExec); b->graphExec = nullptr; }
        cudaGraph_t graph = nullptr;
        CU(cudaStreamBeginCapture(b->ctx->stream, cudaStreamCaptureModeThreadLocal));
        int rc = RFMF_OK;
        for (int i = 0; i < launches && rc == RFMF_OK; ++i) rc = enqueue_run(b, sweeps, true);
        const cudaError_t ec = cudaStreamEndCapture(b->ctx->stream, &graph);
        if (rc != RFMF_OK) { if (graph) cudaGraphDestroy(graph); return rc; }
        if (ec != cudaSuccess) return fail(RFMF_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ec));
        const cudaError_t ei = cudaGraphInstantiate(&b->graphExec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) { b->graphExec = nullptr; return fail(RFMF_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(ei)); }
        b->graphSweeps = sweeps;
        b->graphLaunches = launches;
        return RFMF_OK;
    };
    auto sized = [&](bool& changed) {
        uint64_t end = 0;
        return prepare_phase(b, phase_at(*b, b->hostDone, &end), &changed);
    };
    bool changed = false;
    if (int rc = sized(changed)) return rc;
    if (!b->graphExec || b->graphSweeps != sweeps || b->graphLaunches != launches || changed)
        if (int rc = capture()) return rc;
    for (int r = 0; r < replays; ++r) {
        if (r > 0) {
            if (int rc = sized(changed)) return rc;
            if (changed)
                if (int rc = capture()) return rc;
        }
        CU(cudaGraphLaunch(b->graphExec, b->ctx->stream));
        b->launches += static_cast<int64_t>(launches) * static_cast<int64_t>(b->cls.size());
        for (int i = 0; i < launches; ++i)
            b->hostDone += std::min<uint64_t>(sweeps, b->total - std::min(b->total, b->hostDone));
    }
    for (BatchClass& k : b->cls) k.pendingSweeps = 0;   // item times of replays are not harvested
    return RFMF_OK;
}

static int rfmf_batch_run_timed_impl(rfmf_batch* b, uint64_t sweeps, float* ms) {
    if (!b || !ms) return fail(RFMF_ERR_INVALID, "batch/ms is NULL");
    CU(cudaSetDevice(b->ctx->device));
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    int rc = RFMF_OK;
    if (cudaEventRecord(e0, b->ctx->stream) != cudaSuccess) rc = fail(RFMF_ERR_CUDA, "event record failed");
    if (!rc) rc = enqueue_run(b, sweeps);
    if (!rc && cudaEventRecord(e1, b->ctx->stream) != cudaSuccess) rc = fail(RFMF_ERR_CUDA, "event record failed");
    if (!rc) rc = rfmf_batch_synchronize(b);
    if (!rc && cudaEventElapsedTime(ms, e0, e1) != cudaSuccess) rc = fail(RFMF_ERR_CUDA, "event elapsed failed");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

static int rfmf_batch_stats_impl(rfmf_batch* b, uint64_t* improved_sweeps) {
    if (!b || !improved_sweeps) return fail(RFMF_ERR_INVALID, "batch/out is NULL");
    CU(cudaSetDevice(b->ctx->device));
    CU(cudaStreamSynchronize(b->ctx->stream));
    std::vector<DevChain> hc(b->C);
    CU(cudaMemcpy(hc.data(), b->dChains.p, b->C * sizeof(DevChain), cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < b->C; ++i) improved_sweeps[i] = hc[i].improvedSweeps;
    return RFMF_OK;
}

static int rfmf_batch_synchronize_impl(rfmf_batch* b) {
    if (!b) return fail(RFMF_ERR_INVALID, "batch is NULL");
    CU(cudaSetDevice(b->ctx->device));
    CU(cudaStreamSynchronize(b->ctx->stream));
    for (BatchClass& k : b->cls) {
        if (int rc = harvest_item_times(*b, k)) return rc;
        int32_t ctl[4];
        CU(cudaMemcpy(ctl, k.dCtl.p, sizeof ctl, cudaMemcpyDeviceToHost));
        if (ctl[1] != kDevOk) {
            static const char* names[] = {"ok", "carried cut value disagrees with the spins",
                                          "beta table shorter than the window", "bad work item",
                                          "CSR bulk copy did not complete (do not reuse this context)",
                                          "device CSR failed its check"};
            const int code = ctl[1];
            return fail(RFMF_ERR_DEVICE, "device error %d (%s) on chain %d", code,
                        (code >= 0 && code < 6) ? names[code] : "?", ctl[2]);
        }
    }
    return RFMF_OK;
}

static int rfmf_batch_read_impl(rfmf_batch* b, int8_t* end_spins, int8_t* best_spins,
                               int64_t* cur_vals, int64_t* best_vals, uint64_t* sweeps_done) {
    if (!b) return fail(RFMF_ERR_INVALID, "batch is NULL");
    host_alloc_point();
    int rc = rfmf_batch_synchronize(b);
    if (rc) return rc;
    std::vector<DevChain> hc(b->C);
    CU(cudaMemcpy(hc.data(), b->dChains.p, b->C * sizeof(DevChain), cudaMemcpyDeviceToHost));
    auto unpack = [&](const DevBuf& src, int8_t* dst) -> int {
        std::vector<uint32_t> w(static_cast<size_t>(std::max<int64_t>(b->words, 1)));
        CU(cudaMemcpy(w.data(), src.p, w.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        size_t sp = 0;
        for (int64_t i = 0; i < b->C; ++i) {
            unpack_spins(w.data() + b->chainWordOff[i], b->chainN[i], dst + sp);
            sp += static_cast<size_t>(b->chainN[i]);
        }
        return RFMF_OK;
    };
    if (end_spins && (rc = unpack(b->dBits, end_spins))) return rc;
    if (best_spins && (rc = unpack(b->dBest, best_spins))) return rc;
    for (int64_t i = 0; i < b->C; ++i) {
        if (cur_vals) cur_vals[i] = hc[i].cur;
        if (best_vals) best_vals[i] = hc[i].best;
        if (sweeps_done) sweeps_done[i] = hc[i].sweepsDone;
    }
    return RFMF_OK;
}

static int rfmf_batch_cuts_impl(rfmf_batch* b, int which, int64_t* out_cuts) {
    if (!b || !out_cuts || (which != 0 && which != 1)) return fail(RFMF_ERR_INVALID, "bad arguments");
    if (int rc = rfmf_batch_synchronize(b)) return rc;
    DevBuf d;
    if (int rc = d.alloc(b->C * sizeof(int64_t))) return rc;
    CU(launch_chain_cuts(b->dChains.as<DevChain>(), b->dGraphs.as<DevGraph>(), static_cast<int>(b->C), which,
                         d.as<int64_t>(), b->ctx->stream));
    CU(cudaMemcpyAsync(out_cuts, d.p, b->C * sizeof(int64_t), cudaMemcpyDeviceToHost, b->ctx->stream));
    CU(cudaStreamSynchronize(b->ctx->stream));
    return RFMF_OK;
}

static int rfmf_batch_partitions_impl(rfmf_batch* b, int which, char* out, int64_t stride) {
    if (!b || !out || (which != 0 && which != 1)) return fail(RFMF_ERR_INVALID, "bad arguments");
    int64_t maxN = 0;
    for (int64_t n : b->chainN) maxN = std::max(maxN, n);
    if (stride < maxN) return fail(RFMF_ERR_INVALID, "stride %lld < largest n %lld", (long long)stride, (long long)maxN);
    if (int rc = rfmf_batch_synchronize(b)) return rc;
    // chunks of chains bounded to ~256 MB of device staging and to 65535
    // chains (one grid row per chain: gridDim.y is at most 65535)
    const int64_t per = std::max<int64_t>(
        1, std::min<int64_t>(std::min<int64_t>(b->C, 65535), (int64_t(256) << 20) / std::max<int64_t>(stride, 1)));
    DevBuf d;
    if (int rc = d.alloc(static_cast<size_t>(per * stride))) return rc;
    for (int64_t c0 = 0; c0 < b->C; c0 += per) {
        const int64_t cnt = std::min(per, b->C - c0);
        CU(cudaMemsetAsync(d.p, 0, static_cast<size_t>(cnt * stride), b->ctx->stream));
        CU(launch_chain_partitions(b->dChains.as<DevChain>(), b->dGraphs.as<DevGraph>(), static_cast<int>(c0),
                                   static_cast<int>(cnt), static_cast<int>(maxN), which, d.as<char>(), stride,
                                   b->ctx->stream));
        CU(cudaMemcpyAsync(out + c0 * stride, d.p, static_cast<size_t>(cnt * stride), cudaMemcpyDeviceToHost,
                           b->ctx->stream));
        CU(cudaStreamSynchronize(b->ctx->stream));
    }
    return RFMF_OK;
}

extern "C" int rfmf_batch_info(const rfmf_batch* b, rfmf_batch_plan* out) {
    if (!b || !out) return fail(RFMF_ERR_INVALID, "batch/out is NULL");
    // Shape of the class with the most chains; grid and items over all classes.
    const BatchClass* big = &b->cls[0];
    size_t most = 0;
    int grid = 0, items = 0;
    bool balanced = true;
    for (const BatchClass& k : b->cls) {
        if (k.order.size() > most) { most = k.order.size(); big = &k; }
        grid += k.grid;
        items += k.nitems;
        balanced = balanced && (k.balanced || k.graphs.size() < 2);   // one graph: nothing to balance
    }
    out->nchains = b->C;
    out->total_sweeps = b->total;
    out->threads_per_chain = 32 * big->warps;
    out->chains_per_cta = big->K;
    out->grid = grid;
    out->items = items;
    out->score64 = big->score64 ? 1 : 0;
    out->csr_format = big->fmt + 1;
    out->gain_width = big->dbytes;
    out->smem_bytes = static_cast<int>(big->smem);
    out->balanced = balanced ? 1 : 0;
    out->launch_classes = static_cast<int>(b->cls.size());
    out->launches = b->launches;
    return RFMF_OK;
}

extern "C" int rfmf_batch_destroy(rfmf_batch* b) {
    if (!b) return RFMF_OK;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    delete b;
    return RFMF_OK;
}

// ---------------------------------------------------------------- anneal
static int rfmf_anneal_impl(rfmf_context* ctx, const rfmf_graph* g, int64_t max_weighted_deg,
                           int64_t C, const int8_t* initial_spins, const double* t0s,
                           int64_t nphases, const uint64_t* phases, const uint64_t* iters,
                           const uint64_t* solver_seeds, const rfmf_launch_config* cfg,
                           int8_t* end_spins, int8_t* best_spins, float* kernel_ms,
                           int64_t* kernel_best_vals, int64_t* kernel_final_vals) {
    if (!ctx || !g) return fail(RFMF_ERR_INVALID, "ctx/graph is NULL");
    if (C <= 0 || !initial_spins || !t0s || !solver_seeds)
        return fail(RFMF_ERR_INVALID, "annealGpu needs C > 0 and per-chain arrays");
    (void)max_weighted_deg;   // the graph carries B; accepted for signature parity
    const int64_t n = g->n;
    if (kernel_ms) *kernel_ms = 0.0f;
    if (n == 0 || nphases == 0) {
        // src/anneal_kernels.cu:856-868: inputs returned, cutValueCsr values.
        for (int64_t c = 0; c < C; ++c) {
            if (end_spins) std::memcpy(end_spins + c * n, initial_spins + c * n, n);
            if (best_spins) std::memcpy(best_spins + c * n, initial_spins + c * n, n);
            if (kernel_best_vals) kernel_best_vals[c] = 0;
            if (kernel_final_vals) kernel_final_vals[c] = 0;
        }
        if (n > 0) {
            // Cut values from the device copy of the CSR.
            std::vector<uint32_t> ho(n + 1);
            std::vector<Edge> he(g->m * 2);
            CU(cudaMemcpy(ho.data(), g->offsets.p, (n + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost));
            if (!he.empty()) CU(cudaMemcpy(he.data(), g->edges.p, he.size() * sizeof(Edge), cudaMemcpyDeviceToHost));
            for (int64_t c = 0; c < C; ++c) {
                int64_t v = 0;
                const int8_t* s = initial_spins + c * n;
                for (int64_t x = 0; x < n; ++x)
                    for (uint32_t i = ho[x]; i < ho[x + 1]; ++i)
                        if (he[i].col > x && s[x] != s[he[i].col]) v += he[i].w;
                if (kernel_best_vals) kernel_best_vals[c] = v;
                if (kernel_final_vals) kernel_final_vals[c] = v;
            }
        }
        return RFMF_OK;
    }
    std::vector<const rfmf_graph*> gs(C, g);
    rfmf_batch* b = nullptr;
    int rc = rfmf_batch_create(ctx, C, gs.data(), t0s, solver_seeds, initial_spins, nphases,
                               phases, iters, cfg, &b);
    if (rc) return rc;
    std::unique_ptr<rfmf_batch, int (*)(rfmf_batch*)> guard(b, rfmf_batch_destroy);
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    CU(cudaEventRecord(e0, ctx->stream));
    rc = enqueue_run(b, b->total);
    if (rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
    CU(cudaEventRecord(e1, ctx->stream));
    rc = rfmf_batch_synchronize(b);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (kernel_ms) *kernel_ms = ms;
    return rfmf_batch_read(b, end_spins, best_spins, kernel_final_vals, kernel_best_vals, nullptr);
}

// ---------------------------------------------------------------- autotune
namespace {

// The batch shape a tuned plan is cached under: per distinct graph its n, m,
// B and chain count (sorted), the schedule, the trial length and the knobs
// the caller fixed.
std::string tune_key(int64_t C, const rfmf_graph* const* graphs, int64_t nphases, const uint64_t* phases,
                     const uint64_t* iters, uint64_t trial, const rfmf_launch_config& base) {
    std::map<const rfmf_graph*, int64_t> count;
    for (int64_t i = 0; i < C; ++i) ++count[graphs[i]];
    std::vector<std::tuple<int64_t, int64_t, int64_t, int64_t>> shape;
    for (const auto& kv : count) shape.emplace_back(kv.first->n, kv.first->m, kv.first->B, kv.second);
    std::sort(shape.begin(), shape.end());
    std::string key;
    char buf[96];
    for (const auto& t : shape) {
        std::snprintf(buf, sizeof buf, "g%lld,%lld,%lld,%lld;", (long long)std::get<0>(t), (long long)std::get<1>(t),
                      (long long)std::get<2>(t), (long long)std::get<3>(t));
        key += buf;
    }
    for (int64_t p = 0; p < nphases; ++p) {
        std::snprintf(buf, sizeof buf, "p%llu,%llu;", (unsigned long long)phases[p], (unsigned long long)iters[p]);
        key += buf;
    }
    std::snprintf(buf, sizeof buf, "t%llu;k%d,%d,%d,%d,%d", (unsigned long long)trial, base.threads_per_chain,
                  base.csr_format, base.gain_width, base.score_path, base.chains_per_cta);
    return key + buf;
}

}  // namespace

static int rfmf_autotune_impl(rfmf_context* ctx, int64_t C, const rfmf_graph* const* graphs, const double* t0s,
                              const uint64_t* solver_seeds, const int8_t* initial_spins, int64_t nphases,
                              const uint64_t* phases, const uint64_t* iters, uint64_t trial_sweeps,
                              const rfmf_launch_config* base, rfmf_launch_config* best, int* ncand,
                              rfmf_launch_config* cand, float* cand_us) {
    if (!ctx || !best || !graphs || C <= 0 || nphases < 0 || (nphases > 0 && (!phases || !iters)))
        return fail(RFMF_ERR_INVALID, "bad arguments");
    const rfmf_launch_config b0 = base ? *base : rfmf_launch_config{};
    const uint64_t trial = trial_sweeps ? trial_sweeps : 2048;
    const std::string key = tune_key(C, graphs, nphases, phases, iters, trial, b0);
    auto report = [&](const rfmf_context::TunedPlan& t) {
        *best = t.best;
        if (ncand) {
            const int cap = *ncand;
            *ncand = static_cast<int>(t.us.size());
            for (int k = 0; k < static_cast<int>(t.us.size()) && k < cap; ++k) {
                if (cand_us) cand_us[k] = t.us[k];
                if (cand) cand[k] = t.cand[k];
            }
        }
    };
    {
        std::lock_guard<std::mutex> lk(ctx->tuneMu);
        auto it = ctx->tuneCache.find(key);
        if (it != ctx->tuneCache.end()) {
            report(it->second);
            return RFMF_OK;
        }
    }
    // The schedule compressed to `trial` sweeps, every phase keeping its share.
    uint64_t total = 0;
    for (int64_t p = 0; p < nphases; ++p)
        if (phases[p]) total += iters[p];
    std::vector<uint64_t> it(static_cast<size_t>(std::max<int64_t>(nphases, 1)), 0);
    uint64_t tsum = 0;
    for (int64_t p = 0; p < nphases; ++p) {
        if (!phases[p] || !iters[p] || !total) continue;
        it[p] = std::max<uint64_t>(1, static_cast<uint64_t>(std::llround(static_cast<double>(trial) * iters[p] / total)));
        tsum += it[p];
    }
    if (!tsum) {   // nothing to time: the automatic plan
        *best = b0;
        if (ncand) *ncand = 0;
        return RFMF_OK;
    }
    rfmf_context::TunedPlan tp;
    for (int w : {0, 32, 64, 128}) {
        if (b0.threads_per_chain && w != 0) continue;
        for (int f : {0, 3}) {
            if (b0.csr_format && f != 0) continue;
            rfmf_launch_config c = b0;
            if (w) c.threads_per_chain = w;
            if (f) c.csr_format = f;
            tp.cand.push_back(c);
        }
    }
    int firstErr = RFMF_OK;
    std::string firstMsg;
    float bestUs = -1.0f;
    for (const rfmf_launch_config& c : tp.cand) {
        float fastest = -1.0f;
        for (int rep = 0; rep < 2; ++rep) {
            // Two windows of the trial schedule: the first warms the plan up
            // and teaches it the graphs' costs (which size its work items),
            // the second is timed.
            rfmf_batch* tb = nullptr;
            int rc = rfmf_batch_create(ctx, C, graphs, t0s, solver_seeds, initial_spins, nphases, phases,
                                       it.data(), &c, &tb);
            float ms = 0.0f, warm = 0.0f;
            if (rc == RFMF_OK) rc = rfmf_batch_run_timed(tb, tsum, &warm);
            if (tb) {
                rfmf_batch_destroy(tb);
                tb = nullptr;
            }
            if (rc == RFMF_OK)
                rc = rfmf_batch_create(ctx, C, graphs, t0s, solver_seeds, initial_spins, nphases, phases,
                                       it.data(), &c, &tb);
            if (rc == RFMF_OK) rc = rfmf_batch_run_timed(tb, tsum, &ms);
            if (tb) rfmf_batch_destroy(tb);
            if (rc != RFMF_OK) {
                if (!firstErr) { firstErr = rc; firstMsg = rfmf_last_error(); }
                if (rc != RFMF_ERR_CAPACITY && rc != RFMF_ERR_INVALID) return rc;   // a CUDA failure is not a plan's fault
                fastest = -1.0f;
                break;
            }
            if (fastest < 0.0f || ms < fastest) fastest = ms;
        }
        const float us = fastest < 0.0f ? -1.0f
                                        : static_cast<float>(fastest * 1e3 / (static_cast<double>(C) * tsum));
        tp.us.push_back(us);
        if (us >= 0.0f && (bestUs < 0.0f || us < bestUs)) {
            bestUs = us;
            tp.best = c;
        }
    }
    if (bestUs < 0.0f) return fail(firstErr ? firstErr : RFMF_ERR_CAPACITY, "no candidate plan runs: %s", firstMsg.c_str());
    {
        std::lock_guard<std::mutex> lk(ctx->tuneMu);
        ctx->tuneCache[key] = tp;
    }
    report(tp);
    return RFMF_OK;
}

// C ABI entry points: no C++ exception crosses the boundary.
extern "C" int rfmf_autotune(rfmf_context* ctx, int64_t nchains, const rfmf_graph* const* graphs,
                             const double* t0s, const uint64_t* solver_seeds, const int8_t* initial_spins,
                             int64_t nphases, const uint64_t* phases, const uint64_t* iters,
                             uint64_t trial_sweeps, const rfmf_launch_config* base,
                             rfmf_launch_config* best, int* ncand, rfmf_launch_config* cand,
                             float* cand_us) {
    try {
        return rfmf_autotune_impl(ctx, nchains, graphs, t0s, solver_seeds, initial_spins, nphases, phases, iters,
                                  trial_sweeps, base, best, ncand, cand, cand_us);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_autotune");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_autotune");
    }
}

extern "C" int rfmf_batch_create(rfmf_context* ctx, int64_t C, const rfmf_graph* const* graphs,
                                 const double* t0s, const uint64_t* solver_seeds,
                                 const int8_t* initial_spins, int64_t nphases,
                                 const uint64_t* phases, const uint64_t* iters,
                                 const rfmf_launch_config* cfg, rfmf_batch** out) {
    try {
        return rfmf_batch_create_impl(ctx, C, graphs, t0s, solver_seeds, initial_spins, nphases, phases, iters, cfg, out);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_batch_create");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_batch_create");
    }
}

extern "C" int rfmf_batch_restore(rfmf_context* ctx, int64_t nchains, const rfmf_graph* const* graphs,
                                  const double* t0s, const uint64_t* solver_seeds, int64_t nphases,
                                  const uint64_t* phases, const uint64_t* iters,
                                  const rfmf_launch_config* cfg, const int8_t* end_spins,
                                  const int8_t* best_spins, const int64_t* cur_vals,
                                  const int64_t* best_vals, const uint64_t* sweeps_done, rfmf_batch** out) {
    try {
        if (!best_spins || !cur_vals || !best_vals || !sweeps_done)
            return rfmf::fail(RFMF_ERR_INVALID, "NULL checkpoint array");
        const Resume r{best_spins, cur_vals, best_vals, sweeps_done};
        return rfmf_batch_create_impl(ctx, nchains, graphs, t0s, solver_seeds, end_spins, nphases, phases,
                                      iters, cfg, out, &r);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_batch_restore");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_batch_restore");
    }
}

extern "C" int rfmf_batch_read(rfmf_batch* b, int8_t* end_spins, int8_t* best_spins,
                               int64_t* cur_vals, int64_t* best_vals, uint64_t* sweeps_done) {
    try {
        return rfmf_batch_read_impl(b, end_spins, best_spins, cur_vals, best_vals, sweeps_done);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_batch_read");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_batch_read");
    }
}

extern "C" int rfmf_batch_run(rfmf_batch* b, uint64_t sweeps) {
    try {
        return rfmf_batch_run_impl(b, sweeps);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_batch_run");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_batch_run");
    }
}

extern "C" int rfmf_batch_run_graph(rfmf_batch* b, uint64_t sweeps, int launches, int replays) {
    try {
        return rfmf_batch_run_graph_impl(b, sweeps, launches, replays);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_batch_run_graph");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_batch_run_graph");
    }
}

extern "C" int rfmf_batch_run_timed(rfmf_batch* b, uint64_t sweeps, float* ms) {
    try {
        return rfmf_batch_run_timed_impl(b, sweeps, ms);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_batch_run_timed");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_batch_run_timed");
    }
}

extern "C" int rfmf_batch_stats(rfmf_batch* b, uint64_t* improved_sweeps) {
    try {
        return rfmf_batch_stats_impl(b, improved_sweeps);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_batch_stats");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_batch_stats");
    }
}

extern "C" int rfmf_debug_plan_items(int ngraphs, const int64_t* chains, int max_chains_per_cta,
                                     int warps, const double* level_ns, int64_t slots, int* out_chains_per_item) {
    if (ngraphs < 1 || !chains || max_chains_per_cta < 1 || warps < 1 || !level_ns || slots < 1 ||
        !out_chains_per_item)
        return fail(RFMF_ERR_INVALID, "bad arguments");
    try {
        const int levels = sched_level(max_chains_per_cta, warps);
        std::vector<std::vector<ItemCand>> cand(static_cast<size_t>(ngraphs));
        std::vector<int64_t> ch(chains, chains + ngraphs);
        for (int q = 0; q < ngraphs; ++q)
            for (int K = 1; K <= max_chains_per_cta; ++K) {
                if (K < max_chains_per_cta && sched_level(K + 1, warps) == sched_level(K, warps)) continue;
                cand[q].push_back({K, level_ns[static_cast<size_t>(q) * levels + sched_level(K, warps) - 1]});
            }
        std::vector<int> kg;
        if (!balance_items(cand, ch, slots, kg)) return fail(RFMF_ERR_CAPACITY, "no item sizes fit %lld slots", (long long)slots);
        std::copy(kg.begin(), kg.end(), out_chains_per_item);
        return RFMF_OK;
    } catch (const std::bad_alloc&) {
        return fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_debug_plan_items");
    }
}

extern "C" int rfmf_batch_debug_set_cut(rfmf_batch* b, int64_t chain, int64_t cut) {
    if (!b || chain < 0 || chain >= b->C) return rfmf::fail(RFMF_ERR_INVALID, "batch is NULL or chain out of range");
    CU(cudaSetDevice(b->ctx->device));
    CU(cudaStreamSynchronize(b->ctx->stream));
    char* rec = static_cast<char*>(b->dChains.p) + chain * static_cast<int64_t>(sizeof(DevChain));
    CU(cudaMemcpy(rec + offsetof(DevChain, cur), &cut, sizeof cut, cudaMemcpyHostToDevice));
    return RFMF_OK;
}

extern "C" int rfmf_batch_synchronize(rfmf_batch* b) {
    try {
        return rfmf_batch_synchronize_impl(b);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_batch_synchronize");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_batch_synchronize");
    }
}

extern "C" int rfmf_batch_cuts(rfmf_batch* b, int which, int64_t* out_cuts) {
    try {
        return rfmf_batch_cuts_impl(b, which, out_cuts);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_batch_cuts");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_batch_cuts");
    }
}

extern "C" int rfmf_batch_partitions(rfmf_batch* b, int which, char* out, int64_t stride) {
    try {
        return rfmf_batch_partitions_impl(b, which, out, stride);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_batch_partitions");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_batch_partitions");
    }
}

extern "C" int rfmf_anneal(rfmf_context* ctx, const rfmf_graph* g, int64_t max_weighted_deg,
                           int64_t C, const int8_t* initial_spins, const double* t0s,
                           int64_t nphases, const uint64_t* phases, const uint64_t* iters,
                           const uint64_t* solver_seeds, const rfmf_launch_config* cfg,
                           int8_t* end_spins, int8_t* best_spins, float* kernel_ms,
                           int64_t* kernel_best_vals, int64_t* kernel_final_vals) {
    try {
        return rfmf_anneal_impl(ctx, g, max_weighted_deg, C, initial_spins, t0s, nphases, phases,
                                iters, solver_seeds, cfg, end_spins, best_spins, kernel_ms,
                                kernel_best_vals, kernel_final_vals);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_anneal");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_anneal");
    }
}
