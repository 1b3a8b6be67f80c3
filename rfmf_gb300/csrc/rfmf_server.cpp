// rfmf_server.cpp -- request server over the persistent annealing kernel.
//
// The reference serves one annealGpu call per process launch (main.cu:83-85
// -> src/anneal_kernels.cu:835-884): allocate, copy in, one kernel, copy out,
// free.  Here requests (one annealGpu call's worth of chains each) arrive at
// any time and share the GPU: a worker thread runs launch windows of
// `window_sweeps` sweeps over every admitted chain (continuous batching).
// Between windows it admits queued requests (device state allocated and
// uploaded once), and harvests finished ones (spins and cuts copied out, device
// state freed).  Chains never interact, so every request's results equal a
// standalone rfmf_anneal of its inputs bit for bit, whatever else shares its
// windows.
//
// Launch classes: chains whose kernel variant (gain width, CSR format, score
// path) and warps per chain agree go into one launch per window; a window
// issues one launch per class present, in order on the server's stream.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "rfmf_host.h"

using namespace rfmf;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    GraphHolds graphHold;   // first member: released last
    uint64_t id = 0;
    const rfmf_graph* g = nullptr;
    int64_t C = 0, n = 0, words = 0;
    std::vector<double> t0s;
    std::vector<uint64_t> seeds;
    std::vector<uint32_t> phaseP;
    std::vector<uint64_t> phaseIters;
    uint64_t total = 0;
    int pmax = 1;
    std::vector<uint32_t> initBits;   // C * words
    ChainBeta beta;                   // the context's shared device beta tables
    // launch class
    int dbytes = 1, fmt = kCsrGlobal, W = 1;
    bool s64 = false;
    int64_t devBytes = 0;             // request_device_bytes: counted against max_device_bytes
    // device state (worker thread only)
    DevBuf dBits, dBest, dPhaseP, dPhaseIters;
    int64_t slot0 = -1;               // first of C consecutive chain slots
    int graphSlot = -1, schedSlot = -1;
    uint64_t done = 0;                // sweeps completed by every chain
    bool launched = false;
    bool cancel = false;              // rfmf_cancel on a running request (under the server mutex)
    // status (under the server mutex)
    int state = RFMF_REQ_QUEUED;
    int error = RFMF_OK;
    std::string msg;
    double submitS = 0, startS = 0, finishS = 0;
    uint64_t doneShown = 0;
    // results
    std::vector<uint32_t> endBits, bestBits;
    std::vector<int64_t> cur, best;
};

using ReqPtr = std::shared_ptr<Request>;

// First-fit allocator of consecutive chain slots.
struct SlotRanges {
    std::map<int64_t, int64_t> freeRanges;   // start -> length
    int64_t cap = 0;
    int64_t take(int64_t len) {
        for (auto it = freeRanges.begin(); it != freeRanges.end(); ++it) {
            if (it->second >= len) {
                const int64_t s = it->first, l = it->second;
                freeRanges.erase(it);
                if (l > len) freeRanges[s + len] = l - len;
                return s;
            }
        }
        return -1;
    }
    void give(int64_t s, int64_t len) {
        auto nx = freeRanges.lower_bound(s);
        if (nx != freeRanges.end() && s + len == nx->first) {
            len += nx->second;
            nx = freeRanges.erase(nx);
        }
        if (nx != freeRanges.begin()) {
            auto pv = std::prev(nx);
            if (pv->first + pv->second == s) {
                pv->second += len;
                return;
            }
        }
        freeRanges[s] = len;
    }
    void grow(int64_t newCap) {
        give(cap, newCap - cap);
        cap = newCap;
    }
};

struct ClassKey {
    int dbytes, fmt, W;
    bool s64;
    bool operator<(const ClassKey& o) const {
        return std::tie(dbytes, fmt, W, s64) < std::tie(o.dbytes, o.fmt, o.W, o.s64);
    }
};

}  // namespace

struct rfmf_server {
    rfmf::CtxHold ctxHold;   // first member: released last
    rfmf_context* ctx = nullptr;
    uint64_t window = 4096;
    int64_t maxChains = int64_t(1) << 20;
    int64_t maxDeviceBytes = 0;        // 0: no limit
    rfmf_launch_config lc{};
    Clock::time_point t0;

    std::mutex mu;
    std::condition_variable cvWork, cvDone;
    bool stop = false;
    uint64_t nextId = 1;
    std::deque<ReqPtr> queue;
    std::map<uint64_t, ReqPtr> all;    // every request not yet released
    int64_t runningChains = 0;
    int64_t runningBytes = 0;          // request_device_bytes of the admitted requests
    rfmf_server_stats stats{};


    // worker-owned
    std::thread worker;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // Launch classes of one window run side by side: one stream and one
    // completion event per class, forked from and joined back to `stream`.
    cudaEvent_t fork = nullptr;
    std::vector<cudaStream_t> clsStreams;
    std::vector<cudaEvent_t> clsDone;
    std::vector<ReqPtr> running;
    SlotRanges slots;
    DevBuf dChains, dGraphs, dScheds, dItems, dOrder, dCtl;
    int64_t graphCap = 0, schedCap = 0, itemCap = 0;
    std::map<const rfmf_graph*, std::pair<int, int>> graphSlotOf;   // slot, users
    std::vector<int> freeGraphSlots, freeSchedSlots;
    int graphSlots = 0, schedSlots = 0;
    std::map<const void*, bool> attrSet;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

int64_t grow_to(int64_t have, int64_t need) {
    int64_t c = std::max<int64_t>(have, 64);
    while (c < need) c *= 2;
    return c;
}

// Reallocates a device table to `cap` elements of `esz` bytes, keeping the
// first `keep` elements (no launch is in flight: worker thread, between
// windows).
int grow_table(rfmf_server* s, DevBuf& buf, size_t esz, int64_t keep, int64_t cap) {
    DevBuf nb;
    if (int rc = nb.alloc(static_cast<size_t>(cap) * esz)) return rc;
    if (keep > 0 && buf.p)
        CU(cudaMemcpyAsync(nb.p, buf.p, static_cast<size_t>(keep) * esz, cudaMemcpyDeviceToDevice,
                           s->stream));
    CU(cudaStreamSynchronize(s->stream));
    std::swap(buf.p, nb.p);
    std::swap(buf.bytes, nb.bytes);
    return RFMF_OK;
}

int ensure_attr(rfmf_server* s, const void* k) {
    if (s->attrSet.count(k)) return RFMF_OK;
    cudaFuncAttributes fa{};
    CU(cudaFuncGetAttributes(&fa, k));
    CU(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            s->ctx->smemOptin - static_cast<int>(fa.sharedSizeBytes)));
    CU(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                            cudaSharedmemCarveoutMaxShared));
    s->attrSet[k] = true;
    return RFMF_OK;
}

DevGraph dev_graph(const rfmf_graph* g, int fmt) {
    DevGraph d{};
    d.offsets = g->offsets.as<uint32_t>();
    d.edges = g->edges.as<Edge>();
    d.compact = compact_entries(g, fmt);
    d.n = static_cast<int32_t>(g->n);
    d.words = static_cast<int32_t>((g->n + 31) / 32);
    d.wsum2 = g->wsum2;
    d.offBytes = g->offBytes;
    d.entBytes = (fmt == kCsrUnit16) ? g->u16Bytes : (fmt == kCsrPacked32 ? g->p32Bytes : 0);
    return d;
}

uint32_t csr_bytes(const rfmf_graph* g, int fmt) {
    if (fmt == kCsrUnit16) return g->offBytes + g->u16Bytes;
    if (fmt == kCsrPacked32) return g->offBytes + g->p32Bytes;
    return 0;
}

// Device state of a newly admitted request (worker thread).
int admit(rfmf_server* s, Request& r) {
    host_alloc_point();
    const int64_t CW = r.C * r.words;
    int rc;
    if ((rc = r.dBits.alloc(CW * 4)) || (rc = r.dBest.alloc(CW * 4))) return rc;
    const size_t np = std::max<size_t>(r.phaseP.size(), 1);
    if ((rc = r.dPhaseP.alloc(np * 4)) || (rc = r.dPhaseIters.alloc(np * 8))) return rc;
    cudaStream_t st = s->stream;
    CU(cudaMemcpyAsync(r.dBits.p, r.initBits.data(), CW * 4, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(r.dBest.p, r.initBits.data(), CW * 4, cudaMemcpyHostToDevice, st));
    if (!r.phaseP.empty()) {
        CU(cudaMemcpyAsync(r.dPhaseP.p, r.phaseP.data(), r.phaseP.size() * 4, cudaMemcpyHostToDevice, st));
        CU(cudaMemcpyAsync(r.dPhaseIters.p, r.phaseIters.data(), r.phaseIters.size() * 8,
                           cudaMemcpyHostToDevice, st));
    }

    // chain slots
    r.slot0 = s->slots.take(r.C);
    if (r.slot0 < 0) {
        const int64_t keep = s->slots.cap;
        const int64_t cap = grow_to(s->slots.cap, s->slots.cap + r.C);
        if ((rc = grow_table(s, s->dChains, sizeof(DevChain), keep, cap))) return rc;
        s->slots.grow(cap);
        r.slot0 = s->slots.take(r.C);
    }
    // graph slot (shared by the requests on one graph)
    auto gi = s->graphSlotOf.find(r.g);
    if (gi != s->graphSlotOf.end()) {
        ++gi->second.second;
        r.graphSlot = gi->second.first;
    } else {
        int slot;
        if (!s->freeGraphSlots.empty()) {
            slot = s->freeGraphSlots.back();
            s->freeGraphSlots.pop_back();
        } else {
            slot = s->graphSlots++;
            if (slot >= s->graphCap) {
                const int64_t cap = grow_to(s->graphCap, slot + 1);
                if ((rc = grow_table(s, s->dGraphs, sizeof(DevGraph), s->graphCap, cap))) return rc;
                s->graphCap = cap;
            }
        }
        const DevGraph dg = dev_graph(r.g, r.fmt);
        CU(cudaMemcpyAsync(s->dGraphs.as<DevGraph>() + slot, &dg, sizeof dg, cudaMemcpyHostToDevice, st));
        s->graphSlotOf[r.g] = {slot, 1};
        r.graphSlot = slot;
    }
    // schedule slot
    if (!s->freeSchedSlots.empty()) {
        r.schedSlot = s->freeSchedSlots.back();
        s->freeSchedSlots.pop_back();
    } else {
        r.schedSlot = s->schedSlots++;
        if (r.schedSlot >= s->schedCap) {
            const int64_t cap = grow_to(s->schedCap, r.schedSlot + 1);
            if ((rc = grow_table(s, s->dScheds, sizeof(DevSchedule), s->schedCap, cap))) return rc;
            s->schedCap = cap;
        }
    }
    const DevSchedule ds{r.dPhaseP.as<uint32_t>(), r.dPhaseIters.as<uint64_t>(),
                         static_cast<int32_t>(r.phaseP.size()), 0};
    CU(cudaMemcpyAsync(s->dScheds.as<DevSchedule>() + r.schedSlot, &ds, sizeof ds,
                       cudaMemcpyHostToDevice, st));
    // chain records
    std::vector<DevChain> hc(r.C);
    for (int64_t c = 0; c < r.C; ++c) {
        DevChain& d = hc[c];
        d = DevChain{};
        d.graph = r.graphSlot;
        d.sched = r.schedSlot;
        d.solverSeed = r.seeds[c];
        d.betaEnd = r.beta.end[c];
        d.betaVal = r.beta.val[c];
        d.betaRuns = r.beta.runs[c];
        d.spinBits = r.dBits.as<uint32_t>() + c * r.words;
        d.bestBits = r.dBest.as<uint32_t>() + c * r.words;
        d.cur = kUnsetCut;
        d.best = kUnsetCut;
        d.sweepsDone = 0;
        d.sweepsTotal = r.total;
        d.improvedSweeps = 0;
    }
    CU(cudaMemcpyAsync(s->dChains.as<DevChain>() + r.slot0, hc.data(), r.C * sizeof(DevChain),
                       cudaMemcpyHostToDevice, st));
    CU(cudaStreamSynchronize(st));
    r.initBits.clear();
    r.initBits.shrink_to_fit();
    return RFMF_OK;
}

// Releases a request's device state and slots (worker thread).
void release(rfmf_server* s, Request& r) {
    if (r.slot0 >= 0) s->slots.give(r.slot0, r.C);
    r.slot0 = -1;
    if (r.graphSlot >= 0) {
        auto gi = s->graphSlotOf.find(r.g);
        if (gi != s->graphSlotOf.end() && --gi->second.second == 0) {
            s->freeGraphSlots.push_back(gi->second.first);
            s->graphSlotOf.erase(gi);
        }
        r.graphSlot = -1;
    }
    if (r.schedSlot >= 0) s->freeSchedSlots.push_back(r.schedSlot);
    r.schedSlot = -1;
    r.beta = ChainBeta{};   // drops this request's holds on the shared beta tables
    for (DevBuf* b : {&r.dBits, &r.dBest, &r.dPhaseP, &r.dPhaseIters}) {
        if (b->p) cudaFree(b->p);
        b->p = nullptr;
        b->bytes = 0;
    }
}

// Copies a finished request's state to the host (worker thread).
int harvest(rfmf_server* s, Request& r) {
    host_alloc_point();
    const int64_t CW = r.C * r.words;
    r.endBits.resize(CW);
    r.bestBits.resize(CW);
    r.cur.resize(r.C);
    r.best.resize(r.C);
    cudaStream_t st = s->stream;
    const DevChain* base = s->dChains.as<DevChain>() + r.slot0;
    CU(cudaMemcpyAsync(r.endBits.data(), r.dBits.p, CW * 4, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(r.bestBits.data(), r.dBest.p, CW * 4, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpy2DAsync(r.cur.data(), sizeof(int64_t),
                         reinterpret_cast<const char*>(base) + offsetof(DevChain, cur),
                         sizeof(DevChain), sizeof(int64_t), r.C, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpy2DAsync(r.best.data(), sizeof(int64_t),
                         reinterpret_cast<const char*>(base) + offsetof(DevChain, best),
                         sizeof(DevChain), sizeof(int64_t), r.C, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return RFMF_OK;
}

// One window over the running requests: one launch per launch class, the
// classes side by side on their own streams (a class that fills only part
// of the GPU no longer leaves the rest idle while the next one waits).
// Each class has its own work items, item order and queue/error words.
int run_window(rfmf_server* s, int64_t& launches, float& ms) {
    std::map<ClassKey, std::vector<Request*>> classes;
    for (const ReqPtr& r : s->running) classes[ClassKey{r->dbytes, r->fmt, r->W, r->s64}].push_back(r.get());
    launches = 0;
    ms = 0.0f;
    const int ncls = static_cast<int>(classes.size());
    int64_t need = 0;
    for (const ReqPtr& r : s->running) need += r->C;
    if (need > s->itemCap) {
        const int64_t cap = grow_to(s->itemCap, need);
        int rc;
        if ((rc = grow_table(s, s->dItems, sizeof(DevItem), 0, cap)) ||
            (rc = grow_table(s, s->dOrder, sizeof(int32_t), 0, cap)))
            return rc;
        s->itemCap = cap;
    }
    if (s->dCtl.bytes < static_cast<size_t>(16) * ncls) {
        DevBuf nb;
        if (int rc = nb.alloc(static_cast<size_t>(16) * grow_to(ncls, ncls))) return rc;
        std::swap(s->dCtl.p, nb.p);
        std::swap(s->dCtl.bytes, nb.bytes);
    }
    while (static_cast<int>(s->clsStreams.size()) < ncls) {
        cudaStream_t st = nullptr;
        cudaEvent_t ev = nullptr;
        CU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
            cudaStreamDestroy(st);
            return fail(RFMF_ERR_CUDA, "event creation failed");
        }
        s->clsStreams.push_back(st);
        s->clsDone.push_back(ev);
    }

    // Plan every class on the host; their items and orders go up together.
    struct Plan {
        ClassKey k;
        DevLaunch L;
        int grid, threads;
        size_t smem;
    };
    std::vector<Plan> plans;
    std::vector<DevItem> items;
    std::vector<int32_t> order;
    int ci = 0;
    for (auto& kv : classes) {
        const ClassKey& k = kv.first;
        std::vector<Request*>& reqs = kv.second;
        int maxN = 0, maxWords = 0, pmax = 1;
        uint32_t csrB = 0;
        for (Request* r : reqs) {
            maxN = std::max<int>(maxN, static_cast<int>(r->n));
            maxWords = std::max<int>(maxWords, static_cast<int>(r->words));
            pmax = std::max(pmax, r->pmax);
            csrB = std::max(csrB, csr_bytes(r->g, k.fmt));
        }
        const void* kern = kernel_ptr(k.dbytes, k.fmt, k.s64);
        if (int rc = ensure_attr(s, kern)) return rc;
        cudaFuncAttributes fa{};
        CU(cudaFuncGetAttributes(&fa, kern));
        const int64_t dynMax = s->ctx->smemOptin - static_cast<int64_t>(fa.sharedSizeBytes);
        const uint32_t chainB = chain_layout(maxN, maxWords, pmax, k.W, k.dbytes).total;
        const int kCap = std::min(std::min(16 / k.W, k.W > 1 ? 15 : 16), fa.maxThreadsPerBlock / (32 * k.W));
        const int64_t room = dynMax - kSmemHeader - csrB;
        const int Kmax = room > 0 ? static_cast<int>(std::min<int64_t>(kCap, room / chainB)) : 0;
        if (Kmax < 1)
            return fail(RFMF_ERR_CAPACITY, "launch class needs %u B CSR + %u B per chain", csrB, chainB);
        int occ = 0, Kshape = Kmax;
        for (; Kshape >= 1; --Kshape) {
            const size_t smem = kSmemHeader + csrB + static_cast<size_t>(Kshape) * chainB;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32 * k.W * Kshape, smem) !=
                cudaSuccess) {
                cudaGetLastError();
                occ = 0;
            }
            if (occ > 0) break;
        }
        if (Kshape < 1) return fail(RFMF_ERR_CAPACITY, "no resident configuration for a launch class");
        // Chains grouped by graph; items of K chains, K the smallest that
        // keeps all items resident (else Kshape).
        std::map<int, std::vector<int32_t>> byGraph;
        for (Request* r : reqs)
            for (int64_t c = 0; c < r->C; ++c)
                byGraph[r->graphSlot].push_back(static_cast<int32_t>(r->slot0 + c));
        const int64_t slotsRes = static_cast<int64_t>(occ) * s->ctx->sms;
        auto items_for = [&](int K) {
            int64_t it = 0;
            for (auto& g : byGraph) it += (static_cast<int64_t>(g.second.size()) + K - 1) / K;
            return it;
        };
        int K = 1;
        while (K < Kshape && items_for(K) > slotsRes) ++K;
        const size_t item0 = items.size(), order0 = order.size();
        for (auto& g : byGraph) {
            const std::vector<int32_t>& ch = g.second;
            for (size_t i = 0; i < ch.size(); i += K) {
                const int cnt = static_cast<int>(std::min<size_t>(K, ch.size() - i));
                items.push_back(DevItem{g.first, static_cast<int32_t>(order.size() - order0), cnt, 0});
                for (int q = 0; q < cnt; ++q) order.push_back(ch[i + q]);
            }
        }
        Plan pl{};
        pl.k = k;
        DevLaunch& L = pl.L;
        L.graphs = s->dGraphs.as<DevGraph>();
        L.scheds = s->dScheds.as<DevSchedule>();
        L.chains = s->dChains.as<DevChain>();
        L.items = s->dItems.as<DevItem>() + item0;
        L.order = s->dOrder.as<int32_t>() + order0;
        L.nitems = static_cast<int32_t>(items.size() - item0);
        L.ngraphs = s->graphSlots;
        L.nscheds = s->schedSlots;
        L.warpsPerChain = k.W;
        L.chainsPerCta = Kshape;
        L.maxN = maxN;
        L.maxWords = maxWords;
        L.pmax = pmax;
        L.csrBytes = csrB;
        L.chainBytes = chainB;
        L.queue = s->dCtl.as<int32_t>() + 4 * ci;
        L.error = L.queue + 1;
        L.errorItem = L.queue + 2;
        L.itemNs = nullptr;
        L.window = s->window;
        std::memcpy(L.lut, s->ctx->lut, sizeof L.lut);
        pl.grid = static_cast<int>(std::min<int64_t>(L.nitems, slotsRes));
        pl.threads = 32 * k.W * Kshape;
        pl.smem = kSmemHeader + csrB + static_cast<size_t>(Kshape) * chainB;
        plans.push_back(pl);
        ++ci;
    }
    CU(cudaMemcpyAsync(s->dItems.p, items.data(), items.size() * sizeof(DevItem), cudaMemcpyHostToDevice,
                       s->stream));
    CU(cudaMemcpyAsync(s->dOrder.p, order.data(), order.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                       s->stream));
    CU(cudaMemsetAsync(s->dCtl.p, 0, static_cast<size_t>(16) * ncls, s->stream));
    CU(cudaEventRecord(s->ev0, s->stream));
    const bool fork = ncls > 1;
    if (fork) CU(cudaEventRecord(s->fork, s->stream));
    for (int c = 0; c < ncls; ++c) {
        const Plan& pl = plans[c];
        cudaStream_t st = fork ? s->clsStreams[c] : s->stream;
        if (fork) CU(cudaStreamWaitEvent(st, s->fork, 0));
        CU(launch_anneal(pl.L, pl.k.dbytes, pl.k.fmt, pl.k.s64, pl.grid, pl.threads, pl.smem, st));
        if (fork) {
            CU(cudaEventRecord(s->clsDone[c], st));
            CU(cudaStreamWaitEvent(s->stream, s->clsDone[c], 0));
        }
        ++launches;
    }
    CU(cudaEventRecord(s->ev1, s->stream));
    std::vector<int32_t> ctl(static_cast<size_t>(4) * std::max(ncls, 1), 0);
    CU(cudaMemcpyAsync(ctl.data(), s->dCtl.p, static_cast<size_t>(16) * ncls, cudaMemcpyDeviceToHost, s->stream));
    CU(cudaStreamSynchronize(s->stream));
    CU(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    for (int c = 0; c < ncls; ++c)
        if (ctl[4 * c + 1] != 0)
            return fail(RFMF_ERR_CUDA, "device error %d in a server window (item %d)", ctl[4 * c + 1],
                        ctl[4 * c + 2]);
    return RFMF_OK;
}

void fail_request(Request& r, int code, const std::string& msg, double t) {
    r.state = RFMF_REQ_FAILED;
    r.error = code ? code : RFMF_ERR_CUDA;
    r.msg = msg;
    r.finishS = t;
}

void worker_loop(rfmf_server* s);

// The worker: any host exception (allocation failure) fails the requests it
// holds instead of terminating the process.
void worker_main(rfmf_server* s) {
    cudaSetDevice(s->ctx->device);
    for (;;) {
        try {
            worker_loop(s);
            return;
        } catch (...) {
            std::lock_guard<std::mutex> lk(s->mu);
            const double t = s->now();
            for (ReqPtr& r : s->running) {
                fail_request(*r, RFMF_ERR_NOMEM, "host allocation failed in the server worker", t);
                release(s, *r);
            }
            s->running.clear();
            s->runningChains = 0;
            s->runningBytes = 0;
            s->cvDone.notify_all();
        }
    }
}

// Host allocation failures inside admission, a window or a harvest become
// a status, so the request in hand is failed instead of lost.
template <class F>
int nomem_safe(F&& f, const char* where) {
    try {
        return f();
    } catch (const std::bad_alloc&) {
        return fail(RFMF_ERR_NOMEM, "host allocation failed %s", where);
    }
}

// Running requests that rfmf_cancel marked leave at this window boundary:
// device state and slots freed, state CANCELLED (server mutex held, worker
// thread, no launch in flight).
void drop_cancelled(rfmf_server* s) {
    bool any = false;
    for (size_t i = 0; i < s->running.size();) {
        Request& r = *s->running[i];
        if (!r.cancel) { ++i; continue; }
        release(s, r);
        s->runningChains -= r.C;
        s->runningBytes -= r.devBytes;
        r.state = RFMF_REQ_CANCELLED;
        r.finishS = s->now();
        s->running.erase(s->running.begin() + static_cast<std::ptrdiff_t>(i));
        any = true;
    }
    if (any) s->cvDone.notify_all();
}

void worker_loop(rfmf_server* s) {
    for (;;) {
        std::vector<ReqPtr> admitNow;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cvWork.wait(lk, [&] { return s->stop || !s->queue.empty() || !s->running.empty(); });
            if (s->stop) break;
            drop_cancelled(s);
            while (!s->queue.empty() &&
                   admits(s->runningChains, s->runningBytes, s->queue.front()->C,
                          s->queue.front()->devBytes, s->maxChains, s->maxDeviceBytes)) {
                ReqPtr r = s->queue.front();
                s->queue.pop_front();
                s->runningChains += r->C;
                s->runningBytes += r->devBytes;
                admitNow.push_back(r);
            }
        }
        const auto w0 = Clock::now();
        for (ReqPtr& r : admitNow) {
            const int rc = nomem_safe([&] { return admit(s, *r); }, "while admitting a request");
            std::lock_guard<std::mutex> lk(s->mu);
            if (rc != RFMF_OK) {
                release(s, *r);
                s->runningChains -= r->C;
                s->runningBytes -= r->devBytes;
                fail_request(*r, rc, rfmf_last_error(), s->now());
                s->cvDone.notify_all();
            } else {
                r->state = RFMF_REQ_RUNNING;
                r->startS = s->now();
                s->running.push_back(r);
            }
        }
        if (s->running.empty()) continue;

        int64_t launches = 0;
        float ms = 0.0f;
        const int rc = nomem_safe([&] { return run_window(s, launches, ms); }, "in a launch window");
        std::vector<ReqPtr> finished;
        int64_t chainSweeps = 0;
        if (rc == RFMF_OK) {
            for (ReqPtr& r : s->running) {
                const uint64_t adv = std::min<uint64_t>(s->window, r->total - r->done);
                r->done += adv;
                r->launched = true;
                chainSweeps += static_cast<int64_t>(adv) * r->C;
                if (r->done >= r->total) finished.push_back(r);
            }
        }
        std::string err = rc == RFMF_OK ? std::string() : std::string(rfmf_last_error());
        std::vector<std::pair<ReqPtr, int>> harvested;
        for (ReqPtr& r : finished)
            harvested.push_back({r, nomem_safe([&] { return harvest(s, *r); }, "while reading results")});
        {
            std::lock_guard<std::mutex> lk(s->mu);
            const double t = s->now();
            s->stats.windows += 1;
            s->stats.launches += static_cast<uint64_t>(launches);
            s->stats.chain_sweeps += static_cast<uint64_t>(chainSweeps);
            s->stats.kernel_s += ms * 1e-3;
            s->stats.busy_s += std::chrono::duration<double>(Clock::now() - w0).count();
            for (ReqPtr& r : s->running) r->doneShown = r->done;
            if (rc != RFMF_OK) {
                for (ReqPtr& r : s->running) {
                    fail_request(*r, rc, err, t);
                    release(s, *r);
                }
                s->running.clear();
                s->runningChains = 0;
                s->runningBytes = 0;
            }
            for (auto& h : harvested) {
                Request& r = *h.first;
                if (h.second == RFMF_OK) {
                    r.state = RFMF_REQ_DONE;
                    r.finishS = t;
                } else {
                    fail_request(r, h.second, rfmf_last_error(), t);
                }
                release(s, r);
                s->runningChains -= r.C;
                s->runningBytes -= r.devBytes;
                s->running.erase(std::find(s->running.begin(), s->running.end(), h.first));
            }
            drop_cancelled(s);
            s->cvDone.notify_all();
        }
    }
    // Shut down: device state of whatever is still running.
    std::lock_guard<std::mutex> lk(s->mu);
    for (ReqPtr& r : s->running) release(s, *r);
    s->running.clear();
}

rfmf_request_status status_of(const Request& r) {
    rfmf_request_status st{};
    st.state = r.state;
    st.error = r.error;
    st.sweeps_done = r.doneShown;
    st.sweeps_total = r.total;
    st.submit_s = r.submitS;
    st.start_s = r.startS;
    st.finish_s = r.finishS;
    return st;
}

}  // namespace

static int rfmf_server_create_impl(rfmf_context* ctx, const rfmf_server_config* cfg, rfmf_server** out) {
    if (!ctx || !out) return fail(RFMF_ERR_INVALID, "ctx/out is NULL");
    *out = nullptr;
    auto s = std::unique_ptr<rfmf_server>(new (std::nothrow) rfmf_server());
    if (!s) return fail(RFMF_ERR_NOMEM, "host allocation failed");
    s->ctxHold.set(ctx);
    s->ctx = ctx;
    if (cfg) {
        if (cfg->window_sweeps) s->window = cfg->window_sweeps;
        if (cfg->max_chains < 0) return fail(RFMF_ERR_INVALID, "max_chains must be >= 0");
        if (cfg->max_chains) s->maxChains = cfg->max_chains;
        if (cfg->max_device_bytes < 0) return fail(RFMF_ERR_INVALID, "max_device_bytes must be >= 0");
        s->maxDeviceBytes = cfg->max_device_bytes;
        s->lc = cfg->launch;
    }
    const rfmf_launch_config& c = s->lc;
    if (c.threads_per_chain && c.threads_per_chain != 32 && c.threads_per_chain != 64 &&
        c.threads_per_chain != 128 && c.threads_per_chain != 256)
        return fail(RFMF_ERR_INVALID, "threads_per_chain must be 0, 32, 64, 128 or 256");
    if (c.gain_width != 0 && c.gain_width != 1 && c.gain_width != 4)
        return fail(RFMF_ERR_INVALID, "gain_width must be 0, 1 or 4");
    if (c.csr_format < 0 || c.csr_format > 4) return fail(RFMF_ERR_INVALID, "csr_format must be 0..4");
    if (c.score_path < 0 || c.score_path > 2) return fail(RFMF_ERR_INVALID, "score_path must be 0..2");
    CU(cudaSetDevice(ctx->device));
    CU(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    CU(cudaEventCreate(&s->ev0));
    CU(cudaEventCreate(&s->ev1));
    CU(cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming));
    if (int rc = s->dCtl.alloc(16)) return rc;
    s->t0 = Clock::now();
    rfmf_server* raw = s.get();
    try {
        s->worker = std::thread(worker_main, raw);
    } catch (...) {
        return fail(RFMF_ERR_NOMEM, "cannot start the worker thread");
    }
    *out = s.release();
    return RFMF_OK;
}

extern "C" int rfmf_server_destroy(rfmf_server* s) {
    if (!s) return RFMF_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cvWork.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->ctx->device);
    s->all.clear();
    s->queue.clear();
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->fork) cudaEventDestroy(s->fork);
    for (cudaEvent_t e : s->clsDone) cudaEventDestroy(e);
    for (cudaStream_t st : s->clsStreams) cudaStreamDestroy(st);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return RFMF_OK;
}

static int rfmf_submit_impl(rfmf_server* s, const rfmf_graph* g, int64_t nchains,
                           const int8_t* initial_spins, const double* t0s, int64_t nphases,
                           const uint64_t* phases, const uint64_t* iters,
                           const uint64_t* solver_seeds, uint64_t* request_id) {
    if (!s || !g || !request_id) return fail(RFMF_ERR_INVALID, "server/graph/request_id is NULL");
    if (g->ctx != s->ctx) return fail(RFMF_ERR_INVALID, "graph belongs to another context");
    if (nchains < 1) return fail(RFMF_ERR_INVALID, "nchains must be >= 1");
    if (nchains > s->maxChains)
        return fail(RFMF_ERR_CAPACITY, "request of %lld chains exceeds max_chains %lld",
                    static_cast<long long>(nchains), static_cast<long long>(s->maxChains));
    if (g->n == 0) return fail(RFMF_ERR_INVALID, "graph has no vertices");
    if (!initial_spins || !t0s || !solver_seeds || nphases < 0 || (nphases > 0 && (!phases || !iters)))
        return fail(RFMF_ERR_INVALID, "bad arguments");
    host_alloc_point();
    auto r = std::make_shared<Request>();
    r->g = g;
    r->graphHold.add(g);
    r->C = nchains;
    r->n = g->n;
    r->words = (g->n + 31) / 32;
    r->t0s.assign(t0s, t0s + nchains);
    r->seeds.assign(solver_seeds, solver_seeds + nchains);
    uint64_t total = 0, maxP = 1;
    for (int64_t p = 0; p < nphases; ++p) {
        if (phases[p] > 0x7FFFFFFFull) return fail(RFMF_ERR_CAPACITY, "phase P too large");
        if (iters[p] > kMaxTotalSteps) return fail(RFMF_ERR_CAPACITY, "iters too large");
        r->phaseP.push_back(static_cast<uint32_t>(phases[p]));
        r->phaseIters.push_back(iters[p]);
        if (phases[p]) { total += iters[p]; maxP = std::max<uint64_t>(maxP, phases[p]); }
    }
    if (total > kMaxTotalSteps) return fail(RFMF_ERR_CAPACITY, "total sweeps exceed 1e12");
    for (int64_t c = 0; c < nchains; ++c)
        if (!(t0s[c] > 0.0)) return fail(RFMF_ERR_INVALID, "t0s[%lld] must be > 0", static_cast<long long>(c));
    r->total = total;
    r->pmax = static_cast<int>(std::max<uint64_t>(1, std::min<uint64_t>(maxP, static_cast<uint64_t>(g->n))));
    // Run tables on the submitting thread, never on the worker, where
    // building or uploading them would stall the launch windows: the
    // context's device copies when another batch or request holds the same
    // (t0, sweeps), else built (from the host cache) and uploaded once.
    if (int rc = acquire_beta(s->ctx, r->t0s.data(), nchains, static_cast<int64_t>(total), r->beta))
        return rc;
    // The admission footprint counts the request's beta tables in full even
    // when it shares them with other users.
    r->devBytes = request_device_bytes(nchains, r->words, r->beta.totalRuns,
                                       static_cast<int64_t>(r->phaseP.size()));
    if (s->maxDeviceBytes && r->devBytes > s->maxDeviceBytes)
        return fail(RFMF_ERR_CAPACITY, "request needs %lld device bytes, above max_device_bytes %lld",
                    static_cast<long long>(r->devBytes), static_cast<long long>(s->maxDeviceBytes));

    // launch class
    const rfmf_launch_config& c = s->lc;
    r->dbytes = c.gain_width ? c.gain_width : (g->B <= 127 ? 1 : 4);
    if (r->dbytes == 1 && g->B > 127)
        return fail(RFMF_ERR_INVALID, "int8 gains need max weighted degree <= 127 (B=%lld)",
                    static_cast<long long>(g->B));
    // Warps per chain from the load at submission: the chains running and
    // queued, plus this request's.
    int64_t load = nchains;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        load += s->runningChains;
        for (const ReqPtr& q : s->queue) load += q->C;
    }
    r->W = choose_warps(static_cast<int>(g->n), c, load, s->ctx->sms);
    r->s64 = (c.score_path == 2);
    if (!r->s64) {
        for (int64_t k = 0; k < nchains && !r->s64; ++k)
            if (!compact_key_safe(static_cast<int64_t>(total), t0s[k], g->B, key_bits(g->n, 32 * r->W)))
                r->s64 = true;
        if (r->s64 && c.score_path == 1)
            return fail(RFMF_ERR_INVALID, "int32 scores would overflow for this (t0, B, sweeps)");
    }
    int fmt;
    if (c.csr_format == 0) fmt = g->unit16 ? kCsrUnit16 : (g->packed32 ? kCsrPacked32 : hbm_format(g));
    else if (c.csr_format == 1) { if (!g->unit16) return fail(RFMF_ERR_INVALID, "unit16 CSR needs |w| == 1 and n <= 32768"); fmt = kCsrUnit16; }
    else if (c.csr_format == 2) { if (!g->packed32) return fail(RFMF_ERR_INVALID, "packed32 CSR needs |w| < 2^15 and n <= 65536"); fmt = kCsrPacked32; }
    else fmt = (c.csr_format == 4) ? kCsrGlobal : hbm_format(g);
    // The shared CSR must leave room for about 8 warps of chains per CTA (or
    // the request's chains, if fewer), else the CSR is walked in HBM.
    {
        cudaFuncAttributes fa{};
        CU(cudaFuncGetAttributes(&fa, kernel_ptr(r->dbytes, fmt, r->s64)));
        const int64_t dynMax = s->ctx->smemOptin - static_cast<int64_t>(fa.sharedSizeBytes);
        const uint32_t chainB = chain_layout(static_cast<int>(g->n), static_cast<int>(r->words), r->pmax,
                                             r->W, r->dbytes).total;
        const int64_t kWant = std::min<int64_t>(nchains, std::max(1, 8 / r->W));
        if (!csr_in_hbm(fmt) && static_cast<int64_t>(kSmemHeader) + csr_bytes(g, fmt) + kWant * chainB > dynMax) {
            if (c.csr_format != 0) return fail(RFMF_ERR_CAPACITY, "the shared-memory CSR does not fit");
            fmt = hbm_format(g);
        }
        if (static_cast<int64_t>(kSmemHeader) + chainB > dynMax)
            return fail(RFMF_ERR_CAPACITY, "one chain needs %u B of shared memory", chainB);
    }
    r->fmt = fmt;
    if (nchains * r->words > (int64_t(1) << 34)) return fail(RFMF_ERR_CAPACITY, "request too large");
    r->initBits.assign(static_cast<size_t>(nchains * r->words), 0u);
    for (int64_t k = 0; k < nchains; ++k)
        pack_spins(initial_spins + k * g->n, g->n, r->initBits.data() + k * r->words);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->id = s->nextId++;
        r->submitS = s->now();
        s->queue.push_back(r);
        s->all[r->id] = r;
        *request_id = r->id;
    }
    s->cvWork.notify_one();
    return RFMF_OK;
}

static int rfmf_poll_impl(rfmf_server* s, uint64_t request_id, rfmf_request_status* status) {
    if (!s || !status) return fail(RFMF_ERR_INVALID, "server/status is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(request_id);
    if (it == s->all.end()) return fail(RFMF_ERR_INVALID, "unknown request %llu", static_cast<unsigned long long>(request_id));
    *status = status_of(*it->second);
    return RFMF_OK;
}

static int rfmf_wait_impl(rfmf_server* s, uint64_t request_id, double timeout_s,
                         rfmf_request_status* status) {
    if (!s) return fail(RFMF_ERR_INVALID, "server is NULL");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(request_id);
    if (it == s->all.end()) return fail(RFMF_ERR_INVALID, "unknown request %llu", static_cast<unsigned long long>(request_id));
    ReqPtr r = it->second;
    auto ready = [&] {
        return r->state == RFMF_REQ_DONE || r->state == RFMF_REQ_FAILED || r->state == RFMF_REQ_CANCELLED;
    };
    if (timeout_s < 0) {
        s->cvDone.wait(lk, ready);
    } else if (!s->cvDone.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) {
        if (status) *status = status_of(*r);
        return fail(RFMF_ERR_CAPACITY, "request %llu not done after %g s",
                    static_cast<unsigned long long>(request_id), timeout_s);
    }
    if (status) *status = status_of(*r);
    return RFMF_OK;
}

static int rfmf_result_impl(rfmf_server* s, uint64_t request_id, int8_t* end_spins, int8_t* best_spins,
                           int64_t* best_vals, int64_t* final_vals) {
    if (!s) return fail(RFMF_ERR_INVALID, "server is NULL");
    ReqPtr r;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->all.find(request_id);
        if (it == s->all.end()) return fail(RFMF_ERR_INVALID, "unknown request %llu", static_cast<unsigned long long>(request_id));
        r = it->second;
        if (r->state == RFMF_REQ_FAILED) {
            s->all.erase(it);
            return fail(r->error, "request %llu failed: %s", static_cast<unsigned long long>(request_id), r->msg.c_str());
        }
        if (r->state == RFMF_REQ_CANCELLED) {
            s->all.erase(it);
            return fail(RFMF_ERR_INVALID, "request %llu was cancelled", static_cast<unsigned long long>(request_id));
        }
        if (r->state != RFMF_REQ_DONE)
            return fail(RFMF_ERR_INVALID, "request %llu is not done", static_cast<unsigned long long>(request_id));
        s->all.erase(it);
    }
    for (int64_t c = 0; c < r->C; ++c) {
        if (end_spins) unpack_spins(r->endBits.data() + c * r->words, r->n, end_spins + c * r->n);
        if (best_spins) unpack_spins(r->bestBits.data() + c * r->words, r->n, best_spins + c * r->n);
        if (best_vals) best_vals[c] = r->best[c];
        if (final_vals) final_vals[c] = r->cur[c];
    }
    return RFMF_OK;
}

static int rfmf_cancel_impl(rfmf_server* s, uint64_t request_id) {
    if (!s) return fail(RFMF_ERR_INVALID, "server is NULL");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->all.find(request_id);
        if (it == s->all.end()) return fail(RFMF_ERR_INVALID, "unknown request %llu", static_cast<unsigned long long>(request_id));
        Request& r = *it->second;
        if (r.state == RFMF_REQ_QUEUED) {
            s->queue.erase(std::find(s->queue.begin(), s->queue.end(), it->second));
            r.state = RFMF_REQ_CANCELLED;
            r.finishS = s->now();
            s->cvDone.notify_all();
            return RFMF_OK;
        }
        if (r.state != RFMF_REQ_RUNNING) return RFMF_OK;   // finished: nothing to cancel
        r.cancel = true;
    }
    s->cvWork.notify_one();
    return RFMF_OK;
}

static int rfmf_server_stats_get_impl(rfmf_server* s, rfmf_server_stats* out) {
    if (!s || !out) return fail(RFMF_ERR_INVALID, "server/out is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->queued = out->running = out->done = 0;
    for (auto& kv : s->all) {
        const int st = kv.second->state;
        if (st == RFMF_REQ_QUEUED) ++out->queued;
        else if (st == RFMF_REQ_RUNNING) ++out->running;
        else ++out->done;
    }
    return RFMF_OK;
}

// C ABI entry points: no C++ exception crosses the boundary.
extern "C" int rfmf_server_create(rfmf_context* ctx, const rfmf_server_config* cfg, rfmf_server** out) {
    try {
        return rfmf_server_create_impl(ctx, cfg, out);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_server_create");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_server_create");
    }
}

extern "C" int rfmf_submit(rfmf_server* s, const rfmf_graph* g, int64_t nchains,
                           const int8_t* initial_spins, const double* t0s, int64_t nphases,
                           const uint64_t* phases, const uint64_t* iters,
                           const uint64_t* solver_seeds, uint64_t* request_id) {
    try {
        return rfmf_submit_impl(s, g, nchains, initial_spins, t0s, nphases, phases, iters, solver_seeds, request_id);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_submit");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_submit");
    }
}

extern "C" int rfmf_wait(rfmf_server* s, uint64_t request_id, double timeout_s,
                         rfmf_request_status* status) {
    try {
        return rfmf_wait_impl(s, request_id, timeout_s, status);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_wait");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_wait");
    }
}

extern "C" int rfmf_result(rfmf_server* s, uint64_t request_id, int8_t* end_spins, int8_t* best_spins,
                           int64_t* best_vals, int64_t* final_vals) {
    try {
        return rfmf_result_impl(s, request_id, end_spins, best_spins, best_vals, final_vals);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_result");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_result");
    }
}

extern "C" int rfmf_poll(rfmf_server* s, uint64_t request_id, rfmf_request_status* status) {
    try {
        return rfmf_poll_impl(s, request_id, status);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_poll");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_poll");
    }
}

extern "C" int rfmf_cancel(rfmf_server* s, uint64_t request_id) {
    try {
        return rfmf_cancel_impl(s, request_id);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_cancel");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_cancel");
    }
}

extern "C" int rfmf_server_stats_get(rfmf_server* s, rfmf_server_stats* out) {
    try {
        return rfmf_server_stats_get_impl(s, out);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_server_stats_get");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_server_stats_get");
    }
}
