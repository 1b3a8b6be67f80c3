// rfmf_host.h -- host-side internals shared by the translation units of
// librfmf.so (the C ABI driver, the request server, the no-alloc entry
// point).  Not installed; the public interface is include/rfmf.h.
#ifndef RFMF_HOST_H
#define RFMF_HOST_H

#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "../../include/rfmf.h"
#include "rfmf_device.h"

namespace rfmf {

// Host allocation checkpoint: throws std::bad_alloc when the countdown armed
// by rfmf_debug_fail_host_alloc reaches it (a testing aid; a no-op
// otherwise).
extern std::atomic<int64_t> g_allocCountdown;
inline void host_alloc_point() {
    int64_t c = g_allocCountdown.load(std::memory_order_relaxed);
    while (c > 0) {
        if (g_allocCountdown.compare_exchange_weak(c, c - 1)) {
            if (c == 1) throw std::bad_alloc();
            return;
        }
    }
}

// Kernel entry points (rfmf_anneal.cu).
const void* kernel_ptr(int dbytes, int fmt, bool s64);
cudaError_t launch_anneal(const DevLaunch& L, int dbytes, int fmt, bool s64, int grid,
                          int threads, size_t smem, cudaStream_t stream);

// Output-path kernels (rfmf_ingest.cu).
cudaError_t launch_chain_cuts(const DevChain* chains, const DevGraph* graphs, int C, int which,
                              int64_t* out, cudaStream_t st);
cudaError_t launch_chain_partitions(const DevChain* chains, const DevGraph* graphs, int c0, int count,
                                    int maxN, int which, char* out, int64_t stride, cudaStream_t st);

// Error channel: records the message for rfmf_last_error() (per host thread)
// and returns `code`.
int fail(int code, const char* fmt, ...);
int set_last_error(int code, const char* msg);

#define CU(call)                                                                 \
    do {                                                                         \
        const cudaError_t e_ = (call);                                           \
        if (e_ != cudaSuccess)                                                   \
            return ::rfmf::fail(e_ == cudaErrorMemoryAllocation ? RFMF_ERR_NOMEM \
                                                                : RFMF_ERR_CUDA, \
                                "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

constexpr uint64_t kMaxTotalSteps = 1000000000000ull;   // src/host_common.h:80
constexpr int64_t kMaxBetaRuns = 33000000;              // src/host_common.h:99
constexpr int64_t kGumbelMaxMag = 3617486 + 127;        // src/philox.cuh:44-48

void gumbel_lut(int32_t lut[16]);

// Run-length beta tables of a set of chains: one table per distinct t0,
// chain c reads runs [chainOff[c], chainOff[c] + chainRuns[c]).
// One t0's beta run table over a schedule's sweeps.
struct BetaRun {
    std::vector<int64_t> end;
    std::vector<int32_t> val;
};

struct BetaTables {
    std::vector<int64_t> end;
    std::vector<int32_t> val;
    std::vector<int64_t> chainOff;
    std::vector<int64_t> chainRuns;
};
int build_beta(const double* t0s, int64_t C, int64_t total, BetaTables& bt);
// One t0's run table over `total` sweeps, appended to end/val (the runs of
// src/host_common.cpp:238-294); fails past kMaxBetaRuns entries in end.
int append_runs(double t0, int64_t total, std::vector<int64_t>& end, std::vector<int32_t>& val);
// Refuses t0s whose beta_fixed would overflow int32 within `total` sweeps.
int beta_range_check(const double* t0s, int64_t C, int64_t total);
constexpr int64_t kBetaCacheRuns = int64_t(1) << 24;
constexpr int64_t kDevBetaKeepBytes = int64_t(256) << 20;
bool score_safe_int32(int64_t total, double t0, int64_t B);

// Launch-shape helpers of the planner.
// Warps per chain: at least one per ~768 vertex blocks, more while the batch's
// `chains` leave the SMs (`sms`) short of work; c.threads_per_chain overrides.
constexpr int kMaxAutoWarps = 4;
constexpr int kMaxLatencyWarps = 8;   // widest chain the planner picks for few chains
// Warps an item of `chains` chains of `warps` warps each puts on one of the
// SM's four schedulers (warp w issues from scheduler w mod 4).
inline int sched_level(int chains, int warps) { return (chains * warps + 3) / 4; }
int choose_warps(int maxN, const rfmf_launch_config& c, int64_t chains, int sms);
int key_bits(int64_t n, int T);
bool compact_key_safe(int64_t total, double t0, int64_t B, int kb);

// Owning device buffer.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) {
            if (p) cudaFree(p);
            p = o.p;
            bytes = o.bytes;
            o.p = nullptr;
            o.bytes = 0;
        }
        return *this;
    }
    ~DevBuf() { if (p) cudaFree(p); }
    int alloc(size_t b) {
        bytes = b < 16 ? 16 : b;
        const cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) {
            p = nullptr;
            return fail(e == cudaErrorMemoryAllocation ? RFMF_ERR_NOMEM : RFMF_ERR_CUDA,
                        "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
        }
        return RFMF_OK;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

// One (t0, sweeps) beta run table in device memory, shared by every batch,
// drop-in call and served request of a context that anneals at that t0 over
// that many sweeps (the reference builds and uploads one set per launch,
// src/host_common.cpp:277-294).  Freed when its last user and the context's
// keep-alive list let go of it.
struct DevBetaTable {
    DevBuf end, val;
    int64_t runs = 0;
};
using DevBetaRef = std::shared_ptr<const DevBetaTable>;

// Per-chain view of a set of device tables: chain c reads runs
// [0, runs[c]) of end[c] / val[c]; refs holds one table per distinct t0.
struct ChainBeta {
    std::vector<const int64_t*> end;
    std::vector<const int32_t*> val;
    std::vector<int64_t> runs;
    std::vector<DevBetaRef> refs;
    int64_t totalRuns = 0;   // runs over the distinct t0s (as the reference counts them)
};

// The device tables of C chains: taken from the context when another user
// holds (or recently held) them, else built on the host (from the host-side
// cache) and uploaded once on the context's upload stream, which is
// synchronised before returning, so a launch on any stream may use them.
// Thread-safe.  RFMF_ERR_BETA_RUNS past kMaxBetaRuns runs over the distinct
// t0s, as buildBetaRunTables refuses them.
int acquire_beta(rfmf_context* ctx, const double* t0s, int64_t C, int64_t total, ChainBeta& out);

// Request server admission.  A request's own device state: its spin and
// best-spin words, beta run tables (8 + 4 bytes a run), schedule (4 + 8 bytes
// a phase) and chain records; a DevBuf holds at least 16 bytes.
inline int64_t request_device_bytes(int64_t C, int64_t words, int64_t betaRuns, int64_t nphases) {
    auto buf = [](int64_t b) { return b < 16 ? int64_t(16) : b; };
    const int64_t np = nphases > 1 ? nphases : 1;
    return 2 * buf(C * words * 4) + buf(betaRuns * 8) + buf(betaRuns * 4) + buf(np * 4) +
           buf(np * 8) + C * static_cast<int64_t>(sizeof(DevChain));
}

// The queue head joins the running requests while the admitted chains and
// device bytes stay within max_chains and max_device_bytes (0: no byte
// limit); an idle server admits it regardless, so no request waits forever
// (submission refuses a request that alone exceeds either limit).
inline bool admits(int64_t runningChains, int64_t runningBytes, int64_t C, int64_t bytes,
                   int64_t maxChains, int64_t maxBytes) {
    if (runningChains == 0) return true;
    return runningChains + C <= maxChains && (maxBytes == 0 || runningBytes + bytes <= maxBytes);
}

// One chain's spins (int8, >= 0 is +1) as ceil(n/32) words, bit v = spin +1;
// every word is written (tail bits past n are 0).  Eight spins at a time:
// byte k of m is 1 where spin k >= 0 (its sign bit clear), and multiplying
// by sum_k 2^(56-7k) moves byte k's bit to bit 56+k with no two partial
// products overlapping, so the top byte is the eight bits in order.
static_assert(__BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__, "spin packing assumes little-endian bytes");
inline uint32_t pack_spin_bytes8(const int8_t* s) {
    uint64_t u;
    std::memcpy(&u, s, 8);
    const uint64_t m = (~u >> 7) & 0x0101010101010101ull;
    return static_cast<uint32_t>((m * 0x0102040810204080ull) >> 56);
}

inline void pack_spins(const int8_t* sp, int64_t n, uint32_t* words) {
    const int64_t full = n >> 5;
    for (int64_t w = 0; w < full; ++w) {
        const int8_t* s = sp + 32 * w;
        words[w] = pack_spin_bytes8(s) | (pack_spin_bytes8(s + 8) << 8) |
                   (pack_spin_bytes8(s + 16) << 16) | (pack_spin_bytes8(s + 24) << 24);
    }
    if (n & 31) {
        const int8_t* s = sp + 32 * full;
        uint32_t x = 0;
        for (int j = 0; j < static_cast<int>(n & 31); ++j) x |= static_cast<uint32_t>(s[j] >= 0) << j;
        words[full] = x;
    }
}

// The inverse: spins[v] = +1 where bit v is set, else -1.  Eight at a time:
// the byte replicated eight times and masked with bit k in byte k leaves
// byte k nonzero iff bit k is set; adding 0x7F per byte (no carries: every
// byte is 0 or a single bit <= 0x80) sets its top bit iff nonzero; c * 0xFE
// xor 0xFF per byte is 0x01 (+1) for c = 1 and 0xFF (-1) for c = 0.
inline void unpack_spins(const uint32_t* words, int64_t n, int8_t* sp) {
    const int64_t full = n >> 5;
    for (int64_t w = 0; w < full; ++w) {
        const uint32_t x = words[w];
        for (int q = 0; q < 4; ++q) {
            const uint64_t t = (static_cast<uint64_t>((x >> (8 * q)) & 0xFFu) * 0x0101010101010101ull) &
                               0x8040201008040201ull;
            const uint64_t c = ((t + 0x7F7F7F7F7F7F7F7Full) >> 7) & 0x0101010101010101ull;
            const uint64_t out = ~0ull ^ (c * 0xFEull);
            std::memcpy(sp + 32 * w + 8 * q, &out, 8);
        }
    }
    if (n & 31) {
        const uint32_t x = words[full];
        int8_t* s = sp + 32 * full;
        for (int j = 0; j < static_cast<int>(n & 31); ++j)
            s[j] = static_cast<int8_t>(2 * static_cast<int>((x >> j) & 1u) - 1);
    }
}

}  // namespace rfmf

struct rfmf_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    int sms = 0;
    int smemOptin = 0;
    int32_t lut[16];
    // Beta run tables per (t0 bits, sweeps), kept across batches and
    // requests: most share their t0 ladder and length, and the tables are
    // large (10^5 sweeps already hold ~30k runs per t0).  Dropped wholesale
    // past kBetaCacheRuns runs.
    std::mutex betaMu;
    std::map<std::pair<uint64_t, uint64_t>, std::shared_ptr<const rfmf::BetaRun>> betaCache;
    int64_t betaCachedRuns = 0;
    // Device copies of run tables by (t0 bits, sweeps): live while any batch
    // or request holds them; the most recently acquired stay alive up to
    // kDevBetaKeepBytes in the keep-alive list.  Uploads go through their own
    // stream so that they never wait behind a long launch.
    std::mutex devBetaMu;
    std::map<std::pair<uint64_t, uint64_t>, std::weak_ptr<const rfmf::DevBetaTable>> devBeta;
    std::deque<rfmf::DevBetaRef> devBetaKeep;
    int64_t devBetaKeepBytes = 0;
    uint64_t devBetaUploads = 0;
    cudaStream_t uploadStream = nullptr;
    // Measured plans (rfmf_autotune) by batch shape: the chosen config and
    // every candidate's config and microseconds per chain-sweep.
    struct TunedPlan {
        rfmf_launch_config best;
        std::vector<rfmf_launch_config> cand;
        std::vector<float> us;
    };
    std::mutex tuneMu;
    std::map<std::string, TunedPlan> tuneCache;
    // Holders: the caller's handle plus every graph, batch and server made
    // on the context.  The context is torn down when the last one lets go,
    // so rfmf_context_destroy may come before theirs (a garbage collector
    // finalises objects in any order).
    std::atomic<int> holders{1};
};

namespace rfmf {
// Drop one hold on ctx; the last one destroys its streams and tables.
void let_go(rfmf_context* ctx);

// A graph's, batch's or server's hold on its context.  Declared as the
// object's first member, it is released after every other member (device
// buffers, shared beta tables) is gone.
struct CtxHold {
    rfmf_context* ctx = nullptr;
    CtxHold() = default;
    CtxHold(const CtxHold&) = delete;
    CtxHold& operator=(const CtxHold&) = delete;
    void set(rfmf_context* c) {
        if (ctx) let_go(ctx);
        ctx = c;
        if (c) c->holders.fetch_add(1);
    }
    ~CtxHold() {
        if (ctx) let_go(ctx);
    }
};
}  // namespace rfmf

// A graph in device memory: offsets and 8-byte entries for HBM walks, plus
// the compact entry arrays the shared-memory formats stage from (present
// when the graph qualifies).  All arrays are padded to 16 bytes.
struct rfmf_graph {
    rfmf::CtxHold ctxHold;   // first member: released last
    rfmf_context* ctx = nullptr;
    // Holders: the caller's handle plus every batch and request that runs
    // on the graph; freed when the last one lets go.
    mutable std::atomic<int> holders{1};
    int64_t n = 0, m = 0, B = 0, wsum2 = 0;
    bool unit16 = false, packed32 = false;
    uint32_t offBytes = 0, u16Bytes = 0, p32Bytes = 0;
    rfmf::DevBuf offsets, edges, u16, p32;
    // Learned costs: device time per sweep of one work item, by plan (warps
    // per chain, CSR format), phase group count P and scheduler level (the
    // warps an item puts on each of the SM's four schedulers,
    // sched_level), from the item timings of earlier launches (weight =
    // sweeps observed).  An item's chains run at the pace of its busiest
    // scheduler: on GB300, 13 to 16 one-warp chains of the 50x60 torus take
    // 4.53 us per sweep at P = 1 and 12 take 3.74; and two graphs' relative
    // cost depends on P (at P = 128 a dense graph's row walks double its
    // sweep; at P = 1 its vertex count decides).  They size the work items
    // of later launches of the same plan; they never affect results.
    struct LearnedCost {
        double ns = 0.0, weight = 0.0;
    };
    mutable std::map<std::tuple<int, int, uint32_t, int>, LearnedCost> costs;
    // The item time per sweep at (plan, P, level): from the nearest P (in
    // log2 P) learned under the plan, at the nearest level learned there,
    // scaled to `level` by (level + 3) / (learned level + 3) (measured
    // level-4 / level-3 ratios 1.11 to 1.21); 0 when the plan has none.
    double cost(int warps, int fmt, uint32_t P, int level) const {
        const double lp = std::log2(static_cast<double>(P > 0 ? P : 1));
        double pd = 1e300;
        uint32_t bestP = 0;
        for (auto it = costs.lower_bound({warps, fmt, 0u, 0});
             it != costs.end() && std::get<0>(it->first) == warps && std::get<1>(it->first) == fmt; ++it) {
            const double d = std::fabs(std::log2(static_cast<double>(std::get<2>(it->first))) - lp);
            if (d < pd) { pd = d; bestP = std::get<2>(it->first); }
        }
        if (!bestP) return 0.0;
        int bestL = 0;
        double ns = 0.0;
        for (auto it = costs.lower_bound({warps, fmt, bestP, 0});
             it != costs.end() && std::get<0>(it->first) == warps && std::get<1>(it->first) == fmt &&
             std::get<2>(it->first) == bestP; ++it) {
            const int L = std::get<3>(it->first);
            if (!bestL || std::abs(L - level) < std::abs(bestL - level)) { bestL = L; ns = it->second.ns; }
        }
        return ns * (level + 3.0) / (bestL + 3.0);
    }
    // Before any timing: an estimate of the same quantity from the graph's
    // shape, fitted on GB300 to one-warp chains at 16 per SM (50x60 torus
    // and ER n = 2000 d = 19, phases 128..1): 1.65 us + 1.03 ns per vertex +
    // 3.5 ns per winner-row entry (min(P, n) rows of mean degree 2m/n), the
    // vertex and entry terms spread over the chain's warps, scaled by level
    // as above.  Within 7% of the measured sweep on both graphs at every P.
    double model_cost(int warps, uint32_t P, int level) const {
        const double nn = static_cast<double>(n > 0 ? n : 1);
        const double rows = std::min(static_cast<double>(P > 0 ? P : 1), nn);
        const double us = 1.65 + (1.03e-3 * nn + 3.5e-3 * rows * (2.0 * static_cast<double>(m) / nn)) /
                                     static_cast<double>(warps > 0 ? warps : 1);
        return 1e3 * us * (level + 3.0) / 7.0;
    }
    // Whether a cost was learned under the plan at phase P itself (any level).
    bool learned_at(int warps, int fmt, uint32_t P) const {
        auto it = costs.lower_bound({warps, fmt, P, 0});
        return it != costs.end() && std::get<0>(it->first) == warps && std::get<1>(it->first) == fmt &&
               std::get<2>(it->first) == P;
    }
    void learn(int warps, int fmt, uint32_t P, int level, double ns, double weight) const {
        LearnedCost& c = costs[{warps, fmt, P > 0 ? P : 1u, level}];
        c.ns = (c.ns * c.weight + ns * weight) / (c.weight + weight);
        c.weight += weight;
    }
    // Original vertex ids by dense id (graphs built from an edge list).
    std::vector<int64_t> origIds;
};

namespace rfmf {

// Drop one hold on g; the last one frees it.
void let_go(const rfmf_graph* g);

// The holds a batch or a request keeps on the graphs it runs on, released
// when it is destroyed (so a graph destroyed first stays valid meanwhile).
struct GraphHolds {
    std::vector<const rfmf_graph*> held;
    GraphHolds() = default;
    GraphHolds(const GraphHolds&) = delete;
    GraphHolds& operator=(const GraphHolds&) = delete;
    void add(const rfmf_graph* g) {
        g->holders.fetch_add(1);
        held.push_back(g);
    }
    ~GraphHolds() {
        for (const rfmf_graph* g : held) let_go(g);
    }
};

// The HBM-walk format of a graph: the most compact entries it has.
inline int hbm_format(const rfmf_graph* g) {
    return g->unit16 ? kCsrGlobal16 : (g->packed32 ? kCsrGlobal32 : kCsrGlobal);
}

// The entry array a launch of format `fmt` reads for graph g (the 8-byte
// pairs are DevGraph::edges).
inline const void* compact_entries(const rfmf_graph* g, int fmt) {
    if (fmt == kCsrUnit16 || fmt == kCsrGlobal16) return g->u16.p;
    if (fmt == kCsrPacked32 || fmt == kCsrGlobal32) return g->p32.p;
    return nullptr;
}

}  // namespace rfmf

#endif  // RFMF_HOST_H
