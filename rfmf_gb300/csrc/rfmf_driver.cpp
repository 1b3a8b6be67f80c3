// rfmf_driver.cpp -- host side of librfmf.so: the C ABI of include/rfmf.h.
//
// Replaces the reference's host driver (src/anneal_kernels.cu:498-884:
// runDispatch/runMC/annealGpu) and the helpers of src/host_common.cpp it
// calls.  Differences by design: errors are status codes (the reference
// exits), device state can stay resident across calls (batches), many graphs
// share one persistent launch, and the launch geometry comes from an
// occupancy-driven autotuner instead of the V100 constants of src/tuning.hpp.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../include/rfmf_testing.h"
#include "rfmf_host.h"

using namespace rfmf;

namespace rfmf {

thread_local std::string g_err;
std::atomic<int64_t> g_allocCountdown{0};

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

// Q20 Gumbel quantile table: round(-log(-log((2i+1)/32)) * 2^20), the
// defining formula of src/philox.cuh:26-34 (every entry >= 0.016 away from a
// rounding boundary, so the double evaluation is exact).
void gumbel_lut(int32_t lut[16]) {
    for (int i = 0; i < 16; ++i)
        lut[i] = static_cast<int32_t>(std::lround(-std::log(-std::log((2.0 * i + 1.0) / 32.0)) *
                                                  1048576.0));
}

// betaFixedForStep: round(log(1+step)/t0 * 2^20) in host double
// (src/host_common.h:73-76).  Never evaluated on the device.
inline int32_t beta_fixed(uint64_t step, double t0) {
    const double beta = std::log(1.0 + static_cast<double>(step)) / t0;
    return static_cast<int32_t>(std::round(beta * (1 << 20)));
}

// First 1-based step > s0 whose beta exceeds v.  Starts from the inverse of
// the schedule (beta crosses v+1/2 at step ~ exp((v+1/2) t0 / 2^20) - 1) and
// settles the exact boundary with the same double expression the kernel's
// schedule is defined by, so the table reproduces beta_fixed step for step.
// Returns 0 if beta stays <= v through `total`.
int64_t next_run_start(double t0, int32_t v, int64_t s0, int64_t total) {
    if (beta_fixed(static_cast<uint64_t>(total), t0) <= v) return 0;
    const double guess = std::exp((static_cast<double>(v) + 0.5) * t0 / 1048576.0) - 1.0;
    int64_t s = (guess >= static_cast<double>(total)) ? total
              : std::max<int64_t>(s0 + 1, static_cast<int64_t>(std::ceil(guess)));
    s = std::min(s, total);
    // Bracket [lo, hi]: beta(lo) <= v < beta(hi), growing the step outward.
    int64_t lo = s0, hi = s;
    if (beta_fixed(static_cast<uint64_t>(hi), t0) <= v) {
        int64_t span = 1;
        lo = hi;
        while (true) {
            hi = std::min(total, lo + span);
            if (beta_fixed(static_cast<uint64_t>(hi), t0) > v) break;
            lo = hi;
            span *= 2;
        }
    } else {
        int64_t span = 1;
        while (true) {
            const int64_t cand = std::max(s0, hi - span);
            if (cand == s0 || beta_fixed(static_cast<uint64_t>(cand), t0) <= v) {
                lo = cand;
                break;
            }
            hi = cand;
            span *= 2;
        }
    }
    while (hi - lo > 1) {
        const int64_t mid = lo + (hi - lo) / 2;
        if (beta_fixed(static_cast<uint64_t>(mid), t0) <= v) lo = mid; else hi = mid;
    }
    return hi;
}

// One t0's run-length table over 1-based steps [1, total]; ends are 0-based
// exclusive (src/host_common.h:82-94).  >= 1 run even when total == 0.
int append_runs(double t0, int64_t total, std::vector<int64_t>& end, std::vector<int32_t>& val) {
    if (total <= 0) {
        end.push_back(0);
        val.push_back(0);
        return RFMF_OK;
    }
    int64_t s = 1;
    while (true) {
        if (static_cast<int64_t>(end.size()) >= kMaxBetaRuns)
            return fail(RFMF_ERR_BETA_RUNS,
                        "beta run tables exceed %lld runs (t0=%g, %lld sweeps); runs scale "
                        "with log(sweeps)/t0 * 2^20",
                        static_cast<long long>(kMaxBetaRuns), t0, static_cast<long long>(total));
        const int32_t v = beta_fixed(static_cast<uint64_t>(s), t0);
        const int64_t nxt = next_run_start(t0, v, s, total);
        if (nxt == 0) {
            end.push_back(total);
            val.push_back(v);
            return RFMF_OK;
        }
        end.push_back(nxt - 1);
        val.push_back(v);
        s = nxt;
    }
}

int beta_range_check(const double* t0s, int64_t C, int64_t total) {
    // beta_fixed must stay inside int32: past it the reference's
    // static_cast<int32_t>(round(...)) (src/host_common.h:73-76) is undefined
    // behaviour (x86 and Arm even disagree), so such schedules are refused.
    for (int64_t c = 0; c < C; ++c) {
        const double bmax = std::round(std::log(1.0 + static_cast<double>(total)) / t0s[c] * 1048576.0);
        if (!(bmax < 2147483647.0))
            return fail(RFMF_ERR_INVALID,
                        "t0=%g over %lld sweeps makes beta_fixed overflow int32", t0s[c],
                        static_cast<long long>(total));
    }
    return RFMF_OK;
}

int build_beta(const double* t0s, int64_t C, int64_t total, BetaTables& bt) {
    if (int rc = beta_range_check(t0s, C, total)) return rc;
    std::vector<double> distinct;
    std::vector<int64_t> first, count;
    bt.chainOff.resize(C);
    bt.chainRuns.resize(C);
    for (int64_t c = 0; c < C; ++c) {
        size_t k = 0;
        while (k < distinct.size() && distinct[k] != t0s[c]) ++k;
        if (k == distinct.size()) {
            distinct.push_back(t0s[c]);
            first.push_back(static_cast<int64_t>(bt.end.size()));
            const int rc = append_runs(t0s[c], total, bt.end, bt.val);
            if (rc != RFMF_OK) return rc;
            count.push_back(static_cast<int64_t>(bt.end.size()) - first.back());
        }
        bt.chainOff[c] = first[k];
        bt.chainRuns[c] = count[k];
    }
    return RFMF_OK;
}

namespace {

// The run table of one (t0, sweeps): from the context's cache, or built on
// the calling thread and added.
int cached_runs(rfmf_context* ctx, double t0, int64_t total, std::shared_ptr<const BetaRun>& out) {
    uint64_t bits;
    std::memcpy(&bits, &t0, sizeof bits);
    const auto key = std::make_pair(bits, static_cast<uint64_t>(total));
    {
        std::lock_guard<std::mutex> lk(ctx->betaMu);
        auto it = ctx->betaCache.find(key);
        if (it != ctx->betaCache.end()) {
            out = it->second;
            return RFMF_OK;
        }
    }
    auto tb = std::make_shared<BetaRun>();
    if (int rc = append_runs(t0, total, tb->end, tb->val)) return rc;
    std::lock_guard<std::mutex> lk(ctx->betaMu);
    if (ctx->betaCachedRuns + static_cast<int64_t>(tb->end.size()) > kBetaCacheRuns) {
        ctx->betaCache.clear();
        ctx->betaCachedRuns = 0;
    }
    auto ins = ctx->betaCache.emplace(key, tb);
    if (ins.second) ctx->betaCachedRuns += static_cast<int64_t>(tb->end.size());
    out = ins.first->second;
    return RFMF_OK;
}

}  // namespace

namespace {

// The device copy of one (t0, sweeps) table, uploaded from the host table
// `host` when no batch or request of the context holds it.
int device_table(rfmf_context* ctx, double t0, int64_t total, const BetaRun& host, DevBetaRef& out) {
    uint64_t bits;
    std::memcpy(&bits, &t0, sizeof bits);
    const auto key = std::make_pair(bits, static_cast<uint64_t>(total));
    std::lock_guard<std::mutex> lk(ctx->devBetaMu);
    auto it = ctx->devBeta.find(key);
    if (it != ctx->devBeta.end()) {
        if (DevBetaRef live = it->second.lock()) {
            out = live;
            return RFMF_OK;
        }
    }
    auto t = std::make_shared<DevBetaTable>();
    t->runs = static_cast<int64_t>(host.end.size());
    if (int rc = t->end.alloc(host.end.size() * sizeof(int64_t))) return rc;
    if (int rc = t->val.alloc(host.val.size() * sizeof(int32_t))) return rc;
    if (!ctx->uploadStream) CU(cudaStreamCreateWithFlags(&ctx->uploadStream, cudaStreamNonBlocking));
    CU(cudaMemcpyAsync(t->end.p, host.end.data(), host.end.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                       ctx->uploadStream));
    CU(cudaMemcpyAsync(t->val.p, host.val.data(), host.val.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                       ctx->uploadStream));
    CU(cudaStreamSynchronize(ctx->uploadStream));
    ++ctx->devBetaUploads;
    if (ctx->devBeta.size() > 1024) {
        for (auto e = ctx->devBeta.begin(); e != ctx->devBeta.end();)
            e = e->second.expired() ? ctx->devBeta.erase(e) : std::next(e);
    }
    ctx->devBeta[key] = t;
    ctx->devBetaKeep.push_back(t);
    ctx->devBetaKeepBytes += static_cast<int64_t>(t->end.bytes + t->val.bytes);
    while (ctx->devBetaKeepBytes > kDevBetaKeepBytes && ctx->devBetaKeep.size() > 1) {
        const DevBetaRef& old = ctx->devBetaKeep.front();
        ctx->devBetaKeepBytes -= static_cast<int64_t>(old->end.bytes + old->val.bytes);
        ctx->devBetaKeep.pop_front();
    }
    out = t;
    return RFMF_OK;
}

}  // namespace

int acquire_beta(rfmf_context* ctx, const double* t0s, int64_t C, int64_t total, ChainBeta& out) {
    if (int rc = beta_range_check(t0s, C, total)) return rc;
    CU(cudaSetDevice(ctx->device));
    out = ChainBeta{};
    out.end.resize(C);
    out.val.resize(C);
    out.runs.resize(C);
    std::map<uint64_t, size_t> placed;   // t0 bits -> index into out.refs
    for (int64_t c = 0; c < C; ++c) {
        uint64_t bits;
        std::memcpy(&bits, &t0s[c], sizeof bits);
        auto it = placed.find(bits);
        if (it == placed.end()) {
            std::shared_ptr<const BetaRun> host;
            if (int rc = cached_runs(ctx, t0s[c], total, host)) return rc;
            out.totalRuns += static_cast<int64_t>(host->end.size());
            if (out.totalRuns > kMaxBetaRuns)
                return fail(RFMF_ERR_BETA_RUNS,
                            "beta run tables exceed %lld runs (t0=%g, %lld sweeps); runs scale "
                            "with log(sweeps)/t0 * 2^20",
                            static_cast<long long>(kMaxBetaRuns), t0s[c], static_cast<long long>(total));
            DevBetaRef dev;
            if (int rc = device_table(ctx, t0s[c], total, *host, dev)) return rc;
            it = placed.emplace(bits, out.refs.size()).first;
            out.refs.push_back(std::move(dev));
        }
        const DevBetaTable& t = *out.refs[it->second];
        out.end[c] = t.end.as<int64_t>();
        out.val[c] = t.val.as<int32_t>();
        out.runs[c] = t.runs;
    }
    return RFMF_OK;
}

bool score_safe_int32(int64_t total, double t0, int64_t B) {
    // src/host_common.cpp:296-312
    const double bmax = std::log(1.0 + static_cast<double>(total)) / t0;
    const int64_t bmf = static_cast<int64_t>(std::llround(bmax * (1 << 20)));
    const int64_t limit = static_cast<int64_t>(std::numeric_limits<int32_t>::max()) - kGumbelMaxMag;
    if (bmf > 0 && B > 0 && B > limit / bmf) return false;
    return (bmf * B + kGumbelMaxMag) < static_cast<int64_t>(std::numeric_limits<int32_t>::max());
}

}  // namespace rfmf

// Error channel shared with the other translation units of the library.
namespace rfmf {
int set_last_error(int code, const char* msg) { return fail(code, "%s", msg); }
}  // namespace rfmf

extern "C" int rfmf_debug_fail_host_alloc(int64_t countdown) {
    g_allocCountdown.store(countdown > 0 ? countdown : 0);
    return RFMF_OK;
}

// ------------------------------------------------------------------ misc
extern "C" const char* rfmf_version(void) { return "rfmf_gb300 0.1 (sm_103a)"; }
extern "C" const char* rfmf_last_error(void) { return g_err.c_str(); }

extern "C" int rfmf_context_create(int device, rfmf_context** out) {
    if (!out) return fail(RFMF_ERR_INVALID, "out is NULL");
    *out = nullptr;
    int count = 0;
    CU(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count)
        return fail(RFMF_ERR_INVALID, "device %d out of range (%d devices)", device, count);
    CU(cudaSetDevice(device));
    auto ctx = std::unique_ptr<rfmf_context>(new (std::nothrow) rfmf_context());
    if (!ctx) return fail(RFMF_ERR_NOMEM, "host allocation failed");
    ctx->device = device;
    CU(cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device));
    CU(cudaDeviceGetAttribute(&ctx->smemOptin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    CU(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    gumbel_lut(ctx->lut);
    *out = ctx.release();
    return RFMF_OK;
}

namespace rfmf {
void let_go(rfmf_context* ctx) {
    if (ctx->holders.fetch_sub(1) != 1) return;
    cudaSetDevice(ctx->device);
    {
        std::lock_guard<std::mutex> lk(ctx->devBetaMu);
        ctx->devBetaKeep.clear();
        ctx->devBeta.clear();
    }
    if (ctx->uploadStream) cudaStreamDestroy(ctx->uploadStream);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}
}  // namespace rfmf

extern "C" int rfmf_context_destroy(rfmf_context* ctx) {
    if (!ctx) return RFMF_OK;
    let_go(ctx);
    return RFMF_OK;
}

extern "C" int rfmf_context_info(const rfmf_context* ctx, int* sm_count, int* smem_optin) {
    if (!ctx) return fail(RFMF_ERR_INVALID, "ctx is NULL");
    if (sm_count) *sm_count = ctx->sms;
    if (smem_optin) *smem_optin = ctx->smemOptin;
    return RFMF_OK;
}

extern "C" int rfmf_context_stream(const rfmf_context* ctx, void** stream) {
    if (!ctx || !stream) return fail(RFMF_ERR_INVALID, "ctx/stream is NULL");
    *stream = static_cast<void*>(ctx->stream);
    return RFMF_OK;
}

extern "C" int rfmf_context_beta_cache(rfmf_context* ctx, int64_t* tables, int64_t* device_bytes,
                                       uint64_t* uploads) {
    if (!ctx) return fail(RFMF_ERR_INVALID, "ctx is NULL");
    std::lock_guard<std::mutex> lk(ctx->devBetaMu);
    int64_t live = 0, bytes = 0;
    for (const auto& e : ctx->devBeta) {
        if (DevBetaRef t = e.second.lock()) {
            ++live;
            bytes += static_cast<int64_t>(t->end.bytes + t->val.bytes);
        }
    }
    if (tables) *tables = live;
    if (device_bytes) *device_bytes = bytes;
    if (uploads) *uploads = ctx->devBetaUploads;
    return RFMF_OK;
}

// ----------------------------------------------------------- host helpers
extern "C" int64_t rfmf_total_steps(int64_t nphases, const uint64_t* iters) {
    // src/host_common.cpp:196-210: summed and range-checked in unsigned.
    uint64_t total = 0;
    for (int64_t i = 0; i < nphases; ++i) {
        total += iters[i];
        if (iters[i] > kMaxTotalSteps || total > kMaxTotalSteps) return -1;
    }
    return static_cast<int64_t>(total);
}

extern "C" int32_t rfmf_beta_fixed(uint64_t step, double t0) { return beta_fixed(step, t0); }

extern "C" int rfmf_score_safe_int32(int64_t total_steps, double t0, int64_t delta_bound) {
    return score_safe_int32(total_steps, t0, delta_bound) ? 1 : 0;
}

extern "C" int64_t rfmf_max_weighted_degree(int64_t n, const uint32_t* offsets,
                                            const int32_t* weight) {
    int64_t B = 0;
    for (int64_t v = 0; v < n; ++v) {
        int64_t s = 0;
        for (uint32_t i = offsets[v]; i < offsets[v + 1]; ++i)
            s += std::llabs(static_cast<long long>(weight[i]));
        B = std::max(B, s);
    }
    return B;
}

extern "C" int64_t rfmf_cut_value(int64_t n, const uint32_t* offsets, const int32_t* col,
                                  const int32_t* weight, const int8_t* spin) {
    int64_t value = 0;
    for (int64_t v = 0; v < n; ++v)
        for (uint32_t i = offsets[v]; i < offsets[v + 1]; ++i)
            if (static_cast<int64_t>(col[i]) > v && spin[v] != spin[col[i]]) value += weight[i];
    return value;
}

extern "C" void rfmf_initial_spins(uint64_t seed, int64_t n, int8_t* out) {
    // xoshiro256++ (Blackman & Vigna) seeded by splitmix64; bits drawn one at
    // a time from a 64-bit reservoir, 1 -> +1 (src/rng.hpp:11-58).
    uint64_t s[4];
    uint64_t z = seed;
    for (auto& w : s) {
        z += 0x9e3779b97f4a7c15ULL;
        uint64_t x = z;
        x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
        x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
        w = x ^ (x >> 31);
    }
    auto rotl = [](uint64_t x, int k) { return (x << k) | (x >> (64 - k)); };
    uint64_t buf = 0;
    int avail = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (avail == 0) {
            buf = rotl(s[0] + s[3], 23) + s[0];
            const uint64_t t = s[1] << 17;
            s[2] ^= s[0];
            s[3] ^= s[1];
            s[1] ^= s[2];
            s[0] ^= s[3];
            s[2] ^= t;
            s[3] = rotl(s[3], 45);
            avail = 64;
        }
        out[i] = (buf & 1u) ? 1 : -1;
        buf >>= 1;
        --avail;
    }
}

static int rfmf_beta_tables_impl(const double* t0s, int64_t C, int64_t total_steps,
                                int64_t* run_end, int32_t* run_val, int64_t* chain_off,
                                int64_t cap, int64_t* runs) {
    if (C < 0 || (C > 0 && !t0s) || total_steps < 0) return fail(RFMF_ERR_INVALID, "bad arguments");
    for (int64_t c = 0; c < C; ++c)
        if (!(t0s[c] > 0.0)) return fail(RFMF_ERR_INVALID, "t0s[%lld] must be > 0", (long long)c);
    BetaTables bt;
    const int rc = build_beta(t0s, C, total_steps, bt);
    if (rc != RFMF_OK) return rc;
    const int64_t R = static_cast<int64_t>(bt.end.size());
    for (int64_t i = 0; i < R && i < cap; ++i) {
        if (run_end) run_end[i] = bt.end[i];
        if (run_val) run_val[i] = bt.val[i];
    }
    if (chain_off) for (int64_t c = 0; c < C; ++c) chain_off[c] = bt.chainOff[c];
    if (runs) *runs = R;
    return RFMF_OK;
}

// ------------------------------------------------------------------ graph
namespace {
struct CsrFacts {
    int64_t B = 0, wsum2 = 0;
    bool unit = true, small = true;
};

// The AnnealCsr invariants the kernel's per-vertex gain bookkeeping relies on
// (src/immutable_graph.hpp:44-176): monotone offsets, ids in range, rows
// strictly ascending, no self loops, no zero weights, symmetric with equal
// weights.
int validate_csr(int64_t n, const uint32_t* offsets, const int32_t* col, const int32_t* weight,
                 CsrFacts& f) {
    if (n < 0 || n >= (int64_t(1) << 31)) return fail(RFMF_ERR_INVALID, "n=%lld out of range", (long long)n);
    if (!offsets) return fail(RFMF_ERR_INVALID, "offsets is NULL");
    if (offsets[0] != 0) return fail(RFMF_ERR_INVALID, "offsets[0] must be 0");
    if (offsets[n] > 0 && (!col || !weight)) return fail(RFMF_ERR_INVALID, "col/weight is NULL");
    for (int64_t v = 0; v < n; ++v) {
        if (offsets[v + 1] < offsets[v]) return fail(RFMF_ERR_INVALID, "offsets not monotone at %lld", (long long)v);
        int64_t s = 0;
        for (uint32_t i = offsets[v]; i < offsets[v + 1]; ++i) {
            const int32_t u = col[i];
            if (u < 0 || u >= n) return fail(RFMF_ERR_INVALID, "col[%u]=%d out of range", i, u);
            if (u == v) return fail(RFMF_ERR_INVALID, "self loop at vertex %lld", (long long)v);
            if (i > offsets[v] && col[i - 1] >= u)
                return fail(RFMF_ERR_INVALID, "row %lld not strictly ascending", (long long)v);
            if (weight[i] == 0) return fail(RFMF_ERR_INVALID, "zero weight on edge (%lld,%d)", (long long)v, u);
            if (offsets[u + 1] < offsets[u]) return fail(RFMF_ERR_INVALID, "offsets not monotone at %d", u);
            const int32_t* b = col + offsets[u];
            const int32_t* e = col + offsets[u + 1];
            const int32_t* q = std::lower_bound(b, e, static_cast<int32_t>(v));
            if (q == e || *q != v || weight[q - col] != weight[i])
                return fail(RFMF_ERR_INVALID, "edge (%lld,%d) has no symmetric twin", (long long)v, u);
            s += std::llabs(static_cast<long long>(weight[i]));
            f.wsum2 += weight[i];
            f.unit = f.unit && (weight[i] == 1 || weight[i] == -1);
            f.small = f.small && (weight[i] >= -32767 && weight[i] <= 32767);
        }
        f.B = std::max(f.B, s);
    }
    if (f.B > std::numeric_limits<int32_t>::max())
        return fail(RFMF_ERR_CAPACITY, "max weighted degree %lld exceeds int32", (long long)f.B);
    return RFMF_OK;
}
}  // namespace

static int rfmf_csr_validate_impl(int64_t n, const uint32_t* offsets, const int32_t* col,
                                 const int32_t* weight, int64_t* max_weighted_degree) {
    CsrFacts f;
    const int rc = validate_csr(n, offsets, col, weight, f);
    if (rc == RFMF_OK && max_weighted_degree) *max_weighted_degree = f.B;
    return rc;
}

static int rfmf_graph_create_impl(rfmf_context* ctx, int64_t n, const uint32_t* offsets,
                                 const int32_t* col, const int32_t* weight, rfmf_graph** out) {
    if (!ctx || !out) return fail(RFMF_ERR_INVALID, "ctx/out is NULL");
    *out = nullptr;
    CsrFacts facts;
    if (int rc = validate_csr(n, offsets, col, weight, facts)) return rc;
    const uint64_t m2 = offsets[n];
    const int64_t B = facts.B, wsum2 = facts.wsum2;
    const bool unit = facts.unit, small = facts.small;
    CU(cudaSetDevice(ctx->device));
    auto g = std::unique_ptr<rfmf_graph>(new (std::nothrow) rfmf_graph());
    if (!g) return fail(RFMF_ERR_NOMEM, "host allocation failed");
    g->ctxHold.set(ctx);
    g->ctx = ctx;
    g->n = n;
    g->m = static_cast<int64_t>(m2 / 2);
    g->B = B;
    g->wsum2 = wsum2;
    g->unit16 = unit && n <= 32768 && m2 < (uint64_t(1) << 31);
    g->packed32 = small && n <= 65536 && m2 < (uint64_t(1) << 30);
    const uint64_t ob = (static_cast<uint64_t>(n + 1) * 4u + 15u) & ~uint64_t(15);
    g->offBytes = ob > 0xFFFFFFF0ull ? 0xFFFFFFF0u : static_cast<uint32_t>(ob);
    std::vector<uint32_t> ho(ob / 4, offsets[n]);
    std::memcpy(ho.data(), offsets, (n + 1) * sizeof(uint32_t));
    std::vector<Edge> he(m2);
    for (uint64_t i = 0; i < m2; ++i) he[i] = Edge{col[i], weight[i]};
    int rc = g->offsets.alloc(ob);
    if (rc) return rc;
    rc = g->edges.alloc(m2 * sizeof(Edge));
    if (rc) return rc;
    cudaStream_t st = ctx->stream;
    CU(cudaMemcpyAsync(g->offsets.p, ho.data(), ob, cudaMemcpyHostToDevice, st));
    if (m2) CU(cudaMemcpyAsync(g->edges.p, he.data(), m2 * sizeof(Edge), cudaMemcpyHostToDevice, st));
    std::vector<uint16_t> h16;
    std::vector<uint32_t> h32;
    if (g->unit16) {
        g->u16Bytes = align16(static_cast<uint32_t>(m2 * 2));
        h16.assign(g->u16Bytes / 2, 0);
        for (uint64_t i = 0; i < m2; ++i)
            h16[i] = static_cast<uint16_t>((static_cast<uint32_t>(col[i]) << 1) | (weight[i] < 0 ? 1u : 0u));
        if ((rc = g->u16.alloc(g->u16Bytes))) return rc;
        CU(cudaMemcpyAsync(g->u16.p, h16.data(), g->u16Bytes, cudaMemcpyHostToDevice, st));
    }
    if (g->packed32) {
        g->p32Bytes = align16(static_cast<uint32_t>(m2 * 4));
        h32.assign(g->p32Bytes / 4, 0);
        for (uint64_t i = 0; i < m2; ++i)
            h32[i] = (static_cast<uint32_t>(weight[i]) << 16) | static_cast<uint32_t>(col[i]);
        if ((rc = g->p32.alloc(g->p32Bytes))) return rc;
        CU(cudaMemcpyAsync(g->p32.p, h32.data(), g->p32Bytes, cudaMemcpyHostToDevice, st));
    }
    CU(cudaStreamSynchronize(st));
    *out = g.release();
    return RFMF_OK;
}

namespace rfmf {
void let_go(const rfmf_graph* g) {
    if (g->holders.fetch_sub(1) != 1) return;
    cudaSetDevice(g->ctx->device);
    delete g;
}
}  // namespace rfmf

extern "C" int rfmf_graph_destroy(rfmf_graph* g) {
    if (!g) return RFMF_OK;
    let_go(g);
    return RFMF_OK;
}

extern "C" int rfmf_graph_info(const rfmf_graph* g, int64_t* n, int64_t* m, int64_t* B) {
    if (!g) return fail(RFMF_ERR_INVALID, "graph is NULL");
    if (n) *n = g->n;
    if (m) *m = g->m;
    if (B) *B = g->B;
    return RFMF_OK;
}
// ------------------------------------------------------------------ batch
namespace rfmf {
// Warps per chain: one unless a chain has enough vertex blocks to keep more
// warps busy (about 384 blocks of 8 vertices per extra warp).
int choose_warps(int maxN, const rfmf_launch_config& c, int64_t chains, int sms) {
    if (c.threads_per_chain) return c.threads_per_chain / 32;
    int W = 1;
    const int nblk = (maxN + 7) / 8;
    // About 768 vertex blocks per warp.
    while (W < 4 && nblk >= 384 * 2 * W) W *= 2;
    // Too few chains to fill the SMs: widen each chain while all chains stay
    // within 8 warps per SM and the current width still has a vertex block
    // per thread.  One warp per chain is the most efficient form once chains
    // alone fill the SMs; below that, per-chain latency is what the extra
    // warps buy (GB300, 256 chains of ER n = 2000: 67.5 -> 88.6 M
    // chain-steps/s from one warp to four; 32 chains of ER n = 800: 6.7 -> 11.0).
    const int sized = W;
    while (W < kMaxAutoWarps && chains > 0 && chains * 2 * W <= int64_t(8) * sms && nblk >= 32 * W)
        W *= 2;
    // Two warps for latency alone lose to one on graphs of under 4096
    // vertices (16 vertex blocks per lane) outside the phases heavy in
    // winner rows, which a one-graph batch widens by itself (GB300, 512
    // chains, us per sweep at one / two warps: ER n = 2000 d = 19 P = 128
    // 9.10 / 6.84 but P = 8 2.37 / 3.15 and P = 1 1.98 / 2.23; the 50x60
    // torus 4.11 / 4.10 at P = 128, 2.44 / 3.20 at P = 8); on larger ones
    // two win at every phase (ER n = 5000 d = 5 P = 1 3.57 / 3.15, P = 16
    // 4.43 / 4.24; 70x70 torus and random tree n = 5000 alike); four, where
    // the chains are few enough, win at every phase (256 chains: ER n = 2000
    // 4.65 / 9.10 at P = 128 and 1.89 / 1.98 at P = 1 for four / one).
    if (sized == 1 && W == 2 && nblk < 512) W = 1;
    // Past four warps only for large graphs, where each thread keeps at
    // least four vertex blocks (GB300, 32-64 chains: torus n = 20000 +15% at
    // P = 128 and +29% at P = 1 from four warps to eight, tree n = 10000 +2%
    // / +10%; ER n = 5000 -1% / +5%, so it stays at four).
    while (W >= kMaxAutoWarps && W < kMaxLatencyWarps && chains > 0 && chains * 2 * W <= int64_t(8) * sms &&
           nblk >= 256 * W)
        W *= 2;
    return W;
}

// Bits of the block-iteration field of the compact int32 key (kernel
// key_bits): ceil(log2(blocks per thread)), at least 4.
int key_bits(int64_t n, int T) {
    const int64_t iters = ((n + 7) / 8 + T - 1) / T;
    int kb = 4;
    while ((int64_t(1) << kb) < iters) ++kb;
    return kb;
}

// The kernel's int32 path packs score * 2^kb + (2^kb - 1 - k) into one int:
// (betaMax * B + max|gum| + 1) * 2^kb must stay below 2^31.
bool compact_key_safe(int64_t total, double t0, int64_t B, int kb) {
    const double bmax = std::round(std::log(1.0 + static_cast<double>(std::max<int64_t>(total, 1))) /
                                   t0 * 1048576.0);
    return (bmax * static_cast<double>(B) + static_cast<double>(kGumbelMaxMag) + 1.0) *
               std::ldexp(1.0, kb) < 2147483647.0;
}

}  // namespace rfmf

// C ABI entry points: no C++ exception crosses the boundary.
extern "C" int rfmf_graph_create(rfmf_context* ctx, int64_t n, const uint32_t* offsets,
                                 const int32_t* col, const int32_t* weight, rfmf_graph** out) {
    try {
        return rfmf_graph_create_impl(ctx, n, offsets, col, weight, out);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_graph_create");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_graph_create");
    }
}

extern "C" int rfmf_beta_tables(const double* t0s, int64_t C, int64_t total_steps,
                                int64_t* run_end, int32_t* run_val, int64_t* chain_off,
                                int64_t cap, int64_t* runs) {
    try {
        return rfmf_beta_tables_impl(t0s, C, total_steps, run_end, run_val, chain_off, cap, runs);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_beta_tables");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_beta_tables");
    }
}

extern "C" int rfmf_csr_validate(int64_t n, const uint32_t* offsets, const int32_t* col,
                                 const int32_t* weight, int64_t* max_weighted_degree) {
    try {
        return rfmf_csr_validate_impl(n, offsets, col, weight, max_weighted_degree);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_csr_validate");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_csr_validate");
    }
}
