// rfmf_kernel.cu -- the RFMF sweep kernel for GB300 (sm_103a).
//
// Method (gt-tinker/rfmf, src/anneal_kernels.cu:262-491): per sweep, every
// vertex v draws a Q20 Gumbel key from Philox4x32-10 (key = chain seed,
// counter = (sweep, v>>3)), scores gum + beta*delta(v) with delta(v) the exact
// cut gain of flipping v, and the best score of each group g = v mod P (ties
// to the smallest v) wins; the P winners then flip, exactly as if flipped one
// after another in group order.
//
// GB300 design (not the reference's):
//   * One CTA runs one chain at a time and keeps ALL of that chain's mutable
//     state in shared memory for the whole window: D[v] = spin[v]*S[v] (the
//     per-vertex gain, int32), the spins as bits, and the best-so-far spins
//     as bits.  HBM is touched only for the read-only CSR (L1/L2 resident)
//     and the beta run table.
//   * Persistent CTAs pull chains from a work queue, so many graphs of uneven
//     size run in one launch.
//   * SELECT reads only D (one 16-byte LDS per 4 vertices).  The part of the
//     Philox counter that depends only on the sweep is hoisted out of the
//     vertex loop (rounds 1-3 lose 3 multiplies and 3 xors per block).
//   * The group argmax keeps eight register accumulators per thread (one per
//     Philox lane j) when every thread's lane j always lands in one group
//     (8*T divisible by P), folds them with warp shuffles over packed 64-bit
//     (biased score, ~v) keys, and lands one shared-memory atomic per group
//     per warp.  Other P fall back to one shared atomic per vertex.
//   * FLIP needs no winner-winner correction walk.  With D kept per vertex,
//     negating the winners' D and scattering 2*w*s_b*s_x into D[x] over the
//     winners' rows leaves the winners with D_final, and the cut gain of the
//     whole flip set is exactly (sum delta_pre - sum D_final) / 2 -- the same
//     integer the reference's corr[] formulation (src/anneal_kernels.cu:
//     133-192, 420-440) adds up.
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "rfmf_device.h"

namespace rfmf {

namespace {

// Published Philox4x32 constants (Salmon et al. 2011).
constexpr uint32_t kM0 = 0xD2511F53u;
constexpr uint32_t kM1 = 0xCD9E8D57u;
constexpr uint32_t kW0 = 0x9E3779B9u;
constexpr uint32_t kW1 = 0xBB67AE85u;

__device__ __forceinline__ void mulwide(uint32_t a, uint32_t b, uint32_t& hi,
                                        uint32_t& lo) {
    const uint64_t p = static_cast<uint64_t>(a) * b;
    hi = static_cast<uint32_t>(p >> 32);
    lo = static_cast<uint32_t>(p);
}

// Round keys that stay in registers for a chain's whole window: rounds 3..10
// (index 2..9); rounds 1 and 2 are folded into the per-sweep constants.
struct ChainKeys {
    uint32_t k0[10];
    uint32_t k1[10];
};

__device__ __forceinline__ ChainKeys make_keys(uint64_t seed) {
    ChainKeys k;
    uint32_t a = static_cast<uint32_t>(seed), b = static_cast<uint32_t>(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        k.k0[r] = a;
        k.k1[r] = b;
        a += kW0;
        b += kW1;
    }
    return k;
}

// Per-sweep constants.  The Philox counter is (step_lo, step_hi, b, 0): words
// 0, 1 and 3 are the same for every vertex block of a sweep, so half of round
// 1 and a quarter of rounds 2 and 3 do not depend on b.
struct SweepConst {
    uint32_t A;   // round-1 xor for word 0:  step_hi ^ k0[0]
    uint32_t Cc;  // round-2 xor for word 0:  hi(M1 * w2_r1) ^ k0[1]
    uint32_t Dc;  // round-2 xor for word 2:  lo(M0 * step_lo) ^ k1[1]
    uint32_t E;   // round-3 xor for word 0:  lo(M1 * w2_r1) ^ k0[2]
};

__device__ __forceinline__ SweepConst make_sweep(uint64_t step, const ChainKeys& k) {
    const uint32_t slo = static_cast<uint32_t>(step);
    const uint32_t shi = static_cast<uint32_t>(step >> 32);
    uint32_t hi0, lo0;
    mulwide(kM0, slo, hi0, lo0);
    const uint32_t w2r1 = hi0 ^ k.k1[0];   // counter word 3 (block >> 32) is 0
    uint32_t hi1, lo1;
    mulwide(kM1, w2r1, hi1, lo1);
    SweepConst c;
    c.A = shi ^ k.k0[0];
    c.Cc = hi1 ^ k.k0[1];
    c.Dc = lo0 ^ k.k1[1];
    c.E = lo1 ^ k.k0[2];
    return c;
}

// Philox4x32-10 of counter (step, b, 0) under the chain key.  Bit-identical
// to the reference's philox4x32_10(gumbelBlockCounter(step, b), key)
// (src/philox.cuh:77-119).
__device__ __forceinline__ void philox_block(uint32_t b, const SweepConst& c,
                                             const ChainKeys& k, uint32_t& x0,
                                             uint32_t& x1, uint32_t& x2,
                                             uint32_t& x3) {
    uint32_t hi, lo;
    // round 1
    mulwide(kM1, b, hi, lo);
    uint32_t v0 = hi ^ c.A;
    uint32_t v1 = lo;
    // round 2 (word 2 input is sweep-uniform: its product lives in Cc/E)
    mulwide(kM0, v0, hi, lo);
    v0 = v1 ^ c.Cc;
    uint32_t v2 = hi ^ c.Dc;
    uint32_t v3 = lo;
    // round 3 (word 1 input is sweep-uniform: lo(M1 * w2r1) folded into E)
    uint32_t h0, l0, h1, l1;
    mulwide(kM0, v0, h0, l0);
    mulwide(kM1, v2, h1, l1);
    v0 = h1 ^ c.E;
    v1 = l1;
    v2 = h0 ^ v3 ^ k.k1[2];
    v3 = l0;
#pragma unroll
    for (int r = 3; r < 10; ++r) {
        mulwide(kM0, v0, h0, l0);
        mulwide(kM1, v2, h1, l1);
        v0 = h1 ^ v1 ^ k.k0[r];
        v1 = l1;
        v2 = h0 ^ v3 ^ k.k1[r];
        v3 = l0;
    }
    x0 = v0;
    x1 = v1;
    x2 = v2;
    x3 = v3;
}

// Packed argmax key [biased score : 32 | ~v : 32]: unsigned order = score
// order, ties to the smaller v; 0 is the empty slot (src/philox.cuh:128-152).
__device__ __forceinline__ unsigned long long pack_key(int32_t score, int32_t v) {
    return (static_cast<unsigned long long>(static_cast<uint32_t>(score) ^ 0x80000000u) << 32) |
           static_cast<unsigned long long>(~static_cast<uint32_t>(v));
}

__device__ __forceinline__ int32_t key_vertex(unsigned long long key) {
    return static_cast<int32_t>(~static_cast<uint32_t>(key));
}

__device__ __forceinline__ unsigned long long shfl_xor_u64(unsigned long long x, int m) {
    const uint32_t lo = __shfl_xor_sync(0xFFFFFFFFu, static_cast<uint32_t>(x), m);
    const uint32_t hi = __shfl_xor_sync(0xFFFFFFFFu, static_cast<uint32_t>(x >> 32), m);
    return (static_cast<unsigned long long>(hi) << 32) | lo;
}

__device__ __forceinline__ int spin_of(const uint32_t* bits, int v) {
    return (bits[v >> 5] >> (v & 31)) & 1;
}

__device__ __forceinline__ void raise_error(const DevLaunch& L, int code, int item) {
    if (atomicCAS(L.error, 0, code) == 0) *L.errorItem = item;
}

// Exact int64 sum over the CTA; every thread receives the total.
__device__ __forceinline__ int64_t block_sum(int64_t v, int64_t* red) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, m);
    const int nw = blockDim.x >> 5;
    if (nw == 1) return v;
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    int64_t t = 0;
    for (int w = 0; w < nw; ++w) t += red[w];
    __syncthreads();
    return t;
}

// Shared-memory layout for one chain, sized for the launch's largest graph.
struct Smem {
    int32_t* D;                 // nPad (multiple of 8) per-vertex gains
    uint32_t* bits;             // spin bits
    uint32_t* best;             // best-spin bits
    unsigned long long* slots;  // Pmax packed keys (int32 score mode)
    long long* scoreSlots;      // alias of slots (int64 score mode)
    int32_t* ids;               // Pmax (int64 mode second-pass ids)
    int32_t* win;               // Pmax winners of the current sweep
    int64_t* red;               // 32 block-reduction partials
    int32_t* lut;               // 16
};

__device__ __forceinline__ size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

__device__ __forceinline__ Smem carve(unsigned char* base, const DevLaunch& L, int pmax) {
    Smem s;
    size_t o = 0;
    const size_t nPad = (static_cast<size_t>(L.maxN) + 7) & ~size_t(7);
    s.D = reinterpret_cast<int32_t*>(base + o);          o = align16(o + nPad * 4);
    s.bits = reinterpret_cast<uint32_t*>(base + o);      o = align16(o + static_cast<size_t>(L.maxWords) * 4);
    s.best = reinterpret_cast<uint32_t*>(base + o);      o = align16(o + static_cast<size_t>(L.maxWords) * 4);
    s.slots = reinterpret_cast<unsigned long long*>(base + o);
    s.scoreSlots = reinterpret_cast<long long*>(base + o); o = align16(o + static_cast<size_t>(pmax) * 8);
    s.ids = reinterpret_cast<int32_t*>(base + o);        o = align16(o + static_cast<size_t>(pmax) * 4);
    s.win = reinterpret_cast<int32_t*>(base + o);        o = align16(o + static_cast<size_t>(pmax) * 4);
    s.red = reinterpret_cast<int64_t*>(base + o);        o = align16(o + 32 * 8);
    s.lut = reinterpret_cast<int32_t*>(base + o);
    return s;
}

// ---------------------------------------------------------------- SELECT
// Scores every vertex of the chain from pre-sweep D and leaves, per group,
// the winner in the shared slots.  int32 mode: slots hold packed keys.
// int64 mode: scoreSlots hold the max score, ids the smallest v reaching it.

template <bool kScore64>
struct Acc;

template <>
struct Acc<false> {
    int32_t s[8];
    uint32_t b[8];
};
template <>
struct Acc<true> {
    long long s[8];
    uint32_t b[8];
};

template <bool kScore64>
__device__ __forceinline__ void score_vertex(Acc<kScore64>& a, int j, uint32_t r,
                                             int32_t d, int32_t beta, const int32_t* lut,
                                             uint32_t blk) {
    const int32_t gum = lut[r & 15u] + static_cast<int32_t>(r >> 4);
    if constexpr (kScore64) {
        const long long sc = static_cast<long long>(gum) +
                             static_cast<long long>(beta) * static_cast<long long>(d);
        if (sc > a.s[j]) { a.s[j] = sc; a.b[j] = blk; }
    } else {
        const int32_t sc = gum + beta * d;
        if (sc > a.s[j]) { a.s[j] = sc; a.b[j] = blk; }
    }
}

// Per-vertex fallback (8*T not divisible by P): one shared atomic per vertex.
template <bool kScore64>
__device__ __forceinline__ void score_vertex_atomic(const Smem& s, uint32_t r, int32_t d,
                                                    int32_t beta, int v, int g) {
    const int32_t gum = s.lut[r & 15u] + static_cast<int32_t>(r >> 4);
    if constexpr (kScore64) {
        const long long sc = static_cast<long long>(gum) +
                             static_cast<long long>(beta) * static_cast<long long>(d);
        atomicMax(&s.scoreSlots[g], sc);
    } else {
        atomicMax(&s.slots[g], pack_key(gum + beta * d, v));
    }
}

template <bool kScore64>
__device__ void select_sweep(const Smem& s, int n, int P, int32_t beta, uint64_t step,
                             const ChainKeys& keys) {
    const int T = blockDim.x;
    const int tid = threadIdx.x;
    const int nblk = (n + 7) >> 3;
    const SweepConst sc = make_sweep(step, keys);
    const bool priv = ((8 * T) % P) == 0;

    if (priv) {
        Acc<kScore64> a;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if constexpr (kScore64) a.s[j] = LLONG_MIN; else a.s[j] = INT32_MIN;
            a.b[j] = 0;
        }
        for (int b = tid; b < nblk; b += T) {
            uint32_t x0, x1, x2, x3;
            philox_block(static_cast<uint32_t>(b), sc, keys, x0, x1, x2, x3);
            const int4 d0 = *reinterpret_cast<const int4*>(s.D + 8 * b);
            const int4 d1 = *reinterpret_cast<const int4*>(s.D + 8 * b + 4);
            const uint32_t ub = static_cast<uint32_t>(b);
            if (8 * b + 8 <= n) {
                score_vertex<kScore64>(a, 0, x0 & 0x7FFu, d0.x, beta, s.lut, ub);
                score_vertex<kScore64>(a, 1, (x0 >> 16) & 0x7FFu, d0.y, beta, s.lut, ub);
                score_vertex<kScore64>(a, 2, x1 & 0x7FFu, d0.z, beta, s.lut, ub);
                score_vertex<kScore64>(a, 3, (x1 >> 16) & 0x7FFu, d0.w, beta, s.lut, ub);
                score_vertex<kScore64>(a, 4, x2 & 0x7FFu, d1.x, beta, s.lut, ub);
                score_vertex<kScore64>(a, 5, (x2 >> 16) & 0x7FFu, d1.y, beta, s.lut, ub);
                score_vertex<kScore64>(a, 6, x3 & 0x7FFu, d1.z, beta, s.lut, ub);
                score_vertex<kScore64>(a, 7, (x3 >> 16) & 0x7FFu, d1.w, beta, s.lut, ub);
            } else {
                const int lim = n - 8 * b;   // 1..7 valid lanes in the tail block
                const uint32_t xw[4] = {x0, x1, x2, x3};
                const int32_t dd[8] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w};
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    if (j < lim) {
                        const uint32_t w = xw[j >> 1];
                        const uint32_t r = ((j & 1) ? (w >> 16) : w) & 0x7FFu;
                        score_vertex<kScore64>(a, j, r, dd[j], beta, s.lut, ub);
                    }
                }
            }
        }
        // Thread t's lane j always feeds group (8t + j) mod P.  Fold what can
        // be folded in registers, then land one atomic per distinct group.
        if constexpr (!kScore64) {
            unsigned long long k[8];
#pragma unroll
            for (int j = 0; j < 8; ++j)
                k[j] = (a.s[j] == INT32_MIN) ? 0ull
                                             : pack_key(a.s[j], static_cast<int32_t>(8 * a.b[j] + j));
            if ((256 % P) == 0) {
                // Groups repeat with period P inside a warp's 256 vertices.
                // P in {1, 2, 4}: lane j feeds group j mod P; fold halves.
                if (P <= 4) {
#pragma unroll
                    for (int j = 0; j < 4; ++j) if (k[j + 4] > k[j]) k[j] = k[j + 4];
                }
                if (P <= 2) {
#pragma unroll
                    for (int j = 0; j < 2; ++j) if (k[j + 2] > k[j]) k[j] = k[j + 2];
                }
                if (P == 1) {
                    if (k[1] > k[0]) k[0] = k[1];
                }
                const int lanePeriod = (P >= 8) ? (P >> 3) : 1;   // lanes sharing groups
#pragma unroll
                for (int m = 16; m >= 1; m >>= 1) {
                    if (m >= lanePeriod) {
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const unsigned long long o = shfl_xor_u64(k[j], m);
                            if (o > k[j]) k[j] = o;
                        }
                    }
                }
                const int lane = tid & 31;
                if (lane < lanePeriod) {
                    const int jn = (P < 8) ? P : 8;
#pragma unroll
                    for (int j = 0; j < 8; ++j)
                        if (j < jn && k[j]) atomicMax(&s.slots[(8 * tid + j) % P], k[j]);
                }
            } else {
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    if (k[j]) atomicMax(&s.slots[(8 * tid + j) % P], k[j]);
            }
        } else {
            // int64 scores: max score per group first, then (next barrier)
            // the smallest v among the accumulators that reach it.
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (a.s[j] != LLONG_MIN) atomicMax(&s.scoreSlots[(8 * tid + j) % P], a.s[j]);
            __syncthreads();
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int g = (8 * tid + j) % P;
                if (a.s[j] != LLONG_MIN && a.s[j] == s.scoreSlots[g])
                    atomicMin(&s.ids[g], static_cast<int32_t>(8 * a.b[j] + j));
            }
        }
    } else {
        // General P: every vertex lands its own atomic.
        for (int b = tid; b < nblk; b += T) {
            uint32_t x0, x1, x2, x3;
            philox_block(static_cast<uint32_t>(b), sc, keys, x0, x1, x2, x3);
            const uint32_t xw[4] = {x0, x1, x2, x3};
            const int v0 = 8 * b;
            int g = v0 % P;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int v = v0 + j;
                if (v < n) {
                    const uint32_t w = xw[j >> 1];
                    const uint32_t r = ((j & 1) ? (w >> 16) : w) & 0x7FFu;
                    score_vertex_atomic<kScore64>(s, r, s.D[v], beta, v, g);
                }
                if (++g == P) g = 0;
            }
        }
        if constexpr (kScore64) {
            // Second pass: regenerate the scores, smallest v at the max.
            __syncthreads();
            for (int b = tid; b < nblk; b += T) {
                uint32_t x0, x1, x2, x3;
                philox_block(static_cast<uint32_t>(b), sc, keys, x0, x1, x2, x3);
                const uint32_t xw[4] = {x0, x1, x2, x3};
                const int v0 = 8 * b;
                int g = v0 % P;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int v = v0 + j;
                    if (v < n) {
                        const uint32_t w = xw[j >> 1];
                        const uint32_t r = ((j & 1) ? (w >> 16) : w) & 0x7FFu;
                        const int32_t gum = s.lut[r & 15u] + static_cast<int32_t>(r >> 4);
                        const long long scv = static_cast<long long>(gum) +
                                              static_cast<long long>(beta) * s.D[v];
                        if (scv == s.scoreSlots[g]) atomicMin(&s.ids[g], v);
                    }
                    if (++g == P) g = 0;
                }
            }
        }
    }
}

// ------------------------------------------------------------------ chain
template <bool kScore64>
__device__ void run_chain(const DevLaunch& L, const Smem& s, int item, int pmax) {
    const int T = blockDim.x;
    const int tid = threadIdx.x;
    DevChain& ch = L.chains[item];
    if (ch.graph < 0 || ch.graph >= L.ngraphs || ch.sched < 0 || ch.sched >= L.nscheds) {
        if (tid == 0) raise_error(L, kDevBadItem, item);
        return;
    }
    if (ch.sweepsDone >= ch.sweepsTotal && ch.cur != kUnsetCut) return;
    const DevGraph g = L.graphs[ch.graph];
    const DevSchedule sch = L.scheds[ch.sched];
    const int n = g.n;
    const int words = g.words;
    const uint32_t* __restrict__ off = g.offsets;
    const Edge* __restrict__ edges = g.edges;

    // ---- load state: spin bits (and best bits) into shared memory
    for (int w = tid; w < words; w += T) s.bits[w] = ch.spinBits[w];
    const bool fresh = (ch.cur == kUnsetCut);
    for (int w = tid; w < words; w += T) s.best[w] = fresh ? s.bits[w] : ch.bestBits[w];
    for (int i = tid; i < pmax; i += T) {
        s.slots[i] = kScore64 ? static_cast<unsigned long long>(LLONG_MIN) : 0ull;
        s.ids[i] = INT32_MAX;
    }
    __syncthreads();

    // ---- D[v] = spin[v] * sum_u w(v,u) spin[u]   (zero padding past n)
    const int nPad = (n + 7) & ~7;
    int64_t dsum = 0;
    for (int v = tid; v < nPad; v += T) {
        int32_t d = 0;
        if (v < n) {
            int64_t acc = 0;
            for (uint32_t i = off[v]; i < off[v + 1]; ++i) {
                const Edge e = edges[i];
                acc += spin_of(s.bits, e.col) ? e.w : -e.w;
            }
            d = static_cast<int32_t>(spin_of(s.bits, v) ? acc : -acc);
            dsum += d;
        }
        s.D[v] = d;
    }
    // cut = (sum_directed w - sum_v D[v]) / 4  -- exact integer identity.
    const int64_t cutD = (g.wsum2 - block_sum(dsum, s.red)) / 4;
    int64_t cur = ch.cur, best = ch.best;
    if (fresh) {
        cur = best = cutD;
    } else if (cur != cutD) {
        if (tid == 0) raise_error(L, kDevCutMismatch, item);
    }
    __syncthreads();

    // ---- beta cursor at the window start: first run with end > sweepBegin
    const uint64_t s0 = ch.sweepsDone;
    const uint64_t s1 = (ch.sweepsTotal - s0 > L.window) ? s0 + L.window : ch.sweepsTotal;
    int64_t lo = 0, hi = ch.betaRuns;   // search in [lo, hi)
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (static_cast<uint64_t>(ch.betaEnd[mid]) > s0) hi = mid; else lo = mid + 1;
    }
    int64_t run = lo;
    if (s1 > s0 && (run >= ch.betaRuns ||
                    static_cast<uint64_t>(ch.betaEnd[ch.betaRuns - 1]) < s1)) {
        if (tid == 0) raise_error(L, kDevBetaTable, item);
        return;
    }

    // ---- phase cursor at the window start
    int p = 0;
    uint64_t phaseEnd = 0;
    int P = 1;
    {
        uint64_t acc = 0;
        for (p = 0; p < sch.nphases; ++p) {
            if (sch.phaseP[p] == 0) continue;
            if (acc + sch.phaseIters[p] > s0) break;
            acc += sch.phaseIters[p];
        }
        if (p < sch.nphases) {
            phaseEnd = acc + sch.phaseIters[p];
            P = static_cast<int>(umin(sch.phaseP[p], static_cast<uint32_t>(n)));
        }
    }

    const ChainKeys keys = make_keys(ch.solverSeed);
    uint64_t improved = 0;
    uint64_t betaNext = (s1 > s0) ? static_cast<uint64_t>(ch.betaEnd[run]) : 0;
    int32_t beta = (s1 > s0) ? ch.betaVal[run] : 0;

    for (uint64_t sw = s0; sw < s1; ++sw) {
        // advance phase (skip P == 0 phases and exhausted ones)
        while (sw >= phaseEnd) {
            ++p;
            if (p >= sch.nphases) break;
            if (sch.phaseP[p] == 0) continue;
            phaseEnd += sch.phaseIters[p];
            P = static_cast<int>(umin(sch.phaseP[p], static_cast<uint32_t>(n)));
        }
        if (sw >= betaNext) {
            ++run;
            betaNext = static_cast<uint64_t>(ch.betaEnd[run]);
            beta = ch.betaVal[run];
        }
        const uint64_t step = sw + 1;   // 1-based sweep id

        select_sweep<kScore64>(s, n, P, beta, step, keys);
        __syncthreads();

        // ---- FLIP 1: winners; negate their D, flip their spins
        int64_t loc = 0;
        for (int gi = tid; gi < P; gi += T) {
            int v;
            if constexpr (kScore64) {
                const int32_t id = s.ids[gi];
                v = (id == INT32_MAX) ? -1 : id;
                s.scoreSlots[gi] = LLONG_MIN;
                s.ids[gi] = INT32_MAX;
            } else {
                const unsigned long long k = s.slots[gi];
                s.slots[gi] = 0ull;
                v = k ? key_vertex(k) : -1;
            }
            s.win[gi] = v;
            if (v >= 0) {
                const int32_t d = s.D[v];
                loc += d;
                s.D[v] = -d;
                atomicXor(&s.bits[v >> 5], 1u << (v & 31));
            }
        }
        __syncthreads();

        // ---- FLIP 2: scatter 2*w*s_b*s_x into D[x] over the winners' rows;
        // L consecutive lanes share a row (coalesced CSR walk).
        {
            int lanes = 1;
            while (lanes * 2 * P <= T && lanes < 32) lanes <<= 1;
            const int sub = tid & (lanes - 1);
            for (int gi = tid / lanes; gi < P; gi += T / lanes) {
                const int v = s.win[gi];
                if (v < 0) continue;
                const int sv = spin_of(s.bits, v);
                const uint32_t e1 = off[v + 1];
                for (uint32_t i = off[v] + sub; i < e1; i += lanes) {
                    const Edge e = edges[i];
                    const int sx = spin_of(s.bits, e.col);
                    atomicAdd(&s.D[e.col], (sv == sx) ? 2 * e.w : -2 * e.w);
                }
            }
        }
        __syncthreads();

        // ---- FLIP 3: gain = (sum delta_pre - sum D_final) / 2
        for (int gi = tid; gi < P; gi += T) {
            const int v = s.win[gi];
            if (v >= 0) loc -= s.D[v];
        }
        const int64_t gain = block_sum(loc, s.red) / 2;
        cur += gain;
        if (cur > best) {
            best = cur;
            ++improved;
            for (int w = tid; w < words; w += T) s.best[w] = s.bits[w];
        }
    }
    __syncthreads();

    // ---- write the state back
    for (int w = tid; w < words; w += T) {
        ch.spinBits[w] = s.bits[w];
        ch.bestBits[w] = s.best[w];
    }
    if (tid == 0) {
        ch.cur = cur;
        ch.best = best;
        ch.sweepsDone = s1;
        ch.improvedSweeps += improved;
    }
}

// kMinBlocks sets the register budget through the launch bounds: 2 -> 128,
// 3 -> 80, 4 -> 64 registers per thread at up to 256 threads per CTA.  The
// host picks the variant that keeps every chain resident (see autotune()).
template <bool kScore64, int kMinBlocks>
__global__ void __launch_bounds__(256, kMinBlocks) rfmf_anneal_kernel(const DevLaunch L, int pmax) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Smem s = carve(smem, L, pmax);
    __shared__ int s_item;
    if (threadIdx.x < 16) s.lut[threadIdx.x] = L.lut[threadIdx.x];
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(L.queue, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= L.nchains) break;
        run_chain<kScore64>(L, s, L.order[it], pmax);
        __syncthreads();
    }
}

}  // namespace

size_t smem_bytes(int maxN, int maxWords, int pmax) {
    auto a16 = [](size_t x) { return (x + 15) & ~size_t(15); };
    const size_t nPad = (static_cast<size_t>(maxN) + 7) & ~size_t(7);
    size_t o = a16(nPad * 4);
    o = a16(o + static_cast<size_t>(maxWords) * 4);
    o = a16(o + static_cast<size_t>(maxWords) * 4);
    o = a16(o + static_cast<size_t>(pmax) * 8);
    o = a16(o + static_cast<size_t>(pmax) * 4);
    o = a16(o + static_cast<size_t>(pmax) * 4);
    o = a16(o + 32 * 8);
    o += 16 * 4;
    return o;
}

// Register-budget variants: index 0 -> 128, 1 -> 80, 2 -> 64 registers.
constexpr int kNumVariants = 3;

const void* kernel_ptr(bool score64, int variant) {
    if (score64) {
        switch (variant) {
            case 0: return reinterpret_cast<const void*>(&rfmf_anneal_kernel<true, 2>);
            case 1: return reinterpret_cast<const void*>(&rfmf_anneal_kernel<true, 3>);
            default: return reinterpret_cast<const void*>(&rfmf_anneal_kernel<true, 4>);
        }
    }
    switch (variant) {
        case 0: return reinterpret_cast<const void*>(&rfmf_anneal_kernel<false, 2>);
        case 1: return reinterpret_cast<const void*>(&rfmf_anneal_kernel<false, 3>);
        default: return reinterpret_cast<const void*>(&rfmf_anneal_kernel<false, 4>);
    }
}

int num_variants() { return kNumVariants; }

cudaError_t launch_anneal(const DevLaunch& L, bool score64, int variant, int grid, int threads,
                          size_t smem, int pmax, cudaStream_t stream) {
    void* args[] = {const_cast<DevLaunch*>(&L), &pmax};
    return cudaLaunchKernel(kernel_ptr(score64, variant), dim3(grid), dim3(threads), args, smem,
                            stream);
}

}  // namespace rfmf
