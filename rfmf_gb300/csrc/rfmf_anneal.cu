// rfmf_anneal.cu -- the RFMF sweep kernel for GB300 (sm_103a).
//
// Method (gt-tinker/rfmf, src/anneal_kernels.cu:262-491): per sweep, every
// vertex v draws a Q20 Gumbel key from Philox4x32-10 (key = chain seed,
// counter = (sweep, v>>3)), scores gum + beta*delta(v) with delta(v) the exact
// cut gain of flipping v, and the best score of each group g = v mod P (ties
// to the smallest v) wins; the P winners then flip, exactly as if flipped one
// after another in group order.
//
// GB300 design (not the reference's):
//   * A persistent CTA takes work items of up to K chains of ONE graph.  The
//     graph's CSR is staged once per item into shared memory by bulk async
//     copies (cp.async.bulk + mbarrier) in a compact format (2 bytes per entry
//     for +-1 weights), and K warp groups (W warps each) run K chains side by
//     side on that one copy.  Chains never synchronise with each other: a
//     chain's barriers are __syncwarp (W == 1) or a named barrier of its own.
//   * All mutable chain state stays in shared memory for the whole window:
//     D[v] = spin[v]*S[v] (the per-vertex gain; int8 with a +128 bias when
//     the max weighted degree B <= 127, else int32), the spins as bits, and
//     the best-so-far spins as bits.  Graphs too big for shared memory walk
//     their CSR in HBM instead, in the most compact entry form they allow
//     (2, 4 or 8 bytes); the chain state stays resident.
//   * SELECT reads only D.  The sweep-uniform part of the Philox counter is
//     hoisted (rounds 1-3 lose 3 multiplies and 3 xors per block) and three
//     vertex blocks are in flight per thread.
//   * The group argmax keeps eight register accumulators per thread (one per
//     Philox lane j) whenever every thread's lane j lands in one group, folds
//     them with warp shuffles, and stores one packed (biased score, ~v) key
//     per group; other P fall back to shared-memory atomics.
//   * FLIP has no winner-winner correction walk.  With D kept per vertex,
//     negating the winners' D and scattering 2*w*s_b*s_x into D[x] over the
//     winners' rows leaves every winner holding D_final, and the cut gain of
//     the whole flip set is exactly (sum delta_pre - sum D_final) / 2: the
//     same integer the reference's corr[] formulation (src/anneal_kernels.cu:
//     133-192, 420-440) adds up.  Row walks issue their loads four at a time.
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <type_traits>

#include "rfmf_device.h"

namespace rfmf {

namespace {

// Published Philox4x32 constants (Salmon et al. 2011).
constexpr uint32_t kM0 = 0xD2511F53u;
constexpr uint32_t kM1 = 0xCD9E8D57u;
constexpr uint32_t kW0 = 0x9E3779B9u;
constexpr uint32_t kW1 = 0xBB67AE85u;

// Bound on mbarrier polls while a CSR bulk copy lands (each poll may suspend
// the thread for a hardware-chosen interval); past it the CTA stops taking
// work and the launch reports kDevCopyTimeout.
constexpr int kMaxCopyPolls = 1 << 22;

__device__ __forceinline__ void mulwide(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
    const uint64_t p = static_cast<uint64_t>(a) * b;
    hi = static_cast<uint32_t>(p >> 32);
    lo = static_cast<uint32_t>(p);
}

// Philox round keys, k0[r] = seed_lo + r*W0, k1[r] = seed_hi + r*W1.
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
// 0, 1 and 3 are the same for every vertex block of a sweep.
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

// Philox4x32-10 of counter (step, b, 0) under the chain key; bit-identical to
// philox4x32_10(gumbelBlockCounter(step, b), key) of src/philox.cuh:77-119.
__device__ __forceinline__ void philox_block(uint32_t b, const SweepConst& c,
                                             const ChainKeys& k, uint32_t x[4]) {
    uint32_t hi, lo;
    mulwide(kM1, b, hi, lo);                  // round 1
    uint32_t v0 = hi ^ c.A;
    uint32_t v1 = lo;
    mulwide(kM0, v0, hi, lo);                 // round 2
    v0 = v1 ^ c.Cc;
    uint32_t v2 = hi ^ c.Dc;
    uint32_t v3 = lo;
    uint32_t h0, l0, h1, l1;
    mulwide(kM0, v0, h0, l0);                 // round 3
    mulwide(kM1, v2, h1, l1);
    v0 = h1 ^ c.E;
    v1 = l1;
    v2 = h0 ^ v3 ^ k.k1[2];
    v3 = l0;
#pragma unroll
    for (int r = 3; r < 10; ++r) {            // rounds 4..10
        mulwide(kM0, v0, h0, l0);
        mulwide(kM1, v2, h1, l1);
        v0 = h1 ^ v1 ^ k.k0[r];
        v1 = l1;
        v2 = h0 ^ v3 ^ k.k1[r];
        v3 = l0;
    }
    x[0] = v0;
    x[1] = v1;
    x[2] = v2;
    x[3] = v3;
}

// 11-bit field of lane j (src/philox.cuh:121-126).
__device__ __forceinline__ uint32_t field(const uint32_t x[4], int j) {
    return ((j & 1) ? (x[j >> 1] >> 16) : x[j >> 1]) & 0x7FFu;
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

__device__ __forceinline__ int spin_of(const uint32_t* bits, int v) {
    return (bits[v >> 5] >> (v & 31)) & 1;
}

__device__ __forceinline__ void raise_error(const DevLaunch& L, int code, int item) {
    if (atomicCAS(L.error, 0, code) == 0) *L.errorItem = item;
}

// Barrier of one chain's warp group: __syncwarp for one warp, else named
// barrier grp+1 over the group's 32W threads (barrier 0 is __syncthreads).
__device__ __forceinline__ void group_sync(int grp, int T) {
    if (T == 32) {
        __syncwarp();
    } else {
        asm volatile("bar.sync %0, %1;" ::"r"(grp + 1), "r"(T) : "memory");
    }
}

// ------------------------------------------------------------ D storage
// int32 gains: plain words.
struct D32 {
    static constexpr int32_t kBias = 0;
    // Stored values (D + kBias) of block b; D32 stores D itself.
    __device__ static __forceinline__ void load8raw(const unsigned char* D, int b, int32_t d[8]) {
        load8(D, b, d);
    }
    __device__ static __forceinline__ void load8(const unsigned char* D, int b, int32_t d[8]) {
        const int4 a = *reinterpret_cast<const int4*>(D + 32 * b);
        const int4 c = *reinterpret_cast<const int4*>(D + 32 * b + 16);
        d[0] = a.x; d[1] = a.y; d[2] = a.z; d[3] = a.w;
        d[4] = c.x; d[5] = c.y; d[6] = c.z; d[7] = c.w;
    }
    __device__ static __forceinline__ int32_t get(const unsigned char* D, int v) {
        return reinterpret_cast<const int32_t*>(D)[v];
    }
    __device__ static __forceinline__ void set(unsigned char* D, int v, int32_t d) {
        reinterpret_cast<int32_t*>(D)[v] = d;
    }
    __device__ static __forceinline__ void add(unsigned char* D, int v, int32_t delta) {
        atomicAdd(reinterpret_cast<int*>(D) + v, delta);
    }
};

// int8 gains stored as D + 128 in [1, 255] (|D| <= B <= 127).  Every partial
// sum during a scatter is the gain of some spin configuration, so it stays in
// range and a shifted 32-bit atomicAdd on the containing word never carries
// into the neighbouring byte.  (x ^ 0x80) read as int8 is D.
// Byte k of x sign-extended to 32 bits: prmt with selector nibbles whose msb
// requests sign replication (the __byte_perm intrinsic drops that bit).
template <int k>
__device__ __forceinline__ int32_t sbyte(uint32_t x) {
    int32_t r;
    if constexpr (k == 3) {
        r = static_cast<int32_t>(x) >> 24;
    } else {
        constexpr uint32_t sel = static_cast<uint32_t>(k) | ((8u | k) << 4) | ((8u | k) << 8) |
                                 ((8u | k) << 12);
        asm("prmt.b32 %0, %1, 0, %2;" : "=r"(r) : "r"(x), "n"(sel));
    }
    return r;
}

// Byte k of x zero-extended to 32 bits.
template <int k>
__device__ __forceinline__ int32_t ubyte(uint32_t x) {
    int32_t r;
    if constexpr (k == 3) {
        r = static_cast<int32_t>(x >> 24);
    } else {
        constexpr uint32_t sel = static_cast<uint32_t>(k) | 0x4440u;
        asm("prmt.b32 %0, %1, 0, %2;" : "=r"(r) : "r"(x), "n"(sel));
    }
    return r;
}

struct D8 {
    static constexpr int32_t kBias = 128;
    // Stored values D + 128 of block b (no sign handling: callers fold the
    // bias into a constant).
    __device__ static __forceinline__ void load8raw(const unsigned char* D, int b, int32_t d[8]) {
        const uint2 w = *reinterpret_cast<const uint2*>(D + 8 * b);
        d[0] = ubyte<0>(w.x);
        d[1] = ubyte<1>(w.x);
        d[2] = ubyte<2>(w.x);
        d[3] = ubyte<3>(w.x);
        d[4] = ubyte<0>(w.y);
        d[5] = ubyte<1>(w.y);
        d[6] = ubyte<2>(w.y);
        d[7] = ubyte<3>(w.y);
    }
    __device__ static __forceinline__ void load8(const unsigned char* D, int b, int32_t d[8]) {
        const uint2 w = *reinterpret_cast<const uint2*>(D + 8 * b);
        const uint32_t a = w.x ^ 0x80808080u, c = w.y ^ 0x80808080u;
        d[0] = sbyte<0>(a);
        d[1] = sbyte<1>(a);
        d[2] = sbyte<2>(a);
        d[3] = sbyte<3>(a);
        d[4] = sbyte<0>(c);
        d[5] = sbyte<1>(c);
        d[6] = sbyte<2>(c);
        d[7] = sbyte<3>(c);
    }
    __device__ static __forceinline__ int32_t get(const unsigned char* D, int v) {
        return static_cast<int32_t>(static_cast<int8_t>(D[v] ^ 0x80u));
    }
    __device__ static __forceinline__ void set(unsigned char* D, int v, int32_t d) {
        D[v] = static_cast<unsigned char>(d + 128);
    }
    __device__ static __forceinline__ void add(unsigned char* D, int v, int32_t delta) {
        atomicAdd(reinterpret_cast<unsigned int*>(D + (v & ~3)),
                  static_cast<unsigned int>(delta) << (8 * (v & 3)));
    }
};

// ------------------------------------------------------------ CSR access
struct CsrView {
    const uint32_t* off;
    const void* ent;
};

template <int kFmt>
struct Csr;

template <>
struct Csr<kCsrUnit16> {
    __device__ static __forceinline__ void row(const CsrView& c, int v, uint32_t& lo, uint32_t& hi) {
        lo = c.off[v];
        hi = c.off[v + 1];
    }
    __device__ static __forceinline__ uint32_t raw(const CsrView& c, uint32_t i) {
        return static_cast<const uint16_t*>(c.ent)[i];
    }
    __device__ static __forceinline__ void entry(const CsrView& c, uint32_t i, int& col, int& w) {
        const uint32_t e = static_cast<const uint16_t*>(c.ent)[i];
        col = static_cast<int>(e >> 1);
        w = 1 - 2 * static_cast<int>(e & 1u);
    }
};

template <>
struct Csr<kCsrPacked32> {
    __device__ static __forceinline__ void row(const CsrView& c, int v, uint32_t& lo, uint32_t& hi) {
        lo = c.off[v];
        hi = c.off[v + 1];
    }
    __device__ static __forceinline__ void entry(const CsrView& c, uint32_t i, int& col, int& w) {
        const uint32_t e = static_cast<const uint32_t*>(c.ent)[i];
        col = static_cast<int>(e & 0xFFFFu);
        w = static_cast<int32_t>(e) >> 16;
    }
};

template <>
struct Csr<kCsrGlobal> {
    __device__ static __forceinline__ void row(const CsrView& c, int v, uint32_t& lo, uint32_t& hi) {
        lo = __ldg(c.off + v);
        hi = __ldg(c.off + v + 1);
    }
    __device__ static __forceinline__ void entry(const CsrView& c, uint32_t i, int& col, int& w) {
        const int2 e = __ldg(static_cast<const int2*>(c.ent) + i);
        col = e.x;
        w = e.y;
    }
};

// The compact entries read from HBM on the read-only path: a quarter (16-bit)
// or half (32-bit) of the bytes of the {col, w} pairs per entry.
template <>
struct Csr<kCsrGlobal16> {
    __device__ static __forceinline__ void row(const CsrView& c, int v, uint32_t& lo, uint32_t& hi) {
        lo = __ldg(c.off + v);
        hi = __ldg(c.off + v + 1);
    }
    __device__ static __forceinline__ uint32_t raw(const CsrView& c, uint32_t i) {
        return __ldg(static_cast<const unsigned short*>(c.ent) + i);
    }
    __device__ static __forceinline__ void entry(const CsrView& c, uint32_t i, int& col, int& w) {
        const uint32_t e = raw(c, i);
        col = static_cast<int>(e >> 1);
        w = 1 - 2 * static_cast<int>(e & 1u);
    }
};

template <>
struct Csr<kCsrGlobal32> {
    __device__ static __forceinline__ void row(const CsrView& c, int v, uint32_t& lo, uint32_t& hi) {
        lo = __ldg(c.off + v);
        hi = __ldg(c.off + v + 1);
    }
    __device__ static __forceinline__ void entry(const CsrView& c, uint32_t i, int& col, int& w) {
        const uint32_t e = __ldg(static_cast<const unsigned int*>(c.ent) + i);
        col = static_cast<int>(e & 0xFFFFu);
        w = static_cast<int32_t>(e) >> 16;
    }
};

// ------------------------------------------------------------ chain region
struct ChainSmem {
    unsigned char* D;
    uint32_t* bits;
    uint32_t* best;
    unsigned char* sb;           // spins as bytes (1 = +1), kept equal to bits
    unsigned long long* slots;   // int32 mode: packed keys
    long long* scores;           // int64 mode: max score per group (aliases slots)
    int32_t* ids;                // int64 mode: winner id per group
    int32_t* win;                // winners of the current sweep
    int64_t* red;                // one partial per warp of the group
};

__device__ __forceinline__ ChainSmem carve_chain(unsigned char* base, const DevLaunch& L,
                                                 int dbytes) {
    const ChainLayout c = chain_layout(L.maxN, L.maxWords, L.pmax, L.warpsPerChain, dbytes);
    ChainSmem s;
    s.D = base + c.d;
    s.bits = reinterpret_cast<uint32_t*>(base + c.bits);
    s.best = reinterpret_cast<uint32_t*>(base + c.best);
    s.sb = base + c.sb;
    s.slots = reinterpret_cast<unsigned long long*>(base + c.slots);
    s.scores = reinterpret_cast<long long*>(base + c.slots);
    s.ids = reinterpret_cast<int32_t*>(base + c.ids);
    s.win = reinterpret_cast<int32_t*>(base + c.win);
    s.red = reinterpret_cast<int64_t*>(base + c.red);
    return s;
}

// Exact int64 sum over a chain's warp group; every thread gets the total.
// (The partials buffer is rewritten only after two more group barriers.)
__device__ __forceinline__ int64_t group_sum(int64_t v, const ChainSmem& s, int t, int T, int grp) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, m);
    if (T == 32) return v;
    if ((t & 31) == 0) s.red[t >> 5] = v;
    group_sync(grp, T);
    int64_t tot = 0;
    for (int w = 0; w < (T >> 5); ++w) tot += s.red[w];
    return tot;
}

// int32 sum over a chain's warp group with redux.sync (int8 gains: the sums
// of a sweep's winner gains are bounded by 2 * 127 * P, far inside int32).
__device__ __forceinline__ int32_t group_sum32(int32_t v, const ChainSmem& s, int t, int T, int grp) {
    v = __reduce_add_sync(0xFFFFFFFFu, v);
    if (T == 32) return v;
    if ((t & 31) == 0) s.red[t >> 5] = v;
    group_sync(grp, T);
    int64_t tot = 0;
    for (int w = 0; w < (T >> 5); ++w) tot += s.red[w];
    return static_cast<int32_t>(tot);
}

// ---------------------------------------------------------------- SELECT
// Scores every vertex from pre-sweep D and leaves the winner of every group
// g < P in the chain's slots (int32 mode: packed key; int64 mode: ids[g]).
// Slots start each sweep at their empty value (reset by FLIP's reader).

// Per-phase constants, recomputed only when P changes (no integer division
// or modulo by P inside a sweep).
struct PhaseCfg {
    int P;
    int mode;       // 0: P | 256, groups repeat every P/8 lanes (register fold +
                    //    warp reduction); 1: 8T % P == 0, thread-private groups;
                    // 2: general P, one shared atomic per vertex
    int period;     // mode 0: P/8 (or 1 for P < 8); lanes l and l + period share groups
    int g0;         // mode 1: (8 t) mod P
    int laneShift;  // FLIP scatter: log2 of the lanes that share one row
    uint32_t gmask; // mode 0, P >= 16: the lanes sharing this lane's groups
};

__device__ __forceinline__ PhaseCfg phase_cfg(int P, int t, int T) {
    PhaseCfg c;
    c.P = P;
    c.mode = ((256 % P) == 0) ? 0 : (((8 * T) % P) == 0 ? 1 : 2);
    c.period = (P >= 8) ? (P >> 3) : 1;
    c.g0 = (8 * t) % P;
    int sh = 0;
    while ((2 << sh) * P <= T && sh < 5) ++sh;
    c.laneShift = sh;
    const uint32_t rep = (c.period >= 32) ? 1u : (c.period == 16) ? 0x00010001u
                       : (c.period == 8) ? 0x01010101u : (c.period == 4) ? 0x11111111u : 0x55555555u;
    c.gmask = rep << ((t & 31) & (c.period - 1));
    return c;
}

// Compact int32 argmax key.  A thread visits its vertex blocks b = t + k*T
// for k = 0, 1, ... (at most 2^kb of them); lane j of block k gets
//   key = score * 2^kb + (2^kb - 1 - k),   score = gum + beta * delta,
// so one integer max per vertex keeps the best score and, among equal
// scores, the smallest k, i.e. the smallest vertex (v = 8(t + kT) + j grows
// with k).  With f the 11-bit field and i = f & 15,
//   gum * 2^kb = LUT[i] * 2^kb + (f >> 4) * 2^kb
//              = (LUT[i] * 2^kb - i * 2^(kb-4)) + f * 2^(kb-4)     (kb >= 4)
// so key = TK[i] + f * 2^(kb-4) + (beta * 2^kb) * delta + (2^kb - 1 - k) with a
// 16-entry table TK.  The host enables this path only when
// (betaMax * B + max|gum| + 1) * 2^kb < 2^31 for every chain, so every key and
// partial sum is exact in int32; otherwise the launch takes the int64 path.
//
// Instruction budget per vertex: TK lives in a register (lane L holds
// TK[L & 15]) and is read with one shuffle whose source lane is the Philox
// word itself (a shuffle takes its source lane modulo 32, and lanes L and
// L + 16 hold the same entry, so the low word needs no masking and the high
// one a single shift); the field's multiple f * 2^(kb-4) is one multiply-add
// on the FMA pipe (a mul.hi for the high half-word, whose field sits at bit
// 16); the final add and max fuse into one add-max.
struct KeyCfg {
    int kb;          // bits of the block-iteration field
    uint32_t mulF;   // 2^(kb-4): f * mulF for a low-half field
    uint32_t mulHi;  // 2^(kb+12): umulhi(x & 0x07FF0000, mulHi) = f * 2^(kb-4)
    int32_t tkLane;  // TK[lane & 15]
};

__device__ __forceinline__ int key_bits(int n, int T) {
    const int iters = ((n + 7) / 8 + T - 1) / T;
    int kb = 4;
    while ((1 << kb) < iters) ++kb;
    return kb;
}

__device__ __forceinline__ KeyCfg key_cfg(int n, int T, int t, const int32_t* lut) {
    KeyCfg kc;
    kc.kb = key_bits(n, T);
    kc.mulF = 1u << (kc.kb - 4);
    kc.mulHi = 1u << (kc.kb + 12);
    const int i = t & 15;
    kc.tkLane = lut[i] * (1 << kc.kb) - i * static_cast<int32_t>(kc.mulF);
    return kc;
}

// Keys of one block's 8 vertices folded into acc; lanes j >= lim are skipped
// (the shuffles still run on every lane: the caller keeps the warp converged).
// `tkb` is this lane's TK[lane & 15] plus the block's constant part
// (2^kb - 1 - k) - bias * beta * 2^kb, so the shuffle delivers TK[i] with the
// constant already added and d holds the stored (biased) gains.  All sums are
// modular int32: only the final key is in range, and it is exact.  kF0: kb ==
// 4, the field's multiple is the field itself.
template <bool kMasked, bool kF0>
__device__ __forceinline__ void score8_key(int32_t acc[8], const uint32_t x[4], const int32_t d[8],
                                           int32_t betaK, int32_t tkb, const KeyCfg& kc, int lim) {
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        const uint32_t xs = x[w] >> 16;
        const int32_t tk0 = __shfl_sync(0xFFFFFFFFu, tkb, static_cast<int>(x[w]));
        const int32_t tk1 = __shfl_sync(0xFFFFFFFFu, tkb, static_cast<int>(xs));
        int32_t f0, f1;
        if constexpr (kF0) {
            f0 = static_cast<int32_t>(x[w] & 0x7FFu);
            f1 = static_cast<int32_t>(xs & 0x7FFu);
        } else {
            f0 = static_cast<int32_t>((x[w] & 0x7FFu) * kc.mulF);
            f1 = static_cast<int32_t>(__umulhi(x[w] & 0x07FF0000u, kc.mulHi));
        }
        const int32_t k0 = static_cast<int32_t>(static_cast<uint32_t>(betaK) * static_cast<uint32_t>(d[2 * w]) +
                                                static_cast<uint32_t>(tk0));
        const int32_t k1 = static_cast<int32_t>(static_cast<uint32_t>(betaK) * static_cast<uint32_t>(d[2 * w + 1]) +
                                                static_cast<uint32_t>(tk1));
        if (!kMasked || 2 * w < lim) acc[2 * w] = __viaddmax_s32(k0, f0, acc[2 * w]);
        if (!kMasked || 2 * w + 1 < lim) acc[2 * w + 1] = __viaddmax_s32(k1, f1, acc[2 * w + 1]);
    }
}

// NB vertex blocks b, b + T, ... (block iterations k, k + 1, ...) scored with
// their Philox draws in flight together.
template <int NB, bool kMasked, bool kF0, class DP>
__device__ __forceinline__ void score_blocks(int32_t acc[8], const ChainSmem& s, const SweepConst& sc,
                                             const ChainKeys& keys, int b, int T, int32_t betaK,
                                             int32_t tkb, const KeyCfg& kc, int lim) {
    uint32_t x[NB][4];
    int32_t d[NB][8];
#pragma unroll
    for (int q = 0; q < NB; ++q) philox_block(static_cast<uint32_t>(b + q * T), sc, keys, x[q]);
    if constexpr (NB >= 3) {
        // Three blocks' Philox words in flight; each block's gains are
        // loaded just before it is scored so that they fit the registers.
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            DP::load8raw(s.D, b + q * T, d[0]);
            score8_key<kMasked, kF0>(acc, x[q], d[0], betaK, tkb - q, kc, lim);
        }
    } else {
#pragma unroll
        for (int q = 0; q < NB; ++q) DP::load8raw(s.D, b + q * T, d[q]);
#pragma unroll
        for (int q = 0; q < NB; ++q) score8_key<kMasked, kF0>(acc, x[q], d[q], betaK, tkb - q, kc, lim);
    }
}

// The block loop of select32 (trip counts uniform per warp: its blocks at
// step k are wb + kT .. wb + kT + 31, so the table shuffles run converged):
// three blocks in flight while the whole warp has three full blocks left,
// then two, then a clamped, masked single-block tail.
template <bool kF0, class DP>
__device__ __forceinline__ void select_blocks(int32_t acc[8], const ChainSmem& s, const SweepConst& sc,
                                              const ChainKeys& keys, int n, int t, int T,
                                              int32_t betaK, int32_t tkBase, const KeyCfg& kc) {
    const int nfull = n >> 3;
    const int nblk = (n + 7) >> 3;
    const int wb = t & ~31;
    int b = t, k = 0;
    for (; wb + 2 * T + 31 < nfull - k * T; b += 3 * T, k += 3)
        score_blocks<3, false, kF0, DP>(acc, s, sc, keys, b, T, betaK, tkBase - k, kc, 8);
    for (; wb + T + 31 < nfull - k * T; b += 2 * T, k += 2)
        score_blocks<2, false, kF0, DP>(acc, s, sc, keys, b, T, betaK, tkBase - k, kc, 8);
    for (; wb + k * T < nblk; b += T, ++k) {
        const int bb = (b < nblk) ? b : nblk - 1;
        const int lim = (b < nfull) ? 8 : ((b == nfull) ? (n & 7) : 0);
        score_blocks<1, true, kF0, DP>(acc, s, sc, keys, bb, T, betaK, tkBase - k, kc, lim);
    }
}

// FLIP step 1 for one winner v (or none, v < 0) of group g: publish it, add
// its pre-sweep gain to loc, negate the gain, flip the spin bit and byte.
template <class DP, class Loc>
__device__ __forceinline__ void flip_winner(const ChainSmem& s, int g, int v, Loc& loc) {
    s.win[g] = v;
    if (v >= 0) {
        const int32_t d = DP::get(s.D, v);
        loc += d;
        DP::set(s.D, v, -d);
        atomicXor(&s.bits[v >> 5], 1u << (v & 31));
        s.sb[v] ^= 1u;
    }
}

// FLIP step 2 of a one-warp chain at P >= 64 with +-1 weights in the 16-bit
// CSR (entry = col << 1 | w < 0) and int8 gains: one lane per winner row,
// four entries in flight.  With spins as bits (1 = +1), D[col] changes by +2
// when s_b, s_col and the weight bit XOR to 0, else by -2, added into byte
// lane col & 3 of word col >> 2 (the biased bytes never carry, see D8).
// (At smaller P the generic walk, which spreads a row over several lanes,
// is faster.)
template <int kFmt>
__device__ __forceinline__ void flip2_unit16_d8_warp(const ChainSmem& s, const CsrView& csr, int P, int lane) {
    unsigned int* Dw = reinterpret_cast<unsigned int*>(s.D);
    const unsigned char* sb = s.sb;
    for (int gi = lane; gi < P; gi += 32) {
        const int v = s.win[gi];
        if (v < 0) continue;
        const uint32_t sv = sb[v];
        uint32_t i, hi;
        Csr<kFmt>::row(csr, v, i, hi);
        for (; i + 4 <= hi; i += 4) {
            uint32_t e[4], sx[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) e[j] = Csr<kFmt>::raw(csr, i + j);
#pragma unroll
            for (int j = 0; j < 4; ++j) sx[j] = sb[e[j] >> 1];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t neg = (sv ^ sx[j] ^ e[j]) & 1u;
                atomicAdd(Dw + (e[j] >> 3), (neg ? 0xFFFFFFFEu : 2u) << ((e[j] & 6u) << 2));
            }
        }
        for (; i < hi; ++i) {
            const uint32_t e0 = Csr<kFmt>::raw(csr, i);
            const uint32_t neg = (sv ^ sb[e0 >> 1] ^ e0) & 1u;
            atomicAdd(Dw + (e0 >> 3), (neg ? 0xFFFFFFFEu : 2u) << ((e0 & 6u) << 2));
        }
    }
}

// How select32 hands its winners to FLIP step 1.
enum WinnerHandoff : int {
    kWinSlots = 0,      // packed keys in the group slots (any warp count, any P)
    kWinFlipped = 1,    // FLIP step 1 done here (one-warp chains, P <= 8)
    kWinPublished = 2   // winner ids in s.win (one-warp chains, P >= 16)
};

template <class DP, class Loc>
__device__ int select32(const ChainSmem& s, const int32_t* lut, const KeyCfg& kc, int n,
                         const PhaseCfg& pc, int32_t beta, uint64_t step, const ChainKeys& keys,
                         int t, int T, Loc& loc) {
    const SweepConst sc = make_sweep(step, keys);
    const int P = pc.P;
    const int M = (1 << kc.kb) - 1;
    if (pc.mode != 2) {
        const int32_t betaK = beta * (1 << kc.kb);
        int32_t acc[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[j] = INT32_MIN;
        // Per-sweep part of the table register: (2^kb - 1) - bias * beta * 2^kb.
        const int32_t tkBase = static_cast<int32_t>(static_cast<uint32_t>(kc.tkLane) + static_cast<uint32_t>(M) -
                                                    static_cast<uint32_t>(DP::kBias) * static_cast<uint32_t>(betaK));
        if (kc.kb == 4) select_blocks<true, DP>(acc, s, sc, keys, n, t, T, betaK, tkBase, kc);
        else select_blocks<false, DP>(acc, s, sc, keys, n, t, T, betaK, tkBase, kc);
        const int wb = t & ~31;
        // Group argmax on the compact keys.  Equal keys mean equal score and
        // block iteration k, so they differ only in the thread t (vertex
        // 8(t + kT) + j): the lowest lane holding the maximum wins.  Only the
        // winners are widened to packed (score, v) keys for the slots.
        const int lane = t & 31;
        if (P == 1) {
            // One group: fold the eight accumulators in registers (on equal
            // keys the smaller j, i.e. the smaller vertex, stays), then one
            // warp max; the lowest lane holding it has the smallest vertex
            // (equal keys share the block iteration k) and, in a one-warp
            // chain, flips it itself, so no lane needs its j; in a wider
            // chain it offers its packed key to the group slot (one atomic
            // per warp).  Measured on GB300 at 2048 one-warp chains: -2.4%
            // per P = 1 sweep on ER n = 2000, -13% on n = 256; folding at
            // P = 4 and 8 was slower (the winners' broadcast).
            int32_t m = acc[0];
            int jb = 0;
#pragma unroll
            for (int j = 1; j < 8; ++j)
                if (acc[j] > m) { m = acc[j]; jb = j; }
            const int32_t mx = __reduce_max_sync(0xFFFFFFFFu, m);
            const uint32_t bal = __ballot_sync(0xFFFFFFFFu, m == mx);
            if (lane == __ffs(bal) - 1) {
                const int kk = M - (mx & M);
                const int v = (mx != INT32_MIN) ? 8 * (wb + lane + kk * T) + jb : -1;
                if (T == 32) flip_winner<DP>(s, 0, v, loc);
                else if (v >= 0) atomicMax(&s.slots[0], pack_key(mx >> kc.kb, v));
            }
            return (T == 32) ? kWinFlipped : kWinSlots;
        }
        if (pc.mode == 0 && P <= 8) {
            int32_t mj[8];
            int32_t vj[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                mj[j] = __reduce_max_sync(0xFFFFFFFFu, acc[j]);
                const uint32_t bal = __ballot_sync(0xFFFFFFFFu, acc[j] == mj[j]);
                const int kk = M - (mj[j] & M);
                vj[j] = 8 * (wb + (__ffs(bal) - 1) + kk * T) + j;
            }
            // Groups g < P collect j = g, g + P, ...: larger key, then smaller v.
            if (P <= 4) {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (mj[j + 4] > mj[j] || (mj[j + 4] == mj[j] && vj[j + 4] < vj[j])) {
                        mj[j] = mj[j + 4];
                        vj[j] = vj[j + 4];
                    }
            }
            if (P <= 2) {
#pragma unroll
                for (int j = 0; j < 2; ++j)
                    if (mj[j + 2] > mj[j] || (mj[j + 2] == mj[j] && vj[j + 2] < vj[j])) {
                        mj[j] = mj[j + 2];
                        vj[j] = vj[j + 2];
                    }
            }
            if (P == 1 && (mj[1] > mj[0] || (mj[1] == mj[0] && vj[1] < vj[0]))) {
                mj[0] = mj[1];
                vj[0] = vj[1];
            }
            if (T == 32) {
                // Every lane holds every group's winner: lane g flips group g.
                int mine = -1;
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    if (lane == j) mine = (mj[j] != INT32_MIN) ? vj[j] : -1;
                if (lane < P) flip_winner<DP>(s, lane, mine, loc);
                return kWinFlipped;
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (lane == j && j < P && mj[j] != INT32_MIN)
                    atomicMax(&s.slots[j], pack_key(mj[j] >> kc.kb, vj[j]));
            }
        } else if (pc.mode == 0) {
            // P = 8p, p = P/8 in {2..32}: lanes r, r + p, ... share group 8r + j.
            // Shuffle steps outermost so the eight chains overlap, then one
            // divergent block for the p writing lanes.
            int32_t mx[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) mx[j] = acc[j];
#pragma unroll
            for (int m = 16; m >= 2; m >>= 1) {
                if (m >= pc.period) {
#pragma unroll
                    for (int j = 0; j < 8; ++j) mx[j] = max(mx[j], __shfl_xor_sync(0xFFFFFFFFu, mx[j], m));
                }
            }
            uint32_t bal[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) bal[j] = __ballot_sync(0xFFFFFFFFu, acc[j] == mx[j]) & pc.gmask;
            if (lane < pc.period) {
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int kk = M - (mx[j] & M);
                    const int v = 8 * (wb + (__ffs(bal[j]) - 1) + kk * T) + j;
                    const int g = 8 * lane + j;
                    if (T == 32) s.win[g] = (mx[j] != INT32_MIN) ? v : -1;
                    else if (mx[j] != INT32_MIN) atomicMax(&s.slots[g], pack_key(mx[j] >> kc.kb, v));
                }
            }
            if (T == 32) return kWinPublished;
        } else {
            int g = pc.g0;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (acc[j] != INT32_MIN) {
                    const int kk = M - (acc[j] & M);
                    atomicMax(&s.slots[g], pack_key(acc[j] >> kc.kb, 8 * (t + kk * T) + j));
                }
                if (++g == P) g = 0;
            }
        }
    } else {
        // General P: one shared atomic per vertex, plain score.
        for (int bb = t; 8 * bb < n; bb += T) {
            uint32_t x[4];
            int32_t d[8];
            philox_block(static_cast<uint32_t>(bb), sc, keys, x);
            DP::load8(s.D, bb, d);
            int g = (8 * bb) % P;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int v = 8 * bb + j;
                if (v < n) {
                    const uint32_t r = field(x, j);
                    const int32_t sv = lut[r & 15u] + static_cast<int32_t>(r >> 4) + beta * d[j];
                    atomicMax(&s.slots[g], pack_key(sv, v));
                }
                if (++g == P) g = 0;
            }
        }
    }
    return kWinSlots;
}

// int64 scores (the reference's two-pass path, src/anneal_kernels.cu:348-378,
// taken when annealScoreSafeInt32 fails): max score per group, then the
// smallest v reaching it.
struct Acc64 {
    long long s[8];
    uint32_t b[8];
};

__device__ __forceinline__ void score8_64(Acc64& a, const uint32_t x[4], const int32_t d[8],
                                          int32_t beta, const int32_t* lut, uint32_t b, int lim) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        if (j < lim) {
            const uint32_t r = field(x, j);
            const long long sc = static_cast<long long>(lut[r & 15u] + static_cast<int32_t>(r >> 4)) +
                                 static_cast<long long>(beta) * d[j];
            if (sc > a.s[j]) { a.s[j] = sc; a.b[j] = b; }
        }
    }
}

template <class DP>
__device__ void select64(const ChainSmem& s, const int32_t* lut, int n, const PhaseCfg& pc,
                         int32_t beta, uint64_t step, const ChainKeys& keys, int t, int T,
                         int grp) {
    const SweepConst sc = make_sweep(step, keys);
    const int P = pc.P;
    const bool priv = pc.mode != 2;
    if (priv) {
        Acc64 a;
#pragma unroll
        for (int j = 0; j < 8; ++j) { a.s[j] = LLONG_MIN; a.b[j] = 0; }
        for (int b = t; 8 * b < n; b += T) {
            uint32_t x[4];
            int32_t d[8];
            philox_block(static_cast<uint32_t>(b), sc, keys, x);
            DP::load8(s.D, b, d);
            const int lim = (n - 8 * b < 8) ? (n - 8 * b) : 8;
            score8_64(a, x, d, beta, lut, static_cast<uint32_t>(b), lim);
        }
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (a.s[j] != LLONG_MIN) atomicMax(&s.scores[(8 * t + j) % P], a.s[j]);
        group_sync(grp, T);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int g = (8 * t + j) % P;
            if (a.s[j] != LLONG_MIN && a.s[j] == s.scores[g])
                atomicMin(&s.ids[g], static_cast<int32_t>(8 * a.b[j] + j));
        }
    } else {
        for (int pass = 0; pass < 2; ++pass) {
            for (int b = t; 8 * b < n; b += T) {
                uint32_t x[4];
                int32_t d[8];
                philox_block(static_cast<uint32_t>(b), sc, keys, x);
                DP::load8(s.D, b, d);
                int g = (8 * b) % P;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int v = 8 * b + j;
                    if (v < n) {
                        const uint32_t r = field(x, j);
                        const long long sv =
                            static_cast<long long>(lut[r & 15u] + static_cast<int32_t>(r >> 4)) +
                            static_cast<long long>(beta) * d[j];
                        if (pass == 0) atomicMax(&s.scores[g], sv);
                        else if (sv == s.scores[g]) atomicMin(&s.ids[g], v);
                    }
                    if (++g == P) g = 0;
                }
            }
            if (pass == 0) group_sync(grp, T);
        }
    }
}

// ------------------------------------------------------------------ chain
// Pacing between the chains of one CTA.  The warp scheduler does not share
// issue slots evenly, so chains of one item drift apart within a window (by
// up to ~40% of it measured on GB300), and the CTA then runs its last chains
// with few warps while the others wait at the item barrier.  Every
// kPaceEvery sweeps a chain publishes its progress; one more than kPaceLead
// sweeps ahead of the slowest chain of its CTA yields its issue slots with
// short sleeps (bounded: at most kPaceSleeps of them per check).
constexpr int kPaceEvery = 32;
constexpr int kPaceLead = 64;
constexpr int kPaceSleeps = 32;

// The CTA header holds the pacing state: progress of each warp group at
// bytes 160..223, the number of running groups at 224.
__device__ __forceinline__ volatile int* pace_state() {
    extern __shared__ __align__(128) unsigned char smem[];
    return reinterpret_cast<volatile int*>(smem + 160);
}

__device__ __forceinline__ int slowest_chain(const volatile int* prog) {
    const int active = prog[16];
    int m = INT_MAX;
    for (int q = 0; q < active; ++q) m = min(m, prog[q]);
    return m;
}

template <class DP, int kFmt, bool kS64>
__device__ void run_chain(const DevLaunch& L, const ChainSmem& s, const CsrView& csr,
                          const int32_t* lut, int ci, int t, int T, int grp) {
    volatile int* prog = pace_state();
    DevChain& ch = L.chains[ci];
    if (ch.sweepsDone >= ch.sweepsTotal && ch.cur != kUnsetCut) {
        if (t == 0) prog[grp] = INT_MAX;
        return;
    }
    const DevGraph& g = L.graphs[ch.graph];
    const DevSchedule sch = L.scheds[ch.sched];
    const int n = g.n;
    const int words = g.words;

    // ---- state in: spin bits and best bits; empty group slots
    const bool fresh = (ch.cur == kUnsetCut);
    for (int w = t; w < words; w += T) {
        const uint32_t sb = ch.spinBits[w];
        s.bits[w] = sb;
        s.best[w] = fresh ? sb : ch.bestBits[w];
    }
    for (int i = t; i < L.pmax; i += T) {
        s.slots[i] = kS64 ? static_cast<unsigned long long>(LLONG_MIN) : 0ull;
        s.ids[i] = INT32_MAX;
    }
    const KeyCfg kc = key_cfg(n, T, t, lut);
    group_sync(grp, T);
    const int nPad = (n + 7) & ~7;
    for (int v = t; v < nPad; v += T)
        s.sb[v] = (v < n) ? static_cast<unsigned char>(spin_of(s.bits, v)) : 0;
    group_sync(grp, T);

    // ---- D[v] = spin[v] * sum_u w(v,u) spin[u]; padding past n is 0
    int64_t dsum = 0;
    for (int v = t; v < nPad; v += T) {
        int32_t d = 0;
        if (v < n) {
            uint32_t lo, hi;
            Csr<kFmt>::row(csr, v, lo, hi);
            int32_t acc = 0;
            for (uint32_t i = lo; i < hi; ++i) {
                int col, w;
                Csr<kFmt>::entry(csr, i, col, w);
                acc += s.sb[col] ? w : -w;
            }
            d = s.sb[v] ? acc : -acc;
            dsum += d;
        }
        DP::set(s.D, v, d);
    }
    // cut = (sum over directed entries of w - sum_v D[v]) / 4, exactly.
    const int64_t cutD = (g.wsum2 - group_sum(dsum, s, t, T, grp)) / 4;
    int64_t cur = ch.cur, best = ch.best;
    if (fresh) {
        cur = best = cutD;
    } else if (cur != cutD) {
        if (t == 0) raise_error(L, kDevCutMismatch, ci);
    }

    // ---- window, beta cursor (first run with end > s0), phase cursor
    const uint64_t s0 = ch.sweepsDone;
    const uint64_t s1 = (ch.sweepsTotal - s0 > L.window) ? s0 + L.window : ch.sweepsTotal;
    int64_t run = 0;
    {
        int64_t lo = 0, hi = ch.betaRuns;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (static_cast<uint64_t>(ch.betaEnd[mid]) > s0) hi = mid; else lo = mid + 1;
        }
        run = lo;
    }
    if (s1 > s0 && (run >= ch.betaRuns ||
                    static_cast<uint64_t>(ch.betaEnd[ch.betaRuns - 1]) < s1)) {
        if (t == 0) {
            raise_error(L, kDevBetaTable, ci);
            prog[grp] = INT_MAX;
        }
        return;
    }
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
    PhaseCfg pc = phase_cfg(P, t, T);

    const ChainKeys keys = make_keys(ch.solverSeed);
    // Beta cursor in registers, with the following run prefetched one run
    // ahead (read-only path): a run change costs no dependent global load.
    const int64_t* __restrict__ bEnd = ch.betaEnd;
    const int32_t* __restrict__ bVal = ch.betaVal;
    const int64_t nRuns = ch.betaRuns;
    uint64_t betaNext = (s1 > s0) ? static_cast<uint64_t>(__ldg(bEnd + run)) : 0;
    int32_t beta = (s1 > s0) ? __ldg(bVal + run) : 0;
    uint64_t pfEnd = ~0ull;
    int32_t pfVal = 0;
    if (s1 > s0 && run + 1 < nRuns) {
        pfEnd = static_cast<uint64_t>(__ldg(bEnd + run + 1));
        pfVal = __ldg(bVal + run + 1);
    }
    uint64_t improved = 0;
    group_sync(grp, T);

    for (uint64_t sw = s0; sw < s1; ++sw) {
        if (sw >= phaseEnd) {
            while (sw >= phaseEnd) {
                ++p;
                if (p >= sch.nphases) break;
                if (sch.phaseP[p] == 0) continue;
                phaseEnd += sch.phaseIters[p];
                P = static_cast<int>(umin(sch.phaseP[p], static_cast<uint32_t>(n)));
            }
            pc = phase_cfg(P, t, T);
        }
        if (sw >= betaNext) {
            // Runs are never empty, so one step of the cursor per sweep.
            ++run;
            betaNext = pfEnd;
            beta = pfVal;
            if (run + 1 < nRuns) {
                pfEnd = static_cast<uint64_t>(__ldg(bEnd + run + 1));
                pfVal = __ldg(bVal + run + 1);
            }
        }
        if (((sw - s0) & (kPaceEvery - 1)) == 0) {
            const int mine = static_cast<int>(sw - s0);
            if (t == 0) prog[grp] = mine;
            int lead = mine - slowest_chain(prog);
            for (int q = 0; q < kPaceSleeps && lead > kPaceLead; ++q) {
                __nanosleep(2000);
                lead = mine - slowest_chain(prog);
            }
        }
        const uint64_t step = sw + 1;   // 1-based sweep id

        using Loc = typename std::conditional<std::is_same<DP, D8>::value, int32_t, int64_t>::type;
        Loc loc = 0;
        int handoff = kWinSlots;
        if constexpr (kS64) select64<DP>(s, lut, n, pc, beta, step, keys, t, T, grp);
        else handoff = select32<DP>(s, lut, kc, n, pc, beta, step, keys, t, T, loc);

        // ---- FLIP 1: winners; negate their gains, flip their spins
        if (handoff != kWinFlipped) {
            group_sync(grp, T);
            for (int gi = t; gi < P; gi += T) {
                int v;
                if constexpr (kS64) {
                    const int32_t id = s.ids[gi];
                    v = (id == INT32_MAX) ? -1 : id;
                    s.scores[gi] = LLONG_MIN;
                    s.ids[gi] = INT32_MAX;
                } else if (handoff == kWinPublished) {
                    v = s.win[gi];
                } else {
                    const unsigned long long k = s.slots[gi];
                    s.slots[gi] = 0ull;
                    v = k ? key_vertex(k) : -1;
                }
                flip_winner<DP>(s, gi, v, loc);
            }
        }
        group_sync(grp, T);

        // ---- FLIP 2: D[x] += 2 w s_b s_x over the winners' rows (new spins);
        // `lanes` consecutive threads share a row, four entries in flight.
        bool walked = false;
        if constexpr ((kFmt == kCsrUnit16 || kFmt == kCsrGlobal16) && std::is_same<DP, D8>::value) {
            if (T == 32 && P >= 64) {
                flip2_unit16_d8_warp<kFmt>(s, csr, P, t);
                walked = true;
            }
        }
        if (!walked) {
            const int lanes = 1 << pc.laneShift;
            const int sub = t & (lanes - 1);
            for (int gi = t >> pc.laneShift; gi < P; gi += T >> pc.laneShift) {
                const int v = s.win[gi];
                if (v < 0) continue;
                const int sv = s.sb[v];
                uint32_t lo, hi;
                Csr<kFmt>::row(csr, v, lo, hi);
                uint32_t i = lo + sub;
                for (; i + 3 * lanes < hi; i += 4 * lanes) {
                    int c0, w0, c1, w1, c2, w2, c3, w3;
                    Csr<kFmt>::entry(csr, i, c0, w0);
                    Csr<kFmt>::entry(csr, i + lanes, c1, w1);
                    Csr<kFmt>::entry(csr, i + 2 * lanes, c2, w2);
                    Csr<kFmt>::entry(csr, i + 3 * lanes, c3, w3);
                    const int s0b = s.sb[c0], s1b = s.sb[c1];
                    const int s2b = s.sb[c2], s3b = s.sb[c3];
                    DP::add(s.D, c0, (sv == s0b) ? 2 * w0 : -2 * w0);
                    DP::add(s.D, c1, (sv == s1b) ? 2 * w1 : -2 * w1);
                    DP::add(s.D, c2, (sv == s2b) ? 2 * w2 : -2 * w2);
                    DP::add(s.D, c3, (sv == s3b) ? 2 * w3 : -2 * w3);
                }
                for (; i < hi; i += lanes) {
                    int c0, w0;
                    Csr<kFmt>::entry(csr, i, c0, w0);
                    DP::add(s.D, c0, (sv == s.sb[c0]) ? 2 * w0 : -2 * w0);
                }
            }
        }
        group_sync(grp, T);

        // ---- FLIP 3: gain = (sum delta_pre - sum D_final) / 2
        for (int gi = t; gi < P; gi += T) {
            const int v = s.win[gi];
            if (v >= 0) loc -= DP::get(s.D, v);
        }
        int64_t gain;
        if constexpr (std::is_same<DP, D8>::value) gain = group_sum32(loc, s, t, T, grp) / 2;
        else gain = group_sum(loc, s, t, T, grp) / 2;
        cur += gain;
        if (cur > best) {
            best = cur;
            ++improved;
            for (int w = t; w < words; w += T) s.best[w] = s.bits[w];
        }
    }
    if (t == 0) prog[grp] = INT_MAX;
    group_sync(grp, T);

    // ---- state out
    for (int w = t; w < words; w += T) {
        ch.spinBits[w] = s.bits[w];
        ch.bestBits[w] = s.best[w];
    }
    if (t == 0) {
        ch.cur = cur;
        ch.best = best;
        ch.sweepsDone = s1;
        ch.improvedSweeps += improved;
    }
}

// ------------------------------------------------------------ bulk copy
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mbar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* mbar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(mbar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* mbar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(mbar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Stage graph g's compact CSR into shared memory: thread 0 arms the mbarrier
// with the byte count and issues the bulk copies (<= 64 KB each); every
// thread waits on the phase with a bounded poll.  Returns this thread's
// outcome (false: its polls ran out); the caller makes it CTA-uniform and
// advances the phase.
__device__ bool stage_csr(const DevGraph& g, unsigned char* dst, uint64_t* mbar, uint32_t phase) {
    const uint32_t total = g.offBytes + g.entBytes;
    if (threadIdx.x == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(mbar, total);
        const unsigned char* srcs[2] = {reinterpret_cast<const unsigned char*>(g.offsets),
                                        static_cast<const unsigned char*>(g.compact)};
        const uint32_t sizes[2] = {g.offBytes, g.entBytes};
        uint32_t o = 0;
        for (int k = 0; k < 2; ++k) {
            for (uint32_t c = 0; c < sizes[k]; c += 65536u) {
                const uint32_t len = (sizes[k] - c < 65536u) ? (sizes[k] - c) : 65536u;
                bulk_g2s(dst + o + c, srcs[k] + c, len, mbar);
            }
            o += sizes[k];
        }
    }
    bool ok = false;
    for (int i = 0; i < kMaxCopyPolls && !ok; ++i) ok = mbar_try_wait(mbar, phase);
    return ok;
}

// kDBytes: 1 -> D8, 4 -> D32.
template <int kDBytes, int kFmt, bool kS64>
__global__ void __launch_bounds__(512, 1) rfmf_anneal_kernel(const DevLaunch L) {
    using DP = typename std::conditional<kDBytes == 1, D8, D32>::type;
    extern __shared__ __align__(128) unsigned char smem[];
    int32_t* lut = reinterpret_cast<int32_t*>(smem);                 // 64 B
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + 128);        // 8 B
    int* sItem = reinterpret_cast<int*>(smem + 144);
    volatile int* sProg = pace_state();   // 16 progress words + running-group count
    unsigned char* csrBase = smem + kSmemHeader;
    unsigned char* chainBase = csrBase + L.csrBytes;

    const int T = 32 * L.warpsPerChain;
    const int grp = threadIdx.x / T;
    const int t = threadIdx.x - grp * T;
    const ChainSmem cs = carve_chain(chainBase + static_cast<size_t>(grp) * L.chainBytes, L, kDBytes);

    if (threadIdx.x < 16) lut[threadIdx.x] = L.lut[threadIdx.x];
    if (!csr_in_hbm(kFmt) && threadIdx.x == 0) mbar_init(mbar);
    __syncthreads();

    uint32_t phase = 0;
    int loaded = -1;
    for (;;) {
        if (threadIdx.x == 0) *sItem = atomicAdd(L.queue, 1);
        __syncthreads();
        const int it = *sItem;
        if (it >= L.nitems) break;
        const DevItem item = L.items[it];
        if (item.graph < 0 || item.graph >= L.ngraphs) {
            if (threadIdx.x == 0) raise_error(L, kDevBadItem, it);
            __syncthreads();
            continue;
        }
        uint64_t t0 = 0;
        if (threadIdx.x == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
        const DevGraph& g = L.graphs[item.graph];
        CsrView csr;
        if constexpr (csr_in_hbm(kFmt)) {
            csr.off = g.offsets;
            csr.ent = (kFmt == kCsrGlobal) ? static_cast<const void*>(g.edges) : g.compact;
        } else {
            if (item.graph != loaded) {
                // All threads agree on the outcome, so that a chain's
                // barriers never see part of its warp group leave.
                if (!__syncthreads_and(stage_csr(g, csrBase, mbar, phase))) {
                    // The copy may still be in flight.  Report it, then stay
                    // resident for a second, longer bounded wait: a CTA that
                    // retired with a copy outstanding would leave its target
                    // shared memory to whatever CTA the SM runs next.  The
                    // CTA then takes no more work; the host reports the error
                    // and the context is not to be reused.
                    if (threadIdx.x == 0) raise_error(L, kDevCopyTimeout, it);
                    bool landed = false;
                    for (int i = 0; i < 4 * kMaxCopyPolls && !landed; ++i) landed = mbar_try_wait(mbar, phase);
                    __syncthreads();
                    break;
                }
                phase ^= 1u;
                loaded = item.graph;
            }
            csr.off = reinterpret_cast<const uint32_t*>(csrBase);
            csr.ent = csrBase + g.offBytes;
        }
        const int active = (item.count < L.chainsPerCta) ? item.count : L.chainsPerCta;
        if (threadIdx.x < 16) sProg[threadIdx.x] = (static_cast<int>(threadIdx.x) < active) ? 0 : INT_MAX;
        if (threadIdx.x == 0) sProg[16] = active;
        __syncthreads();
        if (grp < active)
            run_chain<DP, kFmt, kS64>(L, cs, csr, lut, L.order[item.first + grp], t, T, grp);
        __syncthreads();
        if (threadIdx.x == 0 && L.itemNs) {
            uint64_t t1;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
            L.itemNs[it] = t1 - t0;
        }
    }
}

}  // namespace

// ------------------------------------------------------------ host hooks
// Kernel variants: D width {1, 4} x CSR format {unit16, packed32, HBM 8-byte,
// HBM 16-bit, HBM 32-bit} x score {int32, int64}.
template <int DB, bool S>
const void* kernel_for_format(int fmt) {
    switch (fmt) {
        case kCsrUnit16: return reinterpret_cast<const void*>(&rfmf_anneal_kernel<DB, kCsrUnit16, S>);
        case kCsrPacked32: return reinterpret_cast<const void*>(&rfmf_anneal_kernel<DB, kCsrPacked32, S>);
        case kCsrGlobal16: return reinterpret_cast<const void*>(&rfmf_anneal_kernel<DB, kCsrGlobal16, S>);
        case kCsrGlobal32: return reinterpret_cast<const void*>(&rfmf_anneal_kernel<DB, kCsrGlobal32, S>);
        default: return reinterpret_cast<const void*>(&rfmf_anneal_kernel<DB, kCsrGlobal, S>);
    }
}

const void* kernel_ptr(int dbytes, int fmt, bool s64) {
    if (dbytes == 1) return s64 ? kernel_for_format<1, true>(fmt) : kernel_for_format<1, false>(fmt);
    return s64 ? kernel_for_format<4, true>(fmt) : kernel_for_format<4, false>(fmt);
}

cudaError_t launch_anneal(const DevLaunch& L, int dbytes, int fmt, bool s64, int grid,
                          int threads, size_t smem, cudaStream_t stream) {
    void* args[] = {const_cast<DevLaunch*>(&L)};
    return cudaLaunchKernel(kernel_ptr(dbytes, fmt, s64), dim3(grid), dim3(threads), args, smem,
                            stream);
}

}  // namespace rfmf
