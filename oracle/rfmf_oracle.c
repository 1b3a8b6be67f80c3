/*
 * rfmf_oracle.c -- CPU restatement of the RFMF annealer (gt-tinker/rfmf).
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the GPU path is compared against and
 * the timed CPU baseline.  The product never links or calls it.  Written as plain serial C
 * from the reference's algorithm; each function cites the reference lines it
 * restates.  Parity is pinned (see rfmf_oracle.h).
 */
#include "rfmf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------- Philox */
/* Philox4x32-10 (Salmon et al. 2011); multipliers and Weyl constants are the
 * published ones, schedule as in src/philox.cuh:77-98. */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

static inline void philox10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += PHILOX_W0; k1 += PHILOX_W1; }
        const uint64_t p0 = (uint64_t)PHILOX_M0 * c[0];
        const uint64_t p1 = (uint64_t)PHILOX_M1 * c[2];
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        c[1] = (uint32_t)p1;
        c[3] = (uint32_t)p0;
        c[0] = n0;
        c[2] = n2;
    }
}

/* key = solverSeed, counter = (step_lo, step_hi, block_lo, block_hi):
 * src/philox.cuh:100-119. */
void rfmf_oracle_philox_block(uint64_t solver_seed, uint64_t step,
                              uint64_t block, uint32_t out[4]) {
    out[0] = (uint32_t)step;
    out[1] = (uint32_t)(step >> 32);
    out[2] = (uint32_t)block;
    out[3] = (uint32_t)(block >> 32);
    philox10(out, (uint32_t)solver_seed, (uint32_t)(solver_seed >> 32));
}

/* Field j: 16-bit half j&1 of word j>>1, low 11 bits.  src/philox.cuh:121-126 */
uint32_t rfmf_oracle_field(const uint32_t blk[4], uint32_t j) {
    const uint32_t w = blk[j >> 1];
    return ((j & 1u) ? (w >> 16) : (w & 0xFFFFu)) & 0x7FFu;
}

/* ------------------------------------------------------------ Gumbel LUT */
/* coarse[i] = round(-log(-log((2i+1)/32)) * 2^20), the 16-point equiprobable
 * Gumbel quantile table of src/philox.cuh:26-34, evaluated from its defining
 * formula (every entry sits >= 0.016 from a rounding boundary, so the double
 * evaluation is exact on any IEEE libm). */
static void gumbel_lut(int32_t lut[16]) {
    for (int i = 0; i < 16; ++i)
        lut[i] = (int32_t)lround(-log(-log((2.0 * i + 1.0) / 32.0)) * 1048576.0);
}

int32_t rfmf_oracle_gumbel(uint32_t r11) {
    int32_t lut[16];
    gumbel_lut(lut);
    return lut[r11 & 15u] + (int32_t)(r11 >> 4);   /* src/philox.cuh:52-58 */
}

/* ------------------------------------------------------- beta and gates */
int32_t rfmf_oracle_beta_fixed(uint64_t step, double t0) {
    /* src/host_common.h:73-76 */
    const double beta = log(1.0 + (double)step) / t0;
    return (int32_t)round(beta * (double)(1 << 20));
}

int rfmf_oracle_score_safe_int32(int64_t total_steps, double t0,
                                 int64_t delta_bound) {
    /* src/host_common.cpp:296-312: betaMax*B + max|gumbel| < INT32_MAX with an
     * overflow guard before the product. */
    const int64_t kGumbelMaxMag = 3617486 + 127;
    const int64_t int32max = 2147483647;
    const double beta_max = log(1.0 + (double)total_steps) / t0;
    const int64_t bmf = (int64_t)llround(beta_max * (double)(1 << 20));
    const int64_t limit = int32max - kGumbelMaxMag;
    if (bmf > 0 && delta_bound > 0 && delta_bound > limit / bmf) return 0;
    return (bmf * delta_bound + kGumbelMaxMag) < int32max;
}

int64_t rfmf_oracle_max_weighted_degree(int64_t n, const uint32_t* offsets,
                                        const int32_t* weight) {
    /* src/host_common.cpp:314-325 */
    int64_t B = 0;
    for (int64_t v = 0; v < n; ++v) {
        int64_t s = 0;
        for (uint32_t i = offsets[v]; i < offsets[v + 1]; ++i)
            s += llabs((long long)weight[i]);
        if (s > B) B = s;
    }
    return B;
}

int64_t rfmf_oracle_cut_value(int64_t n, const uint32_t* offsets,
                              const int32_t* col, const int32_t* weight,
                              const int8_t* spin) {
    /* src/max_cut.cpp:5-15: edges counted once from their smaller endpoint. */
    int64_t value = 0;
    for (int64_t v = 0; v < n; ++v)
        for (uint32_t i = offsets[v]; i < offsets[v + 1]; ++i)
            if ((int64_t)col[i] > v && spin[v] != spin[col[i]]) value += weight[i];
    return value;
}

/* ------------------------------------------------------- initial spins */
/* xoshiro256++ seeded by splitmix64 (Blackman & Vigna), drawing 1 bit per
 * vertex from a 64-bit reservoir: src/rng.hpp:11-58 with the draw loop of
 * src/host_common.cpp:40-45 (bit 1 -> +1, bit 0 -> -1). */
static inline uint64_t rotl64(uint64_t x, int k) {
    return (x << k) | (x >> (64 - k));
}

void rfmf_oracle_initial_spins(uint64_t seed, int64_t n, int8_t* out) {
    uint64_t s[4];
    uint64_t z = seed;
    for (int i = 0; i < 4; ++i) {
        z += 0x9e3779b97f4a7c15ULL;
        uint64_t x = z;
        x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
        x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
        s[i] = x ^ (x >> 31);
    }
    uint64_t buf = 0;
    int avail = 0;
    for (int64_t v = 0; v < n; ++v) {
        if (avail < 1) {
            const uint64_t result = rotl64(s[0] + s[3], 23) + s[0];
            const uint64_t t = s[1] << 17;
            s[2] ^= s[0];
            s[3] ^= s[1];
            s[1] ^= s[2];
            s[0] ^= s[3];
            s[2] ^= t;
            s[3] = rotl64(s[3], 45);
            buf = result;
            avail = 64;
        }
        out[v] = (buf & 1u) ? (int8_t)1 : (int8_t)-1;
        buf >>= 1;
        avail -= 1;
    }
}

/* -------------------------------------------------------------- anneal */
uint64_t rfmf_oracle_total_sweeps(int64_t nphases, const uint64_t* phases,
                                  const uint64_t* iters) {
    uint64_t t = 0;
    for (int64_t p = 0; p < nphases; ++p)
        if (phases[p] != 0) t += iters[p];
    return t;
}

int rfmf_oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* One chain over sweeps [sweep_begin, sweep_end). */
static void anneal_chain(int64_t n, const uint32_t* off, const int32_t* col,
                         const int32_t* wt, double t0, uint64_t seed,
                         int64_t nphases, const uint64_t* phases,
                         const uint64_t* iters, uint64_t sweep_begin,
                         uint64_t sweep_end, int8_t* spin, int8_t* best_spin,
                         int64_t* cur_io, int64_t* best_io, int64_t* trace,
                         const int32_t lut[16], uint64_t maxP,
                         int64_t* S, int64_t* slot_score, int64_t* slot_v) {
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    int64_t cur = *cur_io, best = *best_io;

    /* Local fields S[v] = sum_u w(v,u) spin[u], rows in CSR (ascending) order:
     * src/anneal_kernels.cu:250-256. */
    for (int64_t v = 0; v < n; ++v) {
        int64_t acc = 0;
        for (uint32_t i = off[v]; i < off[v + 1]; ++i)
            acc += (int64_t)wt[i] * spin[col[i]];
        S[v] = acc;
    }
    (void)maxP;

    const int64_t nblk = (n + 7) >> 3;
    uint64_t sweep = 0;     /* 0-based executed-sweep index */
    for (int64_t p = 0; p < nphases && sweep < sweep_end; ++p) {
        const uint64_t P = phases[p];
        if (P == 0) continue;                     /* src/anneal_kernels.cu:272 */
        const uint64_t ph_begin = sweep, ph_end = sweep + iters[p];
        if (ph_end <= sweep_begin) { sweep = ph_end; continue; }
        uint64_t s0 = ph_begin > sweep_begin ? ph_begin : sweep_begin;
        uint64_t s1 = ph_end < sweep_end ? ph_end : sweep_end;
        for (uint64_t sw = s0; sw < s1; ++sw) {
            const uint64_t step = sw + 1;          /* 1-based sweep id */
            const int64_t beta = rfmf_oracle_beta_fixed(step, t0);

            /* SELECT: every vertex scored from PRE-sweep state; per group the
             * max score wins, ties to the smallest v.
             * src/anneal_kernels.cu:282-346, src/philox.cuh:128-146. */
            for (uint64_t g = 0; g < P; ++g) { slot_score[g] = INT64_MIN; slot_v[g] = -1; }
            uint64_t grp = 0;                       /* v mod P, carried */
            for (int64_t b = 0; b < nblk; ++b) {
                uint32_t blk[4] = {(uint32_t)step, (uint32_t)(step >> 32),
                                   (uint32_t)b, (uint32_t)((uint64_t)b >> 32)};
                philox10(blk, k0, k1);
                for (uint32_t j = 0; j < 8; ++j) {
                    const int64_t v = (b << 3) + j;
                    if (v >= n) break;
                    const uint32_t r = rfmf_oracle_field(blk, j);
                    const int64_t gum = (int64_t)lut[r & 15u] + (int64_t)(r >> 4);
                    const int64_t delta = (int64_t)spin[v] * S[v];
                    const int64_t score = gum + beta * delta;
                    if (score > slot_score[grp]) { slot_score[grp] = score; slot_v[grp] = v; }
                    if (++grp == P) grp = 0;
                }
            }

            /* FLIP, serial in group order reading live S: the reference
             * kernel's corr[] formulation is this computed analytically
             * (src/anneal_kernels.cu:12-15, 133-155, 420-483). */
            for (uint64_t g = 0; g < P; ++g) {
                const int64_t v = slot_v[g];
                if (v < 0) continue;
                cur += (int64_t)spin[v] * S[v];
                spin[v] = (int8_t)-spin[v];
                const int64_t s2 = 2 * (int64_t)spin[v];
                for (uint32_t i = off[v]; i < off[v + 1]; ++i)
                    S[col[i]] += s2 * wt[i];
            }
            /* improved is decided once per sweep, after all flips; bestSpin is
             * the state at the end of the last improving sweep
             * (src/anneal_kernels.cu:432-440, 303-304, 488-490). */
            if (cur > best) {
                best = cur;
                memcpy(best_spin, spin, (size_t)n);
            }
            if (trace) trace[sw - sweep_begin] = cur;
        }
        sweep = ph_end;
    }
    *cur_io = cur;
    *best_io = best;
}

int rfmf_oracle_anneal_window(int64_t n, const uint32_t* offsets,
                              const int32_t* col, const int32_t* weight,
                              int64_t C, const double* t0s,
                              const uint64_t* solver_seeds,
                              int64_t nphases, const uint64_t* phases,
                              const uint64_t* iters,
                              uint64_t sweep_begin, uint64_t sweep_end,
                              int8_t* spins, int8_t* best_spins,
                              int64_t* cur_vals, int64_t* best_vals,
                              int64_t* trace_vals, int nthreads) {
    if (n < 0 || C < 0 || nphases < 0) return -1;
    if (n == 0 || C == 0 || sweep_end <= sweep_begin) return 0;
    uint64_t maxP = 1;
    for (int64_t p = 0; p < nphases; ++p) if (phases[p] > maxP) maxP = phases[p];
    int32_t lut[16];
    gumbel_lut(lut);
    const uint64_t span = sweep_end - sweep_begin;
    int failed = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    #pragma omp parallel num_threads(nthreads)
#else
    (void)nthreads;
#endif
    {
        int64_t* S = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
        int64_t* ss = (int64_t*)malloc(sizeof(int64_t) * (size_t)maxP);
        int64_t* sv = (int64_t*)malloc(sizeof(int64_t) * (size_t)maxP);
        const int ok = S && ss && sv;
        /* Every thread reaches the work-sharing loop, buffers or not. */
#ifdef _OPENMP
        #pragma omp for schedule(dynamic, 1)
#endif
        for (int64_t c = 0; c < C; ++c) {
            if (!ok) {
#ifdef _OPENMP
                #pragma omp atomic write
#endif
                failed = 1;
                continue;
            }
            anneal_chain(n, offsets, col, weight, t0s[c], solver_seeds[c],
                         nphases, phases, iters, sweep_begin, sweep_end,
                         spins + c * n, best_spins + c * n, cur_vals + c,
                         best_vals + c,
                         trace_vals ? trace_vals + (size_t)c * span : NULL,
                         lut, maxP, S, ss, sv);
        }
        free(S); free(ss); free(sv);
    }
    return failed ? -1 : 0;
}
