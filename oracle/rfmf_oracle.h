/*
 * rfmf_oracle.h -- CPU restatement of the RFMF annealer.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (rfmf_gb300/, include/)
 * links, loads or calls this library.  It is the oracle that the GPU path is
 * compared against, and the CPU baseline that bench.py times beside it.
 *
 * Every function restates one piece of the reference (gt-tinker/rfmf); the
 * reference file:line it follows is given beside each declaration.
 *
 * Parity status: pinned.  The primitives (Philox, Gumbel LUT, beta schedule,
 * score gate, xoshiro initial spins, cut value) are checked against the
 * reference's own host code built from its sources (oracle/build_ref.sh), and
 * the full sweep against the reference's committed V100 result logs
 * (oracle/pin_committed_logs.py).
 */
#ifndef RFMF_ORACLE_H
#define RFMF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Philox4x32-10 block for (key = solverSeed, counter = (step, block, 0)).
 * src/philox.cuh:60-119 */
void rfmf_oracle_philox_block(uint64_t solver_seed, uint64_t step,
                              uint64_t block, uint32_t out[4]);

/* Q20 Gumbel from an 11-bit field: LUT[r & 15] + (r >> 4).
 * src/philox.cuh:26-58 */
int32_t rfmf_oracle_gumbel(uint32_t r11);

/* 11-bit field j (0..7) of a Philox block.  src/philox.cuh:121-126 */
uint32_t rfmf_oracle_field(const uint32_t blk[4], uint32_t j);

/* round(log(1+step)/t0 * 2^20), host double.  src/host_common.h:73-76 */
int32_t rfmf_oracle_beta_fixed(uint64_t step, double t0);

/* int32 score-path gate.  src/host_common.cpp:296-312 */
int rfmf_oracle_score_safe_int32(int64_t total_steps, double t0,
                                 int64_t delta_bound);

/* B = max_v sum |w|.  src/host_common.cpp:314-325 */
int64_t rfmf_oracle_max_weighted_degree(int64_t n, const uint32_t* offsets,
                                        const int32_t* weight);

/* Cut value of a +-1 spin vector, each undirected edge once.
 * src/max_cut.cpp:5-15 */
int64_t rfmf_oracle_cut_value(int64_t n, const uint32_t* offsets,
                              const int32_t* col, const int32_t* weight,
                              const int8_t* spin);

/* Initial spins from xoshiro256++ seeded by splitmix64, one bit per vertex.
 * src/rng.hpp:11-58, src/host_common.cpp:40-45 */
void rfmf_oracle_initial_spins(uint64_t seed, int64_t n, int8_t* out);

/*
 * Anneal C independent chains over one CSR graph.
 *
 * Semantics of src/anneal_kernels.cu:262-491 (one sweep = SELECT over all n
 * vertices from pre-sweep state, then the serial "flip winners in group order
 * reading live S" of src/anneal_kernels.cu:12-15), with beta taken from
 * betaFixedForStep per sweep (the run tables of src/host_common.cpp:238-294
 * are an exact encoding of it).
 *
 * Executed sweeps are numbered 0..T-1 over phases with P != 0 (phases with
 * P == 0 are skipped without advancing the step, src/anneal_kernels.cu:272).
 * Only sweeps in [sweep_begin, sweep_end) run; the chain state is carried in
 * and out through spins/best_spins/cur_vals/best_vals, so a run split into
 * windows equals one uninterrupted run.
 *
 * spins, best_spins: C*n int8 (+-1), in/out.  cur_vals, best_vals: C, in/out.
 * trace_vals (optional, C * (sweep_end-sweep_begin)): currentVal after each
 * sweep.  nthreads <= 0 uses all cores.  Returns 0, or -1 on bad arguments.
 */
int rfmf_oracle_anneal_window(int64_t n, const uint32_t* offsets,
                              const int32_t* col, const int32_t* weight,
                              int64_t C, const double* t0s,
                              const uint64_t* solver_seeds,
                              int64_t nphases, const uint64_t* phases,
                              const uint64_t* iters,
                              uint64_t sweep_begin, uint64_t sweep_end,
                              int8_t* spins, int8_t* best_spins,
                              int64_t* cur_vals, int64_t* best_vals,
                              int64_t* trace_vals, int nthreads);

/* Number of executed sweeps of a schedule (sum of iters over P != 0). */
uint64_t rfmf_oracle_total_sweeps(int64_t nphases, const uint64_t* phases,
                                  const uint64_t* iters);

/* Threads the OpenMP runtime would use (for reporting the CPU baseline). */
int rfmf_oracle_max_threads(void);

#ifdef __cplusplus
}
#endif

#endif /* RFMF_ORACLE_H */
