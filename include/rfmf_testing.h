/*
 * rfmf_testing.h -- testing aids exported by librfmf.so.  Not part of the
 * annealer's interface (include/rfmf.h): they exist so that tests can drive
 * the library's failure paths without a GPU fault, and production code has
 * no reason to include this header.
 */
#ifndef RFMF_TESTING_H
#define RFMF_TESTING_H

#include "rfmf.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Overwrite chain `chain`'s carried cut value on the device (after the
 * batch's queued work).  The next launch finds it inconsistent with the
 * chain's spins and the batch reports RFMF_ERR_DEVICE; the context stays
 * usable.  No reference counterpart (the reference has no failure path
 * besides exit). */
int rfmf_batch_debug_set_cut(rfmf_batch* b, int64_t chain, int64_t cut);

/* Injected host allocation failure: the `countdown`-th host allocation
 * checkpoint reached from now on (Gset parsing, batch creation and restore,
 * request submission, admission and result read-out in a server's worker,
 * batch read-out) fails as if
 * the host were out of memory, and the calls above it report RFMF_ERR_NOMEM
 * (a served request fails; the server and the context stay usable).
 * countdown <= 0 disarms it.  Process-wide. */
int rfmf_debug_fail_host_alloc(int64_t countdown);

/* The batch planner's work-item sizing on given costs (no device work):
 * `ngraphs` graphs of one launch class with chains[q] chains each, CTAs of
 * at most `max_chains_per_cta` chains of `warps` warps, `slots` resident
 * CTAs, and level_ns[q * L + l - 1] the time per sweep of an item of graph q
 * at scheduler level l (warps on one SM scheduler, ceil(chains * warps / 4);
 * L = the level of a full CTA).  out_chains_per_item[q] receives graph q's
 * item size: the one-round plan with the smallest makespan, or, when even
 * the largest items need more than one round, sizes that shorten the
 * queue's longest-first list schedule. */
int rfmf_debug_plan_items(int ngraphs, const int64_t* chains, int max_chains_per_cta, int warps,
                          const double* level_ns, int64_t slots, int* out_chains_per_item);

#ifdef __cplusplus
}
#endif

#endif /* RFMF_TESTING_H */
