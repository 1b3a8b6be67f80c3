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

#ifdef __cplusplus
}
#endif

#endif /* RFMF_TESTING_H */
