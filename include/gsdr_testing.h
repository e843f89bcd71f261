/* gsdr_testing.h -- kernel-level entry points for tests and benchmarks.
 *
 * No counterpart in the reference, which only exposes the whole program.
 * gsdr_lcs_decide runs the library's alignment stage on a caller-given list
 * of (pattern, text) pairs: each decision is the reference's kernel_align
 * test (cuda-version/func.cu:828-999), LCS(pattern, text) >= ceil(len * t)
 * over gap-free bases, with len the pattern's raw length.
 */
#ifndef GSDR_TESTING_H
#define GSDR_TESTING_H
#include <stdint.h>

#include "gsdr.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Sequences: seq i is bytes[off[i] .. off[i] + len[i]).  Pair k decides
 * pattern pat[k] against text txt[k]; a pattern index may appear in at most
 * one pair.  mapping: 0 = the plain form's warp grouping, 1 = the batched
 * form's, 2 = the batched form's with the banded one-pair-per-lane kernel for
 * every pair whose band fits 32 words, 3 = the batched form's with the
 * group-banded kernel (one pair per 2..32 lanes) for every pair whose band
 * fits 128 words; greedy: 1 = try the greedy-embedding lower bound first.
 * accept[k] receives 0/1; *ms the device time of the alignment stage. */
int gsdr_lcs_decide(const char* bytes, int64_t n_bytes, const int64_t* off, const int32_t* len,
                    int32_t n_seq, const int32_t* pat, const int32_t* txt, int32_t n_pairs,
                    float t, int32_t mapping, int32_t greedy, uint8_t* accept, double* ms);

/* gsdr_job_run (include/gsdr.h) stopped after max_passes passes (batched) or
 * rounds (plain): the clustering is left unfinished.  For timing settings on
 * the early, full-size passes of a job (gsdr/autotune.py). */
int gsdr_job_run_limited(gsdr_job* job, int32_t max_passes, gsdr_stats* stats);

/* Polls each bounded wait of the alignment kernels (a warp of a multi-warp
 * group waiting for its neighbour's carry words) makes on `device` before it
 * gives up, sets the error flag and returns; polls < 0 restores the default
 * (4,194,304).  With 0 every such wait gives up at once, so a call whose pairs
 * need a multi-warp group returns GSDR_ETIMEOUT: the way tests check that a
 * wait that runs out ends in a status and not in a hang.  The reference has no
 * device-side waits (its errors are read once by checkError,
 * cuda-version/func.cu:1118-1123). */
int gsdr_set_spin_limit(int32_t device, int32_t polls);

#ifdef __cplusplus
}
#endif
#endif
