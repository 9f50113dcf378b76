/*
 * dpg_tune.h -- autotuner of the expansion's launch choices (dpg_tuning in
 * dpg.h).  No counterpart in the reference: its expansion runs on one CPU
 * thread with nothing to tune.
 *
 * The choices that shape the device work of a batch -- which narrow phase
 * the exact check runs (lockstep per-lane walk or (lane, candidate) slots),
 * how many check blocks stay resident per SM, and from which batch size the
 * ball scan walks the key grid -- are timed on the caller's own batch and
 * the fastest is kept in the context.  Results never depend on the choice
 * (every candidate gives identical outputs), only the time does.
 *
 * The winner is cached per workload key: robot kind, primitive count, an
 * 8-bin histogram of the primitive lengths (bins of max_len / 8, counts
 * rounded to 1/16 of P), obstacle count and the batch size rounded to a
 * power of two.  The cache is a text file of one line per key; a key found
 * there is applied without timing.
 */
#ifndef DPG_TUNE_H
#define DPG_TUNE_H

#include <stdint.h>

#include "dpg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dpg_tune_report {
  dpg_tuning chosen;       /* applied to the context */
  dpg_tuning initial;      /* the context's choice before the call */
  double ms_chosen;        /* median device time of the chosen expand (ball scan + check) */
  double ms_initial;       /* the same for the initial choice */
  double seconds;          /* wall time of the search (0 from the cache) */
  int32_t candidates;      /* choices timed */
  int32_t from_cache;      /* 1: the key was in the cache */
  char key[160];           /* the workload key */
} dpg_tune_report;

/* Times every candidate choice on one expand of the N states x_dev (device
 * pointer, N x nx doubles; opts->radius / precision / bands as the caller
 * will expand; outputs go to the tuner's own device buffers), `reps`
 * timed calls each after one warm-up (median), and applies the fastest.
 * cache_path may be NULL (no cache); otherwise a found key is applied
 * directly and a new result is appended.  rep may be NULL. */
int dpg_autotune(dpg_ctx *ctx, const dpg_expand_opts *opts, int64_t N, const double *x_dev, int32_t reps,
                 const char *cache_path, dpg_tune_report *rep);

/* The workload key of the context's primitives and environment for a batch
 * of N nodes (what dpg_autotune caches under). */
int dpg_tune_key(const dpg_ctx *ctx, int64_t N, char *key, int32_t size);

#ifdef __cplusplus
}
#endif
#endif
