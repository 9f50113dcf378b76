/*
 * dpg_bench.h -- measurement helpers exported by libdpg.so for bench.py.
 * No counterpart in the reference (it has no GPU path to measure).
 */
#ifndef DPG_BENCH_H
#define DPG_BENCH_H

#include <stddef.h>
#include <stdint.h>

#include "dpg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Achievable FP32 rate of this device: a register-resident chain of fused
 * multiply-adds on every SM, timed with CUDA events over `iters` launches.
 * Writes TFLOP/s (2 FLOP per FMA).  Returns 0 or a DPG_ERR_* code. */
int dpg_bench_fp32_peak(int device, int iters, double *tflops);

/* Writes `bytes` of scratch on the default stream and waits: evicts the L2
 * between timed iterations. */
int dpg_bench_flush_l2(int device, size_t bytes);

/* The plain GPU drop-in, timed: one dpg_expand per node, in node order,
 * with page-locked host buffers -- what the reference's search loop gets
 * when expand_lazy + check_lazy_trajectory (src/dbastar/dbastar.cpp:806-818)
 * call the GPU for each node it pops (the reference checks the ball
 * lazily; the drop-in checks it in one call).  x: n_nodes x nx host doubles.
 * Outputs per call: node, prim, verdict, first_invalid, end_state, flags
 * (host buffers; no min_gap).  Writes the checked pairs and the wall time in
 * seconds. */
int dpg_bench_per_node_expand(dpg_ctx *ctx, const dpg_expand_opts *opts, int64_t n_nodes, int32_t nx,
                              const double *x, int64_t *pairs, double *seconds);

#ifdef __cplusplus
}
#endif
#endif
