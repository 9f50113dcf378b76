/*
 * dpg_bench.h -- measurement helpers exported by libdpg.so for bench.py.
 * No counterpart in the reference (it has no GPU path to measure).
 */
#ifndef DPG_BENCH_H
#define DPG_BENCH_H

#include <stddef.h>

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

#ifdef __cplusplus
}
#endif
#endif
