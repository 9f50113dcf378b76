/*
 * dpg_mlp.h -- the learned surrogate of the expansion: a BF16 MLP that scores
 * (node, primitive) pairs with a collision logit and a cost-to-go, trained
 * and run on the GB300 by the library's own tensor-core (tcgen05) kernels.
 * No counterpart in the reference: its expansion checks every candidate
 * exactly (check_lazy_trajectory, src/dbastar/dbastar.cpp:391-490) in the
 * shuffled order of Expander::expand_lazy (dbastar.hpp:302-303).  Here the
 * logit orders those lazy checks and the cost-to-go can serve as the A*
 * heuristic; every accepted edge is still verified by the exact checker.
 *
 * All pointers named *_dev are device pointers.  Functions return 0 or a
 * DPG_ERR_* code (dpg.h).
 */
#ifndef DPG_MLP_H
#define DPG_MLP_H

#include <stddef.h>
#include <stdint.h>

#include "dpg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* C[M x N] (FP32, row-major) = A[M x K] * B[N x K]^T with A, B bf16
 * row-major.  impl 0: tcgen05 tensor-core kernel (N a multiple of 16,
 * <= 256; K a multiple of 64); impl 1: CUDA-core reference.  split_k > 1
 * splits K over that many CTAs per row tile (C is zeroed first).  Runs on the
 * current device's default stream and waits. */
int dpg_gemm_bf16(const void *A_dev, const void *B_dev, float *C_dev, int M, int N, int K, int impl,
                  int split_k);

#ifdef __cplusplus
}
#endif
#endif
