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
 * row-major.  impl 0: tcgen05 tensor-core kernel with thread-staged
 * operands (N a multiple of 16, <= 256; K a multiple of 64); impl 2: the
 * same MMA fed by TMA through a multi-stage shared-memory ring (same shape
 * rules; A and B 16-byte aligned; the surrogate's default); impl 1:
 * CUDA-core reference.  split_k > 1
 * splits K over that many CTAs per row tile (C is zeroed first).  Runs on the
 * current device's default stream and waits. */
int dpg_gemm_bf16(const void *A_dev, const void *B_dev, float *C_dev, int M, int N, int K, int impl,
                  int split_k);

/* Failure path of the bounded mbarrier waits of the tensor-core kernels: one
 * CTA allocates tensor memory, waits with at most `polls` polls on an
 * mbarrier that nothing will complete (no copy or MMA is issued), records
 * the timeout, frees the tensor memory and returns.  Returns DPG_ERR_TIMEOUT
 * when the wait gave up, as it must; the device stays usable. */
int dpg_mlp_wait_selftest(int device, uint32_t polls);

/* ---- the surrogate MLP --------------------------------------------------
 * Input row per (node, primitive) pair (96 bf16): normalised node state (16,
 * zero padded), 8x8 occupancy patch around the node (64), the primitive's
 * learned 16-D embedding.  Layers 96 -> 256 -> 256 -> 256 -> 2 with GELU
 * (tanh form: z/2 (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))));
 * outputs [collision logit, cost-to-go].  BF16 weights and activations, FP32
 * accumulation (tcgen05), FP32 master weights, Adam. */
typedef struct dpg_mlp dpg_mlp;

enum { DPG_MLP_W1 = 0, DPG_MLP_B1, DPG_MLP_W2, DPG_MLP_B2, DPG_MLP_W3, DPG_MLP_B3, DPG_MLP_W4, DPG_MLP_B4,
       DPG_MLP_EMB, DPG_MLP_NPARAM };

/* n_prims embedding rows; max_rows = largest batch of pairs per call */
int dpg_mlp_create(dpg_mlp **mlp, int device, int n_prims, int64_t max_rows, uint64_t seed);
void dpg_mlp_destroy(dpg_mlp *mlp);
/* element count of parameter `which` (W1 256x96, W2/W3 256x256, W4 16x256
 * with rows >= 2 held at zero, b1-b3 256, b4 16, EMB n_prims x 16) */
int64_t dpg_mlp_param_size(const dpg_mlp *mlp, int which);
/* host copies of a parameter or of its last gradient (FP32) */
int dpg_mlp_get(const dpg_mlp *mlp, int which, int grad, float *host);
int dpg_mlp_set(dpg_mlp *mlp, int which, const float *host);

/* per node: normalised state + occupancy patch (80 bf16 per node) from the
 * context's environment; x_dev N x nx doubles.  goal (host, nx doubles, may
 * be NULL): the goal the cost-to-go refers to, stored as the normalised
 * offset goal - position in state slots 13.. */
int dpg_mlp_node_features(dpg_ctx *ctx, const double *x_dev, int64_t N, const double *goal, void *feat_dev);

/* scores n pairs: out_dev[n x 2] = [logit, cost-to-go] (FP32) */
int dpg_mlp_forward(dpg_mlp *mlp, const void *node_feat_dev, const uint32_t *node_dev, const uint32_t *prim_dev,
                    int64_t n, float *out_dev);

/* one Adam step on a batch: target_dev[B x 2] = [collision (0/1), cost-to-go];
 * loss = mean(BCE(logit) + 0.5 ctg_weight (ctg - target)^2), returned in *loss */
int dpg_mlp_train_step(dpg_mlp *mlp, const void *node_feat_dev, const uint32_t *node_dev,
                       const uint32_t *prim_dev, const float *target_dev, int64_t B, float lr, float ctg_weight,
                       float *loss);

/* Forward kernels: fused 1 runs the whole MLP per 128-row tile in one
 * persistent tcgen05 kernel (activations kept in shared memory, weights
 * streamed by TMA); fused 2 (default) is the same kernel warp-specialised
 * (a TMA warp, an MMA warp, 16 epilogue warps) so that each layer's
 * epilogue overlaps the next layer's MMAs; fused 0 runs the layer-by-layer
 * GEMMs the training step uses.  Same arithmetic (bf16 operands, FP32
 * accumulation in the same order, same epilogue). */
int dpg_mlp_set_fused(dpg_mlp *mlp, int fused);

/* device time of the last forward / train step (ms) and the FLOPs it ran */
int dpg_mlp_last_timing(const dpg_mlp *mlp, double *ms, double *flops);

#ifdef __cplusplus
}
#endif
#endif
