// check_list.h -- library-internal helpers shared by the translation units
// that run the exact check on lists of (node, primitive) pairs (dpg.cu,
// lazy.cu).  Not part of the ABI.
#pragma once

#include <string>

#include "check_kernels.cuh"
#include "ctx.h"

namespace dpg {

int ctx_fail(dpg_ctx *c, int code, const std::string &msg);
int ctx_ensure(dpg_ctx *c, DevBuf &b, size_t bytes);
PrimView ctx_prim_view(dpg_ctx *c);
EnvView ctx_env_view(const dpg_ctx *c);

// CheckArgs over the context's tables for these nodes (keys and offsets
// prepared) and outputs; prec is DPG_FP32, DPG_FP64 or DPG_FP64_STRICT.
CheckArgs ctx_check_args(dpg_ctx *c, int prec, double contact_band, const NodeView &nv, const PairView &out);

// Processing order of N nodes (x_dev: N x nx, caller's order) on st:
// *perm[pos] = the caller's index of the node at position pos -- Z-order
// cells over the environment, ascending index within a cell, as dpg_expand
// processes a batch.  Batches under kReorderMin nodes keep the caller's
// order (*perm = nullptr).  Uses the context's ordering buffers.
int ctx_spatial_order(dpg_ctx *c, const double *x_dev, int64_t N, cudaStream_t st, const uint32_t **perm);

// node keys / offsets of nv (prep_nodes) on st
void ctx_prep_nodes(dpg_ctx *c, const NodeView &nv, cudaStream_t st);

// Exact check of n pairs given as device arrays node_d / prim_d (indices
// into the N nodes of ca.nv and the uploaded primitives) on st: the pairs
// are grouped by primitive (longest first) and walked by the persistent
// lockstep warps; the result of pair i goes to row dest_d[i] (or i when
// dest_d is null) of the arrays in ca.out.  Pairs with an index out of
// range are skipped and counted in the context's counters (n_bad).  Clears
// the counters first; does not wait.  Records ev[2] / ev[3] around the
// check kernel when `timed`.
int ctx_check_list(dpg_ctx *c, int prec, CheckArgs ca, int64_t n, const uint32_t *node_d, const uint32_t *prim_d,
                   const uint32_t *dest_d, cudaStream_t st, bool timed);

// Exact check of a list already grouped by primitive: the segments of the
// primitives in length order (pv.order) start at c->ord_pbase and their
// work items at c->ord_ibase (scan_totals has written them and the
// counters' n_items); list_node[i] is the node, list_dest[i] the output row
// of list entry i.  Does not wait.
int ctx_check_grouped(dpg_ctx *c, int prec, CheckArgs ca, const uint32_t *list_node, const uint32_t *list_dest,
                      cudaStream_t st);

}  // namespace dpg
