/*
 * dpg_search.h -- db-A* search driven by the batched GPU expansion.
 *
 * Restates the search loop of dbastar() (src/dbastar/dbastar.cpp:523-1058):
 * pop the best open node, goal test, expand (expand_lazy +
 * check_lazy_trajectory), intermediate-goal check (check_goal,
 * dbastar.cpp:492-512), g = g_parent + motion cost + cost_delta_factor *
 * lower_bound_time(x, motion start), novelty radius query on the explored
 * nodes with radius (1 - alpha) * delta, insert or rewire, at most
 * limit_branching_factor novel successors per expanded node
 * (dbastar.cpp:766-920).  Open-list order: lowest f, then highest g, on
 * float scores (compareAStarNode, dbastar.cpp:56-68).
 *
 * GPU form: `batch` open nodes are popped per iteration and expanded in one
 * dpg_expand call.  The reference visits a node's motions in order and stops
 * at the limit, so successors are prepared in rounds: each unfinished node,
 * in pop order, visits its next chunk of valid motions (2 x the limit,
 * doubling per round) until it has `limit` new nodes.  The novelty queries
 * of a round run on the GPU through a uniform grid over position (cell side
 * radius / position weight, nodes counting-sorted by cell, a block of
 * threads per query over the neighbouring cells; FP32 with an FP64 re-test
 * near the radius);
 * neighbour lists are complete: counted (the novelty test), then packed with
 * the time lower bound to each neighbour.  A successor's g counts from its
 * node's g when the batch was popped (with batch = 1 that is the node's g:
 * no successor can lower it), so the GPU also drops the explored neighbours
 * it could never rewire (g + lower bound >= their g when they entered the
 * table; g only decreases), and lists a round's earlier successors only where
 * they can still be accepted (no explored neighbour, or a goal hit).
 * Successor states, goal checks and lower bounds
 * are computed on the GPU with the host arithmetic (no contraction);
 * insertion and rewiring run on the host in order.
 * batch = 1 visits nodes and motions in the reference's order.
 */
#ifndef DPG_SEARCH_H
#define DPG_SEARCH_H

#include <stdint.h>

#include "dpg.h"
#include "dpg_mlp.h"
#include "dpg_roadmap.h"

#ifdef __cplusplus
extern "C" {
#endif

/* heuristics (Options_dbastar::heuristic, dbastar.cpp:600-634) */
#define DPG_HEU_BLIND -1     /* Heu_blind: 0 */
#define DPG_HEU_EUCLIDEAN 0  /* Heu_euclidean: lower_bound_time(x, goal) */
#define DPG_HEU_MLP 1        /* the surrogate's cost-to-go of the (parent, motion) pair */
#define DPG_HEU_ROADMAP 2    /* Heu_roadmap (reference option 1): include/dpg_roadmap.h */

/* termination (Terminate_status, dbastar.hpp:109-117) */
#define DPG_SEARCH_SOLVED 0
#define DPG_SEARCH_MAX_EXPANDS 1
#define DPG_SEARCH_EMPTY_QUEUE 2
#define DPG_SEARCH_MAX_TIME 3

typedef struct dpg_search_opts {
  double delta;                   /* discontinuity bound */
  double alpha;                   /* share of delta for the expansion ball (0.5) */
  double delta_factor_goal;       /* goal tolerance = delta_factor_goal * delta (1) */
  double cost_delta_factor;       /* weight of the jump's time lower bound (1) */
  int32_t limit_branching_factor; /* novel successors per expanded node (20) */
  int32_t batch;                  /* open nodes expanded per GPU call */
  int64_t max_expands;
  double time_limit_ms;
  int32_t heuristic;              /* DPG_HEU_* */
  int32_t precision;              /* DPG_FP32 / DPG_FP64 for the exact checks */
  int32_t shuffle;                /* 1: shuffle each node's candidates (std::mt19937 seeded
                                     with `seed`, then std::shuffle, as expand_lazy);
                                     0: ascending motion index */
  int32_t max_neighbors;          /* unused (kept for layout): neighbour lists are complete,
                                     counted then packed on the GPU */
  uint64_t seed;
  const struct dpg_roadmap *roadmap; /* DPG_HEU_ROADMAP: a roadmap built for this goal */
  double connect_radius_h;           /* its query radius (Options_dbastar::connect_radius_h, 0.5) */
} dpg_search_opts;

typedef struct dpg_search_result {
  int32_t solved;
  int32_t status;                 /* DPG_SEARCH_* */
  double cost;                    /* duration of the solution (actions x dt) */
  float g;                        /* g score of the solution node */
  int32_t path_len;               /* motions in the solution */
  int64_t expands;                /* nodes popped and expanded */
  int64_t nodes;                  /* explored nodes created */
  int64_t checked_pairs;          /* (node, motion) pairs exact-checked */
  double time_ms, expand_ms, novelty_ms, mlp_ms;
  double prepare_ms;              /* successor states, goal checks (host) */
  double insert_ms;               /* insert / rewire and the open list (host) */
  int64_t rounds;                 /* successor rounds (one novelty query each) */
  double table_ms;                /* novelty: explored-node table upload and cell sort */
  double query_ms;                /* novelty: the two query passes and their copies */
} dpg_search_result;

/* Plan from start to goal (nx doubles each) on the context's robot,
 * primitives and environment.  path_motion (max_path ints) and path_state
 * ((max_path + 1) x nx doubles) receive the solution's motions and the node
 * states they start from, when non-NULL.  mlp: the surrogate for
 * DPG_HEU_MLP (else NULL). */
int dpg_search(dpg_ctx *ctx, const dpg_search_opts *opts, const double *start, const double *goal,
               dpg_mlp *mlp, dpg_search_result *res, int32_t *path_motion, double *path_state,
               int32_t max_path);

#ifdef __cplusplus
}
#endif
#endif
