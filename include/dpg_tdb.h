/*
 * dpg_tdb.h -- the checks of tdb-A* (time-aware db-A*, the multi-robot
 * variant) on explicit (node, motion) pairs.
 *
 * Replaces tdbastar's check_lazy_trajectory (src/tdbastar/tdbastar.cpp:
 * 314-447) with LazyTraj::compute (include/dynoplan/tdbastar/
 * tdbastar.hpp:172-214):
 *   - forward: the motion starts at the node (the db-A* transform);
 *     reverse: the motion ends at the node -- translation robots as the
 *     reference's "assumes 2d" branch (:192-197): shifted so that its LAST
 *     state's position is the node's (offset = node - last state); quad2d
 *     and quadrotor as db-A*'s reverse branch (transform_primitiveDirectReverse,
 *     include/dynoplan/dbastar/dbastar.hpp:183-201; dynobench, absent,
 *     restated): the last state takes the node's position and velocity,
 *     every velocity moves by dv = v_node - v_last and every position by
 *     p_node - p_last + (t_k - t_last) dv (the same actions rolled out from
 *     the shifted start);
 *   - verdict as dpg_expand: any state out of bounds -> DPG_OUT_OF_BOUNDS,
 *     else the first colliding state -> DPG_COLLISION, else valid;
 *   - a valid motion is then tested against the constraints: for each
 *     (time, state), time_index = lround((time - node_g) / dt); the state
 *     checked is the motion's state at time_index when 0 <= time_index <
 *     L - 1, or its last state when the motion reaches the goal
 *     (distance(state 0 (forward) / state L-1 (reverse), goal) <= delta)
 *     and time_index >= L - 1; distance(checked, constraint state) <= delta
 *     -> DPG_CONSTRAINT_VIOLATION (the first violated constraint's index
 *     goes to first_invalid).
 * FP64 throughout; one thread per pair.  Node g scores are floats, as
 * AStarNode::gScore.
 */
#ifndef DPG_TDB_H
#define DPG_TDB_H

#include <stdint.h>

#include "dpg.h"

#ifdef __cplusplus
extern "C" {
#endif

#define DPG_CONSTRAINT_VIOLATION 3

typedef struct dpg_tdb_args {
  int32_t reverse;           /* 0 forward, 1 reverse */
  const float *node_g;       /* [N] g score of each node */
  int32_t n_constraints;
  const float *c_time;       /* [n_constraints] */
  const double *c_state;     /* [n_constraints x nx] */
  const double *goal;        /* nx */
  double delta;
} dpg_tdb_args;

/* Check n explicit pairs (node[i], prim[i]) of the N host states x (N x nx).
 * Outputs (host arrays, n entries; end_state n x nx, may be NULL):
 * verdict, first_invalid (state index, or the constraint index for
 * DPG_CONSTRAINT_VIOLATION, or L), end_state (last state of the shifted
 * motion, or the first out-of-bounds one). */
int dpg_tdb_check_pairs(dpg_ctx *ctx, const dpg_tdb_args *args, int64_t N, const double *x, int64_t n,
                        const uint32_t *node, const uint32_t *prim, uint8_t *verdict, int32_t *first_invalid,
                        double *end_state);

#ifdef __cplusplus
}
#endif

#endif /* DPG_TDB_H */
