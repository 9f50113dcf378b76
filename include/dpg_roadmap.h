/*
 * dpg_roadmap.h -- the roadmap heuristic of db-A* (heuristic option 1),
 * its O(S^2) edge checks batched on the GPU.
 *
 * Replaces generate_heuristic_map / build_heuristic_distance_new /
 * compute_heuristic_map_new / Heu_roadmap::h / heuristicCollisionsTree
 * (src/dbastar/heuristics.cpp:6-42, 109-209, 211-228;
 * include/dynoplan/dbastar/heuristics.hpp:143-182):
 *   - the caller supplies the samples (start first, goal last, velocities
 *     zero; heuristics.cpp:17-39 draws them uniformly and keeps the
 *     collision-free ones);
 *   - edge (i, j), i < j: distance(x_i, x_j) < connection_radius and the
 *     straight interpolation between them is valid at `resolution`
 *     (dynobench::check_edge_at_resolution, restated: both ends and the
 *     midpoints of a bisection until segments are at most `resolution`
 *     long; R^n parts linear, angles along the shorter arc, quaternions by
 *     slerp; valid = inside the bounds and separated from every obstacle),
 *     weight lower_bound_time(x_i, x_j);
 *   - Dijkstra from the goal (the last sample) over the undirected graph;
 *     unreachable samples keep DBL_MAX and are their own parent, as the
 *     boost predecessor/distance maps leave them;
 *   - h(x) = max(lower_bound_time_vel(x, goal),
 *                min over samples s with distance(s, x0) <= connect_radius
 *                    of dist[s] + lower_bound_time_pr(s, x0))
 *     with x0 = x with its velocities zero, 1e8 when no sample is in range.
 */
#ifndef DPG_ROADMAP_H
#define DPG_ROADMAP_H

#include <stdint.h>

#include "dpg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dpg_roadmap dpg_roadmap;

/* Build the roadmap for the context's robot and environment (upload the env
 * first).  samples: S x nx host doubles. */
int dpg_roadmap_build(dpg_ctx *ctx, int32_t S, const double *samples, double connection_radius, double resolution,
                      dpg_roadmap **out);
void dpg_roadmap_destroy(dpg_roadmap *rm);

/* Edges sorted by (i, j): *n_edges always; ij (2 per edge) and w when
 * non-NULL and cap >= *n_edges. */
int dpg_roadmap_edges(const dpg_roadmap *rm, int64_t *n_edges, int32_t *ij, double *w, int64_t cap);

/* Dijkstra distances to the goal and parents (S entries each, either may be NULL). */
int dpg_roadmap_distances(const dpg_roadmap *rm, double *dist, int32_t *parent);

/* h(x) for N host states (N x nx doubles) and the goal state, into h[N]. */
int dpg_roadmap_heuristic(const dpg_roadmap *rm, int64_t N, const double *x, const double *goal,
                          double connect_radius, double *h);

/* Validity of N host states (bounds and every obstacle): valid[N] = 1 / 0. */
int dpg_states_valid(dpg_ctx *ctx, int64_t N, const double *x, uint8_t *valid);

#ifdef __cplusplus
}
#endif

#endif /* DPG_ROADMAP_H */
