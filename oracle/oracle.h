/*
 * oracle.h -- FP64 CPU restatement of dynoplan's db-A* node expansion.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * implementation in dynoplan_gb300/: only the test-suite, the smoke check and
 * the CPU-baseline leg of bench.py load it.  The product path never links,
 * loads or calls anything here.
 *
 * What it restates (reference paths are relative to the dynoplan project):
 *   - Expander::expand_lazy            include/dynoplan/dbastar/dbastar.hpp:270-312
 *   - LazyTraj::compute                include/dynoplan/dbastar/dbastar.hpp:174-182
 *   - check_lazy_trajectory            src/dbastar/dbastar.cpp:391-490
 *   - check_goal                       src/dbastar/dbastar.cpp:492-512
 *   - NearestNeighborsNigh::nearestR   include/dynoplan/nigh_custom_spaces.hpp:236-247
 *     with the per-robot product spaces of nigh_factory2
 *                                      include/dynoplan/nigh_custom_spaces.hpp:391-573
 *   - the dynobench models the path calls (step / canonical_state / offset /
 *     transform_primitive / is_state_valid / collision_check).  dynobench is
 *     an empty submodule in the reference, so those are restated from the
 *     reference's call sites and pinned against the reference's own data
 *     (bundled primitives and db-A* output trajectories, see tests/golden).
 *
 * Conventions shared with the CUDA path (the contract both sides implement):
 *   verdict        0 = valid, 1 = collision, 2 = out of bounds
 *   precedence     bounds over collision (the reference runs the bounded
 *                  rollout before any collision query, dbastar.cpp:422-455)
 *   first_invalid  first out-of-bounds state for verdict 2, first colliding
 *                  state for verdict 1, L for verdict 0
 *   end_state      the last state computed: x[L-1], or x[first_invalid] when
 *                  the bounded rollout stopped early (verdict 2)
 *   contact        a robot part and an obstacle collide iff their
 *                  separating-axis gap is <= 0 (touching counts as contact)
 *   ball           primitive p is a neighbour of node n iff
 *                  d(canonical(x_n), start_p) <= radius
 */
#ifndef DYNOPLAN_ORACLE_H
#define DYNOPLAN_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_UNICYCLE1 = 0, ORC_CAR1 = 1, ORC_QUAD3D = 2, ORC_QUAD2D = 3 };

/* min_gap is the min axis-aligned clearance along the checked states when
 * that is <= ORC_GAP_CAP metres, +inf otherwise (NaN for out-of-bounds). */
#define ORC_GAP_CAP 0.05
enum { ORC_VALID = 0, ORC_COLLISION = 1, ORC_OUT_OF_BOUNDS = 2 };

/* Robot description; the field meaning is identical to dpg_robot_desc in
 * include/dpg.h (the two are declared separately so that the oracle has no
 * dependency on the product). */
typedef struct orc_robot {
  int32_t kind;
  int32_t nx, nu;
  int32_t n_parts;
  double dt;
  double w[4];        /* metric block weights */
  double box[2];      /* 2-D robots: collision box length (heading axis), width */
  double hitch;       /* car1: distance from car centre to trailer centre */
  double wheelbase;   /* car1 */
  double radius;      /* quad3d: collision sphere radius */
  double mass;        /* quad3d */
  double arm;         /* quad3d: motor arm length */
  double t2t;         /* quad3d: thrust-to-torque ratio */
  double inertia[3];  /* quad3d: diagonal inertia */
  double ang_gain;    /* quad2d: m*l/I */
  double g;           /* gravity */
} orc_robot;

typedef struct orc_env {
  int32_t dim;        /* 2 or 3 */
  double lo[3], hi[3];/* state position bounds */
  int32_t n_obs;
  const double *obs_lo; /* n_obs x dim */
  const double *obs_hi; /* n_obs x dim */
} orc_env;

typedef struct orc_prims {
  int32_t P;
  const int32_t *len;     /* states per primitive */
  const int64_t *soff;    /* first state row of primitive p */
  const int64_t *aoff;    /* first action row of primitive p */
  const double *states;   /* rows of nx, row-major */
  const double *actions;  /* rows of nu, row-major */
} orc_prims;

typedef struct orc_out {
  int64_t cap;            /* capacity in pairs */
  int64_t n_pairs;        /* written pairs (or required count if > cap) */
  uint32_t *node, *prim;
  uint8_t *verdict;
  int16_t *first_invalid;
  double *end_state;      /* n_pairs x nx */
  double *min_gap;        /* min separating-axis gap along the checked states */
  int64_t n_scanned;      /* node x primitive pairs tested for ball membership */
} orc_out;

/* robot models ------------------------------------------------------------ */
void orc_robot_default(int kind, orc_robot *r);
void orc_step(const orc_robot *r, const double *x, const double *u, double *xn);
void orc_canonical_state(const orc_robot *r, const double *x, double *c);
int  orc_offset_dim(const orc_robot *r);
void orc_offset(const orc_robot *r, const double *x, double *off);
double orc_distance(const orc_robot *r, const double *a, const double *b);
double orc_lower_bound_time(const orc_robot *r, const double *a, const double *b);
int  orc_is_state_valid(const orc_robot *r, const orc_env *e, const double *x);
/* separating-axis gap of the robot at state x against obstacle o (min over parts) */
double orc_state_gap(const orc_robot *r, const orc_env *e, const double *x, int o);
/* rollout of `steps` actions from x0 into xs ((steps+1) x nx) */
void orc_rollout(const orc_robot *r, const double *x0, const double *us, int steps, double *xs);

/* single pair: LazyTraj::compute + check_lazy_trajectory.  Writes the
 * transformed states into xs (L x nx scratch), returns the verdict. */
int orc_check_pair(const orc_robot *r, const orc_env *e, const orc_prims *pr,
                   const double *x_node, int p, double *xs,
                   int16_t *first_invalid, double *end_state, double *min_gap);

/* Batched expand, brute force, single thread: for every node (in order) and
 * every primitive (in order) test ball membership, then check in-ball pairs.
 * Pairs are written node-major, primitives ascending.  Returns 0, or -1 when
 * out->cap is too small (out->n_pairs then holds the required count). */
int orc_expand(const orc_robot *r, const orc_env *e, const orc_prims *pr,
               int64_t N, const double *x, double radius, orc_out *out);

/* Same results as orc_expand, organised like the reference's CPU search
 * (sorted-angle radius query, uniform-grid broadphase, per-pair early exit)
 * and parallelised over nodes with `threads` OpenMP threads.  This is the
 * timed CPU baseline.  Pair order is node-major, primitives ascending. */
int orc_expand_fast(const orc_robot *r, const orc_env *e, const orc_prims *pr,
                    int64_t N, const double *x, double radius, int threads,
                    orc_out *out);

/* check_goal (dbastar.cpp:492-512): index into xs of the first of the states
 * at floor((k+1)/(n+1) * L), k = 0..n-1, within `bound` of goal, or -1. */
int orc_check_goal(const orc_robot *r, const double *xs, int L, const double *goal,
                   double bound, int n_check);

int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
