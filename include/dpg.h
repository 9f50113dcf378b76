/*
 * dpg.h -- C ABI of dynoplan_gb300: the db-A* / iDb-A* node expansion on one
 * GB300 (sm_103a).
 *
 * The boundary replaces, for a BATCH of frontier states, the reference pair
 *
 *   Expander::expand_lazy(Eigen::Ref<const VectorXd> x, std::vector<LazyTraj>&)
 *       include/dynoplan/dbastar/dbastar.hpp:270-312
 *   check_lazy_trajectory(LazyTraj&, Model_robot&, Time_benchmark&,
 *                         TrajWrapper&, Ref<VectorXd>, check_state*, int*, bool)
 *       include/dynoplan/dbastar/dbastar.hpp:334-339, src/dbastar/dbastar.cpp:391-490
 *
 * as called by the search loop at src/dbastar/dbastar.cpp:806-818: for every
 * node x_n and every primitive p with d(canonical(x_n), start_p) <= radius
 * (radius = alpha * delta, dbastar.cpp:585-586) it produces the transformed
 * end state, the bounds/collision verdict and the first invalid state.
 *
 * Conventions
 *   - Every function returns 0 on success or a negative DPG_ERR_* code; no
 *     C++ exception crosses this boundary.  dpg_errstr() names a code and
 *     dpg_last_error() gives the context's last message.
 *   - A context belongs to one host thread at a time (the reference Expander
 *     holds mutable scratch too, dbastar.hpp:233-313).  All device work of a
 *     context runs on its own blocking CUDA stream, so it is ordered after
 *     work already queued on the legacy default stream; device-resident
 *     inputs written on any other stream must be complete (synchronise that
 *     stream) before the call.  Every call has finished its device work
 *     when it returns.
 *   - Input arrays are copied; the caller keeps ownership.  Output arrays
 *     are owned by the caller (host or device memory, see dpg_expand_opts).
 *   - Precision: DPG_FP32 computes rollouts and separating-axis tests in
 *     FP32 and recomputes in FP64, on the GPU, every test whose gap or
 *     bounds margin lies within contact_band of zero, so verdicts and first
 *     invalid states are those of FP64 tests; end states are FP32.
 *     DPG_FP64 runs the same tests and writes the end states in FP64 (the
 *     FP64 canonical state plus the FP64 node offset).  DPG_FP64_STRICT
 *     computes every transform, bounds and collision test in FP64 (1/64 of
 *     the FP32 rate on this GPU).  In every mode the ball test runs in FP32
 *     and is decided in FP64 when the distance lies within ball_band of the
 *     radius, so the neighbour sets are those of an FP64 test.
 */
#ifndef DPG_H
#define DPG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DPG_ABI_VERSION 1

/* error codes */
#define DPG_OK 0
#define DPG_ERR_ARG -1      /* invalid argument */
#define DPG_ERR_OOM -2      /* device or host allocation failed */
#define DPG_ERR_CUDA -3     /* CUDA runtime error (see dpg_last_error) */
#define DPG_ERR_TIMEOUT -4  /* a bounded device wait gave up */
#define DPG_ERR_ABORTED -5  /* dpg_set_abort was raised */
#define DPG_ERR_CAPACITY -6 /* output capacity too small; n_pairs holds the need */
#define DPG_ERR_STATE -7    /* call order (e.g. expand before upload) */
#define DPG_ERR_NODEVICE -8 /* no CUDA device / kernel image not loadable */

/* robot kinds (the dynobench model names) */
#define DPG_ROBOT_UNICYCLE1 0 /* unicycle1_v0: (x,y,theta), (v,w) */
#define DPG_ROBOT_CAR1 1      /* car1_v0: (x,y,theta0,theta1), (v,phi) */
#define DPG_ROBOT_QUAD3D 2    /* quadrotor_v0: (p, q xyzw, v, w), 4 thrusts */
#define DPG_ROBOT_QUAD2D 3    /* quad2d_v0: (x,y,theta,vx,vy,w), 2 thrusts */

/* verdicts (per checked pair) */
#define DPG_VALID 0
#define DPG_COLLISION 1
#define DPG_OUT_OF_BOUNDS 2
#define DPG_UNCHECKED 255 /* dpg_lazy_check: candidate never checked */

/* precision */
#define DPG_FP32 0        /* FP32 tests, FP64 decisions in the bands, FP32 end states */
#define DPG_FP64 1        /* the same tests and decisions, end states in FP64 */
#define DPG_FP64_STRICT 2 /* every transform, bounds and collision test in FP64 */

/* dpg_expand_opts.mode */
#define DPG_MODE_BALL_ONLY 1
/* with DPG_MODE_BALL_ONLY: the reverse ball of tdb-A*'s reverse search --
 * motions keyed on their LAST state (position included) tested against the
 * node's canonical state, the tree nigh_factory_t builds for
 * reverse_search (include/dynoplan/nigh_custom_spaces.hpp:575-693, used at
 * src/tdbastar/tdbastar.cpp:575-576 and tdbastar.hpp:255); unicycle1 and
 * car1, the robots that factory covers.  Check the pairs with
 * dpg_tdb_check_pairs (reverse = 1). */
#define DPG_MODE_REVERSE 2

/* per-pair flags */
#define DPG_FLAG_CONTACT_RECHECK 1 /* verdict recomputed in FP64 (contact/bounds band) */
#define DPG_FLAG_ACCEPTED 2        /* dpg_lazy_check: among the node's first `limit` valid motions */

/* Robot description: the subset of dynobench::Model_robot the expansion uses
 * (nx, nu, ref_dt, distance_weights, collision geometry, dynamics
 * constants).  dpg_robot_default fills the values of each model. */
typedef struct dpg_robot_desc {
  int32_t kind;
  int32_t nx, nu;
  int32_t n_parts;    /* collision parts (car1: car + trailer) */
  double dt;          /* ref_dt */
  double w[4];        /* distance_weights, one per metric block */
  double box[2];      /* planar robots: box length (heading axis), width */
  double hitch;       /* car1: car centre to trailer centre */
  double wheelbase;   /* car1 */
  double radius;      /* quad3d: collision sphere radius */
  double mass;        /* quad3d */
  double arm;         /* quad3d: motor arm length */
  double t2t;         /* quad3d: thrust-to-torque ratio */
  double inertia[3];  /* quad3d: diagonal inertia */
  double ang_gain;    /* quad2d: m*l/I */
  double g;           /* gravity */
} dpg_robot_desc;

typedef struct dpg_expand_opts {
  double radius;          /* ball radius = alpha * delta (dbastar.cpp:585-586) */
  int32_t precision;      /* DPG_FP32, DPG_FP64 or DPG_FP64_STRICT */
  int32_t x_on_device;    /* x is a device pointer */
  int32_t out_on_device;  /* output arrays are device pointers */
  int32_t mode;           /* 0: full expand; DPG_MODE_BALL_ONLY: in-ball pairs only
                             (node, prim), no exact check */
  double contact_band;    /* FP64 re-check band for gaps and bounds (1e-4) */
  double ball_band;       /* FP64 re-check band around the radius (1e-5) */
} dpg_expand_opts;

/* Results, one row per in-ball (node, primitive) pair.  Rows are grouped by
 * primitive, primitives in order of decreasing length.  Within a primitive,
 * nodes come in processing order: ascending index for batches under 2048
 * nodes, else in Z-order of a coarse grid over the environment (64 x 64
 * cells, 16^3 in 3-D), ascending index within a cell -- deterministic, and
 * each node's motions still come in primitive order.  Any array pointer may
 * be NULL to skip that output. */
typedef struct dpg_expand_out {
  int64_t capacity;        /* in: rows available in the arrays below */
  int64_t n_pairs;         /* out: rows produced (or needed, on DPG_ERR_CAPACITY) */
  uint32_t *node;          /* node index */
  uint32_t *prim;          /* primitive index (upload order = Motion::idx) */
  uint8_t *verdict;        /* DPG_VALID / DPG_COLLISION / DPG_OUT_OF_BOUNDS */
  int16_t *first_invalid;  /* first out-of-bounds or colliding state, or L */
  void *end_state;         /* n_pairs x nx, float (DPG_FP32) or double (DPG_FP64, _STRICT) */
  float *min_gap;          /* min axis-aligned clearance along the checked states (costs check
                              time: per-state gap merges and a wider culling margin) */
  uint8_t *flags;          /* DPG_FLAG_* */
  /* counters (out) */
  int64_t n_scanned;       /* node x primitive ball tests */
  int64_t n_contact_recheck;
  int64_t n_ball_recheck;
} dpg_expand_out;

typedef struct dpg_ctx dpg_ctx;

/* version of this header the library was built with */
int dpg_abi_version(void);
const char *dpg_errstr(int code);

/* fills the model constants of `kind` (returns DPG_ERR_ARG for an unknown kind) */
int dpg_robot_default(int32_t kind, dpg_robot_desc *out);

/* Create a context on `device` for the robot.  Replaces robot_factory plus
 * the Expander constructor (dbastar.cpp:532-535, 585-586). */
int dpg_create(dpg_ctx **ctx, int device, const dpg_robot_desc *robot);
void dpg_destroy(dpg_ctx *ctx);
const char *dpg_last_error(const dpg_ctx *ctx);

/* Upload the primitive set: P motions, motion p has len[p] states (rows of
 * nx doubles, concatenated) and len[p]-1 actions (rows of nu doubles).  The
 * index p is Motion::idx.  Replaces load_motion_primitives_new's tables and
 * the T_m tree build (src/ompl/robots.cpp:3061-3174, dbastar.cpp:564-575);
 * the noise and quaternion normalisation of the loader are the caller's
 * (dpg_primitives_prepare in dpg_prim_io.h). */
int dpg_upload_primitives(dpg_ctx *ctx, int32_t P, const int32_t *len,
                          const double *states, const double *actions);

/* Insert P motions (same layout) in front of the uploaded set and re-index:
 * the new motions get indices 0..P-1, motion i of the old set becomes
 * P + i.  Replaces idbA*'s add-primitives step (src/idbastar/idbastar.cpp:
 * 234-291: motions.insert(motions.begin(), ...) then idx = position).  The
 * old tables stay on the device (copied there, not re-sent); every derived
 * table is rebuilt.  Equivalent to uploading the concatenation.  A surrogate
 * (dpg_mlp.h) indexes primitives by position, so one trained before the
 * insert no longer matches. */
int dpg_prepend_primitives(dpg_ctx *ctx, int32_t P, const int32_t *len,
                           const double *states, const double *actions);

/* Upload the environment: state position bounds (dim values each) and
 * n_obs axis-aligned boxes (n_obs x dim corners).  Replaces load_env and the
 * environment broadphase (dbastar.cpp:535). */
int dpg_upload_env(dpg_ctx *ctx, int32_t dim, const double *lo, const double *hi,
                   int32_t n_obs, const double *obs_lo, const double *obs_hi);

/* Expand N frontier states (N x nx doubles).  Returns DPG_ERR_CAPACITY with
 * out->n_pairs set when out->capacity is too small. */
int dpg_expand(dpg_ctx *ctx, const dpg_expand_opts *opts, int64_t N, const double *x,
               dpg_expand_out *out);

/* Exact check of an explicit list of n (node, primitive) pairs -- the lazy
 * check_lazy_trajectory of src/dbastar/dbastar.cpp:391-490 for a batch of
 * candidates chosen by the caller (e.g. ordered by the surrogate, or the
 * pairs a search still needs).  node[i] indexes the N states in x, prim[i]
 * the uploaded primitives.  Outputs are written at the input positions i;
 * opts->radius is ignored; opts->x_on_device applies to x, node and prim;
 * out->capacity must be >= n (out->node / out->prim are not written). */
int dpg_check_pairs(dpg_ctx *ctx, const dpg_expand_opts *opts, int64_t N, const double *x, int64_t n,
                    const uint32_t *node, const uint32_t *prim, dpg_expand_out *out);

/* Lazy exact check of candidate pairs, a batch of nodes at a time: the
 * check loop of the search, src/dbastar/dbastar.cpp:809-919, which walks a
 * node's neighbours (Expander::expand_lazy, dbastar.hpp:270-312) in order,
 * exact-checks each (check_lazy_trajectory, dbastar.cpp:391-490) and stops
 * once limit_branching_factor motions were taken (:916-918).
 *   - The n candidates (node_dev[i], prim_dev[i]) -- e.g. the pairs of a
 *     DPG_MODE_BALL_ONLY expand -- are ranked per node by ascending
 *     score_dev[i * score_stride] (NaN last), ties by ascending primitive
 *     index; score_dev NULL ranks by primitive index (motion order).  A
 *     surrogate's collision logit (dpg_mlp_forward, stride 2) puts the
 *     likely-valid motions first.
 *   - Candidates are exact-checked in rank order, in rounds, until every
 *     node has `limit` valid motions or no candidate left.  The first
 *     `limit` valid candidates of each node in rank order get
 *     DPG_FLAG_ACCEPTED; every accepted motion is exact-checked.
 *   - All pointers are DEVICE pointers (x_dev N x nx doubles).  out's arrays
 *     have a row per candidate (capacity >= n); verdict and flags are
 *     required, the others optional.  Unchecked candidates get verdict
 *     DPG_UNCHECKED; a checked one gets the verdict, first invalid state,
 *     end state and min_gap dpg_check_pairs gives it.  out->node and
 *     out->prim are not used.
 *   - A node may have at most 16384 candidates (DPG_ERR_CAPACITY beyond);
 *     an out-of-range index gives DPG_ERR_ARG.
 *   - stats (may be NULL) receives the counts of checked, valid and
 *     accepted candidates and the number of rounds.
 * No counterpart in the reference as a batch call; per node it takes the
 * same motions as the reference loop would for that neighbour order. */
typedef struct dpg_lazy_stats {
  int64_t n_checked;       /* candidates exact-checked */
  int64_t n_valid;         /* of those, DPG_VALID */
  int64_t n_accepted;      /* candidates with DPG_FLAG_ACCEPTED */
  int32_t rounds;          /* check rounds run */
  int32_t max_candidates;  /* the largest candidate count of a node */
} dpg_lazy_stats;

int dpg_lazy_check(dpg_ctx *ctx, const dpg_expand_opts *opts, int64_t N, const double *x_dev, int64_t n,
                   const uint32_t *node_dev, const uint32_t *prim_dev, const float *score_dev, int32_t score_stride,
                   int32_t limit, dpg_expand_out *out, dpg_lazy_stats *stats);

/* Allocation-free form of dpg_expand.  No counterpart in the reference (its
 * expansion runs on the host).  For callers that cannot allocate device
 * memory while they expand: real-time planning loops that must not block
 * on the device allocator (cudaMalloc can synchronise the device and take
 * milliseconds), and host programs that hand all device memory to their
 * own pool up front, so a cudaMalloc inside the library would fail or
 * break their accounting.  dpg_expand may call cudaMalloc to grow its
 * buffers; this call never allocates: its per-call scratch is one 64 MiB
 * file-scope device array that every GPU loading the library holds until
 * the process exits.
 *   - x_dev (N x nx doubles) and every array in `out` are DEVICE pointers;
 *     out->node and out->prim are required.  opts->x_on_device and
 *     opts->out_on_device are ignored (both are device).
 *   - The scratch must hold, with each term rounded up to 256 bytes,
 *     4*KEYD*N + 4*OFFD*N + 4*ceil32(ceil(N/32))*P + 4*ceil(N/256)*P + 28*P
 *     bytes (KEYD, OFFD: key and offset components of the robot: unicycle1
 *     1, 2; car1 2, 2; quad2d 2, 4; quadrotor 7, 6; ceil32 rounds up to a
 *     multiple of 32).  About 92,000 car1 nodes x 5,000 primitives fit;
 *     larger N x P is rejected with DPG_ERR_ARG and a message that gives
 *     the need.
 *   - All calls share the array, which keeps the last call's contents; the
 *     call clears what must start at zero itself.  Calls whose device work
 *     overlaps (other streams, other host threads, other contexts on the
 *     same GPU) race on it: serialise them.
 *   - The first call on a device looks the array's device address up
 *     (cudaGetSymbolAddress, with that device current).
 *   - It honours DPG_MODE_BALL_ONLY; it does not update dpg_last_timings.
 * Results are identical to dpg_expand's with device outputs. */
int dpg_expand_noalloc(dpg_ctx *ctx, const dpg_expand_opts *opts, int64_t N, const double *x_dev,
                       dpg_expand_out *out);

/* Launch choices of a context (defaults in brackets); dpg_autotune picks
 * them per workload (dpg_tune.h).  Results never depend on them. */
#define DPG_CHECK_LOCKSTEP 0 /* the 32 lanes of a warp walk their pairs' states and candidates */
#define DPG_CHECK_SLOTS 1    /* per chunk of states, (lane, candidate) slots spread over the warp */
typedef struct dpg_tuning {
  int32_t check_variant;       /* DPG_CHECK_* [DPG_CHECK_SLOTS]; FP64_STRICT always walks lockstep */
  int32_t check_blocks_per_sm; /* resident check blocks per SM, 0 = the occupancy maximum [0] */
  int32_t grid_min_nodes;      /* batches from this size scan the ball through the key grid [2048] */
  int32_t pipe_launches;       /* copy ranges of a host-output expand, 1..8 (check launches with
                                  DPG_HOST_OUT_PIPELINED) [8]; each range a fraction of the one
                                  before that the context adapts to its measured copy / check
                                  time, and consecutive ranges under 16 MiB copied together */
  int32_t host_output;         /* DPG_HOST_OUT_* for host output arrays of a batch >= 2048 nodes
                                  [DPG_HOST_OUT_PROGRESS] */
} dpg_tuning;
/* dpg_tuning.host_output: how results reach host output arrays */
#define DPG_HOST_OUT_PIPELINED 0 /* pipe_launches check launches over item ranges of decreasing
                                    size; each range copied (asynchronously when page-locked) once
                                    its launch is done */
#define DPG_HOST_OUT_DIRECT 1    /* page-locked arrays the GPU maps: the check kernel writes them
                                    itself (on the GB300 hosts measured, its stores over the host
                                    link doubled the check time) */
#define DPG_HOST_OUT_PROGRESS 2  /* one check launch; its warps count finished items per range
                                    and the count that completes a range raises a flag in mapped
                                    host memory, on which the host starts that range's copy */
int dpg_get_tuning(const dpg_ctx *ctx, dpg_tuning *t);
int dpg_set_tuning(dpg_ctx *ctx, const dpg_tuning *t);

/* Wait for the context's stream. */
int dpg_sync(dpg_ctx *ctx);
/* Raise (1) or clear (0) the abort flag polled by the device work queue. */
int dpg_set_abort(dpg_ctx *ctx, int32_t flag);

/* Page-locked host buffers (cudaHostAlloc) for inputs and outputs of
 * dpg_expand, so the host<->device copies run at full link speed.  No
 * counterpart in the reference (its expansion never leaves the host). */
void *dpg_host_alloc(size_t bytes);
void dpg_host_free(void *p);

/* Device time of the last dpg_expand, split by stage (milliseconds):
 * t[0] ball scan + compaction, t[1] exact check, t[2] FP64 re-check,
 * t[3] host<->device copies.  Returns the number of stages written. */
int dpg_last_timings(const dpg_ctx *ctx, double *t, int32_t n);

#ifdef __cplusplus
}
#endif
#endif
