/*
 * oracle.c -- FP64 CPU restatement of dynoplan's db-A* node expansion.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Nothing in the product links this.
 *
 * Parity pins (tests/golden, generated by tests/golden/make_golden.py):
 *   unicycle1 step      bundled primitives data/motion_primitives/unicycle1_v0/
 *                       *.msgpack reproduce to 1e-12
 *   quad2d / quad3d     reference db-A* output trajectories in
 *   step                benchmark_initguess/{quad2d,quadrotor_v0}/ (states +
 *                       actions, 6 printed digits) reproduce to print precision
 *   metric              "jump ... delta D min time T" annotations of
 *                       benchmark_initguess/unicycle{1,2}_v0/ reproduce to 6
 *                       digits (block-weighted sum, SO2 wrapped)
 *   angle wrap          the 8 wrapping steps of the bundled unicycle1
 *                       primitives reproduce bit-exactly
 * Unpinned (dynobench is absent): car1 kinematics, collision geometry sizes,
 * state bounds, contact semantics.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define TWO_PI 6.283185307179586476925286766559
#define PI_D 3.1415926535897932384626433832795

/* ---------------------------------------------------------------- robots -- */

void orc_robot_default(int kind, orc_robot *r) {
  memset(r, 0, sizeof(*r));
  r->kind = kind;
  r->g = 9.81;
  switch (kind) {
  case ORC_UNICYCLE1: /* unicycle1_v0: (x, y, theta), (v, w) */
    r->nx = 3; r->nu = 2; r->n_parts = 1; r->dt = 0.1;
    r->w[0] = 1.0; r->w[1] = 0.5;            /* pinned by the jump annotations */
    r->box[0] = 0.5; r->box[1] = 0.25;
    break;
  case ORC_CAR1: /* car1_v0: (x, y, theta0, theta1), (v, phi) */
    r->nx = 4; r->nu = 2; r->n_parts = 2; r->dt = 0.1;
    r->w[0] = 1.0; r->w[1] = 0.5; r->w[2] = 0.5;
    r->box[0] = 0.5; r->box[1] = 0.25;
    r->hitch = 0.5; r->wheelbase = 0.25;
    break;
  case ORC_QUAD3D: /* quadrotor_v0: (p, q xyzw, v, w), 4 thrusts in hover units */
    r->nx = 13; r->nu = 4; r->n_parts = 1; r->dt = 0.01;
    /* SpaceQuad3d block ratios, nigh_custom_spaces.hpp:104-108 */
    r->w[0] = 1.0; r->w[1] = 0.5; r->w[2] = 0.1; r->w[3] = 0.05;
    r->radius = 0.1; r->mass = 0.034; r->arm = 0.046; r->t2t = 0.006;
    r->inertia[0] = 16.571710e-6; r->inertia[1] = 16.655602e-6;
    r->inertia[2] = 29.261652e-6;
    break;
  case ORC_QUAD2D: /* quad2d_v0: (x, y, theta, vx, vy, w), 2 thrusts in hover units */
    r->nx = 6; r->nu = 2; r->n_parts = 1; r->dt = 0.01;
    /* SpaceQuad2d block ratios, nigh_custom_spaces.hpp:70-74 */
    r->w[0] = 1.0; r->w[1] = 0.5; r->w[2] = 0.2; r->w[3] = 0.1;
    r->box[0] = 0.5; r->box[1] = 0.25;
    r->ang_gain = 34.0;
    break;
  default:
    break;
  }
}

static double so2_dist(double a, double b) {
  double d = fabs(a - b);
  d = fmod(d, TWO_PI);
  return d > PI_D ? TWO_PI - d : d;
}

static double norm3(double a, double b, double c) { return sqrt(a * a + b * b + c * c); }

/* Angle normalisation of the planar models' step: x - 2 pi floor((x + pi) /
 * 2 pi), i.e. [-pi, pi).  Pinned bit-exactly by the 8 wrapping steps of the
 * reference's bundled unicycle1 primitives. */
static double wrap_angle(double x) { return x - TWO_PI * floor((x + PI_D) / TWO_PI); }

static void quat_mul(const double *a, const double *b, double *o) {
  /* Hamilton product, (x, y, z, w) storage */
  double ax = a[0], ay = a[1], az = a[2], aw = a[3];
  double bx = b[0], by = b[1], bz = b[2], bw = b[3];
  o[0] = aw * bx + ax * bw + ay * bz - az * by;
  o[1] = aw * by - ax * bz + ay * bw + az * bx;
  o[2] = aw * bz + ax * by - ay * bx + az * bw;
  o[3] = aw * bw - ax * bx - ay * by - az * bz;
}

/* Explicit Euler step of each model from the current state.  The quad2d and
 * quad3d forms were pinned against reference output trajectories (explicit in
 * every component, body-frame quaternion exponential), the unicycle1 form
 * against the reference's bundled primitives. */
void orc_step(const orc_robot *r, const double *x, const double *u, double *xn) {
  const double dt = r->dt;
  switch (r->kind) {
  case ORC_UNICYCLE1: {
    const double c = cos(x[2]), s = sin(x[2]);
    xn[0] = x[0] + u[0] * c * dt;
    xn[1] = x[1] + u[0] * s * dt;
    xn[2] = wrap_angle(x[2] + u[1] * dt);
  } break;
  case ORC_CAR1: {
    const double v = u[0], phi = u[1];
    xn[0] = x[0] + v * cos(x[2]) * dt;
    xn[1] = x[1] + v * sin(x[2]) * dt;
    xn[2] = wrap_angle(x[2] + v / r->wheelbase * tan(phi) * dt);
    xn[3] = wrap_angle(x[3] + v / r->hitch * sin(x[2] - x[3]) * dt);
  } break;
  case ORC_QUAD2D: {
    const double th = x[2];
    const double acc = (u[0] + u[1]) * r->g * 0.5; /* thrust / mass */
    xn[0] = x[0] + x[3] * dt;
    xn[1] = x[1] + x[4] * dt;
    xn[2] = wrap_angle(x[2] + x[5] * dt);
    xn[3] = x[3] - acc * sin(th) * dt;
    xn[4] = x[4] + (acc * cos(th) - r->g) * dt;
    xn[5] = x[5] + r->ang_gain * r->g * 0.5 * (u[0] - u[1]) * dt;
  } break;
  case ORC_QUAD3D: {
    const double *p = x, *q = x + 3, *v = x + 7, *w = x + 10;
    const double fu = r->mass * r->g * 0.25;
    const double f0 = u[0] * fu, f1 = u[1] * fu, f2 = u[2] * fu, f3 = u[3] * fu;
    const double F = f0 + f1 + f2 + f3;
    const double lever = r->arm / sqrt(2.0);
    const double tx = lever * (-f0 - f1 + f2 + f3);
    const double ty = lever * (-f0 + f1 + f2 - f3);
    const double tz = r->t2t * (-f0 + f1 - f2 + f3);
    const double qx = q[0], qy = q[1], qz = q[2], qw = q[3];
    /* third column of R(q) times thrust/mass, minus gravity */
    const double am = F / r->mass;
    const double ax = 2.0 * (qx * qz + qy * qw) * am;
    const double ay = 2.0 * (qy * qz - qx * qw) * am;
    const double az = (1.0 - 2.0 * (qx * qx + qy * qy)) * am - r->g;
    const double Jx = r->inertia[0], Jy = r->inertia[1], Jz = r->inertia[2];
    const double hx = Jx * w[0], hy = Jy * w[1], hz = Jz * w[2];
    const double cx = w[1] * hz - w[2] * hy;
    const double cy = w[2] * hx - w[0] * hz;
    const double cz = w[0] * hy - w[1] * hx;
    const double wdx = (tx - cx) / Jx, wdy = (ty - cy) / Jy, wdz = (tz - cz) / Jz;
    /* q <- q (x) exp(w dt / 2), then renormalised */
    double e[4], qn[4];
    const double hvx = 0.5 * dt * w[0], hvy = 0.5 * dt * w[1], hvz = 0.5 * dt * w[2];
    const double th = norm3(hvx, hvy, hvz);
    const double sc = th > 1e-12 ? sin(th) / th : 1.0;
    e[0] = hvx * sc; e[1] = hvy * sc; e[2] = hvz * sc; e[3] = cos(th);
    quat_mul(q, e, qn);
    const double nq = sqrt(qn[0] * qn[0] + qn[1] * qn[1] + qn[2] * qn[2] + qn[3] * qn[3]);
    xn[0] = p[0] + v[0] * dt; xn[1] = p[1] + v[1] * dt; xn[2] = p[2] + v[2] * dt;
    xn[3] = qn[0] / nq; xn[4] = qn[1] / nq; xn[5] = qn[2] / nq; xn[6] = qn[3] / nq;
    xn[7] = v[0] + ax * dt; xn[8] = v[1] + ay * dt; xn[9] = v[2] + az * dt;
    xn[10] = w[0] + wdx * dt; xn[11] = w[1] + wdy * dt; xn[12] = w[2] + wdz * dt;
  } break;
  default:
    break;
  }
}

/* Components zeroed by canonical_state and returned by offset
 * (Expander::expand_lazy, dbastar.hpp:273-274).  unicycle1 and car1 are
 * translation invariant (the reuse-collision-shape path asserts an offset of
 * dimension 2, dbastar.cpp:462-469); quad2d and quad3d use the velocity
 * invariance, offset = (position, velocity). */
static int offset_components(int kind, int *idx) {
  switch (kind) {
  case ORC_UNICYCLE1:
  case ORC_CAR1:
    idx[0] = 0; idx[1] = 1;
    return 2;
  case ORC_QUAD2D:
    idx[0] = 0; idx[1] = 1; idx[2] = 3; idx[3] = 4;
    return 4;
  case ORC_QUAD3D:
    idx[0] = 0; idx[1] = 1; idx[2] = 2; idx[3] = 7; idx[4] = 8; idx[5] = 9;
    return 6;
  }
  return 0;
}

int orc_offset_dim(const orc_robot *r) {
  int idx[8];
  return offset_components(r->kind, idx);
}

void orc_canonical_state(const orc_robot *r, const double *x, double *c) {
  int idx[8];
  int k = offset_components(r->kind, idx);
  memcpy(c, x, sizeof(double) * (size_t)r->nx);
  for (int i = 0; i < k; i++) c[idx[i]] = 0.0;
}

void orc_offset(const orc_robot *r, const double *x, double *off) {
  int idx[8];
  int k = offset_components(r->kind, idx);
  for (int i = 0; i < k; i++) off[i] = x[idx[i]];
}

/* Weighted product metric of nigh_factory2 (nigh_custom_spaces.hpp:391-573):
 * the sum of the weighted block distances; L2 blocks, SO2 wrapped angle,
 * SO3 = acos(|<qa, qb>|) (the key's w-first quaternion constructor,
 * nigh_custom_spaces.hpp:547, permutes both operands alike, which leaves the
 * dot product unchanged). */
double orc_distance(const orc_robot *r, const double *a, const double *b) {
  const double *w = r->w;
  switch (r->kind) {
  case ORC_UNICYCLE1:
    return w[0] * hypot(a[0] - b[0], a[1] - b[1]) + w[1] * so2_dist(a[2], b[2]);
  case ORC_CAR1:
    return w[0] * hypot(a[0] - b[0], a[1] - b[1]) + w[1] * so2_dist(a[2], b[2]) +
           w[2] * so2_dist(a[3], b[3]);
  case ORC_QUAD2D:
    return w[0] * hypot(a[0] - b[0], a[1] - b[1]) + w[1] * so2_dist(a[2], b[2]) +
           w[2] * hypot(a[3] - b[3], a[4] - b[4]) + w[3] * fabs(a[5] - b[5]);
  case ORC_QUAD3D: {
    double dq = fabs(a[3] * b[3] + a[4] * b[4] + a[5] * b[5] + a[6] * b[6]);
    if (dq > 1.0) dq = 1.0;
    return w[0] * norm3(a[0] - b[0], a[1] - b[1], a[2] - b[2]) + w[1] * acos(dq) +
           w[2] * norm3(a[7] - b[7], a[8] - b[8], a[9] - b[9]) +
           w[3] * norm3(a[10] - b[10], a[11] - b[11], a[12] - b[12]);
  }
  }
  return 0.0;
}

/* Time lower bound used by the g-score (dbastar.cpp:843-847).  The unicycle1
 * form (max of distance over max speed per block, 0.5 m/s and 0.5 rad/s) is
 * pinned by the "min time" annotations; the others follow the same form
 * with the speed limits listed here. */
double orc_lower_bound_time(const orc_robot *r, const double *a, const double *b) {
  double t0, t1, t2 = 0, t3 = 0;
  switch (r->kind) {
  case ORC_UNICYCLE1:
    t0 = hypot(a[0] - b[0], a[1] - b[1]) / 0.5;
    t1 = so2_dist(a[2], b[2]) / 0.5;
    return fmax(t0, t1);
  case ORC_CAR1:
    t0 = hypot(a[0] - b[0], a[1] - b[1]) / 0.5;
    t1 = so2_dist(a[2], b[2]) / 0.5;
    t2 = so2_dist(a[3], b[3]) / 0.5;
    return fmax(fmax(t0, t1), t2);
  case ORC_QUAD2D:
    t0 = hypot(a[0] - b[0], a[1] - b[1]) / 2.0;
    t1 = so2_dist(a[2], b[2]) / 4.0;
    t2 = hypot(a[3] - b[3], a[4] - b[4]) / 4.0;
    t3 = fabs(a[5] - b[5]) / 8.0;
    return fmax(fmax(t0, t1), fmax(t2, t3));
  case ORC_QUAD3D: {
    double dq = fabs(a[3] * b[3] + a[4] * b[4] + a[5] * b[5] + a[6] * b[6]);
    if (dq > 1.0) dq = 1.0;
    t0 = norm3(a[0] - b[0], a[1] - b[1], a[2] - b[2]) / 4.0;
    t1 = acos(dq) / 8.0;
    t2 = norm3(a[7] - b[7], a[8] - b[8], a[9] - b[9]) / 4.0;
    t3 = norm3(a[10] - b[10], a[11] - b[11], a[12] - b[12]) / 8.0;
    return fmax(fmax(t0, t1), fmax(t2, t3));
  }
  }
  return 0.0;
}

static int pos_dim(const orc_robot *r) { return r->kind == ORC_QUAD3D ? 3 : 2; }

/* is_state_valid: position inside the environment bounds (inclusive). */
int orc_is_state_valid(const orc_robot *r, const orc_env *e, const double *x) {
  const int d = pos_dim(r);
  for (int i = 0; i < d; i++)
    if (!(x[i] >= e->lo[i] && x[i] <= e->hi[i])) return 0;
  return 1;
}

/* Separating-axis gap between an oriented box (centre c, yaw th, half
 * extents a along the heading and b across) and an axis-aligned box (centre
 * o, half extents H).  Positive: separated by at least that much along one
 * axis; <= 0: overlapping or touching. */
static double obb_aabb_gap(double cx, double cy, double ct, double st, double a, double b,
                           double ox, double oy, double Hx, double Hy) {
  const double ac = fabs(ct), as = fabs(st);
  const double dx = cx - ox, dy = cy - oy;
  const double gx = fabs(dx) - (a * ac + b * as + Hx);
  const double gy = fabs(dy) - (a * as + b * ac + Hy);
  const double du = dx * ct + dy * st, dv = -dx * st + dy * ct;
  const double gu = fabs(du) - (a + Hx * ac + Hy * as);
  const double gv = fabs(dv) - (b + Hx * as + Hy * ac);
  return fmax(fmax(gx, gy), fmax(gu, gv));
}

/* Axis-aligned clearance between a part's bounding box and an obstacle: the
 * quantity reported as min_gap (a lower bound of the separating-axis gap). */
static double obb_aabb_clearance(double cx, double cy, double ct, double st, double a,
                                 double b, double ox, double oy, double Hx, double Hy) {
  const double ac = fabs(ct), as = fabs(st);
  const double gx = fabs(cx - ox) - (a * ac + b * as + Hx);
  const double gy = fabs(cy - oy) - (a * as + b * ac + Hy);
  return fmax(gx, gy);
}

/* Sphere against axis-aligned box: exact signed distance minus the radius. */
static double sphere_aabb_gap(const double *p, double rad, const double *o, const double *H) {
  double d[3], m = -1e300, s = 0;
  for (int i = 0; i < 3; i++) {
    d[i] = fabs(p[i] - o[i]) - H[i];
    m = fmax(m, d[i]);
    if (d[i] > 0) s += d[i] * d[i];
  }
  return (m <= 0 ? m : sqrt(s)) - rad;
}

typedef struct part_pose { double cx, cy, ct, st; } part_pose;

/* Robot part poses at state x (transformation_collision_geometries).  car1:
 * trailer centre = position - hitch * (cos theta1, sin theta1), yaw theta1,
 * as the reference's car/trailer transform (src/ompl/robots.cpp:2428-2449). */
static int part_poses(const orc_robot *r, const double *x, part_pose *pp) {
  switch (r->kind) {
  case ORC_UNICYCLE1:
  case ORC_QUAD2D:
    pp[0].cx = x[0]; pp[0].cy = x[1]; pp[0].ct = cos(x[2]); pp[0].st = sin(x[2]);
    return 1;
  case ORC_CAR1: {
    pp[0].cx = x[0]; pp[0].cy = x[1]; pp[0].ct = cos(x[2]); pp[0].st = sin(x[2]);
    const double c1 = cos(x[3]), s1 = sin(x[3]);
    pp[1].cx = x[0] - r->hitch * c1; pp[1].cy = x[1] - r->hitch * s1;
    pp[1].ct = c1; pp[1].st = s1;
    return 2;
  }
  }
  return 0;
}

static void obs_centre(const orc_env *e, int o, double *c, double *H) {
  for (int i = 0; i < e->dim; i++) {
    const double lo = e->obs_lo[(size_t)o * e->dim + i], hi = e->obs_hi[(size_t)o * e->dim + i];
    c[i] = 0.5 * (lo + hi);
    H[i] = 0.5 * (hi - lo);
  }
}

double orc_state_gap(const orc_robot *r, const orc_env *e, const double *x, int o) {
  double c[3], H[3];
  obs_centre(e, o, c, H);
  if (r->kind == ORC_QUAD3D) return sphere_aabb_gap(x, r->radius, c, H);
  part_pose pp[2];
  const int np = part_poses(r, x, pp);
  double g = 1e300;
  for (int k = 0; k < np; k++)
    g = fmin(g, obb_aabb_gap(pp[k].cx, pp[k].cy, pp[k].ct, pp[k].st, 0.5 * r->box[0],
                             0.5 * r->box[1], c[0], c[1], H[0], H[1]));
  return g;
}

/* min over parts of the axis-aligned clearance (the min_gap quantity) */
static double state_clearance(const orc_robot *r, const double *x, const double *c,
                              const double *H, const part_pose *pp, int np) {
  if (r->kind == ORC_QUAD3D) {
    double m = -1e300;
    for (int i = 0; i < 3; i++) m = fmax(m, fabs(x[i] - c[i]) - H[i] - r->radius);
    return m;
  }
  double g = 1e300;
  for (int k = 0; k < np; k++)
    g = fmin(g, obb_aabb_clearance(pp[k].cx, pp[k].cy, pp[k].ct, pp[k].st, 0.5 * r->box[0],
                                   0.5 * r->box[1], c[0], c[1], H[0], H[1]));
  return g;
}

void orc_rollout(const orc_robot *r, const double *x0, const double *us, int steps, double *xs) {
  const int nx = r->nx;
  memcpy(xs, x0, sizeof(double) * (size_t)nx);
  for (int k = 0; k < steps; k++)
    orc_step(r, xs + (size_t)k * nx, us + (size_t)k * r->nu, xs + (size_t)(k + 1) * nx);
}

static int is_rollout_robot(int kind) { return kind == ORC_QUAD2D || kind == ORC_QUAD3D; }

/* LazyTraj::compute (dbastar.hpp:174-182) with the bounds callback, i.e. the
 * transform_primitive of the robot: translation robots shift every state by
 * the offset; velocity-invariant robots shift the start and roll the
 * primitive's actions out again, stopping at the first invalid state.
 * Returns the index of the first out-of-bounds state, or L. */
static int transform_bounded(const orc_robot *r, const orc_env *e, const orc_prims *pr,
                             const double *off, int p, double *xs) {
  const int nx = r->nx, L = pr->len[p];
  const double *S = pr->states + (size_t)pr->soff[p] * nx;
  int idx[8];
  const int k = offset_components(r->kind, idx);
  if (!is_rollout_robot(r->kind)) {
    memcpy(xs, S, sizeof(double) * (size_t)L * nx);
    for (int s = 0; s < L; s++)
      for (int i = 0; i < k; i++) xs[(size_t)s * nx + idx[i]] += off[i];
    /* bounds over all states, first invalid (dbastar.cpp:446-455) */
    for (int s = 0; s < L; s++)
      if (!orc_is_state_valid(r, e, xs + (size_t)s * nx)) return s;
    return L;
  }
  const double *A = pr->actions + (size_t)pr->aoff[p] * r->nu;
  memcpy(xs, S, sizeof(double) * (size_t)nx);
  for (int i = 0; i < k; i++) xs[idx[i]] += off[i];
  for (int s = 0; s < L; s++) {
    if (!orc_is_state_valid(r, e, xs + (size_t)s * nx)) return s;
    if (s + 1 < L) orc_step(r, xs + (size_t)s * nx, A + (size_t)s * r->nu, xs + (size_t)(s + 1) * nx);
  }
  return L;
}

int orc_check_pair(const orc_robot *r, const orc_env *e, const orc_prims *pr,
                   const double *x_node, int p, double *xs, int16_t *first_invalid,
                   double *end_state, double *min_gap) {
  const int nx = r->nx, L = pr->len[p];
  double off[8];
  orc_offset(r, x_node, off);
  const int first_oob = transform_bounded(r, e, pr, off, p, xs);
  if (first_oob < L) {
    *first_invalid = (int16_t)first_oob;
    memcpy(end_state, xs + (size_t)first_oob * nx, sizeof(double) * (size_t)nx);
    *min_gap = NAN;
    return ORC_OUT_OF_BOUNDS;
  }
  memcpy(end_state, xs + (size_t)(L - 1) * nx, sizeof(double) * (size_t)nx);
  /* is_motion_collision_free over every state (dbastar.cpp:461-485) */
  double mg = INFINITY; /* no obstacle: +inf */
  for (int s = 0; s < L; s++) {
    const double *x = xs + (size_t)s * nx;
    part_pose pp[2];
    const int np = r->kind == ORC_QUAD3D ? 0 : part_poses(r, x, pp);
    int hit = 0;
    for (int o = 0; o < e->n_obs; o++) {
      double c[3], H[3];
      obs_centre(e, o, c, H);
      mg = fmin(mg, state_clearance(r, x, c, H, pp, np));
      double g;
      if (r->kind == ORC_QUAD3D) {
        g = sphere_aabb_gap(x, r->radius, c, H);
      } else {
        g = 1e300;
        for (int q = 0; q < np; q++)
          g = fmin(g, obb_aabb_gap(pp[q].cx, pp[q].cy, pp[q].ct, pp[q].st, 0.5 * r->box[0],
                                   0.5 * r->box[1], c[0], c[1], H[0], H[1]));
      }
      if (g <= 0.0) hit = 1;
    }
    if (hit) {
      *first_invalid = (int16_t)s;
      *min_gap = mg <= ORC_GAP_CAP ? mg : INFINITY;
      return ORC_COLLISION;
    }
  }
  *first_invalid = (int16_t)L;
  *min_gap = mg <= ORC_GAP_CAP ? mg : INFINITY;
  return ORC_VALID;
}

static int max_len(const orc_prims *pr) {
  int m = 0;
  for (int p = 0; p < pr->P; p++) m = pr->len[p] > m ? pr->len[p] : m;
  return m;
}

int orc_expand(const orc_robot *r, const orc_env *e, const orc_prims *pr, int64_t N,
               const double *x, double radius, orc_out *out) {
  const int nx = r->nx;
  double *c = (double *)malloc(sizeof(double) * nx);
  double *xs = (double *)malloc(sizeof(double) * (size_t)max_len(pr) * nx);
  int64_t np = 0;
  for (int64_t n = 0; n < N; n++) {
    const double *xn = x + (size_t)n * nx;
    orc_canonical_state(r, xn, c);
    for (int p = 0; p < pr->P; p++) {
      const double d = orc_distance(r, c, pr->states + (size_t)pr->soff[p] * nx);
      if (!(d <= radius)) continue;
      if (np < out->cap) {
        int16_t fi;
        double mg;
        out->node[np] = (uint32_t)n;
        out->prim[np] = (uint32_t)p;
        out->verdict[np] = (uint8_t)orc_check_pair(r, e, pr, xn, p, xs, &fi,
                                                   out->end_state + (size_t)np * nx, &mg);
        out->first_invalid[np] = fi;
        if (out->min_gap) out->min_gap[np] = mg;
      }
      np++;
    }
  }
  free(c);
  free(xs);
  out->n_pairs = np;
  out->n_scanned = N * (int64_t)pr->P;
  return np > out->cap ? -1 : 0;
}

int orc_check_goal(const orc_robot *r, const double *xs, int L, const double *goal,
                   double bound, int n_check) {
  for (int k = 0; k < n_check; k++) {
    const int idx = (int)((float)(k + 1) / (float)(n_check + 1) * (float)L);
    if (orc_distance(r, xs + (size_t)idx * r->nx, goal) <= bound) return idx;
  }
  return -1;
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------ fast CPU baseline -- */
/* Radius query by a sorted-angle window (the metric is bounded below by
 * w1 * so2(theta) for every planar robot) and a uniform-grid broadphase over
 * the obstacles; per-pair early exit at the first colliding state. */

typedef struct grid {
  int dim, n[3];
  double lo[3], cell[3];
  int *start; /* cells+1 */
  int *items;
} grid;

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

static void grid_build(grid *g, const orc_env *e) {
  g->dim = e->dim;
  int cells = 1;
  for (int i = 0; i < 3; i++) { g->n[i] = 1; g->lo[i] = 0; g->cell[i] = 1; }
  for (int i = 0; i < e->dim; i++) {
    const double ext = e->hi[i] - e->lo[i];
    int n = (int)(ext / 0.5);
    g->n[i] = clampi(n, 1, 256);
    g->lo[i] = e->lo[i];
    g->cell[i] = ext / g->n[i];
    cells *= g->n[i];
  }
  int *cnt = (int *)calloc((size_t)cells + 1, sizeof(int));
  int lohi[3][2];
  for (int pass = 0; pass < 2; pass++) {
    for (int o = 0; o < e->n_obs; o++) {
      for (int i = 0; i < 3; i++) { lohi[i][0] = 0; lohi[i][1] = 0; }
      for (int i = 0; i < e->dim; i++) {
        lohi[i][0] = clampi((int)floor((e->obs_lo[(size_t)o * e->dim + i] - g->lo[i]) / g->cell[i]), 0, g->n[i] - 1);
        lohi[i][1] = clampi((int)floor((e->obs_hi[(size_t)o * e->dim + i] - g->lo[i]) / g->cell[i]), 0, g->n[i] - 1);
      }
      for (int a = lohi[0][0]; a <= lohi[0][1]; a++)
        for (int b = lohi[1][0]; b <= lohi[1][1]; b++)
          for (int z = lohi[2][0]; z <= lohi[2][1]; z++) {
            const int cidx = (z * g->n[1] + b) * g->n[0] + a;
            if (pass == 0) cnt[cidx + 1]++;
            else g->items[cnt[cidx]++] = o;
          }
    }
    if (pass == 0) {
      for (int i = 0; i < cells; i++) cnt[i + 1] += cnt[i];
      g->start = (int *)malloc(sizeof(int) * ((size_t)cells + 1));
      memcpy(g->start, cnt, sizeof(int) * ((size_t)cells + 1));
      g->items = (int *)malloc(sizeof(int) * ((size_t)cnt[cells] + 1));
    }
  }
  free(cnt);
}

static void grid_free(grid *g) { free(g->start); free(g->items); }

/* does any obstacle overlapping the query box [qlo, qhi] give gap <= 0 */
static int grid_collide(const grid *g, const orc_robot *r, const orc_env *e, const double *x,
                        const part_pose *pp, int np) {
  if (r->kind == ORC_QUAD3D) {
    int lo[3], hi[3];
    for (int i = 0; i < 3; i++) {
      lo[i] = clampi((int)floor((x[i] - r->radius - g->lo[i]) / g->cell[i]), 0, g->n[i] - 1);
      hi[i] = clampi((int)floor((x[i] + r->radius - g->lo[i]) / g->cell[i]), 0, g->n[i] - 1);
    }
    for (int z = lo[2]; z <= hi[2]; z++)
      for (int b = lo[1]; b <= hi[1]; b++)
        for (int a = lo[0]; a <= hi[0]; a++) {
          const int cidx = (z * g->n[1] + b) * g->n[0] + a;
          for (int t = g->start[cidx]; t < g->start[cidx + 1]; t++) {
            double c[3], H[3];
            obs_centre(e, g->items[t], c, H);
            if (sphere_aabb_gap(x, r->radius, c, H) <= 0.0) return 1;
          }
        }
    return 0;
  }
  const double a = 0.5 * r->box[0], b = 0.5 * r->box[1];
  for (int q = 0; q < np; q++) {
    const double ac = fabs(pp[q].ct), as = fabs(pp[q].st);
    const double ex = a * ac + b * as, ey = a * as + b * ac;
    const int x0 = clampi((int)floor((pp[q].cx - ex - g->lo[0]) / g->cell[0]), 0, g->n[0] - 1);
    const int x1 = clampi((int)floor((pp[q].cx + ex - g->lo[0]) / g->cell[0]), 0, g->n[0] - 1);
    const int y0 = clampi((int)floor((pp[q].cy - ey - g->lo[1]) / g->cell[1]), 0, g->n[1] - 1);
    const int y1 = clampi((int)floor((pp[q].cy + ey - g->lo[1]) / g->cell[1]), 0, g->n[1] - 1);
    for (int yy = y0; yy <= y1; yy++)
      for (int xx = x0; xx <= x1; xx++) {
        const int cidx = yy * g->n[0] + xx;
        for (int t = g->start[cidx]; t < g->start[cidx + 1]; t++) {
          double c[3], H[3];
          obs_centre(e, g->items[t], c, H);
          if (obb_aabb_gap(pp[q].cx, pp[q].cy, pp[q].ct, pp[q].st, a, b, c[0], c[1], H[0], H[1]) <= 0.0)
            return 1;
        }
      }
  }
  return 0;
}

static int check_pair_fast(const orc_robot *r, const orc_env *e, const orc_prims *pr,
                           const grid *g, const double *x_node, int p, double *xs,
                           int16_t *first_invalid, double *end_state) {
  const int nx = r->nx, L = pr->len[p];
  double off[8];
  orc_offset(r, x_node, off);
  const int first_oob = transform_bounded(r, e, pr, off, p, xs);
  if (first_oob < L) {
    *first_invalid = (int16_t)first_oob;
    memcpy(end_state, xs + (size_t)first_oob * nx, sizeof(double) * (size_t)nx);
    return ORC_OUT_OF_BOUNDS;
  }
  memcpy(end_state, xs + (size_t)(L - 1) * nx, sizeof(double) * (size_t)nx);
  for (int s = 0; s < L; s++) {
    const double *xx = xs + (size_t)s * nx;
    part_pose pp[2];
    const int np = r->kind == ORC_QUAD3D ? 0 : part_poses(r, xx, pp);
    if (grid_collide(g, r, e, xx, pp, np)) {
      *first_invalid = (int16_t)s;
      return ORC_COLLISION;
    }
  }
  *first_invalid = (int16_t)L;
  return ORC_VALID;
}

typedef struct ang_key { double th; int p; } ang_key;
static int cmp_ang(const void *a, const void *b) {
  const double x = ((const ang_key *)a)->th, y = ((const ang_key *)b)->th;
  return x < y ? -1 : (x > y ? 1 : 0);
}
static int cmp_int(const void *a, const void *b) {
  return *(const int *)a - *(const int *)b;
}
static double wrap_pi(double a) {
  a = fmod(a + PI_D, TWO_PI);
  if (a < 0) a += TWO_PI;
  return a - PI_D;
}

/* neighbours of canonical key c, ascending primitive index; returns count */
static int radius_query_fast(const orc_robot *r, const orc_prims *pr, const ang_key *keys,
                             const double *c, double radius, int *outp) {
  const int nx = r->nx;
  int n = 0;
  if (r->kind == ORC_QUAD3D) {
    for (int p = 0; p < pr->P; p++)
      if (orc_distance(r, c, pr->states + (size_t)pr->soff[p] * nx) <= radius) outp[n++] = p;
    return n;
  }
  /* window on theta (component 2); every metric here has w1 * so2(dtheta) */
  const double win = radius / r->w[1] + 1e-9;
  if (win >= PI_D) {
    for (int p = 0; p < pr->P; p++)
      if (orc_distance(r, c, pr->states + (size_t)pr->soff[p] * nx) <= radius) outp[n++] = p;
    return n;
  }
  const double th = wrap_pi(c[2]);
  double lo = th - win, hi = th + win;
  double ranges[2][2];
  int nr = 0;
  if (lo < -PI_D) { ranges[nr][0] = lo + TWO_PI; ranges[nr][1] = PI_D; nr++; lo = -PI_D; }
  if (hi > PI_D) { ranges[nr][0] = -PI_D; ranges[nr][1] = hi - TWO_PI; nr++; hi = PI_D; }
  ranges[nr][0] = lo; ranges[nr][1] = hi; nr++;
  for (int t = 0; t < nr; t++) {
    int a = 0, b = pr->P;
    while (a < b) { /* first key >= lo */
      const int m = (a + b) / 2;
      if (keys[m].th < ranges[t][0]) a = m + 1; else b = m;
    }
    for (int i = a; i < pr->P && keys[i].th <= ranges[t][1]; i++) {
      const int p = keys[i].p;
      if (orc_distance(r, c, pr->states + (size_t)pr->soff[p] * nx) <= radius) outp[n++] = p;
    }
  }
  qsort(outp, (size_t)n, sizeof(int), cmp_int);
  /* windows may overlap near +-pi: drop duplicates */
  int m = 0;
  for (int i = 0; i < n; i++)
    if (m == 0 || outp[m - 1] != outp[i]) outp[m++] = outp[i];
  return m;
}

int orc_expand_fast(const orc_robot *r, const orc_env *e, const orc_prims *pr, int64_t N,
                    const double *x, double radius, int threads, orc_out *out) {
  const int nx = r->nx, P = pr->P;
  grid g;
  grid_build(&g, e);
  ang_key *keys = (ang_key *)malloc(sizeof(ang_key) * (size_t)P);
  for (int p = 0; p < P; p++) {
    keys[p].th = wrap_pi(pr->states[(size_t)pr->soff[p] * nx + 2]);
    keys[p].p = p;
  }
  qsort(keys, (size_t)P, sizeof(ang_key), cmp_ang);
  int64_t *cnt = (int64_t *)calloc((size_t)N + 1, sizeof(int64_t));
  const int ML = max_len(pr);
  if (threads < 1) threads = 1;
  /* pass 1: radius queries (counts) */
#pragma omp parallel num_threads(threads)
  {
    int *nb = (int *)malloc(sizeof(int) * (size_t)P);
    double *c = (double *)malloc(sizeof(double) * nx);
#pragma omp for schedule(dynamic, 64)
    for (int64_t n = 0; n < N; n++) {
      orc_canonical_state(r, x + (size_t)n * nx, c);
      cnt[n + 1] = radius_query_fast(r, pr, keys, c, radius, nb);
    }
    free(nb);
    free(c);
  }
  for (int64_t n = 0; n < N; n++) cnt[n + 1] += cnt[n];
  const int64_t total = cnt[N];
  out->n_pairs = total;
  out->n_scanned = N * (int64_t)P;
  if (total > out->cap) {
    free(cnt); free(keys); grid_free(&g);
    return -1;
  }
  /* pass 2: neighbour lists and checks */
#pragma omp parallel num_threads(threads)
  {
    int *nb = (int *)malloc(sizeof(int) * (size_t)P);
    double *c = (double *)malloc(sizeof(double) * nx);
    double *xs = (double *)malloc(sizeof(double) * (size_t)ML * nx);
#pragma omp for schedule(dynamic, 16)
    for (int64_t n = 0; n < N; n++) {
      const double *xn = x + (size_t)n * nx;
      orc_canonical_state(r, xn, c);
      const int k = radius_query_fast(r, pr, keys, c, radius, nb);
      for (int i = 0; i < k; i++) {
        const int64_t j = cnt[n] + i;
        int16_t fi;
        out->node[j] = (uint32_t)n;
        out->prim[j] = (uint32_t)nb[i];
        out->verdict[j] = (uint8_t)check_pair_fast(r, e, pr, &g, xn, nb[i], xs, &fi,
                                                   out->end_state + (size_t)j * nx);
        out->first_invalid[j] = fi;
        if (out->min_gap) out->min_gap[j] = NAN;
      }
    }
    free(nb);
    free(c);
    free(xs);
  }
  free(cnt);
  free(keys);
  grid_free(&g);
  return 0;
}
