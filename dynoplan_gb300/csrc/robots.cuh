// robots.cuh -- device-side robot models of the expansion (sm_103a).
//
// One traits struct per dynobench model the expansion supports.  Each gives
// the compile-time shape (state/control sizes, collision parts, which state
// components canonical_state zeroes and offset returns) and the FP64 dynamics
// step used by the per-primitive canonical rollout.  The formulas restate the
// dynobench models the reference calls from Expander::expand_lazy and
// check_lazy_trajectory (include/dynoplan/dbastar/dbastar.hpp:270-312,
// src/dbastar/dbastar.cpp:391-490); the quad2d/quad3d steps follow the
// reference's recorded trajectories (benchmark_initguess/quad2d,
// benchmark_initguess/quadrotor_v0): explicit Euler from the current state,
// body-frame quaternion exponential.
#pragma once

#include <cstdint>

#include "dpg.h"

namespace dpg {

// Model constants on the device (dpg_robot_desc, flattened).
struct RobotParams {
  double dt;
  double w[4];
  double half_len, half_wid;  // planar collision box half extents
  double hitch, wheelbase;
  double radius;
  double mass, lever, t2t;     // lever = arm / sqrt(2) (X configuration)
  double inertia[3];
  double ang_gain, g;
};

// Translation robots: canonical_state zeroes (x, y); offset = (x, y).
// Velocity-invariant robots: canonical_state zeroes position and velocity;
// offset = (position, velocity); transform_primitive rolls the actions out
// again from the shifted start.
template <int KIND> struct Robot;

template <> struct Robot<DPG_ROBOT_UNICYCLE1> {
  static constexpr int NX = 3, NU = 2, PARTS = 1, POSD = 2, VELOFF = 0;
  static constexpr bool ROLLOUT = false, SPHERE = false;
  static constexpr int KEYD = 1;  // kept key components: theta
  static constexpr int CHUNK = 8;  // states per culling chunk
  static constexpr int CHECK_BLOCKS = 4;  // check_pairs blocks per SM (register bound)
  static constexpr int SLOT_BLOCKS = 4;  // slot-parallel check: 64 registers a thread
  static constexpr bool BOUNDS_SLOTS = false;  // bounds tests walked per lane (the slot form: car1 2.07 -> 2.28 ms)
  __host__ __device__ static int key_comp(int i) { return 2; }
  __host__ __device__ static int vel_comp(int i) { return -1; }
};

template <> struct Robot<DPG_ROBOT_CAR1> {
  static constexpr int NX = 4, NU = 2, PARTS = 2, POSD = 2, VELOFF = 0;
  static constexpr bool ROLLOUT = false, SPHERE = false;
  static constexpr int KEYD = 2;  // theta0, theta1
  static constexpr int CHUNK = 8;
  static constexpr int CHECK_BLOCKS = 4;  // measured: 4 beats 3, 5 and 6 here
  static constexpr int SLOT_BLOCKS = 4;  // slot-parallel check: 64 registers a thread
  static constexpr bool BOUNDS_SLOTS = false;  // bounds tests walked per lane (the slot form: car1 2.07 -> 2.28 ms)
  __host__ __device__ static int key_comp(int i) { return 2 + i; }
  __host__ __device__ static int vel_comp(int i) { return -1; }
};

template <> struct Robot<DPG_ROBOT_QUAD2D> {
  static constexpr int NX = 6, NU = 2, PARTS = 1, POSD = 2, VELOFF = 2;
  static constexpr bool ROLLOUT = true, SPHERE = false;
  static constexpr int KEYD = 2;  // theta, w
  static constexpr int CHUNK = 16;  // dt 0.01: ten times the states of the others per second
  static constexpr int CHECK_BLOCKS = 4;
  static constexpr int SLOT_BLOCKS = 4;  // slot-parallel check: 64 registers a thread
  static constexpr bool BOUNDS_SLOTS = false;  // bounds tests walked per lane
  __host__ __device__ static int key_comp(int i) { return i == 0 ? 2 : 5; }
  __host__ __device__ static int vel_comp(int i) { return 3 + i; }
};

template <> struct Robot<DPG_ROBOT_QUAD3D> {
  static constexpr int NX = 13, NU = 4, PARTS = 1, POSD = 3, VELOFF = 3;
  static constexpr bool ROLLOUT = true, SPHERE = true;
  static constexpr int KEYD = 7;  // quaternion (4), w (3)
  static constexpr int CHUNK = 16;
  static constexpr int CHECK_BLOCKS = 5;  // measured: 5 beats 4 and 6 here
  static constexpr int SLOT_BLOCKS = 4;  // slot-parallel check: 64 registers a thread
  static constexpr bool BOUNDS_SLOTS = true;   // bounds tests as (lane, state) slots when few lanes need them (11.45 -> 10.65 ms)
  __host__ __device__ static int key_comp(int i) { return i < 4 ? 3 + i : 6 + i; }
  __host__ __device__ static int vel_comp(int i) { return 7 + i; }
};

constexpr double kPi = 3.1415926535897932384626433832795;
constexpr double kTwoPi = 6.283185307179586476925286766559;

// wrapped angle distance, FP64, the oracle's formula (fabs, fmod, reflect)
__device__ __forceinline__ double so2_dist64(double a, double b) {
  double d = fabs(a - b);
  if (d >= kTwoPi) d = fmod(d, kTwoPi);  // (fmod(d, 2 pi) = d below 2 pi)
  return d > kPi ? kTwoPi - d : d;
}

// Angle normalisation of the planar steps, x - 2 pi floor((x + pi) / 2 pi):
// [-pi, pi), the form the reference's unicycle1 primitives show.  Products
// and differences are rounded separately (no FMA contraction) to match the
// plain C evaluation.
__device__ __forceinline__ double wrap_angle64(double x) {
  return __dsub_rn(x, __dmul_rn(kTwoPi, floor(__dadd_rn(x, kPi) / kTwoPi)));
}

// FP64 explicit Euler step (robot-specific).
template <int KIND>
__device__ void step64(const RobotParams &rp, const double *x, const double *u, double *xn);

template <>
__device__ inline void step64<DPG_ROBOT_UNICYCLE1>(const RobotParams &rp, const double *x,
                                                    const double *u, double *xn) {
  double s, c;
  sincos(x[2], &s, &c);
  xn[0] = x[0] + u[0] * c * rp.dt;
  xn[1] = x[1] + u[0] * s * rp.dt;
  xn[2] = wrap_angle64(x[2] + u[1] * rp.dt);
}

template <>
__device__ inline void step64<DPG_ROBOT_CAR1>(const RobotParams &rp, const double *x,
                                               const double *u, double *xn) {
  double s, c;
  sincos(x[2], &s, &c);
  xn[0] = x[0] + u[0] * c * rp.dt;
  xn[1] = x[1] + u[0] * s * rp.dt;
  xn[2] = wrap_angle64(x[2] + u[0] / rp.wheelbase * tan(u[1]) * rp.dt);
  xn[3] = wrap_angle64(x[3] + u[0] / rp.hitch * sin(x[2] - x[3]) * rp.dt);
}

template <>
__device__ inline void step64<DPG_ROBOT_QUAD2D>(const RobotParams &rp, const double *x,
                                                 const double *u, double *xn) {
  const double dt = rp.dt;
  double s, c;
  sincos(x[2], &s, &c);
  const double acc = (u[0] + u[1]) * rp.g * 0.5;
  xn[0] = x[0] + x[3] * dt;
  xn[1] = x[1] + x[4] * dt;
  xn[2] = wrap_angle64(x[2] + x[5] * dt);
  xn[3] = x[3] - acc * s * dt;
  xn[4] = x[4] + (acc * c - rp.g) * dt;
  xn[5] = x[5] + rp.ang_gain * rp.g * 0.5 * (u[0] - u[1]) * dt;
}

template <>
__device__ inline void step64<DPG_ROBOT_QUAD3D>(const RobotParams &rp, const double *x,
                                                 const double *u, double *xn) {
  const double dt = rp.dt;
  const double fu = rp.mass * rp.g * 0.25;
  const double f0 = u[0] * fu, f1 = u[1] * fu, f2 = u[2] * fu, f3 = u[3] * fu;
  const double F = f0 + f1 + f2 + f3;
  const double tx = rp.lever * (-f0 - f1 + f2 + f3);
  const double ty = rp.lever * (-f0 + f1 + f2 - f3);
  const double tz = rp.t2t * (-f0 + f1 - f2 + f3);
  const double qx = x[3], qy = x[4], qz = x[5], qw = x[6];
  const double am = F / rp.mass;
  const double ax = 2.0 * (qx * qz + qy * qw) * am;
  const double ay = 2.0 * (qy * qz - qx * qw) * am;
  const double az = (1.0 - 2.0 * (qx * qx + qy * qy)) * am - rp.g;
  const double wx = x[10], wy = x[11], wz = x[12];
  const double Jx = rp.inertia[0], Jy = rp.inertia[1], Jz = rp.inertia[2];
  const double hx = Jx * wx, hy = Jy * wy, hz = Jz * wz;
  const double cx = wy * hz - wz * hy, cy = wz * hx - wx * hz, cz = wx * hy - wy * hx;
  // q <- q (x) exp(w dt / 2), renormalised in FP64
  const double vx = 0.5 * dt * wx, vy = 0.5 * dt * wy, vz = 0.5 * dt * wz;
  const double th = sqrt(vx * vx + vy * vy + vz * vz);
  double sth, cth;
  sincos(th, &sth, &cth);
  const double sc = th > 1e-12 ? sth / th : 1.0;
  const double ex = vx * sc, ey = vy * sc, ez = vz * sc, ew = cth;
  const double nx_ = qw * ex + qx * ew + qy * ez - qz * ey;
  const double ny_ = qw * ey - qx * ez + qy * ew + qz * ex;
  const double nz_ = qw * ez + qx * ey - qy * ex + qz * ew;
  const double nw_ = qw * ew - qx * ex - qy * ey - qz * ez;
  const double nq = sqrt(nx_ * nx_ + ny_ * ny_ + nz_ * nz_ + nw_ * nw_);
  xn[0] = x[0] + x[7] * dt;
  xn[1] = x[1] + x[8] * dt;
  xn[2] = x[2] + x[9] * dt;
  xn[3] = nx_ / nq;
  xn[4] = ny_ / nq;
  xn[5] = nz_ / nq;
  xn[6] = nw_ / nq;
  xn[7] = x[7] + ax * dt;
  xn[8] = x[8] + ay * dt;
  xn[9] = x[9] + az * dt;
  xn[10] = wx + (tx - cx) / Jx * dt;
  xn[11] = wy + (ty - cy) / Jy * dt;
  xn[12] = wz + (tz - cz) / Jz * dt;
}

// FP64 metric restricted to the kept key components plus the per-primitive
// constant part (the weighted norms of the components the node's canonical
// state zeroes).  Exactly the oracle's distance(canonical(x), start_p).
template <int KIND>
__device__ double key_dist64(const RobotParams &rp, const double *xnode, const double *start);

template <>
__device__ inline double key_dist64<DPG_ROBOT_UNICYCLE1>(const RobotParams &rp, const double *xn,
                                                          const double *s) {
  return rp.w[0] * hypot(0.0 - s[0], 0.0 - s[1]) + rp.w[1] * so2_dist64(xn[2], s[2]);
}
template <>
__device__ inline double key_dist64<DPG_ROBOT_CAR1>(const RobotParams &rp, const double *xn,
                                                     const double *s) {
  return rp.w[0] * hypot(0.0 - s[0], 0.0 - s[1]) + rp.w[1] * so2_dist64(xn[2], s[2]) +
         rp.w[2] * so2_dist64(xn[3], s[3]);
}
template <>
__device__ inline double key_dist64<DPG_ROBOT_QUAD2D>(const RobotParams &rp, const double *xn,
                                                       const double *s) {
  return rp.w[0] * hypot(0.0 - s[0], 0.0 - s[1]) + rp.w[1] * so2_dist64(xn[2], s[2]) +
         rp.w[2] * hypot(0.0 - s[3], 0.0 - s[4]) + rp.w[3] * fabs(xn[5] - s[5]);
}
template <>
__device__ inline double key_dist64<DPG_ROBOT_QUAD3D>(const RobotParams &rp, const double *xn,
                                                       const double *s) {
  double dq = fabs(xn[3] * s[3] + xn[4] * s[4] + xn[5] * s[5] + xn[6] * s[6]);
  dq = dq > 1.0 ? 1.0 : dq;
  const double p = sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
  const double v = sqrt(s[7] * s[7] + s[8] * s[8] + s[9] * s[9]);
  const double a = xn[10] - s[10], b = xn[11] - s[11], c = xn[12] - s[12];
  return rp.w[0] * p + rp.w[1] * acos(dq) + rp.w[2] * v + rp.w[3] * sqrt(a * a + b * b + c * c);
}

}  // namespace dpg
