// metric.cuh -- the robots' full-state metric and time lower bounds on the
// device (the definitions of the oracle, oracle/oracle.c, and of the host
// search code): distance = sum of weighted block distances (L2 blocks,
// wrapped |d theta| for SO2, quaternion angle for SO3); lower_bound_time =
// max over blocks of block distance / block max speed, split into the
// position/rotation blocks (lbt_pr) and the velocity blocks (lbt_vel).
#pragma once

#include "robots.cuh"

namespace dpg {

// full-state metric, FP32 (the novelty query's first test) and FP64
template <int KIND>
__device__ float full_dist32(const float4 w, const float *a, const float *b) {
  auto so2f = [](float x, float y) {
    float d = fabsf(x - y);
    if (d >= 6.2831853071795865f) d = fmodf(d, 6.2831853071795865f);
    return d > 3.1415926535897932f ? 6.2831853071795865f - d : d;
  };
  if constexpr (KIND == DPG_ROBOT_UNICYCLE1) {
    return w.x * hypotf(a[0] - b[0], a[1] - b[1]) + w.y * so2f(a[2], b[2]);
  } else if constexpr (KIND == DPG_ROBOT_CAR1) {
    return w.x * hypotf(a[0] - b[0], a[1] - b[1]) + w.y * so2f(a[2], b[2]) + w.z * so2f(a[3], b[3]);
  } else if constexpr (KIND == DPG_ROBOT_QUAD2D) {
    return w.x * hypotf(a[0] - b[0], a[1] - b[1]) + w.y * so2f(a[2], b[2]) + w.z * hypotf(a[3] - b[3], a[4] - b[4]) +
           w.w * fabsf(a[5] - b[5]);
  } else {
    float dq = fminf(1.f, fabsf(a[3] * b[3] + a[4] * b[4] + a[5] * b[5] + a[6] * b[6]));
    auto l3 = [](float x, float y, float z) { return sqrtf(x * x + y * y + z * z); };
    return w.x * l3(a[0] - b[0], a[1] - b[1], a[2] - b[2]) + w.y * acosf(dq) +
           w.z * l3(a[7] - b[7], a[8] - b[8], a[9] - b[9]) + w.w * l3(a[10] - b[10], a[11] - b[11], a[12] - b[12]);
  }
}

template <int KIND>
__device__ double full_dist64(const RobotParams &rp, const double *a, const double *b) {
  auto so2d = [](double x, double y) {
    double d = fabs(x - y);
    if (d >= kTwoPi) d = fmod(d, kTwoPi);
    return d > kPi ? kTwoPi - d : d;
  };
  if constexpr (KIND == DPG_ROBOT_UNICYCLE1) {
    return rp.w[0] * hypot(a[0] - b[0], a[1] - b[1]) + rp.w[1] * so2d(a[2], b[2]);
  } else if constexpr (KIND == DPG_ROBOT_CAR1) {
    return rp.w[0] * hypot(a[0] - b[0], a[1] - b[1]) + rp.w[1] * so2d(a[2], b[2]) + rp.w[2] * so2d(a[3], b[3]);
  } else if constexpr (KIND == DPG_ROBOT_QUAD2D) {
    return rp.w[0] * hypot(a[0] - b[0], a[1] - b[1]) + rp.w[1] * so2d(a[2], b[2]) +
           rp.w[2] * hypot(a[3] - b[3], a[4] - b[4]) + rp.w[3] * fabs(a[5] - b[5]);
  } else {
    double dq = fmin(1.0, fabs(a[3] * b[3] + a[4] * b[4] + a[5] * b[5] + a[6] * b[6]));
    auto l3 = [](double x, double y, double z) { return sqrt(x * x + y * y + z * z); };
    return rp.w[0] * l3(a[0] - b[0], a[1] - b[1], a[2] - b[2]) + rp.w[1] * acos(dq) +
           rp.w[2] * l3(a[7] - b[7], a[8] - b[8], a[9] - b[9]) + rp.w[3] * l3(a[10] - b[10], a[11] - b[11], a[12] - b[12]);
  }
}


__device__ __forceinline__ double qangle64(const double *a, const double *b) {
  return acos(fmin(1.0, fabs(a[3] * b[3] + a[4] * b[4] + a[5] * b[5] + a[6] * b[6])));
}

// lower bound of the time between the position / rotation parts (max speeds
// unicycle1, car1 0.5 m/s, 0.5 rad/s; quad2d 2 m/s, 4 rad/s; quadrotor 4 m/s, 8 rad/s)
template <int KIND>
__device__ double lbt_pr64(const double *a, const double *b) {
  if constexpr (KIND == DPG_ROBOT_UNICYCLE1) {
    return fmax(hypot(a[0] - b[0], a[1] - b[1]) / 0.5, so2_dist64(a[2], b[2]) / 0.5);
  } else if constexpr (KIND == DPG_ROBOT_CAR1) {
    return fmax(fmax(hypot(a[0] - b[0], a[1] - b[1]) / 0.5, so2_dist64(a[2], b[2]) / 0.5),
                so2_dist64(a[3], b[3]) / 0.5);
  } else if constexpr (KIND == DPG_ROBOT_QUAD2D) {
    return fmax(hypot(a[0] - b[0], a[1] - b[1]) / 2.0, so2_dist64(a[2], b[2]) / 4.0);
  } else {
    const double dp = sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
    return fmax(dp / 4.0, qangle64(a, b) / 8.0);
  }
}

// ... and between the velocity parts (0 for the kinematic robots; quad2d
// 4 m/s^2-equivalent and 8 rad/s^2, quadrotor 4 and 8)
template <int KIND>
__device__ double lbt_vel64(const double *a, const double *b) {
  if constexpr (KIND == DPG_ROBOT_QUAD2D) {
    return fmax(hypot(a[3] - b[3], a[4] - b[4]) / 4.0, fabs(a[5] - b[5]) / 8.0);
  } else if constexpr (KIND == DPG_ROBOT_QUAD3D) {
    auto l3 = [](double x, double y, double z) { return sqrt(x * x + y * y + z * z); };
    return fmax(l3(a[7] - b[7], a[8] - b[8], a[9] - b[9]) / 4.0, l3(a[10] - b[10], a[11] - b[11], a[12] - b[12]) / 8.0);
  } else {
    return 0.0;
  }
}

}  // namespace dpg
