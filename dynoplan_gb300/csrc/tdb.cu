// tdb.cu -- tdb-A*'s checks of explicit (node, motion) pairs
// (include/dpg_tdb.h): forward or reverse transform, bounds and collision
// verdict, then the constraint test.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "ctx.h"
#include "dpg_tdb.h"
#include "metric.cuh"
#include "state_check.cuh"

using namespace dpg;

namespace {

struct TdbView {
  const double *st64;  // canonical FP64 states [S][NX]
  const int64_t *soff;
  const int32_t *len;
  int reverse;
  const float *node_g;
  int nc;
  const float *c_time;
  const double *c_state;
  const double *goal;
  double delta;
};

// state k of motion p applied at node x.  Forward: the motion starts at the
// node.  Reverse: the motion ends at the node -- translation robots shift
// the positions so that the last one is the node's; the rollout robots
// (db-A*'s transform_primitiveDirectReverse, include/dynoplan/dbastar/
// dbastar.hpp:183-201) take the offset (position, velocity) at the last
// state: velocities shifted by dv = v_node - v_last, positions by
// p_node - p_last + (t_k - t_last) dv, which is the same actions' rollout
// from the shifted start (no dynamics term depends on position or velocity).
template <int KIND>
__device__ void tdb_state(const RobotParams &rp, const TdbView &tv, const double *x, int64_t s0, int L, int k,
                          double *out) {
  using R = Robot<KIND>;
  const double *c = tv.st64 + (s0 + k) * R::NX;
#pragma unroll
  for (int i = 0; i < R::NX; i++) out[i] = c[i];
  if (tv.reverse) {
    const double *last = tv.st64 + (s0 + L - 1) * R::NX;
    const double tk = (k - (L - 1)) * rp.dt;  // time from the last state (<= 0)
#pragma unroll
    for (int i = 0; i < R::POSD; i++) out[i] += x[i] - last[i];
#pragma unroll
    for (int i = 0; i < R::VELOFF; i++) {
      const double dv = x[R::vel_comp(i)] - last[R::vel_comp(i)];
      out[i] += tk * dv;
      out[R::vel_comp(i)] += dv;
    }
    return;
  }
  const double t = k * rp.dt;
#pragma unroll
  for (int i = 0; i < R::POSD; i++) out[i] += x[i];
#pragma unroll
  for (int i = 0; i < R::VELOFF; i++) {
    out[i] += t * x[R::vel_comp(i)];
    out[R::vel_comp(i)] += x[R::vel_comp(i)];
  }
}

template <int KIND>
__global__ void tdb_check(RobotParams rp, EnvView ev, TdbView tv, const double *xn, int64_t n, const uint32_t *node,
                          const uint32_t *prim, uint8_t *verdict, int32_t *first_invalid, double *end_state) {
  using R = Robot<KIND>;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int p = (int)prim[i];
  const int L = tv.len[p];
  const int64_t s0 = tv.soff[p];
  const double *x = xn + (int64_t)node[i] * R::NX;
  double s[R::NX];
  int k_oob = L;
  for (int k = 0; k < L && k_oob == L; k++) {
    tdb_state<KIND>(rp, tv, x, s0, L, k, s);
    if (!state_in_bounds64<KIND>(ev, s)) k_oob = k;
  }
  uint8_t v = DPG_VALID;
  int fi = L, er = L - 1;
  if (k_oob < L) {
    v = DPG_OUT_OF_BOUNDS;
    fi = er = k_oob;
  } else {
    for (int k = 0; k < L; k++) {
      tdb_state<KIND>(rp, tv, x, s0, L, k, s);
      if (state_collides64<KIND>(rp, ev, s)) {
        v = DPG_COLLISION;
        fi = k;
        break;
      }
    }
  }
  if (v == DPG_VALID && tv.nc > 0) {
    tdb_state<KIND>(rp, tv, x, s0, L, tv.reverse ? L - 1 : 0, s);
    const bool reaches = full_dist64<KIND>(rp, s, tv.goal) <= tv.delta;
    const float g = tv.node_g[node[i]];
    for (int c = 0; c < tv.nc; c++) {
      const float t_off = tv.c_time[c] - g;  // float, as time_offset
      const long long idx = llround((double)t_off / rp.dt);
      int k = -1;
      if (reaches && idx >= L - 1) k = L - 1;
      if (idx >= 0 && idx < L - 1) k = (int)idx;
      if (k < 0) continue;
      tdb_state<KIND>(rp, tv, x, s0, L, k, s);
      if (full_dist64<KIND>(rp, s, tv.c_state + (int64_t)c * R::NX) <= tv.delta) {
        v = DPG_CONSTRAINT_VIOLATION;
        fi = c;
        break;
      }
    }
  }
  verdict[i] = v;
  first_invalid[i] = fi;
  if (end_state) tdb_state<KIND>(rp, tv, x, s0, L, er, end_state + i * R::NX);
}

template <class F> void with_kind_t(int kind, F &&f) {
  switch (kind) {
    case DPG_ROBOT_UNICYCLE1: f(std::integral_constant<int, DPG_ROBOT_UNICYCLE1>{}); break;
    case DPG_ROBOT_CAR1: f(std::integral_constant<int, DPG_ROBOT_CAR1>{}); break;
    case DPG_ROBOT_QUAD3D: f(std::integral_constant<int, DPG_ROBOT_QUAD3D>{}); break;
    case DPG_ROBOT_QUAD2D: f(std::integral_constant<int, DPG_ROBOT_QUAD2D>{}); break;
  }
}

// device copy of a host array (freed by the owner's destructor)
struct Dev {
  void *p = nullptr;
  ~Dev() { cudaFree(p); }
  bool put(const void *h, size_t bytes) {
    if (!bytes) return true;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return false;
    return !h || cudaMemcpy(p, h, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
  }
};

}  // namespace

extern "C" int dpg_tdb_check_pairs(dpg_ctx *c, const dpg_tdb_args *a, int64_t N, const double *x, int64_t n,
                                   const uint32_t *node, const uint32_t *prim, uint8_t *verdict,
                                   int32_t *first_invalid, double *end_state) {
  if (!c || !a || N < 0 || n < 0 || (n > 0 && (!x || !node || !prim || !verdict || !first_invalid))) return DPG_ERR_ARG;
  if (!c->have_prims || !c->have_env) return DPG_ERR_STATE;
  const int kind = c->robot.kind, nx = c->robot.nx;
  if (a->n_constraints < 0 || (a->n_constraints > 0 && (!a->c_time || !a->c_state || !a->node_g || !a->goal)))
    return DPG_ERR_ARG;
  for (int64_t i = 0; i < n; i++)
    if ((int64_t)node[i] >= N || (int64_t)prim[i] >= c->P) {
      c->err = "tdb_check_pairs: node or motion index out of range";
      return DPG_ERR_ARG;
    }
  if (n == 0) return DPG_OK;
  cudaSetDevice(c->device);
  Dev dx, dnode, dprim, dg, dct, dcs, dgoal, dv, dfi, des;
  const int nc = a->n_constraints;
  if (!dx.put(x, sizeof(double) * N * nx) || !dnode.put(node, 4 * n) || !dprim.put(prim, 4 * n) ||
      !dg.put(a->node_g, a->node_g ? sizeof(float) * N : 0) || !dct.put(a->c_time, sizeof(float) * nc) ||
      !dcs.put(a->c_state, sizeof(double) * nc * nx) || !dgoal.put(a->goal, a->goal ? sizeof(double) * nx : 0) ||
      !dv.put(nullptr, n) || !dfi.put(nullptr, 4 * n) || !des.put(nullptr, end_state ? sizeof(double) * n * nx : 0))
    return DPG_ERR_OOM;
  TdbView tv{static_cast<const double *>(c->st64.p), static_cast<const int64_t *>(c->soff.p),
             static_cast<const int32_t *>(c->len.p), a->reverse != 0, static_cast<const float *>(dg.p), nc,
             static_cast<const float *>(dct.p), static_cast<const double *>(dcs.p),
             static_cast<const double *>(dgoal.p), a->delta};
  EnvView ev{};
  ev.dim = c->dim;
  for (int i = 0; i < 3; i++) { ev.lo[i] = c->lo[i]; ev.hi[i] = c->hi[i]; }
  ev.n_obs = c->n_obs;
  ev.obs32 = c->obs32.p;
  ev.obs64 = c->obs64.p;
  with_kind_t(kind, [&](auto K) {
    constexpr int KIND = decltype(K)::value;
    tdb_check<KIND><<<(unsigned)((n + 127) / 128), 128>>>(
        c->rp, ev, tv, static_cast<const double *>(dx.p), n, static_cast<const uint32_t *>(dnode.p),
        static_cast<const uint32_t *>(dprim.p), static_cast<uint8_t *>(dv.p), static_cast<int32_t *>(dfi.p),
        static_cast<double *>(des.p));
  });
  cudaError_t e = cudaMemcpy(verdict, dv.p, n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(first_invalid, dfi.p, 4 * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && end_state) e = cudaMemcpy(end_state, des.p, sizeof(double) * n * nx, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    c->err = std::string("tdb_check_pairs: ") + cudaGetErrorString(e);
    return DPG_ERR_CUDA;
  }
  return DPG_OK;
}
