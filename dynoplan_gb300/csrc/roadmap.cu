// roadmap.cu -- the roadmap heuristic (include/dpg_roadmap.h): GPU edge
// checks and heuristic queries, host Dijkstra.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <queue>
#include <string>
#include <vector>

#include "ctx.h"
#include "dpg_roadmap.h"
#include "metric.cuh"
#include "state_check.cuh"

using namespace dpg;

namespace {

// shortest signed angle from a to b, in [-pi, pi)
__device__ __forceinline__ double dangle(double a, double b) {
  double d = fmod(b - a + kPi, kTwoPi);
  if (d < 0) d += kTwoPi;
  return d - kPi;
}

// point at t in [0, 1] of the straight interpolation from a to b
template <int KIND>
__device__ void interp64(const double *a, const double *b, double t, double *out) {
  using R = Robot<KIND>;
#pragma unroll
  for (int i = 0; i < R::NX; i++) out[i] = a[i] + t * (b[i] - a[i]);
  if constexpr (KIND == DPG_ROBOT_QUAD3D) {
    double bq[4], dot = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) dot += a[3 + i] * b[3 + i];
    const double sg = dot < 0 ? -1.0 : 1.0;
#pragma unroll
    for (int i = 0; i < 4; i++) bq[i] = sg * b[3 + i];
    dot = fabs(dot);
    double wa = 1.0 - t, wb = t;
    if (dot < 0.9995) {
      const double th = acos(dot), s = sin(th);
      wa = sin((1.0 - t) * th) / s;
      wb = sin(t * th) / s;
    }
    double n = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      out[3 + i] = wa * a[3 + i] + wb * bq[i];
      n += out[3 + i] * out[3 + i];
    }
    n = sqrt(n);
#pragma unroll
    for (int i = 0; i < 4; i++) out[3 + i] /= n;
  } else {
    out[2] = a[2] + t * dangle(a[2], b[2]);
    if (KIND == DPG_ROBOT_CAR1) out[3] = a[3] + t * dangle(a[3], b[3]);
  }
}

template <int KIND>
__device__ double lbt64(const double *a, const double *b) {
  return fmax(lbt_pr64<KIND>(a, b), lbt_vel64<KIND>(a, b));
}

// 16 x 16 threads per block over (j, i); thread (i, j), i < j: one candidate edge
template <int KIND>
__global__ void roadmap_edges(RobotParams rp, EnvView ev, const double *xs, int S, double radius, double res,
                              int64_t cap, unsigned long long *count, int2 *ij, double *w) {
  using R = Robot<KIND>;
  const int i = blockIdx.y * 16 + threadIdx.y, j = blockIdx.x * 16 + threadIdx.x;
  if (i >= j || j >= S) return;
  const double *a = xs + (int64_t)i * R::NX, *b = xs + (int64_t)j * R::NX;
  const double d = full_dist64<KIND>(rp, a, b);
  if (!(d < radius)) return;
  int depth = 0;  // bisection depth: segments of d / 2^depth <= res
  for (double seg = d; seg > res && depth < 20; seg *= 0.5) depth++;
  const int n = 1 << depth;
  double x[R::NX];
  for (int k = 0; k <= n; k++) {
    interp64<KIND>(a, b, (double)k / (double)n, x);
    if (!state_free64<KIND>(rp, ev, x)) return;
  }
  const unsigned long long slot = atomicAdd(count, 1ull);
  if ((int64_t)slot < cap) {
    ij[slot] = make_int2(i, j);
    w[slot] = lbt64<KIND>(a, b);
  }
}

// thread per query: the roadmap heuristic of state x
template <int KIND>
__global__ void roadmap_h(RobotParams rp, const double *xs, const double *dist, int S, const double *q, int64_t N,
                          const double *goal, double connect, double *h) {
  using R = Robot<KIND>;
  const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= N) return;
  const double *x = q + n * R::NX;
  double x0[R::NX];
#pragma unroll
  for (int i = 0; i < R::NX; i++) x0[i] = x[i];
#pragma unroll
  for (int i = 0; i < R::VELOFF; i++) x0[R::vel_comp(i)] = 0.0;
  if (KIND == DPG_ROBOT_QUAD2D) x0[5] = 0.0;
  if (KIND == DPG_ROBOT_QUAD3D) x0[10] = x0[11] = x0[12] = 0.0;
  double best = 1e8;
  for (int s = 0; s < S; s++) {
    const double *p = xs + (int64_t)s * R::NX;
    if (full_dist64<KIND>(rp, p, x0) <= connect) best = fmin(best, dist[s] + lbt_pr64<KIND>(p, x0));
  }
  h[n] = fmax(lbt_vel64<KIND>(x, goal), best);
}

template <int KIND>
__global__ void states_valid(RobotParams rp, EnvView ev, const double *x, int64_t N, uint8_t *valid) {
  using R = Robot<KIND>;
  const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n < N) valid[n] = state_free64<KIND>(rp, ev, x + n * R::NX) ? 1 : 0;
}

template <class F> void with_kind_r(int kind, F &&f) {
  switch (kind) {
    case DPG_ROBOT_UNICYCLE1: f(std::integral_constant<int, DPG_ROBOT_UNICYCLE1>{}); break;
    case DPG_ROBOT_CAR1: f(std::integral_constant<int, DPG_ROBOT_CAR1>{}); break;
    case DPG_ROBOT_QUAD3D: f(std::integral_constant<int, DPG_ROBOT_QUAD3D>{}); break;
    case DPG_ROBOT_QUAD2D: f(std::integral_constant<int, DPG_ROBOT_QUAD2D>{}); break;
  }
}

EnvView env_view(const dpg_ctx *c) {
  EnvView ev{};
  ev.dim = c->dim;
  for (int i = 0; i < 3; i++) { ev.lo[i] = c->lo[i]; ev.hi[i] = c->hi[i]; }
  ev.n_obs = c->n_obs;
  ev.obs32 = c->obs32.p;
  ev.obs64 = c->obs64.p;
  return ev;
}

}  // namespace

struct dpg_roadmap {
  int device = 0, kind = 0, nx = 0, S = 0;
  RobotParams rp{};
  std::vector<double> samples, dist;
  std::vector<int32_t> parent;
  std::vector<int2> edges;
  std::vector<double> w;
  double *d_samples = nullptr, *d_dist = nullptr;
};

extern "C" {

void dpg_roadmap_destroy(dpg_roadmap *rm) {
  if (!rm) return;
  cudaSetDevice(rm->device);
  cudaFree(rm->d_samples);
  cudaFree(rm->d_dist);
  delete rm;
}

int dpg_roadmap_build(dpg_ctx *c, int32_t S, const double *samples, double connection_radius, double resolution,
                      dpg_roadmap **out) {
  if (!c || !out || S < 1 || !samples || !(connection_radius > 0) || !(resolution > 0)) return DPG_ERR_ARG;
  if (!c->have_env) return DPG_ERR_STATE;
  *out = nullptr;
  cudaSetDevice(c->device);
  const int nx = c->robot.nx;
  auto *rm = new dpg_roadmap();
  rm->device = c->device;
  rm->kind = c->robot.kind;
  rm->nx = nx;
  rm->S = S;
  rm->rp = c->rp;
  rm->samples.assign(samples, samples + (size_t)S * nx);
  auto fail_rm = [&](int code) {
    dpg_roadmap_destroy(rm);
    return code;
  };
  if (cudaMalloc(&rm->d_samples, sizeof(double) * S * nx) != cudaSuccess ||
      cudaMalloc(&rm->d_dist, sizeof(double) * S) != cudaSuccess)
    return fail_rm(DPG_ERR_OOM);
  cudaMemcpy(rm->d_samples, samples, sizeof(double) * S * nx, cudaMemcpyHostToDevice);
  // edges, with the capacity grown to the count when a first pass overflows
  const EnvView ev = env_view(c);
  int64_t cap = std::min<int64_t>((int64_t)S * (S - 1) / 2, (int64_t)1 << 20);
  unsigned long long *d_count = nullptr;
  int2 *d_ij = nullptr;
  double *d_w = nullptr;
  unsigned long long n_edges = 0;
  if (cudaMalloc(&d_count, sizeof(unsigned long long)) != cudaSuccess) return fail_rm(DPG_ERR_OOM);
  for (int pass = 0; pass < 2; pass++) {
    cudaFree(d_ij);
    cudaFree(d_w);
    d_ij = nullptr;
    d_w = nullptr;
    if (cap > 0 && (cudaMalloc(&d_ij, sizeof(int2) * cap) != cudaSuccess ||
                    cudaMalloc(&d_w, sizeof(double) * cap) != cudaSuccess)) {
      cudaFree(d_count);
      return fail_rm(DPG_ERR_OOM);
    }
    cudaMemset(d_count, 0, sizeof(unsigned long long));
    const dim3 grid((unsigned)((S + 15) / 16), (unsigned)((S + 15) / 16)), block(16, 16);
    with_kind_r(rm->kind, [&](auto K) {
      constexpr int KIND = decltype(K)::value;
      roadmap_edges<KIND><<<grid, block>>>(rm->rp, ev, rm->d_samples, S, connection_radius, resolution, cap,
                                           d_count, d_ij, d_w);
    });
    if (cudaMemcpy(&n_edges, d_count, sizeof(n_edges), cudaMemcpyDeviceToHost) != cudaSuccess) {
      cudaFree(d_count);
      return fail_rm(DPG_ERR_CUDA);
    }
    if ((int64_t)n_edges <= cap) break;
    cap = (int64_t)n_edges;
  }
  rm->edges.resize(n_edges);
  rm->w.resize(n_edges);
  if (n_edges) {
    cudaMemcpy(rm->edges.data(), d_ij, sizeof(int2) * n_edges, cudaMemcpyDeviceToHost);
    cudaMemcpy(rm->w.data(), d_w, sizeof(double) * n_edges, cudaMemcpyDeviceToHost);
  }
  cudaFree(d_count);
  cudaFree(d_ij);
  cudaFree(d_w);
  if (cudaGetLastError() != cudaSuccess) return fail_rm(DPG_ERR_CUDA);
  // deterministic edge order
  std::vector<size_t> order(n_edges);
  for (size_t k = 0; k < n_edges; k++) order[k] = k;
  std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
    return rm->edges[a].x != rm->edges[b].x ? rm->edges[a].x < rm->edges[b].x : rm->edges[a].y < rm->edges[b].y;
  });
  std::vector<int2> e2(n_edges);
  std::vector<double> w2(n_edges);
  for (size_t k = 0; k < n_edges; k++) {
    e2[k] = rm->edges[order[k]];
    w2[k] = rm->w[order[k]];
  }
  rm->edges.swap(e2);
  rm->w.swap(w2);
  // Dijkstra from the goal (the last sample) over the undirected graph
  std::vector<std::vector<std::pair<int, double>>> adj(S);
  for (size_t k = 0; k < n_edges; k++) {
    adj[rm->edges[k].x].push_back({rm->edges[k].y, rm->w[k]});
    adj[rm->edges[k].y].push_back({rm->edges[k].x, rm->w[k]});
  }
  rm->dist.assign(S, DBL_MAX);
  rm->parent.resize(S);
  for (int s = 0; s < S; s++) rm->parent[s] = s;
  using QI = std::pair<double, int>;
  std::priority_queue<QI, std::vector<QI>, std::greater<QI>> pq;
  rm->dist[S - 1] = 0.0;
  pq.push({0.0, S - 1});
  while (!pq.empty()) {
    const auto [d, u] = pq.top();
    pq.pop();
    if (d > rm->dist[u]) continue;
    for (const auto &[v, wv] : adj[u])
      if (d + wv < rm->dist[v]) {
        rm->dist[v] = d + wv;
        rm->parent[v] = u;
        pq.push({rm->dist[v], v});
      }
  }
  cudaMemcpy(rm->d_dist, rm->dist.data(), sizeof(double) * S, cudaMemcpyHostToDevice);
  *out = rm;
  return DPG_OK;
}

int dpg_roadmap_edges(const dpg_roadmap *rm, int64_t *n_edges, int32_t *ij, double *w, int64_t cap) {
  if (!rm || !n_edges) return DPG_ERR_ARG;
  const int64_t n = (int64_t)rm->edges.size();
  *n_edges = n;
  if ((ij || w) && cap < n) return DPG_ERR_CAPACITY;
  for (int64_t k = 0; k < n && (ij || w); k++) {
    if (ij) {
      ij[2 * k] = rm->edges[k].x;
      ij[2 * k + 1] = rm->edges[k].y;
    }
    if (w) w[k] = rm->w[k];
  }
  return DPG_OK;
}

int dpg_roadmap_distances(const dpg_roadmap *rm, double *dist, int32_t *parent) {
  if (!rm) return DPG_ERR_ARG;
  if (dist) std::memcpy(dist, rm->dist.data(), sizeof(double) * rm->S);
  if (parent) std::memcpy(parent, rm->parent.data(), sizeof(int32_t) * rm->S);
  return DPG_OK;
}

int dpg_roadmap_heuristic(const dpg_roadmap *rm, int64_t N, const double *x, const double *goal,
                          double connect_radius, double *h) {
  if (!rm || N < 0 || (N > 0 && (!x || !h)) || !goal) return DPG_ERR_ARG;
  if (N == 0) return DPG_OK;
  cudaSetDevice(rm->device);
  const int nx = rm->nx;
  double *d_x = nullptr, *d_goal = nullptr, *d_h = nullptr;
  if (cudaMalloc(&d_x, sizeof(double) * N * nx) != cudaSuccess || cudaMalloc(&d_goal, sizeof(double) * nx) != cudaSuccess ||
      cudaMalloc(&d_h, sizeof(double) * N) != cudaSuccess) {
    cudaFree(d_x);
    cudaFree(d_goal);
    return DPG_ERR_OOM;
  }
  cudaMemcpy(d_x, x, sizeof(double) * N * nx, cudaMemcpyHostToDevice);
  cudaMemcpy(d_goal, goal, sizeof(double) * nx, cudaMemcpyHostToDevice);
  with_kind_r(rm->kind, [&](auto K) {
    constexpr int KIND = decltype(K)::value;
    roadmap_h<KIND><<<(unsigned)((N + 127) / 128), 128>>>(rm->rp, rm->d_samples, rm->d_dist, rm->S, d_x, N, d_goal,
                                                          connect_radius, d_h);
  });
  const cudaError_t e = cudaMemcpy(h, d_h, sizeof(double) * N, cudaMemcpyDeviceToHost);
  cudaFree(d_x);
  cudaFree(d_goal);
  cudaFree(d_h);
  return e == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

int dpg_states_valid(dpg_ctx *c, int64_t N, const double *x, uint8_t *valid) {
  if (!c || N < 0 || (N > 0 && (!x || !valid))) return DPG_ERR_ARG;
  if (!c->have_env) return DPG_ERR_STATE;
  if (N == 0) return DPG_OK;
  cudaSetDevice(c->device);
  const int nx = c->robot.nx;
  double *d_x = nullptr;
  uint8_t *d_v = nullptr;
  if (cudaMalloc(&d_x, sizeof(double) * N * nx) != cudaSuccess || cudaMalloc(&d_v, N) != cudaSuccess) {
    cudaFree(d_x);
    return DPG_ERR_OOM;
  }
  cudaMemcpy(d_x, x, sizeof(double) * N * nx, cudaMemcpyHostToDevice);
  const EnvView ev = env_view(c);
  with_kind_r(c->robot.kind, [&](auto K) {
    constexpr int KIND = decltype(K)::value;
    states_valid<KIND><<<(unsigned)((N + 255) / 256), 256>>>(c->rp, ev, d_x, N, d_v);
  });
  const cudaError_t e = cudaMemcpy(valid, d_v, N, cudaMemcpyDeviceToHost);
  cudaFree(d_x);
  cudaFree(d_v);
  return e == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

}  // extern "C"
