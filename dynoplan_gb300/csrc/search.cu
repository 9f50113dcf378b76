// search.cu -- db-A* over the batched GPU expansion (include/dpg_search.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <queue>
#include <random>
#include <string>
#include <vector>

#include "ctx.h"
#include "dpg_mlp.h"
#include "dpg_search.h"
#include "metric.cuh"
#include "mlp_kernels.cuh"

using namespace dpg;

namespace {

// the surrogate's cost-to-go output is in units of this many seconds
constexpr double kCtgScale = 10.0;
constexpr double kTwoPiH = 6.283185307179586476925286766559;
constexpr double kPiH = 3.1415926535897932384626433832795;

double so2(double a, double b) {
  double d = std::fabs(a - b);
  if (d >= kTwoPiH) d = std::fmod(d, kTwoPiH);  // (fmod(d, 2 pi) = d below 2 pi)
  return d > kPiH ? kTwoPiH - d : d;
}
double n3(double a, double b, double c) { return std::sqrt(a * a + b * b + c * c); }

// robot metric and time lower bound: the definitions the checker's tables use
// (weighted sum of block distances; lower_bound_time = max over blocks of
// distance / max speed)
double distance(const dpg_robot_desc &r, const double *a, const double *b) {
  const double *w = r.w;
  switch (r.kind) {
    case DPG_ROBOT_UNICYCLE1: return w[0] * std::hypot(a[0] - b[0], a[1] - b[1]) + w[1] * so2(a[2], b[2]);
    case DPG_ROBOT_CAR1:
      return w[0] * std::hypot(a[0] - b[0], a[1] - b[1]) + w[1] * so2(a[2], b[2]) + w[2] * so2(a[3], b[3]);
    case DPG_ROBOT_QUAD2D:
      return w[0] * std::hypot(a[0] - b[0], a[1] - b[1]) + w[1] * so2(a[2], b[2]) +
             w[2] * std::hypot(a[3] - b[3], a[4] - b[4]) + w[3] * std::fabs(a[5] - b[5]);
    default: {
      double dq = std::fabs(a[3] * b[3] + a[4] * b[4] + a[5] * b[5] + a[6] * b[6]);
      dq = std::min(dq, 1.0);
      return w[0] * n3(a[0] - b[0], a[1] - b[1], a[2] - b[2]) + w[1] * std::acos(dq) +
             w[2] * n3(a[7] - b[7], a[8] - b[8], a[9] - b[9]) + w[3] * n3(a[10] - b[10], a[11] - b[11], a[12] - b[12]);
    }
  }
}

double lower_bound_time(const dpg_robot_desc &r, const double *a, const double *b) {
  switch (r.kind) {
    case DPG_ROBOT_UNICYCLE1:
      return std::max(std::hypot(a[0] - b[0], a[1] - b[1]) / 0.5, so2(a[2], b[2]) / 0.5);
    case DPG_ROBOT_CAR1:
      return std::max(std::max(std::hypot(a[0] - b[0], a[1] - b[1]) / 0.5, so2(a[2], b[2]) / 0.5), so2(a[3], b[3]) / 0.5);
    case DPG_ROBOT_QUAD2D:
      return std::max(std::max(std::hypot(a[0] - b[0], a[1] - b[1]) / 2.0, so2(a[2], b[2]) / 4.0),
                      std::max(std::hypot(a[3] - b[3], a[4] - b[4]) / 4.0, std::fabs(a[5] - b[5]) / 8.0));
    default: {
      double dq = std::fabs(a[3] * b[3] + a[4] * b[4] + a[5] * b[5] + a[6] * b[6]);
      dq = std::min(dq, 1.0);
      return std::max(std::max(n3(a[0] - b[0], a[1] - b[1], a[2] - b[2]) / 4.0, std::acos(dq) / 8.0),
                      std::max(n3(a[7] - b[7], a[8] - b[8], a[9] - b[9]) / 4.0,
                               n3(a[10] - b[10], a[11] - b[11], a[12] - b[12]) / 8.0));
    }
  }
}

// the host `lower_bound_time` (max over blocks of distance / max speed)
template <int KIND>
__device__ double lbt_exact(const double *a, const double *b) {
  auto mx = [](double x, double y) { return x < y ? y : x; };  // std::max
  if constexpr (KIND == DPG_ROBOT_UNICYCLE1) {
    return mx(hypot(a[0] - b[0], a[1] - b[1]) / 0.5, so2_dist64(a[2], b[2]) / 0.5);
  } else if constexpr (KIND == DPG_ROBOT_CAR1) {
    return mx(mx(hypot(a[0] - b[0], a[1] - b[1]) / 0.5, so2_dist64(a[2], b[2]) / 0.5), so2_dist64(a[3], b[3]) / 0.5);
  } else if constexpr (KIND == DPG_ROBOT_QUAD2D) {
    return mx(mx(hypot(a[0] - b[0], a[1] - b[1]) / 2.0, so2_dist64(a[2], b[2]) / 4.0),
              mx(hypot(a[3] - b[3], a[4] - b[4]) / 4.0, fabs(a[5] - b[5]) / 8.0));
  } else {
    auto n3 = [](double x, double y, double z) {
      return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
    };
    double dq = fabs(__dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(a[3], b[3]), __dmul_rn(a[4], b[4])), __dmul_rn(a[5], b[5])),
                               __dmul_rn(a[6], b[6])));
    dq = dq < 1.0 ? dq : 1.0;
    return mx(mx(n3(a[0] - b[0], a[1] - b[1], a[2] - b[2]) / 4.0, acos(dq) / 8.0),
              mx(n3(a[7] - b[7], a[8] - b[8], a[9] - b[9]) / 4.0, n3(a[10] - b[10], a[11] - b[11], a[12] - b[12]) / 8.0));
  }
}

// the time lower bound in FP32 (the rewire filter's first test)
template <int KIND>
__device__ float lbt32(const float *a, const float *b) {
  auto so2f = [](float x, float y) {
    float d = fabsf(x - y);
    if (d >= 6.2831853071795865f) d = fmodf(d, 6.2831853071795865f);
    return d > 3.1415926535897932f ? 6.2831853071795865f - d : d;
  };
  if constexpr (KIND == DPG_ROBOT_UNICYCLE1) {
    return fmaxf(hypotf(a[0] - b[0], a[1] - b[1]) * 2.f, so2f(a[2], b[2]) * 2.f);
  } else if constexpr (KIND == DPG_ROBOT_CAR1) {
    return fmaxf(fmaxf(hypotf(a[0] - b[0], a[1] - b[1]) * 2.f, so2f(a[2], b[2]) * 2.f), so2f(a[3], b[3]) * 2.f);
  } else if constexpr (KIND == DPG_ROBOT_QUAD2D) {
    return fmaxf(fmaxf(hypotf(a[0] - b[0], a[1] - b[1]) * 0.5f, so2f(a[2], b[2]) * 0.25f),
                 fmaxf(hypotf(a[3] - b[3], a[4] - b[4]) * 0.25f, fabsf(a[5] - b[5]) * 0.125f));
  } else {
    auto l3 = [](float x, float y, float z) { return sqrtf(x * x + y * y + z * z); };
    const float dq = fminf(1.f, fabsf(a[3] * b[3] + a[4] * b[4] + a[5] * b[5] + a[6] * b[6]));
    return fmaxf(fmaxf(l3(a[0] - b[0], a[1] - b[1], a[2] - b[2]) * 0.25f, acosf(dq) * 0.125f),
                 fmaxf(l3(a[7] - b[7], a[8] - b[8], a[9] - b[9]) * 0.25f,
                       l3(a[10] - b[10], a[11] - b[11], a[12] - b[12]) * 0.125f));
  }
}

// ---- novelty radius query through a uniform grid over position ----------
// Every metric here is >= w0 * |position difference|, so a target within
// `radius` lies in the query's cell or a neighbouring one when the cell side
// is radius / w0 (slightly enlarged for rounding).  Each round the targets
// are counting-sorted by cell (count, scan, scatter, rows gathered into that
// order); a block per query scans the neighbouring cells' contiguous ranges.
// Neighbour lists are sorted on the host, so the order within a list does
// not matter.
struct Grid {
  float lo[3];
  float inv_cs;
  int n[3];
};

template <int KIND>
__device__ __forceinline__ int grid_coord(const Grid &g, const float *x, int d) {
  const int c = (int)floorf((x[d] - g.lo[d]) * g.inv_cs);
  return min(max(c, 0), g.n[d] - 1);
}

template <int KIND>
__global__ void grid_count(Grid g, const float *rows, int n, int *cell_of, int *cnt) {
  using R = Robot<KIND>;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float *x = rows + (int64_t)i * R::NX;
  int c = grid_coord<KIND>(g, x, 0) + g.n[0] * grid_coord<KIND>(g, x, 1);
  if (R::POSD == 3) c += g.n[0] * g.n[1] * grid_coord<KIND>(g, x, 2);
  cell_of[i] = c;
  atomicAdd(&cnt[c], 1);
}

// single block: start = exclusive prefix of cnt over n_cells cells
static __global__ void __launch_bounds__(1024) grid_scan(int n_cells, const int *cnt, int *start) {
  __shared__ int part[1024];
  const int t = threadIdx.x, per = (n_cells + 1023) / 1024;
  const int b = min(n_cells, t * per), e = min(n_cells, b + per);
  int sum = 0;
  for (int i = b; i < e; i++) sum += cnt[i];
  part[t] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const int v = t >= off ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int run = part[t] - sum;
  for (int i = b; i < e; i++) {
    start[i] = run;
    run += cnt[i];
  }
}

static __global__ void grid_scatter(int n, const int *cell_of, const int *start, int *fill, int *sorted) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = cell_of[i];
  sorted[start[c] + atomicAdd(&fill[c], 1)] = i;
}

// rows[sorted[j]] -> out[j]: the targets' FP32 rows in cell order
static __global__ void gather_rows(const float *rows, const int *sorted, int n, int nx, float *out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)n * nx) return;
  const int64_t j = i / nx;
  out[i] = rows[(int64_t)sorted[j] * nx + (i - j * nx)];
}

// Block of 256 threads per query over the neighbouring cells (the 3 (2-D) or
// 9 (3-D) runs of cells contiguous in the cell order; targets' FP32 rows in
// cell order, so the loads are coalesced); lower_only: targets t < q.  One
// pass: count_all[q] = every neighbour within the radius, count[q] = the kept
// ones (all of them without a filter), whose ids and time lower bounds are
// collected in shared memory and written as one run at offset[q], a range
// the block takes from the list counter *fill (the order of the runs, and
// within a run, is arbitrary: the host sorts each list by id).  A query with
// more kept neighbours than the shared buffer holds scans its cells again to
// write them; runs past `cap` are not written (the host grows the lists and
// repeats the round's queries).  Rewire filter (gsnap set): a neighbour with
// g + lbt >= the g it entered the table with is dropped (g only decreases,
// so it could never be rewired).  t_ok (lower_only queries): targets that can
// still be accepted as new nodes this round; the others are skipped (a
// successor with an explored neighbour in the radius and no goal hit is
// never accepted).
constexpr int kQueryBuf = 512;  // kept neighbours a query collects in shared memory

template <int KIND>
__global__ void __launch_bounds__(256) grid_query(RobotParams rp, float4 w32, Grid g, const double *q64,
                                                  const float *q32, int Q, const double *t64, const float *ts32,
                                                  const int *start, const int *cnt, const int *sorted, double radius,
                                                  float band, int lower_only, const unsigned char *t_ok,
                                                  const double *gq, const float *gsnap, int *count, int *count_all,
                                                  int64_t *offset, unsigned long long *fill, int64_t cap, int *ids,
                                                  double *lbt_out) {
  using R = Robot<KIND>;
  __shared__ int s_in, s_keep, s_put;
  __shared__ int64_t s_at;
  __shared__ int s_id[kQueryBuf];
  __shared__ double s_lb[kQueryBuf];
  const int q = blockIdx.x;
  if (threadIdx.x == 0) { s_in = 0; s_keep = 0; s_put = 0; }
  __syncthreads();
  float a[R::NX];
#pragma unroll
  for (int i = 0; i < R::NX; i++) a[i] = q32[(int64_t)q * R::NX + i];
  int c0[3] = {0, 0, 0};
#pragma unroll
  for (int d = 0; d < R::POSD; d++) c0[d] = grid_coord<KIND>(g, a, d);
  const float gq32 = gq ? (float)gq[q] : 0.f;
  const int zr = R::POSD == 3 ? 1 : 0;
  // the neighbours of the cells around the query: fn(t, lb) for each kept one;
  // returns this thread's count of neighbours within the radius
  auto scan = [&](auto fn) -> int {
    int my_in = 0;
    for (int dz = -zr; dz <= zr; dz++)
      for (int dy = -1; dy <= 1; dy++) {
        const int cy = c0[1] + dy, cz = c0[2] + dz;
        if (cy < 0 || cz < 0 || cy >= g.n[1] || (R::POSD == 3 && cz >= g.n[2])) continue;
        const int x0 = max(c0[0] - 1, 0), x1 = min(c0[0] + 1, g.n[0] - 1);
        const int row = g.n[0] * (cy + g.n[1] * cz);
        const int s = start[row + x0], e = start[row + x1] + cnt[row + x1];
        for (int j = s + (int)threadIdx.x; j < e; j += blockDim.x) {
          const int t = sorted[j];
          if (lower_only && (t >= q || (t_ok && !t_ok[t]))) continue;
          const float *b = ts32 + (int64_t)j * R::NX;
          float bb[R::NX];
#pragma unroll
          for (int k = 0; k < R::NX; k++) bb[k] = b[k];
          const float d = full_dist32<KIND>(w32, a, bb);
          bool in = d <= (float)radius;
          if (fabsf(d - (float)radius) <= band)
            in = full_dist64<KIND>(rp, q64 + (int64_t)q * R::NX, t64 + (int64_t)t * R::NX) <= radius;
          if (!in) continue;
          // (FP32 first: a neighbour clearly out by more than 1e-3 (1 + g) is
          // dropped; the rest are decided, and their bound kept, in FP64)
          bool keep = true, exact = lbt_out != nullptr;
          double lb = 0.0;
          if (gsnap) {
            const float gs = gsnap[t];
            if (gq32 + lbt32<KIND>(a, bb) > gs + 1e-3f * (1.f + fabsf(gs))) {
              keep = false;
              exact = false;
            } else {
              exact = true;
            }
          }
          if (exact) {
            lb = lbt_exact<KIND>(q64 + (int64_t)q * R::NX, t64 + (int64_t)t * R::NX);
            if (gsnap) keep = __dadd_rn(gq[q], lb) < (double)gsnap[t];
          }
          my_in++;
          if (keep) fn(t, lb);
        }
      }
    return my_in;
  };
  int my_in = scan([&](int t, double lb) {
    const int slot = atomicAdd(&s_keep, 1);
    if (slot < kQueryBuf) {
      s_id[slot] = t;
      s_lb[slot] = lb;
    }
  });
  for (int o = 16; o > 0; o >>= 1) my_in += __shfl_down_sync(0xffffffffu, my_in, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(&s_in, my_in);
  __syncthreads();
  const int n = s_keep;
  if (threadIdx.x == 0) {
    s_at = (int64_t)atomicAdd(fill, (unsigned long long)n);
    count[q] = n;
    if (count_all) count_all[q] = s_in;
    offset[q] = s_at;
  }
  __syncthreads();
  const int64_t at = s_at;
  if (at + n > cap) return;  // the host grows the lists and repeats the queries
  if (n <= kQueryBuf) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      ids[at + i] = s_id[i];
      if (lbt_out) lbt_out[at + i] = s_lb[i];
    }
  } else {  // more than the buffer: the same scan again, writing straight to the list
    scan([&](int t, double lb) {
      const int slot = atomicAdd(&s_put, 1);
      if (slot < n) {
        ids[at + slot] = t;
        if (lbt_out) lbt_out[at + slot] = lb;
      }
    });
  }
}

// ok[i] = successor i can be accepted as a new node: no explored neighbour in
// the radius, or it meets the goal (chosen index != -1, prep rows of width prow)
static __global__ void acceptable(int Q, const int *count_all, const double *prep, int prow, int nx,
                                  unsigned char *ok) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Q) return;
  ok[i] = (count_all[i] == 0 || prep[(int64_t)i * prow + nx] != -1.0) ? 1 : 0;
}

template <class F> void with_kind_s(int kind, F &&f) {
  switch (kind) {
    case DPG_ROBOT_UNICYCLE1: f(std::integral_constant<int, DPG_ROBOT_UNICYCLE1>{}); break;
    case DPG_ROBOT_CAR1: f(std::integral_constant<int, DPG_ROBOT_CAR1>{}); break;
    case DPG_ROBOT_QUAD3D: f(std::integral_constant<int, DPG_ROBOT_QUAD3D>{}); break;
    case DPG_ROBOT_QUAD2D: f(std::integral_constant<int, DPG_ROBOT_QUAD2D>{}); break;
  }
}

struct Node {
  float g = 0, h = 0, f = 0;  // float scores, as AStarNode (dbastar.hpp:62-64)
  int parent = -1;
  int motion = -1;
  int inter = -1;             // intermediate state index when a goal was met inside the motion
  int version = 0;
  bool in_open = false;
};

struct HeapItem {
  float f, g;
  int id, version;
};
struct NbrLbt {  // a rewire candidate and the time lower bound to it
  int id;
  double lbt;
};
struct HeapCmp {  // lowest f first, then highest g (compareAStarNode)
  bool operator()(const HeapItem &a, const HeapItem &b) const {
    if (a.f != b.f) return a.f > b.f;
    return a.g < b.g;
  }
};

// ---- successors of a round on the GPU ------------------------------------
// The host restatement's arithmetic, every product and sum rounded on its
// own (no contraction), as the host restatement computes them.
template <int KIND>
__device__ void transform_exact(const RobotParams &rp, const double *st64, int64_t s0, int k, const double *x,
                                double *o) {
  using R = Robot<KIND>;
  const double *c = st64 + (s0 + k) * R::NX;
#pragma unroll
  for (int j = 0; j < R::NX; j++) o[j] = c[j];
  const double t = __dmul_rn((double)k, rp.dt);
#pragma unroll
  for (int i = 0; i < R::POSD; i++) {
    o[i] = __dadd_rn(o[i], x[i]);
    if (R::VELOFF) {
      o[i] = __dadd_rn(o[i], __dmul_rn(t, x[R::vel_comp(i)]));
      o[R::vel_comp(i)] = __dadd_rn(o[R::vel_comp(i)], x[R::vel_comp(i)]);
    }
  }
}

// the host `distance` (weighted sum of block distances), terms rounded on their own
template <int KIND>
__device__ double distance_exact(const RobotParams &rp, const double *a, const double *b) {
  const double *w = rp.w;
  if constexpr (KIND == DPG_ROBOT_UNICYCLE1) {
    return __dadd_rn(__dmul_rn(w[0], hypot(a[0] - b[0], a[1] - b[1])), __dmul_rn(w[1], so2_dist64(a[2], b[2])));
  } else if constexpr (KIND == DPG_ROBOT_CAR1) {
    return __dadd_rn(__dadd_rn(__dmul_rn(w[0], hypot(a[0] - b[0], a[1] - b[1])), __dmul_rn(w[1], so2_dist64(a[2], b[2]))),
                     __dmul_rn(w[2], so2_dist64(a[3], b[3])));
  } else if constexpr (KIND == DPG_ROBOT_QUAD2D) {
    double d = __dadd_rn(__dmul_rn(w[0], hypot(a[0] - b[0], a[1] - b[1])), __dmul_rn(w[1], so2_dist64(a[2], b[2])));
    d = __dadd_rn(d, __dmul_rn(w[2], hypot(a[3] - b[3], a[4] - b[4])));
    return __dadd_rn(d, __dmul_rn(w[3], fabs(a[5] - b[5])));
  } else {
    auto n3 = [](double x, double y, double z) {
      return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
    };
    double dq = fabs(__dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(a[3], b[3]), __dmul_rn(a[4], b[4])), __dmul_rn(a[5], b[5])),
                               __dmul_rn(a[6], b[6])));
    dq = fmin(dq, 1.0);
    double d = __dadd_rn(__dmul_rn(w[0], n3(a[0] - b[0], a[1] - b[1], a[2] - b[2])), __dmul_rn(w[1], acos(dq)));
    d = __dadd_rn(d, __dmul_rn(w[2], n3(a[7] - b[7], a[8] - b[8], a[9] - b[9])));
    return __dadd_rn(d, __dmul_rn(w[3], n3(a[10] - b[10], a[11] - b[11], a[12] - b[12])));
  }
}

// Candidate i = (batch node cn[i], motion cp[i]): the motion's last state at
// the node, or the first of its states at floor((k + 1) / 5 L), k = 0..3,
// within goal_tol of the goal (check_goal, dbastar.cpp:492-512); the chosen
// index (-1: the last state), the duration up to it, the time lower bound from
// the node to the motion's start and from the state to the goal, and the
// candidate's g = (g of the node when popped + duration) + cost_delta_factor x
// that lower bound.  out rows [nx + 4]: state, chosen, cost, lbt from the node,
// lbt to the goal; gq[i] = g; q64 / q32 = the state.
template <int KIND>
__global__ void prepare_successors(RobotParams rp, const double *st64, const int64_t *soff, const int32_t *len,
                                   const double *bx, const float *gpop, const int *cn, const int *cp, int Q,
                                   const double *goal, double goal_tol, double cdf, double *out, double *gq,
                                   double *q64, float *q32) {
  using R = Robot<KIND>;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Q) return;
  const int p = cp[i], L = len[p];
  const int64_t s0 = soff[p];
  const double *x = bx + (int64_t)cn[i] * R::NX;
  double *row = out + (int64_t)i * (R::NX + 4);
  double xe[R::NX], xi[R::NX], x0[R::NX];
  transform_exact<KIND>(rp, st64, s0, L - 1, x, xe);
  transform_exact<KIND>(rp, st64, s0, 0, x, x0);
  int chosen = -1;
  for (int k = 0; k < 4; k++) {
    const int idx = (int)__fmul_rn(__fdiv_rn((float)(k + 1), 5.0f), (float)L);
    if (idx >= L) continue;
    transform_exact<KIND>(rp, st64, s0, idx, x, xi);
    if (distance_exact<KIND>(rp, xi, goal) <= goal_tol) {
#pragma unroll
      for (int j = 0; j < R::NX; j++) xe[j] = xi[j];
      chosen = idx;
      break;
    }
  }
#pragma unroll
  for (int j = 0; j < R::NX; j++) {
    row[j] = xe[j];
    q64[(int64_t)i * R::NX + j] = xe[j];
    q32[(int64_t)i * R::NX + j] = (float)xe[j];
  }
  const double cost = __dmul_rn((double)(chosen != -1 ? chosen : L - 1), rp.dt);
  const double lbt_par = lbt_exact<KIND>(x, x0);
  row[R::NX] = (double)chosen;
  row[R::NX + 1] = cost;
  row[R::NX + 2] = lbt_par;
  row[R::NX + 3] = lbt_exact<KIND>(xe, goal);
  gq[i] = __dadd_rn(__dadd_rn((double)gpop[cn[i]], cost), __dmul_rn(cdf, lbt_par));
}

template <class T> struct DVec {  // growable device array
  T *p = nullptr;
  size_t cap = 0;
  ~DVec() { if (p) cudaFree(p); }
  bool reserve(size_t n) {
    if (n <= cap) return true;
    size_t nc = std::max<size_t>(n, cap * 2 + 1024);
    T *q = nullptr;
    if (cudaMalloc(&q, sizeof(T) * nc) != cudaSuccess) return false;
    if (p) {
      cudaMemcpy(q, p, sizeof(T) * cap, cudaMemcpyDeviceToDevice);
      cudaFree(p);
    }
    p = q;
    cap = nc;
    return true;
  }
};

}  // namespace


extern "C" int dpg_search(dpg_ctx *c, const dpg_search_opts *o, const double *start, const double *goal,
                          dpg_mlp *mlp, dpg_search_result *res, int32_t *path_motion, double *path_state,
                          int32_t max_path) {
  if (!c || !o || !start || !goal || !res) return DPG_ERR_ARG;
  if (!c->have_prims || !c->have_env) return DPG_ERR_STATE;
  if (!(o->delta > 0) || !(o->alpha > 0 && o->alpha < 1) || o->batch < 1 || o->limit_branching_factor < 1)
    return DPG_ERR_ARG;
  if (o->heuristic == DPG_HEU_MLP && !mlp) return DPG_ERR_ARG;
  if (o->heuristic == DPG_HEU_ROADMAP && !o->roadmap) return DPG_ERR_ARG;
  std::memset(res, 0, sizeof(*res));
  const auto t_start = std::chrono::steady_clock::now();
  auto elapsed_ms = [&] {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
  };
  const dpg_robot_desc &r = c->robot;
  const int nx = r.nx, P = c->P;
  int rc = DPG_OK;
  const double goal_tol = o->delta_factor_goal * o->delta;
  const double nov_radius = (1.0 - o->alpha) * o->delta;
  std::mt19937 rng((uint32_t)o->seed);

  // explored nodes (host) + their states mirrored on the GPU for the queries
  std::vector<Node> nodes;
  std::vector<double> xs;  // [nodes][nx]
  DVec<double> t64;
  DVec<float> t32;
  auto add_node = [&](const double *x) {
    nodes.emplace_back();
    xs.insert(xs.end(), x, x + nx);
    return (int)nodes.size() - 1;
  };
  // novelty grid over position: cell side = radius / w0 (slightly enlarged),
  // at most 256 cells a side in 2-D and 40 in 3-D
  Grid grid{};
  int n_cells = 1;
  {
    const int pd = r.kind == DPG_ROBOT_QUAD3D ? 3 : 2;
    double cs = nov_radius / std::max(r.w[0], 1e-12) * (1.0 + 1e-5) + 1e-6;
    for (int d = 0; d < pd; d++) cs = std::max(cs, (c->hi[d] - c->lo[d]) / (pd == 3 ? 40.0 : 256.0));
    grid.inv_cs = (float)(1.0 / cs);
    for (int d = 0; d < 3; d++) {
      grid.lo[d] = (float)c->lo[d];
      grid.n[d] = d < pd ? std::max(1, (int)std::ceil((c->hi[d] - c->lo[d]) / cs)) : 1;
      n_cells *= grid.n[d];
    }
  }
  // cell-sorted copies of the explored nodes (t_*) and of a round's successors (s_*)
  DVec<int> tab_cnt, tab_start, tab_fill, tab_cell, tab_sorted, rnd_cnt, rnd_start, rnd_fill, rnd_cell, rnd_sorted;
  DVec<unsigned char> ok_d;
  DVec<float> tab_rows, rnd_rows;
  if (!tab_cnt.reserve(n_cells) || !tab_start.reserve(n_cells) || !tab_fill.reserve(n_cells) ||
      !rnd_cnt.reserve(n_cells) || !rnd_start.reserve(n_cells) || !rnd_fill.reserve(n_cells))
    return DPG_ERR_OOM;
  // counting sort of n rows by cell; rows_out = the FP32 rows in that order
  auto sort_by_cell = [&](const float *rows, int n, DVec<int> &cnt, DVec<int> &start, DVec<int> &fill,
                          DVec<int> &cell, DVec<int> &sorted, DVec<float> &rows_out) -> bool {
    if (!cell.reserve(std::max(n, 1)) || !sorted.reserve(std::max(n, 1)) ||
        !rows_out.reserve((size_t)std::max(n, 1) * nx))
      return false;
    cudaMemset(cnt.p, 0, sizeof(int) * n_cells);
    cudaMemset(fill.p, 0, sizeof(int) * n_cells);
    with_kind_s(r.kind, [&](auto Kd) {
      constexpr int KIND = decltype(Kd)::value;
      if (n > 0) grid_count<KIND><<<(n + 255) / 256, 256>>>(grid, rows, n, cell.p, cnt.p);
      grid_scan<<<1, 1024>>>(n_cells, cnt.p, start.p);
      if (n > 0) grid_scatter<<<(n + 255) / 256, 256>>>(n, cell.p, start.p, fill.p, sorted.p);
      if (n > 0)
        gather_rows<<<(unsigned)(((int64_t)n * nx + 255) / 256), 256>>>(rows, sorted.p, n, nx, rows_out.p);
    });
    return true;
  };
  // the table's g values as uploaded with each node: never below a node's
  // current g (g only decreases), so the rewire filter against them is exact
  DVec<float> gsnap;
  size_t uploaded = 0;
  auto sync_table = [&]() -> bool {
    const size_t n = nodes.size();
    if (!t64.reserve(n * nx) || !t32.reserve(n * nx) || !gsnap.reserve(n)) return false;
    if (n > uploaded) {
      std::vector<float> f(xs.begin() + uploaded * nx, xs.end()), gs(n - uploaded);
      for (size_t i = uploaded; i < n; i++) gs[i - uploaded] = nodes[i].g;
      cudaMemcpy(t64.p + uploaded * nx, xs.data() + uploaded * nx, sizeof(double) * (n - uploaded) * nx,
                 cudaMemcpyHostToDevice);
      cudaMemcpy(t32.p + uploaded * nx, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice);
      cudaMemcpy(gsnap.p + uploaded, gs.data(), sizeof(float) * gs.size(), cudaMemcpyHostToDevice);
      uploaded = n;
      return sort_by_cell(t32.p, (int)n, tab_cnt, tab_start, tab_fill, tab_cell, tab_sorted, tab_rows);
    }
    return true;
  };
  auto heuristic = [&](const double *x) -> float {
    if (o->heuristic == DPG_HEU_BLIND) return 0.f;
    if (o->heuristic == DPG_HEU_ROADMAP) {
      double h = 0;
      dpg_roadmap_heuristic(o->roadmap, 1, x, goal, o->connect_radius_h, &h);
      return (float)h;
    }
    return (float)lower_bound_time(r, x, goal);
  };

  std::priority_queue<HeapItem, std::vector<HeapItem>, HeapCmp> open;
  const int s0 = add_node(start);
  nodes[s0].g = 0;
  nodes[s0].h = heuristic(start);
  nodes[s0].f = nodes[s0].g + nodes[s0].h;
  nodes[s0].in_open = true;
  open.push({nodes[s0].f, nodes[s0].g, s0, 0});

  // per-iteration device buffers
  DVec<double> q64, b64, prep, goal_d, gq, lbt_tab, lbt_self;
  DVec<float> gpop_d;
  DVec<int> cand, cnt_all;
  std::vector<int> cnp;
  std::vector<double> prep_h;
  if (!goal_d.reserve(nx)) return DPG_ERR_OOM;
  cudaMemcpy(goal_d.p, goal, sizeof(double) * nx, cudaMemcpyHostToDevice);
  DVec<float> q32;
  DVec<int> cnt_tab, ids_tab, cnt_self, ids_self;
  DVec<int64_t> off_tab, off_self;
  DVec<unsigned long long> list_fill;  // the two lists' counters
  DVec<uint32_t> pnode, pprim;
  DVec<float> mlp_out;
  DVec<__nv_bfloat16> feat;
  std::vector<uint32_t> h_node, h_prim;
  std::vector<uint8_t> h_verdict;
  std::vector<int16_t> h_fi;
  int solution = -1;
  int status = DPG_SEARCH_EMPTY_QUEUE;
  const float4 w32 = make_float4((float)r.w[0], (float)r.w[1], (float)r.w[2], (float)r.w[3]);

  while (true) {
    if (res->expands >= o->max_expands) { status = DPG_SEARCH_MAX_EXPANDS; break; }
    if (elapsed_ms() > o->time_limit_ms) { status = DPG_SEARCH_MAX_TIME; break; }
    if (open.empty()) { status = DPG_SEARCH_EMPTY_QUEUE; break; }
    // pop up to `batch` nodes
    std::vector<int> batch;
    while (!open.empty() && (int)batch.size() < o->batch &&
           res->expands + (int64_t)batch.size() < o->max_expands) {
      const HeapItem it = open.top();
      open.pop();
      Node &n = nodes[it.id];
      if (!n.in_open || it.version != n.version) continue;  // stale entry
      n.in_open = false;
      batch.push_back(it.id);
    }
    if (batch.empty()) continue;
    bool solved = false;
    for (int id : batch) {
      res->expands++;
      if (distance(r, &xs[(size_t)id * nx], goal) < goal_tol) {  // dbastar.cpp:790-800
        solution = id;
        solved = true;
        break;
      }
    }
    if (solved) { status = DPG_SEARCH_SOLVED; break; }

    // expand the batch: every in-ball pair, exact-checked
    const int B = (int)batch.size();
    std::vector<double> bx((size_t)B * nx);
    for (int i = 0; i < B; i++) std::memcpy(&bx[(size_t)i * nx], &xs[(size_t)batch[i] * nx], sizeof(double) * nx);
    int64_t cap = std::max<int64_t>(1024, (int64_t)B * P);  // every pair of the batch
    dpg_expand_out eo{};
    dpg_expand_opts eopt{};
    eopt.radius = o->alpha * o->delta;
    eopt.precision = o->precision;
    eopt.contact_band = 1e-4;
    eopt.ball_band = 1e-5;
    const double te0 = elapsed_ms();
    for (;;) {
      h_node.resize(cap); h_prim.resize(cap); h_verdict.resize(cap); h_fi.resize(cap);
      eo = dpg_expand_out{};
      eo.capacity = cap;
      eo.node = h_node.data(); eo.prim = h_prim.data(); eo.verdict = h_verdict.data(); eo.first_invalid = h_fi.data();
      rc = dpg_expand(c, &eopt, B, bx.data(), &eo);
      if (rc == DPG_ERR_CAPACITY) { cap = eo.n_pairs; continue; }
      break;
    }
    if (rc) return rc;
    res->expand_ms += elapsed_ms() - te0;
    res->checked_pairs += eo.n_pairs;

    // valid motions per batch node, in expand_lazy's order
    std::vector<std::vector<int>> per_node(B);
    for (int64_t i = 0; i < eo.n_pairs; i++)
      if (h_verdict[i] == DPG_VALID) per_node[h_node[i]].push_back((int)h_prim[i]);
    for (int b = 0; b < B; b++) {
      std::sort(per_node[b].begin(), per_node[b].end());
      if (o->shuffle) std::shuffle(per_node[b].begin(), per_node[b].end(), rng);
    }
    // the batch's states and g when popped on the device (successor
    // preparation, features); a successor's g counts from its node's g at
    // pop time
    std::vector<float> gpop(B);
    for (int b = 0; b < B; b++) gpop[b] = nodes[batch[b]].g;
    if (!b64.reserve((size_t)B * nx) || !gpop_d.reserve(B)) return DPG_ERR_OOM;
    cudaMemcpy(b64.p, bx.data(), sizeof(double) * bx.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(gpop_d.p, gpop.data(), sizeof(float) * B, cudaMemcpyHostToDevice);
    if (o->heuristic == DPG_HEU_MLP) {  // node features of the batch, goal-conditioned
      const double tm0 = elapsed_ms();
      if (!feat.reserve((size_t)B * kMlpNodeFeat)) return DPG_ERR_OOM;
      if ((rc = dpg_mlp_node_features(c, b64.p, B, goal, feat.p))) return rc;
      res->mlp_ms += elapsed_ms() - tm0;
    }

    // Rounds of (prepare, query, insert/rewire): in each round every
    // unfinished node, in pop order, visits its next chunk of motions (2 x the
    // limit, doubling per round) until it has `limit` new nodes.  With one
    // node per batch this is the reference's visiting order.
    const int limit = o->limit_branching_factor;
    std::vector<size_t> pos(B, 0), chunk(B, (size_t)2 * limit);
    std::vector<int> n_new(B, 0);
    std::vector<char> finished(B, 0);
    for (int b = 0; b < B; b++) finished[b] = per_node[b].empty();
    std::vector<int> first(B + 1, 0), c_node, c_prim, c_chosen;
    std::vector<NbrLbt> nbl;
    std::vector<double> c_x, c_cost, c_lbtpar, c_hlbt;
    while (std::find(finished.begin(), finished.end(), 0) != finished.end()) {
      // successors of the round: end state (or the state meeting the goal),
      // transformed motion start, cost
      const double tp0 = elapsed_ms();
      c_node.clear(); c_prim.clear();
      for (int b = 0; b < B; b++) {
        first[b] = (int)c_prim.size();
        if (finished[b]) continue;
        const size_t e = std::min(per_node[b].size(), pos[b] + chunk[b]);
        for (size_t j = pos[b]; j < e; j++) {
          c_node.push_back(b);
          c_prim.push_back(per_node[b][j]);
        }
      }
      first[B] = (int)c_prim.size();
      const int Q = (int)c_prim.size();
      if (Q == 0) {
        res->prepare_ms += elapsed_ms() - tp0;
        break;
      }
      // on the GPU: every candidate's end (or goal) state, start state,
      // goal-check index and cost; the states stay there as the query rows
      const size_t prow = (size_t)nx + 4;
      if (!q64.reserve((size_t)Q * nx) || !q32.reserve((size_t)Q * nx) || !cand.reserve(2 * (size_t)Q) ||
          !prep.reserve((size_t)Q * prow) || !gq.reserve(Q))
        return DPG_ERR_OOM;
      cnp.resize(2 * (size_t)Q);
      std::copy(c_node.begin(), c_node.end(), cnp.begin());
      std::copy(c_prim.begin(), c_prim.end(), cnp.begin() + Q);
      cudaMemcpy(cand.p, cnp.data(), sizeof(int) * cnp.size(), cudaMemcpyHostToDevice);
      with_kind_s(r.kind, [&](auto Kd) {
        constexpr int KIND = decltype(Kd)::value;
        prepare_successors<KIND><<<(Q + 127) / 128, 128>>>(
            c->rp, static_cast<const double *>(c->st64.p), static_cast<const int64_t *>(c->soff.p),
            static_cast<const int32_t *>(c->len.p), b64.p, gpop_d.p, cand.p, cand.p + Q, Q, goal_d.p, goal_tol,
            o->cost_delta_factor, prep.p, gq.p, q64.p, q32.p);
      });
      prep_h.resize((size_t)Q * prow);
      if (cudaMemcpy(prep_h.data(), prep.p, sizeof(double) * prep_h.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
        return DPG_ERR_CUDA;
      c_x.resize((size_t)Q * nx);
      c_chosen.resize(Q);
      c_cost.resize(Q);
      c_lbtpar.resize(Q);
      c_hlbt.resize(Q);
      for (int q = 0; q < Q; q++) {
        const double *row = &prep_h[(size_t)q * prow];
        std::memcpy(&c_x[(size_t)q * nx], row, sizeof(double) * nx);
        c_chosen[q] = (int)row[nx];
        c_cost[q] = row[nx + 1];
        c_lbtpar[q] = row[nx + 2];
        c_hlbt[q] = row[nx + 3];
      }
      res->prepare_ms += elapsed_ms() - tp0;

      // novelty: successors vs explored nodes, and vs earlier successors of
      // the round; the id capacity grows until every list is complete
      const double tn0 = elapsed_ms();
      res->rounds++;
      const double tt0 = elapsed_ms();
      if (!sync_table() || !cnt_tab.reserve(Q) || !cnt_self.reserve(Q) || !cnt_all.reserve(Q)) return DPG_ERR_OOM;
      res->table_ms += elapsed_ms() - tt0;
      // the round's successors sorted by cell too, for the lower-index query
      if (!sort_by_cell(q32.p, Q, rnd_cnt, rnd_start, rnd_fill, rnd_cell, rnd_sorted, rnd_rows) ||
          !ok_d.reserve(Q))
        return DPG_ERR_OOM;
      // one pass per query set: the explored neighbours that pass the rewire
      // filter (all of them are counted for the novelty test) and every
      // earlier successor of the round within the radius, each with its time
      // lower bound, in packed lists (a run per query, offsets from the device)
      std::vector<int> ct(Q), ca(Q), cs(Q), it, is;
      std::vector<double> lt, ls;
      std::vector<int64_t> ot(Q), os(Q);
      unsigned long long nts[2] = {0, 0};
      if (!off_tab.reserve(Q) || !off_self.reserve(Q) || !list_fill.reserve(2)) return DPG_ERR_OOM;
      auto query = [&]() {  // a block per query
        cudaMemsetAsync(list_fill.p, 0, sizeof(unsigned long long) * 2);
        with_kind_s(r.kind, [&](auto Kd) {
          constexpr int KIND = decltype(Kd)::value;
          grid_query<KIND><<<(unsigned)Q, 256>>>(c->rp, w32, grid, q64.p, q32.p, Q, t64.p, tab_rows.p, tab_start.p,
                                                 tab_cnt.p, tab_sorted.p, nov_radius, 1e-5f, 0, nullptr, gq.p,
                                                 gsnap.p, cnt_tab.p, cnt_all.p, off_tab.p, list_fill.p,
                                                 (int64_t)std::min(ids_tab.cap, lbt_tab.cap), ids_tab.p, lbt_tab.p);
          // which successors can be accepted follows from the explored-table counts
          acceptable<<<(Q + 255) / 256, 256>>>(Q, cnt_all.p, prep.p, (int)prow, nx, ok_d.p);
          grid_query<KIND><<<(unsigned)Q, 256>>>(c->rp, w32, grid, q64.p, q32.p, Q, q64.p, rnd_rows.p, rnd_start.p,
                                                 rnd_cnt.p, rnd_sorted.p, nov_radius, 1e-5f, 1, ok_d.p, nullptr,
                                                 nullptr, cnt_self.p, nullptr, off_self.p, list_fill.p + 1,
                                                 (int64_t)std::min(ids_self.cap, lbt_self.cap), ids_self.p,
                                                 lbt_self.p);
        });
        return cudaMemcpy(nts, list_fill.p, sizeof(nts), cudaMemcpyDeviceToHost) == cudaSuccess;
      };
      const double tq0 = elapsed_ms();
      if (!ids_tab.reserve(1024) || !lbt_tab.reserve(1024) || !ids_self.reserve(1024) || !lbt_self.reserve(1024) ||
          !query())
        return DPG_ERR_CUDA;
      if (nts[0] > std::min(ids_tab.cap, lbt_tab.cap) || nts[1] > std::min(ids_self.cap, lbt_self.cap)) {
        // lists past the capacity: grow them, query again
        if (!ids_tab.reserve(nts[0]) || !lbt_tab.reserve(nts[0]) || !ids_self.reserve(nts[1]) ||
            !lbt_self.reserve(nts[1]) || !query())
          return DPG_ERR_OOM;
      }
      const int64_t nt = (int64_t)nts[0], ns = (int64_t)nts[1];
      cudaMemcpy(ct.data(), cnt_tab.p, sizeof(int) * Q, cudaMemcpyDeviceToHost);
      cudaMemcpy(ca.data(), cnt_all.p, sizeof(int) * Q, cudaMemcpyDeviceToHost);
      cudaMemcpy(cs.data(), cnt_self.p, sizeof(int) * Q, cudaMemcpyDeviceToHost);
      cudaMemcpy(ot.data(), off_tab.p, sizeof(int64_t) * Q, cudaMemcpyDeviceToHost);
      cudaMemcpy(os.data(), off_self.p, sizeof(int64_t) * Q, cudaMemcpyDeviceToHost);
      it.resize((size_t)nt);
      is.resize((size_t)ns);
      lt.resize((size_t)nt);
      ls.resize((size_t)ns);
      if (nt) {
        cudaMemcpy(it.data(), ids_tab.p, sizeof(int) * nt, cudaMemcpyDeviceToHost);
        cudaMemcpy(lt.data(), lbt_tab.p, sizeof(double) * nt, cudaMemcpyDeviceToHost);
      }
      if (ns) {
        cudaMemcpy(is.data(), ids_self.p, sizeof(int) * ns, cudaMemcpyDeviceToHost);
        cudaMemcpy(ls.data(), lbt_self.p, sizeof(double) * ns, cudaMemcpyDeviceToHost);
      }
      if (cudaGetLastError() != cudaSuccess) return DPG_ERR_CUDA;
      res->query_ms += elapsed_ms() - tq0;
      res->novelty_ms += elapsed_ms() - tn0;

      // learned heuristic: the surrogate's cost-to-go of every (node, motion)
      // successor, never below the time lower bound
      std::vector<float> pred;
      std::vector<double> hroad;  // the roadmap heuristic of every successor of the round
      if (o->heuristic == DPG_HEU_ROADMAP) {
        hroad.resize(Q);
        if ((rc = dpg_roadmap_heuristic(o->roadmap, Q, c_x.data(), goal, o->connect_radius_h, hroad.data())))
          return rc;
      }
      if (o->heuristic == DPG_HEU_MLP) {
        const double tm0 = elapsed_ms();
        if (!pnode.reserve(Q) || !pprim.reserve(Q) || !mlp_out.reserve((size_t)Q * 2)) return DPG_ERR_OOM;
        cudaMemcpy(pnode.p, c_node.data(), sizeof(uint32_t) * Q, cudaMemcpyHostToDevice);
        cudaMemcpy(pprim.p, c_prim.data(), sizeof(uint32_t) * Q, cudaMemcpyHostToDevice);
        if ((rc = dpg_mlp_forward(mlp, feat.p, pnode.p, pprim.p, Q, mlp_out.p))) return rc;
        pred.resize((size_t)Q * 2);
        cudaMemcpy(pred.data(), mlp_out.p, sizeof(float) * Q * 2, cudaMemcpyDeviceToHost);
        res->mlp_ms += elapsed_ms() - tm0;
      }

      // insert or rewire, in pop order and the motions' order (dbastar.cpp:809-919)
      const double ti0 = elapsed_ms();
      std::vector<int> accepted_as(Q, -1);  // node id of an accepted successor
      for (int b = 0; b < B; b++) {
        if (finished[b]) continue;
        const int parent = batch[b];
        for (int ci = first[b]; ci < first[b + 1]; ci++) {
          pos[b]++;
          const double *cx = &c_x[(size_t)ci * nx];
          double h = (o->heuristic == DPG_HEU_BLIND) ? 0.0 : c_hlbt[ci];
          if (o->heuristic == DPG_HEU_ROADMAP) h = hroad[ci];
          if (o->heuristic == DPG_HEU_MLP) h = std::max(h, kCtgScale * std::max(0.0, (double)pred[2 * (size_t)ci + 1]));
          const double g = (double)gpop[b] + c_cost[ci] + o->cost_delta_factor * c_lbtpar[ci];
          // rewire candidates: the filtered explored neighbours and the
          // accepted earlier successors, by node id, with their lower bounds
          nbl.clear();
          for (int k = 0; k < ct[ci]; k++) nbl.push_back({it[ot[ci] + k], lt[ot[ci] + k]});
          bool self_nbr = false;
          for (int k = 0; k < cs[ci]; k++) {
            const int other = is[os[ci] + k];
            if (accepted_as[other] >= 0) {
              nbl.push_back({accepted_as[other], ls[os[ci] + k]});
              self_nbr = true;
            }
          }
          std::sort(nbl.begin(), nbl.end(), [](const NbrLbt &x, const NbrLbt &y) { return x.id < y.id; });
          if ((ca[ci] == 0 && !self_nbr) || c_chosen[ci] != -1) {
            const int id = add_node(cx);
            Node &n = nodes[id];
            n.g = (float)g;
            n.h = (float)h;
            n.f = n.g + n.h;
            n.parent = parent;
            n.motion = c_prim[ci];
            n.inter = c_chosen[ci];
            n.in_open = true;
            open.push({n.f, n.g, id, n.version});
            accepted_as[ci] = id;
            n_new[b]++;
          } else {
            for (const NbrLbt &e : nbl) {
              Node &n = nodes[e.id];
              const double tentative = g + e.lbt;
              if (tentative < n.g) {
                n.g = (float)tentative;
                n.f = n.g + n.h;
                n.parent = parent;
                n.motion = c_prim[ci];
                n.inter = -1;
                n.version++;
                n.in_open = true;
                open.push({n.f, n.g, e.id, n.version});
              }
            }
          }
          if (n_new[b] >= limit) break;
        }
        if (n_new[b] >= limit || pos[b] >= per_node[b].size()) finished[b] = 1;
        else chunk[b] *= 2;  // chunk used up below the limit: a larger one next round
      }
      res->insert_ms += elapsed_ms() - ti0;
    }
  }
  res->status = status;
  res->nodes = (int64_t)nodes.size();
  res->time_ms = elapsed_ms();
  if (solution >= 0) {
    res->solved = 1;
    res->g = nodes[solution].g;
    std::vector<int> chain;
    for (int id = solution; id != -1; id = nodes[id].parent) chain.push_back(id);
    std::reverse(chain.begin(), chain.end());
    res->path_len = (int32_t)chain.size() - 1;
    double cost = 0;
    for (size_t i = 1; i < chain.size(); i++) {
      const Node &n = nodes[chain[i]];
      const int L = c->h_len[n.motion];
      cost += (n.inter != -1 ? n.inter : L - 1) * r.dt;
    }
    res->cost = cost;
    for (int i = 0; i < res->path_len && i < max_path; i++) {
      if (path_motion) path_motion[i] = nodes[chain[i + 1]].motion;
    }
    if (path_state)
      for (int i = 0; i <= res->path_len && i <= max_path; i++)
        std::memcpy(path_state + (size_t)i * nx, &xs[(size_t)chain[i] * nx], sizeof(double) * nx);
  }
  (void)mlp;
  (void)P;
  return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}
