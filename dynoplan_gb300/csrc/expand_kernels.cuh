// expand_kernels.cuh -- sm_103a kernels of the batched db-A* expansion.
//
// Pipeline for one dpg_expand (N frontier states x P primitives):
//   (node_tiles, nn_prefix, cell_scan, cell_scatter, gather_nodes: batches
//    of >= kReorderMin nodes are processed in spatial order)
//   prep_nodes      node keys / offsets, component-major FP32
//   nn_grid         ball membership through the primitives' key-space grid
//                   (batches >= 2048 nodes, one- or two-component keys), or
//   nn_mask         the same by testing every primitive: bitmask
//                   M[prim][word] + per-(node tile, prim) counts; FP64 re-test
//                   of |d - r| <= ball_band
//   nn_prefix       per-primitive exclusive prefix over node tiles
//   scan_totals     per-primitive bases in length order, work-item bases
//   nn_emit         pair lists grouped by primitive, nodes in processing order
//   check_pairs     persistent warps over (primitive, 32 nodes) work items
//                   (check_kernels.cuh); they also restore the caller's node
//                   ids of a spatially ordered batch
//
// The reference does this per node with a KD-tree radius query and a
// per-motion fcl AABB tree (include/dynoplan/dbastar/dbastar.hpp:270-312,
// src/dbastar/dbastar.cpp:391-490).  Here the pairs of one primitive share
// every per-state quantity (canonical pose, orientation, action), so a warp
// walks one primitive for 32 nodes in lockstep: pose rows are broadcast
// loads, obstacles are broadcast shared-memory reads, and only the node
// offset differs per lane.
#pragma once

#include <algorithm>
#include <cfloat>
#include <cstdint>

#include "robots.cuh"

namespace dpg {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kNNThreads = 256;   // 8 warps = 8 bitmask words = 256 nodes
constexpr int kNNTile = 256;      // primitives staged per shared-memory tile
constexpr int kCheckThreads = 256;
constexpr int kMaxCullObs = 128;   // per-lane candidate bitmask covers this many obstacles
constexpr float kGapCap = 0.05f;   // min_gap is exact up to this clearance, +inf above

constexpr int kMaxSub = 8;  // check launches per expand (item ranges)

struct DevCounters {
  unsigned long long n_pairs;
  unsigned long long n_items;
  unsigned long long next_sub[kMaxSub];  // work-queue position of each check launch
  unsigned long long n_recheck;
  unsigned long long n_ball_recheck;
  unsigned long long n_overflow;
  unsigned long long range_done[kMaxSub];  // items finished per copy range (DPG_HOST_OUT_PROGRESS)
  int status;  // 0 ok, DPG_ERR_ABORTED
  unsigned n_bad;  // dpg_check_pairs: pairs whose node or primitive index is out of range
};

template <class Real> struct __align__(sizeof(Real) * 4) Pose { Real cx, cy, c, s; };
template <class Real> struct __align__(sizeof(Real) * 4) Obs2 { Real cx, cy, hx, hy; };
template <class Real> struct Obs3 { Real cx, cy, cz, hx, hy, hz; };

// Device view of the primitive tables (one set per precision where needed).
struct PrimView {
  int P;
  int64_t S;                 // state rows
  const int32_t *len;        // [P]
  const int64_t *soff;       // [P] first state row
  const int64_t *krow;       // [P] row of the state the ball test keys on (first; last in reverse)
  const int32_t *order;      // [P] primitive ids, decreasing length
  const float *key32;        // [KEYD][P] kept key components, angles wrapped
  const float *kconst32;     // [P] constant part of the metric
  const double *st64;        // [S][NX] canonical states (row-major)
  const float *st32;         // [S][NX]
  const Pose<float> *pose32; // [PARTS][S] (3-D: cx,cy,c = position, s unused)
  const Pose<double> *pose64;
  const double *pbox;        // [P][2*POSD]: lo..., hi... of the state positions
  const float *pbox32;       // the same, rounded outward
  const int64_t *coff;       // [P] first chunk row of primitive p
  const float *cbox32;       // [sum chunks][2*POSD]: centre..., half... of the parts'
                             //   bounding box over Robot::CHUNK states (outward rounded)
  const float *tbox32;       // [P][2*POSD]: the same over the whole primitive
};

struct NodeView {
  int64_t N;
  const double *x64;   // [N][NX] raw node states
  float *key32;        // [KEYD][N]
  float *off32;        // [POSD+VELOFF][N]
};

struct EnvView {
  int dim;
  double lo[3], hi[3];
  int n_obs;
  const void *obs32;   // Obs2<float> / Obs3<float>
  const void *obs64;
};

struct PairView {
  int64_t cap;
  uint32_t *node;
  uint32_t *prim;
  uint8_t *verdict;
  int16_t *first_invalid;
  void *end_state;     // float or double rows of NX
  float *min_gap;
  uint8_t *flags;
  const uint32_t *out_index;  // when set, results of pair i go to row out_index[i]
  // when set (host arrays the GPU writes directly), the check also writes
  // each pair's caller node id and primitive there
  uint32_t *node_host, *prim_host;
};

__device__ __forceinline__ float wrap_pi_f64(double a) {
  double w = fmod(a + kPi, kTwoPi);
  if (w < 0) w += kTwoPi;
  return (float)(w - kPi);
}

// wrapped-angle distance of two angles already in [-pi, pi)
__device__ __forceinline__ float so2w(float a, float b) {
  const float d = fabsf(a - b);
  return fminf(d, (float)kTwoPi - d);
}

// --------------------------------------------------------------- prep ----

template <int KIND>
__global__ void prep_nodes(NodeView nv) {
  using R = Robot<KIND>;
  const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= nv.N) return;
  const double *x = nv.x64 + n * R::NX;
#pragma unroll
  for (int i = 0; i < R::KEYD; i++) {
    const int c = R::key_comp(i);
    const bool angle = (KIND != DPG_ROBOT_QUAD3D) && c == 2 || (KIND == DPG_ROBOT_CAR1 && c == 3);
    nv.key32[i * nv.N + n] = angle ? wrap_pi_f64(x[c]) : (float)x[c];
  }
#pragma unroll
  for (int i = 0; i < R::POSD; i++) nv.off32[i * nv.N + n] = (float)x[i];
#pragma unroll
  for (int i = 0; i < R::VELOFF; i++) nv.off32[(R::POSD + i) * nv.N + n] = (float)x[R::vel_comp(i)];
}

// ------------------------------------------------- spatial order of nodes ---
// The exact check walks 32 nodes of one primitive per warp; nodes that are
// close in space see the same obstacles and collide at similar steps, so the
// batch is processed in Z-order of a 64 x 64 (2-D) or 16^3 (3-D) cell grid
// over the environment, nodes of a cell by ascending index (deterministic).
constexpr int kOrderCells = 4096;
constexpr int64_t kReorderMin = 2048;  // smaller batches keep the caller's order

// Z-order cell of node n
template <int KIND>
__device__ __forceinline__ uint32_t cell_code(const double *x64, int64_t n, const EnvView &ev) {
  using R = Robot<KIND>;
  constexpr int bits = R::POSD == 3 ? 4 : 6;
  uint32_t code = 0;
#pragma unroll
  for (int d = 0; d < R::POSD; d++) {
    const double ext = ev.hi[d] - ev.lo[d];
    double u = ext > 0 ? (x64[n * R::NX + d] - ev.lo[d]) / ext : 0.0;
    u = u != u ? 0.0 : fmin(fmax(u, 0.0), 1.0);  // NaN / outside: clamp
    const uint32_t q = min((uint32_t)(u * (1 << bits)), (uint32_t)((1 << bits) - 1));
#pragma unroll
    for (int b = 0; b < bits; b++) code |= ((q >> b) & 1u) << (R::POSD * b + d);
  }
  return code;
}

// Stable counting sort of the nodes by cell, over tiles of `tile` consecutive
// nodes (a multiple of 256, one block each).  node_tiles gives every node its
// rank among the earlier nodes of its tile in the same cell, and writes the
// tile's count per cell (cnt[b][c], every cell); nn_prefix turns the counts
// into per-cell prefixes over the tiles and cell totals, cell_scan the totals
// into cell starts, and cell_scatter puts node n at start[c] + prefix[b][c] +
// rank.  The nodes of a cell come in ascending index whatever the thread
// schedule, in O(N) for any distribution of the nodes over the cells.
template <int KIND>
__global__ void __launch_bounds__(256) node_tiles(const double *x64, int64_t N, EnvView ev, int64_t tile,
                                                  uint32_t *cell, uint32_t *rank, uint32_t *cnt) {
  __shared__ uint32_t hist[kOrderCells];
  __shared__ uint32_t sc[256];
  for (int c = threadIdx.x; c < kOrderCells; c += 256) hist[c] = 0u;
  __syncthreads();
  const int64_t t0 = blockIdx.x * tile, t1 = min(N, t0 + tile);
  for (int64_t base = t0; base < t1; base += 256) {  // block-uniform loop over the tile's chunks
    const int64_t n = base + threadIdx.x;
    const bool live = n < t1;
    const uint32_t c = live ? cell_code<KIND>(x64, n, ev) : 0xffffffffu;
    sc[threadIdx.x] = c;
    __syncthreads();
    if (live) {
      uint32_t r = hist[c];
      for (int j = 0; j < (int)threadIdx.x; j++) r += sc[j] == c ? 1u : 0u;
      cell[n] = c;
      rank[n] = r;
    }
    __syncthreads();
    if (live) atomicAdd(&hist[c], 1u);
    __syncthreads();
  }
  uint32_t *out = cnt + (int64_t)blockIdx.x * kOrderCells;
  for (int c = threadIdx.x; c < kOrderCells; c += 256) out[c] = hist[c];
}

// single block: start = exclusive prefix of cnt over n cells
static __global__ void __launch_bounds__(1024) cell_scan(int n, const uint32_t *cnt, uint32_t *start) {
  __shared__ uint32_t part[1024];
  const int t = threadIdx.x, per = (n + 1023) / 1024;
  const int b = min(n, t * per), e = min(n, b + per);
  uint32_t sum = 0;
  for (int i = b; i < e; i++) sum += cnt[i];
  part[t] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const uint32_t v = t >= off ? part[t - off] : 0u;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  uint32_t run = part[t] - sum;
  for (int i = b; i < e; i++) {
    start[i] = run;
    run += cnt[i];
  }
}

static __global__ void cell_scatter(int64_t N, int64_t tile, const uint32_t *cell, const uint32_t *rank,
                                    const uint32_t *tile_pre, const uint32_t *start, uint32_t *perm) {
  const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= N) return;
  const uint32_t c = cell[n];
  perm[start[c] + tile_pre[(n / tile) * kOrderCells + c] + rank[n]] = (uint32_t)n;
}

// tile length of the node sort: 256 nodes, longer for huge batches so that
// the per-tile counts (tiles x kOrderCells) stay within 2048 tiles
inline int64_t order_tile(int64_t N) { return 256 * std::max<int64_t>(1, (N + 256 * 2048 - 1) / (256 * 2048)); }

template <int NX>
__global__ void gather_nodes(const double *in, const uint32_t *perm, int64_t N, double *out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= N * NX) return;
  const int64_t n = i / NX;
  out[i] = in[(int64_t)perm[n] * NX + (i - n * NX)];
}

// pair lists back to the caller's node numbering (the pairs the emit step
// wrote: none when the list overflowed the capacity)
static __global__ void unpermute_nodes(const DevCounters *ctr, int64_t cap, const uint32_t *perm, uint32_t *node) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t n = ctr->n_overflow ? 0 : min((int64_t)ctr->n_pairs, cap);
  if (i < n) node[i] = perm[node[i]];
}

// ------------------------------------------------------------ ball scan ---

template <int KIND>
__device__ __forceinline__ float key_dist32(const float4 w, const float *nk,
                                            const float *sk, int stride, float kc) {
  if constexpr (KIND == DPG_ROBOT_UNICYCLE1) {
    return kc + w.y * so2w(nk[0], sk[0]);
  } else if constexpr (KIND == DPG_ROBOT_CAR1) {
    return kc + w.y * so2w(nk[0], sk[0]) + w.z * so2w(nk[1], sk[stride]);
  } else if constexpr (KIND == DPG_ROBOT_QUAD2D) {
    return kc + w.y * so2w(nk[0], sk[0]) + w.w * fabsf(nk[1] - sk[stride]);
  } else {
    float dq = fabsf(nk[0] * sk[0] + nk[1] * sk[stride] + nk[2] * sk[2 * stride] +
                     nk[3] * sk[3 * stride]);
    dq = fminf(dq, 1.0f);
    const float a = nk[4] - sk[4 * stride], b = nk[5] - sk[5 * stride],
                c = nk[6] - sk[6 * stride];
    return kc + w.y * acosf(dq) + w.w * sqrtf(a * a + b * b + c * c);
  }
}

// Ball membership of 256 nodes (blockIdx.x) against the primitives of
// `tiles_per_y` tiles of kNNTile (blockIdx.y), so that small node batches
// still fill the GPU.
// mask[p * Wpad + w] bit l  <=>  node 32 w + l is within radius of prim p
// (primitive-major rows of Wpad >= W words; words past W are never written).
// cnt[b * P + p] = members of prim p among the block's nodes.
template <int KIND>
__global__ void __launch_bounds__(kNNThreads) nn_mask(RobotParams rp, PrimView pv, NodeView nv,
                                                      float4 w32, float radius, double radius64, float band,
                                                      int64_t Wpad, int tiles_per_y, uint32_t *mask, uint32_t *cnt,
                                                      DevCounters *ctr) {
  using R = Robot<KIND>;
  __shared__ float sk[R::KEYD * kNNTile];
  __shared__ float skc[kNNTile];
  __shared__ uint32_t scnt[kNNThreads / 32][kNNTile];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t w = (int64_t)blockIdx.x * (kNNThreads / 32) + warp;  // bitmask word
  const int64_t n = w * 32 + lane;
  const bool live = n < nv.N;
  float nk[R::KEYD];
#pragma unroll
  for (int i = 0; i < R::KEYD; i++) nk[i] = live ? nv.key32[i * nv.N + n] : 0.f;
  unsigned long long rechecks = 0;

  const int p_begin = blockIdx.y * tiles_per_y * kNNTile;
  const int p_end = min(pv.P, p_begin + tiles_per_y * kNNTile);
  for (int p0 = p_begin; p0 < p_end; p0 += kNNTile) {
    const int tp = min(kNNTile, pv.P - p0);
    __syncthreads();
    for (int t = threadIdx.x; t < tp; t += blockDim.x) {
#pragma unroll
      for (int i = 0; i < R::KEYD; i++) sk[i * kNNTile + t] = pv.key32[i * pv.P + p0 + t];
      skc[t] = pv.kconst32[p0 + t];
    }
    __syncthreads();
    for (int j0 = 0; j0 < tp; j0 += 32) {
      uint32_t mine = 0;
      const int jn = min(32, tp - j0);
      for (int jj = 0; jj < jn; jj++) {
        const int j = j0 + jj;
        bool in = false;
        if (live) {
          const float d = key_dist32<KIND>(w32, nk, &sk[j], kNNTile, skc[j]);
          in = d <= radius;
          if (fabsf(d - radius) <= band) {  // decide in FP64
            const int p = p0 + j;
            const double d64 = key_dist64<KIND>(rp, nv.x64 + n * R::NX, pv.st64 + pv.krow[p] * R::NX);
            in = d64 <= radius64;
            rechecks++;
          }
        }
        const uint32_t word = __ballot_sync(kFull, in);
        if (lane == jj) mine = word;
      }
      const int p = p0 + j0 + lane;
      if (p < pv.P && w * 32 < nv.N) mask[(int64_t)p * Wpad + w] = mine;
      scnt[warp][j0 + lane] = __popc(mine);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < tp; t += blockDim.x) {
      uint32_t s = 0;
#pragma unroll
      for (int k = 0; k < kNNThreads / 32; k++) s += scnt[k][t];
      cnt[(int64_t)blockIdx.x * pv.P + p0 + t] = s;
    }
  }
  // warp-aggregated counter update
  for (int o = 16; o > 0; o >>= 1) rechecks += __shfl_down_sync(kFull, rechecks, o);
  if (lane == 0 && rechecks) atomicAdd(&ctr->n_ball_recheck, rechecks);
}

// Key-space grid of the primitives (robots whose kept key has one or two
// components): cells over key component 0 (an angle, periodic) and
// component 1 (an angle for car1, periodic; the angular rate for quad2d,
// linear over the primitives' range), primitives listed by cell (CSR).
struct KeyGrid {
  int n0, n1;              // cells per component (n1 = 1 for one component)
  float inv0, lo1, inv1;   // cell = floor((k + pi) inv0), floor((k - lo1) inv1)
  const uint32_t *start;   // [n0 n1 + 1]
  const float4 *tab;       // [P] (key 0, key 1, constant part, primitive id bits)
};

__host__ __device__ __forceinline__ int kg_clamp(int c, int n) { return c < 0 ? 0 : (c >= n ? n - 1 : c); }

// Ball membership through the key grid: thread per node, each node tests the
// primitives of the cells within h0 / h1 (the radius plus the band over the
// component's weight, widened; negative = the whole range) of its key, with
// the same FP32 test and FP64 band decision as nn_mask, so the bitmask and
// the counts are the same.  The mask must be zero on entry; members set
// their bit with atomicOr.  cnt[b][p] is counted in shared memory when
// SCNT (P <= kGridSmemP), else by global atomics into a zeroed cnt.
constexpr int kGridSmemP = 12288;
template <int KIND, bool SCNT>
__global__ void __launch_bounds__(kNNThreads) nn_grid(RobotParams rp, PrimView pv, NodeView nv, KeyGrid kg,
                                                      float4 w32, float radius, double radius64, float band,
                                                      float h0, float h1, int64_t Wpad, uint32_t *mask, uint32_t *cnt,
                                                      DevCounters *ctr) {
  using R = Robot<KIND>;
  static_assert(R::KEYD <= 2, "key grid: one or two key components");
  constexpr bool kPer1 = KIND == DPG_ROBOT_CAR1;  // second component an angle
  constexpr float kPiF = 3.14159265f;
  extern __shared__ uint32_t scnt[];
  if (SCNT) {
    for (int t = threadIdx.x; t < pv.P; t += blockDim.x) scnt[t] = 0;
    __syncthreads();
  }
  const int lane = threadIdx.x & 31;
  const int64_t w = (int64_t)blockIdx.x * (kNNThreads / 32) + (threadIdx.x >> 5);
  const int64_t n = w * 32 + lane;
  unsigned long long rechecks = 0;
  if (n < nv.N) {
    float nk[2];
    nk[0] = nv.key32[n];
    nk[1] = R::KEYD > 1 ? nv.key32[nv.N + n] : 0.f;
    // cell ranges; a NaN key or a range of a whole period takes every cell
    // (node angles are wrapped to [-pi, pi] and h0 inv0 <= n0, so the
    // conversions stay small)
    int a0 = 0, a1 = kg.n0 - 1, b0 = 0, b1 = kg.n1 - 1;
    if (h0 >= 0.f) {
      const float f0 = floorf((nk[0] - h0 + kPiF) * kg.inv0), f1 = floorf((nk[0] + h0 + kPiF) * kg.inv0);
      if (f1 - f0 + 1.f < (float)kg.n0) { a0 = (int)f0; a1 = (int)f1; }
    }
    if (R::KEYD > 1 && h1 >= 0.f) {
      if (kPer1) {
        const float f0 = floorf((nk[1] - h1 + kPiF) * kg.inv1), f1 = floorf((nk[1] + h1 + kPiF) * kg.inv1);
        if (f1 - f0 + 1.f < (float)kg.n1) { b0 = (int)f0; b1 = (int)f1; }
      } else {
        b0 = kg_clamp((int)floorf(fmaxf((nk[1] - h1 - kg.lo1) * kg.inv1, -1.f)), kg.n1);
        b1 = kg_clamp((int)floorf(fminf((nk[1] + h1 - kg.lo1) * kg.inv1, (float)kg.n1)), kg.n1);
      }
    }
    const double *xn = nv.x64 + n * R::NX;
    const uint32_t bit = 1u << lane;
    for (int a = a0; a <= a1; a++) {
      const int ca = ((a % kg.n0) + kg.n0) % kg.n0;
      for (int b = b0; b <= b1;) {  // runs of cells contiguous in the row
        const int cb = kPer1 ? ((b % kg.n1) + kg.n1) % kg.n1 : b;
        const int last = kPer1 ? min(b1, b + (kg.n1 - 1 - cb)) : b1;
        const uint32_t s = kg.start[ca * kg.n1 + cb], e = kg.start[ca * kg.n1 + cb + (last - b) + 1];
        for (uint32_t i = s; i < e; i += 4) {  // four table loads in flight
          float4 t[4];
#pragma unroll
          for (int u = 0; u < 4; u++) t[u] = i + u < e ? kg.tab[i + u] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
          for (int u = 0; u < 4; u++) {
            if (i + u >= e) break;
            const float sk[2] = {t[u].x, t[u].y};
            const float d = key_dist32<KIND>(w32, nk, sk, 1, t[u].z);
            bool in = d <= radius;
            const int p = __float_as_int(t[u].w);
            if (fabsf(d - radius) <= band) {  // decide in FP64
              in = key_dist64<KIND>(rp, xn, pv.st64 + pv.krow[p] * R::NX) <= radius64;
              rechecks++;
            }
            if (in) {
              atomicOr(&mask[(int64_t)p * Wpad + w], bit);
              if (SCNT) atomicAdd(&scnt[p], 1u);
              else atomicAdd(&cnt[(int64_t)blockIdx.x * pv.P + p], 1u);
            }
          }
        }
        b = last + 1;
      }
    }
  }
  if (SCNT) {
    __syncthreads();
    for (int t = threadIdx.x; t < pv.P; t += blockDim.x) cnt[(int64_t)blockIdx.x * pv.P + t] = scnt[t];
  }
  for (int o = 16; o > 0; o >>= 1) rechecks += __shfl_down_sync(kFull, rechecks, o);
  if (lane == 0 && rechecks) atomicAdd(&ctr->n_ball_recheck, rechecks);
}

// per primitive: cnt[b][p] -> exclusive prefix over b; tot[p] = total.
// Block = 32 primitives (lanes) x 8 segments of the node tiles (warps).
static __global__ void __launch_bounds__(256) nn_prefix(int P, int B, uint32_t *cnt, uint32_t *tot) {
  __shared__ uint32_t part[8][32];
  const int pl = threadIdx.x & 31, sg = threadIdx.x >> 5;
  const int p = blockIdx.x * 32 + pl;
  const int per = (B + 7) / 8;
  const int b0 = min(B, sg * per), b1 = min(B, b0 + per);
  uint32_t s = 0;
  if (p < P) {
#pragma unroll 8
    for (int b = b0; b < b1; b++) s += cnt[(int64_t)b * P + p];
  }
  part[sg][pl] = s;
  __syncthreads();
  uint32_t run = 0;
  for (int k = 0; k < sg; k++) run += part[k][pl];
  if (p >= P) return;
  for (int b = b0; b < b1; b++) {
    const uint32_t c = cnt[(int64_t)b * P + p];
    cnt[(int64_t)b * P + p] = run;
    run += c;
  }
  if (sg == 7) tot[p] = run;
}

// Single block: bases of each primitive's pair segment and of its work
// items, in the order of decreasing primitive length.
static __global__ void __launch_bounds__(1024) scan_totals(int P, const int32_t *order, const uint32_t *tot,
                                                    unsigned long long *pbase,
                                                    unsigned long long *ord_pbase,
                                                    unsigned long long *ord_ibase, int64_t cap,
                                                    DevCounters *ctr) {
  __shared__ unsigned long long sp[1024], si[1024];
  const int t = threadIdx.x, T = blockDim.x;
  const int per = (P + T - 1) / T;
  const int b = t * per, e = min(P, b + per);
  unsigned long long a = 0, c = 0;
  for (int i = b; i < e; i++) {
    const uint32_t v = tot[order[i]];
    a += v;
    c += (v + 31) / 32;
  }
  sp[t] = a;
  si[t] = c;
  __syncthreads();
  for (int off = 1; off < T; off <<= 1) {  // inclusive Hillis-Steele
    unsigned long long va = 0, vc = 0;
    if (t >= off) { va = sp[t - off]; vc = si[t - off]; }
    __syncthreads();
    sp[t] += va;
    si[t] += vc;
    __syncthreads();
  }
  unsigned long long ra = sp[t] - a, rc = si[t] - c;
  for (int i = b; i < e; i++) {
    const int p = order[i];
    const uint32_t v = tot[p];
    ord_pbase[i] = ra;
    ord_ibase[i] = rc;
    pbase[p] = ra;
    ra += v;
    rc += (v + 31) / 32;
  }
  if (t == T - 1) {
    ord_pbase[P] = sp[T - 1];
    ord_ibase[P] = si[T - 1];
    ctr->n_pairs = sp[T - 1];
    const bool overflow = (int64_t)sp[T - 1] > cap;
    ctr->n_overflow = overflow ? 1 : 0;
    ctr->n_items = overflow ? 0 : si[T - 1];
    for (int i = 0; i < kMaxSub; i++) ctr->next_sub[i] = 0;
  }
}

// item_pos[item] = the order position whose work items hold it (a warp per
// position writes its run, lane by lane): the check kernel's item ->
// primitive lookup in one load instead of a binary search over ord_ibase.
// Nothing when the pairs overflowed the capacity (no items then).
static __global__ void item_positions(int P, const unsigned long long *ord_ibase, const DevCounters *ctr,
                                      uint32_t *item_pos) {
  const int i = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (i >= P || ctr->n_overflow) return;
  for (unsigned long long it = ord_ibase[i] + lane; it < ord_ibase[i + 1]; it += 32) item_pos[it] = (uint32_t)i;
}

// Pair lists from the primitive-major bitmask.  Warp per (primitive p, run of
// kEmitGroups groups of 32 mask words; a group = 4 node tiles); lane = word.
// The run's words are loaded up front (kEmitGroups loads in flight); for each
// group the warp scans the popcounts, expands the bits into node ids in
// shared memory in order, and writes the group's pairs as one contiguous run
// (coalesced stores) starting at pbase[p] + loc[first tile of the run][p].
constexpr int kEmitGroups = 8;
static __global__ void __launch_bounds__(256) nn_emit(int P, int64_t W, int64_t Wpad, const uint32_t *mask,
                                               const uint32_t *loc, const unsigned long long *pbase,
                                               int64_t cap, uint32_t *pair_node, uint32_t *pair_prim) {
  __shared__ uint32_t stage[8][32 * 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t G = Wpad / 32;                               // groups per row
  const int64_t R = (G + kEmitGroups - 1) / kEmitGroups;     // runs per row
  const int64_t gw = (int64_t)blockIdx.x * 8 + warp;
  const int64_t p = gw / R, g0 = (gw - p * R) * kEmitGroups;
  if (p >= P) return;  // warp-uniform
  uint32_t words[kEmitGroups];
#pragma unroll
  for (int k = 0; k < kEmitGroups; k++) {
    const int64_t w = (g0 + k) * 32 + lane;
    words[k] = w < W ? mask[p * Wpad + w] : 0u;
  }
  unsigned long long base = 0;
  bool have_base = false;
#pragma unroll
  for (int k = 0; k < kEmitGroups; k++) {
    const int c = __popc(words[k]);
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(kFull, incl, 31);
    if (total == 0) continue;  // warp-uniform
    if (!have_base) {  // first non-empty group: the tile prefix of the run's first tile
      base = pbase[p] + loc[(g0 * 4) * P + p];
      have_base = true;
    }
    const int64_t w = (g0 + k) * 32 + lane;
    uint32_t m = words[k];
    int j = incl - c;
    __syncwarp();
    while (m) {
      const int bit = __ffs(m) - 1;
      m &= m - 1;
      stage[warp][j++] = (uint32_t)(w * 32 + bit);
    }
    __syncwarp();
    for (int i = lane; i < total; i += 32) {
      const unsigned long long pos = base + i;
      if ((int64_t)pos < cap) {
        pair_node[pos] = stage[warp][i];
        pair_prim[pos] = (uint32_t)p;
      }
    }
    base += total;
  }
}

// --------------------------------------------------- upload-time tables ---

// Canonical FP64 rollout of every primitive from its stored start with its
// stored actions (velocity-invariant robots); one thread per primitive.
template <int KIND>
__global__ void rollout_primitives(RobotParams rp, int P, const int32_t *len, const int64_t *soff,
                                   const int64_t *aoff, const double *actions, double *st64) {
  using R = Robot<KIND>;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  double *x = st64 + soff[p] * R::NX;
  const double *u = actions + aoff[p] * R::NU;
  for (int k = 0; k + 1 < len[p]; k++) step64<KIND>(rp, x + k * R::NX, u + k * R::NU, x + (k + 1) * R::NX);
}

// Pose rows from canonical states; FP64 and the FP32 rounding of it.
template <int KIND>
__global__ void build_poses(RobotParams rp, int64_t S, const double *st64, Pose<double> *pose64,
                            Pose<float> *pose32, float *st32) {
  using R = Robot<KIND>;
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= S) return;
  const double *x = st64 + s * R::NX;
  for (int c = 0; c < R::NX; c++) st32[s * R::NX + c] = (float)x[c];
  Pose<double> ps[2];
  if constexpr (R::SPHERE) {
    ps[0] = Pose<double>{x[0], x[1], x[2], 0.0};
  } else {
    double sn, cs;
    sincos(x[2], &sn, &cs);
    ps[0] = Pose<double>{x[0], x[1], cs, sn};
    if (R::PARTS > 1) {
      double s1, c1;
      sincos(x[3], &s1, &c1);
      ps[1] = Pose<double>{x[0] - rp.hitch * c1, x[1] - rp.hitch * s1, c1, s1};
    }
  }
  for (int q = 0; q < R::PARTS; q++) {
    pose64[q * S + s] = ps[q];
    pose32[q * S + s] = Pose<float>{(float)ps[q].cx, (float)ps[q].cy, (float)ps[q].c, (float)ps[q].s};
  }
}

// Per primitive: key components (angles wrapped), constant metric part,
// swept position box of the canonical states.
template <int KIND>
// keys_only: just the key tables (soff then gives each primitive's key row,
// e.g. its last state for the reverse ball)
__global__ void build_keys(RobotParams rp, int P, const int32_t *len, const int64_t *soff,
                           const double *st64, float *key32, float *kconst32, double *pbox, float *pbox32,
                           bool keys_only = false) {
  using R = Robot<KIND>;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const double *s = st64 + soff[p] * R::NX;
#pragma unroll
  for (int i = 0; i < R::KEYD; i++) {
    const int c = R::key_comp(i);
    const bool angle = (KIND != DPG_ROBOT_QUAD3D) && c == 2 || (KIND == DPG_ROBOT_CAR1 && c == 3);
    key32[i * P + p] = angle ? wrap_pi_f64(s[c]) : (float)s[c];
  }
  double kc;
  if constexpr (R::POSD == 2) {
    kc = rp.w[0] * hypot(s[0], s[1]);
    if (R::VELOFF) kc += rp.w[2] * hypot(s[3], s[4]);
  } else {
    kc = rp.w[0] * sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]) +
         rp.w[2] * sqrt(s[7] * s[7] + s[8] * s[8] + s[9] * s[9]);
  }
  kconst32[p] = (float)kc;
  if (keys_only) return;
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int k = 0; k < len[p]; k++)
    for (int i = 0; i < R::POSD; i++) {
      lo[i] = fmin(lo[i], s[k * R::NX + i]);
      hi[i] = fmax(hi[i], s[k * R::NX + i]);
    }
  for (int i = 0; i < R::POSD; i++) {
    pbox[(int64_t)p * 2 * R::POSD + i] = lo[i];
    pbox[(int64_t)p * 2 * R::POSD + R::POSD + i] = hi[i];
    pbox32[(int64_t)p * 2 * R::POSD + i] = __double2float_rd(lo[i]);
    pbox32[(int64_t)p * 2 * R::POSD + R::POSD + i] = __double2float_ru(hi[i]);
  }
}

// Culling boxes: per chunk of Robot::CHUNK states, the bounding box of every
// collision part over those canonical states; per primitive, the union.
// FP64, then rounded outward to FP32 (centre to nearest, half extent up by
// the centre's rounding error).
template <int KIND>
__global__ void build_chunks(RobotParams rp, int P, const int32_t *len, const int64_t *soff,
                             const int64_t *coff, const Pose<double> *pose64, int64_t S,
                             float *cbox32, float *tbox32) {
  using R = Robot<KIND>;
  constexpr int D = R::POSD;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  double tlo[3] = {1e300, 1e300, 1e300}, thi[3] = {-1e300, -1e300, -1e300};
  const int L = len[p];
  for (int c = 0; c * R::CHUNK < L; c++) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int k = c * R::CHUNK; k < min(L, (c + 1) * R::CHUNK); k++) {
      for (int q = 0; q < R::PARTS; q++) {
        const Pose<double> ps = pose64[q * S + soff[p] + k];
        if constexpr (R::SPHERE) {
          const double v[3] = {ps.cx, ps.cy, ps.c};
          for (int i = 0; i < 3; i++) {
            lo[i] = fmin(lo[i], v[i] - rp.radius);
            hi[i] = fmax(hi[i], v[i] + rp.radius);
          }
        } else {
          const double ac = fabs(ps.c), as = fabs(ps.s);
          const double ex = rp.half_len * ac + rp.half_wid * as, ey = rp.half_len * as + rp.half_wid * ac;
          lo[0] = fmin(lo[0], ps.cx - ex); hi[0] = fmax(hi[0], ps.cx + ex);
          lo[1] = fmin(lo[1], ps.cy - ey); hi[1] = fmax(hi[1], ps.cy + ey);
        }
      }
    }
    float *cb = cbox32 + (coff[p] + c) * 2 * D;
    for (int i = 0; i < D; i++) {
      const double cen = 0.5 * (lo[i] + hi[i]), half = 0.5 * (hi[i] - lo[i]);
      const float c32 = (float)cen;
      cb[i] = c32;
      cb[D + i] = __double2float_ru(half + fabs(cen - (double)c32));
      tlo[i] = fmin(tlo[i], lo[i]);
      thi[i] = fmax(thi[i], hi[i]);
    }
  }
  float *tb = tbox32 + (int64_t)p * 2 * D;
  for (int i = 0; i < D; i++) {
    const double cen = 0.5 * (tlo[i] + thi[i]), half = 0.5 * (thi[i] - tlo[i]);
    const float c32 = (float)cen;
    tb[i] = c32;
    tb[D + i] = __double2float_ru(half + fabs(cen - (double)c32));
  }
}

}  // namespace dpg

namespace dpg {

// ---- explicit pair lists (dpg_check_pairs): group pairs by primitive -----
// Pairs with node >= N or prim >= P (caller-supplied device lists) are
// counted in ctr->n_bad and left out of every table; the call then fails.
static __global__ void pairs_hist(const uint32_t *node, const uint32_t *prim, int64_t n, int64_t N, int P,
                                  uint32_t *hist, DevCounters *ctr) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t p = prim[i];
  if (p >= (uint32_t)P || (int64_t)node[i] >= N) {
    atomicAdd(&ctr->n_bad, 1u);
    return;
  }
  atomicAdd(&hist[p], 1u);
}

// position of pair i inside its primitive's segment (order within a segment
// is arbitrary; results are written back at the input positions)
// sorted_idx receives the output row of each pair: dest[i] when given (the
// lazy rounds write into the rows of the whole candidate list), else i.
static __global__ void pairs_scatter(const uint32_t *node, const uint32_t *prim, int64_t n, int64_t N, int P,
                                     const unsigned long long *pbase, uint32_t *fill, uint32_t *sorted_node,
                                     uint32_t *sorted_idx, const uint32_t *dest) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t p = prim[i];
  if (p >= (uint32_t)P || (int64_t)node[i] >= N) return;  // counted by pairs_hist
  const unsigned long long pos = pbase[p] + atomicAdd(&fill[p], 1u);
  sorted_node[pos] = node[i];
  sorted_idx[pos] = dest ? dest[i] : (uint32_t)i;
}

}  // namespace dpg
