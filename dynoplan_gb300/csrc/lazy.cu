// lazy.cu -- lazy batched exact check (dpg_lazy_check, include/dpg.h).
//
// The reference checks a node's neighbours lazily: Expander::expand_lazy
// returns the in-ball motions in shuffled order (include/dynoplan/dbastar/
// dbastar.hpp:270-312) and the search loop exact-checks them one by one,
// stopping once limit_branching_factor motions were taken
// (src/dbastar/dbastar.cpp:809-919, cap at :916-918).  Here a whole batch of
// nodes runs that loop at once:
//
//   lz_hist, lz_scan, lz_scatter   candidates grouped by node (CSR)
//   lz_sort                        each node's candidates ranked by
//                                  (score, primitive index), a bitonic sort
//                                  in shared memory, one block per node
//   rounds of
//     lz_select                    every node short of `limit` valid motions
//                                  takes its next ceil((limit - valid) * f)
//                                  ranked candidates
//     lz_tile_count, nn_prefix,    the round's list grouped by primitive
//     scan_totals, lz_tile_scatter (longest first) with the nodes in the
//                                  spatial order of dpg_expand (tiles of 256
//                                  Z-ordered nodes), so the lockstep warps
//                                  see neighbouring nodes as in a full expand
//     exact check of the list      the persistent lockstep warps of
//                                  check_kernels.cuh, results written to the
//                                  candidates' own rows
//     lz_update                    walks the new results in rank order and
//                                  marks the first `limit` valid candidates
//                                  of each node DPG_FLAG_ACCEPTED
//
// f starts at 1.25 for scored candidates (a surrogate ranks likely-valid
// motions first) and 2.5 in motion order, then follows the measured yield
// of the previous round (checked / valid, x1.15, clamped to [1, 16]).  What a
// node accepts depends only on its ranking and the exact verdicts: the first
// `limit` valid candidates in rank order, or all of its valid ones.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>

#include "check_list.h"

using namespace dpg;

namespace {

struct LazyCounters {
  unsigned long long checked;   // pairs checked this round (lz_update)
  unsigned long long valid;     // valid verdicts among them
  unsigned long long accepted;  // accepted in total
  unsigned long long active;    // nodes still short of `limit` with candidates left
  unsigned int max_seg;
  unsigned int n_bad;
};

template <class T> T *P_(DevBuf &b) { return static_cast<T *>(b.p); }

// order-preserving map of a float to u32 (NaN last)
__device__ __forceinline__ uint32_t ord_score(float f) {
  if (f != f) return 0xffffffffu;
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void lz_hist(const uint32_t *node, const uint32_t *prim, int64_t n, int64_t N, int P, uint32_t *cnt,
                        LazyCounters *ctr) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t v = node[i];
  if ((int64_t)v >= N || prim[i] >= (uint32_t)P) {
    atomicAdd(&ctr->n_bad, 1u);
    return;
  }
  atomicAdd(&cnt[v], 1u);
}

// exclusive scan of cnt[0..N) into off[0..N]; the largest count into ctr
__global__ void __launch_bounds__(1024) lz_scan(const uint32_t *cnt, int64_t N, uint32_t *off, LazyCounters *ctr) {
  __shared__ unsigned long long part[1024];
  const int t = threadIdx.x, T = blockDim.x;
  const int64_t per = (N + T - 1) / T, b = t * per, e = min(N, b + per);
  unsigned long long a = 0;
  uint32_t mx = 0;
  for (int64_t i = b; i < e; i++) {
    a += cnt[i];
    mx = max(mx, cnt[i]);
  }
  part[t] = a;
  __syncthreads();
  for (int d = 1; d < T; d <<= 1) {  // inclusive Hillis-Steele over the thread sums
    const unsigned long long v = t >= d ? part[t - d] : 0ull;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  unsigned long long run = part[t] - a;
  for (int64_t i = b; i < e; i++) {
    off[i] = (uint32_t)run;
    run += cnt[i];
  }
  if (t == T - 1) off[N] = (uint32_t)part[T - 1];
  atomicMax(&ctr->max_seg, mx);
}

__global__ void lz_scatter(const uint32_t *node, const uint32_t *prim, int64_t n, int64_t N, int P,
                           const uint32_t *off, uint32_t *fill, uint32_t *rank) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t v = node[i];
  if ((int64_t)v >= N || prim[i] >= (uint32_t)P) return;
  rank[off[v] + atomicAdd(&fill[v], 1u)] = (uint32_t)i;
}

// One block per node (grid-stride): the node's candidates sorted by
// (score, primitive) ascending with a bitonic network over the next power
// of two; `cap` (a power of two) entries of shared memory.
constexpr int kSortThreads = 256;
__global__ void __launch_bounds__(kSortThreads) lz_sort(const uint32_t *off, uint32_t *rank, const uint32_t *prim,
                                                        const float *score, int stride, int64_t N) {
  extern __shared__ unsigned long long sk[];  // S keys, then S values (S <= the launch's power of two)
  for (int64_t v = blockIdx.x; v < N; v += gridDim.x) {
    const uint32_t b = off[v], m = off[v + 1] - b;
    if (m <= 1) continue;  // block-uniform
    uint32_t S = 1;
    while (S < m) S <<= 1;
    uint32_t *sv = reinterpret_cast<uint32_t *>(sk + S);
    for (uint32_t i = threadIdx.x; i < S; i += kSortThreads) {
      if (i < m) {
        const uint32_t idx = rank[b + i];
        const uint32_t hi = score ? ord_score(score[(int64_t)idx * stride]) : 0u;
        sk[i] = ((unsigned long long)hi << 32) | prim[idx];
        sv[i] = idx;
      } else {
        sk[i] = ~0ull;
        sv[i] = 0u;
      }
    }
    __syncthreads();
    for (uint32_t k = 2; k <= S; k <<= 1) {
      for (uint32_t j = k >> 1; j > 0; j >>= 1) {
        for (uint32_t i = threadIdx.x; i < S; i += kSortThreads) {
          const uint32_t l = i ^ j;
          if (l > i) {
            const unsigned long long a = sk[i], c = sk[l];
            const bool asc = (i & k) == 0;
            if ((a > c) == asc) {
              sk[i] = c;
              sk[l] = a;
              const uint32_t t = sv[i];
              sv[i] = sv[l];
              sv[l] = t;
            }
          }
        }
        __syncthreads();
      }
    }
    for (uint32_t i = threadIdx.x; i < m; i += kSortThreads) rank[b + i] = sv[i];
    __syncthreads();
  }
}

// nodes short of `limit` valid motions take their next ranked candidates:
// ranks [cur, next)
__global__ void lz_select(int64_t N, const uint32_t *off, const uint32_t *cur, uint32_t *next, const uint32_t *valid,
                          int limit, float f) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= N) return;
  const uint32_t seg = off[v + 1] - off[v], c = cur[v];
  if ((int)valid[v] >= limit || c >= seg) {
    next[v] = c;
    return;
  }
  const uint32_t want = (uint32_t)ceilf((float)(limit - (int)valid[v]) * f);
  next[v] = c + min(seg - c, max(want, 1u));
}

// Tiles of 256 nodes in processing order (perm: position -> node, or the
// identity): per tile, how many of the round's candidates each primitive
// has (table[tile][P]).
__global__ void __launch_bounds__(256) lz_tile_count(int64_t N, const uint32_t *perm, const uint32_t *off,
                                                     const uint32_t *rank, const uint32_t *cur, const uint32_t *next,
                                                     const uint32_t *prim, int P, uint32_t *table) {
  extern __shared__ uint32_t hist[];
  for (int i = threadIdx.x; i < P; i += blockDim.x) hist[i] = 0u;
  __syncthreads();
  const int64_t pos = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (pos < N) {
    const uint32_t v = perm ? perm[pos] : (uint32_t)pos, b = off[v];
    for (uint32_t r = cur[v]; r < next[v]; r++) atomicAdd(&hist[prim[rank[b + r]]], 1u);
  }
  __syncthreads();
  uint32_t *t = table + (int64_t)blockIdx.x * P;
  for (int i = threadIdx.x; i < P; i += blockDim.x) t[i] = hist[i];
}

// the round's list: entry at pbase[p] + (tile prefix) + (rank in the tile);
// within a tile the order is arbitrary (the nodes of a tile are neighbours)
__global__ void __launch_bounds__(256) lz_tile_scatter(int64_t N, const uint32_t *perm, const uint32_t *off,
                                                       const uint32_t *rank, const uint32_t *cur,
                                                       const uint32_t *next, const uint32_t *prim, int P,
                                                       const uint32_t *table, const unsigned long long *pbase,
                                                       uint32_t *l_node, uint32_t *l_dest) {
  extern __shared__ uint32_t hist[];
  for (int i = threadIdx.x; i < P; i += blockDim.x) hist[i] = 0u;
  __syncthreads();
  const int64_t pos = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (pos < N) {
    const uint32_t v = perm ? perm[pos] : (uint32_t)pos, b = off[v];
    const uint32_t *t = table + (int64_t)blockIdx.x * P;
    for (uint32_t r = cur[v]; r < next[v]; r++) {
      const uint32_t idx = rank[b + r], p = prim[idx];
      const unsigned long long slot = pbase[p] + t[p] + atomicAdd(&hist[p], 1u);
      l_node[slot] = v;
      l_dest[slot] = idx;
    }
  }
}

// the first `limit` valid candidates in rank order are accepted
__global__ void lz_update(int64_t N, const uint32_t *off, const uint32_t *rank, uint32_t *cur, const uint32_t *next,
                          uint32_t *valid, int limit, const uint8_t *verdict, uint8_t *flags, LazyCounters *ctr) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= N) return;
  const uint32_t b = off[v], seg = off[v + 1] - b, c0 = cur[v], c1 = next[v];
  uint32_t ok = valid[v], nval = 0, nacc = 0;
  for (uint32_t r = c0; r < c1; r++) {
    const uint32_t idx = rank[b + r];
    if (verdict[idx] == DPG_VALID) {
      nval++;
      if ((int)ok < limit) {
        flags[idx] |= DPG_FLAG_ACCEPTED;
        ok++;
        nacc++;
      }
    }
  }
  valid[v] = ok;
  cur[v] = c1;
  if (c1 > c0) {
    atomicAdd(&ctr->checked, (unsigned long long)(c1 - c0));
    if (nval) atomicAdd(&ctr->valid, (unsigned long long)nval);
    if (nacc) atomicAdd(&ctr->accepted, (unsigned long long)nacc);
  }
  if ((int)ok < limit && c1 < seg) atomicAdd(&ctr->active, 1ull);
}

}  // namespace

extern "C" int dpg_lazy_check(dpg_ctx *c, const dpg_expand_opts *opts, int64_t N, const double *x_dev, int64_t n,
                              const uint32_t *node_dev, const uint32_t *prim_dev, const float *score_dev,
                              int32_t score_stride, int32_t limit, dpg_expand_out *out, dpg_lazy_stats *stats) {
  if (!c || !opts || !out) return DPG_ERR_ARG;
  if (!c->have_prims || !c->have_env) return ctx_fail(c, DPG_ERR_STATE, "lazy_check: upload primitives and env first");
  if (N < 0 || n < 0 || (N > 0 && !x_dev) || (n > 0 && (!node_dev || !prim_dev)))
    return ctx_fail(c, DPG_ERR_ARG, "lazy_check: bad arrays");
  if (n > (int64_t)0xfffffffeLL || N > (int64_t)1 << 31) return ctx_fail(c, DPG_ERR_ARG, "lazy_check: too many pairs");
  if (limit < 1) return ctx_fail(c, DPG_ERR_ARG, "lazy_check: limit < 1");
  if (score_dev && score_stride < 1) return ctx_fail(c, DPG_ERR_ARG, "lazy_check: score_stride < 1");
  if (!out->verdict || !out->flags) return ctx_fail(c, DPG_ERR_ARG, "lazy_check: verdict and flags are required");
  if (out->capacity < n) {
    out->n_pairs = n;
    return ctx_fail(c, DPG_ERR_CAPACITY, "lazy_check: capacity below n");
  }
  const int prec = opts->precision;
  if (prec != DPG_FP32 && prec != DPG_FP64 && prec != DPG_FP64_STRICT)
    return ctx_fail(c, DPG_ERR_ARG, "lazy_check: precision");
  if (*(volatile int *)c->h_abort) return ctx_fail(c, DPG_ERR_ABORTED, "lazy_check: abort flag raised");
  if (cudaSetDevice(c->device) != cudaSuccess) return ctx_fail(c, DPG_ERR_CUDA, "lazy_check: cudaSetDevice");
  dpg_lazy_stats st_out{};
  out->n_pairs = n;
  out->n_scanned = 0;
  out->n_contact_recheck = 0;
  out->n_ball_recheck = 0;
  if (stats) *stats = st_out;
  if (n == 0 || N == 0) return DPG_OK;

  const int kind = c->robot.kind, P = c->P;
  const int kd = kind == DPG_ROBOT_QUAD3D ? 7 : (kind == DPG_ROBOT_UNICYCLE1 ? 1 : 2);
  const int od = kind == DPG_ROBOT_QUAD3D ? 6 : (kind == DPG_ROBOT_QUAD2D ? 4 : 2);
  cudaStream_t st = c->stream;
  int rc;
  const size_t nz = (size_t)n, Nz = (size_t)N;
  if ((rc = ctx_ensure(c, c->nkey32, sizeof(float) * kd * Nz)) || (rc = ctx_ensure(c, c->noff32, sizeof(float) * od * Nz)) ||
      (rc = ctx_ensure(c, c->lz_off, 4 * (Nz + 1))) || (rc = ctx_ensure(c, c->lz_cnt, 4 * Nz)) ||
      (rc = ctx_ensure(c, c->lz_cur, 4 * Nz)) || (rc = ctx_ensure(c, c->lz_next, 4 * Nz)) ||
      (rc = ctx_ensure(c, c->lz_valid, 4 * Nz)) || (rc = ctx_ensure(c, c->lz_rank, 4 * nz)) ||
      (rc = ctx_ensure(c, c->lz_lnode, 4 * nz)) ||
      (rc = ctx_ensure(c, c->lz_ldest, 4 * nz)) || (rc = ctx_ensure(c, c->lz_ctr, sizeof(LazyCounters))))
    return rc;
  if (!c->h_lz) {
    if (cudaHostAlloc(&c->h_lz, sizeof(LazyCounters), cudaHostAllocDefault) != cudaSuccess)
      return ctx_fail(c, DPG_ERR_OOM, "lazy_check: cudaHostAlloc");
  }
  LazyCounters *d_lz = P_<LazyCounters>(c->lz_ctr), *h_lz = static_cast<LazyCounters *>(c->h_lz);
  uint32_t *off = P_<uint32_t>(c->lz_off), *cnt = P_<uint32_t>(c->lz_cnt), *cur = P_<uint32_t>(c->lz_cur),
           *nxt = P_<uint32_t>(c->lz_next), *valid = P_<uint32_t>(c->lz_valid), *rank = P_<uint32_t>(c->lz_rank);
  auto sync_counters = [&]() -> int {
    if (cudaMemcpyAsync(h_lz, d_lz, sizeof(LazyCounters), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return ctx_fail(c, DPG_ERR_CUDA, std::string("lazy_check: ") + cudaGetErrorString(cudaGetLastError()));
    return DPG_OK;
  };

  // outputs start unchecked, flags clear
  if (cudaMemsetAsync(out->verdict, DPG_UNCHECKED, nz, st) != cudaSuccess ||
      cudaMemsetAsync(out->flags, 0, nz, st) != cudaSuccess || cudaMemsetAsync(d_lz, 0, sizeof(LazyCounters), st) ||
      cudaMemsetAsync(cnt, 0, 4 * Nz, st) || cudaMemsetAsync(cur, 0, 4 * Nz, st) ||
      cudaMemsetAsync(valid, 0, 4 * Nz, st))
    return ctx_fail(c, DPG_ERR_CUDA, "lazy_check: memset");
  NodeView nv{N, x_dev, P_<float>(c->nkey32), P_<float>(c->noff32)};
  ctx_prep_nodes(c, nv, st);
  // candidates by node, ranked
  const unsigned gn = (unsigned)((n + 255) / 256), gN = (unsigned)((N + 255) / 256);
  lz_hist<<<gn, 256, 0, st>>>(node_dev, prim_dev, n, N, P, cnt, d_lz);
  lz_scan<<<1, 1024, 0, st>>>(cnt, N, off, d_lz);
  cudaMemsetAsync(cnt, 0, 4 * Nz, st);
  lz_scatter<<<gn, 256, 0, st>>>(node_dev, prim_dev, n, N, P, off, cnt, rank);
  if ((rc = sync_counters())) return rc;
  if (h_lz->n_bad)
    return ctx_fail(c, DPG_ERR_ARG, "lazy_check: " + std::to_string(h_lz->n_bad) + " pairs have node >= N or prim >= P");
  const uint32_t max_seg = h_lz->max_seg;
  uint32_t S = 1;
  while (S < max_seg) S <<= 1;
  const size_t smem = (size_t)S * 12;
  if (smem > 200 * 1024)
    return ctx_fail(c, DPG_ERR_CAPACITY, "lazy_check: a node has " + std::to_string(max_seg) +
                                             " candidates (at most 16384 are ranked)");
  if (max_seg > 1) {
    cudaFuncSetAttribute(lz_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(smem, 1024));
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lz_sort, kSortThreads, smem);
    const int64_t grid = std::min<int64_t>(N, (int64_t)c->sm_count * std::max(per_sm, 1) * 8);
    lz_sort<<<(unsigned)grid, kSortThreads, smem, st>>>(off, rank, prim_dev, score_dev, score_stride, N);
  }
  PairView po{};
  po.verdict = out->verdict;
  po.first_invalid = out->first_invalid;
  po.end_state = out->end_state;
  po.min_gap = out->min_gap;
  po.flags = out->flags;
  const CheckArgs ca = ctx_check_args(c, prec, opts->contact_band, nv, po);
  // processing order of the nodes and the per-tile primitive table
  const uint32_t *perm = nullptr;
  if ((rc = ctx_spatial_order(c, x_dev, N, st, &perm))) return rc;
  const int64_t tiles = (N + 255) / 256;
  const size_t hsm = sizeof(uint32_t) * (size_t)P;
  if (hsm > 200 * 1024) return ctx_fail(c, DPG_ERR_ARG, "lazy_check: more than 51200 primitives");
  if ((rc = ctx_ensure(c, c->lz_table, sizeof(uint32_t) * (size_t)P * tiles)) ||
      (rc = ctx_ensure(c, c->tot, sizeof(uint32_t) * P)) || (rc = ctx_ensure(c, c->pbase, 8 * (size_t)P)) ||
      (rc = ctx_ensure(c, c->ord_pbase, 8 * ((size_t)P + 1))) || (rc = ctx_ensure(c, c->ord_ibase, 8 * ((size_t)P + 1))))
    return rc;
  cudaFuncSetAttribute(lz_tile_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hsm);
  cudaFuncSetAttribute(lz_tile_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hsm);
  uint32_t *table = P_<uint32_t>(c->lz_table), *tot = P_<uint32_t>(c->tot);
  unsigned long long *pbase = P_<unsigned long long>(c->pbase);
  float f = score_dev ? 1.25f : 2.5f;
  int rounds = 0;
  long long n_checked = 0, n_valid = 0, n_recheck = 0;
  for (;;) {
    cudaMemsetAsync(d_lz, 0, sizeof(LazyCounters), st);
    cudaMemsetAsync(c->d_ctr, 0, sizeof(DevCounters), st);
    lz_select<<<gN, 256, 0, st>>>(N, off, cur, nxt, valid, limit, f);
    lz_tile_count<<<(unsigned)tiles, 256, hsm, st>>>(N, perm, off, rank, cur, nxt, prim_dev, P, table);
    nn_prefix<<<(unsigned)((P + 31) / 32), 256, 0, st>>>(P, (int)tiles, table, tot);
    scan_totals<<<1, 1024, 0, st>>>(P, P_<int32_t>(c->order), tot, pbase, P_<unsigned long long>(c->ord_pbase),
                                    P_<unsigned long long>(c->ord_ibase), n, c->d_ctr);
    lz_tile_scatter<<<(unsigned)tiles, 256, hsm, st>>>(N, perm, off, rank, cur, nxt, prim_dev, P, table, pbase,
                                                        P_<uint32_t>(c->lz_lnode), P_<uint32_t>(c->lz_ldest));
    if ((rc = ctx_check_grouped(c, prec, ca, P_<uint32_t>(c->lz_lnode), P_<uint32_t>(c->lz_ldest), st))) return rc;
    lz_update<<<gN, 256, 0, st>>>(N, off, rank, cur, nxt, valid, limit, out->verdict, out->flags, d_lz);
    if (cudaMemcpyAsync(c->h_ctr, c->d_ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return ctx_fail(c, DPG_ERR_CUDA, "lazy_check: counters");
    if ((rc = sync_counters())) return rc;
    rounds++;
    n_checked += (long long)h_lz->checked;
    n_valid += (long long)h_lz->valid;
    n_recheck += (long long)c->h_ctr->n_recheck;
    st_out.n_accepted += (int64_t)h_lz->accepted;
    if (c->h_ctr->status == DPG_ERR_ABORTED) return ctx_fail(c, DPG_ERR_ABORTED, "lazy_check: aborted");
    if (h_lz->active == 0 || h_lz->checked == 0) break;
    // next round: as many candidates as the last round's yield suggests
    const double yield = (double)h_lz->valid / (double)h_lz->checked;
    f = (float)std::clamp(yield > 0 ? 1.15 / yield : 16.0, 1.0, 16.0);
  }
  st_out.n_checked = n_checked;
  st_out.n_valid = n_valid;
  st_out.rounds = rounds;
  st_out.max_candidates = (int32_t)max_seg;
  out->n_contact_recheck = n_recheck;
  if (stats) *stats = st_out;
  return DPG_OK;
}
