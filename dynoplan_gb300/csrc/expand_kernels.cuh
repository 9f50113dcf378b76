// expand_kernels.cuh -- sm_103a kernels of the batched db-A* expansion.
//
// Pipeline for one dpg_expand (N frontier states x P primitives):
//   prep_nodes      node keys / offsets, component-major FP32
//   nn_mask         ball membership bitmask M[word][prim] + per-(node tile,
//                   prim) counts; FP64 re-test of |d - r| <= ball_band
//   nn_prefix       per-primitive exclusive prefix over node tiles
//   scan_totals     per-primitive bases in length order, work-item bases
//   nn_emit         pair lists grouped by primitive, nodes ascending
//   check_pairs     persistent warps over (primitive, 32 nodes) work items
//   recheck_pairs   FP64 re-check of pairs flagged near contact or bounds
//
// The reference does this per node with a KD-tree radius query and a
// per-motion fcl AABB tree (include/dynoplan/dbastar/dbastar.hpp:270-312,
// src/dbastar/dbastar.cpp:391-490).  Here the pairs of one primitive share
// every per-state quantity (canonical pose, orientation, action), so a warp
// walks one primitive for 32 nodes in lockstep: pose rows are broadcast
// loads, obstacles are broadcast shared-memory reads, and only the node
// offset differs per lane.
#pragma once

#include <cfloat>
#include <cstdint>

#include "robots.cuh"

namespace dpg {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kNNThreads = 256;   // 8 warps = 8 bitmask words = 256 nodes
constexpr int kNNTile = 256;      // primitives staged per shared-memory tile
constexpr int kCheckThreads = 256;

struct DevCounters {
  unsigned long long n_pairs;
  unsigned long long n_items;
  unsigned long long next_item;
  unsigned long long n_recheck;
  unsigned long long n_ball_recheck;
  unsigned long long n_overflow;
  int status;  // 0 ok, DPG_ERR_ABORTED
  int pad;
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
  const int32_t *order;      // [P] primitive ids, decreasing length
  const float *key32;        // [KEYD][P] kept key components, angles wrapped
  const float *kconst32;     // [P] constant part of the metric
  const double *st64;        // [S][NX] canonical states (row-major)
  const float *st32;         // [S][NX]
  const Pose<float> *pose32; // [PARTS][S] (3-D: cx,cy,c = position, s unused)
  const Pose<double> *pose64;
  const double *pbox;        // [P][2*POSD]: lo..., hi...
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
  uint32_t *recheck;   // pair indices flagged for the FP64 re-check
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

// ------------------------------------------------------------ ball scan ---

template <int KIND>
__device__ __forceinline__ float key_dist32(const RobotParams &rp, const float *nk,
                                            const float *sk, int stride, float kc) {
  if constexpr (KIND == DPG_ROBOT_UNICYCLE1) {
    return kc + (float)rp.w[1] * so2w(nk[0], sk[0]);
  } else if constexpr (KIND == DPG_ROBOT_CAR1) {
    return kc + (float)rp.w[1] * so2w(nk[0], sk[0]) + (float)rp.w[2] * so2w(nk[1], sk[stride]);
  } else if constexpr (KIND == DPG_ROBOT_QUAD2D) {
    return kc + (float)rp.w[1] * so2w(nk[0], sk[0]) + (float)rp.w[3] * fabsf(nk[1] - sk[stride]);
  } else {
    float dq = fabsf(nk[0] * sk[0] + nk[1] * sk[stride] + nk[2] * sk[2 * stride] +
                     nk[3] * sk[3 * stride]);
    dq = fminf(dq, 1.0f);
    const float a = nk[4] - sk[4 * stride], b = nk[5] - sk[5 * stride],
                c = nk[6] - sk[6 * stride];
    return kc + (float)rp.w[1] * acosf(dq) + (float)rp.w[3] * sqrtf(a * a + b * b + c * c);
  }
}

// Ball membership of 256 nodes (one block) against all primitives.
// mask[w * Ppad + p] bit l  <=>  node 32 w + l is within radius of prim p.
// cnt[b * P + p] = members of prim p among the block's nodes.
template <int KIND>
__global__ void __launch_bounds__(kNNThreads) nn_mask(RobotParams rp, PrimView pv, NodeView nv,
                                                      float radius, double radius64, float band, int Ppad,
                                                      uint32_t *mask, uint32_t *cnt,
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

  for (int p0 = 0; p0 < pv.P; p0 += kNNTile) {
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
          const float d = key_dist32<KIND>(rp, nk, &sk[j], kNNTile, skc[j]);
          in = d <= radius;
          if (fabsf(d - radius) <= band) {  // decide in FP64
            const int p = p0 + j;
            const double d64 = key_dist64<KIND>(rp, nv.x64 + n * R::NX, pv.st64 + pv.soff[p] * R::NX);
            in = d64 <= radius64;
            rechecks++;
          }
        }
        const uint32_t word = __ballot_sync(kFull, in);
        if (lane == jj) mine = word;
      }
      const int p = p0 + j0 + lane;
      if (p < Ppad && w * 32 < nv.N) mask[w * (int64_t)Ppad + p] = mine;
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

// per primitive: cnt[b][p] -> exclusive prefix over b; tot[p] = total
__global__ void nn_prefix(int P, int B, uint32_t *cnt, uint32_t *tot) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  uint32_t run = 0;
  for (int b = 0; b < B; b++) {
    const uint32_t c = cnt[(int64_t)b * P + p];
    cnt[(int64_t)b * P + p] = run;
    run += c;
  }
  tot[p] = run;
}

// Single block: bases of each primitive's pair segment and of its work
// items, in the order of decreasing primitive length.
__global__ void __launch_bounds__(1024) scan_totals(int P, const int32_t *order, const uint32_t *tot,
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
    ctr->next_item = 0;
  }
}

// Warp per (node tile b, 32 primitives); lane = primitive.
__global__ void __launch_bounds__(256) nn_emit(int P, int Ppad, int64_t W, const uint32_t *mask,
                                               const uint32_t *loc, const unsigned long long *pbase,
                                               int64_t cap, uint32_t *pair_node, uint32_t *pair_prim) {
  const int lane = threadIdx.x & 31;
  const int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int p = g * 32 + lane;
  const int64_t b = blockIdx.y;
  if (p >= P) return;
  unsigned long long pos = pbase[p] + loc[b * P + p];
  for (int k = 0; k < kNNThreads / 32; k++) {
    const int64_t w = b * (kNNThreads / 32) + k;
    if (w >= W) break;
    uint32_t word = mask[w * Ppad + p];
    while (word) {
      const int bit = __ffs(word) - 1;
      word &= word - 1;
      if ((int64_t)pos < cap) {
        pair_node[pos] = (uint32_t)(w * 32 + bit);
        pair_prim[pos] = (uint32_t)p;
      }
      pos++;
    }
  }
}

// ------------------------------------------------------ exact checking ---

template <class Real> struct StepGeom {
  // per state, per part: pose and its axis-aligned half extents
  Real cx[2], cy[2], c[2], s[2], ex[2], ey[2];
};

// Collision test of one state against all obstacles (planar box parts).
// Updates the lane's min axis-aligned clearance; returns 0 clear, 1 hit,
// 2 ambiguous (|gap| <= band, FP32 path only).
template <class Real, bool BAND, int PARTS>
__device__ __forceinline__ int test_planar(const StepGeom<Real> &G, Real px0, Real py0, Real px1,
                                           Real py1, const Obs2<Real> *obs, int n_obs, Real a,
                                           Real b, Real band, Real &mg) {
  int res = 0;
  for (int o = 0; o < n_obs; o++) {
    const Obs2<Real> ob = obs[o];
#pragma unroll
    for (int q = 0; q < PARTS; q++) {
      const Real px = q == 0 ? px0 : px1, py = q == 0 ? py0 : py1;
      const Real dx = px - ob.cx, dy = py - ob.cy;
      const Real g = fmax(fabs(dx) - (G.ex[q] + ob.hx), fabs(dy) - (G.ey[q] + ob.hy));
      mg = fmin(mg, g);
      if (g <= band) {
        const Real ac = fabs(G.c[q]), as = fabs(G.s[q]);
        const Real du = dx * G.c[q] + dy * G.s[q], dv = dy * G.c[q] - dx * G.s[q];
        const Real gu = fabs(du) - (a + ob.hx * ac + ob.hy * as);
        const Real gv = fabs(dv) - (b + ob.hx * as + ob.hy * ac);
        const Real gs = fmax(g, fmax(gu, gv));
        if (BAND) {
          if (gs <= band) res = max(res, gs < -band ? 1 : 2);
        } else {
          if (gs <= Real(0)) res = 1;
        }
      }
    }
  }
  return res;
}

template <class Real, bool BAND>
__device__ __forceinline__ int test_sphere(Real px, Real py, Real pz, const Obs3<Real> *obs,
                                           int n_obs, Real rad, Real band, Real &mg) {
  int res = 0;
  for (int o = 0; o < n_obs; o++) {
    const Obs3<Real> ob = obs[o];
    const Real dx = fabs(px - ob.cx) - ob.hx, dy = fabs(py - ob.cy) - ob.hy,
               dz = fabs(pz - ob.cz) - ob.hz;
    const Real m = fmax(dx, fmax(dy, dz));
    const Real g = m - rad;
    mg = fmin(mg, g);
    if (g <= band) {
      const Real ux = fmax(dx, Real(0)), uy = fmax(dy, Real(0)), uz = fmax(dz, Real(0));
      const Real gs = (m <= Real(0) ? m : sqrt(ux * ux + uy * uy + uz * uz)) - rad;
      if (BAND) {
        if (gs <= band) res = max(res, gs < -band ? 1 : 2);
      } else {
        if (gs <= Real(0)) res = 1;
      }
    }
  }
  return res;
}

// bounds of a position component: 0 inside, 1 outside, 2 ambiguous
template <class Real, bool BAND>
__device__ __forceinline__ int bound_test(Real v, double lo, double hi, Real band) {
  if (BAND) {
    if (v < Real(lo) - band || v > Real(hi) + band) return 1;
    if (v <= Real(lo) + band || v >= Real(hi) - band) return 2;
    return 0;
  } else {
    return (v >= Real(lo) && v <= Real(hi)) ? 0 : 1;
  }
}

struct CheckArgs {
  RobotParams rp;
  PrimView pv;
  NodeView nv;
  EnvView ev;
  PairView out;
  const unsigned long long *ord_pbase;
  const unsigned long long *ord_ibase;
  DevCounters *ctr;
  const volatile int *abort_flag;
  double band;
};

template <class Real> __device__ __forceinline__ const Pose<Real> *pose_table(const PrimView &pv);
template <> __device__ __forceinline__ const Pose<float> *pose_table<float>(const PrimView &pv) { return pv.pose32; }
template <> __device__ __forceinline__ const Pose<double> *pose_table<double>(const PrimView &pv) { return pv.pose64; }

template <class Real> __device__ __forceinline__ Real node_off(const NodeView &nv, int64_t n, int i, int nx, int comp);
template <> __device__ __forceinline__ float node_off<float>(const NodeView &nv, int64_t n, int i, int nx, int comp) {
  return nv.off32[i * nv.N + n];
}
template <> __device__ __forceinline__ double node_off<double>(const NodeView &nv, int64_t n, int i, int nx, int comp) {
  return nv.x64[n * nx + comp];
}

// One (primitive, node) pair: the transformed trajectory is
//   position_k = canonical_k + offset_pos + k*dt*offset_vel,
//   velocity_k = canonical_k + offset_vel, other components = canonical_k,
// which is the translation of the stored states (unicycle1, car1) and the
// exact re-rollout from the shifted start (quad2d, quad3d: no dynamics term
// depends on position or velocity).  LOCKSTEP: the 32 lanes of a warp share
// the primitive and advance over its states together.
template <int KIND, class Real, bool BAND, bool LOCKSTEP, class OutT>
__device__ void check_one(const CheckArgs &A, const void *obs_sm, int p, int64_t pair,
                          uint32_t node, bool active, uint8_t flag_bits) {
  using R = Robot<KIND>;
  const PrimView &pv = A.pv;
  const RobotParams &rp = A.rp;
  const int L = pv.len[p];
  const int64_t s0 = pv.soff[p];
  const Pose<Real> *pose = pose_table<Real>(pv);
  const Real band = BAND ? Real(A.band) : Real(0);

  Real off[R::POSD + R::VELOFF];
#pragma unroll
  for (int i = 0; i < R::POSD; i++) off[i] = active ? node_off<Real>(A.nv, node, i, R::NX, i) : Real(0);
#pragma unroll
  for (int i = 0; i < R::VELOFF; i++)
    off[R::POSD + i] = active ? node_off<Real>(A.nv, node, R::POSD + i, R::NX, R::vel_comp(i)) : Real(0);

  // bounds pre-check on the swept box of the trajectory (FP64)
  bool need_bounds = true;
  if (active) {
    const double *bx = pv.pbox + (int64_t)p * 2 * R::POSD;
    const double *x64 = A.nv.x64 + (int64_t)node * R::NX;
    const double tmax = (L - 1) * rp.dt;
    bool inside = true;
#pragma unroll
    for (int i = 0; i < R::POSD; i++) {
      double lo = bx[i] + x64[i], hi = bx[R::POSD + i] + x64[i];
      if (R::VELOFF) {
        const double sv = tmax * x64[R::vel_comp(i)];
        lo += fmin(sv, 0.0);
        hi += fmax(sv, 0.0);
      }
      inside = inside && lo > A.ev.lo[i] + A.band && hi < A.ev.hi[i] - A.band;
    }
    need_bounds = !inside;
  }

  bool done = !active, collided = false;
  int first_oob = L, first_col = L, amb = 0;
  Real mg = Real(INFINITY);  // no obstacle: +inf
  const Real hl = Real(rp.half_len), hw = Real(rp.half_wid), rad = Real(rp.radius);

  for (int k = 0; k < L; k++) {
    if (LOCKSTEP) {
      if (!__any_sync(kFull, !done)) break;
    } else if (done) {
      break;
    }
    // per-state geometry, shared by all lanes of the warp
    StepGeom<Real> G;
#pragma unroll
    for (int q = 0; q < R::PARTS; q++) {
      const Pose<Real> ps = pose[q * pv.S + s0 + k];
      G.cx[q] = ps.cx; G.cy[q] = ps.cy; G.c[q] = ps.c; G.s[q] = ps.s;
      if (!R::SPHERE) {
        const Real ac = fabs(ps.c), as = fabs(ps.s);
        G.ex[q] = hl * ac + hw * as;
        G.ey[q] = hl * as + hw * ac;
      }
    }
    if (done) continue;
    const Real t = Real(k) * Real(rp.dt);
    Real sx = off[0], sy = off[1], sz = Real(0);
    if (R::VELOFF) { sx += t * off[R::POSD + 0]; sy += t * off[R::POSD + 1]; }
    if (R::POSD == 3) { sz = off[2]; if (R::VELOFF) sz += t * off[R::POSD + 2]; }
    const Real px0 = G.cx[0] + sx, py0 = G.cy[0] + sy;
    if (need_bounds) {
      int bt = bound_test<Real, BAND>(px0, A.ev.lo[0], A.ev.hi[0], band);
      bt = max(bt, bound_test<Real, BAND>(py0, A.ev.lo[1], A.ev.hi[1], band));
      if (R::POSD == 3) bt = max(bt, bound_test<Real, BAND>(G.c[0] + sz, A.ev.lo[2], A.ev.hi[2], band));
      if (bt == 2) { amb = 1; done = true; continue; }
      if (bt == 1) { first_oob = k; done = true; continue; }
    }
    if (collided) continue;
    int res;
    if constexpr (R::SPHERE) {
      res = test_sphere<Real, BAND>(px0, py0, G.c[0] + sz, (const Obs3<Real> *)obs_sm, A.ev.n_obs, rad, band, mg);
    } else {
      const Real px1 = R::PARTS > 1 ? G.cx[R::PARTS - 1] + sx : px0;
      const Real py1 = R::PARTS > 1 ? G.cy[R::PARTS - 1] + sy : py0;
      res = test_planar<Real, BAND, R::PARTS>(G, px0, py0, px1, py1, (const Obs2<Real> *)obs_sm,
                                              A.ev.n_obs, hl, hw, band, mg);
    }
    if (res == 2) { amb = 1; done = true; continue; }
    if (res == 1) {
      collided = true;
      first_col = k;
      if (!need_bounds) done = true;
    }
  }
  if (!active) return;
  const PairView &o = A.out;
  if (amb) {  // hand the pair to the FP64 re-check
    const unsigned long long slot = atomicAdd(&A.ctr->n_recheck, 1ull);
    o.recheck[slot] = (uint32_t)pair;
    return;
  }
  uint8_t verdict;
  int fi;
  if (first_oob < L) { verdict = DPG_OUT_OF_BOUNDS; fi = first_oob; }
  else if (collided) { verdict = DPG_COLLISION; fi = first_col; }
  else { verdict = DPG_VALID; fi = L; }
  const int er = first_oob < L ? first_oob : L - 1;  // end-state row
  if (o.verdict) o.verdict[pair] = verdict;
  if (o.first_invalid) o.first_invalid[pair] = (int16_t)fi;
  if (o.min_gap) o.min_gap[pair] = verdict == DPG_OUT_OF_BOUNDS ? __int_as_float(0x7fc00000) : (float)mg;
  if (o.flags) o.flags[pair] = flag_bits;
  if (o.end_state) {
    OutT *es = (OutT *)o.end_state + pair * R::NX;
    const Real t = Real(er) * Real(rp.dt);
    const int64_t row = s0 + er;
#pragma unroll
    for (int c = 0; c < R::NX; c++) {
      Real v = sizeof(Real) == 4 ? Real(pv.st32[row * R::NX + c]) : Real(pv.st64[row * R::NX + c]);
      if (c < R::POSD) {
        v += off[c];
        if (R::VELOFF) v += t * off[R::POSD + c];
      }
#pragma unroll
      for (int i = 0; i < R::VELOFF; i++)
        if (c == R::vel_comp(i)) v += off[R::POSD + i];
      es[c] = (OutT)v;
    }
  }
}

template <class Real, int KIND>
__device__ void load_obstacles(const EnvView &ev, void *sm) {
  using R = Robot<KIND>;
  if constexpr (R::SPHERE) {
    const Obs3<Real> *src = (const Obs3<Real> *)(sizeof(Real) == 4 ? ev.obs32 : ev.obs64);
    Obs3<Real> *dst = (Obs3<Real> *)sm;
    for (int i = threadIdx.x; i < ev.n_obs; i += blockDim.x) dst[i] = src[i];
  } else {
    const Obs2<Real> *src = (const Obs2<Real> *)(sizeof(Real) == 4 ? ev.obs32 : ev.obs64);
    Obs2<Real> *dst = (Obs2<Real> *)sm;
    for (int i = threadIdx.x; i < ev.n_obs; i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
}

// Persistent warps: each warp takes the next work item (primitive in order
// of decreasing length, next 32 of its nodes) from a device counter.
template <int KIND, class Real, bool BAND>
__global__ void __launch_bounds__(kCheckThreads) check_pairs(CheckArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  load_obstacles<Real, KIND>(A.ev, smem);
  const int lane = threadIdx.x & 31;
  const int P = A.pv.P;
  const unsigned long long n_items = A.ctr->n_items;
  while (true) {
    unsigned long long item = 0;
    int stop = 0;
    if (lane == 0) {
      stop = *A.abort_flag;
      item = stop ? n_items : atomicAdd(&A.ctr->next_item, 1ull);
    }
    item = __shfl_sync(kFull, item, 0);
    stop = __shfl_sync(kFull, stop, 0);
    if (stop) {
      if (lane == 0) A.ctr->status = DPG_ERR_ABORTED;
      break;
    }
    if (item >= n_items) break;
    // order position i with ord_ibase[i] <= item < ord_ibase[i+1]
    int lo = 0, hi = P;  // invariant: ord_ibase[lo] <= item < ord_ibase[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (A.ord_ibase[mid] <= item) lo = mid; else hi = mid;
    }
    const int p = A.pv.order[lo];
    const unsigned long long j = item - A.ord_ibase[lo];
    const unsigned long long first = A.ord_pbase[lo] + 32ull * j;
    const unsigned long long end = A.ord_pbase[lo + 1];
    const unsigned long long pair = first + lane;
    const bool active = pair < end;
    const uint32_t node = active ? A.out.node[pair] : 0u;
    check_one<KIND, Real, BAND, true, Real>(A, smem, p, (int64_t)pair, node, active, 0);
  }
}

// FP64 re-check of flagged pairs, one thread per pair.
template <int KIND>
__global__ void __launch_bounds__(kCheckThreads) recheck_pairs(CheckArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  load_obstacles<double, KIND>(A.ev, smem);
  const unsigned long long n = A.ctr->n_recheck;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const uint32_t pair = A.out.recheck[i];
    const int p = (int)A.out.prim[pair];
    check_one<KIND, double, false, false, float>(A, smem, p, pair, A.out.node[pair], true,
                                          DPG_FLAG_CONTACT_RECHECK);
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
__global__ void build_keys(RobotParams rp, int P, const int32_t *len, const int64_t *soff,
                           const double *st64, float *key32, float *kconst32, double *pbox) {
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
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int k = 0; k < len[p]; k++)
    for (int i = 0; i < R::POSD; i++) {
      lo[i] = fmin(lo[i], s[k * R::NX + i]);
      hi[i] = fmax(hi[i], s[k * R::NX + i]);
    }
  for (int i = 0; i < R::POSD; i++) {
    pbox[(int64_t)p * 2 * R::POSD + i] = lo[i];
    pbox[(int64_t)p * 2 * R::POSD + R::POSD + i] = hi[i];
  }
}

}  // namespace dpg
