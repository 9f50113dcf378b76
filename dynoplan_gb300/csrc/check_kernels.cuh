// check_kernels.cuh -- exact checking of (primitive, node) pairs on sm_103a.
//
// Replaces LazyTraj::compute + check_lazy_trajectory
// (include/dynoplan/dbastar/dbastar.hpp:166-230, src/dbastar/dbastar.cpp:391-490)
// for every in-ball pair of a batch.
//
// Work decomposition: persistent warps take (primitive, 32 nodes) items from a
// device counter, longest primitives first.  The 32 lanes walk the same
// primitive in lockstep, so the per-state pose rows are warp-broadcast loads
// and the lanes differ only by their node offset.
//
// Transform: position_k = canonical_k + p0 (+ k*dt*v0), velocity_k =
// canonical_k + v0, other components canonical_k.  That is the translation of
// the stored states (unicycle1, car1) and, exactly, the re-rollout from the
// shifted start for quad2d / quadrotor (no dynamics term depends on position
// or velocity); the canonical rollout is FP64, once per upload.
//
// Obstacles (shared memory) are culled per lane in two levels, both with a
// margin of band + slack (+ kGapCap when min_gap is an output) so nothing that
// could touch the robot, fall in the FP64 band or set min_gap is dropped:
//   1. against the bounding box of the whole transformed primitive (once per
//      pair; bitmask over <= kMaxCullObs obstacles),
//   2. against the box of each chunk of R::CHUNK states (from the level-1 set),
// then every state tests its chunk's candidates (separating axes, AABB early
// reject).  Bounds tests run only in chunks whose box is not inside the
// bounds, and a chunk in which no lane has an obstacle or bounds test to make
// is stepped over as a whole.  A test whose FP32 gap lies within `band` of zero, and a bounds
// test within `band` of a bound, is recomputed in FP64 from the FP64 tables
// on the spot, so verdicts equal the FP64 oracle's.
#pragma once

#include <type_traits>

#include "expand_kernels.cuh"

namespace dpg {

struct CheckArgs {
  RobotParams rp;
  PrimView pv;
  NodeView nv;
  EnvView ev;
  PairView out;
  const unsigned long long *ord_pbase;
  const unsigned long long *ord_ibase;
  const uint32_t *item_pos;  // item -> order position (null: binary search over ord_ibase)
  DevCounters *ctr;
  const volatile int *abort_flag;
  double band;       // FP64 re-check band (0 on the FP64 path)
  float cull_margin; // obstacle culling margin
  // FP32 copies of the constants the state loop uses (GB300 runs FP64 and
  // double->float conversions at 1/64 of the FP32 rate)
  float dt32, half_len32, half_wid32, radius32, band32;
  float lo32[3], hi32[3];
  // this launch takes work items [n_items cum[sub] / cum[nsub],
  // n_items cum[sub + 1] / cum[nsub]) (integer weights; nsub <= 1: all items)
  int sub, nsub;
  int sub_cum[kMaxSub + 1];
  // progress-driven copies (one launch, nsub = 1): the items fall into
  // n_ranges ranges by the same weights; a warp adds the items it finished
  // in a range to range_done when it moves to the next range or stops (after
  // a fence), and the add that completes a range sets range_flag[j] (mapped
  // host memory) after a system fence
  int n_ranges;
  int *range_flag;
  // when set, the pair's node id is written back through it (processing
  // order -> caller's numbering) once the pair is checked
  const uint32_t *perm;
  // slot variant: byte offset of the per-warp scratch in dynamic shared memory
  int slot_offset;
};

// Obstacle culling margin: every obstacle within the FP64 band, plus a slack
// for the FP32 box arithmetic, and within the min_gap cap when min_gap is an
// output (without it, obstacles farther than the band change no result).
inline float cull_margin(bool min_gap, double band) { return (min_gap ? kGapCap : 0.f) + (float)band + 1e-3f; }

template <class Real> __device__ __forceinline__ const Pose<Real> *pose_table(const PrimView &pv);
template <> __device__ __forceinline__ const Pose<float> *pose_table<float>(const PrimView &pv) { return pv.pose32; }
template <> __device__ __forceinline__ const Pose<double> *pose_table<double>(const PrimView &pv) { return pv.pose64; }

// node offset component i (position i < POSD, then velocity)
template <class Real> __device__ __forceinline__ Real node_off(const NodeView &nv, int64_t n, int i, int nx, int comp);
template <> __device__ __forceinline__ float node_off<float>(const NodeView &nv, int64_t n, int i, int nx, int comp) {
  return nv.off32[i * nv.N + n];
}
template <> __device__ __forceinline__ double node_off<double>(const NodeView &nv, int64_t n, int i, int nx, int comp) {
  return nv.x64[n * nx + comp];
}

// ------------------------------------------------------------ narrow phase --

// Oriented box (pose c,s; half extents a,b; axis-aligned half extents ex,ey)
// against an obstacle box.  Returns 0 clear, 1 contact, 2 ambiguous (|gap| <=
// band, FP32 path).  mg takes the axis-aligned clearance.
template <class Real, bool BAND>
__device__ __forceinline__ int planar_test(Real px, Real py, Real c, Real s, Real ex, Real ey,
                                           const Obs2<Real> &ob, Real a, Real b, Real band, Real &mg) {
  const Real dx = px - ob.cx, dy = py - ob.cy;
  const Real g = fmax(fabs(dx) - (ex + ob.hx), fabs(dy) - (ey + ob.hy));
  mg = fmin(mg, g);
  if (g > band) return 0;
  const Real ac = fabs(c), as = fabs(s);
  const Real du = dx * c + dy * s, dv = dy * c - dx * s;
  const Real gu = fabs(du) - (a + ob.hx * ac + ob.hy * as);
  const Real gv = fabs(dv) - (b + ob.hx * as + ob.hy * ac);
  const Real gs = fmax(g, fmax(gu, gv));
  if (BAND) {
    if (gs > band) return 0;
    return gs < -band ? 1 : 2;
  }
  return gs <= Real(0) ? 1 : 0;
}

template <class Real, bool BAND>
__device__ __forceinline__ int sphere_test(Real px, Real py, Real pz, const Obs3<Real> &ob, Real rad,
                                           Real band, Real &mg) {
  const Real dx = fabs(px - ob.cx) - ob.hx, dy = fabs(py - ob.cy) - ob.hy, dz = fabs(pz - ob.cz) - ob.hz;
  const Real m = fmax(dx, fmax(dy, dz));
  const Real g = m - rad;
  mg = fmin(mg, g);
  if (g > band) return 0;
  const Real ux = fmax(dx, Real(0)), uy = fmax(dy, Real(0)), uz = fmax(dz, Real(0));
  const Real gs = (m <= Real(0) ? m : sqrt(ux * ux + uy * uy + uz * uz)) - rad;
  if (BAND) {
    if (gs > band) return 0;
    return gs < -band ? 1 : 2;
  }
  return gs <= Real(0) ? 1 : 0;
}

// FP64 position component i of state k (affine transform of the FP64 table)
template <int KIND>
__device__ __forceinline__ double pos64(const CheckArgs &A, int64_t row, int k, const double *x64, int i) {
  using R = Robot<KIND>;
  const Pose<double> ps = A.pv.pose64[row];  // part 0 = the state position
  double v = (i == 0 ? ps.cx : (i == 1 ? ps.cy : ps.c)) + x64[i];
  if (R::VELOFF) v += (double(k) * A.rp.dt) * x64[R::vel_comp(i)];
  return v;
}

// FP64 separating-axis gap of part q at state k against obstacle o (the
// oracle's formula, from the FP64 tables).
template <int KIND>
__device__ double gap64(const CheckArgs &A, int64_t s0, int k, int q, const double *x64, int o) {
  using R = Robot<KIND>;
  const RobotParams &rp = A.rp;
  double sx = x64[0], sy = x64[1], sz = R::POSD == 3 ? x64[2] : 0.0;
  if (R::VELOFF) {
    const double t = double(k) * rp.dt;
    sx += t * x64[R::vel_comp(0)];
    sy += t * x64[R::vel_comp(1)];
    if (R::POSD == 3) sz += t * x64[R::vel_comp(2)];
  }
  const Pose<double> ps = A.pv.pose64[q * A.pv.S + s0 + k];
  if constexpr (R::SPHERE) {
    const Obs3<double> ob = ((const Obs3<double> *)A.ev.obs64)[o];
    const double dx = fabs(ps.cx + sx - ob.cx) - ob.hx, dy = fabs(ps.cy + sy - ob.cy) - ob.hy,
                 dz = fabs(ps.c + sz - ob.cz) - ob.hz;
    const double m = fmax(dx, fmax(dy, dz));
    const double ux = fmax(dx, 0.0), uy = fmax(dy, 0.0), uz = fmax(dz, 0.0);
    return (m <= 0 ? m : sqrt(ux * ux + uy * uy + uz * uz)) - rp.radius;
  } else {
    const Obs2<double> ob = ((const Obs2<double> *)A.ev.obs64)[o];
    const double px = ps.cx + sx, py = ps.cy + sy;
    const double ac = fabs(ps.c), as = fabs(ps.s);
    const double a = rp.half_len, b = rp.half_wid;
    const double dx = px - ob.cx, dy = py - ob.cy;
    const double gx = fabs(dx) - (a * ac + b * as + ob.hx);
    const double gy = fabs(dy) - (a * as + b * ac + ob.hy);
    const double du = dx * ps.c + dy * ps.s, dv = -dx * ps.s + dy * ps.c;
    const double gu = fabs(du) - (a + ob.hx * ac + ob.hy * as);
    const double gv = fabs(dv) - (b + ob.hx * as + ob.hy * ac);
    return fmax(fmax(gx, gy), fmax(gu, gv));
  }
}

// box (centre cen, half hf) against obstacle box, with margin
template <int D, class Real>
__device__ __forceinline__ bool near_box(const float *cen, const float *hf, const void *obs_sm, int o, float M) {
  if constexpr (D == 2) {
    const Obs2<Real> ob = ((const Obs2<Real> *)obs_sm)[o];
    return fabsf(cen[0] - (float)ob.cx) <= hf[0] + (float)ob.hx + M &&
           fabsf(cen[1] - (float)ob.cy) <= hf[1] + (float)ob.hy + M;
  } else {
    const Obs3<Real> ob = ((const Obs3<Real> *)obs_sm)[o];
    return fabsf(cen[0] - (float)ob.cx) <= hf[0] + (float)ob.hx + M &&
           fabsf(cen[1] - (float)ob.cy) <= hf[1] + (float)ob.hy + M &&
           fabsf(cen[2] - (float)ob.cz) <= hf[2] + (float)ob.hz + M;
  }
}


// ------------------------------------------------------------- one pair ----

// NW: words of the per-lane obstacle bitmasks (obstacles <= 32 NW); 0 = no
// culling (more than kMaxCullObs obstacles), every state tests every obstacle.
// ES64: write the end state in FP64 (the FP64 canonical row plus the FP64
// node offset) while the tests run in Real.
template <int KIND, class Real, bool BAND, int NW, bool LOCKSTEP, bool ES64 = false>
__device__ void check_one(const CheckArgs &A, const void *obs_sm, int p, int64_t pair, uint32_t node,
                          bool active) {
  using R = Robot<KIND>;
  constexpr int D = R::POSD, V = R::VELOFF;
  const PrimView &pv = A.pv;
  const RobotParams &rp = A.rp;
  const int L = pv.len[p];
  const int64_t s0 = pv.soff[p];
  const Pose<Real> *pose = pose_table<Real>(pv);
  constexpr bool F32 = sizeof(Real) == 4;
  const Real band = BAND ? (F32 ? Real(A.band32) : Real(A.band)) : Real(0);
  const Real dtR = F32 ? Real(A.dt32) : Real(rp.dt);
  Real loR[3], hiR[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    loR[i] = F32 ? Real(A.lo32[i]) : Real(A.ev.lo[i]);
    hiR[i] = F32 ? Real(A.hi32[i]) : Real(A.ev.hi[i]);
  }
  const double *x64 = A.nv.x64 + (int64_t)(active ? node : 0) * R::NX;
  const int n_obs = A.ev.n_obs;

  Real off[D + V];
#pragma unroll
  for (int i = 0; i < D; i++) off[i] = active ? node_off<Real>(A.nv, node, i, R::NX, i) : Real(0);
#pragma unroll
  for (int i = 0; i < V; i++) off[D + i] = active ? node_off<Real>(A.nv, node, D + i, R::NX, R::vel_comp(i)) : Real(0);

  // bounds pre-check on the swept box of the positions: inside with a margin
  // (band + slack for the arithmetic) means no state needs a bounds test
  bool need_bounds = true;
  if (active) {
    const double *bx = pv.pbox + (int64_t)p * 2 * D;
    const float *bx32 = pv.pbox32 + (int64_t)p * 2 * D;
    const Real tmax = Real(L - 1) * dtR;
    const Real slack = F32 ? Real(1e-3f) : Real(0);
    bool inside = true;
#pragma unroll
    for (int i = 0; i < D; i++) {
      Real lo = (F32 ? Real(bx32[i]) : Real(bx[i])) + off[i];
      Real hi = (F32 ? Real(bx32[D + i]) : Real(bx[D + i])) + off[i];
      if (V) {
        const Real sv = tmax * off[D + i];
        lo += fmin(sv, Real(0));
        hi += fmax(sv, Real(0));
      }
      inside = inside && lo > loR[i] + band + slack && hi < hiR[i] - band - slack;
    }
    need_bounds = !inside;
  }

  // level-1 culling: obstacles near the whole transformed primitive
  constexpr bool CULL = NW > 0;
  constexpr int NWA = NW > 0 ? NW : 1;
  uint32_t l1[NWA] = {};
  const float M = A.cull_margin;
  if (CULL && active) {
    const float *tb = pv.tbox32 + (int64_t)p * 2 * D;
    const float tmax = float(L - 1) * A.dt32;
    float cen[D], hf[D];
#pragma unroll
    for (int i = 0; i < D; i++) {
      cen[i] = tb[i] + (float)off[i];
      hf[i] = tb[D + i];
      if (V) {
        const float sv = tmax * (float)off[D + i];
        cen[i] += 0.5f * sv;
        hf[i] += 0.5f * fabsf(sv);
      }
    }
#pragma unroll
    for (int w = 0; w < NWA; w++) {  // word by word: the masks stay in registers
      uint32_t bits = 0u;
      const int o0 = 32 * w, o1 = min(n_obs, o0 + 32);
      for (int o = o0; o < o1; o++)
        if (near_box<D, Real>(cen, hf, obs_sm, o, M)) bits |= 1u << (o - o0);
      l1[w] = bits;
    }
  }

  bool done = !active, collided = false, rechecked = false;
  int first_oob = L, first_col = L;
  Real mg = Real(INFINITY);
  const Real hl = F32 ? Real(A.half_len32) : Real(rp.half_len);
  const Real hw = F32 ? Real(A.half_wid32) : Real(rp.half_wid);
  const Real rad = F32 ? Real(A.radius32) : Real(rp.radius);
  uint32_t cm[NWA] = {};
  bool nb = need_bounds;  // bounds tests in the current chunk

  for (int k = 0; k < L; k++) {
    if (LOCKSTEP) {
      if (!__any_sync(kFull, !done)) break;
    } else if (done) {
      break;
    }
    const Real t = Real(k) * dtR;
    // at each chunk start: the chunk's box (the parts over its R::CHUNK states,
    // transformed), level-2 culling, and whether its states need bounds tests
    if (CULL && (k % R::CHUNK) == 0) {
      const float *cb = pv.cbox32 + (pv.coff[p] + k / R::CHUNK) * 2 * D;
      const float t0 = float(k) * A.dt32, t1 = float(min(L - 1, k + R::CHUNK - 1)) * A.dt32;
      float cen[D], hf[D];
#pragma unroll
      for (int i = 0; i < D; i++) {
        cen[i] = cb[i] + (float)off[i];
        hf[i] = cb[D + i];
        if (V) {
          const float v = (float)off[D + i];
          cen[i] += 0.5f * (t0 + t1) * v;
          hf[i] += 0.5f * (t1 - t0) * fabsf(v);
        }
      }
      if (!done && !collided) {
#pragma unroll
        for (int w = 0; w < NWA; w++) {
          uint32_t m = l1[w], c = 0;
          while (m) {
            const int b = __ffs(m) - 1;
            m &= m - 1;
            if (near_box<D, Real>(cen, hf, obs_sm, 32 * w + b, M)) c |= 1u << b;
          }
          cm[w] = c;
        }
      }
      // the box holds every state position of the chunk: inside the bounds
      // with the band and an arithmetic slack, no state of it is out
      if (need_bounds) {
        bool in = true;
#pragma unroll
        for (int i = 0; i < D; i++)
          in = in && cen[i] - hf[i] > A.lo32[i] + A.band32 + 1e-3f && cen[i] + hf[i] < A.hi32[i] - A.band32 - 1e-3f;
        nb = !in;
      }
      // no lane has an obstacle test or a bounds test to make in this chunk:
      // its states change nothing (no contact, no bound, no min_gap update)
      if (LOCKSTEP) {
        uint32_t any = 0u;
#pragma unroll
        for (int w = 0; w < NWA; w++) any |= cm[w];
        const bool idle = done || ((collided || any == 0u) && !nb);
        if (__all_sync(kFull, idle)) {
          k += R::CHUNK - 1;
          continue;
        }
      }
    }
    if (done) continue;
    // per-state geometry (identical for the 32 lanes)
    Pose<Real> ps[R::PARTS];
#pragma unroll
    for (int q = 0; q < R::PARTS; q++) ps[q] = pose[q * pv.S + s0 + k];
    Real sx = off[0], sy = off[1], sz = Real(0);
    if (V) { sx += t * off[D + 0]; sy += t * off[D + 1]; }
    if (D == 3) { sz = off[2]; if (V) sz += t * off[D + 2]; }
    if (nb) {
      const Real pv3[3] = {ps[0].cx + sx, ps[0].cy + sy, ps[0].c + sz};
      int bt = 0;
#pragma unroll
      for (int i = 0; i < D; i++) {
        int r;
        if (BAND) {
          const Real v = pv3[i];
          const Real lo = loR[i], hi = hiR[i];
          r = (v < lo - band || v > hi + band) ? 1 : ((v <= lo + band || v >= hi - band) ? 2 : 0);
          if (r == 2) {  // decide in FP64
            const double v64 = pos64<KIND>(A, s0 + k, k, x64, i);
            r = (v64 >= A.ev.lo[i] && v64 <= A.ev.hi[i]) ? 0 : 1;
            rechecked = true;
          }
        } else {
          r = (pv3[i] >= loR[i] && pv3[i] <= hiR[i]) ? 0 : 1;
        }
        bt |= r;
      }
      if (bt) { first_oob = k; done = true; continue; }
    }
    if (collided) continue;
    bool hit = false;
    auto test_obstacle = [&](int o) {
      if constexpr (R::SPHERE) {
        const Obs3<Real> ob = ((const Obs3<Real> *)obs_sm)[o];
        int r = sphere_test<Real, BAND>(ps[0].cx + sx, ps[0].cy + sy, ps[0].c + sz, ob, rad, band, mg);
        if (BAND && r == 2) { r = gap64<KIND>(A, s0, k, 0, x64, o) <= 0.0 ? 1 : 0; rechecked = true; }
        hit |= r == 1;
      } else {
        const Obs2<Real> ob = ((const Obs2<Real> *)obs_sm)[o];
#pragma unroll
        for (int q = 0; q < R::PARTS; q++) {
          const Real ac = fabs(ps[q].c), as = fabs(ps[q].s);
          const Real ex = hl * ac + hw * as, ey = hl * as + hw * ac;
          int r = planar_test<Real, BAND>(ps[q].cx + sx, ps[q].cy + sy, ps[q].c, ps[q].s, ex, ey, ob, hl, hw,
                                          band, mg);
          if (BAND && r == 2) { r = gap64<KIND>(A, s0, k, q, x64, o) <= 0.0 ? 1 : 0; rechecked = true; }
          hit |= r == 1;
        }
      }
    };
    if (CULL) {
#pragma unroll
      for (int w = 0; w < NWA; w++) {
        uint32_t m = cm[w];
        while (m) {
          const int b = __ffs(m) - 1;
          m &= m - 1;
          test_obstacle(32 * w + b);
        }
      }
    } else {
      for (int o = 0; o < n_obs; o++) test_obstacle(o);
    }
    if (hit) {
      collided = true;
      first_col = k;
      if (!need_bounds) done = true;
    }
  }

  const unsigned rmask = LOCKSTEP ? __ballot_sync(kFull, active && rechecked) : 0u;
  if (LOCKSTEP && (threadIdx.x & 31) == 0 && rmask) atomicAdd(&A.ctr->n_recheck, (unsigned long long)__popc(rmask));
  if (!active) return;
  const PairView &o = A.out;
  if (A.perm) o.node[pair] = A.perm[node];
  uint8_t verdict;
  int fi;
  if (first_oob < L) { verdict = DPG_OUT_OF_BOUNDS; fi = first_oob; }
  else if (collided) { verdict = DPG_COLLISION; fi = first_col; }
  else { verdict = DPG_VALID; fi = L; }
  const int er = first_oob < L ? first_oob : L - 1;  // end-state row
  const int64_t row_out = o.out_index ? (int64_t)o.out_index[pair] : pair;
  if (o.node_host) {
    o.node_host[row_out] = A.perm ? A.perm[node] : node;
    o.prim_host[row_out] = (uint32_t)p;
  }
  if (o.verdict) o.verdict[row_out] = verdict;
  if (o.first_invalid) o.first_invalid[row_out] = (int16_t)fi;
  if (o.min_gap)
    o.min_gap[row_out] = verdict == DPG_OUT_OF_BOUNDS ? __int_as_float(0x7fc00000)
                                                   : ((float)mg <= kGapCap ? (float)mg : __int_as_float(0x7f800000));
  if (o.flags) o.flags[row_out] = rechecked ? DPG_FLAG_CONTACT_RECHECK : 0;
  if (ES64 && o.end_state) {
    double *es = (double *)o.end_state + row_out * R::NX;
    const double t = double(er) * rp.dt;
    const double *xs = pv.st64 + (s0 + er) * R::NX;
#pragma unroll
    for (int c = 0; c < R::NX; c++) {
      double v = xs[c];
      if (c < D) {
        v += x64[c];
        if (V) v += t * x64[R::vel_comp(c)];
      }
#pragma unroll
      for (int i = 0; i < V; i++)
        if (c == R::vel_comp(i)) v += x64[R::vel_comp(i)];
      es[c] = v;
    }
  } else if (o.end_state) {
    Real *es = (Real *)o.end_state + row_out * R::NX;
    const Real t = Real(er) * dtR;
    const int64_t row = s0 + er;
#pragma unroll
    for (int c = 0; c < R::NX; c++) {
      Real v = sizeof(Real) == 4 ? Real(pv.st32[row * R::NX + c]) : Real(pv.st64[row * R::NX + c]);
      if (c < D) {
        v += off[c];
        if (V) v += t * off[D + c];
      }
#pragma unroll
      for (int i = 0; i < V; i++)
        if (c == R::vel_comp(i)) v += off[D + i];
      es[c] = v;
    }
  }
}

// ------------------------------------------------- slot-parallel variant --
//
// The lockstep walk above makes every state cost the largest candidate count
// of any lane: lanes with fewer candidates (most have none) wait.  This
// variant keeps the walk over chunks of R::CHUNK states but runs the narrow
// phase as a list of (lane, chunk, candidate obstacle) slots spread over the
// warp's 32 lanes; a slot tests its obstacle against every state of its chunk
// (all parts) and stops at its first contact.  One narrow round takes
// consecutive chunks until the warp has about a round of slots (car1 chunks
// average about 10 slots a warp), at most 32 states; chunks after a lane's
// first contact are tested speculatively and discarded by the fold.  Per lane
// and state, the contacts, the FP64 decisions and the minimum axis-aligned gap
// are merged in shared memory; each lane then folds the states up to its first
// contact, which gives exactly the per-state results of the sequential walk
// (every candidate is tested at every state up to the first contact).  FP32
// tests with FP64 decisions in the band; the bounds tests stay per lane.

constexpr int kSlotFill = 16;  // a narrow round stops taking chunks at this many slots

template <int CH, int PARTS, int NW> struct SlotScratch {
  static constexpr int GMAX = 32 / CH;  // chunks a round can take (32 hit bits)
  static constexpr int MGS = 16;        // states a round takes when min_gap is an output
  Pose<float> pose[32 * PARTS];         // the round's pose rows, [s * PARTS + q]
  float2 ext[32 * PARTS];               // planar robots: axis-aligned half extents of each part
  unsigned cm[GMAX][NW][32];            // per chunk, word and lane: the chunk's candidates
  unsigned l1[NW][32];                  // per word and lane: level-1 candidates
  unsigned mg[MGS][32];                 // per state and lane: min axis-aligned gap (order-preserving bits)
  unsigned hit[32];                     // per lane: bit s = contact at state k0 + s
  unsigned rc[32];                      // per lane: bit s = a test at k0 + s was decided in FP64
  // (the bounds slots of a chunk use hit / rc before the narrow phase does:
  // bit j = state j of the chunk out of bounds / decided in FP64)
};

__device__ __forceinline__ unsigned ord_gap(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unord_gap(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

template <int KIND, int NW>
constexpr size_t slot_scratch_bytes() {
  return sizeof(SlotScratch<Robot<KIND>::CHUNK, Robot<KIND>::PARTS, NW>);
}

template <int KIND, int NW, bool ES64>
__device__ void check_one_slots(const CheckArgs &A, const void *obs_sm,
                                SlotScratch<Robot<KIND>::CHUNK, Robot<KIND>::PARTS, NW> &S, int p, int64_t pair,
                                uint32_t node, bool active) {
  using R = Robot<KIND>;
  using Scratch = SlotScratch<Robot<KIND>::CHUNK, Robot<KIND>::PARTS, NW>;
  constexpr int D = R::POSD, V = R::VELOFF, CH = R::CHUNK, PARTS = R::PARTS;
  static_assert(NW > 0, "the slot variant needs the candidate bitmasks");
  static_assert(CH <= 16 && Scratch::MGS % CH == 0, "5-bit state counts; whole chunks under the min_gap limit");
  const int lane = threadIdx.x & 31;
  const PrimView &pv = A.pv;
  const RobotParams &rp = A.rp;
  const int L = pv.len[p];
  const int64_t s0 = pv.soff[p];
  const Pose<float> *pose = pv.pose32;
  const float band = A.band32, dt = A.dt32;
  const double *x64 = A.nv.x64 + (int64_t)(active ? node : 0) * R::NX;
  const int n_obs = A.ev.n_obs;
  const bool want_mg = A.out.min_gap != nullptr;  // per-state gap merges only for that output
  const int GL = want_mg ? Scratch::MGS / CH : Scratch::GMAX;

  float off[D + V];
#pragma unroll
  for (int i = 0; i < D; i++) off[i] = active ? node_off<float>(A.nv, node, i, R::NX, i) : 0.f;
#pragma unroll
  for (int i = 0; i < V; i++) off[D + i] = active ? node_off<float>(A.nv, node, D + i, R::NX, R::vel_comp(i)) : 0.f;

  // bounds pre-check on the swept box of the positions (as check_one)
  bool need_bounds = true;
  if (active) {
    const float *bx32 = pv.pbox32 + (int64_t)p * 2 * D;
    const float tmax = float(L - 1) * dt;
    bool inside = true;
#pragma unroll
    for (int i = 0; i < D; i++) {
      float lo = bx32[i] + off[i], hi = bx32[D + i] + off[i];
      if (V) {
        const float sv = tmax * off[D + i];
        lo += fminf(sv, 0.f);
        hi += fmaxf(sv, 0.f);
      }
      inside = inside && lo > A.lo32[i] + band + 1e-3f && hi < A.hi32[i] - band - 1e-3f;
    }
    need_bounds = !inside;
  }

  // level-1 culling against the whole transformed primitive
  const float M = A.cull_margin;
  {
    const float *tb = pv.tbox32 + (int64_t)p * 2 * D;
    const float tmax = float(L - 1) * dt;
    float cen[D], hf[D];
#pragma unroll
    for (int i = 0; i < D; i++) {
      cen[i] = tb[i] + off[i];
      hf[i] = tb[D + i];
      if (V) {
        const float sv = tmax * off[D + i];
        cen[i] += 0.5f * sv;
        hf[i] += 0.5f * fabsf(sv);
      }
    }
#pragma unroll
    for (int w = 0; w < NW; w++) {
      uint32_t bits = 0u;
      if (active) {
        const int o0 = 32 * w, o1 = min(n_obs, o0 + 32);
        for (int o = o0; o < o1; o++)
          if (near_box<D, float>(cen, hf, obs_sm, o, M)) bits |= 1u << (o - o0);
      }
      S.l1[w][lane] = bits;
    }
  }

  bool done = !active, collided = false, rechecked = false;
  int first_oob = L, first_col = L;
  float mg = INFINITY;
  const float hl = A.half_len32, hw = A.half_wid32, rad = A.radius32;

  for (int k0 = 0; k0 < L;) {
    if (!__any_sync(kFull, !done)) break;
    // the round's chunks: level-2 culling, bounds tests, per-chunk state and candidate counts
    uint32_t nsts = 0u, ncs = 0u;  // chunk g: states to test (5 bits at 5g), candidates (8 bits at 8g)
    int n_lane = 0;                // this lane's slots in the round
    int G = 0, kk = k0;
    while (true) {
      const int kend = min(L, kk + CH);
      int nc = 0;
      bool nb = false;
      if (!done) {
        const float *cb = pv.cbox32 + (pv.coff[p] + kk / CH) * 2 * D;
        const float t0 = float(kk) * dt, t1 = float(kend - 1) * dt;
        float cen[D], hf[D];
#pragma unroll
        for (int i = 0; i < D; i++) {
          cen[i] = cb[i] + off[i];
          hf[i] = cb[D + i];
          if (V) {
            const float v = off[D + i];
            cen[i] += 0.5f * (t0 + t1) * v;
            hf[i] += 0.5f * (t1 - t0) * fabsf(v);
          }
        }
        if (!collided) {
#pragma unroll
          for (int w = 0; w < NW; w++) {
            uint32_t m = S.l1[w][lane], c = 0;
            while (m) {
              const int b = __ffs(m) - 1;
              m &= m - 1;
              if (near_box<D, float>(cen, hf, obs_sm, 32 * w + b, M)) c |= 1u << b;
            }
            S.cm[G][w][lane] = c;
            nc += __popc(c);
          }
        }
        if (need_bounds) {
          bool in = true;
#pragma unroll
          for (int i = 0; i < D; i++)
            in = in && cen[i] - hf[i] > A.lo32[i] + band + 1e-3f && cen[i] + hf[i] < A.hi32[i] - band - 1e-3f;
          nb = !in;
        }
      }
      // bounds tests of the chunk's states, up to each lane's first state out.
      // Few lanes with tests: (lane, state) slots over the warp, each lane's
      // first state out (and the FP64 decisions up to it) from bitmasks, as
      // the sequential walk finds them; else each lane walks its states.
      int j_oob = CH;
      bool walk = nb;
      if constexpr (R::BOUNDS_SLOTS) {
        const unsigned nbm = __ballot_sync(kFull, nb);
        const int nbs = __popc(nbm) * (kend - kk);
        if (nbm && nbs <= 64) {
          walk = false;
          const int ns = kend - kk;
          S.hit[lane] = 0u;
          S.rc[lane] = 0u;
          __syncwarp();
          for (int base = 0; base < nbs; base += 32) {
            const int t = base + lane;
            const int li = t / ns, j = t - li * ns;
            const int owner = t < nbs ? (int)__fns(nbm, 0u, li + 1) : 0;
            float osh[D + V];
  #pragma unroll
            for (int i = 0; i < D + V; i++) osh[i] = __shfl_sync(kFull, off[i], owner);
            const uint32_t onode = __shfl_sync(kFull, node, owner);
            if (t < nbs) {
              const int k = kk + j;
              const Pose<float> ps = pose[s0 + k];  // part 0 = the state position
              const float tk = float(k) * dt;
              const float pv3[3] = {ps.cx + osh[0] + (V ? tk * osh[D] : 0.f), ps.cy + osh[1] + (V ? tk * osh[D + 1] : 0.f),
                                    D == 3 ? ps.c + osh[2] + (V ? tk * osh[D + 2] : 0.f) : 0.f};
              int bt = 0;
              bool amb = false;
  #pragma unroll
              for (int i = 0; i < D; i++) {
                const float v = pv3[i], lo = A.lo32[i], hi = A.hi32[i];
                int r = (v < lo - band || v > hi + band) ? 1 : ((v <= lo + band || v >= hi - band) ? 2 : 0);
                if (r == 2) {  // decide in FP64
                  const double v64 = pos64<KIND>(A, s0 + k, k, A.nv.x64 + (int64_t)onode * R::NX, i);
                  r = (v64 >= A.ev.lo[i] && v64 <= A.ev.hi[i]) ? 0 : 1;
                  amb = true;
                }
                bt |= r;
              }
              if (bt) atomicOr(&S.hit[owner], 1u << j);
              if (amb) atomicOr(&S.rc[owner], 1u << j);
            }
          }
          __syncwarp();
          if (nb) {
            const unsigned bo = S.hit[lane];
            const int first = bo ? __ffs(bo) - 1 : CH;
            if (bo) j_oob = first;
            if (S.rc[lane] & (bo ? ((2u << first) - 1u) : 0xffffffffu)) rechecked = true;
          }
          __syncwarp();  // the next chunk's slots and the narrow phase reuse the masks
        }
      }
      if (walk) {
        for (int k = kk; k < kend; k++) {
          const Pose<float> ps = pose[s0 + k];  // part 0 = the state position
          const float t = float(k) * dt;
          const float pv3[3] = {ps.cx + off[0] + (V ? t * off[D] : 0.f), ps.cy + off[1] + (V ? t * off[D + 1] : 0.f),
                                D == 3 ? ps.c + off[2] + (V ? t * off[D + 2] : 0.f) : 0.f};
          int bt = 0;
#pragma unroll
          for (int i = 0; i < D; i++) {
            const float v = pv3[i], lo = A.lo32[i], hi = A.hi32[i];
            int r = (v < lo - band || v > hi + band) ? 1 : ((v <= lo + band || v >= hi - band) ? 2 : 0);
            if (r == 2) {  // decide in FP64
              const double v64 = pos64<KIND>(A, s0 + k, k, x64, i);
              r = (v64 >= A.ev.lo[i] && v64 <= A.ev.hi[i]) ? 0 : 1;
              rechecked = true;
            }
            bt |= r;
          }
          if (bt) {
            j_oob = k - kk;
            break;
          }
        }
      }
      const int nst = (!done && !collided) ? min(kend - kk, j_oob) : 0;
      if (nst == 0) nc = 0;
      nsts |= (uint32_t)nst << (5 * G);
      ncs |= (uint32_t)nc << (8 * G);
      n_lane += nc;
      if (!done && j_oob < CH) {  // later states of this lane are never tested
        first_oob = kk + j_oob;
        done = true;
      }
      G++;
      kk = kend;
      if (G >= GL || kk >= L) break;
      if (__reduce_add_sync(kFull, (unsigned)n_lane) >= (unsigned)kSlotFill) break;
    }
    const int nS = kk - k0;  // states of the round, <= 32 (<= MGS with min_gap)
    // the narrow phase as (lane, chunk, candidate) slots
    int pre = n_lane;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int v = __shfl_up_sync(kFull, pre, d);
      if (lane >= d) pre += v;
    }
    const int T = __shfl_sync(kFull, pre, 31);
    pre -= n_lane;  // exclusive prefix
    if (T > 0) {
      for (int e = lane; e < nS * PARTS; e += 32) {
        const int j = e / PARTS, q = e % PARTS;
        const Pose<float> ps = pose[(int64_t)q * pv.S + s0 + k0 + j];
        S.pose[e] = ps;
        const float ac = fabsf(ps.c), as = fabsf(ps.s);
        S.ext[e] = make_float2(hl * ac + hw * as, hl * as + hw * ac);
      }
      if (want_mg)
        for (int j = 0; j < nS; j++) S.mg[j][lane] = ord_gap(INFINITY);
      S.hit[lane] = 0u;
      S.rc[lane] = 0u;
      __syncwarp();
      for (int base = 0; base < T; base += 32) {
        const int t = base + lane;
        int owner = 0;  // the last lane whose exclusive prefix is <= t
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
          const int cand = owner + step;
          const int pv_ = __shfl_sync(kFull, pre, cand & 31);
          if (cand < 32 && pv_ <= t) owner = cand;
        }
        const int opre = __shfl_sync(kFull, pre, owner);
        const uint32_t onsts = __shfl_sync(kFull, nsts, owner);
        const uint32_t oncs = __shfl_sync(kFull, ncs, owner);
        const uint32_t onode = __shfl_sync(kFull, node, owner);
        float osh[D + V];
#pragma unroll
        for (int i = 0; i < D + V; i++) osh[i] = __shfl_sync(kFull, off[i], owner);
        if (t < T) {
          // the slot's chunk g and candidate index within it
          int cidx = t - opre, g = 0;
          for (; g < Scratch::GMAX - 1; g++) {
            const int c = (oncs >> (8 * g)) & 255u;
            if (cidx < c) break;
            cidx -= c;
          }
          const int onst = (onsts >> (5 * g)) & 31u;
          int o = -1;
#pragma unroll
          for (int w = 0; w < NW; w++) {
            if (o < 0) {
              const uint32_t ow = S.cm[g][w][owner];
              const int c = __popc(ow);
              if (cidx < c) o = 32 * w + (int)__fns(ow, 0u, cidx + 1);
              else cidx -= c;
            }
          }
          if (o >= 0 && o < n_obs) {
            const double *ox64 = A.nv.x64 + (int64_t)onode * R::NX;
            using Ob = std::conditional_t<R::SPHERE, Obs3<float>, Obs2<float>>;
            const Ob ob = ((const Ob *)obs_sm)[o];
            const int sb = g * CH;  // the chunk's first state in the round
            for (int j = 0; j < onst; j++) {
              const int sj = sb + j, k = k0 + sj;
              float sx = osh[0], sy = osh[1], sz = 0.f;
              if (V) {
                const float tk = float(k) * dt;
                sx += tk * osh[D + 0];
                sy += tk * osh[D + 1];
                if (D == 3) sz = osh[2] + tk * osh[D + 2];
              } else if (D == 3) {
                sz = osh[2];
              }
              float gmin = INFINITY;
              bool hit = false;
#pragma unroll
              for (int q = 0; q < PARTS; q++) {
                int r;
                const Pose<float> ps = S.pose[sj * PARTS + q];
                if constexpr (R::SPHERE) {
                  r = sphere_test<float, true>(ps.cx + sx, ps.cy + sy, ps.c + sz, ob, rad, band, gmin);
                } else {
                  // axis-aligned reject first; the oriented axes only within the band
                  const float2 ex = S.ext[sj * PARTS + q];
                  const float dx = ps.cx + sx - ob.cx, dy = ps.cy + sy - ob.cy;
                  const float ga = fmaxf(fabsf(dx) - (ex.x + ob.hx), fabsf(dy) - (ex.y + ob.hy));
                  gmin = fminf(gmin, ga);
                  if (ga > band) {
                    r = 0;
                  } else {
                    float unused = INFINITY;
                    r = planar_test<float, true>(ps.cx + sx, ps.cy + sy, ps.c, ps.s, ex.x, ex.y, ob, hl, hw, band,
                                                 unused);
                  }
                }
                if (r == 2) {  // decide in FP64
                  r = gap64<KIND>(A, s0, k, q, ox64, o) <= 0.0 ? 1 : 0;
                  atomicOr(&S.rc[owner], 1u << sj);
                }
                hit |= r == 1;
              }
              // gaps above the cap are reported as +inf: only smaller ones are merged
              if (want_mg && gmin <= kGapCap) atomicMin(&S.mg[sj][owner], ord_gap(gmin));
              if (hit) {
                atomicOr(&S.hit[owner], 1u << sj);
                break;  // later states of this candidate lie past the lane's first contact
              }
            }
          }
        }
      }
      __syncwarp();
      if (n_lane > 0) {
        const unsigned h = S.hit[lane];
        const int last = h ? __ffs(h) - 1 : nS - 1;
        if (want_mg)
          for (int j = 0; j <= last; j++) mg = fminf(mg, unord_gap(S.mg[j][lane]));
        if (S.rc[lane] & (last >= 31 ? 0xffffffffu : ((2u << last) - 1u))) rechecked = true;
        if (h) {
          collided = true;
          first_col = k0 + last;
        }
      }
      __syncwarp();  // the next round reuses the scratch
    }
    if (!done && collided && !need_bounds) done = true;
    k0 = kk;
  }

  const unsigned rmask = __ballot_sync(kFull, active && rechecked);
  if (lane == 0 && rmask) atomicAdd(&A.ctr->n_recheck, (unsigned long long)__popc(rmask));
  if (!active) return;
  const PairView &o = A.out;
  if (A.perm) o.node[pair] = A.perm[node];
  uint8_t verdict;
  int fi;
  if (first_oob < L) { verdict = DPG_OUT_OF_BOUNDS; fi = first_oob; }
  else if (collided) { verdict = DPG_COLLISION; fi = first_col; }
  else { verdict = DPG_VALID; fi = L; }
  const int er = first_oob < L ? first_oob : L - 1;  // end-state row
  const int64_t row_out = o.out_index ? (int64_t)o.out_index[pair] : pair;
  if (o.node_host) {
    o.node_host[row_out] = A.perm ? A.perm[node] : node;
    o.prim_host[row_out] = (uint32_t)p;
  }
  if (o.verdict) o.verdict[row_out] = verdict;
  if (o.first_invalid) o.first_invalid[row_out] = (int16_t)fi;
  if (o.min_gap)
    o.min_gap[row_out] = verdict == DPG_OUT_OF_BOUNDS ? __int_as_float(0x7fc00000)
                                                   : (mg <= kGapCap ? mg : __int_as_float(0x7f800000));
  if (o.flags) o.flags[row_out] = rechecked ? DPG_FLAG_CONTACT_RECHECK : 0;
  if (o.end_state) {
    if constexpr (ES64) {
      double *es = (double *)o.end_state + row_out * R::NX;
      const double t = double(er) * rp.dt;
      const double *xs = pv.st64 + (s0 + er) * R::NX;
#pragma unroll
      for (int c = 0; c < R::NX; c++) {
        double v = xs[c];
        if (c < D) {
          v += x64[c];
          if (V) v += t * x64[R::vel_comp(c)];
        }
#pragma unroll
        for (int i = 0; i < V; i++)
          if (c == R::vel_comp(i)) v += x64[R::vel_comp(i)];
        es[c] = v;
      }
    } else {
      float *es = (float *)o.end_state + row_out * R::NX;
      const float t = float(er) * dt;
      const int64_t row = s0 + er;
#pragma unroll
      for (int c = 0; c < R::NX; c++) {
        float v = pv.st32[row * R::NX + c];
        if (c < D) {
          v += off[c];
          if (V) v += t * off[D + c];
        }
#pragma unroll
        for (int i = 0; i < V; i++)
          if (c == R::vel_comp(i)) v += off[D + i];
        es[c] = v;
      }
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

// Persistent warps over (primitive, 32 nodes) work items.
// SLOTS: the slot-parallel narrow phase (FP32 tests with the band, NW > 0);
// its per-warp scratch follows the obstacles at A.slot_offset.
template <int KIND, class Real, bool BAND, int NW, bool ES64 = false, bool SLOTS = false>
__global__ void __launch_bounds__(kCheckThreads, SLOTS ? Robot<KIND>::SLOT_BLOCKS : Robot<KIND>::CHECK_BLOCKS)
    check_pairs(CheckArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  load_obstacles<Real, KIND>(A.ev, smem);
  const int lane = threadIdx.x & 31;
  const int P = A.pv.P;
  const unsigned long long n_all = A.ctr->n_items;
  const int nsub = A.nsub > 0 ? A.nsub : 1;
  const unsigned long long i_lo = nsub > 1 ? n_all * A.sub_cum[A.sub] / A.sub_cum[nsub] : 0ull;
  const unsigned long long n_items = nsub > 1 ? n_all * A.sub_cum[A.sub + 1] / A.sub_cum[nsub] : n_all;
  int cur_range = -1;        // progress-driven copies: the range of this warp's items,
  unsigned long long cur_cnt = 0;  // and how many of them it finished
  auto flush_range = [&]() {  // warp-uniform
    if (cur_cnt == 0) return;
    __threadfence();  // this lane's result writes, before the count
    __syncwarp();
    if (lane == 0) {
      const int nr = A.n_ranges, tot = A.sub_cum[nr], j = cur_range;
      const unsigned long long lo = n_all * A.sub_cum[j] / tot;
      const unsigned long long hi = j + 1 == nr ? n_all : n_all * A.sub_cum[j + 1] / tot;
      if (atomicAdd(&A.ctr->range_done[j], cur_cnt) + cur_cnt == hi - lo) {
        __threadfence_system();
        reinterpret_cast<volatile int *>(A.range_flag)[j] = 1;
      }
    }
    cur_cnt = 0;
  };
  while (true) {
    unsigned long long item = 0;
    int stop = 0;
    if (lane == 0) {
      stop = *A.abort_flag;
      item = stop ? n_items : i_lo + atomicAdd(&A.ctr->next_sub[A.sub], 1ull);
    }
    item = __shfl_sync(kFull, item, 0);
    stop = __shfl_sync(kFull, stop, 0);
    if (stop) {
      if (lane == 0) A.ctr->status = DPG_ERR_ABORTED;
      break;
    }
    if (item >= n_items) break;
    if (A.n_ranges > 1) {
      const int nr = A.n_ranges, tot = A.sub_cum[nr];
      int j = 0;
      while (j + 1 < nr && item >= n_all * A.sub_cum[j + 1] / tot) j++;
      if (j != cur_range) {
        flush_range();
        cur_range = j;
      }
      cur_cnt++;
    }
    // order position lo with ord_ibase[lo] <= item < ord_ibase[lo + 1]
    int lo = 0;
    if (A.item_pos) {
      lo = (int)A.item_pos[item];
    } else {
      int hi = P;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (A.ord_ibase[mid] <= item) lo = mid; else hi = mid;
      }
    }
    const int p = A.pv.order[lo];
    const unsigned long long j = item - A.ord_ibase[lo];
    const unsigned long long first = A.ord_pbase[lo] + 32ull * j;
    const unsigned long long end = A.ord_pbase[lo + 1];
    const unsigned long long pair = first + lane;
    const bool active = pair < end;
    const uint32_t node = active ? A.out.node[pair] : 0u;
    if constexpr (SLOTS) {
      using Scratch = SlotScratch<Robot<KIND>::CHUNK, Robot<KIND>::PARTS, NW>;
      Scratch *scr = reinterpret_cast<Scratch *>(smem + A.slot_offset) + (threadIdx.x >> 5);
      check_one_slots<KIND, NW, ES64>(A, smem, *scr, p, (int64_t)pair, node, active);
    } else {
      check_one<KIND, Real, BAND, NW, true, ES64>(A, smem, p, (int64_t)pair, node, active);
    }
  }
  if (A.n_ranges > 1) flush_range();
}

}  // namespace dpg
