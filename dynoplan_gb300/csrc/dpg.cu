// dpg.cu -- host side of the C ABI in include/dpg.h: contexts, device
// tables, and the launch sequence of one batched expansion.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <mutex>
#include <vector>

#include "dpg.h"
#include "check_kernels.cuh"
#include "dpg_mlp.h"
#include "mlp_kernels.cuh"

#include "check_list.h"
#include "ctx.h"

using namespace dpg;

namespace {

int fail(dpg_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}

#define CUDA_TRY(ctx, call)                                                        \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return fail((ctx), e_ == cudaErrorMemoryAllocation ? DPG_ERR_OOM : DPG_ERR_CUDA, \
                  std::string(#call) + ": " + cudaGetErrorString(e_));             \
  } while (0)

int ensure(dpg_ctx *c, DevBuf &b, size_t bytes) {
  if (b.bytes >= bytes && b.p) return DPG_OK;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
  size_t want = std::max<size_t>(bytes, 256);
  cudaError_t e = cudaMalloc(&b.p, want);
  if (e != cudaSuccess) {
    b.p = nullptr;
    return fail(c, DPG_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  b.bytes = want;
  return DPG_OK;
}

void release(DevBuf &b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
}

template <class T> T *P_(DevBuf &b) { return static_cast<T *>(b.p); }

bool kind_ok(int k) { return k >= DPG_ROBOT_UNICYCLE1 && k <= DPG_ROBOT_QUAD2D; }

RobotParams to_params(const dpg_robot_desc &r) {
  RobotParams p{};
  p.dt = r.dt;
  for (int i = 0; i < 4; i++) p.w[i] = r.w[i];
  p.half_len = 0.5 * r.box[0];
  p.half_wid = 0.5 * r.box[1];
  p.hitch = r.hitch;
  p.wheelbase = r.wheelbase;
  p.radius = r.radius;
  p.mass = r.mass;
  p.lever = r.arm / std::sqrt(2.0);
  p.t2t = r.t2t;
  for (int i = 0; i < 3; i++) p.inertia[i] = r.inertia[i];
  p.ang_gain = r.ang_gain;
  p.g = r.g;
  return p;
}

int pos_dim(int kind) { return kind == DPG_ROBOT_QUAD3D ? 3 : 2; }

int key_dim(int kind) {
  switch (kind) {
    case DPG_ROBOT_UNICYCLE1: return Robot<DPG_ROBOT_UNICYCLE1>::KEYD;
    case DPG_ROBOT_CAR1: return Robot<DPG_ROBOT_CAR1>::KEYD;
    case DPG_ROBOT_QUAD2D: return Robot<DPG_ROBOT_QUAD2D>::KEYD;
    default: return Robot<DPG_ROBOT_QUAD3D>::KEYD;
  }
}
int off_dim(int kind) {
  switch (kind) {
    case DPG_ROBOT_QUAD2D: return 4;
    case DPG_ROBOT_QUAD3D: return 6;
    default: return 2;
  }
}
bool is_rollout(int kind) { return kind == DPG_ROBOT_QUAD2D || kind == DPG_ROBOT_QUAD3D; }

// dispatch a functor templated on the robot kind
template <class F> void with_kind(int kind, F &&f) {
  switch (kind) {
    case DPG_ROBOT_UNICYCLE1: f(std::integral_constant<int, DPG_ROBOT_UNICYCLE1>{}); break;
    case DPG_ROBOT_CAR1: f(std::integral_constant<int, DPG_ROBOT_CAR1>{}); break;
    case DPG_ROBOT_QUAD3D: f(std::integral_constant<int, DPG_ROBOT_QUAD3D>{}); break;
    case DPG_ROBOT_QUAD2D: f(std::integral_constant<int, DPG_ROBOT_QUAD2D>{}); break;
  }
}

}  // namespace

// The exact check of the pair list on `st`: lockstep warps over (primitive,
// 32 nodes) items, with obstacle culling when the candidate masks cover
// every obstacle.
// prec: DPG_FP32 (FP32 tests, FP64 decisions in the band, FP32 end states),
// DPG_FP64 (the same tests, FP64 end states), DPG_FP64_STRICT (every test in
// FP64).
template <int KIND>
static void launch_check(dpg_ctx *c, const CheckArgs &ca, int prec, cudaStream_t st) {
  const bool fp64 = prec == DPG_FP64_STRICT;
  using R = Robot<KIND>;
  // obstacle bitmask words per lane: the fewest that cover the obstacles
  // (fewer registers), none above kMaxCullObs (no culling)
  const int nw = c->n_obs <= 32 ? 1 : c->n_obs <= 64 ? 2 : c->n_obs <= 96 ? 3 : c->n_obs <= kMaxCullObs ? 4 : 0;
  const size_t ob = fp64 ? (R::SPHERE ? sizeof(Obs3<double>) : sizeof(Obs2<double>))
                         : (R::SPHERE ? sizeof(Obs3<float>) : sizeof(Obs2<float>));
  const size_t sm_obs = (ob * std::max(c->n_obs, 1) + 15) / 16 * 16;
  // the slot-parallel narrow phase for FP32 tests with culling
  const bool slots = !fp64 && nw > 0 && c->tune.check_variant == DPG_CHECK_SLOTS;
  CheckArgs a = ca;
  a.slot_offset = (int)sm_obs;
  auto go = [&](auto kern, size_t scratch = 0) {
    const size_t sm = sm_obs + scratch * (kCheckThreads / 32);
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCheckThreads, sm);
    if (c->tune.check_blocks_per_sm > 0) per_sm = std::min(per_sm, c->tune.check_blocks_per_sm);
    kern<<<c->sm_count * std::max(per_sm, 1), kCheckThreads, sm, st>>>(a);
  };
  auto by_words = [&](auto real, auto band, auto es64) {
    using Real = decltype(real);
    constexpr bool BAND = decltype(band)::value, ES64 = decltype(es64)::value;
    constexpr bool F32 = sizeof(Real) == 4;
    switch (nw) {
      case 1: slots ? go(check_pairs<KIND, Real, BAND, 1, ES64, F32>, slot_scratch_bytes<KIND, 1>()) : go(check_pairs<KIND, Real, BAND, 1, ES64>); break;
      case 2: slots ? go(check_pairs<KIND, Real, BAND, 2, ES64, F32>, slot_scratch_bytes<KIND, 2>()) : go(check_pairs<KIND, Real, BAND, 2, ES64>); break;
      case 3: slots ? go(check_pairs<KIND, Real, BAND, 3, ES64, F32>, slot_scratch_bytes<KIND, 3>()) : go(check_pairs<KIND, Real, BAND, 3, ES64>); break;
      case 4: slots ? go(check_pairs<KIND, Real, BAND, 4, ES64, F32>, slot_scratch_bytes<KIND, 4>()) : go(check_pairs<KIND, Real, BAND, 4, ES64>); break;
      default: go(check_pairs<KIND, Real, BAND, 0, ES64>); break;
    }
  };
  if (fp64) by_words(0.0, std::false_type{}, std::false_type{});
  else if (prec == DPG_FP64) by_words(0.0f, std::true_type{}, std::true_type{});
  else by_words(0.0f, std::true_type{}, std::false_type{});
}

static bool prec_ok(int p) { return p == DPG_FP32 || p == DPG_FP64 || p == DPG_FP64_STRICT; }

// primitive tiles per nn_mask block: small node batches are split over the
// primitives too, for about two blocks per SM
static int nn_tiles_per_y(int P, int64_t B, int sm_count) {
  const int ntiles = std::max(1, (P + kNNTile - 1) / kNNTile);
  const int64_t want = std::max<int64_t>(1, (2 * (int64_t)sm_count + B - 1) / std::max<int64_t>(B, 1));
  const int y = (int)std::min<int64_t>(ntiles, want);
  return (ntiles + y - 1) / y;
}

// Ball scan of the nv.N nodes against the pv.P primitives: bitmask words
// (P x Wpad, primitive-major), per-tile counts cnt[B][P] turned into prefixes,
// totals tot[P].
// Batches of at least tune.grid_min_nodes nodes of a robot with a key grid test only the
// primitives of the cells near their key; smaller batches test every
// primitive (split over the primitives too, to fill the GPU).  Both give the
// same mask and counts.
// (an expand whose results go to host buffers runs tune.pipe_launches <=
// kMaxSub check launches, one work-queue counter each)

constexpr size_t kMinCopyBytes = 16u << 20;  // smallest group of copy ranges copied together

// Cumulative item weights of the copy ranges of a host-buffer expand: each
// range `decay` times the one before, so a range's result copy overlaps the
// next ranges' check and the last, exposed copy is small.  The decay follows
// the ratio of copy time to check time (dpg_expand adapts it after each call:
// car1's copies take about 0.6 of its check, so 3/4; the quadrotor's about as
// long as its check, so equal ranges).  cum[0] = 0, cum[n] = the total.
static void pipe_weights(int n, int *cum, double decay) {
  cum[0] = 0;
  double w = 1000.0;
  for (int j = 0; j < n; j++) {
    cum[j + 1] = cum[j] + (int)w;
    w *= decay;
  }
}
template <int KIND>
static void launch_ball(const dpg_ctx *c, const PrimView &pv, const NodeView &nv, double radius, double ball_band,
                        int64_t Wpad, int64_t B, int64_t W, uint32_t *mask, uint32_t *cnt, uint32_t *tot,
                        DevCounters *ctr, cudaStream_t st, bool allow_grid = true) {
  using R = Robot<KIND>;
  const RobotParams &rp = c->rp;
  const int P = pv.P;
  const float4 w32 = make_float4((float)rp.w[0], (float)rp.w[1], (float)rp.w[2], (float)rp.w[3]);
  bool done = false;
  if constexpr (R::KEYD <= 2) {
    if (allow_grid && c->kg.n0 > 0 && nv.N >= c->tune.grid_min_nodes) {
      // half-width of the cell range along a key component: radius plus band
      // over its weight, widened; -1 = every cell
      auto half = [&](double wk, bool periodic) -> float {
        const double h = (radius + ball_band) / wk * (1.0 + 1e-4) + 1e-3;
        if (!(wk > 0) || !std::isfinite(h) || (periodic && h >= kPi)) return -1.f;
        return (float)h;
      };
      const float h0 = half(rp.w[1], true);
      const float h1 = half(KIND == DPG_ROBOT_CAR1 ? rp.w[2] : rp.w[3], KIND == DPG_ROBOT_CAR1);
      cudaMemsetAsync(mask, 0, sizeof(uint32_t) * (size_t)P * Wpad, st);
      if (P <= kGridSmemP) {
        nn_grid<KIND, true><<<(unsigned)B, kNNThreads, sizeof(uint32_t) * P, st>>>(
            rp, pv, nv, c->kg, w32, (float)radius, radius, (float)ball_band, h0, h1, Wpad, mask, cnt, ctr);
      } else {
        cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * (size_t)B * P, st);
        nn_grid<KIND, false><<<(unsigned)B, kNNThreads, 0, st>>>(rp, pv, nv, c->kg, w32, (float)radius, radius,
                                                                 (float)ball_band, h0, h1, Wpad, mask, cnt, ctr);
      }
      done = true;
    }
  }
  if (!done) {
    const int tpy = nn_tiles_per_y(P, B, c->sm_count);
    const dim3 ng((unsigned)B, (unsigned)((P + tpy * kNNTile - 1) / (tpy * kNNTile)));
    nn_mask<KIND><<<ng, kNNThreads, 0, st>>>(rp, pv, nv, w32, (float)radius, radius, (float)ball_band, Wpad, tpy,
                                             mask, cnt, ctr);
  }
  nn_prefix<<<(unsigned)((P + 31) / 32), 256, 0, st>>>(P, (int)B, cnt, tot);
}

extern "C" {

int dpg_abi_version(void) { return DPG_ABI_VERSION; }

const char *dpg_errstr(int code) {
  switch (code) {
    case DPG_OK: return "ok";
    case DPG_ERR_ARG: return "invalid argument";
    case DPG_ERR_OOM: return "out of memory";
    case DPG_ERR_CUDA: return "CUDA error";
    case DPG_ERR_TIMEOUT: return "device wait timed out";
    case DPG_ERR_ABORTED: return "aborted";
    case DPG_ERR_CAPACITY: return "output capacity too small";
    case DPG_ERR_STATE: return "invalid call order";
    case DPG_ERR_NODEVICE: return "no usable CUDA device";
  }
  return "unknown error";
}

int dpg_robot_default(int32_t kind, dpg_robot_desc *r) {
  if (!r || !kind_ok(kind)) return DPG_ERR_ARG;
  std::memset(r, 0, sizeof(*r));
  r->kind = kind;
  r->g = 9.81;
  switch (kind) {
    case DPG_ROBOT_UNICYCLE1:
      r->nx = 3; r->nu = 2; r->n_parts = 1; r->dt = 0.1;
      r->w[0] = 1.0; r->w[1] = 0.5;
      r->box[0] = 0.5; r->box[1] = 0.25;
      break;
    case DPG_ROBOT_CAR1:
      r->nx = 4; r->nu = 2; r->n_parts = 2; r->dt = 0.1;
      r->w[0] = 1.0; r->w[1] = 0.5; r->w[2] = 0.5;
      r->box[0] = 0.5; r->box[1] = 0.25;
      r->hitch = 0.5; r->wheelbase = 0.25;
      break;
    case DPG_ROBOT_QUAD3D:
      r->nx = 13; r->nu = 4; r->n_parts = 1; r->dt = 0.01;
      r->w[0] = 1.0; r->w[1] = 0.5; r->w[2] = 0.1; r->w[3] = 0.05;
      r->radius = 0.1; r->mass = 0.034; r->arm = 0.046; r->t2t = 0.006;
      r->inertia[0] = 16.571710e-6; r->inertia[1] = 16.655602e-6; r->inertia[2] = 29.261652e-6;
      break;
    case DPG_ROBOT_QUAD2D:
      r->nx = 6; r->nu = 2; r->n_parts = 1; r->dt = 0.01;
      r->w[0] = 1.0; r->w[1] = 0.5; r->w[2] = 0.2; r->w[3] = 0.1;
      r->box[0] = 0.5; r->box[1] = 0.25;
      r->ang_gain = 34.0;
      break;
  }
  return DPG_OK;
}

int dpg_create(dpg_ctx **out, int device, const dpg_robot_desc *robot) {
  if (!out || !robot || !kind_ok(robot->kind)) return DPG_ERR_ARG;
  *out = nullptr;
  dpg_robot_desc def;
  dpg_robot_default(robot->kind, &def);
  if (robot->nx != def.nx || robot->nu != def.nu || robot->n_parts != def.n_parts || !(robot->dt > 0))
    return DPG_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) return DPG_ERR_NODEVICE;
  dpg_ctx *c = new (std::nothrow) dpg_ctx();
  if (!c) return DPG_ERR_OOM;
  c->device = device;
  c->robot = *robot;
  c->rp = to_params(*robot);
  int rc = DPG_OK;
  do {
    if (cudaSetDevice(device) != cudaSuccess) { rc = DPG_ERR_NODEVICE; break; }
    if (cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
      rc = DPG_ERR_NODEVICE; break;
    }
    // a blocking stream: ordered after the caller's work on the legacy
    // default stream, which produces device-resident inputs
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamDefault) != cudaSuccess) { rc = DPG_ERR_CUDA; break; }
    if (cudaMalloc(&c->d_ctr, sizeof(DevCounters)) != cudaSuccess) { rc = DPG_ERR_OOM; break; }
    if (cudaHostAlloc(&c->h_ctr, 2 * sizeof(DevCounters), cudaHostAllocDefault) != cudaSuccess) { rc = DPG_ERR_OOM; break; }
    if (cudaHostAlloc(&c->h_abort, sizeof(int), cudaHostAllocMapped) != cudaSuccess) { rc = DPG_ERR_OOM; break; }
    *c->h_abort = 0;
    if (cudaHostGetDevicePointer(&c->d_abort, c->h_abort, 0) != cudaSuccess) { rc = DPG_ERR_CUDA; break; }
    for (auto &e : c->ev)
      if (cudaEventCreate(&e) != cudaSuccess) { rc = DPG_ERR_CUDA; break; }
  } while (0);
  if (rc != DPG_OK) {
    dpg_destroy(c);
    return rc;
  }
  *out = c;
  return DPG_OK;
}

void dpg_destroy(dpg_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->cstream) cudaStreamSynchronize(c->cstream);
  if (c->xstream) cudaStreamSynchronize(c->xstream);
  DevBuf *bufs[] = {&c->len, &c->soff, &c->aoff, &c->order, &c->key32, &c->kconst32, &c->st64,
                    &c->st32, &c->act64, &c->pose32, &c->pose64, &c->pbox, &c->pbox32, &c->obs32, &c->obs64,
                    &c->x64, &c->nkey32, &c->noff32, &c->mask, &c->cnt, &c->tot, &c->pbase,
                    &c->ord_pbase, &c->ord_ibase, &c->item_pos, &c->p_node, &c->p_prim, &c->p_verdict, &c->p_fi,
                    &c->p_end, &c->p_gap, &c->p_flags, &c->coff, &c->cbox32, &c->tbox32,
                    &c->q_node, &c->q_prim, &c->q_sorted, &c->q_idx, &c->q_fill,
                    &c->ord_cell, &c->ord_perm, &c->ord_cnt, &c->ord_start, &c->ord_rank, &c->ord_tiles, &c->x64s,
                    &c->kg_start, &c->kg_tab, &c->lz_off, &c->lz_cnt, &c->lz_cur, &c->lz_next, &c->lz_valid,
                    &c->lz_rank, &c->lz_lnode, &c->lz_ldest, &c->lz_ctr, &c->lz_table, &c->rkey32, &c->rkconst32, &c->rkrow};
  for (DevBuf *b : bufs) release(*b);
  if (c->d_ctr) cudaFree(c->d_ctr);
  if (c->h_ctr) cudaFreeHost(c->h_ctr);
  if (c->h_bases) cudaFreeHost(c->h_bases);
  if (c->h_lz) cudaFreeHost(c->h_lz);
  if (c->h_rflag) cudaFreeHost(c->h_rflag);
  for (auto &e : c->ev_sub)
    if (e) cudaEventDestroy(e);
  if (c->ev_tot) cudaEventDestroy(c->ev_tot);
  if (c->ev_ball) cudaEventDestroy(c->ev_ball);
  for (auto &e : c->ev_cl)
    if (e) cudaEventDestroy(e);
  if (c->cstream) cudaStreamDestroy(c->cstream);
  if (c->xstream) cudaStreamDestroy(c->xstream);
  if (c->h_abort) cudaFreeHost(c->h_abort);
  for (auto &e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char *dpg_last_error(const dpg_ctx *c) { return c ? c->err.c_str() : "null context"; }

}  // extern "C"

// Host index, raw device tables and every derived table of a primitive set.
// `states` / `actions` are host arrays (H2D) or device arrays (D2D, `kind`).
// Key-space grid of the primitives for robots with one or two key
// components: about two primitives per cell, primitives listed by cell in
// id order.  Built from the device key table the ball scan reads, so a
// primitive's cell is that of the key it is tested with.
static int build_key_grid(dpg_ctx *c, int P) {
  const int kind = c->robot.kind, kd = key_dim(kind);
  c->kg = KeyGrid{};
  if (kd > 2) return DPG_OK;
  std::vector<float> key((size_t)kd * P), kc(P);
  CUDA_TRY(c, cudaMemcpy(key.data(), c->key32.p, sizeof(float) * kd * P, cudaMemcpyDeviceToHost));
  CUDA_TRY(c, cudaMemcpy(kc.data(), c->kconst32.p, sizeof(float) * P, cudaMemcpyDeviceToHost));
  KeyGrid g{};
  if (kd == 1) {
    g.n0 = std::clamp(P / 2, 1, 4096);
    g.n1 = 1;
  } else {
    g.n0 = g.n1 = std::clamp((int)std::lround(std::sqrt(P / 2.0)), 1, 128);
  }
  const bool per1 = kind == DPG_ROBOT_CAR1;
  g.inv0 = (float)(g.n0 / kTwoPi);
  if (kd > 1 && per1) {
    g.inv1 = (float)(g.n1 / kTwoPi);
  } else if (kd > 1) {
    float lo = 0.f, hi = 0.f;
    bool any = false;
    for (int p = 0; p < P; p++) {
      const float k = key[(size_t)P + p];
      if (!std::isfinite(k)) continue;
      lo = any ? std::min(lo, k) : k;
      hi = any ? std::max(hi, k) : k;
      any = true;
    }
    g.lo1 = lo;
    g.inv1 = hi > lo ? (float)(g.n1 / ((double)hi - lo)) : 0.f;
  }
  // same float arithmetic as the query's ranges; NaN keys (never members) in cell 0
  auto cell = [](float f, int n) { return std::isfinite(f) ? kg_clamp((int)std::max(-1.f, std::min(f, (float)n)), n) : 0; };
  const float piF = 3.14159265f;
  const int ncell = g.n0 * g.n1;
  std::vector<uint32_t> cid(P), start(ncell + 1, 0u);
  for (int p = 0; p < P; p++) {
    const int c0 = cell(std::floor((key[p] + piF) * g.inv0), g.n0);
    int c1 = 0;
    if (kd > 1) {
      const float k1 = key[(size_t)P + p];
      c1 = per1 ? cell(std::floor((k1 + piF) * g.inv1), g.n1) : cell(std::floor((k1 - g.lo1) * g.inv1), g.n1);
    }
    cid[p] = (uint32_t)(c0 * g.n1 + c1);
    start[cid[p] + 1]++;
  }
  for (int i = 0; i < ncell; i++) start[i + 1] += start[i];
  std::vector<float4> tab(P);
  std::vector<uint32_t> fill(start.begin(), start.end() - 1);
  for (int p = 0; p < P; p++) {
    float id;
    std::memcpy(&id, &p, sizeof id);
    tab[fill[cid[p]]++] = make_float4(key[p], kd > 1 ? key[(size_t)P + p] : 0.f, kc[p], id);
  }
  int rc;
  if ((rc = ensure(c, c->kg_start, sizeof(uint32_t) * (ncell + 1))) ||
      (rc = ensure(c, c->kg_tab, sizeof(float4) * P)))
    return rc;
  CUDA_TRY(c, cudaMemcpy(c->kg_start.p, start.data(), sizeof(uint32_t) * (ncell + 1), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(c->kg_tab.p, tab.data(), sizeof(float4) * P, cudaMemcpyHostToDevice));
  g.start = P_<uint32_t>(c->kg_start);
  g.tab = P_<float4>(c->kg_tab);
  c->kg = g;
  return DPG_OK;
}

static int load_tables(dpg_ctx *c, int32_t P, const int32_t *len, const double *states, const double *actions,
                       cudaMemcpyKind copy) {
  const int nx = c->robot.nx, nu = c->robot.nu, kind = c->robot.kind;
  c->h_len.assign(len, len + P);
  c->h_soff.resize(P);
  c->h_aoff.resize(P);
  c->h_coff.resize(P);
  int64_t S = 0, A = 0, NC = 0;
  int chunk = 0;
  with_kind(kind, [&](auto K) { chunk = Robot<decltype(K)::value>::CHUNK; });
  for (int p = 0; p < P; p++) {
    if (len[p] < 1 || len[p] > 32767) return fail(c, DPG_ERR_ARG, "upload_primitives: length out of [1, 32767]");
    c->h_soff[p] = S;
    c->h_aoff[p] = A;
    c->h_coff[p] = NC;
    NC += (len[p] + chunk - 1) / chunk;
    S += len[p];
    A += len[p] - 1;
  }
  c->h_order.resize(P);
  std::iota(c->h_order.begin(), c->h_order.end(), 0);
  std::stable_sort(c->h_order.begin(), c->h_order.end(),
                   [&](int a, int b) { return c->h_len[a] > c->h_len[b]; });
  CUDA_TRY(c, cudaSetDevice(c->device));
  int rc;
  const int pd = pos_dim(kind), kd = key_dim(kind), parts = c->robot.n_parts;
  if ((rc = ensure(c, c->len, sizeof(int32_t) * P)) ||
      (rc = ensure(c, c->soff, sizeof(int64_t) * P)) ||
      (rc = ensure(c, c->aoff, sizeof(int64_t) * P)) ||
      (rc = ensure(c, c->order, sizeof(int32_t) * P)) ||
      (rc = ensure(c, c->key32, sizeof(float) * kd * P)) ||
      (rc = ensure(c, c->kconst32, sizeof(float) * P)) ||
      (rc = ensure(c, c->st64, sizeof(double) * nx * S)) ||
      (rc = ensure(c, c->st32, sizeof(float) * nx * S)) ||
      (rc = ensure(c, c->act64, sizeof(double) * nu * std::max<int64_t>(A, 1))) ||
      (rc = ensure(c, c->pose32, sizeof(Pose<float>) * parts * S)) ||
      (rc = ensure(c, c->pose64, sizeof(Pose<double>) * parts * S)) ||
      (rc = ensure(c, c->pbox, sizeof(double) * 2 * pd * P)) ||
      (rc = ensure(c, c->pbox32, sizeof(float) * 2 * pd * P)) ||
      (rc = ensure(c, c->coff, sizeof(int64_t) * P)) ||
      (rc = ensure(c, c->cbox32, sizeof(float) * 2 * pd * NC)) ||
      (rc = ensure(c, c->tbox32, sizeof(float) * 2 * pd * P)) ||
      (rc = ensure(c, c->rkey32, sizeof(float) * kd * P)) || (rc = ensure(c, c->rkconst32, sizeof(float) * P)) ||
      (rc = ensure(c, c->rkrow, sizeof(int64_t) * P)))
    return rc;
  std::vector<int64_t> last_row(P);
  for (int p = 0; p < P; p++) last_row[p] = c->h_soff[p] + len[p] - 1;
  cudaStream_t st = c->stream;
  CUDA_TRY(c, cudaMemcpyAsync(c->len.p, len, sizeof(int32_t) * P, cudaMemcpyHostToDevice, st));
  CUDA_TRY(c, cudaMemcpyAsync(c->soff.p, c->h_soff.data(), sizeof(int64_t) * P, cudaMemcpyHostToDevice, st));
  CUDA_TRY(c, cudaMemcpyAsync(c->aoff.p, c->h_aoff.data(), sizeof(int64_t) * P, cudaMemcpyHostToDevice, st));
  CUDA_TRY(c, cudaMemcpyAsync(c->order.p, c->h_order.data(), sizeof(int32_t) * P, cudaMemcpyHostToDevice, st));
  CUDA_TRY(c, cudaMemcpyAsync(c->coff.p, c->h_coff.data(), sizeof(int64_t) * P, cudaMemcpyHostToDevice, st));
  CUDA_TRY(c, cudaMemcpyAsync(c->rkrow.p, last_row.data(), sizeof(int64_t) * P, cudaMemcpyHostToDevice, st));
  CUDA_TRY(c, cudaMemcpyAsync(c->st64.p, states, sizeof(double) * nx * S, copy, st));
  if (A > 0) CUDA_TRY(c, cudaMemcpyAsync(c->act64.p, actions, sizeof(double) * nu * A, copy, st));
  const RobotParams rp = c->rp;
  with_kind(kind, [&](auto K) {
    constexpr int KIND = decltype(K)::value;
    if (is_rollout(KIND))
      rollout_primitives<KIND><<<(P + 127) / 128, 128, 0, st>>>(rp, P, P_<int32_t>(c->len), P_<int64_t>(c->soff),
                                                                 P_<int64_t>(c->aoff), P_<double>(c->act64),
                                                                 P_<double>(c->st64));
    build_poses<KIND><<<(unsigned)((S + 255) / 256), 256, 0, st>>>(rp, S, P_<double>(c->st64),
                                                                  P_<Pose<double>>(c->pose64),
                                                                  P_<Pose<float>>(c->pose32), P_<float>(c->st32));
    build_keys<KIND><<<(P + 127) / 128, 128, 0, st>>>(rp, P, P_<int32_t>(c->len), P_<int64_t>(c->soff),
                                                       P_<double>(c->st64), P_<float>(c->key32),
                                                       P_<float>(c->kconst32), P_<double>(c->pbox),
                                                       P_<float>(c->pbox32));
    build_keys<KIND><<<(P + 127) / 128, 128, 0, st>>>(rp, P, P_<int32_t>(c->len), P_<int64_t>(c->rkrow),
                                                       P_<double>(c->st64), P_<float>(c->rkey32),
                                                       P_<float>(c->rkconst32), nullptr, nullptr, true);
    build_chunks<KIND><<<(P + 127) / 128, 128, 0, st>>>(rp, P, P_<int32_t>(c->len), P_<int64_t>(c->soff),
                                                         P_<int64_t>(c->coff), P_<Pose<double>>(c->pose64), S,
                                                         P_<float>(c->cbox32), P_<float>(c->tbox32));
  });
  CUDA_TRY(c, cudaGetLastError());
  CUDA_TRY(c, cudaStreamSynchronize(st));
  if ((rc = build_key_grid(c, P)) != DPG_OK) return rc;
  c->P = P;
  c->S = S;
  c->A = A;
  c->have_prims = true;
  return DPG_OK;
}

extern "C" {

int dpg_upload_primitives(dpg_ctx *c, int32_t P, const int32_t *len, const double *states,
                          const double *actions) {
  if (!c) return DPG_ERR_ARG;
  if (P <= 0 || !len || !states || !actions) return fail(c, DPG_ERR_ARG, "upload_primitives: empty input");
  return load_tables(c, P, len, states, actions, cudaMemcpyHostToDevice);
}

int dpg_prepend_primitives(dpg_ctx *c, int32_t P, const int32_t *len, const double *states,
                           const double *actions) {
  if (!c) return DPG_ERR_ARG;
  if (P <= 0 || !len || !states || !actions) return fail(c, DPG_ERR_ARG, "prepend_primitives: empty input");
  if (!c->have_prims) return load_tables(c, P, len, states, actions, cudaMemcpyHostToDevice);
  const int nx = c->robot.nx, nu = c->robot.nu;
  int64_t S = 0, A = 0;
  for (int p = 0; p < P; p++) {
    if (len[p] < 1 || len[p] > 32767) return fail(c, DPG_ERR_ARG, "prepend_primitives: length out of [1, 32767]");
    S += len[p];
    A += len[p] - 1;
  }
  // the combined raw tables, new motions first; the old ones stay on the device
  // (for rollout robots their rows are the canonical rollout of the stored
  // start and actions, which the derivation reproduces exactly)
  std::vector<int32_t> all(len, len + P);
  all.insert(all.end(), c->h_len.begin(), c->h_len.end());
  CUDA_TRY(c, cudaSetDevice(c->device));
  DevBuf st{}, ac{};
  int rc;
  if ((rc = ensure(c, st, sizeof(double) * nx * (S + c->S))) ||
      (rc = ensure(c, ac, sizeof(double) * nu * std::max<int64_t>(A + c->A, 1)))) {
    release(st);
    release(ac);
    return rc;
  }
  cudaStream_t s = c->stream;
  double *st_p = P_<double>(st), *ac_p = P_<double>(ac);
  cudaError_t e = cudaMemcpyAsync(st_p, states, sizeof(double) * nx * S, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(st_p + nx * S, c->st64.p, sizeof(double) * nx * c->S, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && A > 0)
    e = cudaMemcpyAsync(ac_p, actions, sizeof(double) * nu * A, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && c->A > 0)
    e = cudaMemcpyAsync(ac_p + nu * A, c->act64.p, sizeof(double) * nu * c->A, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    release(st);
    release(ac);
    return fail(c, DPG_ERR_CUDA, std::string("prepend_primitives: ") + cudaGetErrorString(e));
  }
  rc = load_tables(c, (int32_t)all.size(), all.data(), st_p, ac_p, cudaMemcpyDeviceToDevice);
  release(st);
  release(ac);
  return rc;
}

int dpg_upload_env(dpg_ctx *c, int32_t dim, const double *lo, const double *hi, int32_t n_obs,
                   const double *obs_lo, const double *obs_hi) {
  if (!c) return DPG_ERR_ARG;
  if (dim != pos_dim(c->robot.kind)) return fail(c, DPG_ERR_ARG, "upload_env: dim does not match the robot");
  if (!lo || !hi || n_obs < 0 || (n_obs > 0 && (!obs_lo || !obs_hi)))
    return fail(c, DPG_ERR_ARG, "upload_env: missing arrays");
  const int max_obs = 4096;
  if (n_obs > max_obs) return fail(c, DPG_ERR_ARG, "upload_env: more than 4096 obstacles");
  for (int i = 0; i < dim; i++)
    if (!(lo[i] <= hi[i])) return fail(c, DPG_ERR_ARG, "upload_env: bounds lo > hi");
  CUDA_TRY(c, cudaSetDevice(c->device));
  std::vector<float> o32;
  std::vector<double> o64;
  for (int o = 0; o < n_obs; o++) {
    double cen[3], half[3];
    for (int i = 0; i < dim; i++) {
      const double a = obs_lo[(size_t)o * dim + i], b = obs_hi[(size_t)o * dim + i];
      if (!(a <= b)) return fail(c, DPG_ERR_ARG, "upload_env: obstacle lo > hi");
      cen[i] = 0.5 * (a + b);
      half[i] = 0.5 * (b - a);
    }
    for (int i = 0; i < dim; i++) { o64.push_back(cen[i]); o32.push_back((float)cen[i]); }
    for (int i = 0; i < dim; i++) { o64.push_back(half[i]); o32.push_back((float)half[i]); }
  }
  int rc;
  const size_t n32 = std::max<size_t>(o32.size(), 1), n64 = std::max<size_t>(o64.size(), 1);
  if ((rc = ensure(c, c->obs32, sizeof(float) * n32)) || (rc = ensure(c, c->obs64, sizeof(double) * n64)))
    return rc;
  if (n_obs > 0) {
    CUDA_TRY(c, cudaMemcpy(c->obs32.p, o32.data(), sizeof(float) * o32.size(), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->obs64.p, o64.data(), sizeof(double) * o64.size(), cudaMemcpyHostToDevice));
  }
  c->dim = dim;
  for (int i = 0; i < 3; i++) { c->lo[i] = i < dim ? lo[i] : 0; c->hi[i] = i < dim ? hi[i] : 0; }
  c->n_obs = n_obs;
  c->have_env = true;
  return DPG_OK;
}

int dpg_sync(dpg_ctx *c) {
  if (!c) return DPG_ERR_ARG;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return DPG_OK;
}

int dpg_set_abort(dpg_ctx *c, int32_t flag) {
  if (!c) return DPG_ERR_ARG;
  *(volatile int *)c->h_abort = flag ? 1 : 0;
  return DPG_OK;
}

void *dpg_host_alloc(size_t bytes) {
  void *p = nullptr;
  if (cudaHostAlloc(&p, std::max<size_t>(bytes, 1), cudaHostAllocDefault) != cudaSuccess) return nullptr;
  return p;
}

void dpg_host_free(void *p) {
  if (p) cudaFreeHost(p);
}

int dpg_last_timings(const dpg_ctx *c, double *t, int32_t n) {
  if (!c || !t || n < 0) return DPG_ERR_ARG;
  const int k = std::min(n, 4);
  for (int i = 0; i < k; i++) t[i] = c->timings[i];
  return k;
}

int dpg_get_tuning(const dpg_ctx *c, dpg_tuning *t) {
  if (!c || !t) return DPG_ERR_ARG;
  *t = c->tune;
  return DPG_OK;
}

int dpg_set_tuning(dpg_ctx *c, const dpg_tuning *t) {
  if (!c || !t) return DPG_ERR_ARG;
  if ((t->check_variant != DPG_CHECK_LOCKSTEP && t->check_variant != DPG_CHECK_SLOTS) ||
      t->check_blocks_per_sm < 0 || t->check_blocks_per_sm > 32 || t->grid_min_nodes < 0 ||
      t->pipe_launches < 1 || t->pipe_launches > kMaxSub ||
      (t->host_output != DPG_HOST_OUT_PIPELINED && t->host_output != DPG_HOST_OUT_DIRECT &&
       t->host_output != DPG_HOST_OUT_PROGRESS))
    return fail(c, DPG_ERR_ARG, "set_tuning: value out of range");
  c->tune = *t;
  return DPG_OK;
}

int dpg_expand(dpg_ctx *c, const dpg_expand_opts *opts, int64_t N, const double *x, dpg_expand_out *out) {
  if (!c || !opts || !out) return DPG_ERR_ARG;
  if (!c->have_prims || !c->have_env) return fail(c, DPG_ERR_STATE, "expand: upload primitives and env first");
  if (N < 0 || (N > 0 && !x)) return fail(c, DPG_ERR_ARG, "expand: bad node array");
  if (N > (int64_t)1 << 31) return fail(c, DPG_ERR_ARG, "expand: more than 2^31 nodes");
  if (!(opts->radius >= 0) || !prec_ok(opts->precision))
    return fail(c, DPG_ERR_ARG, "expand: bad radius or precision");
  if (out->capacity < 0 || out->capacity > (int64_t)0xffffffffLL)
    return fail(c, DPG_ERR_ARG, "expand: capacity out of range");
  const bool reverse = (opts->mode & DPG_MODE_REVERSE) != 0;
  if (reverse && !(opts->mode & DPG_MODE_BALL_ONLY))
    return fail(c, DPG_ERR_ARG, "expand: DPG_MODE_REVERSE gives the reverse ball only (with DPG_MODE_BALL_ONLY)");
  if (reverse && c->robot.kind != DPG_ROBOT_UNICYCLE1 && c->robot.kind != DPG_ROBOT_CAR1)
    return fail(c, DPG_ERR_ARG, "expand: the reverse ball is defined for unicycle1 and car1");
  if (*(volatile int *)c->h_abort) return fail(c, DPG_ERR_ABORTED, "expand: abort flag raised");
  CUDA_TRY(c, cudaSetDevice(c->device));
  const int kind = c->robot.kind, nx = c->robot.nx, P = c->P;
  const int kd = key_dim(kind), od = off_dim(kind);
  const int prec = opts->precision;
  const bool fp64 = prec == DPG_FP64_STRICT;  // every test in FP64
  const int64_t cap = out->capacity;
  const int64_t W = (N + 31) / 32;
  const int64_t Wpad = (W + 31) / 32 * 32;  // mask row: words of a primitive, whole emit groups
  const int64_t B = (N + kNNThreads - 1) / kNNThreads;
  const size_t es_bytes = prec != DPG_FP32 ? sizeof(double) : sizeof(float);
  cudaStream_t st = c->stream;
  int rc;
  if ((rc = ensure(c, c->x64, sizeof(double) * nx * std::max<int64_t>(N, 1))) ||
      (rc = ensure(c, c->nkey32, sizeof(float) * kd * std::max<int64_t>(N, 1))) ||
      (rc = ensure(c, c->noff32, sizeof(float) * od * std::max<int64_t>(N, 1))) ||
      (rc = ensure(c, c->mask, sizeof(uint32_t) * (size_t)std::max<int64_t>(Wpad, 32) * P)) ||
      (rc = ensure(c, c->cnt, sizeof(uint32_t) * (size_t)std::max<int64_t>(B, 1) * P)) ||
      (rc = ensure(c, c->tot, sizeof(uint32_t) * P)) ||
      (rc = ensure(c, c->pbase, sizeof(unsigned long long) * P)) ||
      (rc = ensure(c, c->ord_pbase, sizeof(unsigned long long) * (P + 1))) ||
      (rc = ensure(c, c->ord_ibase, sizeof(unsigned long long) * (P + 1))) ||
      // work items: at most one per 32 pairs of the capacity plus one partial item per primitive
      (rc = ensure(c, c->item_pos, sizeof(uint32_t) * (size_t)(std::max<int64_t>(cap, 0) / 32 + P + 1))))
    return rc;
  // batches of at least kReorderMin nodes are processed in spatial order
  const bool reorder = N >= kReorderMin;
  if (reorder &&
      ((rc = ensure(c, c->ord_cell, sizeof(uint32_t) * N)) || (rc = ensure(c, c->ord_perm, sizeof(uint32_t) * N)) ||
       (rc = ensure(c, c->ord_cnt, sizeof(uint32_t) * kOrderCells)) ||
       (rc = ensure(c, c->ord_start, sizeof(uint32_t) * kOrderCells)) ||
       (rc = ensure(c, c->ord_rank, sizeof(uint32_t) * N)) ||
       (rc = ensure(c, c->ord_tiles, sizeof(uint32_t) * kOrderCells * (size_t)((N + order_tile(N) - 1) / order_tile(N)))) ||
       (rc = ensure(c, c->x64s, sizeof(double) * nx * N))))
    return rc;
  // pair arrays: the caller's device arrays when given, else the arena
  const bool dev_out = opts->out_on_device != 0;
  const size_t capz = (size_t)std::max<int64_t>(cap, 1);
  PairView pv_out{};
  pv_out.cap = cap;
  if (dev_out) {
    if ((rc = ensure(c, c->p_node, 4 * capz)) || (rc = ensure(c, c->p_prim, 4 * capz))) return rc;
    pv_out.node = out->node ? out->node : P_<uint32_t>(c->p_node);
    pv_out.prim = out->prim ? out->prim : P_<uint32_t>(c->p_prim);
    pv_out.verdict = out->verdict;
    pv_out.first_invalid = out->first_invalid;
    pv_out.end_state = out->end_state;
    pv_out.min_gap = out->min_gap;
    pv_out.flags = out->flags;
  } else {
    if ((rc = ensure(c, c->p_node, 4 * capz)) || (rc = ensure(c, c->p_prim, 4 * capz)) ||
        (rc = ensure(c, c->p_verdict, capz)) || (rc = ensure(c, c->p_fi, 2 * capz)) ||
        (rc = ensure(c, c->p_end, es_bytes * nx * capz)) || (rc = ensure(c, c->p_gap, 4 * capz)) ||
        (rc = ensure(c, c->p_flags, capz)))
      return rc;
    pv_out.node = P_<uint32_t>(c->p_node);
    pv_out.prim = P_<uint32_t>(c->p_prim);
    pv_out.verdict = out->verdict ? P_<uint8_t>(c->p_verdict) : nullptr;
    pv_out.first_invalid = out->first_invalid ? P_<int16_t>(c->p_fi) : nullptr;
    pv_out.end_state = out->end_state ? c->p_end.p : nullptr;
    pv_out.min_gap = out->min_gap ? P_<float>(c->p_gap) : nullptr;
    pv_out.flags = out->flags ? P_<uint8_t>(c->p_flags) : nullptr;
  }

  // host outputs in page-locked memory the GPU maps (dpg_host_alloc,
  // cudaHostAlloc, cudaHostRegister): the check kernel writes every result
  // there itself, node ids and primitives included, so no copy follows it
  bool direct = false;
  if (!dev_out && c->tune.host_output == DPG_HOST_OUT_DIRECT && !(opts->mode & DPG_MODE_BALL_ONLY) && cap > 0) {
    void *hp[7] = {out->node, out->prim, out->verdict, out->first_invalid, out->end_state, out->min_gap, out->flags};
    void *dp[7] = {};
    direct = out->node && out->prim;
    for (int i = 0; i < 7 && direct; i++) {
      if (!hp[i]) continue;
      cudaPointerAttributes at{};
      if (cudaPointerGetAttributes(&at, hp[i]) != cudaSuccess || at.type != cudaMemoryTypeHost || !at.devicePointer) {
        cudaGetLastError();
        direct = false;
      } else {
        dp[i] = at.devicePointer;
      }
    }
    if (direct) {
      pv_out.node_host = static_cast<uint32_t *>(dp[0]);
      pv_out.prim_host = static_cast<uint32_t *>(dp[1]);
      pv_out.verdict = static_cast<uint8_t *>(dp[2]);
      pv_out.first_invalid = static_cast<int16_t *>(dp[3]);
      pv_out.end_state = dp[4];
      pv_out.min_gap = static_cast<float *>(dp[5]);
      pv_out.flags = static_cast<uint8_t *>(dp[6]);
    }
  }

  // host-buffer outputs of a checked batch in spatial order: the check runs as
  // tune.pipe_launches launches over item ranges and each range's results are copied out
  // while the next range is checked
  const bool pipelined = !dev_out && !direct && !(opts->mode & DPG_MODE_BALL_ONLY) && reorder && cap > 0;
  // one check launch whose warps flag finished copy ranges in mapped memory
  const bool progress = pipelined && c->tune.host_output == DPG_HOST_OUT_PROGRESS;
  const int n_ranges = pipelined ? c->tune.pipe_launches : 1;
  const double decay = c->pipe_decay;  // the copy ranges' sizes for this call
  size_t last_bytes = 0;               // bytes of the last range's copies
  if (progress && !c->h_rflag) {
    CUDA_TRY(c, cudaHostAlloc(&c->h_rflag, sizeof(int) * kMaxSub, cudaHostAllocMapped));
    CUDA_TRY(c, cudaHostGetDevicePointer(&c->d_rflag, c->h_rflag, 0));
  }
  if (progress)
    for (int j = 0; j < kMaxSub; j++) reinterpret_cast<volatile int *>(c->h_rflag)[j] = 0;
  if (pipelined) {
    if (!c->cstream) {
      CUDA_TRY(c, cudaStreamCreateWithFlags(&c->cstream, cudaStreamNonBlocking));
      CUDA_TRY(c, cudaStreamCreateWithFlags(&c->xstream, cudaStreamNonBlocking));
      for (auto &e : c->ev_sub) CUDA_TRY(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      CUDA_TRY(c, cudaEventCreateWithFlags(&c->ev_tot, cudaEventDisableTiming));
      CUDA_TRY(c, cudaEventCreateWithFlags(&c->ev_ball, cudaEventDisableTiming));
      for (auto &e : c->ev_cl) CUDA_TRY(c, cudaEventCreate(&e));
    }
    if (c->h_bases_n < (size_t)P + 1) {
      if (c->h_bases) cudaFreeHost(c->h_bases);
      c->h_bases = nullptr;
      c->h_bases_n = 0;
      CUDA_TRY(c, cudaHostAlloc(&c->h_bases, 2 * sizeof(unsigned long long) * (P + 1), cudaHostAllocDefault));
      c->h_bases_n = (size_t)P + 1;
    }
  }

  CUDA_TRY(c, cudaEventRecord(c->ev[0], st));
  if (N > 0) {
    if (opts->x_on_device)
      CUDA_TRY(c, cudaMemcpyAsync(c->x64.p, x, sizeof(double) * nx * N, cudaMemcpyDeviceToDevice, st));
    else
      CUDA_TRY(c, cudaMemcpyAsync(c->x64.p, x, sizeof(double) * nx * N, cudaMemcpyHostToDevice, st));
  }
  CUDA_TRY(c, cudaMemsetAsync(c->d_ctr, 0, sizeof(DevCounters), st));
  CUDA_TRY(c, cudaEventRecord(c->ev[1], st));

  PrimView pv{};
  pv.P = P;
  pv.S = c->S;
  pv.len = P_<int32_t>(c->len);
  pv.soff = P_<int64_t>(c->soff);
  pv.krow = P_<int64_t>(c->soff);
  pv.order = P_<int32_t>(c->order);
  pv.key32 = P_<float>(c->key32);
  pv.kconst32 = P_<float>(c->kconst32);
  pv.st64 = P_<double>(c->st64);
  pv.st32 = P_<float>(c->st32);
  pv.pose32 = P_<Pose<float>>(c->pose32);
  pv.pose64 = P_<Pose<double>>(c->pose64);
  pv.pbox = P_<double>(c->pbox);
  pv.pbox32 = P_<float>(c->pbox32);
  pv.coff = P_<int64_t>(c->coff);
  pv.cbox32 = P_<float>(c->cbox32);
  pv.tbox32 = P_<float>(c->tbox32);
  if (reverse) {  // the ball keys on each primitive's last state (the key grid holds start keys)
    pv.key32 = P_<float>(c->rkey32);
    pv.kconst32 = P_<float>(c->rkconst32);
    pv.krow = P_<int64_t>(c->rkrow);
  }
  NodeView nv{N, P_<double>(c->x64), P_<float>(c->nkey32), P_<float>(c->noff32)};
  EnvView ev{};
  ev.dim = c->dim;
  for (int i = 0; i < 3; i++) { ev.lo[i] = c->lo[i]; ev.hi[i] = c->hi[i]; }
  ev.n_obs = c->n_obs;
  ev.obs32 = c->obs32.p;
  ev.obs64 = c->obs64.p;
  const RobotParams rp = c->rp;
  const double band = opts->contact_band > 0 ? opts->contact_band : 1e-4;
  const double ball_band = opts->ball_band > 0 ? opts->ball_band : 1e-5;
  DevCounters *ctr = c->d_ctr;

  CheckArgs ca{};
  ca.rp = rp;
  ca.pv = pv;
  ca.nv = nv;
  ca.ev = ev;
  ca.out = pv_out;
  ca.ord_pbase = P_<unsigned long long>(c->ord_pbase);
  ca.ord_ibase = P_<unsigned long long>(c->ord_ibase);
  ca.item_pos = P_<uint32_t>(c->item_pos);
  ca.ctr = ctr;
  ca.abort_flag = c->d_abort;
  ca.band = fp64 ? 0.0 : band;
  ca.cull_margin = cull_margin(pv_out.min_gap != nullptr, band);
  ca.dt32 = (float)rp.dt;
  ca.half_len32 = (float)rp.half_len;
  ca.half_wid32 = (float)rp.half_wid;
  ca.radius32 = (float)rp.radius;
  ca.band32 = (float)ca.band;
  for (int i = 0; i < 3; i++) { ca.lo32[i] = (float)c->lo[i]; ca.hi32[i] = (float)c->hi[i]; }

  cudaError_t launch_err = cudaSuccess;
  with_kind(kind, [&](auto K) {
    constexpr int KIND = decltype(K)::value;
    using R = Robot<KIND>;
    if (reorder) {  // nodes by Z-order cell, then index; the pipeline runs on the sorted copy
      const unsigned nb = (unsigned)((N + 255) / 256);
      const int64_t tile = order_tile(N), ntile = (N + tile - 1) / tile;
      node_tiles<KIND><<<(unsigned)ntile, 256, 0, st>>>(P_<double>(c->x64), N, ev, tile, P_<uint32_t>(c->ord_cell),
                                                         P_<uint32_t>(c->ord_rank), P_<uint32_t>(c->ord_tiles));
      nn_prefix<<<kOrderCells / 32, 256, 0, st>>>(kOrderCells, (int)ntile, P_<uint32_t>(c->ord_tiles),
                                                  P_<uint32_t>(c->ord_cnt));
      cell_scan<<<1, 1024, 0, st>>>(kOrderCells, P_<uint32_t>(c->ord_cnt), P_<uint32_t>(c->ord_start));
      cell_scatter<<<nb, 256, 0, st>>>(N, tile, P_<uint32_t>(c->ord_cell), P_<uint32_t>(c->ord_rank),
                                       P_<uint32_t>(c->ord_tiles), P_<uint32_t>(c->ord_start),
                                       P_<uint32_t>(c->ord_perm));
      gather_nodes<R::NX><<<(unsigned)((N * R::NX + 255) / 256), 256, 0, st>>>(
          P_<double>(c->x64), P_<uint32_t>(c->ord_perm), N, P_<double>(c->x64s));
      nv.x64 = P_<double>(c->x64s);
      ca.nv = nv;
    }
    if (N > 0) {
      prep_nodes<KIND><<<(unsigned)((N + 255) / 256), 256, 0, st>>>(nv);
      launch_ball<KIND>(c, pv, nv, opts->radius, ball_band, Wpad, B, W, P_<uint32_t>(c->mask),
                        P_<uint32_t>(c->cnt), P_<uint32_t>(c->tot), ctr, st, !reverse);
    } else {
      cudaMemsetAsync(c->tot.p, 0, sizeof(uint32_t) * P, st);
    }
    scan_totals<<<1, 1024, 0, st>>>(P, P_<int32_t>(c->order), P_<uint32_t>(c->tot),
                                    P_<unsigned long long>(c->pbase), P_<unsigned long long>(c->ord_pbase),
                                    P_<unsigned long long>(c->ord_ibase), cap, ctr);
    if (!(opts->mode & DPG_MODE_BALL_ONLY))
      item_positions<<<(unsigned)(((int64_t)P * 32 + 255) / 256), 256, 0, st>>>(
          P, P_<unsigned long long>(c->ord_ibase), ctr, P_<uint32_t>(c->item_pos));
    if (N > 0) {
      nn_emit<<<(unsigned)((P * ((Wpad / 32 + kEmitGroups - 1) / kEmitGroups) + 7) / 8), 256, 0, st>>>(
          P, W, Wpad, P_<uint32_t>(c->mask), P_<uint32_t>(c->cnt), P_<unsigned long long>(c->pbase), cap,
          pv_out.node, pv_out.prim);
    }
    cudaEventRecord(c->ev[2], st);
    launch_err = cudaGetLastError();
  });
  if (launch_err != cudaSuccess)
    return fail(c, DPG_ERR_CUDA, std::string("expand launch: ") + cudaGetErrorString(launch_err));
  if (pipelined) {  // what the host needs to place the copies: counters and item / pair bases
    CUDA_TRY(c, cudaMemcpyAsync(c->h_ctr, ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(c, cudaMemcpyAsync(c->h_bases, c->ord_ibase.p, sizeof(unsigned long long) * (P + 1),
                                cudaMemcpyDeviceToHost, st));
    CUDA_TRY(c, cudaMemcpyAsync(c->h_bases + c->h_bases_n, c->ord_pbase.p, sizeof(unsigned long long) * (P + 1),
                                cudaMemcpyDeviceToHost, st));
    CUDA_TRY(c, cudaEventRecord(c->ev_tot, st));
    CUDA_TRY(c, cudaEventRecord(c->ev_ball, st));
    CUDA_TRY(c, cudaStreamWaitEvent(c->xstream, c->ev_ball, 0));
  }
  with_kind(kind, [&](auto K) {
    constexpr int KIND = decltype(K)::value;
    if (!(opts->mode & DPG_MODE_BALL_ONLY)) {
      // exact check: persistent grid, obstacles in shared memory; node ids go
      // back to the caller's numbering as each pair is done.  Pipelined: the
      // launches alternate between two streams (disjoint item ranges and
      // work-queue counters), so the next range's blocks take the SMs that
      // the previous range's last items leave idle
      ca.perm = reorder ? P_<uint32_t>(c->ord_perm) : nullptr;
      ca.nsub = pipelined && !progress ? n_ranges : 1;
      ca.n_ranges = progress ? n_ranges : 0;
      ca.range_flag = progress ? c->d_rflag : nullptr;
      pipe_weights(n_ranges, ca.sub_cum, decay);
      for (int j = 0; j < ca.nsub; j++) {
        ca.sub = j;
        cudaStream_t s = pipelined && (j & 1) ? c->xstream : st;
        launch_check<KIND>(c, ca, prec, s);
        if (pipelined) cudaEventRecord(c->ev_sub[j], s);
      }
      if (pipelined && ca.nsub > 1) {  // join: the last launch on the second stream
        const int last_x = ca.nsub % 2 == 0 ? ca.nsub - 1 : ca.nsub - 2;
        cudaStreamWaitEvent(st, c->ev_sub[last_x], 0);
      }
    } else if (reorder && cap > 0) {  // ball only: pairs, no check
      unpermute_nodes<<<(unsigned)((cap + 255) / 256), 256, 0, st>>>(ctr, cap, P_<uint32_t>(c->ord_perm),
                                                                    pv_out.node);
    }
    cudaEventRecord(c->ev[3], st);
    cudaEventRecord(c->ev[4], st);
    launch_err = cudaGetLastError();
  });
  if (launch_err != cudaSuccess)
    return fail(c, DPG_ERR_CUDA, std::string("expand launch: ") + cudaGetErrorString(launch_err));
  if (pipelined) {
    // copy each check launch's pairs (a contiguous range: items are laid out
    // in pair order) on the copy stream as soon as that launch is done
    CUDA_TRY(c, cudaEventSynchronize(c->ev_tot));
    const DevCounters h0 = c->h_ctr[0];
    if (!h0.n_overflow && h0.n_pairs > 0) {
      const unsigned long long *ib = c->h_bases, *pb = c->h_bases + c->h_bases_n;
      auto pair_at = [&](unsigned long long item) -> int64_t {
        if (item >= h0.n_items) return (int64_t)h0.n_pairs;
        const int lo = (int)(std::upper_bound(ib, ib + P, item) - ib) - 1;  // ib[lo] <= item < ib[lo + 1]
        return (int64_t)(pb[lo] + 32ull * (item - ib[lo]));
      };
      struct { void *dst; void *src; size_t b; } cp[] = {
          {out->node, c->p_node.p, 4}, {out->prim, c->p_prim.p, 4}, {out->verdict, c->p_verdict.p, 1},
          {out->first_invalid, c->p_fi.p, 2}, {out->end_state, c->p_end.p, es_bytes * nx},
          {out->min_gap, c->p_gap.p, 4}, {out->flags, c->p_flags.p, 1}};
      const int np = n_ranges;
      int cum[kMaxSub + 1];
      pipe_weights(np, cum, decay);
      size_t bpp = 0;  // bytes copied per pair
      for (const auto &f : cp)
        if (f.dst) bpp += f.b;
      // consecutive ranges are copied together until a group holds
      // kMinCopyBytes (each copy call costs host time; small batches get
      // fewer, larger copies); the last range closes the last group
      int64_t ga = -1;
      for (int j = 0; j < np; j++) {
        const int64_t a = pair_at(h0.n_items * cum[j] / cum[np]), e = pair_at(h0.n_items * cum[j + 1] / cum[np]);
        if (progress) {
          // the range's flag, or the end of the check (an abort or an error:
          // the copies below then read final memory and the sync reports it)
          if (e > a)
            for (uint64_t it = 0; !reinterpret_cast<volatile int *>(c->h_rflag)[j]; it++)
              if ((it & 255) == 255 && cudaStreamQuery(st) != cudaErrorNotReady) break;
        } else {
          CUDA_TRY(c, cudaStreamWaitEvent(c->cstream, c->ev_sub[j], 0));
        }
        if (ga < 0) ga = a;
        const bool last = j == np - 1;
        if (!last && (size_t)(e - ga) * bpp < kMinCopyBytes) continue;
        if (last) CUDA_TRY(c, cudaEventRecord(c->ev_cl[0], c->cstream));
        if (e > ga)
          for (const auto &f : cp)
            if (f.dst) {
              CUDA_TRY(c, cudaMemcpyAsync(static_cast<char *>(f.dst) + ga * f.b, static_cast<char *>(f.src) + ga * f.b,
                                          (e - ga) * f.b, cudaMemcpyDeviceToHost, c->cstream));
              if (last) last_bytes += (e - ga) * f.b;
            }
        if (last) CUDA_TRY(c, cudaEventRecord(c->ev_cl[1], c->cstream));
        ga = -1;
      }
    }
    CUDA_TRY(c, cudaStreamWaitEvent(c->cstream, c->ev[4], 0));
    CUDA_TRY(c, cudaEventRecord(c->ev[5], c->cstream));
  }
  CUDA_TRY(c, cudaMemcpyAsync(c->h_ctr + 1, ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(c, cudaStreamSynchronize(st));
  if (pipelined) CUDA_TRY(c, cudaStreamSynchronize(c->cstream));
  const DevCounters h = c->h_ctr[1];
  out->n_pairs = (int64_t)h.n_pairs;
  out->n_scanned = N * (int64_t)P;
  out->n_contact_recheck = (int64_t)h.n_recheck;
  out->n_ball_recheck = (int64_t)h.n_ball_recheck;
  if (h.status == DPG_ERR_ABORTED) return fail(c, DPG_ERR_ABORTED, "expand: aborted");
  if ((int64_t)h.n_pairs > cap) return fail(c, DPG_ERR_CAPACITY, "expand: output capacity too small");
  const int64_t np = (int64_t)h.n_pairs;
  if (pipelined) {
    // copied above
  } else if (!dev_out && !direct && np > 0) {
    struct { void *dst; void *src; size_t b; } cp[] = {
        {out->node, c->p_node.p, 4}, {out->prim, c->p_prim.p, 4}, {out->verdict, c->p_verdict.p, 1},
        {out->first_invalid, c->p_fi.p, 2}, {out->end_state, c->p_end.p, es_bytes * nx},
        {out->min_gap, c->p_gap.p, 4}, {out->flags, c->p_flags.p, 1}};
    const int n_copy = (opts->mode & DPG_MODE_BALL_ONLY) ? 2 : 7;  // pairs only: node, prim
    for (int i = 0; i < n_copy; i++)
      if (cp[i].dst) CUDA_TRY(c, cudaMemcpyAsync(cp[i].dst, cp[i].src, cp[i].b * np, cudaMemcpyDeviceToHost, st));
  }
  if (!pipelined) {
    CUDA_TRY(c, cudaEventRecord(c->ev[5], st));
    CUDA_TRY(c, cudaStreamSynchronize(st));
  }
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev[1], c->ev[2]); c->timings[0] = ms;
  cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]); c->timings[1] = ms;
  cudaEventElapsedTime(&ms, c->ev[3], c->ev[4]); c->timings[2] = ms;
  float t_in = 0, t_out = 0;
  cudaEventElapsedTime(&t_in, c->ev[0], c->ev[1]);
  cudaEventElapsedTime(&t_out, c->ev[4], c->ev[5]);
  c->timings[3] = t_in + t_out;
  if (pipelined && last_bytes >= (1u << 20) && np > 0 && c->timings[1] > 0) {
    // the next call's range decay: this call's copy time (at the rate of its
    // last range, whose copies run after the check) over its check time
    float cl = 0;
    if (cudaEventElapsedTime(&cl, c->ev_cl[0], c->ev_cl[1]) == cudaSuccess && cl > 0) {
      size_t bpp = 0;  // bytes copied per pair
      const size_t b1[7] = {4, 4, 1, 2, (size_t)es_bytes * nx, 4, 1};
      void *d1[7] = {out->node, out->prim, out->verdict, out->first_invalid, out->end_state, out->min_gap, out->flags};
      for (int i = 0; i < 7; i++)
        if (d1[i]) bpp += b1[i];
      const double copy_ms = (double)bpp * (double)np * (double)cl / (double)last_bytes;
      c->pipe_decay = std::min(1.0, std::max(0.75, copy_ms / (double)c->timings[1]));
    }
  }
  return DPG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free batched expand (dpg_expand_noalloc, declared in dpg.h).
//
// Who needs it: callers that must not allocate device memory at expand time
// -- real-time planning loops that cannot block on the device allocator
// (cudaMalloc may synchronise the device), and host programs that hand all
// device memory to their own pool up front.  dpg_expand may grow its
// per-context buffers with cudaMalloc on any call; this entry point never
// does.
//
// Its per-call scratch (node keys and offsets, ball bitmask, per-tile counts,
// segment bases, work-queue counters) lives in one file-scope device array of
// kNoAllocScratchBytes.  Every GPU that loads this library holds that array
// until the process exits.  All calls share it and it keeps the contents of
// the last call: the counters are cleared at the start of every call, and
// calls whose device work overlaps (two streams, two host threads) race on it.
// The first call on a device looks the array's device address up with
// cudaGetSymbolAddress (once per device, with that device current).
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;  // 64 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_addr[kNoAllocMaxDevices] = {};

// device address of g_noalloc_scratch on `device` (which must be current)
int noalloc_scratch(dpg_ctx *c, int device, unsigned char **out) {
  if (device < 0 || device >= kNoAllocMaxDevices) return fail(c, DPG_ERR_ARG, "noalloc: device index too large");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[device]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(c, DPG_ERR_CUDA, std::string("noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_noalloc_addr[device] = p;
  }
  *out = static_cast<unsigned char *>(g_noalloc_addr[device]);
  return DPG_OK;
}

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

}  // namespace

extern "C" {

int dpg_expand_noalloc(dpg_ctx *c, const dpg_expand_opts *opts, int64_t N, const double *x_dev,
                       dpg_expand_out *out) {
  if (!c || !opts || !out) return DPG_ERR_ARG;
  if (!c->have_prims || !c->have_env) return fail(c, DPG_ERR_STATE, "noalloc: upload primitives and env first");
  if (N < 0 || (N > 0 && !x_dev)) return fail(c, DPG_ERR_ARG, "noalloc: bad node array");
  if (!out->node || !out->prim)
    return fail(c, DPG_ERR_ARG, "noalloc: the caller provides device arrays for node and prim");
  if (!(opts->radius >= 0) || !prec_ok(opts->precision))
    return fail(c, DPG_ERR_ARG, "noalloc: bad radius or precision");
  if (out->capacity < 0 || out->capacity > (int64_t)0xffffffffLL)
    return fail(c, DPG_ERR_ARG, "noalloc: capacity out of range");
  if (opts->mode & DPG_MODE_REVERSE) return fail(c, DPG_ERR_ARG, "noalloc: no reverse ball (use dpg_expand)");
  if (*(volatile int *)c->h_abort) return fail(c, DPG_ERR_ABORTED, "noalloc: abort flag raised");
  CUDA_TRY(c, cudaSetDevice(c->device));
  const int kind = c->robot.kind, P = c->P;
  const int kd = key_dim(kind), od = off_dim(kind);
  const int prec = opts->precision;
  const bool fp64 = prec == DPG_FP64_STRICT;  // every test in FP64
  const int64_t cap = out->capacity;
  const int64_t W = (N + 31) / 32;
  const int64_t Wpad = (W + 31) / 32 * 32;
  const int64_t B = (N + kNNThreads - 1) / kNNThreads;

  // carve the scratch; reject sizes beyond the array
  size_t off_key = 0;
  size_t off_off = off_key + align256(sizeof(float) * kd * (size_t)N);
  size_t off_mask = off_off + align256(sizeof(float) * od * (size_t)N);
  size_t off_cnt = off_mask + align256(sizeof(uint32_t) * (size_t)Wpad * P);
  size_t off_tot = off_cnt + align256(sizeof(uint32_t) * (size_t)B * P);
  size_t off_pbase = off_tot + align256(sizeof(uint32_t) * (size_t)P);
  size_t off_opb = off_pbase + align256(sizeof(unsigned long long) * (size_t)P);
  size_t off_oib = off_opb + align256(sizeof(unsigned long long) * ((size_t)P + 1));
  size_t off_ctr = off_oib + align256(sizeof(unsigned long long) * ((size_t)P + 1));
  const size_t need = off_ctr + align256(sizeof(DevCounters));
  if (need > kNoAllocScratchBytes)
    return fail(c, DPG_ERR_ARG, "noalloc: N x P too large for the " + std::to_string(kNoAllocScratchBytes >> 20) +
                                    " MiB scratch (needs " + std::to_string(need) + " bytes)");
  unsigned char *base = nullptr;
  int rc;
  if ((rc = noalloc_scratch(c, c->device, &base))) return rc;
  float *nkey32 = reinterpret_cast<float *>(base + off_key);
  float *noff32 = reinterpret_cast<float *>(base + off_off);
  uint32_t *mask = reinterpret_cast<uint32_t *>(base + off_mask);
  uint32_t *cnt = reinterpret_cast<uint32_t *>(base + off_cnt);
  uint32_t *tot = reinterpret_cast<uint32_t *>(base + off_tot);
  unsigned long long *pbase = reinterpret_cast<unsigned long long *>(base + off_pbase);
  unsigned long long *ord_pbase = reinterpret_cast<unsigned long long *>(base + off_opb);
  unsigned long long *ord_ibase = reinterpret_cast<unsigned long long *>(base + off_oib);
  DevCounters *ctr = reinterpret_cast<DevCounters *>(base + off_ctr);

  cudaStream_t st = c->stream;
  CUDA_TRY(c, cudaMemsetAsync(ctr, 0, sizeof(DevCounters), st));  // counters start at zero

  PrimView pv{};
  pv.P = P;
  pv.S = c->S;
  pv.len = P_<int32_t>(c->len);
  pv.soff = P_<int64_t>(c->soff);
  pv.krow = P_<int64_t>(c->soff);
  pv.order = P_<int32_t>(c->order);
  pv.key32 = P_<float>(c->key32);
  pv.kconst32 = P_<float>(c->kconst32);
  pv.st64 = P_<double>(c->st64);
  pv.st32 = P_<float>(c->st32);
  pv.pose32 = P_<Pose<float>>(c->pose32);
  pv.pose64 = P_<Pose<double>>(c->pose64);
  pv.pbox = P_<double>(c->pbox);
  pv.pbox32 = P_<float>(c->pbox32);
  pv.coff = P_<int64_t>(c->coff);
  pv.cbox32 = P_<float>(c->cbox32);
  pv.tbox32 = P_<float>(c->tbox32);
  NodeView nv{N, x_dev, nkey32, noff32};
  EnvView ev{};
  ev.dim = c->dim;
  for (int i = 0; i < 3; i++) { ev.lo[i] = c->lo[i]; ev.hi[i] = c->hi[i]; }
  ev.n_obs = c->n_obs;
  ev.obs32 = c->obs32.p;
  ev.obs64 = c->obs64.p;
  PairView po{};
  po.cap = cap;
  po.node = out->node;
  po.prim = out->prim;
  po.verdict = out->verdict;
  po.first_invalid = out->first_invalid;
  po.end_state = out->end_state;
  po.min_gap = out->min_gap;
  po.flags = out->flags;
  const RobotParams rp = c->rp;
  const double band = opts->contact_band > 0 ? opts->contact_band : 1e-4;
  const double ball_band = opts->ball_band > 0 ? opts->ball_band : 1e-5;
  CheckArgs ca{};
  ca.rp = rp;
  ca.pv = pv;
  ca.nv = nv;
  ca.ev = ev;
  ca.out = po;
  ca.ord_pbase = ord_pbase;
  ca.ord_ibase = ord_ibase;
  ca.ctr = ctr;
  ca.abort_flag = c->d_abort;
  ca.band = fp64 ? 0.0 : band;
  ca.cull_margin = cull_margin(po.min_gap != nullptr, band);
  ca.dt32 = (float)rp.dt;
  ca.half_len32 = (float)rp.half_len;
  ca.half_wid32 = (float)rp.half_wid;
  ca.radius32 = (float)rp.radius;
  ca.band32 = (float)ca.band;
  for (int i = 0; i < 3; i++) { ca.lo32[i] = (float)c->lo[i]; ca.hi32[i] = (float)c->hi[i]; }

  cudaError_t launch_err = cudaSuccess;
  with_kind(kind, [&](auto K) {
    constexpr int KIND = decltype(K)::value;
    using R = Robot<KIND>;
    if (N > 0) {
      prep_nodes<KIND><<<(unsigned)((N + 255) / 256), 256, 0, st>>>(nv);
      launch_ball<KIND>(c, pv, nv, opts->radius, ball_band, Wpad, B, W, mask, cnt, tot, ctr, st);
    } else {
      cudaMemsetAsync(tot, 0, sizeof(uint32_t) * P, st);
    }
    scan_totals<<<1, 1024, 0, st>>>(P, P_<int32_t>(c->order), tot, pbase, ord_pbase, ord_ibase, cap, ctr);
    if (N > 0) {
      nn_emit<<<(unsigned)((P * ((Wpad / 32 + kEmitGroups - 1) / kEmitGroups) + 7) / 8), 256, 0, st>>>(
          P, W, Wpad, mask, cnt, pbase, cap, po.node, po.prim);
    }
    if (!(opts->mode & DPG_MODE_BALL_ONLY)) launch_check<KIND>(c, ca, prec, st);
    launch_err = cudaGetLastError();
  });
  if (launch_err != cudaSuccess)
    return fail(c, DPG_ERR_CUDA, std::string("noalloc launch: ") + cudaGetErrorString(launch_err));
  CUDA_TRY(c, cudaMemcpyAsync(c->h_ctr, ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(c, cudaStreamSynchronize(st));
  const DevCounters h = *c->h_ctr;
  out->n_pairs = (int64_t)h.n_pairs;
  out->n_scanned = N * (int64_t)P;
  out->n_contact_recheck = (int64_t)h.n_recheck;
  out->n_ball_recheck = (int64_t)h.n_ball_recheck;
  if (h.status == DPG_ERR_ABORTED) return fail(c, DPG_ERR_ABORTED, "noalloc: aborted");
  if ((int64_t)h.n_pairs > cap) return fail(c, DPG_ERR_CAPACITY, "noalloc: output capacity too small");
  return DPG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Node features of the surrogate MLP (include/dpg_mlp.h): normalised state
// and the occupancy patch of the context's environment around each node.
extern "C" int dpg_mlp_node_features(dpg_ctx *c, const double *x_dev, int64_t N, const double *goal,
                                     void *feat_dev) {
  if (!c || N < 0 || (N > 0 && (!x_dev || !feat_dev))) return DPG_ERR_ARG;
  if (!c->have_env) return fail(c, DPG_ERR_STATE, "node_features: upload the environment first");
  if (N == 0) return DPG_OK;
  CUDA_TRY(c, cudaSetDevice(c->device));
  NodeView nv{N, x_dev, nullptr, nullptr};
  EnvView ev{};
  ev.dim = c->dim;
  for (int i = 0; i < 3; i++) { ev.lo[i] = c->lo[i]; ev.hi[i] = c->hi[i]; }
  ev.n_obs = c->n_obs;
  ev.obs32 = c->obs32.p;
  ev.obs64 = c->obs64.p;
  GoalView gv{};
  gv.has = goal ? 1 : 0;
  for (int i = 0; i < 3 && goal; i++) gv.g[i] = i < c->dim ? goal[i] : 0.0;
  with_kind(c->robot.kind, [&](auto K) {
    constexpr int KIND = decltype(K)::value;
    mlp_node_features<KIND><<<(unsigned)((N + 127) / 128), 128, 0, c->stream>>>(
        nv, ev, gv, static_cast<__nv_bfloat16 *>(feat_dev));
  });
  CUDA_TRY(c, cudaGetLastError());
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return DPG_OK;
}

// ---------------------------------------------------------------------------
// Helpers shared with lazy.cu (check_list.h).
namespace dpg {

int ctx_fail(dpg_ctx *c, int code, const std::string &msg) { return fail(c, code, msg); }
int ctx_ensure(dpg_ctx *c, DevBuf &b, size_t bytes) { return ensure(c, b, bytes); }

PrimView ctx_prim_view(dpg_ctx *c) {
  PrimView pv{};
  pv.P = c->P;
  pv.S = c->S;
  pv.len = P_<int32_t>(c->len);
  pv.soff = P_<int64_t>(c->soff);
  pv.krow = P_<int64_t>(c->soff);
  pv.order = P_<int32_t>(c->order);
  pv.key32 = P_<float>(c->key32);
  pv.kconst32 = P_<float>(c->kconst32);
  pv.st64 = P_<double>(c->st64);
  pv.st32 = P_<float>(c->st32);
  pv.pose32 = P_<Pose<float>>(c->pose32);
  pv.pose64 = P_<Pose<double>>(c->pose64);
  pv.pbox = P_<double>(c->pbox);
  pv.pbox32 = P_<float>(c->pbox32);
  pv.coff = P_<int64_t>(c->coff);
  pv.cbox32 = P_<float>(c->cbox32);
  pv.tbox32 = P_<float>(c->tbox32);
  return pv;
}

EnvView ctx_env_view(const dpg_ctx *c) {
  EnvView ev{};
  ev.dim = c->dim;
  for (int i = 0; i < 3; i++) { ev.lo[i] = c->lo[i]; ev.hi[i] = c->hi[i]; }
  ev.n_obs = c->n_obs;
  ev.obs32 = c->obs32.p;
  ev.obs64 = c->obs64.p;
  return ev;
}

CheckArgs ctx_check_args(dpg_ctx *c, int prec, double contact_band, const NodeView &nv, const PairView &out) {
  const RobotParams rp = c->rp;
  const double band = contact_band > 0 ? contact_band : 1e-4;
  CheckArgs ca{};
  ca.rp = rp;
  ca.pv = ctx_prim_view(c);
  ca.nv = nv;
  ca.ev = ctx_env_view(c);
  ca.out = out;
  ca.ord_pbase = P_<unsigned long long>(c->ord_pbase);
  ca.ord_ibase = P_<unsigned long long>(c->ord_ibase);
  ca.ctr = c->d_ctr;
  ca.abort_flag = c->d_abort;
  ca.band = prec == DPG_FP64_STRICT ? 0.0 : band;
  ca.cull_margin = cull_margin(out.min_gap != nullptr, band);
  ca.dt32 = (float)rp.dt;
  ca.half_len32 = (float)rp.half_len;
  ca.half_wid32 = (float)rp.half_wid;
  ca.radius32 = (float)rp.radius;
  ca.band32 = (float)ca.band;
  for (int i = 0; i < 3; i++) { ca.lo32[i] = (float)c->lo[i]; ca.hi32[i] = (float)c->hi[i]; }
  return ca;
}

int ctx_spatial_order(dpg_ctx *c, const double *x_dev, int64_t N, cudaStream_t st, const uint32_t **perm) {
  *perm = nullptr;
  if (N < kReorderMin) return DPG_OK;
  const int64_t tile = order_tile(N), ntile = (N + tile - 1) / tile;
  int rc;
  if ((rc = ensure(c, c->ord_cell, sizeof(uint32_t) * N)) || (rc = ensure(c, c->ord_perm, sizeof(uint32_t) * N)) ||
      (rc = ensure(c, c->ord_cnt, sizeof(uint32_t) * kOrderCells)) ||
      (rc = ensure(c, c->ord_start, sizeof(uint32_t) * kOrderCells)) ||
      (rc = ensure(c, c->ord_rank, sizeof(uint32_t) * N)) ||
      (rc = ensure(c, c->ord_tiles, sizeof(uint32_t) * kOrderCells * (size_t)ntile)))
    return rc;
  const EnvView ev = ctx_env_view(c);
  with_kind(c->robot.kind, [&](auto K) {
    constexpr int KIND = decltype(K)::value;
    node_tiles<KIND><<<(unsigned)ntile, 256, 0, st>>>(x_dev, N, ev, tile, P_<uint32_t>(c->ord_cell),
                                                       P_<uint32_t>(c->ord_rank), P_<uint32_t>(c->ord_tiles));
    nn_prefix<<<kOrderCells / 32, 256, 0, st>>>(kOrderCells, (int)ntile, P_<uint32_t>(c->ord_tiles),
                                                P_<uint32_t>(c->ord_cnt));
    cell_scan<<<1, 1024, 0, st>>>(kOrderCells, P_<uint32_t>(c->ord_cnt), P_<uint32_t>(c->ord_start));
    cell_scatter<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(N, tile, P_<uint32_t>(c->ord_cell),
                                                             P_<uint32_t>(c->ord_rank), P_<uint32_t>(c->ord_tiles),
                                                             P_<uint32_t>(c->ord_start), P_<uint32_t>(c->ord_perm));
  });
  CUDA_TRY(c, cudaGetLastError());
  *perm = P_<uint32_t>(c->ord_perm);
  return DPG_OK;
}

void ctx_prep_nodes(dpg_ctx *c, const NodeView &nv, cudaStream_t st) {
  if (nv.N <= 0) return;
  with_kind(c->robot.kind, [&](auto K) {
    constexpr int KIND = decltype(K)::value;
    prep_nodes<KIND><<<(unsigned)((nv.N + 255) / 256), 256, 0, st>>>(nv);
  });
}

int ctx_check_list(dpg_ctx *c, int prec, CheckArgs ca, int64_t n, const uint32_t *node_d, const uint32_t *prim_d,
                   const uint32_t *dest_d, cudaStream_t st, bool timed) {
  const int P = c->P;
  int rc;
  if ((rc = ensure(c, c->tot, sizeof(uint32_t) * P)) || (rc = ensure(c, c->q_fill, sizeof(uint32_t) * P)) ||
      (rc = ensure(c, c->pbase, sizeof(unsigned long long) * P)) ||
      (rc = ensure(c, c->ord_pbase, sizeof(unsigned long long) * (P + 1))) ||
      (rc = ensure(c, c->ord_ibase, sizeof(unsigned long long) * (P + 1))) ||
      (rc = ensure(c, c->q_sorted, 4 * (size_t)std::max<int64_t>(n, 1))) ||
      (rc = ensure(c, c->q_idx, 4 * (size_t)std::max<int64_t>(n, 1))))
    return rc;
  ca.ord_pbase = P_<unsigned long long>(c->ord_pbase);
  ca.ord_ibase = P_<unsigned long long>(c->ord_ibase);
  ca.ctr = c->d_ctr;
  ca.out.cap = n;
  ca.out.node = P_<uint32_t>(c->q_sorted);
  ca.out.prim = nullptr;
  ca.out.out_index = P_<uint32_t>(c->q_idx);
  ca.perm = nullptr;
  ca.sub = 0;
  ca.nsub = 1;
  CUDA_TRY(c, cudaMemsetAsync(c->d_ctr, 0, sizeof(DevCounters), st));
  CUDA_TRY(c, cudaMemsetAsync(c->tot.p, 0, sizeof(uint32_t) * P, st));
  CUDA_TRY(c, cudaMemsetAsync(c->q_fill.p, 0, sizeof(uint32_t) * P, st));
  if (n == 0) return DPG_OK;
  const int64_t N = ca.nv.N;
  cudaError_t launch_err = cudaSuccess;
  with_kind(c->robot.kind, [&](auto K) {
    constexpr int KIND = decltype(K)::value;
    pairs_hist<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(node_d, prim_d, n, N, P, P_<uint32_t>(c->tot), c->d_ctr);
    scan_totals<<<1, 1024, 0, st>>>(P, P_<int32_t>(c->order), P_<uint32_t>(c->tot), P_<unsigned long long>(c->pbase),
                                    P_<unsigned long long>(c->ord_pbase), P_<unsigned long long>(c->ord_ibase), n,
                                    c->d_ctr);
    pairs_scatter<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(node_d, prim_d, n, N, P,
                                                               P_<unsigned long long>(c->pbase),
                                                               P_<uint32_t>(c->q_fill), P_<uint32_t>(c->q_sorted),
                                                               P_<uint32_t>(c->q_idx), dest_d);
    if (timed) cudaEventRecord(c->ev[2], st);
    launch_check<KIND>(c, ca, prec, st);
    if (timed) cudaEventRecord(c->ev[3], st);
    launch_err = cudaGetLastError();
  });
  if (launch_err != cudaSuccess)
    return fail(c, DPG_ERR_CUDA, std::string("check launch: ") + cudaGetErrorString(launch_err));
  return DPG_OK;
}

int ctx_check_grouped(dpg_ctx *c, int prec, CheckArgs ca, const uint32_t *list_node, const uint32_t *list_dest,
                      cudaStream_t st) {
  ca.ord_pbase = P_<unsigned long long>(c->ord_pbase);
  ca.ord_ibase = P_<unsigned long long>(c->ord_ibase);
  ca.ctr = c->d_ctr;
  ca.out.node = const_cast<uint32_t *>(list_node);
  ca.out.prim = nullptr;
  ca.out.out_index = list_dest;
  ca.perm = nullptr;
  ca.sub = 0;
  ca.nsub = 1;
  cudaError_t launch_err = cudaSuccess;
  with_kind(c->robot.kind, [&](auto K) {
    constexpr int KIND = decltype(K)::value;
    launch_check<KIND>(c, ca, prec, st);
    launch_err = cudaGetLastError();
  });
  if (launch_err != cudaSuccess)
    return fail(c, DPG_ERR_CUDA, std::string("check launch: ") + cudaGetErrorString(launch_err));
  return DPG_OK;
}

}  // namespace dpg

// ---------------------------------------------------------------------------
// Exact check of an explicit pair list (dpg_check_pairs, dpg.h): the pairs
// are grouped by primitive (longest first) so the same persistent warps as
// in dpg_expand walk one primitive per warp; results go back to the input
// positions.
extern "C" int dpg_check_pairs(dpg_ctx *c, const dpg_expand_opts *opts, int64_t N, const double *x, int64_t n,
                               const uint32_t *node, const uint32_t *prim, dpg_expand_out *out) {
  if (!c || !opts || !out) return DPG_ERR_ARG;
  if (!c->have_prims || !c->have_env) return fail(c, DPG_ERR_STATE, "check_pairs: upload primitives and env first");
  if (N < 0 || n < 0 || (N > 0 && !x) || (n > 0 && (!node || !prim)))
    return fail(c, DPG_ERR_ARG, "check_pairs: bad arrays");
  if (n > (int64_t)0xffffffffLL || N > (int64_t)1 << 31) return fail(c, DPG_ERR_ARG, "check_pairs: too many pairs");
  if (out->capacity < n) {
    out->n_pairs = n;
    return fail(c, DPG_ERR_CAPACITY, "check_pairs: capacity below n");
  }
  if (!prec_ok(opts->precision)) return fail(c, DPG_ERR_ARG, "check_pairs: precision");
  if (*(volatile int *)c->h_abort) return fail(c, DPG_ERR_ABORTED, "check_pairs: abort flag raised");
  CUDA_TRY(c, cudaSetDevice(c->device));
  out->n_pairs = n;
  out->n_scanned = 0;
  out->n_contact_recheck = 0;
  out->n_ball_recheck = 0;
  if (n == 0) return DPG_OK;
  const int kind = c->robot.kind, nx = c->robot.nx, P = c->P;
  const int kd = key_dim(kind), od = off_dim(kind);
  const int prec = opts->precision;
  const size_t es_bytes = prec != DPG_FP32 ? sizeof(double) : sizeof(float);
  const bool dev_in = opts->x_on_device != 0, dev_out = opts->out_on_device != 0;
  cudaStream_t st = c->stream;
  int rc;
  if ((rc = ensure(c, c->x64, sizeof(double) * nx * std::max<int64_t>(N, 1))) ||
      (rc = ensure(c, c->nkey32, sizeof(float) * kd * std::max<int64_t>(N, 1))) ||
      (rc = ensure(c, c->noff32, sizeof(float) * od * std::max<int64_t>(N, 1))))
    return rc;
  const uint32_t *node_d = node, *prim_d = prim;
  const double *x_d = x;
  if (!dev_in) {  // host lists: reject out-of-range indices before any copy
    for (int64_t i = 0; i < n; i++)
      if ((int64_t)node[i] >= N || prim[i] >= (uint32_t)P)
        return fail(c, DPG_ERR_ARG, "check_pairs: pair " + std::to_string(i) + " has node >= N or prim >= P");
    if ((rc = ensure(c, c->q_node, 4 * (size_t)n)) || (rc = ensure(c, c->q_prim, 4 * (size_t)n))) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(c->x64.p, x, sizeof(double) * nx * std::max<int64_t>(N, 0), cudaMemcpyHostToDevice, st));
    CUDA_TRY(c, cudaMemcpyAsync(c->q_node.p, node, 4 * n, cudaMemcpyHostToDevice, st));
    CUDA_TRY(c, cudaMemcpyAsync(c->q_prim.p, prim, 4 * n, cudaMemcpyHostToDevice, st));
    node_d = P_<uint32_t>(c->q_node);
    prim_d = P_<uint32_t>(c->q_prim);
    x_d = P_<double>(c->x64);
  }
  PairView po{};
  if (dev_out) {
    po.verdict = out->verdict;
    po.first_invalid = out->first_invalid;
    po.end_state = out->end_state;
    po.min_gap = out->min_gap;
    po.flags = out->flags;
  } else {
    const size_t nz = (size_t)n;
    if ((rc = ensure(c, c->p_verdict, nz)) || (rc = ensure(c, c->p_fi, 2 * nz)) ||
        (rc = ensure(c, c->p_end, es_bytes * nx * nz)) || (rc = ensure(c, c->p_gap, 4 * nz)) ||
        (rc = ensure(c, c->p_flags, nz)))
      return rc;
    po.verdict = out->verdict ? P_<uint8_t>(c->p_verdict) : nullptr;
    po.first_invalid = out->first_invalid ? P_<int16_t>(c->p_fi) : nullptr;
    po.end_state = out->end_state ? c->p_end.p : nullptr;
    po.min_gap = out->min_gap ? P_<float>(c->p_gap) : nullptr;
    po.flags = out->flags ? P_<uint8_t>(c->p_flags) : nullptr;
  }
  NodeView nv{N, x_d, P_<float>(c->nkey32), P_<float>(c->noff32)};
  const CheckArgs ca = ctx_check_args(c, prec, opts->contact_band, nv, po);

  CUDA_TRY(c, cudaEventRecord(c->ev[1], st));
  ctx_prep_nodes(c, nv, st);
  if ((rc = ctx_check_list(c, prec, ca, n, node_d, prim_d, nullptr, st, true)) != DPG_OK) return rc;
  CUDA_TRY(c, cudaMemcpyAsync(c->h_ctr, c->d_ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, st));
  if (!dev_out) {
    struct { void *dst; void *src; size_t b; } cp[] = {
        {out->verdict, c->p_verdict.p, 1}, {out->first_invalid, c->p_fi.p, 2},
        {out->end_state, c->p_end.p, es_bytes * nx}, {out->min_gap, c->p_gap.p, 4}, {out->flags, c->p_flags.p, 1}};
    for (auto &e : cp)
      if (e.dst) CUDA_TRY(c, cudaMemcpyAsync(e.dst, e.src, e.b * n, cudaMemcpyDeviceToHost, st));
  }
  CUDA_TRY(c, cudaStreamSynchronize(st));
  const DevCounters h = *c->h_ctr;
  out->n_contact_recheck = (int64_t)h.n_recheck;
  if (h.n_bad)
    return fail(c, DPG_ERR_ARG, "check_pairs: " + std::to_string(h.n_bad) +
                                    " pairs have node >= N or prim >= P (left unchecked)");
  if (h.status == DPG_ERR_ABORTED) return fail(c, DPG_ERR_ABORTED, "check_pairs: aborted");
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev[1], c->ev[2]);
  c->timings[0] = ms;
  cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
  c->timings[1] = ms;
  c->timings[2] = 0;
  c->timings[3] = 0;
  return DPG_OK;
}
