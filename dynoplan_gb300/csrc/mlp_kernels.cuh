// mlp_kernels.cuh -- element-wise and data-movement kernels of the surrogate
// MLP (the GEMMs are gemm_kernels.cuh).
//
// Input row of a (node, primitive) pair, 128 bf16 (K of the first GEMM is a
// multiple of 64; columns 96..127 are zero):
//   [0, 16)   node state, normalised (position to [-1, 1] over the
//             environment box, angles / pi, velocities / 4), zero padded
//   [16, 80)  8 x 8 occupancy patch around the node: cell (i, j) is 1 when its
//             box overlaps an obstacle (0.75 m cells, patch centred on the
//             node, world-aligned)
//   [80, 96)  the primitive's learned 16-D embedding
// Outputs per pair: [collision logit, cost-to-go].
#pragma once

#include <cuda_bf16.h>

#include "expand_kernels.cuh"
#include "gemm_kernels.cuh"

namespace dpg {

constexpr int kMlpIn = 128, kMlpNodeFeat = 80, kMlpEmb = 16, kMlpHidden = 256, kMlpOutPad = 16;
constexpr int kOccSide = 8;
constexpr float kOccCell = 0.75f;

// goal the cost-to-go refers to: slots 13.. of the state block hold
// (goal - position), normalised like the position
struct GoalView {
  int has;
  double g[3];
};

// per node: normalised state + occupancy patch (80 bf16)
template <int KIND>
__global__ void mlp_node_features(NodeView nv, EnvView ev, GoalView gv, __nv_bfloat16 *feat) {
  using R = Robot<KIND>;
  const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= nv.N) return;
  const double *x = nv.x64 + n * R::NX;
  __nv_bfloat16 *f = feat + n * kMlpNodeFeat;
  float s[16];
#pragma unroll
  for (int i = 0; i < 16; i++) s[i] = 0.f;
  for (int i = 0; i < R::POSD; i++) {
    const double ext = ev.hi[i] - ev.lo[i];
    s[i] = ext > 0 ? (float)(2.0 * (x[i] - ev.lo[i]) / ext - 1.0) : 0.f;
  }
  int k = R::POSD;
  if constexpr (KIND == DPG_ROBOT_QUAD3D) {
    for (int i = 3; i < 13 && k < 16; i++) s[k++] = (float)(i >= 7 ? x[i] / 4.0 : x[i]);
  } else {
    for (int i = R::POSD; i < R::NX && k < 16; i++) {
      const bool angle = i == 2 || (KIND == DPG_ROBOT_CAR1 && i == 3);
      s[k++] = angle ? wrap_pi_f64(x[i]) * 0.31830988618f : (float)(x[i] / 4.0);
    }
  }
  if (gv.has)
    for (int i = 0; i < R::POSD; i++) {
      const double ext = ev.hi[i] - ev.lo[i];
      s[13 + i] = ext > 0 ? (float)(2.0 * (gv.g[i] - x[i]) / ext) : 0.f;
    }
#pragma unroll
  for (int i = 0; i < 16; i++) f[i] = __float2bfloat16_rn(s[i]);
  const float px = (float)x[0], py = (float)x[1];
  const float h = 0.5f * kOccCell;
  for (int c = 0; c < kOccSide * kOccSide; c++) {
    const float cx = px + ((c % kOccSide) - 3.5f) * kOccCell, cy = py + ((c / kOccSide) - 3.5f) * kOccCell;
    float occ = 0.f;
    if (ev.dim == 2) {
      const Obs2<float> *ob = (const Obs2<float> *)ev.obs32;
      for (int o = 0; o < ev.n_obs && occ == 0.f; o++)
        if (fabsf(cx - ob[o].cx) <= h + ob[o].hx && fabsf(cy - ob[o].cy) <= h + ob[o].hy) occ = 1.f;
    } else {
      const Obs3<float> *ob = (const Obs3<float> *)ev.obs32;
      const float pz = (float)x[2];
      for (int o = 0; o < ev.n_obs && occ == 0.f; o++)
        if (fabsf(cx - ob[o].cx) <= h + ob[o].hx && fabsf(cy - ob[o].cy) <= h + ob[o].hy &&
            fabsf(pz - ob[o].cz) <= h + ob[o].hz)
          occ = 1.f;
    }
    f[16 + c] = __float2bfloat16_rn(occ);
  }
}

// X[b] = [node_feat[node[b]] | emb[prim[b]]], one thread per 16-byte chunk
// Thread per (8-column chunk c, row b), rows fastest; when XT is set the
// rows are also written transposed (XT[col * B_pad + b]: consecutive threads
// store consecutive rows of a column).
static __global__ void mlp_assemble(const __nv_bfloat16 *node_feat, const __nv_bfloat16 *emb, const uint32_t *node,
                             const uint32_t *prim, int64_t B, int64_t B_pad, __nv_bfloat16 *X,
                             __nv_bfloat16 *XT) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int c = (int)(i / B_pad);
  const int64_t b = i - (int64_t)c * B_pad;
  if (c >= kMlpIn / 8) return;
  uint4 v = make_uint4(0, 0, 0, 0);
  if (b < B) {
    if (c < kMlpNodeFeat / 8)
      v = reinterpret_cast<const uint4 *>(node_feat + (int64_t)node[b] * kMlpNodeFeat)[c];
    else if (c < (kMlpNodeFeat + kMlpEmb) / 8)
      v = reinterpret_cast<const uint4 *>(emb + (int64_t)prim[b] * kMlpEmb)[c - kMlpNodeFeat / 8];
  }
  reinterpret_cast<uint4 *>(X + b * kMlpIn)[c] = v;
  if (XT) {
    const __nv_bfloat16 *h = reinterpret_cast<const __nv_bfloat16 *>(&v);
#pragma unroll
    for (int j = 0; j < 8; j++) XT[(int64_t)(8 * c + j) * B_pad + b] = h[j];
  }
}

__device__ __forceinline__ float softplus(float x) { return x > 20.f ? x : log1pf(__expf(x)); }
__device__ __forceinline__ float sigmoid(float x) { return 1.f / (1.f + __expf(-x)); }

// loss = mean_b [softplus(l) - y l  +  0.5 w (c - t)^2]; dY (bf16, B x 64,
// columns >= 2 zero) = d loss / d [l, c]; loss accumulated into *loss_sum
// (ctg_weight = hp[1]: the step's hyper-parameters live in device memory so a
// captured training step can be replayed with new values)
// When dYT is set, also the first kMlpOutPad columns of dY transposed
// (dYT[j * B_pad + b]) and the head's bias gradient (column sums of the bf16
// dY, two non-zero columns) added into db.
static __global__ void mlp_loss(const float *out, const float *target, int64_t B, int64_t B_pad, const float *hp,
                         __nv_bfloat16 *dY, float *loss_sum, __nv_bfloat16 *dYT, float *db) {
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const float ctg_weight = hp[1];
  float l = 0.f, g0 = 0.f, g1 = 0.f;
  if (b < B_pad) {
    __align__(16) __nv_bfloat16 row[64];
#pragma unroll
    for (int j = 0; j < 64; j++) row[j] = __float2bfloat16_rn(0.f);
    if (b < B) {  // a NaN target leaves its head out of the loss
      const float lg = out[b * 2], ct = out[b * 2 + 1];
      const float y = target[b * 2], t = target[b * 2 + 1];
      const float inv = 1.f / (float)B;
      if (!isnan(y)) {
        l += softplus(lg) - y * lg;
        row[0] = __float2bfloat16_rn((sigmoid(lg) - y) * inv);
      }
      if (!isnan(t)) {
        l += 0.5f * ctg_weight * (ct - t) * (ct - t);
        row[1] = __float2bfloat16_rn(ctg_weight * (ct - t) * inv);
      }
    }
    uint4 *dst = reinterpret_cast<uint4 *>(dY + b * 64);
#pragma unroll
    for (int j = 0; j < 8; j++) dst[j] = reinterpret_cast<const uint4 *>(row)[j];
    if (dYT) {
#pragma unroll
      for (int j = 0; j < kMlpOutPad; j++) dYT[j * B_pad + b] = row[j];
    }
    g0 = __bfloat162float(row[0]);
    g1 = __bfloat162float(row[1]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    l += __shfl_down_sync(0xffffffffu, l, o);
    g0 += __shfl_down_sync(0xffffffffu, g0, o);
    g1 += __shfl_down_sync(0xffffffffu, g1, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (l != 0.f) atomicAdd(loss_sum, l);
    if (db && g0 != 0.f) atomicAdd(db, g0);
    if (db && g1 != 0.f) atomicAdd(db + 1, g1);
  }
}

// dZ = dH * gelu'(Z) (gelu' kept in bf16 by the forward epilogue): the
// epilogue of dH = dZnext * W.  Optionally also
// dZ transposed (dzT[col * ldt + row], the K-major operand of the
// weight-gradient GEMM) and partial bias gradients: the column sums of the
// bf16 dZ over each warp's 32 rows, stored (no atomics) at row
// 4 blockIdx.x + (warp % 4) of dpart [M / 32 x ld], summed by sum_rows_f32.
// The partial sums need whole warps of rows: M a multiple of 128.
struct EpiGeluGrad {
  const __nv_bfloat16 *dgelu;
  __nv_bfloat16 *dz;
  int ld;
  __nv_bfloat16 *dzT = nullptr;
  int64_t ldt = 0;
  float *dpart = nullptr;
  __device__ void operator()(int row, int c0, const float *v) const {
    __align__(16) __nv_bfloat16 h[16], d[16];
    const uint4 *gd = reinterpret_cast<const uint4 *>(dgelu + (int64_t)row * ld + c0);
    reinterpret_cast<uint4 *>(d)[0] = gd[0];
    reinterpret_cast<uint4 *>(d)[1] = gd[1];
#pragma unroll
    for (int j = 0; j < 16; j++) h[j] = __float2bfloat16_rn(v[j] * __bfloat162float(d[j]));
    uint4 *dst = reinterpret_cast<uint4 *>(dz + (int64_t)row * ld + c0);
    dst[0] = reinterpret_cast<const uint4 *>(h)[0];
    dst[1] = reinterpret_cast<const uint4 *>(h)[1];
    float *prow = dpart ? dpart + ((int64_t)blockIdx.x * 4 + ((threadIdx.x >> 5) & 3)) * ld + c0 : nullptr;
    if (dzT) {  // the transposed store also sums the staged columns
      store_transposed16(dzT, ldt, row, c0, h, prow);
    } else if (prow) {
      const int lane = threadIdx.x & 31;
      float mine = 0.f;  // lane j < 16 keeps column c0 + j
#pragma unroll
      for (int j = 0; j < 16; j++) {
        float t = __bfloat162float(h[j]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == j) mine = t;
      }
      if (lane < 16) prow[lane] = mine;
    }
  }
};

// dE[prim[b]] += dX[b, 80:96]: the epilogue of the 16-column product
// dZ1 * W1[:, 80:96] (the embedding part of the layer-1 input gradient)
struct EpiEmbGrad {
  const uint32_t *prim;
  float *demb;
  int64_t B;
  __device__ void operator()(int row, int c0, const float *v) const {
    if (row >= B) return;
    float4 *dst = reinterpret_cast<float4 *>(demb + (int64_t)prim[row] * kMlpEmb);
#pragma unroll
    for (int j = 0; j < 4; j++) atomicAdd(dst + j, make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]));
  }
};

// out[C x R] = in[R x C]^T (bf16), 32x32 tiles
static __global__ void transpose_bf16(const __nv_bfloat16 *in, __nv_bfloat16 *out, int64_t R, int64_t C) {
  __shared__ __nv_bfloat16 t[32][33];
  const int64_t r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int64_t r = r0 + i, c = c0 + threadIdx.x;
    t[i][threadIdx.x] = (r < R && c < C) ? in[r * C + c] : __float2bfloat16_rn(0.f);
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int64_t c = c0 + i, r = r0 + threadIdx.x;
    if (c < C && r < R) out[c * R + r] = t[threadIdx.x][i];
  }
}

// out[j] += sum_r part[r * ld + j] for j < n.  Block = 32 columns x 8 warps;
// gridDim.y splits the rows; one atomic per (block, column).
static __global__ void __launch_bounds__(256) sum_rows_f32(const float *part, int64_t rows, int ld, int n,
                                                           float *out) {
  __shared__ float red[8][33];
  const int j = blockIdx.x * 32 + (threadIdx.x & 31), sg = threadIdx.x >> 5;
  const int64_t per = (rows + gridDim.y - 1) / gridDim.y;
  const int64_t r0 = blockIdx.y * per, r1 = min(rows, r0 + per);
  float s = 0.f;
  if (j < n) {
#pragma unroll 4
    for (int64_t r = r0 + sg; r < r1; r += 8) s += part[r * ld + j];
  }
  red[sg][threadIdx.x & 31] = s;
  __syncthreads();
  if (sg == 0 && j < n) {
    float t = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++) t += red[k][threadIdx.x];
    atomicAdd(out + j, t);
  }
}

// Adam over every parameter in one launch: segment s is elements
// [start[s], start[s + 1]) of the concatenation; the bf16 copy (w16) and the
// transposed bf16 copy (wT[(k % cols) * ldT + k / cols]) are written when set.
struct AdamSeg {
  float *w, *m, *v;
  const float *g;
  __nv_bfloat16 *w16, *wT;
  int cols, ldT;
};
constexpr int kAdamSegs = 9;
struct AdamArgs {
  AdamSeg seg[kAdamSegs];
  int64_t start[kAdamSegs + 1];
};
static __global__ void adam_all(AdamArgs a, const float *hp, float b1, float b2, float eps) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= a.start[kAdamSegs]) return;
  int s = 0;
  while (s + 1 < kAdamSegs && i >= a.start[s + 1]) s++;
  const AdamSeg &q = a.seg[s];
  const int64_t k = i - a.start[s];
  const float lr = hp[0], bc1 = hp[2], bc2 = hp[3];
  const float gi = q.g[k];
  const float mi = b1 * q.m[k] + (1.f - b1) * gi;
  const float vi = b2 * q.v[k] + (1.f - b2) * gi * gi;
  q.m[k] = mi;
  q.v[k] = vi;
  const float wi = q.w[k] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  q.w[k] = wi;
  if (q.w16) q.w16[k] = __float2bfloat16_rn(wi);
  if (q.wT) q.wT[(k % q.cols) * q.ldT + k / q.cols] = __float2bfloat16_rn(wi);
}

static __global__ void f32_to_bf16(const float *in, __nv_bfloat16 *out, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = __float2bfloat16_rn(in[i]);
}

// ---------------------------------------------------------------------------
// Fused forward: the whole MLP for 128-row tiles in one persistent kernel.
//
// One CTA per SM (512 threads) walks tiles m0 = 128 * (blockIdx.x + k *
// gridDim.x).  A tile's activations live in one 64 KB shared-memory buffer
// (128 rows x 256 bf16, SW128 K-major): the gathered input [node features |
// embedding | 0] first, then H1, H2, H3, each written over the previous
// one once the layer's MMAs have read it.  Accumulators (128 x 256 FP32)
// sit in TMEM; the epilogue adds the bias, applies GELU and writes bf16
// back into the buffer.  W1..W3 stream by TMA in 64-column chunks (32 KB)
// into four stages -- a whole layer -- while the previous epilogue runs;
// W4 (16 x 256) stays resident.  Thread 0 issues every TMA and MMA.
// Every wait is bounded: on expiry the kernel sets *err, drains its copies
// and MMAs (bounded), frees TMEM and returns.
struct FusedArgs {
  const __nv_bfloat16 *node_feat, *emb;
  const uint32_t *node, *prim;
  const float *b1, *b2, *b3, *b4;
  float *out;  // [B x 2]
  int64_t B;
  int *err;
};
constexpr int kFusedThreads = 512;  // 16 warps: 4 per accumulator lane quarter
constexpr uint32_t kActBytes = 128 * kMlpHidden * 2;        // 64 KB
constexpr uint32_t kWChunk = kMlpHidden * 128;              // 256 rows x 64 bf16 = 32 KB
constexpr uint32_t kW4Bytes = kMlpOutPad * kMlpHidden * 2;  // 8 KB
constexpr size_t kFusedSmem = 1024 + kActBytes + 4 * kWChunk + kW4Bytes + 256;

static __global__ void __launch_bounds__(kFusedThreads, 1)
    mlp_forward_fused(const __grid_constant__ CUtensorMap tw1, const __grid_constant__ CUtensorMap tw2,
                      const __grid_constant__ CUtensorMap tw3, const __grid_constant__ CUtensorMap tw4, FusedArgs a) {
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = umma::smem_u32(smem_raw);
  unsigned char *act = smem_raw + ((1024 - (raw & 1023)) & 1023);
  unsigned char *wst = act + kActBytes;           // 4 weight stages
  unsigned char *w4 = wst + 4 * kWChunk;          // resident W4, 4 k-blocks of 16 rows
  uint64_t *wfull = reinterpret_cast<uint64_t *>(w4 + kW4Bytes);  // [4]
  uint64_t *w4full = wfull + 4;
  uint64_t *done = w4full + 1;
  uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t n_tiles = (a.B + 127) / 128;
  __shared__ __align__(16) float sbias[3][kMlpHidden];  // b1..b3, read by the epilogues
  for (int i = tid; i < 3 * kMlpHidden; i += kFusedThreads)
    sbias[i / kMlpHidden][i % kMlpHidden] = (i < kMlpHidden ? a.b1 : (i < 2 * kMlpHidden ? a.b2 : a.b3))[i % kMlpHidden];
  const void *wmap[3] = {&tw1, &tw2, &tw3};
  constexpr uint32_t kIdesc = umma::idesc_bf16_f32(128, kMlpHidden);
  constexpr uint32_t kIdesc4 = umma::idesc_bf16_f32(128, kMlpOutPad);

  if (tid == 0) {
    for (int s = 0; s < 4; s++) umma::mbar_init(&wfull[s], 1);
    umma::mbar_init(w4full, 1);
    umma::mbar_init(done, 1);
    umma::mbar_fence_init();
  }
  if (warp == 0) {
    umma::tmem_alloc(tslot, 256);
    umma::tmem_relinquish();
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;

  // thread 0's bookkeeping: phase of each weight stage, loads in flight
  uint32_t wphase = 0;      // bit s: parity of the next completion of stage s
  uint32_t inflight = 0;    // bit s: a load into stage s not yet waited for
  uint32_t done_phase = 0;  // parity of the next `done` completion
  bool w4_inflight = false;
  auto load_layer = [&](int l) {  // all chunks of W(l+1), l = 0..2
    const int chunks = (l == 0 ? kMlpIn : kMlpHidden) / 64;
    for (int j = 0; j < chunks; j++) {
      umma::mbar_arrive_expect_tx(&wfull[j], kWChunk);
      umma::tma_load_2d(wst + j * kWChunk, wmap[l], 64 * j, 0, &wfull[j]);
      inflight |= 1u << j;
    }
  };
  if (tid == 0 && blockIdx.x < n_tiles) {
    umma::mbar_arrive_expect_tx(w4full, kW4Bytes);
    for (int j = 0; j < 4; j++) umma::tma_load_2d(w4 + j * (kMlpOutPad * 128), &tw4, 64 * j, 0, w4full);
    w4_inflight = true;
    load_layer(0);
  }
  bool w4_ready = false;
  bool bad = false;  // this thread saw a wait expire; block-wide decisions use __syncthreads_or

  for (int64_t t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    const int64_t m0 = t * 128;
    // ---- gather the input rows into the buffer (k-blocks 0 and 1)
    for (int i = tid; i < 128 * (kMlpIn / 8); i += kFusedThreads) {
      const int r = i / (kMlpIn / 8), c = i % (kMlpIn / 8);
      const int64_t b = m0 + r;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (b < a.B) {
        if (c < kMlpNodeFeat / 8)
          v = reinterpret_cast<const uint4 *>(a.node_feat + (int64_t)a.node[b] * kMlpNodeFeat)[c];
        else if (c < (kMlpNodeFeat + kMlpEmb) / 8)
          v = reinterpret_cast<const uint4 *>(a.emb + (int64_t)a.prim[b] * kMlpEmb)[c - kMlpNodeFeat / 8];
      }
      *reinterpret_cast<uint4 *>(act + umma::kmajor_offset(128, r, c)) = v;
    }
    umma::fence_proxy_async_smem();
    umma::fence_before_sync();
    __syncthreads();

    for (int l = 0; l < 4; l++) {
      // ---- MMAs of layer l (thread 0)
      if (tid == 0) {
        umma::fence_after_sync();
        const uint32_t a0 = umma::smem_u32(act);
        if (l < 3) {
          const int chunks = (l == 0 ? kMlpIn : kMlpHidden) / 64;
          for (int j = 0; j < chunks && !bad; j++) {
            if (!umma::mbar_wait(&wfull[j], (wphase >> j) & 1)) { bad = true; break; }
            wphase ^= 1u << j;
            inflight &= ~(1u << j);
            umma::fence_after_sync();
            const uint32_t b0 = umma::smem_u32(wst + j * kWChunk), ak = a0 + j * (128 * 128);
#pragma unroll
            for (int kk = 0; kk < 4; kk++)
              umma::mma_bf16(tmem, umma::sdesc_kmajor_sw128(ak + kk * 32), umma::sdesc_kmajor_sw128(b0 + kk * 32),
                             kIdesc, (j > 0 || kk > 0) ? 1u : 0u);
          }
        } else {
          if (!w4_ready) {
            if (umma::mbar_wait(w4full, 0)) {
              w4_ready = true;
              w4_inflight = false;
            } else {
              bad = true;
            }
          }
          for (int j = 0; j < 4 && !bad; j++) {
            const uint32_t b0 = umma::smem_u32(w4 + j * (kMlpOutPad * 128)), ak = a0 + j * (128 * 128);
#pragma unroll
            for (int kk = 0; kk < 4; kk++)
              umma::mma_bf16(tmem, umma::sdesc_kmajor_sw128(ak + kk * 32), umma::sdesc_kmajor_sw128(b0 + kk * 32),
                             kIdesc4, (j > 0 || kk > 0) ? 1u : 0u);
          }
        }
        umma::commit(done);  // also after an expired wait: arrives once the issued MMAs are done
      }
      // ---- wait for the accumulator; refill the weight stages
      if (umma::mbar_wait(done, done_phase)) done_phase ^= 1u;
      else bad = true;
      if (tid == 0 && !bad) {
        if (l == 0) load_layer(1);
        else if (l == 1) load_layer(2);
        else if (l == 2 && t + gridDim.x < n_tiles) load_layer(0);  // the next tile's W1
      }
      umma::fence_after_sync();
      // ---- epilogue: warps w, w + 4, w + 8, w + 12 share accumulator lanes
      // 32 (w % 4), 64 columns each
      const int q = warp & 3, h = warp >> 2, row = 32 * q + lane;
      const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16);
      if (l < 3 && !bad) {
        const float *bias = sbias[l];
#pragma unroll 1
        for (int c0 = 64 * h; c0 < 64 * (h + 1); c0 += 32) {
          float v[32];
          umma::tmem_ld32(lane_addr + c0, v);
          __align__(16) __nv_bfloat162 hb[16];
#pragma unroll
          for (int j = 0; j < 16; j++)
            hb[j] = __floats2bfloat162_rn(gelu(v[2 * j] + bias[c0 + 2 * j]), gelu(v[2 * j + 1] + bias[c0 + 2 * j + 1]));
#pragma unroll
          for (int k = 0; k < 4; k++)
            *reinterpret_cast<uint4 *>(act + umma::kmajor_offset(128, row, c0 / 8 + k)) =
                reinterpret_cast<const uint4 *>(hb)[k];
        }
        umma::fence_proxy_async_smem();
      } else if (l == 3 && !bad && h == 0) {
        float v[16];
        umma::tmem_ld16(lane_addr, v);
        const int64_t b = m0 + row;
        if (b < a.B) {
          a.out[b * 2] = v[0] + a.b4[0];
          a.out[b * 2 + 1] = v[1] + a.b4[1];
        }
      }
      umma::fence_before_sync();
      bad = __syncthreads_or(bad);  // the same decision in every thread
      if (bad) break;
    }
    if (bad) break;
  }
  if (bad && tid == 0) {
    atomicExch(a.err, 1);
    // copies still in flight land, and MMAs finish, before the memory goes
    for (int s = 0; s < 4; s++)
      if (inflight & (1u << s)) umma::mbar_wait(&wfull[s], (wphase >> s) & 1, 1u << 20);
    if (w4_inflight) umma::mbar_wait(w4full, 0, 1u << 20);
    umma::mbar_wait(done, done_phase, 1u << 20);
  }
  if (!bad && tid == 0 && w4_inflight) umma::mbar_wait(w4full, 0, 1u << 20);  // no tile: W4 never used
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, 256);
}


// ---------------------------------------------------------------------------
// The same forward, warp-specialised so that the input gather and each
// layer's epilogue overlap the MMAs.  Warps 0-15 run the epilogues, warp 16
// (one lane) streams W1..W3 by TMA through a 3-stage ring of 64-column
// K-chunks (10 chunks a tile, each stage freed as its MMAs complete), warp
// 17 (one lane) issues the MMAs, warps 18-25 gather the next tile's input
// rows into their own buffer while the current tile is computed.  The
// epilogue of layer l writes H_l one 64-column k-block at a time, every warp
// taking 16 columns of its lane quarter, and each finished k-block releases
// the MMAs of layer l+1 over it (mbarrier hready[j], 512 arrivals); layers
// alternate between two TMEM accumulators of 256 columns (512 allocated),
// so layer l+1 accumulates while layer l's accumulator is still being read.
// H_l is written over H_{l-1} in place: layer l's MMAs are complete before
// its epilogue writes (accfull), and layer l+1 reads only k-blocks already
// written.  The input buffer is refilled once the tile's layer-0 MMAs are
// complete (xfree).  Every wait is bounded: on expiry the kernel sets *err,
// waits (bounded) for its copies and MMAs in flight, frees TMEM and returns.
constexpr int kFused2Threads = 832;  // 16 epilogue warps + TMA warp + MMA warp + 8 gather warps
constexpr int kF2EpiThreads = 512;
constexpr int kF2GatherThreads = 256;
constexpr int kF2Stages = 3;
constexpr uint32_t kXBytes = 128 * kMlpIn * 2;  // 32 KB: the input rows of a tile
constexpr size_t kFused2Smem = 1024 + kXBytes + kActBytes + kF2Stages * kWChunk + kW4Bytes + 256;

static __global__ void __launch_bounds__(kFused2Threads, 1)
    mlp_forward_fused2(const __grid_constant__ CUtensorMap tw1, const __grid_constant__ CUtensorMap tw2,
                       const __grid_constant__ CUtensorMap tw3, const __grid_constant__ CUtensorMap tw4, FusedArgs a) {
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = umma::smem_u32(smem_raw);
  unsigned char *xin = smem_raw + ((1024 - (raw & 1023)) & 1023);
  unsigned char *act = xin + kXBytes;
  unsigned char *wst = act + kActBytes;             // kF2Stages weight stages
  unsigned char *w4 = wst + kF2Stages * kWChunk;    // resident W4, 4 k-blocks of 16 rows
  uint64_t *wfull = reinterpret_cast<uint64_t *>(w4 + kW4Bytes);  // [kF2Stages]
  uint64_t *wempty = wfull + kF2Stages;                           // [kF2Stages]
  uint64_t *hready = wempty + kF2Stages;                          // [4]
  uint64_t *w4full = hready + 4;
  uint64_t *xready = w4full + 1;
  uint64_t *xfree = xready + 1;
  uint64_t *accfull = xfree + 1;
  uint64_t *drain = accfull + 1;
  uint32_t *tslot = reinterpret_cast<uint32_t *>(drain + 1);
  __shared__ __align__(16) float sbias[3][kMlpHidden];
  __shared__ int s_bad, s_consumed, s_w4_done;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t n_tiles = (a.B + 127) / 128;
  for (int i = tid; i < 3 * kMlpHidden; i += kFused2Threads)
    sbias[i / kMlpHidden][i % kMlpHidden] = (i < kMlpHidden ? a.b1 : (i < 2 * kMlpHidden ? a.b2 : a.b3))[i % kMlpHidden];
  constexpr uint32_t kIdesc = umma::idesc_bf16_f32(128, kMlpHidden);
  constexpr uint32_t kIdesc4 = umma::idesc_bf16_f32(128, kMlpOutPad);
  if (tid == 0) {
    for (int s = 0; s < kF2Stages; s++) {
      umma::mbar_init(&wfull[s], 1);
      umma::mbar_init(&wempty[s], 1);
    }
    for (int j = 0; j < 4; j++) umma::mbar_init(&hready[j], kF2EpiThreads);
    umma::mbar_init(w4full, 1);
    umma::mbar_init(xready, kF2GatherThreads);
    umma::mbar_init(xfree, 1);
    umma::mbar_init(accfull, 1);
    umma::mbar_init(drain, 1);
    umma::mbar_fence_init();
    s_bad = 0;
    s_consumed = 0;
    s_w4_done = 0;
  }
  if (warp == 0) {
    umma::tmem_alloc(tslot, 512);
    umma::tmem_relinquish();
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;
  volatile int *bad = &s_bad;

  if (warp == 16) {
    // ---- TMA producer: W4 once, then W1 (2 chunks), W2, W3 (4 each) per tile
    if (lane == 0 && blockIdx.x < n_tiles) {
      const void *wmap[3] = {&tw1, &tw2, &tw3};
      umma::mbar_arrive_expect_tx(w4full, kW4Bytes);
      for (int j = 0; j < 4; j++) umma::tma_load_2d(w4 + j * (kMlpOutPad * 128), &tw4, 64 * j, 0, w4full);
      int cnt = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < n_tiles && ok; t += gridDim.x)
        for (int l = 0; l < 3 && ok; l++)
          for (int j = 0; j < (l == 0 ? kMlpIn : kMlpHidden) / 64; j++, cnt++) {
            const int s = cnt % kF2Stages;
            if ((cnt >= kF2Stages && !umma::mbar_wait(&wempty[s], ((cnt / kF2Stages) - 1) & 1)) || *bad) {
              *bad = 1;
              ok = false;
              break;
            }
            umma::mbar_arrive_expect_tx(&wfull[s], kWChunk);
            umma::tma_load_2d(wst + s * kWChunk, wmap[l], 64 * j, 0, &wfull[s]);
          }
      // Copies still in flight land before the block's memory goes: once the
      // MMA thread has stopped (it publishes s_w4_done; waited for at most
      // ~2 s of SM clock, far beyond any batch), the loads it did not consume
      // are waited for, bounded.
      const long long t0 = clock64();
      while (*(volatile int *)&s_w4_done == 0 && clock64() - t0 < 4000000000ll) {
      }
      if (*bad) {
        const int cons = *(volatile int *)&s_consumed;
        for (int i = cons; i < cnt; i++) umma::mbar_wait(&wfull[i % kF2Stages], (i / kF2Stages) & 1, 1u << 20);
      }
      if (*(volatile int *)&s_w4_done != 2) umma::mbar_wait(w4full, 0, 1u << 20);  // W4 never waited for
    }
  } else if (warp == 17) {
    // ---- MMA issuer
    if (lane == 0) {
      int cnt = 0, it = 0;
      bool w4_ready = false, ok = true, issued_any = false;
      for (int64_t t = blockIdx.x; t < n_tiles && ok; t += gridDim.x, it++) {
        if (!umma::mbar_wait(xready, it & 1) || *bad) { ok = false; break; }
        for (int l = 0; l < 4 && ok; l++) {
          const uint32_t acc = tmem + 256u * (uint32_t)(l & 1);
          const uint32_t a0 = umma::smem_u32(l == 0 ? xin : act);
          const int chunks = l == 0 ? kMlpIn / 64 : kMlpHidden / 64;
          if (l == 3 && !w4_ready) {
            if (!umma::mbar_wait(w4full, 0)) { ok = false; break; }
            w4_ready = true;
          }
          for (int j = 0; j < chunks; j++) {
            if (l > 0 && !umma::mbar_wait(&hready[j], (it * 3 + l - 1) & 1)) { ok = false; break; }
            if (l < 3) {
              if (!umma::mbar_wait(&wfull[cnt % kF2Stages], (cnt / kF2Stages) & 1)) { ok = false; break; }
              *(volatile int *)&s_consumed = cnt + 1;
            }
            if (*bad) { ok = false; break; }
            umma::fence_after_sync();
            const uint32_t ak = a0 + j * (128 * 128);
            const uint32_t b0 = l < 3 ? umma::smem_u32(wst + (cnt % kF2Stages) * kWChunk)
                                      : umma::smem_u32(w4 + j * (kMlpOutPad * 128));
#pragma unroll
            for (int kk = 0; kk < 4; kk++)
              umma::mma_bf16(acc, umma::sdesc_kmajor_sw128(ak + kk * 32), umma::sdesc_kmajor_sw128(b0 + kk * 32),
                             l < 3 ? kIdesc : kIdesc4, (j > 0 || kk > 0) ? 1u : 0u);
            issued_any = true;
            if (l < 3) {
              umma::commit(&wempty[cnt % kF2Stages]);
              cnt++;
            }
          }
          if (!ok) break;
          if (l == 0) umma::commit(xfree);  // the input buffer may be refilled once these MMAs are done
          umma::commit(accfull);
        }
      }
      if (!ok) *bad = 1;
      if (issued_any) {  // the MMAs issued are complete before the memory goes
        umma::commit(drain);
        umma::mbar_wait(drain, 0, 1u << 20);
      }
      *(volatile int *)&s_consumed = cnt;
      __threadfence_block();
      *(volatile int *)&s_w4_done = w4_ready ? 2 : 1;
    }
  } else if (warp >= 18) {
    // ---- gather warps: the input rows of each tile into xin, once the
    // previous tile's layer-0 MMAs have read it
    const int gt = tid - 18 * 32;
    int it = 0;
    for (int64_t t = blockIdx.x; t < n_tiles && !*bad; t += gridDim.x, it++) {
      if (it > 0 && !umma::mbar_wait(xfree, (it - 1) & 1)) { *bad = 1; break; }
      // two threads a row: the row's indices once, then its eight 16-byte
      // chunks (node features 0-9, embedding 10-11, zero 12-15) loaded
      // together before any store
      static_assert(kF2GatherThreads == 256 && kMlpIn == 128, "two gather threads per row, 8 chunks each");
      const int r = gt >> 1, c0 = 8 * (gt & 1);
      const int64_t b = t * 128 + r;
      uint4 v[8];
#pragma unroll
      for (int k = 0; k < 8; k++) v[k] = make_uint4(0, 0, 0, 0);
      if (b < a.B) {
        const uint4 *nf = reinterpret_cast<const uint4 *>(a.node_feat + (int64_t)a.node[b] * kMlpNodeFeat);
        const uint4 *em = reinterpret_cast<const uint4 *>(a.emb + (int64_t)a.prim[b] * kMlpEmb);
#pragma unroll
        for (int k = 0; k < 8; k++) {
          const int c = c0 + k;
          if (c < kMlpNodeFeat / 8) v[k] = nf[c];
          else if (c < (kMlpNodeFeat + kMlpEmb) / 8) v[k] = em[c - kMlpNodeFeat / 8];
        }
      }
#pragma unroll
      for (int k = 0; k < 8; k++) *reinterpret_cast<uint4 *>(xin + umma::kmajor_offset(128, r, c0 + k)) = v[k];
      umma::fence_proxy_async_smem();
      umma::mbar_arrive(xready);
    }
  } else {
    // ---- epilogue warps: per layer H_l by k-blocks, then the outputs
    const int q = warp & 3, h = warp >> 2, row = 32 * q + lane;
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16);
    int it = 0;
    for (int64_t t = blockIdx.x; t < n_tiles && !*bad; t += gridDim.x, it++) {
      const int64_t m0 = t * 128;
      bool ok = true;
      for (int l = 0; l < 3 && ok; l++) {
        if (!umma::mbar_wait(accfull, (it * 4 + l) & 1)) { *bad = 1; ok = false; break; }
        umma::fence_after_sync();
        const uint32_t acc = 256u * (uint32_t)(l & 1);
        const float *bias = sbias[l];
        for (int j = 0; j < 4; j++) {
          const int c0 = 64 * j + 16 * h;
          float v[16];
          umma::tmem_ld16(lane_addr + acc + c0, v);
          __align__(16) __nv_bfloat162 hb[8];
#pragma unroll
          for (int k = 0; k < 8; k++)
            hb[k] = __floats2bfloat162_rn(gelu(v[2 * k] + bias[c0 + 2 * k]), gelu(v[2 * k + 1] + bias[c0 + 2 * k + 1]));
          *reinterpret_cast<uint4 *>(act + umma::kmajor_offset(128, row, c0 / 8)) = reinterpret_cast<const uint4 *>(hb)[0];
          *reinterpret_cast<uint4 *>(act + umma::kmajor_offset(128, row, c0 / 8 + 1)) =
              reinterpret_cast<const uint4 *>(hb)[1];
          umma::fence_proxy_async_smem();
          umma::fence_before_sync();
          umma::mbar_arrive(&hready[j]);
        }
      }
      if (!ok) break;
      if (!umma::mbar_wait(accfull, (it * 4 + 3) & 1)) { *bad = 1; break; }
      umma::fence_after_sync();
      if (h == 0) {
        float v[16];
        umma::tmem_ld16(lane_addr + 256u, v);
        const int64_t b = m0 + row;
        if (b < a.B) {
          a.out[b * 2] = v[0] + a.b4[0];
          a.out[b * 2 + 1] = v[1] + a.b4[1];
        }
      }
      umma::fence_before_sync();
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  if (tid == 0 && s_bad) atomicExch(a.err, 1);
  umma::fence_after_sync();
  if (warp == 0) umma::tmem_dealloc(tmem, 512);
}

}  // namespace dpg
