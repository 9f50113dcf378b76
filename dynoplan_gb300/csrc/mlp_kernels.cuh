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
static __global__ void mlp_assemble(const __nv_bfloat16 *node_feat, const __nv_bfloat16 *emb, const uint32_t *node,
                             const uint32_t *prim, int64_t B, int64_t B_pad, __nv_bfloat16 *X) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t b = i / (kMlpIn / 8);
  const int c = (int)(i % (kMlpIn / 8));
  if (b >= B_pad) return;
  uint4 v = make_uint4(0, 0, 0, 0);
  if (b < B) {
    if (c < kMlpNodeFeat / 8)
      v = reinterpret_cast<const uint4 *>(node_feat + (int64_t)node[b] * kMlpNodeFeat)[c];
    else if (c < (kMlpNodeFeat + kMlpEmb) / 8)
      v = reinterpret_cast<const uint4 *>(emb + (int64_t)prim[b] * kMlpEmb)[c - kMlpNodeFeat / 8];
  }
  reinterpret_cast<uint4 *>(X + b * kMlpIn)[c] = v;
}

__device__ __forceinline__ float softplus(float x) { return x > 20.f ? x : log1pf(__expf(x)); }
__device__ __forceinline__ float sigmoid(float x) { return 1.f / (1.f + __expf(-x)); }

// loss = mean_b [softplus(l) - y l  +  0.5 w (c - t)^2]; dY (bf16, B x 64,
// columns >= 2 zero) = d loss / d [l, c]; loss accumulated into *loss_sum
static __global__ void mlp_loss(const float *out, const float *target, int64_t B, int64_t B_pad, float ctg_weight,
                         __nv_bfloat16 *dY, float *loss_sum) {
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  float l = 0.f;
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
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0 && l != 0.f) atomicAdd(loss_sum, l);
}

// dZ = dH * gelu'(Z): the epilogue of dH = dZnext * W
struct EpiGeluGrad {
  const float *pre;
  __nv_bfloat16 *dz;
  int ld;
  __device__ void operator()(int row, int c0, const float *v) const {
    __align__(16) __nv_bfloat16 h[16];
    float z[16];
    load16(pre + (int64_t)row * ld + c0, z);
#pragma unroll
    for (int j = 0; j < 16; j++) h[j] = __float2bfloat16_rn(v[j] * gelu_grad(z[j]));
    uint4 *dst = reinterpret_cast<uint4 *>(dz + (int64_t)row * ld + c0);
    dst[0] = reinterpret_cast<const uint4 *>(h)[0];
    dst[1] = reinterpret_cast<const uint4 *>(h)[1];
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

// out[j] = sum_b in[b * ld + j] for j < n (bias gradients), block per column group
static __global__ void column_sums_bf16(const __nv_bfloat16 *in, int64_t B, int ld, int n, float *out) {
  const int j = blockIdx.x * 32 + threadIdx.x;
  float s = 0.f;
  if (j < n)
    for (int64_t b = blockIdx.y * blockDim.y + threadIdx.y; b < B; b += (int64_t)gridDim.y * blockDim.y)
      s += __bfloat162float(in[b * ld + j]);
  __shared__ float red[8][33];
  red[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && j < n) {
    float t = 0.f;
    for (int i = 0; i < blockDim.y; i++) t += red[i][threadIdx.x];
    atomicAdd(out + j, t);
  }
}

// Adam on FP32 master weights; writes the bf16 copy (and, if wT, its
// transpose of a rows x cols matrix)
static __global__ void adam_update(float *w, const float *g, float *m, float *v, int64_t n, float lr, float b1, float b2,
                            float eps, float bc1, float bc2, __nv_bfloat16 *w16, __nv_bfloat16 *wT, int rows,
                            int cols) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  w[i] = wi;
  if (w16) w16[i] = __float2bfloat16_rn(wi);
  if (wT) wT[(int64_t)(i % cols) * rows + i / cols] = __float2bfloat16_rn(wi);
}

static __global__ void f32_to_bf16(const float *in, __nv_bfloat16 *out, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = __float2bfloat16_rn(in[i]);
}

}  // namespace dpg
