// gemm_kernels.cuh -- BF16 GEMM on the 5th-generation tensor cores (sm_103a).
//
//   C[M x N] = A[M x K] * B[N x K]^T      A, B bf16 row-major (K contiguous),
//                                          FP32 accumulation in tensor memory
//
// One CTA of 128 threads computes a 128-row tile with every N column (N a
// multiple of 16, <= 256) in one tcgen05.mma chain of M=128 x N x K=16
// instructions; gridDim.y splits K.  K is consumed in chunks of 64 (one
// 128-byte swizzle atom) staged into two shared-memory buffers: threads
// stage chunk i+1 while the tensor cores run chunk i; an mbarrier that the
// MMA commit arrives on tells the stagers when a buffer is free again.
// Every wait is bounded: on expiry the kernel sets *err, drains, frees its
// tensor memory and returns.  The epilogue reads one accumulator row per
// thread (tcgen05.ld 32x32b) and hands 16 columns at a time to `Epi`.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

#include "umma.cuh"

namespace dpg {

constexpr int kGemmThreads = 128;
constexpr int kGemmKChunk = 64;

__host__ __device__ constexpr int tmem_cols_for(int n) {
  return n <= 32 ? 32 : (n <= 64 ? 64 : (n <= 128 ? 128 : 256));
}
__host__ __device__ constexpr size_t gemm_smem_bytes(int N) {
  // two stages of (A 128x64 + B Nx64) bf16, 1024-aligned, + barriers + slack
  return 2 * (size_t)(128 * 128 + N * 128) + 1024 + 64;
}

template <int N, class Epi>
__global__ void __launch_bounds__(kGemmThreads) gemm_bf16_tn(const __nv_bfloat16 *__restrict__ A,
                                                              const __nv_bfloat16 *__restrict__ B, int M,
                                                              int K, int k_per_split, Epi epi, int *err) {
  static_assert(N % 16 == 0 && N >= 16 && N <= 256, "N");
  extern __shared__ unsigned char smem_raw[];
  // 1024-byte aligned stage buffers
  const uint32_t raw = umma::smem_u32(smem_raw);
  unsigned char *base = smem_raw + ((1024 - (raw & 1023)) & 1023);
  constexpr int kA = 128 * 128, kB = N * 128;
  unsigned char *tileA[2] = {base, base + kA + kB};
  unsigned char *tileB[2] = {base + kA, base + 2 * kA + kB};
  uint64_t *mbar = reinterpret_cast<uint64_t *>(base + 2 * (kA + kB));
  uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + 2);
  __shared__ int s_bad;

  const int m0 = blockIdx.x * 128;
  const int kbeg = blockIdx.y * k_per_split;
  const int kend = min(K, kbeg + k_per_split);
  const int nchunks = (kend - kbeg) / kGemmKChunk;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr uint32_t kCols = tmem_cols_for(N);
  constexpr uint32_t idesc = umma::idesc_bf16_f32(128, N);

  if (threadIdx.x == 0) {
    umma::mbar_init(&mbar[0], 1);
    umma::mbar_init(&mbar[1], 1);
    umma::mbar_fence_init();
    s_bad = 0;
  }
  if (warp == 0) {
    umma::tmem_alloc(tslot, kCols);
    umma::tmem_relinquish();
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;
  const int rows_valid = min(128, M - m0);

  bool bad = false;
  int issued = 0;  // chunks whose MMAs were issued (identical in every thread)
  for (int i = 0; i < nchunks && !bad; i++) {
    const int s = i & 1;
    if (i >= 2) {  // buffer s is free once the MMAs of chunk i-2 are done
      bool ok = umma::mbar_wait(&mbar[s], ((i - 2) >> 1) & 1);
      if (__syncthreads_or(!ok)) { bad = true; break; }
    }
    const int k0 = kbeg + i * kGemmKChunk;
    umma::stage_kmajor(tileA[s], A + (int64_t)m0 * K, K, 128, rows_valid, k0, 1);
    umma::stage_kmajor(tileB[s], B, K, N, N, k0, 1);
    umma::fence_proxy_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      umma::fence_after_sync();
      const uint32_t a0 = umma::smem_u32(tileA[s]), b0 = umma::smem_u32(tileB[s]);
#pragma unroll
      for (int kk = 0; kk < kGemmKChunk / 16; kk++)
        umma::mma_bf16(tmem, umma::sdesc_kmajor_sw128(a0 + kk * 32), umma::sdesc_kmajor_sw128(b0 + kk * 32),
                       idesc, (i > 0 || kk > 0) ? 1u : 0u);
      umma::commit(&mbar[s]);
    }
    issued = i + 1;
  }
  if (!bad && nchunks > 0) {  // all MMAs done
    const int last = nchunks - 1;
    bool ok = umma::mbar_wait(&mbar[last & 1], (last >> 1) & 1);
    bad = __syncthreads_or(!ok);
  }
  if (bad) {
    if (threadIdx.x == 0) atomicExch(err, 1);
    // let in-flight MMAs finish before the tensor memory is released
    if (issued > 0) umma::mbar_wait(&mbar[(issued - 1) & 1], ((issued - 1) >> 1) & 1, 1u << 20);
  } else if (nchunks > 0) {
    umma::fence_after_sync();
    const int row = 32 * warp + lane;
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * warp) << 16);
#pragma unroll 1
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      umma::tmem_ld16(lane_addr + c0, v);
      if (m0 + row < M) epi(m0 + row, c0, v);
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, kCols);
}

// ---- TMA-fed, warp-specialised form ------------------------------------------
//
// Same contract and tile (128 rows x all N columns in TMEM, K in 64-wide
// SW128 k-blocks), but the operands arrive by TMA (cp.async.bulk.tensor,
// 128-byte swizzle written by the copy engine) into a ring of S stages:
// thread 0 of warp 0 issues the loads, thread 0 of warp 1 the MMAs; a stage
// is refilled once the MMAs that read it have committed to its `empty`
// barrier.  All four warps run the epilogue.  Rows beyond M load as zeros.
// Every wait is bounded; on expiry the kernel sets *err, waits (bounded)
// for its copies and MMAs in flight, frees its tensor memory and returns.
__host__ __device__ constexpr int tma_stages(int N) {
  return (110 * 1024) / (128 * 128 + N * 128) < 2 ? 2
         : ((110 * 1024) / (128 * 128 + N * 128) > 4 ? 4 : (110 * 1024) / (128 * 128 + N * 128));
}
// deeper ring for long K (one CTA per SM): up to 200 KB of stages
__host__ __device__ constexpr int tma_stages_deep(int N) {
  return (200 * 1024) / (128 * 128 + N * 128) < 2 ? 2
         : ((200 * 1024) / (128 * 128 + N * 128) > 6 ? 6 : (200 * 1024) / (128 * 128 + N * 128));
}
__host__ __device__ constexpr size_t gemm_tma_smem_bytes(int N, int S) {
  return (size_t)S * (128 * 128 + N * 128) + 1024 + 256;
}

constexpr int kTmaThreads = 256;  // 8 warps: all of them drain the accumulator

template <int N, class Epi, int S = tma_stages(N)>
__global__ void __launch_bounds__(kTmaThreads) gemm_bf16_tma(const __grid_constant__ CUtensorMap tmA,
                                                               const __grid_constant__ CUtensorMap tmB, int M,
                                                               int K, int k_per_split, Epi epi, int *err) {
  static_assert(N % 16 == 0 && N >= 16 && N <= 256, "N");
  static_assert(S >= 2, "stages");
  constexpr uint32_t kA = 128 * 128, kB = N * 128, kStage = kA + kB;
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = umma::smem_u32(smem_raw);
  unsigned char *base = smem_raw + ((1024 - (raw & 1023)) & 1023);
  uint64_t *full = reinterpret_cast<uint64_t *>(base + S * kStage);
  uint64_t *empty = full + S;
  uint64_t *done = empty + S;
  uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
  __shared__ int s_bad;

  const int m0 = blockIdx.x * 128;
  const int kbeg = blockIdx.y * k_per_split;
  const int kend = min(K, kbeg + k_per_split);
  const int nchunks = (kend - kbeg) / kGemmKChunk;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr uint32_t kCols = tmem_cols_for(N);
  constexpr uint32_t idesc = umma::idesc_bf16_f32(128, N);

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; s++) {
      umma::mbar_init(&full[s], 1);
      umma::mbar_init(&empty[s], 1);
    }
    umma::mbar_init(done, 1);
    umma::mbar_fence_init();
    s_bad = 0;
  }
  if (warp == 0) {
    umma::tmem_alloc(tslot, kCols);
    umma::tmem_relinquish();
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;

  int loads = 0;  // (thread 0) chunks whose loads were issued
  if (threadIdx.x == 0) {
    // producer
    for (int i = 0; i < nchunks; i++) {
      const int s = i % S;
      if (i >= S && !umma::mbar_wait(&empty[s], ((i / S) - 1) & 1)) {
        s_bad = 1;
        break;
      }
      if (*(volatile int *)&s_bad) break;
      unsigned char *a = base + s * kStage;
      umma::mbar_arrive_expect_tx(&full[s], kStage);
      umma::tma_load_2d(a, &tmA, kbeg + i * kGemmKChunk, m0, &full[s]);
      umma::tma_load_2d(a + kA, &tmB, kbeg + i * kGemmKChunk, 0, &full[s]);
      loads = i + 1;
    }
  } else if (threadIdx.x == 32) {
    // MMA issuer
    for (int i = 0; i < nchunks; i++) {
      const int s = i % S;
      if (!umma::mbar_wait(&full[s], (i / S) & 1)) {
        s_bad = 1;
        break;
      }
      umma::fence_after_sync();
      const uint32_t a0 = umma::smem_u32(base + s * kStage), b0 = a0 + kA;
#pragma unroll
      for (int kk = 0; kk < kGemmKChunk / 16; kk++)
        umma::mma_bf16(tmem, umma::sdesc_kmajor_sw128(a0 + kk * 32), umma::sdesc_kmajor_sw128(b0 + kk * 32),
                       idesc, (i > 0 || kk > 0) ? 1u : 0u);
      umma::commit(&empty[s]);
    }
    umma::commit(done);  // arrives once every MMA issued above is complete
  }
  // everyone: the accumulator is final once `done` completes
  const bool ok = nchunks > 0 && umma::mbar_wait(done, 0);
  const bool bad = __syncthreads_or(!ok || s_bad) && nchunks > 0;
  if (bad) {
    if (threadIdx.x == 0) {
      atomicExch(err, 1);
      // copies still in flight land before the block's shared memory goes
      for (int i = max(0, loads - S); i < loads; i++) umma::mbar_wait(&full[i % S], (i / S) & 1, 1u << 20);
    }
  } else if (nchunks > 0) {
    // warp w reads accumulator lanes 32 (w % 4) ...; warps 0-3 and 4-7 split
    // the columns in halves (all columns in warps 0-3 when N / 2 is not a
    // multiple of 16)
    constexpr int kHalves = (N % 32 == 0) ? 2 : 1, kNC = N / kHalves;
    const int q = warp & 3, h = warp >> 2;
    if (h < kHalves) {
      umma::fence_after_sync();
      const int row = 32 * q + lane;
      const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16);
#pragma unroll 1
      for (int c0 = h * kNC; c0 < (h + 1) * kNC; c0 += 16) {
        float v[16];
        umma::tmem_ld16(lane_addr + c0, v);
        if (m0 + row < M) epi(m0 + row, c0, v);
      }
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, kCols);
}

// ---- epilogues ---------------------------------------------------------------
// 16 consecutive FP32 values as four 16-byte stores (dst 16-byte aligned)
__device__ __forceinline__ void store16(float *dst, const float *v) {
#pragma unroll
  for (int j = 0; j < 4; j++)
    reinterpret_cast<float4 *>(dst)[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
}
__device__ __forceinline__ void load16(const float *src, float *v) {
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const float4 t = reinterpret_cast<const float4 *>(src)[j];
    v[4 * j] = t.x; v[4 * j + 1] = t.y; v[4 * j + 2] = t.z; v[4 * j + 3] = t.w;
  }
}

struct EpiStoreF32 {  // C = acc (ldc = row stride, only columns < n_valid)
  float *C;
  int ldc, n_valid;
  __device__ void operator()(int row, int c0, const float *v) const {
    float *dst = C + (int64_t)row * ldc + c0;
    if (c0 + 16 <= n_valid && (ldc & 3) == 0) {
      store16(dst, v);
      return;
    }
#pragma unroll
    for (int j = 0; j < 16; j++)
      if (c0 + j < n_valid) dst[j] = v[j];
  }
};
struct EpiAtomicF32 {  // C += acc (split-K partial sums)
  float *C;
  int ldc, n_valid;
  __device__ void operator()(int row, int c0, const float *v) const {
    float *dst = C + (int64_t)row * ldc + c0;
    if (c0 + 16 <= n_valid && (ldc & 3) == 0) {  // 16-byte vector atomics
#pragma unroll
      for (int j = 0; j < 4; j++)
        atomicAdd(reinterpret_cast<float4 *>(dst) + j, make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]));
      return;
    }
#pragma unroll
    for (int j = 0; j < 16; j++)
      if (c0 + j < n_valid) atomicAdd(dst + j, v[j]);
  }
};

// GELU in its tanh form (Hendrycks & Gimpel, "Gaussian Error Linear Units",
// 2016): gelu(z) = z/2 (1 + tanh(u)), u = sqrt(2/pi) (z + 0.044715 z^3), with
// the hardware tanh (tanh.approx.f32, max relative error about 2^-11, below
// the bf16 rounding the activations get).
__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
constexpr float kGeluA = 0.7978845608028654f, kGeluB = 0.044715f;
__device__ __forceinline__ float gelu(float z) {
  const float t = tanh_fast(kGeluA * z * fmaf(kGeluB * z, z, 1.0f));
  return 0.5f * z * (1.0f + t);
}
__device__ __forceinline__ float gelu_grad(float z) {
  const float t = tanh_fast(kGeluA * z * fmaf(kGeluB * z, z, 1.0f));
  const float du = kGeluA * fmaf(3.0f * kGeluB * z, z, 1.0f);
  return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * du;
}

// Transposed store of a warp's 32 rows x 16 columns of bf16 (lane = row,
// h = the lane's 16 values of columns c0..c0+15): staged in shared memory,
// then written as 16-byte runs, dst[(c0 + c) * ldt + row0 + r] for the warp's
// first row row0.  With colsum set, lanes c < 16 also write the sum over the
// 32 rows of column c0 + c to colsum[c].  All 32 lanes must call it (M a
// multiple of 32); row0 and ldt multiples of 8.
__device__ __forceinline__ void store_transposed16(__nv_bfloat16 *dst, int64_t ldt, int row, int c0,
                                                   const __nv_bfloat16 *h, float *colsum = nullptr) {
  __shared__ __align__(16) __nv_bfloat16 tbuf[kTmaThreads / 32][16][40];  // 80-byte rows
  const int w = (threadIdx.x >> 5) % (kTmaThreads / 32), lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < 16; j++) tbuf[w][j][lane] = h[j];
  __syncwarp();
  const int row0 = row - lane;
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const int q = lane + 32 * k, c = q >> 2, part = q & 3;  // column c, rows 8 part .. 8 part + 7
    const uint4 val = *reinterpret_cast<const uint4 *>(&tbuf[w][c][8 * part]);
    *reinterpret_cast<uint4 *>(dst + (int64_t)(c0 + c) * ldt + row0 + 8 * part) = val;
  }
  if (colsum && lane < 16) {
    float t = 0.f;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const uint4 val = *reinterpret_cast<const uint4 *>(&tbuf[w][lane][8 * k]);
      const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&val);
#pragma unroll
      for (int i = 0; i < 8; i++) t += __bfloat162float(e[i]);
    }
    colsum[lane] = t;
  }
  __syncwarp();
}

// z = acc + bias; keeps gelu'(z) in bf16 for the backward pass when
// dgelu != nullptr; writes gelu(z) in bf16, and also transposed (actT[col *
// ldt + row], the K-major operand of the weight-gradient GEMM) when actT !=
// nullptr (M a multiple of 32)
struct EpiBiasGelu {
  const float *bias;
  __nv_bfloat16 *dgelu;
  __nv_bfloat16 *act;
  int ld;
  __nv_bfloat16 *actT = nullptr;
  int64_t ldt = 0;
  __device__ void operator()(int row, int c0, const float *v) const {
    __align__(16) __nv_bfloat16 h[16];
    float z[16];
    load16(bias + c0, z);
#pragma unroll
    for (int j = 0; j < 16; j++) z[j] += v[j];
    if (dgelu) {
      __align__(16) __nv_bfloat16 d[16];
#pragma unroll
      for (int j = 0; j < 16; j++) d[j] = __float2bfloat16_rn(gelu_grad(z[j]));
      uint4 *gd = reinterpret_cast<uint4 *>(dgelu + (int64_t)row * ld + c0);
      gd[0] = reinterpret_cast<const uint4 *>(d)[0];
      gd[1] = reinterpret_cast<const uint4 *>(d)[1];
    }
#pragma unroll
    for (int j = 0; j < 16; j++) h[j] = __float2bfloat16_rn(gelu(z[j]));
    uint4 *dst = reinterpret_cast<uint4 *>(act + (int64_t)row * ld + c0);
    dst[0] = reinterpret_cast<const uint4 *>(h)[0];
    dst[1] = reinterpret_cast<const uint4 *>(h)[1];
    if (actT) store_transposed16(actT, ldt, row, c0, h);
  }
};
// out = acc + bias (FP32), first n_valid columns
struct EpiBias {
  const float *bias;
  float *out;
  int ld, n_valid;
  __device__ void operator()(int row, int c0, const float *v) const {
#pragma unroll
    for (int j = 0; j < 16; j++)
      if (c0 + j < n_valid) out[(int64_t)row * ld + c0 + j] = v[j] + bias[c0 + j];
  }
};

// ---- SIMT reference (CUDA cores, FP32 accumulation) ---------------------------
static __global__ void gemm_bf16_ref(const __nv_bfloat16 *A, const __nv_bfloat16 *B, float *C, int M, int N, int K) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)M * N) return;
  const int m = (int)(i / N), n = (int)(i % N);
  float s = 0.f;
  for (int k = 0; k < K; k++) s += __bfloat162float(A[(int64_t)m * K + k]) * __bfloat162float(B[(int64_t)n * K + k]);
  C[i] = s;
}

}  // namespace dpg
