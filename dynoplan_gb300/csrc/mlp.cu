// mlp.cu -- host side of include/dpg_mlp.h: the tcgen05 BF16 GEMM and the
// surrogate MLP built on it.
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "dpg.h"
#include "dpg_mlp.h"
#include "gemm_kernels.cuh"

using namespace dpg;

namespace {

template <int N, class Epi>
cudaError_t launch_gemm_n(const __nv_bfloat16 *A, const __nv_bfloat16 *B, int M, int K, int split, Epi epi,
                          int *err, cudaStream_t st) {
  auto kern = gemm_bf16_tn<N, Epi>;
  const size_t sm = gemm_smem_bytes(N);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  const int kchunks = K / kGemmKChunk;
  const int per = (kchunks + split - 1) / split * kGemmKChunk;
  dim3 grid((M + 127) / 128, (K + per - 1) / per);
  kern<<<grid, kGemmThreads, sm, st>>>(A, B, M, K, per, epi, err);
  return cudaGetLastError();
}

// N (multiple of 16, <= 256) as a template argument
template <class Epi>
cudaError_t launch_gemm(int N, const __nv_bfloat16 *A, const __nv_bfloat16 *B, int M, int K, int split, Epi epi,
                        int *err, cudaStream_t st) {
  switch (N) {
#define DPG_GEMM_CASE(n) \
  case n:                \
    return launch_gemm_n<n>(A, B, M, K, split, epi, err, st);
    DPG_GEMM_CASE(16) DPG_GEMM_CASE(32) DPG_GEMM_CASE(48) DPG_GEMM_CASE(64) DPG_GEMM_CASE(80)
    DPG_GEMM_CASE(96) DPG_GEMM_CASE(112) DPG_GEMM_CASE(128) DPG_GEMM_CASE(144) DPG_GEMM_CASE(160)
    DPG_GEMM_CASE(176) DPG_GEMM_CASE(192) DPG_GEMM_CASE(208) DPG_GEMM_CASE(224) DPG_GEMM_CASE(240)
    DPG_GEMM_CASE(256)
#undef DPG_GEMM_CASE
  }
  return cudaErrorInvalidValue;
}

int *g_err = nullptr;  // per-process device error word of the bounded waits (device 0 context)

}  // namespace

extern "C" int dpg_gemm_bf16(const void *A_dev, const void *B_dev, float *C_dev, int M, int N, int K, int impl,
                             int split_k) {
  if (!A_dev || !B_dev || !C_dev || M <= 0 || N <= 0 || K <= 0) return DPG_ERR_ARG;
  const auto *A = static_cast<const __nv_bfloat16 *>(A_dev);
  const auto *B = static_cast<const __nv_bfloat16 *>(B_dev);
  if (impl == 1) {
    const int64_t n = (int64_t)M * N;
    gemm_bf16_ref<<<(unsigned)((n + 255) / 256), 256>>>(A, B, C_dev, M, N, K);
    return cudaDeviceSynchronize() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
  }
  if (impl != 0 || N % 16 || N > 256 || K % kGemmKChunk || split_k < 1) return DPG_ERR_ARG;
  if (!g_err && cudaMalloc(&g_err, sizeof(int)) != cudaSuccess) return DPG_ERR_OOM;
  cudaMemset(g_err, 0, sizeof(int));
  cudaError_t e;
  if (split_k > 1) {
    cudaMemset(C_dev, 0, sizeof(float) * (size_t)M * N);
    e = launch_gemm(N, A, B, M, K, split_k, EpiAtomicF32{C_dev, N, N}, g_err, 0);
  } else {
    e = launch_gemm(N, A, B, M, K, 1, EpiStoreF32{C_dev, N, N}, g_err, 0);
  }
  if (e != cudaSuccess) return DPG_ERR_CUDA;
  if (cudaDeviceSynchronize() != cudaSuccess) return DPG_ERR_CUDA;
  int h = 0;
  cudaMemcpy(&h, g_err, sizeof(int), cudaMemcpyDeviceToHost);
  return h ? DPG_ERR_TIMEOUT : DPG_OK;
}
