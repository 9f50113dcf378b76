// bench_util.cu -- measurement helpers of include/dpg_bench.h.
#include <cuda_runtime.h>

#include <chrono>
#include <vector>

#include "dpg.h"
#include "dpg_bench.h"

namespace {

// 8 independent FMA chains per thread keep the FP32 pipes busy.
__global__ void __launch_bounds__(256) fma_chain(float *out, int reps, float a, float b) {
  float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  float x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < reps; i++) {
#pragma unroll
    for (int j = 0; j < 16; j++) {
      x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
      x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
    }
  }
  const float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 123.456f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

}  // namespace

extern "C" int dpg_bench_fp32_peak(int device, int iters, double *tflops) {
  if (!tflops || iters <= 0) return DPG_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return DPG_ERR_NODEVICE;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * 8, threads = 256, reps = 4096;
  float *out = nullptr;
  if (cudaMalloc(&out, sizeof(float) * blocks * threads) != cudaSuccess) return DPG_ERR_OOM;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  fma_chain<<<blocks, threads>>>(out, reps, 0.999f, 1e-4f);  // warm-up
  cudaEventRecord(a);
  for (int i = 0; i < iters; i++) fma_chain<<<blocks, threads>>>(out, reps, 0.999f, 1e-4f);
  cudaEventRecord(b);
  cudaEventSynchronize(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  const double flops = 2.0 * 8 * 16 * (double)reps * blocks * threads * iters;
  *tflops = flops / (ms * 1e-3) / 1e12;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

extern "C" int dpg_bench_flush_l2(int device, size_t bytes) {
  if (cudaSetDevice(device) != cudaSuccess) return DPG_ERR_NODEVICE;
  static void *buf = nullptr;
  static size_t have = 0;
  if (have < bytes) {
    if (buf) cudaFree(buf);
    buf = nullptr;
    have = 0;
    if (cudaMalloc(&buf, bytes) != cudaSuccess) return DPG_ERR_OOM;
    have = bytes;
  }
  cudaMemsetAsync(buf, (int)(bytes & 0xff), bytes, 0);
  return cudaDeviceSynchronize() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

extern "C" int dpg_bench_per_node_expand(dpg_ctx *ctx, const dpg_expand_opts *opts, int64_t n_nodes, int32_t nx,
                                         const double *x, int64_t *pairs, double *seconds) {
  if (!ctx || !opts || !x || !pairs || !seconds || n_nodes < 0 || nx < 1) return DPG_ERR_ARG;
  dpg_expand_opts o = *opts;
  o.x_on_device = 0;
  o.out_on_device = 0;
  int64_t cap = 0;
  void *buf[7] = {};
  auto release = [&]() {
    for (void *&p : buf) {
      dpg_host_free(p);
      p = nullptr;
    }
  };
  auto grow = [&](int64_t rows) -> bool {
    release();
    const size_t sz[7] = {4, 4, 1, 2, (size_t)8 * nx, 4, 1};
    for (int i = 0; i < 7; i++)
      if (!(buf[i] = dpg_host_alloc(sz[i] * (size_t)rows))) return false;
    cap = rows;
    return true;
  };
  if (!grow(1 << 14)) {
    release();
    return DPG_ERR_OOM;
  }
  int64_t total = 0;
  int rc = DPG_OK;
  const auto t0 = std::chrono::steady_clock::now();
  for (int64_t i = 0; i < n_nodes && rc == DPG_OK; i++) {
    for (;;) {
      dpg_expand_out out{};
      out.capacity = cap;
      out.node = (uint32_t *)buf[0];
      out.prim = (uint32_t *)buf[1];
      out.verdict = (uint8_t *)buf[2];
      out.first_invalid = (int16_t *)buf[3];
      out.end_state = buf[4];
      out.min_gap = nullptr;  // the reference's outputs: no clearance diagnostic
      out.flags = (uint8_t *)buf[6];
      rc = dpg_expand(ctx, &o, 1, x + i * nx, &out);
      if (rc == DPG_ERR_CAPACITY) {
        if (!grow(out.n_pairs)) {
          rc = DPG_ERR_OOM;
          break;
        }
        continue;
      }
      if (rc == DPG_OK) total += out.n_pairs;
      break;
    }
  }
  const auto t1 = std::chrono::steady_clock::now();
  release();
  *pairs = total;
  *seconds = std::chrono::duration<double>(t1 - t0).count();
  return rc;
}
