// mlp.cu -- host side of include/dpg_mlp.h: the tcgen05 BF16 GEMM and the
// surrogate MLP built on it.
#include <cuda_runtime.h>

#include <type_traits>

#include <cstring>
#include <string>

#include "dpg.h"
#include "dpg_mlp.h"
#include "gemm_kernels.cuh"

using namespace dpg;

namespace {

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

// tensor map of a row-major bf16 matrix [rows x k] read in boxes of
// 64 columns (one 128-byte swizzle row) x box_rows rows
bool make_kmajor_map(CUtensorMap *m, const void *ptr, uint64_t rows, uint64_t k, uint32_t box_rows) {
  const EncodeTiledFn fn = encode_tiled();
  if (!fn || (reinterpret_cast<uintptr_t>(ptr) & 15) || k % kGemmKChunk) return false;
  const cuuint64_t dims[2] = {k, rows};
  const cuuint64_t strides[1] = {k * sizeof(__nv_bfloat16)};
  const cuuint32_t box[2] = {(cuuint32_t)kGemmKChunk, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool g_gemm_tma = true;  // surrogate GEMMs through the TMA-fed kernel

template <int N, class Epi>
cudaError_t launch_gemm_n(const __nv_bfloat16 *A, const __nv_bfloat16 *B, int M, int K, int split, Epi epi,
                          int *err, cudaStream_t st, bool tma) {
  const int kchunks = K / kGemmKChunk;
  const int per = (kchunks + split - 1) / split * kGemmKChunk;
  dim3 grid((M + 127) / 128, (K + per - 1) / per);
  CUtensorMap ta, tb;
  if (tma && make_kmajor_map(&ta, A, (uint64_t)M, (uint64_t)K, 128) && make_kmajor_map(&tb, B, N, (uint64_t)K, N)) {
    // long K per CTA (the split-K weight gradients): the deep ring, one CTA per SM
    if constexpr (std::is_same<Epi, EpiAtomicF32>::value) {
      if (per >= 8 * kGemmKChunk) {
        constexpr int S = tma_stages_deep(N);
        auto kern = gemm_bf16_tma<N, Epi, S>;
        const size_t sm = gemm_tma_smem_bytes(N, S);
        static cudaError_t attr = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (attr != cudaSuccess) return attr;
        kern<<<grid, kTmaThreads, sm, st>>>(ta, tb, M, K, per, epi, err);
        return cudaGetLastError();
      }
    }
    constexpr int S = tma_stages(N);
    auto kern = gemm_bf16_tma<N, Epi, S>;
    const size_t sm = gemm_tma_smem_bytes(N, S);
    static cudaError_t attr = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (attr != cudaSuccess) return attr;
    kern<<<grid, kTmaThreads, sm, st>>>(ta, tb, M, K, per, epi, err);
    return cudaGetLastError();
  }
  auto kern = gemm_bf16_tn<N, Epi>;
  const size_t sm = gemm_smem_bytes(N);
  static cudaError_t attr = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (attr != cudaSuccess) return attr;
  kern<<<grid, kGemmThreads, sm, st>>>(A, B, M, K, per, epi, err);
  return cudaGetLastError();
}

// N (multiple of 16, <= 256) as a template argument
template <class Epi>
cudaError_t launch_gemm(int N, const __nv_bfloat16 *A, const __nv_bfloat16 *B, int M, int K, int split, Epi epi,
                        int *err, cudaStream_t st, bool tma = g_gemm_tma) {
  switch (N) {
#define DPG_GEMM_CASE(n) \
  case n:                \
    return launch_gemm_n<n>(A, B, M, K, split, epi, err, st, tma);
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
  if ((impl != 0 && impl != 2) || N % 16 || N > 256 || K % kGemmKChunk || split_k < 1) return DPG_ERR_ARG;
  const bool tma = impl == 2;
  if (tma && !encode_tiled()) return DPG_ERR_NODEVICE;
  if (!g_err && cudaMalloc(&g_err, sizeof(int)) != cudaSuccess) return DPG_ERR_OOM;
  cudaMemset(g_err, 0, sizeof(int));
  cudaError_t e;
  if (split_k > 1) {
    cudaMemset(C_dev, 0, sizeof(float) * (size_t)M * N);
    e = launch_gemm(N, A, B, M, K, split_k, EpiAtomicF32{C_dev, N, N}, g_err, 0, tma);
  } else {
    e = launch_gemm(N, A, B, M, K, 1, EpiStoreF32{C_dev, N, N}, g_err, 0, tma);
  }
  if (e != cudaSuccess) return DPG_ERR_CUDA;
  if (cudaDeviceSynchronize() != cudaSuccess) return DPG_ERR_CUDA;
  int h = 0;
  cudaMemcpy(&h, g_err, sizeof(int), cudaMemcpyDeviceToHost);
  return h ? DPG_ERR_TIMEOUT : DPG_OK;
}

// ---------------------------------------------------------------------------
// Failure path of the bounded waits (dpg_mlp_wait_selftest): the protocol of
// the tensor-core kernels -- TMEM allocated by warp 0, mbarriers initialised
// by thread 0, a bounded wait, on give-up an error word and the TMEM freed --
// with nothing issued that could complete the barrier, so the wait runs out
// with no copy or MMA in flight.
namespace {

__global__ void __launch_bounds__(128) wait_selftest(int *err, uint32_t polls) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  if (threadIdx.x == 0) {
    umma::mbar_init(&bar, 1);
    umma::mbar_fence_init();
  }
  if (threadIdx.x < 32) {
    umma::tmem_alloc(&tslot, 32);
    umma::tmem_relinquish();
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  // the consumer's wait: no producer arrives on `bar`
  const bool ok = threadIdx.x == 0 ? umma::mbar_wait(&bar, 0, polls) : true;
  const bool bad = __syncthreads_or(!ok);
  if (bad && threadIdx.x == 0) atomicExch(err, 1);
  umma::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) umma::tmem_dealloc(tslot, 32);
}

}  // namespace

extern "C" int dpg_mlp_wait_selftest(int device, uint32_t polls) {
  if (polls == 0 || polls > (1u << 24)) return DPG_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return DPG_ERR_NODEVICE;
  int *err = nullptr;
  if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) return DPG_ERR_OOM;
  cudaMemset(err, 0, sizeof(int));
  wait_selftest<<<1, 128>>>(err, polls);
  int h = 0;
  const cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(err);
  if (e != cudaSuccess) return DPG_ERR_CUDA;
  return h ? DPG_ERR_TIMEOUT : DPG_OK;
}

// ---------------------------------------------------------------------------
// The surrogate MLP (include/dpg_mlp.h).
#include <cmath>
#include <vector>

#include "mlp_kernels.cuh"

struct dpg_mlp {
  int device = 0;
  int P = 0;
  int64_t max_rows = 0, rows_pad = 0;
  cudaStream_t stream = nullptr;
  // FP32 master parameters, gradients, Adam moments
  float *w[DPG_MLP_NPARAM] = {}, *g[DPG_MLP_NPARAM] = {}, *m[DPG_MLP_NPARAM] = {}, *v[DPG_MLP_NPARAM] = {};
  int64_t n[DPG_MLP_NPARAM] = {};
  // bf16 operands: W16[l] [out x in], WT16[l] its transpose (layer 4 padded
  // to K = 64), emb16 the embedding table
  __nv_bfloat16 *W16[4] = {}, *WT16[4] = {}, *emb16 = nullptr;
  // activations and backward buffers (rows_pad rows)
  __nv_bfloat16 *X = nullptr, *H[3] = {}, *dZa = nullptr, *dZb = nullptr, *dY = nullptr, *T1 = nullptr,
                *T2 = nullptr;
  // training: the activations and loss gradient transposed ([cols x rows_pad],
  // the K-major operands of the weight-gradient GEMMs), written by the
  // producing kernels; T2 holds X^T, T1 the current layer's dZ^T
  __nv_bfloat16 *HT[3] = {}, *dYT = nullptr;
  float *dpart = nullptr;  // per-warp partial bias gradients [rows_pad / 32 x 256]
  __nv_bfloat16 *G[3] = {};  // gelu'(pre-activation) of layers 1-3 (training)
  float *out = nullptr, *loss = nullptr;
  int *err = nullptr;
  int step = 0;
  int fused = 2;  // forward kernel: 2 mlp_forward_fused2, 1 mlp_forward_fused, 0 layer GEMMs
  int sm_count = 0;
  // training-step inputs copied to fixed buffers, hyper-parameters in device
  // memory [lr, ctg_weight, 1 - b1^t, 1 - b2^t]: the step is captured once
  // per (batch size, feature table) as a CUDA graph and replayed
  uint32_t *in_node = nullptr, *in_prim = nullptr;
  float *in_target = nullptr, *hp = nullptr, *hp_host = nullptr;
  cudaGraphExec_t graph = nullptr;
  int64_t graph_B = -1;
  const void *graph_feat = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double last_ms = 0, last_flops = 0;
};

namespace {

constexpr int kIn[4] = {kMlpIn, kMlpHidden, kMlpHidden, kMlpHidden};
constexpr int kOut[4] = {kMlpHidden, kMlpHidden, kMlpHidden, kMlpOutPad};
constexpr int kDY = 64;  // loss-gradient row width (K of the dH3 GEMM)

__global__ void init_normal(float *w, int64_t n, float stdev, uint64_t seed, int rows_valid, int cols) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  auto mix = [](uint64_t x) {
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
  };
  const uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1);
  const uint64_t a = mix(z), b = mix(z ^ 0xD1B54A32D192ED03ull);
  const float u1 = (float)(((a >> 11) + 1) * (1.0 / 9007199254740993.0));
  const float u2 = (float)((b >> 11) * (1.0 / 9007199254740992.0));
  const float r = sqrtf(-2.f * logf(u1)) * cosf(6.2831853f * u2);
  w[i] = (i / cols < rows_valid) ? stdev * r : 0.f;
}

int64_t pad128(int64_t n) { return (n + 127) / 128 * 128; }

// bf16 copy of parameter `which` (and, for weights, the transpose)
void refresh_bf16(dpg_mlp *M, int which, cudaStream_t st) {
  const int64_t n = M->n[which];
  if (which == DPG_MLP_EMB) {
    f32_to_bf16<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(M->w[which], M->emb16, n);
    return;
  }
  if (which % 2) return;  // biases stay FP32
  const int l = which / 2, rows = kOut[l], cols = kIn[l];
  f32_to_bf16<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(M->w[which], M->W16[l], n);
  dim3 tb(32, 8), tg((cols + 31) / 32, (rows + 31) / 32);
  if (l < 3) {
    transpose_bf16<<<tg, tb, 0, st>>>(M->W16[l], M->WT16[l], rows, cols);
  } else {  // [16 x 256] -> [256 x 16] -> rows of 64 (zero padded)
    transpose_bf16<<<tg, tb, 0, st>>>(M->W16[l], M->T1, rows, cols);
    cudaMemsetAsync(M->WT16[3], 0, sizeof(__nv_bfloat16) * kMlpHidden * kDY, st);
    cudaMemcpy2DAsync(M->WT16[3], kDY * sizeof(__nv_bfloat16), M->T1, kMlpOutPad * sizeof(__nv_bfloat16),
                      kMlpOutPad * sizeof(__nv_bfloat16), kMlpHidden, cudaMemcpyDeviceToDevice, st);
  }
}

template <class T> cudaError_t dalloc(T **p, size_t count) {
  return cudaMalloc((void **)p, sizeof(T) * std::max<size_t>(count, 1));
}

// forward of rows [0, B) of the assembled X; keeps gelu'(Z) (bf16) and the
// activations transposed (HT) when train
cudaError_t forward_rows(dpg_mlp *M, int64_t B, bool train, float *out, cudaStream_t st) {
  const int64_t Bp = pad128(B);
  cudaError_t e;
  const __nv_bfloat16 *in = M->X;
  for (int l = 0; l < 3; l++) {
    EpiBiasGelu epi{M->w[2 * l + 1], train ? M->G[l] : nullptr, M->H[l], kMlpHidden, train ? M->HT[l] : nullptr, Bp};
    e = launch_gemm(kMlpHidden, in, M->W16[l], (int)Bp, kIn[l], 1, epi, M->err, st);
    if (e != cudaSuccess) return e;
    in = M->H[l];
  }
  return launch_gemm(kMlpOutPad, M->H[2], M->W16[3], (int)Bp, kMlpHidden, 1, EpiBias{M->w[DPG_MLP_B4], out, 2, 2},
                     M->err, st);
}

double forward_flops(int64_t Bp) {
  return 2.0 * Bp * ((double)kMlpIn * kMlpHidden + 2.0 * kMlpHidden * kMlpHidden + kMlpHidden * kMlpOutPad);
}

int check_err(dpg_mlp *M) {
  int h = 0;
  cudaMemcpy(&h, M->err, sizeof(int), cudaMemcpyDeviceToHost);
  return h ? DPG_ERR_TIMEOUT : DPG_OK;
}

}  // namespace

extern "C" {

int dpg_mlp_create(dpg_mlp **out, int device, int n_prims, int64_t max_rows, uint64_t seed) {
  if (!out || n_prims <= 0 || max_rows <= 0 || max_rows > ((int64_t)1 << 31) - 128) return DPG_ERR_ARG;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return DPG_ERR_NODEVICE;
  dpg_mlp *M = new dpg_mlp();
  M->device = device;
  M->P = n_prims;
  cudaDeviceGetAttribute(&M->sm_count, cudaDevAttrMultiProcessorCount, device);
  M->max_rows = max_rows;
  M->rows_pad = pad128(max_rows);
  const int64_t R = M->rows_pad;
  const int64_t sizes[DPG_MLP_NPARAM] = {(int64_t)kMlpHidden * kMlpIn, kMlpHidden, (int64_t)kMlpHidden * kMlpHidden,
                                         kMlpHidden, (int64_t)kMlpHidden * kMlpHidden, kMlpHidden,
                                         (int64_t)kMlpOutPad * kMlpHidden, kMlpOutPad, (int64_t)n_prims * kMlpEmb};
  // blocking: ordered after the caller's legacy-default-stream work
  bool ok = cudaStreamCreateWithFlags(&M->stream, cudaStreamDefault) == cudaSuccess;
  for (int i = 0; i < DPG_MLP_NPARAM && ok; i++) {
    M->n[i] = sizes[i];
    ok = dalloc(&M->w[i], sizes[i]) == cudaSuccess && dalloc(&M->g[i], sizes[i]) == cudaSuccess &&
         dalloc(&M->m[i], sizes[i]) == cudaSuccess && dalloc(&M->v[i], sizes[i]) == cudaSuccess;
  }
  for (int l = 0; l < 4 && ok; l++)
    ok = dalloc(&M->W16[l], (size_t)kOut[l] * kIn[l]) == cudaSuccess &&
         dalloc(&M->WT16[l], l < 3 ? (size_t)kOut[l] * kIn[l] : (size_t)kMlpHidden * kDY) == cudaSuccess;
  ok = ok && dalloc(&M->emb16, (size_t)n_prims * kMlpEmb) == cudaSuccess &&
       dalloc(&M->X, (size_t)R * kMlpIn) == cudaSuccess && dalloc(&M->dZa, (size_t)R * kMlpHidden) == cudaSuccess &&
       dalloc(&M->dZb, (size_t)R * kMlpHidden) == cudaSuccess && dalloc(&M->dY, (size_t)R * kDY) == cudaSuccess &&
       dalloc(&M->T1, (size_t)R * kMlpHidden) == cudaSuccess && dalloc(&M->T2, (size_t)R * kMlpHidden) == cudaSuccess &&
       dalloc(&M->out, (size_t)R * 2) == cudaSuccess && dalloc(&M->loss, 1) == cudaSuccess &&
       dalloc(&M->err, 1) == cudaSuccess;
  for (int l = 0; l < 3 && ok; l++)
    ok = dalloc(&M->H[l], (size_t)R * kMlpHidden) == cudaSuccess && dalloc(&M->G[l], (size_t)R * kMlpHidden) == cudaSuccess &&
         dalloc(&M->HT[l], (size_t)R * kMlpHidden) == cudaSuccess;
  ok = ok && dalloc(&M->dYT, (size_t)R * kMlpOutPad) == cudaSuccess &&
       dalloc(&M->dpart, (size_t)(R / 32) * kMlpHidden) == cudaSuccess;
  ok = ok && cudaEventCreate(&M->e0) == cudaSuccess && cudaEventCreate(&M->e1) == cudaSuccess;
  ok = ok && dalloc(&M->in_node, R) == cudaSuccess && dalloc(&M->in_prim, R) == cudaSuccess &&
       dalloc(&M->in_target, 2 * R) == cudaSuccess && dalloc(&M->hp, 4) == cudaSuccess &&
       cudaHostAlloc(&M->hp_host, 4 * sizeof(float), cudaHostAllocDefault) == cudaSuccess;
  if (!ok) {
    dpg_mlp_destroy(M);
    return DPG_ERR_OOM;
  }
  cudaStream_t st = M->stream;
  cudaMemsetAsync(M->err, 0, sizeof(int), st);
  const float stdv[DPG_MLP_NPARAM] = {1.f / sqrtf(96.f), 0, 1.f / 16.f, 0, 1.f / 16.f, 0, 1.f / 16.f, 0, 0.5f};
  for (int i = 0; i < DPG_MLP_NPARAM; i++) {
    const int64_t n = M->n[i];
    const int cols = (i == DPG_MLP_EMB) ? kMlpEmb : ((i % 2 == 0) ? kIn[i / 2] : (int)n);
    const int rows_valid = (i == DPG_MLP_W4) ? 2 : (int)(n / cols);
    if (stdv[i] > 0)
      init_normal<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(M->w[i], n, stdv[i], seed + 7919ull * (i + 1),
                                                               rows_valid, cols);
    else
      cudaMemsetAsync(M->w[i], 0, sizeof(float) * n, st);
    cudaMemsetAsync(M->m[i], 0, sizeof(float) * n, st);
    cudaMemsetAsync(M->v[i], 0, sizeof(float) * n, st);
    cudaMemsetAsync(M->g[i], 0, sizeof(float) * n, st);
  }
  for (int i = 0; i < DPG_MLP_NPARAM; i++) refresh_bf16(M, i, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) {
    dpg_mlp_destroy(M);
    return DPG_ERR_CUDA;
  }
  *out = M;
  return DPG_OK;
}

void dpg_mlp_destroy(dpg_mlp *M) {
  if (!M) return;
  cudaSetDevice(M->device);
  if (M->stream) cudaStreamSynchronize(M->stream);
  for (int i = 0; i < DPG_MLP_NPARAM; i++) {
    cudaFree(M->w[i]);
    cudaFree(M->g[i]);
    cudaFree(M->m[i]);
    cudaFree(M->v[i]);
  }
  for (int l = 0; l < 4; l++) {
    cudaFree(M->W16[l]);
    cudaFree(M->WT16[l]);
  }
  for (int l = 0; l < 3; l++) {
    cudaFree(M->H[l]);
    cudaFree(M->G[l]);
    cudaFree(M->HT[l]);
  }
  cudaFree(M->dYT);
  cudaFree(M->dpart);
  void *bufs[] = {M->emb16, M->X,   M->dZa,     M->dZb,     M->dY,     M->T1,  M->T2,
                  M->out,   M->loss, M->err, M->in_node, M->in_prim, M->in_target, M->hp};
  for (void *b : bufs) cudaFree(b);
  if (M->hp_host) cudaFreeHost(M->hp_host);
  if (M->graph) cudaGraphExecDestroy(M->graph);
  if (M->e0) cudaEventDestroy(M->e0);
  if (M->e1) cudaEventDestroy(M->e1);
  if (M->stream) cudaStreamDestroy(M->stream);
  delete M;
}

int64_t dpg_mlp_param_size(const dpg_mlp *M, int which) {
  return (M && which >= 0 && which < DPG_MLP_NPARAM) ? M->n[which] : -1;
}

int dpg_mlp_get(const dpg_mlp *M, int which, int grad, float *host) {
  if (!M || !host || which < 0 || which >= DPG_MLP_NPARAM) return DPG_ERR_ARG;
  cudaSetDevice(M->device);
  cudaStreamSynchronize(M->stream);
  return cudaMemcpy(host, grad ? M->g[which] : M->w[which], sizeof(float) * M->n[which], cudaMemcpyDeviceToHost) ==
                 cudaSuccess
             ? DPG_OK
             : DPG_ERR_CUDA;
}

int dpg_mlp_set(dpg_mlp *M, int which, const float *host) {
  if (!M || !host || which < 0 || which >= DPG_MLP_NPARAM) return DPG_ERR_ARG;
  cudaSetDevice(M->device);
  if (cudaMemcpyAsync(M->w[which], host, sizeof(float) * M->n[which], cudaMemcpyHostToDevice, M->stream) != cudaSuccess)
    return DPG_ERR_CUDA;
  refresh_bf16(M, which, M->stream);
  return cudaStreamSynchronize(M->stream) == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

int dpg_mlp_forward(dpg_mlp *M, const void *node_feat_dev, const uint32_t *node_dev, const uint32_t *prim_dev,
                    int64_t n, float *out_dev) {
  if (!M || !node_feat_dev || !node_dev || !prim_dev || !out_dev || n < 0) return DPG_ERR_ARG;
  cudaSetDevice(M->device);
  cudaStream_t st = M->stream;
  const auto *nf = static_cast<const __nv_bfloat16 *>(node_feat_dev);
  cudaMemsetAsync(M->err, 0, sizeof(int), st);
  cudaEventRecord(M->e0, st);
  double flops = 0;
  CUtensorMap tw[4];
  const bool fused = M->fused && n > 0 && make_kmajor_map(&tw[0], M->W16[0], kMlpHidden, kMlpIn, kMlpHidden) &&
                     make_kmajor_map(&tw[1], M->W16[1], kMlpHidden, kMlpHidden, kMlpHidden) &&
                     make_kmajor_map(&tw[2], M->W16[2], kMlpHidden, kMlpHidden, kMlpHidden) &&
                     make_kmajor_map(&tw[3], M->W16[3], kMlpOutPad, kMlpHidden, kMlpOutPad);
  if (fused) {  // one persistent kernel, one CTA per SM
    FusedArgs fa{nf, M->emb16, node_dev, prim_dev, M->w[DPG_MLP_B1], M->w[DPG_MLP_B2], M->w[DPG_MLP_B3],
                 M->w[DPG_MLP_B4], out_dev, n, M->err};
    const int64_t tiles = (n + 127) / 128;
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, std::max(M->sm_count, 1));
    if (M->fused == 2) {  // warp-specialised: epilogues overlap the next layer's MMAs
      if (cudaFuncSetAttribute(mlp_forward_fused2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFused2Smem) !=
          cudaSuccess)
        return DPG_ERR_CUDA;
      mlp_forward_fused2<<<grid, kFused2Threads, kFused2Smem, st>>>(tw[0], tw[1], tw[2], tw[3], fa);
    } else {
      if (cudaFuncSetAttribute(mlp_forward_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFusedSmem) !=
          cudaSuccess)
        return DPG_ERR_CUDA;
      mlp_forward_fused<<<grid, kFusedThreads, kFusedSmem, st>>>(tw[0], tw[1], tw[2], tw[3], fa);
    }
    if (cudaGetLastError() != cudaSuccess) return DPG_ERR_CUDA;
    flops = forward_flops(pad128(n));
  }
  for (int64_t r0 = 0; r0 < n && !fused; r0 += M->max_rows) {
    const int64_t B = std::min(M->max_rows, n - r0), Bp = pad128(B);
    const int64_t chunks = Bp * (kMlpIn / 8);
    mlp_assemble<<<(unsigned)((chunks + 255) / 256), 256, 0, st>>>(nf, M->emb16, node_dev + r0, prim_dev + r0, B, Bp,
                                                                    M->X, nullptr);
    if (forward_rows(M, B, false, out_dev + 2 * r0, st) != cudaSuccess) return DPG_ERR_CUDA;
    flops += forward_flops(Bp);
  }
  cudaEventRecord(M->e1, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return DPG_ERR_CUDA;
  float ms = 0;
  cudaEventElapsedTime(&ms, M->e0, M->e1);
  M->last_ms = ms;
  M->last_flops = flops;
  return check_err(M);
}

}  // extern "C"

// Every device operation of one training step, reading the batch from the
// fixed input buffers and the hyper-parameters from M->hp (capturable).
static cudaError_t enqueue_train(dpg_mlp *M, const __nv_bfloat16 *nf, int64_t B, cudaStream_t st) {
  const int64_t Bp = pad128(B);
  // split-K of the weight-gradient GEMMs (K = the batch): about one CTA per SM
  auto split_for = [&](int rows) {
    const int tiles = (rows + 127) / 128;
    return (int)std::max<int64_t>(1, std::min<int64_t>(std::max(M->sm_count, 1) / tiles, Bp / 512));
  };
  cudaMemsetAsync(M->err, 0, sizeof(int), st);
  cudaMemsetAsync(M->loss, 0, sizeof(float), st);
  for (int i = 0; i < DPG_MLP_NPARAM; i++) cudaMemsetAsync(M->g[i], 0, sizeof(float) * M->n[i], st);
  const int64_t chunks = Bp * (kMlpIn / 8);
  mlp_assemble<<<(unsigned)((chunks + 255) / 256), 256, 0, st>>>(nf, M->emb16, M->in_node, M->in_prim, B, Bp, M->X,
                                                                  M->T2);
  cudaError_t e = forward_rows(M, B, true, M->out, st);
  if (e != cudaSuccess) return e;
  mlp_loss<<<(unsigned)((Bp + 255) / 256), 256, 0, st>>>(M->out, M->in_target, B, Bp, M->hp, M->dY, M->loss, M->dYT,
                                                          M->g[DPG_MLP_B4]);
  // the transposed operands and the bias gradients come from the kernels that
  // produce the activations and dZ (Bp is a multiple of 128: whole warps of rows)
  auto bias_grad = [&](int which) {  // the partial column sums of the last dZ into g[which]
    sum_rows_f32<<<dim3(kMlpHidden / 32, 32), 256, 0, st>>>(M->dpart, Bp / 32, kMlpHidden, kMlpHidden, M->g[which]);
  };
  // layer 4: dW4 = dY^T H3 (16 rows), dZ3 = (dY W4) * gelu'(Z3) with dZ3^T and db3
  e = launch_gemm(kMlpHidden, M->dYT, M->HT[2], kMlpOutPad, (int)Bp, split_for(kMlpOutPad),
                  EpiAtomicF32{M->g[DPG_MLP_W4], kMlpHidden, kMlpHidden}, M->err, st);
  if (e == cudaSuccess)
    e = launch_gemm(kMlpHidden, M->dY, M->WT16[3], (int)Bp, kDY, 1,
                    EpiGeluGrad{M->G[2], M->dZa, kMlpHidden, M->T1, Bp, M->dpart}, M->err, st);
  if (e == cudaSuccess) bias_grad(DPG_MLP_B3);
  __nv_bfloat16 *dz = M->dZa, *dz_next = M->dZb;
  for (int l = 2; l >= 0 && e == cudaSuccess; l--) {  // layers 3, 2, 1: dZ^T in T1
    const __nv_bfloat16 *h_inT = l > 0 ? M->HT[l - 1] : M->T2;
    e = launch_gemm(kIn[l], M->T1, h_inT, kMlpHidden, (int)Bp, split_for(kMlpHidden),
                    EpiAtomicF32{M->g[2 * l], kIn[l], kIn[l]},
                    M->err, st);
    if (e != cudaSuccess) break;
    if (l > 0)
      e = launch_gemm(kMlpHidden, dz, M->WT16[l], (int)Bp, kMlpHidden, 1,
                      EpiGeluGrad{M->G[l - 1], dz_next, kMlpHidden, M->T1, Bp, M->dpart}, M->err, st);
    if (e == cudaSuccess && l > 0) bias_grad(2 * (l - 1) + 1);
    else
      // only the embedding columns 80..95 of dX are needed: rows 80..95 of W1^T
      e = launch_gemm(kMlpEmb, dz, M->WT16[0] + (size_t)kMlpNodeFeat * kMlpHidden, (int)Bp, kMlpHidden, 1,
                      EpiEmbGrad{M->in_prim, M->g[DPG_MLP_EMB], B}, M->err, st);
    std::swap(dz, dz_next);
  }
  if (e != cudaSuccess) return e;
  // Adam on every parameter and the bf16 operand copies, one launch
  static_assert(kAdamSegs == DPG_MLP_NPARAM, "one Adam segment per parameter");
  AdamArgs aa{};
  for (int i = 0; i < DPG_MLP_NPARAM; i++) {
    AdamSeg &q = aa.seg[i];
    q = AdamSeg{M->w[i], M->m[i], M->v[i], M->g[i], nullptr, nullptr, 1, 1};
    if (i == DPG_MLP_EMB) {
      q.w16 = M->emb16;
    } else if (i % 2 == 0) {  // weights [out x in]: bf16 copy and its transpose
      const int l = i / 2;
      q.w16 = M->W16[l];
      q.wT = M->WT16[l];
      q.cols = kIn[l];
      q.ldT = l < 3 ? kOut[l] : kDY;  // layer 4: [256 x 64] rows, columns >= 16 stay zero
    }
    aa.start[i + 1] = aa.start[i] + M->n[i];
  }
  adam_all<<<(unsigned)((aa.start[DPG_MLP_NPARAM] + 255) / 256), 256, 0, st>>>(aa, M->hp, 0.9f, 0.999f, 1e-8f);
  return cudaGetLastError();
}

extern "C" {

int dpg_mlp_train_step(dpg_mlp *M, const void *node_feat_dev, const uint32_t *node_dev, const uint32_t *prim_dev,
                       const float *target_dev, int64_t B, float lr, float ctg_weight, float *loss) {
  if (!M || !node_feat_dev || !node_dev || !prim_dev || !target_dev || B <= 0 || B > M->max_rows) return DPG_ERR_ARG;
  cudaSetDevice(M->device);
  cudaStream_t st = M->stream;
  const auto *nf = static_cast<const __nv_bfloat16 *>(node_feat_dev);
  // this step's batch and hyper-parameters into the fixed buffers
  M->step++;
  M->hp_host[0] = lr;
  M->hp_host[1] = ctg_weight;
  M->hp_host[2] = 1.f - powf(0.9f, (float)M->step);
  M->hp_host[3] = 1.f - powf(0.999f, (float)M->step);
  cudaMemcpyAsync(M->in_node, node_dev, sizeof(uint32_t) * B, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(M->in_prim, prim_dev, sizeof(uint32_t) * B, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(M->in_target, target_dev, sizeof(float) * 2 * B, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(M->hp, M->hp_host, 4 * sizeof(float), cudaMemcpyHostToDevice, st);
  // the step as a CUDA graph, captured on first use for this batch size and
  // feature table; without a graph (capture refused) the step runs eagerly
  if (!(M->graph && M->graph_B == B && M->graph_feat == nf)) {
    if (M->graph) cudaGraphExecDestroy(M->graph);
    M->graph = nullptr;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      const cudaError_t e = enqueue_train(M, nf, B, st);
      const cudaError_t ee = cudaStreamEndCapture(st, &g);
      if (e == cudaSuccess && ee == cudaSuccess && g && cudaGraphInstantiate(&M->graph, g, 0) == cudaSuccess) {
        M->graph_B = B;
        M->graph_feat = nf;
      } else {
        M->graph = nullptr;
      }
      if (g) cudaGraphDestroy(g);
    }
    cudaGetLastError();  // a refused capture leaves no error behind
  }
  cudaEventRecord(M->e0, st);
  if (M->graph) {
    if (cudaGraphLaunch(M->graph, st) != cudaSuccess) return DPG_ERR_CUDA;
  } else if (enqueue_train(M, nf, B, st) != cudaSuccess) {
    return DPG_ERR_CUDA;
  }
  cudaEventRecord(M->e1, st);
  float hl = 0;
  cudaMemcpyAsync(&hl, M->loss, sizeof(float), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return DPG_ERR_CUDA;
  if (loss) *loss = hl / (float)B;
  float ms = 0;
  cudaEventElapsedTime(&ms, M->e0, M->e1);
  M->last_ms = ms;
  // forward + the two backward GEMMs per layer
  M->last_flops = 3.0 * forward_flops(pad128(B));
  return check_err(M);
}

int dpg_mlp_set_fused(dpg_mlp *M, int fused) {
  if (!M) return DPG_ERR_ARG;
  if (fused < 0 || fused > 2) return DPG_ERR_ARG;
  M->fused = fused;
  return DPG_OK;
}

int dpg_mlp_last_timing(const dpg_mlp *M, double *ms, double *flops) {
  if (!M) return DPG_ERR_ARG;
  if (ms) *ms = M->last_ms;
  if (flops) *flops = M->last_flops;
  return DPG_OK;
}

}  // extern "C"
