// Diagnostics: the sustained FP64 / FP32 FMA issue rates of the current GPU, used to state the roofline
// of the FP64-bound kernels (no counterpart in the reference).  Eight independent FMA chains per thread,
// grid of 8 CTAs x 256 threads per SM, timed with CUDA events after a warm-up launch.
#include "mrg_internal.h"

namespace {
template <typename T, int IT>
__global__ void __launch_bounds__(256) k_fma_rate(T* out, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
#pragma unroll 4
  for (int i = 0; i < IT; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
int rate(double* r, cudaStream_t s) {
  constexpr int IT = sizeof(T) == 8 ? 2048 : 32768;
  int dev = 0, nsm = 0;
  MRG_CUDA(cudaGetDevice(&dev));
  MRG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = nsm * 8, threads = 256;
  T* out = nullptr;
  MRG_CUDA(cudaMallocAsync(&out, (size_t)blocks * threads * sizeof(T), s));
  cudaEvent_t e0, e1;
  MRG_CUDA(cudaEventCreate(&e0));
  MRG_CUDA(cudaEventCreate(&e1));
  k_fma_rate<T, IT><<<blocks, threads, 0, s>>>(out, (T)0.999, (T)0.001);
  MRG_CUDA(cudaEventRecord(e0, s));
  for (int k = 0; k < 3; ++k) k_fma_rate<T, IT><<<blocks, threads, 0, s>>>(out, (T)0.999, (T)0.001);
  MRG_CUDA(cudaEventRecord(e1, s));
  MRG_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  MRG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(out, s);
  *r = 3.0 * (double)blocks * threads * IT * 8 / (ms * 1e-3);
  return MRG_OK;
}
}  // namespace

extern "C" int mrg_measure_fma_rates(double* fp64_fma_per_s, double* fp32_fma_per_s, mrg_stream_t stream) {
  if (!fp64_fma_per_s || !fp32_fma_per_s) return mrg_fail(MRG_EINVAL, "mrg_measure_fma_rates: null argument");
  int rc = rate<double>(fp64_fma_per_s, (cudaStream_t)stream);
  if (rc) return rc;
  return rate<float>(fp32_fma_per_s, (cudaStream_t)stream);
}
