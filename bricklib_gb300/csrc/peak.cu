// Arithmetic-rate probes for the compute roofline: a kernel of independent FMA
// chains per thread, timed with CUDA events on the given stream.
#include "bk_common.cuh"

namespace bk {

template <typename T, int CHAINS>
__global__ void __launch_bounds__(256) fma_rate_kernel(T *sink, int iters, T b, T c) {
  T a[CHAINS];
#pragma unroll
  for (int q = 0; q < CHAINS; ++q) a[q] = (T)(threadIdx.x + q);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int q = 0; q < CHAINS; ++q) a[q] = fma(a[q], b, c);
  }
  T s = 0;
#pragma unroll
  for (int q = 0; q < CHAINS; ++q) s += a[q];
  if (s == (T)1234.5678) sink[threadIdx.x] = s;  // keeps the chains alive
}

}  // namespace bk

using namespace bk;

extern "C" int bk_measure_fma_rate(int dtype, void *stream, double *flops_per_s) {
  if (!flops_per_s || (dtype != BK_F64 && dtype != BK_F32)) return fail(BK_ERR_ARG, "bk_measure_fma_rate: bad arguments");
  int dev = 0, sms = 0;
  BK_CUDA(cudaGetDevice(&dev));
  BK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  cudaStream_t s = as_stream(stream);
  void *sink = nullptr;
  BK_CUDA(cudaMalloc(&sink, 256 * sizeof(double)));
  const int blocks = sms * 8, threads = 256, chains = 8;
  const int iters = dtype == BK_F64 ? 256 : 8192;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0, s);
    if (dtype == BK_F64)
      fma_rate_kernel<double, chains><<<blocks, threads, 0, s>>>((double *)sink, iters, 0.999999, 1e-7);
    else
      fma_rate_kernel<float, chains><<<blocks, threads, 0, s>>>((float *)sink, iters, 0.9999f, 1e-4f);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (err != cudaSuccess) return cuda_fail(err, "fma rate kernel");
  *flops_per_s = 2.0 * blocks * threads * chains * (double)iters / (best * 1e-3);
  return BK_OK;
}
