// Seeded synthetic inputs generated on the device.  Element n of seed s is
// lo + (hi - lo) * u, u = (splitmix64(s + n) >> 11) * 2^-53, evaluated with
// separately rounded double operations so the values equal a host evaluation
// of the same formula bit for bit.
#include "bk_common.cuh"

namespace bk {

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

template <typename T>
__global__ void __launch_bounds__(256)
fill_uniform_kernel(T *dat, unsigned long long n, unsigned long long seed, double lo, double span) {
  for (unsigned long long p = blockIdx.x * 256ull + threadIdx.x; p < n; p += (unsigned long long)gridDim.x * 256ull) {
    const double u = (double)(splitmix64(seed + p) >> 11) * (1.0 / 9007199254740992.0);
    const double v = __dadd_rn(lo, __dmul_rn(span, u));
    Elem<T>::store(dat + p, (typename Elem<T>::acc)v);
  }
}

}  // namespace bk

using namespace bk;

extern "C" int bk_fill_uniform(void *dat, size_t n, int dtype, uint64_t seed, double lo, double hi, void *stream) {
  if (n == 0) return BK_OK;
  if (!dat || !dtype_ok(dtype)) return fail(BK_ERR_ARG, "bk_fill_uniform: bad arguments");
  int dev = 0, sms = 0;
  BK_CUDA(cudaGetDevice(&dev));
  BK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  unsigned long long blocks = (n + 255) / 256;
  if (blocks > (unsigned long long)sms * 64) blocks = (unsigned long long)sms * 64;
  cudaStream_t s = as_stream(stream);
  switch (dtype) {
    case BK_F64: fill_uniform_kernel<double><<<(unsigned)blocks, 256, 0, s>>>((double *)dat, n, seed, lo, hi - lo); break;
    case BK_F32: fill_uniform_kernel<float><<<(unsigned)blocks, 256, 0, s>>>((float *)dat, n, seed, lo, hi - lo); break;
    case BK_BF16:
      fill_uniform_kernel<__nv_bfloat16><<<(unsigned)blocks, 256, 0, s>>>((__nv_bfloat16 *)dat, n, seed, lo, hi - lo);
      break;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "fill kernel launch");
  return BK_OK;
}
