// Shared helpers of libbrick_gb300: status handling, element types, layout math.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include <string>

#include "bricklib_gb300.h"

namespace bk {

// ---------------------------------------------------------------- status

void set_error(const std::string &msg);
int fail(int status, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

#define BK_CUDA(call)                                   \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return bk::cuda_fail(e_, #call); \
  } while (0)

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Device word of error flags, one per device, set by kernels with atomicOr.
int *device_error_word();
constexpr int FLAG_BOUNDS = 1;
constexpr int FLAG_TIMEOUT = 2;

inline size_t dtype_size(int dt) { return dt == BK_F64 ? 8 : dt == BK_F32 ? 4 : 2; }
inline bool dtype_ok(int dt) { return dt == BK_F64 || dt == BK_F32 || dt == BK_BF16; }

// ---------------------------------------------------------------- element types

template <typename T> struct Elem;
template <> struct Elem<double> {
  typedef double acc;
  static __device__ __forceinline__ double load(const double *p) { return __ldg(p); }
  static __device__ __forceinline__ void store(double *p, double v) { *p = v; }
};
template <> struct Elem<float> {
  typedef float acc;
  static __device__ __forceinline__ float load(const float *p) { return __ldg(p); }
  static __device__ __forceinline__ void store(float *p, float v) { *p = v; }
};
template <> struct Elem<__nv_bfloat16> {
  typedef float acc;
  static __device__ __forceinline__ float load(const __nv_bfloat16 *p) { return __bfloat162float(*p); }
  static __device__ __forceinline__ void store(__nv_bfloat16 *p, float v) { *p = __float2bfloat16_rn(v); }
};

// ---------------------------------------------------------------- layout

// In-brick offset of element (k,j,i) for brick dims B and fold F (all (k,j,i)).
struct Layout {
  int bk, bj, bi, fk, fj, fi;
  __host__ __device__ __forceinline__ int offset(int k, int j, int i) const {
    const int vl = fk * fj * fi;
    const int vec = ((k / fk) * (bj / fj) + j / fj) * (bi / fi) + i / fi;
    const int lane = ((k % fk) * fj + j % fj) * fi + i % fi;
    return vec * vl + lane;
  }
  __host__ __device__ __forceinline__ int size() const { return bk * bj * bi; }
  // true when offset(k,j,i) == (k*bj + j)*bi + i for every element
  __host__ bool row_major() const {
    for (int k = 0; k < bk; ++k)
      for (int j = 0; j < bj; ++j)
        for (int i = 0; i < bi; ++i)
          if (offset(k, j, i) != (k * bj + j) * bi + i) return false;
    return true;
  }
};

int check_layout(const bk_layout *lay, Layout *out);
int check_field(const bk_field *f, const Layout &L, const char *name);
int check_disjoint(const bk_field *in, const bk_field *out, size_t brick_elems);

}  // namespace bk
