// Precision-form support: field conversion between storage types, FP64 error norms of
// one field against a reference field, and the seeded sum-of-sines initial field.
#include <mutex>
#include <vector>

#include "bk_common.cuh"

namespace bk {

template <typename T> __device__ __forceinline__ double to_f64(T x);
template <> __device__ __forceinline__ double to_f64<double>(double x) { return x; }
template <> __device__ __forceinline__ double to_f64<float>(float x) { return (double)x; }
template <> __device__ __forceinline__ double to_f64<__nv_bfloat16>(__nv_bfloat16 x) { return (double)__bfloat162float(x); }

template <typename D> __device__ __forceinline__ D from_f64(double x);
template <> __device__ __forceinline__ double from_f64<double>(double x) { return x; }
template <> __device__ __forceinline__ float from_f64<float>(double x) { return __double2float_rn(x); }
template <> __device__ __forceinline__ __nv_bfloat16 from_f64<__nv_bfloat16>(double x) { return __double2bfloat16(x); }

// One CTA per brick of the list; the brick's BRICKSIZE elements, in storage order.
template <typename S, typename D>
__global__ void __launch_bounds__(256)
convert_kernel(const S *__restrict__ src, unsigned long long sstep, D *__restrict__ dst, unsigned long long dstep,
               const unsigned *__restrict__ blist, unsigned nlist, int bsize, long long schunks, long long dchunks, int *err) {
  for (unsigned n = blockIdx.x; n < nlist; n += gridDim.x) {
    const unsigned b = blist[n];
    if ((long long)b >= schunks || (long long)b >= dchunks) {
      if (threadIdx.x == 0) atomicOr(err, FLAG_BOUNDS);
      continue;
    }
    const S *s = src + (size_t)b * sstep;
    D *d = dst + (size_t)b * dstep;
    for (int e = threadIdx.x; e < bsize; e += blockDim.x) d[e] = from_f64<D>(to_f64<S>(s[e]));
  }
}

// Partial norms per CTA: [max |a - r|, sum (a - r)^2, max |r|, sum r^2], in FP64.
template <typename A, typename Rt>
__global__ void __launch_bounds__(256)
norms_partial_kernel(const A *__restrict__ a, unsigned long long astep, const Rt *__restrict__ r, unsigned long long rstep,
                     const unsigned *__restrict__ blist, unsigned nlist, int bsize, long long achunks, long long rchunks,
                     double4 *partial, int *err) {
  double mx = 0.0, ss = 0.0, mr = 0.0, sr = 0.0;
  for (unsigned n = blockIdx.x; n < nlist; n += gridDim.x) {
    const unsigned b = blist[n];
    if ((long long)b >= achunks || (long long)b >= rchunks) {
      if (threadIdx.x == 0) atomicOr(err, FLAG_BOUNDS);
      continue;
    }
    const A *pa = a + (size_t)b * astep;
    const Rt *pr = r + (size_t)b * rstep;
    for (int e = threadIdx.x; e < bsize; e += blockDim.x) {
      const double x = to_f64<A>(pa[e]), y = to_f64<Rt>(pr[e]);
      const double d = x - y;
      mx = fmax(mx, fabs(d));
      ss = fma(d, d, ss);
      mr = fmax(mr, fabs(y));
      sr = fma(y, y, sr);
    }
  }
  __shared__ double4 red[256];
  red[threadIdx.x] = make_double4(mx, ss, mr, sr);
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      double4 p = red[threadIdx.x], q = red[threadIdx.x + w];
      red[threadIdx.x] = make_double4(fmax(p.x, q.x), p.y + q.y, fmax(p.z, q.z), p.w + q.w);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(256) norms_final_kernel(const double4 *partial, int nparts, double *out) {
  __shared__ double4 red[256];
  double4 acc = make_double4(0.0, 0.0, 0.0, 0.0);
  for (int p = threadIdx.x; p < nparts; p += blockDim.x) {
    const double4 q = partial[p];
    acc = make_double4(fmax(acc.x, q.x), acc.y + q.y, fmax(acc.z, q.z), acc.w + q.w);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      double4 p = red[threadIdx.x], q = red[threadIdx.x + w];
      red[threadIdx.x] = make_double4(fmax(p.x, q.x), p.y + q.y, fmax(p.z, q.z), p.w + q.w);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = red[0].x;
    out[1] = red[0].y;
    out[2] = red[0].z;
    out[3] = red[0].w;
  }
}

// Number of partial-norm blocks for a list of nlist bricks (at most NORM_BLOCKS).
constexpr int NORM_BLOCKS = 1024;
inline int norm_blocks(unsigned nlist) { return (int)(nlist < (unsigned)NORM_BLOCKS ? (nlist ? nlist : 1) : NORM_BLOCKS); }

template <typename A, typename Rt>
int launch_norms_typed(const bk_field *a, const bk_field *r, const unsigned *blist, unsigned nlist, int bsize,
                       double4 *partial, double *out_dev, int *err, cudaStream_t s) {
  const int blocks = norm_blocks(nlist);
  norms_partial_kernel<A, Rt><<<blocks, 256, 0, s>>>(
      reinterpret_cast<const A *>(a->dat) + a->offset, a->step, reinterpret_cast<const Rt *>(r->dat) + r->offset,
      r->step, blist, nlist, bsize, a->chunks, r->chunks, partial, err);
  norms_final_kernel<<<1, 256, 0, s>>>(partial, blocks, out_dev);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "norm kernels launch");
  return BK_OK;
}

// The partial-sum scratch (NORM_BLOCKS x 4 doubles) and the 4-double result live in
// scratch: pointers chosen by the caller of this function.
int launch_norms(const bk_field *a, const bk_field *r, const unsigned *blist, unsigned nlist, int bsize,
                 double4 *partial, double *out_dev, cudaStream_t s) {
  int *err = device_error_word();
  if (!err) return fail(BK_ERR_CUDA, "device error word unavailable");
#define BK_NORM_CASE(DA, TA, DR, TR) \
  if (a->dtype == DA && r->dtype == DR) return launch_norms_typed<TA, TR>(a, r, blist, nlist, bsize, partial, out_dev, err, s);
  BK_NORM_CASE(BK_F64, double, BK_F64, double)
  BK_NORM_CASE(BK_F32, float, BK_F64, double)
  BK_NORM_CASE(BK_BF16, __nv_bfloat16, BK_F64, double)
  BK_NORM_CASE(BK_F32, float, BK_F32, float)
  BK_NORM_CASE(BK_BF16, __nv_bfloat16, BK_BF16, __nv_bfloat16)
  BK_NORM_CASE(BK_F64, double, BK_F32, float)
  BK_NORM_CASE(BK_F64, double, BK_BF16, __nv_bfloat16)
  BK_NORM_CASE(BK_F32, float, BK_BF16, __nv_bfloat16)
  BK_NORM_CASE(BK_BF16, __nv_bfloat16, BK_F32, float)
#undef BK_NORM_CASE
  return fail(BK_ERR_ARG, "unknown dtype pair");
}

int check_pair(const bk_field *a, const bk_field *r, const bk_layout *lay, const unsigned *blist, unsigned nlist,
               Layout *L) {
  int s = check_layout(lay, L);
  if (s) return s;
  if ((s = check_field(a, *L, "first"))) return s;
  if ((s = check_field(r, *L, "second"))) return s;
  if (nlist && !blist) return fail(BK_ERR_ARG, "brick list is NULL");
  return BK_OK;
}

// Per-device scratch of the allocating norms entry point: grown on demand, kept until exit.
static std::mutex g_scratch_mu;
static std::vector<void *> g_scratch;

static void *norm_scratch() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if ((int)g_scratch.size() <= dev) g_scratch.resize(dev + 1, nullptr);
  if (!g_scratch[dev]) {
    void *p = nullptr;
    if (cudaMalloc(&p, sizeof(double4) * NORM_BLOCKS + sizeof(double) * 4) != cudaSuccess) return nullptr;
    g_scratch[dev] = p;
  }
  return g_scratch[dev];
}

// Seeded sum of `nw` sines with random integer wave numbers and phases on the periodic
// interior plus `noise` uniform noise, written to every brick of an init_grid layout
// (brick index = linear grid position).  Evaluated in FP32 (sinf), stored in the field's
// type: every storage type of one study starts from these values.
__device__ __forceinline__ unsigned long long sm64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
__device__ __forceinline__ double u01(unsigned long long seed, unsigned long long n) {
  return (double)(sm64(seed + n) >> 11) * (1.0 / 9007199254740992.0);
}

struct SinesArgs {
  void *dat;
  unsigned long long step, offset;
  int dtype;
  int gk, gj, gi;   // grid dims in bricks
  int gbk, gbj, gbi;  // ghost bricks per side
  int nk, nj, ni;   // interior elements per axis
  Layout L;
  int nw;
  float kv[64][3];
  float ph[64];
  unsigned long long nseed;
  double noise;
};

__global__ void __launch_bounds__(256) sines_kernel(const SinesArgs a) {
  const long long nb = (long long)a.gk * a.gj * a.gi;
  const int bsize = a.L.size();
  for (long long b = blockIdx.x; b < nb; b += gridDim.x) {
    const int bi = (int)(b % a.gi), bj = (int)((b / a.gi) % a.gj), bk = (int)(b / ((long long)a.gi * a.gj));
    for (int e = threadIdx.x; e < bsize; e += blockDim.x) {
      const int k = e / (a.L.bj * a.L.bi), j = (e / a.L.bi) % a.L.bj, i = e % a.L.bi;
      // position relative to the interior origin, wrapped into the periodic interior
      int z = (bk - a.gbk) * a.L.bk + k, y = (bj - a.gbj) * a.L.bj + j, x = (bi - a.gbi) * a.L.bi + i;
      z = ((z % a.nk) + a.nk) % a.nk;
      y = ((y % a.nj) + a.nj) % a.nj;
      x = ((x % a.ni) + a.ni) % a.ni;
      float v = 0.0f;
      for (int m = 0; m < a.nw; ++m) {
        const float arg = 6.28318530717958647692f * (a.kv[m][0] * z / a.nk + a.kv[m][1] * y / a.nj + a.kv[m][2] * x / a.ni) + a.ph[m];
        v += sinf(arg) / a.nw;
      }
      const unsigned long long idx = ((unsigned long long)z * a.nj + y) * a.ni + x;
      const double val = (double)v + a.noise * (2.0 * u01(a.nseed, idx) - 1.0);
      const size_t off = (size_t)b * a.step + a.offset + a.L.offset(k, j, i);
      switch (a.dtype) {
        case BK_F64: reinterpret_cast<double *>(a.dat)[off] = val; break;
        case BK_F32: reinterpret_cast<float *>(a.dat)[off] = (float)val; break;
        default: reinterpret_cast<__nv_bfloat16 *>(a.dat)[off] = __float2bfloat16_rn((float)val); break;
      }
    }
  }
}

}  // namespace bk

using namespace bk;

extern "C" {

int bk_convert(const bk_field *src, const bk_field *dst, const unsigned *blist, unsigned nlist, const bk_layout *lay,
               void *stream) {
  Layout L;
  int s = check_pair(src, dst, lay, blist, nlist, &L);
  if (s) return s;
  if (nlist == 0) return BK_OK;
  int *err = device_error_word();
  if (!err) return fail(BK_ERR_CUDA, "device error word unavailable");
  const unsigned grid = nlist < (1u << 30) ? nlist : (1u << 30);
  cudaStream_t st = as_stream(stream);
#define BK_CONV_CASE(DS, TS, DD, TD)                                                                        \
  if (src->dtype == DS && dst->dtype == DD) {                                                               \
    convert_kernel<TS, TD><<<grid, 256, 0, st>>>(reinterpret_cast<const TS *>(src->dat) + src->offset, src->step, \
                                                  reinterpret_cast<TD *>(dst->dat) + dst->offset, dst->step, blist,  \
                                                  nlist, L.size(), src->chunks, dst->chunks, err);          \
  } else
  BK_CONV_CASE(BK_F64, double, BK_F32, float)
  BK_CONV_CASE(BK_F64, double, BK_BF16, __nv_bfloat16)
  BK_CONV_CASE(BK_F32, float, BK_F64, double)
  BK_CONV_CASE(BK_BF16, __nv_bfloat16, BK_F64, double)
  BK_CONV_CASE(BK_F32, float, BK_BF16, __nv_bfloat16)
  BK_CONV_CASE(BK_BF16, __nv_bfloat16, BK_F32, float)
  BK_CONV_CASE(BK_F64, double, BK_F64, double)
  BK_CONV_CASE(BK_F32, float, BK_F32, float)
  BK_CONV_CASE(BK_BF16, __nv_bfloat16, BK_BF16, __nv_bfloat16)
  return fail(BK_ERR_ARG, "unknown dtype pair");
#undef BK_CONV_CASE
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "convert kernel launch");
  return BK_OK;
}

int bk_field_norms(const bk_field *a, const bk_field *ref, const unsigned *blist, unsigned nlist,
                   const bk_layout *lay, void *stream, double out[4]) {
  Layout L;
  int s = check_pair(a, ref, lay, blist, nlist, &L);
  if (s) return s;
  if (!out) return fail(BK_ERR_ARG, "out is NULL");
  for (int q = 0; q < 4; ++q) out[q] = 0.0;
  if (nlist == 0) return BK_OK;
  void *scratch = norm_scratch();
  if (!scratch) return fail(BK_ERR_NOMEM, "norm scratch allocation failed");
  double4 *partial = reinterpret_cast<double4 *>(scratch);
  double *res = reinterpret_cast<double *>(partial + NORM_BLOCKS);
  cudaStream_t st = as_stream(stream);
  if ((s = launch_norms(a, ref, blist, nlist, L.size(), partial, res, st))) return s;
  BK_CUDA(cudaMemcpyAsync(out, res, sizeof(double) * 4, cudaMemcpyDeviceToHost, st));
  BK_CUDA(cudaStreamSynchronize(st));
  return BK_OK;
}

int bk_fill_sines(const bk_field *f, const bk_layout *lay, const long grid_bricks[3], const long ghost_bricks[3],
                  int nwaves, uint64_t seed, double noise, void *stream) {
  Layout L;
  int s = check_layout(lay, &L);
  if (s) return s;
  if ((s = check_field(f, L, "sines"))) return s;
  if (!grid_bricks || !ghost_bricks || nwaves < 1 || nwaves > 64) return fail(BK_ERR_ARG, "bk_fill_sines: bad arguments");
  SinesArgs a{};
  a.dat = f->dat;
  a.step = f->step;
  a.offset = f->offset;
  a.dtype = f->dtype;
  a.gk = (int)grid_bricks[0]; a.gj = (int)grid_bricks[1]; a.gi = (int)grid_bricks[2];
  a.gbk = (int)ghost_bricks[0]; a.gbj = (int)ghost_bricks[1]; a.gbi = (int)ghost_bricks[2];
  a.nk = (a.gk - 2 * a.gbk) * L.bk; a.nj = (a.gj - 2 * a.gbj) * L.bj; a.ni = (a.gi - 2 * a.gbi) * L.bi;
  if (a.nk <= 0 || a.nj <= 0 || a.ni <= 0) return fail(BK_ERR_ARG, "bk_fill_sines: no interior");
  if ((long long)a.gk * a.gj * a.gi > f->chunks) return fail(BK_ERR_ARG, "bk_fill_sines: grid larger than the storage");
  a.L = L;
  a.nw = nwaves;
  // wave numbers in 1..4 and phases from the seed, as the oracle's orc_fill_sines
  for (int m = 0; m < nwaves; ++m) {
    for (int d = 0; d < 3; ++d) {
      unsigned long long x = seed + (unsigned long long)(4 * m + d);
      x += 0x9E3779B97F4A7C15ull;
      x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
      x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
      x ^= x >> 31;
      a.kv[m][d] = (float)(1 + (int)((double)(x >> 11) * (1.0 / 9007199254740992.0) * 4.0));
    }
    unsigned long long x = seed + (unsigned long long)(4 * m + 3);
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    a.ph[m] = (float)(6.283185307179586 * (double)(x >> 11) * (1.0 / 9007199254740992.0));
  }
  {
    unsigned long long x = seed ^ 0x5eedull;
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    a.nseed = x ^ (x >> 31);
  }
  a.noise = noise;
  const long long nb = (long long)a.gk * a.gj * a.gi;
  const unsigned grid = nb < (1ll << 30) ? (unsigned)nb : (1u << 30);
  sines_kernel<<<grid, 256, 0, as_stream(stream)>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "sines kernel launch");
  return BK_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Norms without allocation.
//
// Some callers cannot call cudaMalloc: a serving loop with a latency budget (cudaMalloc and
// cudaFree can synchronise the device and stall every stream) or a process whose device
// memory is all reserved up front by another allocator.  bk_field_norms_noalloc gives them
// the FP64 error norms with no allocation at all: its scratch -- one partial per listed
// brick, the 4-double result and an error word -- is the file-scope array below, which every
// GPU that loads this library holds until the process exits.  All calls share it and it
// keeps the last call's contents; calls whose work overlaps on the GPU (on different
// streams, or from several host threads) race on it.
namespace bk {

constexpr int NOALLOC_MAX_BRICKS = BK_NORMS_NOALLOC_MAX_BRICKS;
// [0, MAX): per-brick partials; [MAX]: result (x, y, z, w); [MAX + 1].x: error word
static __device__ __align__(256) double4 g_noalloc_scratch[NOALLOC_MAX_BRICKS + 2];

static std::mutex g_noalloc_mu;
static std::vector<double4 *> g_noalloc_addr;  // device address of the array, per device

// Device address of g_noalloc_scratch for the current device (looked up once per device,
// with that device current; the host-side name of the array is not a device address).
static int noalloc_scratch(double4 **p) {
  int dev = 0;
  BK_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if ((int)g_noalloc_addr.size() <= dev) g_noalloc_addr.resize(dev + 1, nullptr);
  if (!g_noalloc_addr[dev]) {
    void *addr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_addr[dev] = reinterpret_cast<double4 *>(addr);
  }
  *p = g_noalloc_addr[dev];
  return BK_OK;
}

// One partial-norm block per listed brick, then one final block over those partials.
template <typename A, typename Rt>
int launch_norms_per_brick(const bk_field *a, const bk_field *r, const unsigned *blist, unsigned nlist, int bsize,
                           double4 *partial, double *out_dev, int *err, cudaStream_t s) {
  norms_partial_kernel<A, Rt><<<nlist, 256, 0, s>>>(
      reinterpret_cast<const A *>(a->dat) + a->offset, a->step, reinterpret_cast<const Rt *>(r->dat) + r->offset,
      r->step, blist, nlist, bsize, a->chunks, r->chunks, partial, err);
  norms_final_kernel<<<1, 256, 0, s>>>(partial, (int)nlist, out_dev);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "no-alloc norm kernels launch");
  return BK_OK;
}

}  // namespace bk

extern "C" int bk_field_norms_noalloc(const bk_field *a, const bk_field *ref, const unsigned *blist, unsigned nlist,
                                      const bk_layout *lay, void *stream, double out[4]) {
  using namespace bk;
  Layout L;
  int s = check_pair(a, ref, lay, blist, nlist, &L);
  if (s) return s;
  if (!out) return fail(BK_ERR_ARG, "out is NULL");
  if (nlist > (unsigned)NOALLOC_MAX_BRICKS)
    return fail(BK_ERR_ARG, "bk_field_norms_noalloc: " + std::to_string(nlist) +
                                " bricks exceed its static scratch of " + std::to_string(NOALLOC_MAX_BRICKS) +
                                " bricks; split the list and combine (max of maxima, sum of sums)");
  for (int q = 0; q < 4; ++q) out[q] = 0.0;
  if (nlist == 0) return BK_OK;
  double4 *scratch = nullptr;
  if ((s = noalloc_scratch(&scratch))) return s;
  double4 *partial = scratch;
  double *res = reinterpret_cast<double *>(scratch + NOALLOC_MAX_BRICKS);
  int *err = reinterpret_cast<int *>(scratch + NOALLOC_MAX_BRICKS + 1);
  cudaStream_t st = as_stream(stream);
  BK_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));  // the word starts each call at zero
#define BK_NORM_CASE(DA, TA, DR, TR)                                                                  \
  if (a->dtype == DA && ref->dtype == DR) {                                                           \
    s = launch_norms_per_brick<TA, TR>(a, ref, blist, nlist, L.size(), partial, res, err, st);       \
  } else
  BK_NORM_CASE(BK_F64, double, BK_F64, double)
  BK_NORM_CASE(BK_F32, float, BK_F64, double)
  BK_NORM_CASE(BK_BF16, __nv_bfloat16, BK_F64, double)
  BK_NORM_CASE(BK_F32, float, BK_F32, float)
  BK_NORM_CASE(BK_BF16, __nv_bfloat16, BK_BF16, __nv_bfloat16)
  BK_NORM_CASE(BK_F64, double, BK_F32, float)
  BK_NORM_CASE(BK_F64, double, BK_BF16, __nv_bfloat16)
  BK_NORM_CASE(BK_F32, float, BK_BF16, __nv_bfloat16)
  BK_NORM_CASE(BK_BF16, __nv_bfloat16, BK_F32, float)
  return fail(BK_ERR_ARG, "unknown dtype pair");
#undef BK_NORM_CASE
  if (s) return s;
  int herr = 0;
  BK_CUDA(cudaMemcpyAsync(out, res, sizeof(double) * 4, cudaMemcpyDeviceToHost, st));
  BK_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  BK_CUDA(cudaStreamSynchronize(st));
  if (herr) return fail(BK_ERR_BOUNDS, "bk_field_norms_noalloc: a listed brick index was out of range and skipped");
  return BK_OK;
}
