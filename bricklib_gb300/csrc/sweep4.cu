// Four-dimensional bricks (weak/main-4d.cpp): Brick<Dim<4,4,4,4>, Dim<fold>> with a runtime
// tap list, e.g. the 9-point star of stencils/mpi9pt.py.  Persistent CTAs of 256 threads: a
// brick's (4+2R)^4 neighbourhood is gathered into shared memory by asynchronous copies (the
// source slot and in-brick offset of every tile element from a table the CTA builds once)
// while the previous brick is computed, one element per thread.  Out-of-range list or adjacency entries are clamped / skipped and
// raise the device error flag, as in the 3-D kernels.
#include "bk_common.cuh"

namespace bk {

struct Layout4 {
  int b[4], f[4];  // (l, k, j, i), outermost first
  __host__ __device__ __forceinline__ int size() const { return b[0] * b[1] * b[2] * b[3]; }
  // in-brick offset: folds right-aligned, vector index over the fold blocks, lane inside
  __host__ __device__ __forceinline__ int offset(int l, int k, int j, int i) const {
    const int vl = f[0] * f[1] * f[2] * f[3];
    const int vec = (((l / f[0]) * (b[1] / f[1]) + k / f[1]) * (b[2] / f[2]) + j / f[2]) * (b[3] / f[3]) + i / f[3];
    const int lane = (((l % f[0]) * f[1] + k % f[1]) * f[2] + j % f[2]) * f[3] + i % f[3];
    return vec * vl + lane;
  }
};

struct Taps4 {
  int n;
  int toff[BK_MAX_TAPS4];  // offsets in the (4+2R)^4 tile
  double c[BK_MAX_TAPS4];
  float cf[BK_MAX_TAPS4];
};

// Element copy global -> shared through the asynchronous copy path (4 or 8 bytes).
template <int BYTES>
__device__ __forceinline__ void cp_async_elem(unsigned dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(dst), "l"(src), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_async_commit4() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait4() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Persistent CTAs walk the brick list with a stride of the grid, pipelined: while brick j is
// computed from one tile buffer, brick j+1's neighbourhood is gathered into the other by
// asynchronous copies, and brick j+2's list and adjacency entries are staged (three
// adjacency slots, so no slot is rewritten while read).  Two block barriers per brick.
template <typename T, typename AT, int R>
__global__ void __launch_bounds__(256)
sweep4_kernel(const unsigned *__restrict__ adj, unsigned nbricks, const T *__restrict__ in, unsigned long long in_step,
              long long in_chunks, T *__restrict__ out, unsigned long long out_step, long long out_chunks,
              const unsigned *__restrict__ blist, unsigned nlist, const Layout4 L, const Taps4 tp, int *err) {
  static_assert(sizeof(T) == sizeof(AT) && (sizeof(T) == 4 || sizeof(T) == 8), "the tile holds the storage type");
  constexpr int B = 4, E = B + 2 * R, TILE = E * E * E * E;
  constexpr unsigned NONE = 0xFFFFFFFFu;
  // dynamic shared memory: tile[2][TILE], then where every tile element comes from (offset in
  // its brick, adjacency slot): fixed by the layout, so computed once per CTA
  extern __shared__ __align__(16) unsigned char smem4[];
  T(*tile)[TILE] = reinterpret_cast<T(*)[TILE]>(smem4);
  unsigned short *toffs = reinterpret_cast<unsigned short *>(smem4 + 2 * TILE * sizeof(T));
  unsigned char *tslot = reinterpret_cast<unsigned char *>(toffs + TILE);
  __shared__ unsigned nbr[3][81];
  const int t = threadIdx.x;
  for (int e = t; e < TILE; e += blockDim.x) {
    int r = e;
    const int ii = r % E; r /= E;
    const int jj = r % E; r /= E;
    const int kk = r % E;
    const int ll = r / E;
    const int ql = ll < R ? -1 : (ll >= R + B ? 1 : 0), qk = kk < R ? -1 : (kk >= R + B ? 1 : 0);
    const int qj = jj < R ? -1 : (jj >= R + B ? 1 : 0), qi = ii < R ? -1 : (ii >= R + B ? 1 : 0);
    tslot[e] = (unsigned char)(((ql + 1) * 3 + (qk + 1)) * 9 + (qj + 1) * 3 + (qi + 1));
    toffs[e] = (unsigned short)L.offset(ll - R - ql * B, kk - R - qk * B, jj - R - qj * B, ii - R - qi * B);
  }
  const unsigned long long gs = gridDim.x;
  // this thread's adjacency entry (slot t < 81) of list entry n; slot 40 carries NONE for a
  // brick that is not computed (past the list, or out of range: flagged)
  auto fetch = [&](unsigned long long n) -> unsigned {
    if (t >= 81) return 0u;
    if (n >= nlist) return t == 40 ? NONE : 0u;
    const unsigned b = blist[n];
    if (b >= nbricks) {
      if (t == 40) {
        atomicOr(err, FLAG_BOUNDS);
        return NONE;
      }
      return 0u;
    }
    unsigned v = adj[(size_t)b * 81 + t];
    if ((long long)v >= in_chunks || (t == 40 && (long long)v >= out_chunks)) {
      atomicOr(err, FLAG_BOUNDS);
      v = t == 40 ? NONE : 0u;
    }
    return v;
  };
  auto issue = [&](int slot, int buf) {
    const unsigned *nb = nbr[slot];
    if (nb[40] != NONE) {
      const unsigned base = (unsigned)__cvta_generic_to_shared(&tile[buf][0]);
      for (int e = t; e < TILE; e += blockDim.x)
        cp_async_elem<sizeof(T)>(base + e * (unsigned)sizeof(T), in + (size_t)nb[tslot[e]] * in_step + toffs[e]);
    }
    cp_async_commit4();
  };
  const unsigned long long n0 = blockIdx.x;
  {
    const unsigned a0 = fetch(n0), a1 = fetch(n0 + gs);
    if (t < 81) {
      nbr[0][t] = a0;
      nbr[1][t] = a1;
    }
  }
  unsigned ahead = fetch(n0 + 2 * gs);
  __syncthreads();  // tables and the first two adjacency slots
  issue(0, 0);
  int j = 0;
  for (unsigned long long n = n0; n < nlist; n += gs, ++j) {
    const int cur = j % 3, nxt = (j + 1) % 3, far = (j + 2) % 3, buf = j & 1;
    __syncthreads();  // the previous brick's compute is done with tile[buf ^ 1] and slot far
    issue(nxt, buf ^ 1);
    if (t < 81) nbr[far][t] = ahead;
    ahead = fetch(n + 3 * gs);
    cp_async_wait4<1>();  // this thread's copies for brick n have landed
    __syncthreads();      // ... and everybody else's
    const unsigned ob = nbr[cur][40];
    if (ob != NONE && t < B * B * B * B) {
      const int i = t % B, jj = (t / B) % B, k = (t / (B * B)) % B, l = t / (B * B * B);
      const T *c = tile[buf] + (((l + R) * E + (k + R)) * E + (jj + R)) * E + (i + R);
      AT v;
      if constexpr (sizeof(AT) == 8) {
        v = tp.c[0] * c[tp.toff[0]];
        for (int q = 1; q < tp.n; ++q) v = fma(tp.c[q], c[tp.toff[q]], v);
      } else {
        v = tp.cf[0] * c[tp.toff[0]];
        for (int q = 1; q < tp.n; ++q) v = fmaf(tp.cf[q], c[tp.toff[q]], v);
      }
      Elem<T>::store(out + (size_t)ob * out_step + L.offset(l, k, jj, i), v);
    }
  }
  cp_async_wait4<0>();  // no copy may outlive the kernel
}

template <typename T, typename AT, int R>
static int launch4(const unsigned *adj, unsigned nbricks, const bk_field *in, const bk_field *out, const unsigned *blist,
                   unsigned nlist, const Layout4 &L, const Taps4 &tp, int *err, cudaStream_t s) {
  // persistent CTAs (each builds its tile table once): as many as fit on the GPU
  auto kern = sweep4_kernel<T, AT, R>;
  constexpr int E = 4 + 2 * R, TILE = E * E * E * E;
  constexpr size_t smem = 2 * TILE * sizeof(T) + TILE * 3;
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e0 = cudaGetDevice(&dev);
  if (e0 == cudaSuccess) e0 = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e0 == cudaSuccess && smem > 48 * 1024) e0 = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e0 == cudaSuccess) e0 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem);
  if (e0 != cudaSuccess) return cuda_fail(e0, "sweep4 launch setup");
  long long grid = (long long)sms * (per_sm > 0 ? per_sm : 1);
  if (grid > nlist) grid = nlist;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, 256, smem, s>>>(
      adj, nbricks, reinterpret_cast<const T *>(in->dat) + in->offset, in->step, in->chunks,
      reinterpret_cast<T *>(out->dat) + out->offset, out->step, out->chunks, blist, nlist, L, tp, err);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "sweep4 launch");
  return BK_OK;
}

}  // namespace bk

using namespace bk;

extern "C" {

int bk_sweep4(const unsigned *adj, unsigned nbricks, const bk_field *in, const bk_field *out, const unsigned *blist,
              unsigned nlist, const bk_stencil4 *st, const bk_layout4 *lay, void *stream) {
  if (!st || !lay || !in || !out) return fail(BK_ERR_ARG, "stencil, layout and fields are required");
  Layout4 L;
  for (int d = 0; d < 4; ++d) {
    L.b[d] = lay->bdim[d];
    L.f[d] = lay->fold[d];
    if (L.b[d] != 4) return fail(BK_ERR_UNSUPPORTED, "4-D sweeps take 4x4x4x4 bricks (weak/main-4d.cpp)");
    if (L.f[d] <= 0 || L.b[d] % L.f[d]) return fail(BK_ERR_ARG, "fold must divide the brick dims");
  }
  if (!in->dat || !out->dat || in->chunks <= 0 || out->chunks <= 0) return fail(BK_ERR_ARG, "fields need storage");
  if (in->offset + 256 > in->step || out->offset + 256 > out->step)
    return fail(BK_ERR_ARG, "field: offset + brick size exceeds step");
  if (in->dtype != out->dtype || (in->dtype != BK_F64 && in->dtype != BK_F32))
    return fail(BK_ERR_UNSUPPORTED, "4-D sweeps: FP64 or FP32 storage, the same for in and out");
  if (in->dat == out->dat && in->step == out->step) {
    const size_t lo = in->offset < out->offset ? in->offset : out->offset;
    const size_t hi = in->offset < out->offset ? out->offset : in->offset;
    if (hi - lo < 256) return fail(BK_ERR_ARG, "in and out fields overlap");
  }
  if (st->npoints < 1 || st->npoints > BK_MAX_TAPS4) return fail(BK_ERR_ARG, "4-D stencil npoints out of range");
  int r = 0;
  for (int t = 0; t < st->npoints; ++t)
    for (int d = 0; d < 4; ++d) r = abs(st->offsets[t][d]) > r ? abs(st->offsets[t][d]) : r;
  if (r > 2) return fail(BK_ERR_UNSUPPORTED, "4-D stencils of radius up to 2");
  if (nlist == 0) return BK_OK;
  if (!adj || !blist || nbricks == 0) return fail(BK_ERR_ARG, "adjacency, brick list and nbricks are required");
  const int R = r <= 1 ? 1 : 2, E = 4 + 2 * R;
  Taps4 tp;
  tp.n = st->npoints;
  for (int t = 0; t < tp.n; ++t) {
    const int *o = st->offsets[t];
    tp.toff[t] = ((o[0] * E + o[1]) * E + o[2]) * E + o[3];
    tp.c[t] = st->coeff[t];
    tp.cf[t] = (float)st->coeff[t];
  }
  int *err = device_error_word();
  if (!err) return fail(BK_ERR_CUDA, "device error word unavailable");
  cudaStream_t s = as_stream(stream);
  if (in->dtype == BK_F64)
    return R == 1 ? launch4<double, double, 1>(adj, nbricks, in, out, blist, nlist, L, tp, err, s)
                  : launch4<double, double, 2>(adj, nbricks, in, out, blist, nlist, L, tp, err, s);
  return R == 1 ? launch4<float, float, 1>(adj, nbricks, in, out, blist, nlist, L, tp, err, s)
                : launch4<float, float, 2>(adj, nbricks, in, out, blist, nlist, L, tp, err, s);
}

}  // extern "C"
