// Four-dimensional bricks (weak/main-4d.cpp): Brick<Dim<4,4,4,4>, Dim<fold>> with a runtime
// tap list, e.g. the 9-point star of stencils/mpi9pt.py.  Persistent CTAs of 128 threads: the
// part of a brick's neighbourhood the stencil reads (centre and faces for a star, the whole
// radius-R box otherwise) is gathered into shared memory by asynchronous copies while the
// previous brick is computed, one output per thread.  The copies follow a table the CTA builds
// once from the layout: one entry per 16-byte block of a tile row, a single 16-byte copy where
// the block's elements are consecutive in their brick, else one copy per element.  Out-of-range
// list or adjacency entries are clamped / skipped and raise the device error flag, as in the
// 3-D kernels.
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
  int toff[BK_MAX_TAPS4];  // offsets in the E x E x E x EI tile (Tile4)
  double c[BK_MAX_TAPS4];
  float cf[BK_MAX_TAPS4];
  double mzero;  // -0.0: the addend that makes a product a multiply-add (FP64 register operands)
};

// Element copy global -> shared through the asynchronous copy path (4, 8 or 16 bytes).
template <int BYTES>
__device__ __forceinline__ void cp_async_elem(unsigned dst, const void *src) {
  if (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(dst), "l"(src), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_async_commit4() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait4() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Tile of one brick's neighbourhood: E = 4 + 2R along l, k, j; along i the halo is rounded up
// to whole 16-byte blocks (RP elements a side), EI = 4 + 2 RP, so that each block of a row lies
// in one brick and the centre blocks start 16-byte aligned.
template <typename T, int R>
struct Tile4 {
  static constexpr int ES = (int)sizeof(T), VE = 16 / ES, RP = (R + VE - 1) / VE * VE;
  static constexpr int E = 4 + 2 * R, EI = 4 + 2 * RP, ROWS = E * E * E, NBLK = EI / VE;
  static constexpr int NENT = ROWS * NBLK, TILE = ROWS * EI;
  static constexpr size_t SMEM = 2 * (size_t)TILE * ES + (size_t)NENT * 8;
};

// Persistent CTAs walk the brick list with a stride of the grid, pipelined: while brick j is
// computed from one tile buffer, brick j+1's neighbourhood is gathered into the other by
// asynchronous copies, and brick j+2's list and adjacency entries are staged (three
// adjacency slots, so no slot is rewritten while read).  Two block barriers per brick.
// star: every tap has at most one non-zero offset (only centre and face elements are read);
// vec: the input field's bricks start 16-byte aligned (16-byte copies allowed).
constexpr int NT4 = 128;  // threads per CTA, each computing two of a brick's 256 points

template <typename T, typename AT, int R>
__global__ void __launch_bounds__(NT4)
sweep4_kernel(const unsigned *__restrict__ adj, unsigned nbricks, const T *__restrict__ in, unsigned long long in_step,
              long long in_chunks, T *__restrict__ out, unsigned long long out_step, long long out_chunks,
              const unsigned *__restrict__ blist, unsigned nlist, const Layout4 L, const Taps4 tp, int star, int vec,
              int *err) {
  static_assert(sizeof(T) == sizeof(AT) && (sizeof(T) == 4 || sizeof(T) == 8), "the tile holds the storage type");
  typedef Tile4<T, R> G;
  constexpr int B = 4, E = G::E, EI = G::EI, VE = G::VE, RP = G::RP, NBLK = G::NBLK, NENT = G::NENT, TILE = G::TILE;
  static_assert(TILE < (1 << 14), "tile offsets take 14 bits");
  constexpr unsigned NONE = 0xFFFFFFFFu;
  // dynamic shared memory: tile[2][TILE], then the copy table (room for every (row, block);
  // filled with the blocks that have elements to copy, nent of them, in any order): per entry
  // a word slot (7 bits) | tile offset (14) << 7 | element mask (VE bits) << 21 | kind << 30
  // (1 one 16-byte copy, 2 one copy per element of the mask) and a word of the elements'
  // in-brick offsets (8 bits each)
  extern __shared__ __align__(16) unsigned char smem4[];
  T(*tile)[TILE] = reinterpret_cast<T(*)[TILE]>(smem4);
  unsigned *plan = reinterpret_cast<unsigned *>(smem4 + 2 * TILE * sizeof(T));
  unsigned *srcw = plan + NENT;
  __shared__ unsigned nbr[3][81];
  __shared__ unsigned nent;  // entries of the compacted table
  // FP64: the coefficients of a star of this radius and -0.0, read into per-thread registers
  // (on GB300 a DFMA with a constant-bank coefficient, and a DMUL, issue a fifth slower)
  constexpr int MT = 8 * R + 1;
  __shared__ double cs4[MT + 1];
  const int t = threadIdx.x;
  if (t == 0) nent = 0;
  if (t <= MT) cs4[t] = t == MT ? tp.mzero : t < tp.n ? tp.c[t] : 0.0;
  __syncthreads();
  for (int e = t; e < NENT; e += blockDim.x) {
    const int row = e / NBLK, blk = e - row * NBLK;
    const int l = row / (E * E) - R, k = (row / E) % E - R, j = row % E - R;  // in-brick, may lie outside
    const int ql = l < 0 ? -1 : (l >= B ? 1 : 0), qk = k < 0 ? -1 : (k >= B ? 1 : 0);
    const int qj = j < 0 ? -1 : (j >= B ? 1 : 0);
    const int i0 = blk * VE - RP;  // the block's first i
    const int qi = i0 < 0 ? -1 : (i0 >= B ? 1 : 0);
    const int outside = (ql != 0) + (qk != 0) + (qj != 0) + (qi != 0);
    unsigned mask = 0, sw = 0;
    bool consecutive = true;
    int s0 = -1;
    for (int q = 0; q < VE; ++q) {
      const int i = i0 + q;
      if (i < -R || i >= B + R || (star && outside > 1)) continue;
      const int so = L.offset(l - ql * B, k - qk * B, j - qj * B, i - qi * B);
      if (q == 0) s0 = so;
      if (so != s0 + q) consecutive = false;
      mask |= 1u << q;
      sw |= (unsigned)so << (8 * q);
    }
    unsigned w = 0;
    if (mask) {
      const unsigned slot = (unsigned)(((ql + 1) * 3 + (qk + 1)) * 9 + (qj + 1) * 3 + (qi + 1));
      const bool v16 = vec && consecutive && mask == (1u << VE) - 1u && s0 % VE == 0;
      w = slot | ((unsigned)(row * EI + blk * VE) << 7) | (mask << 21) | ((v16 ? 1u : 2u) << 30);
      // only blocks with elements to copy enter the table (a star reads its centre and faces:
      // 288 of 648 entries for FP32 radius 1), in any order
      const unsigned at = atomicAdd(&nent, 1u);
      plan[at] = w;
      srcw[at] = sw;
    }
  }
  const unsigned long long gs = gridDim.x;
  // Staging of list entry n's adjacency row (thread t < 81 holds slot t): the list entry is
  // loaded two iterations and the adjacency row one iteration before the row is staged, so no
  // iteration waits for a load it issued.  check() gives the staged value: slot 40 carries
  // NONE for a brick that is not computed (past the list, or out of range: flagged).
  auto load_b = [&](unsigned long long n) -> unsigned { return (t < 81 && n < nlist) ? blist[n] : NONE; };
  auto load_v = [&](unsigned b) -> unsigned { return (t < 81 && b < nbricks) ? adj[(size_t)b * 81 + t] : 0u; };
  auto check = [&](unsigned long long n, unsigned b, unsigned v) -> unsigned {
    if (n >= nlist) return t == 40 ? NONE : 0u;
    if (b >= nbricks) {
      if (t == 40) {
        atomicOr(err, FLAG_BOUNDS);
        return NONE;
      }
      return 0u;
    }
    if ((long long)v >= in_chunks || (t == 40 && (long long)v >= out_chunks)) {
      atomicOr(err, FLAG_BOUNDS);
      return t == 40 ? NONE : 0u;
    }
    return v;
  };
  auto issue = [&](int slot, int buf) {
    const unsigned *nb = nbr[slot];
    if (nb[40] != NONE) {
      const unsigned base = (unsigned)__cvta_generic_to_shared(&tile[buf][0]);
      // entries t, t + NT4, ... of the table (a compile-time count per thread)
      constexpr int NPT = (NENT + NT4 - 1) / NT4;
      const int ne = (int)nent;
#pragma unroll
      for (int m = 0; m < NPT; ++m) {
        const int e = t + NT4 * m;
        if (e >= ne) break;
        const unsigned w = plan[e];
        const T *src = in + (size_t)nb[w & 127u] * in_step;
        const unsigned dst = base + ((w >> 7) & 0x3FFFu) * (unsigned)sizeof(T);
        const unsigned sw = srcw[e];
        if ((w >> 30) == 1u) {
          cp_async_elem<16>(dst, src + (sw & 255u));
        } else {
#pragma unroll
          for (int q = 0; q < VE; ++q)
            if ((w >> (21 + q)) & 1u) cp_async_elem<sizeof(T)>(dst + q * (unsigned)sizeof(T), src + ((sw >> (8 * q)) & 255u));
        }
      }
    }
    cp_async_commit4();
  };
  const unsigned long long n0 = blockIdx.x;
  {
    const unsigned b0 = load_b(n0), b1 = load_b(n0 + gs);
    const unsigned a0 = check(n0, b0, load_v(b0)), a1 = check(n0 + gs, b1, load_v(b1));
    if (t < 81) {
      nbr[0][t] = a0;
      nbr[1][t] = a1;
    }
  }
  unsigned ba = load_b(n0 + 2 * gs);  // list entry n + 2 gs and its adjacency row
  unsigned va = load_v(ba);
  unsigned bb = load_b(n0 + 3 * gs);  // list entry n + 3 gs
  __syncthreads();  // tables and the first two adjacency slots
  issue(0, 0);
  // this thread's output elements t and t + NT4: their tile positions and in-brick offsets (the
  // layout's divisions by the fold, once per kernel instead of once per brick)
  static_assert(2 * NT4 == B * B * B * B, "two points per thread");
  int ctile[2], oofs[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int pt = t + NT4 * h;
    const int oi = pt % B, oj = (pt / B) % B, ok = (pt / (B * B)) % B, ol = pt / (B * B * B);
    ctile[h] = (((ol + R) * E + (ok + R)) * E + (oj + R)) * EI + (oi + RP);
    oofs[h] = L.offset(ol, ok, oj, oi);
  }
  // the tap list of a star of this radius fits MT entries: offsets held in registers for the
  // whole kernel (the loop over a runtime count read them from the parameters per tap)
  int toffr[MT];
#pragma unroll
  for (int q = 0; q < MT; ++q) toffr[q] = q < tp.n ? tp.toff[q] : 0;
  constexpr bool F64 = sizeof(AT) == 8;
  AT cr[MT];
#pragma unroll
  for (int q = 0; q < MT; ++q) cr[q] = F64 ? (AT)cs4[q] : (AT)0;
  const AT mz = F64 ? (AT)cs4[MT] : (AT)0;
  auto coefq = [&](int q) -> AT {
    if constexpr (sizeof(AT) == 8) return tp.c[q];
    else return tp.cf[q];
  };
  // the product of the first tap: FP64 as a multiply-add onto -0 (the same bits)
  auto first = [&](AT k, AT x) -> AT {
    if constexpr (F64) return fma(k, x, mz);
    else return k * x;
  };
  int jb = 0;
  for (unsigned long long n = n0; n < nlist; n += gs, ++jb) {
    const int cur = jb % 3, nxt = (jb + 1) % 3, far = (jb + 2) % 3, buf = jb & 1;
    __syncthreads();  // the previous brick's compute is done with tile[buf ^ 1] and slot far
    issue(nxt, buf ^ 1);
    const unsigned staged = check(n + 2 * gs, ba, va);
    if (t < 81) nbr[far][t] = staged;
    ba = bb;
    va = load_v(bb);
    bb = load_b(n + 4 * gs);
    cp_async_wait4<1>();  // this thread's copies for brick n have landed
    __syncthreads();      // ... and everybody else's
    const unsigned ob = nbr[cur][40];
    if (ob != NONE) {
      const T *c0 = tile[buf] + ctile[0], *c1 = tile[buf] + ctile[1];
      AT v0, v1;
      if (tp.n <= MT) {
        // up to MT taps (a radius-R star): unrolled, the offsets and coefficients from
        // registers, the taps past n predicated off; the thread's two points side by side
        const AT k0 = F64 ? cr[0] : coefq(0);
        v0 = first(k0, c0[toffr[0]]);
        v1 = first(k0, c1[toffr[0]]);
#pragma unroll
        for (int q = 1; q < MT; ++q)
          if (q < tp.n) {
            const AT kq = F64 ? cr[q] : coefq(q);
            v0 = fma(kq, c0[toffr[q]], v0);
            v1 = fma(kq, c1[toffr[q]], v1);
          }
      } else {
        v0 = coefq(0) * c0[tp.toff[0]];
        v1 = coefq(0) * c1[tp.toff[0]];
        for (int q = 1; q < tp.n; ++q) {
          v0 = fma(coefq(q), c0[tp.toff[q]], v0);
          v1 = fma(coefq(q), c1[tp.toff[q]], v1);
        }
      }
      T *ob0 = out + (size_t)ob * out_step;
      Elem<T>::store(ob0 + oofs[0], v0);
      Elem<T>::store(ob0 + oofs[1], v1);
    }
  }
  cp_async_wait4<0>();  // no copy may outlive the kernel
}

template <typename T, typename AT, int R>
static int launch4(const unsigned *adj, unsigned nbricks, const bk_field *in, const bk_field *out, const unsigned *blist,
                   unsigned nlist, const Layout4 &L, Taps4 tp, const int (*offs)[4], int star, cudaStream_t s) {
  // persistent CTAs (each builds its copy table once): as many as fit on the GPU
  typedef Tile4<T, R> G;
  auto kern = sweep4_kernel<T, AT, R>;
  constexpr size_t smem = G::SMEM;
  for (int t = 0; t < tp.n; ++t)
    tp.toff[t] = ((offs[t][0] * G::E + offs[t][1]) * G::E + offs[t][2]) * G::EI + offs[t][3];
  const char *ibase = reinterpret_cast<const char *>(in->dat) + in->offset * sizeof(T);
  const int vec = reinterpret_cast<uintptr_t>(ibase) % 16 == 0 && (in->step * sizeof(T)) % 16 == 0;
  int *err = device_error_word();
  if (!err) return fail(BK_ERR_CUDA, "device error word unavailable");
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e0 = cudaGetDevice(&dev);
  if (e0 == cudaSuccess) e0 = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e0 == cudaSuccess && smem > 48 * 1024) e0 = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e0 == cudaSuccess) e0 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT4, smem);
  if (e0 != cudaSuccess) return cuda_fail(e0, "sweep4 launch setup");
  long long grid = (long long)sms * (per_sm > 0 ? per_sm : 1);
  if (grid > nlist) grid = nlist;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, NT4, smem, s>>>(
      adj, nbricks, reinterpret_cast<const T *>(in->dat) + in->offset, in->step, in->chunks,
      reinterpret_cast<T *>(out->dat) + out->offset, out->step, out->chunks, blist, nlist, L, tp, star, vec, err);
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
  {
    const int s_ = check_disjoint(in, out, 256);
    if (s_) return s_;
  }
  if (st->npoints < 1 || st->npoints > BK_MAX_TAPS4) return fail(BK_ERR_ARG, "4-D stencil npoints out of range");
  int r = 0;
  for (int t = 0; t < st->npoints; ++t)
    for (int d = 0; d < 4; ++d) r = abs(st->offsets[t][d]) > r ? abs(st->offsets[t][d]) : r;
  if (r > 2) return fail(BK_ERR_UNSUPPORTED, "4-D stencils of radius up to 2");
  if (nlist == 0) return BK_OK;
  if (!adj || !blist || nbricks == 0) return fail(BK_ERR_ARG, "adjacency, brick list and nbricks are required");
  const int R = r <= 1 ? 1 : 2;
  Taps4 tp;
  tp.n = st->npoints;
  tp.mzero = -0.0;
  int star = 1;
  for (int t = 0; t < tp.n; ++t) {
    const int *o = st->offsets[t];
    star = star && ((o[0] != 0) + (o[1] != 0) + (o[2] != 0) + (o[3] != 0) <= 1);
    tp.c[t] = st->coeff[t];
    tp.cf[t] = (float)st->coeff[t];
  }
  cudaStream_t s = as_stream(stream);
  if (in->dtype == BK_F64)
    return R == 1 ? launch4<double, double, 1>(adj, nbricks, in, out, blist, nlist, L, tp, st->offsets, star, s)
                  : launch4<double, double, 2>(adj, nbricks, in, out, blist, nlist, L, tp, st->offsets, star, s);
  return R == 1 ? launch4<float, float, 1>(adj, nbricks, in, out, blist, nlist, L, tp, st->offsets, star, s)
                : launch4<float, float, 2>(adj, nbricks, in, out, blist, nlist, L, tp, st->offsets, star, s);
}

}  // extern "C"
