// The brick stencil sweep kernel (templated; instantiated per element type in
// sweep_f64.cu / sweep_f32.cu / sweep_bf16.cu).
//
// One CTA computes NB bricks at a time (NB = threads / (BJ*BI)).  For each brick it
//   1. reads the brick's 27 adjacency entries (BrickInfo::adj, brick.h:96-111) into
//      shared memory, clamping out-of-range indices to brick 0 and raising a flag;
//   2. gathers the extended tile (BK+2R) x (BJ+2R) x (BI+2R) from the centre brick
//      and its neighbours into shared memory in row-major order, converting from the
//      storage type to the accumulation type once per element (star stencils skip
//      the edge and corner regions they never read);
//   3. lets each thread compute one (j, i) column of BK outputs from shared memory
//      and store it, coalesced, into the output field of brick adj[b][13].
// The tap structure is compile-time for the star / cube families and a runtime list
// (offsets into the tile, coefficients in the parameter constant bank) for the
// generic family.
#pragma once

#include "bk_common.cuh"

namespace bk {

// FAM_CUBESYM: a cube whose coefficients are mirror-symmetric in each axis,
// c(dk, dj, di) = c(|dk|, |dj|, |di|); computed from pair sums (see sweep2_kernel.cuh)
// FAM_CUBESYM_IJ: in addition c(dk, dj, di) == c(dk, di, dj) (i <-> j swap symmetry)
enum Family { FAM_GENERIC = 0, FAM_STAR = 1, FAM_CUBE = 2, FAM_CUBESYM = 3, FAM_CUBESYM_IJ = 4 };
// Taps index of the mirror-symmetric coefficient of (|dk|, |dj|, |di|), radius r: the
// symmetric table lives after the full cube table (at most 125 entries)
__host__ __device__ constexpr int sym_index(int ak, int aj, int ai, int r) {
  return 200 + (ak * (r + 1) + aj) * (r + 1) + ai;
}
enum AccMode { ACCM_NATIVE = 0, ACCM_COMP = 1, ACCM_FF = 2 };

// One domain of a batch (device table entry).
struct BatchDomain {
  const unsigned *adj;
  unsigned nbricks;
  unsigned stencil;
  unsigned char *f0, *f1;  // field bases (dat + offset), bytes
  unsigned long long step_bytes;
  long long chunks;
};

struct SweepArgs {
  const unsigned *adj;
  unsigned nbricks;
  const void *in;
  unsigned long long in_step, in_off;
  long long in_chunks;
  void *out;
  unsigned long long out_step, out_off;
  long long out_chunks;
  const unsigned *blist;
  unsigned nlist;
  int *err;
  Layout L;
  // batch mode: work items (domain, brick) instead of blist, per-domain fields by parity
  const BatchDomain *doms;
  const uint2 *work;
  unsigned ndom;
  int parity;
  // bounded waits of the TMA-fed kernels give up after wait_ns (0: one second)
  unsigned long long wait_ns;
  // test hook (BK_TEST_WITHHOLD_COPY): the TMA star kernel's first CTA posts its first
  // stage's byte count but never issues one of that stage's copies, so that stage's wait runs
  // out; nothing is left in flight.  Zero in normal use.
  int withhold;
};

// Taps with a packed-FP32 coefficient pair (every star up to radius 5).
constexpr int TAP_PAIRS = 32;

// Coefficients in kernel order; passed by value (kernel parameter constant bank).
struct Taps {
  int n;
  int pre, post;  // BK_OP_* applied to every input value / to the sum
  int toff[BK_MAX_TAPS];  // generic family: tap offset in tile elements from the centre
  float cf[BK_MAX_TAPS];   // coefficient rounded to float (the high part)
  float cl[BK_MAX_TAPS];   // float(c - cf): the low part, for float-float arithmetic
  double c[BK_MAX_TAPS];
  float2 cp[TAP_PAIRS];    // (cf, cf) of the first taps: operands of packed FP32 arithmetic
  int kj;                  // mirror-symmetric cube also symmetric under the k <-> j swap
  // mirror-symmetric cubes: (cf, cf) of class (|dk|, |dj|, |di|) at ((|dk| (R+1) + |dj|) (R+1) + |di|)
  float2 sp[27];
  // {1.0, -0.0}, which the native FP64 kernels hold in registers (F64Ops); set by the host so
  // that the compiler cannot fold them back into plain additions and products
  double one_mz[2];
};

__host__ __device__ constexpr int sweep_threads(int tpb) { return tpb < 128 ? 128 : tpb; }

template <typename AT> __device__ __forceinline__ AT coef(const Taps &tp, int t);
template <> __device__ __forceinline__ double coef<double>(const Taps &tp, int t) { return tp.c[t]; }
template <> __device__ __forceinline__ float coef<float>(const Taps &tp, int t) { return tp.cf[t]; }

// Neumaier compensated accumulation of one partial into (s, comp).
__device__ __forceinline__ double absval(double x) { return fabs(x); }
__device__ __forceinline__ float absval(float x) { return fabsf(x); }

template <typename AT>
__device__ __forceinline__ void neumaier(AT &s, AT &comp, AT p) {
  const AT t = s + p;
  comp += (absval(s) >= absval(p)) ? ((s - t) + p) : ((p - t) + s);
  s = t;
}

// Pointwise operations of non-linear stencils (BK_OP_RELU = max(x, 0), BK_OP_ABS = |x|).
// The FP64 versions work on the sign bit, so they do not occupy the FP64 pipe.
__device__ __forceinline__ float op_apply(float x, int op) {
  return op == BK_OP_RELU ? fmaxf(x, 0.0f) : (op == BK_OP_ABS ? fabsf(x) : x);
}
__device__ __forceinline__ double op_apply(double x, int op) {
  const long long b = __double_as_longlong(x);
  if (op == BK_OP_RELU) return b < 0 ? 0.0 : x;
  if (op == BK_OP_ABS) return __longlong_as_double(b & 0x7FFFFFFFFFFFFFFFll);
  return x;
}
__device__ __forceinline__ float2 op_apply(float2 x, int op) {  // hi carries the sign of hi + lo
  if (op == BK_OP_RELU) return x.x < 0.0f ? make_float2(0.0f, 0.0f) : x;
  if (op == BK_OP_ABS) return x.x < 0.0f ? make_float2(-x.x, -x.y) : x;
  return x;
}

// ---------------------------------------------------------------- float-float (FP64 storage)
//
// A double x is held as hi + lo, two floats obtained from its bit pattern with integer
// operations only (the FP64 pipe of GB300 runs at 1/64 of the FP32 rate, and so do the
// double<->float conversions): hi carries the sign, exponent and top 23 stored mantissa
// bits (truncated), lo the next 23 bits, i.e. 47 significant bits, relative error
// below 2^-47.  |x| must be below 2^128; |x| below 2^-126 reads as 0.
__device__ __forceinline__ float2 split_f64(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned h32 = (unsigned)(b >> 32), l32 = (unsigned)b;
  const unsigned sign = h32 & 0x80000000u;
  const int e = (int)((h32 >> 20) & 0x7FFu) - 1023;
  const unsigned m23 = ((h32 & 0xFFFFFu) << 3) | (l32 >> 29);
  float hi, lo;
  if (e >= -126 && e <= 127) {
    hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | m23);
    // next 23 mantissa bits; bit 0 weighs 2^(e-46).  (2^23 + r) * 2^(e-46) - 2^23 * 2^(e-46)
    // is r * 2^(e-46), exact
    const unsigned r = (l32 & 0x1FFFFFFFu) >> 6;
    const int el = e + 104;
    lo = el >= 1 ? __uint_as_float(((unsigned)el << 23) | r) - __uint_as_float((unsigned)el << 23) : 0.0f;
    lo = __uint_as_float(__float_as_uint(lo) | sign);
  } else if (e > 127) {
    hi = __uint_as_float(sign | 0x7F800000u);
    lo = 0.0f;
  } else {
    hi = __uint_as_float(sign);
    lo = 0.0f;
  }
  return make_float2(hi, lo);
}

// Knuth's TwoSum: s + err == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &err) {
  s = a + b;
  const float bp = s - a;
  err = (a - (s - bp)) + (b - bp);
}

// The double nearest (within 2^-52 relative) to the float-float value h + l, |l| <= ulp(h)/2,
// built from the two bit patterns with integer operations.
__device__ __forceinline__ double ff_to_f64(float h, float l) {
  const unsigned bh = __float_as_uint(h);
  const unsigned eh = (bh >> 23) & 0xFFu;
  if (eh == 0) return 0.0;
  if (eh == 0xFFu) return __longlong_as_double((long long)(((unsigned long long)(bh & 0x80000000u) << 32) | 0x7FF0000000000000ull));
  long long M = (long long)((1ull << 52) | ((unsigned long long)(bh & 0x7FFFFFu) << 29));
  int E = (int)eh - 127 + 1023;
  const unsigned bl = __float_as_uint(l);
  const unsigned el = (bl >> 23) & 0xFFu;
  if (el != 0) {
    const long long ml = (long long)((1u << 23) | (bl & 0x7FFFFFu));
    const int sh = (int)el - (int)eh + 29;  // <= 5
    long long add = sh >= 0 ? (ml << sh) : (sh > -40 ? (ml >> (-sh)) : 0);
    M += ((bl ^ bh) & 0x80000000u) ? -add : add;
    if (M < (1ll << 52)) {
      M <<= 1;
      E -= 1;
    }
  }
  const unsigned long long bits = ((unsigned long long)(bh & 0x80000000u) << 32) |
                                  ((unsigned long long)E << 52) | ((unsigned long long)M & ((1ull << 52) - 1));
  return __longlong_as_double((long long)bits);
}

// Float-float sum a + b (both hi + lo pairs): TwoSum of the high parts, the low parts and the
// rounding error added, then renormalised with the fast two-sum.
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
  float s, e;
  two_sum(a.x, b.x, s, e);
  e += a.y + b.y;
  const float h = s + e;
  return make_float2(h, e - (h - s));
}

// Dot2-style accumulation of c * x: (s, corr) with s + corr ~ sum of products.
struct FFAcc {
  float s, corr;
  // products are formed with __fmul_rn so that they are never contracted into a
  // following addition: TwoSum and the FMA error term need the rounded product itself
  __device__ __forceinline__ void first(float ch, float cl, float2 x) {
    s = __fmul_rn(ch, x.x);
    corr = fmaf(ch, x.x, -s);
    corr = fmaf(ch, x.y, corr);
    corr = fmaf(cl, x.x, corr);
  }
  __device__ __forceinline__ void add(float ch, float cl, float2 x) {
    const float p = __fmul_rn(ch, x.x);
    float t, err;
    two_sum(s, p, t, err);
    s = t;
    corr += fmaf(ch, x.x, -p) + err;
    corr = fmaf(ch, x.y, corr);
    corr = fmaf(cl, x.x, corr);
  }
  // moves the correction into s (s + corr unchanged): keeps |corr| near ulp(s) so the
  // FP32 rounding of later correction terms stays at the 2^-48 level
  __device__ __forceinline__ void renorm() {
    float t, e;
    two_sum(s, corr, t, e);
    s = t;
    corr = e;
  }
  __device__ __forceinline__ double result() const {
    float h, l;
    two_sum(s, corr, h, l);
    return ff_to_f64(h, l);
  }
};

template <int EJ, int EI, int R, int FAM>
__device__ __forceinline__ double stencil_point_ff(const float2 *__restrict__ c, const Taps &tp) {
  constexpr int SJ = EI, SK = EJ * EI;
  FFAcc a;
  if (FAM == FAM_STAR) {
    a.first(tp.cf[0], tp.cl[0], c[0]);
#pragma unroll
    for (int d = 1; d <= R; ++d) {
      const int t = 1 + 6 * (d - 1);
      a.add(tp.cf[t + 0], tp.cl[t + 0], c[d]);
      a.add(tp.cf[t + 1], tp.cl[t + 1], c[-d]);
      a.add(tp.cf[t + 2], tp.cl[t + 2], c[d * SJ]);
      a.add(tp.cf[t + 3], tp.cl[t + 3], c[-d * SJ]);
      a.add(tp.cf[t + 4], tp.cl[t + 4], c[d * SK]);
      a.add(tp.cf[t + 5], tp.cl[t + 5], c[-d * SK]);
      a.renorm();
    }
  } else if (FAM == FAM_CUBE) {
#pragma unroll
    for (int dk = -R; dk <= R; ++dk)
#pragma unroll
      for (int dj = -R; dj <= R; ++dj)
#pragma unroll
        for (int di = -R; di <= R; ++di) {
          const int t = ((dk + R) * (2 * R + 1) + (dj + R)) * (2 * R + 1) + (di + R);
          const float2 x = c[dk * SK + dj * SJ + di];
          if (t == 0) a.first(tp.cf[0], tp.cl[0], x);
          else a.add(tp.cf[t], tp.cl[t], x);
          if (di == R) a.renorm();
        }
  } else {
    a.first(tp.cf[0], tp.cl[0], c[tp.toff[0]]);
    for (int t = 1; t < tp.n; ++t) {
      a.add(tp.cf[t], tp.cl[t], c[tp.toff[t]]);
      if ((t & 7) == 7) a.renorm();
    }
  }
  return a.result();
}

// Element type of the shared-memory tile and the load that fills it.
template <typename T, int ACC>
struct TileOf {
  typedef typename Elem<T>::acc type;
  static __device__ __forceinline__ type load(const T *p) { return Elem<T>::load(p); }
};
template <>
struct TileOf<double, ACCM_FF> {
  typedef float2 type;
  static __device__ __forceinline__ float2 load(const double *p) { return split_f64(__ldg(p)); }
};

// One output point; c points at the centre element in the tile.
template <typename AT, int EJ, int EI, int R, int FAM, int ACC>
__device__ __forceinline__ AT stencil_point(const AT *__restrict__ c, const Taps &tp) {
  constexpr int SJ = EI, SK = EJ * EI;
  if (FAM == FAM_STAR) {
    if (ACC == ACCM_NATIVE) {
      AT v = coef<AT>(tp, 0) * c[0];
#pragma unroll
      for (int d = 1; d <= R; ++d) {
        const int t = 1 + 6 * (d - 1);
        v = fma(coef<AT>(tp, t + 0), c[d], v);
        v = fma(coef<AT>(tp, t + 1), c[-d], v);
        v = fma(coef<AT>(tp, t + 2), c[d * SJ], v);
        v = fma(coef<AT>(tp, t + 3), c[-d * SJ], v);
        v = fma(coef<AT>(tp, t + 4), c[d * SK], v);
        v = fma(coef<AT>(tp, t + 5), c[-d * SK], v);
      }
      return v;
    } else {
      // partial 0: the i row (centre and i taps) as an FMA chain; every j / k tap is
      // its own partial; partials are combined with Neumaier's compensated sum
      AT row = coef<AT>(tp, 0) * c[0];
#pragma unroll
      for (int d = 1; d <= R; ++d) {
        const int t = 1 + 6 * (d - 1);
        row = fma(coef<AT>(tp, t + 0), c[d], row);
        row = fma(coef<AT>(tp, t + 1), c[-d], row);
      }
      AT s = row, comp = AT(0);
#pragma unroll
      for (int d = 1; d <= R; ++d) {
        const int t = 1 + 6 * (d - 1);
        neumaier(s, comp, coef<AT>(tp, t + 2) * c[d * SJ]);
        neumaier(s, comp, coef<AT>(tp, t + 3) * c[-d * SJ]);
        neumaier(s, comp, coef<AT>(tp, t + 4) * c[d * SK]);
        neumaier(s, comp, coef<AT>(tp, t + 5) * c[-d * SK]);
      }
      return s + comp;
    }
  } else if (FAM == FAM_CUBE) {
    if (ACC == ACCM_NATIVE) {
      AT v = AT(0);
#pragma unroll
      for (int dk = -R; dk <= R; ++dk)
#pragma unroll
        for (int dj = -R; dj <= R; ++dj)
#pragma unroll
          for (int di = -R; di <= R; ++di) {
            const int t = ((dk + R) * (2 * R + 1) + (dj + R)) * (2 * R + 1) + (di + R);
            const AT x = c[dk * SK + dj * SJ + di];
            v = (t == 0) ? coef<AT>(tp, 0) * x : fma(coef<AT>(tp, t), x, v);
          }
      return v;
    } else {
      // each (dk, dj) row of 2R+1 taps is an FMA chain; rows are Neumaier-summed
      AT s = AT(0), comp = AT(0);
#pragma unroll
      for (int dk = -R; dk <= R; ++dk)
#pragma unroll
        for (int dj = -R; dj <= R; ++dj) {
          const int t0 = ((dk + R) * (2 * R + 1) + (dj + R)) * (2 * R + 1);
          AT row = coef<AT>(tp, t0) * c[dk * SK + dj * SJ - R];
#pragma unroll
          for (int di = -R + 1; di <= R; ++di)
            row = fma(coef<AT>(tp, t0 + di + R), c[dk * SK + dj * SJ + di], row);
          if (dk == -R && dj == -R) s = row;
          else neumaier(s, comp, row);
        }
      return s + comp;
    }
  } else {
    if (ACC == ACCM_NATIVE) {
      AT v = coef<AT>(tp, 0) * c[tp.toff[0]];
      for (int t = 1; t < tp.n; ++t) v = fma(coef<AT>(tp, t), c[tp.toff[t]], v);
      return v;
    } else {
      AT s = coef<AT>(tp, 0) * c[tp.toff[0]], comp = AT(0);
      for (int t = 1; t < tp.n; ++t) neumaier(s, comp, coef<AT>(tp, t) * c[tp.toff[t]]);
      return s + comp;
    }
  }
}

template <typename T, int BK, int BJ, int BI, int R, int FAM, bool RM, int ACC>
__global__ void __launch_bounds__(sweep_threads(BJ * BI))
sweep_kernel(const SweepArgs a, const Taps tp) {
  typedef typename TileOf<T, ACC>::type AT;
  constexpr int TPB = BJ * BI;
  constexpr int NT = sweep_threads(TPB);
  constexpr int NB = NT / TPB;
  constexpr int EK = BK + 2 * R, EJ = BJ + 2 * R, EI = BI + 2 * R;
  constexpr int TILE = EK * EJ * EI;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  AT *tiles = reinterpret_cast<AT *>(smem_raw);
  unsigned *nbrs = reinterpret_cast<unsigned *>(smem_raw + sizeof(AT) * TILE * NB);

  const int slot = threadIdx.x / TPB, lt = threadIdx.x % TPB;
  AT *tile = tiles + slot * TILE;
  unsigned *nbr = nbrs + slot * 28;
  const T *in = reinterpret_cast<const T *>(a.in) + a.in_off;
  T *out = reinterpret_cast<T *>(a.out) + a.out_off;

  for (long long base = (long long)blockIdx.x * NB; base < a.nlist; base += (long long)gridDim.x * NB) {
    const long long n = base + slot;
    // all 27 slots are written every iteration, whatever the threads per brick (16 for 4^3)
    for (int sl = lt; sl < 27; sl += TPB) {
      unsigned v = 0;
      int ok = 0;
      if (n < a.nlist) {
        const unsigned b = a.blist[n];
        if (b < a.nbricks) {
          v = a.adj[(size_t)b * 27 + sl];
          ok = 1;
          // the centre entry is also the output brick: out of range skips the brick
          if (sl == 13 && ((long long)v >= a.out_chunks || (long long)v >= a.in_chunks)) ok = 0;
          if ((long long)v >= a.in_chunks || !ok) { atomicOr(a.err, FLAG_BOUNDS); v = 0; }
        } else if (sl == 13) {
          atomicOr(a.err, FLAG_BOUNDS);
        }
      }
      nbr[sl] = v;
      if (sl == 13) nbr[27] = ok;
    }
    __syncthreads();
    const bool active = nbr[27] != 0;
    if (active) {
      for (int e = lt; e < TILE; e += TPB) {
        const int kk = e / (EJ * EI), rem = e - kk * (EJ * EI);
        const int jj = rem / EI, ii = rem - jj * EI;
        const int qk = kk < R ? -1 : (kk >= R + BK ? 1 : 0);
        const int qj = jj < R ? -1 : (jj >= R + BJ ? 1 : 0);
        const int qi = ii < R ? -1 : (ii >= R + BI ? 1 : 0);
        if (FAM == FAM_STAR && ((qk != 0) + (qj != 0) + (qi != 0)) > 1) continue;
        const int lk = kk - R - qk * BK, lj = jj - R - qj * BJ, li = ii - R - qi * BI;
        const unsigned nb = nbr[(qk + 1) * 9 + (qj + 1) * 3 + (qi + 1)];
        const int o = RM ? (lk * BJ + lj) * BI + li : a.L.offset(lk, lj, li);
        tile[e] = op_apply(TileOf<T, ACC>::load(in + (size_t)nb * a.in_step + o), tp.pre);
      }
    }
    __syncthreads();
    if (active) {
      const int j = lt / BI, i = lt - (lt / BI) * BI;
      T *ob = out + (size_t)nbr[13] * a.out_step;
#pragma unroll 1
      for (int k = 0; k < BK; ++k) {
        const AT *c = tile + ((k + R) * EJ + (j + R)) * EI + (i + R);
        typename Elem<T>::acc v;
        if constexpr (ACC == ACCM_FF) v = stencil_point_ff<EJ, EI, R, FAM>(c, tp);
        else v = stencil_point<AT, EJ, EI, R, FAM, ACC>(c, tp);
        const int o = RM ? (k * BJ + j) * BI + i : a.L.offset(k, j, i);
        Elem<T>::store(ob + o, op_apply(v, tp.post));
      }
    }
    __syncthreads();
  }
}

template <typename T, int BK, int BJ, int BI, int R, int FAM, bool RM, int ACC>
int launch_sweep(const SweepArgs &a, const Taps &tp, cudaStream_t s) {
  typedef typename TileOf<T, ACC>::type AT;
  constexpr int TPB = BJ * BI;
  constexpr int NT = sweep_threads(TPB);
  constexpr int NB = NT / TPB;
  constexpr int TILE = (BK + 2 * R) * (BJ + 2 * R) * (BI + 2 * R);
  constexpr size_t smem = sizeof(AT) * TILE * NB + sizeof(unsigned) * 28 * NB;
  static_assert(smem <= 227 * 1024, "tile too large");
  auto kern = sweep_kernel<T, BK, BJ, BI, R, FAM, RM, ACC>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(sweep)");
  }
  long long grid = ((long long)a.nlist + NB - 1) / NB;
  if (grid > (1ll << 30)) grid = 1ll << 30;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, NT, smem, s>>>(a, tp);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "sweep kernel launch");
  return BK_OK;
}

// Which instantiation a sweep needs.
struct SweepPlan {
  int dtype;
  int shape;  // 0: 8x8x8, 1: 4x4x4, 2: 16x8x8, 3: 8x8x32
  bool rm;
  bool v2;    // row-major and aligned: the pipelined kernel applies
  bool tma;   // star stencil on row-major 8x8x8 bricks, TMA-describable field: the TMA kernel applies
  bool sym;   // cube with mirror-symmetric coefficients (sym_index table filled)
  bool symij; // ... and symmetric under the i <-> j swap
  bool ops;   // pointwise pre / post operations (one-shot kernels only)
  bool out_pair;  // every output brick starts on a boundary of two elements (pair stores)
  bool istream;   // FP64 mirror-symmetric 8x8x8 cubes: columns streamed along i
  int fam;
  int r;
  int acc;
  const int (*offs)[3];  // tap offsets in kernel order (generic family)
  const int *toff1;      // generic-family tile offsets for the one-shot kernel
};

int sweep_dispatch_f64(const SweepPlan &p, const SweepArgs &a, Taps &tp, cudaStream_t s);
int sweep_dispatch_f32(const SweepPlan &p, const SweepArgs &a, Taps &tp, cudaStream_t s);
int sweep_dispatch_bf16(const SweepPlan &p, const SweepArgs &a, Taps &tp, cudaStream_t s);
int sweep_dispatch_tma(const SweepPlan &p, const SweepArgs &a, Taps &tp, cudaStream_t s);
bool tma_eligible(const SweepPlan &p, const bk_field *in);
// Whether a TMA sweep takes the row-run kernel (2- and 4-byte storage; BK_TMA_ROW=0 selects
// per-brick staging).
bool tma_row(const SweepPlan &p);

}  // namespace bk
