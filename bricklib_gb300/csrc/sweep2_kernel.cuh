// Pipelined brick sweep for row-major brick layouts (sweep_kernel covers the rest).
//
// Persistent CTAs walk the brick list in groups of NB bricks (every gridDim.x-th group; a
// contiguous share of the list per CTA for the FP64 mirror-symmetric cubes streamed along i,
// sym_cube_istream).  For every group:
//   * the 27 adjacency entries of each brick are staged in shared memory;
//   * every thread issues its share of the group's gather as asynchronous global->shared
//     copies (cp.async, 16 bytes where the layout allows) into one of two tile buffers,
//     following a per-thread plan computed once at kernel start: each plan entry is one
//     vector of the brick's neighbourhood -- centre brick, faces (stars) or the full
//     (BK+2R) x (BJ+2R) x (BI+2RP) box (cubes) -- packed as (adjacency slot, source
//     offset in the neighbour brick, destination offset in the tile);
//   * while those copies are in flight the previous group is computed from the other
//     buffer.
// Compute: each thread owns one (j, i) column of a brick; the column's k-extended values
// sit in registers, so k-direction taps cost no shared-memory loads; star stencils read
// the i / j taps from the tile, cube stencils walk the (2R+1)^2 columns (the 8x8x8 cube
// paths: a column pair per lane, or, streamed along i, two rows per lane).  Float-float
// mode converts the raw FP64 tile into float pairs in one pass before computing.
#pragma once

#include "sweep_kernel.cuh"

namespace bk {

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

template <int BYTES>
__device__ __forceinline__ void cp_async(unsigned dst, const void *src) {
  if (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(dst), "l"(src), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// FP64 arithmetic on register operands only.  On GB300 a DADD, a DMUL, or a DFMA that reads its
// coefficient from the constant bank issues about a fifth slower than a DFMA whose operands are
// all registers (standalone probe, 16 warps per SM: 0.80 against 0.955 of the DFMA rate), so the
// native FP64 kernels write a + b as fma(1, a, b) and c * x as fma(c, x, -0), with 1 and -0 in
// registers, and read their coefficients from shared memory into registers.  The bits are those
// of the plain operations: 1 * a is exact and -0 is the identity of every sum (signed zeros
// included), so each form rounds once, as the plain operation does.  The operands come from a
// shared-memory block (F64Ops::NHEAD doubles, then the coefficients, filled from Taps::one_mz
// and c; stars and cubes), or, for the class-sum stream, whose tile leaves no room for the
// block without losing a resident CTA per SM, straight from the kernel parameters at an index
// carrying a zero the compiler cannot see through (so the loads are neither folded into
// constant operands nor hoisted).  Measured: the stream runs the same from either source; the
// 27-point cube ran 22.4 GStencil/s from the shared block and 19.0 from parameter loads.
__device__ __forceinline__ int opaque_zero() {
  int z;
  asm volatile("mov.u32 %0, 0;\n" : "=r"(z));
  return z;
}
struct F64Ops {
  static constexpr int NHEAD = 2;
  double one, mz;
  __device__ __forceinline__ static F64Ops load(const double *cs) { return F64Ops{cs[0], cs[1]}; }
  __device__ __forceinline__ static F64Ops load(const Taps &tp) {
    const int z = opaque_zero();
    return F64Ops{tp.one_mz[z], tp.one_mz[z + 1]};
  }
  __device__ __forceinline__ double add(double a, double b) const { return fma(one, a, b); }
  __device__ __forceinline__ double mul(double c, double x) const { return fma(c, x, mz); }
};
// coefficient t of Taps::c as a per-thread register operand, loaded at each call
__device__ __forceinline__ double f64_coef(const Taps &tp, int t) { return tp.c[t + opaque_zero()]; }

__device__ __forceinline__ void store_stream(double *p, double v) { __stcs(p, v); }
__device__ __forceinline__ void store_stream(float *p, float v) { __stcs(p, v); }
__device__ __forceinline__ void store_stream(__nv_bfloat16 *p, float v) { *p = __float2bfloat16_rn(v); }

__device__ __forceinline__ float to_acc(__nv_bfloat16 x) { return __bfloat162float(x); }
__device__ __forceinline__ float to_acc(float x) { return x; }
__device__ __forceinline__ double to_acc(double x) { return x; }

// Two adjacent elements (i, i+1) of a brick row in FP32: one 8-byte (FP32) or 4-byte (BF16)
// shared-memory load, one store of the same width.  bf16 -> fp32 is exact (the bf16 bits are
// the high half of the fp32 word); fp32 -> bf16 rounds to nearest even as the scalar path.
__device__ __forceinline__ float2 ld_pair(const float *p) { return *reinterpret_cast<const float2 *>(p); }
__device__ __forceinline__ float2 ld_pair(const __nv_bfloat16 *p) {
  const unsigned u = *reinterpret_cast<const unsigned *>(p);
  return make_float2(__uint_as_float(u << 16), __uint_as_float(u & 0xFFFF0000u));
}
__device__ __forceinline__ void st_pair(float *p, float2 v) { __stcs(reinterpret_cast<float2 *>(p), v); }
__device__ __forceinline__ void st_pair(__nv_bfloat16 *p, float2 v) {
  *reinterpret_cast<__nv_bfloat162 *>(p) = __floats2bfloat162_rn(v.x, v.y);
}
__device__ __forceinline__ double2 ld_pair(const double *p) { return *reinterpret_cast<const double2 *>(p); }
__device__ __forceinline__ void st_pair(double *p, double2 v) { __stcs(reinterpret_cast<double2 *>(p), v); }
__device__ __forceinline__ float2 pair_of(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ double2 pair_of(double a, double b) { return make_double2(a, b); }

__host__ __device__ constexpr int cmin(int a, int b) { return a < b ? a : b; }
__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }

// Smallest row length >= need (a multiple of ve) for which the 32/bi consecutive rows
// read by one warp map to pairwise disjoint bank sets (8-byte elements: per half warp).
__host__ __device__ constexpr bool rows_disjoint(int ei, int bi, int es) {
  const int words_row = ei * es / 4 > 0 ? ei * es / 4 : 1;  // row stride in 4-byte words
  const int seg = (bi * es + 3) / 4;                          // words one row segment covers
  const int lanes = es == 8 ? 16 : 32;
  const int rows = lanes / bi > 0 ? lanes / bi : 1;
  if (seg * rows > 32) return true;  // the warp needs several wavefronts whatever the stride
  for (int a = 0; a < rows; ++a)
    for (int b = a + 1; b < rows; ++b)
      for (int x = 0; x < seg; ++x)
        for (int y = 0; y < seg; ++y)
          if ((a * words_row + x) % 32 == (b * words_row + y) % 32) return false;
  return true;
}
__host__ __device__ constexpr int conflict_free_row(int need, int bi, int es, int ve) {
  int ei = need;
  for (int t = 0; t < 64; ++t, ei += ve)
    if (rows_disjoint(ei, bi, es)) return ei;
  return need;
}

// 16-element FP32 tile rows with XOR-permuted 16-byte units for the FP32 class-sum stream (1),
// or rows padded to 20 elements (0)
#ifndef BK_CS_SWZ
#define BK_CS_SWZ 1
#endif

// bricks (warps) per CTA of the column-pair cube kernels: one, so that a CTA's barriers wait
// for no other warp (GB300, FP32 cube125 at 512^3: 191 / 171 GStencil/s with one / two)
// class-sum streams of 4- / 2-byte storage: about this many consecutive groups per chunk of a
// CTA's walk
#ifndef BK_CS_CHUNK
#define BK_CS_CHUNK 16
#endif

// resident two-warp CTAs per SM asked of the register allocator for the compensated FP32 / BF16
// class-sum stream (0: none).  GB300, cube125 at 512^3, FP32 / BF16 GStencil/s: none (182 / 146
// registers) 99.3 / 110.7; 6 (168, some spilled) 114.5 / 109.0; 8 (128, 50-80 bytes spilled)
// 119.8 / 112.8; 10 (96, 100-150 bytes spilled) 114.1 / 109.1
#ifndef BK_CS_COMP_MINB
#define BK_CS_COMP_MINB 8
#endif

#ifndef BK_PAIR_NB
#define BK_PAIR_NB 1
#endif
constexpr int PAIR_NB = BK_PAIR_NB;

// IST: the class-sum stream of the mirror-symmetric cubes (sym_cube_istream for FP64,
// sym_cube_istream4 for 4- and 2-byte storage), one warp per 8x8x8 brick (two for the
// compensated 4- and 2-byte stream, one row per thread).
template <typename T, int BK, int BJ, int BI, int R, int FAM, int ACC, bool IST = false>
struct Sweep2Cfg {
  static constexpr int ES = (int)sizeof(T);
  static constexpr int VB = cmin(16, BI * ES);  // bytes per copy
  static constexpr int VE = VB / ES;            // elements per copy
  static constexpr int RP = (R + VE - 1) / VE * VE;  // i halo rounded up to whole copies
  static constexpr int EK = BK + 2 * R, EJ = BJ + 2 * R;
  // Tile row length, at least BI + 2*RP, chosen against shared-memory bank conflicts.
  // 8-byte elements in 8-wide rows: a half warp reads two rows; lanes are assigned to
  // rows in the order 0,2,1,3 so those two rows are two apart, and a row length of
  // 4 (mod 8) elements puts them 16 banks apart.  Otherwise: pad until the rows one warp
  // reads fall in disjoint banks.
  static constexpr bool PERM = ES == 8 && BI == 8;
  static constexpr int NEED = BI + 2 * RP;
  // the class-sum stream of 4- / 2-byte storage reads 4 columns of 32 rows at once (16 / 8
  // bytes per lane).  FP32: rows of 16 elements with the 16-byte units of row jj XOR-permuted by
  // (jj >> 1) & 3 (SWZ), which puts the 8 rows of a quarter warp in distinct 4-bank groups
  // (conflict free) with no padding -- a smaller tile, more CTAs per SM.  BF16: rows of 24
  // (two-way within a half warp, which reads half the bytes of the FP32 case)
  static constexpr bool CS4 = IST && ES <= 4;
  static constexpr bool SWZ = BK_CS_SWZ && CS4 && ES == 4 && BI + 2 * RP == 16;
  static constexpr int EI = CS4 ? (ES == 4 ? (SWZ ? 16 : 20) : 24)
                          : PERM ? (NEED % 8 <= 4 ? NEED - NEED % 8 + 4 : NEED - NEED % 8 + 12)
                                 : conflict_free_row(NEED, BI, ES, VE);
  static constexpr int TILE = EK * EJ * EI;  // elements per brick tile
  // position within tile row jj of column ii (SWZ: the row's 16-byte units permuted)
  static __host__ __device__ __forceinline__ int col(int jj, int ii) {
    return SWZ ? ((((ii >> 2) ^ ((jj >> 1) & 3)) << 2) | (ii & 3)) : ii;
  }
  static constexpr int TILE_BYTES = (TILE * ES + 15) / 16 * 16;
  // Column pairs: one warp per 8x8x8 brick, each lane computing columns (i0, i0 + 1) from
  // 8-byte (FP32) / 4-byte (BF16) row loads, for the cubes whose per-plane row values or
  // symmetry-class sums fit a sliding window along k (FP32 arithmetic on 2- and 4-byte
  // storage; GB300 at 512^3, GStencil/s against one column per thread: FP32 cube27 313 / 287,
  // cube125 191 / 156; BF16 cube27 412 / 302, cube125 235 / 139).
  static constexpr bool PAIR = BK == 8 && BJ == 8 && BI == 8 && ACC == ACCM_NATIVE &&
                               (FAM == FAM_CUBESYM || FAM == FAM_CUBESYM_IJ || (FAM == FAM_CUBE && R == 1 && ES <= 4));
  static constexpr bool WARP1 = PAIR || CS4;  // one warp per brick (the compensated stream: two)
  // rows of the brick per thread in the FP32 / BF16 class-sum stream: two in native arithmetic
  // (one warp per brick), one under compensated accumulation (two warps per brick), whose Dot2
  // state per row would otherwise cap the SM at 8 warps (255 registers)
  static constexpr int CSROWS = CS4 && ACC == ACCM_COMP ? 1 : 2;
  static constexpr int TPB = CS4 ? BK * BJ / CSROWS : WARP1 ? BJ * BI / 2 : BJ * BI;
  // vectors of the neighbourhood (per brick)
  static constexpr int NV_CENTRE = BK * BJ * (BI / VE);
  static constexpr int NV_KF = R * BJ * (BI / VE);   // one k face
  static constexpr int NV_JF = BK * R * (BI / VE);   // one j face
  static constexpr int NV_IF = BK * BJ * (RP / VE);  // one i face
  static constexpr int NV_STAR = NV_CENTRE + 2 * (NV_KF + NV_JF + NV_IF);
  static constexpr int NV_CUBE = EK * EJ * (NEED / VE);  // the row padding is never fetched
  static constexpr int NV = FAM == FAM_STAR ? NV_STAR : NV_CUBE;
  static constexpr int EPT = (NV + TPB - 1) / TPB;  // plan entries per thread
  // float-float converts each raw FP64 tile into float pairs in place (same 8 bytes)
  static constexpr int FTILE_BYTES = 0;
  // bricks per CTA: as many as fit 128 threads and a ~100 KB shared-memory budget
  static constexpr int PER_BRICK = 2 * TILE_BYTES + FTILE_BYTES + 3 * 36 * 4;
  static constexpr int NB = CS4 ? 1 : PAIR ? PAIR_NB : cmax(1, cmin(cmax(1, 128 / TPB), (100 * 1024) / PER_BRICK));
  static constexpr int NT = TPB * NB;
  // native FP64 arithmetic on register operands (F64Ops).  Stars and cubes read them from a
  // shared-memory block after the tiles and the adjacency slots (F64Ops head, then the taps'
  // coefficients); the class-sum streams read them from the kernel parameters (a block would cost
  // them a resident CTA per SM, and they measured the same either way).
  static constexpr bool F64R = ES == 8 && ACC == ACCM_NATIVE;
  static constexpr bool SYMF = FAM == FAM_CUBESYM || FAM == FAM_CUBESYM_IJ;
  static constexpr bool F64S = F64R && (FAM == FAM_STAR || FAM == FAM_CUBE);
  static constexpr int NCOEF = FAM == FAM_STAR ? 1 + 6 * R : (2 * R + 1) * (2 * R + 1) * (2 * R + 1);
  static constexpr int COEFB = F64S ? ((F64Ops::NHEAD + NCOEF) * 8 + 15) / 16 * 16 : 0;
  static constexpr int SMEM = NB * PER_BRICK + COEFB;
  // resident CTAs asked of the register allocator: the native FP32 / BF16 class-sum stream
  // (one warp per CTA) at <= 170 registers fits three warps per scheduler (12 per SM), which its
  // shared memory also allows; the compensated stream (two warps per CTA): BK_CS_COMP_MINB
  static constexpr int MINB = CS4 ? (ACC == ACCM_NATIVE ? 12 : BK_CS_COMP_MINB) : 0;
};

// Tile coordinates (kk, jj, ii) of plan vector g for the star / cube neighbourhood.
template <typename C, int BK, int BJ, int BI, int R, int FAM>
__device__ __forceinline__ void plan_coords(int g, int &kk, int &jj, int &ii) {
  constexpr int VE = C::VE, RP = C::RP;
  if (FAM != FAM_STAR) {
    constexpr int RV = C::NEED / VE;
    kk = g / (C::EJ * RV);
    const int r = g - kk * (C::EJ * RV);
    jj = r / RV;
    ii = (r - jj * RV) * VE;
    return;
  }
  constexpr int BV = BI / VE;
  // regions: centre, k-lo, k-hi, j-lo, j-hi, i-lo, i-hi
  if (g < C::NV_CENTRE) {
    kk = g / (BJ * BV);
    const int r = g - kk * (BJ * BV);
    jj = r / BV;
    ii = (r - jj * BV) * VE;
    kk += R; jj += R; ii += RP;
    return;
  }
  g -= C::NV_CENTRE;
  if (g < 2 * C::NV_KF) {
    const int hi = g >= C::NV_KF;
    g -= hi * C::NV_KF;
    kk = g / (BJ * BV);
    const int r = g - kk * (BJ * BV);
    jj = r / BV;
    ii = (r - jj * BV) * VE;
    kk += hi ? R + BK : 0; jj += R; ii += RP;
    return;
  }
  g -= 2 * C::NV_KF;
  if (g < 2 * C::NV_JF) {
    const int hi = g >= C::NV_JF;
    g -= hi * C::NV_JF;
    kk = g / (R * BV);
    const int r = g - kk * (R * BV);
    jj = r / BV;
    ii = (r - jj * BV) * VE;
    kk += R; jj += hi ? R + BJ : 0; ii += RP;
    return;
  }
  g -= 2 * C::NV_JF;
  {
    constexpr int IV = RP / VE;
    const int hi = g >= C::NV_IF;
    g -= hi * C::NV_IF;
    kk = g / (BJ * IV);
    const int r = g - kk * (BJ * IV);
    jj = r / IV;
    ii = (r - jj * IV) * VE;
    kk += R; jj += R; ii += hi ? RP + BI : 0;
  }
}

// Class-sum streams: a brick that continues a stream reads only the tile columns from ICUT on
// (the W of the earlier columns come from the previous brick).  Its plan lists first the copies
// of columns from ICUT on (NS of each row's NEED / VE copies lie wholly before ICUT), then the
// others, so a continued brick issues a prefix of the plan.
template <typename C, int R>
struct StreamPlan {
  static constexpr int ICUT = C::ES == 8 ? C::RP + R : C::RP + 4;
  static constexpr int RV = C::NEED / C::VE;               // copies per tile row
  static constexpr int NS = ICUT / C::VE;                   // of them wholly before ICUT
  static constexpr int NN = RV - NS;
  static constexpr int NVN = C::EK * C::EJ * NN;            // copies a continued brick needs
};

// Packed plan entry: slot (5 bits) | source element offset in the neighbour brick (13 bits)
// | destination element offset in the tile (14 bits).  All three fit for bricks up to 8192
// elements and tiles up to 16384 elements (checked on the host).  SORD: the stream order above.
template <typename C, int BK, int BJ, int BI, int R, int FAM, bool SORD = false>
__device__ __forceinline__ unsigned plan_entry(int g) {
  int kk, jj, ii;
  if constexpr (SORD) {
    typedef StreamPlan<C, R> P;
    static_assert(FAM != FAM_STAR, "streams are for cubes");
    int row, chunk;
    if (g < P::NVN) {
      row = g / P::NN;
      chunk = P::NS + g % P::NN;
    } else {
      row = (g - P::NVN) / P::NS;
      chunk = (g - P::NVN) % P::NS;
    }
    kk = row / C::EJ;
    jj = row % C::EJ;
    ii = chunk * C::VE;
  } else {
    plan_coords<C, BK, BJ, BI, R, FAM>(g, kk, jj, ii);
  }
  const int qk = kk < R ? -1 : (kk >= R + BK ? 1 : 0);
  const int qj = jj < R ? -1 : (jj >= R + BJ ? 1 : 0);
  const int qi = ii < C::RP ? -1 : (ii >= C::RP + BI ? 1 : 0);
  const int lk = kk - R - qk * BK, lj = jj - R - qj * BJ, li = ii - C::RP - qi * BI;
  const unsigned slot = (unsigned)((qk + 1) * 9 + (qj + 1) * 3 + (qi + 1));
  const unsigned src = (unsigned)((lk * BJ + lj) * BI + li);
  const unsigned dst = (unsigned)((kk * C::EJ + jj) * C::EI + C::col(jj, ii));
  return slot | (src << 5) | (dst << 18);
}

// Columns (i0, i0 + 1) of row j of one 8x8x8 brick, every k, from its staged tile, in FP32
// arithmetic: mirror-symmetric cubes (radius 1 or 2, pair sums) and the radius-1 cube.  Plane
// kk of the tile yields the 2R + 2 values x(kk, j + dj, i0 - R .. i0 + 1 + R) of every row
// dj = -R..R (aligned pair loads); a symmetric cube reduces them at once to its class sums
// q(kk).  Output plane k is complete once plane k + 2R is in, and is then summed term by term
// in the order of the one-column code below (class by class: c0 q(k), then c_d (q(k-d) +
// q(k+d)); the plain cube: dj, di, dk), so both give identical results.  Only the last 2R + 1
// planes are live.
template <typename C, typename T, int R, int FAM>
__device__ __forceinline__ void cube_pair_columns(const T *rt, T *ob, const int j, const int i0, const Taps &tp) {
  constexpr int BK = 8, PK = 64, SK = C::EJ * C::EI, SJ = C::EI, RP = C::RP;
  constexpr int NK = BK + 2 * R, NR = 2 * R + 1, W = 2 * R + 2;
  static_assert(R == 1 || R == 2, "cube radius");
  typedef typename Elem<T>::acc AT;
  const T *col = rt + (j + R) * SJ + (i0 + RP);  // (plane 0, row j, column i0)
  // x[kk][r][m] = x(kk, j + r - R, i0 + m - R)
  AT x[NK][NR][W];
  auto load_plane = [&](int kk) {
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      const T *p = col + kk * SK + (r - R) * SJ;
      if constexpr (R == 1) {
        const auto c = ld_pair(p);
        x[kk][r][0] = to_acc(p[-1]);
        x[kk][r][1] = c.x;
        x[kk][r][2] = c.y;
        x[kk][r][3] = to_acc(p[2]);
      } else {
        const auto l = ld_pair(p - 2), c = ld_pair(p), h = ld_pair(p + 2);
        x[kk][r][0] = l.x;
        x[kk][r][1] = l.y;
        x[kk][r][2] = c.x;
        x[kk][r][3] = c.y;
        x[kk][r][4] = h.x;
        x[kk][r][5] = h.y;
      }
    }
  };
  if constexpr (FAM == FAM_CUBE) {
#pragma unroll
    for (int kk = 0; kk < NK; ++kk) {
      load_plane(kk);
      if (kk >= 2 * R) {
        const int k = kk - 2 * R;
        AT acc[2];
#pragma unroll
        for (int dj = -R; dj <= R; ++dj)
#pragma unroll
          for (int di = -R; di <= R; ++di)
#pragma unroll
            for (int dk = -R; dk <= R; ++dk) {
              const int t = ((dk + R) * (2 * R + 1) + (dj + R)) * (2 * R + 1) + (di + R);
              const AT c = coef<AT>(tp, t);
#pragma unroll
              for (int o = 0; o < 2; ++o) {
                const AT v = x[k + R + dk][dj + R][R + o + di];
                acc[o] = (dj == -R && di == -R && dk == -R) ? c * v : fma(c, v, acc[o]);
              }
            }
        st_pair(ob + k * PK, pair_of(acc[0], acc[1]));
      }
    }
  } else {
    constexpr bool IJ = FAM == FAM_CUBESYM_IJ;
    constexpr int NC = IJ ? (R + 1) * (R + 2) / 2 : (R + 1) * (R + 1);
    AT q[NC][NK][2];
    // sum of x(kk, j +- b, i +- a) over the distinct sign choices, for output column i0 + o
    auto ring = [&](int kk, int b, int a, int o) -> AT {
      const int m = R + o;
      if (a == 0 && b == 0) return x[kk][R][m];
      if (b == 0) return x[kk][R][m - a] + x[kk][R][m + a];
      if (a == 0) return x[kk][R - b][m] + x[kk][R + b][m];
      return (x[kk][R - b][m - a] + x[kk][R - b][m + a]) + (x[kk][R + b][m - a] + x[kk][R + b][m + a]);
    };
#pragma unroll
    for (int kk = 0; kk < NK; ++kk) {
      load_plane(kk);
      {
        int cls = 0;
#pragma unroll
        for (int b = 0; b <= R; ++b)
#pragma unroll
          for (int a = 0; a <= (IJ ? b : R); ++a, ++cls)
#pragma unroll
            for (int o = 0; o < 2; ++o)
              q[cls][kk][o] = (IJ && a != b) ? ring(kk, b, a, o) + ring(kk, a, b, o) : ring(kk, b, a, o);
      }
      if (kk >= 2 * R) {
        const int k = kk - 2 * R;
        AT acc[2];
        int cls = 0;
#pragma unroll
        for (int b = 0; b <= R; ++b)
#pragma unroll
          for (int a = 0; a <= (IJ ? b : R); ++a, ++cls) {
            const AT c0 = coef<AT>(tp, sym_index(0, b, a, R));
#pragma unroll
            for (int o = 0; o < 2; ++o)
              acc[o] = (a == 0 && b == 0) ? c0 * q[cls][k + R][o] : fma(c0, q[cls][k + R][o], acc[o]);
#pragma unroll
            for (int d = 1; d <= R; ++d) {
              const AT cd = coef<AT>(tp, sym_index(d, b, a, R));
#pragma unroll
              for (int o = 0; o < 2; ++o) acc[o] = fma(cd, q[cls][k + R - d][o] + q[cls][k + R + d][o], acc[o]);
            }
          }
        st_pair(ob + k * PK, pair_of(acc[0], acc[1]));
      }
    }
  }
}

// FP64 mirror-symmetric cubes on column pairs with fewer FP64 operations: plane by plane the
// row sums V_b(m) = x(j - b, m) + x(j + b, m) of the 2R + 2 columns are shared by both outputs,
// the class sums T(b, a) = V_b(i - a) + V_b(i + a) come from them, and every class sum of plane
// kk goes straight into the 2R + 1 output planes it reaches (one multiply-add each, as many
// operations as the pair sums q(k - d) + q(k + d) but no window of class sums to keep).  The
// 125-point cube with i <-> j symmetry: 52.5 FP64 operations per point instead of 58.5.  The
// summation order differs from the one-column code (results agree to rounding).
template <typename C, typename T, int R, bool IJ>
__device__ __forceinline__ void sym_cube_pair_shared(const T *rt, T *ob, const int j, const int i0, const Taps &tp) {
  constexpr int BK = 8, PK = 64, SK = C::EJ * C::EI, SJ = C::EI, RP = C::RP;
  constexpr int NK = BK + 2 * R, W = 2 * R + 2;
  static_assert(R == 1 || R == 2, "cube radius");
  typedef typename Elem<T>::acc AT;
  const T *col = rt + (j + R) * SJ + (i0 + RP);  // (plane 0, row j, column i0)
  AT acc[BK][2];
#pragma unroll
  for (int kk = 0; kk < NK; ++kk) {
    // V[b][m] = sum of x(kk, j +- b, i0 + m - R) (b = 0: the row itself)
    AT V[R + 1][W];
#pragma unroll
    for (int b = 0; b <= R; ++b) {
      AT lo[W], hi[W];
#pragma unroll
      for (int sg = 0; sg < (b ? 2 : 1); ++sg) {
        const T *p = col + kk * SK + (sg ? b : -b) * SJ;
        AT *dst = sg ? hi : lo;
        if constexpr (R == 1) {
          const auto c = ld_pair(p);
          dst[0] = to_acc(p[-1]);
          dst[1] = c.x;
          dst[2] = c.y;
          dst[3] = to_acc(p[2]);
        } else {
          const auto l = ld_pair(p - 2), c = ld_pair(p), h = ld_pair(p + 2);
          dst[0] = l.x;
          dst[1] = l.y;
          dst[2] = c.x;
          dst[3] = c.y;
          dst[4] = h.x;
          dst[5] = h.y;
        }
      }
#pragma unroll
      for (int m = 0; m < W; ++m) V[b][m] = b ? lo[m] + hi[m] : lo[m];
    }
#pragma unroll
    for (int o = 0; o < 2; ++o) {
      const int mc = R + o;
      auto Tba = [&](int b, int a) -> AT { return a == 0 ? V[b][mc] : V[b][mc - a] + V[b][mc + a]; };
      int cls = 0;
#pragma unroll
      for (int b = 0; b <= R; ++b)
#pragma unroll
        for (int a = 0; a <= (IJ ? b : R); ++a, ++cls) {
          const AT qv = (IJ && a != b) ? Tba(b, a) + Tba(a, b) : Tba(b, a);
#pragma unroll
          for (int k = 0; k < BK; ++k) {
            const int dk = kk - R - k;
            if (dk < -R || dk > R) continue;
            const AT c = coef<AT>(tp, sym_index(dk < 0 ? -dk : dk, b, a, R));
            if (dk == -R && cls == 0) acc[k][o] = c * qv;
            else acc[k][o] = fma(c, qv, acc[k][o]);
          }
        }
    }
    if (kk >= 2 * R) st_pair(ob + (kk - 2 * R) * PK, pair_of(acc[kk - 2 * R][0], acc[kk - 2 * R][1]));
  }
}

// FP64 mirror-symmetric cubes streamed along i.  With the CTA walking a contiguous share of
// the brick list, consecutive entries that are i-neighbours (the next brick's column of
// i-lo neighbours is this brick's centre column, and its centre column this brick's i-hi
// column) form one stream.  For each tile column ii a lane forms, for its rows (k0, j) and
// (k0 + 1, j), the class sums Q(c, b) = sum of x(k +- c, j +- b, ii) (from the row sums
// H_b(k') = x(k', j - b) + x(k', j + b), shared by both rows) and from them
// W_a(ii) = sum over (c, b) of coef(c, b, a) Q(c, b), a = 0..R.  The output at column i is
// W_0(i) + sum over a of (W_a(i - a) + W_a(i + a)).  The W of a brick's last 2R columns carry
// over to the next brick of a stream, so a brick costs 8 columns instead of 8 + 2R: the
// 125-point cube takes 43 FP64 operations per point, 37 when its coefficients are also
// symmetric under k <-> j (Q(c, b) + Q(b, c) share one multiply-add).  Each W depends on one
// input column only, so a brick's outputs are the same bits whether the W of its first 2R
// columns were carried or computed from its own tile.  Output (k, j, i) is parked in the tile
// at its own input position, whose column was consumed R steps earlier (the CTA is this one
// warp), and the finished brick leaves in whole-warp 512-byte stores.  All arithmetic runs on
// register operands (F64Ops).
template <typename C, int R, bool KJ>
__device__ __forceinline__ void sym_cube_istream(double *rt, double *ob, const int lane, const Taps &tp,
                                                 double (&W)[2][R + 1][2 * R + 1], const bool cont) {
  constexpr int SK = C::EJ * C::EI, SJ = C::EI, RP = C::RP, NW = 2 * R + 1;
  static_assert(R == 1 || R == 2, "cube radius");
  const int k0 = 2 * (lane >> 3), j = lane & 7;
  // register operands (F64Ops): the class coefficients coef(c, b, a), 1 and -0
  static_assert(C::F64R && C::SYMF, "native FP64 classes");
  const F64Ops f = F64Ops::load(tp);
  // the class coefficients coef(c, b, a), held for the brick
  double cf[R + 1][R + 1][R + 1];
#pragma unroll
  for (int c = 0; c <= R; ++c)
#pragma unroll
    for (int b = 0; b <= (KJ ? c : R); ++b)
#pragma unroll
      for (int a = 0; a <= R; ++a) cf[c][b][a] = f64_coef(tp, sym_index(c, b, a, R));
  double *col = rt + (k0 + R) * SK + (j + R) * SJ;  // tile row of brick-local (k0, j), column 0
  // W_a of tile column ii for both rows, pushed into the window (newest at NW - 1)
  auto column = [&](const int ii) {
    double H[R + 1][2 * R + 2];  // H[b][q]: plane k0 - R + q
#pragma unroll
    for (int q = 0; q < 2 * R + 2; ++q) {
      const double *p = col + (q - R) * SK + ii;
      H[0][q] = p[0];
#pragma unroll
      for (int b = 1; b <= R; ++b) H[b][q] = f.add(p[-b * SJ], p[b * SJ]);
    }
    double Q[2][R + 1][R + 1];
#pragma unroll
    for (int o = 0; o < 2; ++o) {
#pragma unroll
      for (int b = 0; b <= R; ++b) {
        Q[o][0][b] = H[b][R + o];
#pragma unroll
        for (int c = 1; c <= R; ++c) Q[o][c][b] = f.add(H[b][R + o - c], H[b][R + o + c]);
      }
      if constexpr (KJ) {
#pragma unroll
        for (int c = 1; c <= R; ++c)
#pragma unroll
          for (int b = 0; b < c; ++b) Q[o][c][b] = f.add(Q[o][c][b], Q[o][b][c]);
      }
    }
    // W of both rows
#pragma unroll
    for (int a = 0; a <= R; ++a) {
      double w[2];
#pragma unroll
      for (int c = 0; c <= R; ++c)
#pragma unroll
        for (int b = 0; b <= (KJ ? c : R); ++b)
#pragma unroll
          for (int o = 0; o < 2; ++o)
            w[o] = (c == 0 && b == 0) ? f.mul(cf[0][0][a], Q[o][0][0]) : fma(cf[c][b][a], Q[o][c][b], w[o]);
#pragma unroll
      for (int o = 0; o < 2; ++o) {
#pragma unroll
        for (int m = 0; m + 1 < NW; ++m) W[o][a][m] = W[o][a][m + 1];
        W[o][a][NW - 1] = w[o];
      }
    }
  };
  if (!cont) {
#pragma unroll
    for (int ii = RP - R; ii < RP + R; ++ii) column(ii);
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    column(RP + R + i);  // the window now ends at column i + R: output i is complete
    __syncwarp();        // every lane is past column RP + i
#pragma unroll
    for (int o = 0; o < 2; ++o) {
      double v = W[o][0][R];
#pragma unroll
      for (int a = 1; a <= R; ++a) v = f.add(v, f.add(W[o][a][R - a], W[o][a][R + a]));
      col[o * SK + RP + i] = v;
    }
  }
  __syncwarp();
  // 64 outputs per store: lane l writes elements 2l, 2l + 1 of rows 8q .. 8q + 7
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int e = q * 64 + 2 * lane, k = e >> 6, jj = (e >> 3) & 7, i = e & 7;
    st_pair(ob + e, ld_pair(rt + (k + R) * SK + (jj + R) * SJ + RP + i));
  }
}

// ---------------------------------------------------------------------------------------
// Mirror-symmetric cubes on 4- and 2-byte storage in FP32 arithmetic, streamed along i: the
// class sums of sym_cube_istream, four tile columns per step.  A lane owns rows (k0, j) and
// (k0 + 1, j) of the brick as in the FP64 stream, and reads each of the 2R + 1 rows j - R ..
// j + R of the 2R + 2 planes it needs as one 16-byte (FP32) / 8-byte (BF16) load of four
// columns; all arithmetic runs on column pairs (i, i + 1) in packed FP32 (FADD2 / FFMA2):
//   H_b  = x(j - b) + x(j + b)                        per plane, shared by both rows
//   Q(c, b) = H_b(k - c) + H_b(k + c)                 per row; Q(c, b) += Q(b, c) under k <-> j
//   W_a  = sum over classes of coef(c, b, a) Q(c, b)  a = 0..R
//   out(i) = W_0(i) + sum over a of (W_a(i - a) + W_a(i + a))
// (per point 37 FP32 operations for the 125-point cube with k <-> j symmetry, in 19 packed
// instructions).  W of the columns already computed carry from one brick of a stream to the
// next (two 4-column groups), so a continued brick reads only its own eight columns.  Each W
// depends on one column only and the output sums run in a fixed order, so a brick's outputs
// are the same bits however it was reached.
// Compensated accumulation (ACCM_COMP): every W sum runs as Dot2 (the error of each product by
// FMA, of each addition by TwoSum, summed apart and added at the end) and the output sum is
// Neumaier-compensated with the W errors folded in; the remaining error is that of the
// additions in H and Q, about the error of the one-column compensated code.

__device__ __forceinline__ float2 neg2(float2 v) { return make_float2(-v.x, -v.y); }

// four consecutive tile elements as two column pairs
// (one 16-byte / 8-byte shared-memory load each: the address is 16 / 8-byte aligned by the
// tile layout, stated to the compiler by the vector load itself)
// (shared-memory byte address sa)
__device__ __forceinline__ void ld_quad(float *, unsigned sa, float2 &a, float2 &b) {
  float x, y, z, w;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];\n" : "=f"(x), "=f"(y), "=f"(z), "=f"(w) : "r"(sa));
  a = make_float2(x, y);
  b = make_float2(z, w);
}
__device__ __forceinline__ void ld_quad(__nv_bfloat16 *, unsigned sa, float2 &a, float2 &b) {
  unsigned ux, uy;
  asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];\n" : "=r"(ux), "=r"(uy) : "r"(sa));
  a = make_float2(__uint_as_float(ux << 16), __uint_as_float(ux & 0xFFFF0000u));
  b = make_float2(__uint_as_float(uy << 16), __uint_as_float(uy & 0xFFFF0000u));
}
// four consecutive parked outputs -> tile: one 16-byte (FP32) / 8-byte (BF16) shared store at
// shared-memory byte address sa (aligned by the tile layout)
__device__ __forceinline__ void sts_quad(float *, unsigned sa, const float (&v)[4]) {
  asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};\n" ::"r"(sa), "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3])
               : "memory");
}
__device__ __forceinline__ void sts_quad(__nv_bfloat16 *, unsigned sa, const float (&v)[4]) {
  const __nv_bfloat162 lo = __floats2bfloat162_rn(v[0], v[1]), hi = __floats2bfloat162_rn(v[2], v[3]);
  asm volatile("st.shared.v2.u32 [%0], {%1, %2};\n" ::"r"(sa), "r"(*reinterpret_cast<const unsigned *>(&lo)),
               "r"(*reinterpret_cast<const unsigned *>(&hi))
               : "memory");
}
// four parked outputs (tile) -> global memory: one 16-byte (FP32) / 8-byte (BF16) store
__device__ __forceinline__ void st_quad(float *g, const float *t) {
  __stcs(reinterpret_cast<float4 *>(g), *reinterpret_cast<const float4 *>(t));
}
__device__ __forceinline__ void st_quad(__nv_bfloat16 *g, const __nv_bfloat16 *t) {
  __stcs(reinterpret_cast<uint2 *>(g), *reinterpret_cast<const uint2 *>(t));
}

// W of the current and previous 4-column groups of a stream, per row o, a = 0..R and column
// pair; with the Dot2 error terms of each W under compensated accumulation.
template <int R, bool COMP, int NO>
struct CsWin {
  float2 p[NO][R + 1][2], c[NO][R + 1][2];
  float2 ep[COMP ? NO : 1][R + 1][2], ec[COMP ? NO : 1][R + 1][2];
};

// W_a (and errors) of the four tile columns c0 .. c0 + 3 for the NO rows (k0 .. k0 + NO - 1, j)
// of this thread.  base: tile row j of plane k0 (brick-local (k0 - R, j - R)); rows j .. j + 2R
// are read.
template <typename C, typename T, int R, bool KJ, bool COMP, int NO>
__device__ __forceinline__ void cs_group(const T *base, const int j, const int c0, const Taps &tp,
                                         float2 (&W)[NO][R + 1][2], float2 (&E)[COMP ? NO : 1][R + 1][2]) {
  constexpr int SK = C::EJ * C::EI, SJ = C::EI;
  float2 Q[NO][R + 1][R + 1][2];  // [o][c][b][pair]
  const unsigned sb = smem_u32(base);
#pragma unroll
  for (int q = 0; q < 2 * R + NO; ++q) {  // tile plane k0 + q: brick-local plane k0 - R + q
    float2 v[2 * R + 1][2];
#pragma unroll
    for (int rr = 0; rr <= 2 * R; ++rr)
      ld_quad((T *)nullptr, sb + (unsigned)((q * SK + rr * SJ + C::col(j + rr, c0)) * (int)sizeof(T)), v[rr][0],
              v[rr][1]);
    float2 H[R + 1][2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      H[0][h] = v[R][h];
#pragma unroll
      for (int b = 1; b <= R; ++b) H[b][h] = __fadd2_rn(v[R - b][h], v[R + b][h]);
    }
#pragma unroll
    for (int o = 0; o < NO; ++o) {
      const int dk = q - R - o;  // offset of this plane from row k0 + o
      if (dk < -R || dk > R) continue;
      const int c = dk < 0 ? -dk : dk;
#pragma unroll
      for (int b = 0; b <= R; ++b)
#pragma unroll
        for (int h = 0; h < 2; ++h)
          Q[o][c][b][h] = dk == -c ? H[b][h] : __fadd2_rn(Q[o][c][b][h], H[b][h]);
    }
  }
#pragma unroll
  for (int o = 0; o < NO; ++o) {
    if constexpr (KJ) {
#pragma unroll
      for (int c = 1; c <= R; ++c)
#pragma unroll
        for (int b = 0; b < c; ++b)
#pragma unroll
          for (int h = 0; h < 2; ++h) Q[o][c][b][h] = __fadd2_rn(Q[o][c][b][h], Q[o][b][c][h]);
    }
#pragma unroll
    for (int a = 0; a <= R; ++a)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float2 w = make_float2(0.f, 0.f), e = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c <= R; ++c)
#pragma unroll
          for (int b = 0; b <= (KJ ? c : R); ++b) {
            const float2 cf = tp.sp[(c * (R + 1) + b) * (R + 1) + a];
            const float2 x = Q[o][c][b][h];
            if constexpr (!COMP) {
              w = (c == 0 && b == 0) ? __fmul2_rn(cf, x) : __ffma2_rn(cf, x, w);
            } else {
              const float2 pr = __fmul2_rn(cf, x);
              const float2 pe = __ffma2_rn(cf, x, neg2(pr));  // the product's rounding error, exact
              if (c == 0 && b == 0) {
                w = pr;
                e = pe;
              } else {  // TwoSum(w, pr): sm + ew == w + pr exactly
                const float2 sm = __fadd2_rn(w, pr);
                const float2 bb = __fadd2_rn(sm, neg2(w));
                const float2 ew = __fadd2_rn(__fadd2_rn(w, neg2(__fadd2_rn(sm, neg2(bb)))), __fadd2_rn(pr, neg2(bb)));
                e = __fadd2_rn(e, __fadd2_rn(ew, pe));
                w = sm;
              }
            }
          }
        W[o][a][h] = w;
        if constexpr (COMP) E[o][a][h] = e;
      }
  }
}

// W_a (or its error) at column rel of the current group (rel in [-4, 8): previous, current,
// next group), for row o.
template <int R, int NO>
__device__ __forceinline__ float cs_at(const float2 (&P)[NO][R + 1][2], const float2 (&Cc)[NO][R + 1][2],
                                       const float2 (&N)[NO][R + 1][2], int o, int a, int rel) {
  const float2 (*g)[R + 1][2] = rel < 0 ? P : rel < 4 ? Cc : N;
  const int m = (rel + 4) & 3;
  const float2 v = g[o][a][m >> 1];
  return (m & 1) ? v.y : v.x;
}

// Outputs of the current group's four columns c0 .. c0 + 3 for the thread's NO rows, parked in
// the tile at their own input positions (park: tile row prow = j + R of plane k0 + R), one
// vector store per row (the four columns are one 16-byte unit of the row, also under the FP32
// swizzle; the eight lanes of a quarter warp hit distinct banks).
template <typename C, typename T, int R, bool COMP, int NO>
__device__ __forceinline__ void cs_out(T *park, const int prow, const int c0, const CsWin<R, COMP, NO> &S,
                                       const float2 (&Wn)[NO][R + 1][2], const float2 (&En)[COMP ? NO : 1][R + 1][2]) {
  constexpr int SK = C::EJ * C::EI;
  static_assert(C::SWZ || C::EI % 4 == 0, "four parked columns stay in one aligned unit");
  const unsigned pb = smem_u32(park + C::col(prow, c0));
#pragma unroll
  for (int o = 0; o < NO; ++o) {
    float q[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      float v;
      if constexpr (!COMP) {
        v = cs_at<R, NO>(S.p, S.c, Wn, o, 0, t);
#pragma unroll
        for (int a = 1; a <= R; ++a) v += cs_at<R, NO>(S.p, S.c, Wn, o, a, t - a) + cs_at<R, NO>(S.p, S.c, Wn, o, a, t + a);
      } else {
        float sm = cs_at<R, NO>(S.p, S.c, Wn, o, 0, t), cm = 0.f;
        float es = cs_at<R, NO>(S.ep, S.ec, En, o, 0, t);
#pragma unroll
        for (int a = 1; a <= R; ++a) {
          neumaier(sm, cm, cs_at<R, NO>(S.p, S.c, Wn, o, a, t - a));
          neumaier(sm, cm, cs_at<R, NO>(S.p, S.c, Wn, o, a, t + a));
          es += cs_at<R, NO>(S.ep, S.ec, En, o, a, t - a) + cs_at<R, NO>(S.ep, S.ec, En, o, a, t + a);
        }
        v = sm + (cm + es);
      }
      q[t] = v;
    }
    sts_quad((T *)nullptr, pb + (unsigned)(o * SK * (int)sizeof(T)), q);
  }
}

template <int R, bool COMP, int NO>
__device__ __forceinline__ void cs_shift(CsWin<R, COMP, NO> &S, const float2 (&Wn)[NO][R + 1][2],
                                         const float2 (&En)[COMP ? NO : 1][R + 1][2]) {
#pragma unroll
  for (int o = 0; o < NO; ++o)
#pragma unroll
    for (int a = 0; a <= R; ++a)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        S.p[o][a][h] = S.c[o][a][h];
        S.c[o][a][h] = Wn[o][a][h];
        if constexpr (COMP) {
          S.ep[o][a][h] = S.ec[o][a][h];
          S.ec[o][a][h] = En[o][a][h];
        }
      }
}

// One brick of the stream: its eight output columns (groups at tile columns RP and RP + 4), the
// W of groups RP - 4 and RP computed here unless the stream continues (cont), then the brick
// leaves in whole-warp stores (16 / 8 bytes per lane) when the output brick is aligned for them.
// A thread (lane of the brick's TPB threads) owns rows (k0 .. k0 + NO - 1, j); with two warps per
// brick the syncs around the parking are block barriers.
template <typename C, typename T, int R, bool KJ, bool COMP>
__device__ __forceinline__ void sym_cube_istream4(T *rt, T *ob, const int lane, const Taps &tp,
                                                  CsWin<R, COMP, C::CSROWS> &S, const bool cont) {
  constexpr int SK = C::EJ * C::EI, SJ = C::EI, RP = C::RP, NO = C::CSROWS, TPB = C::TPB;
  static_assert(R == 1 || R == 2, "cube radius");
  static_assert(RP >= 4 && C::NEED >= RP + 12, "the four column groups of a brick fit the tile row");
  static_assert(TPB * NO == 64 && (TPB == 32 || TPB == 64), "the brick's 64 rows over its threads");
  auto sync = [] {
    if constexpr (TPB == 32) __syncwarp();
    else __syncthreads();
  };
  const int k0 = NO * (lane >> 3), j = lane & 7;
  const T *base = rt + k0 * SK + j * SJ;
  T *park = rt + (k0 + R) * SK + (j + R) * SJ;
  float2 Wn[NO][R + 1][2], En[COMP ? NO : 1][R + 1][2];
  if (!cont) {
    cs_group<C, T, R, KJ, COMP, NO>(base, j, RP - 4, tp, S.p, S.ep);
    cs_group<C, T, R, KJ, COMP, NO>(base, j, RP, tp, S.c, S.ec);
  }
  cs_group<C, T, R, KJ, COMP, NO>(base, j, RP + 4, tp, Wn, En);
  sync();  // every thread is past its reads of columns RP .. RP + 7
  cs_out<C, T, R, COMP, NO>(park, j + R, RP, S, Wn, En);
  cs_shift<R, COMP, NO>(S, Wn, En);
  cs_group<C, T, R, KJ, COMP, NO>(base, j, RP + 8, tp, Wn, En);  // the i-hi columns: never parked over
  cs_out<C, T, R, COMP, NO>(park, j + R, RP + 4, S, Wn, En);
  cs_shift<R, COMP, NO>(S, Wn, En);
  sync();  // the parked outputs of every thread are in the tile
  constexpr int AL = 4 * (int)sizeof(T);
  if ((reinterpret_cast<uintptr_t>(ob) & (AL - 1)) == 0) {
#pragma unroll
    for (int q = 0; q < 512 / (4 * TPB); ++q) {
      const int e = q * 4 * TPB + 4 * lane, k = e >> 6, jj = (e >> 3) & 7, i = e & 7;
      st_quad(ob + e, rt + (k + R) * SK + (jj + R) * SJ + C::col(jj + R, RP + i));
    }
  } else {
#pragma unroll
    for (int q = 0; q < 512 / TPB; ++q) {
      const int e = q * TPB + lane, k = e >> 6, jj = (e >> 3) & 7, i = e & 7;
      ob[e] = rt[(k + R) * SK + (jj + R) * SJ + C::col(jj + R, RP + i)];
    }
  }
}

// One brick's outputs from its staged tile (the compute of sweep2_kernel): each of the BJ*BI
// threads (lt) owns one (j, i) column, or, for the column-pair cubes, each of the BJ*BI/2
// threads a pair of columns.
// out_brick: the output field's brick (field base + centre brick x step).
// cs: the native FP64 register-operand block (F64Ops) in shared memory (stars and cubes).
template <typename T, int BK, int BJ, int BI, int R, int FAM, int ACC>
__device__ __forceinline__ void sweep2_brick(const T *rt, T *out_brick, int lt, const Taps &tp, const double *cs) {
  typedef Sweep2Cfg<T, BK, BJ, BI, R, FAM, ACC> C;
  typedef typename Elem<T>::acc AT;
  constexpr int EJ = C::EJ, EI = C::EI, SK = EJ * EI, SJ = EI, RP = C::RP;
  if constexpr (C::PAIR) {
    // lane -> (row, column pair); 16-byte pairs: rows 0,2,1,3 per quarter warp, two rows apart
    const int q = lt >> 2, i0 = 2 * (lt & 3);
    const int jp = C::PERM ? (q & 4) | ((q & 1) << 1) | ((q >> 1) & 1) : q;
    if constexpr (C::ES == 8)
      sym_cube_pair_shared<C, T, R, FAM == FAM_CUBESYM_IJ>(rt, out_brick + (size_t)(jp * BI + i0), jp, i0, tp);
    else
      cube_pair_columns<C, T, R, FAM>(rt, out_brick + (size_t)(jp * BI + i0), jp, i0, tp);
    return;
  }
  int j = lt / BI;
  const int i = lt - j * BI;
  if (C::PERM) j = (j & ~3) | ((j & 1) << 1) | ((j >> 1) & 1);  // rows 0,2,1,3 per warp
  T *ob = out_brick + (size_t)(j * BI + i);
  const int cofs = (j + R) * SJ + (i + RP);  // column (j, i) at kk = 0
  if constexpr (ACC == ACCM_FF) {
    const float2 *ft = reinterpret_cast<const float2 *>(rt);
    if constexpr (FAM == FAM_STAR) {
      float2 w[BK + 2 * R];
#pragma unroll
      for (int kk = 0; kk < BK + 2 * R; ++kk) w[kk] = ft[kk * SK + cofs];
#pragma unroll
      for (int k = 0; k < BK; ++k) {
        const float2 *c = ft + (k + R) * SK + cofs;
        FFAcc acc;
        acc.first(tp.cf[0], tp.cl[0], w[k + R]);
#pragma unroll
        for (int d = 1; d <= R; ++d) {
          const int t = 1 + 6 * (d - 1);
          acc.add(tp.cf[t + 0], tp.cl[t + 0], c[d]);
          acc.add(tp.cf[t + 1], tp.cl[t + 1], c[-d]);
          acc.add(tp.cf[t + 2], tp.cl[t + 2], c[d * SJ]);
          acc.add(tp.cf[t + 3], tp.cl[t + 3], c[-d * SJ]);
          acc.add(tp.cf[t + 4], tp.cl[t + 4], w[k + R + d]);
          acc.add(tp.cf[t + 5], tp.cl[t + 5], w[k + R - d]);
          acc.renorm();
        }
        store_stream(ob + k * BJ * BI, acc.result());
      }
    } else if constexpr (FAM == FAM_CUBE) {
      FFAcc acc[BK];
#pragma unroll
      for (int dj = -R; dj <= R; ++dj)
#pragma unroll
        for (int di = -R; di <= R; ++di) {
          float2 w[BK + 2 * R];
#pragma unroll
          for (int kk = 0; kk < BK + 2 * R; ++kk) w[kk] = ft[kk * SK + cofs + dj * SJ + di];
#pragma unroll
          for (int k = 0; k < BK; ++k) {
#pragma unroll
            for (int dk = -R; dk <= R; ++dk) {
              const int t = ((dk + R) * (2 * R + 1) + (dj + R)) * (2 * R + 1) + (di + R);
              if (dj == -R && di == -R && dk == -R) acc[k].first(tp.cf[t], tp.cl[t], w[k + R + dk]);
              else acc[k].add(tp.cf[t], tp.cl[t], w[k + R + dk]);
            }
            acc[k].renorm();
          }
        }
#pragma unroll
      for (int k = 0; k < BK; ++k) store_stream(ob + k * BJ * BI, acc[k].result());
    } else if constexpr (FAM == FAM_CUBESYM || FAM == FAM_CUBESYM_IJ) {
      // mirror-symmetric cube in float-float: the pair-sum evaluation of the native path below
      // with float-float additions and Dot2 products
      constexpr bool IJ = FAM == FAM_CUBESYM_IJ;
      FFAcc acc[BK];
      auto ring = [&](const float2 *c, int b, int a) -> float2 {
        if (a == 0 && b == 0) return c[0];
        if (b == 0) return ff_add(c[-a], c[a]);
        if (a == 0) return ff_add(c[-b * SJ], c[b * SJ]);
        return ff_add(ff_add(c[-b * SJ - a], c[-b * SJ + a]), ff_add(c[b * SJ - a], c[b * SJ + a]));
      };
#pragma unroll
      for (int b = 0; b <= R; ++b)
#pragma unroll
        for (int a = 0; a <= (IJ ? b : R); ++a) {
          float2 q[BK + 2 * R];
#pragma unroll
          for (int kk = 0; kk < BK + 2 * R; ++kk) {
            const float2 *c = ft + kk * SK + cofs;
            q[kk] = (IJ && a != b) ? ff_add(ring(c, b, a), ring(c, a, b)) : ring(c, b, a);
          }
#pragma unroll
          for (int k = 0; k < BK; ++k) {
            const int t0 = sym_index(0, b, a, R);
            if (a == 0 && b == 0) acc[k].first(tp.cf[t0], tp.cl[t0], q[k + R]);
            else acc[k].add(tp.cf[t0], tp.cl[t0], q[k + R]);
#pragma unroll
            for (int d = 1; d <= R; ++d) {
              const int t = sym_index(d, b, a, R);
              acc[k].add(tp.cf[t], tp.cl[t], ff_add(q[k + R - d], q[k + R + d]));
            }
            acc[k].renorm();
          }
        }
#pragma unroll
      for (int k = 0; k < BK; ++k) store_stream(ob + k * BJ * BI, acc[k].result());
    } else {
#pragma unroll 1
      for (int k = 0; k < BK; ++k) {
        const float2 *c = ft + (k + R) * SK + cofs;
        FFAcc acc;
        acc.first(tp.cf[0], tp.cl[0], c[tp.toff[0]]);
        for (int t = 1; t < tp.n; ++t) {
          acc.add(tp.cf[t], tp.cl[t], c[tp.toff[t]]);
          if ((t & 7) == 7) acc.renorm();
        }
        store_stream(ob + k * BJ * BI, acc.result());
      }
    }
  } else if constexpr (C::F64S && FAM == FAM_STAR) {
    // the per-point operations of the star below, taps outer over the column's points, on
    // register operands (F64Ops), every multiply-add with its value freshly loaded
    const F64Ops f = F64Ops::load(cs);
    double cr[1 + 6 * R];
#pragma unroll
    for (int t = 0; t < 1 + 6 * R; ++t) cr[t] = cs[F64Ops::NHEAD + t];
    const double *c0 = reinterpret_cast<const double *>(rt) + R * SK + cofs;  // point k at c0[k * SK]
    double acc[BK];
#pragma unroll
    for (int k = 0; k < BK; ++k) acc[k] = f.mul(cr[0], c0[k * SK]);
#pragma unroll
    for (int d = 1; d <= R; ++d) {
      const int t = 1 + 6 * (d - 1);
      const int off[6] = {d, -d, d * SJ, -d * SJ, d * SK, -d * SK};
#pragma unroll
      for (int q = 0; q < 6; ++q)
#pragma unroll
        for (int k = 0; k < BK; ++k) acc[k] = fma(cr[t + q], c0[k * SK + off[q]], acc[k]);
    }
#pragma unroll
    for (int k = 0; k < BK; ++k) store_stream(reinterpret_cast<double *>(ob) + k * BJ * BI, acc[k]);
  } else if constexpr (C::F64S && FAM == FAM_CUBE) {
    // the per-point operations of the cube below ((dj, di) outer, dk inner), taps outer over the
    // column's points, on register operands (F64Ops), every multiply-add with its value freshly
    // loaded
    const F64Ops f = F64Ops::load(cs);
    const double *c0 = reinterpret_cast<const double *>(rt) + cofs;  // plane kk at c0[kk * SK]
    double acc[BK];
#pragma unroll
    for (int dj = -R; dj <= R; ++dj)
#pragma unroll
      for (int di = -R; di <= R; ++di)
#pragma unroll
        for (int dk = -R; dk <= R; ++dk) {
          const int t = ((dk + R) * (2 * R + 1) + (dj + R)) * (2 * R + 1) + (di + R);
          const double cf = cs[F64Ops::NHEAD + t];
#pragma unroll
          for (int k = 0; k < BK; ++k) {
            const double x = c0[(k + R + dk) * SK + dj * SJ + di];
            acc[k] = (dj == -R && di == -R && dk == -R) ? f.mul(cf, x) : fma(cf, x, acc[k]);
          }
        }
#pragma unroll
    for (int k = 0; k < BK; ++k) store_stream(reinterpret_cast<double *>(ob) + k * BJ * BI, acc[k]);
  } else {
    if constexpr (FAM == FAM_STAR) {
      AT w[BK + 2 * R];
#pragma unroll
      for (int kk = 0; kk < BK + 2 * R; ++kk) w[kk] = to_acc(rt[kk * SK + cofs]);
#pragma unroll
      for (int k = 0; k < BK; ++k) {
        const T *c = rt + (k + R) * SK + cofs;
        AT v;
        if constexpr (ACC == ACCM_NATIVE) {
          v = coef<AT>(tp, 0) * w[k + R];
#pragma unroll
          for (int d = 1; d <= R; ++d) {
            const int t = 1 + 6 * (d - 1);
            v = fma(coef<AT>(tp, t + 0), to_acc(c[d]), v);
            v = fma(coef<AT>(tp, t + 1), to_acc(c[-d]), v);
            v = fma(coef<AT>(tp, t + 2), to_acc(c[d * SJ]), v);
            v = fma(coef<AT>(tp, t + 3), to_acc(c[-d * SJ]), v);
            v = fma(coef<AT>(tp, t + 4), w[k + R + d], v);
            v = fma(coef<AT>(tp, t + 5), w[k + R - d], v);
          }
        } else {
          AT row = coef<AT>(tp, 0) * w[k + R];
#pragma unroll
          for (int d = 1; d <= R; ++d) {
            const int t = 1 + 6 * (d - 1);
            row = fma(coef<AT>(tp, t + 0), to_acc(c[d]), row);
            row = fma(coef<AT>(tp, t + 1), to_acc(c[-d]), row);
          }
          AT s = row, comp = AT(0);
#pragma unroll
          for (int d = 1; d <= R; ++d) {
            const int t = 1 + 6 * (d - 1);
            neumaier(s, comp, coef<AT>(tp, t + 2) * to_acc(c[d * SJ]));
            neumaier(s, comp, coef<AT>(tp, t + 3) * to_acc(c[-d * SJ]));
            neumaier(s, comp, coef<AT>(tp, t + 4) * w[k + R + d]);
            neumaier(s, comp, coef<AT>(tp, t + 5) * w[k + R - d]);
          }
          v = s + comp;
        }
        store_stream(ob + k * BJ * BI, v);
      }
    } else if constexpr (FAM == FAM_CUBESYM || FAM == FAM_CUBESYM_IJ) {
      // Mirror-symmetric cube: for every (b, a) = (|dj|, |di|) the column
      //   q[kk] = sum of x(kk, j +- b, i +- a) over the distinct sign choices
      // is formed with additions, then
      //   out(k) += c(0,b,a) q[k] + sum_{c>=1} c(c,b,a) (q[k-c] + q[k+c]).
      // Per point: 69 instead of 125 floating-point operations for R = 2 (27 multiply-adds,
      // 42 additions), 18 instead of 27 for R = 1.  With the i <-> j swap symmetry the
      // columns of (b, a) and (a, b) share their coefficients and are added first: 58.5
      // operations for R = 2.
      static_assert(ACC == ACCM_NATIVE, "symmetric cubes: native arithmetic");
      constexpr bool IJ = FAM == FAM_CUBESYM_IJ;
      AT acc[BK];
      // sum of x(kk, j +- b, i +- a) over the distinct sign choices
      auto ring = [&](const T *c, int b, int a) -> AT {
        if (a == 0 && b == 0) return to_acc(c[0]);
        if (b == 0) return to_acc(c[-a]) + to_acc(c[a]);
        if (a == 0) return to_acc(c[-b * SJ]) + to_acc(c[b * SJ]);
        return (to_acc(c[-b * SJ - a]) + to_acc(c[-b * SJ + a])) + (to_acc(c[b * SJ - a]) + to_acc(c[b * SJ + a]));
      };
#pragma unroll
      for (int b = 0; b <= R; ++b)
#pragma unroll
        for (int a = 0; a <= (IJ ? b : R); ++a) {
          AT q[BK + 2 * R];
#pragma unroll
          for (int kk = 0; kk < BK + 2 * R; ++kk) {
            const T *c = rt + kk * SK + cofs;
            q[kk] = (IJ && a != b) ? ring(c, b, a) + ring(c, a, b) : ring(c, b, a);
          }
#pragma unroll
          for (int k = 0; k < BK; ++k) {
            const AT c0 = coef<AT>(tp, sym_index(0, b, a, R));
            if (a == 0 && b == 0) acc[k] = c0 * q[k + R];
            else acc[k] = fma(c0, q[k + R], acc[k]);
#pragma unroll
            for (int d = 1; d <= R; ++d)
              acc[k] = fma(coef<AT>(tp, sym_index(d, b, a, R)), q[k + R - d] + q[k + R + d], acc[k]);
          }
        }
#pragma unroll
      for (int k = 0; k < BK; ++k) store_stream(ob + k * BJ * BI, acc[k]);
    } else if constexpr (FAM == FAM_CUBE) {
      AT acc[BK], comp[BK];
#pragma unroll
      for (int dj = -R; dj <= R; ++dj)
#pragma unroll
        for (int di = -R; di <= R; ++di) {
          AT w[BK + 2 * R];
#pragma unroll
          for (int kk = 0; kk < BK + 2 * R; ++kk) w[kk] = to_acc(rt[kk * SK + cofs + dj * SJ + di]);
#pragma unroll
          for (int k = 0; k < BK; ++k) {
            if constexpr (ACC == ACCM_NATIVE) {
#pragma unroll
              for (int dk = -R; dk <= R; ++dk) {
                const int t = ((dk + R) * (2 * R + 1) + (dj + R)) * (2 * R + 1) + (di + R);
                if (dj == -R && di == -R && dk == -R) acc[k] = coef<AT>(tp, t) * w[k + R + dk];
                else acc[k] = fma(coef<AT>(tp, t), w[k + R + dk], acc[k]);
              }
            } else {
              // the 2R+1 k taps of this column as one FMA chain, columns Neumaier-summed
              const int t0 = ((0) * (2 * R + 1) + (dj + R)) * (2 * R + 1) + (di + R);
              AT col = coef<AT>(tp, t0) * w[k];
#pragma unroll
              for (int dk = -R + 1; dk <= R; ++dk) {
                const int t = ((dk + R) * (2 * R + 1) + (dj + R)) * (2 * R + 1) + (di + R);
                col = fma(coef<AT>(tp, t), w[k + R + dk], col);
              }
              if (dj == -R && di == -R) {
                acc[k] = col;
                comp[k] = AT(0);
              } else {
                neumaier(acc[k], comp[k], col);
              }
            }
          }
        }
#pragma unroll
      for (int k = 0; k < BK; ++k) {
        if constexpr (ACC == ACCM_NATIVE) store_stream(ob + k * BJ * BI, acc[k]);
        else store_stream(ob + k * BJ * BI, acc[k] + comp[k]);
      }
    } else {
#pragma unroll 1
      for (int k = 0; k < BK; ++k) {
        const T *c = rt + (k + R) * SK + cofs;
        AT v;
        if constexpr (ACC == ACCM_NATIVE) {
          v = coef<AT>(tp, 0) * to_acc(c[tp.toff[0]]);
          for (int t = 1; t < tp.n; ++t) v = fma(coef<AT>(tp, t), to_acc(c[tp.toff[t]]), v);
        } else {
          AT s = coef<AT>(tp, 0) * to_acc(c[tp.toff[0]]), comp = AT(0);
          for (int t = 1; t < tp.n; ++t) neumaier(s, comp, coef<AT>(tp, t) * to_acc(c[tp.toff[t]]));
          v = s + comp;
        }
        store_stream(ob + k * BJ * BI, v);
      }
    }
  }
}

// IST: FP64 mirror-symmetric cubes streamed along i (sym_cube_istream): each CTA takes a
// contiguous share of the list instead of every gridDim.x-th group.
template <typename T, int BK, int BJ, int BI, int R, int FAM, int ACC, bool BATCH, bool IST>
__global__ void __launch_bounds__(Sweep2Cfg<T, BK, BJ, BI, R, FAM, ACC, IST>::NT,
                                  Sweep2Cfg<T, BK, BJ, BI, R, FAM, ACC, IST>::MINB)
sweep2_kernel(const SweepArgs a, const Taps tp) {
  typedef Sweep2Cfg<T, BK, BJ, BI, R, FAM, ACC, IST> C;
  constexpr int TPB = C::TPB, NB = C::NB, EPT = C::EPT;
  static_assert(!IST || (C::ES == 8 && C::PAIR && NB == 1 && (FAM == FAM_CUBESYM || FAM == FAM_CUBESYM_IJ)) ||
                    (C::ES <= 4 && C::CS4 && NB == 1 && FAM == FAM_CUBESYM && ACC != ACCM_FF),
                "class-sum streams: mirror-symmetric cubes, FP64 (native) or FP32 / BF16 storage, one brick per CTA");
  // streams run along the list, plain or batch mode (in batch mode a stream continues only
  // within one domain's field)
  constexpr bool STREAM = IST;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char *raw0 = smem_raw;                               // [NB] tiles, buffer 0
  unsigned char *raw1 = smem_raw + NB * C::TILE_BYTES;          // [NB] tiles, buffer 1
  unsigned *nbrs = reinterpret_cast<unsigned *>(smem_raw + 2 * NB * C::TILE_BYTES + NB * C::FTILE_BYTES);
  // nbrs slot (36 words): [0..26] adjacency, [27] active, [28..29] input field base,
  // [30..31] output field base, [32..33] / [34..35] input / output storage step (elements)
  // nbrs: [3][NB][28]: adjacency of the groups being computed, copied and staged
  // (three slots, so staging the group after next never overwrites one still read);
  // entry [27] is the brick's active flag

  const int slot = threadIdx.x / TPB, lt = threadIdx.x - slot * TPB;
  unsigned plan[EPT];
#pragma unroll
  for (int e = 0; e < EPT; ++e) {
    const int g = e * TPB + lt;
    plan[e] = g < C::NV ? plan_entry<C, BK, BJ, BI, R, FAM, IST>(g) : 0xFFFFFFFFu;
  }

  const long long ngroups = ((long long)a.nlist + NB - 1) / NB;
  // This CTA's groups.  Plain: every gridDim.x-th.  Streams of 4- / 2-byte storage: chunks of
  // CH consecutive groups, chunk c to CTA c mod gridDim.x, so that at any time the CTAs work on
  // neighbouring stretches of the list in step -- the j and k neighbours a brick's tile reads
  // were just read by the CTAs on the neighbouring rows and are still in L2 (with a contiguous
  // share per CTA they came many bricks apart in time, and the kernel read 2.6 times its
  // algorithmic bytes from DRAM); CH is about 16, chosen so the chunks fill whole rounds.
  // FP64 streams, bound by the FP64 pipe, keep one contiguous share per CTA (fewer stream
  // restarts, each of which computes 2R more columns).
  constexpr bool CHUNKED = STREAM && C::ES <= 4;
  const long long G = gridDim.x;
  long long CH = 1;
  if constexpr (CHUNKED) {
    const long long rounds = (ngroups + G * BK_CS_CHUNK - 1) / (G * BK_CS_CHUNK);
    CH = (ngroups + G * rounds - 1) / (G * rounds);
    if (CH < 1) CH = 1;
  }
  // a position in this CTA's walk: the group and, chunked, its place in its chunk
  struct Walk {
    long long g;
    long long pos;
  };
  auto advance = [&](Walk w) -> Walk {
    if constexpr (CHUNKED) return w.pos + 1 < CH ? Walk{w.g + 1, w.pos + 1} : Walk{w.g + 1 + (G - 1) * CH, 0};
    else if constexpr (STREAM) return Walk{w.g + 1, 0};
    else return Walk{w.g + G, 0};
  };
  const long long g0 = CHUNKED ? (long long)blockIdx.x * CH
                       : STREAM ? (long long)blockIdx.x * ngroups / G : (long long)blockIdx.x;
  const long long gend = STREAM && !CHUNKED ? ((long long)blockIdx.x + 1) * ngroups / G : ngroups;

  // Adjacency of a group: fetched into registers two groups ahead (its global-load latency
  // hides under the current group's compute), stored into one of three nbrs slots.
  constexpr int APT = (27 + TPB - 1) / TPB;  // adjacency entries per thread
  unsigned av[APT];
  int aok[APT];
  unsigned long long fin = 0, fout = 0, fsin = 0, fsout = 0;  // held by the thread of slot 13
  auto fetch_adj = [&](long long grp) {
    const long long n = grp * NB + slot;
#pragma unroll
    for (int q = 0; q < APT; ++q) {
      const int sl = lt + q * TPB;
      unsigned v = 0;
      int ok = 0;
      if (sl < 27 && grp < gend && n < a.nlist) {
        const unsigned *adj;
        unsigned b, nbricks;
        long long in_chunks, out_chunks;
        if constexpr (BATCH) {
          const uint2 w = a.work[n];
          const bool dok = w.x < a.ndom;
          const BatchDomain &D = a.doms[dok ? w.x : 0];
          adj = D.adj;
          b = dok ? w.y : 0xFFFFFFFFu;
          nbricks = D.nbricks;
          in_chunks = out_chunks = D.chunks;
          if (sl == 13) {
            fin = reinterpret_cast<unsigned long long>(a.parity ? D.f1 : D.f0);
            fout = reinterpret_cast<unsigned long long>(a.parity ? D.f0 : D.f1);
            fsin = fsout = D.step_bytes / sizeof(T);
          }
        } else {
          adj = a.adj;
          b = a.blist[n];
          nbricks = a.nbricks;
          in_chunks = a.in_chunks;
          out_chunks = a.out_chunks;
          if (sl == 13) {
            fin = reinterpret_cast<unsigned long long>(reinterpret_cast<const T *>(a.in) + a.in_off);
            fout = reinterpret_cast<unsigned long long>(reinterpret_cast<T *>(a.out) + a.out_off);
            fsin = a.in_step;
            fsout = a.out_step;
          }
        }
        if (b < nbricks) {
          v = adj[(size_t)b * 27 + sl];
          ok = 1;
          if (sl == 13 && ((long long)v >= out_chunks || (long long)v >= in_chunks)) ok = 0;
          if ((long long)v >= in_chunks || !ok) { atomicOr(a.err, FLAG_BOUNDS); v = 0; }
        } else if (sl == 13) {
          atomicOr(a.err, FLAG_BOUNDS);
        }
      }
      av[q] = v;
      aok[q] = ok;
    }
  };
  auto store_adj = [&](int ns) {
    unsigned *nbr = nbrs + (ns * NB + slot) * 36;
#pragma unroll
    for (int q = 0; q < APT; ++q) {
      const int sl = lt + q * TPB;
      if (sl < 27) {
        nbr[sl] = av[q];
        if (sl == 13) {
          nbr[27] = aok[q];
          *reinterpret_cast<unsigned long long *>(nbr + 28) = fin;
          *reinterpret_cast<unsigned long long *>(nbr + 30) = fout;
          *reinterpret_cast<unsigned long long *>(nbr + 32) = fsin;
          *reinterpret_cast<unsigned long long *>(nbr + 34) = fsout;
        }
      }
    }
  };
  // issue the asynchronous gather of the group staged in nbrs[ns] into raw buffer buf
  // Whether the stream continues from the group whose adjacency is in nbrs[prev] into the group
  // in nbrs[ns]: both ran, and the latter's i-lo and centre columns of neighbours are the
  // former's centre and i-hi columns (lanes 0..17 of every warp check one slot pair each, so
  // all warps of a brick reach the same answer).
  auto continues = [&](int prev, int ns) -> bool {
    const unsigned *nb = nbrs + ns * 36, *pv = nbrs + prev * 36;
    bool same = true;
    const int wl = lt & 31;
    if (wl < 18) {
      const int s9 = wl < 9 ? wl : wl - 9, sh = wl < 9 ? 0 : 1;
      const int base = (s9 / 3) * 9 + (s9 % 3) * 3;  // (dk, dj) = (s9 / 3 - 1, s9 % 3 - 1), di = -1
      same = nb[base + sh] == pv[base + sh + 1];
    }
    // the same input field: in batch mode consecutive items may belong to different domains
    same = same && *reinterpret_cast<const unsigned long long *>(nb + 28) ==
                       *reinterpret_cast<const unsigned long long *>(pv + 28);
    return __all_sync(0xFFFFFFFFu, same) && pv[27] != 0 && nb[27] != 0;
  };
  // issue the asynchronous gather of the group staged in nbrs[ns] into raw buffer buf; a
  // continued stream reads only the tile columns from ICUT on (the W of the columns before
  // come from the previous brick), so copies wholly before ICUT are skipped
  // plan entries a continued brick issues: those of the first NVN copies (warp-uniform bound)
  constexpr int EPTN = STREAM ? (StreamPlan<C, R>::NVN + TPB - 1) / TPB : EPT;
  auto issue = [&](int buf, int ns, bool cont) {
    const unsigned *nbr = nbrs + (ns * NB + slot) * 36;
    if (nbr[27]) {
      unsigned char *tile = (buf ? raw1 : raw0) + slot * C::TILE_BYTES;
      const unsigned tbase = smem_u32(tile);
      const T *in = reinterpret_cast<const T *>(*reinterpret_cast<const unsigned long long *>(nbr + 28));
      const size_t step = *reinterpret_cast<const unsigned long long *>(nbr + 32);
      const int ne = STREAM && cont ? EPTN : EPT;
#pragma unroll
      for (int e = 0; e < EPT; ++e) {
        const unsigned p = plan[e];
        const bool need = !(STREAM && cont) || e * TPB + lt < StreamPlan<C, R>::NVN;
        if (e < ne && need && p != 0xFFFFFFFFu) {
          const unsigned sl = p & 31u, src = (p >> 5) & 8191u, dst = p >> 18;
          const T *g = in + (size_t)nbr[sl] * step + src;
          cp_async<C::VB>(tbase + dst * C::ES, g);
        }
      }
    }
    cp_async_commit();
  };

  // native FP64 stars and cubes: the register-operand block (F64Ops), read after the prologue's
  // barrier
  const double *cs = reinterpret_cast<const double *>(smem_raw + NB * C::PER_BRICK);
  if constexpr (C::F64S) {
    double *csw = reinterpret_cast<double *>(smem_raw + NB * C::PER_BRICK);
    for (int e = threadIdx.x; e < F64Ops::NHEAD + C::NCOEF; e += C::NT)
      csw[e] = e < F64Ops::NHEAD ? tp.one_mz[e] : tp.c[e - F64Ops::NHEAD];
  }

  // prologue: adjacency of the first two groups, copies of the first
  Walk w1{g0, 0};
  Walk w2 = advance(w1), w3 = advance(w2);  // the next group and the one after
  long long grp = g0;
  fetch_adj(grp);
  store_adj(0);
  fetch_adj(w2.g);
  store_adj(1);
  __syncthreads();
  issue(0, 0, false);

  // i-streaming: W of the last 2R columns of the previous brick (sym_cube_istream), or of the
  // last two 4-column groups (sym_cube_istream4)
  double W[IST && C::ES == 8 ? 2 : 1][IST && C::ES == 8 ? R + 1 : 1][IST && C::ES == 8 ? 2 * R + 1 : 1];
  CsWin<R, ACC == ACCM_COMP, C::CSROWS> S4;

  for (int it = 0; grp < gend; grp = w2.g, w2 = w3, w3 = advance(w3), ++it) {
    const int cur = it & 1, nxt = cur ^ 1;
    const int ncur = it % 3, nnxt = (it + 1) % 3, nfar = (it + 2) % 3;
    __syncthreads();     // nbrs[nnxt] visible; every thread is done with raw[nxt] and nbrs[nfar]
    issue(nxt, nnxt, STREAM && continues(ncur, nnxt));
    fetch_adj(w3.g);  // lands while this group computes
    cp_async_wait<1>();  // this thread's copies for the current group have landed
    __syncthreads();     // ... and everybody else's

    const unsigned *nbr = nbrs + (ncur * NB + slot) * 36;
    const bool active = nbr[27] != 0;
    const T *rt = reinterpret_cast<const T *>((cur ? raw1 : raw0) + slot * C::TILE_BYTES);
    if constexpr (ACC == ACCM_FF) {
      // one pass, in place: raw doubles -> float pairs (each thread its own elements)
      float2 *ft = reinterpret_cast<float2 *>(const_cast<T *>(rt));
      if (active)
        for (int e = lt; e < C::TILE; e += TPB) ft[e] = split_f64(reinterpret_cast<const double *>(rt)[e]);
      __syncthreads();
    }
    if constexpr (IST) {
      // the stream continues when the previous group (list entry grp - 1, adjacency still in
      // nbrs[nfar]) ran and its centre and i-hi columns of neighbours are this brick's i-lo
      // and centre columns
      // (the same test the gather of this group was issued with: its skipped columns are the
      // ones a continued stream does not read)
      const bool cont = STREAM && it > 0 && continues(nfar, ncur);
      if (active) {
        T *out = reinterpret_cast<T *>(*reinterpret_cast<const unsigned long long *>(nbr + 30));
        const size_t ostep = *reinterpret_cast<const unsigned long long *>(nbr + 34);
        T *ob = out + (size_t)nbr[13] * ostep;
        T *tile = const_cast<T *>(rt);  // this brick's buffer until the next barrier
        if constexpr (C::ES == 8) {
          if (tp.kj) sym_cube_istream<C, R, true>(tile, ob, lt, tp, W, cont);
          else sym_cube_istream<C, R, false>(tile, ob, lt, tp, W, cont);
        } else {
          constexpr bool CM = ACC == ACCM_COMP;
          if (tp.kj) sym_cube_istream4<C, T, R, true, CM>(tile, ob, lt, tp, S4, cont);
          else sym_cube_istream4<C, T, R, false, CM>(tile, ob, lt, tp, S4, cont);
        }
      }
    } else if (active) {
      T *out = reinterpret_cast<T *>(*reinterpret_cast<const unsigned long long *>(nbr + 30));
      const size_t ostep = *reinterpret_cast<const unsigned long long *>(nbr + 34);
      sweep2_brick<T, BK, BJ, BI, R, FAM, ACC>(rt, out + (size_t)nbr[13] * ostep, lt, tp, cs);
    }
    store_adj(nfar);  // group it + 2; read after the next iteration's first barrier
  }
  cp_async_wait<0>();  // no copy may outlive the kernel
}

template <typename T, int BK, int BJ, int BI, int R, int FAM, int ACC, bool BATCH = false, bool IST = false>
int launch_sweep2(const SweepArgs &a, const Taps &tp, cudaStream_t s, int grid_cap = 0) {
  typedef Sweep2Cfg<T, BK, BJ, BI, R, FAM, ACC, IST> C;
  static_assert(C::SMEM <= 227 * 1024, "tile too large");
  static_assert(BK * BJ * BI <= 8192 && C::TILE <= 16384, "plan entry fields overflow");
  auto kern = sweep2_kernel<T, BK, BJ, BI, R, FAM, ACC, BATCH, IST>;
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess && C::SMEM > 48 * 1024)
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, C::NT, C::SMEM);
  if (e != cudaSuccess) return cuda_fail(e, "sweep2 launch setup");
  if (per_sm < 1) return fail(BK_ERR_UNSUPPORTED, "sweep2 kernel does not fit on an SM");
  const long long groups = ((long long)a.nlist + C::NB - 1) / C::NB;
  long long grid = (long long)sms * per_sm;
  if (grid_cap > 0 && grid > grid_cap) grid = grid_cap;
  if (grid > groups) grid = groups;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, C::NT, C::SMEM, s>>>(a, tp);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "sweep2 kernel launch");
  return BK_OK;
}

// Tile geometry the host needs for generic-family tap offsets.
template <typename T, int BK, int BJ, int BI, int R>
struct Sweep2Geom {
  typedef Sweep2Cfg<T, BK, BJ, BI, R, FAM_GENERIC, ACCM_NATIVE> C;
  static constexpr int EJ = C::EJ, EI = C::EI;
};

}  // namespace bk
