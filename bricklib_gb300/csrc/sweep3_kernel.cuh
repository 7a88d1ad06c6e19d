// Star-stencil brick sweep fed by the Tensor Memory Accelerator (row-major 8x8x8 bricks).
//
// The input field is described to the TMA unit as a 3-D tensor (j*BI + i, k, brick) with
// the brick's storage step as the outer stride, so every piece of a brick's star
// neighbourhood is one tiled bulk copy of whole k-plane rows, issued by one thread:
//   centre   box (BJ*BI, BK) of brick adj[b][13]
//   k faces  box (BJ*BI, R)  of bricks adj[b][4] (last R planes) and adj[b][22] (first R)
//   j faces  box (R*BI, BK)  of bricks adj[b][10] (last R rows of every plane) and
//            adj[b][16] (first R rows)
//   i faces  either the whole bricks adj[b][12] and adj[b][14] (an i face is BJ*BK separate
//            pieces of R elements in memory, which cost as many L2 sectors as the whole brick
//            but BJ*BK times as many copy requests; whole bricks also give the i taps the
//            centre's plane stride), or, with NI, box (IW, BJ, BK) of a 4-D view (i, j, k,
//            brick), IW = R rounded up to whole 16-byte units: less shared memory per brick.
// Each region lands densely in its own 128-byte aligned slice of a stage buffer; a stage
// holds NB bricks.  Persistent CTAs, warp-specialised:
//   * the last warp is the producer: its lanes 0..7*NB-1 each own one (brick, region) pair;
//     they load brick-list entries eight groups and adjacency entries four groups ahead, and
//     for each group wait until the consumers have released the stage (mbarrier "empty"), then
//     post the stage's byte count and issue the copies (mbarrier "full");
//   * the other warps are consumers: wait for "full", compute, arrive on "empty".  Every
//     thread computes one (j, i) column of its brick: k taps from registers, i / j taps from
//     shared memory, the region (centre or face) chosen per lane.
// No block-wide barrier runs in the loop.  Every wait gives up after about a second, sets a
// device error flag and stops the CTA (the producer then waits, again bounded, for its
// copies still in flight).  Summation order is that of the pipelined kernel.
#pragma once

#include <cuda.h>

#include "sweep2_kernel.cuh"

namespace bk {

// The box shapes over one input field: whole brick, k face, j face (3-D view), the narrow
// i face (4-D view), and for the row-run kernel the same three 3-D boxes spanning a run of
// consecutive bricks (NB + 2 whole bricks, NB k faces, NB j faces).
struct TmaMaps {
  CUtensorMap m[7];
};

constexpr int TMA_MAX_STAGES = 4;

template <typename T, int BK, int BJ, int BI, int R, bool NI>
struct StarTmaCfg {
  static constexpr int ES = (int)sizeof(T);
  static constexpr int IW = NI ? cmin(BI, (R + 16 / ES - 1) / (16 / ES) * (16 / ES)) : BI;  // i-face columns held
  static constexpr int TPB = BJ * BI;
  static constexpr int NB = cmax(1, cmin(4, 128 / TPB));  // bricks per stage (7*NB producer lanes)
  static constexpr int NC = NB * TPB;                     // consumer threads
  static constexpr int NT = NC + 32;                      // + the producer warp
  static constexpr int al(int b) { return (b + 127) / 128 * 128; }
  static constexpr int B_C = BK * BJ * BI * ES, B_KF = R * BJ * BI * ES, B_JF = BK * R * BI * ES,
                       B_IF = BK * BJ * IW * ES;
  static constexpr int O_C = 0, O_KL = al(B_C), O_KH = O_KL + al(B_KF), O_JL = O_KH + al(B_KF),
                       O_JH = O_JL + al(B_JF), O_IL = O_JH + al(B_JF), O_IH = O_IL + al(B_IF);
  static constexpr int BRICK = O_IH + al(B_IF);               // bytes of one brick's stage buffer
  static constexpr int TX = B_C + 2 * (B_KF + B_JF + B_IF);  // bytes the copies of one brick deliver
  // after the stage buffers: full[4], empty[4] mbarriers, centre brick index [4][NB], abort word,
  // the FP64 register-operand block (F64Ops head, then NTAP coefficients; 8-byte aligned)
  static constexpr int NTAP = 1 + 6 * R;
  static constexpr int O_COEF = 64 + 4 * TMA_MAX_STAGES * NB + 16;
  static constexpr int META = O_COEF + 8 * (F64Ops::NHEAD + NTAP);
  static constexpr int smem(int stages) { return 128 + stages * NB * BRICK + META; }  // + base alignment slack
};

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}
// Wait for the phase of the given parity to complete; gives up after limit_ns (about one
// second by default).
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned parity,
                                                  unsigned long long limit_ns = 1000000000ull) {
  unsigned long long t0 = 0;
  for (unsigned n = 0;; ++n) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((n & 63u) == 63u) {
      const unsigned long long t = global_ns();
      if (!t0) t0 = t;
      else if (t - t0 > limit_ns) return false;
    }
  }
}
__device__ __forceinline__ void tma_load_3d(unsigned dst, const CUtensorMap *map, int x, int y, int z, unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_load_4d(unsigned dst, const CUtensorMap *map, int x, int y, int z, int w,
                                            unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void prefetch_l2(const void *p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(p), "r"(bytes) : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
// Named barrier over `count` threads with an OR reduction of `pred` (uniform result).
__device__ __forceinline__ bool bar_red_or(int id, int count, bool pred) {
  unsigned r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.or.pred q, %2, %3, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}\n"
      : "=r"(r)
      : "r"((unsigned)pred), "r"(id), "r"(count)
      : "memory");
  return r != 0;
}

// A producer lane's look-ahead over the brick list and the adjacency: the list entry of
// iteration it + 2D and the adjacency entry of iteration it + D load at iteration it, so each
// load has D iterations to arrive before it is used (one memory latency per iteration would
// otherwise bound the producer).
template <int D>
struct EntryRing {
  unsigned b[2 * D], v[D];
  template <class LB, class LA>
  __device__ __forceinline__ void init(long long g0, long long gstep, LB load_b, LA load_adj) {
#pragma unroll
    for (int d = 0; d < 2 * D; ++d) b[d] = load_b(g0 + d * gstep);
#pragma unroll
    for (int d = 0; d < D; ++d) v[d] = load_adj(b[d]);
  }
  // the entries of the current iteration are b[0], v[0]; move to the next one
  template <class LB, class LA>
  __device__ __forceinline__ void advance(long long g, long long gstep, LB load_b, LA load_adj) {
    const unsigned nv = load_adj(b[D]);
    const unsigned nb = load_b(g + 2 * D * gstep);
#pragma unroll
    for (int d = 0; d + 1 < D; ++d) v[d] = v[d + 1];
    v[D - 1] = nv;
#pragma unroll
    for (int d = 0; d + 1 < 2 * D; ++d) b[d] = b[d + 1];
    b[2 * D - 1] = nb;
  }
};
constexpr int PRODUCER_LOOKAHEAD = 4;

// One consumer thread's column (fixed j, i; every k plane) of a star stencil over staged
// regions, stored to `ob` (plane stride BJ*BI).  Offsets are in elements from `buf`: cKL / cC /
// cKH address plane 0 of the column in the k-lo face, the centre and the k-hi face (plane
// stride BJ*BI); oi / oj address the i / j taps (index 2(d-1) is +d, 2(d-1)+1 is -d) with
// plane strides si / sj.  Float-float accumulation reads the stage as float pairs.
template <typename T, int BK, int BJ, int BI, int R, int ACC>
__device__ __forceinline__ void star_column(const unsigned char *buf, const int cKL, const int cC, const int cKH,
                                            const int (&oi)[2 * R], const int (&si)[2 * R], const int (&oj)[2 * R],
                                            const int (&sj)[2 * R], T *ob, const Taps &tp) {
  typedef typename Elem<T>::acc AT;
  constexpr int PK = BJ * BI;
  if constexpr (ACC == ACCM_FF) {
    const float2 *f = reinterpret_cast<const float2 *>(buf);
    float2 w[BK + 2 * R];
#pragma unroll
    for (int kk = 0; kk < R; ++kk) w[kk] = f[cKL + kk * PK];
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) w[R + kk] = f[cC + kk * PK];
#pragma unroll
    for (int kk = 0; kk < R; ++kk) w[R + BK + kk] = f[cKH + kk * PK];
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      FFAcc acc;
      acc.first(tp.cf[0], tp.cl[0], w[k + R]);
#pragma unroll
      for (int d = 1; d <= R; ++d) {
        const int t = 1 + 6 * (d - 1), q = 2 * (d - 1);
        acc.add(tp.cf[t + 0], tp.cl[t + 0], f[oi[q] + k * si[q]]);
        acc.add(tp.cf[t + 1], tp.cl[t + 1], f[oi[q + 1] + k * si[q + 1]]);
        acc.add(tp.cf[t + 2], tp.cl[t + 2], f[oj[q] + k * sj[q]]);
        acc.add(tp.cf[t + 3], tp.cl[t + 3], f[oj[q + 1] + k * sj[q + 1]]);
        acc.add(tp.cf[t + 4], tp.cl[t + 4], w[k + R + d]);
        acc.add(tp.cf[t + 5], tp.cl[t + 5], w[k + R - d]);
        acc.renorm();
      }
      store_stream(ob + k * PK, acc.result());
    }
  } else {
    const T *f = reinterpret_cast<const T *>(buf);
    AT w[BK + 2 * R];
#pragma unroll
    for (int kk = 0; kk < R; ++kk) w[kk] = to_acc(f[cKL + kk * PK]);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) w[R + kk] = to_acc(f[cC + kk * PK]);
#pragma unroll
    for (int kk = 0; kk < R; ++kk) w[R + BK + kk] = to_acc(f[cKH + kk * PK]);
    if constexpr (ACC == ACCM_NATIVE && sizeof(AT) == 4) {
      // two k planes per packed FP32 multiply-add (FFMA2): per point the same operations in
      // the same order as the scalar path below, so the results are identical
      static_assert(BK % 2 == 0, "k planes in pairs");
      auto cc = [&](int t) { return tp.cp[t]; };
      static_assert(1 + 6 * R <= TAP_PAIRS, "coefficient pairs");
#pragma unroll
      for (int k = 0; k < BK; k += 2) {
        auto ld2 = [&](int o, int st) { return make_float2(to_acc(f[o + k * st]), to_acc(f[o + (k + 1) * st])); };
        float2 v = __fmul2_rn(cc(0), make_float2(w[k + R], w[k + R + 1]));
#pragma unroll
        for (int d = 1; d <= R; ++d) {
          const int t = 1 + 6 * (d - 1), q = 2 * (d - 1);
          v = __ffma2_rn(cc(t + 0), ld2(oi[q], si[q]), v);
          v = __ffma2_rn(cc(t + 1), ld2(oi[q + 1], si[q + 1]), v);
          v = __ffma2_rn(cc(t + 2), ld2(oj[q], sj[q]), v);
          v = __ffma2_rn(cc(t + 3), ld2(oj[q + 1], sj[q + 1]), v);
          v = __ffma2_rn(cc(t + 4), make_float2(w[k + R + d], w[k + R + 1 + d]), v);
          v = __ffma2_rn(cc(t + 5), make_float2(w[k + R - d], w[k + R + 1 - d]), v);
        }
        store_stream(ob + k * PK, v.x);
        store_stream(ob + (k + 1) * PK, v.y);
      }
    } else
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      AT v;
      if constexpr (ACC == ACCM_NATIVE) {
        v = coef<AT>(tp, 0) * w[k + R];
#pragma unroll
        for (int d = 1; d <= R; ++d) {
          const int t = 1 + 6 * (d - 1), q = 2 * (d - 1);
          v = fma(coef<AT>(tp, t + 0), to_acc(f[oi[q] + k * si[q]]), v);
          v = fma(coef<AT>(tp, t + 1), to_acc(f[oi[q + 1] + k * si[q + 1]]), v);
          v = fma(coef<AT>(tp, t + 2), to_acc(f[oj[q] + k * sj[q]]), v);
          v = fma(coef<AT>(tp, t + 3), to_acc(f[oj[q + 1] + k * sj[q + 1]]), v);
          v = fma(coef<AT>(tp, t + 4), w[k + R + d], v);
          v = fma(coef<AT>(tp, t + 5), w[k + R - d], v);
        }
      } else {
        AT row = coef<AT>(tp, 0) * w[k + R];
#pragma unroll
        for (int d = 1; d <= R; ++d) {
          const int t = 1 + 6 * (d - 1), q = 2 * (d - 1);
          row = fma(coef<AT>(tp, t + 0), to_acc(f[oi[q] + k * si[q]]), row);
          row = fma(coef<AT>(tp, t + 1), to_acc(f[oi[q + 1] + k * si[q + 1]]), row);
        }
        AT s = row, comp = AT(0);
#pragma unroll
        for (int d = 1; d <= R; ++d) {
          const int t = 1 + 6 * (d - 1), q = 2 * (d - 1);
          neumaier(s, comp, coef<AT>(tp, t + 2) * to_acc(f[oj[q] + k * sj[q]]));
          neumaier(s, comp, coef<AT>(tp, t + 3) * to_acc(f[oj[q + 1] + k * sj[q + 1]]));
          neumaier(s, comp, coef<AT>(tp, t + 4) * w[k + R + d]);
          neumaier(s, comp, coef<AT>(tp, t + 5) * w[k + R - d]);
        }
        v = s + comp;
      }
      store_stream(ob + k * PK, v);
    }
  }
}

// The native FP64 column: the same operations in the same order per point as star_column, on
// register operands only (F64Ops; the coefficients cr read from shared memory once per thread),
// with the loop over the column's BK points innermost, so that consecutive multiply-adds share
// one coefficient and each takes its other factor straight from a shared-memory load.
template <int BK, int BJ, int BI, int R>
__device__ __forceinline__ void star_column_f64(const unsigned char *buf, const int cKL, const int cC, const int cKH,
                                                const int (&oi)[2 * R], const int (&si)[2 * R], const int (&oj)[2 * R],
                                                const int (&sj)[2 * R], double *ob, const double (&cr)[1 + 6 * R],
                                                const F64Ops &f64) {
  constexpr int PK = BJ * BI;
  const double *f = reinterpret_cast<const double *>(buf);
  // plane kk in [-R, BK + R) of this column: k-lo face, centre or k-hi face
  auto kv = [&](int kk) { return kk < 0 ? f[cKL + (kk + R) * PK] : kk >= BK ? f[cKH + (kk - BK) * PK] : f[cC + kk * PK]; };
  double acc[BK];
#pragma unroll
  for (int k = 0; k < BK; ++k) acc[k] = f64.mul(cr[0], kv(k));
#pragma unroll
  for (int d = 1; d <= R; ++d) {
    const int t = 1 + 6 * (d - 1), q = 2 * (d - 1);
#pragma unroll
    for (int k = 0; k < BK; ++k) acc[k] = fma(cr[t + 0], f[oi[q] + k * si[q]], acc[k]);
#pragma unroll
    for (int k = 0; k < BK; ++k) acc[k] = fma(cr[t + 1], f[oi[q + 1] + k * si[q + 1]], acc[k]);
#pragma unroll
    for (int k = 0; k < BK; ++k) acc[k] = fma(cr[t + 2], f[oj[q] + k * sj[q]], acc[k]);
#pragma unroll
    for (int k = 0; k < BK; ++k) acc[k] = fma(cr[t + 3], f[oj[q + 1] + k * sj[q + 1]], acc[k]);
#pragma unroll
    for (int k = 0; k < BK; ++k) acc[k] = fma(cr[t + 4], kv(k + d), acc[k]);
#pragma unroll
    for (int k = 0; k < BK; ++k) acc[k] = fma(cr[t + 5], kv(k - d), acc[k]);
  }
#pragma unroll
  for (int k = 0; k < BK; ++k) store_stream(ob + k * PK, acc[k]);
}

template <typename T, int BK, int BJ, int BI, int R, int ACC, bool NI>
__global__ void __launch_bounds__(StarTmaCfg<T, BK, BJ, BI, R, NI>::NT)
sweep_star_tma_kernel(const __grid_constant__ TmaMaps maps, const SweepArgs a, const Taps tp, const int S) {
  typedef StarTmaCfg<T, BK, BJ, BI, R, NI> C;
  typedef typename Elem<T>::acc AT;
  constexpr int NB = C::NB, TPB = C::TPB, IW = C::IW, PK = BJ * BI;
  static_assert(7 * NB <= 32, "one producer lane per (brick, region)");
  static_assert(TPB % 32 == 0, "whole warps per brick");
  static_assert(C::ES == 8 || ACC != ACCM_FF, "float-float needs FP64 storage");

  extern __shared__ __align__(16) unsigned char smem_raw[];
  const unsigned raw = smem_u32(smem_raw);
  const unsigned pad = (128u - (raw & 127u)) & 127u;
  unsigned char *sm = smem_raw + pad;  // 128-byte aligned stage buffers
  const unsigned sbase = raw + pad;
  const unsigned full0 = sbase + S * NB * C::BRICK, empty0 = full0 + 8 * TMA_MAX_STAGES;
  unsigned *outb = reinterpret_cast<unsigned *>(sm + S * NB * C::BRICK + 64);  // [S][NB]
  volatile int *abort_word = reinterpret_cast<volatile int *>(sm + S * NB * C::BRICK + 64 + 4 * TMA_MAX_STAGES * NB);

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, C::NC / 32);
    }
    *abort_word = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    fence_proxy_async_smem();
  }
  static_assert(C::NT >= F64Ops::NHEAD + C::NTAP, "one thread per entry");
  double *coef_s = reinterpret_cast<double *>(sm + S * NB * C::BRICK + C::O_COEF);
  if (threadIdx.x < F64Ops::NHEAD + C::NTAP)
    coef_s[threadIdx.x] = threadIdx.x < F64Ops::NHEAD ? tp.one_mz[threadIdx.x] : tp.c[threadIdx.x - F64Ops::NHEAD];
  __syncthreads();

  const long long ngroups = ((long long)a.nlist + NB - 1) / NB;
  const long long g0 = blockIdx.x, gstep = gridDim.x;
  const int lane = threadIdx.x & 31;
  const unsigned long long lim = a.wait_ns ? a.wait_ns : 1000000000ull;

  if (threadIdx.x >= C::NC) {
    // ------------------------------------------------------------------ producer warp
    const bool prod = lane < 7 * NB;
    const int pbs = lane / 7, prg = lane - (lane / 7) * 7;  // brick slot, region
    // region prg: 0 centre, 1 k-lo, 2 k-hi, 3 j-lo, 4 j-hi, 5 i-lo, 6 i-hi
    const int pslot = prg == 0 ? 13 : prg == 1 ? 4 : prg == 2 ? 22 : prg == 3 ? 10 : prg == 4 ? 16 : prg == 5 ? 12 : 14;
    const int pmap = prg == 1 || prg == 2 ? 1 : prg == 3 || prg == 4 ? 2 : (NI && prg >= 5 ? 3 : 0);
    const int px = prg == 3 ? (BJ - R) * BI : (NI && prg == 5 ? BI - IW : 0), py = prg == 1 ? BK - R : 0;
    const int poff = prg == 0 ? C::O_C : prg == 1 ? C::O_KL : prg == 2 ? C::O_KH : prg == 3 ? C::O_JL
                   : prg == 4 ? C::O_JH : prg == 5 ? C::O_IL : C::O_IH;
    // brick-list entry of this lane's brick in group grp (0xFFFFFFFF: none)
    auto load_b = [&](long long grp) -> unsigned {
      const long long n = grp * NB + pbs;
      return (prod && grp < ngroups && n < (long long)a.nlist) ? a.blist[n] : 0xFFFFFFFFu;
    };
    auto load_adj = [&](unsigned b) -> unsigned {
      return (prod && b < a.nbricks) ? a.adj[(size_t)b * 27 + pslot] : 0u;
    };
    // lanes 7*NB .. 8*NB-1 prefetch the centre bricks of the group PF iterations ahead into
    // L2 (no shared memory involved), so that the copies find them there.  They prefetch
    // brick b of the list itself: adjacency lists hold every brick as its own centre
    // (slot 13); where one does not, the hint is merely wasted.
    constexpr int PF = 2;
    const bool pfl = lane >= 7 * NB && lane < 8 * NB;
    const int pfs = lane - 7 * NB;
    auto load_pf = [&](long long grp) -> unsigned {
      const long long n = grp * NB + pfs;
      return (pfl && grp < ngroups && n < (long long)a.nlist) ? a.blist[n] : 0xFFFFFFFFu;
    };
    unsigned pf = load_pf(g0 + PF * gstep);
    const char *in_bytes = reinterpret_cast<const char *>(a.in) + a.in_off * C::ES;
    EntryRing<PRODUCER_LOOKAHEAD> ring;
    ring.init(g0, gstep, load_b, load_adj);
    int it = 0, st = 0;
    unsigned ph = 0;  // (it / S) & 1
    for (long long g = g0; g < ngroups; g += gstep, ++it) {
      // every lane waits (acquire), the warp agrees on the outcome
      const bool freed = it < S || mbar_wait_bounded(empty0 + 8 * st, ph ^ 1u, lim);
      if (!__all_sync(0xFFFFFFFFu, freed)) {
        if (lane == 0) atomicOr(a.err, FLAG_TIMEOUT);
        *abort_word = 1;
        break;
      }
      if (__any_sync(0xFFFFFFFFu, *abort_word != 0)) break;
      // checks of this group's entries
      const unsigned bq = ring.b[0];
      unsigned v = ring.v[0];
      int act = 0;
      if (prod && bq != 0xFFFFFFFFu) {
        if (bq >= a.nbricks) {
          if (prg == 0) atomicOr(a.err, FLAG_BOUNDS);
        } else {
          act = prg != 0 || ((long long)v < a.out_chunks && (long long)v < a.in_chunks);
          if ((long long)v >= a.in_chunks || !act) {
            atomicOr(a.err, FLAG_BOUNDS);
            v = 0;
          }
        }
      }
      const int bact = __shfl_sync(0xFFFFFFFFu, act, pbs * 7 < 32 ? pbs * 7 : 0);
      const unsigned m = __ballot_sync(0xFFFFFFFFu, prod && prg == 0 && bact);
      if (prod && prg == 0) outb[st * NB + pbs] = bact ? v : 0xFFFFFFFFu;
      __syncwarp();  // the centre indices are written before the phase can complete
      const unsigned bar = full0 + 8 * st;
      if (lane == 0) mbar_arrive_expect_tx(bar, (unsigned)__popc(m) * (unsigned)C::TX);
      __syncwarp();
      // the test hook withholds the i-hi copy of the first brick of this CTA's first stage
      const bool withheld = a.withhold && blockIdx.x == 0 && it == 0 && pbs == 0 && prg == 6;
      if (prod && bact && !withheld)
      {
        if (pmap == 3) tma_load_4d(sbase + (st * NB + pbs) * C::BRICK + poff, &maps.m[3], px, 0, 0, (int)v, bar);
        else tma_load_3d(sbase + (st * NB + pbs) * C::BRICK + poff, &maps.m[pmap], px, py, (int)v, bar);
      }
      // advance the prefetch pipeline
      ring.advance(g, gstep, load_b, load_adj);
      if (++st == S) {
        st = 0;
        ph ^= 1u;
      }
      if (pfl && (long long)pf < a.in_chunks)
        prefetch_l2(in_bytes + (size_t)pf * a.in_step * C::ES, (unsigned)(BK * BJ * BI * C::ES));
      pf = load_pf(g + (PF + 1) * gstep);
    }
    // copies of the last S issued iterations may still be in flight after an abort: wait for
    // each of those stages (bounded; a stage whose wait runs out has had the whole limit for
    // its copies to land)
    if (lane == 0)
      for (int q = it - S > 0 ? it - S : 0; q < it; ++q)
        mbar_wait_bounded(full0 + 8 * (q % S), (unsigned)(q / S) & 1u, lim);
    return;
  }

  // -------------------------------------------------------------------- consumer warps
  const int bs = threadIdx.x / TPB, lt = threadIdx.x - bs * TPB;
  const int j = lt / BI, i = lt - j * BI;
  // per-lane shared-memory element offsets (from the brick's stage buffer) and k strides
  // of the i and j taps: index 2(d-1) is +d, 2(d-1)+1 is -d
  int oi[2 * R], si[2 * R], oj[2 * R], sj[2 * R];
  constexpr int eC = C::O_C / C::ES, eKL = C::O_KL / C::ES, eKH = C::O_KH / C::ES, eJL = C::O_JL / C::ES,
                eJH = C::O_JH / C::ES, eIL = C::O_IL / C::ES, eIH = C::O_IH / C::ES;
#pragma unroll
  for (int d = 1; d <= R; ++d) {
#pragma unroll
    for (int sg = 0; sg < 2; ++sg) {
      const int q = 2 * (d - 1) + sg;
      const int ii = sg ? i - d : i + d;
      if (ii >= BI) { oi[q] = eIH + j * IW + (ii - BI); si[q] = BJ * IW; }
      else if (ii < 0) { oi[q] = eIL + j * IW + (IW + ii); si[q] = BJ * IW; }
      else { oi[q] = eC + j * BI + ii; si[q] = PK; }
      const int jj = sg ? j - d : j + d;
      if (jj >= BJ) { oj[q] = eJH + (jj - BJ) * BI + i; sj[q] = R * BI; }
      else if (jj < 0) { oj[q] = eJL + (R + jj) * BI + i; sj[q] = R * BI; }
      else { oj[q] = eC + jj * BI + i; sj[q] = PK; }
    }
  }

  constexpr bool F64R = ACC == ACCM_NATIVE && C::ES == 8;  // FP64 column with register coefficients
  double cr[C::NTAP];
#pragma unroll
  for (int t = 0; t < C::NTAP; ++t) cr[t] = F64R ? coef_s[F64Ops::NHEAD + t] : 0.0;
  const F64Ops f64 = F64R ? F64Ops::load(coef_s) : F64Ops{0.0, 0.0};

  int st = 0;
  unsigned ph = 0;  // phase parity of the stage's current use
  for (long long g = g0; g < ngroups; g += gstep) {
    const bool ok = __all_sync(0xFFFFFFFFu, mbar_wait_bounded(full0 + 8 * st, ph, lim));
    if (!ok) {
      atomicOr(a.err, FLAG_TIMEOUT);
      *abort_word = 1;
    }
    const unsigned ob_idx = outb[st * NB + bs];
    const bool active = ok && ob_idx != 0xFFFFFFFFu;
    unsigned char *buf = sm + (st * NB + bs) * C::BRICK;
    if constexpr (ACC == ACCM_FF) {
      // in place, each thread its own elements: raw doubles -> float pairs; the brick's
      // threads then meet on a named barrier that also agrees on stopping
      if (active) {
        double *dv = reinterpret_cast<double *>(buf);
        float2 *fv = reinterpret_cast<float2 *>(buf);
        for (int e = lt; e < C::BRICK / 8; e += TPB) fv[e] = split_f64(dv[e]);
      }
      if (bar_red_or(1 + bs, TPB, !ok)) break;
    } else {
      if (!ok) break;
    }
    if (active) {
      T *ob = reinterpret_cast<T *>(a.out) + a.out_off + (size_t)ob_idx * a.out_step + (size_t)(j * BI + i);
      if constexpr (F64R)
        star_column_f64<BK, BJ, BI, R>(buf, eKL + j * BI + i, eC + j * BI + i, eKH + j * BI + i, oi, si, oj, sj,
                                       reinterpret_cast<double *>(ob), cr, f64);
      else
        star_column<T, BK, BJ, BI, R, ACC>(buf, eKL + j * BI + i, eC + j * BI + i, eKH + j * BI + i, oi, si, oj, sj,
                                           ob, tp);
    }
    // the float-float conversion wrote the stage through the generic proxy; order those
    // writes before the copies that refill it
    if constexpr (ACC == ACCM_FF) fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) mbar_arrive(empty0 + 8 * st);
    if (++st == S) {
      st = 0;
      ph ^= 1u;
    }
  }
}

// Host: encode the four box shapes over the input field.  Returns false when the field
// does not meet the bulk-tensor rules (16-byte aligned base, strides multiple of 16 bytes).
bool star_tma_maps(const SweepArgs &a, int dtype, int bk, int bj, int bi, int r, int iw, TmaMaps *maps);
// The run boxes m[4..6] over consecutive bricks (after star_tma_maps): slot_box whole bricks, nb
// k faces, nb j faces; false when the field cannot be described that way (the kernel then
// copies brick by brick).
bool row_group_maps(const SweepArgs &a, int dtype, int bk, int bj, int bi, int r, int nb, int slot_box,
                    TmaMaps *maps);
// Pipeline depth: the host thread's bk_set_pipeline_depth value when set, else BK_TMA_STAGES
// (2..4) when set, else `dflt`.
int tma_stages(int dflt);
int pipeline_depth_override();
void set_pipeline_depth_override(int stages);

template <typename T, int BK, int BJ, int BI, int R, int ACC, bool NI>
int launch_star_tma(const SweepArgs &a, const Taps &tp, int dtype, cudaStream_t s, int grid_cap = 0) {
  typedef StarTmaCfg<T, BK, BJ, BI, R, NI> C;
  // default depth 2: on GB300 more resident CTAs beat deeper pipelines (FP32 star7 at 512^3:
  // 602 / 490 GStencil/s with 2 / 3 stages)
  const int S = tma_stages(2);
  const int smem = C::smem(S);
  if (smem > 227 * 1024) return fail(BK_ERR_UNSUPPORTED, "TMA sweep stage buffers exceed shared memory");
  TmaMaps maps;
  if (!star_tma_maps(a, dtype, BK, BJ, BI, R, C::IW, &maps)) return fail(BK_ERR_UNSUPPORTED, "field not describable to the TMA unit");
  auto kern = sweep_star_tma_kernel<T, BK, BJ, BI, R, ACC, NI>;
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, C::NT, smem);
  if (e != cudaSuccess) return cuda_fail(e, "star TMA sweep launch setup");
  if (per_sm < 1) return fail(BK_ERR_UNSUPPORTED, "star TMA sweep does not fit on an SM");
  const long long groups = ((long long)a.nlist + C::NB - 1) / C::NB;
  long long grid = (long long)sms * per_sm;
  if (grid_cap > 0 && grid > grid_cap) grid = grid_cap;
  if (grid > groups) grid = groups;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, C::NT, smem, s>>>(maps, a, tp, S);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "star TMA sweep launch");
  return BK_OK;
}

}  // namespace bk
