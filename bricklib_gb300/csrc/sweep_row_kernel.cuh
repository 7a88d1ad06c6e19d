// Star-stencil brick sweep over runs of i-adjacent bricks, fed by the Tensor Memory
// Accelerator (2- and 4-byte storage, row-major 8x8x8 bricks).
//
// A brick list in grid order is made of rows of bricks that are neighbours along i (the
// reference's drivers sweep bricks in that order).  The kernel takes the list in segments of
// NB entries and splits every segment into runs: maximal stretches of entries where entry n+1
// is entry n's i-hi neighbour (adjacency slot 14) and entry n is entry n+1's i-lo neighbour
// (slot 12).  One pipeline stage holds one run of L bricks:
//   slots 0 .. L+1  whole bricks: the run's i-lo neighbour, the L centre bricks, the run's
//                   i-hi neighbour (box (BJ*BI, BK) of the 3-D view (j*BI + i, k, brick));
//   faces           brick n's k faces (box (BJ*BI, R)) and j faces (box (R*BI, BK)), each
//                   type in its own array of NB.
// Brick n's i taps read the slots either side of its own, so a run loads L + 2 whole bricks
// where per-brick staging loads 3 L.  A list that is not in grid order runs as runs of one
// brick.  A run of NB bricks whose slots are consecutive bricks in storage, and whose k / j
// neighbours are too (a dense grid in grid order), takes five copies instead of 5 NB + 2: the
// NB + 2 slots, and each face type of the NB bricks, as one box over consecutive bricks; the
// copy-instruction rate, not the bytes, bounds this staging.  Persistent CTAs, warp-specialised like the per-brick kernel: the last warp produces
// (lanes 0 .. 7*NB-1 each own one (entry, region) pair of the segment; list and adjacency
// entries load several segments ahead), the other warps consume (brick slot n+1 belongs to
// consumer warp n, whose lanes compute one (j, i, i+1) column pair each).  The number of
// stages a segment takes is known only to the producer, so it ends the stream with a marker
// stage that carries no copies.  Every wait is bounded (about a second), after which the CTA
// sets a device error flag and stops.  Summation order is that of the pipelined kernel.
#pragma once

#include "sweep3_kernel.cuh"

namespace bk {

// bricks per copy of a run's whole-brick slots (divides NB + 2)
#ifndef BK_ROW_SLOT_BOX
#define BK_ROW_SLOT_BOX 6
#endif
constexpr int SLOT_BOX = BK_ROW_SLOT_BOX;

template <typename T, int R>
struct RowTmaCfg {
  static constexpr int BK = 8, BJ = 8, BI = 8, PK = BJ * BI;
  static constexpr int ES = (int)sizeof(T);
  static constexpr int NB = 4;           // list entries per segment, bricks per stage at most
  static constexpr int NC = NB * 32;     // consumer threads: one warp per brick slot
  static constexpr int NT = NC + 32;     // + the producer warp
  static constexpr int al(int b) { return (b + 127) / 128 * 128; }
  static constexpr int B_C = BK * BJ * BI * ES, B_KF = R * BJ * BI * ES, B_JF = BK * R * BI * ES;
  static constexpr int PC = B_C;         // pitch of the whole-brick slots
  // faces after the slots, by type: NB k-lo faces, NB k-hi, NB j-lo, NB j-hi (a run of
  // consecutive bricks fills each type with one copy)
  static constexpr int FKL = (NB + 2) * PC, FKH = FKL + NB * B_KF, FJL = FKH + NB * B_KF, FJH = FJL + NB * B_JF;
  static constexpr int STAGE = FJH + NB * B_JF;      // bytes of one stage
  static_assert(B_C % 128 == 0 && B_KF % 128 == 0 && B_JF % 128 == 0, "copies land on 128-byte boundaries");
  static constexpr int TXB = B_C + 2 * (B_KF + B_JF);  // bytes one run brick brings
  // after the stages: full[4], empty[4] mbarriers, centre brick index [4][NB], abort word
  static constexpr int META = 64 + 4 * TMA_MAX_STAGES * NB + 16;
  static constexpr int smem(int stages) { return 128 + stages * STAGE + META; }
};

// Element offsets (from the stage base, plane 0) of one thread's taps for columns (i0, i0+1):
// a[m + MI] = the aligned pair (i0 + 2m, i0 + 2m + 1), m = -MI..MI, MI = ceil(R/2) (m = 0 is the
// centre; the others may sit in the slots either side); oj / sj the j taps (index 2(d-1) is +d,
// 2(d-1)+1 is -d) and their plane strides; kl / kh plane 0 of the k faces.
template <int R>
struct RowPairTaps {
  int a[2 * ((R + 1) / 2) + 1];
  int oj[2 * R], sj[2 * R];
  int kl, kh;
};

// Columns (i0, i0+1) of a star stencil over every k plane, with FP32 arithmetic: packed FFMA2
// on the column pair (native), or scalar compensated sums per column.  Per point the terms and
// their order are those of the per-brick kernels: centre, then for d = 1..R: i+d, i-d, j+d,
// j-d, k+d, k-d; a pair tap at odd distance d joins the halves of two aligned pairs.
template <typename T, int R, int ACC>
__device__ __forceinline__ void star_pair_column(const T *f, const RowPairTaps<R> &o, T *ob, const Taps &tp) {
  constexpr int BK = 8, PK = 64, MI = (R + 1) / 2;
  float2 w[BK + 2 * R];
#pragma unroll
  for (int kk = 0; kk < R; ++kk) w[kk] = ld_pair(f + o.kl + kk * PK);
#pragma unroll
  for (int kk = 0; kk < BK; ++kk) w[R + kk] = ld_pair(f + o.a[MI] + kk * PK);
#pragma unroll
  for (int kk = 0; kk < R; ++kk) w[R + BK + kk] = ld_pair(f + o.kh + kk * PK);
#pragma unroll
  for (int k = 0; k < BK; ++k) {
    float2 A[2 * MI + 1];
#pragma unroll
    for (int m = 0; m < 2 * MI + 1; ++m) A[m] = m == MI ? w[k + R] : ld_pair(f + o.a[m] + k * PK);
    auto ip = [&](int d) {  // taps (i0 + d, i0 + 1 + d)
      return (d & 1) ? make_float2(A[MI + (d - 1) / 2].y, A[MI + (d + 1) / 2].x) : A[MI + d / 2];
    };
    auto im = [&](int d) {  // taps (i0 - d, i0 + 1 - d)
      return (d & 1) ? make_float2(A[MI - (d + 1) / 2].y, A[MI - (d - 1) / 2].x) : A[MI - d / 2];
    };
    auto jt = [&](int q) { return ld_pair(f + o.oj[q] + k * o.sj[q]); };
    float2 v;
    if constexpr (ACC == ACCM_NATIVE) {
      auto cc = [&](int t) { return tp.cp[t]; };
      static_assert(1 + 6 * R <= TAP_PAIRS, "coefficient pairs");
      v = __fmul2_rn(cc(0), w[k + R]);
#pragma unroll
      for (int d = 1; d <= R; ++d) {
        const int t = 1 + 6 * (d - 1), q = 2 * (d - 1);
        v = __ffma2_rn(cc(t + 0), ip(d), v);
        v = __ffma2_rn(cc(t + 1), im(d), v);
        v = __ffma2_rn(cc(t + 2), jt(q), v);
        v = __ffma2_rn(cc(t + 3), jt(q + 1), v);
        v = __ffma2_rn(cc(t + 4), w[k + R + d], v);
        v = __ffma2_rn(cc(t + 5), w[k + R - d], v);
      }
    } else {
      float2 row;
      row.x = coef<float>(tp, 0) * w[k + R].x;
      row.y = coef<float>(tp, 0) * w[k + R].y;
#pragma unroll
      for (int d = 1; d <= R; ++d) {
        const int t = 1 + 6 * (d - 1);
        const float2 p = ip(d), m = im(d);
        row.x = fmaf(coef<float>(tp, t + 0), p.x, row.x);
        row.y = fmaf(coef<float>(tp, t + 0), p.y, row.y);
        row.x = fmaf(coef<float>(tp, t + 1), m.x, row.x);
        row.y = fmaf(coef<float>(tp, t + 1), m.y, row.y);
      }
      float2 acc = row, comp = make_float2(0.0f, 0.0f);
#pragma unroll
      for (int d = 1; d <= R; ++d) {
        const int t = 1 + 6 * (d - 1), q = 2 * (d - 1);
        const float2 jp = jt(q), jm = jt(q + 1);
        neumaier(acc.x, comp.x, coef<float>(tp, t + 2) * jp.x);
        neumaier(acc.y, comp.y, coef<float>(tp, t + 2) * jp.y);
        neumaier(acc.x, comp.x, coef<float>(tp, t + 3) * jm.x);
        neumaier(acc.y, comp.y, coef<float>(tp, t + 3) * jm.y);
        neumaier(acc.x, comp.x, coef<float>(tp, t + 4) * w[k + R + d].x);
        neumaier(acc.y, comp.y, coef<float>(tp, t + 4) * w[k + R + d].y);
        neumaier(acc.x, comp.x, coef<float>(tp, t + 5) * w[k + R - d].x);
        neumaier(acc.y, comp.y, coef<float>(tp, t + 5) * w[k + R - d].y);
      }
      v = make_float2(acc.x + comp.x, acc.y + comp.y);
    }
    st_pair(ob + k * PK, v);
  }
}

template <typename T, int R, int ACC>
__global__ void __launch_bounds__(RowTmaCfg<T, R>::NT)
sweep_star_row_kernel(const __grid_constant__ TmaMaps maps, const SweepArgs a, const Taps tp, const int S,
                      const int group_maps) {
  typedef RowTmaCfg<T, R> C;
  constexpr int NB = C::NB, BK = C::BK, BJ = C::BJ, BI = C::BI, PK = C::PK, E = C::ES;
  constexpr unsigned NONE = 0xFFFFFFFFu;  // slot without a brick in this stage
  constexpr unsigned END = 0xFFFFFFFEu;   // no further stages
  constexpr unsigned ALL = 0xFFFFFFFFu;
  static_assert(7 * NB <= 28, "one producer lane per (entry, region), four prefetch lanes");
  static_assert(E <= 4, "2- and 4-byte storage");

  extern __shared__ __align__(16) unsigned char smem_raw[];
  const unsigned raw = smem_u32(smem_raw);
  const unsigned pad = (128u - (raw & 127u)) & 127u;
  unsigned char *sm = smem_raw + pad;  // 128-byte aligned stages
  const unsigned sbase = raw + pad;
  const unsigned full0 = sbase + S * C::STAGE, empty0 = full0 + 8 * TMA_MAX_STAGES;
  unsigned *outb = reinterpret_cast<unsigned *>(sm + S * C::STAGE + 64);  // [S][NB]
  volatile int *abort_word = reinterpret_cast<volatile int *>(sm + S * C::STAGE + 64 + 4 * TMA_MAX_STAGES * NB);

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, C::NC / 32);
    }
    *abort_word = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    fence_proxy_async_smem();
  }
  __syncthreads();

  const long long nseg = ((long long)a.nlist + NB - 1) / NB;
  const long long g0 = blockIdx.x, gstep = gridDim.x;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x >= C::NC) {
    // ------------------------------------------------------------------ producer warp
    const bool prod = lane < 7 * NB;
    const int pbs = lane / 7, prg = lane - (lane / 7) * 7;  // segment entry, region
    // region prg: 0 centre, 1 k-lo, 2 k-hi, 3 j-lo, 4 j-hi, 5 i-lo, 6 i-hi
    const int pslot = prg == 0 ? 13 : prg == 1 ? 4 : prg == 2 ? 22 : prg == 3 ? 10 : prg == 4 ? 16 : prg == 5 ? 12 : 14;
    const int pmap = prg == 1 || prg == 2 ? 1 : prg == 3 || prg == 4 ? 2 : 0;
    const int px = prg == 3 ? (BJ - R) * BI : 0, py = prg == 1 ? BK - R : 0;
    // faces only: the type's array and its pitch
    const int fbase = prg == 1 ? C::FKL : prg == 2 ? C::FKH : prg == 3 ? C::FJL : C::FJH;
    const int fpitch = prg == 1 || prg == 2 ? C::B_KF : C::B_JF;
    auto load_b = [&](long long grp) -> unsigned {
      const long long n = grp * NB + pbs;
      return (prod && grp < nseg && n < (long long)a.nlist) ? a.blist[n] : NONE;
    };
    auto load_adj = [&](unsigned b) -> unsigned {
      return (prod && b < a.nbricks) ? a.adj[(size_t)b * 27 + pslot] : 0u;
    };
    // lanes 28..31 prefetch the centre bricks of the segment PF iterations ahead into L2
    constexpr int PF = 2;
    const bool pfl = lane >= 7 * NB && lane < 8 * NB;
    const int pfs = lane - 7 * NB;
    auto load_pf = [&](long long grp) -> unsigned {
      const long long n = grp * NB + pfs;
      return (pfl && grp < nseg && n < (long long)a.nlist) ? a.blist[n] : NONE;
    };
    unsigned pf = load_pf(g0 + PF * gstep);
    const char *in_bytes = reinterpret_cast<const char *>(a.in) + a.in_off * E;
    EntryRing<PRODUCER_LOOKAHEAD> ring;
    ring.init(g0, gstep, load_b, load_adj);
    int it = 0, st = 0;                // stages issued, current stage
    unsigned ph = 0;                   // (it / S) & 1
    bool stop = false;
    for (long long g = g0; g < nseg && !stop; g += gstep) {
      // checks of this segment's entries: out-of-range faces read brick 0, an entry whose
      // brick or centre is out of range is skipped; both raise the bounds flag
      const unsigned bq = ring.b[0];
      unsigned v = ring.v[0];
      int act = 0;
      if (prod && bq != NONE) {
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
      // entries that run (bit n), and entries n, n+1 that are i-neighbours of each other (bit n)
      const unsigned am = __ballot_sync(ALL, prod && prg == 0 && act);
      const unsigned vn = __shfl_down_sync(ALL, v, 1);   // lane 7n+6 <- centre of entry n+1
      const unsigned vp = __shfl_up_sync(ALL, v, 12);    // lane 7(n+1)+5 <- centre of entry n
      const unsigned c1 = __ballot_sync(ALL, prod && prg == 6 && pbs + 1 < NB && v == vn);
      const unsigned c2 = __ballot_sync(ALL, prod && prg == 5 && pbs >= 1 && v == vp);
      unsigned bm = 0, cm = 0;
#pragma unroll
      for (int n = 0; n < NB; ++n) {
        if ((am >> (7 * n)) & 1u) bm |= 1u << n;
        if (n + 1 < NB && ((c1 >> (7 * n + 6)) & 1u) && ((c2 >> (7 * n + 12)) & 1u)) cm |= 1u << n;
      }
      ring.advance(g, gstep, load_b, load_adj);
      unsigned todo = bm;
      while (todo) {  // one stage per run; warp-uniform
        const int s0 = __ffs(todo) - 1;
        int e = s0 + 1;
        while (e < NB && ((todo >> e) & 1u) && ((cm >> (e - 1)) & 1u)) ++e;
        todo &= ~((1u << e) - 1u);
        const bool freed = it < S || mbar_wait_bounded(empty0 + 8 * st, ph ^ 1u);
        if (!__all_sync(ALL, freed)) {
          if (lane == 0) atomicOr(a.err, FLAG_TIMEOUT);
          *abort_word = 1;
          stop = true;
          break;
        }
        if (__any_sync(ALL, *abort_word != 0)) {
          stop = true;
          break;
        }
        const int L = e - s0;
        const int src = s0 + lane < NB ? s0 + lane : NB - 1;
        const unsigned cv = __shfl_sync(ALL, v, 7 * src);
        if (lane < NB) outb[st * NB + lane] = lane < L ? cv : NONE;
        __syncwarp();  // the centre indices are written before the phase can complete
        const unsigned bar = full0 + 8 * st;
        if (lane == 0) mbar_arrive_expect_tx(bar, (unsigned)(L * C::TXB + 2 * C::B_C));
        __syncwarp();
        // a full run over consecutive bricks: entry n's region r is region r of entry 0 plus
        // n, and the slots run from the i-lo neighbour to the i-hi one without a gap
        bool group = false;
        if (group_maps && L == NB) {
          const unsigned first = __shfl_sync(ALL, v, prg < 7 ? prg : 0);  // region prg of entry 0
          const unsigned c0 = __shfl_sync(ALL, v, 0), cl = __shfl_sync(ALL, v, 7 * (NB - 1));
          const bool ok = !prod || (prg <= 4 ? v == first + (unsigned)pbs
                                             : prg == 5 ? (pbs != 0 || v + 1u == c0) : (pbs != NB - 1 || v == cl + 1u));
          group = __all_sync(ALL, ok);
        }
        const unsigned stage = sbase + st * C::STAGE;
        if (group) {
          if (lane == 5)  // slots 0 .. NB+1, SLOT_BOX bricks per copy
#pragma unroll
            for (int q = 0; q < (NB + 2) / SLOT_BOX; ++q)
              tma_load_3d(stage + q * SLOT_BOX * C::PC, &maps.m[4], 0, 0, (int)v + q * SLOT_BOX, bar);
          else if (lane >= 1 && lane <= 4)
            tma_load_3d(stage + fbase, &maps.m[pmap + 4], px, py, (int)v, bar);
        } else if (prod && pbs >= s0 && pbs < e) {
          const int slot = pbs - s0 + 1;
          if (prg == 0) tma_load_3d(stage + slot * C::PC, &maps.m[0], 0, 0, (int)v, bar);
          else if (prg == 5) {
            if (pbs == s0) tma_load_3d(stage, &maps.m[0], 0, 0, (int)v, bar);
          } else if (prg == 6) {
            if (pbs == e - 1) tma_load_3d(stage + (L + 1) * C::PC, &maps.m[0], 0, 0, (int)v, bar);
          } else {
            tma_load_3d(stage + fbase + (slot - 1) * fpitch, &maps.m[pmap], px, py, (int)v, bar);
          }
        }
        ++it;
        if (++st == S) {
          st = 0;
          ph ^= 1u;
        }
      }
      if (pfl && (long long)pf < a.in_chunks)
        prefetch_l2(in_bytes + (size_t)pf * a.in_step * E, (unsigned)C::B_C);
      pf = load_pf(g + (PF + 1) * gstep);
    }
    if (!stop) {
      // the end marker: a stage whose phase completes without copies
      const bool freed = it < S || mbar_wait_bounded(empty0 + 8 * st, ph ^ 1u);
      if (__all_sync(ALL, freed)) {
        if (lane < NB) outb[st * NB + lane] = END;
        __syncwarp();
        if (lane == 0) mbar_arrive(full0 + 8 * st);
        ++it;
      } else {
        if (lane == 0) atomicOr(a.err, FLAG_TIMEOUT);
        *abort_word = 1;
      }
    }
    // copies of the last S issued stages may still be in flight after an abort
    if (lane == 0)
      for (int q = it - S > 0 ? it - S : 0; q < it; ++q)
        if (!mbar_wait_bounded(full0 + 8 * (q % S), (unsigned)(q / S) & 1u)) break;
    return;
  }

  // -------------------------------------------------------------------- consumer warps
  // one warp per brick slot; lane = (j, pair of i columns)
  const int bs = threadIdx.x >> 5;
  const int j = lane >> 2, i0 = 2 * (lane & 3);
  const int slot = bs + 1;
  constexpr int SE = C::PC / E;  // slot pitch in elements
  constexpr int MI = (R + 1) / 2;

  RowPairTaps<R> o;
#pragma unroll
  for (int m = -MI; m <= MI; ++m) {
    const int c = i0 + 2 * m;
    o.a[m + MI] = (c >= BI ? (slot + 1) * SE + (c - BI) : c < 0 ? (slot - 1) * SE + (c + BI) : slot * SE + c) + j * BI;
  }
#pragma unroll
  for (int d = 1; d <= R; ++d) {
#pragma unroll
    for (int sg = 0; sg < 2; ++sg) {
      const int q = 2 * (d - 1) + sg;
      const int jj = sg ? j - d : j + d;
      if (jj >= BJ) { o.oj[q] = (C::FJH + bs * C::B_JF) / E + (jj - BJ) * BI + i0; o.sj[q] = R * BI; }
      else if (jj < 0) { o.oj[q] = (C::FJL + bs * C::B_JF) / E + (R + jj) * BI + i0; o.sj[q] = R * BI; }
      else { o.oj[q] = slot * SE + jj * BI + i0; o.sj[q] = PK; }
    }
  }
  o.kl = (C::FKL + bs * C::B_KF) / E + j * BI + i0;
  o.kh = (C::FKH + bs * C::B_KF) / E + j * BI + i0;

  int st = 0;
  unsigned ph = 0;
  for (;;) {
    const bool ok = __all_sync(ALL, mbar_wait_bounded(full0 + 8 * st, ph));
    if (!ok) {
      atomicOr(a.err, FLAG_TIMEOUT);
      *abort_word = 1;
      break;
    }
    const unsigned ob_idx = outb[st * NB + bs];
    if (ob_idx == END) break;
    if (ob_idx != NONE) {
      T *ob = reinterpret_cast<T *>(a.out) + a.out_off + (size_t)ob_idx * a.out_step + (size_t)(j * BI + i0);
      star_pair_column<T, R, ACC>(reinterpret_cast<const T *>(sm + st * C::STAGE), o, ob, tp);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(empty0 + 8 * st);
    if (++st == S) {
      st = 0;
      ph ^= 1u;
    }
  }
}

template <typename T, int R, int ACC>
int launch_star_row(const SweepArgs &a, const Taps &tp, int dtype, cudaStream_t s) {
  typedef RowTmaCfg<T, R> C;
  // Defaults measured on GB300 at 512^3 (GStencil/s, grouped copies with 2 / 3 stages, brick by
  // brick with 2): FP32 star7 578 / 735 / 704, star13 635 / 629 / 619, star25 528 / 457 / 491;
  // BF16 star7 938 / 921 / 821, star13 700 / 699 / 616, star25 483 / 481 / 503.
  constexpr bool group_default = !(C::ES == 2 && R == 4);
  const int S = tma_stages(C::ES == 4 && R == 1 ? 3 : 2);
  const int smem = C::smem(S);
  if (smem > 227 * 1024) return fail(BK_ERR_UNSUPPORTED, "row TMA sweep stages exceed shared memory");
  TmaMaps maps;
  if (!star_tma_maps(a, dtype, C::BK, C::BJ, C::BI, R, C::BI, &maps))
    return fail(BK_ERR_UNSUPPORTED, "field not describable to the TMA unit");
  // BK_TMA_GROUP=0 / 1 keeps every run on brick-by-brick copies / allows grouped copies
  const char *ge = getenv("BK_TMA_GROUP");
  const bool group = ge ? ge[0] != '0' : group_default;
  static_assert((C::NB + 2) % SLOT_BOX == 0, "slot copies");
  const int group_maps = group && row_group_maps(a, dtype, C::BK, C::BJ, C::BI, R, C::NB, SLOT_BOX, &maps);
  auto kern = sweep_star_row_kernel<T, R, ACC>;
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, C::NT, smem);
  if (e != cudaSuccess) return cuda_fail(e, "row TMA sweep launch setup");
  if (per_sm < 1) return fail(BK_ERR_UNSUPPORTED, "row TMA sweep does not fit on an SM");
  const long long segs = ((long long)a.nlist + C::NB - 1) / C::NB;
  long long grid = (long long)sms * per_sm;
  if (grid > segs) grid = segs;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, C::NT, smem, s>>>(maps, a, tp, S, group_maps);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "row TMA sweep launch");
  return BK_OK;
}

}  // namespace bk
