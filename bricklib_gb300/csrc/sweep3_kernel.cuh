// Star-stencil brick sweep fed by the Tensor Memory Accelerator (row-major 8x8x8 bricks).
//
// The input field is described to the TMA unit as a 4-D tensor (i, j, k, brick) with the
// brick's storage step as the outer stride, so every piece of a brick's star
// neighbourhood is one tiled bulk copy issued by one thread:
//   centre   box (BI, BJ, BK) of brick adj[b][13]
//   k faces  box (BI, BJ, R)  of bricks adj[b][4] (last R planes) and adj[b][22] (first R)
//   j faces  box (BI, R, BK)  of bricks adj[b][10] (last R rows) and adj[b][16] (first R)
//   i faces  box (IW, BJ, BK) of bricks adj[b][12] (last IW columns) and adj[b][14] (first
//            IW), IW = R rounded up to whole 16-byte units
// Each region lands densely in its own 128-byte aligned slice of a stage buffer; a stage
// holds NB bricks and completes on one mbarrier (transaction bytes).  Persistent CTAs keep
// S-1 groups of copies in flight ahead of the group they compute.  Warp 0 is the producer:
// its lanes 0..7*NB-1 each own one (brick, region) pair, load that region's adjacency entry
// one group before it is needed and issue its copy.  Every thread computes one (j, i)
// column of its brick: k taps from registers, i / j taps from shared memory, the region
// (centre or face) chosen per lane.  Summation order is that of the pipelined kernel.
#pragma once

#include <cuda.h>

#include "sweep2_kernel.cuh"

namespace bk {

// The four box shapes over one input field: centre, k face, j face, i face.
struct TmaMaps {
  CUtensorMap m[4];
};

template <typename T, int BK, int BJ, int BI, int R>
struct StarTmaCfg {
  static constexpr int ES = (int)sizeof(T);
  static constexpr int VE = 16 / ES;                        // elements per 16 bytes
  static constexpr int IW = cmin(BI, (R + VE - 1) / VE * VE);  // i-face columns fetched
  static constexpr int TPB = BJ * BI;
  static constexpr int NB = cmax(1, cmin(4, 128 / TPB));  // bricks per CTA (7*NB producer lanes)
  static constexpr int NT = NB * TPB;
  static constexpr int al(int b) { return (b + 127) / 128 * 128; }
  static constexpr int B_C = BK * BJ * BI * ES, B_KF = R * BJ * BI * ES, B_JF = BK * R * BI * ES,
                       B_IF = BK * BJ * IW * ES;
  static constexpr int O_C = 0, O_KL = al(B_C), O_KH = O_KL + al(B_KF), O_JL = O_KH + al(B_KF),
                       O_JH = O_JL + al(B_JF), O_IL = O_JH + al(B_JF), O_IH = O_IL + al(B_IF);
  static constexpr int BRICK = O_IH + al(B_IF);  // bytes of one brick's stage buffer
  static constexpr int TX = B_C + 2 * (B_KF + B_JF + B_IF);  // bytes the copies of one brick deliver
  static constexpr int S = cmax(2, cmin(4, (48 * 1024) / (NB * BRICK)));  // pipeline stages
  // after the stage buffers: S mbarriers (8 B each), then S*NB centre brick indices
  static constexpr int META = 8 * 4 + 4 * 4 * 4;
  static constexpr int SMEM = 128 + S * NB * BRICK + META;  // + slack to align the base to 128 B
};

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
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
// Wait for the phase of the given parity to complete; gives up after about one second.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned parity) {
  unsigned long long t0 = 0;
  for (unsigned n = 0;; ++n) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((n & 63u) == 63u) {
      const unsigned long long t = global_ns();
      if (!t0) t0 = t;
      else if (t - t0 > 1000000000ull) return false;
    }
  }
}
__device__ __forceinline__ void tma_load_4d(unsigned dst, const CUtensorMap *map, int x, int y, int z, int w,
                                            unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

template <typename T, int BK, int BJ, int BI, int R, int ACC>
__global__ void __launch_bounds__(StarTmaCfg<T, BK, BJ, BI, R>::NT)
sweep_star_tma_kernel(const __grid_constant__ TmaMaps maps, const SweepArgs a, const Taps tp) {
  typedef StarTmaCfg<T, BK, BJ, BI, R> C;
  typedef typename Elem<T>::acc AT;
  constexpr int NB = C::NB, S = C::S, TPB = C::TPB, IW = C::IW, PK = BJ * BI;
  static_assert(7 * NB <= 32, "one producer lane per (brick, region)");
  static_assert(C::ES == 8 || ACC != ACCM_FF, "float-float needs FP64 storage");

  extern __shared__ __align__(16) unsigned char smem_raw[];
  const unsigned raw = smem_u32(smem_raw);
  const unsigned pad = (128u - (raw & 127u)) & 127u;
  unsigned char *sm = smem_raw + pad;  // 128-byte aligned stage buffers
  const unsigned sbase = raw + pad;
  const unsigned bar0 = sbase + S * NB * C::BRICK;
  unsigned *outb = reinterpret_cast<unsigned *>(sm + S * NB * C::BRICK + 32);  // [S][NB]

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) mbar_init(bar0 + 8 * s, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    fence_proxy_async_smem();
  }
  __syncthreads();

  const long long ngroups = ((long long)a.nlist + NB - 1) / NB;
  const int lane = threadIdx.x & 31;
  const bool prod = threadIdx.x < 32 && lane < 7 * NB;
  const int pbs = lane / 7, prg = lane - (lane / 7) * 7;  // producer lane: brick slot, region
  // region prg: 0 centre, 1 k-lo, 2 k-hi, 3 j-lo, 4 j-hi, 5 i-lo, 6 i-hi
  const int pslot = prg == 0 ? 13 : prg == 1 ? 4 : prg == 2 ? 22 : prg == 3 ? 10 : prg == 4 ? 16 : prg == 5 ? 12 : 14;
  const int pmap = (prg + 1) >> 1;
  const int px = prg == 5 ? BI - IW : 0, py = prg == 3 ? BJ - R : 0, pz = prg == 1 ? BK - R : 0;
  const int poff = prg == 0 ? C::O_C : prg == 1 ? C::O_KL : prg == 2 ? C::O_KH : prg == 3 ? C::O_JL
                 : prg == 4 ? C::O_JH : prg == 5 ? C::O_IL : C::O_IH;
  unsigned pv = 0;  // prefetched adjacency entry of this lane's (brick, region)
  int pact = 0;     // centre lanes: the brick is valid

  auto fetch = [&](long long grp) {
    pv = 0;
    pact = 0;
    if (!prod) return;
    const long long n = grp * NB + pbs;
    if (grp >= ngroups || n >= a.nlist) return;
    const unsigned b = a.blist[n];
    if (b >= a.nbricks) {
      if (prg == 0) atomicOr(a.err, FLAG_BOUNDS);
      return;
    }
    unsigned v = a.adj[(size_t)b * 27 + pslot];
    pact = prg != 0 || ((long long)v < a.out_chunks && (long long)v < a.in_chunks);
    if ((long long)v >= a.in_chunks || !pact) {
      atomicOr(a.err, FLAG_BOUNDS);
      v = 0;
    }
    pv = v;
  };
  // warp 0: copies of the group whose adjacency is in (pv, pact) into stage st
  auto issue = [&](int st) {
    const int act = __shfl_sync(0xFFFFFFFFu, pact, pbs * 7 < 32 ? pbs * 7 : 0);
    const unsigned m = __ballot_sync(0xFFFFFFFFu, prod && prg == 0 && act);
    const unsigned bar = bar0 + 8 * st;
    if (lane == 0) mbar_arrive_expect_tx(bar, (unsigned)__popc(m) * (unsigned)C::TX);
    __syncwarp();
    if (prod && act)
      tma_load_4d(sbase + (st * NB + pbs) * C::BRICK + poff, &maps.m[pmap], px, py, pz, (int)pv, bar);
    if (prod && prg == 0) outb[st * NB + pbs] = act ? pv : 0xFFFFFFFFu;
  };

  const long long g0 = blockIdx.x;
  const long long gstep = gridDim.x;
  if (threadIdx.x < 32) {
    for (int p = 0; p < S - 1; ++p) {
      const long long g = g0 + p * gstep;
      if (g < ngroups) {
        fetch(g);
        issue(p);
      }
    }
    fetch(g0 + (S - 1) * gstep);
  }

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

  int it = 0, timed_out = 0;
  for (long long g = g0; g < ngroups; g += gstep, ++it) {
    // stage (it-1) % S is free again; a wait that gave up anywhere ends the CTA's loop
    if (__syncthreads_or(timed_out)) break;
    const int st = it % S;
    if (threadIdx.x < 32) {
      const long long gi = g + (S - 1) * gstep;
      if (gi < ngroups) {
        issue((it + S - 1) % S);
        fetch(gi + gstep);
      }
    }
    if (!mbar_wait_bounded(bar0 + 8 * st, (unsigned)(it / S) & 1u)) {
      atomicOr(a.err, FLAG_TIMEOUT);
      timed_out = 1;
    }
    const unsigned ob_idx = outb[st * NB + bs];
    const bool active = !timed_out && ob_idx != 0xFFFFFFFFu;
    unsigned char *buf = sm + (st * NB + bs) * C::BRICK;
    if constexpr (ACC == ACCM_FF) {
      // in place, each thread its own elements: raw doubles -> float pairs
      if (active) {
        double *dv = reinterpret_cast<double *>(buf);
        float2 *fv = reinterpret_cast<float2 *>(buf);
        for (int e = lt; e < C::BRICK / 8; e += TPB) fv[e] = split_f64(dv[e]);
      }
      __syncthreads();
    }
    if (active) {
      T *ob = reinterpret_cast<T *>(a.out) + a.out_off + (size_t)ob_idx * a.out_step + (size_t)(j * BI + i);
      if constexpr (ACC == ACCM_FF) {
        const float2 *f = reinterpret_cast<const float2 *>(buf);
        float2 w[BK + 2 * R];
#pragma unroll
        for (int kk = 0; kk < R; ++kk) w[kk] = f[eKL + (kk * BJ + j) * BI + i];
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) w[R + kk] = f[eC + (kk * BJ + j) * BI + i];
#pragma unroll
        for (int kk = 0; kk < R; ++kk) w[R + BK + kk] = f[eKH + (kk * BJ + j) * BI + i];
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
        for (int kk = 0; kk < R; ++kk) w[kk] = to_acc(f[eKL + (kk * BJ + j) * BI + i]);
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) w[R + kk] = to_acc(f[eC + (kk * BJ + j) * BI + i]);
#pragma unroll
        for (int kk = 0; kk < R; ++kk) w[R + BK + kk] = to_acc(f[eKH + (kk * BJ + j) * BI + i]);
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
    // the float-float conversion wrote the stage through the generic proxy; order those
    // writes before the copies that refill it
    if constexpr (ACC == ACCM_FF) fence_proxy_async_smem();
  }
  // after a wait gave up: wait (bounded) for the copies still in flight into this CTA's
  // stages (iterations it-1 .. it+S-2 were issued and not consumed)
  if (__syncthreads_or(timed_out) && threadIdx.x == 0) {
    for (int q = it - 1; q < it + S - 1; ++q) {
      if (q < 0) continue;
      const long long gq = g0 + (long long)q * gstep;
      if (gq >= ngroups) break;
      if (!mbar_wait_bounded(bar0 + 8 * (q % S), (unsigned)(q / S) & 1u)) break;
    }
  }
}

// Host: encode the four box shapes over the input field.  Returns false when the field
// does not meet the bulk-tensor rules (16-byte aligned base, strides multiple of 16 bytes).
bool star_tma_maps(const SweepArgs &a, int dtype, int bk, int bj, int bi, int r, int iw, TmaMaps *maps);

template <typename T, int BK, int BJ, int BI, int R, int ACC>
int launch_star_tma(const SweepArgs &a, const Taps &tp, int dtype, cudaStream_t s, int grid_cap = 0) {
  typedef StarTmaCfg<T, BK, BJ, BI, R> C;
  static_assert(C::SMEM <= 227 * 1024, "stage buffers too large");
  TmaMaps maps;
  if (!star_tma_maps(a, dtype, BK, BJ, BI, R, C::IW, &maps)) return fail(BK_ERR_UNSUPPORTED, "field not describable to the TMA unit");
  auto kern = sweep_star_tma_kernel<T, BK, BJ, BI, R, ACC>;
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess && C::SMEM > 48 * 1024)
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, C::NT, C::SMEM);
  if (e != cudaSuccess) return cuda_fail(e, "star TMA sweep launch setup");
  if (per_sm < 1) return fail(BK_ERR_UNSUPPORTED, "star TMA sweep does not fit on an SM");
  const long long groups = ((long long)a.nlist + C::NB - 1) / C::NB;
  long long grid = (long long)sms * per_sm;
  if (grid_cap > 0 && grid > grid_cap) grid = grid_cap;
  if (grid > groups) grid = groups;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, C::NT, C::SMEM, s>>>(maps, a, tp);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "star TMA sweep launch");
  return BK_OK;
}

}  // namespace bk
