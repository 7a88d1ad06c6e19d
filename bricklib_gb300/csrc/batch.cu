// Batched form: many independent domains of different sizes and stencils advanced
// together.  One persistent sweep launch per step walks a global work list of
// (domain, brick) pairs; one ghost-fill launch per step walks a global list of
// (domain, dst, src) brick pairs; T steps are captured once into a CUDA graph and replayed.
//
// Each CTA slot (TPB = BJ*BI threads, one brick at a time) resolves its own domain: the
// domain table gives the adjacency list, the two ping-pong fields and the stencil, so one
// CTA can hold bricks of different domains and stencils.  Tiles are sized for radius 2,
// the largest of the batched shapes (7/13-point stars, 27/125-point cubes).
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "sweep_kernel.cuh"

namespace bk {

constexpr int BATCH_RMAX = 2;
constexpr int BATCH_MAX_ST = 8;
constexpr int BATCH_MAX_TAPS = 125;

struct BatchDomain {  // device table entry
  const unsigned *adj;
  unsigned nbricks;
  unsigned stencil;
  unsigned char *f0, *f1;  // field bases (dat + offset), bytes
  unsigned long long step_bytes;
  long long chunks;
};

struct BatchTaps {
  int n[BATCH_MAX_ST], fam[BATCH_MAX_ST], r[BATCH_MAX_ST];
  float cf[BATCH_MAX_ST][BATCH_MAX_TAPS];
  double c[BATCH_MAX_ST][BATCH_MAX_TAPS];
};

template <typename AT> __device__ __forceinline__ AT bcoef(const BatchTaps &tp, int s, int t);
template <> __device__ __forceinline__ float bcoef<float>(const BatchTaps &tp, int s, int t) { return tp.cf[s][t]; }
template <> __device__ __forceinline__ double bcoef<double>(const BatchTaps &tp, int s, int t) { return tp.c[s][t]; }

// Stencil point on a radius-2 tile for a star or cube of radius R (kernel tap order as bk_sweep).
template <typename AT, int EJ, int EI, int R, int FAM, int ACC>
__device__ __forceinline__ AT batch_point(const AT *__restrict__ c, const BatchTaps &tp, int s) {
  constexpr int SJ = EI, SK = EJ * EI;
  if (FAM == FAM_STAR) {
    AT v = bcoef<AT>(tp, s, 0) * c[0];
    AT comp = AT(0);
#pragma unroll
    for (int d = 1; d <= R; ++d) {
      const int t = 1 + 6 * (d - 1);
      if (ACC == ACCM_NATIVE) {
        v = fma(bcoef<AT>(tp, s, t + 0), c[d], v);
        v = fma(bcoef<AT>(tp, s, t + 1), c[-d], v);
        v = fma(bcoef<AT>(tp, s, t + 2), c[d * SJ], v);
        v = fma(bcoef<AT>(tp, s, t + 3), c[-d * SJ], v);
        v = fma(bcoef<AT>(tp, s, t + 4), c[d * SK], v);
        v = fma(bcoef<AT>(tp, s, t + 5), c[-d * SK], v);
      } else {
        neumaier(v, comp, bcoef<AT>(tp, s, t + 0) * c[d]);
        neumaier(v, comp, bcoef<AT>(tp, s, t + 1) * c[-d]);
        neumaier(v, comp, bcoef<AT>(tp, s, t + 2) * c[d * SJ]);
        neumaier(v, comp, bcoef<AT>(tp, s, t + 3) * c[-d * SJ]);
        neumaier(v, comp, bcoef<AT>(tp, s, t + 4) * c[d * SK]);
        neumaier(v, comp, bcoef<AT>(tp, s, t + 5) * c[-d * SK]);
      }
    }
    return v + comp;
  } else {
    AT v = AT(0), comp = AT(0);
#pragma unroll
    for (int dk = -R; dk <= R; ++dk)
#pragma unroll
      for (int dj = -R; dj <= R; ++dj) {
        const int t0 = ((dk + R) * (2 * R + 1) + (dj + R)) * (2 * R + 1);
        AT row = bcoef<AT>(tp, s, t0) * c[dk * SK + dj * SJ - R];
#pragma unroll
        for (int di = -R + 1; di <= R; ++di) row = fma(bcoef<AT>(tp, s, t0 + di + R), c[dk * SK + dj * SJ + di], row);
        if (dk == -R && dj == -R) v = row;
        else if (ACC == ACCM_NATIVE) v += row;
        else neumaier(v, comp, row);
      }
    return v + comp;
  }
}

template <typename T, int BK, int BJ, int BI, bool RM, int ACC>
__global__ void __launch_bounds__(sweep_threads(BJ * BI))
batch_sweep_kernel(const BatchDomain *__restrict__ doms, unsigned ndom, const uint2 *__restrict__ work, unsigned nwork,
                   int parity, const BatchTaps tp, Layout L, int *err) {
  typedef typename Elem<T>::acc AT;
  constexpr int R = BATCH_RMAX;
  constexpr int TPB = BJ * BI, NT = sweep_threads(TPB), NB = NT / TPB;
  constexpr int EK = BK + 2 * R, EJ = BJ + 2 * R, EI = BI + 2 * R, TILE = EK * EJ * EI;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  AT *tiles = reinterpret_cast<AT *>(smem_raw);
  unsigned *meta = reinterpret_cast<unsigned *>(smem_raw + sizeof(AT) * TILE * NB);  // [NB][32]

  const int slot = threadIdx.x / TPB, lt = threadIdx.x - slot * TPB;
  AT *tile = tiles + slot * TILE;
  unsigned *nbr = meta + slot * 32;  // [0..26] adjacency, [27] active, [28] domain, [29] stencil

  for (long long base = (long long)blockIdx.x * NB; base < nwork; base += (long long)gridDim.x * NB) {
    const long long n = base + slot;
    for (int sl = lt; sl < 27; sl += TPB) {
      unsigned v = 0;
      int ok = 0;
      unsigned d = 0, s = 0;
      if (n < nwork) {
        const uint2 w = work[n];
        d = w.x;
        if (d < ndom) {
          const BatchDomain &D = doms[d];
          s = D.stencil;
          if (w.y < D.nbricks && s < BATCH_MAX_ST) {
            v = D.adj[(size_t)w.y * 27 + sl];
            ok = 1;
            if (sl == 13 && (long long)v >= D.chunks) ok = 0;
            if ((long long)v >= D.chunks || !ok) { atomicOr(err, FLAG_BOUNDS); v = 0; }
          } else if (sl == 13) {
            atomicOr(err, FLAG_BOUNDS);
          }
        } else if (sl == 13) {
          atomicOr(err, FLAG_BOUNDS);
        }
      }
      nbr[sl] = v;
      if (sl == 13) {
        nbr[27] = ok;
        nbr[28] = d;
        nbr[29] = s;
      }
    }
    __syncthreads();
    const bool active = nbr[27] != 0;
    if (active) {
      const BatchDomain &D = doms[nbr[28]];
      const int s = (int)nbr[29];
      const int fam = tp.fam[s], r = tp.r[s];
      const T *in = reinterpret_cast<const T *>(parity ? D.f1 : D.f0);
      const size_t step = D.step_bytes / sizeof(T);
      for (int e = lt; e < TILE; e += TPB) {
        const int kk = e / (EJ * EI), rem = e - kk * (EJ * EI);
        const int jj = rem / EI, ii = rem - jj * EI;
        const int rk = kk - R, rj = jj - R, ri = ii - R;  // coordinates relative to the brick origin
        const int ok = rk < 0 ? -rk : (rk >= BK ? rk - BK + 1 : 0);
        const int oj = rj < 0 ? -rj : (rj >= BJ ? rj - BJ + 1 : 0);
        const int oi = ri < 0 ? -ri : (ri >= BI ? ri - BI + 1 : 0);
        // outside this stencil's reach: never read
        if (ok > r || oj > r || oi > r) continue;
        if (fam == FAM_STAR && ((ok != 0) + (oj != 0) + (oi != 0)) > 1) continue;
        const int qk = rk < 0 ? -1 : (rk >= BK ? 1 : 0);
        const int qj = rj < 0 ? -1 : (rj >= BJ ? 1 : 0);
        const int qi = ri < 0 ? -1 : (ri >= BI ? 1 : 0);
        const int lk = rk - qk * BK, lj = rj - qj * BJ, li = ri - qi * BI;
        const unsigned nb = nbr[(qk + 1) * 9 + (qj + 1) * 3 + (qi + 1)];
        const int o = RM ? (lk * BJ + lj) * BI + li : L.offset(lk, lj, li);
        tile[e] = Elem<T>::load(in + (size_t)nb * step + o);
      }
    }
    __syncthreads();
    if (active) {
      const BatchDomain &D = doms[nbr[28]];
      const int s = (int)nbr[29];
      const int fam = tp.fam[s], r = tp.r[s];
      T *out = reinterpret_cast<T *>(parity ? D.f0 : D.f1);
      const size_t step = D.step_bytes / sizeof(T);
      const int j = lt / BI, i = lt - (lt / BI) * BI;
      T *ob = out + (size_t)nbr[13] * step;
#pragma unroll 1
      for (int k = 0; k < BK; ++k) {
        const AT *c = tile + ((k + R) * EJ + (j + R)) * EI + (i + R);
        AT v;
        if (fam == FAM_STAR) v = (r == 1) ? batch_point<AT, EJ, EI, 1, FAM_STAR, ACC>(c, tp, s)
                                          : batch_point<AT, EJ, EI, 2, FAM_STAR, ACC>(c, tp, s);
        else v = (r == 1) ? batch_point<AT, EJ, EI, 1, FAM_CUBE, ACC>(c, tp, s)
                          : batch_point<AT, EJ, EI, 2, FAM_CUBE, ACC>(c, tp, s);
        const int o = RM ? (k * BJ + j) * BI + i : L.offset(k, j, i);
        Elem<T>::store(ob + o, v);
      }
    }
    __syncthreads();
  }
}

// One CTA per (domain, dst, src) entry: copies the brick field of the current input.
template <typename W>
__global__ void __launch_bounds__(256)
batch_fill_kernel(const BatchDomain *__restrict__ doms, unsigned ndom, const uint3 *__restrict__ pairs, unsigned npairs,
                  int parity, unsigned words, int *err) {
  for (unsigned p = blockIdx.x; p < npairs; p += gridDim.x) {
    const uint3 e = pairs[p];
    if (e.x >= ndom) {
      if (threadIdx.x == 0) atomicOr(err, FLAG_BOUNDS);
      continue;
    }
    const BatchDomain &D = doms[e.x];
    if ((long long)e.y >= D.chunks || (long long)e.z >= D.chunks) {
      if (threadIdx.x == 0) atomicOr(err, FLAG_BOUNDS);
      continue;
    }
    unsigned char *base = parity ? D.f1 : D.f0;
    const W *s = reinterpret_cast<const W *>(base + (size_t)e.z * D.step_bytes);
    W *d = reinterpret_cast<W *>(base + (size_t)e.y * D.step_bytes);
    for (unsigned w = threadIdx.x; w < words; w += blockDim.x) d[w] = s[w];
  }
}

template <typename T, int BK, int BJ, int BI, bool RM, int ACC>
int launch_batch_sweep(const BatchDomain *doms, unsigned ndom, const uint2 *work, unsigned nwork, int parity,
                       const BatchTaps &tp, const Layout &L, int *err, int grid_cap, cudaStream_t s) {
  typedef typename Elem<T>::acc AT;
  constexpr int TPB = BJ * BI, NT = sweep_threads(TPB), NB = NT / TPB;
  constexpr int TILE = (BK + 4) * (BJ + 4) * (BI + 4);
  constexpr size_t smem = sizeof(AT) * TILE * NB + sizeof(unsigned) * 32 * NB;
  static_assert(smem <= 227 * 1024, "batch tile too large");
  auto kern = batch_sweep_kernel<T, BK, BJ, BI, RM, ACC>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(batch)");
  }
  long long grid = ((long long)nwork + NB - 1) / NB;
  if (grid_cap > 0 && grid > grid_cap) grid = grid_cap;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, NT, smem, s>>>(doms, ndom, work, nwork, parity, tp, L, err);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "batch sweep launch");
  return BK_OK;
}

}  // namespace bk

using namespace bk;

struct bk_batch {
  int device = 0;
  Layout L{};
  bool rm = true;
  int shape = 0;
  int dtype = BK_F32;
  int acc = ACCM_NATIVE;
  unsigned ndom = 0, nwork = 0, npairs = 0;
  BatchDomain *d_doms = nullptr;
  uint2 *d_work = nullptr;
  uint3 *d_pairs = nullptr;
  BatchTaps taps{};
  int parity = 0;
  int grid_cap = 0;
  int *err = nullptr;
  std::map<std::pair<int, int>, cudaGraphExec_t> graphs;  // (steps, parity) -> graph
};

namespace bk {

static int batch_shape(const Layout &L) {
  if (L.bk == 8 && L.bj == 8 && L.bi == 8) return 0;
  if (L.bk == 4 && L.bj == 4 && L.bi == 4) return 1;
  if (L.bk == 16 && L.bj == 8 && L.bi == 8) return 2;
  if (L.bk == 8 && L.bj == 8 && L.bi == 32) return 3;
  return -1;
}

template <typename T, int ACC>
static int batch_dispatch_t(bk_batch *b, cudaStream_t s) {
#define BK_BCASE(BK_, BJ_, BI_)                                                                                  \
  return b->rm ? launch_batch_sweep<T, BK_, BJ_, BI_, true, ACC>(b->d_doms, b->ndom, b->d_work, b->nwork,        \
                                                                  b->parity, b->taps, b->L, b->err, b->grid_cap, s) \
               : launch_batch_sweep<T, BK_, BJ_, BI_, false, ACC>(b->d_doms, b->ndom, b->d_work, b->nwork,       \
                                                                   b->parity, b->taps, b->L, b->err, b->grid_cap, s);
  switch (b->shape) {
    case 0: BK_BCASE(8, 8, 8)
    case 1: BK_BCASE(4, 4, 4)
    case 2: BK_BCASE(16, 8, 8)
    case 3: BK_BCASE(8, 8, 32)
  }
#undef BK_BCASE
  return fail(BK_ERR_UNSUPPORTED, "batch: brick shape");
}

static int batch_sweep(bk_batch *b, cudaStream_t s) {
  if (b->dtype == BK_F32) return b->acc == ACCM_COMP ? batch_dispatch_t<float, ACCM_COMP>(b, s) : batch_dispatch_t<float, ACCM_NATIVE>(b, s);
  if (b->dtype == BK_BF16)
    return b->acc == ACCM_COMP ? batch_dispatch_t<__nv_bfloat16, ACCM_COMP>(b, s) : batch_dispatch_t<__nv_bfloat16, ACCM_NATIVE>(b, s);
  return batch_dispatch_t<double, ACCM_NATIVE>(b, s);
}

static int batch_fill(bk_batch *b, cudaStream_t s) {
  if (!b->npairs) return BK_OK;
  const size_t bytes = (size_t)b->L.size() * dtype_size(b->dtype);
  const unsigned grid = b->npairs < (1u << 30) ? b->npairs : (1u << 30);
  if (bytes % 16 == 0)
    batch_fill_kernel<uint4><<<grid, 256, 0, s>>>(b->d_doms, b->ndom, b->d_pairs, b->npairs, b->parity, (unsigned)(bytes / 16), b->err);
  else
    batch_fill_kernel<unsigned short><<<grid, 256, 0, s>>>(b->d_doms, b->ndom, b->d_pairs, b->npairs, b->parity, (unsigned)(bytes / 2), b->err);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "batch fill launch");
  return BK_OK;
}

static void batch_free(bk_batch *b) {
  for (auto &g : b->graphs) cudaGraphExecDestroy(g.second);
  b->graphs.clear();
  if (b->d_doms) cudaFree(b->d_doms);
  if (b->d_work) cudaFree(b->d_work);
  if (b->d_pairs) cudaFree(b->d_pairs);
  b->d_doms = nullptr;
  b->d_work = nullptr;
  b->d_pairs = nullptr;
}

}  // namespace bk

extern "C" {

int bk_batch_create(bk_batch **out, const bk_batch_domain *doms, unsigned ndom, const bk_stencil *sts, unsigned nst,
                    const bk_layout *lay, int dtype, int acc) {
  if (!out || !doms || !ndom || !sts || !nst) return fail(BK_ERR_ARG, "bk_batch_create: bad arguments");
  *out = nullptr;
  if (nst > (unsigned)BATCH_MAX_ST) return fail(BK_ERR_ARG, "bk_batch_create: at most 8 stencils");
  if (!dtype_ok(dtype)) return fail(BK_ERR_ARG, "bk_batch_create: dtype");
  Layout L;
  int s = check_layout(lay, &L);
  if (s) return s;
  const int shape = batch_shape(L);
  if (shape < 0) return fail(BK_ERR_UNSUPPORTED, "bk_batch_create: brick dims must be 8x8x8, 4x4x4, 16x8x8 or 8x8x32");
  if (L.bk < BATCH_RMAX || L.bj < BATCH_RMAX || L.bi < BATCH_RMAX) return fail(BK_ERR_UNSUPPORTED, "bricks smaller than radius 2");
  bk_batch *b = new bk_batch();
  b->L = L;
  b->rm = L.row_major();
  b->shape = shape;
  b->dtype = dtype;
  if (acc == BK_ACC_COMPENSATED && dtype != BK_F64) b->acc = ACCM_COMP;
  else if (acc == BK_ACC_NATIVE) b->acc = ACCM_NATIVE;
  else {
    delete b;
    return fail(BK_ERR_UNSUPPORTED, "bk_batch_create: accumulation mode");
  }
  // stencils: star or cube of radius <= 2, coefficients in kernel order
  for (unsigned q = 0; q < nst; ++q) {
    const bk_stencil &st = sts[q];
    int r = 0, star = 1;
    if (st.npoints < 1 || st.npoints > BATCH_MAX_TAPS) { delete b; return fail(BK_ERR_UNSUPPORTED, "batch stencil size"); }
    for (int t = 0; t < st.npoints; ++t) {
      int nz = 0;
      for (int d = 0; d < 3; ++d) {
        const int a = abs(st.offsets[t][d]);
        r = a > r ? a : r;
        nz += a != 0;
      }
      if (nz > 1) star = 0;
    }
    const bool is_star = star && st.npoints == 1 + 6 * r && r >= 1 && r <= 2;
    const bool is_cube = !star && st.npoints == (2 * r + 1) * (2 * r + 1) * (2 * r + 1) && r >= 1 && r <= 2;
    if (!is_star && !is_cube) { delete b; return fail(BK_ERR_UNSUPPORTED, "batch stencils: stars and cubes of radius 1 or 2"); }
    std::vector<int> seen(st.npoints, 0);
    for (int t = 0; t < st.npoints; ++t) {
      const int dk = st.offsets[t][0], dj = st.offsets[t][1], di = st.offsets[t][2];
      int idx;
      if (is_star) {
        const int dd = abs(dk) + abs(dj) + abs(di);
        idx = dd == 0 ? 0 : 1 + 6 * (dd - 1) + (di ? (di > 0 ? 0 : 1) : dj ? (dj > 0 ? 2 : 3) : (dk > 0 ? 4 : 5));
      } else {
        idx = ((dk + r) * (2 * r + 1) + (dj + r)) * (2 * r + 1) + (di + r);
      }
      if (idx < 0 || idx >= st.npoints || seen[idx]++) { delete b; return fail(BK_ERR_UNSUPPORTED, "batch stencil: repeated tap"); }
      b->taps.c[q][idx] = st.coeff[t];
      b->taps.cf[q][idx] = (float)st.coeff[t];
    }
    b->taps.n[q] = st.npoints;
    b->taps.fam[q] = is_star ? FAM_STAR : FAM_CUBE;
    b->taps.r[q] = r;
  }
  // domain table, work list and fill list
  std::vector<BatchDomain> hd(ndom);
  std::vector<uint2> work;
  std::vector<uint3> pairs;
  const size_t es = dtype_size(dtype);
  for (unsigned d = 0; d < ndom; ++d) {
    const bk_batch_domain &D = doms[d];
    if (!D.adj || !D.dat || D.chunks <= 0 || D.nbricks == 0 || D.stencil < 0 || (unsigned)D.stencil >= nst ||
        D.off0 + (size_t)L.size() > D.step || D.off1 + (size_t)L.size() > D.step ||
        (D.off0 < D.off1 ? D.off1 - D.off0 : D.off0 - D.off1) < (size_t)L.size() || (D.nlist && !D.blist) ||
        (D.npairs && !D.pairs)) {
      delete b;
      return fail(BK_ERR_ARG, "bk_batch_create: domain " + std::to_string(d) + " is malformed");
    }
    unsigned char *base = reinterpret_cast<unsigned char *>(D.dat);
    hd[d] = BatchDomain{D.adj, D.nbricks, (unsigned)D.stencil, base + D.off0 * es, base + D.off1 * es, D.step * es, D.chunks};
    for (unsigned n = 0; n < D.nlist; ++n) work.push_back(make_uint2(d, D.blist[n]));
    for (unsigned p = 0; p < D.npairs; ++p) pairs.push_back(make_uint3(d, D.pairs[2 * p], D.pairs[2 * p + 1]));
  }
  b->ndom = ndom;
  b->nwork = (unsigned)work.size();
  b->npairs = (unsigned)pairs.size();
  cudaError_t e = cudaGetDevice(&b->device);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_doms, sizeof(BatchDomain) * ndom);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_work, sizeof(uint2) * (work.size() ? work.size() : 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_pairs, sizeof(uint3) * (pairs.size() ? pairs.size() : 1));
  if (e == cudaSuccess) e = cudaMemcpy(b->d_doms, hd.data(), sizeof(BatchDomain) * ndom, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && work.size()) e = cudaMemcpy(b->d_work, work.data(), sizeof(uint2) * work.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && pairs.size()) e = cudaMemcpy(b->d_pairs, pairs.data(), sizeof(uint3) * pairs.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    batch_free(b);
    delete b;
    return cuda_fail(e, "bk_batch_create");
  }
  b->err = device_error_word();
  if (!b->err) {
    batch_free(b);
    delete b;
    return fail(BK_ERR_CUDA, "device error word unavailable");
  }
  *out = b;
  return BK_OK;
}

int bk_batch_set_grid(bk_batch *b, int max_ctas) {
  if (!b || max_ctas < 0) return fail(BK_ERR_ARG, "bk_batch_set_grid: bad arguments");
  b->grid_cap = max_ctas;
  for (auto &g : b->graphs) cudaGraphExecDestroy(g.second);
  b->graphs.clear();
  return BK_OK;
}

int bk_batch_run(bk_batch *b, int steps, int fill_every, int use_graph, void *stream) {
  if (!b || steps < 0 || fill_every < 0) return fail(BK_ERR_ARG, "bk_batch_run: bad arguments");
  if (steps == 0) return BK_OK;
  cudaStream_t user = as_stream(stream);
  auto enqueue = [&](cudaStream_t s) -> int {
    int st = BK_OK;
    for (int t = 0; t < steps && st == BK_OK; ++t) {
      if (fill_every && t % fill_every == 0) st = batch_fill(b, s);
      if (st == BK_OK) st = batch_sweep(b, s);
      b->parity ^= 1;
    }
    return st;
  };
  if (!use_graph) return enqueue(user);
  const auto key = std::make_pair(steps * 64 + fill_every, b->parity);
  auto it = b->graphs.find(key);
  if (it == b->graphs.end()) {
    static thread_local cudaStream_t priv = nullptr;
    static thread_local int priv_dev = -1;
    int dev = 0;
    BK_CUDA(cudaGetDevice(&dev));
    if (!priv || priv_dev != dev) {
      BK_CUDA(cudaStreamCreateWithFlags(&priv, cudaStreamNonBlocking));
      priv_dev = dev;
    }
    const int parity0 = b->parity;
    BK_CUDA(cudaStreamBeginCapture(priv, cudaStreamCaptureModeThreadLocal));
    int st = enqueue(priv);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(priv, &g);
    b->parity = parity0;
    if (st != BK_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture(batch)");
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate(batch)");
    it = b->graphs.emplace(key, exec).first;
  }
  BK_CUDA(cudaGraphLaunch(it->second, user));
  if (steps % 2) b->parity ^= 1;
  return BK_OK;
}

int bk_batch_parity(const bk_batch *b) { return b ? b->parity : -1; }

int bk_batch_destroy(bk_batch *b) {
  if (!b) return BK_OK;
  cudaDeviceSynchronize();
  batch_free(b);
  delete b;
  return BK_OK;
}

}  // extern "C"
