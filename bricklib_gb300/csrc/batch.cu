// Batched form: many independent domains of different sizes and stencils advanced
// together.  Persistent sweep launches walk a global work list of (domain, brick) pairs;
// domains that keep ghost bricks add one ghost-fill launch per step over a global list of
// (domain, dst, src) brick pairs (domains whose adjacency wraps the periodic boundary need
// none); T steps are captured once into a CUDA graph and replayed.
//
// The work list is sorted by stencil; each step launches one persistent kernel per stencil
// over that stencil's segment, specialised at compile time for its family and radius.  Each
// CTA slot (BJ*BI threads, one brick at a time) resolves its own domain from the domain
// table -- adjacency list, ping-pong fields, storage step -- so a CTA can hold bricks of
// several domains.
#include <algorithm>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "batch_common.cuh"
#include "sweep2_kernel.cuh"
#include "sweep3_kernel.cuh"

namespace bk {

// Per-stencil sweep over a segment of the global work list: the one-shot brick kernel
// (sweep_kernel) with every slot resolving its own domain -- adjacency, ping-pong fields and
// storage step come from the domain table, so one CTA can hold bricks of several domains.
template <typename T, int BK, int BJ, int BI, int R, int FAM, bool RM, int ACC>
__global__ void __launch_bounds__(sweep_threads(BJ * BI))
batch_sweep_kernel(const BatchDomain *__restrict__ doms, unsigned ndom, const uint2 *__restrict__ work, unsigned nwork,
                   int parity, const Taps tp, Layout L, int *err) {
  typedef typename TileOf<T, ACC>::type AT;
  constexpr int TPB = BJ * BI, NT = sweep_threads(TPB), NB = NT / TPB;
  constexpr int EK = BK + 2 * R, EJ = BJ + 2 * R, EI = BI + 2 * R, TILE = EK * EJ * EI;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  AT *tiles = reinterpret_cast<AT *>(smem_raw);
  unsigned *meta = reinterpret_cast<unsigned *>(smem_raw + sizeof(AT) * TILE * NB);  // [NB][32]

  const int slot = threadIdx.x / TPB, lt = threadIdx.x - slot * TPB;
  AT *tile = tiles + slot * TILE;
  unsigned *nbr = meta + slot * 32;  // [0..26] adjacency, [27] active, [28] domain

  for (long long base = (long long)blockIdx.x * NB; base < nwork; base += (long long)gridDim.x * NB) {
    const long long n = base + slot;
    for (int sl = lt; sl < 27; sl += TPB) {
      unsigned v = 0, d = 0;
      int ok = 0;
      if (n < nwork) {
        const uint2 w = work[n];
        d = w.x;
        if (d < ndom && w.y < doms[d].nbricks) {
          const BatchDomain &D = doms[d];
          v = D.adj[(size_t)w.y * 27 + sl];
          ok = 1;
          if (sl == 13 && (long long)v >= D.chunks) ok = 0;
          if ((long long)v >= D.chunks || !ok) { atomicOr(err, FLAG_BOUNDS); v = 0; }
        } else if (sl == 13) {
          atomicOr(err, FLAG_BOUNDS);
        }
      }
      nbr[sl] = v;
      if (sl == 13) {
        nbr[27] = ok;
        nbr[28] = d;
      }
    }
    __syncthreads();
    const bool active = nbr[27] != 0;
    if (active) {
      const BatchDomain &D = doms[nbr[28]];
      const T *in = reinterpret_cast<const T *>(parity ? D.f1 : D.f0);
      const size_t step = D.step_bytes / sizeof(T);
      for (int e = lt; e < TILE; e += TPB) {
        const int kk = e / (EJ * EI), rem = e - kk * (EJ * EI);
        const int jj = rem / EI, ii = rem - jj * EI;
        const int qk = kk < R ? -1 : (kk >= R + BK ? 1 : 0);
        const int qj = jj < R ? -1 : (jj >= R + BJ ? 1 : 0);
        const int qi = ii < R ? -1 : (ii >= R + BI ? 1 : 0);
        if (FAM == FAM_STAR && ((qk != 0) + (qj != 0) + (qi != 0)) > 1) continue;
        const int lk = kk - R - qk * BK, lj = jj - R - qj * BJ, li = ii - R - qi * BI;
        const unsigned nb = nbr[(qk + 1) * 9 + (qj + 1) * 3 + (qi + 1)];
        const int o = RM ? (lk * BJ + lj) * BI + li : L.offset(lk, lj, li);
        tile[e] = op_apply(TileOf<T, ACC>::load(in + (size_t)nb * step + o), tp.pre);
      }
    }
    __syncthreads();
    if (active) {
      const BatchDomain &D = doms[nbr[28]];
      T *out = reinterpret_cast<T *>(parity ? D.f0 : D.f1);
      const size_t step = D.step_bytes / sizeof(T);
      const int j = lt / BI, i = lt - (lt / BI) * BI;
      T *ob = out + (size_t)nbr[13] * step;
#pragma unroll 1
      for (int k = 0; k < BK; ++k) {
        const AT *c = tile + ((k + R) * EJ + (j + R)) * EI + (i + R);
        typename Elem<T>::acc v;
        if constexpr (ACC == ACCM_FF) v = stencil_point_ff<EJ, EI, R, FAM>(c, tp);
        else v = stencil_point<AT, EJ, EI, R, FAM, ACC>(c, tp);
        const int o = RM ? (k * BJ + j) * BI + i : L.offset(k, j, i);
        Elem<T>::store(ob + o, op_apply(v, tp.post));
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

// A domain whose cells are not whole bricks: its fields, brick grid (device) and cell counts.
struct WrapDomain {
  unsigned char *f0, *f1;
  unsigned long long step_bytes;
  const unsigned *grid;  // gk x gj x gi positions -> brick
  long long chunks;
  int g[3], n[3], r;     // brick grid (k, j, i) with one ghost brick per side, cells, stencil radius
};

// Cell-level periodic wrap of the input fields: every cell within r of a domain's box and
// outside it takes the value at its periodic image (always a cell inside the box, which
// nothing here writes).  Cell (z, y, x), z in [-r, n + r), sits in brick position
// floor(z / bk) + 1 (the ghost layer is position 0).  One block row (blockIdx.y) per domain.
template <typename W>
__global__ void __launch_bounds__(256)
wrap_fill_kernel(const WrapDomain *__restrict__ doms, unsigned ndom, int parity, Layout L, int *err) {
  const unsigned d = blockIdx.y;
  if (d >= ndom) return;
  const WrapDomain D = doms[d];
  const int r = D.r, e0 = D.n[0] + 2 * r, e1 = D.n[1] + 2 * r, e2 = D.n[2] + 2 * r;
  const long long box = (long long)e0 * e1 * e2;
  unsigned char *base = parity ? D.f1 : D.f0;
  const int bd[3] = {L.bk, L.bj, L.bi};
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < box; c += (long long)gridDim.x * blockDim.x) {
    int q[3];
    q[2] = (int)(c % e2) - r;
    q[1] = (int)((c / e2) % e1) - r;
    q[0] = (int)(c / ((long long)e2 * e1)) - r;
    if (q[0] >= 0 && q[0] < D.n[0] && q[1] >= 0 && q[1] < D.n[1] && q[2] >= 0 && q[2] < D.n[2]) continue;
    int pd[3], od[3], ps[3], os[3];
    bool ok = true;
    for (int a = 0; a < 3; ++a) {
      const int w = ((q[a] % D.n[a]) + D.n[a]) % D.n[a];  // periodic image, in the box
      pd[a] = (q[a] + bd[a]) / bd[a];                     // floor(q / b) + 1 for q >= -b
      od[a] = q[a] + bd[a] - pd[a] * bd[a];
      ps[a] = w / bd[a] + 1;
      os[a] = w - (ps[a] - 1) * bd[a];
      ok = ok && pd[a] >= 0 && pd[a] < D.g[a];
    }
    if (!ok) {  // a radius deeper than one ghost brick
      atomicOr(err, FLAG_BOUNDS);
      continue;
    }
    const unsigned bdst = D.grid[((long long)pd[0] * D.g[1] + pd[1]) * D.g[2] + pd[2]];
    const unsigned bsrc = D.grid[((long long)ps[0] * D.g[1] + ps[1]) * D.g[2] + ps[2]];
    if ((long long)bdst >= D.chunks || (long long)bsrc >= D.chunks) {
      atomicOr(err, FLAG_BOUNDS);
      continue;
    }
    const W *src = reinterpret_cast<const W *>(base + (size_t)bsrc * D.step_bytes) + L.offset(os[0], os[1], os[2]);
    W *dst = reinterpret_cast<W *>(base + (size_t)bdst * D.step_bytes) + L.offset(od[0], od[1], od[2]);
    *dst = *src;
  }
}

template <typename T, int BK, int BJ, int BI, int R, int FAM, bool RM, int ACC>
int launch_batch_sweep(const BatchDomain *doms, unsigned ndom, const uint2 *work, unsigned nwork, int parity,
                       const Taps &tp, const Layout &L, int *err, int grid_cap, cudaStream_t s) {
  typedef typename TileOf<T, ACC>::type AT;
  constexpr int TPB = BJ * BI, NT = sweep_threads(TPB), NB = NT / TPB;
  constexpr int TILE = (BK + 2 * R) * (BJ + 2 * R) * (BI + 2 * R);
  constexpr size_t smem = sizeof(AT) * TILE * NB + sizeof(unsigned) * 32 * NB;
  static_assert(smem <= 227 * 1024, "batch tile too large");
  auto kern = batch_sweep_kernel<T, BK, BJ, BI, R, FAM, RM, ACC>;
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

template <typename T, int ACC>
int batch_dispatch(const BatchStencil &bs, const BatchDomain *doms, unsigned ndom, const uint2 *work, unsigned nwork,
                   int parity, const Layout &L, int *err, int grid_cap, bool aligned, cudaStream_t s) {
  const SweepPlan &p = bs.plan;
  // the pipelined kernel in batch mode for row-major layouts and aligned fields (every field
  // base is 16-byte aligned when the storages come from cudaMalloc and offsets are whole
  // bricks); the one-shot batch kernel below serves the rest
  const bool v2 = aligned && p.rm && !p.ops && !(ACC == ACCM_FF && (p.fam == FAM_CUBE || p.r >= 4)) &&
                  !getenv("BK_SWEEP_ONESHOT");
  if (v2) {
    SweepArgs a{};
    a.nlist = nwork;
    a.err = err;
    a.L = L;
    a.doms = doms;
    a.work = work;
    a.ndom = ndom;
    a.parity = parity;
    Taps &tp = const_cast<Taps &>(bs.taps);
#define BK_B2(BK_, BJ_, BI_, R_, FAM_)                                                        \
  if (p.r == R_ && p.fam == FAM_) {                                                          \
    if (FAM_ == FAM_GENERIC) {                                                               \
      typedef Sweep2Geom<T, BK_, BJ_, BI_, R_> G;                                            \
      for (int t = 0; t < tp.n; ++t)                                                         \
        tp.toff[t] = (p.offs[t][0] * G::EJ + p.offs[t][1]) * G::EI + p.offs[t][2];           \
    }                                                                                        \
    return launch_sweep2<T, BK_, BJ_, BI_, R_, FAM_, ACC, true>(a, tp, s, grid_cap);         \
  }
#define BK_B2SET(BK_, BJ_, BI_)                                                               \
  BK_B2(BK_, BJ_, BI_, 1, FAM_STAR) BK_B2(BK_, BJ_, BI_, 2, FAM_STAR) BK_B2(BK_, BJ_, BI_, 4, FAM_STAR) \
  BK_B2(BK_, BJ_, BI_, 1, FAM_CUBE) BK_B2(BK_, BJ_, BI_, 2, FAM_CUBE)
    if (p.shape == 0) {
      if constexpr ((sizeof(T) <= 4 && (ACC == ACCM_NATIVE || ACC == ACCM_COMP)) || (sizeof(T) == 8 && ACC == ACCM_NATIVE)) {
        // mirror-symmetric cubes: the class sums streamed along each domain's runs of bricks, as
        // the plain sweep streams them (the same bits as the plain sweep of the same bricks)
        if (p.sym && p.fam == FAM_CUBE && p.r == 1) return launch_sweep2<T, 8, 8, 8, 1, FAM_CUBESYM, ACC, true, true>(a, tp, s, grid_cap);
        if (p.sym && p.fam == FAM_CUBE && p.r == 2) return launch_sweep2<T, 8, 8, 8, 2, FAM_CUBESYM, ACC, true, true>(a, tp, s, grid_cap);
      }
      if constexpr (ACC == ACCM_NATIVE) {  // mirror-symmetric cubes: the pair-sum variant
        if (p.symij && p.fam == FAM_CUBE && p.r == 1) return launch_sweep2<T, 8, 8, 8, 1, FAM_CUBESYM_IJ, ACC, true>(a, tp, s, grid_cap);
        if (p.symij && p.fam == FAM_CUBE && p.r == 2) return launch_sweep2<T, 8, 8, 8, 2, FAM_CUBESYM_IJ, ACC, true>(a, tp, s, grid_cap);
        if (p.sym && p.fam == FAM_CUBE && p.r == 1) return launch_sweep2<T, 8, 8, 8, 1, FAM_CUBESYM, ACC, true>(a, tp, s, grid_cap);
        if (p.sym && p.fam == FAM_CUBE && p.r == 2) return launch_sweep2<T, 8, 8, 8, 2, FAM_CUBESYM, ACC, true>(a, tp, s, grid_cap);
      }
      BK_B2SET(8, 8, 8)
    }
    if constexpr (ACC == ACCM_NATIVE && sizeof(T) == 4) {
      if (p.shape == 1) { BK_B2SET(4, 4, 4) }
    }
    if constexpr (ACC == ACCM_NATIVE) {  // FP32 and FP64: the brick dims the autotuner tries
      if (p.shape == 2) { BK_B2SET(16, 8, 8) }
      if (p.shape == 3) { BK_B2SET(8, 8, 32) }
    }
#undef BK_B2SET
#undef BK_B2
  }
#define BK_BC(BK_, BJ_, BI_, R_, FAM_, RM_)                                                              \
  if (p.r == R_ && p.fam == FAM_ && p.rm == RM_)                                                         \
    return launch_batch_sweep<T, BK_, BJ_, BI_, R_, FAM_, RM_, ACC>(doms, ndom, work, nwork, parity, bs.taps, L, \
                                                                     err, grid_cap, s);
#define BK_BSET(BK_, BJ_, BI_)                                                                            \
  BK_BC(BK_, BJ_, BI_, 1, FAM_STAR, true) BK_BC(BK_, BJ_, BI_, 2, FAM_STAR, true)                         \
  BK_BC(BK_, BJ_, BI_, 4, FAM_STAR, true) BK_BC(BK_, BJ_, BI_, 1, FAM_CUBE, true)                         \
  BK_BC(BK_, BJ_, BI_, 2, FAM_CUBE, true) BK_BC(BK_, BJ_, BI_, 4, FAM_GENERIC, true)                      \
  BK_BC(BK_, BJ_, BI_, 4, FAM_GENERIC, false)
  if (p.shape == 0) { BK_BSET(8, 8, 8) }
  if constexpr (ACC == ACCM_NATIVE) {
    if (p.shape == 1) { BK_BSET(4, 4, 4) }
    // FP32 and FP64: the brick dims the autotuner tries, with folds that are not row-major too
    if (p.shape == 2) { BK_BSET(16, 8, 8) }
    if (p.shape == 3) { BK_BSET(8, 8, 32) }
  }
#undef BK_BSET
#undef BK_BC
  return fail(BK_ERR_UNSUPPORTED, "batch: no kernel for this brick shape / stencil / storage / accumulation");
}

}  // namespace bk

using namespace bk;

struct bk_batch {
  int device = 0;
  Layout L{};
  int dtype = BK_F32;
  int acc = ACCM_NATIVE;
  unsigned ndom = 0, nwork = 0, npairs = 0;
  BatchDomain *d_doms = nullptr;
  uint2 *d_work = nullptr;  // sorted by stencil
  uint3 *d_pairs = nullptr;
  std::vector<BatchStencil> sts;
  std::vector<std::pair<unsigned, unsigned>> seg;  // per stencil: (first work item, count)
  int parity = 0;
  int grid_cap = 0;
  int stages = 0;  // pipeline depth of the TMA-fed star sweeps (0: the kernels' defaults)
  bool aligned = true;  // every field base and step 16-byte aligned: the pipelined kernel applies
  int *err = nullptr;
  std::map<std::pair<int, int>, cudaGraphExec_t> graphs;  // (steps, fill, parity) -> graph
  // Arena mode: every domain's storage is a range of bricks of one storage (same step and
  // field offsets).  The batch then is one brick set: a global adjacency (each domain's
  // entries shifted by its first brick), global work and fill lists, and a step is the plain
  // sweep (bk_sweep) per stencil segment and one plain ghost fill -- so star stencils take the
  // TMA-fed kernels, which read whole bricks through one tensor map of the arena.
  bool arena = false;
  unsigned total = 0;             // bricks of the arena
  unsigned *d_gadj = nullptr;     // total x 27
  unsigned *d_gwork = nullptr;    // global brick ids, sorted by stencil (segments as seg)
  unsigned *d_gpairs = nullptr;   // global (dst, src) pairs
  unsigned ngpairs = 0;
  bk_field field[2]{};            // field[0] at off0, field[1] at off1
  std::vector<bk_stencil> csts;
  int acc_mode = BK_ACC_NATIVE;
  bk_layout lay{};
  // The stencil segments of a step are independent (each writes its own domains' bricks):
  // with `concurrent` they run as parallel branches -- one stream each, forked from the
  // caller's stream and joined before the next step -- so one segment's last wave overlaps
  // the others' work, in a captured graph as in eager runs.
  int concurrent = 1;
  std::vector<cudaStream_t> lanes;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
  // domains of partial bricks: their descriptors and brick grids on the device, the cells of
  // the largest wrap box (the fill's grid size)
  WrapDomain *d_wrap = nullptr;
  unsigned *d_wgrid = nullptr;
  unsigned nwrap = 0;
  long long wrap_cells = 0;
  std::vector<int> radius;  // per stencil
};

namespace bk {

int plan_stencil(const bk_stencil *st, const Layout &L, int dtype, int acc, SweepPlan *plan, Taps *tp);

// Launchers shared with the server (serve.cu): one stencil over a work segment, and the
// batched ghost fill.
int batch_launch_sweep(const BatchStencil &bs, int dtype, const BatchDomain *doms, unsigned ndom, const uint2 *work,
                       unsigned nwork, int parity, const Layout &L, int *err, int grid_cap, bool aligned,
                       cudaStream_t s) {
  if (!nwork) return BK_OK;
  const int acc = bs.plan.acc;
  if (dtype == BK_F32)
    return acc == ACCM_COMP ? batch_dispatch<float, ACCM_COMP>(bs, doms, ndom, work, nwork, parity, L, err, grid_cap, aligned, s)
                            : batch_dispatch<float, ACCM_NATIVE>(bs, doms, ndom, work, nwork, parity, L, err, grid_cap, aligned, s);
  if (dtype == BK_F64)
    return acc == ACCM_FF ? batch_dispatch<double, ACCM_FF>(bs, doms, ndom, work, nwork, parity, L, err, grid_cap, aligned, s)
                          : batch_dispatch<double, ACCM_NATIVE>(bs, doms, ndom, work, nwork, parity, L, err, grid_cap, aligned, s);
  return fail(BK_ERR_UNSUPPORTED, "batch: BF16 storage is not instantiated");
}

int batch_launch_fill(const BatchDomain *doms, unsigned ndom, const uint3 *pairs, unsigned npairs, int parity,
                      size_t brick_bytes, int *err, cudaStream_t s) {
  if (!npairs) return BK_OK;
  const unsigned grid = npairs < (1u << 30) ? npairs : (1u << 30);
  if (brick_bytes % 16 == 0)
    batch_fill_kernel<uint4><<<grid, 256, 0, s>>>(doms, ndom, pairs, npairs, parity, (unsigned)(brick_bytes / 16), err);
  else
    batch_fill_kernel<unsigned short><<<grid, 256, 0, s>>>(doms, ndom, pairs, npairs, parity, (unsigned)(brick_bytes / 2), err);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "batch fill launch");
  return BK_OK;
}

static int batch_sweep_segment(bk_batch *b, size_t q, cudaStream_t s);

// Stencil radius of a batch stencil (the depth of the wrap fill).
static int wrap_radius(const bk_batch *b, int stencil) { return b->radius[stencil]; }

// Streams and events of the parallel segment branches (made on first use).
static int batch_lanes(bk_batch *b) {
  const size_t n = b->seg.size();
  if (b->lanes.size() == n) return BK_OK;
  if (!b->fork) BK_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
  while (b->lanes.size() < n) {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    BK_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    b->lanes.push_back(st);
    BK_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    b->joins.push_back(ev);
  }
  return BK_OK;
}

static int batch_sweep(bk_batch *b, cudaStream_t s) {
  size_t live = 0;
  for (const auto &sg : b->seg) live += sg.second ? 1 : 0;
  if (b->concurrent && live > 1) {
    int st = batch_lanes(b);
    if (st) return st;
    BK_CUDA(cudaEventRecord(b->fork, s));
    for (size_t q = 0; q < b->seg.size(); ++q) {
      if (!b->seg[q].second) continue;
      BK_CUDA(cudaStreamWaitEvent(b->lanes[q], b->fork, 0));
      if ((st = batch_sweep_segment(b, q, b->lanes[q]))) return st;
      BK_CUDA(cudaEventRecord(b->joins[q], b->lanes[q]));
      BK_CUDA(cudaStreamWaitEvent(s, b->joins[q], 0));
    }
    return BK_OK;
  }
  for (size_t q = 0; q < b->seg.size(); ++q) {
    const int st = batch_sweep_segment(b, q, s);
    if (st) return st;
  }
  return BK_OK;
}

// One stencil segment of a step: a plain sweep over the arena's global list, or the batch-mode
// kernel over (domain, brick) work items.
static int batch_sweep_segment(bk_batch *b, size_t q, cudaStream_t s) {
  const unsigned first = b->seg[q].first, count = b->seg[q].second;
  if (!count) return BK_OK;
  if (b->arena) {
    const bk_field &fin = b->field[b->parity], &fout = b->field[b->parity ^ 1];
    const int prev = pipeline_depth_override();
    set_pipeline_depth_override(b->stages);
    const int st = bk_sweep(b->d_gadj, b->total, &fin, &fout, b->d_gwork + first, count, &b->csts[q], &b->lay,
                            b->acc_mode, s);
    set_pipeline_depth_override(prev);
    return st;
  }
  return batch_launch_sweep(b->sts[q], b->dtype, b->d_doms, b->ndom, b->d_work + first, count, b->parity, b->L,
                            b->err, b->grid_cap, b->aligned, s);
}

static int batch_wrap_fill(bk_batch *b, cudaStream_t s) {
  if (!b->nwrap) return BK_OK;
  const unsigned bx = (unsigned)std::min<long long>((b->wrap_cells + 255) / 256, 64);
  const dim3 grid(bx, b->nwrap);
  const size_t es = dtype_size(b->dtype);
  if (es == 8) wrap_fill_kernel<unsigned long long><<<grid, 256, 0, s>>>(b->d_wrap, b->nwrap, b->parity, b->L, b->err);
  else if (es == 4) wrap_fill_kernel<unsigned><<<grid, 256, 0, s>>>(b->d_wrap, b->nwrap, b->parity, b->L, b->err);
  else wrap_fill_kernel<unsigned short><<<grid, 256, 0, s>>>(b->d_wrap, b->nwrap, b->parity, b->L, b->err);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "batch wrap fill launch");
  return BK_OK;
}

static int batch_fill(bk_batch *b, cudaStream_t s) {
  int st = batch_wrap_fill(b, s);
  if (st) return st;
  if (b->arena) return b->ngpairs ? bk_ghost_fill(b->d_gpairs, b->ngpairs, &b->field[b->parity], &b->lay, s) : BK_OK;
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
  if (b->d_wrap) cudaFree(b->d_wrap);
  if (b->d_wgrid) cudaFree(b->d_wgrid);
  b->d_wrap = nullptr;
  b->d_wgrid = nullptr;
  for (auto st : b->lanes) cudaStreamDestroy(st);
  for (auto ev : b->joins) cudaEventDestroy(ev);
  if (b->fork) cudaEventDestroy(b->fork);
  b->lanes.clear();
  b->joins.clear();
  b->fork = nullptr;
  if (b->d_doms) cudaFree(b->d_doms);
  if (b->d_work) cudaFree(b->d_work);
  if (b->d_pairs) cudaFree(b->d_pairs);
  if (b->d_gadj) cudaFree(b->d_gadj);
  if (b->d_gwork) cudaFree(b->d_gwork);
  if (b->d_gpairs) cudaFree(b->d_gpairs);
  b->d_doms = nullptr;
  b->d_work = nullptr;
  b->d_pairs = nullptr;
  b->d_gadj = b->d_gwork = b->d_gpairs = nullptr;
}

// Adjacency of one arena domain: its entries shifted by the domain's first brick; an entry
// outside the domain is clamped to the domain's brick 0 and flagged, as the sweeps do.
__global__ void arena_adj_kernel(const unsigned *__restrict__ adj, unsigned nbricks, unsigned first,
                                 unsigned *__restrict__ gadj, int *err) {
  const size_t n = (size_t)nbricks * 27;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    unsigned v = adj[p];
    if (v >= nbricks) {
      atomicOr(err, FLAG_BOUNDS);
      v = 0;
    }
    gadj[(size_t)first * 27 + p] = first + v;
  }
}

// Arena mode when every domain's storage is a brick range of one storage (see bk_batch);
// BK_OK also when the domains are not laid out that way (the batch then stays per domain).
static int batch_arena(bk_batch *b, const bk_batch_domain *doms, unsigned ndom, const bk_stencil *sts, unsigned nst,
                       const bk_layout *lay, int acc) {
  const size_t es = dtype_size(b->dtype);
  const bk_batch_domain &D0 = doms[0];
  uintptr_t base = reinterpret_cast<uintptr_t>(D0.dat);
  for (unsigned d = 1; d < ndom; ++d) base = std::min(base, reinterpret_cast<uintptr_t>(doms[d].dat));
  const size_t stepb = D0.step * es;
  std::vector<std::pair<unsigned long long, unsigned long long>> ranges(ndom);  // (first brick, end)
  for (unsigned d = 0; d < ndom; ++d) {
    const bk_batch_domain &D = doms[d];
    const uintptr_t p = reinterpret_cast<uintptr_t>(D.dat);
    if (D.step != D0.step || D.off0 != D0.off0 || D.off1 != D0.off1 || (p - base) % stepb || D.nbricks > (unsigned long long)D.chunks)
      return BK_OK;
    ranges[d] = {(p - base) / stepb, (p - base) / stepb + (unsigned long long)D.chunks};
  }
  std::vector<std::pair<unsigned long long, unsigned long long>> sorted = ranges;
  std::sort(sorted.begin(), sorted.end());
  for (unsigned d = 1; d < ndom; ++d)
    if (sorted[d].first < sorted[d - 1].second) return BK_OK;  // overlapping domains
  unsigned long long total = 0, sum = 0;
  for (const auto &r : ranges) {
    total = std::max(total, r.second);
    sum += r.second - r.first;
  }
  // the ranges must tile the arena exactly (separate allocations that merely happen to be
  // step-aligned would leave gaps the global tables would span)
  if (total != sum || total > 0x7FFFFFFFull) return BK_OK;
  // host lists: global work per stencil, global fill pairs
  std::vector<std::vector<unsigned>> per_st(nst);
  std::vector<unsigned> gpairs;
  for (unsigned d = 0; d < ndom; ++d) {
    const bk_batch_domain &D = doms[d];
    const unsigned first = (unsigned)ranges[d].first;
    for (unsigned n = 0; n < D.nlist; ++n)
      per_st[D.stencil].push_back(D.blist[n] < D.nbricks ? first + D.blist[n] : 0xFFFFFFFFu);
    for (unsigned q = 0; q < D.npairs; ++q) {
      const unsigned dst = D.pairs[2 * q], src = D.pairs[2 * q + 1];
      gpairs.push_back(dst < D.nbricks ? first + dst : 0xFFFFFFFFu);
      gpairs.push_back(src < D.nbricks ? first + src : 0xFFFFFFFFu);
    }
  }
  std::vector<unsigned> gwork;
  b->seg.clear();
  for (unsigned q = 0; q < nst; ++q) {
    b->seg.emplace_back((unsigned)gwork.size(), (unsigned)per_st[q].size());
    gwork.insert(gwork.end(), per_st[q].begin(), per_st[q].end());
  }
  cudaError_t e = cudaMalloc(&b->d_gadj, sizeof(unsigned) * 27 * (size_t)total);
  if (e == cudaSuccess) e = cudaMemset(b->d_gadj, 0, sizeof(unsigned) * 27 * (size_t)total);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_gwork, sizeof(unsigned) * (gwork.size() ? gwork.size() : 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_gpairs, sizeof(unsigned) * (gpairs.size() ? gpairs.size() : 2));
  if (e == cudaSuccess && gwork.size())
    e = cudaMemcpy(b->d_gwork, gwork.data(), sizeof(unsigned) * gwork.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && gpairs.size())
    e = cudaMemcpy(b->d_gpairs, gpairs.data(), sizeof(unsigned) * gpairs.size(), cudaMemcpyHostToDevice);
  for (unsigned d = 0; d < ndom && e == cudaSuccess; ++d) {
    const size_t n = (size_t)doms[d].nbricks * 27;
    const unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 4096);
    arena_adj_kernel<<<grid, 256>>>(doms[d].adj, doms[d].nbricks, (unsigned)ranges[d].first, b->d_gadj, b->err);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "bk_batch_create (arena)");
  b->total = (unsigned)total;
  b->ngpairs = (unsigned)(gpairs.size() / 2);
  void *dat = reinterpret_cast<void *>(base);
  b->field[0] = bk_field{dat, (long)total, D0.step, D0.off0, b->dtype};
  b->field[1] = bk_field{dat, (long)total, D0.step, D0.off1, b->dtype};
  b->csts.assign(sts, sts + nst);
  b->acc_mode = acc;
  b->lay = *lay;
  b->arena = true;
  return BK_OK;
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
  bk_batch *b = new bk_batch();
  b->L = L;
  b->dtype = dtype;
  b->sts.resize(nst);
  for (unsigned q = 0; q < nst; ++q) {
    if ((s = plan_stencil(&sts[q], L, dtype, acc, &b->sts[q].plan, &b->sts[q].taps))) {
      delete b;
      return s;
    }
  }
  b->acc = b->sts[0].plan.acc;
  for (unsigned q = 0; q < nst; ++q) {
    int r = 0;
    for (int t = 0; t < sts[q].npoints; ++t)
      for (int a = 0; a < 3; ++a) r = std::max(r, std::abs(sts[q].offsets[t][a]));
    b->radius.push_back(r);
  }
  // domain table, work list sorted by stencil, fill list
  std::vector<BatchDomain> hd(ndom);
  std::vector<std::vector<uint2>> per_st(nst);
  std::vector<uint3> pairs;
  std::vector<WrapDomain> wdoms;
  std::vector<unsigned> wgrids;
  const size_t es = dtype_size(dtype);
  for (unsigned d = 0; d < ndom; ++d) {
    const bk_batch_domain &D = doms[d];
    const size_t gap = D.off0 < D.off1 ? D.off1 - D.off0 : D.off0 - D.off1;
    if (!D.adj || !D.dat || D.chunks <= 0 || D.nbricks == 0 || D.stencil < 0 || (unsigned)D.stencil >= nst ||
        D.off0 + (size_t)L.size() > D.step || D.off1 + (size_t)L.size() > D.step || gap < (size_t)L.size() ||
        (D.nlist && !D.blist) || (D.npairs && !D.pairs)) {
      delete b;
      return fail(BK_ERR_ARG, "bk_batch_create: domain " + std::to_string(d) + " is malformed");
    }
    unsigned char *base = reinterpret_cast<unsigned char *>(D.dat);
    hd[d] = BatchDomain{D.adj, D.nbricks, (unsigned)D.stencil, base + D.off0 * es, base + D.off1 * es, D.step * es, D.chunks};
    if (D.n[0] || D.n[1] || D.n[2]) {
      const int bdim[3] = {L.bk, L.bj, L.bi};
      bool ok = D.grid != nullptr;
      for (int a = 0; a < 3 && ok; ++a)
        ok = D.n[a] > 0 && D.gdims[a] == (D.n[a] + bdim[a] - 1) / bdim[a] + 2 && wrap_radius(b, D.stencil) <= bdim[a] &&
             wrap_radius(b, D.stencil) <= D.n[a];
      if (!ok) {
        delete b;
        return fail(BK_ERR_ARG, "bk_batch_create: domain " + std::to_string(d) +
                                    ": partial bricks need the grid, n cells per axis (at least the stencil radius) "
                                    "and gdims = n / bdim rounded up + 2 (stencil radius at most a brick)");
      }
      WrapDomain w{};
      w.f0 = base + D.off0 * es;
      w.f1 = base + D.off1 * es;
      w.step_bytes = D.step * es;
      w.chunks = D.chunks;
      w.r = wrap_radius(b, D.stencil);
      for (int a = 0; a < 3; ++a) {
        w.g[a] = (int)D.gdims[a];
        w.n[a] = (int)D.n[a];
      }
      const size_t gsize = (size_t)D.gdims[0] * D.gdims[1] * D.gdims[2];
      w.grid = reinterpret_cast<const unsigned *>(wgrids.size());  // offset, rebased after the upload
      wgrids.insert(wgrids.end(), D.grid, D.grid + gsize);
      wdoms.push_back(w);
      b->wrap_cells = std::max<long long>(b->wrap_cells, (long long)(w.n[0] + 2 * w.r) * (w.n[1] + 2 * w.r) *
                                                             (w.n[2] + 2 * w.r));
    }
    if ((reinterpret_cast<uintptr_t>(base) | (D.off0 * es) | (D.off1 * es) | (D.step * es)) % 16) b->aligned = false;
    for (unsigned n = 0; n < D.nlist; ++n) per_st[D.stencil].push_back(make_uint2(d, D.blist[n]));
    for (unsigned p = 0; p < D.npairs; ++p) pairs.push_back(make_uint3(d, D.pairs[2 * p], D.pairs[2 * p + 1]));
  }
  std::vector<uint2> work;
  for (unsigned q = 0; q < nst; ++q) {
    b->seg.emplace_back((unsigned)work.size(), (unsigned)per_st[q].size());
    work.insert(work.end(), per_st[q].begin(), per_st[q].end());
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
  if (e == cudaSuccess && wdoms.size()) {
    e = cudaMalloc(&b->d_wgrid, sizeof(unsigned) * wgrids.size());
    if (e == cudaSuccess) e = cudaMemcpy(b->d_wgrid, wgrids.data(), sizeof(unsigned) * wgrids.size(), cudaMemcpyHostToDevice);
    for (auto &w : wdoms) w.grid = b->d_wgrid + reinterpret_cast<size_t>(w.grid);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_wrap, sizeof(WrapDomain) * wdoms.size());
    if (e == cudaSuccess) e = cudaMemcpy(b->d_wrap, wdoms.data(), sizeof(WrapDomain) * wdoms.size(), cudaMemcpyHostToDevice);
    b->nwrap = (unsigned)wdoms.size();
  }
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
  if ((s = batch_arena(b, doms, ndom, sts, nst, lay, acc)) != BK_OK) {
    batch_free(b);
    delete b;
    return s;
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

int bk_batch_set_stages(bk_batch *b, int stages) {
  if (!b || (stages != 0 && (stages < 2 || stages > TMA_MAX_STAGES)))
    return fail(BK_ERR_ARG, "bk_batch_set_stages: stages must be 0 or 2..4");
  b->stages = stages;
  for (auto &g : b->graphs) cudaGraphExecDestroy(g.second);
  b->graphs.clear();
  return BK_OK;
}

int bk_batch_set_concurrent(bk_batch *b, int on) {
  if (!b) return fail(BK_ERR_ARG, "bk_batch_set_concurrent: bad arguments");
  b->concurrent = on ? 1 : 0;
  for (auto &g : b->graphs) cudaGraphExecDestroy(g.second);
  b->graphs.clear();
  return BK_OK;
}

int bk_batch_parity(const bk_batch *b) { return b ? b->parity : -1; }

int bk_batch_is_arena(const bk_batch *b) { return b ? (b->arena ? 1 : 0) : -1; }

int bk_batch_destroy(bk_batch *b) {
  if (!b) return BK_OK;
  cudaDeviceSynchronize();
  batch_free(b);
  delete b;
  return BK_OK;
}

}  // extern "C"
