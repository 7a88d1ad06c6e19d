// Four-dimensional bricks (weak/main-4d.cpp): Brick<Dim<4,4,4,4>, Dim<fold>> with a runtime
// tap list, e.g. the 9-point star of stencils/mpi9pt.py.  Persistent CTAs of 128 threads, two
// outputs per thread: the part of a brick's neighbourhood the stencil reads (centre and faces for
// a star, the whole radius-R box otherwise) is gathered into a shared-memory tile by asynchronous
// copies while earlier bricks are computed (two bricks in flight for FP32 at radius 1, one
// otherwise).  The copies follow a table the CTA builds once from the layout, one word per copy:
// a 16-byte copy where a block of a tile row's centre (or a whole i halo) is consecutive and
// aligned in its brick, else one copy per element.  Out-of-range list entries, and out-of-range
// adjacency entries in the slots the tile reads, are clamped / skipped and raise the device error
// flag, as in the 3-D kernels.
#include "bk_common.cuh"

namespace bk {

struct Layout4 {
  int b[4], f[4];  // (l, k, j, i), outermost first
  int lf[4];       // log2 of the folds: a fold divides the brick's 4, so it is 1, 2 or 4
  __host__ __device__ __forceinline__ int size() const { return b[0] * b[1] * b[2] * b[3]; }
  // in-brick offset of (l, k, j, i), each in [0, 4): folds right-aligned, vector index over
  // the fold blocks, lane inside (the reference's accessor formula, with shifts and masks)
  __host__ __device__ __forceinline__ int offset(int l, int k, int j, int i) const {
    const int vl = f[0] * f[1] * f[2] * f[3];
    const int vec = ((((l >> lf[0]) * (4 >> lf[1]) + (k >> lf[1])) * (4 >> lf[2]) + (j >> lf[2])) * (4 >> lf[3])) +
                    (i >> lf[3]);
    const int lane = (((l & (f[0] - 1)) * f[1] + (k & (f[1] - 1))) * f[2] + (j & (f[2] - 1))) * f[3] + (i & (f[3] - 1));
    return vec * vl + lane;
  }
};

struct Taps4 {
  int n;
  int toff[BK_MAX_TAPS4];  // tile offsets (Tile4::toff)
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

// Tile of one brick's neighbourhood: E = 4 + 2R rows along each of l, k, j.  A row holds its 4
// centre elements from C0 (a whole number of 16-byte blocks, >= R) and R halo elements either
// side; the rows of an (l, k) plane are P apart (P >= 4 + 2R, a whole number of blocks) and the
// planes Q apart, so row (l, k, j) spans [(l E + k) Q + j P + C0 - R, ... + C0 + 4 + R): a row's
// i-hi halo may share a 16-byte block with the unused front of the next row, and every centre
// block starts 16-byte aligned.  For 4-byte storage Q = E P + 4: the two k planes a warp's
// points span then fall on complementary shared-memory banks (E P alone is 0 or 16 mod 32).
// A tap (dl, dk, dj, di) is the fixed tile offset (dl E + dk) Q + dj P + di from any point.
// STARONLY: the table holds a star's centre and face elements only.
template <typename T, int R, bool STARONLY>
struct Tile4 {
  static constexpr int ES = (int)sizeof(T), VE = 16 / ES;
  static constexpr int C0 = (R + VE - 1) / VE * VE, P = (4 + 2 * R + VE - 1) / VE * VE;
  static constexpr int E = 4 + 2 * R, ROWS = E * E * E, NBC = 4 / VE, NSEG = NBC + 2;
  static constexpr int Q = E * P + (ES == 4 ? 4 : 0);
  static constexpr int TILE = (E * E - 1) * Q + (E - 1) * P + C0 + 4 + R;
  // copy table words: one per tile element the stencil can read, at most
  static constexpr int NTAB = STARONLY ? 256 + 512 * R : ROWS * (4 + 2 * R);
  // tile buffers: S - 1 bricks in flight (FP64 sweeps are bound by the FP64 pipe and keep the
  // resident CTAs instead)
  static constexpr int S = (R == 1 && ES == 4) ? 3 : 2;
  static constexpr int TILEA = (TILE + VE - 1) / VE * VE;  // buffer stride, whole 16-byte blocks
  static constexpr size_t SMEM = S * (size_t)TILEA * ES + (size_t)NTAB * 4;
  __host__ __device__ static constexpr int toff(int dl, int dk, int dj, int di) { return (dl * E + dk) * Q + dj * P + di; }
};

// Persistent CTAs walk the brick list with a stride of the grid, pipelined over S tile buffers:
// while brick j is computed, the neighbourhoods of bricks j+1 .. j+S-1 are being gathered by
// asynchronous copies, brick j+S's list and adjacency entries are staged into shared memory
// (S + 1 adjacency slots, so no slot is rewritten while read), brick j+S+1's and j+S+2's
// adjacency entries and brick j+S+3's list entry are in flight in registers.  Only the
// adjacency slots the tile reads are staged (9 of 81 for a star), by the CTA's last threads.
// One block barrier per brick.
// star: every tap has at most one non-zero offset (only centre and face elements are read);
// canon: the taps are exactly the star of radius R, passed in the order centre, then along l,
// k, j, i the distances -R..-1, 1..R (tile offsets known at compile time);
// vec: the input field's bricks start 16-byte aligned (16-byte copies allowed).
constexpr int NT4 = 128;  // threads per CTA, each computing two of a brick's 256 points

template <typename T, typename AT, int R, bool CANON>
__global__ void __launch_bounds__(NT4)
sweep4_kernel(const unsigned *__restrict__ adj, unsigned nbricks, const T *__restrict__ in, unsigned long long in_step,
              long long in_chunks, T *__restrict__ out, unsigned long long out_step, long long out_chunks,
              const unsigned *__restrict__ blist, unsigned nlist, const Layout4 L, const Taps4 tp, int star, int vec,
              int *err) {
  static_assert(sizeof(T) == sizeof(AT) && (sizeof(T) == 4 || sizeof(T) == 8), "the tile holds the storage type");
  typedef Tile4<T, R, CANON> G;
  constexpr int B = 4, E = G::E, VE = G::VE, C0 = G::C0, NBC = G::NBC, NSEG = G::NSEG;
  constexpr int NTAB = G::NTAB, TILEA = G::TILEA, S = G::S, NSLOT = S + 1;
  static_assert(G::TILE < (1 << 14), "tile offsets take 14 bits");
  constexpr unsigned NONE = 0xFFFFFFFFu;
  // dynamic shared memory: tile[S][TILEA], then the copy table, one word per copy: adjacency
  // slot (7 bits) | tile offset (14) << 7 | in-brick offset of the (first) element (8) << 21.
  // 16-byte copies fill it from the front (n16 of them), one-element copies from the back (nel).
  extern __shared__ __align__(16) unsigned char smem4[];
  T(*tile)[TILEA] = reinterpret_cast<T(*)[TILEA]>(smem4);
  unsigned *plan = reinterpret_cast<unsigned *>(smem4 + S * TILEA * sizeof(T));
  __shared__ unsigned nbr[NSLOT][81];
  __shared__ unsigned n16, nel, needm[3], nneed;
  __shared__ unsigned char need[81];  // the adjacency slots the tile reads, the centre (40) first
  // FP64: the coefficients of a star of this radius and -0.0, read into per-thread registers
  // (on GB300 a DFMA with a constant-bank coefficient, and a DMUL, issue a fifth slower)
  constexpr int MT = 8 * R + 1;
  __shared__ double cs4[MT + 1];
  const int t = threadIdx.x;
  if (t == 0) {
    n16 = nel = 0;
    needm[0] = needm[2] = 0;
    needm[1] = 1u << (40 - 32);
  }
  if (t <= MT) cs4[t] = t == MT ? tp.mzero : t < tp.n ? tp.c[t] : 0.0;
  __syncthreads();
  for (int e = t; e < G::ROWS * NSEG; e += blockDim.x) {
    const int row = e / NSEG, seg = e - row * NSEG;
    const int l = row / (E * E) - R, k = (row / E) % E - R, j = row % E - R;  // in-brick, may lie outside
    const int ql = l < 0 ? -1 : (l >= B ? 1 : 0), qk = k < 0 ? -1 : (k >= B ? 1 : 0);
    const int qj = j < 0 ? -1 : (j >= B ? 1 : 0);
    // the segment: one 16-byte block of the row's centre, or the R halo elements on one side
    const int qi = seg < NBC ? 0 : (seg == NBC ? -1 : 1);
    const int i0 = seg < NBC ? seg * VE : (seg == NBC ? -R : B);
    const int cnt = seg < NBC ? VE : R;
    const int dst0 = (row / E) * G::Q + (row % E) * G::P + C0 + i0;
    const int outside = (ql != 0) + (qk != 0) + (qj != 0) + (qi != 0);
    if (star && outside > 1) continue;  // a star reads centre and face elements only
    const unsigned slot = (unsigned)(((ql + 1) * 3 + (qk + 1)) * 9 + (qj + 1) * 3 + (qi + 1));
    int so[VE];
    bool consecutive = true;
#pragma unroll
    for (int q = 0; q < VE; ++q) {
      so[q] = q < cnt ? L.offset(l - ql * B, k - qk * B, j - qj * B, i0 + q - qi * B) : 0;
      if (q < cnt && so[q] != so[0] + q) consecutive = false;
    }
    atomicOr(&needm[slot >> 5], 1u << (slot & 31u));
    if (vec && consecutive && cnt == VE && so[0] % VE == 0 && dst0 % VE == 0) {
      plan[atomicAdd(&n16, 1u)] = slot | ((unsigned)dst0 << 7) | ((unsigned)so[0] << 21);
    } else {
#pragma unroll
      for (int q = 0; q < VE; ++q)
        if (q < cnt) plan[NTAB - 1 - atomicAdd(&nel, 1u)] = slot | ((unsigned)(dst0 + q) << 7) | ((unsigned)so[q] << 21);
    }
  }
  __syncthreads();
  if (t == 0) {
    unsigned c = 0;
    need[c++] = 40;
    for (int q = 0; q < 81; ++q)
      if (q != 40 && ((needm[q >> 5] >> (q & 31)) & 1u)) need[c++] = (unsigned char)q;
    nneed = c;
  }
  __syncthreads();
  // list positions in 32 bits: the host holds lists below 2^31 entries, so n + (S + 3) gs stays
  // far below 2^32
  const unsigned gs = gridDim.x;
  // Staging of list entry n's adjacency entries: thread t < nneed holds slot need[t].  check()
  // gives the staged value: slot 40 carries NONE for a brick that is not computed (past the
  // list, or out of range: flagged).
  // (the last threads of the CTA: warp 0 issues the most copies)
  const int nstage = (int)nneed, ts = NT4 - 1 - t;
  const bool stager = ts < nstage;
  const unsigned myslot = stager ? need[ts] : 0u;
  const bool ctr = stager && myslot == 40u;
  auto load_b = [&](unsigned n) -> unsigned { return (stager && n < nlist) ? blist[n] : NONE; };
  auto load_v = [&](unsigned b) -> unsigned { return (stager && b < nbricks) ? adj[(size_t)b * 81 + myslot] : 0u; };
  auto check = [&](unsigned n, unsigned b, unsigned v) -> unsigned {
    if (n >= nlist) return ctr ? NONE : 0u;
    if (b >= nbricks) {
      if (ctr) {
        atomicOr(err, FLAG_BOUNDS);
        return NONE;
      }
      return 0u;
    }
    if ((long long)v >= in_chunks || (ctr && (long long)v >= out_chunks)) {
      if (stager) atomicOr(err, FLAG_BOUNDS);
      return ctr ? NONE : 0u;
    }
    return v;
  };
  auto issue = [&](int slot, int buf) {
    const unsigned *nb = nbr[slot];
    if (nb[40] != NONE) {
      const unsigned base = (unsigned)__cvta_generic_to_shared(&tile[buf][0]);
      const int a16 = (int)n16, ael = (int)nel;
      // entries t, t + NT4, ... of each part of the table (compile-time counts per thread)
      constexpr int NP16 = (G::ROWS * NSEG + NT4 - 1) / NT4, NPEL = (NTAB + NT4 - 1) / NT4;
#pragma unroll
      for (int m = 0; m < NP16; ++m) {
        const int e = t + NT4 * m;
        if (e >= a16) break;
        const unsigned w = plan[e];
        cp_async_elem<16>(base + ((w >> 7) & 0x3FFFu) * (unsigned)sizeof(T), in + (size_t)nb[w & 127u] * in_step + (w >> 21));
      }
#pragma unroll
      for (int m = 0; m < NPEL; ++m) {
        const int e = t + NT4 * m;
        if (e >= ael) break;
        const unsigned w = plan[NTAB - 1 - e];
        cp_async_elem<sizeof(T)>(base + ((w >> 7) & 0x3FFFu) * (unsigned)sizeof(T),
                                 in + (size_t)nb[w & 127u] * in_step + (w >> 21));
      }
    }
    cp_async_commit4();
  };
  const unsigned n0 = blockIdx.x;
  // bricks n0 .. n0 + (S-1) gs staged into slots 0 .. S-1
#pragma unroll
  for (int q = 0; q < S; ++q) {
    const unsigned nq = n0 + q * gs;
    const unsigned bq = load_b(nq);
    const unsigned aq = check(nq, bq, load_v(bq));
    if (stager) nbr[q][myslot] = aq;
  }
  // in flight: list entries n0 + S gs (bA), + (S+1) gs (bB), + (S+2) gs (bC); adjacency of bA, bB
  unsigned bA = load_b(n0 + S * gs), bB = load_b(n0 + (S + 1) * gs), bC = load_b(n0 + (S + 2) * gs);
  unsigned vA = load_v(bA), vB = load_v(bB);
  __syncthreads();  // the first S adjacency slots
#pragma unroll
  for (int q = 0; q + 1 < S; ++q) issue(q, q);
  // this thread's output elements t and t + NT4: their tile positions and in-brick offsets
  static_assert(2 * NT4 == B * B * B * B, "two points per thread");
  int ctile[2], oofs[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int pt = t + NT4 * h;
    const int oi = pt % B, oj = (pt / B) % B, ok = (pt / (B * B)) % B, ol = pt / (B * B * B);
    ctile[h] = G::toff(ol + R, ok + R, oj + R, oi) + C0;
    oofs[h] = L.offset(ol, ok, oj, oi);
  }
  // the tap list of a star of this radius fits MT entries: offsets held in registers for the
  // whole kernel (the loop over a runtime count read them from the parameters per tap)
  int toffr[CANON ? 1 : MT];
#pragma unroll
  for (int q = 0; q < (CANON ? 1 : MT); ++q) toffr[q] = q < tp.n ? tp.toff[q] : 0;
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
  int sc = 0, sb = 0;  // slot and buffer of brick jb (jb mod NSLOT, jb mod S)
  for (unsigned n = n0; n < nlist; n += gs) {
    const int sl = sc + S - 1 - (sc + S - 1 >= NSLOT ? NSLOT : 0);  // brick jb + S - 1
    const int bl = sb == 0 ? S - 1 : sb - 1;                        // its buffer, (jb + S - 1) mod S
    const int sf = sc == 0 ? NSLOT - 1 : sc - 1;                    // brick jb + S: slot (jb - 1) mod NSLOT
    cp_async_wait4<S - 2>();  // this thread's copies for brick jb have landed
    // one barrier per brick: everybody's copies for brick jb have landed, and everybody is done
    // with brick jb-1's compute (its buffer bl and slot sf) and has staged brick jb+S-1 (slot sl)
    __syncthreads();
    issue(sl, bl);
    const unsigned staged = check(n + S * gs, bA, vA);
    if (stager) nbr[sf][myslot] = staged;
    bA = bB;
    vA = vB;
    bB = bC;
    vB = load_v(bC);
    bC = load_b(n + (S + 3) * gs);
    const int cur = sc, buf = sb;
    sc = sc + 1 == NSLOT ? 0 : sc + 1;
    sb = sb + 1 == S ? 0 : sb + 1;
    const unsigned ob = nbr[cur][40];
    if (ob != NONE) {
      const T *c0 = tile[buf] + ctile[0], *c1 = tile[buf] + ctile[1];
      AT v0, v1;
      if constexpr (CANON) {
        // the star of radius R in its canonical order: every tile offset a constant
        const AT k0 = F64 ? cr[0] : coefq(0);
        v0 = first(k0, c0[0]);
        v1 = first(k0, c1[0]);
#pragma unroll
        for (int ax = 0; ax < 4; ++ax)
#pragma unroll
          for (int d = -R; d <= R; ++d) {
            if (d == 0) continue;
            const int q = 1 + 2 * R * ax + (d < 0 ? d + R : d + R - 1);
            const int o = d * (ax == 0 ? E * G::Q : ax == 1 ? G::Q : ax == 2 ? G::P : 1);
            const AT kq = F64 ? cr[q] : coefq(q);
            v0 = fma(kq, c0[o], v0);
            v1 = fma(kq, c1[o], v1);
          }
      } else if (tp.n <= MT) {
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
  typedef Tile4<T, R, false> G;  // the tile geometry (the table size depends on canon)
  for (int t = 0; t < tp.n; ++t) tp.toff[t] = G::toff(offs[t][0], offs[t][1], offs[t][2], offs[t][3]);
  // the star of radius R, each tap once: coefficients passed in the canonical order (centre,
  // then along l, k, j, i the distances -R..-1, 1..R) and summed in that order
  constexpr int MT = 8 * R + 1;
  bool canon = star && tp.n == MT;
  if (canon) {
    double c[MT];
    bool seen[MT] = {};
    for (int t = 0; t < tp.n && canon; ++t) {
      int ax = -1, d = 0;
      for (int a = 0; a < 4; ++a)
        if (offs[t][a]) ax = a, d = offs[t][a];
      const int q = ax < 0 ? 0 : 1 + 2 * R * ax + (d < 0 ? d + R : d + R - 1);
      if (seen[q]) canon = false;
      seen[q] = true;
      c[q] = tp.c[t];
    }
    if (canon)
      for (int q = 0; q < MT; ++q) {
        tp.c[q] = c[q];
        tp.cf[q] = (float)c[q];
      }
  }
  auto kern = canon ? sweep4_kernel<T, AT, R, true> : sweep4_kernel<T, AT, R, false>;
  const size_t smem = canon ? Tile4<T, R, true>::SMEM : G::SMEM;
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
    L.lf[d] = L.f[d] == 1 ? 0 : (L.f[d] == 2 ? 1 : 2);
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
  if (nlist >= (1u << 31)) return fail(BK_ERR_ARG, "4-D brick lists hold fewer than 2^31 entries");
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
