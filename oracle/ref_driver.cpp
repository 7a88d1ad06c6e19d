/*
 * ref_driver.cpp -- drives bricklib's own CPU brick path, compiled from the
 * reference's headers where they lie (see oracle/Makefile, target `ref`).
 *
 * TEST INFRASTRUCTURE ONLY: it produces golden vectors and pins the C
 * restatement in brick_oracle.c.  Nothing in the product links it.
 *
 * What it runs is the reference's single-node CPU path of stencils/3axis.cpp
 * d3pt7() (:14-92), generalised to a runtime tap list:
 *   init_grid<3>            include/bricksetup.h:73-90
 *   BrickStorage::allocate  include/brick.h:68-75 (bIn / bOut interleaved, 3axis.cpp:26-28)
 *   copyToBrick<3>          include/bricksetup.h:172-181
 *   accessor brick kernel   3axis.cpp:51-66 (bOut[b][k][j][i] = sum c * bIn[b][k+dk][j+dj][i+di])
 *   array kernel            3axis.cpp:32-37 (_TILEFOR over the ghost-inclusive region)
 *   compareBrick<3>         include/brickcompare.h:30-57 (tolerance 1e-6, cmpconst.h:7)
 *   copyFromBrick<3>        include/bricksetup.h:213-221
 * The generated-code kernels (brick("x.py", ...)) need the vecscatter code generator at
 * build time and are not built here.
 */
#include <cstring>
#include <vector>

#include "brick.h"
#include "bricksetup.h"
#include "brickcompare.h"

namespace {

constexpr long GZ = 8;       // ghost zone, elements (stencils.h:14)
constexpr long PADDING = 8;  // array padding, elements (stencils.h:15)

template <unsigned BK, unsigned BJ, unsigned BI, typename Fold>
struct Lay {
  typedef Brick<Dim<BK, BJ, BI>, Fold> B;
  static constexpr unsigned bk = BK, bj = BJ, bi = BI;
};

template <typename L>
void offsets(long *out) {
  unsigned *grid_ptr;
  auto bInfo = init_grid<3>(grid_ptr, {1, 1, 1});
  auto bStorage = BrickStorage::allocate(bInfo.nbricks, L::B::BRICKSIZE);
  typename L::B br(&bInfo, bStorage, 0);
  for (unsigned k = 0; k < L::bk; ++k)
    for (unsigned j = 0; j < L::bj; ++j)
      for (unsigned i = 0; i < L::bi; ++i)
        out[(k * L::bj + j) * L::bi + i] = (long)(&br[0][k][j][i] - br.dat);
  free(grid_ptr);
  free(bInfo.adj);
}

template <typename L>
int sweep(long n, const double *in_arr, int npts, const int *offs, const double *coeff,
          double *out_brick, double *out_arr) {
  const long STRIDE = n + 2 * (GZ + PADDING), STRIDEG = n + 2 * GZ;
  const long gk = STRIDEG / L::bk, gj = STRIDEG / L::bj, gi = STRIDEG / L::bi;
  const long sz = STRIDE * STRIDE * STRIDE;
  unsigned *grid_ptr;
  auto bInfo = init_grid<3>(grid_ptr, {gi, gj, gk});
  const unsigned bsize = L::B::BRICKSIZE;
  auto bStorage = BrickStorage::allocate(bInfo.nbricks, bsize * 2);
  typename L::B bIn(&bInfo, bStorage, 0);
  typename L::B bOut(&bInfo, bStorage, bsize);
  std::memset(bStorage.dat.get(), 0, sizeof(bElem) * bStorage.chunks * bStorage.step);

  bElem *in_ptr = (bElem *)aligned_alloc(ALIGN, sizeof(bElem) * sz);
  std::memcpy(in_ptr, in_arr, sizeof(bElem) * sz);
  copyToBrick<3>({STRIDEG, STRIDEG, STRIDEG}, {PADDING, PADDING, PADDING}, {0, 0, 0}, in_ptr, grid_ptr, bIn);

  // array kernel, ghost-inclusive region like _TILEFOR (stencils.h:28-35)
  std::memset(out_arr, 0, sizeof(bElem) * sz);
  for (long k = PADDING; k < PADDING + STRIDEG; ++k)
    for (long j = PADDING; j < PADDING + STRIDEG; ++j)
      for (long i = PADDING; i < PADDING + STRIDEG; ++i) {
        bElem v = coeff[0] * in_ptr[((k + offs[0]) * STRIDE + j + offs[1]) * STRIDE + i + offs[2]];
        for (int t = 1; t < npts; ++t)
          v = v + coeff[t] * in_ptr[((k + offs[3 * t]) * STRIDE + j + offs[3 * t + 1]) * STRIDE + i + offs[3 * t + 2]];
        out_arr[(k * STRIDE + j) * STRIDE + i] = v;
      }

  // accessor brick kernel over interior bricks (3axis.cpp:51-66)
  auto grid = grid_ptr;
  for (long tk = GZ / L::bk; tk < gk - GZ / L::bk; ++tk)
    for (long tj = GZ / L::bj; tj < gj - GZ / L::bj; ++tj)
      for (long ti = GZ / L::bi; ti < gi - GZ / L::bi; ++ti) {
        unsigned b = grid[(tk * gj + tj) * gi + ti];
        for (long k = 0; k < L::bk; ++k)
          for (long j = 0; j < L::bj; ++j)
            for (long i = 0; i < L::bi; ++i) {
              bElem v = coeff[0] * bIn[b][k + offs[0]][j + offs[1]][i + offs[2]];
              for (int t = 1; t < npts; ++t)
                v = v + coeff[t] * bIn[b][k + offs[3 * t]][j + offs[3 * t + 1]][i + offs[3 * t + 2]];
              bOut[b][k][j][i] = v;
            }
      }

  bool ok = compareBrick<3>({n, n, n}, {PADDING, PADDING, PADDING}, {GZ, GZ, GZ}, out_arr, grid_ptr, bOut);
  std::memset(out_brick, 0, sizeof(bElem) * sz);
  copyFromBrick<3>({n, n, n}, {PADDING, PADDING, PADDING}, {GZ, GZ, GZ}, out_brick, grid_ptr, bOut);

  free(in_ptr);
  free(grid_ptr);
  free(bInfo.adj);
  return ok ? 1 : 0;
}

// The cond kernel of stencils/3axis.cpp:94-163 (d3cond): array and accessor brick versions
// with the reference's expression, coeff[0..6] in its order.
int cond_sweep(long n, const double *in_arr, const double *coeff, double *out_brick, double *out_arr) {
  typedef Brick<Dim<8, 8, 8>, Dim<4, 8>> B;
  const long STRIDE = n + 2 * (GZ + PADDING), STRIDEG = n + 2 * GZ, gb = STRIDEG / 8;
  const long sz = STRIDE * STRIDE * STRIDE;
  unsigned *grid_ptr;
  auto bInfo = init_grid<3>(grid_ptr, {gb, gb, gb});
  auto bStorage = BrickStorage::allocate(bInfo.nbricks, 1024);
  B bIn(&bInfo, bStorage, 0), bOut(&bInfo, bStorage, 512);
  std::memset(bStorage.dat.get(), 0, sizeof(bElem) * bStorage.chunks * bStorage.step);
  bElem *in_ptr = (bElem *)aligned_alloc(ALIGN, sizeof(bElem) * sz);
  std::memcpy(in_ptr, in_arr, sizeof(bElem) * sz);
  copyToBrick<3>({STRIDEG, STRIDEG, STRIDEG}, {PADDING, PADDING, PADDING}, {0, 0, 0}, in_ptr, grid_ptr, bIn);
  auto arr_in = (bElem(*)[STRIDE][STRIDE])in_ptr;
  auto arr_out = (bElem(*)[STRIDE][STRIDE])out_arr;
  std::memset(out_arr, 0, sizeof(bElem) * sz);
  using std::max;
  for (long k = PADDING; k < PADDING + STRIDEG; ++k)
    for (long j = PADDING; j < PADDING + STRIDEG; ++j)
      for (long i = PADDING; i < PADDING + STRIDEG; ++i) {
        bElem partial = coeff[5] * max(arr_in[k + 1][j][i], 0.0) + coeff[6] * max(arr_in[k - 1][j][i], 0.0) +
                        coeff[3] * max(arr_in[k][j + 1][i], 0.0) + coeff[4] * max(arr_in[k][j - 1][i], 0.0) +
                        coeff[1] * max(arr_in[k][j][i + 1], 0.0) + coeff[2] * max(arr_in[k][j][i - 1], 0.0) +
                        coeff[0] * max(arr_in[k][j][i], 0.0);
        arr_out[k][j][i] = partial > 0 ? partial : -partial;
      }
  auto grid = (unsigned(*)[gb][gb])grid_ptr;
  for (long tk = 1; tk < gb - 1; ++tk)
    for (long tj = 1; tj < gb - 1; ++tj)
      for (long ti = 1; ti < gb - 1; ++ti) {
        unsigned b = grid[tk][tj][ti];
        for (long k = 0; k < 8; ++k)
          for (long j = 0; j < 8; ++j)
            for (long i = 0; i < 8; ++i) {
              bElem partial =
                  coeff[5] * max(bIn[b][k + 1][j][i], 0.0) + coeff[6] * max(bIn[b][k - 1][j][i], 0.0) +
                  coeff[3] * max(bIn[b][k][j + 1][i], 0.0) + coeff[4] * max(bIn[b][k][j - 1][i], 0.0) +
                  coeff[1] * max(bIn[b][k][j][i + 1], 0.0) + coeff[2] * max(bIn[b][k][j][i - 1], 0.0) +
                  coeff[0] * max(bIn[b][k][j][i], 0.0);
              bOut[b][k][j][i] = partial > 0 ? partial : -partial;
            }
      }
  bool ok = compareBrick<3>({n, n, n}, {PADDING, PADDING, PADDING}, {GZ, GZ, GZ}, out_arr, grid_ptr, bOut);
  std::memset(out_brick, 0, sizeof(bElem) * sz);
  copyFromBrick<3>({n, n, n}, {PADDING, PADDING, PADDING}, {GZ, GZ, GZ}, out_brick, grid_ptr, bOut);
  free(in_ptr);
  free(grid_ptr);
  free(bInfo.adj);
  return ok ? 1 : 0;
}

// ------------------------------------------------------------------ 4-D (weak/main-4d.cpp)
// Brick<Dim<4,4,4,4>, Dim<VFOLD>> with the folds of main-4d.cpp:33-52 (AVX512 (2,4),
// AVX2 (2,2), scalar (1)), init_grid<4>, copyToBrick<4> / copyFromBrick<4> / compareBrick<4>
// and the accessor form of the mpi9pt.py kernel generalised to a runtime 4-D tap list; ghost
// zone 2*TILE = 8 and array padding 4 as in main-4d.cpp:29-31.
constexpr long GZ4 = 8, PAD4 = 4;

template <typename Fold>
void offsets4(long *out) {
  typedef Brick<Dim<4, 4, 4, 4>, Fold> B;
  unsigned *grid_ptr;
  auto bInfo = init_grid<4>(grid_ptr, {1, 1, 1, 1});
  auto bStorage = BrickStorage::allocate(bInfo.nbricks, B::BRICKSIZE);
  B br(&bInfo, bStorage, 0);
  for (unsigned l = 0; l < 4; ++l)
    for (unsigned k = 0; k < 4; ++k)
      for (unsigned j = 0; j < 4; ++j)
        for (unsigned i = 0; i < 4; ++i) out[((l * 4 + k) * 4 + j) * 4 + i] = (long)(&br[0][l][k][j][i] - br.dat);
  free(grid_ptr);
  free(bInfo.adj);
}

template <typename Fold>
int sweep4(long n, const double *in_arr, int npts, const int *offs, const double *coeff, double *out_brick,
           double *out_arr) {
  typedef Brick<Dim<4, 4, 4, 4>, Fold> B;
  const long S = n + 2 * (GZ4 + PAD4), SG = n + 2 * GZ4, gb = SG / 4;
  const long sz = S * S * S * S;
  unsigned *grid_ptr;
  auto bInfo = init_grid<4>(grid_ptr, {gb, gb, gb, gb});
  auto bStorage = BrickStorage::allocate(bInfo.nbricks, B::BRICKSIZE * 2);
  B bIn(&bInfo, bStorage, 0), bOut(&bInfo, bStorage, B::BRICKSIZE);
  std::memset(bStorage.dat.get(), 0, sizeof(bElem) * bStorage.chunks * bStorage.step);
  bElem *in_ptr = (bElem *)aligned_alloc(ALIGN, sizeof(bElem) * sz);
  std::memcpy(in_ptr, in_arr, sizeof(bElem) * sz);
  copyToBrick<4>({SG, SG, SG, SG}, {PAD4, PAD4, PAD4, PAD4}, {0, 0, 0, 0}, in_ptr, grid_ptr, bIn);
  auto at = [&](long l, long k, long j, long i) { return in_ptr[((l * S + k) * S + j) * S + i]; };
  std::memset(out_arr, 0, sizeof(bElem) * sz);
  for (long l = PAD4; l < PAD4 + SG; ++l)
    for (long k = PAD4; k < PAD4 + SG; ++k)
      for (long j = PAD4; j < PAD4 + SG; ++j)
        for (long i = PAD4; i < PAD4 + SG; ++i) {
          bElem v = coeff[0] * at(l + offs[0], k + offs[1], j + offs[2], i + offs[3]);
          for (int t = 1; t < npts; ++t)
            v = v + coeff[t] * at(l + offs[4 * t], k + offs[4 * t + 1], j + offs[4 * t + 2], i + offs[4 * t + 3]);
          out_arr[((l * S + k) * S + j) * S + i] = v;
        }
  auto grid = (unsigned(*)[gb][gb][gb])grid_ptr;
  const long g = GZ4 / 4;
  for (long tl = g; tl < gb - g; ++tl)
    for (long tk = g; tk < gb - g; ++tk)
      for (long tj = g; tj < gb - g; ++tj)
        for (long ti = g; ti < gb - g; ++ti) {
          unsigned b = grid[tl][tk][tj][ti];
          for (long l = 0; l < 4; ++l)
            for (long k = 0; k < 4; ++k)
              for (long j = 0; j < 4; ++j)
                for (long i = 0; i < 4; ++i) {
                  bElem v = coeff[0] * bIn[b][l + offs[0]][k + offs[1]][j + offs[2]][i + offs[3]];
                  for (int t = 1; t < npts; ++t)
                    v = v + coeff[t] * bIn[b][l + offs[4 * t]][k + offs[4 * t + 1]][j + offs[4 * t + 2]]
                                          [i + offs[4 * t + 3]];
                  bOut[b][l][k][j][i] = v;
                }
        }
  bool ok = compareBrick<4>({n, n, n, n}, {PAD4, PAD4, PAD4, PAD4}, {GZ4, GZ4, GZ4, GZ4}, out_arr, grid_ptr, bOut);
  std::memset(out_brick, 0, sizeof(bElem) * sz);
  copyFromBrick<4>({n, n, n, n}, {PAD4, PAD4, PAD4, PAD4}, {GZ4, GZ4, GZ4, GZ4}, out_brick, grid_ptr, bOut);
  free(in_ptr);
  free(grid_ptr);
  free(bInfo.adj);
  return ok ? 1 : 0;
}

typedef Lay<8, 8, 8, Dim<4, 8>> L0;     // CUDA fold (stencils/cudavfold.h:9)
typedef Lay<8, 8, 8, Dim<8>> L1;        // AVX-512 fold (stencils/cpuvfold.h:12-13)
typedef Lay<8, 8, 8, Dim<2, 2>> L2;     // docs/usingbricks.md example fold
typedef Lay<8, 8, 8, Dim<2, 4, 4>> L3;  // three-level fold
typedef Lay<4, 4, 4, Dim<4, 4>> L4;     // 4^3 bricks
typedef Lay<16, 8, 8, Dim<4, 8>> L5;    // 16x8x8 bricks
typedef Lay<8, 8, 32, Dim<4, 8>> L6;    // 8x8x32 bricks

}  // namespace

extern "C" {

/* Layout ids: 0 (8,8,8)/(4,8)  1 (8,8,8)/(8)  2 (8,8,8)/(2,2)  3 (8,8,8)/(2,4,4)
 *             4 (4,4,4)/(4,4)  5 (16,8,8)/(4,8)  6 (8,8,32)/(4,8) */
int ref_layout_offsets(int layout, long *out) {
  switch (layout) {
    case 0: offsets<L0>(out); return 0;
    case 1: offsets<L1>(out); return 0;
    case 2: offsets<L2>(out); return 0;
    case 3: offsets<L3>(out); return 0;
    case 4: offsets<L4>(out); return 0;
    case 5: offsets<L5>(out); return 0;
    case 6: offsets<L6>(out); return 0;
  }
  return -1;
}

int ref_init_grid(long gk, long gj, long gi, unsigned *grid, unsigned *adj) {
  unsigned *grid_ptr;
  auto bInfo = init_grid<3>(grid_ptr, {gi, gj, gk});
  std::memcpy(grid, grid_ptr, sizeof(unsigned) * gk * gj * gi);
  std::memcpy(adj, bInfo.adj, sizeof(unsigned) * 27 * bInfo.nbricks);
  free(grid_ptr);
  free(bInfo.adj);
  return 0;
}

/* One sweep on an n^3 interior with an 8-cell ghost zone and 8-cell array padding.
 * in_arr, out_brick, out_arr: (n+32)^3 arrays.  Returns 1 when compareBrick matches. */
int ref_sweep(int layout, long n, const double *in_arr, int npts, const int *offs, const double *coeff,
              double *out_brick, double *out_arr) {
  switch (layout) {
    case 0: return sweep<L0>(n, in_arr, npts, offs, coeff, out_brick, out_arr);
    case 1: return sweep<L1>(n, in_arr, npts, offs, coeff, out_brick, out_arr);
    case 4: return sweep<L4>(n, in_arr, npts, offs, coeff, out_brick, out_arr);
  }
  return -1;
}

/* 4-D: fold ids 0 (2,4)  1 (2,2)  2 (1) of Brick<Dim<4,4,4,4>, Dim<fold>>; out[256] in (l,k,j,i). */
int ref_layout_offsets4(int fold, long *out) {
  switch (fold) {
    case 0: offsets4<Dim<2, 4>>(out); return 0;
    case 1: offsets4<Dim<2, 2>>(out); return 0;
    case 2: offsets4<Dim<1>>(out); return 0;
  }
  return -1;
}

int ref_init_grid4(long gl, long gk, long gj, long gi, unsigned *grid, unsigned *adj) {
  unsigned *grid_ptr;
  auto bInfo = init_grid<4>(grid_ptr, {gi, gj, gk, gl});
  std::memcpy(grid, grid_ptr, sizeof(unsigned) * gl * gk * gj * gi);
  std::memcpy(adj, bInfo.adj, sizeof(unsigned) * 81 * bInfo.nbricks);
  free(grid_ptr);
  free(bInfo.adj);
  return 0;
}

/* One 4-D sweep on an n^4 interior (ghost 8, padding 4): arrays (n+24)^4, taps (dl,dk,dj,di). */
int ref_sweep4(int fold, long n, const double *in_arr, int npts, const int *offs, const double *coeff,
               double *out_brick, double *out_arr) {
  switch (fold) {
    case 0: return sweep4<Dim<2, 4>>(n, in_arr, npts, offs, coeff, out_brick, out_arr);
    case 2: return sweep4<Dim<1>>(n, in_arr, npts, offs, coeff, out_brick, out_arr);
  }
  return -1;
}

/* The reference's cond kernel (3axis.cpp:94-163) on an n^3 interior; coeff[0..6]. */
int ref_cond(long n, const double *in_arr, const double *coeff, double *out_brick, double *out_arr) {
  return cond_sweep(n, in_arr, coeff, out_brick, out_arr);
}

}  // extern "C"
