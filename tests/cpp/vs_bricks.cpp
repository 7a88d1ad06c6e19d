// A CPU brick program in the reference's single-node style (stencils/3axis.cpp d3pt7,
// :14-92): a padded array, init_grid, copyToBrick into interleaved bIn / bOut, a per-brick
// loop whose body is a brick("vs_star7.py", ...) statement, and compareBrick against the
// array loop.  It is not compiled as written: bricklib_gb300.dsl.vecscatter lowers the
// brick(...) loop first, as the reference's build runs its code generator first.  The loop
// runs twice (the second pass reuses the device brick list), then once more over the bricks
// in device memory.  Exit status 0 and "result match" on success.
#define BRICK_TOLERANCE 1e-12

#include <cstdio>
#include <random>
#include <vector>

#include "brick.h"
#include "brick-gb300.h"
#include "brickcompare.h"
#include "bricksetup.h"

#define N 64
#define TILE 8
#define GZ TILE
#define PADDING 8
#define STRIDE (N + 2 * (GZ + PADDING))
#define STRIDEG (N + 2 * GZ)
#define STRIDEB ((N + 2 * GZ) / TILE)
#define GB (GZ / TILE)

typedef Brick<Dim<8, 8, 8>, Dim<4, 8>> Brick3D;

bElem coeff[7];

static void sweep_bricks(unsigned (*grid)[STRIDEB][STRIDEB], Brick3D &bIn, Brick3D &bOut) {
#pragma omp parallel for collapse(2)
  for (long tk = GB; tk < STRIDEB - GB; ++tk)
    for (long tj = GB; tj < STRIDEB - GB; ++tj)
      for (long ti = GB; ti < STRIDEB - GB; ++ti) {
        unsigned b = grid[tk][tj][ti];
        brick("vs_star7.py", VSVEC, (8, 8, 8), (4, 8), b);
      }
}

int main() {
  std::mt19937_64 mt(20261204);
  std::uniform_real_distribution<bElem> u(-1, 1);
  for (auto &c : coeff) c = u(mt);
  const long size = (long)STRIDE * STRIDE * STRIDE;
  std::vector<bElem> in(size), out(size, 0.0);
  for (auto &x : in) x = u(mt);
  bElem(*a)[STRIDE][STRIDE] = (bElem(*)[STRIDE][STRIDE])in.data();
  bElem(*o)[STRIDE][STRIDE] = (bElem(*)[STRIDE][STRIDE])out.data();
  for (long k = PADDING; k < PADDING + STRIDEG; ++k)  // the array loop over interior and ghost
    for (long j = PADDING; j < PADDING + STRIDEG; ++j)
      for (long i = PADDING; i < PADDING + STRIDEG; ++i)
        if (k >= PADDING + GZ && k < PADDING + GZ + N && j >= PADDING + GZ && j < PADDING + GZ + N &&
            i >= PADDING + GZ && i < PADDING + GZ + N)
          o[k][j][i] = coeff[0] * a[k][j][i] + coeff[1] * a[k][j][i + 1] + coeff[2] * a[k][j][i - 1] +
                       coeff[3] * a[k][j + 1][i] + coeff[4] * a[k][j - 1][i] + coeff[5] * a[k + 1][j][i] +
                       coeff[6] * a[k - 1][j][i];

  unsigned *grid_ptr;
  BrickInfo<3> bInfo = init_grid<3>(grid_ptr, {STRIDEB, STRIDEB, STRIDEB});
  unsigned(*grid)[STRIDEB][STRIDEB] = (unsigned(*)[STRIDEB][STRIDEB])grid_ptr;
  BrickStorage bStorage = BrickStorage::allocate(bInfo.nbricks, 1024);
  Brick3D bIn(&bInfo, bStorage, 0), bOut(&bInfo, bStorage, 512);
  copyToBrick<3>({STRIDEG, STRIDEG, STRIDEG}, {PADDING, PADDING, PADDING}, {0, 0, 0}, in.data(), grid_ptr, bIn);

  int bad = 0;
  for (int pass = 0; pass < 2; ++pass) {  // host bricks, twice
    for (long q = 0; q < bInfo.nbricks; ++q)
      for (long e = 0; e < 512; ++e) bStorage.dat.get()[q * 1024 + 512 + e] = 0.0;
    sweep_bricks(grid, bIn, bOut);
    if (!compareBrick<3>({N, N, N}, {PADDING, PADDING, PADDING}, {GZ, GZ, GZ}, out.data(), grid_ptr, bOut)) ++bad;
  }
  // the same loop over bricks in device memory (output field zeroed before the copy)
  for (long q = 0; q < bInfo.nbricks; ++q)
    for (long e = 0; e < 512; ++e) bStorage.dat.get()[q * 1024 + 512 + e] = 0.0;
  BrickInfo<3> bInfo_dev = movBrickInfo(bInfo, cudaMemcpyHostToDevice);
  BrickStorage bStorage_dev = movBrickStorage(bStorage, cudaMemcpyHostToDevice);
  Brick3D dIn(&bInfo_dev, bStorage_dev, 0), dOut(&bInfo_dev, bStorage_dev, 512);
  sweep_bricks(grid, dIn, dOut);
  BrickStorage back = movBrickStorage(bStorage_dev, cudaMemcpyDeviceToHost);
  Brick3D hOut(&bInfo, back, 512);
  if (!compareBrick<3>({N, N, N}, {PADDING, PADDING, PADDING}, {GZ, GZ, GZ}, out.data(), grid_ptr, hOut)) ++bad;
  printf(bad ? "result mismatch (%d of 3 passes)\n" : "result match\n", bad);
  return bad ? 1 : 0;
}
