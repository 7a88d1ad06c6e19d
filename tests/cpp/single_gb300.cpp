// The reference's single-node CUDA test (single/cuda.cpp -> stencils/3axis.cu d3pt7cu)
// written against the GB300 engine's source-compatible headers: the same init_grid /
// BrickStorage / Brick / copyToBrick / movBrickInfo / movBrickStorage / compareBrick calls,
// with the per-brick CUDA kernel replaced by brickSweep.  Runs the 7-point stencil of
// 3axis.cu (coeff[0..6]) and the 13/25-point stars, 27- and 125-point cubes on an N^3
// interior, and compares every result with the array kernel at 1e-12.
// Exit status 0 and "result match" on success.
#define BRICK_TOLERANCE 1e-12

#include <cstdio>
#include <random>
#include <stdexcept>
#include <vector>

#include "brick.h"
#include "brick-decomp.h"
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

struct Tap { int dk, dj, di; };

static std::vector<Tap> star(int r) {
  std::vector<Tap> t{{0, 0, 0}};
  for (int d = 1; d <= r; ++d) {
    t.push_back({0, 0, d}); t.push_back({0, 0, -d});
    t.push_back({0, d, 0}); t.push_back({0, -d, 0});
    t.push_back({d, 0, 0}); t.push_back({-d, 0, 0});
  }
  return t;
}

static std::vector<Tap> cube(int r) {
  std::vector<Tap> t;
  for (int k = -r; k <= r; ++k)
    for (int j = -r; j <= r; ++j)
      for (int i = -r; i <= r; ++i) t.push_back({k, j, i});
  return t;
}

// single/mpi.cpp:58-121 on one GPU: a BrickDecomp layout, the reference's adjacency symmetry
// check, then the periodic exchange + the 7-point sweep against the array kernel on a
// periodically wrapped array.
static void decomp_check(std::mt19937_64 &mt) {
  std::uniform_real_distribution<bElem> u(-1, 1);
  BrickDecomp<3, 8, 8, 8> bDecomp({N, N, N}, GZ, 2);
  bDecomp.initialize(skin3d_good);
  BrickInfo<3> bInfo = bDecomp.getBrickInfo();
  const long bSize = cal_size<8, 8, 8>::value;
  auto bStorage = bInfo.allocate(bSize * 2);
  std::vector<unsigned> grid(STRIDEB * STRIDEB * STRIDEB);
  for (long k = 0; k < STRIDEB; ++k)
    for (long j = 0; j < STRIDEB; ++j)
      for (long i = 0; i < STRIDEB; ++i) grid[(k * STRIDEB + j) * STRIDEB + i] = bDecomp[k][j][i];
  for (long k = 1; k < STRIDEB - 1; ++k)
    for (long j = 1; j < STRIDEB - 1; ++j)
      for (long i = 1; i < STRIDEB - 1; ++i) {
        const unsigned l = grid[(k * STRIDEB + j) * STRIDEB + i];
        for (long id = 0; id < 27; ++id)
          if (bInfo.adj[bInfo.adj[l][id]][26 - id] != l) throw std::runtime_error("decomp: adjacency not symmetric");
      }
  // interior values only; the exchange fills the ghost bricks
  const long size = (long)STRIDE * STRIDE * STRIDE;
  std::vector<bElem> in(size, 0.0), out(size, 0.0);
  bElem(*a)[STRIDE][STRIDE] = (bElem(*)[STRIDE][STRIDE])in.data();
  for (long k = PADDING + GZ; k < PADDING + GZ + N; ++k)
    for (long j = PADDING + GZ; j < PADDING + GZ + N; ++j)
      for (long i = PADDING + GZ; i < PADDING + GZ + N; ++i) a[k][j][i] = u(mt);
  Brick3D bIn(&bInfo, bStorage, 0);
  copyToBrick<3>({STRIDEG, STRIDEG, STRIDEG}, {PADDING, PADDING, PADDING}, {0, 0, 0}, in.data(), grid.data(), bIn);
  // the array's periodic wrap (ghost cells <- the opposite interior cells)
  auto wrap = [](long x) { return PADDING + GZ + ((x - PADDING - GZ) % N + N) % N; };
  for (long k = PADDING; k < PADDING + STRIDEG; ++k)
    for (long j = PADDING; j < PADDING + STRIDEG; ++j)
      for (long i = PADDING; i < PADDING + STRIDEG; ++i) a[k][j][i] = a[wrap(k)][wrap(j)][wrap(i)];
  bElem(*o)[STRIDE][STRIDE] = (bElem(*)[STRIDE][STRIDE])out.data();
  const bElem c[7] = {0.4, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1};
  for (long k = PADDING + GZ; k < PADDING + GZ + N; ++k)
    for (long j = PADDING + GZ; j < PADDING + GZ + N; ++j)
      for (long i = PADDING + GZ; i < PADDING + GZ + N; ++i)
        o[k][j][i] = c[0] * a[k][j][i] + c[1] * a[k][j][i + 1] + c[2] * a[k][j][i - 1] + c[3] * a[k][j + 1][i] +
                     c[4] * a[k][j - 1][i] + c[5] * a[k + 1][j][i] + c[6] * a[k - 1][j][i];
  BrickInfo<3> bInfo_dev = movBrickInfo(bInfo, cudaMemcpyHostToDevice);
  BrickStorage bStorage_dev = movBrickStorage(bStorage, cudaMemcpyHostToDevice);
  Brick3D bIn_dev(&bInfo_dev, bStorage_dev, 0), bOut_dev(&bInfo_dev, bStorage_dev, bSize);
  std::vector<unsigned> interior;
  for (long k = GB; k < STRIDEB - GB; ++k)
    for (long j = GB; j < STRIDEB - GB; ++j)
      for (long i = GB; i < STRIDEB - GB; ++i) interior.push_back(grid[(k * STRIDEB + j) * STRIDEB + i]);
  unsigned *blist_dev = nullptr;
  gpuCheck(bk_device_malloc((void **)&blist_dev, interior.size() * sizeof(unsigned)));
  gpuCheck(bk_memcpy(blist_dev, interior.data(), interior.size() * sizeof(unsigned), 0, nullptr));
  BrickStencil st;
  st.add(0, 0, 0, c[0]).add(0, 0, 1, c[1]).add(0, 0, -1, c[2]).add(0, 1, 0, c[3]).add(0, -1, 0, c[4]);
  st.add(1, 0, 0, c[5]).add(-1, 0, 0, c[6]);
  bDecomp.exchange(bStorage_dev);
  brickSweep(bIn_dev, bOut_dev, blist_dev, (unsigned)interior.size(), st);
  int flags = 0;
  gpuCheck(bk_error_flags(nullptr, &flags));
  if (flags) throw std::runtime_error("decomp: device error flags");
  BrickStorage back = movBrickStorage(bStorage_dev, cudaMemcpyDeviceToHost);
  Brick3D bOut_host(&bInfo, back, bSize);
  if (!compareBrick<3>({N, N, N}, {PADDING, PADDING, PADDING}, {GZ, GZ, GZ}, out.data(), grid.data(), bOut_host))
    throw std::runtime_error("decomp: result mismatch!");
  gpuCheck(bk_device_free(blist_dev));
  gpuCheck(bk_device_free(bInfo_dev.adj));
  printf("decomp match\n");
}

// weak/main-4d.cpp's brick path on one GPU: Brick<Dim<4,4,4,4>, Dim<2,4>>, init_grid<4>,
// copyToBrick<4>, the 9-point star of stencils/mpi9pt.py through brickSweep4, compareBrick<4>
// against the array kernel (ghost 8, padding 4).
static void four_d_check(std::mt19937_64 &mt) {
  typedef Brick<Dim<4, 4, 4, 4>, Dim<2, 4>> Brick4D;
  const long n4 = 16, gz = 8, pad = 4, S = n4 + 2 * (gz + pad), SG = n4 + 2 * gz, gb = SG / 4;
  std::uniform_real_distribution<bElem> u(-1, 1);
  unsigned *grid_ptr;
  auto bInfo = init_grid<4>(grid_ptr, {gb, gb, gb, gb});
  auto bStorage = BrickStorage::allocate(bInfo.nbricks, 512);
  Brick4D bIn(&bInfo, bStorage, 0);
  std::vector<bElem> in(S * S * S * S), out(S * S * S * S, 0.0);
  for (auto &x : in) x = u(mt);
  copyToBrick<4>({SG, SG, SG, SG}, {pad, pad, pad, pad}, {0, 0, 0, 0}, in.data(), grid_ptr, bIn);
  auto at = [&](long l, long k, long j, long i) { return in[((l * S + k) * S + j) * S + i]; };
  const bElem alpha = 0.2, beta = 0.1;
  for (long l = pad + gz; l < pad + gz + n4; ++l)
    for (long k = pad + gz; k < pad + gz + n4; ++k)
      for (long j = pad + gz; j < pad + gz + n4; ++j)
        for (long i = pad + gz; i < pad + gz + n4; ++i)
          out[((l * S + k) * S + j) * S + i] =
              alpha * at(l, k, j, i) + beta * at(l, k, j, i + 1) + beta * at(l, k, j, i - 1) + beta * at(l, k, j + 1, i) +
              beta * at(l, k, j - 1, i) + beta * at(l, k + 1, j, i) + beta * at(l, k - 1, j, i) +
              beta * at(l + 1, k, j, i) + beta * at(l - 1, k, j, i);
  std::vector<unsigned> interior;
  const long g = gz / 4;
  for (long tl = g; tl < gb - g; ++tl)
    for (long tk = g; tk < gb - g; ++tk)
      for (long tj = g; tj < gb - g; ++tj)
        for (long ti = g; ti < gb - g; ++ti) interior.push_back(grid_ptr[((tl * gb + tk) * gb + tj) * gb + ti]);
  unsigned *blist_dev = nullptr;
  gpuCheck(bk_device_malloc((void **)&blist_dev, interior.size() * sizeof(unsigned)));
  gpuCheck(bk_memcpy(blist_dev, interior.data(), interior.size() * sizeof(unsigned), 0, nullptr));
  BrickInfo<4> bInfo_dev = movBrickInfo(bInfo, cudaMemcpyHostToDevice);
  BrickStorage bStorage_dev = movBrickStorage(bStorage, cudaMemcpyHostToDevice);
  Brick4D bIn_dev(&bInfo_dev, bStorage_dev, 0), bOut_dev(&bInfo_dev, bStorage_dev, 256);
  BrickStencil4 st;
  st.add(0, 0, 0, 0, alpha).add(0, 0, 0, 1, beta).add(0, 0, 0, -1, beta).add(0, 0, 1, 0, beta).add(0, 0, -1, 0, beta);
  st.add(0, 1, 0, 0, beta).add(0, -1, 0, 0, beta).add(1, 0, 0, 0, beta).add(-1, 0, 0, 0, beta);
  brickSweep4(bIn_dev, bOut_dev, blist_dev, (unsigned)interior.size(), st);
  int flags = 0;
  gpuCheck(bk_error_flags(nullptr, &flags));
  if (flags) throw std::runtime_error("4-D: device error flags");
  BrickStorage back = movBrickStorage(bStorage_dev, cudaMemcpyDeviceToHost);
  Brick4D bOut_host(&bInfo, back, 256);
  if (!compareBrick<4>({n4, n4, n4, n4}, {pad, pad, pad, pad}, {gz, gz, gz, gz}, out.data(), grid_ptr, bOut_host))
    throw std::runtime_error("4-D: result mismatch!");
  gpuCheck(bk_device_free(blist_dev));
  gpuCheck(bk_device_free(bInfo_dev.adj));
  free(grid_ptr);
  free(bInfo.adj);
  printf("d4pt9 match\n");
}

int main() {
  std::mt19937_64 mt(20261203);
  std::uniform_real_distribution<bElem> u(-1, 1);

  unsigned *grid_ptr;
  auto bInfo = init_grid<3>(grid_ptr, {STRIDEB, STRIDEB, STRIDEB});
  auto grid = (unsigned(*)[STRIDEB][STRIDEB])grid_ptr;

  // interior brick list on the device (the blocks of d3pt7_brick_trans, 3axis.cu:167)
  std::vector<unsigned> interior;
  for (long tk = GB; tk < STRIDEB - GB; ++tk)
    for (long tj = GB; tj < STRIDEB - GB; ++tj)
      for (long ti = GB; ti < STRIDEB - GB; ++ti) interior.push_back(grid[tk][tj][ti]);
  unsigned *blist_dev = nullptr;
  gpuCheck(bk_device_malloc((void **)&blist_dev, interior.size() * sizeof(unsigned)));
  gpuCheck(bk_memcpy(blist_dev, interior.data(), interior.size() * sizeof(unsigned), 0, nullptr));

  const long size = (long)STRIDE * STRIDE * STRIDE;
  std::vector<bElem> in(size), out(size, 0.0);
  for (auto &x : in) x = u(mt);
  bElem(*arr_in)[STRIDE][STRIDE] = (bElem(*)[STRIDE][STRIDE])in.data();
  bElem(*arr_out)[STRIDE][STRIDE] = (bElem(*)[STRIDE][STRIDE])out.data();

  auto bSize = cal_size<8, 8, 8>::value;
  auto bStorage = BrickStorage::allocate(bInfo.nbricks, bSize * 2);
  Brick3D bIn(&bInfo, bStorage, 0);
  Brick3D bOut(&bInfo, bStorage, bSize);
  copyToBrick<3>({STRIDEG, STRIDEG, STRIDEG}, {PADDING, PADDING, PADDING}, {0, 0, 0}, in.data(), grid_ptr, bIn);

  BrickInfo<3> bInfo_dev = movBrickInfo(bInfo, cudaMemcpyHostToDevice);
  BrickStorage bStorage_dev = movBrickStorage(bStorage, cudaMemcpyHostToDevice);
  Brick3D bIn_dev(&bInfo_dev, bStorage_dev, 0);
  Brick3D bOut_dev(&bInfo_dev, bStorage_dev, bSize);

  struct Case { const char *name; std::vector<Tap> taps; };
  std::vector<Case> cases = {{"d3pt7", star(1)}, {"d3pt13", star(2)}, {"d3pt25", star(4)},
                             {"d3pt27", cube(1)}, {"d3pt125", cube(2)}};
  for (auto &c : cases) {
    BrickStencil st;
    std::vector<bElem> coeff;
    for (auto &t : c.taps) {
      coeff.push_back(u(mt));
      st.add(t.dk, t.dj, t.di, coeff.back());
    }
    // array kernel (3axis.cpp:32-37 generalised to the tap list)
    for (long k = PADDING + GZ; k < PADDING + GZ + N; ++k)
      for (long j = PADDING + GZ; j < PADDING + GZ + N; ++j)
        for (long i = PADDING + GZ; i < PADDING + GZ + N; ++i) {
          bElem v = 0;
          for (size_t t = 0; t < c.taps.size(); ++t)
            v += coeff[t] * arr_in[k + c.taps[t].dk][j + c.taps[t].dj][i + c.taps[t].di];
          arr_out[k][j][i] = v;
        }
    brickSweep(bIn_dev, bOut_dev, blist_dev, (unsigned)interior.size(), st);
    int flags = 0;
    gpuCheck(bk_error_flags(nullptr, &flags));
    if (flags) throw std::runtime_error("device error flags");
    BrickStorage back = movBrickStorage(bStorage_dev, cudaMemcpyDeviceToHost);
    Brick3D bOut_host(&bInfo, back, bSize);
    if (!compareBrick<3>({N, N, N}, {PADDING, PADDING, PADDING}, {GZ, GZ, GZ}, out.data(), grid_ptr, bOut_host))
      throw std::runtime_error(std::string(c.name) + ": result mismatch!");
    printf("%s match\n", c.name);
  }
  gpuCheck(bk_device_free(blist_dev));
  gpuCheck(bk_device_free(bInfo_dev.adj));
  free(grid_ptr);
  free(bInfo.adj);
  decomp_check(mt);
  four_d_check(mt);
  printf("result match\n");
  return 0;
}
