// Host-only check of include/brick.h and include/bricksetup.h: writes, as raw binary
// to the file named by argv[1],
//   the in-brick offsets &b[0][k][j][i] - b.dat for seven brick-dims / fold pairs,
//   then grid and adjacency of init_grid<3>(grid, {5, 4, 3}),
// for comparison with the golden vectors of the reference accessor.
#include <cstdio>
#include <vector>

#include "brick.h"
#include "bricksetup.h"

template <typename B, unsigned BK, unsigned BJ, unsigned BI>
static void offsets(FILE *f) {
  unsigned *grid_ptr;
  auto bInfo = init_grid<3>(grid_ptr, {1, 1, 1});
  auto st = BrickStorage::allocate(bInfo.nbricks, B::BRICKSIZE);
  B br(&bInfo, st, 0);
  for (unsigned k = 0; k < BK; ++k)
    for (unsigned j = 0; j < BJ; ++j)
      for (unsigned i = 0; i < BI; ++i) {
        long o = (long)(&br[0][k][j][i] - br.dat);
        fwrite(&o, sizeof o, 1, f);
      }
  free(grid_ptr);
  free(bInfo.adj);
}

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  FILE *f = fopen(argv[1], "wb");
  if (!f) return 2;
  offsets<Brick<Dim<8, 8, 8>, Dim<4, 8>>, 8, 8, 8>(f);
  offsets<Brick<Dim<8, 8, 8>, Dim<8>>, 8, 8, 8>(f);
  offsets<Brick<Dim<8, 8, 8>, Dim<2, 2>>, 8, 8, 8>(f);
  offsets<Brick<Dim<8, 8, 8>, Dim<2, 4, 4>>, 8, 8, 8>(f);
  offsets<Brick<Dim<4, 4, 4>, Dim<4, 4>>, 4, 4, 4>(f);
  offsets<Brick<Dim<16, 8, 8>, Dim<4, 8>>, 16, 8, 8>(f);
  offsets<Brick<Dim<8, 8, 32>, Dim<4, 8>>, 8, 8, 32>(f);
  unsigned *grid_ptr;
  auto bInfo = init_grid<3>(grid_ptr, {5, 4, 3});
  fwrite(grid_ptr, sizeof(unsigned), 60, f);
  fwrite(&bInfo.adj[0][0], sizeof(unsigned), 60 * 27, f);
  fclose(f);
  free(grid_ptr);
  free(bInfo.adj);
  return 0;
}
