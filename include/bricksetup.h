/*
 * bricksetup.h -- grid setup and array <-> brick copies (host), source-compatible with
 * the reference's include/bricksetup.h: init_grid<dims> (:73-90), iter_grid (:139-159),
 * copyToBrick (:172-195) and copyFromBrick (:197-221).
 *
 * Dimension lists are contiguous-first (i, j, k), as in the reference.  The iteration is
 * written as a flat odometer over brick-grid positions and in-brick coordinates; element
 * access goes through Brick::at, the same address computation as bIn[b][k][j][i].
 */
#ifndef BRICK_SETUP_H
#define BRICK_SETUP_H

#include <stdlib.h>

#include <algorithm>
#include <vector>

#include "brick.h"

/**
 * Dense grid of bricks: grid_ptr[p] = p over prod(dimlist) bricks, and the neighbour of
 * brick p at offset (q_0 .. q_{dims-1}) (outermost first, each in {-1,0,1}) is the brick at
 * linear position p + sum_c q_c * stride_c, or brick 0 when that position is outside the
 * whole grid (the reference tests the linear position, bricksetup.h:44-47, so a step past
 * the edge of a row lands on the neighbouring row).  grid_ptr is malloc'ed; the caller
 * frees it and bInfo.adj.
 */
template <unsigned dims>
BrickInfo<dims> init_grid(unsigned *&grid_ptr, const std::vector<long> &dimlist) {
  long size = 1;
  std::vector<long> stride;  // contiguous-first
  for (long a : dimlist) {
    stride.push_back(size);
    size *= a;
  }
  grid_ptr = (unsigned *)malloc(sizeof(unsigned) * size);
  for (long p = 0; p < size; ++p) grid_ptr[p] = (unsigned)p;
  BrickInfo<dims> bInfo((unsigned)size);
  constexpr unsigned NS = static_power<3, dims>::value;
#pragma omp parallel for
  for (long p = 0; p < size; ++p) {
    for (unsigned s = 0; s < NS; ++s) {
      // slot digits, outermost dimension first
      long q = p;
      unsigned rem = s;
      for (unsigned d = 0; d < dims; ++d) {
        const unsigned pw = [](unsigned e) { unsigned v = 1; while (e--) v *= 3; return v; }(dims - 1 - d);
        const int digit = (int)(rem / pw);
        rem %= pw;
        q += (digit - 1) * stride[dims - 1 - d];
      }
      bInfo.adj[p][s] = (q >= 0 && q < size) ? grid_ptr[q] : 0u;
    }
  }
  return bInfo;
}

/**
 * Visit every element of the region dimlist (skipping `padding` in the array and `ghost`
 * in both) side by side in bricks and in the array: f(brick element, array element).
 * The array has extent dimlist + 2*(padding+ghost) per axis; the brick grid has
 * (dimlist + 2*ghost) / BDim bricks per axis.
 */
template <unsigned dims, typename F, typename T, unsigned... BDims>
inline void iter_grid(const std::vector<long> &dimlist, const std::vector<long> &padding,
                      const std::vector<long> &ghost, bElem *arr, unsigned *grid_ptr,
                      Brick<Dim<BDims...>, T> &brick, F f) {
  const long bd_outer_first[] = {(long)BDims...};
  long tile[dims], s0[dims], s1[dims], astride[dims], gstride[dims];
  long sa = 1, sg = 1;
  for (unsigned c = 0; c < dims; ++c) {  // contiguous-first
    tile[c] = bd_outer_first[dims - 1 - c];
    s0[c] = ghost[c] / tile[c];
    s1[c] = (dimlist[c] + ghost[c]) / tile[c];
    astride[c] = sa;
    gstride[c] = sg;
    sa *= dimlist[c] + 2 * (padding[c] + ghost[c]);
    sg *= (dimlist[c] + 2 * ghost[c]) / tile[c];
  }
  long nbr = 1;
  for (unsigned c = 0; c < dims; ++c) nbr *= s1[c] - s0[c];
  const long bsize = cal_size<BDims...>::value;
#pragma omp parallel for
  for (long n = 0; n < nbr; ++n) {
    long s[dims], rem = n;
    for (unsigned c = 0; c < dims; ++c) {
      s[c] = s0[c] + rem % (s1[c] - s0[c]);
      rem /= s1[c] - s0[c];
    }
    long g = 0;
    for (unsigned c = 0; c < dims; ++c) g += s[c] * gstride[c];
    const unsigned b = grid_ptr[g];
    for (long e = 0; e < bsize; ++e) {
      int x[dims];
      long er = e, aoff = 0;
      for (unsigned c = 0; c < dims; ++c) {
        const long l = er % tile[c];
        er /= tile[c];
        x[dims - 1 - c] = (int)l;
        aoff += (padding[c] + s[c] * tile[c] + l) * astride[c];
      }
      f(brick.at(b, x), arr + aoff);
    }
  }
}

template <unsigned dims, typename T>
inline void copyToBrick(const std::vector<long> &dimlist, const std::vector<long> &padding,
                        const std::vector<long> &ghost, bElem *arr, unsigned *grid_ptr, T &brick) {
  iter_grid<dims>(dimlist, padding, ghost, arr, grid_ptr, brick, [](bElem &br, bElem *a) { br = *a; });
}

template <unsigned dims, typename T>
inline void copyToBrick(const std::vector<long> &dimlist, bElem *arr, unsigned *grid_ptr, T &brick) {
  std::vector<long> zero(dimlist.size(), 0);
  copyToBrick<dims>(dimlist, zero, zero, arr, grid_ptr, brick);
}

template <unsigned dims, typename T>
inline void copyFromBrick(const std::vector<long> &dimlist, const std::vector<long> &padding,
                          const std::vector<long> &ghost, bElem *arr, unsigned *grid_ptr, T &brick) {
  iter_grid<dims>(dimlist, padding, ghost, arr, grid_ptr, brick, [](bElem &br, bElem *a) { *a = br; });
}

#endif  // BRICK_SETUP_H
