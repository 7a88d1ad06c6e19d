/*
 * brickcompare.h -- compare bricks with an array, source-compatible with the reference's
 * include/brickcompare.h (compareBrick, :30-80) and include/cmpconst.h (BRICK_TOLERANCE).
 *
 * An element passes when diff < tol or diff < (|brick| + |array|) * tol
 * (brickcompare.h:37).  BRICK_TOLERANCE defaults to the reference's 1e-6; define it
 * before including this header for a tighter check (the FP64 parity tests use 1e-12).
 */
#ifndef BRICK_BRICKCOMPARE_H
#define BRICK_BRICKCOMPARE_H

#include <cmath>
#include <vector>

#include "bricksetup.h"

#ifndef BRICK_TOLERANCE
#define BRICK_TOLERANCE 1e-6
#endif

template <unsigned dims, typename T>
inline bool compareBrick(const std::vector<long> &dimlist, const std::vector<long> &padding,
                         const std::vector<long> &ghost, bElem *arr, unsigned *grid_ptr, T &brick) {
  bool ok = true;
  iter_grid<dims>(dimlist, padding, ghost, arr, grid_ptr, brick, [&ok](bElem &br, bElem *a) {
    const double diff = std::abs((double)br - (double)*a);
    if (!((diff < BRICK_TOLERANCE) || (diff < (std::abs((double)br) + std::abs((double)*a)) * BRICK_TOLERANCE))) {
#pragma omp atomic write
      ok = false;
    }
  });
  return ok;
}

template <unsigned dims, typename T>
inline bool compareBrick(const std::vector<long> &dimlist, bElem *arr, unsigned *grid_ptr, T &brick) {
  std::vector<long> zero(dimlist.size(), 0);
  return compareBrick<dims, T>(dimlist, zero, zero, arr, grid_ptr, brick);
}

#endif  // BRICK_BRICKCOMPARE_H
