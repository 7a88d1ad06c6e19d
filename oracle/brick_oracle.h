/*
 * brick_oracle.h -- CPU restatement of bricklib's single-node brick stencil path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA sweep in
 * bricklib_gb300: only the test suite, the smoke check and the CPU-baseline leg
 * of the benchmark load it.  The product path never calls it and never falls
 * back to it.
 *
 * Every function restates the behaviour of a reference file (cited per
 * function, paths relative to the bricklib source tree).  Arithmetic is plain
 * IEEE double, evaluated in tap order, compiled with -ffp-contract=off so the
 * result is the same on x86-64 and aarch64.
 *
 * Index conventions used throughout: triples are (k, j, i) with i the
 * contiguous axis.  A brick grid of gk x gj x gi bricks stores the brick at grid
 * position (bk, bj, bi) in grid[(bk * gj + bj) * gi + bi].
 */
#ifndef BRICK_ORACLE_H
#define BRICK_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Seeded uniform values in [lo, hi): splitmix64 stream, element n uses state seed + n. */
void orc_fill_uniform(double *a, long n, uint64_t seed, double lo, double hi);

/* Sum of `nw` seeded random-phase sines on an N^3 periodic domain plus `noise`
 * uniform noise, written into a padded array (dims nk x nj x ni, the N^3
 * interior starts at `org` in every axis; cells outside the interior get the
 * periodic continuation). */
void orc_fill_sines(double *a, const long dims[3], const long org[3], const long n[3],
                    int nw, uint64_t seed, double noise);

/* init_grid (bricksetup.h:73-90 with init_iter/init_fill :30-71): grid[p] = p
 * and adj[b][27] holds the neighbour at (dk, dj, di) in slot
 * (dk+1)*9 + (dj+1)*3 + (di+1).  The neighbour is looked up at linear grid
 * position p + (dk*gj + dj)*gi + di and is brick 0 only when that position falls
 * outside the whole grid (a step past a row's edge wraps to the next row). */
void orc_init_grid(unsigned *grid, unsigned *adj, long gk, long gj, long gi);

/* In-brick element offset for brick dims bdim (k,j,i) and vector fold
 * fold (k,j,i; 1 = not folded), as computed by _BrickAccessor
 * (brick.h:213-327): vectors ordered (k/fk, j/fj, i/fi), lanes (k%fk, j%fj, i%fi). */
long orc_brick_offset(const int bdim[3], const int fold[3], int k, int j, int i);

/* copyToBrick / copyFromBrick (bricksetup.h:139-221, iter_grid).
 * dim: region size (k,j,i) in elements; pad, ghost: array padding and ghost (k,j,i);
 * to_brick = 1 copies array -> bricks, 0 copies bricks -> array.
 * The array has dims dim + 2*(pad+ghost); the brick grid has (dim + 2*ghost)/bdim bricks
 * per axis, and the copy covers grid positions ghost/bdim .. (dim+ghost)/bdim - 1. */
void orc_copy_brick(int to_brick, const long dim[3], const long pad[3], const long ghost[3],
                    double *arr, const unsigned *grid, double *dat, long step, long off,
                    const int bdim[3], const int fold[3]);

/* Brick sweep with the accessor's semantics (3axis.cpp:51-66 generalised to any
 * tap list): for every brick b in blist and every element (k,j,i) of it,
 *   out[b](k,j,i) = sum_t coeff[t] * in[b](k+dk_t, j+dj_t, i+di_t)
 * evaluated left to right, reading neighbour bricks through adj.  Offsets must
 * satisfy |d| <= brick dim on their axis.  Runs on `nthreads` OpenMP threads
 * (<= 0: the OpenMP default). */
void orc_brick_sweep(const unsigned *adj, const double *in, long in_step, long in_off,
                     double *out, long out_step, long out_off,
                     const unsigned *blist, long nlist,
                     const int bdim[3], const int fold[3],
                     int npts, const int *offs, const double *coeff, int nthreads);

/* The same sweep for non-linear stencils: out = post(sum_t coeff[t] * pre(in)), op 0 none,
 * 1 max(x, 0.0), 2 |x| written as x > 0 ? x : -x (the cond kernel, stencils/3axis.cpp:94-163). */
void orc_brick_sweep_ops(const unsigned *adj, const double *in, long in_step, long in_off,
                         double *out, long out_step, long out_off,
                         const unsigned *blist, long nlist,
                         const int bdim[3], const int fold[3],
                         int npts, const int *offs, const double *coeff, int pre, int post, int nthreads);

/* Same sweep, float storage with float accumulation in tap order (FP32 form). */
void orc_brick_sweep_f32(const unsigned *adj, const float *in, long in_step, long in_off,
                         float *out, long out_step, long out_off,
                         const unsigned *blist, long nlist,
                         const int bdim[3], const int fold[3],
                         int npts, const int *offs, const double *coeff, int nthreads);

/* Array sweep (arr_func, 3axis.cpp:32-37; ST_CPU, stencils/fake.h:44-351):
 * out[p] = sum_t coeff[t] * in[p + off_t] for every p in the box lo..hi-1 (k,j,i)
 * of a dense array with dims (k,j,i). */
void orc_array_sweep(const double *in, double *out, const long dims[3],
                     const long lo[3], const long hi[3],
                     int npts, const int *offs, const double *coeff, int nthreads);

/* Array sweep with pointwise operations (see orc_brick_sweep_ops). */
void orc_array_sweep_ops(const double *in, double *out, const long dims[3],
                         const long lo[3], const long hi[3],
                         int npts, const int *offs, const double *coeff, int pre, int post, int nthreads);

/* Periodic ghost fill of a padded array: every cell of the box
 * org - ghost .. org + n + ghost - 1 outside the interior org .. org + n - 1 gets the
 * value of the interior cell at the wrapped position (the one-rank periodic
 * exchange of array-mpi.h:146-205 on a periodic Cartesian communicator,
 * weak/args.cpp:105-108). */
void orc_array_periodic_fill(double *a, const long dims[3], const long org[3],
                             const long n[3], const long ghost[3]);

/* Periodic ghost-brick plan for an init_grid layout of (n+2g) bricks per axis
 * (g ghost bricks each side): for every ghost grid position the (dst, src)
 * storage indices, src being the interior brick at the wrapped grid position
 * (strong/args.cpp:36-55 wrap).  Returns the number of pairs written into
 * pairs[2*count] (pass pairs = NULL to count only). */
long orc_periodic_plan(const unsigned *grid, const long nb[3], const long gb[3], unsigned *pairs);

/* Apply a (dst, src) brick plan: copies `belems` elements at offset `off` of each chunk. */
void orc_apply_plan(double *dat, long step, long off, long belems, const unsigned *pairs, long npairs);

/* compareBrick (brickcompare.h:30-57): element-wise over the region, passes when
 * diff < tol || diff < (|a|+|b|)*tol.  Returns the number of failing elements;
 * writes max |a-b| and max |a| of the array side to stats[0], stats[1]. */
long orc_compare_brick(const long dim[3], const long pad[3], const long ghost[3],
                       const double *arr, const unsigned *grid, const double *dat,
                       long step, long off, const int bdim[3], const int fold[3],
                       double tol, double *stats);

/* OpenMP thread count actually used by the parallel regions. */
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
