/*
 * brick_oracle.c -- CPU restatement of bricklib's brick stencil path.
 *
 * TEST INFRASTRUCTURE ONLY (see brick_oracle.h).  Built with
 *   gcc -O2 -fopenmp -ffp-contract=off -fPIC -shared
 * so that every double operation is a separately rounded IEEE operation in the
 * order written, on x86-64 and aarch64 alike.
 */
#include "brick_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

/* 53 random bits -> [0, 1) */
static inline double u01(uint64_t seed, uint64_t n) {
  return (double)(splitmix64(seed + n) >> 11) * (1.0 / 9007199254740992.0);
}

void orc_fill_uniform(double *a, long n, uint64_t seed, double lo, double hi) {
#pragma omp parallel for schedule(static)
  for (long p = 0; p < n; ++p) a[p] = lo + (hi - lo) * u01(seed, (uint64_t)p);
}

static inline long wrap(long x, long n) {
  long r = x % n;
  return r < 0 ? r + n : r;
}

void orc_fill_sines(double *a, const long dims[3], const long org[3], const long n[3],
                    int nw, uint64_t seed, double noise) {
  /* wave m: integer wave numbers in 1..4 per axis, phase in [0, 2pi), amplitude 1/nw */
  int kv[64][3];
  double ph[64];
  if (nw > 64) nw = 64;
  for (int m = 0; m < nw; ++m) {
    for (int d = 0; d < 3; ++d) kv[m][d] = 1 + (int)(u01(seed, (uint64_t)(4 * m + d)) * 4.0);
    ph[m] = 2.0 * M_PI * u01(seed, (uint64_t)(4 * m + 3));
  }
  const uint64_t nseed = splitmix64(seed ^ 0x5eedull);
#pragma omp parallel for collapse(2) schedule(static)
  for (long k = 0; k < dims[0]; ++k)
    for (long j = 0; j < dims[1]; ++j)
      for (long i = 0; i < dims[2]; ++i) {
        long z = wrap(k - org[0], n[0]), y = wrap(j - org[1], n[1]), x = wrap(i - org[2], n[2]);
        double v = 0.0;
        for (int m = 0; m < nw; ++m)
          v += sin(2.0 * M_PI * ((double)kv[m][0] * z / n[0] + (double)kv[m][1] * y / n[1] +
                                 (double)kv[m][2] * x / n[2]) + ph[m]) / nw;
        uint64_t idx = (uint64_t)((z * n[1] + y) * n[2] + x);
        v += noise * (2.0 * u01(nseed, idx) - 1.0);
        a[(k * dims[1] + j) * dims[2] + i] = v;
      }
}

void orc_init_grid(unsigned *grid, unsigned *adj, long gk, long gj, long gi) {
  long size = gk * gj * gi;
  for (long p = 0; p < size; ++p) grid[p] = (unsigned)p;
#pragma omp parallel for collapse(2) schedule(static)
  for (long k = 0; k < gk; ++k)
    for (long j = 0; j < gj; ++j)
      for (long i = 0; i < gi; ++i) {
        unsigned b = grid[(k * gj + j) * gi + i];
        for (int dk = -1; dk <= 1; ++dk)
          for (int dj = -1; dj <= 1; ++dj)
            for (int di = -1; di <= 1; ++di) {
              /* init_fill tests the neighbour's linear position against the whole
               * grid (bricksetup.h:44-47), not each axis: a neighbour past an edge
               * of a row or plane lands on the adjacent row or plane, and only a
               * position before the first or after the last brick becomes 0. */
              long q = ((k + dk) * gj + (j + dj)) * gi + (i + di);
              unsigned v = (q >= 0 && q < size) ? grid[q] : 0;
              adj[(size_t)b * 27 + (dk + 1) * 9 + (dj + 1) * 3 + (di + 1)] = v;
            }
      }
}

long orc_brick_offset(const int bdim[3], const int fold[3], int k, int j, int i) {
  const long fk = fold[0], fj = fold[1], fi = fold[2];
  const long vl = fk * fj * fi;
  long vec = ((k / fk) * (bdim[1] / fj) + j / fj) * (bdim[2] / fi) + i / fi;
  long lane = ((k % fk) * fj + j % fj) * fi + i % fi;
  return vec * vl + lane;
}

static long *offset_table(const int bdim[3], const int fold[3]) {
  long bs = (long)bdim[0] * bdim[1] * bdim[2];
  long *t = (long *)malloc(sizeof(long) * (size_t)bs);
  for (int k = 0; k < bdim[0]; ++k)
    for (int j = 0; j < bdim[1]; ++j)
      for (int i = 0; i < bdim[2]; ++i)
        t[((long)k * bdim[1] + j) * bdim[2] + i] = orc_brick_offset(bdim, fold, k, j, i);
  return t;
}

void orc_copy_brick(int to_brick, const long dim[3], const long pad[3], const long ghost[3],
                    double *arr, const unsigned *grid, double *dat, long step, long off,
                    const int bdim[3], const int fold[3]) {
  long adims[3], gdims[3], s0[3], s1[3];
  for (int d = 0; d < 3; ++d) {
    adims[d] = dim[d] + 2 * (pad[d] + ghost[d]);
    gdims[d] = (dim[d] + 2 * ghost[d]) / bdim[d];
    s0[d] = ghost[d] / bdim[d];
    s1[d] = (dim[d] + ghost[d]) / bdim[d];
  }
  long *ot = offset_table(bdim, fold);
#pragma omp parallel for collapse(2) schedule(static)
  for (long sk = s0[0]; sk < s1[0]; ++sk)
    for (long sj = s0[1]; sj < s1[1]; ++sj)
      for (long si = s0[2]; si < s1[2]; ++si) {
        unsigned b = grid[(sk * gdims[1] + sj) * gdims[2] + si];
        double *bp = dat + (size_t)b * step + off;
        for (int k = 0; k < bdim[0]; ++k)
          for (int j = 0; j < bdim[1]; ++j)
            for (int i = 0; i < bdim[2]; ++i) {
              long ak = pad[0] + sk * bdim[0] + k, aj = pad[1] + sj * bdim[1] + j,
                   ai = pad[2] + si * bdim[2] + i;
              double *ap = arr + (ak * adims[1] + aj) * adims[2] + ai;
              double *e = bp + ot[((long)k * bdim[1] + j) * bdim[2] + i];
              if (to_brick) *e = *ap;
              else *ap = *e;
            }
      }
  free(ot);
}

/* radius per axis of a tap list */
static void tap_radius(int npts, const int *offs, int r[3]) {
  r[0] = r[1] = r[2] = 0;
  for (int t = 0; t < npts; ++t)
    for (int d = 0; d < 3; ++d) {
      int a = abs(offs[3 * t + d]);
      if (a > r[d]) r[d] = a;
    }
}

/* The part of a brick's extended tile (bdim + 2r per axis) that a tap list reads: per tile
 * row (k, j) the column range [lo, hi); lo >= hi when no tap reads the row.  A star reads its
 * centre brick and the faces it reaches, a cube its whole neighbourhood. */
typedef struct {
  int ek, ej, ei;
  int *lo, *hi;
} tile_rows;

static tile_rows rows_read(int npts, const int *offs, const int bdim[3], const int r[3]) {
  tile_rows t;
  t.ek = bdim[0] + 2 * r[0];
  t.ej = bdim[1] + 2 * r[1];
  t.ei = bdim[2] + 2 * r[2];
  t.lo = (int *)malloc(sizeof(int) * (size_t)t.ek * t.ej);
  t.hi = (int *)malloc(sizeof(int) * (size_t)t.ek * t.ej);
  for (long q = 0; q < (long)t.ek * t.ej; ++q) {
    t.lo[q] = t.ei;
    t.hi[q] = 0;
  }
  for (int p = 0; p < npts; ++p) {
    const int dk = offs[3 * p], dj = offs[3 * p + 1], di = offs[3 * p + 2];
    for (int k = 0; k < bdim[0]; ++k)
      for (int j = 0; j < bdim[1]; ++j) {
        const long q = (long)(k + r[0] + dk) * t.ej + (j + r[1] + dj);
        if (r[2] + di < t.lo[q]) t.lo[q] = r[2] + di;
        if (r[2] + di + bdim[2] > t.hi[q]) t.hi[q] = r[2] + di + bdim[2];
      }
  }
  return t;
}

static void rows_free(tile_rows *t) {
  free(t->lo);
  free(t->hi);
}

/* 1 when the in-brick layout is row-major (element (k,j,i) at (k*bj + j)*bi + i): brick rows are
 * then contiguous and copy as one run. */
static int layout_row_major(const int bdim[3], const long *ot) {
  const long bs = (long)bdim[0] * bdim[1] * bdim[2];
  for (long p = 0; p < bs; ++p)
    if (ot[p] != p) return 0;
  return 1;
}

/* Gather the rows of brick b's extended tile that the taps read, through adj, the way the
 * accessor resolves an out-of-brick index: neighbour slot from the sign of the overflow
 * (brick.h:232-245), element from the in-brick remainder.  A tile row spans up to three
 * bricks along i (the i-lo neighbour, the brick itself, the i-hi neighbour). */
#define DEFINE_GATHER(NAME, T)                                                                    \
  static void NAME(const unsigned *adj, const T *in, long step, long off, unsigned b,            \
                   const int bdim[3], const int r[3], const long *ot, int rm, const tile_rows *tr, \
                   T *tile) {                                                                    \
    const int ej = tr->ej, ei = tr->ei, bi = bdim[2];                                            \
    for (int k = 0; k < tr->ek; ++k) {                                                           \
      const int kk = k - r[0], qk = kk < 0 ? -1 : (kk >= bdim[0] ? 1 : 0);                       \
      const int lk = kk - qk * bdim[0];                                                          \
      for (int j = 0; j < ej; ++j) {                                                             \
        const int lo = tr->lo[(long)k * ej + j], hi = tr->hi[(long)k * ej + j];                  \
        if (lo >= hi) continue;                                                                  \
        const int jj = j - r[1], qj = jj < 0 ? -1 : (jj >= bdim[1] ? 1 : 0);                     \
        const int lj = jj - qj * bdim[1];                                                        \
        T *trow = tile + ((long)k * ej + j) * ei;                                                \
        for (int qi = -1; qi <= 1; ++qi) {                                                       \
          const int s0 = qi < 0 ? 0 : (qi == 0 ? r[2] : r[2] + bi);                              \
          const int s1 = qi < 0 ? r[2] : (qi == 0 ? r[2] + bi : ei);                             \
          const int a = s0 > lo ? s0 : lo, e = s1 < hi ? s1 : hi;                                \
          if (a >= e) continue;                                                                  \
          const unsigned nb = adj[(size_t)b * 27 + (qk + 1) * 9 + (qj + 1) * 3 + (qi + 1)];      \
          const T *src = in + (size_t)nb * step + off;                                           \
          const long row = ((long)lk * bdim[1] + lj) * bi + (a - r[2] - qi * bi);                \
          if (rm) memcpy(trow + a, src + row, sizeof(T) * (size_t)(e - a));                      \
          else                                                                                   \
            for (int i = a; i < e; ++i) trow[i] = src[ot[row + (i - a)]];                        \
        }                                                                                        \
      }                                                                                          \
    }                                                                                            \
  }

DEFINE_GATHER(gather_f64, double)
DEFINE_GATHER(gather_f32, float)

static inline double op_apply(double x, int op) {
  if (op == 1) return x > 0.0 ? x : 0.0;  /* max(x, 0.0) */
  if (op == 2) return x > 0 ? x : -x;     /* partial > 0 ? partial : -partial */
  return x;
}

/* acc(k,j,i) = sum_t coeff[t] * tile(k+r+dk, j+r+dj, i+r+di), every point summing its taps left
 * to right.  Any brick dims: taps outermost, over whole brick rows. */
#define DEFINE_TAPS(NAME, T)                                                                      \
  static void NAME(const T *restrict tile, int ej, int ei, const int r[3], const int bdim[3],    \
                   int npts, const int *offs, const double *coeff, T *restrict acc) {           \
    const int bk = bdim[0], bj = bdim[1], bi = bdim[2];                                          \
    for (int t = 0; t < npts; ++t) {                                                             \
      const T c = (T)coeff[t];                                                                   \
      const int dk = offs[3 * t], dj = offs[3 * t + 1], di = offs[3 * t + 2];                    \
      for (int k = 0; k < bk; ++k)                                                               \
        for (int j = 0; j < bj; ++j) {                                                           \
          const T *src = tile + ((long)(k + r[0] + dk) * ej + (j + r[1] + dj)) * ei + r[2] + di; \
          T *dst = acc + ((long)k * bj + j) * bi;                                                \
          if (t == 0)                                                                            \
            for (int i = 0; i < bi; ++i) dst[i] = c * src[i];                                    \
          else                                                                                   \
            for (int i = 0; i < bi; ++i) dst[i] = dst[i] + c * src[i];                           \
        }                                                                                        \
    }                                                                                            \
  }

/* 8^3 bricks: rows outermost, the row's eight sums held in registers across the taps (tap t of
 * the row at tile offset toff[t] from the row's centre); the same operations per point in the
 * same order as above. */
#define DEFINE_TAPS_888(NAME, T)                                                                  \
  static void NAME(const T *restrict tile, int ej, int ei, const int r[3], int npts,             \
                   const long *toff, const T *cf, T *restrict acc) {                            \
    for (int k = 0; k < 8; ++k)                                                                  \
      for (int j = 0; j < 8; ++j) {                                                              \
        const T *base = tile + ((long)(k + r[0]) * ej + (j + r[1])) * ei + r[2];                 \
        T a[8];                                                                                  \
        const T *s0 = base + toff[0];                                                            \
        for (int i = 0; i < 8; ++i) a[i] = cf[0] * s0[i];                                        \
        for (int t = 1; t < npts; ++t) {                                                         \
          const T c = cf[t];                                                                     \
          const T *s = base + toff[t];                                                           \
          for (int i = 0; i < 8; ++i) a[i] = a[i] + c * s[i];                                    \
        }                                                                                        \
        memcpy(acc + (k * 8 + j) * 8, a, sizeof(a));                                             \
      }                                                                                          \
  }

DEFINE_TAPS(taps_f64, double)
DEFINE_TAPS(taps_f32, float)
DEFINE_TAPS_888(taps_f64_888, double)
DEFINE_TAPS_888(taps_f32_888, float)

/* tile offsets of the taps from a row's centre element, for the 8^3 path */
static long *tap_offsets(int npts, const int *offs, int ej, int ei) {
  long *t = (long *)malloc(sizeof(long) * (size_t)(npts > 0 ? npts : 1));
  for (int p = 0; p < npts; ++p) t[p] = ((long)offs[3 * p] * ej + offs[3 * p + 1]) * ei + offs[3 * p + 2];
  return t;
}

#define BK_ORC_MAX_TAPS 1024

static int is_888(const int bdim[3]) { return bdim[0] == 8 && bdim[1] == 8 && bdim[2] == 8; }

void orc_brick_sweep(const unsigned *adj, const double *in, long in_step, long in_off,
                     double *out, long out_step, long out_off,
                     const unsigned *blist, long nlist,
                     const int bdim[3], const int fold[3],
                     int npts, const int *offs, const double *coeff, int nthreads) {
  orc_brick_sweep_ops(adj, in, in_step, in_off, out, out_step, out_off, blist, nlist, bdim, fold, npts, offs,
                      coeff, 0, 0, nthreads);
}

void orc_brick_sweep_ops(const unsigned *adj, const double *in, long in_step, long in_off,
                         double *out, long out_step, long out_off,
                         const unsigned *blist, long nlist,
                         const int bdim[3], const int fold[3],
                         int npts, const int *offs, const double *coeff, int pre, int post, int nthreads) {
  int r[3];
  tap_radius(npts, offs, r);
  tile_rows tr = rows_read(npts, offs, bdim, r);
  const long bs = (long)bdim[0] * bdim[1] * bdim[2];
  long *ot = offset_table(bdim, fold);
  const int rm = layout_row_major(bdim, ot), b8 = is_888(bdim);
  long *toff = tap_offsets(npts, offs, tr.ej, tr.ei);
  if (nthreads <= 0) nthreads = orc_max_threads();
#pragma omp parallel num_threads(nthreads)
  {
    double *tile = (double *)malloc(sizeof(double) * (size_t)tr.ek * tr.ej * tr.ei);
    double *acc = (double *)malloc(sizeof(double) * (size_t)bs);
#pragma omp for schedule(static)
    for (long n = 0; n < nlist; ++n) {
      unsigned b = blist[n];
      gather_f64(adj, in, in_step, in_off, b, bdim, r, ot, rm, &tr, tile);
      if (pre)
        for (long q = 0; q < (long)tr.ek * tr.ej; ++q)
          for (int i = tr.lo[q]; i < tr.hi[q]; ++i) tile[q * tr.ei + i] = op_apply(tile[q * tr.ei + i], pre);
      if (b8) taps_f64_888(tile, tr.ej, tr.ei, r, npts, toff, coeff, acc);
      else taps_f64(tile, tr.ej, tr.ei, r, bdim, npts, offs, coeff, acc);
      double *ob = out + (size_t)b * out_step + out_off;
      if (rm && !post) memcpy(ob, acc, sizeof(double) * (size_t)bs);
      else
        for (long p = 0; p < bs; ++p) ob[ot[p]] = op_apply(acc[p], post);
    }
    free(tile);
    free(acc);
  }
  free(ot);
  free(toff);
  rows_free(&tr);
}

void orc_brick_sweep_f32(const unsigned *adj, const float *in, long in_step, long in_off,
                         float *out, long out_step, long out_off,
                         const unsigned *blist, long nlist,
                         const int bdim[3], const int fold[3],
                         int npts, const int *offs, const double *coeff, int nthreads) {
  int r[3];
  tap_radius(npts, offs, r);
  tile_rows tr = rows_read(npts, offs, bdim, r);
  const long bs = (long)bdim[0] * bdim[1] * bdim[2];
  long *ot = offset_table(bdim, fold);
  const int rm = layout_row_major(bdim, ot), b8 = is_888(bdim);
  long *toff = tap_offsets(npts, offs, tr.ej, tr.ei);
  float cf[BK_ORC_MAX_TAPS];
  for (int t = 0; t < npts && t < BK_ORC_MAX_TAPS; ++t) cf[t] = (float)coeff[t];
  if (nthreads <= 0) nthreads = orc_max_threads();
#pragma omp parallel num_threads(nthreads)
  {
    float *tile = (float *)malloc(sizeof(float) * (size_t)tr.ek * tr.ej * tr.ei);
    float *acc = (float *)malloc(sizeof(float) * (size_t)bs);
#pragma omp for schedule(static)
    for (long n = 0; n < nlist; ++n) {
      unsigned b = blist[n];
      gather_f32(adj, in, in_step, in_off, b, bdim, r, ot, rm, &tr, tile);
      if (b8 && npts <= BK_ORC_MAX_TAPS) taps_f32_888(tile, tr.ej, tr.ei, r, npts, toff, cf, acc);
      else taps_f32(tile, tr.ej, tr.ei, r, bdim, npts, offs, coeff, acc);
      float *ob = out + (size_t)b * out_step + out_off;
      for (long p = 0; p < bs; ++p) ob[ot[p]] = acc[p];
    }
    free(tile);
    free(acc);
  }
  free(ot);
  free(toff);
  rows_free(&tr);
}

void orc_array_sweep(const double *in, double *out, const long dims[3],
                     const long lo[3], const long hi[3],
                     int npts, const int *offs, const double *coeff, int nthreads) {
  orc_array_sweep_ops(in, out, dims, lo, hi, npts, offs, coeff, 0, 0, nthreads);
}

void orc_array_sweep_ops(const double *in, double *out, const long dims[3],
                         const long lo[3], const long hi[3],
                         int npts, const int *offs, const double *coeff, int pre, int post, int nthreads) {
  const long sj = dims[2], sk = dims[1] * dims[2];
  if (nthreads <= 0) nthreads = orc_max_threads();
#pragma omp parallel for collapse(2) schedule(static) num_threads(nthreads)
  for (long k = lo[0]; k < hi[0]; ++k)
    for (long j = lo[1]; j < hi[1]; ++j)
      for (long i = lo[2]; i < hi[2]; ++i) {
        const long p = k * sk + j * sj + i;
        double v = coeff[0] * op_apply(in[p + offs[0] * sk + offs[1] * sj + offs[2]], pre);
        for (int t = 1; t < npts; ++t)
          v = v + coeff[t] * op_apply(in[p + offs[3 * t] * sk + offs[3 * t + 1] * sj + offs[3 * t + 2]], pre);
        out[p] = op_apply(v, post);
      }
}

void orc_array_periodic_fill(double *a, const long dims[3], const long org[3],
                             const long n[3], const long ghost[3]) {
  long lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = org[d] - ghost[d];
    hi[d] = org[d] + n[d] + ghost[d];
  }
  /* axis by axis over the full extended box: faces first, then edges and corners
   * pick up already-wrapped values, which equals wrapping every axis at once */
  for (int ax = 0; ax < 3; ++ax) {
#pragma omp parallel for collapse(2) schedule(static)
    for (long k = lo[0]; k < hi[0]; ++k)
      for (long j = lo[1]; j < hi[1]; ++j)
        for (long i = lo[2]; i < hi[2]; ++i) {
          long c[3] = {k, j, i};
          if (c[ax] >= org[ax] && c[ax] < org[ax] + n[ax]) continue;
          long s[3] = {k, j, i};
          s[ax] = org[ax] + wrap(c[ax] - org[ax], n[ax]);
          a[(k * dims[1] + j) * dims[2] + i] = a[(s[0] * dims[1] + s[1]) * dims[2] + s[2]];
        }
  }
}

long orc_periodic_plan(const unsigned *grid, const long nb[3], const long gb[3], unsigned *pairs) {
  long G[3];
  for (int d = 0; d < 3; ++d) G[d] = nb[d] + 2 * gb[d];
  long cnt = 0;
  for (long k = 0; k < G[0]; ++k)
    for (long j = 0; j < G[1]; ++j)
      for (long i = 0; i < G[2]; ++i) {
        long c[3] = {k, j, i};
        int ghost = 0;
        long s[3];
        for (int d = 0; d < 3; ++d) {
          if (c[d] < gb[d] || c[d] >= gb[d] + nb[d]) ghost = 1;
          s[d] = gb[d] + wrap(c[d] - gb[d], nb[d]);
        }
        if (!ghost) continue;
        if (pairs) {
          pairs[2 * cnt] = grid[(k * G[1] + j) * G[2] + i];
          pairs[2 * cnt + 1] = grid[(s[0] * G[1] + s[1]) * G[2] + s[2]];
        }
        ++cnt;
      }
  return cnt;
}

void orc_apply_plan(double *dat, long step, long off, long belems, const unsigned *pairs, long npairs) {
#pragma omp parallel for schedule(static)
  for (long p = 0; p < npairs; ++p)
    memcpy(dat + (size_t)pairs[2 * p] * step + off, dat + (size_t)pairs[2 * p + 1] * step + off,
           sizeof(double) * (size_t)belems);
}

long orc_compare_brick(const long dim[3], const long pad[3], const long ghost[3],
                       const double *arr, const unsigned *grid, const double *dat,
                       long step, long off, const int bdim[3], const int fold[3],
                       double tol, double *stats) {
  long adims[3], gdims[3], s0[3], s1[3];
  for (int d = 0; d < 3; ++d) {
    adims[d] = dim[d] + 2 * (pad[d] + ghost[d]);
    gdims[d] = (dim[d] + 2 * ghost[d]) / bdim[d];
    s0[d] = ghost[d] / bdim[d];
    s1[d] = (dim[d] + ghost[d]) / bdim[d];
  }
  long *ot = offset_table(bdim, fold);
  long bad = 0;
  double maxdiff = 0.0, maxref = 0.0;
#pragma omp parallel for collapse(2) schedule(static) reduction(+ : bad) reduction(max : maxdiff, maxref)
  for (long sk = s0[0]; sk < s1[0]; ++sk)
    for (long sj = s0[1]; sj < s1[1]; ++sj)
      for (long si = s0[2]; si < s1[2]; ++si) {
        unsigned b = grid[(sk * gdims[1] + sj) * gdims[2] + si];
        const double *bp = dat + (size_t)b * step + off;
        for (int k = 0; k < bdim[0]; ++k)
          for (int j = 0; j < bdim[1]; ++j)
            for (int i = 0; i < bdim[2]; ++i) {
              long ak = pad[0] + sk * bdim[0] + k, aj = pad[1] + sj * bdim[1] + j,
                   ai = pad[2] + si * bdim[2] + i;
              double a = arr[(ak * adims[1] + aj) * adims[2] + ai];
              double e = bp[ot[((long)k * bdim[1] + j) * bdim[2] + i]];
              double diff = fabs(e - a);
              int ok = (diff < tol) || (diff < (fabs(e) + fabs(a)) * tol);
              if (!ok) ++bad;
              if (diff > maxdiff) maxdiff = diff;
              if (fabs(a) > maxref) maxref = fabs(a);
            }
      }
  free(ot);
  if (stats) {
    stats[0] = maxdiff;
    stats[1] = maxref;
  }
  return bad;
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
