// copyToBrick / copyFromBrick on the device (include/bricksetup.h:139-221).
//
// The region `dim` (k,j,i elements) of a dense array with `pad` padding and `ghost` ghost
// cells per side is copied to / from the bricks whose grid positions are ghost/B ..
// (dim+ghost)/B - 1 per axis; grid_dev maps grid positions (row-major over
// (dim + 2*ghost)/B bricks per axis) to storage indices.  One CTA per brick: the CTA's
// threads walk the brick in row-major (k, j, i) order, so array rows are read and written
// contiguously and the brick side through the fold layout; row-major bricks with 16-byte
// rows move as 16-byte vectors.  A negative `pad` addresses an
// array that holds the region without (all of) its ghost cells.
#include "bk_common.cuh"

namespace bk {

struct CopyArgs {
  long long adim[3];   // array extents (k, j, i)
  long long a0[3];     // array index of grid position s0 element 0: pad + s0*B
  int s0[3], ns[3];    // first grid position and count per axis
  int gd[3];           // grid extents per axis
  Layout L;
  unsigned long long step, offset;
  long long chunks;
};

template <typename T, bool TO_BRICK>
__global__ void __launch_bounds__(256)
array_brick_kernel(T *arr, const unsigned *__restrict__ grid, T *dat, const CopyArgs a, int *err) {
  const long long nb = (long long)a.ns[0] * a.ns[1] * a.ns[2];
  const int bsize = a.L.size();
  for (long long q = blockIdx.x; q < nb; q += gridDim.x) {
    const int si = (int)(q % a.ns[2]), sj = (int)((q / a.ns[2]) % a.ns[1]), sk = (int)(q / ((long long)a.ns[1] * a.ns[2]));
    const long long gpos = ((long long)(a.s0[0] + sk) * a.gd[1] + (a.s0[1] + sj)) * a.gd[2] + (a.s0[2] + si);
    const unsigned b = grid[gpos];
    if ((long long)b >= a.chunks) {
      if (threadIdx.x == 0) atomicOr(err, FLAG_BOUNDS);
      continue;
    }
    T *bp = dat + (size_t)b * a.step + a.offset;
    for (int e = threadIdx.x; e < bsize; e += blockDim.x) {
      const int k = e / (a.L.bj * a.L.bi), j = (e / a.L.bi) % a.L.bj, i = e % a.L.bi;
      const long long ak = a.a0[0] + (long long)sk * a.L.bk + k;
      const long long aj = a.a0[1] + (long long)sj * a.L.bj + j;
      const long long ai = a.a0[2] + (long long)si * a.L.bi + i;
      T *ap = arr + (ak * a.adim[1] + aj) * a.adim[2] + ai;
      T *ep = bp + a.L.offset(k, j, i);
      if (TO_BRICK) *ep = *ap;
      else *ap = *ep;
    }
  }
}

// Row-major bricks whose rows are whole 16-byte vectors on both sides: one CTA per brick
// (blockIdx = brick position within the region, i fastest), one thread per 16-byte vector
// of a brick row, the row index of each thread computed once.  Bricks are read and written
// in whole rows; array rows in 16-byte pieces of bi elements.
template <bool TO_BRICK>
__global__ void array_brick_rows_kernel(char *arr, const unsigned *__restrict__ grid, char *dat, const CopyArgs a,
                                        int es, int *err) {
  const int vpr = a.L.bi * es / 16;  // vectors per brick row
  const int r = threadIdx.x / vpr, c = threadIdx.x - r * vpr;
  const int k = r / a.L.bj, j = r - k * a.L.bj;
  const int si = blockIdx.x, sj = blockIdx.y, sk = blockIdx.z;
  const long long gpos = ((long long)(a.s0[0] + sk) * a.gd[1] + (a.s0[1] + sj)) * a.gd[2] + (a.s0[2] + si);
  const unsigned b = grid[gpos];
  if ((long long)b >= a.chunks) {
    if (threadIdx.x == 0) atomicOr(err, FLAG_BOUNDS);
    return;
  }
  const long long ak = a.a0[0] + (long long)sk * a.L.bk + k, aj = a.a0[1] + (long long)sj * a.L.bj + j;
  const long long ai = a.a0[2] + (long long)si * a.L.bi;
  uint4 *ap = reinterpret_cast<uint4 *>(arr + ((ak * a.adim[1] + aj) * a.adim[2] + ai) * es) + c;
  uint4 *bp = reinterpret_cast<uint4 *>(dat + ((size_t)b * a.step + a.offset + (size_t)r * a.L.bi) * es) + c;
  if (TO_BRICK) *bp = *ap;
  else *ap = *bp;
}

static int array_brick(bool to_brick, void *arr, const long dim[3], const long pad[3], const long ghost[3],
                       const unsigned *grid, const bk_field *f, const bk_layout *lay, void *stream) {
  Layout L;
  int s = check_layout(lay, &L);
  if (s) return s;
  if ((s = check_field(f, L, "brick"))) return s;
  if (!arr || !dim || !pad || !ghost || !grid) return fail(BK_ERR_ARG, "array <-> brick copy: NULL argument");
  CopyArgs a{};
  const int bd[3] = {L.bk, L.bj, L.bi};
  for (int d = 0; d < 3; ++d) {
    if (dim[d] <= 0 || ghost[d] < 0 || ghost[d] % bd[d] || dim[d] % bd[d] || pad[d] + ghost[d] < 0)
      return fail(BK_ERR_ARG, "array <-> brick copy: region and ghost must be multiples of the brick dims "
                              "and the array must hold the region");
    a.adim[d] = dim[d] + 2 * (pad[d] + ghost[d]);
    a.s0[d] = (int)(ghost[d] / bd[d]);
    a.ns[d] = (int)(dim[d] / bd[d]);
    a.gd[d] = (int)((dim[d] + 2 * ghost[d]) / bd[d]);
    a.a0[d] = pad[d] + (long long)a.s0[d] * bd[d];
  }
  a.L = L;
  a.step = f->step;
  a.offset = f->offset;
  a.chunks = f->chunks;
  int *err = device_error_word();
  if (!err) return fail(BK_ERR_CUDA, "device error word unavailable");
  const long long nb = (long long)a.ns[0] * a.ns[1] * a.ns[2];
  const unsigned g = nb < (1ll << 30) ? (unsigned)nb : (1u << 30);
  cudaStream_t st = as_stream(stream);
  const size_t es = dtype_size(f->dtype);
  const bool rows16 = L.row_major() && (L.bi * es) % 16 == 0 && L.size() * es / 16 <= 1024 &&
                      reinterpret_cast<uintptr_t>(arr) % 16 == 0 && (a.a0[2] * es) % 16 == 0 && (a.adim[2] * es) % 16 == 0 &&
                      reinterpret_cast<uintptr_t>(f->dat) % 16 == 0 && (f->offset * es) % 16 == 0 && (f->step * es) % 16 == 0 &&
                      a.ns[1] <= 65535 && a.ns[0] <= 65535;
  if (rows16 && nb > 0) {
    const dim3 grid3((unsigned)a.ns[2], (unsigned)a.ns[1], (unsigned)a.ns[0]);
    const unsigned nt = (unsigned)(L.size() * es / 16);
    if (to_brick)
      array_brick_rows_kernel<true><<<grid3, nt, 0, st>>>((char *)arr, grid, (char *)f->dat, a, (int)es, err);
    else
      array_brick_rows_kernel<false><<<grid3, nt, 0, st>>>((char *)arr, grid, (char *)f->dat, a, (int)es, err);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "array <-> brick copy launch");
    return BK_OK;
  }
  switch (f->dtype) {
    case BK_F64:
      if (to_brick) array_brick_kernel<double, true><<<g, 256, 0, st>>>((double *)arr, grid, (double *)f->dat, a, err);
      else array_brick_kernel<double, false><<<g, 256, 0, st>>>((double *)arr, grid, (double *)f->dat, a, err);
      break;
    case BK_F32:
      if (to_brick) array_brick_kernel<float, true><<<g, 256, 0, st>>>((float *)arr, grid, (float *)f->dat, a, err);
      else array_brick_kernel<float, false><<<g, 256, 0, st>>>((float *)arr, grid, (float *)f->dat, a, err);
      break;
    default:
      if (to_brick)
        array_brick_kernel<unsigned short, true><<<g, 256, 0, st>>>((unsigned short *)arr, grid, (unsigned short *)f->dat, a, err);
      else
        array_brick_kernel<unsigned short, false><<<g, 256, 0, st>>>((unsigned short *)arr, grid, (unsigned short *)f->dat, a, err);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "array <-> brick copy launch");
  return BK_OK;
}

}  // namespace bk

using namespace bk;

extern "C" {

int bk_copy_to_bricks(const void *arr, const long dim[3], const long pad[3], const long ghost[3], const unsigned *grid,
                      const bk_field *f, const bk_layout *lay, void *stream) {
  return array_brick(true, const_cast<void *>(arr), dim, pad, ghost, grid, f, lay, stream);
}

int bk_copy_from_bricks(void *arr, const long dim[3], const long pad[3], const long ghost[3], const unsigned *grid,
                        const bk_field *f, const bk_layout *lay, void *stream) {
  return array_brick(false, arr, dim, pad, ghost, grid, f, lay, stream);
}

}  // extern "C"
