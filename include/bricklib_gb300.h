/*
 * bricklib_gb300.h -- C ABI of the GB300 brick stencil engine (libbrick_gb300.so).
 *
 * This is the boundary a bricklib user binds instead of the reference's device
 * layer.  Every entry point is plain C: device pointers, host pointers, sizes and
 * a cudaStream_t passed as `void *` (NULL = the legacy default stream).  No call
 * exits, traps or throws; each returns a bk_status and leaves a message for
 * bk_last_error() (thread-local).  Calls are stream-ordered and do not
 * synchronise unless their description says so.
 *
 * Data model (the reference's, include/brick.h):
 *   BrickStorage  `chunks` chunks of `step` elements each (brick.h:53-82)
 *   BrickInfo<3>  unsigned adj[nbricks][27]; slot (dk+1)*9+(dj+1)*3+(di+1) holds the
 *                 storage index of the neighbour at (dk,dj,di), 13 = the brick itself
 *                 (brick.h:96-127)
 *   Brick         a field inside the storage: element (k,j,i) of brick b lives at
 *                 dat[adj-resolved b * step + offset + layout(k,j,i)] (brick.h:353-395)
 * layout(k,j,i) is the vector-fold order of _BrickAccessor (brick.h:213-327): with
 * brick dims (BK,BJ,BI) and fold (FK,FJ,FI) the vector index is
 * ((k/FK)*(BJ/FJ) + j/FJ)*(BI/FI) + i/FI and the lane ((k%FK)*FJ + j%FJ)*FI + i%FI.
 * Triples are always (k, j, i) with i contiguous.
 */
#ifndef BRICKLIB_GB300_H
#define BRICKLIB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BK_ABI_VERSION 1
#define BK_MAX_TAPS 343 /* a radius-3 cube */

typedef enum bk_status {
  BK_OK = 0,
  BK_ERR_ARG = 1,         /* invalid argument (message says which) */
  BK_ERR_CUDA = 2,        /* a CUDA runtime call failed */
  BK_ERR_NOMEM = 3,       /* device or host allocation failed */
  BK_ERR_UNSUPPORTED = 4, /* valid request the library has no kernel for */
  BK_ERR_BOUNDS = 5,      /* a kernel met an out-of-range brick index and skipped it */
  BK_ERR_BUDGET = 6,      /* serving: request exceeds the HBM budget */
  BK_ERR_STATE = 7,       /* call not valid in the object's current state */
  BK_ERR_TIMEOUT = 8      /* a bounded device wait gave up */
} bk_status;

typedef enum bk_dtype { BK_F64 = 0, BK_F32 = 1, BK_BF16 = 2 } bk_dtype;

/* Arithmetic of a sweep.
 * BK_ACC_NATIVE      accumulate in the storage type (FP32 for BF16 storage)
 * BK_ACC_COMPENSATED FP32/BF16 storage: FP32 accumulation with Neumaier compensation
 * BK_ACC_FLOATFLOAT  FP64 storage: products and sums in float-float (pairs of FP32,
 *                    error-free transforms of Dekker 1971 / Knuth TwoSum), relative
 *                    error below 1e-13 per point; the FP64 units are not used */
typedef enum bk_acc { BK_ACC_NATIVE = 0, BK_ACC_COMPENSATED = 1, BK_ACC_FLOATFLOAT = 2 } bk_acc;

/* Brick dims and vector fold, (k, j, i); a fold of 1 means that axis is not folded.
 * Brick<Dim<8,8,8>, Dim<4,8>> is {{8,8,8},{1,4,8}}. */
typedef struct bk_layout {
  int bdim[3];
  int fold[3];
} bk_layout;

/* One field of a BrickStorage on the device: Brick(bInfo, storage, offset). */
typedef struct bk_field {
  void *dat;     /* device pointer to BrickStorage::dat */
  long chunks;   /* BrickStorage::chunks */
  size_t step;   /* BrickStorage::step, elements per chunk */
  size_t offset; /* Brick offset within a chunk, elements */
  int dtype;     /* bk_dtype of the elements */
} bk_field;

/* A stencil: out(k,j,i) = sum_t coeff[t] * in(k+off[t][0], j+off[t][1], i+off[t][2]).
 * The reference compiles each stencil from a Python script (stencils/7pt.py, mpi*.py)
 * into one kernel; here the tap list is data. |offset| on each axis must not exceed
 * the brick dim on that axis (the accessor reaches one neighbour brick, brick.h:232-245). */
/* Pointwise operations around the weighted sum, for non-linear stencils such as the
 * reference's cond kernel (stencils/cond.py, 3axis.cpp:94-163):
 *   out = post( sum_t coeff[t] * pre(in(...)) )
 * BK_OP_RELU is max(x, 0), BK_OP_ABS is |x|.  Both default to BK_OP_NONE (zero-filled). */
#define BK_OP_NONE 0
#define BK_OP_RELU 1
#define BK_OP_ABS 2

typedef struct bk_stencil {
  int npoints;
  int offsets[BK_MAX_TAPS][3];
  double coeff[BK_MAX_TAPS];
  int pre_op;  /* applied to every input value */
  int post_op; /* applied to the sum */
} bk_stencil;

/* ------------------------------------------------------------------ runtime */

int bk_abi_version(void);
/* Message of the last failed call on this host thread ("" if none). */
const char *bk_last_error(void);
/* Select the CUDA device for this host thread. */
int bk_set_device(int device);
int bk_device_synchronize(void);
int bk_stream_synchronize(void *stream);

/* Device memory.  bk_device_malloc replaces gpuMalloc in movBrickInfo /
 * movBrickStorage (include/brick-gpu.h:42-103); bk_device_free replaces the
 * gpuFree deleter of the device BrickStorage (brick-gpu.h:97-101). */
int bk_device_malloc(void **dptr, size_t bytes);
int bk_device_free(void *dptr);
/* Page-locked host memory for copies that overlap with kernels.  It is mapped into the
 * device's address space at the same address, so it can also hold a field that kernels
 * of this library read or write directly: an output field in it receives a sweep's results
 * straight over the CPU-GPU link (NVLink-C2C on GB300), with no separate device-to-host copy. */
int bk_host_malloc(void **hptr, size_t bytes);
int bk_host_free(void *hptr);
/* Stream-ordered copy; kind: 0 host->device, 1 device->host, 2 device->device. */
int bk_memcpy(void *dst, const void *src, size_t bytes, int kind, void *stream);
int bk_memset(void *dptr, int value, size_t bytes, void *stream);

/* movBrickInfo(bInfo, cudaMemcpyHostToDevice) (include/brick-gpu.h:42-55):
 * allocates nbricks*27 unsigned on the device and copies the adjacency list.
 * Synchronous, like the reference's cudaMemcpy. Free with bk_device_free. */
int bk_info_to_device(const unsigned *adj_host, unsigned nbricks, unsigned **adj_dev);
/* movBrickStorage(bStorage, cudaMemcpyHostToDevice) (include/brick-gpu.h:84-103):
 * allocates chunks*step elements and copies them.  Synchronous. */
int bk_storage_to_device(const void *host, long chunks, size_t step, int dtype, void **dev);
/* movBrickStorage(bStorage, cudaMemcpyDeviceToHost) into caller memory.  Synchronous. */
int bk_storage_to_host(const void *dev, long chunks, size_t step, int dtype, void *host);

/* Measured FMA rate of the current device for BK_F64 or BK_F32 (flop/s, an FMA counted
 * as 2), from a kernel of independent FMA chains timed with CUDA events on `stream`.
 * Synchronous.  Used as the compute roofline of the sweep; no reference counterpart. */
int bk_measure_fma_rate(int dtype, void *stream, double *flops_per_s);

/* Seeded synthetic input on the device: element p of dat (n elements of dtype) becomes
 * lo + (hi - lo) * u with u = (splitmix64(seed + p) >> 11) * 2^-53, in separately
 * rounded double arithmetic, then converted to the storage type.  Stands in for the
 * reference's unseeded randomArray (src/multiarray.cpp:13-40). */
int bk_fill_uniform(void *dat, size_t n, int dtype, uint64_t seed, double lo, double hi, void *stream);

/* ------------------------------------------------------------------ the sweep */

/* Validate a stencil for a layout; on success writes the radius (max |offset|) and the
 * kernel family used: 1 star (taps on the axes), 2 cube (full (2r+1)^3 box), 0 generic. */
int bk_stencil_check(const bk_stencil *st, const bk_layout *lay, int *radius, int *family);

/* One stencil sweep over a brick list.  Replaces the per-brick CUDA kernels of the
 * reference -- d3pt7_brick / d3pt7_brick_trans (stencils/3axis.cu:12-37), brick_kernel
 * (weak/main.cu:35-43, strong/main.cu:85-111) -- and their launch (one kernel over the
 * listed bricks instead of one 32-thread block per grid position, weak/main.cu:277-282).
 *   adj        device BrickInfo adjacency, nbricks x 27
 *   in, out    fields (may share a storage, e.g. interleaved bIn/bOut at offsets 0 and 512,
 *              stencils/3axis.cu:119-121; in and out must not overlap element-wise)
 *   blist      device list of nlist brick indices to compute (e.g. the interior bricks
 *              grid[GB..STRIDEB-GB)^3 of 3axis.cu:167)
 * Neighbour or list indices >= chunks/nbricks are clamped to brick 0 and reported by
 * bk_error_flags() as BK_ERR_BOUNDS; the kernel never reads outside the storage.
 * Four kernels implement it: two TMA-fed ones for 7/13/25-point stars on row-major 8x8x8
 * bricks with 16-byte aligned input (FP32 / BF16: runs of i-adjacent list entries share
 * their i-neighbour bricks; FP64: per-brick staging), a pipelined one (row-major layouts,
 * 16-byte aligned input; FP64 mirror-symmetric cubes carry per-column sums along runs of
 * i-adjacent list entries, so a list in grid order is fastest) and a one-shot one
 * (everything).  The FP32 / BF16 row kernel and the cube kernels on 8x8x8 bricks store
 * output pairs: they need every output brick to start on a two-element boundary, and
 * other output fields take per-element stores.  The environment variables
 * BK_SWEEP_ONESHOT=1 and BK_SWEEP_PIPELINED=1 override the built-in choice (used by the
 * parity tests); BK_TMA_ROW=0 selects per-brick staging for FP32 / BF16, BK_TMA_GROUP=0/1
 * turns the row kernel's grouped copies of full runs off/on, BK_TMA_STAGES (2..4) and
 * BK_TMA_IFACE (narrow / whole) tune the TMA-fed kernels, BK_SWEEP_ISTREAM=0 computes
 * FP64 mirror-symmetric cubes one brick at a time. */
int bk_sweep(const unsigned *adj, unsigned nbricks, const bk_field *in, const bk_field *out,
             const unsigned *blist, unsigned nlist, const bk_stencil *st, const bk_layout *lay,
             int acc, void *stream);

/* Which kernel bk_sweep would launch for these fields, stencil, layout and accumulation
 * (no launch): *name = "sweep_star_row_kernel", "sweep_star_tma_kernel", "sweep2_kernel" or
 * "sweep_kernel" (a static string).  No reference counterpart: a diagnostic of this implementation. */
int bk_sweep_kernel(const bk_field *in, const bk_field *out, const bk_stencil *st, const bk_layout *lay,
                    int acc, const char **name);

/* Reads and clears the device error word set by kernels of this library on the
 * current device (synchronises the stream).  *flags = 0 when all launches were clean;
 * bit 0: out-of-range brick index clamped; bit 1: bounded wait timed out. */
int bk_error_flags(void *stream, int *flags);

/* ------------------------------------------------------------------ 4-D bricks */

/* Four-dimensional bricks (weak/main-4d.cpp: Brick<Dim<4,4,4,4>, Dim<VFOLD>>, the 9-point
 * star of stencils/mpi9pt.py).  bdim / fold and tap offsets are (l, k, j, i), outermost
 * first; folds apply to the innermost dimensions as in the 3-D layout.  Adjacency lists hold
 * 81 entries per brick, slot ((dl+1)*3 + (dk+1))*9 + (dj+1)*3 + (di+1) (init_grid<4>). */
#define BK_MAX_TAPS4 81

typedef struct bk_layout4 {
  int bdim[4];
  int fold[4];
} bk_layout4;

typedef struct bk_stencil4 {
  int npoints;
  int offsets[BK_MAX_TAPS4][4];
  double coeff[BK_MAX_TAPS4];
} bk_stencil4;

/* One 4-D sweep over the listed bricks: out = sum c_t * in(l+dl, k+dk, j+dj, i+di).  4x4x4x4
 * bricks, FP64 or FP32 storage (native arithmetic), radius up to 2, lists of fewer than 2^31
 * bricks.  Same field, list and error conventions as bk_sweep.  A tap list that is exactly the
 * star of its radius is summed in the order centre, then along l, k, j, i the distances -R..-1,
 * 1..R, whatever order it is listed in; any other tap list in its listed order. */
int bk_sweep4(const unsigned *adj, unsigned nbricks, const bk_field *in, const bk_field *out, const unsigned *blist,
              unsigned nlist, const bk_stencil4 *st, const bk_layout4 *lay, void *stream);

/* ------------------------------------------------------------------ ghost zones */

/* Ghost-zone fill / periodic wrap on the device.  For every (dst, src) pair of brick
 * storage indices copies the field's BRICKSIZE elements of brick src into brick dst.
 * Replaces, on one GPU, the periodic BrickDecomp::exchange of a single rank
 * (include/brick-mpi.h:466-499 on the periodic communicator of weak/args.cpp:105-108)
 * and the D2H / MPI / H2D round trip around it (weak/main.cu:251-275). */
int bk_ghost_fill(const unsigned *pairs, unsigned npairs, const bk_field *f, const bk_layout *lay,
                  void *stream);

/* Host helper: periodic (dst, src) plan for an init_grid layout of nb+2*gb bricks per axis
 * (gb ghost bricks each side, grid as returned by init_grid).  Writes up to `cap` pairs
 * and returns the count needed in *npairs (call with pairs = NULL to size). */
int bk_periodic_plan(const unsigned *grid, const long nb[3], const long gb[3], unsigned *pairs,
                     long cap, long *npairs);

/* Batched contiguous copies inside device memory: the reference's RegionLink / cudaCopy
 * (strong/main.cu:60-83).  links: device array of nlinks {from, to, bytes} triples (uint64
 * each); bytes must be a multiple of 8.  All CTAs share every link, so a few large links
 * (the regions of a BrickDecomp exchange) use the whole GPU. */
int bk_region_copy(const uint64_t *links, unsigned nlinks, void *stream);

/* ------------------------------------------------------------------ BrickDecomp layout */

/* BrickDecomp's layout producer without MPI (include/brick-mpi.h:178-464): the storage
 * order in which the inner region, each skin region (in skin-list order, page padded) and
 * each ghost region are contiguous runs of bricks; the grid (position -> brick), the
 * BrickInfo adjacency and the ghost / skin region records.  On one GPU with periodic
 * boundaries the exchange (brick-mpi.h:466-499 with one rank) copies skin[i] into ghost[i]
 * for every record: bk_decomp_exchange_links writes those copies as bk_region_copy links.
 * Conventions are the reference's: dimension 0 is the contiguous one; a region / neighbour
 * is a BitSet bit field (bitset.h: side +p of dimension p-1 is bit p, side -p is bit 31+p). */
typedef struct bk_decomp bk_decomp;

/* g_region of brick-mpi.h:185-193: neighbour set, skin-list range [skin_st, skin_ed), first
 * brick pos, length len (bricks, including first_pad / last_pad padding bricks). */
typedef struct bk_decomp_region {
  uint64_t neighbor;
  unsigned skin_st, skin_ed, pos, len, first_pad, last_pad;
} bk_decomp_region;

/* BrickDecomp(dims, depth, numfield) + initialize(skinlist) (brick-mpi.h:298-464).
 *   dim        1..4
 *   dims       interior size per dimension in elements, contiguous dimension first
 *   bdims      brick dims, contiguous dimension first
 *   depth      ghost depth in elements (a multiple of every brick dim)
 *   elem_bytes bytes of one element (sizeof(bElem)); with numfield interleaved fields a brick
 *              occupies bdims product x elem_bytes x numfield bytes
 *   pagesize   page padding granule in bytes (the reference uses sysconf(_SC_PAGESIZE));
 *              1 gives the unpadded layout of DECOMP_PAGEUNALIGN builds
 *   skinlist   nskin regions, e.g. the reference's skin3d_good order */
int bk_decomp_create(int dim, const unsigned *dims, const unsigned *bdims, unsigned depth, unsigned numfield,
                     size_t elem_bytes, long pagesize, const uint64_t *skinlist, unsigned nskin, bk_decomp **out);
/* nbricks (storage chunks, = sep_pos[2]), grid positions (product of dims + 2 x ghost
 * bricks), number of ghost (= skin) records, sep_pos[3] (inner / skin / ghost ends). */
int bk_decomp_info(const bk_decomp *d, unsigned *nbricks, size_t *grid_size, unsigned *nregions, unsigned *sep_pos);
/* grid[position] = brick, position = sum of coordinate x stride, dimension 0 fastest. */
int bk_decomp_grid(const bk_decomp *d, unsigned *grid);
/* nbricks x 3^dim adjacency (slot = sum of (offset_d + 1) x 3^d; 0 outside the grid). */
int bk_decomp_adjacency(const bk_decomp *d, unsigned *adj);
/* ghost and skin records (nregions each) and the per-skin-list-entry sizes (nskin). */
int bk_decomp_regions(const bk_decomp *d, bk_decomp_region *ghost, bk_decomp_region *skin, long *skin_size);
/* The periodic single-GPU exchange of a storage at `dat` with chunk stride step_bytes as
 * nregions {from, to, bytes} links (host array of 3 x nregions) for bk_region_copy. */
int bk_decomp_exchange_links(const bk_decomp *d, const void *dat, size_t step_bytes, uint64_t *links);
void bk_decomp_destroy(bk_decomp *d);

/* ------------------------------------------------------------------ precision form */

/* Element-wise conversion of the listed bricks of field src into field dst (any pair of
 * storage types; round to nearest even).  Used to start FP32 / BF16 runs from the same
 * values as an FP64 run. */
int bk_convert(const bk_field *src, const bk_field *dst, const unsigned *blist, unsigned nlist,
               const bk_layout *lay, void *stream);

/* FP64 error norms of field a against field ref over the listed bricks, reduced on the
 * device in FP64: out[0] = max |a - ref|, out[1] = sum (a - ref)^2, out[2] = max |ref|,
 * out[3] = sum ref^2.  Synchronises the stream.  Its partial sums live in a device buffer
 * the library allocates on the first call per device and keeps until exit. */
int bk_field_norms(const bk_field *a, const bk_field *ref, const unsigned *blist, unsigned nlist,
                   const bk_layout *lay, void *stream, double out[4]);

/* bk_field_norms without any allocation, for callers that cannot call cudaMalloc: a
 * serving loop with a latency budget (cudaMalloc / cudaFree can synchronise the device and
 * stall every stream) or a process whose device memory is all reserved up front by another
 * allocator.  No counterpart in the reference.
 * Same inputs and outputs as bk_field_norms; its scratch (one FP64 partial per listed brick,
 * the result and an error word, ~512 KiB) is a file-scope static device array that every GPU
 * loading this library holds until exit, so nlist may not exceed
 * BK_NORMS_NOALLOC_MAX_BRICKS (larger lists: split them and combine -- max of the maxima,
 * sum of the sums).  Calls no cudaMalloc / cudaFree.  The first call on a device looks up
 * the array's device address (cudaGetSymbolAddress) for that device; make that first call
 * before any stream capture.  All calls share the array and it keeps the last call's
 * contents: calls whose work overlaps on the GPU race.  Synchronises the stream.  One
 * difference from bk_field_norms: a listed brick out of range (skipped, never read) makes
 * this call return BK_ERR_BOUNDS itself, where bk_field_norms returns BK_OK and raises the
 * bounds bit of bk_error_flags. */
#define BK_NORMS_NOALLOC_MAX_BRICKS 16384
int bk_field_norms_noalloc(const bk_field *a, const bk_field *ref, const unsigned *blist, unsigned nlist,
                           const bk_layout *lay, void *stream, double out[4]);

/* Seeded initial field: the sum of `nwaves` sines with integer wave numbers in 1..4 and
 * random phases on the periodic interior, plus `noise` times uniform[-1,1) noise, written
 * to every brick of an init_grid layout of grid_bricks (k,j,i) bricks with ghost_bricks
 * ghost bricks per side (brick index = linear grid position).  Ghost bricks receive the
 * periodic continuation.  Evaluated in FP32 and stored in the field's type. */
int bk_fill_sines(const bk_field *f, const bk_layout *lay, const long grid_bricks[3],
                  const long ghost_bricks[3], int nwaves, uint64_t seed, double noise, void *stream);

/* ------------------------------------------------------------------ array <-> bricks */

/* copyToBrick / copyFromBrick (include/bricksetup.h:172-221) on the device: the region
 * dim (k,j,i) of a device array of extent dim + 2*(pad + ghost) is copied to / from the
 * bricks at grid positions ghost/B .. (dim+ghost)/B - 1, grid (device, row-major over
 * (dim + 2*ghost)/B bricks per axis) mapping positions to storage indices, as the host
 * copies do with grid_ptr.  The array has the field's element type.  pad may be negative
 * down to -ghost (an array holding the region without its ghost cells).  The reference
 * times these host copies as "To"/"From" in stencils/copy.cpp:32-58. */
int bk_copy_to_bricks(const void *arr, const long dim[3], const long pad[3], const long ghost[3],
                      const unsigned *grid, const bk_field *f, const bk_layout *lay, void *stream);
int bk_copy_from_bricks(void *arr, const long dim[3], const long pad[3], const long ghost[3],
                        const unsigned *grid, const bk_field *f, const bk_layout *lay, void *stream);

/* ------------------------------------------------------------------ time steps */

/* T time steps, ping-pong between fields a and b (weak/main.cu:277-282): before every
 * `fill_every`-th step (0 = never) the ghost plan is applied to the current input field,
 * then the sweep runs over blist.  After the call the newest values are in a when T is
 * even and in b when T is odd.  With use_graph != 0 the T steps are captured once into a
 * CUDA graph and replayed (launch-bound small domains). */
int bk_steps(const unsigned *adj, unsigned nbricks, const bk_field *a, const bk_field *b,
             const unsigned *blist, unsigned nlist, const unsigned *pairs, unsigned npairs,
             const bk_stencil *st, const bk_layout *lay, int acc, int steps, int fill_every,
             int use_graph, void *stream);

/* ------------------------------------------------------------------ batched form */

/* One domain of a batch: an independent brick grid with two ping-pong fields in one
 * device storage, the bricks to compute each step and its ghost plan (host arrays, copied
 * at creation).  The reference advances several subdomains in one launch in
 * strong/main.cu:85-100 (brick_kernel over Brick3D barr[], subdomain = blockIdx.x / strideb);
 * a batch generalises that to domains of any size and stencil. */
typedef struct bk_batch_domain {
  const unsigned *adj;   /* device adjacency, nbricks x 27 */
  unsigned nbricks;
  void *dat;             /* device storage holding both fields */
  long chunks;
  size_t step;           /* elements per chunk */
  size_t off0, off1;     /* element offsets of the two ping-pong fields */
  const unsigned *blist; /* host: bricks computed every step */
  unsigned nlist;
  const unsigned *pairs; /* host: ghost plan, npairs (dst, src) brick pairs */
  unsigned npairs;
  int stencil;           /* index into the batch's stencil array */
  /* Domains whose cell counts are not whole bricks (e.g. 40 cells on 16-wide bricks): n holds
   * the domain's cells (k, j, i), the brick grid covers them rounded up to whole bricks plus
   * one ghost brick per side, and grid (host, gdims (k, j, i) bricks, position (k*gj + j)*gi + i
   * -> brick) locates every cell.  Before every step a cell-level wrap fill writes each cell
   * within the stencil radius outside the domain with the value at its periodic image; cells
   * of partial bricks past n are computed by the sweep but belong to no domain.  n = {0,0,0}:
   * whole bricks (periodic wrap through the adjacency or the ghost plan, as above). */
  long n[3];
  long gdims[3];
  const unsigned *grid;
} bk_batch_domain;

typedef struct bk_batch bk_batch;

/* Build a batch: domains share one layout, one storage type and one accumulation mode; up to
 * 8 stencils, any that bk_sweep accepts.  Builds on the device the global (domain, brick) work
 * list, sorted by stencil, and the (domain, dst, src) fill list.  When the domains' storages
 * are brick ranges of one storage (same step and field offsets, ranges tiling it), the batch
 * is one brick set instead: a global adjacency (each domain's entries shifted by its first
 * brick), global work and fill lists, and steps of plain bk_sweep / bk_ghost_fill calls.
 * Per-domain storages take FP64 or FP32.  Field 0 (off0) holds the input of the first step. */
int bk_batch_create(bk_batch **batch, const bk_batch_domain *doms, unsigned ndom, const bk_stencil *stencils,
                    unsigned nstencils, const bk_layout *lay, int dtype, int acc);
/* Cap the number of CTAs of the persistent sweep launch (0 = one CTA per work group);
 * the autotuner's block-count knob. */
int bk_batch_set_grid(bk_batch *batch, int max_ctas);
/* Advance every domain `steps` steps: before every `fill_every`-th step (0 = never) the ghost
 * plans and the wrap fill of partial-brick domains are applied to the current input fields,
 * then one launch per stencil sweeps that stencil's segment of the work list.  With use_graph the sequence is captured once per
 * (steps, fill_every, parity) into a CUDA graph kept by the batch and replayed on later calls. */
int bk_batch_run(bk_batch *batch, int steps, int fill_every, int use_graph, void *stream);
/* Pipeline depth (2..4 stages of staged bricks) of the TMA-fed star sweeps launched from the
 * calling host thread; 0 restores each kernel's own default (3 for 4-byte radius-1 stars, else
 * 2).  Fewer stages leave room for more resident CTAs.  Returns BK_ERR_ARG for other values. */
int bk_set_pipeline_depth(int stages);
/* The calling thread's setting (0: the kernels' defaults). */
int bk_get_pipeline_depth(void);
/* Pipeline depth of the batch's TMA-fed star sweeps (0: the kernels' defaults; see
 * bk_set_pipeline_depth), the autotuner's launch-shape knob.  Drops the batch's captured graphs. */
int bk_batch_set_stages(bk_batch *batch, int stages);
/* on (default): the stencil segments of a step run as parallel branches (one stream each,
 * joined before the next step), so one segment's last wave overlaps the others' work; 0: one
 * after another on the caller's stream.  Drops the batch's captured graphs. */
int bk_batch_set_concurrent(bk_batch *batch, int on);
/* Which field (0 or 1) holds the newest values. */
int bk_batch_parity(const bk_batch *batch);
/* 1 when the batch's domains are brick ranges of one storage (a common brick step, ranges
 * tiling it without gaps) and the batch therefore runs as one brick set through the plain
 * sweep kernels; 0 for domains in storages of their own; -1 for NULL. */
int bk_batch_is_arena(const bk_batch *batch);
/* Synchronises the device and releases the batch's device memory and graphs; the domains'
 * storages belong to the caller. */
int bk_batch_destroy(bk_batch *batch);

/* ------------------------------------------------------------------ serving form */

/* One stencil job: a periodic domain of n (k,j,i) interior cells (multiples of the server's
 * brick dims), advanced `steps` steps with `stencil` in storage type dtype (BK_F64 or
 * BK_F32) and accumulation acc.  input / output are host arrays of n[0]*n[1]*n[2] elements
 * (k, j, i; i contiguous) that must stay valid until the job completes; page-locked memory
 * (bk_host_malloc) lets their copies overlap with other jobs' work. */
typedef struct bk_job_desc {
  long n[3];
  const bk_stencil *stencil;
  int steps;
  int dtype;
  int acc;
  const void *input;
  void *output;
} bk_job_desc;

typedef struct bk_server_report {
  unsigned long long submitted, admitted, completed, rejected, ticks;
  double p50_s, p99_s, mean_s, max_s; /* latency: submission to output on the host */
  double gstencil_s;                  /* completed point-steps / (last completion - first submission) */
  double span_s;
  size_t hbm_budget, hbm_peak;        /* bytes admitted against the budget: limit and peak */
} bk_server_report;

typedef struct bk_server bk_server;

/* Start a server on the current device: jobs are admitted first-in first-out while their
 * device bytes (storage, adjacency, staging, work lists) fit in hbm_budget and fewer than
 * max_active jobs run.  Every active job advances one step per scheduler tick; jobs join
 * and leave between ticks.  Layout: a row-major brick layout (e.g. 8x8x8, fold (4,8)). */
int bk_server_create(bk_server **server, size_t hbm_budget, const bk_layout *lay, int max_active);
/* Queue a job (thread safe).  BK_ERR_BUDGET when the job alone exceeds the budget. */
int bk_server_submit(bk_server *server, const bk_job_desc *job, unsigned long long *id);
/* Wait up to timeout_s for a job; BK_ERR_TIMEOUT if it is not done by then.  On success
 * the output array holds the result and *latency_s the submission-to-result time. */
int bk_server_wait(bk_server *server, unsigned long long id, double timeout_s, double *latency_s);
/* Wait up to timeout_s for every submitted job. */
int bk_server_drain(bk_server *server, double timeout_s);
int bk_server_stats(bk_server *server, bk_server_report *stats);
/* Stop the scheduler (jobs not yet done are abandoned), free all device memory. */
int bk_server_destroy(bk_server *server);

#ifdef __cplusplus
}
#endif
#endif /* BRICKLIB_GB300_H */
