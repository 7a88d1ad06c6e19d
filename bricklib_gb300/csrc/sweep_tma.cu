// Star stencils on row-major 8x8x8 bricks through the TMA-fed kernel: tensor-map encoding
// and the instantiations for every storage type.
#include <cstdlib>
#include <cstring>

#include "sweep_row_kernel.cuh"

namespace bk {

// cuTensorMapEncodeTiled, looked up through the runtime so that the library does not link
// the CUDA driver library directly (it loads on machines without a GPU driver).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (EncodeTiledFn) nullptr;
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

bool star_tma_maps(const SweepArgs &a, int dtype, int bk, int bj, int bi, int r, int iw, TmaMaps *maps) {
  const EncodeTiledFn encode = encode_tiled();
  if (!encode) return false;
  const size_t es = dtype_size(dtype);
  const CUtensorMapDataType ty = dtype == BK_F64   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64
                                 : dtype == BK_F32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                                   : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
  const char *base = reinterpret_cast<const char *>(a.in) + a.in_off * es;
  const size_t plane = (size_t)bj * bi;
  // bulk-tensor rules: 16-byte aligned base and strides, box rows of whole 16-byte units
  // (the j-face box is r*bi elements wide and starts at (bj - r)*bi)
  if (reinterpret_cast<uintptr_t>(base) % 16 || (a.in_step * es) % 16 || ((size_t)bi * es) % 16) return false;
  if (plane > 256 || a.in_chunks < 1 || a.in_chunks > 0x7FFFFFFFll || a.in_step * es >= (1ull << 40)) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)plane, (cuuint64_t)bk, (cuuint64_t)a.in_chunks};
  const cuuint64_t strides[2] = {(cuuint64_t)(plane * es), (cuuint64_t)(a.in_step * es)};
  const cuuint32_t boxes[3][3] = {{(cuuint32_t)plane, (cuuint32_t)bk, 1},
                                  {(cuuint32_t)plane, (cuuint32_t)r, 1},
                                  {(cuuint32_t)(r * bi), (cuuint32_t)bk, 1}};
  const cuuint32_t estr[3] = {1, 1, 1};
  for (int m = 0; m < 3; ++m) {
    const CUresult e = encode(&maps->m[m], ty, 3, const_cast<char *>(base), dims, strides, boxes[m], estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (e != CUDA_SUCCESS) return false;
  }
  // narrow i faces: box (iw, bj, bk) of the 4-D view (i, j, k, brick)
  const cuuint64_t dims4[4] = {(cuuint64_t)bi, (cuuint64_t)bj, (cuuint64_t)bk, (cuuint64_t)a.in_chunks};
  const cuuint64_t strides4[3] = {(cuuint64_t)(bi * es), (cuuint64_t)(plane * es), (cuuint64_t)(a.in_step * es)};
  const cuuint32_t box4[4] = {(cuuint32_t)iw, (cuuint32_t)bj, (cuuint32_t)bk, 1};
  const cuuint32_t estr4[4] = {1, 1, 1, 1};
  if (((size_t)iw * es) % 16 || ((size_t)(bi - iw) * es) % 16) return false;
  return encode(&maps->m[3], ty, 4, const_cast<char *>(base), dims4, strides4, box4, estr4,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool row_group_maps(const SweepArgs &a, int dtype, int bk, int bj, int bi, int r, int nb, int slot_box,
                    TmaMaps *maps) {
  const EncodeTiledFn encode = encode_tiled();
  if (!encode) return false;
  const size_t es = dtype_size(dtype);
  const CUtensorMapDataType ty = dtype == BK_F64   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64
                                 : dtype == BK_F32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                                   : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
  const char *base = reinterpret_cast<const char *>(a.in) + a.in_off * es;
  const size_t plane = (size_t)bj * bi;
  if (a.in_chunks < nb + 2) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)plane, (cuuint64_t)bk, (cuuint64_t)a.in_chunks};
  const cuuint64_t strides[2] = {(cuuint64_t)(plane * es), (cuuint64_t)(a.in_step * es)};
  const cuuint32_t boxes[3][3] = {{(cuuint32_t)plane, (cuuint32_t)bk, (cuuint32_t)slot_box},
                                  {(cuuint32_t)plane, (cuuint32_t)r, (cuuint32_t)nb},
                                  {(cuuint32_t)(r * bi), (cuuint32_t)bk, (cuuint32_t)nb}};
  const cuuint32_t estr[3] = {1, 1, 1};
  for (int m = 0; m < 3; ++m) {
    const CUresult e = encode(&maps->m[4 + m], ty, 3, const_cast<char *>(base), dims, strides, boxes[m], estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (e != CUDA_SUCCESS) return false;
  }
  return true;
}

// Pipeline depth of the TMA-fed star kernels on this host thread (bk_set_pipeline_depth; 0:
// each kernel's default).
static thread_local int g_stages = 0;
int pipeline_depth_override() { return g_stages; }
void set_pipeline_depth_override(int stages) { g_stages = stages; }

int tma_stages(int dflt) {
  if (g_stages >= 2 && g_stages <= TMA_MAX_STAGES) return g_stages;
  const char *e = getenv("BK_TMA_STAGES");
  if (!e) return dflt;
  const int v = atoi(e);
  return v >= 2 && v <= TMA_MAX_STAGES ? v : dflt;
}

// i faces: narrow boxes (less shared memory, more copy requests) or whole bricks; BK_TMA_IFACE
// = narrow / whole overrides the per-type default
static bool narrow_iface(int dtype) {
  const char *e = getenv("BK_TMA_IFACE");
  if (e && !strcmp(e, "narrow")) return true;
  if (e && !strcmp(e, "whole")) return false;
  return dtype == BK_F64;
}

bool tma_row(const SweepPlan &p) {
  if (!p.tma || p.dtype == BK_F64 || p.acc == ACCM_FF || !p.out_pair) return false;
  const char *e = getenv("BK_TMA_ROW");
  return !(e && !strcmp(e, "0"));
}

#define BK_TMA_CASE(T_, R_, ACC_)                                                    \
  if (p.r == R_ && p.acc == ACC_)                                                   \
    return narrow_iface(p.dtype) ? launch_star_tma<T_, 8, 8, 8, R_, ACC_, true>(a, tp, p.dtype, s) \
                                 : launch_star_tma<T_, 8, 8, 8, R_, ACC_, false>(a, tp, p.dtype, s);
#define BK_TMA_RADII(T_, ACC_) BK_TMA_CASE(T_, 1, ACC_) BK_TMA_CASE(T_, 2, ACC_) BK_TMA_CASE(T_, 4, ACC_)
#define BK_ROW_CASE(T_, R_, ACC_) \
  if (p.r == R_ && p.acc == ACC_) return launch_star_row<T_, R_, ACC_>(a, tp, p.dtype, s);
#define BK_ROW_RADII(T_, ACC_) BK_ROW_CASE(T_, 1, ACC_) BK_ROW_CASE(T_, 2, ACC_) BK_ROW_CASE(T_, 4, ACC_)

int sweep_dispatch_tma(const SweepPlan &p, const SweepArgs &a, Taps &tp, cudaStream_t s) {
  if (p.fam != FAM_STAR || p.shape != 0 || !p.rm)
    return fail(BK_ERR_UNSUPPORTED, "the TMA sweep covers star stencils on row-major 8x8x8 bricks");
  switch (p.dtype) {
    case BK_F64:
      BK_TMA_RADII(double, ACCM_NATIVE)
      BK_TMA_RADII(double, ACCM_FF)
      break;
    case BK_F32:
      if (tma_row(p)) {
        BK_ROW_RADII(float, ACCM_NATIVE)
        BK_ROW_RADII(float, ACCM_COMP)
        break;
      }
      BK_TMA_RADII(float, ACCM_NATIVE)
      BK_TMA_RADII(float, ACCM_COMP)
      break;
    case BK_BF16:
      if (tma_row(p)) {
        BK_ROW_RADII(__nv_bfloat16, ACCM_NATIVE)
        BK_ROW_RADII(__nv_bfloat16, ACCM_COMP)
        break;
      }
      BK_TMA_RADII(__nv_bfloat16, ACCM_NATIVE)
      BK_TMA_RADII(__nv_bfloat16, ACCM_COMP)
      break;
  }
  return fail(BK_ERR_UNSUPPORTED, "no TMA sweep kernel for this storage type / radius / accumulation");
}

// Whether a sweep with these fields can take the TMA kernel (host-side rules only).
bool tma_eligible(const SweepPlan &p, const bk_field *in) {
  if (p.fam != FAM_STAR || p.shape != 0 || !p.rm || p.ops) return false;
  if (!(p.r == 1 || p.r == 2 || p.r == 4)) return false;
  const size_t es = dtype_size(in->dtype);
  const char *base = reinterpret_cast<const char *>(in->dat) + in->offset * es;
  return reinterpret_cast<uintptr_t>(base) % 16 == 0 && (in->step * es) % 16 == 0 && in->chunks <= 0x7FFFFFFFll;
}

}  // namespace bk

using namespace bk;

extern "C" int bk_set_pipeline_depth(int stages) {
  if (stages != 0 && (stages < 2 || stages > TMA_MAX_STAGES))
    return fail(BK_ERR_ARG, "bk_set_pipeline_depth: stages must be 0 (the kernels' defaults) or 2..4");
  set_pipeline_depth_override(stages);
  return BK_OK;
}

extern "C" int bk_get_pipeline_depth(void) { return pipeline_depth_override(); }
