// Instantiations of the sweep kernels for float storage.
#include "sweep2_kernel.cuh"

namespace bk {

#define BK_CASE(BK_, BJ_, BI_, R_, FAM_, RM_, ACC_)                   \
  if (p.r == R_ && p.fam == FAM_ && p.rm == RM_ && p.acc == ACC_)     \
    return launch_sweep<float, BK_, BJ_, BI_, R_, FAM_, RM_, ACC_>(a, tp, s);

#define BK_SHAPE_SET(BK_, BJ_, BI_, ACC_)          \
  BK_CASE(BK_, BJ_, BI_, 1, FAM_STAR, true, ACC_)  \
  BK_CASE(BK_, BJ_, BI_, 2, FAM_STAR, true, ACC_)  \
  BK_CASE(BK_, BJ_, BI_, 4, FAM_STAR, true, ACC_)  \
  BK_CASE(BK_, BJ_, BI_, 1, FAM_CUBE, true, ACC_)  \
  BK_CASE(BK_, BJ_, BI_, 2, FAM_CUBE, true, ACC_)  \
  BK_CASE(BK_, BJ_, BI_, 4, FAM_GENERIC, true, ACC_) \
  BK_CASE(BK_, BJ_, BI_, 4, FAM_GENERIC, false, ACC_)

// pipelined kernel (row-major layouts, aligned fields); the generic family's tap offsets
// are rebased onto that kernel's padded tile
#define BK_CASE2(BK_, BJ_, BI_, R_, FAM_, ACC_)                                         \
  if (p.r == R_ && p.fam == FAM_ && p.acc == ACC_) {                                    \
    if (FAM_ == FAM_GENERIC) {                                                          \
      typedef Sweep2Geom<float, BK_, BJ_, BI_, R_> G;                                     \
      for (int t = 0; t < tp.n; ++t)                                                    \
        tp.toff[t] = (p.offs[t][0] * G::EJ + p.offs[t][1]) * G::EI + p.offs[t][2];      \
    }                                                                                   \
    return launch_sweep2<float, BK_, BJ_, BI_, R_, FAM_, ACC_>(a, tp, s);                 \
  }

#define BK_SHAPE_SET2(BK_, BJ_, BI_, ACC_)   \
  BK_CASE2(BK_, BJ_, BI_, 1, FAM_STAR, ACC_) \
  BK_CASE2(BK_, BJ_, BI_, 2, FAM_STAR, ACC_) \
  BK_CASE2(BK_, BJ_, BI_, 4, FAM_STAR, ACC_) \
  BK_CASE2(BK_, BJ_, BI_, 1, FAM_CUBE, ACC_) \
  BK_CASE2(BK_, BJ_, BI_, 2, FAM_CUBE, ACC_) \
  BK_CASE2(BK_, BJ_, BI_, 4, FAM_GENERIC, ACC_)

int sweep_dispatch_f32(const SweepPlan &p, const SweepArgs &a, Taps &tp, cudaStream_t s) {
  if (p.v2) {
    if (p.shape == 0) {
      // mirror-symmetric cubes: class sums streamed along i (native or compensated arithmetic)
      if (p.sym && p.fam == FAM_CUBE && p.istream && (p.acc == ACCM_NATIVE || p.acc == ACCM_COMP)) {
        if (p.acc == ACCM_NATIVE && p.r == 1) return launch_sweep2<float, 8, 8, 8, 1, FAM_CUBESYM, ACCM_NATIVE, false, true>(a, tp, s);
        if (p.acc == ACCM_NATIVE && p.r == 2) return launch_sweep2<float, 8, 8, 8, 2, FAM_CUBESYM, ACCM_NATIVE, false, true>(a, tp, s);
        if (p.r == 1) return launch_sweep2<float, 8, 8, 8, 1, FAM_CUBESYM, ACCM_COMP, false, true>(a, tp, s);
        if (p.r == 2) return launch_sweep2<float, 8, 8, 8, 2, FAM_CUBESYM, ACCM_COMP, false, true>(a, tp, s);
      }
      // ... one brick at a time on column pairs (BK_SWEEP_ISTREAM=0)
      if (p.sym && p.fam == FAM_CUBE && p.acc == ACCM_NATIVE) {
        if (p.symij && p.r == 1) return launch_sweep2<float, 8, 8, 8, 1, FAM_CUBESYM_IJ, ACCM_NATIVE>(a, tp, s);
        if (p.symij && p.r == 2) return launch_sweep2<float, 8, 8, 8, 2, FAM_CUBESYM_IJ, ACCM_NATIVE>(a, tp, s);
        if (p.r == 1) return launch_sweep2<float, 8, 8, 8, 1, FAM_CUBESYM, ACCM_NATIVE>(a, tp, s);
        if (p.r == 2) return launch_sweep2<float, 8, 8, 8, 2, FAM_CUBESYM, ACCM_NATIVE>(a, tp, s);
      }
      BK_SHAPE_SET2(8, 8, 8, ACCM_NATIVE)
      BK_SHAPE_SET2(8, 8, 8, ACCM_COMP)
    } else if (p.shape == 1) {
      BK_SHAPE_SET2(4, 4, 4, ACCM_NATIVE)
    } else if (p.shape == 2) {
      BK_SHAPE_SET2(16, 8, 8, ACCM_NATIVE)
    } else if (p.shape == 3) {
      BK_SHAPE_SET2(8, 8, 32, ACCM_NATIVE)
    }
  }
  // the generic family of the one-shot kernel uses the host-computed offsets
  if (p.fam == FAM_GENERIC)
    for (int t = 0; t < tp.n; ++t) tp.toff[t] = p.toff1[t];
  if (p.shape == 0) {
    BK_SHAPE_SET(8, 8, 8, ACCM_NATIVE)
    BK_SHAPE_SET(8, 8, 8, ACCM_COMP)
  } else if (p.shape == 1) {
    BK_SHAPE_SET(4, 4, 4, ACCM_NATIVE)
  } else if (p.shape == 2) {
    BK_SHAPE_SET(16, 8, 8, ACCM_NATIVE)
  } else if (p.shape == 3) {
    BK_SHAPE_SET(8, 8, 32, ACCM_NATIVE)
  }
  return fail(BK_ERR_UNSUPPORTED, "no f32 sweep kernel for this brick shape / stencil / accumulation");
}

}  // namespace bk
