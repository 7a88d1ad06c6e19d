// Instantiations of the sweep kernel for double storage.
#include "sweep_kernel.cuh"

namespace bk {

#define BK_CASE(BK_, BJ_, BI_, R_, FAM_, RM_, ACC_)                   \
  if (p.r == R_ && p.fam == FAM_ && p.rm == RM_ && p.acc == ACC_)     \
    return launch_sweep<double, BK_, BJ_, BI_, R_, FAM_, RM_, ACC_>(a, tp, s);

#define BK_SHAPE_SET(BK_, BJ_, BI_, ACC_)          \
  BK_CASE(BK_, BJ_, BI_, 1, FAM_STAR, true, ACC_)  \
  BK_CASE(BK_, BJ_, BI_, 2, FAM_STAR, true, ACC_)  \
  BK_CASE(BK_, BJ_, BI_, 4, FAM_STAR, true, ACC_)  \
  BK_CASE(BK_, BJ_, BI_, 1, FAM_CUBE, true, ACC_)  \
  BK_CASE(BK_, BJ_, BI_, 2, FAM_CUBE, true, ACC_)  \
  BK_CASE(BK_, BJ_, BI_, 4, FAM_GENERIC, true, ACC_) \
  BK_CASE(BK_, BJ_, BI_, 4, FAM_GENERIC, false, ACC_)

int sweep_dispatch_f64(const SweepPlan &p, const SweepArgs &a, const Taps &tp, cudaStream_t s) {
  if (p.shape == 0) {
    BK_SHAPE_SET(8, 8, 8, ACCM_NATIVE)
    BK_SHAPE_SET(8, 8, 8, ACCM_FF)

  } else if (p.shape == 1) {
    BK_SHAPE_SET(4, 4, 4, ACCM_NATIVE)
  } else if (p.shape == 2) {
    BK_SHAPE_SET(16, 8, 8, ACCM_NATIVE)
  } else if (p.shape == 3) {
    BK_SHAPE_SET(8, 8, 32, ACCM_NATIVE)
  }
  return fail(BK_ERR_UNSUPPORTED, "no f64 sweep kernel for this brick shape / stencil / accumulation");
}

}  // namespace bk
