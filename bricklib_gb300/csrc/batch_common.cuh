// Types shared by the batched form (batch.cu) and the server (serve.cu).
#pragma once

#include "sweep_kernel.cuh"

namespace bk {

constexpr int BATCH_MAX_ST = 8;


// What one per-stencil launch needs besides the work segment.
struct BatchStencil {
  SweepPlan plan;  // family, radius, accumulation, shape, row-major
  Taps taps;
};

int plan_stencil(const bk_stencil *st, const Layout &L, int dtype, int acc, SweepPlan *plan, Taps *tp);
int batch_launch_sweep(const BatchStencil &bs, int dtype, const BatchDomain *doms, unsigned ndom, const uint2 *work,
                       unsigned nwork, int parity, const Layout &L, int *err, int grid_cap, bool aligned,
                       cudaStream_t s);
int batch_launch_fill(const BatchDomain *doms, unsigned ndom, const uint3 *pairs, unsigned npairs, int parity,
                      size_t brick_bytes, int *err, cudaStream_t s);

}  // namespace bk
