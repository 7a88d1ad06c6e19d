// Host side of the sweep: stencil analysis, kernel selection, bk_sweep and bk_steps.
#include <cstdlib>
#include <cstring>
#include <string>

#include "sweep_kernel.cuh"

namespace bk {

int ghost_fill(const unsigned *pairs, unsigned npairs, const bk_field *f, const Layout &L, cudaStream_t s);

constexpr int GENERIC_R = 4;  // tile radius of the generic-family kernels

static int star_index(int dk, int dj, int di) {
  if (!dk && !dj && !di) return 0;
  const int d = abs(dk) + abs(dj) + abs(di);
  const int base = 1 + 6 * (d - 1);
  if (di) return base + (di > 0 ? 0 : 1);
  if (dj) return base + (dj > 0 ? 2 : 3);
  return base + (dk > 0 ? 4 : 5);
}

static int shape_of(const Layout &L) {
  if (L.bk == 8 && L.bj == 8 && L.bi == 8) return 0;
  if (L.bk == 4 && L.bj == 4 && L.bi == 4) return 1;
  if (L.bk == 16 && L.bj == 8 && L.bi == 8) return 2;
  if (L.bk == 8 && L.bj == 8 && L.bi == 32) return 3;
  return -1;
}

// Classify a tap list and lay its coefficients out in kernel order.
static int analyze(const bk_stencil *st, const Layout &L, SweepPlan *plan, Taps *tp) {
  if (!st) return fail(BK_ERR_ARG, "stencil is NULL");
  const int n = st->npoints;
  if (n < 1 || n > BK_MAX_TAPS) return fail(BK_ERR_ARG, "stencil npoints out of range");
  int r = 0;
  bool star = true;
  const int bd[3] = {L.bk, L.bj, L.bi};
  for (int t = 0; t < n; ++t) {
    int nz = 0;
    for (int d = 0; d < 3; ++d) {
      const int a = abs(st->offsets[t][d]);
      if (a > bd[d]) return fail(BK_ERR_ARG, "stencil offset exceeds the brick dim on its axis");
      if (a > r) r = a;
      nz += a != 0;
    }
    if (nz > 1) star = false;
  }
  if (r > GENERIC_R) return fail(BK_ERR_UNSUPPORTED, "stencil radius above 4");
  // exact-set tests: every canonical tap present exactly once
  int fam = FAM_GENERIC;
  static thread_local int seen[BK_MAX_TAPS];
  if (star && n == 1 + 6 * r && (r == 1 || r == 2 || r == 4)) {
    memset(seen, 0, sizeof(int) * n);
    bool ok = true;
    for (int t = 0; t < n && ok; ++t) {
      const int idx = star_index(st->offsets[t][0], st->offsets[t][1], st->offsets[t][2]);
      if (idx < 0 || idx >= n || seen[idx]++) ok = false;
    }
    if (ok) fam = FAM_STAR;
  } else if (n == (2 * r + 1) * (2 * r + 1) * (2 * r + 1) && (r == 1 || r == 2)) {
    memset(seen, 0, sizeof(int) * n);
    bool ok = true;
    const int w = 2 * r + 1;
    for (int t = 0; t < n && ok; ++t) {
      const int idx = ((st->offsets[t][0] + r) * w + (st->offsets[t][1] + r)) * w + st->offsets[t][2] + r;
      if (seen[idx]++) ok = false;
    }
    if (ok) fam = FAM_CUBE;
  }
  plan->rm = L.row_major();
  if (!plan->rm) fam = FAM_GENERIC;
  plan->fam = fam;
  plan->r = fam == FAM_GENERIC ? GENERIC_R : r;
  plan->shape = shape_of(L);
  if (st->pre_op < BK_OP_NONE || st->pre_op > BK_OP_ABS || st->post_op < BK_OP_NONE || st->post_op > BK_OP_ABS)
    return fail(BK_ERR_ARG, "stencil pre_op / post_op must be BK_OP_NONE, BK_OP_RELU or BK_OP_ABS");
  plan->ops = st->pre_op != BK_OP_NONE || st->post_op != BK_OP_NONE;
  if (!tp) return BK_OK;
  tp->n = n;
  tp->pre = st->pre_op;
  tp->post = st->post_op;
  tp->one_mz[0] = 1.0;
  tp->one_mz[1] = -0.0;
  static thread_local int offs[BK_MAX_TAPS][3];
  static thread_local int toff1[BK_MAX_TAPS];
  const int EJ = L.bj + 2 * GENERIC_R, EI = L.bi + 2 * GENERIC_R;
  for (int t = 0; t < n; ++t) {
    const int dk = st->offsets[t][0], dj = st->offsets[t][1], di = st->offsets[t][2];
    int idx = t;
    if (fam == FAM_STAR) idx = star_index(dk, dj, di);
    else if (fam == FAM_CUBE) idx = ((dk + r) * (2 * r + 1) + (dj + r)) * (2 * r + 1) + (di + r);
    tp->c[idx] = st->coeff[t];
    tp->cf[idx] = (float)st->coeff[t];
    tp->cl[idx] = (float)(st->coeff[t] - (double)tp->cf[idx]);
    toff1[idx] = (dk * EJ + dj) * EI + di;
    tp->toff[idx] = toff1[idx];
    offs[idx][0] = dk;
    offs[idx][1] = dj;
    offs[idx][2] = di;
  }
  plan->offs = offs;
  plan->toff1 = toff1;
  // mirror symmetry of a cube in every axis: c(dk,dj,di) == c(|dk|,|dj|,|di|) exactly
  plan->sym = plan->symij = false;
  tp->kj = 0;
  if (fam == FAM_CUBE) {
    const int w = 2 * r + 1;
    bool sym = true;
    for (int t = 0; t < w * w * w && sym; ++t) {
      const int dk = t / (w * w) - r, dj = (t / w) % w - r, di = t % w - r;
      const int m = ((abs(dk) + r) * w + (abs(dj) + r)) * w + (abs(di) + r);
      sym = tp->c[t] == tp->c[m];
    }
    if (sym) {
      plan->sym = true;
      for (int ak = 0; ak <= r; ++ak)
        for (int aj = 0; aj <= r; ++aj)
          for (int ai = 0; ai <= r; ++ai) {
            const int m = ((ak + r) * w + (aj + r)) * w + (ai + r), q = sym_index(ak, aj, ai, r);
            tp->c[q] = tp->c[m];
            tp->cf[q] = tp->cf[m];
            tp->cl[q] = tp->cl[m];
            tp->sp[(ak * (r + 1) + aj) * (r + 1) + ai] = make_float2(tp->cf[m], tp->cf[m]);
          }
      bool ij = true;
      for (int ak = 0; ak <= r; ++ak)
        for (int aj = 0; aj <= r; ++aj)
          for (int ai = 0; ai <= r; ++ai) ij = ij && tp->c[sym_index(ak, aj, ai, r)] == tp->c[sym_index(ak, ai, aj, r)];
      plan->symij = ij;
      bool kj = true;
      for (int ak = 0; ak <= r; ++ak)
        for (int aj = 0; aj <= r; ++aj)
          for (int ai = 0; ai <= r; ++ai) kj = kj && tp->c[sym_index(ak, aj, ai, r)] == tp->c[sym_index(aj, ak, ai, r)];
      tp->kj = kj;
    }
  }
  for (int t = 0; t < TAP_PAIRS; ++t) tp->cp[t] = make_float2(tp->cf[t], tp->cf[t]);
  return BK_OK;
}

// Field / stencil / accumulation checks and the kernel choice (everything but the brick lists).
static int plan_sweep(const bk_field *in, const bk_field *out, const bk_stencil *st, const bk_layout *lay, int acc,
                      SweepPlan *plan, Taps *tp, Layout *Lout) {
  Layout L;
  int s = check_layout(lay, &L);
  if (s) return s;
  if ((s = check_field(in, L, "in"))) return s;
  if ((s = check_field(out, L, "out"))) return s;
  if (in->dtype != out->dtype) return fail(BK_ERR_ARG, "in and out fields must have the same dtype");
  if ((s = check_disjoint(in, out, (size_t)L.size()))) return s;
  if ((s = analyze(st, L, plan, tp))) return s;
  if (plan->shape < 0) return fail(BK_ERR_UNSUPPORTED, "brick dims must be 8x8x8, 4x4x4, 16x8x8 or 8x8x32");
  plan->dtype = in->dtype;
  if (acc == BK_ACC_NATIVE) plan->acc = ACCM_NATIVE;
  else if (acc == BK_ACC_COMPENSATED && in->dtype != BK_F64) plan->acc = ACCM_COMP;
  else if (acc == BK_ACC_COMPENSATED) return fail(BK_ERR_UNSUPPORTED, "compensated accumulation is for FP32 / BF16 storage");
  else if (acc == BK_ACC_FLOATFLOAT && in->dtype == BK_F64) plan->acc = ACCM_FF;
  else if (acc == BK_ACC_FLOATFLOAT) return fail(BK_ERR_UNSUPPORTED, "float-float arithmetic is for FP64 storage");
  else return fail(BK_ERR_UNSUPPORTED, "accumulation mode not available");
  // the pipelined kernel copies whole 16-byte (or brick-row) vectors: it needs a row-major
  // layout and vector-aligned input addresses
  {
    const size_t es = dtype_size(in->dtype);
    const size_t vb = (size_t)L.bi * es < 16 ? (size_t)L.bi * es : 16;
    const size_t ve = vb / es;
    plan->v2 = plan->rm && !plan->ops && (reinterpret_cast<uintptr_t>(in->dat) % 16 == 0) && in->step % ve == 0 &&
               in->offset % ve == 0 && !getenv("BK_SWEEP_ONESHOT");
    // float-float cubes and the radius-4 star are bound by the FP32 pipes; the one-shot
    // kernel's single tile buffer keeps twice as many CTAs resident and wins there
    // (measured on GB300: cube125 18.6 vs 12.8, cube27 61 vs 46, star25 17 vs 15 GStencil/s)
    // (mirror-symmetric float-float cubes, on pair sums, stay on the pipelined kernel)
    if (plan->acc == ACCM_FF && ((plan->fam == FAM_CUBE && !(plan->sym && plan->shape == 0)) || plan->r >= 4) &&
        !getenv("BK_SWEEP_PIPELINED"))
      plan->v2 = false;
    // the column-pair kernels (cubes on 8x8x8 bricks, the FP32 / BF16 star row kernel) store
    // two adjacent outputs at once: every output brick must start on a two-element boundary
    const char *obase = reinterpret_cast<const char *>(out->dat) + out->offset * es;
    plan->out_pair = reinterpret_cast<uintptr_t>(obase) % (2 * es) == 0 && (out->step * es) % (2 * es) == 0;
    if (plan->fam == FAM_CUBE && plan->shape == 0 && !plan->out_pair) plan->v2 = false;
    // star stencils on 8x8x8 row-major bricks: the TMA-fed kernel, unless a kernel is forced
    plan->tma = tma_eligible(*plan, in) && !getenv("BK_SWEEP_ONESHOT") && !getenv("BK_SWEEP_PIPELINED");
    // mirror-symmetric cubes: the pipelined kernel streams class sums along i -- FP64 in native
    // arithmetic, FP32 / BF16 in native or compensated FP32 (BK_SWEEP_ISTREAM=0: one brick at a
    // time on column pairs)
    const char *ist = getenv("BK_SWEEP_ISTREAM");
    plan->istream = plan->v2 && plan->sym && plan->shape == 0 && !(ist && !strcmp(ist, "0")) &&
                    (in->dtype == BK_F64 ? plan->acc == ACCM_NATIVE
                                         : (plan->acc == ACCM_NATIVE || plan->acc == ACCM_COMP));
  }
  *Lout = L;
  return BK_OK;
}

static int prepare(const unsigned *adj, unsigned nbricks, const bk_field *in, const bk_field *out,
                   const unsigned *blist, const bk_stencil *st, const bk_layout *lay, int acc,
                   SweepPlan *plan, Taps *tp, SweepArgs *a) {
  Layout L;
  int s = plan_sweep(in, out, st, lay, acc, plan, tp, &L);
  if (s) return s;
  if (!adj || !blist || nbricks == 0) return fail(BK_ERR_ARG, "adjacency, brick list and nbricks are required");
  int *err = device_error_word();
  if (!err) return fail(BK_ERR_CUDA, "device error word unavailable");
  *a = SweepArgs{adj, nbricks, in->dat, in->step, in->offset, in->chunks,
                 out->dat, out->step, out->offset, out->chunks, blist, 0, err, L};
  // test hook: make one bounded wait of the TMA star kernel run out (5 ms limit), so that the
  // timeout path -- flag, stop, drain -- can be exercised; never set in normal use
  if (plan->tma && !tma_row(*plan) && getenv("BK_TEST_WITHHOLD_COPY")) {
    a->withhold = 1;
    a->wait_ns = 5000000ull;
  }
  return BK_OK;
}

static int dispatch(const SweepPlan &p, const SweepArgs &a, Taps &tp, cudaStream_t s) {
  if (p.tma) return sweep_dispatch_tma(p, a, tp, s);
  switch (p.dtype) {
    case BK_F64: return sweep_dispatch_f64(p, a, tp, s);
    case BK_F32: return sweep_dispatch_f32(p, a, tp, s);
    case BK_BF16: return sweep_dispatch_bf16(p, a, tp, s);
  }
  return fail(BK_ERR_ARG, "unknown dtype");
}

// Taps is ~5.5 KB; keep one per host thread instead of on the stack of every call.
static Taps &thread_taps() {
  static thread_local Taps t;
  return t;
}

// Stencil analysis and accumulation mode for kernels outside this file (the batch).
int plan_stencil(const bk_stencil *st, const Layout &L, int dtype, int acc, SweepPlan *plan, Taps *tp) {
  int s = analyze(st, L, plan, tp);
  if (s) return s;
  if (plan->shape < 0) return fail(BK_ERR_UNSUPPORTED, "brick dims must be 8x8x8, 4x4x4, 16x8x8 or 8x8x32");
  plan->dtype = dtype;
  plan->v2 = false;
  plan->tma = false;
  if (acc == BK_ACC_NATIVE) plan->acc = ACCM_NATIVE;
  else if (acc == BK_ACC_COMPENSATED && dtype != BK_F64) plan->acc = ACCM_COMP;
  else if (acc == BK_ACC_FLOATFLOAT && dtype == BK_F64) plan->acc = ACCM_FF;
  else return fail(BK_ERR_UNSUPPORTED, "accumulation mode not available for this storage type");
  return BK_OK;
}

}  // namespace bk

using namespace bk;

extern "C" {

int bk_stencil_check(const bk_stencil *st, const bk_layout *lay, int *radius, int *family) {
  Layout L;
  int s = check_layout(lay, &L);
  if (s) return s;
  SweepPlan p{};
  if ((s = analyze(st, L, &p, nullptr))) return s;
  int r = 0;
  for (int t = 0; t < st->npoints; ++t)
    for (int d = 0; d < 3; ++d) r = abs(st->offsets[t][d]) > r ? abs(st->offsets[t][d]) : r;
  if (radius) *radius = r;
  if (family) *family = p.fam;
  return BK_OK;
}

int bk_sweep_kernel(const bk_field *in, const bk_field *out, const bk_stencil *st, const bk_layout *lay, int acc,
                    const char **name) {
  if (!name) return fail(BK_ERR_ARG, "name is NULL");
  SweepPlan plan{};
  Layout L;
  static thread_local Taps tp;  // the coefficient analysis decides the symmetric-cube routes
  int s = plan_sweep(in, out, st, lay, acc, &plan, &tp, &L);
  if (s) return s;
  *name = plan.tma ? (tma_row(plan) ? "sweep_star_row_kernel" : "sweep_star_tma_kernel")
          : plan.v2 ? "sweep2_kernel" : "sweep_kernel";
  return BK_OK;
}

int bk_sweep(const unsigned *adj, unsigned nbricks, const bk_field *in, const bk_field *out,
             const unsigned *blist, unsigned nlist, const bk_stencil *st, const bk_layout *lay,
             int acc, void *stream) {
  if (nlist == 0) return BK_OK;
  SweepPlan plan{};
  SweepArgs a{};
  Taps &tp = thread_taps();
  int s = prepare(adj, nbricks, in, out, blist, st, lay, acc, &plan, &tp, &a);
  if (s) return s;
  a.nlist = nlist;
  return dispatch(plan, a, tp, as_stream(stream));
}

int bk_steps(const unsigned *adj, unsigned nbricks, const bk_field *a, const bk_field *b,
             const unsigned *blist, unsigned nlist, const unsigned *pairs, unsigned npairs,
             const bk_stencil *st, const bk_layout *lay, int acc, int steps, int fill_every,
             int use_graph, void *stream) {
  if (steps < 0 || fill_every < 0) return fail(BK_ERR_ARG, "steps and fill_every must be >= 0");
  if (steps == 0 || nlist == 0) return BK_OK;
  if (fill_every && npairs && !pairs) return fail(BK_ERR_ARG, "pairs is NULL");
  SweepPlan plan{};
  SweepArgs fwd{}, bwd{};
  Taps &tp = thread_taps();
  int s = prepare(adj, nbricks, a, b, blist, st, lay, acc, &plan, &tp, &fwd);
  if (s) return s;
  if ((s = prepare(adj, nbricks, b, a, blist, st, lay, acc, &plan, &tp, &bwd))) return s;
  fwd.nlist = bwd.nlist = nlist;
  Layout L = fwd.L;

  cudaStream_t user = as_stream(stream);
  cudaStream_t cap = user;
  cudaGraph_t graph = nullptr;
  if (use_graph) {
    static thread_local cudaStream_t priv = nullptr;
    static thread_local int priv_dev = -1;
    int dev = 0;
    BK_CUDA(cudaGetDevice(&dev));
    if (!priv || priv_dev != dev) {
      BK_CUDA(cudaStreamCreateWithFlags(&priv, cudaStreamNonBlocking));
      priv_dev = dev;
    }
    cap = priv;
    BK_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
  }
  for (int t = 0; t < steps && s == BK_OK; ++t) {
    const bk_field *cur = (t % 2 == 0) ? a : b;
    if (fill_every && npairs && t % fill_every == 0) s = ghost_fill(pairs, npairs, cur, L, cap);
    if (s == BK_OK) s = dispatch(plan, (t % 2 == 0) ? fwd : bwd, tp, cap);
  }
  if (use_graph) {
    cudaError_t e = cudaStreamEndCapture(cap, &graph);
    if (s != BK_OK) {
      if (graph) cudaGraphDestroy(graph);
      return s;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    e = cudaGraphLaunch(exec, user);
    // the executable graph is released only after its launch has finished
    cudaError_t e2 = (e == cudaSuccess) ? cudaStreamSynchronize(user) : cudaSuccess;
    cudaGraphExecDestroy(exec);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamSynchronize(graph)");
  }
  return s;
}

}  // extern "C"
