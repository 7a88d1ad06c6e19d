// Serving form: a continuous-batching stencil server.
//
// Clients submit jobs (a periodic domain, a stencil, a step count, a storage type, host
// input and output arrays) from any thread.  One scheduler thread owns the GPU work:
//   admission  FIFO, against an HBM byte budget and a cap on active jobs; a job's storage,
//              adjacency and staging array come from the stream-ordered allocator on an
//              admission stream, its input is copied in and scattered into bricks there,
//              and the tick stream waits on that before the job's first step;
//   ticks      every active job advances one step per tick: one persistent sweep launch per
//              (storage type, stencil) group over a work list of all active jobs' bricks.
//              Jobs join and leave between ticks, so work of jobs that arrived at different
//              times overlaps;
//   retirement after its last step a job's newest field is gathered into an array and
//              copied to the client's output on a retire stream; a host callback on that
//              stream stamps the completion time, releases its budget and wakes waiters.
// Domains use the init_grid layout (brick index = grid position, one ghost brick per side);
// the periodic boundary goes through the adjacency, which points every interior brick's
// neighbours across the boundary at the interior bricks a periodic ghost fill would copy,
// so no fill runs between steps and the ghost bricks stay unused.  No device-side wait
// exists: the only waits are host waits with timeouts.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "batch_common.cuh"

namespace bk {

using Clock = std::chrono::steady_clock;

// Periodic adjacency of a (gk, gj, gi) brick grid (brick = position, one ghost brick per side):
// the neighbour (k + dk, j + dj, i + di) of every brick, wrapped into the interior
// 1 .. g - 2 of each axis.  For an interior brick this is the init_grid neighbour
// (bricksetup.h:44-47) wherever that is interior, and the source of the periodic ghost fill
// wherever it is a ghost brick.
__global__ void grid_adj_kernel(unsigned *adj, int gk, int gj, int gi) {
  const long long size = (long long)gk * gj * gi;
  const int nk = gk - 2, nj = gj - 2, ni = gi - 2;
  for (long long p = blockIdx.x * 256ll + threadIdx.x; p < size * 27; p += (long long)gridDim.x * 256) {
    const long long b = p / 27;
    const int s = (int)(p - b * 27);
    const int dk = s / 9 - 1, dj = (s / 3) % 3 - 1, di = s % 3 - 1;
    const int k = (int)(b / ((long long)gj * gi)), j = (int)((b / gi) % gj), i = (int)(b % gi);
    const int wk = 1 + ((k + dk - 1) % nk + nk) % nk, wj = 1 + ((j + dj - 1) % nj + nj) % nj,
              wi = 1 + ((i + di - 1) % ni + ni) % ni;
    adj[p] = (unsigned)(((long long)wk * gj + wj) * gi + wi);
  }
}

__global__ void identity_kernel(unsigned *g, long long n) {
  for (long long p = blockIdx.x * 256ll + threadIdx.x; p < n; p += (long long)gridDim.x * 256) g[p] = (unsigned)p;
}

struct JobRow {
  unsigned dom;
  int gk, gj, gi;
  unsigned long long work_off;
};

// interior bricks of every job, in position order
__global__ void expand_work_kernel(const JobRow *rows, unsigned nrows, uint2 *work) {
  const JobRow r = rows[blockIdx.x];
  const int nk = r.gk - 2, nj = r.gj - 2, ni = r.gi - 2;
  const long long n = (long long)nk * nj * ni;
  for (long long l = threadIdx.x; l < n; l += blockDim.x) {
    const int i = (int)(l % ni), j = (int)((l / ni) % nj), k = (int)(l / ((long long)ni * nj));
    const unsigned p = (unsigned)(((long long)(k + 1) * r.gj + (j + 1)) * r.gi + (i + 1));
    work[r.work_off + l] = make_uint2(r.dom, p);
  }
}

enum JobState { JOB_PENDING = 0, JOB_ACTIVE = 1, JOB_RETIRING = 2, JOB_DONE = 3, JOB_FAILED = 4, JOB_CANCELLED = 5 };

struct Job {
  unsigned long long id = 0;
  long n[3] = {0, 0, 0};
  int g[3] = {0, 0, 0};
  long long nbricks = 0;
  int dtype = BK_F32, acc = BK_ACC_NATIVE;
  int steps = 0, left = 0;
  int group = -1;
  bk_stencil stencil{};
  const void *input = nullptr;
  void *output = nullptr;
  size_t bytes = 0;
  // device
  void *storage = nullptr;
  unsigned *adj = nullptr, *grid = nullptr;
  void *staging = nullptr;
  cudaEvent_t ready = nullptr;
  int flip = 0;  // 1: field B is f0 (admitted at odd parity)
  // timing
  Clock::time_point t_submit, t_admit, t_done;
  std::atomic<int> state{JOB_PENDING};
  std::string error;
};

struct Group {
  int dtype, acc;
  bk_stencil st;
  BatchStencil bs;
};

}  // namespace bk

using namespace bk;

struct bk_server {
  int device = 0;
  Layout L{};
  size_t budget = 0;
  int max_active = 0;
  std::atomic<size_t> used{0};
  size_t peak = 0;
  cudaStream_t s_tick = nullptr, s_admit = nullptr, s_retire = nullptr;
  int *err = nullptr;
  std::thread th;
  std::mutex mu;  // pending, jobs, stats
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Job>> pending;
  std::map<unsigned long long, std::shared_ptr<Job>> jobs;
  std::vector<std::shared_ptr<Job>> active;
  std::vector<Group> groups;
  unsigned long long next_id = 1;
  std::atomic<bool> stop{false};
  // the current tick program
  bool dirty = true;
  BatchDomain *d_doms = nullptr;
  uint2 *d_work = nullptr;
  JobRow *d_rows = nullptr;
  std::vector<std::pair<int, std::pair<unsigned, unsigned>>> work_seg;  // group -> (offset, count)
  unsigned ndom = 0;
  int parity = 0;
  std::deque<cudaEvent_t> inflight;
  // pinned staging for table uploads
  std::vector<unsigned char *> ring;
  std::vector<cudaEvent_t> ring_ev;
  std::vector<size_t> ring_cap;
  unsigned ring_next = 0;
  // stats
  std::vector<double> lat;
  double work_done = 0.0;  // stencil point-steps of completed jobs
  Clock::time_point t_first, t_last;
  bool any = false;
  unsigned long long submitted = 0, admitted = 0, completed = 0, rejected = 0, ticks = 0;
  std::string fatal;
};

namespace bk {

static size_t job_bytes(const Layout &L, const Job &j) {
  const size_t es = dtype_size(j.dtype);
  const size_t bs = (size_t)L.size();
  const size_t interior = (size_t)(j.g[0] - 2) * (j.g[1] - 2) * (j.g[2] - 2);
  return (size_t)j.nbricks * (2 * bs * es + 27 * 4 + 4) + (size_t)j.n[0] * j.n[1] * j.n[2] * es +
         interior * sizeof(uint2) + sizeof(BatchDomain) + 4096;
}

static int group_of(bk_server *S, const Job &j) {
  for (size_t q = 0; q < S->groups.size(); ++q) {
    const Group &g = S->groups[q];
    if (g.dtype == j.dtype && g.acc == j.acc && g.st.npoints == j.stencil.npoints &&
        !memcmp(g.st.offsets, j.stencil.offsets, sizeof(int) * 3 * j.stencil.npoints) &&
        !memcmp(g.st.coeff, j.stencil.coeff, sizeof(double) * j.stencil.npoints))
      return (int)q;
  }
  Group g;
  g.dtype = j.dtype;
  g.acc = j.acc;
  g.st = j.stencil;
  if (plan_stencil(&g.st, S->L, j.dtype, j.acc, &g.bs.plan, &g.bs.taps) != BK_OK) return -1;
  S->groups.push_back(g);
  return (int)S->groups.size() - 1;
}

static void CUDART_CB on_job_done(void *arg) {
  // runs on a driver thread: no CUDA calls here
  auto *pr = reinterpret_cast<std::pair<bk_server *, std::shared_ptr<Job>> *>(arg);
  bk_server *S = pr->first;
  std::shared_ptr<Job> j = pr->second;
  delete pr;
  j->t_done = Clock::now();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    const double l = std::chrono::duration<double>(j->t_done - j->t_submit).count();
    S->lat.push_back(l);
    S->work_done += (double)j->n[0] * j->n[1] * j->n[2] * j->steps;
    if (!S->any || j->t_done > S->t_last) S->t_last = j->t_done;
    S->any = true;
    S->completed++;
    S->used -= j->bytes;
    j->state = JOB_DONE;
  }
  S->cv_done.notify_all();
  S->cv_work.notify_all();
}

static int admit(bk_server *S, const std::shared_ptr<Job> &j) {
  cudaStream_t s = S->s_admit;
  const size_t es = dtype_size(j->dtype);
  const size_t field = (size_t)j->nbricks * 2 * S->L.size() * es;
  const size_t arr = (size_t)j->n[0] * j->n[1] * j->n[2] * es;
  BK_CUDA(cudaMallocAsync(&j->storage, field, s));
  BK_CUDA(cudaMallocAsync((void **)&j->adj, (size_t)j->nbricks * 27 * 4, s));
  BK_CUDA(cudaMallocAsync((void **)&j->grid, (size_t)j->nbricks * 4, s));
  BK_CUDA(cudaMallocAsync(&j->staging, arr, s));
  BK_CUDA(cudaMemcpyAsync(j->staging, j->input, arr, cudaMemcpyHostToDevice, s));
  grid_adj_kernel<<<(unsigned)std::min<long long>((j->nbricks * 27 + 255) / 256, 4096), 256, 0, s>>>(j->adj, j->g[0], j->g[1], j->g[2]);
  identity_kernel<<<(unsigned)std::min<long long>((j->nbricks + 255) / 256, 4096), 256, 0, s>>>(j->grid, j->nbricks);
  BK_CUDA(cudaGetLastError());
  // field A = offset 0 gets the input; field B = offset BRICKSIZE
  bk_field fa{j->storage, (long)j->nbricks, (size_t)2 * S->L.size(), 0, j->dtype};
  bk_layout lay{{S->L.bk, S->L.bj, S->L.bi}, {S->L.fk, S->L.fj, S->L.fi}};
  const long gh[3] = {S->L.bk, S->L.bj, S->L.bi};
  const long pad[3] = {-gh[0], -gh[1], -gh[2]};
  int st = bk_copy_to_bricks(j->staging, j->n, pad, gh, j->grid, &fa, &lay, s);
  if (st) return st;
  BK_CUDA(cudaFreeAsync(j->staging, s));
  j->staging = nullptr;
  BK_CUDA(cudaEventCreateWithFlags(&j->ready, cudaEventDisableTiming));
  BK_CUDA(cudaEventRecord(j->ready, s));
  j->flip = S->parity;
  j->t_admit = Clock::now();
  j->left = j->steps;
  j->state = JOB_ACTIVE;
  return BK_OK;
}

static int retire(bk_server *S, const std::shared_ptr<Job> &j, cudaEvent_t after_tick) {
  cudaStream_t s = S->s_retire;
  BK_CUDA(cudaStreamWaitEvent(s, after_tick, 0));
  const size_t es = dtype_size(j->dtype);
  const size_t arr = (size_t)j->n[0] * j->n[1] * j->n[2] * es;
  BK_CUDA(cudaMallocAsync(&j->staging, arr, s));
  // the newest values are in f_parity (parity after the last tick), f0 = A unless flipped
  const int newest_f = S->parity;                   // 0: f0, 1: f1
  const int field_b = (newest_f ^ j->flip) ? 1 : 0;  // which of A (0) / B (1)
  bk_field f{j->storage, (long)j->nbricks, (size_t)2 * S->L.size(), (size_t)(field_b ? S->L.size() : 0), j->dtype};
  bk_layout lay{{S->L.bk, S->L.bj, S->L.bi}, {S->L.fk, S->L.fj, S->L.fi}};
  const long gh[3] = {S->L.bk, S->L.bj, S->L.bi};
  const long pad[3] = {-gh[0], -gh[1], -gh[2]};
  int st = bk_copy_from_bricks(j->staging, j->n, pad, gh, j->grid, &f, &lay, s);
  if (st) return st;
  BK_CUDA(cudaMemcpyAsync(j->output, j->staging, arr, cudaMemcpyDeviceToHost, s));
  BK_CUDA(cudaFreeAsync(j->staging, s));
  BK_CUDA(cudaFreeAsync(j->storage, s));
  BK_CUDA(cudaFreeAsync(j->adj, s));
  BK_CUDA(cudaFreeAsync(j->grid, s));
  j->staging = j->storage = nullptr;
  j->adj = j->grid = nullptr;
  j->state = JOB_RETIRING;
  auto *arg = new std::pair<bk_server *, std::shared_ptr<Job>>(S, j);
  cudaError_t e = cudaLaunchHostFunc(s, on_job_done, arg);
  if (e != cudaSuccess) {
    delete arg;
    return cuda_fail(e, "cudaLaunchHostFunc");
  }
  return BK_OK;
}

// pinned staging slot of at least `bytes`, free of pending copies
static unsigned char *ring_slot(bk_server *S, size_t bytes, int *slot) {
  const unsigned K = (unsigned)S->ring.size();
  const unsigned r = S->ring_next++ % K;
  cudaEventSynchronize(S->ring_ev[r]);
  if (S->ring_cap[r] < bytes) {
    if (S->ring[r]) cudaFreeHost(S->ring[r]);
    S->ring[r] = nullptr;
    size_t cap = std::max(bytes, (size_t)1 << 20);
    if (cudaMallocHost((void **)&S->ring[r], cap) != cudaSuccess) {
      S->ring_cap[r] = 0;
      return nullptr;
    }
    S->ring_cap[r] = cap;
  }
  *slot = (int)r;
  return S->ring[r];
}

// rebuild the domain table and work list of the active jobs
static int rebuild(bk_server *S) {
  cudaStream_t s = S->s_tick;
  std::vector<std::shared_ptr<Job>> order = S->active;
  std::stable_sort(order.begin(), order.end(), [](const std::shared_ptr<Job> &a, const std::shared_ptr<Job> &b) {
    return a->group < b->group;
  });
  const unsigned n = (unsigned)order.size();
  std::vector<BatchDomain> doms(n);
  std::vector<JobRow> rows(n);
  S->work_seg.clear();
  unsigned long long woff = 0;
  for (unsigned d = 0; d < n; ++d) {
    const Job &j = *order[d];
    const size_t es = dtype_size(j.dtype);
    unsigned char *A = reinterpret_cast<unsigned char *>(j.storage);
    unsigned char *Bf = A + (size_t)S->L.size() * es;
    doms[d] = BatchDomain{j.adj, (unsigned)j.nbricks, (unsigned)j.group, j.flip ? Bf : A, j.flip ? A : Bf,
                          (unsigned long long)2 * S->L.size() * es, j.nbricks};
    const unsigned long long nint = (unsigned long long)(j.g[0] - 2) * (j.g[1] - 2) * (j.g[2] - 2);
    rows[d] = JobRow{d, j.g[0], j.g[1], j.g[2], woff};
    if (S->work_seg.empty() || S->work_seg.back().first != j.group)
      S->work_seg.push_back({j.group, {(unsigned)woff, 0}});
    S->work_seg.back().second.second += (unsigned)nint;
    woff += nint;
  }
  // new device buffers (stream ordered); the previous ones are freed after the ticks using them
  if (S->d_doms) BK_CUDA(cudaFreeAsync(S->d_doms, s));
  if (S->d_work) BK_CUDA(cudaFreeAsync(S->d_work, s));
  if (S->d_rows) BK_CUDA(cudaFreeAsync(S->d_rows, s));
  S->d_doms = nullptr;
  S->d_work = nullptr;
  S->d_rows = nullptr;
  S->ndom = n;
  if (!n) return BK_OK;
  BK_CUDA(cudaMallocAsync((void **)&S->d_doms, sizeof(BatchDomain) * n, s));
  BK_CUDA(cudaMallocAsync((void **)&S->d_rows, sizeof(JobRow) * n, s));
  BK_CUDA(cudaMallocAsync((void **)&S->d_work, sizeof(uint2) * std::max<unsigned long long>(woff, 1), s));
  const size_t bytes = sizeof(BatchDomain) * n + sizeof(JobRow) * n;
  int slot = 0;
  unsigned char *h = ring_slot(S, bytes, &slot);
  if (!h) return fail(BK_ERR_NOMEM, "server: pinned staging");
  memcpy(h, doms.data(), sizeof(BatchDomain) * n);
  memcpy(h + sizeof(BatchDomain) * n, rows.data(), sizeof(JobRow) * n);
  BK_CUDA(cudaMemcpyAsync(S->d_doms, h, sizeof(BatchDomain) * n, cudaMemcpyHostToDevice, s));
  BK_CUDA(cudaMemcpyAsync(S->d_rows, h + sizeof(BatchDomain) * n, sizeof(JobRow) * n, cudaMemcpyHostToDevice, s));
  BK_CUDA(cudaEventRecord(S->ring_ev[slot], s));
  expand_work_kernel<<<n, 256, 0, s>>>(S->d_rows, n, S->d_work);
  BK_CUDA(cudaGetLastError());
  S->active = order;
  return BK_OK;
}

static int tick(bk_server *S) {
  cudaStream_t s = S->s_tick;
  for (auto &ws : S->work_seg) {
    const Group &g = S->groups[ws.first];
    // job storages come from cudaMallocAsync and hold two whole-brick fields: aligned
    int st = batch_launch_sweep(g.bs, g.dtype, S->d_doms, S->ndom, S->d_work + ws.second.first, ws.second.second,
                                S->parity, S->L, S->err, 0, true, s);
    if (st) return st;
  }
  S->parity ^= 1;
  S->ticks++;
  return BK_OK;
}

static void serve_loop(bk_server *S) {
  cudaSetDevice(S->device);
  const int MAXQ = 3;
  while (!S->stop) {
    // admission
    std::vector<std::shared_ptr<Job>> admitted;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      if (S->pending.empty() && S->active.empty())
        S->cv_work.wait_for(lk, std::chrono::milliseconds(2), [&] { return S->stop || !S->pending.empty(); });
      while (!S->pending.empty() && (int)S->active.size() + (int)admitted.size() < S->max_active) {
        std::shared_ptr<Job> j = S->pending.front();
        if (S->used + j->bytes > S->budget) break;  // FIFO: wait until memory frees up
        S->pending.pop_front();
        S->used += j->bytes;
        S->peak = std::max(S->peak, (size_t)S->used);
        admitted.push_back(j);
      }
    }
    if (S->stop) break;
    for (auto &j : admitted) {
      int g = group_of(S, *j);
      int st = g < 0 ? BK_ERR_UNSUPPORTED : BK_OK;
      j->group = g;
      if (st == BK_OK) st = admit(S, j);
      if (st != BK_OK) {
        std::lock_guard<std::mutex> lk(S->mu);
        j->error = bk_last_error();
        j->state = JOB_FAILED;
        S->used -= j->bytes;
        S->cv_done.notify_all();
        continue;
      }
      cudaStreamWaitEvent(S->s_tick, j->ready, 0);  // first step after the job's data is in
      S->active.push_back(j);
      S->admitted++;
      S->dirty = true;
    }
    if (S->active.empty()) continue;
    if (S->dirty) {
      int st = rebuild(S);
      if (st != BK_OK) {
        S->fatal = bk_last_error();
        break;
      }
      S->dirty = false;
    }
    int st = tick(S);
    if (st != BK_OK) {
      S->fatal = bk_last_error();
      break;
    }
    cudaEvent_t ev = nullptr;
    cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    cudaEventRecord(ev, S->s_tick);
    // retire finished jobs
    std::vector<std::shared_ptr<Job>> still;
    for (auto &j : S->active) {
      if (--j->left > 0) {
        still.push_back(j);
        continue;
      }
      if (retire(S, j, ev) != BK_OK) {
        std::lock_guard<std::mutex> lk(S->mu);
        j->error = bk_last_error();
        j->state = JOB_FAILED;
        S->cv_done.notify_all();
      }
      S->dirty = true;
    }
    S->active.swap(still);
    S->inflight.push_back(ev);
    while ((int)S->inflight.size() > MAXQ) {  // bounded run-ahead of the host
      cudaEventSynchronize(S->inflight.front());
      cudaEventDestroy(S->inflight.front());
      S->inflight.pop_front();
    }
  }
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (!S->stop && S->fatal.empty()) S->fatal = "scheduler stopped";
  }
  S->cv_done.notify_all();
}

}  // namespace bk

extern "C" {

int bk_server_create(bk_server **out, size_t hbm_budget, const bk_layout *lay, int max_active) {
  if (!out || hbm_budget == 0 || max_active < 1) return fail(BK_ERR_ARG, "bk_server_create: bad arguments");
  *out = nullptr;
  Layout L;
  int s = check_layout(lay, &L);
  if (s) return s;
  if (!L.row_major()) return fail(BK_ERR_UNSUPPORTED, "bk_server_create: the server uses row-major brick layouts");
  bk_server *S = new bk_server();
  S->L = L;
  S->budget = hbm_budget;
  S->max_active = max_active;
  cudaError_t e = cudaGetDevice(&S->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S->s_tick, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S->s_admit, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S->s_retire, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    // keep freed blocks in the stream-ordered pool instead of returning them to the driver
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, S->device) == cudaSuccess) {
      unsigned long long thr = ~0ull;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
  }
  const int K = 8;
  S->ring.assign(K, nullptr);
  S->ring_cap.assign(K, 0);
  S->ring_ev.assign(K, nullptr);
  for (int r = 0; r < K && e == cudaSuccess; ++r) e = cudaEventCreateWithFlags(&S->ring_ev[r], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    delete S;
    return cuda_fail(e, "bk_server_create");
  }
  S->err = device_error_word();
  if (!S->err) {
    delete S;
    return fail(BK_ERR_CUDA, "device error word unavailable");
  }
  S->th = std::thread(serve_loop, S);
  *out = S;
  return BK_OK;
}

int bk_server_submit(bk_server *S, const bk_job_desc *d, unsigned long long *id) {
  if (!S || !d || !id || !d->stencil || !d->input || !d->output || d->steps < 1 ||
      (d->dtype != BK_F64 && d->dtype != BK_F32))
    return fail(BK_ERR_ARG, "bk_server_submit: bad arguments");
  auto j = std::make_shared<Job>();
  const int bd[3] = {S->L.bk, S->L.bj, S->L.bi};
  for (int a = 0; a < 3; ++a) {
    if (d->n[a] <= 0 || d->n[a] % bd[a]) return fail(BK_ERR_ARG, "bk_server_submit: domain edges must be multiples of the brick dims");
    j->n[a] = d->n[a];
    j->g[a] = (int)(d->n[a] / bd[a]) + 2;
  }
  j->nbricks = (long long)j->g[0] * j->g[1] * j->g[2];
  j->dtype = d->dtype;
  j->acc = d->acc;
  j->steps = d->steps;
  j->stencil = *d->stencil;
  j->input = d->input;
  j->output = d->output;
  j->bytes = job_bytes(S->L, *j);
  // validate the stencil for this layout now, so a bad job fails at submission
  SweepPlan p{};
  std::unique_ptr<Taps> tp(new Taps());
  int st = plan_stencil(&j->stencil, S->L, j->dtype, j->acc, &p, tp.get());
  if (st) return st;
  std::lock_guard<std::mutex> lk(S->mu);
  if (!S->fatal.empty()) return fail(BK_ERR_STATE, "server stopped: " + S->fatal);
  if (j->bytes > S->budget) {
    S->rejected++;
    return fail(BK_ERR_BUDGET, "bk_server_submit: job needs " + std::to_string(j->bytes) + " bytes, budget is " +
                                   std::to_string(S->budget));
  }
  j->id = S->next_id++;
  j->t_submit = Clock::now();
  if (!S->submitted) S->t_first = j->t_submit;
  S->submitted++;
  S->jobs[j->id] = j;
  S->pending.push_back(j);
  *id = j->id;
  S->cv_work.notify_all();
  return BK_OK;
}

int bk_server_wait(bk_server *S, unsigned long long id, double timeout_s, double *latency_s) {
  if (!S) return fail(BK_ERR_ARG, "bk_server_wait: server is NULL");
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->jobs.find(id);
  if (it == S->jobs.end()) return fail(BK_ERR_ARG, "bk_server_wait: unknown job id");
  std::shared_ptr<Job> j = it->second;
  const bool ok = S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] {
    const int st = j->state.load();
    return st == JOB_DONE || st == JOB_FAILED || st == JOB_CANCELLED || !S->fatal.empty();
  });
  if (!ok) return fail(BK_ERR_TIMEOUT, "bk_server_wait: job " + std::to_string(id) + " not done in time");
  if (j->state == JOB_FAILED) return fail(BK_ERR_CUDA, "job failed: " + j->error);
  if (j->state != JOB_DONE) return fail(BK_ERR_STATE, "job did not complete: " + S->fatal);
  if (latency_s) *latency_s = std::chrono::duration<double>(j->t_done - j->t_submit).count();
  return BK_OK;
}

int bk_server_drain(bk_server *S, double timeout_s) {
  if (!S) return fail(BK_ERR_ARG, "bk_server_drain: server is NULL");
  std::unique_lock<std::mutex> lk(S->mu);
  const bool ok = S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] {
    return S->completed + S->rejected >= S->submitted || !S->fatal.empty();
  });
  if (!S->fatal.empty()) return fail(BK_ERR_STATE, "server stopped: " + S->fatal);
  if (!ok) return fail(BK_ERR_TIMEOUT, "bk_server_drain: jobs still running");
  return BK_OK;
}

int bk_server_stats(bk_server *S, bk_server_report *o) {
  if (!S || !o) return fail(BK_ERR_ARG, "bk_server_stats: bad arguments");
  std::lock_guard<std::mutex> lk(S->mu);
  memset(o, 0, sizeof(*o));
  o->submitted = S->submitted;
  o->admitted = S->admitted;
  o->completed = S->completed;
  o->rejected = S->rejected;
  o->ticks = S->ticks;
  o->hbm_budget = S->budget;
  o->hbm_peak = S->peak;
  std::vector<double> l = S->lat;
  if (!l.empty()) {
    std::sort(l.begin(), l.end());
    auto q = [&](double f) { return l[std::min(l.size() - 1, (size_t)(f * (l.size() - 1) + 0.5))]; };
    o->p50_s = q(0.50);
    o->p99_s = q(0.99);
    o->max_s = l.back();
    double sum = 0;
    for (double x : l) sum += x;
    o->mean_s = sum / l.size();
  }
  if (S->any) {
    const double span = std::chrono::duration<double>(S->t_last - S->t_first).count();
    o->span_s = span;
    o->gstencil_s = span > 0 ? S->work_done / span / 1e9 : 0.0;
  }
  return BK_OK;
}

int bk_server_destroy(bk_server *S) {
  if (!S) return BK_OK;
  S->stop = true;
  S->cv_work.notify_all();
  if (S->th.joinable()) S->th.join();
  cudaDeviceSynchronize();
  for (auto &kv : S->jobs) {
    Job &j = *kv.second;
    if (j.storage) cudaFree(j.storage);
    if (j.adj) cudaFree(j.adj);
    if (j.grid) cudaFree(j.grid);
    if (j.ready) cudaEventDestroy(j.ready);
  }
  for (auto ev : S->inflight) cudaEventDestroy(ev);
  if (S->d_doms) cudaFree(S->d_doms);
  if (S->d_work) cudaFree(S->d_work);
  if (S->d_rows) cudaFree(S->d_rows);
  for (size_t r = 0; r < S->ring.size(); ++r) {
    if (S->ring[r]) cudaFreeHost(S->ring[r]);
    if (S->ring_ev[r]) cudaEventDestroy(S->ring_ev[r]);
  }
  cudaStreamDestroy(S->s_tick);
  cudaStreamDestroy(S->s_admit);
  cudaStreamDestroy(S->s_retire);
  delete S;
  return BK_OK;
}

}  // extern "C"
