// Runtime part of the C ABI: status strings, device memory, BrickInfo / BrickStorage
// moves, the device error word, and the host-side periodic plan.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "bk_common.cuh"

namespace bk {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int status, const std::string &msg) {
  g_last_error = msg;
  return status;
}

int cuda_fail(cudaError_t e, const char *what) {
  char buf[512];
  snprintf(buf, sizeof buf, "%s: %s (%d)", what, cudaGetErrorString(e), (int)e);
  g_last_error = buf;
  return e == cudaErrorMemoryAllocation ? BK_ERR_NOMEM : BK_ERR_CUDA;
}

// One device word per device for kernel-side error flags, allocated on first use.
static std::mutex g_err_mu;
static std::vector<int *> g_err_words;

int *device_error_word() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(g_err_mu);
  if ((int)g_err_words.size() <= dev) g_err_words.resize(dev + 1, nullptr);
  if (!g_err_words[dev]) {
    int *p = nullptr;
    if (cudaMalloc(&p, sizeof(int)) != cudaSuccess) return nullptr;
    if (cudaMemset(p, 0, sizeof(int)) != cudaSuccess) return nullptr;
    g_err_words[dev] = p;
  }
  return g_err_words[dev];
}

int check_layout(const bk_layout *lay, Layout *out) {
  if (!lay) return fail(BK_ERR_ARG, "layout is NULL");
  for (int d = 0; d < 3; ++d) {
    if (lay->bdim[d] <= 0 || lay->fold[d] <= 0 || lay->bdim[d] % lay->fold[d] != 0)
      return fail(BK_ERR_ARG, "brick dims must be positive multiples of the fold");
  }
  long sz = (long)lay->bdim[0] * lay->bdim[1] * lay->bdim[2];
  if (sz > 8192) return fail(BK_ERR_ARG, "brick larger than 8192 elements");
  *out = Layout{lay->bdim[0], lay->bdim[1], lay->bdim[2], lay->fold[0], lay->fold[1], lay->fold[2]};
  return BK_OK;
}

int check_field(const bk_field *f, const Layout &L, const char *name) {
  if (!f) return fail(BK_ERR_ARG, std::string(name) + " field is NULL");
  if (!f->dat) return fail(BK_ERR_ARG, std::string(name) + " field has no data pointer");
  if (!dtype_ok(f->dtype)) return fail(BK_ERR_ARG, std::string(name) + " field has an unknown dtype");
  if (f->chunks <= 0) return fail(BK_ERR_ARG, std::string(name) + " field has no chunks");
  if (f->offset + (size_t)L.size() > f->step)
    return fail(BK_ERR_ARG, std::string(name) + " field: offset + brick size exceeds step");
  return BK_OK;
}

// A sweep reads `in` and writes `out`, so no output element may be an input element.  Fields
// in separate storages are disjoint; fields of one storage (same base and step, the
// interleaved bIn / bOut of stencils/3axis.cpp:26-28) are disjoint when their offsets are a
// brick apart.  Anything else whose byte ranges meet (one storage seen with two steps, or two
// storages that overlap in memory) is rejected.
int check_disjoint(const bk_field *in, const bk_field *out, size_t brick_elems) {
  const size_t es_in = dtype_size(in->dtype), es_out = dtype_size(out->dtype);
  if (in->dat == out->dat && in->step == out->step && es_in == es_out) {
    const size_t lo = in->offset < out->offset ? in->offset : out->offset;
    const size_t hi = in->offset < out->offset ? out->offset : in->offset;
    if (hi - lo < brick_elems) return fail(BK_ERR_ARG, "in and out fields overlap");
    return BK_OK;
  }
  const uintptr_t a0 = reinterpret_cast<uintptr_t>(in->dat), b0 = reinterpret_cast<uintptr_t>(out->dat);
  const uintptr_t a1 = a0 + (uintptr_t)in->chunks * in->step * es_in;
  const uintptr_t b1 = b0 + (uintptr_t)out->chunks * out->step * es_out;
  if (a0 < b1 && b0 < a1)
    return fail(BK_ERR_ARG, "in and out fields share storage bytes with a different base or step");
  return BK_OK;
}

}  // namespace bk

using namespace bk;

extern "C" {

int bk_abi_version(void) { return BK_ABI_VERSION; }

const char *bk_last_error(void) { return g_last_error.c_str(); }

int bk_set_device(int device) {
  BK_CUDA(cudaSetDevice(device));
  return BK_OK;
}

int bk_device_synchronize(void) {
  BK_CUDA(cudaDeviceSynchronize());
  return BK_OK;
}

int bk_stream_synchronize(void *stream) {
  BK_CUDA(cudaStreamSynchronize(as_stream(stream)));
  return BK_OK;
}

int bk_device_malloc(void **dptr, size_t bytes) {
  if (!dptr) return fail(BK_ERR_ARG, "dptr is NULL");
  *dptr = nullptr;
  if (bytes == 0) return BK_OK;
  BK_CUDA(cudaMalloc(dptr, bytes));
  return BK_OK;
}

int bk_device_free(void *dptr) {
  if (dptr) BK_CUDA(cudaFree(dptr));
  return BK_OK;
}

int bk_host_malloc(void **hptr, size_t bytes) {
  if (!hptr) return fail(BK_ERR_ARG, "hptr is NULL");
  *hptr = nullptr;
  if (bytes == 0) return BK_OK;
  // mapped: kernels of this library may read or write it at the same address (an output field
  // in this memory receives a sweep's results straight over the CPU-GPU link)
  BK_CUDA(cudaHostAlloc(hptr, bytes, cudaHostAllocMapped | cudaHostAllocPortable));
  void *dptr = nullptr;
  cudaError_t e = cudaHostGetDevicePointer(&dptr, *hptr, 0);
  if (e != cudaSuccess || dptr != *hptr) {
    cudaFreeHost(*hptr);
    *hptr = nullptr;
    return e != cudaSuccess ? cuda_fail(e, "cudaHostGetDevicePointer")
                            : fail(BK_ERR_UNSUPPORTED, "page-locked memory is not at the same device address");
  }
  return BK_OK;
}

int bk_host_free(void *hptr) {
  if (hptr) BK_CUDA(cudaFreeHost(hptr));
  return BK_OK;
}

int bk_memcpy(void *dst, const void *src, size_t bytes, int kind, void *stream) {
  if (bytes == 0) return BK_OK;
  if (!dst || !src) return fail(BK_ERR_ARG, "bk_memcpy: NULL pointer");
  cudaMemcpyKind k;
  switch (kind) {
    case 0: k = cudaMemcpyHostToDevice; break;
    case 1: k = cudaMemcpyDeviceToHost; break;
    case 2: k = cudaMemcpyDeviceToDevice; break;
    default: return fail(BK_ERR_ARG, "bk_memcpy: kind must be 0, 1 or 2");
  }
  BK_CUDA(cudaMemcpyAsync(dst, src, bytes, k, as_stream(stream)));
  return BK_OK;
}

int bk_memset(void *dptr, int value, size_t bytes, void *stream) {
  if (bytes == 0) return BK_OK;
  if (!dptr) return fail(BK_ERR_ARG, "bk_memset: NULL pointer");
  BK_CUDA(cudaMemsetAsync(dptr, value, bytes, as_stream(stream)));
  return BK_OK;
}

int bk_info_to_device(const unsigned *adj_host, unsigned nbricks, unsigned **adj_dev) {
  if (!adj_host || !adj_dev || nbricks == 0) return fail(BK_ERR_ARG, "bk_info_to_device: bad arguments");
  *adj_dev = nullptr;
  size_t bytes = (size_t)nbricks * 27 * sizeof(unsigned);
  unsigned *p = nullptr;
  BK_CUDA(cudaMalloc(&p, bytes));
  cudaError_t e = cudaMemcpy(p, adj_host, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(p);
    return cuda_fail(e, "cudaMemcpy(adj)");
  }
  *adj_dev = p;
  return BK_OK;
}

int bk_storage_to_device(const void *host, long chunks, size_t step, int dtype, void **dev) {
  if (!host || !dev || chunks <= 0 || step == 0 || !dtype_ok(dtype))
    return fail(BK_ERR_ARG, "bk_storage_to_device: bad arguments");
  *dev = nullptr;
  size_t bytes = (size_t)chunks * step * dtype_size(dtype);
  void *p = nullptr;
  BK_CUDA(cudaMalloc(&p, bytes));
  cudaError_t e = cudaMemcpy(p, host, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(p);
    return cuda_fail(e, "cudaMemcpy(storage)");
  }
  *dev = p;
  return BK_OK;
}

int bk_storage_to_host(const void *dev, long chunks, size_t step, int dtype, void *host) {
  if (!host || !dev || chunks <= 0 || step == 0 || !dtype_ok(dtype))
    return fail(BK_ERR_ARG, "bk_storage_to_host: bad arguments");
  BK_CUDA(cudaMemcpy(host, dev, (size_t)chunks * step * dtype_size(dtype), cudaMemcpyDeviceToHost));
  return BK_OK;
}

int bk_error_flags(void *stream, int *flags) {
  if (!flags) return fail(BK_ERR_ARG, "flags is NULL");
  int *w = device_error_word();
  if (!w) return fail(BK_ERR_CUDA, "device error word unavailable");
  int h = 0;
  BK_CUDA(cudaMemcpyAsync(&h, w, sizeof(int), cudaMemcpyDeviceToHost, as_stream(stream)));
  BK_CUDA(cudaMemsetAsync(w, 0, sizeof(int), as_stream(stream)));
  BK_CUDA(cudaStreamSynchronize(as_stream(stream)));
  *flags = h;
  return BK_OK;
}

int bk_periodic_plan(const unsigned *grid, const long nb[3], const long gb[3], unsigned *pairs,
                     long cap, long *npairs) {
  if (!grid || !nb || !gb || !npairs) return fail(BK_ERR_ARG, "bk_periodic_plan: bad arguments");
  long G[3];
  for (int d = 0; d < 3; ++d) {
    if (nb[d] <= 0 || gb[d] < 0 || gb[d] > nb[d])
      return fail(BK_ERR_ARG, "bk_periodic_plan: need 0 <= ghost bricks <= interior bricks");
    G[d] = nb[d] + 2 * gb[d];
  }
  long cnt = 0;
  for (long k = 0; k < G[0]; ++k)
    for (long j = 0; j < G[1]; ++j)
      for (long i = 0; i < G[2]; ++i) {
        const long c[3] = {k, j, i};
        bool ghost = false;
        long s[3];
        for (int d = 0; d < 3; ++d) {
          if (c[d] < gb[d] || c[d] >= gb[d] + nb[d]) ghost = true;
          long r = (c[d] - gb[d]) % nb[d];
          s[d] = gb[d] + (r < 0 ? r + nb[d] : r);
        }
        if (!ghost) continue;
        if (pairs && cnt < cap) {
          pairs[2 * cnt] = grid[(k * G[1] + j) * G[2] + i];
          pairs[2 * cnt + 1] = grid[(s[0] * G[1] + s[1]) * G[2] + s[2]];
        }
        ++cnt;
      }
  *npairs = cnt;
  if (pairs && cnt > cap) return fail(BK_ERR_ARG, "bk_periodic_plan: capacity too small");
  return BK_OK;
}

}  // extern "C"
