// Ghost-zone fill / periodic wrap and batched region copies on the device.
#include "bk_common.cuh"

namespace bk {

// (dst, src) brick pairs; `words` words of W bytes per brick field.  Bricks of at most 256
// words: a CTA takes GF_PAIRS pairs at a time, each thread loading its word of every pair
// before storing any (more bytes in flight per SM); larger bricks: one pair per CTA step.
constexpr int GF_PAIRS = 4;
template <typename W>
__global__ void __launch_bounds__(256)
ghost_fill_kernel(const unsigned *__restrict__ pairs, unsigned npairs, unsigned char *dat,
                  unsigned long long step_bytes, unsigned long long off_bytes, unsigned words,
                  long long chunks, int *err) {
  if (words <= blockDim.x) {
    const unsigned t = threadIdx.x;
    for (unsigned p0 = blockIdx.x * GF_PAIRS; p0 < npairs; p0 += gridDim.x * GF_PAIRS) {
      W v[GF_PAIRS];
      W *d[GF_PAIRS];
#pragma unroll
      for (int q = 0; q < GF_PAIRS; ++q) {
        d[q] = nullptr;
        const unsigned p = p0 + q;
        if (p >= npairs) continue;
        const unsigned dst = pairs[2 * p], src = pairs[2 * p + 1];
        if ((long long)dst >= chunks || (long long)src >= chunks) {
          if (t == 0) atomicOr(err, FLAG_BOUNDS);
          continue;
        }
        if (t < words) {
          v[q] = reinterpret_cast<const W *>(dat + (size_t)src * step_bytes + off_bytes)[t];
          d[q] = reinterpret_cast<W *>(dat + (size_t)dst * step_bytes + off_bytes) + t;
        }
      }
#pragma unroll
      for (int q = 0; q < GF_PAIRS; ++q)
        if (d[q]) *d[q] = v[q];
    }
    return;
  }
  for (unsigned p = blockIdx.x; p < npairs; p += gridDim.x) {
    const unsigned dst = pairs[2 * p], src = pairs[2 * p + 1];
    if ((long long)dst >= chunks || (long long)src >= chunks) {
      if (threadIdx.x == 0) atomicOr(err, FLAG_BOUNDS);
      continue;
    }
    const W *s = reinterpret_cast<const W *>(dat + (size_t)src * step_bytes + off_bytes);
    W *d = reinterpret_cast<W *>(dat + (size_t)dst * step_bytes + off_bytes);
    for (unsigned w = threadIdx.x; w < words; w += blockDim.x) d[w] = s[w];
  }
}

// strong/main.cu:76-83 cudaCopy over {from, to, bytes} links.  Every CTA walks every link
// and copies its share of it (16-byte words where the link allows, else 8-byte words), so
// both many small links and a few large ones spread over the whole grid.
__global__ void __launch_bounds__(256) region_copy_kernel(const uint64_t *__restrict__ links, unsigned nlinks) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, nt = (uint64_t)gridDim.x * blockDim.x;
  for (unsigned l = 0; l < nlinks; ++l) {
    const uint64_t from = links[3 * l], to = links[3 * l + 1], bytes = links[3 * l + 2];
    if (((from | to | bytes) & 15) == 0) {
      const uint4 *s = reinterpret_cast<const uint4 *>(from);
      uint4 *d = reinterpret_cast<uint4 *>(to);
      const uint64_t n = bytes / 16;
      uint64_t w = t;
      for (; w + 3 * nt < n; w += 4 * nt) {  // four loads in flight before the stores
        const uint4 a = s[w], b = s[w + nt], c = s[w + 2 * nt], e = s[w + 3 * nt];
        d[w] = a;
        d[w + nt] = b;
        d[w + 2 * nt] = c;
        d[w + 3 * nt] = e;
      }
      for (; w < n; w += nt) d[w] = s[w];
    } else {
      const uint64_t *s = reinterpret_cast<const uint64_t *>(from);
      uint64_t *d = reinterpret_cast<uint64_t *>(to);
      for (uint64_t w = t; w < bytes / 8; w += nt) d[w] = s[w];
    }
  }
}

int ghost_fill(const unsigned *pairs, unsigned npairs, const bk_field *f, const Layout &L, cudaStream_t s) {
  if (npairs == 0) return BK_OK;
  int *err = device_error_word();
  if (!err) return fail(BK_ERR_CUDA, "device error word unavailable");
  const size_t es = dtype_size(f->dtype);
  const unsigned long long step_b = f->step * es, off_b = f->offset * es;
  const size_t bytes = (size_t)L.size() * es;
  const uintptr_t base = reinterpret_cast<uintptr_t>(f->dat);
  const unsigned groups = (npairs + GF_PAIRS - 1) / GF_PAIRS;
  const unsigned grid = groups < (1u << 30) ? groups : (1u << 30);
  unsigned char *dat = reinterpret_cast<unsigned char *>(f->dat);
  if (((base | step_b | off_b | bytes) & 15) == 0)
    ghost_fill_kernel<uint4><<<grid, 256, 0, s>>>(pairs, npairs, dat, step_b, off_b, (unsigned)(bytes / 16), f->chunks, err);
  else if (((base | step_b | off_b | bytes) & 7) == 0)
    ghost_fill_kernel<uint2><<<grid, 256, 0, s>>>(pairs, npairs, dat, step_b, off_b, (unsigned)(bytes / 8), f->chunks, err);
  else
    ghost_fill_kernel<unsigned short><<<grid, 256, 0, s>>>(pairs, npairs, dat, step_b, off_b, (unsigned)(bytes / 2), f->chunks, err);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "ghost fill launch");
  return BK_OK;
}

}  // namespace bk

using namespace bk;

extern "C" {

int bk_ghost_fill(const unsigned *pairs, unsigned npairs, const bk_field *f, const bk_layout *lay,
                  void *stream) {
  Layout L;
  int st = check_layout(lay, &L);
  if (st) return st;
  if ((st = check_field(f, L, "ghost"))) return st;
  if (npairs && !pairs) return fail(BK_ERR_ARG, "pairs is NULL");
  return ghost_fill(pairs, npairs, f, L, as_stream(stream));
}

int bk_region_copy(const uint64_t *links, unsigned nlinks, void *stream) {
  if (nlinks == 0) return BK_OK;
  if (!links) return fail(BK_ERR_ARG, "links is NULL");
  int dev = 0, sms = 0;
  BK_CUDA(cudaGetDevice(&dev));
  BK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  region_copy_kernel<<<(unsigned)sms * 4, 256, 0, as_stream(stream)>>>(links, nlinks);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "region copy launch");
  return BK_OK;
}

}  // extern "C"
