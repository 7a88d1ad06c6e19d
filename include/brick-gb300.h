/*
 * brick-gb300.h -- the device layer of the brick API on the GB300 engine; include it
 * where bricklib code includes brick-cuda.h (include/brick-cuda.h, brick-gpu.h).
 *
 *   gpuCheck(x)        checks a cudaError_t or bk_status; on failure prints the call and
 *                      exits (the reference's _gpuCheck, brick-gpu.h:27-33).  Unlike the
 *                      reference macro (brick-gpu.h:16-22) it checks in every build.
 *   movBrickInfo       brick-gpu.h:42-55, adjacency copied by bk_info_to_device
 *   movBrickInfoDeep   brick-gpu.h:64-76
 *   movBrickStorage    brick-gpu.h:84-103, device memory owned by a shared_ptr whose
 *                      deleter is bk_device_free
 *   brickSweep         one sweep of a bk_stencil over a device brick list: what a
 *                      brick("x.py", VSVEC, (8,8,8), (4,8), b) kernel launched over the
 *                      listed bricks computes (stencils/3axis.cu:28-37, weak/main.cu:35-43)
 *   brickGhostFill     device ghost-zone fill from (dst, src) brick pairs
 *
 * A Brick passed to brickSweep must be built on the host struct returned by
 * movBrickInfo (device adjacency pointer, host struct) and a device BrickStorage.
 */
#ifndef BRICK_GB300_H
#define BRICK_GB300_H

#include <cuda_runtime_api.h>

#include <cassert>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <memory>

#include "brick.h"
#include "bricklib_gb300.h"

#define gpuMemcpyKind cudaMemcpyKind
#define gpuMemcpyHostToDevice cudaMemcpyHostToDevice
#define gpuMemcpyDeviceToHost cudaMemcpyDeviceToHost
#define gpuSuccess 0

namespace brick_gb300 {

inline void check_status(long e, bool is_cuda, const char *call, const char *file, int line) {
  if (e == 0) return;
  const char *msg = is_cuda ? cudaGetErrorString((cudaError_t)e) : bk_last_error();
  fprintf(stderr, "\"%s\" at %d in %s\n\treturned %ld\n-> %s\n", call, line, file, e, msg);
  exit(EXIT_FAILURE);
}
inline void check_any(cudaError_t e, const char *c, const char *f, int l) { check_status((long)e, true, c, f, l); }
inline void check_any(int e, const char *c, const char *f, int l) { check_status((long)e, false, c, f, l); }

template <typename T> struct dtype_of;
template <> struct dtype_of<double> { static constexpr int value = BK_F64; };
template <> struct dtype_of<float> { static constexpr int value = BK_F32; };

template <typename BrickT> struct layout_of;
template <unsigned... BDims, unsigned... Folds>
struct layout_of<Brick<Dim<BDims...>, Dim<Folds...>>> {
  static bk_layout get() {
    typedef Brick<Dim<BDims...>, Dim<Folds...>> B;
    static_assert(B::DIMS == 3, "the GB300 sweep is three-dimensional");
    bk_layout l;
    for (unsigned d = 0; d < 3; ++d) {
      l.bdim[d] = (int)B::BD::get(d);
      l.fold[d] = (int)brick_detail::fold_of<typename B::BD, typename B::FD>(d);
    }
    return l;
  }
};

}  // namespace brick_gb300

#define gpuCheck(x) brick_gb300::check_any((x), #x, __FILE__, __LINE__)

template <unsigned dims>
BrickInfo<dims> movBrickInfo(BrickInfo<dims> &bInfo, cudaMemcpyKind kind) {
  assert(kind == cudaMemcpyHostToDevice || kind == cudaMemcpyDeviceToHost);
  BrickInfo<dims> ret = bInfo;
  const size_t size = (size_t)bInfo.nbricks * static_power<3, dims>::value * sizeof(unsigned);
  if (kind == cudaMemcpyHostToDevice) {
    unsigned *p = nullptr;
    if (dims == 3) {
      gpuCheck(bk_info_to_device(&bInfo.adj[0][0], bInfo.nbricks, &p));
    } else {  // 3^dims entries per brick
      gpuCheck(bk_device_malloc((void **)&p, size));
      gpuCheck(bk_memcpy(p, &bInfo.adj[0][0], size, 0, nullptr));
      gpuCheck(bk_stream_synchronize(nullptr));
    }
    ret.adj = (typename BrickInfo<dims>::adjlist)p;
  } else {
    ret.adj = (typename BrickInfo<dims>::adjlist)malloc(size);
    gpuCheck(bk_memcpy(ret.adj, bInfo.adj, size, 1, nullptr));
    gpuCheck(bk_stream_synchronize(nullptr));
  }
  return ret;
}

template <unsigned dims>
BrickInfo<dims> *movBrickInfoDeep(BrickInfo<dims> &bInfo, cudaMemcpyKind kind) {
  BrickInfo<dims> temp = movBrickInfo(bInfo, kind);
  BrickInfo<dims> *ret = nullptr;
  if (kind == cudaMemcpyHostToDevice) {
    gpuCheck(bk_device_malloc((void **)&ret, sizeof(BrickInfo<dims>)));
    gpuCheck(bk_memcpy(ret, &temp, sizeof(BrickInfo<dims>), 0, nullptr));
    gpuCheck(bk_stream_synchronize(nullptr));
  } else {
    ret = (BrickInfo<dims> *)malloc(sizeof(BrickInfo<dims>));
    memcpy(ret, &temp, sizeof(BrickInfo<dims>));
  }
  return ret;
}

inline BrickStorage movBrickStorage(BrickStorage &bStorage, cudaMemcpyKind kind) {
  assert(kind == cudaMemcpyHostToDevice || kind == cudaMemcpyDeviceToHost);
  BrickStorage ret = bStorage;
  const int dt = brick_gb300::dtype_of<bElem>::value;
  if (kind == cudaMemcpyHostToDevice) {
    void *p = nullptr;
    gpuCheck(bk_storage_to_device(bStorage.dat.get(), bStorage.chunks, bStorage.step, dt, &p));
    ret.dat = std::shared_ptr<bElem>((bElem *)p, [](bElem *q) { bk_device_free(q); });
  } else {
    bElem *h = (bElem *)malloc((size_t)bStorage.chunks * bStorage.step * sizeof(bElem));
    gpuCheck(bk_storage_to_host(bStorage.dat.get(), bStorage.chunks, bStorage.step, dt, h));
    ret.dat = std::shared_ptr<bElem>(h, [](bElem *q) { free(q); });
  }
  return ret;
}

/// bk_field view of a Brick whose storage lives on the device.
template <typename BrickT>
inline bk_field brickField(const BrickT &b) {
  bk_field f;
  f.dat = b.bStorage.dat.get();
  f.chunks = b.bStorage.chunks;
  f.step = b.bStorage.step;
  f.offset = (size_t)(b.dat - b.bStorage.dat.get());
  f.dtype = brick_gb300::dtype_of<bElem>::value;
  return f;
}

/// Tap-list builder: BrickStencil st; st.add(0,0,1, c1).add(0,0,-1, c2) ...
struct BrickStencil : bk_stencil {
  BrickStencil() : bk_stencil() {}
  BrickStencil &add(int dk, int dj, int di, double c) {
    if (npoints < BK_MAX_TAPS) {
      offsets[npoints][0] = dk;
      offsets[npoints][1] = dj;
      offsets[npoints][2] = di;
      coeff[npoints] = c;
      ++npoints;
    }
    return *this;
  }
};

template <typename BrickT>
inline void brickSweep(BrickT &bIn, BrickT &bOut, const unsigned *blist_dev, unsigned nlist, const bk_stencil &st,
                       int acc = BK_ACC_NATIVE, cudaStream_t stream = 0) {
  const bk_field in = brickField(bIn), out = brickField(bOut);
  const bk_layout lay = brick_gb300::layout_of<BrickT>::get();
  gpuCheck(bk_sweep(&bIn.bInfo->adj[0][0], bIn.bInfo->nbricks, &in, &out, blist_dev, nlist, &st, &lay, acc,
                    (void *)stream));
}

/// 4-D tap-list builder: BrickStencil4 st; st.add(dl, dk, dj, di, c) ...
struct BrickStencil4 : bk_stencil4 {
  BrickStencil4() : bk_stencil4() {}
  BrickStencil4 &add(int dl, int dk, int dj, int di, double c) {
    if (npoints < BK_MAX_TAPS4) {
      offsets[npoints][0] = dl;
      offsets[npoints][1] = dk;
      offsets[npoints][2] = dj;
      offsets[npoints][3] = di;
      coeff[npoints] = c;
      ++npoints;
    }
    return *this;
  }
};

/// One sweep of a 4-D Brick<Dim<4,4,4,4>, Dim<fold>> (weak/main-4d.cpp) over a device brick list.
template <typename BrickT>
inline void brickSweep4(BrickT &bIn, BrickT &bOut, const unsigned *blist_dev, unsigned nlist, const bk_stencil4 &st,
                        cudaStream_t stream = 0) {
  static_assert(BrickT::DIMS == 4, "brickSweep4 takes four-dimensional bricks");
  typedef typename BrickT::BD BD;
  typedef typename BrickT::FD FD;
  bk_layout4 lay;
  for (unsigned d = 0; d < 4; ++d) {
    lay.bdim[d] = (int)BD::get(d);
    lay.fold[d] = (int)brick_detail::fold_of<BD, FD>(d);
  }
  const bk_field in = brickField(bIn), out = brickField(bOut);
  gpuCheck(bk_sweep4(&bIn.bInfo->adj[0][0], bIn.bInfo->nbricks, &in, &out, blist_dev, nlist, &st, &lay,
                     (void *)stream));
}

template <typename BrickT>
inline void brickGhostFill(BrickT &b, const unsigned *pairs_dev, unsigned npairs, cudaStream_t stream = 0) {
  const bk_field f = brickField(b);
  const bk_layout lay = brick_gb300::layout_of<BrickT>::get();
  gpuCheck(bk_ghost_fill(pairs_dev, npairs, &f, &lay, (void *)stream));
}

#endif  // BRICK_GB300_H
