/*
 * brick-vs.h -- runtime of the brick(...) statements that bricklib_gb300.dsl.vecscatter lowers.
 *
 * In the reference a `brick("x.py", VEC, (dims), (fold), b);` statement inside a per-brick
 * loop becomes, through its code generator (include/vecscatter.h:62,
 * codegen/vecscatter:145-186), code that computes brick b.  The lowering tool of this engine
 * keeps the loop, makes it record the bricks it visits on a per-statement Site, and follows
 * it with one Site::sweep -- a bk_sweep of the script's tap list over all of them:
 *
 *   { static bk_vs::Site s; s.begin();
 *     for (...) for (...) for (...) { unsigned b = grid[tk][tj][ti]; s.visit(b); }
 *     s.sweep(bIn, bOut, BrickStencil().add(0, 0, 0, (coeff[0])) ...); }
 *
 * Bricks whose storage is device memory (movBrickInfo / movBrickStorage) are swept in place.
 * Bricks in host memory -- a CPU program such as stencils/3axis.cpp -- run on device mirrors:
 * the adjacency and the storages are copied to the device before the sweep and the output
 * storage back after it, so the program sees its results where the reference's generated CPU
 * code would have written them.  The brick list stays on the device between calls and is
 * uploaded again only when the loop visited other bricks.  Sweeps are synchronous (the next
 * host statement may read the output).  A Site is not shared between host threads.
 */
#ifndef BRICK_VS_H
#define BRICK_VS_H

#include <cuda_runtime_api.h>

#include <cstring>
#include <memory>
#include <vector>

#include "brick-gb300.h"

namespace bk_vs {

/// The tap list with pointwise operations (the cond stencil: pre max(x, 0), post |x|).
inline bk_stencil with_ops(bk_stencil st, int pre, int post) {
  st.pre_op = pre;
  st.post_op = post;
  return st;
}

/// Whether p points into device memory.
inline bool on_device(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear the error of a pointer the runtime does not know
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

/// A device buffer kept between calls, grown on demand.
class DevBuf {
 public:
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() {
    if (p_) bk_device_free(p_);
  }
  void *get(size_t bytes) {
    if (bytes > n_) {
      if (p_) gpuCheck(bk_device_free(p_));
      p_ = nullptr;
      gpuCheck(bk_device_malloc(&p_, bytes));
      n_ = bytes;
    }
    return p_;
  }
  void *ptr() const { return p_; }

 private:
  void *p_ = nullptr;
  size_t n_ = 0;
};

/// One lowered brick(...) statement.
class Site {
 public:
  void begin() { list_.clear(); }
  void visit(unsigned b) { list_.push_back(b); }

  template <typename BrickT>
  void sweep(BrickT &bIn, BrickT &bOut, const bk_stencil &st) {
    if (list_.empty()) return;
    if (list_ != uploaded_) {
      gpuCheck(bk_memcpy(dlist_.get(list_.size() * sizeof(unsigned)), list_.data(), list_.size() * sizeof(unsigned),
                         0, nullptr));
      uploaded_ = list_;
    }
    const unsigned *dl = static_cast<const unsigned *>(dlist_.ptr());
    const unsigned n = (unsigned)list_.size();
    if (on_device(bIn.bStorage.dat.get())) {
      brickSweep(bIn, bOut, dl, n, st);
      gpuCheck(bk_stream_synchronize(nullptr));
      return;
    }
    // host bricks: device mirrors of the adjacency and of the storages around the sweep
    typedef typename BrickT::myBrickInfo Info;
    Info dinfo = *bIn.bInfo;
    const size_t adj_bytes = (size_t)dinfo.nbricks * sizeof(dinfo.adj[0]);
    dinfo.adj = reinterpret_cast<typename Info::adjlist>(adj_.get(adj_bytes));
    gpuCheck(bk_memcpy(dinfo.adj, bIn.bInfo->adj, adj_bytes, 0, nullptr));
    const bool same = bIn.bStorage.dat.get() == bOut.bStorage.dat.get();
    BrickStorage din = mirror(bIn.bStorage, in_, true);
    BrickStorage dout = same ? din : mirror(bOut.bStorage, out_, false);
    BrickT mi(&dinfo, din, (unsigned)(bIn.dat - bIn.bStorage.dat.get()));
    BrickT mo(&dinfo, dout, (unsigned)(bOut.dat - bOut.bStorage.dat.get()));
    brickSweep(mi, mo, dl, n, st);
    gpuCheck(bk_memcpy(bOut.bStorage.dat.get(), dout.dat.get(), bytes_of(bOut.bStorage), 1, nullptr));
    gpuCheck(bk_stream_synchronize(nullptr));
  }

 private:
  static size_t bytes_of(const BrickStorage &s) { return (size_t)s.chunks * s.step * sizeof(bElem); }
  // a device storage of the same shape (not owning buf's memory), with the host contents if copy
  static BrickStorage mirror(const BrickStorage &h, DevBuf &buf, bool copy) {
    BrickStorage d;
    d.chunks = h.chunks;
    d.step = h.step;
    bElem *p = static_cast<bElem *>(buf.get(bytes_of(h)));
    d.dat = std::shared_ptr<bElem>(p, [](bElem *) {});
    if (copy) gpuCheck(bk_memcpy(p, h.dat.get(), bytes_of(h), 0, nullptr));
    return d;
  }
  std::vector<unsigned> list_, uploaded_;
  DevBuf dlist_, adj_, in_, out_;
};

}  // namespace bk_vs

#endif  // BRICK_VS_H
