/*
 * brick-decomp.h -- BrickDecomp<dim, BDims...> without MPI, for one GB300: the reference's
 * decomposition (include/brick-mpi.h:178-464) computed by the library (bk_decomp_*), with
 * the same public members and grid access, and exchange() as the periodic wrap of a single
 * domain on the device (brick-mpi.h:466-499 on one periodic rank: ghost[i] <- skin[i]).
 *
 *   BrickDecomp<3, 8, 8, 8> bDecomp({512, 512, 512}, 8);   // dims contiguous first, depth
 *   bDecomp.initialize(skin3d_good);
 *   BrickInfo<3> bInfo = bDecomp.getBrickInfo();           // adjacency owned by bDecomp
 *   unsigned b = bDecomp[k][j][i];                         // grid position -> brick
 *   bDecomp.exchange(deviceStorage);                       // periodic ghost refresh
 *
 * There is no communicator and no rank map: every neighbour of the domain is the domain.
 * Define DECOMP_PAGEUNALIGN for the unpadded layout, as the reference does.
 */
#ifndef BRICK_GB300_DECOMP_H
#define BRICK_GB300_DECOMP_H

#include <unistd.h>

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "bitset.h"
#include "brick-gb300.h"
#include "brick.h"
#include "bricklib_gb300.h"

/// skin orders of the reference (src/brick-mpi.cpp:25-112): data, kept identical
inline const std::vector<BitSet> skin3d_good = {
    {1}, {1, -3}, {1, 2, -3}, {1, 2}, {1, 2, 3}, {2, 3}, {2}, {2, -3}, {-1, 2, -3}, {-1, 2}, {-1, 2, 3},
    {-1, 3}, {-1}, {-3}, {-1, -3}, {-1, -2, -3}, {-1, -2}, {-1, -2, 3}, {-2, 3}, {-2}, {-2, -3},
    {1, -2, -3}, {1, -2}, {1, -2, 3}, {1, 3}, {3}};
inline const std::vector<BitSet> skin3d_normal = {
    {-1, -2, -3}, {-2, -3}, {1, -2, -3}, {-1, -3}, {-3}, {1, -3}, {-1, 2, -3}, {2, -3}, {1, 2, -3},
    {-1, -2}, {-2}, {1, -2}, {-1}, {}, {1}, {-1, 2}, {2}, {1, 2}, {-1, -2, 3}, {-2, 3}, {1, -2, 3},
    {-1, 3}, {3}, {1, 3}, {-1, 2, 3}, {2, 3}, {1, 2, 3}};

template <unsigned dim, unsigned... BDims>
class BrickDecomp {
 public:
  typedef struct {
    BitSet neighbor;     ///< the neighbour the region is exchanged with
    unsigned skin_st;    ///< first skin-list entry of the region
    unsigned skin_ed;    ///< one past the last skin-list entry
    unsigned pos;        ///< first brick
    unsigned len;        ///< bricks, including the padding bricks below
    unsigned first_pad;
    unsigned last_pad;
  } g_region;
  std::vector<g_region> ghost;   ///< ghost regions
  std::vector<g_region> skin;    ///< skin regions; ghost[i] receives skin[i]
  unsigned sep_pos[3];           ///< ends of the inner, skin and ghost brick ranges
  std::vector<BitSet> skinlist;  ///< the skin order the layout was built with
  std::vector<long> skin_size;   ///< bricks per skin-list entry (padding included)

  /// dims: interior elements per dimension, contiguous first; depth: ghost elements
  BrickDecomp(const std::vector<unsigned> &dims, const unsigned depth, unsigned numfield = 1)
      : dims_(dims), depth_(depth), numfield_(numfield) {
    if (dims.size() != dim) throw std::runtime_error("BrickDecomp: one size per dimension");
  }
  BrickDecomp(const BrickDecomp &) = delete;
  BrickDecomp &operator=(const BrickDecomp &) = delete;

  void initialize(const std::vector<BitSet> &skinlist_in) {
    release();
    skinlist = skinlist_in;
    std::vector<unsigned> bd = {BDims...};
    std::vector<unsigned> bdims(bd.rbegin(), bd.rend());  // contiguous first
    std::vector<uint64_t> sk;
    for (auto &b : skinlist) sk.push_back(b.set);
#ifdef DECOMP_PAGEUNALIGN
    const long page = 1;
#else
    const long page = sysconf(_SC_PAGESIZE);
#endif
    check(bk_decomp_create((int)dim, dims_.data(), bdims.data(), depth_, numfield_, sizeof(bElem), page, sk.data(),
                           (unsigned)sk.size(), &h_));
    size_t gsize = 0;
    unsigned nreg = 0;
    check(bk_decomp_info(h_, &nbricks_, &gsize, &nreg, sep_pos));
    grid_.resize(gsize);
    check(bk_decomp_grid(h_, grid_.data()));
    bInfo_ = new BrickInfo<dim>(nbricks_);
    check(bk_decomp_adjacency(h_, &bInfo_->adj[0][0]));
    std::vector<bk_decomp_region> g(nreg), s(nreg);
    skin_size.assign(skinlist.size(), 0);
    check(bk_decomp_regions(h_, g.data(), s.data(), skin_size.data()));
    ghost.clear();
    skin.clear();
    for (unsigned q = 0; q < nreg; ++q) {
      ghost.push_back(conv(g[q]));
      skin.push_back(conv(s[q]));
    }
    stride_.assign(dim, 1);
    for (unsigned d = 1; d < dim; ++d) {
      const unsigned bprev = bdims[d - 1];
      stride_[d] = stride_[d - 1] * (dims_[d - 1] / bprev + 2 * (depth_ / bprev));
    }
  }

  /// grid access, outermost dimension first: bDecomp[k][j][i] (grid_access of brick-mpi.h)
  struct access {
    const BrickDecomp *self;
    size_t ref;
    unsigned d;
    access operator[](int i) const { return {self, ref + (size_t)i * self->stride_[d - 1], d - 1}; }
    operator unsigned() const { return self->grid_[ref]; }
  };
  access operator[](int i) const { return access{this, 0, dim}[i]; }

  /// the decomposition's BrickInfo (adjacency owned by this object)
  BrickInfo<dim> getBrickInfo() const { return *bInfo_; }

  /// periodic ghost refresh of a device storage built on this decomposition
  void exchange(BrickStorage &bStorage, cudaStream_t stream = 0) {
    const void *dat = bStorage.dat.get();
    if (dat != links_for_) {
      std::vector<uint64_t> links(3 * ghost.size());
      check(bk_decomp_exchange_links(h_, dat, bStorage.step * sizeof(bElem), links.data()));
      if (!links_dev_) check(bk_device_malloc(&links_dev_, links.size() * sizeof(uint64_t) + 8));
      check(bk_memcpy(links_dev_, links.data(), links.size() * sizeof(uint64_t), 0, (void *)stream));
      links_for_ = dat;
    }
    check(bk_region_copy((const uint64_t *)links_dev_, (unsigned)ghost.size(), (void *)stream));
  }

  ~BrickDecomp() { release(); }

 private:
  std::vector<unsigned> dims_;
  unsigned depth_, numfield_;
  bk_decomp *h_ = nullptr;
  unsigned nbricks_ = 0;
  std::vector<unsigned> grid_;
  std::vector<size_t> stride_;
  BrickInfo<dim> *bInfo_ = nullptr;
  void *links_dev_ = nullptr;
  const void *links_for_ = nullptr;

  static g_region conv(const bk_decomp_region &r) {
    return g_region{BitSet(r.neighbor), r.skin_st, r.skin_ed, r.pos, r.len, r.first_pad, r.last_pad};
  }
  static void check(int s) {
    if (s != BK_OK) throw std::runtime_error(std::string("BrickDecomp: ") + bk_last_error());
  }
  void release() {
    if (h_) bk_decomp_destroy(h_);
    h_ = nullptr;
    if (bInfo_) {
      free(bInfo_->adj);
      delete bInfo_;
      bInfo_ = nullptr;
    }
    if (links_dev_) bk_device_free(links_dev_);
    links_dev_ = nullptr;
    links_for_ = nullptr;
  }
};

#endif  // BRICK_GB300_DECOMP_H
