/*
 * ref_decomp.cpp -- runs the reference's own BrickDecomp layout producer
 * (include/brick-mpi.h:168-464: the constructor :298-316 and initialize :322-464, with
 * allneighbors and the skin orders of src/brick-mpi.cpp:9-112), compiled from the reference
 * sources where they lie (oracle/Makefile, target `ref`), against the declarations-only
 * oracle/mpi_decls/mpi.h: initialize makes no MPI call.
 *
 * TEST INFRASTRUCTURE ONLY: it writes the tests/golden/decomp_*.npz fixtures that pin the
 * product's bk_decomp_* layouts.  Nothing in the product links it.
 *
 * Two inputs the reference takes from its build and host are set per call here:
 *   - the page size: initialize reads sysconf(_SC_PAGESIZE) (brick-mpi.h:343); the call below
 *     is routed to page_size() for this translation unit only;
 *   - the element size: bElem is double in this build, and a brick of another element size
 *     is described by scaling the page instead.  The layout depends on the brick bytes only
 *     through the ratio brick bytes : page bytes (brick-mpi.h:344-351), so a page of
 *     P x 8 / elem_bytes bytes with 8-byte elements gives the layout of elem_bytes-byte
 *     elements with a page of P bytes.
 */
#include <unistd.h>

#include <cstdint>
#include <cstring>
#include <vector>

namespace {
long g_page = 4096;
long page_size(int) { return g_page; }
}  // namespace

#define sysconf page_size
#include "brick-mpi.h"
#undef sysconf

namespace {

// Flat grid position (dimension 0 fastest) -> brick, read through the reference's
// grid_access chain (brick-mpi.h:46-75): d[c_{n-1}]...[c_0].
template <unsigned dim, unsigned... BD>
unsigned grid_at(BrickDecomp<dim, BD...> &d, const std::vector<unsigned> &c);
template <>
unsigned grid_at<2, 8, 8>(BrickDecomp<2, 8, 8> &d, const std::vector<unsigned> &c) { return d[c[1]][c[0]]; }
template <>
unsigned grid_at<3, 8, 8, 8>(BrickDecomp<3, 8, 8, 8> &d, const std::vector<unsigned> &c) {
  return d[c[2]][c[1]][c[0]];
}
template <>
unsigned grid_at<3, 4, 4, 4>(BrickDecomp<3, 4, 4, 4> &d, const std::vector<unsigned> &c) {
  return d[c[2]][c[1]][c[0]];
}
template <>
unsigned grid_at<4, 4, 4, 4, 4>(BrickDecomp<4, 4, 4, 4, 4> &d, const std::vector<unsigned> &c) {
  return d[c[3]][c[2]][c[1]][c[0]];
}

// info: [0] nbricks (BrickInfo size = sep_pos[2]), [1..3] sep_pos, [4] grid positions,
// [5] ghost (= skin) records.  grid / adj / regions / skin_size are written when non-null:
// regions holds 2 x nregions records of 7 int64 (neighbor set, skin_st, skin_ed, pos, len,
// first_pad, last_pad), ghost records first.
template <unsigned dim, unsigned... BD>
int run(const unsigned *dims, unsigned depth, unsigned numfield, const uint64_t *skin, unsigned nskin, long *info,
        unsigned *grid, unsigned *adj, long long *regions, long *skin_size) {
  constexpr unsigned bd[] = {BD...};
  std::vector<unsigned> dv(dims, dims + dim);
  BrickDecomp<dim, BD...> d(dv, depth, numfield);
  std::vector<BitSet> sl;
  for (unsigned q = 0; q < nskin; ++q) sl.emplace_back(BitSet(skin[q]));
  d.initialize(sl);
  std::vector<unsigned> t(dim);
  long gsize = 1;
  for (unsigned q = 0; q < dim; ++q) {
    // bdims are listed outermost first; dims contiguous first (brick-mpi.h:307-315)
    t[q] = dims[q] / bd[dim - 1 - q] + 2 * (depth / bd[dim - 1 - q]);
    gsize *= t[q];
  }
  BrickInfo<dim> bi = d.getBrickInfo();
  info[0] = (long)bi.nbricks;
  for (int q = 0; q < 3; ++q) info[1 + q] = d.sep_pos[q];
  info[4] = gsize;
  info[5] = (long)d.ghost.size();
  if (grid) {
    std::vector<unsigned> c(dim, 0);
    for (long p = 0; p < gsize; ++p) {
      long r = p;
      for (unsigned q = 0; q < dim; ++q) {
        c[q] = (unsigned)(r % t[q]);
        r /= t[q];
      }
      grid[p] = grid_at<dim, BD...>(d, c);
    }
  }
  if (adj) {
    constexpr unsigned w = static_power<3, dim>::value;
    for (unsigned b = 0; b < bi.nbricks; ++b)
      for (unsigned s = 0; s < w; ++s) adj[(size_t)b * w + s] = bi.adj[b][s];
  }
  if (regions) {
    auto put = [](long long *o, const typename BrickDecomp<dim, BD...>::g_region &g) {
      const long long v[7] = {(long long)g.neighbor.set, g.skin_st, g.skin_ed, g.pos, g.len, g.first_pad, g.last_pad};
      std::memcpy(o, v, sizeof(v));
    };
    const size_t n = d.ghost.size();
    for (size_t q = 0; q < n; ++q) {
      put(regions + 7 * q, d.ghost[q]);
      put(regions + 7 * (n + q), d.skin[q]);
    }
  }
  if (skin_size)
    for (size_t q = 0; q < d.skin_size.size(); ++q) skin_size[q] = d.skin_size[q];
  return 0;
}

}  // namespace

extern std::vector<BitSet> skin3d_good, skin3d_normal;  // src/brick-mpi.cpp:25-82

extern "C" {

/* The reference's skin orders (which: 0 skin3d_good, 1 skin3d_normal) as BitSet words; returns
 * the count (out may be null to ask for it). */
int ref_skin_list(int which, uint64_t *out) {
  const std::vector<BitSet> &l = which == 0 ? skin3d_good : skin3d_normal;
  if (out)
    for (size_t q = 0; q < l.size(); ++q) out[q] = l[q].set;
  return (int)l.size();
}

/* allneighbors(0, 1, dim, .) (src/brick-mpi.cpp:9-23): every region of dim dimensions, the empty
 * one included, in the reference's enumeration order; returns the count. */
int ref_allneighbors(int dim, uint64_t *out) {
  std::vector<BitSet> n;
  allneighbors(0, 1, dim, n);
  if (out)
    for (size_t q = 0; q < n.size(); ++q) out[q] = n[q].set;
  return (int)n.size();
}

/* BrickDecomp<dim, bdim...>(dims, depth, numfield).initialize(skin) of the reference.
 * bcase: 0 -> <3, 8,8,8>, 1 -> <3, 4,4,4>, 2 -> <2, 8,8>, 3 -> <4, 4,4,4,4>.
 * elem_bytes / pagesize: see the file comment.  Returns 0, or -1 for an unknown case. */
int ref_decomp(int bcase, const unsigned *dims, unsigned depth, unsigned numfield, long elem_bytes, long pagesize,
               const uint64_t *skin, unsigned nskin, long *info, unsigned *grid, unsigned *adj,
               long long *regions, long *skin_size) {
  if (elem_bytes <= 0 || pagesize <= 0) return -1;
  g_page = pagesize * (long)sizeof(bElem) / elem_bytes;
  if (g_page < 1) g_page = 1;
  switch (bcase) {
    case 0: return run<3, 8, 8, 8>(dims, depth, numfield, skin, nskin, info, grid, adj, regions, skin_size);
    case 1: return run<3, 4, 4, 4>(dims, depth, numfield, skin, nskin, info, grid, adj, regions, skin_size);
    case 2: return run<2, 8, 8>(dims, depth, numfield, skin, nskin, info, grid, adj, regions, skin_size);
    case 3: return run<4, 4, 4, 4, 4>(dims, depth, numfield, skin, nskin, info, grid, adj, regions, skin_size);
  }
  return -1;
}

}  // extern "C"
