// BrickDecomp's layout producer without MPI (include/brick-mpi.h:178-464 of the reference):
// the brick storage order that keeps every skin region and every ghost region a contiguous
// run of bricks, its grid and adjacency, and the (ghost, skin) region records whose
// pairwise copies are the exchange.  On one GPU with periodic boundaries every neighbour
// is the domain itself, so the exchange is a handful of large device copies, ghost[i] <-
// skin[i] (brick-mpi.h:466-499 with one rank).
//
// Conventions follow the reference: dimension d = 0 is the contiguous one (i); a region or
// neighbour is a set of signed dimension numbers (+d / -d for the high / low side of
// dimension d-1, 1-based) encoded as the reference's BitSet bit field (bitset.h: +p is bit
// p, -p is bit 31 + p).
#include <cstdint>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "bk_common.cuh"

namespace bk {

namespace {

inline uint64_t sbit(long p) { return 1ull << (uint64_t)(p < 0 ? 31 - p : p); }
inline bool has(uint64_t set, long p) { return (set & sbit(p)) != 0; }
inline bool subset(uint64_t a, uint64_t b) { return (a & b) == a; }  // a <= b
inline long popcount(uint64_t s) { return __builtin_popcountll(s); }
// the opposite sides: +p <-> -p (bitset.h operator!)
inline uint64_t flip_sides(uint64_t s) {
  const uint64_t mask = (1ull << 32) - 1ull;
  return ((s & mask) << 31) | (s >> 31);
}

// every neighbour set of `dim` dimensions in the reference's order (brick-mpi.cpp:9-23):
// for dimension idx = 1..dim the choices are +idx, none, -idx, the first dimension varying
// slowest
void neighbour_sets(uint64_t cur, long idx, long dim, std::vector<uint64_t> &out) {
  if (idx > dim) {
    out.push_back(cur);
    return;
  }
  neighbour_sets(cur ^ sbit(idx), idx + 1, dim, out);
  neighbour_sets(cur, idx + 1, dim, out);
  neighbour_sets(cur ^ sbit(-idx), idx + 1, dim, out);
}

}  // namespace

struct Decomp {
  int dim = 0;
  std::vector<unsigned> dims, g_depth, t_dims, stride;  // in bricks, contiguous first
  std::vector<uint64_t> skinlist;
  std::vector<long> skin_size;
  std::vector<unsigned> grid;  // grid position -> brick index
  std::vector<unsigned> adj;   // brick index -> 3^dim neighbours
  std::vector<bk_decomp_region> ghost, skin;
  unsigned sep_pos[3] = {0, 0, 0};
  unsigned nbricks = 0;
  unsigned factor = 1;
  unsigned adj_width = 1;

  long region_size(uint64_t region) const {
    long n = 1;
    for (int d = 0; d < dim; ++d)
      n *= (has(region, d + 1) || has(region, -d - 1)) ? g_depth[d] : dims[d] - 2 * g_depth[d];
    return n;
  }
  // padding (bricks) that makes the region end on a page boundary (brick-mpi.h:364-370)
  long pad_of(uint64_t region) const {
    return (long)factor - (region_size(region) + factor - 1) % factor - 1;
  }
  // Number the bricks of `region` as seen from `owner` (the domain itself when 0, else the
  // neighbour on that side, whose skin maps into this domain's ghost zone) in grid order,
  // the last dimension outermost (brick-mpi.h:220-260).
  void number(uint64_t owner, uint64_t region, unsigned &pos) {
    long ref = 0;
    for (int d = 0; d < dim; ++d) {
      if (has(owner, d + 1)) ref += (long)dims[d] * stride[d];
      if (has(owner, -d - 1)) ref -= (long)dims[d] * stride[d];
    }
    number_dim(region, ref, dim - 1, pos);
  }
  void number_dim(uint64_t region, long ref, int d, unsigned &pos) {
    if (d < 0) {
      grid[ref] = pos++;
      return;
    }
    if (has(region, d + 1) || has(region, -d - 1)) {
      const long first = has(region, d + 1) ? dims[d] : g_depth[d];  // high skin / low skin
      for (unsigned i = 0; i < g_depth[d]; ++i) number_dim(region, ref + (first + i) * (long)stride[d], d - 1, pos);
    } else {
      for (unsigned i = 2 * g_depth[d]; i < dims[d]; ++i) number_dim(region, ref + (long)i * stride[d], d - 1, pos);
    }
  }
  void number_aligned(uint64_t owner, uint64_t region, unsigned &pos) {
    number(owner, region, pos);
    pos = (pos + factor - 1) / factor * factor;
  }
  // adjacency of grid position p: 3^dim entries, dimension dim-1 most significant, 0 outside
  // the grid (brick-mpi.h:262-290)
  void adjacency_of(long p, unsigned *out) const {
    const unsigned w = adj_width;
    for (unsigned s = 0; s < w; ++s) {
      long q = p;
      bool inside = true;
      unsigned rest = s;
      for (int d = 0; d < dim && inside; ++d) {
        const int o = (int)(rest % 3) - 1;
        rest /= 3;
        const long c = (p / stride[d]) % t_dims[d] + o;
        if (c < 0 || c >= (long)t_dims[d]) inside = false;
        q += (long)o * stride[d];
      }
      out[s] = inside ? grid[q] : 0u;
    }
  }

  int build() {
    const size_t gsize = [&] {
      size_t g = 1;
      stride.assign(dim, 0);
      t_dims.assign(dim, 0);
      for (int d = 0; d < dim; ++d) {
        stride[d] = (unsigned)g;
        t_dims[d] = dims[d] + 2 * g_depth[d];
        g *= t_dims[d];
      }
      return g;
    }();
    if (gsize > 0xFFFFFFFFull) return fail(BK_ERR_ARG, "decomposition grid too large");
    grid.assign(gsize, 0u);
    unsigned pos = factor;  // bricks 0 .. factor-1 stay unused (brick 0 is the "outside" entry)

    const size_t ns = skinlist.size();
    std::vector<bool> pad_first(ns);
    for (size_t l = 0; l < ns; ++l) {
      const uint64_t prev = l ? skinlist[l - 1] : 0, next = l + 1 < ns ? skinlist[l + 1] : 0;
      pad_first[l] = popcount(prev & skinlist[l]) < popcount(skinlist[l] & next);
    }
    std::vector<unsigned> st_pos;
    number_aligned(0, 0, pos);  // the inner region
    st_pos.push_back(pos);
    sep_pos[0] = pos;
    skin_size.clear();
    for (size_t l = 0; l < ns; ++l) {
      const unsigned before = pos;
      if (pad_first[l]) pos += (unsigned)pad_of(skinlist[l]);
      if (skinlist[l]) number_aligned(0, skinlist[l], pos);
      st_pos.push_back(pos);
      skin_size.push_back((long)pos - (long)before);
    }
    sep_pos[1] = pos;

    // ghost zones: for every neighbour n, the skin regions of n that face this domain (those
    // containing the opposite sides of n), in skin-list order, as maximal contiguous runs
    std::vector<uint64_t> nsets;
    neighbour_sets(0, 1, dim, nsets);
    ghost.clear();
    skin.clear();
    for (uint64_t n : nsets) {
      if (!n) continue;
      const uint64_t in = flip_sides(n);
      bk_decomp_region g{}, s{};
      g.neighbor = n;
      s.neighbor = in;
      long start = -1;
      auto close = [&](size_t end) {
        g.last_pad = s.last_pad = pad_first[end - 1] ? 0u : (unsigned)pad_of(skinlist[end - 1]);
        g.skin_ed = s.skin_ed = (unsigned)end;
        g.len = pos - g.pos;
        s.len = st_pos[end] - s.pos;
        ghost.push_back(g);
        skin.push_back(s);
        start = -1;
      };
      for (size_t l = 0; l < ns; ++l) {
        if (subset(in, skinlist[l])) {
          if (start < 0) {
            start = (long)l;
            g.skin_st = s.skin_st = (unsigned)l;
            g.first_pad = s.first_pad = pad_first[l] ? (unsigned)pad_of(skinlist[l]) : 0u;
            g.pos = pos;
            s.pos = st_pos[l];
          }
          if (pad_first[l]) pos += (unsigned)pad_of(skinlist[l]);
          number_aligned(n, skinlist[l], pos);
        } else if (start >= 0) {
          close(l);
        }
      }
      if (start >= 0) close(ns);
    }
    sep_pos[2] = pos;
    nbricks = pos;

    adj_width = 1;
    for (int d = 0; d < dim; ++d) adj_width *= 3;
    adj.assign((size_t)nbricks * adj_width, 0u);
    for (size_t p = 0; p < gsize; ++p) adjacency_of((long)p, &adj[(size_t)grid[p] * adj_width]);
    return BK_OK;
  }
};

}  // namespace bk

using namespace bk;

struct bk_decomp {
  Decomp d;
};

extern "C" {

int bk_decomp_create(int dim, const unsigned *dims, const unsigned *bdims, unsigned depth, unsigned numfield,
                     size_t elem_bytes, long pagesize, const uint64_t *skinlist, unsigned nskin, bk_decomp **out) {
  if (!out) return fail(BK_ERR_ARG, "out is NULL");
  *out = nullptr;
  if (dim < 1 || dim > 4) return fail(BK_ERR_UNSUPPORTED, "decompositions of 1 to 4 dimensions");
  if (!dims || !bdims || (nskin && !skinlist)) return fail(BK_ERR_ARG, "dims, bdims and skinlist are required");
  if (numfield < 1 || elem_bytes < 1 || pagesize < 1) return fail(BK_ERR_ARG, "numfield, elem_bytes and pagesize must be >= 1");
  Decomp D;
  D.dim = dim;
  size_t bsize = elem_bytes * numfield;
  for (int d = 0; d < dim; ++d) {
    if (!bdims[d] || depth % bdims[d] || dims[d] % bdims[d])
      return fail(BK_ERR_ARG, "the domain and the ghost depth must be whole bricks in every dimension");
    D.dims.push_back(dims[d] / bdims[d]);
    D.g_depth.push_back(depth / bdims[d]);
    if (D.dims[d] < 2 * D.g_depth[d]) return fail(BK_ERR_ARG, "the domain must be at least two ghost depths wide");
    bsize *= bdims[d];
  }
  // bricks fill whole pages (brick-mpi.h:344-352)
  const size_t page = (size_t)pagesize;
  if ((bsize > page ? bsize : page) % (bsize < page ? bsize : page))
    return fail(BK_ERR_ARG, "brick size must be a factor or a multiple of the page size");
  D.factor = bsize < page ? (unsigned)(page / bsize) : 1u;
  for (unsigned l = 0; l < nskin; ++l) {
    for (long b = 0; b < 64; ++b)
      if ((skinlist[l] >> b) & 1ull) {
        const long p = b > 31 ? 31 - b : b;
        if (p == 0 || (p > 0 && p > dim) || (p < 0 && -p > dim) || (p > 0 && has(skinlist[l], -p)))
          return fail(BK_ERR_ARG, "skin list entry names a side outside the dimensions (or both sides)");
      }
    D.skinlist.push_back(skinlist[l]);
  }
  int s = D.build();
  if (s) return s;
  bk_decomp *h = new (std::nothrow) bk_decomp;
  if (!h) return fail(BK_ERR_ARG, "out of host memory");
  h->d = std::move(D);
  *out = h;
  return BK_OK;
}

int bk_decomp_info(const bk_decomp *h, unsigned *nbricks, size_t *grid_size, unsigned *nregions, unsigned *sep_pos) {
  if (!h) return fail(BK_ERR_ARG, "decomposition is NULL");
  if (nbricks) *nbricks = h->d.nbricks;
  if (grid_size) *grid_size = h->d.grid.size();
  if (nregions) *nregions = (unsigned)h->d.ghost.size();
  if (sep_pos)
    for (int q = 0; q < 3; ++q) sep_pos[q] = h->d.sep_pos[q];
  return BK_OK;
}

int bk_decomp_grid(const bk_decomp *h, unsigned *grid) {
  if (!h || !grid) return fail(BK_ERR_ARG, "decomposition and grid are required");
  memcpy(grid, h->d.grid.data(), h->d.grid.size() * sizeof(unsigned));
  return BK_OK;
}

int bk_decomp_adjacency(const bk_decomp *h, unsigned *adj) {
  if (!h || !adj) return fail(BK_ERR_ARG, "decomposition and adj are required");
  memcpy(adj, h->d.adj.data(), h->d.adj.size() * sizeof(unsigned));
  return BK_OK;
}

int bk_decomp_regions(const bk_decomp *h, bk_decomp_region *ghost, bk_decomp_region *skin, long *skin_size) {
  if (!h) return fail(BK_ERR_ARG, "decomposition is NULL");
  if (ghost) memcpy(ghost, h->d.ghost.data(), h->d.ghost.size() * sizeof(bk_decomp_region));
  if (skin) memcpy(skin, h->d.skin.data(), h->d.skin.size() * sizeof(bk_decomp_region));
  if (skin_size) memcpy(skin_size, h->d.skin_size.data(), h->d.skin_size.size() * sizeof(long));
  return BK_OK;
}

int bk_decomp_exchange_links(const bk_decomp *h, const void *dat, size_t step_bytes, uint64_t *links) {
  if (!h || !dat || !links) return fail(BK_ERR_ARG, "decomposition, storage and links are required");
  if (step_bytes % 8) return fail(BK_ERR_ARG, "step_bytes must be a multiple of 8");
  const uint64_t base = reinterpret_cast<uint64_t>(dat);
  for (size_t i = 0; i < h->d.ghost.size(); ++i) {
    const bk_decomp_region &g = h->d.ghost[i], &s = h->d.skin[i];
    const uint64_t nb = (uint64_t)(g.len - g.first_pad - g.last_pad);
    links[3 * i] = base + (uint64_t)(s.pos + s.first_pad) * step_bytes;      // from the skin
    links[3 * i + 1] = base + (uint64_t)(g.pos + g.first_pad) * step_bytes;  // to the ghost zone
    links[3 * i + 2] = nb * step_bytes;
  }
  return BK_OK;
}

void bk_decomp_destroy(bk_decomp *h) { delete h; }

}  // extern "C"
