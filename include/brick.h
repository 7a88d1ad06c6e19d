/*
 * brick.h -- source-compatible brick data structures for the GB300 engine.
 *
 * Same names, members and semantics as the reference's include/brick.h so that code
 * written against bricklib compiles unchanged: BrickStorage (brick.h:53-82),
 * BrickInfo<dims> (:96-127), Dim<...>, Brick<Dim<BDims...>, Dim<Folds...>> with
 * VECLEN, BRICKSIZE, operator[] element access and neighbor<...>() (:353-395).
 *
 * The element accessor is written afresh: bIn[b][k][j][i] records one index per
 * dimension and the last [] resolves them at once -- for each axis the neighbour
 * direction q = floor(x / D) in {-1, 0, 1} and the in-brick coordinate x - q*D; the
 * adjacency slot sum((q_d+1) * 3^(dims-1-d)); and the folded in-brick offset
 *   vector = row-major index of (x_d / F_d), lane = row-major index of (x_d % F_d),
 *   offset = vector * VECLEN + lane,
 * where folds are right-aligned to the brick dims (Dim<4,8> on Dim<8,8,8> folds j by 4
 * and i by 8).  This is the layout of the reference accessor (brick.h:213-327).
 * Indices may reach one brick beyond each face, as in the reference.
 *
 * Host code only needs this header; the GPU sweep is reached through
 * bricklib_gb300.h / brick-gb300.h.
 */
#ifndef BRICK_H
#define BRICK_H

#include <stdlib.h>

#include <memory>
#include <type_traits>

#ifndef bElem
#define bElem double
#endif

/// BrickStorage allocation alignment (bytes)
#define ALIGN 2048

#if defined(__CUDACC__)
#define FORCUDA __host__ __device__
#else
#define FORCUDA
#endif

/// base^exp at compile time
template <unsigned base, unsigned exp>
struct static_power {
  static constexpr unsigned value = base * static_power<base, exp - 1>::value;
};
template <unsigned base>
struct static_power<base, 0> {
  static constexpr unsigned value = 1;
};

/// Product of a list of numbers at compile time
template <unsigned... xs>
struct cal_size {
  static constexpr unsigned value = 1;
};
template <unsigned x, unsigned... xs>
struct cal_size<x, xs...> {
  static constexpr unsigned value = x * cal_size<xs...>::value;
};

/// Storage of bricks: `chunks` chunks of `step` elements.
struct BrickStorage {
  std::shared_ptr<bElem> dat;
  long chunks = 0;
  size_t step = 0;
  void *mmap_info = nullptr;

  static BrickStorage allocate(long chunks, size_t step) {
    BrickStorage b;
    b.chunks = chunks;
    b.step = step;
    size_t bytes = (size_t)chunks * step * sizeof(bElem);
    bytes = (bytes + ALIGN - 1) / ALIGN * ALIGN;
    b.dat = std::shared_ptr<bElem>((bElem *)aligned_alloc(ALIGN, bytes), [](bElem *p) { free(p); });
    return b;
  }
};

/// Adjacency list of bricks: adj[b][3^dims], centre slot 3^dims / 2.
template <unsigned dims>
struct BrickInfo {
  typedef unsigned (*adjlist)[static_power<3, dims>::value];
  adjlist adj;
  unsigned nbricks;

  explicit BrickInfo(unsigned nbricks) : nbricks(nbricks) {
    adj = (adjlist)malloc((size_t)nbricks * static_power<3, dims>::value * sizeof(unsigned));
  }

  BrickStorage allocate(long step) { return BrickStorage::allocate(nbricks, step); }
};

template <unsigned... Ds>
struct Dim {};

namespace brick_detail {

template <unsigned... Ds>
struct ulist {
  static constexpr unsigned n = sizeof...(Ds);
  FORCUDA static constexpr unsigned get(unsigned i) {
    const unsigned v[sizeof...(Ds) + 1] = {Ds..., 0u};
    return v[i];
  }
};

// fold of axis d (0 = outermost) with folds right-aligned to the brick dims
template <typename BD, typename FD>
FORCUDA constexpr unsigned fold_of(unsigned d) {
  return d + FD::n >= BD::n ? FD::get(d + FD::n - BD::n) : 1u;
}

}  // namespace brick_detail

template <typename...>
struct Brick;

template <typename BrickT, unsigned Level>
struct BrickRef;

template <unsigned... BDims, unsigned... Folds>
struct Brick<Dim<BDims...>, Dim<Folds...>> {
  typedef Brick<Dim<BDims...>, Dim<Folds...>> mytype;
  typedef BrickInfo<sizeof...(BDims)> myBrickInfo;
  typedef brick_detail::ulist<BDims...> BD;
  typedef brick_detail::ulist<Folds...> FD;

  static constexpr unsigned DIMS = sizeof...(BDims);
  static constexpr unsigned VECLEN = cal_size<Folds...>::value;
  static constexpr unsigned BRICKSIZE = cal_size<BDims...>::value;

  myBrickInfo *bInfo;
  size_t step;
  bElem *dat;
  BrickStorage bStorage;

  Brick(myBrickInfo *bInfo, const BrickStorage &brickStorage, unsigned offset) : bInfo(bInfo) {
    bStorage = brickStorage;
    dat = bStorage.dat.get() + offset;
    step = (unsigned)bStorage.step;
  }

  /// Storage address of element x[0..DIMS) (outermost first) of brick b.
  FORCUDA inline bElem &at(unsigned b, const int *x) {
    unsigned slot = 0, vec = 0, lane = 0;
    for (unsigned d = 0; d < DIMS; ++d) {
      const int D = (int)BD::get(d);
      const int q = x[d] < 0 ? -1 : (x[d] >= D ? 1 : 0);
      const unsigned l = (unsigned)(x[d] - q * D);
      const unsigned F = brick_detail::fold_of<BD, FD>(d);
      slot = slot * 3 + (unsigned)(q + 1);
      vec = vec * (D / F) + l / F;
      lane = lane * F + l % F;
    }
    return dat[(size_t)bInfo->adj[b][slot] * step + vec * VECLEN + lane];
  }

  FORCUDA inline BrickRef<mytype, 1> operator[](unsigned b);

  /// Pointer to the start of the neighbour brick at offsets (0/1/2 per axis, 1 = same).
  template <unsigned... Offsets>
  FORCUDA inline bElem *neighbor(unsigned b) {
    static_assert(sizeof...(Offsets) == DIMS, "one offset per dimension");
    const unsigned o[] = {Offsets...};
    unsigned slot = 0;
    for (unsigned d = 0; d < DIMS; ++d) slot = slot * 3 + o[d];
    return &dat[(size_t)bInfo->adj[b][slot] * step];
  }
};

/// Partially indexed brick: Level indices given so far (the brick index counts as the first).
template <typename BrickT, unsigned Level>
struct BrickRef {
  BrickT *par;
  unsigned b;
  int x[BrickT::DIMS];

  FORCUDA inline typename std::conditional<Level == BrickT::DIMS, bElem &, BrickRef<BrickT, Level + 1>>::type
  operator[](int i) {
    return index(i, std::integral_constant<bool, Level == BrickT::DIMS>());
  }

 private:
  FORCUDA inline bElem &index(int i, std::true_type) {
    x[Level - 1] = i;
    return par->at(b, x);
  }
  FORCUDA inline BrickRef<BrickT, Level + 1> index(int i, std::false_type) {
    BrickRef<BrickT, Level + 1> r;
    r.par = par;
    r.b = b;
    for (unsigned d = 0; d + 1 < Level; ++d) r.x[d] = x[d];
    r.x[Level - 1] = i;
    return r;
  }
};

template <unsigned... BDims, unsigned... Folds>
FORCUDA inline BrickRef<Brick<Dim<BDims...>, Dim<Folds...>>, 1> Brick<Dim<BDims...>, Dim<Folds...>>::operator[](
    unsigned b) {
  BrickRef<mytype, 1> r;
  r.par = this;
  r.b = b;
  return r;
}

#endif  // BRICK_H
