/*
 * bitset.h -- the set of signed dimension numbers that names a region or a neighbour of a
 * brick decomposition (include/bitset.h of the reference, same bit layout so that skin lists
 * written for the reference carry over): side +p (high side of dimension p-1) is bit p,
 * side -p is bit 31 + p.
 */
#ifndef BRICK_GB300_BITSET_H
#define BRICK_GB300_BITSET_H

#include <cstdint>
#include <initializer_list>

struct BitSet {
  static const long zero = 31;  ///< bit of "-0"; -p is bit zero + p

  static inline uint64_t to_set(long pos) { return 1ull << (uint64_t)(pos < 0 ? zero - pos : pos); }

  uint64_t set;

  BitSet() : set(0) {}
  BitSet(uint64_t s) : set(s) {}
  BitSet(std::initializer_list<int> l) : set(0) {
    for (int p : l) set ^= to_set(p);
  }

  inline BitSet &flip(long pos) {
    set ^= to_set(pos);
    return *this;
  }
  inline long size() const { return __builtin_popcountll(set); }
  inline bool get(long pos) const { return (set & to_set(pos)) != 0; }
  inline BitSet operator&(BitSet a) const { return set & a.set; }
  inline BitSet operator|(BitSet a) const { return set | a.set; }
  inline BitSet operator^(BitSet a) const { return set ^ a.set; }
  inline operator bool() const { return set != 0; }
  inline bool operator<=(BitSet a) const { return (set & a.set) == set; }  ///< subset
  inline bool operator>=(BitSet a) const { return (set & a.set) == a.set; }  ///< superset
  /// every side replaced by the opposite side
  inline BitSet operator!() const {
    const uint64_t mask = (1ull << (uint64_t)(zero + 1)) - 1ull;
    return BitSet(((set & mask) << (uint64_t)zero) | (set >> (uint64_t)zero));
  }
};

#endif  // BRICK_GB300_BITSET_H
