// ttg::MultiIndex<N> — the keys of the potrf flowgraph (Key1/Key2/Key3 of examples/potrf/pmw.h:14-16),
// with the interface of ttg/util/multiindex.h:12-60: construction from integers, operator[],
// equality, hashing and printing.
#pragma once
#include <array>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <initializer_list>
#include <ostream>

namespace ttg {

template <std::size_t Rank, typename Int = int>
struct MultiIndex {
  static constexpr std::size_t max_index = 1u << 21;  // the reference's key-space bound
  std::array<Int, Rank> idx{};

  MultiIndex() = default;
  template <typename... Ints, typename = std::enable_if_t<(sizeof...(Ints) == Rank) &&
                                                          (std::is_integral_v<std::decay_t<Ints>> && ...)>>
  MultiIndex(Ints... ints) : idx{static_cast<Int>(ints)...} {}
  MultiIndex(std::initializer_list<Int> il) {
    std::size_t i = 0;
    for (auto v : il) {
      if (i < Rank) idx[i++] = v;
    }
  }
  Int& operator[](std::size_t i) { return idx[i]; }
  const Int& operator[](std::size_t i) const { return idx[i]; }
  static constexpr std::size_t size() { return Rank; }
  bool operator==(const MultiIndex& o) const { return idx == o.idx; }
  bool operator!=(const MultiIndex& o) const { return idx != o.idx; }
  bool operator<(const MultiIndex& o) const { return idx < o.idx; }
  std::size_t hash() const {
    std::uint64_t h = 1469598103934665603ull;
    for (auto v : idx) {
      h ^= static_cast<std::uint64_t>(static_cast<std::int64_t>(v));
      h *= 1099511628211ull;
    }
    return static_cast<std::size_t>(h);
  }
  friend std::ostream& operator<<(std::ostream& o, const MultiIndex& k) {
    o << "{";
    for (std::size_t i = 0; i < Rank; ++i) o << (i ? ", " : "") << k.idx[i];
    return o << "}";
  }
  template <typename Archive>
  void serialize(Archive& ar) {
    for (auto& v : idx) ar& v;
  }
};

}  // namespace ttg

namespace std {
template <std::size_t R, typename I>
struct hash<ttg::MultiIndex<R, I>> {
  std::size_t operator()(const ttg::MultiIndex<R, I>& k) const { return k.hash(); }
};
}  // namespace std
