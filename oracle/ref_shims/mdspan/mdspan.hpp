// Minimal stand-in for the subset of Kokkos::mdspan (C++23 std::mdspan) that
// the reference's MACIS headers use: dynamic extents, layout_left (column
// major), element access by operator(), data_handle(), extent(r), size().
#pragma once
#include <array>
#include <cstddef>
#include <type_traits>

namespace Kokkos {

template <class IndexType, std::size_t Rank>
struct dextents {
  using index_type = IndexType;
  static constexpr std::size_t rank() { return Rank; }
};

struct layout_left {};

template <class T, class Extents, class Layout = layout_left>
class mdspan {
 public:
  static constexpr std::size_t R = Extents::rank();
  using element_type = T;
  using value_type = std::remove_cv_t<T>;
  using index_type = std::size_t;
  using size_type = std::size_t;
  using extents_type = Extents;
  using layout_type = Layout;
  using data_handle_type = T*;
  using reference = T&;

  mdspan() = default;
  template <class... I, class = std::enable_if_t<sizeof...(I) == R>>
  mdspan(T* p, I... e) : p_(p), ext_{static_cast<std::size_t>(e)...} {}
  // mdspan<T> -> mdspan<const T>
  template <class U, class = std::enable_if_t<std::is_convertible_v<U*, T*> && !std::is_same_v<U, T>>>
  mdspan(const mdspan<U, Extents, Layout>& o) : p_(o.data_handle()) {
    for (std::size_t r = 0; r < R; ++r) ext_[r] = o.extent(r);
  }

  static constexpr std::size_t rank() { return R; }
  T* data_handle() const { return p_; }
  std::size_t extent(std::size_t r) const { return ext_[r]; }
  std::size_t size() const {
    std::size_t s = 1;
    for (std::size_t r = 0; r < R; ++r) s *= ext_[r];
    return s;
  }
  std::size_t stride(std::size_t r) const {
    std::size_t s = 1;
    for (std::size_t q = 0; q < r; ++q) s *= ext_[q];
    return s;
  }
  template <class... I, class = std::enable_if_t<sizeof...(I) == R>>
  T& operator()(I... i) const {
    const std::size_t idx[R] = {static_cast<std::size_t>(i)...};
    std::size_t off = 0, s = 1;
    for (std::size_t r = 0; r < R; ++r) {
      off += idx[r] * s;
      s *= ext_[r];
    }
    return p_[off];
  }

 private:
  T* p_ = nullptr;
  std::array<std::size_t, R> ext_{};
};

}  // namespace Kokkos
