// Minimal, project-written subset of the Boost.uBLAS *tensor* extension API.
//
// The reference library (OpenMP-BLAS) takes its operands as
// boost::numeric::ublas::tensor_core<Engine> objects.  Boost is not a
// dependency of this project, so this header provides just the surface the
// reference's hot-path headers and tests touch, with the same names and
// meaning:
//   * layout::first_order (column-major: strides {1, M}) and
//     layout::last_order (row-major: strides {N, 1})
//       (reference test/test.mtv.cpp:49-50 and 100-101 build BLIS strides
//        this way);
//   * extents<N>           - fixed-rank shape with operator[] / data();
//   * tensor_core<Engine>  - dense owning tensor: extents(), strides(),
//                            data(), begin()/end(), size(), size(i),
//                            operator[], value_type, layout_type;
//   * tensor_static_rank<T, N, L> = tensor_core over std::vector<T>
//       (used by reference include/utils.hpp:18-19);
//   * is_matrix / is_vector / is_scalar / product on extents;
//   * the `integral` concept (reference include/utils.hpp:22).
//
// When a real Boost.uBLAS tensor installation is on the include path ahead
// of this directory, it is used instead; nothing here is specific to CUDA.
#ifndef GBBLAS_COMPAT_UBLAS_TENSOR_HPP
#define GBBLAS_COMPAT_UBLAS_TENSOR_HPP

#include <algorithm>
#include <array>
#include <concepts>
#include <cstddef>
#include <functional>
#include <initializer_list>
#include <numeric>
#include <stdexcept>
#include <type_traits>
#include <vector>

namespace boost::numeric::ublas {

template <class T>
concept integral = std::is_integral_v<T>;

namespace layout {
/// Column-major: the first index varies fastest.
struct first_order {};
/// Row-major: the last index varies fastest.
struct last_order {};
}  // namespace layout

/// Fixed-rank extents.  Rank 2 is all the BLAS paths use.
template <std::size_t N>
class extents {
 public:
  using value_type = std::size_t;
  using base_type = std::array<std::size_t, N>;
  using const_iterator = typename base_type::const_iterator;

  constexpr extents() noexcept : m_{} {}
  constexpr extents(std::initializer_list<std::size_t> l) : m_{} {
    if (l.size() != N) throw std::length_error("extents: wrong number of dimensions");
    std::copy(l.begin(), l.end(), m_.begin());
  }
  template <integral... Is>
    requires(sizeof...(Is) == N && N != 1)
  constexpr explicit extents(Is... is) noexcept : m_{static_cast<std::size_t>(is)...} {}

  constexpr std::size_t operator[](std::size_t i) const noexcept { return m_[i]; }
  constexpr std::size_t& operator[](std::size_t i) noexcept { return m_[i]; }
  constexpr std::size_t at(std::size_t i) const { return m_.at(i); }
  constexpr std::size_t const* data() const noexcept { return m_.data(); }
  static constexpr std::size_t size() noexcept { return N; }
  constexpr const_iterator begin() const noexcept { return m_.begin(); }
  constexpr const_iterator end() const noexcept { return m_.end(); }
  constexpr bool empty() const noexcept { return N == 0; }
  constexpr base_type const& base() const noexcept { return m_; }

  friend constexpr bool operator==(extents const& a, extents const& b) noexcept { return a.m_ == b.m_; }

 private:
  base_type m_;
};

/// Number of elements the extents describe.
template <std::size_t N>
constexpr std::size_t product(extents<N> const& e) noexcept {
  std::size_t p = N == 0 ? 0 : 1;
  for (std::size_t i = 0; i < N; ++i) p *= e[i];
  return p;
}

template <std::size_t N>
constexpr std::size_t size(extents<N> const&) noexcept {
  return N;
}

/// Every extent is 1.
template <std::size_t N>
constexpr bool is_scalar(extents<N> const& e) noexcept {
  if (N == 0) return false;
  for (std::size_t i = 0; i < N; ++i)
    if (e[i] != 1) return false;
  return true;
}

/// A vector: exactly one of the first two extents is larger than 1, the other
/// and all further extents are 1 (so (1,n) and (n,1) with n > 1).
template <std::size_t N>
constexpr bool is_vector(extents<N> const& e) noexcept {
  if constexpr (N == 0) {
    return false;
  } else if constexpr (N == 1) {
    return e[0] > 1;
  } else {
    for (std::size_t i = 2; i < N; ++i)
      if (e[i] != 1) return false;
    return (e[0] > 1 && e[1] == 1) || (e[0] == 1 && e[1] > 1);
  }
}

/// A matrix: the first two extents are both larger than 1, the rest are 1.
template <std::size_t N>
constexpr bool is_matrix(extents<N> const& e) noexcept {
  if constexpr (N < 2) {
    return false;
  } else {
    for (std::size_t i = 2; i < N; ++i)
      if (e[i] != 1) return false;
    return e[0] > 1 && e[1] > 1;
  }
}

/// Dense strides of `e` under `Layout`.
template <class Layout, std::size_t N>
constexpr std::array<std::size_t, N> to_strides(extents<N> const& e) noexcept {
  std::array<std::size_t, N> w{};
  if constexpr (N == 0) {
    return w;
  } else if constexpr (std::is_same_v<Layout, layout::first_order>) {
    w[0] = 1;
    for (std::size_t i = 1; i < N; ++i) w[i] = w[i - 1] * e[i - 1];
  } else {
    w[N - 1] = 1;
    for (std::size_t i = N - 1; i > 0; --i) w[i - 1] = w[i] * e[i];
  }
  return w;
}

/// Strides object with the array-like interface the reference uses
/// (operator[], data(), begin(), end()).
template <std::size_t N>
class strides {
 public:
  using value_type = std::size_t;
  constexpr strides() noexcept : w_{} {}
  constexpr explicit strides(std::array<std::size_t, N> const& w) noexcept : w_(w) {}
  constexpr std::size_t operator[](std::size_t i) const noexcept { return w_[i]; }
  constexpr std::size_t const* data() const noexcept { return w_.data(); }
  static constexpr std::size_t size() noexcept { return N; }
  constexpr auto begin() const noexcept { return w_.begin(); }
  constexpr auto end() const noexcept { return w_.end(); }

 private:
  std::array<std::size_t, N> w_;
};

template <class ExtentsType, class LayoutType, class ContainerType>
struct tensor_engine {
  using extents_type = ExtentsType;
  using layout_type = LayoutType;
  using container_type = ContainerType;
};

template <class Engine>
class tensor_core;

/// Dense owning tensor over a contiguous container.
template <std::size_t N, class L, class Container>
class tensor_core<tensor_engine<extents<N>, L, Container>> {
 public:
  using engine_type = tensor_engine<::boost::numeric::ublas::extents<N>, L, Container>;
  using container_type = Container;
  using value_type = typename Container::value_type;
  using layout_type = L;
  using extents_type = ::boost::numeric::ublas::extents<N>;
  using strides_type = ::boost::numeric::ublas::strides<N>;
  using size_type = std::size_t;
  using reference = value_type&;
  using const_reference = value_type const&;
  using pointer = value_type*;
  using const_pointer = value_type const*;
  using iterator = typename Container::iterator;
  using const_iterator = typename Container::const_iterator;

  tensor_core() = default;

  explicit tensor_core(extents_type const& e)
      : e_(e), w_(to_strides<L>(e)), data_(product(e)) {}

  tensor_core(extents_type const& e, value_type const& v)
      : e_(e), w_(to_strides<L>(e)), data_(product(e), v) {}

  template <integral... Is>
    requires(sizeof...(Is) == N && N != 1)
  explicit tensor_core(Is... is) : tensor_core(extents_type(is...)) {}

  extents_type const& extents() const noexcept { return e_; }
  strides_type const& strides() const noexcept { return w_; }

  pointer data() noexcept { return data_.data(); }
  const_pointer data() const noexcept { return data_.data(); }

  size_type size() const noexcept { return data_.size(); }
  size_type size(size_type r) const { return e_.at(r); }
  static constexpr size_type rank() noexcept { return N; }
  bool empty() const noexcept { return data_.empty(); }

  reference operator[](size_type i) { return data_[i]; }
  const_reference operator[](size_type i) const { return data_[i]; }

  template <integral... Is>
    requires(sizeof...(Is) == N)
  reference operator()(Is... is) {
    std::size_t idx[] = {static_cast<std::size_t>(is)...};
    std::size_t off = 0;
    for (std::size_t k = 0; k < N; ++k) off += idx[k] * w_[k];
    return data_[off];
  }
  template <integral... Is>
    requires(sizeof...(Is) == N)
  const_reference operator()(Is... is) const {
    std::size_t idx[] = {static_cast<std::size_t>(is)...};
    std::size_t off = 0;
    for (std::size_t k = 0; k < N; ++k) off += idx[k] * w_[k];
    return data_[off];
  }

  iterator begin() noexcept { return data_.begin(); }
  iterator end() noexcept { return data_.end(); }
  const_iterator begin() const noexcept { return data_.begin(); }
  const_iterator end() const noexcept { return data_.end(); }
  const_iterator cbegin() const noexcept { return data_.cbegin(); }
  const_iterator cend() const noexcept { return data_.cend(); }

  container_type& base() noexcept { return data_; }
  container_type const& base() const noexcept { return data_; }

 private:
  extents_type e_{};
  strides_type w_{};
  container_type data_{};
};

template <class T, std::size_t N, class L = layout::first_order>
using tensor_static_rank = tensor_core<tensor_engine<extents<N>, L, std::vector<T>>>;

}  // namespace boost::numeric::ublas

#endif  // GBBLAS_COMPAT_UBLAS_TENSOR_HPP
