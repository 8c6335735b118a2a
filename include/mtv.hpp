// mtv.hpp - drop-in amt::mtv / amt::vtm running on the GB300.
//
// Same templates and argument order as the reference's include/mtv.hpp
// (mtv 100-162, vtm 164-236).  Validation happens at call time
// (std::runtime_error), the callable does the work.  Like the reference,
// A's strides are taken from its layout (A must be dense), and
//   mtv: column-major A ACCUMULATES y += A x, row-major A OVERWRITES y = A x;
//   vtm: y = v^T A; column-major A overwrites y, row-major A accumulates.
// Unlike the reference, vtm is correct for every shape and layout (the
// reference builds A^T's strides from the wrong extent, lines 224-227, and is
// right only for square column-major A).
#ifndef GBBLAS_AMT_MTV_HPP
#define GBBLAS_AMT_MTV_HPP

#include <boost/numeric/ublas/tensor.hpp>
#include <optional>
#include <stdexcept>
#include <type_traits>

#include "gbblas.h"
#include "utils.hpp"

namespace amt {

namespace gpu::detail {

template <typename Out, typename E1, typename E2>
constexpr void mv_static_checks() {
  using value_type1 = typename boost::numeric::ublas::tensor_core<E1>::value_type;
  using value_type2 = typename boost::numeric::ublas::tensor_core<E2>::value_type;
  using out_value_type = typename boost::numeric::ublas::tensor_core<Out>::value_type;
  static_assert(std::is_same_v<value_type1, value_type2> && std::is_same_v<out_value_type, value_type2>,
                "both tensor type and result type must be of same value_type");
  static_assert(std::is_same_v<out_value_type, float> || std::is_same_v<out_value_type, double>,
                "amt::mtv / amt::vtm on the GPU support float and double");
}

}  // namespace gpu::detail

/// y = A x (see the header comment for overwrite/accumulate).
template <typename Out, typename E1, typename E2>
constexpr auto mtv(boost::numeric::ublas::tensor_core<Out>& c, boost::numeric::ublas::tensor_core<E1> const& a,
                   boost::numeric::ublas::tensor_core<E2> const& b, std::optional<std::size_t> num_threads) {
  gpu::detail::mv_static_checks<Out, E1, E2>();
  using layout_type = typename boost::numeric::ublas::tensor_core<E1>::layout_type;
  using T = typename boost::numeric::ublas::tensor_core<Out>::value_type;
  (void)num_threads;
  auto const& na = a.extents();
  auto const& nb = b.extents();
  auto const& nc = c.extents();
  if (!(boost::numeric::ublas::is_matrix(na) && boost::numeric::ublas::is_vector(nb) &&
        boost::numeric::ublas::is_vector(nc)))
    throw std::runtime_error("amt::mtv(c, a, b): c and b must be vectors, and a must be a matrix");
  if (na[1] != boost::numeric::ublas::product(nb) || na[0] != boost::numeric::ublas::product(nc))
    throw std::runtime_error("amt::mtv(c, a, b): dimension mismatch");
  const auto M = static_cast<int64_t>(na[0]), N = static_cast<int64_t>(na[1]);
  T* yp = c.data();
  T const* ap = a.data();
  T const* xp = b.data();
  return [yp, ap, xp, M, N] {
    constexpr gbblas_layout L = gpu::layout_of<layout_type>();
    gbblas_status s;
    if constexpr (std::is_same_v<T, float>)
      s = gbblas_smtv_host(L, M, N, ap, xp, yp);
    else
      s = gbblas_dmtv_host(L, M, N, ap, xp, yp);
    gpu::check(s, "amt::mtv");
  };
}

/// y = v^T A.
template <typename Out, typename E1, typename E2>
constexpr auto vtm(boost::numeric::ublas::tensor_core<Out>& c, boost::numeric::ublas::tensor_core<E1> const& a,
                   boost::numeric::ublas::tensor_core<E2> const& b, std::optional<std::size_t> num_threads) {
  gpu::detail::mv_static_checks<Out, E1, E2>();
  using layout_type = typename boost::numeric::ublas::tensor_core<E1>::layout_type;
  using T = typename boost::numeric::ublas::tensor_core<Out>::value_type;
  (void)num_threads;
  auto const& na = a.extents();
  auto const& nb = b.extents();
  auto const& nc = c.extents();
  if (!(boost::numeric::ublas::is_matrix(na) && boost::numeric::ublas::is_vector(nb) &&
        boost::numeric::ublas::is_vector(nc)))
    throw std::runtime_error("amt::vtm(c, a, b): c and b must be vectors, and a must be a matrix");
  if (na[1] != boost::numeric::ublas::product(nc) || na[0] != boost::numeric::ublas::product(nb))
    throw std::runtime_error("amt::vtm(c, a, b): dimension mismatch");
  const auto M = static_cast<int64_t>(na[0]), N = static_cast<int64_t>(na[1]);
  T* yp = c.data();
  T const* ap = a.data();
  T const* vp = b.data();
  return [yp, ap, vp, M, N] {
    constexpr gbblas_layout L = gpu::layout_of<layout_type>();
    gbblas_status s;
    if constexpr (std::is_same_v<T, float>)
      s = gbblas_svtm_host(L, M, N, ap, vp, yp);
    else
      s = gbblas_dvtm_host(L, M, N, ap, vp, yp);
    gpu::check(s, "amt::vtm");
  };
}

}  // namespace amt

#endif  // GBBLAS_AMT_MTV_HPP
