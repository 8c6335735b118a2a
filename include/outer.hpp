// outer.hpp - drop-in amt::outer_prod running on the GB300.
//
// Same template, argument order and checks as the reference's
// include/outer.hpp:67-119: C += a b^T for vectors a (NA elements) and b (NB
// elements) into the NA x NB matrix C of either layout; the callable does
// the work.  Each element is one fused multiply-add, as the reference's inner
// loop (include/simd_loop.hpp:42-47), so results agree bit for bit.
#ifndef GBBLAS_AMT_OUTER_HPP
#define GBBLAS_AMT_OUTER_HPP

#include <boost/numeric/ublas/tensor.hpp>
#include <optional>
#include <stdexcept>
#include <type_traits>

#include "gbblas.h"
#include "utils.hpp"

namespace amt {

/// C += a b^T.  `num_threads` is accepted and ignored (the work runs on the GPU).
template <typename Out, typename E1, typename E2>
constexpr auto outer_prod(boost::numeric::ublas::tensor_core<Out>& c, boost::numeric::ublas::tensor_core<E1> const& a,
                          boost::numeric::ublas::tensor_core<E2> const& b, std::optional<std::size_t> num_threads) {
  using value_type1 = typename boost::numeric::ublas::tensor_core<E1>::value_type;
  using value_type2 = typename boost::numeric::ublas::tensor_core<E2>::value_type;
  using T = typename boost::numeric::ublas::tensor_core<Out>::value_type;
  using layout_type = typename boost::numeric::ublas::tensor_core<Out>::layout_type;
  static_assert(std::is_same_v<value_type1, value_type2> && std::is_same_v<T, value_type2>,
                "both tensor type and result type must be of same value_type");
  static_assert(std::is_same_v<T, float> || std::is_same_v<T, double>,
                "amt::outer_prod on the GPU supports float and double");
  (void)num_threads;
  auto const& na = a.extents();
  auto const& nb = b.extents();
  auto const& nc = c.extents();
  if (!(boost::numeric::ublas::is_vector(na) && boost::numeric::ublas::is_vector(nb)))
    throw std::runtime_error("amt::outer_prod(c, a, b): both tensor must be vector");
  const std::size_t NA = boost::numeric::ublas::product(na), NB = boost::numeric::ublas::product(nb);
  if (nc[0] != NA || nc[1] != NB) throw std::runtime_error("amt::outer_prod(c, a, b): dimension mismatch");
  T* cp = c.data();
  T const* ap = a.data();
  T const* bp = b.data();
  const auto M = static_cast<int64_t>(NA), N = static_cast<int64_t>(NB);
  return [cp, ap, bp, M, N] {
    constexpr gbblas_layout L = gpu::layout_of<layout_type>();
    gbblas_status s;
    if constexpr (std::is_same_v<T, float>)
      s = gbblas_souter_host(L, M, N, ap, bp, cp);
    else
      s = gbblas_douter_host(L, M, N, ap, bp, cp);
    gpu::check(s, "amt::outer_prod");
  };
}

}  // namespace amt

#endif  // GBBLAS_AMT_OUTER_HPP
