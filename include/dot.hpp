// dot.hpp - drop-in amt::dot_prod / amt::dot_prod_tuning_param on the GB300.
//
// Same templates and argument order as the reference's include/dot.hpp
// (dot_prod 176-224, dot_prod_tuning_param 92-141): validation at call time
// (std::runtime_error for non-vectors or unequal sizes), the callable
// captures `c` by reference and assigns the result to it.  The CPU block
// sizes of dot_prod_tuning_param have no meaning on the GPU; they must be
// non-zero and otherwise do not change the result.
#ifndef GBBLAS_AMT_DOT_HPP
#define GBBLAS_AMT_DOT_HPP

#include <boost/numeric/ublas/tensor.hpp>
#include <optional>
#include <stdexcept>
#include <type_traits>

#include "gbblas.h"
#include "utils.hpp"

namespace amt {

namespace gpu::detail {

template <typename Out, typename E1, typename E2>
constexpr std::size_t dot_checks(boost::numeric::ublas::tensor_core<E1> const& a,
                                 boost::numeric::ublas::tensor_core<E2> const& b) {
  using V1 = typename boost::numeric::ublas::tensor_core<E1>::value_type;
  using V2 = typename boost::numeric::ublas::tensor_core<E2>::value_type;
  static_assert(std::is_same_v<V1, V2> && std::is_same_v<Out, V2>,
                "both tensor type and result type must be of same value_type");
  static_assert(std::is_same_v<Out, float> || std::is_same_v<Out, double>,
                "amt::dot_prod on the GPU supports float and double");
  if (!(boost::numeric::ublas::is_vector(a.extents()) && boost::numeric::ublas::is_vector(b.extents())))
    throw std::runtime_error("amt::dot_prod(a, b): both tensors must be vectors");
  const std::size_t na = boost::numeric::ublas::product(a.extents());
  if (na != boost::numeric::ublas::product(b.extents()))
    throw std::runtime_error("amt::dot_prod(a, b): both vectors must be of the same size");
  return na;
}

template <typename Out>
inline void dot_run(Out& c, Out const* a, Out const* b, std::size_t n) {
  gbblas_status s;
  if constexpr (std::is_same_v<Out, float>)
    s = gbblas_sdot_host(static_cast<int64_t>(n), a, b, &c);
  else
    s = gbblas_ddot_host(static_cast<int64_t>(n), a, b, &c);
  check(s, "amt::dot_prod");
}

}  // namespace gpu::detail

template <typename Out, typename E1, typename E2>
constexpr auto dot_prod(Out& c, boost::numeric::ublas::tensor_core<E1> const& a,
                        boost::numeric::ublas::tensor_core<E2> const& b,
                        std::optional<std::size_t> num_threads = std::nullopt) {
  (void)num_threads;
  const std::size_t n = gpu::detail::dot_checks<Out, E1, E2>(a, b);
  Out const* ap = a.data();
  Out const* bp = b.data();
  return [&c, ap, bp, n] { gpu::detail::dot_run<Out>(c, ap, bp, n); };
}

template <typename Out, typename E1, typename E2>
constexpr auto dot_prod_tuning_param(Out& c, boost::numeric::ublas::tensor_core<E1> const& a,
                                     boost::numeric::ublas::tensor_core<E2> const& b, std::size_t const b1,
                                     std::size_t const b2, std::size_t const b3,
                                     std::optional<std::size_t> num_threads) {
  (void)num_threads;
  const std::size_t n = gpu::detail::dot_checks<Out, E1, E2>(a, b);
  if (b1 == 0 || b2 == 0 || b3 == 0)
    throw std::runtime_error("amt::dot_prod_tuning_param: block sizes must be non-zero");
  Out const* ap = a.data();
  Out const* bp = b.data();
  return [&c, ap, bp, n] { gpu::detail::dot_run<Out>(c, ap, bp, n); };
}

}  // namespace amt

#endif  // GBBLAS_AMT_DOT_HPP
