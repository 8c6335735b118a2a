// el_wise_op.hpp - drop-in amt::el_op running on the GB300.
//
// Same functions and argument order as the reference's
// include/el_wise_op.hpp:33-121: c[i] = a[i] op b[i] over c.size() elements
// of the tensors' storage, run at once (these functions return nothing, as
// in the reference).  The operation runs on the GPU, so the predicate of
// apply / apply_ops must be one of std::plus, std::minus, std::multiplies or
// std::divides (any specialisation); other callables are rejected at compile
// time.  Unlike the reference (whose size check is commented out, lines
// 55-60), a or b with fewer elements than c is reported with
// std::runtime_error instead of being read past its end.
#ifndef GBBLAS_AMT_EL_WISE_OP_HPP
#define GBBLAS_AMT_EL_WISE_OP_HPP

#include <boost/numeric/ublas/tensor.hpp>
#include <functional>
#include <optional>
#include <stdexcept>
#include <type_traits>

#include "gbblas.h"
#include "utils.hpp"

namespace amt::el_op {

namespace detail {

template <typename P, template <typename...> class F>
struct is_functor : std::false_type {};
template <template <typename...> class F, typename... A>
struct is_functor<F<A...>, F> : std::true_type {};

template <typename P>
constexpr gbblas_ew_op op_of() {
  using D = std::decay_t<P>;
  if constexpr (is_functor<D, std::plus>::value)
    return GBBLAS_EW_ADD;
  else if constexpr (is_functor<D, std::minus>::value)
    return GBBLAS_EW_SUB;
  else if constexpr (is_functor<D, std::multiplies>::value)
    return GBBLAS_EW_MUL;
  else {
    static_assert(is_functor<D, std::divides>::value,
                  "amt::el_op on the GPU: the predicate must be std::plus, std::minus, std::multiplies or "
                  "std::divides");
    return GBBLAS_EW_DIV;
  }
}

}  // namespace detail

template <typename Out, typename E1, typename E2, typename Predicate>
auto apply(boost::numeric::ublas::tensor_core<Out>& c, boost::numeric::ublas::tensor_core<E1> const& a,
           boost::numeric::ublas::tensor_core<E2> const& b, std::optional<std::size_t>, Predicate&&) {
  using T = typename boost::numeric::ublas::tensor_core<Out>::value_type;
  using value_type1 = typename boost::numeric::ublas::tensor_core<E1>::value_type;
  using value_type2 = typename boost::numeric::ublas::tensor_core<E2>::value_type;
  static_assert(std::is_same_v<T, value_type1> && std::is_same_v<T, value_type2>,
                "all the value types must be of same value type");
  static_assert(std::is_same_v<T, float> || std::is_same_v<T, double>,
                "amt::el_op on the GPU supports float and double");
  constexpr gbblas_ew_op op = detail::op_of<Predicate>();
  const std::size_t n = c.size();
  if (a.size() < n || b.size() < n)
    throw std::runtime_error("amt::el_op::apply(c, a, b): a and b need at least c.size() elements");
  gbblas_status s;
  if constexpr (std::is_same_v<T, float>)
    s = gbblas_sew_host(op, static_cast<int64_t>(n), a.data(), b.data(), c.data());
  else
    s = gbblas_dew_host(op, static_cast<int64_t>(n), a.data(), b.data(), c.data());
  gpu::check(s, "amt::el_op");
}

template <typename Out, typename E1, typename E2>
constexpr auto add(boost::numeric::ublas::tensor_core<Out>& c, boost::numeric::ublas::tensor_core<E1> const& a,
                   boost::numeric::ublas::tensor_core<E2> const& b, std::optional<std::size_t> num_threads) {
  apply(c, a, b, num_threads, std::plus<>{});
}

template <typename Out, typename E1, typename E2>
constexpr auto sub(boost::numeric::ublas::tensor_core<Out>& c, boost::numeric::ublas::tensor_core<E1> const& a,
                   boost::numeric::ublas::tensor_core<E2> const& b, std::optional<std::size_t> num_threads) {
  apply(c, a, b, num_threads, std::minus<>{});
}

template <typename Out, typename E1, typename E2>
constexpr auto mul(boost::numeric::ublas::tensor_core<Out>& c, boost::numeric::ublas::tensor_core<E1> const& a,
                   boost::numeric::ublas::tensor_core<E2> const& b, std::optional<std::size_t> num_threads) {
  apply(c, a, b, num_threads, std::multiplies<>{});
}

template <typename Out, typename E1, typename E2>
constexpr auto div(boost::numeric::ublas::tensor_core<Out>& c, boost::numeric::ublas::tensor_core<E1> const& a,
                   boost::numeric::ublas::tensor_core<E2> const& b, std::optional<std::size_t> num_threads) {
  apply(c, a, b, num_threads, std::divides<>{});
}

template <typename Out, typename E1, typename E2, typename Predicate>
constexpr auto apply_ops(boost::numeric::ublas::tensor_core<Out>& c, boost::numeric::ublas::tensor_core<E1> const& a,
                         boost::numeric::ublas::tensor_core<E2> const& b, std::optional<std::size_t> num_threads,
                         Predicate&& pred) {
  apply(c, a, b, num_threads, std::forward<Predicate>(pred));
}

}  // namespace amt::el_op

#endif  // GBBLAS_AMT_EL_WISE_OP_HPP
