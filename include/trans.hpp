// trans.hpp - drop-in amt::transpose running on the GB300.
//
// Same templates and argument order as the reference's include/trans.hpp:
//   transpose(c, a, num_threads)  c = a^T out of place, honouring both
//                                 tensors' strides (reference lines 103-145);
//   transpose(a, num_threads)     a transposed in place (lines 147-169).
// The callable does the work.  The reference's in-place form swaps
// a[i*rows + j] with a[j*cols + i] and so is only a transpose for square
// matrices (for others it writes outside the matrix); this header accepts
// square matrices only and throws std::runtime_error otherwise.
#ifndef GBBLAS_AMT_TRANS_HPP
#define GBBLAS_AMT_TRANS_HPP

#include <boost/numeric/ublas/tensor.hpp>
#include <optional>
#include <stdexcept>
#include <type_traits>

#include "gbblas.h"
#include "utils.hpp"

namespace amt {

/// c = a^T.
template <typename Out, typename E>
constexpr auto transpose(boost::numeric::ublas::tensor_core<Out>& c, boost::numeric::ublas::tensor_core<E> const& a,
                         std::optional<std::size_t> num_threads) {
  using T = typename boost::numeric::ublas::tensor_core<Out>::value_type;
  using value_type = typename boost::numeric::ublas::tensor_core<E>::value_type;
  static_assert(std::is_same_v<T, value_type>, "input value type and result value type must be of same value type");
  static_assert(std::is_same_v<T, float> || std::is_same_v<T, double>,
                "amt::transpose on the GPU supports float and double");
  (void)num_threads;
  auto const& na = a.extents();
  auto const& nc = c.extents();
  if (!(boost::numeric::ublas::is_matrix(na) && boost::numeric::ublas::is_matrix(nc)))
    throw std::runtime_error("amt::transpose(c, a): a and c must be the matrices");
  if (!((na[0] == nc[1]) && (na[1] == nc[0]))) throw std::runtime_error("amt::transpose(c, a): dimension mismatch");
  T* cp = c.data();
  T const* ap = a.data();
  const auto M = static_cast<int64_t>(na[0]), N = static_cast<int64_t>(na[1]);
  const auto rsa = static_cast<int64_t>(a.strides()[0]), csa = static_cast<int64_t>(a.strides()[1]);
  const auto rsc = static_cast<int64_t>(c.strides()[0]), csc = static_cast<int64_t>(c.strides()[1]);
  return [cp, ap, M, N, rsa, csa, rsc, csc] {
    gbblas_status s;
    if constexpr (std::is_same_v<T, float>)
      s = gbblas_stranspose_host(M, N, ap, rsa, csa, cp, rsc, csc);
    else
      s = gbblas_dtranspose_host(M, N, ap, rsa, csa, cp, rsc, csc);
    gpu::check(s, "amt::transpose");
  };
}

/// a = a^T in place (square matrices).
template <typename E>
constexpr auto transpose(boost::numeric::ublas::tensor_core<E>& a, std::optional<std::size_t> num_threads) {
  using T = typename boost::numeric::ublas::tensor_core<E>::value_type;
  static_assert(std::is_same_v<T, float> || std::is_same_v<T, double>,
                "amt::transpose on the GPU supports float and double");
  (void)num_threads;
  auto const& na = a.extents();
  if (!boost::numeric::ublas::is_matrix(na)) throw std::runtime_error("amt::transpose(a): a must be a matrix");
  if (na[0] != na[1])
    throw std::runtime_error("amt::transpose(a): in-place transpose needs a square matrix");
  T* ap = a.data();
  const auto n = static_cast<int64_t>(na[0]);
  return [ap, n] {
    gbblas_status s;
    if constexpr (std::is_same_v<T, float>)
      s = gbblas_stranspose_inplace_host(n, ap);
    else
      s = gbblas_dtranspose_inplace_host(n, ap);
    gpu::check(s, "amt::transpose");
  };
}

}  // namespace amt

#endif  // GBBLAS_AMT_TRANS_HPP
