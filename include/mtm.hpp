// mtm.hpp - drop-in amt::mtm running on the GB300.
//
// Same template, argument order and behaviour as the reference's
// include/mtm.hpp:208-267: validate at call time (std::runtime_error for
// non-matrices or mismatched extents, static_assert for mixed value types),
// return a nullary callable, and ACCUMULATE C += A * B when it is invoked.
// Any mix of first_order / last_order operands and any strides are accepted.
// The callable stages the host buffers through the GPU
// (gbblas_?gemm_host) and returns once C holds the result; num_threads is
// accepted for source compatibility and ignored (the GPU schedules itself).
#ifndef GBBLAS_AMT_MTM_HPP
#define GBBLAS_AMT_MTM_HPP

#include <boost/numeric/ublas/tensor.hpp>
#include <optional>
#include <stdexcept>
#include <type_traits>

#include "gbblas.h"
#include "utils.hpp"

namespace amt {

/// C += A * B.  An optional fifth argument picks the arithmetic
/// (amt::gpu::accuracy): for float the default is fp32 FMA, the
/// reference's; for double the default is the library's (tensor-core digits
/// kept within the FP64 error bound where faster), fp64 forces FP64 FMAs.
template <typename Out, typename E1, typename E2>
constexpr auto mtm(boost::numeric::ublas::tensor_core<Out>& c, boost::numeric::ublas::tensor_core<E1> const& a,
                   boost::numeric::ublas::tensor_core<E2> const& b, std::optional<std::size_t> num_threads,
                   gpu::accuracy acc = gpu::accuracy::fp32) {
  using value_type1 = typename boost::numeric::ublas::tensor_core<E1>::value_type;
  using value_type2 = typename boost::numeric::ublas::tensor_core<E2>::value_type;
  using out_value_type = typename boost::numeric::ublas::tensor_core<Out>::value_type;
  static_assert(std::is_same_v<value_type1, value_type2> && std::is_same_v<out_value_type, value_type2>,
                "both tensor type and result type must be of same value_type");
  static_assert(std::is_same_v<out_value_type, float> || std::is_same_v<out_value_type, double>,
                "amt::mtm on the GPU supports float and double");
  (void)num_threads;

  auto const& na = a.extents();
  auto const& nb = b.extents();
  auto const& nc = c.extents();
  if (!(boost::numeric::ublas::is_matrix(na) && boost::numeric::ublas::is_matrix(nb) &&
        boost::numeric::ublas::is_matrix(nc)))
    throw std::runtime_error("amt::mtm(c, a, b): a, b and c must be matrices");
  if (!(na[0] == nc[0] && na[1] == nb[0] && nc[1] == nb[1]))
    throw std::runtime_error("amt::mtm(c, a, b): dimension mismatch");

  auto* cp = c.data();
  auto const* ap = a.data();
  auto const* bp = b.data();
  auto const* wc = c.strides().data();
  auto const* wa = a.strides().data();
  auto const* wb = b.strides().data();
  auto const* nap = na.data();
  auto const* nbp = nb.data();
  return [cp, ap, bp, wc, wa, wb, nap, nbp, acc] {
    const auto M = static_cast<int64_t>(nap[0]), K = static_cast<int64_t>(nap[1]),
               N = static_cast<int64_t>(nbp[1]);
    gbblas_status s;
    if constexpr (std::is_same_v<out_value_type, float>)
      s = gbblas_sgemm_host(M, N, K, ap, (int64_t)wa[0], (int64_t)wa[1], bp, (int64_t)wb[0], (int64_t)wb[1], cp,
                            (int64_t)wc[0], (int64_t)wc[1], static_cast<gbblas_accuracy>(acc));
    else if (acc == gpu::accuracy::fp32)
      s = gbblas_dgemm_host(M, N, K, ap, (int64_t)wa[0], (int64_t)wa[1], bp, (int64_t)wb[0], (int64_t)wb[1], cp,
                            (int64_t)wc[0], (int64_t)wc[1]);
    else
      s = gbblas_dgemm_ex_host(M, N, K, ap, (int64_t)wa[0], (int64_t)wa[1], bp, (int64_t)wb[0], (int64_t)wb[1], cp,
                               (int64_t)wc[0], (int64_t)wc[1], static_cast<gbblas_accuracy>(acc));
    gpu::check(s, "amt::mtm");
  };
}

}  // namespace amt

#endif  // GBBLAS_AMT_MTM_HPP
