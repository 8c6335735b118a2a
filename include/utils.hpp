// utils.hpp - the helpers reference callers reach through the hot-path
// headers (reference include/utils.hpp): make_tensor, the layout traits,
// tag types, nearest_mul_of_x and the panel packers.  Host-side utilities;
// the compute path is in mtm.hpp / mtv.hpp / dot.hpp, which call the GPU.
#ifndef GBBLAS_AMT_UTILS_HPP
#define GBBLAS_AMT_UTILS_HPP

#include <algorithm>
#include <boost/numeric/ublas/tensor.hpp>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "gbblas.h"

namespace amt {

namespace ub = boost::numeric::ublas;
using shape_t = ub::extents<2u>;

template <typename T, typename L>
using tensor_t = ub::tensor_static_rank<T, 2, L>;

/// M x N tensor of layout L, value-initialised (reference include/utils.hpp:21-31).
template <typename T, typename L = ub::layout::first_order>
auto make_tensor(ub::integral auto M, ub::integral auto N) {
  return tensor_t<T, L>(static_cast<std::size_t>(M), static_cast<std::size_t>(N));
}

/// M x N tensor of layout L with every element set to `val`.
template <typename T, typename L = ub::layout::first_order>
auto make_tensor(ub::integral auto M, ub::integral auto N, T val) {
  auto t = tensor_t<T, L>(static_cast<std::size_t>(M), static_cast<std::size_t>(N));
  std::fill(t.begin(), t.end(), val);
  return t;
}

/// Largest multiple of M not above N.
constexpr std::size_t nearest_mul_of_x(std::size_t N, std::size_t M) noexcept { return N - (N % M); }

template <typename T>
struct is_first_order : std::false_type {};
template <>
struct is_first_order<ub::layout::first_order> : std::true_type {};
template <typename T>
constexpr bool is_first_order_v = is_first_order<T>::value;

template <typename T>
struct is_last_order : std::false_type {};
template <>
struct is_last_order<ub::layout::last_order> : std::true_type {};
template <typename T>
constexpr bool is_last_order_v = is_last_order<T>::value;

namespace tag {
struct trans {};
struct inplace {};
struct outplace {};
}  // namespace tag

/// Copy an m x n panel (rows wi[0] apart, columns wi[1] apart) into `out`,
/// one column of m values after another, columns `wo` apart
/// (reference include/utils.hpp:99-118).
template <typename ValueType, typename SizeType>
void pack(ValueType* out, SizeType const wo, ValueType const* in, SizeType const* wi, SizeType const m,
          SizeType const n) noexcept {
  for (SizeType col = 0; col < n; ++col)
    for (SizeType row = 0; row < m; ++row) out[wo * col + row] = in[wi[1] * col + wi[0] * row];
}

/// Transposed packing: walks rows of `in` instead of columns
/// (reference include/utils.hpp:120-141).
template <typename ValueType, typename SizeType>
void pack(ValueType* out, SizeType const wo, ValueType const* in, SizeType const* wi, SizeType const m,
          SizeType const n, tag::trans) noexcept {
  for (SizeType row = 0; row < n; ++row)
    for (SizeType col = 0; col < m; ++col) out[wo * row + col] = in[wi[0] * row + wi[1] * col];
}

namespace gpu {

/// GEMM arithmetic (see gbblas_accuracy in gbblas.h).  float: fp32 (the
/// default), bf16x3, fp8, automatic, bf16x6, fp16x3.  double: fp32 (the default:
/// gbblas_dgemm's - automatic unless GBBLAS_DGEMM_FP64=1), automatic (the
/// guarded tensor-core digits where faster), fp64 (the FP64 pipes),
/// fp64_digits7 / fp64_digits8 (unguarded tensor-core digits).
enum class accuracy : int {
  fp32 = GBBLAS_ACCURACY_FP32,
  bf16x3 = GBBLAS_ACCURACY_BF16X3,
  fp8 = GBBLAS_ACCURACY_FP8,
  automatic = GBBLAS_ACCURACY_AUTO,
  bf16x6 = GBBLAS_ACCURACY_BF16X6,
  fp64 = GBBLAS_ACCURACY_FP64,
  fp64_digits7 = GBBLAS_ACCURACY_FP64_DIGITS7,
  fp64_digits8 = GBBLAS_ACCURACY_FP64_DIGITS8,
  fp16x3 = GBBLAS_ACCURACY_FP16X3,
};

/// Throw std::runtime_error for a failed C-ABI call (the reference reports
/// every misuse by throwing std::runtime_error).
inline void check(gbblas_status s, const char* what) {
  if (s != GBBLAS_STATUS_SUCCESS)
    throw std::runtime_error(std::string(what) + ": " + gbblas_status_string(s) + ": " + gbblas_last_error());
}

template <typename L>
constexpr gbblas_layout layout_of() noexcept {
  return std::is_same_v<L, ub::layout::last_order> ? GBBLAS_LAST_ORDER : GBBLAS_FIRST_ORDER;
}

}  // namespace gpu
}  // namespace amt

#endif  // GBBLAS_AMT_UTILS_HPP
