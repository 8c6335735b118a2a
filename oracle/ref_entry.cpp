// ref_entry.cpp - C entry points over the reference's own hot-path headers.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
// the reference's unmodified include/{mtm,mtv,dot}.hpp (read where they lie,
// never copied) and the project's uBLAS-tensor compat shim into
// oracle/_ref/libamt_ref.so.  Tests use it to pin the C restatement in
// oracle/oracle.c and tests/golden/make_golden.py uses it to write golden
// vectors.  It exists only where the reference sources exist.
//
// Each entry copies the caller's dense buffers into uBLAS tensors of the
// requested layout, runs the reference's deferred callable exactly as its
// tests do (e.g. `amt::mtm(C, A, B, std::nullopt)();`, test/test.mtm.cpp:70),
// and copies the result back.  Layout 0 = first_order (column-major),
// 1 = last_order (row-major).
#include <algorithm>
#include <cstddef>
#include <cstring>
#include <exception>
#include <optional>

#include <dot.hpp>
#include <mtm.hpp>
#include <mtv.hpp>

namespace ub = boost::numeric::ublas;

namespace {

template <class T, class L>
using mat = ub::tensor_static_rank<T, 2, L>;

template <class T, class L>
mat<T, L> load(std::size_t r, std::size_t c, T const* src) {
  mat<T, L> t(r, c);
  std::memcpy(t.data(), src, r * c * sizeof(T));
  return t;
}

template <class T, class LC, class LA, class LB>
int mtm_case(std::size_t M, std::size_t N, std::size_t K, T const* A, T const* B, T* C) {
  auto a = load<T, LA>(M, K, A);
  auto b = load<T, LB>(K, N, B);
  auto c = load<T, LC>(M, N, C);
  amt::mtm(c, a, b, std::nullopt)();
  std::memcpy(C, c.data(), M * N * sizeof(T));
  return 0;
}

template <class T, class LC, class LA>
int mtm_lb(int lb, std::size_t M, std::size_t N, std::size_t K, T const* A, T const* B, T* C) {
  return lb ? mtm_case<T, LC, LA, ub::layout::last_order>(M, N, K, A, B, C)
            : mtm_case<T, LC, LA, ub::layout::first_order>(M, N, K, A, B, C);
}

template <class T, class LC>
int mtm_la(int la, int lb, std::size_t M, std::size_t N, std::size_t K, T const* A, T const* B, T* C) {
  return la ? mtm_lb<T, LC, ub::layout::last_order>(lb, M, N, K, A, B, C)
            : mtm_lb<T, LC, ub::layout::first_order>(lb, M, N, K, A, B, C);
}

template <class T>
int mtm_any(int lc, int la, int lb, std::size_t M, std::size_t N, std::size_t K, T const* A, T const* B,
            T* C) {
  try {
    return lc ? mtm_la<T, ub::layout::last_order>(la, lb, M, N, K, A, B, C)
              : mtm_la<T, ub::layout::first_order>(la, lb, M, N, K, A, B, C);
  } catch (std::exception const&) {
    return 1;
  }
}

// x and y are built as (1, n) first_order tensors, as test/test.mtv.cpp:37-43 does.
template <class T, class LA, bool Transposed>
int mv_case(std::size_t M, std::size_t N, T const* A, T const* x, T* y) {
  auto a = load<T, LA>(M, N, A);
  std::size_t nx = Transposed ? M : N, ny = Transposed ? N : M;
  auto xv = load<T, ub::layout::first_order>(1, nx, x);
  auto yv = load<T, ub::layout::first_order>(1, ny, y);
  if constexpr (Transposed)
    amt::vtm(yv, a, xv, std::nullopt)();
  else
    amt::mtv(yv, a, xv, std::nullopt)();
  std::memcpy(y, yv.data(), ny * sizeof(T));
  return 0;
}

template <class T, bool Transposed>
int mv_any(int la, std::size_t M, std::size_t N, T const* A, T const* x, T* y) {
  try {
    return la ? mv_case<T, ub::layout::last_order, Transposed>(M, N, A, x, y)
              : mv_case<T, ub::layout::first_order, Transposed>(M, N, A, x, y);
  } catch (std::exception const&) {
    return 1;
  }
}

template <class T>
T dot_any(std::size_t n, T const* a, T const* b) {
  auto av = load<T, ub::layout::first_order>(1, n, a);
  auto bv = load<T, ub::layout::first_order>(1, n, b);
  T r{};
  amt::dot_prod(r, av, bv, std::nullopt)();
  return r;
}

template <class T>
T dot_tuning_any(std::size_t n, T const* a, T const* b, std::size_t b1, std::size_t b2, std::size_t b3) {
  auto av = load<T, ub::layout::first_order>(1, n, a);
  auto bv = load<T, ub::layout::first_order>(1, n, b);
  T r{};
  amt::dot_prod_tuning_param(r, av, bv, b1, b2, b3, std::nullopt)();
  return r;
}

}  // namespace

extern "C" {

int ref_sgemm(int lc, int la, int lb, std::size_t M, std::size_t N, std::size_t K, float const* A,
              float const* B, float* C) {
  return mtm_any<float>(lc, la, lb, M, N, K, A, B, C);
}
int ref_dgemm(int lc, int la, int lb, std::size_t M, std::size_t N, std::size_t K, double const* A,
              double const* B, double* C) {
  return mtm_any<double>(lc, la, lb, M, N, K, A, B, C);
}
int ref_smtv(int la, std::size_t M, std::size_t N, float const* A, float const* x, float* y) {
  return mv_any<float, false>(la, M, N, A, x, y);
}
int ref_dmtv(int la, std::size_t M, std::size_t N, double const* A, double const* x, double* y) {
  return mv_any<double, false>(la, M, N, A, x, y);
}
int ref_svtm(int la, std::size_t M, std::size_t N, float const* A, float const* v, float* y) {
  return mv_any<float, true>(la, M, N, A, v, y);
}
int ref_dvtm(int la, std::size_t M, std::size_t N, double const* A, double const* v, double* y) {
  return mv_any<double, true>(la, M, N, A, v, y);
}
float ref_sdot(std::size_t n, float const* a, float const* b) { return dot_any<float>(n, a, b); }
double ref_ddot(std::size_t n, double const* a, double const* b) { return dot_any<double>(n, a, b); }
float ref_sdot_tuning(std::size_t n, float const* a, float const* b, std::size_t b1, std::size_t b2,
                      std::size_t b3) {
  return dot_tuning_any<float>(n, a, b, b1, b2, b3);
}
double ref_ddot_tuning(std::size_t n, double const* a, double const* b, std::size_t b1, std::size_t b2,
                       std::size_t b3) {
  return dot_tuning_any<double>(n, a, b, b1, b2, b3);
}

// The reference's panel packers (include/utils.hpp:99-141) on a raw buffer.
void ref_spack(float* out, std::size_t wo, float const* in, std::size_t const* wi, std::size_t m,
               std::size_t n, int trans) {
  if (trans)
    amt::pack(out, wo, in, wi, m, n, amt::tag::trans{});
  else
    amt::pack(out, wo, in, wi, m, n);
}

// Cache geometry as the reference sees it (include/cache_manager.hpp:204-208).
void ref_cache_info(std::size_t size[3], std::size_t assoc[3], std::size_t line[3]) {
  for (std::size_t k = 0; k < 3; ++k) {
    size[k] = amt::cache_manager::size(k);
    assoc[k] = amt::cache_manager::assoc(k);
    line[k] = amt::cache_manager::line_size(k);
  }
}

}  // extern "C"
