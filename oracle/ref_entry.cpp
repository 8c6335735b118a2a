// ref_entry.cpp - C entry points over the reference's own hot-path headers.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
// the reference's unmodified include/{mtm,mtv,dot,outer,trans,el_wise_op}.hpp
// (read where they lie,
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
#include <el_wise_op.hpp>
#include <mtm.hpp>
#include <mtv.hpp>
#include <outer.hpp>
#include <trans.hpp>

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

// a and b as (1, n) first_order vectors, as test/test.outer_prod.cpp:37-38 builds them.
template <class T, class LC>
int outer_case(std::size_t M, std::size_t N, T const* a, T const* b, T* C) {
  auto av = load<T, ub::layout::first_order>(1, M, a);
  auto bv = load<T, ub::layout::first_order>(1, N, b);
  auto c = load<T, LC>(M, N, C);
  amt::outer_prod(c, av, bv, std::nullopt)();
  std::memcpy(C, c.data(), M * N * sizeof(T));
  return 0;
}

template <class T>
int outer_any(int lc, std::size_t M, std::size_t N, T const* a, T const* b, T* C) {
  try {
    return lc ? outer_case<T, ub::layout::last_order>(M, N, a, b, C)
              : outer_case<T, ub::layout::first_order>(M, N, a, b, C);
  } catch (std::exception const&) {
    return 1;
  }
}

// C = A^T for dense A (M x N, layout la) into dense C (N x M, layout lc).
template <class T, class LA, class LC>
int transpose_case(std::size_t M, std::size_t N, T const* A, T* C) {
  auto a = load<T, LA>(M, N, A);
  mat<T, LC> c(N, M);
  amt::transpose(c, a, std::nullopt)();
  std::memcpy(C, c.data(), M * N * sizeof(T));
  return 0;
}

template <class T>
int transpose_any(int la, int lc, std::size_t M, std::size_t N, T const* A, T* C) {
  try {
    if (la)
      return lc ? transpose_case<T, ub::layout::last_order, ub::layout::last_order>(M, N, A, C)
                : transpose_case<T, ub::layout::last_order, ub::layout::first_order>(M, N, A, C);
    return lc ? transpose_case<T, ub::layout::first_order, ub::layout::last_order>(M, N, A, C)
              : transpose_case<T, ub::layout::first_order, ub::layout::first_order>(M, N, A, C);
  } catch (std::exception const&) {
    return 1;
  }
}

// In place on a square n x n (the only shape the reference handles in place).
template <class T>
int transpose_inplace_any(std::size_t n, T* A) {
  try {
    auto a = load<T, ub::layout::first_order>(n, n, A);
    amt::transpose(a, std::nullopt)();
    std::memcpy(A, a.data(), n * n * sizeof(T));
    return 0;
  } catch (std::exception const&) {
    return 1;
  }
}

template <class T>
int ew_case(int op, std::size_t n, T const* a, T const* b, T* c) {
  auto av = load<T, ub::layout::first_order>(1, n, a);
  auto bv = load<T, ub::layout::first_order>(1, n, b);
  auto cv = load<T, ub::layout::first_order>(1, n, c);
  switch (op) {
    case 0: amt::el_op::add(cv, av, bv, std::nullopt); break;
    case 1: amt::el_op::sub(cv, av, bv, std::nullopt); break;
    case 2: amt::el_op::mul(cv, av, bv, std::nullopt); break;
    default: amt::el_op::div(cv, av, bv, std::nullopt); break;
  }
  std::memcpy(c, cv.data(), n * sizeof(T));
  return 0;
}

template <class T>
int ew_any(int op, std::size_t n, T const* a, T const* b, T* c) {
  try {
    return ew_case(op, n, a, b, c);
  } catch (std::exception const&) {
    return 1;
  }
}

}  // namespace

extern "C" {

int ref_souter(int lc, std::size_t M, std::size_t N, float const* a, float const* b, float* C) {
  return outer_any<float>(lc, M, N, a, b, C);
}
int ref_douter(int lc, std::size_t M, std::size_t N, double const* a, double const* b, double* C) {
  return outer_any<double>(lc, M, N, a, b, C);
}
int ref_stranspose(int la, int lc, std::size_t M, std::size_t N, float const* A, float* C) {
  return transpose_any<float>(la, lc, M, N, A, C);
}
int ref_dtranspose(int la, int lc, std::size_t M, std::size_t N, double const* A, double* C) {
  return transpose_any<double>(la, lc, M, N, A, C);
}
int ref_stranspose_inplace(std::size_t n, float* A) { return transpose_inplace_any<float>(n, A); }
int ref_dtranspose_inplace(std::size_t n, double* A) { return transpose_inplace_any<double>(n, A); }
int ref_sew(int op, std::size_t n, float const* a, float const* b, float* c) { return ew_any<float>(op, n, a, b, c); }
int ref_dew(int op, std::size_t n, double const* a, double const* b, double* c) {
  return ew_any<double>(op, n, a, b, c);
}


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
