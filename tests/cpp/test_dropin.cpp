// Drop-in test of include/{mtm,mtv,dot,outer,trans,el_wise_op}.hpp: the
// reference's own test cases (test/test.mtm.cpp, test.mtv.cpp, test.vtm.cpp,
// test.dot_prod.cpp, test.pack.cpp, test.outer_prod.cpp, test.trans.cpp)
// rewritten without Catch2/BLIS/Eigen, calling the amt:: templates
// exactly as the reference's tests do - `amt::mtm(rres, A, B, std::nullopt)();`
// - and checking the results against the CPU oracle (oracle/oracle.c), the
// reference's arithmetic restated.  Built and run by tests/test_dropin_cpp.py.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <optional>
#include <stdexcept>
#include <vector>

#include <dot.hpp>
#include <el_wise_op.hpp>
#include <mtm.hpp>
#include <mtv.hpp>
#include <outer.hpp>
#include <trans.hpp>

extern "C" {
int orc_sgemm(size_t, size_t, size_t, const float*, ptrdiff_t, ptrdiff_t, const float*, ptrdiff_t, ptrdiff_t, float*,
              ptrdiff_t, ptrdiff_t);
int orc_dgemm(size_t, size_t, size_t, const double*, ptrdiff_t, ptrdiff_t, const double*, ptrdiff_t, ptrdiff_t,
              double*, ptrdiff_t, ptrdiff_t);
void orc_smtv(int, size_t, size_t, const float*, const float*, float*);
void orc_dmtv(int, size_t, size_t, const double*, const double*, double*);
void orc_svtm(int, size_t, size_t, const float*, const float*, float*);
void orc_dvtm(int, size_t, size_t, const double*, const double*, double*);
void orc_souter(int, size_t, size_t, const float*, const float*, float*);
void orc_douter(int, size_t, size_t, const double*, const double*, double*);
}

namespace ub = boost::numeric::ublas;

static int g_checks = 0, g_failures = 0;
#define REQUIRE(cond)                                                               \
  do {                                                                              \
    ++g_checks;                                                                     \
    if (!(cond)) {                                                                  \
      if (++g_failures < 20) std::fprintf(stderr, "FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond); \
    }                                                                               \
  } while (0)

// Catch2's default Approx: relative 100 * FLT_EPSILON.
static bool approx(double a, double b) {
  const double eps = 100.0 * 1.1920929e-7;
  return std::fabs(a - b) <= eps * (std::max(std::fabs(a), std::fabs(b)) + 1.0);
}

// test/test_utils.hpp: integer values in [0, 99]
template <typename T, typename C>
void rand_gen(C& c) {
  std::generate(c.begin(), c.end(), [] { return static_cast<T>(std::rand() % 100); });
}

template <typename T>
int oracle_gemm(size_t M, size_t N, size_t K, const T* A, ptrdiff_t rsa, ptrdiff_t csa, const T* B, ptrdiff_t rsb,
                ptrdiff_t csb, T* C, ptrdiff_t rsc, ptrdiff_t csc) {
  if constexpr (std::is_same_v<T, float>)
    return orc_sgemm(M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc);
  else
    return orc_dgemm(M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc);
}

// One of the eight (C, A, B) layout mixes of test/test.mtm.cpp.
template <typename T, typename LC, typename LA, typename LB>
void mtm_case() {
  for (std::size_t sz = 2; sz < 32; ++sz) {
    auto A = amt::make_tensor<T, LA>(sz, sz);
    auto B = amt::make_tensor<T, LB>(sz, sz);
    rand_gen<T>(A);
    rand_gen<T>(B);
    auto lres = amt::make_tensor<T, LC>(sz, sz);
    auto rres = amt::make_tensor<T, LC>(sz, sz);
    auto wa = A.strides(), wb = B.strides(), wc = lres.strides();
    oracle_gemm<T>(sz, sz, sz, A.data(), wa[0], wa[1], B.data(), wb[0], wb[1], lres.data(), wc[0], wc[1]);
    amt::mtm(rres, A, B, std::nullopt)();
    for (std::size_t i = 0; i < rres.size(); ++i) REQUIRE(rres[i] == lres[i]);  // integer data: exact
  }
  // non-square, K crossing the reference's K blocking, C accumulated
  auto A = amt::make_tensor<T, LA>(37, 600);
  auto B = amt::make_tensor<T, LB>(600, 29);
  rand_gen<T>(A);
  rand_gen<T>(B);
  auto lres = amt::make_tensor<T, LC>(37, 29, T(3));
  auto rres = amt::make_tensor<T, LC>(37, 29, T(3));
  auto wa = A.strides(), wb = B.strides(), wc = lres.strides();
  oracle_gemm<T>(37, 29, 600, A.data(), wa[0], wa[1], B.data(), wb[0], wb[1], lres.data(), wc[0], wc[1]);
  amt::mtm(rres, A, B, std::nullopt)();
  for (std::size_t i = 0; i < rres.size(); ++i) REQUIRE(rres[i] == lres[i]);
  if constexpr (std::is_same_v<T, double>) {
    // every double arithmetic is exact on these integers
    for (auto acc : {amt::gpu::accuracy::fp64, amt::gpu::accuracy::automatic, amt::gpu::accuracy::fp64_digits7,
                     amt::gpu::accuracy::fp64_digits8}) {
      auto r2 = amt::make_tensor<T, LC>(37, 29, T(3));
      amt::mtm(r2, A, B, std::nullopt, acc)();
      for (std::size_t i = 0; i < r2.size(); ++i) REQUIRE(r2[i] == lres[i]);
    }
  }
}

template <typename T>
void mtm_all() {
  using F = ub::layout::first_order;
  using L = ub::layout::last_order;
  mtm_case<T, F, F, F>();
  mtm_case<T, F, F, L>();
  mtm_case<T, F, L, F>();
  mtm_case<T, L, F, F>();
  mtm_case<T, F, L, L>();
  mtm_case<T, L, F, L>();
  mtm_case<T, L, L, F>();
  mtm_case<T, L, L, L>();
}

template <typename T, typename LA, bool Vtm>
void mv_case() {
  constexpr int lay = std::is_same_v<LA, ub::layout::last_order> ? 1 : 0;
  for (std::size_t M = 2; M < 512; M += 37) {
    for (std::size_t N : {M, M + 5, (M + 1) / 2 + 1}) {
      auto A = amt::make_tensor<T, LA>(M, N);
      rand_gen<T>(A);
      std::size_t nin = Vtm ? M : N, nout = Vtm ? N : M;
      auto v = amt::make_tensor<T>(1, nin);
      rand_gen<T>(v);
      auto rres = amt::make_tensor<T>(1, nout, T(5));
      std::vector<T> lres(nout, T(5));
      if constexpr (Vtm) {
        if constexpr (std::is_same_v<T, float>)
          orc_svtm(lay, M, N, A.data(), v.data(), lres.data());
        else
          orc_dvtm(lay, M, N, A.data(), v.data(), lres.data());
        amt::vtm(rres, A, v, std::nullopt)();
      } else {
        if constexpr (std::is_same_v<T, float>)
          orc_smtv(lay, M, N, A.data(), v.data(), lres.data());
        else
          orc_dmtv(lay, M, N, A.data(), v.data(), lres.data());
        amt::mtv(rres, A, v, std::nullopt)();
      }
      for (std::size_t i = 0; i < nout; ++i) REQUIRE(approx(rres[i], lres[i]));
    }
  }
}

template <typename T>
void dot_case() {
  // test/test.dot_prod.cpp: iota . iota against the closed form
  for (std::size_t s = 2; s < (1u << 17) + 2; s += (s < 300 ? 1 : 1009)) {
    auto a = amt::make_tensor<T>(1ul, s);
    std::iota(a.begin(), a.end(), 1);
    T my_res{};
    amt::dot_prod(my_res, a, a, std::nullopt)();
    const double exact = double(s) * double(s + 1) * double(2 * s + 1) / 6.0;
    REQUIRE(approx(my_res, exact));
    T tuned{};
    amt::dot_prod_tuning_param(tuned, a, a, 64, 128, 4096, std::nullopt)();
    REQUIRE(tuned == my_res);
  }
}

void pack_case() {
  // test/test.pack.cpp:48-123
  auto in = amt::make_tensor<float>(3, 3);
  std::iota(in.begin(), in.end(), 1.f);
  auto out = amt::make_tensor<float>(3, 3);
  std::iota(out.begin(), out.end(), 1.f);
  auto const& n = in.extents();
  auto const& w = in.strides();
  for (std::size_t i = 0; i < n[0]; i += 2) {
    auto ib = std::min<std::size_t>(2, n[0] - i);
    amt::pack(out.data() + i * n[1], ib, in.data() + i * w[0], w.data(), ib, n[1]);
  }
  const int plain[9][2] = {{0, 0}, {1, 1}, {2, 6}, {3, 2}, {4, 3}, {5, 7}, {6, 4}, {7, 5}, {8, 8}};
  for (auto& p : plain) REQUIRE(in[p[0]] == out[p[1]]);
  std::iota(out.begin(), out.end(), 1.f);
  for (std::size_t i = 0; i < n[0]; i += 2) {
    auto ib = std::min<std::size_t>(2, n[0] - i);
    amt::pack(out.data() + i * n[1], ib, in.data() + i * w[1], w.data(), ib, n[1], amt::tag::trans{});
  }
  const int trans[9][2] = {{0, 0}, {1, 2}, {2, 4}, {3, 1}, {4, 3}, {5, 5}, {6, 6}, {7, 7}, {8, 8}};
  for (auto& p : trans) REQUIRE(in[p[0]] == out[p[1]]);
}

// test/test.outer_prod.cpp: square and rectangular sizes 2..33, both layouts
template <typename T, typename LC>
void outer_case() {
  constexpr int lay = std::is_same_v<LC, ub::layout::last_order> ? 1 : 0;
  for (std::size_t m = 2; m < 34; m += 3) {
    for (std::size_t n = 2; n < 34; n += 5) {
      auto a = amt::make_tensor<T>(1ul, m);
      auto b = amt::make_tensor<T>(1ul, n);
      rand_gen<T>(a);
      rand_gen<T>(b);
      auto lres = amt::make_tensor<T, LC>(m, n, T(1));
      auto rres = amt::make_tensor<T, LC>(m, n, T(1));
      if constexpr (std::is_same_v<T, float>)
        orc_souter(lay, m, n, a.data(), b.data(), lres.data());
      else
        orc_douter(lay, m, n, a.data(), b.data(), lres.data());
      amt::outer_prod(rres, a, b, std::nullopt)();
      for (std::size_t i = 0; i < rres.size(); ++i) REQUIRE(rres[i] == lres[i]);
    }
  }
}

// test/test.trans.cpp: out of place (every layout pair) and in place, sizes 2..31
template <typename T, typename LA, typename LC>
void trans_case() {
  for (std::size_t sz = 2; sz < 32; ++sz) {
    for (std::size_t n2 : {sz, sz + 3}) {
      auto A = amt::make_tensor<T, LA>(sz, n2);
      rand_gen<T>(A);
      auto C = amt::make_tensor<T, LC>(n2, sz);
      amt::transpose(C, A, std::nullopt)();
      for (std::size_t i = 0; i < sz; ++i)
        for (std::size_t j = 0; j < n2; ++j) REQUIRE(C(j, i) == A(i, j));
    }
    auto S = amt::make_tensor<T, LA>(sz, sz);
    rand_gen<T>(S);
    auto orig = S;
    amt::transpose(S, std::nullopt)();
    for (std::size_t i = 0; i < sz; ++i)
      for (std::size_t j = 0; j < sz; ++j) REQUIRE(S(i, j) == orig(j, i));
  }
}

template <typename T>
void el_wise_case() {
  for (std::size_t n : {1ul, 7ul, 1000ul, 4099ul}) {
    auto a = amt::make_tensor<T>(1ul, n);
    auto b = amt::make_tensor<T>(1ul, n);
    auto c = amt::make_tensor<T>(1ul, n);
    rand_gen<T>(a);
    std::generate(b.begin(), b.end(), [] { return static_cast<T>(std::rand() % 100 + 1); });
    amt::el_op::add(c, a, b, std::nullopt);
    for (std::size_t i = 0; i < n; ++i) REQUIRE(c[i] == a[i] + b[i]);
    amt::el_op::sub(c, a, b, std::nullopt);
    for (std::size_t i = 0; i < n; ++i) REQUIRE(c[i] == a[i] - b[i]);
    amt::el_op::mul(c, a, b, std::nullopt);
    for (std::size_t i = 0; i < n; ++i) REQUIRE(c[i] == a[i] * b[i]);
    amt::el_op::div(c, a, b, std::nullopt);
    for (std::size_t i = 0; i < n; ++i) REQUIRE(c[i] == a[i] / b[i]);
    amt::el_op::apply_ops(c, a, b, std::nullopt, std::multiplies<T>{});
    for (std::size_t i = 0; i < n; ++i) REQUIRE(c[i] == a[i] * b[i]);
  }
}

void error_cases() {
  // shape errors throw std::runtime_error when the callable is created
  auto A = amt::make_tensor<float>(4, 5);
  auto B = amt::make_tensor<float>(6, 3);
  auto C = amt::make_tensor<float>(4, 3);
  bool threw = false;
  try {
    auto f = amt::mtm(C, A, B, std::nullopt);
    (void)f;
  } catch (std::runtime_error const&) {
    threw = true;
  }
  REQUIRE(threw);
  threw = false;
  auto v = amt::make_tensor<float>(1, 4);
  auto y = amt::make_tensor<float>(1, 4);
  try {
    auto f = amt::mtv(y, A, v, std::nullopt);
    (void)f;
  } catch (std::runtime_error const&) {
    threw = true;
  }
  REQUIRE(threw);
  threw = false;
  auto notvec = amt::make_tensor<float>(2, 2);
  float r = 0;
  try {
    auto f = amt::dot_prod(r, notvec, notvec);
    (void)f;
  } catch (std::runtime_error const&) {
    threw = true;
  }
  REQUIRE(threw);
  threw = false;
  auto rect = amt::make_tensor<float>(3, 5);
  try {
    auto f = amt::transpose(rect, std::nullopt);  // in place needs a square matrix
    (void)f;
  } catch (std::runtime_error const&) {
    threw = true;
  }
  REQUIRE(threw);
  threw = false;
  auto o = amt::make_tensor<float>(4, 4);
  try {
    auto f = amt::outer_prod(o, v, notvec, std::nullopt);
    (void)f;
  } catch (std::runtime_error const&) {
    threw = true;
  }
  REQUIRE(threw);
}

int main() {
  std::srand(1);
  pack_case();
  error_cases();
  mtm_all<float>();
  mtm_all<double>();
  mv_case<float, ub::layout::first_order, false>();
  mv_case<float, ub::layout::last_order, false>();
  mv_case<double, ub::layout::first_order, false>();
  mv_case<double, ub::layout::last_order, false>();
  mv_case<float, ub::layout::first_order, true>();
  mv_case<float, ub::layout::last_order, true>();
  mv_case<double, ub::layout::first_order, true>();
  mv_case<double, ub::layout::last_order, true>();
  dot_case<float>();
  dot_case<double>();
  outer_case<float, ub::layout::first_order>();
  outer_case<float, ub::layout::last_order>();
  outer_case<double, ub::layout::first_order>();
  outer_case<double, ub::layout::last_order>();
  trans_case<float, ub::layout::first_order, ub::layout::first_order>();
  trans_case<float, ub::layout::first_order, ub::layout::last_order>();
  trans_case<float, ub::layout::last_order, ub::layout::first_order>();
  trans_case<double, ub::layout::last_order, ub::layout::last_order>();
  el_wise_case<float>();
  el_wise_case<double>();
  std::printf("%d checks, %d failures\n", g_checks, g_failures);
  return g_failures == 0 ? 0 : 1;
}
