// inputs.cu - the seeded synthetic inputs of the benchmark configurations
// and parity tests (host code only, no kernel).
//
// The reference fills its benchmark operands with ones (src/mtm.cpp:204-205,
// make_tensor(..., 1.)) and its tests with rand() % 100
// (test/test_utils.hpp:4-8); the GB300 configurations instead draw
// U[-1,1) values from std::mt19937_64 with a fixed seed, operand after
// operand.  std::mt19937_64's output sequence is fixed by the C++ standard,
// and the mapping from a 64-bit draw to a value below uses exact integer
// arithmetic and one exact subtraction, so every machine and language that
// follows it gets the same bits: the CPU oracle restates the generator
// independently, and both benchmark arms and the parity tests compute on
// identical inputs.
#include <cmath>
#include <random>

#include "common.cuh"

namespace {

// U[-1, 1): (draw >> 11) * 2^-52 - 1 in double, (draw >> 40) * 2^-23 - 1 in
// float.  Both products are exact, and so is the subtraction.
inline double u64_to_f64(uint64_t x) { return (double)(x >> 11) * 0x1.0p-52 - 1.0; }
inline float u64_to_f32(uint64_t x) { return (float)(x >> 40) * 0x1.0p-23f - 1.0f; }

// Wide-range set: s * m * 2^e from two draws d1, d2: s = -1 if bit 63 of d1
// is set, m = 1 + (d1 bits 11..62) * 2^-52 (double) or 1 + (d1 bits 40..62)
// * 2^-23 (float), e = ((d2 >> 32) mod 21) - 10.
inline int wide_exp(uint64_t d2) { return (int)((d2 >> 32) % 21u) - 10; }
inline double wide_f64(uint64_t d1, uint64_t d2) {
  const double m = 1.0 + (double)((d1 >> 11) & ((1ull << 52) - 1)) * 0x1.0p-52;
  const double v = std::ldexp(m, wide_exp(d2));
  return (d1 >> 63) ? -v : v;
}
inline float wide_f32(uint64_t d1, uint64_t d2) {
  const float m = 1.0f + (float)((d1 >> 40) & ((1u << 23) - 1)) * 0x1.0p-23f;
  const float v = std::ldexp(m, wide_exp(d2));
  return (d1 >> 63) ? -v : v;
}

}  // namespace

extern "C" gbblas_status gbblas_seeded_fill(uint64_t seed, int32_t kind, int64_t nseg, const int64_t* counts,
                                            float* const* out_f32, double* const* out_f64) {
  using namespace gbblas;
  if (kind != GBBLAS_FILL_UNIFORM && kind != GBBLAS_FILL_WIDE) {
    set_error("gbblas_seeded_fill: unknown kind %d", (int)kind);
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  if (nseg < 0 || (nseg > 0 && !counts)) {
    set_error("gbblas_seeded_fill: bad segment list");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  for (int64_t s = 0; s < nseg; ++s) {
    if (counts[s] < 0) {
      set_error("gbblas_seeded_fill: negative count in segment %lld", (long long)s);
      return GBBLAS_STATUS_INVALID_VALUE;
    }
  }
  std::mt19937_64 gen(seed);
  for (int64_t s = 0; s < nseg; ++s) {
    float* f = out_f32 ? out_f32[s] : nullptr;
    double* d = out_f64 ? out_f64[s] : nullptr;
    const int64_t n = counts[s];
    if (kind == GBBLAS_FILL_UNIFORM) {
      if (f && d) {
        for (int64_t i = 0; i < n; ++i) {
          const uint64_t x = gen();
          f[i] = u64_to_f32(x);
          d[i] = u64_to_f64(x);
        }
      } else if (f) {
        for (int64_t i = 0; i < n; ++i) f[i] = u64_to_f32(gen());
      } else if (d) {
        for (int64_t i = 0; i < n; ++i) d[i] = u64_to_f64(gen());
      } else {
        gen.discard((unsigned long long)n);
      }
    } else {
      for (int64_t i = 0; i < n; ++i) {
        const uint64_t d1 = gen();
        const uint64_t d2 = gen();
        if (f) f[i] = wide_f32(d1, d2);
        if (d) d[i] = wide_f64(d1, d2);
      }
    }
  }
  return GBBLAS_STATUS_SUCCESS;
}
