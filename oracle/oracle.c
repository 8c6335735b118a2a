/*
 * oracle.c - CPU restatement of OpenMP-BLAS's dense hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed
 * CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline / reference arm may load it, and only as the checker or as the
 * CPU number beside the GPU one.  The GPU library never calls it.
 *
 * Parity pinning: tests/test_oracle_golden.py checks this restatement
 * against the reference's own known-answer tests (test/test.pack.cpp:8-83,
 * the closed-form dot of test/test.dot_prod.cpp:20-27) and against golden
 * vectors produced by the reference headers themselves, compiled unmodified
 * by oracle/Makefile into oracle/_ref/ (tests/golden/make_golden.py).
 *
 * What is restated (reference file:line):
 *   - cache geometry read through sysconf, including the slip that stores the
 *     L3 associativity into the L2 slot   include/cache_manager.hpp:107-150
 *   - register-tile sizes MR x NR         include/cpuinfo.hpp:167-223,
 *                                          include/mtm.hpp:26-39
 *   - cache-block sizes kc/mc/nc          include/mtm.hpp:41-80
 *   - panel packing (plain and transposed) include/utils.hpp:99-141
 *   - Goto 5-loop GEMM, C += A*B          include/mtm.hpp:83-110,116-206
 *   - MR x NR micro-kernel + C update     include/simd_loop.hpp:106-190
 *   - mtv, column-major (accumulates)     include/mtv.hpp:15-70,
 *                                          include/simd_loop.hpp:52-78
 *   - mtv, row-major (overwrites)         include/mtv.hpp:72-98,
 *                                          include/simd_loop.hpp:21-35
 *   - vtm (see orc_?vtm below: the reference's stride bug is NOT restated;
 *     the oracle computes y = v^T A with the reference's per-layout
 *     overwrite/accumulate rule)         include/mtv.hpp:164-236
 *   - dot in three size regimes           include/dot.hpp:16-54,143-174
 *   - dot with caller-given blocks        include/dot.hpp:59-90
 *   - outer product, C += a b^T           include/outer.hpp:14-119,
 *                                          include/simd_loop.hpp:42-47
 *   - transpose, out of place and square in place
 *                                          include/trans.hpp:33-169,
 *                                          include/simd_loop.hpp:194-238
 *   - element-wise + - * /                include/el_wise_op.hpp:33-112
 *
 * Element layouts follow uBLAS: "first order" = column-major (strides
 * {1, rows}), "last order" = row-major (strides {cols, 1}).
 */
#include <math.h>
#include <omp.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define ORC_FIRST_ORDER 0 /* column-major */
#define ORC_LAST_ORDER 1  /* row-major */

/* ------------------------------------------------------------------------ */
/* Cache geometry.                                                           */
/* ------------------------------------------------------------------------ */

typedef struct {
  size_t size[3];
  size_t assoc[3];
  size_t line[3];
} orc_cache_t;

static orc_cache_t g_cache;
static int g_cache_ready = 0;

/* Read one value from /sys/devices/system/cpu/cpu0/cache/index<i>/<leaf>.
 * Used when sysconf reports nothing (glibc on aarch64 often returns 0 for
 * the _SC_LEVEL*_CACHE_* names). */
static long sysfs_cache_value(int level, const char* want_type, const char* leaf) {
  for (int idx = 0; idx < 8; ++idx) {
    char path[256], buf[64];
    snprintf(path, sizeof path, "/sys/devices/system/cpu/cpu0/cache/index%d/level", idx);
    FILE* f = fopen(path, "r");
    if (!f) continue;
    int lv = 0;
    if (fscanf(f, "%d", &lv) != 1) lv = 0;
    fclose(f);
    if (lv != level) continue;
    snprintf(path, sizeof path, "/sys/devices/system/cpu/cpu0/cache/index%d/type", idx);
    f = fopen(path, "r");
    if (!f) continue;
    buf[0] = 0;
    if (fscanf(f, "%63s", buf) != 1) buf[0] = 0;
    fclose(f);
    if (strcmp(buf, want_type) != 0 && strcmp(buf, "Unified") != 0) continue;
    snprintf(path, sizeof path, "/sys/devices/system/cpu/cpu0/cache/index%d/%s", idx, leaf);
    f = fopen(path, "r");
    if (!f) continue;
    long v = 0;
    char unit = 0;
    int got = fscanf(f, "%ld%c", &v, &unit);
    fclose(f);
    if (got >= 1) {
      if (got == 2 && (unit == 'K' || unit == 'k')) v *= 1024;
      if (got == 2 && (unit == 'M' || unit == 'm')) v *= 1024 * 1024;
      return v;
    }
  }
  return 0;
}

static long cache_query(int sc_name, int level, const char* leaf) {
  long v = sysconf(sc_name);
  if (v > 0) return v;
  return sysfs_cache_value(level, "Data", leaf);
}

/* include/cache_manager.hpp:107-150.  The reference writes the L3
 * associativity into the L2 slot (lines 133-135) and never fills the L3
 * associativity, which keeps its default of 1 (line 35).  Block sizes below
 * depend on that, so the slip is restated. */
static void cache_init(void) {
  if (g_cache_ready) return;
  orc_cache_t c;
  for (int i = 0; i < 3; ++i) {
    c.size[i] = 0;
    c.assoc[i] = 1;
    c.line[i] = 0;
  }
  long v;
  if ((v = cache_query(_SC_LEVEL1_DCACHE_SIZE, 1, "size")) > 0) c.size[0] = (size_t)v;
  if ((v = cache_query(_SC_LEVEL2_CACHE_SIZE, 2, "size")) > 0) c.size[1] = (size_t)v;
  if ((v = cache_query(_SC_LEVEL3_CACHE_SIZE, 3, "size")) > 0) c.size[2] = (size_t)v;
  if ((v = cache_query(_SC_LEVEL1_DCACHE_ASSOC, 1, "ways_of_associativity")) > 0) c.assoc[0] = (size_t)(int8_t)v;
  if ((v = cache_query(_SC_LEVEL2_CACHE_ASSOC, 2, "ways_of_associativity")) > 0) c.assoc[1] = (size_t)(int8_t)v;
  if ((v = cache_query(_SC_LEVEL3_CACHE_ASSOC, 3, "ways_of_associativity")) > 0) c.assoc[1] = (size_t)(int8_t)v;
  if ((v = cache_query(_SC_LEVEL1_DCACHE_LINESIZE, 1, "coherency_line_size")) > 0) c.line[0] = (size_t)v;
  if ((v = cache_query(_SC_LEVEL2_CACHE_LINESIZE, 2, "coherency_line_size")) > 0) c.line[1] = (size_t)v;
  if ((v = cache_query(_SC_LEVEL3_CACHE_LINESIZE, 3, "coherency_line_size")) > 0) c.line[2] = (size_t)v;
  /* A machine that reports nothing at all would make the reference divide by
   * zero; such a machine gets a conventional 64 B / 48 KiB / 2 MiB / 32 MiB
   * geometry instead so the oracle stays defined. */
  for (int i = 0; i < 3; ++i)
    if (c.line[i] == 0) c.line[i] = 64;
  if (c.size[0] == 0) c.size[0] = 48u << 10;
  if (c.size[1] == 0) c.size[1] = 2u << 20;
  if (c.size[2] == 0) c.size[2] = 32u << 20;
  g_cache = c;
  g_cache_ready = 1;
}

static size_t cache_sets(int k) { return g_cache.size[k] / (g_cache.line[k] * g_cache.assoc[k]); }

void orc_cache_info(size_t out_size[3], size_t out_assoc[3], size_t out_line[3]) {
  cache_init();
  for (int i = 0; i < 3; ++i) {
    out_size[i] = g_cache.size[i];
    out_assoc[i] = g_cache.assoc[i];
    out_line[i] = g_cache.line[i];
  }
}

/* ------------------------------------------------------------------------ */
/* Register tile (include/cpuinfo.hpp:167-223 with the Skylake table, 256-bit */
/* vectors).  The compile-time square root there is a bisection that stops   */
/* when its interval closes (include/utils.hpp:185-201).                      */
/* ------------------------------------------------------------------------ */

static double ct_sqrt_rec(double res, double l, double r) {
  while (l != r) {
    double mid = (r + l) / 2.;
    if (mid * mid >= res)
      r = mid;
    else
      l = mid + 1.;
  }
  return r;
}

static size_t ceil_sz(double x) {
  size_t ip = (size_t)x;
  return (size_t)(x > (double)ip ? x + 1 : x);
}

/* Skylake: fma latency 4, loads 7 (256-bit), fma/load throughput 0.5. */
static void reg_tile(size_t elem_size, size_t* mr, size_t* nr) {
  double lat = 4. + 2. * 7.;
  double thr = 3. / (1. / 0.5 + 2. / 0.5);
  double elements = (double)(256 / (elem_size * 8));
  size_t mrxnr = (size_t)(elements * lat * thr);
  size_t m = ceil_sz(ct_sqrt_rec((double)mrxnr, 1., (double)mrxnr) / elements) * (size_t)elements;
  size_t n = ceil_sz((elements * lat * thr) / (double)m);
  *mr = m;
  *nr = n + (n & 1u);
}

typedef struct {
  size_t MR, NR, KB, MB, NB;
} orc_partition_t;

/* include/mtm.hpp:19-81.  For double with a row-major C the register tile is
 * transposed (lines 26-39). */
static orc_partition_t partition(size_t elem_size, int out_layout) {
  cache_init();
  orc_partition_t p;
  size_t mr, nr;
  reg_tile(elem_size, &mr, &nr);
  if (elem_size == sizeof(double) && out_layout == ORC_LAST_ORDER) {
    p.MR = nr;
    p.NR = mr;
  } else {
    p.MR = mr;
    p.NR = nr;
  }
  {
    size_t assoc = g_cache.assoc[0] == 1 ? 8u : g_cache.assoc[0];
    size_t sets = g_cache.size[0] / (g_cache.line[0] * assoc);
    double W = (double)assoc;
    double ratio = (double)p.NR / (double)p.MR;
    size_t CA = (size_t)ceil((W - 1.) / (1. + ratio));
    p.KB = (CA * sets * g_cache.line[0]) / (p.MR * elem_size);
  }
  {
    size_t assoc = g_cache.assoc[1];
    size_t sets = g_cache.size[1] / (g_cache.line[1] * assoc);
    size_t CA = (assoc - 1) >> 1;
    size_t sz = (CA * sets * g_cache.line[1]) / (p.KB * elem_size);
    p.MB = sz - sz % p.MR;
  }
  {
    size_t assoc = g_cache.assoc[2] == 1 ? 16u : g_cache.assoc[2];
    size_t sets = g_cache.size[2] / (g_cache.line[2] * assoc);
    size_t CB = (assoc - 1) >> 1;
    size_t sz = (CB * sets * g_cache.line[2]) / (p.KB * elem_size);
    p.NB = sz - sz % p.NR;
  }
  if (p.KB == 0) p.KB = 1;
  if (p.MB == 0) p.MB = p.MR;
  if (p.NB == 0) p.NB = p.NR;
  return p;
}

void orc_partition(size_t elem_size, int out_layout, size_t out[5]) {
  orc_partition_t p = partition(elem_size, out_layout);
  out[0] = p.MR;
  out[1] = p.NR;
  out[2] = p.KB;
  out[3] = p.MB;
  out[4] = p.NB;
}

/* Maximum threads, as omp_get_max_threads() (include/thread_utils.hpp:13-19). */
int orc_max_threads(void) { return omp_get_max_threads(); }
void orc_set_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
}

/* ------------------------------------------------------------------------ */
/* Type-generic parts, instantiated for float and double.                   */
/* ------------------------------------------------------------------------ */

/* Fused multiply-add by element type (the contraction the reference's
 * -ffast-math build applies to `c += a * b`). */
static inline float fmas_(float a, float b, float c) { return fmaf(a, b, c); }
static inline double fmad_(double a, double b, double c) { return fma(a, b, c); }

/* Correctly rounded IEEE quotients, exempt from -ffast-math (which may turn
 * a float division into a reciprocal estimate plus a Newton step). */
__attribute__((optimize("no-fast-math"), noinline)) static float divs_(float a, float b) { return a / b; }
__attribute__((optimize("no-fast-math"), noinline)) static double divd_(double a, double b) { return a / b; }

#define ORC_T float
#define ORC_S s
#include "oracle_impl.inc"
#undef ORC_T
#undef ORC_S

#define ORC_T double
#define ORC_S d
#include "oracle_impl.inc"
#undef ORC_T
#undef ORC_S

/* ------------------------------------------------------------------------ */
/* Higher-precision references used for error reports.                      */
/* ------------------------------------------------------------------------ */

/* sum_i a_i b_i in long double, plus sum_i |a_i b_i| (the dot's condition
 * scale).  Sequential, so it is exact enough to judge FP32 and FP64 dots. */
void orc_sdot_exact(size_t n, const float* a, const float* b, double* dot, double* absdot) {
  long double s = 0, t = 0;
  for (size_t i = 0; i < n; ++i) {
    long double p = (long double)a[i] * (long double)b[i];
    s += p;
    t += p < 0 ? -p : p;
  }
  *dot = (double)s;
  *absdot = (double)t;
}

void orc_ddot_exact(size_t n, const double* a, const double* b, double* dot, double* absdot) {
  long double s = 0, t = 0;
  for (size_t i = 0; i < n; ++i) {
    long double p = (long double)a[i] * (long double)b[i];
    s += p;
    t += p < 0 ? -p : p;
  }
  *dot = (double)s;
  *absdot = (double)t;
}

/* Sampled entries of A*B (general strides, float inputs) in long double, with
 * the matching entries of |A|*|B|.  rows/cols hold `count` (i, j) pairs. */
/* The same for double operands: each product and the sums in long double
 * (64 significand bits on x86, 113 on aarch64), far below the 2^-53
 * relative errors the double-precision paths are measured at. */
void orc_dgemm_sample_exact(size_t K, const double* A, ptrdiff_t rsa, ptrdiff_t csa, const double* B,
                            ptrdiff_t rsb, ptrdiff_t csb, size_t count, const int64_t* rows,
                            const int64_t* cols, double* out, double* absout) {
#pragma omp parallel for schedule(static)
  for (size_t s = 0; s < count; ++s) {
    long double acc = 0, aacc = 0;
    const double* ai = A + rows[s] * rsa;
    const double* bj = B + cols[s] * csb;
    for (size_t k = 0; k < K; ++k) {
      long double p = (long double)ai[k * csa] * (long double)bj[k * rsb];
      acc += p;
      aacc += p < 0 ? -p : p;
    }
    out[s] = (double)acc;
    absout[s] = (double)aacc;
  }
}

void orc_sgemm_sample_exact(size_t K, const float* A, ptrdiff_t rsa, ptrdiff_t csa, const float* B,
                            ptrdiff_t rsb, ptrdiff_t csb, size_t count, const int64_t* rows,
                            const int64_t* cols, double* out, double* absout) {
#pragma omp parallel for schedule(static)
  for (size_t s = 0; s < count; ++s) {
    long double acc = 0, aacc = 0;
    const float* ai = A + rows[s] * rsa;
    const float* bj = B + cols[s] * csb;
    for (size_t k = 0; k < K; ++k) {
      long double p = (long double)ai[k * csa] * (long double)bj[k * rsb];
      acc += p;
      aacc += p < 0 ? -p : p;
    }
    out[s] = (double)acc;
    absout[s] = (double)aacc;
  }
}

/* ------------------------------------------------------------------------ */
/* Seeded inputs: MT19937-64 (Matsumoto & Nishimura, "Tables of 64-bit      */
/* Mersenne Twisters", 2000; the engine std::mt19937_64 names) and the      */
/* value mappings of the benchmark configurations.  The GPU library draws   */
/* the same values through the C++ standard library's engine; this is an    */
/* independent restatement from the published algorithm, so the two        */
/* checking each other pins both.                                           */
/* ------------------------------------------------------------------------ */

#define MT64_N 312
#define MT64_M 156

typedef struct {
  uint64_t mt[MT64_N];
  int i;
} orc_mt64_t;

static void mt64_seed(orc_mt64_t* g, uint64_t seed) {
  g->mt[0] = seed;
  for (int i = 1; i < MT64_N; ++i)
    g->mt[i] = 6364136223846793005ULL * (g->mt[i - 1] ^ (g->mt[i - 1] >> 62)) + (uint64_t)i;
  g->i = MT64_N;
}

static inline uint64_t mt64_twist(uint64_t upper_from, uint64_t lower_from, uint64_t far) {
  const uint64_t x = (upper_from & 0xFFFFFFFF80000000ULL) | (lower_from & 0x7FFFFFFFULL);
  return far ^ (x >> 1) ^ ((x & 1ULL) ? 0xB5026F5AA96619E9ULL : 0ULL);
}

static uint64_t mt64_next(orc_mt64_t* g) {
  if (g->i >= MT64_N) {
    int k = 0;
    for (; k < MT64_N - MT64_M; ++k) g->mt[k] = mt64_twist(g->mt[k], g->mt[k + 1], g->mt[k + MT64_M]);
    for (; k < MT64_N - 1; ++k) g->mt[k] = mt64_twist(g->mt[k], g->mt[k + 1], g->mt[k + MT64_M - MT64_N]);
    g->mt[MT64_N - 1] = mt64_twist(g->mt[MT64_N - 1], g->mt[0], g->mt[MT64_M - 1]);
    g->i = 0;
  }
  uint64_t x = g->mt[g->i++];
  x ^= (x >> 29) & 0x5555555555555555ULL;
  x ^= (x << 17) & 0x71D67FFFEDA60000ULL;
  x ^= (x << 37) & 0xFFF7EEE000000000ULL;
  x ^= x >> 43;
  return x;
}

/* The first n raw 64-bit outputs of the engine seeded with `seed`. */
void orc_mt64_raw(uint64_t seed, int64_t n, uint64_t* out) {
  orc_mt64_t g;
  mt64_seed(&g, seed);
  for (int64_t i = 0; i < n; ++i) out[i] = mt64_next(&g);
}

/* kind 0: U[-1,1) - double (x >> 11) 2^-52 - 1, float (x >> 40) 2^-23 - 1.
 * kind 1: wide range s m 2^e from two draws d1, d2 - s from bit 63 of d1,
 * m = 1 + (d1 bits 11..62) 2^-52 (double) or 1 + (d1 bits 40..62) 2^-23
 * (float), e = ((d2 >> 32) mod 21) - 10.  Segments are drawn one after the
 * other from one engine; NULL outputs are drawn and skipped. */
int orc_seeded_fill(uint64_t seed, int kind, int64_t nseg, const int64_t* counts, float* const* f32,
                    double* const* f64) {
  if (kind != 0 && kind != 1) return 1;
  orc_mt64_t g;
  mt64_seed(&g, seed);
  for (int64_t s = 0; s < nseg; ++s) {
    float* f = f32 ? f32[s] : NULL;
    double* d = f64 ? f64[s] : NULL;
    for (int64_t i = 0; i < counts[s]; ++i) {
      const uint64_t x = mt64_next(&g);
      if (kind == 0) {
        if (f) f[i] = (float)(x >> 40) * 0x1.0p-23f - 1.0f;
        if (d) d[i] = (double)(x >> 11) * 0x1.0p-52 - 1.0;
      } else {
        const uint64_t x2 = mt64_next(&g);
        const int e = (int)((x2 >> 32) % 21u) - 10;
        if (f) {
          const float v = ldexpf(1.0f + (float)((x >> 40) & ((1u << 23) - 1)) * 0x1.0p-23f, e);
          f[i] = (x >> 63) ? -v : v;
        }
        if (d) {
          const double v = ldexp(1.0 + (double)((x >> 11) & ((1ULL << 52) - 1)) * 0x1.0p-52, e);
          d[i] = (x >> 63) ? -v : v;
        }
      }
    }
  }
  return 0;
}
