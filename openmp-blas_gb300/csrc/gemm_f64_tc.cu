// gemm_f64_tc.cu - double-precision C += A * B on the BF16 tensor cores
// (Ozaki scheme: exact integer digit products).
//
// GB300's FP64 pipes deliver about 1.25 TFLOP/s; its BF16 tensor cores more
// than a thousand times that.  This path turns one FP64 GEMM into integer
// GEMMs the tensor cores compute exactly:
//
//   1. Scales: every row i of A gets e_i with max_k |a_ik| < 2^e_i (the
//      exponent frexp gives), every column j of B likewise f_j.  A row or
//      column holding Inf or NaN is marked; its outputs become NaN.
//   2. Digits: x = a_ik / 2^e_i lies in (-1, 1).  F = round(x * 2^(8S-1)) is
//      an integer below 2^(8S-1) in magnitude (|x - F 2^(1-8S)| <= 2^-8S),
//      written in balanced base 256: F = sum_s D_s 256^(S-1-s) with
//      D_1..D_{S-1} in [-128, 127] and D_0 in [-128, 128], so every digit is
//      an integer a BF16 holds exactly.  S digit planes per operand, K-major
//      (A as M x K, B as its transpose N x K), zero-padded, in one arena.
//      Integer arithmetic on the FP64 bit pattern: no FP64 instructions.
//   3. GEMM: C_ij += 2^(e_i + f_j) sum_{w<S} 2^(-14-8w) G_w(i,j), where
//      G_w = sum_k sum_{s+t=w} D_s(a_ik) E_t(b_kj) - every digit product of
//      weight w (s + t > S-1 dropped).  The products are integers of at most
//      2^14, so a group's sum over 128 of K is at most 7 * 128 * 2^14 < 2^24
//      in magnitude and the FP32 accumulation in TMEM is exact.  Every 128 of
//      K the epilogue converts each group to an integer and adds it, shifted
//      by its weight, into two 64-bit accumulators per output (exact for K
//      up to 2^20); at the end of the tile it rounds their 128-bit sum once
//      to FP64 (integer operations; the power of two goes into the exponent
//      field) and adds it into C - one FP64 instruction per output.
//
// Error: the only roundings are the digit truncation (2^-8S of the scale),
// the dropped digit products and the final conversion and addition, so
// |C_ij - exact| <= (S+1) 2^-8S K 2^(e_i+f_j) + 2 ulp, i.e. with S = 7
// about 4 K 2^-53 max_k|a_ik| max_k|b_kj|.  The FP64 pipe's own bound is
// K 2^-53 sum_k |a_ik| |b_kj|: the two agree where each row's and column's
// magnitudes are comparable; rows mixing very large and very small values
// lose relative accuracy in their small entries.
//
// The guard (7 digits, G = 1; what AUTO runs): one more plane per operand,
// P = max(|D_0| - 1, 0) <= |x| 2^7, whose products summed over the first
// 32 of K of every 128-K chunk bound sum_k |a_ik||b_kj| from below.  An
// epilogue warp keeps its 32 x 16 block only where that bound makes the
// digit error smaller than the FP64 pipes' bound; other blocks leave C
// alone and are recomputed on the FP64 pipes by dgemm_fixup_kernel.
//
// The method is the published Ozaki scheme (error-free splitting of
// floating-point matrix products into exactly computable ones, by Ozaki,
// Ogita, Oishi and Rump), here with balanced base-256 integer digits.
//
// Kernel (persistent, one CTA per SM, tiles of 128 x 32 in static
// round-robin order): per 32-K stage one 3-D TMA copy per operand brings all
// S digit planes (64-byte rows, 64-byte swizzle).  Per 16 of K the MMA lane
// issues S tcgen05.mma kind::f16: digit s of A against digits 0..S-1-s of B
// (stacked in shared memory, so one MMA with N = 32 (S - s)) into the
// accumulator columns of groups s..S-1 (group w at column 32 w of a
// 256-column TMEM buffer; two buffers, so the epilogue folds one 128-K chunk
// while the MMAs fill the next).  Warp roles as in gemm_tc.cu: warp 0
// streams A, warp 10 B, warp 1 allocates TMEM and issues the MMAs, warps
// 2-9 fold (warp w: TMEM lane quarter w % 4 = 32 tile rows, 16 of the 32
// columns).  Every wait is bounded; a wait that gives up records
// GBBLAS_STATUS_TIMEOUT, and the CTA drains its copies and MMAs, frees TMEM
// and returns.
//
// Replaces the double-precision mtm of the reference (include/mtm.hpp:
// 208-267 with include/simd_loop.hpp:132-158): guarded under AUTO (the
// library's default for double where it is faster than the FP64 pipes),
// unguarded for GBBLAS_ACCURACY_FP64_DIGITS7 / 8.  Roofline: the tensor pipe and shared-memory
// bandwidth; 2*M*N*K algorithmic flops (the tensor cores execute
// S(S+1)/2 times that in BF16 products).
#include <cuda.h>
#include <cuda_bf16.h>

#include <climits>
#include <cstdlib>
#include <mutex>

#include "common.cuh"
#include "tc_ptx.cuh"
#include "tma_map.cuh"

namespace gbblas {
namespace {

using namespace tc;

constexpr int kBM = 128;  // tile rows (TMEM lanes)
constexpr int kBN = 32;   // tile columns per digit group
constexpr int kBK = 32;   // K per stage: one 64-byte row of BF16
constexpr int kEpiWarps = 8;
constexpr int kThreads = 32 * (3 + kEpiWarps);  // A producer, MMA, 8 epilogue, B producer
constexpr int kBProdWarp = 2 + kEpiWarps;
constexpr uint32_t kBufCols = 256;  // one TMEM buffer: S <= 8 groups x 32 columns
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s
constexpr size_t kSmemLimit = 232448;             // 227 KB per CTA
constexpr int kBadExp = INT_MAX;                  // scale marker: the row / column holds Inf or NaN
constexpr int kZeroExp = (int)0x80808080;          // scale of an all-zero row (the fill byte 0x80)

// S digits; G = 1 adds the guard plane (P = max(|D_0| - 1, 0), whose
// product sum bounds sum_k |a_ik||b_kj| from below) and its accumulator in
// TMEM column slot S.
template <int S, int G>
struct DgCfg {
  static_assert(S >= 4 && S + G <= 8, "4 to 8 digits, and a free TMEM slot for the guard");
  static constexpr int NP = S + G;              // planes per operand in the arena
  static constexpr uint32_t kATile = kBM * 64;  // one plane of A: 128 rows x 64 bytes
  static constexpr uint32_t kBTile = kBN * 64;  // one of B^T: 32 rows x 64 bytes
  static constexpr uint32_t kAStage = S * kATile;
  static constexpr uint32_t kBStage = S * kBTile;
  static constexpr uint32_t kStageBytes = kAStage + kBStage;
  // the guard planes' 32 K at the start of each chunk, in a slot of their own
  // (a lower bound over part of K is still a lower bound; the digit stages
  // keep their size, so three of them still fit)
  static constexpr uint32_t kGuardBytes = G ? kATile + kBTile : 0;
  // stages per TMEM chunk: a group's sum over the chunk stays below 2^24
  // (S * chunk * 2^14 with chunk = 128 K for S <= 7, 64 K for S = 8)
  static constexpr int kChunk = S <= 7 ? 4 : 2;
  // longest K: the 64-bit accumulators stay below 2^62 (each chunk adds
  // less than 2^48 to hi and to lo)
  static constexpr int64_t kMaxK = 1 << 20;
  static constexpr size_t kBarBytes = 256;
  static constexpr int kStagesFit = (int)((kSmemLimit - 1024 - kBarBytes - kGuardBytes) / kStageBytes);
  static constexpr int kStages = kStagesFit > 4 ? 4 : kStagesFit;
  static constexpr size_t kSmem = 1024 + (size_t)kStages * kStageBytes + kGuardBytes + kBarBytes;
  static_assert(kStages >= 2, "need a double-buffered stage ring");
  static_assert((uint64_t)S * kChunk * kBK * 16384 < (1u << 24), "chunk sums must stay exact in FP32");
  static_assert(kStageBytes % 1024 == 0, "stages stay 1024-byte aligned");
  static_assert((2 * 4 + 2 * 2 + 2 + 1) * 8 + 8 <= kBarBytes, "barrier area too small");
};

// One GEMM (device-side view).
struct DgProblem {
  int M, N, num_kt, tiles_m, tiles_n, total_tiles;
  int tile_begin, tile_end;  // this launch's tiles (a slice of 0 .. total_tiles - 1)
  double* C;
  int64_t rsc, csc;
  const int* ea;  // [rows of A, padded] row scales
  const int* eb;  // [columns of B, padded] column scales
  // guarded form: the 32 x 16 blocks the guard rejected (block b of tile t
  // = t * 8 + epilogue warp), recomputed on the FP64 pipes from A and B
  int* fix_count;
  int* fix_list;
  const double* A;
  const double* B;
  int64_t rsa, csa, rsb, csb;
  int64_t K;
};

// Guard: a block's digit result is kept when every output has
// sum_k P(a_ik) P(b_kj) >= 2^14, i.e. sum_k |a_ik||b_kj| >= 2^(e_i + f_j):
// the digit error (at most 9 2^-56 K 2^(e_i + f_j) with 7 digits) is then
// below 0.3 K eps sum_k |a_ik||b_kj| and, with the two final roundings,
// inside the FP64 pipes' bound 2 K eps (|A||B| + |C|).
constexpr int kGuardMin = 1 << 14;
constexpr int kGuardCap = 1 << 30;  // the guard sums saturate here (int32)

// ------------------------------------------------------ operand preparation
// Row scales: e[r] = the exponent frexp gives for max_k |src(r, k)| (so the
// row's magnitudes lie below 2^e), element (r, k) at src[r*rs + k*cs].  The
// array starts filled with the byte 0x80 (kZeroExp: an all-zero row); every
// CTA takes 32 rows x 256 K, reads them along whichever side is contiguous,
// and atomicMax-es its rows' exponents in - kBadExp (INT_MAX) for a row
// holding Inf or NaN, which then stays.
// One launch serves both operands: CTAs below a.blocks take A, the rest B
// (B^T: rows = columns of B); block 0 also clears the fix-up count.
constexpr int kScaleTK = 256;

// One operand of the preparation kernels (A, or B read as its transpose).
struct DgOperand {
  const double* src;
  int64_t rows, K, rs, cs;  // element (r, k) at src[r*rs + k*cs]
  int* e;                   // row scales
  __nv_bfloat16* out;       // digit planes
  int64_t plane_stride, pitch;
  int tiles_k;              // CTAs per 32 rows (K tiles of the kernel at hand)
  int blocks;               // CTAs of this operand
};

// Magnitudes compare as their bit patterns with the sign cleared (IEEE
// order), so the scan runs on the integer pipes: GB300's FP64 pipes would
// bound it (fabs / fmax / isfinite on doubles are FP64 instructions).
constexpr unsigned long long kAbsMask = 0x7FFFFFFFFFFFFFFFull;
constexpr unsigned long long kInfBits = 0x7FF0000000000000ull;  // |a| >= this: Inf or NaN

__device__ __forceinline__ unsigned long long abs_bits(const double* p) {
  return (unsigned long long)__double_as_longlong(__ldg(p)) & kAbsMask;
}

__global__ void __launch_bounds__(256) row_scale_kernel(const DgOperand oa, const DgOperand ob, int* fix_count) {
  __shared__ unsigned long long part_max[8][33];
  const bool is_a = (int)blockIdx.x < oa.blocks;
  const DgOperand& o = is_a ? oa : ob;
  const int blk = is_a ? (int)blockIdx.x : (int)blockIdx.x - oa.blocks;
  const double* __restrict__ src = o.src;
  const int64_t rows = o.rows, K = o.K, rs = o.rs, cs = o.cs;
  int* __restrict__ e_out = o.e;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (blockIdx.x == 0 && tid == 0 && fix_count) *fix_count = 0;
  const int64_t r0 = (int64_t)(blk / o.tiles_k) * 32, k0 = (int64_t)(blk % o.tiles_k) * kScaleTK;
  unsigned long long amax;  // largest |a| bit pattern; >= kInfBits marks Inf / NaN
  if (cs == 1) {
    // warp w: rows w, w+8, w+16, w+24; lanes along K
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = warp + 8 * i;
      unsigned long long m = 0;
      if (r0 + r < rows) {
        const double* p = src + (r0 + r) * rs + k0;
        unsigned long long v[kScaleTK / 32];
#pragma unroll
        for (int j = 0; j < kScaleTK / 32; ++j) v[j] = (k0 + lane + 32 * j < K) ? abs_bits(p + lane + 32 * j) : 0ull;
#pragma unroll
        for (int j = 0; j < kScaleTK / 32; ++j) m = v[j] > m ? v[j] : m;
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long x = __shfl_xor_sync(0xffffffffu, m, off);
        m = x > m ? x : m;
      }
      if (lane == 0) part_max[0][r] = m;
    }
    __syncthreads();
    if (tid >= 32) return;
    amax = part_max[0][lane];
  } else {
    // thread (slice w, row lane): 32 consecutive K of row lane; a warp reads
    // 32 consecutive rows at each k
    unsigned long long m = 0;
    if (r0 + lane < rows) {
      const double* p = src + (r0 + lane) * rs;
      unsigned long long v[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int64_t k = k0 + warp * 32 + j;
        v[j] = k < K ? abs_bits(p + k * cs) : 0ull;
      }
#pragma unroll
      for (int j = 0; j < 32; ++j) m = v[j] > m ? v[j] : m;
    }
    part_max[warp][lane] = m;
    __syncthreads();
    if (tid >= 32) return;
    for (int w = 1; w < 8; ++w) m = part_max[w][lane] > m ? part_max[w][lane] : m;
    amax = m;
  }
  // warp 0: one row per lane
  if (r0 + lane >= rows) return;
  if (amax >= kInfBits) {
    atomicMax(e_out + r0 + lane, kBadExp);
  } else if (amax != 0) {
    // the frexp exponent: |a| = f 2^e with f in [0.5, 1)
    const int ex = (int)(amax >> 52);
    const int e = ex != 0 ? ex - 1022 : (64 - __clzll((long long)amax)) - 1074;
    atomicMax(e_out + r0 + lane, e);
  }
}

// The scale of a row as the digit and GEMM kernels use it (kBadExp aside):
// an all-zero (or padding) row keeps kZeroExp and gets 0.
__device__ __forceinline__ int used_exp(int e) { return e == kZeroExp ? 0 : e; }

// Balanced base-256 digits of round(a * 2^(8S-1-e)), most significant first,
// from the bit pattern of a (|a| < 2^e; integer operations only).
template <int S>
__device__ __forceinline__ void f64_digits(double a, int e, int (&d)[S]) {
  if (e == kBadExp) {  // the row's outputs become NaN; its digits do not matter
#pragma unroll
    for (int s = 0; s < S; ++s) d[s] = 0;
    return;
  }
  const long long bits = __double_as_longlong(a);
  const int ex = (int)((bits >> 52) & 0x7ff);
  long long m = bits & ((1ll << 52) - 1);
  int p2;  // a = +-m * 2^p2
  if (ex != 0) {
    m |= 1ll << 52;
    p2 = ex - 1075;
  } else {
    p2 = -1074;
  }
  const int sh = p2 + 8 * S - 1 - e;  // F = m * 2^sh, rounded; sh <= 8S - 54 for |a| < 2^e
  long long F;
  if (m == 0)
    F = 0;
  else if (sh >= 0)
    F = m << sh;
  else if (sh > -63)
    F = (m + (1ll << (-sh - 1))) >> (-sh);
  else
    F = 0;
  if (bits < 0) F = -F;
#pragma unroll
  for (int s = S - 1; s > 0; --s) {
    const int lo = (int)(((F & 0xff) ^ 0x80) - 0x80);  // in [-128, 127]
    d[s] = lo;
    F = (F - lo) >> 8;  // exact: the low byte is now zero
  }
  d[0] = (int)F;  // in [-128, 128]
}

// Digit planes of one operand, written K-major into the arena: plane s of
// row r at out[s * plane_stride + r * pitch + k], for every padded row
// (< rows_pad) and padded k (< k_pad); zero outside rows x K.  G = 1 adds
// plane S, the guard plane max(|D_0| - 1, 0).  One launch for both
// operands (CTAs below a.blocks: A).  A CTA takes
// 32 rows x 32 K (8 KB of FP64 staged in shared memory, read along whichever
// side is contiguous); thread t then makes the digits of 4 consecutive K of
// one row and writes 8 bytes per plane.
template <int S, int G>
__global__ void __launch_bounds__(256) digits_kernel(const DgOperand oa, const DgOperand ob) {
  __shared__ double tile[32][33];
  const bool is_a = (int)blockIdx.x < oa.blocks;
  const DgOperand& o = is_a ? oa : ob;
  const int blk = is_a ? (int)blockIdx.x : (int)blockIdx.x - oa.blocks;
  const double* __restrict__ src = o.src;
  const int64_t rows = o.rows, K = o.K, rs = o.rs, cs = o.cs, plane_stride = o.plane_stride, pitch = o.pitch;
  const int* __restrict__ e_row = o.e;
  __nv_bfloat16* __restrict__ out = o.out;
  const int tid = threadIdx.x;
  const int64_t r0 = (int64_t)(blk / o.tiles_k) * 32, k0 = (int64_t)(blk % o.tiles_k) * 32;
  if (cs == 1) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int idx = tid + 256 * i, r = idx >> 5, k = idx & 31;
      tile[r][k] = (r0 + r < rows && k0 + k < K) ? __ldg(src + (r0 + r) * rs + k0 + k) : 0.0;
    }
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int idx = tid + 256 * i, r = idx & 31, k = idx >> 5;
      tile[r][k] = (r0 + r < rows && k0 + k < K) ? __ldg(src + (r0 + r) * rs + (k0 + k) * cs) : 0.0;
    }
  }
  __syncthreads();
  const int r = tid >> 3, kq = (tid & 7) * 4;
  const int e = e_row[r0 + r] == kBadExp ? kBadExp : used_exp(e_row[r0 + r]);
  int d[4][S];
#pragma unroll
  for (int j = 0; j < 4; ++j) f64_digits<S>(tile[r][kq + j], e, d[j]);
  __nv_bfloat16* dst = out + (r0 + r) * pitch + k0 + kq;
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const __nv_bfloat162 h01 = __floats2bfloat162_rn((float)d[0][s], (float)d[1][s]);  // exact: |d| <= 128
    const __nv_bfloat162 h23 = __floats2bfloat162_rn((float)d[2][s], (float)d[3][s]);
    uint2 w;
    w.x = *reinterpret_cast<const uint32_t*>(&h01);
    w.y = *reinterpret_cast<const uint32_t*>(&h23);
    *reinterpret_cast<uint2*>(dst + s * plane_stride) = w;
  }
  if constexpr (G) {  // guard plane: max(|D_0| - 1, 0) <= |x| 2^7
    auto g = [](int d) { return (float)max(abs(d) - 1, 0); };
    const __nv_bfloat162 h01 = __floats2bfloat162_rn(g(d[0][0]), g(d[1][0]));
    const __nv_bfloat162 h23 = __floats2bfloat162_rn(g(d[2][0]), g(d[3][0]));
    uint2 w;
    w.x = *reinterpret_cast<const uint32_t*>(&h01);
    w.y = *reinterpret_cast<const uint32_t*>(&h23);
    *reinterpret_cast<uint2*>(dst + S * plane_stride) = w;
  }
}

// ---------------------------------------------------------------- GEMM
// (hi 2^32 + lo) 2^e2 rounded once to the nearest double (ties to even),
// with integer operations only: the 128-bit value's top 53 bits and the
// round bit, the scale added to the exponent field.  A result below the
// normal range (or above it) goes through ldexp, so it may round twice.
__device__ __forceinline__ double i128_scaled_to_double(long long hi, long long lo, int e2) {
  const __int128 v = ((__int128)hi << 32) + (__int128)lo;
  if (v == 0) return 0.0;
  const bool neg = v < 0;
  const unsigned __int128 m = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
  const unsigned long long mh = (unsigned long long)(m >> 64), ml = (unsigned long long)m;
  const int n = mh ? 128 - __clzll((long long)mh) : 64 - __clzll((long long)ml);  // bit length, >= 1
  unsigned long long mant;  // 2^52 <= mant < 2^53
  int exp2;                 // value = mant 2^exp2
  if (n <= 53) {
    mant = ml << (53 - n);
    exp2 = e2 - (53 - n);
  } else {
    const int sh = n - 53;
    mant = (unsigned long long)(m >> sh);
    const unsigned __int128 rem = m & ((((unsigned __int128)1) << sh) - 1);
    const unsigned __int128 half = ((unsigned __int128)1) << (sh - 1);
    exp2 = e2 + sh;
    if (rem > half || (rem == half && (mant & 1ull))) {
      ++mant;
      if (mant == (1ull << 53)) {
        mant >>= 1;
        ++exp2;
      }
    }
  }
  const int be = exp2 + 52 + 1023;  // biased exponent of mant 2^exp2
  if (be <= 0 || be >= 2047) return ldexp(neg ? -(double)mant : (double)mant, exp2);
  return __longlong_as_double((neg ? (long long)(1ull << 63) : 0ll) | ((long long)be << 52) |
                              (long long)(mant & ((1ull << 52) - 1)));
}

// Output tile t (static round-robin over the CTAs): grouped raster, 8 tile
// rows per band, so the CTAs running at one time share A's and B's digit
// tiles in L2.
__device__ __forceinline__ void dg_tile(const DgProblem& p, int t, int& m0, int& n0) {
  constexpr int kGroup = 8;
  const int group_span = kGroup * p.tiles_n;
  const int g = t / group_span;
  const int first_m = g * kGroup;
  const int gm = min(p.tiles_m - first_m, kGroup);
  const int in_g = t % group_span;
  m0 = (first_m + in_g % gm) * kBM;
  n0 = (in_g / gm) * kBN;
}

template <int S, int G>
__global__ void __launch_bounds__(kThreads, 1)
    dgemm_digits_kernel(const __grid_constant__ CUtensorMap tm_a, const __grid_constant__ CUtensorMap tm_b,
                        const __grid_constant__ CUtensorMap tm_ga, const __grid_constant__ CUtensorMap tm_gb,
                        const DgProblem p, int* __restrict__ err) {
  using CF = DgCfg<S, G>;
  constexpr int ST = CF::kStages;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  // stage st: A digit planes 0..S-1 (8 KB each), then B's (2 KB each); after
  // the stages the guard slot (G: A's guard tile, then B's)
  auto a_tile = [&](int st, int d) { return smem + (size_t)st * CF::kStageBytes + (size_t)d * CF::kATile; };
  auto b_tile = [&](int st) { return smem + (size_t)st * CF::kStageBytes + CF::kAStage; };
  unsigned char* guard_a = smem + (size_t)ST * CF::kStageBytes;
  unsigned char* guard_b = guard_a + CF::kATile;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)ST * CF::kStageBytes + CF::kGuardBytes);
  uint64_t* full = bars;        // [ST]  TMA -> MMA (both producers)
  uint64_t* empty = full + 4;   // [ST]  MMA -> TMA
  uint64_t* tfull = empty + 4;  // [2]   MMA -> epilogue: chunk in TMEM buffer b
  uint64_t* tempty = tfull + 2;  // [2]  epilogue -> MMA: buffer b drained
  uint64_t* gfull = tempty + 2;  // [1]  TMA -> MMA: the guard slot (both producers)
  uint64_t* gempty = gfull + 1;  // [1]  MMA -> TMA
  uint64_t* accf = gempty + 1;   // [1]  every MMA of this CTA finished
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accf + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      mbar_init(&full[s], 2);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], kEpiWarps);
    }
    mbar_init(gfull, 2);
    mbar_init(gempty, 1);
    mbar_init(accf, 1);
    *abort_flag = 0;
    fence_mbar_init();
    prefetch_tensormap(&tm_a);
    prefetch_tensormap(&tm_b);
    if (G) {
      prefetch_tensormap(&tm_ga);
      prefetch_tensormap(&tm_gb);
    }
  }
  if (warp == 1) {
    tmem_alloc(tmem_slot, 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  auto fail = [&]() {
    *abort_flag = 1;
    atomicExch(err, (int)GBBLAS_STATUS_TIMEOUT);
  };

  int issued = 0;  // A producer: stages whose copies were issued
  if ((warp == 0 || warp == kBProdWarp) && lane == 0) {
    // producers: warp 0 brings A's digit planes, warp 10 B's, into the same stages
    const bool is_a = warp == 0;
    int n_issued = 0, g_issued = 0;
    bool stop = false;
    for (int t = p.tile_begin + (int)blockIdx.x; t < p.tile_end && !stop; t += gridDim.x) {
      int m0, n0;
      dg_tile(p, t, m0, n0);
      for (int kt = 0; kt < p.num_kt; ++kt) {
        if (G && kt % CF::kChunk == 0) {
          // the guard planes' first 32 K of this chunk, once the MMAs of the
          // previous chunk's guard product have read the slot
          if (g_issued > 0 && !mbar_wait_bounded(gempty, (g_issued - 1) & 1, abort_flag, kWaitLimitNs)) {
            fail();
            stop = true;
            break;
          }
          if (is_a) {
            mbar_arrive_expect_tx(gfull, CF::kATile);
            tma_load_3d(guard_a, &tm_ga, gfull, kt * kBK, m0, 0);
          } else {
            mbar_arrive_expect_tx(gfull, CF::kBTile);
            tma_load_3d(guard_b, &tm_gb, gfull, kt * kBK, n0, 0);
          }
          ++g_issued;
        }
        const int s = n_issued % ST, round = n_issued / ST;
        if (round > 0 && !mbar_wait_bounded(&empty[s], (round - 1) & 1, abort_flag, kWaitLimitNs)) {
          fail();
          stop = true;
          break;
        }
        if (is_a) {
          mbar_arrive_expect_tx(&full[s], CF::kAStage);
          tma_load_3d(a_tile(s, 0), &tm_a, &full[s], kt * kBK, m0, 0);
        } else {
          mbar_arrive_expect_tx(&full[s], CF::kBStage);
          tma_load_3d(b_tile(s), &tm_b, &full[s], kt * kBK, n0, 0);
        }
        ++n_issued;
      }
    }
    if (is_a) issued = n_issued;
  } else if (warp == 1) {
    if (lane == 0) {
      int consumed = 0, chunk_g = 0, g_used = 0;
      bool stop = false;
      for (int t = p.tile_begin + (int)blockIdx.x; t < p.tile_end && !stop; t += gridDim.x) {
        for (int kt = 0; kt < p.num_kt; ++kt) {
          const int s = consumed % ST, round = consumed / ST;
          const bool chunk_first = (kt % CF::kChunk) == 0;
          const bool chunk_last = ((kt + 1) % CF::kChunk) == 0 || kt + 1 == p.num_kt;
          if (chunk_first) ++chunk_g;
          const int chunk = chunk_g - 1, b = chunk & 1;
          if (chunk_first && chunk >= 2) {  // buffer b drained by the epilogue
            if (!mbar_wait_bounded(&tempty[b], ((chunk >> 1) - 1) & 1, abort_flag, kWaitLimitNs)) {
              fail();
              stop = true;
              break;
            }
            tc_fence_after();
          }
          if (!mbar_wait_bounded(&full[s], round & 1, abort_flag, kWaitLimitNs)) {
            fail();
            stop = true;
            break;
          }
          tc_fence_after();
          const uint32_t acc = tmem + (uint32_t)b * kBufCols;
          const uint32_t b0 = smem_u32(b_tile(s));
          if (G && chunk_first) {
            // guard plane x guard plane over the chunk's first 32 K -> slot S
            if (!mbar_wait_bounded(gfull, g_used & 1, abort_flag, kWaitLimitNs)) {
              fail();
              stop = true;
              break;
            }
            tc_fence_after();
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk)
              mma_f16(acc + 32u * S, sw64_kmajor_desc(smem_u32(guard_a) + kk * 32),
                      sw64_kmajor_desc(smem_u32(guard_b) + kk * 32), idesc_bf16_f32(kBM, kBN), kk == 0 ? 0u : 1u);
            mma_commit(gempty);
            ++g_used;
          }
#pragma unroll
          for (int kk = 0; kk < kBK / 16; ++kk) {
            const uint32_t off = kk * 32;  // 16 BF16 of K inside the swizzled 64-byte row
#pragma unroll
            for (int d = 0; d < S; ++d) {
              // digit d of A x digits 0..S-1-d of B (stacked: N = 32 (S - d))
              // -> groups d..S-1; the first MMA of a chunk (N = 32 S) clears all
              mma_f16(acc + 32u * d, sw64_kmajor_desc(smem_u32(a_tile(s, d)) + off), sw64_kmajor_desc(b0 + off),
                      idesc_bf16_f32(kBM, kBN * (S - d)), (chunk_first && kk == 0 && d == 0) ? 0u : 1u);
            }
          }
          mma_commit(&empty[s]);
          if (chunk_last) mma_commit(&tfull[b]);
          ++consumed;
        }
      }
      mma_commit(accf);
      if (*abort_flag) {
        int never = 0;
        (void)mbar_wait_bounded(accf, 0, &never, kWaitLimitNs);
      }
    }
  } else if (warp >= 2 && warp < 2 + kEpiWarps) {
    // epilogue: TMEM lane quarter q = warp % 4 (tile rows 32q..32q+31), 16
    // columns (half h) of each group's 32
    const int q = warp & 3, h = (warp - 2) >> 2;
    const uint32_t trow = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(16 * h);
    const int nchunks = (p.num_kt + CF::kChunk - 1) / CF::kChunk;
    int chunk_g = 0;
    bool ok = true;
    for (int t = p.tile_begin + (int)blockIdx.x; t < p.tile_end && ok; t += gridDim.x) {
      int m0, n0;
      dg_tile(p, t, m0, n0);
      // sum_w G_w 2^(8(S-1-w)) = hi 2^32 + lo, exactly: groups w < S-4 go
      // into hi (shifted by 8(S-5-w)), the last four into lo (8(S-1-w))
      long long hi[16], lo[16];
      int gsum[16];  // guard: sum of P(a) P(b) (saturating)
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        hi[j] = lo[j] = 0;
        gsum[j] = 0;
      }
      auto fold = [&](int d, const float (&v)[16]) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const long long g = (long long)__float2int_rn(v[j]);  // exact: an integer below 2^24
          if (d < S - 4)
            hi[j] += g << (8 * (S - 5 - d));
          else
            lo[j] += g << (8 * (S - 1 - d));
        }
      };
      auto take = [&](int slot, const float (&v)[16]) {
        if (slot < S) {
          fold(slot, v);
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) gsum[j] = min(gsum[j] + __float2int_rn(v[j]), kGuardCap);
        }
      };
      for (int c = 0; c < nchunks; ++c, ++chunk_g) {
        const int b = chunk_g & 1;
        const bool ready =
            __all_sync(0xffffffffu, mbar_wait_bounded(&tfull[b], (chunk_g >> 1) & 1, abort_flag, kWaitLimitNs));
        if (!ready) {
          if (lane == 0) fail();
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t tb = trow + (uint32_t)b * kBufCols;
#pragma unroll
        for (int d = 0; d < S + G; d += 2) {  // slots d, d + 1 (slot S: the guard)
          float v0[16], v1[16];
          tmem_ld16(tb + 32u * d, v0);
          if (d + 1 < S + G) tmem_ld16(tb + 32u * (d + 1), v1);
          tmem_ld_wait();
          take(d, v0);
          if (d + 1 < S + G) take(d + 1, v1);
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&tempty[b]);
      }
      if (!ok) break;
      if (__shfl_sync(0xffffffffu, *abort_flag, 0)) break;
      const int row = m0 + q * 32 + lane;
      if constexpr (G) {
        // every output of this warp's 32 x 16 block must pass, else the
        // block goes to the FP64 fix-up and C is left alone here
        bool pass = true;
        if (row < p.M) {
#pragma unroll
          for (int j = 0; j < 16; ++j)
            if (n0 + 16 * h + j < p.N && gsum[j] < kGuardMin) pass = false;
        }
        if (!__all_sync(0xffffffffu, pass)) {
          if (lane == 0) p.fix_list[atomicAdd(p.fix_count, 1)] = t * kEpiWarps + (warp - 2);
          continue;
        }
      }
      if (row < p.M) {
        // C += r for the thread's 16 outputs: all loads first, then all
        // stores (the outputs are distinct: a valid C has non-zero strides),
        // 16-byte accesses where the row segment is contiguous and aligned
        const int ei = p.ea[row] == kBadExp ? kBadExp : used_exp(p.ea[row]);
        double* crow = p.C + (int64_t)row * p.rsc;
        const int cn = n0 + 16 * h;
        const int nv = min(16, p.N - cn);
        const bool vec = p.csc == 1 && nv == 16 && (reinterpret_cast<uintptr_t>(crow + cn) & 15) == 0;
        double cv[16];
        int ej[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int e = j < nv ? p.eb[cn + j] : 0;
          ej[j] = e == kBadExp ? kBadExp : used_exp(e);
        }
        if (vec) {
#pragma unroll
          for (int j = 0; j < 16; j += 2) {
            const double2 t = *reinterpret_cast<const double2*>(crow + cn + j);
            cv[j] = t.x;
            cv[j + 1] = t.y;
          }
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) cv[j] = j < nv ? crow[(int64_t)(cn + j) * p.csc] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          // hi 2^32 + lo in units of 2^(e_i + f_j - 14 - 8(S-1))
          if (ei == kBadExp || ej[j] == kBadExp)
            cv[j] += __longlong_as_double(0x7ff8000000000000ll);  // NaN
          else
            cv[j] += i128_scaled_to_double(hi[j], lo[j], ei + ej[j] - 14 - 8 * (S - 1));
        }
        if (vec) {
#pragma unroll
          for (int j = 0; j < 16; j += 2) *reinterpret_cast<double2*>(crow + cn + j) = make_double2(cv[j], cv[j + 1]);
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j)
            if (j < nv) crow[(int64_t)(cn + j) * p.csc] = cv[j];
        }
      }
    }
  }

  // ---- teardown: drain in-flight copies if the pipeline stopped early, make
  // sure every MMA finished (warp 1 waited on accf after an abort), free TMEM
  if (warp == 0 && lane == 0 && *abort_flag) {
    int never = 0;
    const int from = issued > ST ? issued - ST : 0;
    for (int k = from; k < issued; ++k) (void)mbar_wait_bounded(&full[k % ST], (k / ST) & 1, &never, kWaitLimitNs / 2);
    // copies of B the A producer did not match complete on no barrier it
    // waits for: give them 100 us to land
    const uint64_t t0 = global_timer_ns();
    while (global_timer_ns() - t0 < 100000ull) {
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// FP64-pipe recomputation of the blocks the guard rejected: CTA i takes
// list entries i, i + grid, ...; block (tile t, epilogue warp w) covers tile
// rows 32 (w % 4) .. +31 and columns 16 ((w - 2) / 4) .. +15; thread
// (row lane, column pair) sums its two outputs over k in order with fused
// multiply-adds and adds them into C (the FP64 FMA kernel's arithmetic).
__global__ void __launch_bounds__(256) dgemm_fixup_kernel(const DgProblem p) {
  const int n = *p.fix_count;
  const int lane = threadIdx.x & 31, pair = threadIdx.x >> 5;
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const int id = p.fix_list[i];
    const int t = id / kEpiWarps, w = 2 + id % kEpiWarps;
    int m0, n0;
    dg_tile(p, t, m0, n0);
    const int row = m0 + 32 * (w & 3) + lane;
    const int c0 = n0 + 16 * ((w - 2) >> 2) + 2 * pair;
    if (row >= p.M) continue;
    const double* a = p.A + (int64_t)row * p.rsa;
    double s0 = 0.0, s1 = 0.0;
    const bool has1 = c0 + 1 < p.N;
    if (c0 < p.N) {
      const double* b0 = p.B + (int64_t)c0 * p.csb;
      for (int64_t k = 0; k < p.K; ++k) {
        const double av = a[k * p.csa];
        s0 = fma(av, b0[k * p.rsb], s0);
        if (has1) s1 = fma(av, b0[k * p.rsb + p.csb], s1);
      }
      p.C[(int64_t)row * p.rsc + (int64_t)c0 * p.csc] += s0;
      if (has1) p.C[(int64_t)row * p.rsc + (int64_t)(c0 + 1) * p.csc] += s1;
    }
  }
}

// ------------------------------------------------------------ host side
inline int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }
inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

template <int S, int G>
void dg_setup(DeviceCtx* c) {
  static std::mutex mu;
  static bool done[64] = {false};
  std::lock_guard<std::mutex> lk(mu);
  if (!done[c->device & 63]) {
    cudaFuncSetAttribute(dgemm_digits_kernel<S, G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)DgCfg<S, G>::kSmem);
    done[c->device & 63] = true;
  }
}

template <int S, int G>
gbblas_status launch_digits(DeviceCtx* c, int64_t M, int64_t N, int64_t K, const double* A, int64_t rsa,
                            int64_t csa, const double* B, int64_t rsb, int64_t csb, double* C, int64_t rsc,
                            int64_t csc, cudaStream_t stream, int max_ctas, int slices) {
  using CF = DgCfg<S, G>;
  constexpr int NP = CF::NP;
  if (K > CF::kMaxK) {
    set_error("dgemm (FP64 digits): K = %lld exceeds %lld", (long long)K, (long long)CF::kMaxK);
    return GBBLAS_STATUS_NOT_SUPPORTED;
  }
  if (M > (1 << 30) || N > (1 << 30)) {
    set_error("dgemm (FP64 digits): problem too large for the tile grid");
    return GBBLAS_STATUS_NOT_SUPPORTED;
  }
  const int64_t Mp = round_up(M, kBM), Np = round_up(N, kBN), Kp = round_up(K, kBK);
  const size_t off_ea = kScratchZeroBytes;
  const size_t off_eb = off_ea + align256(sizeof(int) * (size_t)Mp);
  const size_t off_a = off_eb + align256(sizeof(int) * (size_t)Np);
  const size_t a_plane = (size_t)(Mp * Kp), b_plane = (size_t)(Np * Kp);
  const size_t off_b = off_a + align256((size_t)NP * a_plane * sizeof(__nv_bfloat16));
  const int64_t tiles = (Mp / kBM) * (Np / kBN);
  const size_t off_fix = off_b + align256((size_t)NP * b_plane * sizeof(__nv_bfloat16));
  const size_t bytes = off_fix + (G ? align256(sizeof(int) * (size_t)(1 + tiles * kEpiWarps)) : 0);
  void* scratch = nullptr;
  GB_TRY(get_scratch(c, stream, bytes, &scratch));
  char* base = static_cast<char*>(scratch);
  int* ea = reinterpret_cast<int*>(base + off_ea);
  int* eb = reinterpret_cast<int*>(base + off_eb);
  auto* da = reinterpret_cast<__nv_bfloat16*>(base + off_a);
  auto* db = reinterpret_cast<__nv_bfloat16*>(base + off_b);
  int* err = reinterpret_cast<int*>(base + kErrWordOffset);

  // scales: rows of A over K; columns of B (element (n, k) = B[k*rsb + n*csb])
  int* fix_count = G ? reinterpret_cast<int*>(base + off_fix) : nullptr;
  GB_CUDA_TRY(cudaMemsetAsync(ea, 0x80, off_a - off_ea, stream));  // kZeroExp everywhere (ea and eb)
  const int stk = (int)((K + kScaleTK - 1) / kScaleTK);
  const int tiles_k = (int)(Kp / 32);
  DgOperand oa{A, M, K, rsa, csa, ea, da, (int64_t)a_plane, Kp, stk, (int)((Mp / 32) * stk)};
  DgOperand ob{B, N, K, csb, rsb, eb, db, (int64_t)b_plane, Kp, stk, (int)((Np / 32) * stk)};
  if ((double)(Mp + Np) / 32 * tiles_k >= 2.0e9) {
    set_error("dgemm (FP64 digits): operands too large for one preparation launch");
    return GBBLAS_STATUS_NOT_SUPPORTED;
  }
  row_scale_kernel<<<(unsigned)(oa.blocks + ob.blocks), 256, 0, stream>>>(oa, ob, fix_count);
  GB_TRY(check_launch("row_scale_kernel"));
  oa.tiles_k = ob.tiles_k = tiles_k;
  oa.blocks = (int)((Mp / 32) * tiles_k);
  ob.blocks = (int)((Np / 32) * tiles_k);
  digits_kernel<S, G><<<(unsigned)(oa.blocks + ob.blocks), 256, 0, stream>>>(oa, ob);
  GB_TRY(check_launch("digits_kernel"));

  CUtensorMap ma, mb;
  GB_TRY(make_map(&ma, da, (uint64_t)Mp, (uint64_t)Kp, (uint64_t)S, kBM, false, 64));
  GB_TRY(make_map(&mb, db, (uint64_t)Np, (uint64_t)Kp, (uint64_t)S, kBN, false, 64));
  CUtensorMap mga = ma, mgb = mb;  // the guard planes (plane S of each arena)
  if (G) {
    GB_TRY(make_map(&mga, da + (size_t)S * a_plane, (uint64_t)Mp, (uint64_t)Kp, 1, kBM, false, 64));
    GB_TRY(make_map(&mgb, db + (size_t)S * b_plane, (uint64_t)Np, (uint64_t)Kp, 1, kBN, false, 64));
  }
  DgProblem p;
  p.M = (int)M;
  p.N = (int)N;
  p.num_kt = (int)(Kp / kBK);
  p.tiles_m = (int)(Mp / kBM);
  p.tiles_n = (int)(Np / kBN);
  if (tiles * kEpiWarps >= (1ll << 31)) {
    set_error("dgemm (FP64 digits): too many tiles");
    return GBBLAS_STATUS_NOT_SUPPORTED;
  }
  p.total_tiles = (int)tiles;
  p.C = C;
  p.rsc = rsc;
  p.csc = csc;
  p.ea = ea;
  p.eb = eb;
  p.fix_count = fix_count;  // cleared by row_scale_kernel
  p.fix_list = G ? fix_count + 1 : nullptr;
  p.A = A;
  p.B = B;
  p.rsa = rsa;
  p.csa = csa;
  p.rsb = rsb;
  p.csb = csb;
  p.K = K;
  dg_setup<S, G>(c);
  int grid = (int)std::min<int64_t>(tiles, c->num_sms);
  if (max_ctas > 0 && grid > max_ctas) grid = max_ctas;
  // slices: consecutive tile ranges of whole waves, one launch each (higher-
  // priority work on other streams gets the SMs between them)
  const int64_t waves = (tiles + grid - 1) / grid;
  const int64_t nsl = std::max<int64_t>(1, std::min<int64_t>(slices, waves));
  for (int64_t sl = 0; sl < nsl; ++sl) {
    p.tile_begin = (int)(grid * (waves * sl / nsl));
    p.tile_end = (int)std::min<int64_t>(tiles, grid * (waves * (sl + 1) / nsl));
    dgemm_digits_kernel<S, G><<<grid, kThreads, CF::kSmem, stream>>>(ma, mb, mga, mgb, p, err);
    GB_TRY(check_launch("dgemm_digits_kernel"));
  }
  if constexpr (G) {
    // the rejected blocks (usually none: the kernel reads the count and returns)
    dgemm_fixup_kernel<<<(unsigned)(max_ctas > 0 ? std::min(max_ctas, 2 * c->num_sms) : 2 * c->num_sms), 256, 0,
                         stream>>>(p);
    GB_TRY(check_launch("dgemm_fixup_kernel"));
  }
  return GBBLAS_STATUS_SUCCESS;
}

}  // namespace

int dgemm_digits_count(gbblas_accuracy acc) {
  return acc == GBBLAS_ACCURACY_FP64_DIGITS7 ? 7 : (acc == GBBLAS_ACCURACY_FP64_DIGITS8 ? 8 : 0);
}

int64_t dgemm_digits_max_k(int digits) { return digits == 8 ? DgCfg<8, 0>::kMaxK : DgCfg<7, 0>::kMaxK; }

// Scratch one call takes (scales, digit planes, fix-up list), as launch_digits lays it out.
size_t dgemm_digits_scratch_bytes(int digits, bool guarded, int64_t M, int64_t N, int64_t K) {
  const int64_t Mp = round_up(M, kBM), Np = round_up(N, kBN), Kp = round_up(K, kBK);
  const int64_t np = digits + (guarded ? 1 : 0);
  const int64_t tiles = (Mp / kBM) * (Np / kBN);
  return kScratchZeroBytes + align256(sizeof(int) * (size_t)Mp) + align256(sizeof(int) * (size_t)Np) +
         align256((size_t)(np * Mp * Kp) * 2) + align256((size_t)(np * Np * Kp) * 2) +
         (guarded ? align256(sizeof(int) * (size_t)(1 + tiles * kEpiWarps)) : 0);
}

void dgemm_digits_prepare(DeviceCtx* c) {
  dg_setup<7, 0>(c);
  dg_setup<8, 0>(c);
  dg_setup<7, 1>(c);
}

gbblas_status launch_dgemm_digits(DeviceCtx* c, int digits, bool guarded, int64_t M, int64_t N, int64_t K,
                                  const double* A, int64_t rsa, int64_t csa, const double* B, int64_t rsb,
                                  int64_t csb, double* C, int64_t rsc, int64_t csc, cudaStream_t stream, int max_ctas,
                                  int slices) {
  if (M == 0 || N == 0 || K == 0) return GBBLAS_STATUS_SUCCESS;
  if (guarded && digits == 7)
    return launch_digits<7, 1>(c, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, stream, max_ctas, slices);
  if (!guarded && digits == 7)
    return launch_digits<7, 0>(c, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, stream, max_ctas, slices);
  if (!guarded && digits == 8)
    return launch_digits<8, 0>(c, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, stream, max_ctas, slices);
  set_error("dgemm (FP64 digits): %d digits%s not supported", digits, guarded ? " with the guard" : "");
  return GBBLAS_STATUS_INVALID_VALUE;
}

}  // namespace gbblas
