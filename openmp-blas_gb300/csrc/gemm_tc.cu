// gemm_tc.cu - GEMM on the 5th-generation tensor cores, single and grouped:
// FP32-accurate (split-BF16; split-FP16 on scaled operands) and low-accuracy
// (FP8-E4M3, block-scaled).
// C += A * B for float A, B, C of any layout; a group is any number of
// independent problems of any shapes.
//
//   1. Operand preparation, written K-major (A as M x K, B as its transpose
//      N x K) into one arena per operand kind: all problems' rows stacked,
//      one common K pitch.  One pair of TMA tensor maps then covers every
//      problem of the group.
//      split-BF16: every FP32 element a becomes P BF16 pieces
//        p0 = bf16_rn(a), p1 = bf16_rn(a - p0), p2 = bf16_rn(a - p0 - p1),
//        piece planes one after another (split_rows_kernel, a warp per row,
//        where K is contiguous; prep_group_kernel's tiles otherwise).
//      split-FP16: every row of A / column of B is scaled by 2^(15 - e), e
//        the frexp exponent of its largest magnitude, and split
//        h = fp16_rn(v), l = fp16_rn(v - h); the epilogue multiplies by
//        2^(e_i + f_j - 30) again.  K contiguous: f16_row_prep_kernel, a CTA
//        per row, does both in one read; rows contiguous: the exponents from
//        f16_col_scale_kernel's column reduction, the pieces from
//        prep_group_kernel; other layouts: f16_scale_kernel and
//        prep_group_kernel on tiles.  All routes give the same bits.
//      prep_group_kernel, FP8: every 128-element K-block of a row becomes
//        128 E4M3 values and one power-of-two scale, kept as its UE8M0
//        exponent byte in 512-byte atoms (128 rows of one K-block) beside
//        the arena, laid out the way tcgen05.cp moves them into TMEM.
//   2. gemm_split_kernel (persistent, one CTA per SM): a device-side tile
//      scheduler hands out 128 x 128 output tiles of all problems (largest K
//      first) through an atomic counter.  K is walked in chunks: each chunk
//      accumulates in one of two TMEM buffers while the epilogue warps fold
//      the previous chunk into FP32 registers with round-to-nearest adds; the
//      registers go into C once per tile.  The chunk buffers carry over from
//      tile to tile, so a tile's epilogue overlaps the next tile's MMAs.
//      Split-BF16 (tcgen05.mma kind::f16, BF16 in, FP32 accumulate): C += sum
//      of the piece products p_i(A) p_j(B) with i + j < P, into two TMEM
//      accumulators - p0*p0 alone, and every smaller product together (so
//      small terms are summed at their own scale); chunks of 512 K (P = 2) or
//      128 K (P = 3): the tensor core's own accumulation over long K is
//      measurably less accurate than FP32.
//        P = 2 ("bf16x3"):  p0p0 + (p0p1 + p1p0)                     3 MMAs
//        P = 3 ("bf16x6"):  p0p0 + (p0p1 + p1p0 + p0p2 + p1p1 + p2p0) 6 MMAs
//      Three pieces hold all 24 significand bits of an FP32 value and the
//      dropped products are below 2^-23 of |a||b|: bf16x6 is at least as
//      accurate as FP32 FMA arithmetic.  bf16x3 keeps about 16 bits.
//      FP8 (tcgen05.mma kind::mxf8f6f4 block_scale, E4M3 in, FP32
//      accumulate): the tensor core applies the row and column block scales
//      itself (UE8M0 scales copied from the stage into TMEM by tcgen05.cp
//      ahead of each slice's MMAs); chunks of 512 K as for the split.
//
// Warp roles (320 threads; FP8: 192):
//   warp 0      tile scheduler + TMA producer: takes the next tile from the
//               global counter, publishes it in a shared-memory tile ring,
//               then streams its K slices (128 bytes of K of all P pieces of
//               A and of B: one 3-D tiled bulk copy per operand, 128-byte
//               swizzle; FP8 adds the two 512-byte scale atoms) into a
//               stage ring;
//   warp 1      allocates TMEM and issues the MMAs (one elected lane);
//               tcgen05.commit frees a stage once its MMAs have read it and
//               signals a TMEM chunk buffer as full;
//   warps 2-9   epilogue: tcgen05.ld each finished chunk (warp w reads TMEM
//   (FP8: 2-5)  lanes 32*(w%4)..+31 = tile rows; with 8 warps, warps 2-5
//               take the first 64 columns, 6-9 the other 64) into FP32
//               registers, release the buffer, add the registers into C
//               (single CTAs: 32 x 32 blocks staged in shared memory and
//               added by TMA reduce-add stores where C's layout allows).
// Every mbarrier wait is bounded (2 s by %globaltimer); a wait that gives up
// records GBBLAS_STATUS_TIMEOUT in the stream's error word, the CTA drains
// its in-flight copies (bounded again), lets its MMAs finish, frees TMEM and
// returns.
//
// Replaces the FP32 path of the reference's mtm (include/mtm.hpp:116-206)
// when the caller asks for GBBLAS_ACCURACY_BF16X3 / BF16X6 / FP8, and runs
// the batched form of it.  Roofline: tensor pipe; 2*M*N*K algorithmic flops
// per problem (split-BF16 issues 3 or 6 times that in BF16 products).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "tc_ptx.cuh"
#include "tma_map.cuh"

namespace gbblas {
namespace {

using namespace tc;

constexpr int kBM = 128;
constexpr int kBN = 128;
constexpr int kBK = 64;  // K padding of the BF16 arenas: 64 bf16 = one 128-byte row
// K slices folded into FP32 registers per chunk: three-product split every
// 512 of K, six-product split every 128 (the tensor core's accumulation over
// a 512-K chunk made the six-product result's max relative error worse than
// plain FP32 on operands spanning 2^+-10; at 128 it is 5x better, within 1 %
// of the speed), FP8 every 512 (four scale blocks).
constexpr int kChunkTiles3 = 8;
constexpr int kChunkTiles6 = 2;
// The FP16 split (22 of 24 bits) folds every 128 of K as well.  Folding
// every 256 measured 2.3 % faster at 8192^3 (458 -> 469 TFLOP/s) with
// sampled errors still 3-10x below plain FP32's, but over all entries of a
// 1024^3 product of wide-range operands its largest elementwise relative
// error (0.217, at an entry near zero) exceeded plain FP32's (0.133).
constexpr int kChunkTilesF16 = 2;
constexpr int kChunkTilesFp8 = 2;  // FP8 stages are 256 K deep
constexpr int kTileRing = 4;     // tiles in flight between scheduler and consumers
constexpr int kMaxStages = 8;    // operand stages in flight (as many as shared memory holds, up to this)
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s
constexpr size_t kSmemLimit = 232448;             // 227 KB per CTA

// Kernel modes: 2 / 3 = FP32 split into that many BF16 pieces; kModeFp8 =
// E4M3 operands with one power-of-two scale per 128 elements along K;
// kModeF16 = FP32 scaled by a power of two per row of A / column of B and
// split into two FP16 pieces (11 significand bits each), three products.
constexpr int kModeFp8 = 8;
constexpr int kModeF16 = 12;
// kModeF16 with the AUTO guard (host-side plan mode; the kernels run kModeF16)
constexpr int kModeF16Guard = kTcModeF16Guard;

template <int MODE>
struct ModeTraits {
  static constexpr bool fp8 = MODE == kModeFp8;
  static constexpr bool f16 = MODE == kModeF16;
  static constexpr int P = fp8 ? 1 : (f16 ? 2 : MODE);  // operand planes per operand
  // Bytes of K per operand row in one K sub-tile (128-byte swizzle).  The
  // six-product split measured slower with 64-byte rows (32-K stages, 4 in
  // shared memory instead of 2): 245 vs 269 TFLOP/s at 8192^3.
  static constexpr int kRowBytes = 128;
  static constexpr int kKSteps = kRowBytes / 32;  // MMAs of 32 bytes of K per sub-tile
  // K sub-tiles per stage: one for the split, two for FP8 (256 E4M3: twice
  // the MMAs per barrier round trip, the per-stage hand-offs being what
  // bounds the four-MMA FP8 stage).
  static constexpr int kSub = fp8 ? 2 : 1;
  static constexpr int kBKe = fp8 ? 128 * kSub : kRowBytes / 2;  // K elements per stage
  // slices per TMEM chunk (the six-product and the FP16 split every 128 of
  // K, the three-product split and FP8 every 512)
  static constexpr int kChunk = fp8 ? kChunkTilesFp8 : (MODE == 2 ? kChunkTiles3 : (f16 ? kChunkTilesF16 : kChunkTiles6));
  // Epilogue warps: 8 for the split, each 32 tile rows x 64 columns (with
  // 128 FP32 accumulators per thread the kernel ran out of registers and
  // spilled); 4 for FP8, each 32 rows x 128 columns (no spills).
  static constexpr int kEpiWarps = fp8 ? 4 : 8;
  static constexpr int kCols = kBN * 4 / kEpiWarps;  // tile columns per epilogue thread
  // Single CTAs load B with a second producer warp (after the epilogue
  // warps): one thread issuing every copy caps what TMA delivers into the
  // SM (measured 43-46 B/cycle for 64 KB stages from one issuing thread,
  // 66-68 from two).  CTA pairs keep one producer; the warp then idles.
  static constexpr int kBProdWarp = 2 + kEpiWarps;
  static constexpr int kThreads = 64 + 32 * kEpiWarps + 32;
  // TMEM: two chunk buffers (the MMAs may run one chunk ahead of the
  // epilogue), main + correction accumulators for the split (2 x 256
  // columns), one accumulator for FP8 (2 x 128 columns, then one 8-column
  // scale slot per stage from column 256).
  static constexpr int kBufs = 2;
  static constexpr uint32_t kBufCols = fp8 ? kBN : 2 * kBN;
  static constexpr uint32_t kSfCol0 = 2 * kBN;
};

template <int MODE, bool PAIR>
struct TcCfg {
  static constexpr int P = ModeTraits<MODE>::P;
  static constexpr uint32_t kRow = ModeTraits<MODE>::kRowBytes;
  static constexpr uint32_t kABytes = kBM * kRow;  // one K sub-tile of A (this CTA's rows)
  static constexpr uint32_t kBBytes = (PAIR ? kBN / 2 : kBN) * kRow;  // B^T rows this CTA stages
  static constexpr int kSub = ModeTraits<MODE>::kSub;
  // FP8: the stage's scale atoms (512 bytes per 128-K block) of A, then of B
  static constexpr uint32_t kSfBytes = ModeTraits<MODE>::fp8 ? 2 * 512 * kSub : 0;
  static constexpr uint32_t kStageBytes = P * kSub * (kABytes + kBBytes) + kSfBytes;
  // what each producer of a single CTA brings per stage (A part, B part)
  static constexpr uint32_t kAStageBytes = P * kSub * kABytes + kSfBytes / 2;
  static constexpr uint32_t kBStageBytes = P * kSub * kBBytes + kSfBytes / 2;
  static constexpr uint32_t kTmemCols = 512;
  static constexpr size_t kBarBytes = 1024;  // mbarriers, tile ring, TMEM slot, abort flag
  // Single CTAs: per epilogue warp one 32 x 32 float block (4 KB, 1024-aligned)
  // that a TMA reduce-add store adds into C (where C's layout allows it)
  static constexpr bool kTmaC = !PAIR;
  static constexpr size_t kEpiScratch = kTmaC ? (size_t)ModeTraits<MODE>::kEpiWarps * 4096 : 0;
  static constexpr int kStagesFit = (int)((kSmemLimit - 1024 - kBarBytes - kEpiScratch) / kStageBytes);
  static constexpr int kStages = kStagesFit > kMaxStages ? kMaxStages : kStagesFit;
  static constexpr size_t kSmem = 1024 /*alignment slack*/ + (size_t)kStages * kStageBytes + kEpiScratch + kBarBytes;
  static_assert(!(PAIR && ModeTraits<MODE>::fp8), "FP8 runs on single CTAs");
  static_assert(ModeTraits<MODE>::kBufs * ModeTraits<MODE>::kBufCols <= kTmemCols, "chunk buffers exceed TMEM");
  static_assert(!ModeTraits<MODE>::fp8 || ModeTraits<MODE>::kSfCol0 + 8 * kSub * kStages <= kTmemCols,
                "scale slots exceed TMEM");
  static_assert((2 * kMaxStages + 2 * 4 + 2 * kTileRing + 1) * 8 + (kTileRing + 3) * 4 <= kBarBytes,
                "barrier area too small");
  static_assert(kStages >= 2, "need at least a double-buffered stage ring");
  static_assert(kSmem <= kSmemLimit, "exceeds the 227 KB per-CTA shared memory limit");
  static_assert(kStageBytes % 1024 == 0 && kABytes % 1024 == 0 && kBBytes % 1024 == 0,
                "operand tiles must stay 1024-byte aligned for the 128- / 64-byte swizzle");
  static_assert(kTmemCols <= 512, "TMEM has 512 columns");
};

// One GEMM of a group, as the kernel sees it (device memory).
struct TcProblem {
  CUtensorMap c_map;  // FP8 with c_tma: C as a float tensor, 32 x 32 boxes, 128-byte swizzle
  int c_tma;          // 1: the epilogue adds into C with TMA reduce-add stores
  int M, N;
  int num_kt;      // K stages of this (sub)problem: 64 of K (BF16) or 256 (FP8) each
  int kt0;         // its first K stage (a split-K part covers stages kt0 .. kt0 + num_kt - 1)
  int a_row;       // first row of this problem in the A arena (piece 0)
  int b_row;       // first row in the B^T arena (piece 0)
  int tiles_m, tiles_n;
  int tile_start;  // first global tile index of this problem
  int overwrite;   // 1: the epilogue stores (a split-K partial), 0: C += result
  float* C;
  int64_t rsc, csc;
};

// One split-K problem's final step: C += sum over s of part[s] (in order of
// s, so the result does not depend on which part finished first); parts are
// M x pitch row-major, `parts` x M x pitch floats in all.
struct SplitReduce {
  float* C;
  int64_t rsc, csc;
  const float* part;
  int M, N, pitch, parts;
};

// One operand matrix to split or quantise (device memory).
struct SplitJob {
  const float* src;
  int64_t rows, K, rs, cs;  // logical rows x K, element (r, k) at src[r*rs + k*cs]
  int64_t dst_row;          // first row in the arena
  int tiles_r, tiles_k;     // preparation tiles (PrepTile) covering padded rows x padded K
  int tile_start;
  int col_start;            // first CTA of f16_col_scale_kernel (operands whose rows are contiguous)
};

// ------------------------------------------------------ operand preparation
// Tile of one preparation CTA: TR rows x TK along K (16 KB of FP32).
template <int MODE>
struct PrepTile {
  static constexpr int TK = MODE == kModeFp8 ? 128 : 64;  // one FP8 scale block / one BF16 slice
  static constexpr int TR = 4096 / TK;                    // 32 / 64 rows
  static constexpr int LD = TK + 4;                       // shared row pitch (floats), 16-byte multiple
};

// For every job, writes its rows_pad x k_pad operand into the arena (row pitch
// `pitch` elements), zero outside rows x K:
//  * split-BF16 (MODE 2, 3): MODE pieces p0 = bf16_rn(a), p1 = bf16_rn(a - p0),
//    ... (piece p at out + p * piece_stride);
//  * FP8: E4M3 bytes and one power-of-two scale per (row, 128-K block).
//    Block scale s = 2^e with e the smallest integer such that
//    amax * 2^-e <= 448 (the largest finite E4M3), so v * 2^-e is exact and
//    only the E4M3 rounding (nearest-even, saturating) loses bits.  All-zero
//    (and padding) blocks get s = 1.  The scale is stored as its UE8M0 byte
//    e + 127, repeated in the four bytes of a 32-bit word (one per 32-K
//    sub-block of the MMA), words in 512-byte atoms of 128 arena rows and
//    one K-block, the atoms of a row block consecutive along K:
//    row R = 128 a + 32 j + i of K-block kb at word
//    a * scale_stride + 128 kb + 4 i + j  (scale_stride = 128 x the K-blocks;
//    each atom in the layout tmem_cp_scales expects).
// One CTA per tile.  Interior tiles of 16-byte-aligned sources are read with
// 128-bit loads along whichever dimension is contiguous; edge tiles and other
// strides element by element (still coalesced along the contiguous side).
// FP16 split: every row is scaled by 2^(15 - e), e the frexp exponent of its
// largest magnitude (f16_scale_kernel), so it lies below 2^15 and inside
// FP16's range.
constexpr int kF16ScaleTop = 15;

// Magnitude bits of a float (comparable as unsigned integers), and the same
// with zero mapped above every finite magnitude (for the smallest nonzero).
__device__ __forceinline__ unsigned mag_bits(float v) { return __float_as_uint(v) & 0x7FFFFFFFu; }
__device__ __forceinline__ unsigned nz_bits(float v) {
  const unsigned m = mag_bits(v);
  return m ? m : 0xFFFFFFFFu;
}

// Edge / strided tiles of f16_scale_kernel: value i of a thread (element
// tid + 256 i of the 64 x 64 tile, as magnitude bits mx / nonzero bits mn)
// into the rows' maxima and nonzero minima.  K contiguous: it lies in row
// tid / 64 + 4 i and a warp's 32 lanes hold 32 K of that row (one shared
// atomic per warp and row); otherwise all 16 lie in row tid % 64.
__device__ __forceinline__ void f16_scale_tile_rows(const unsigned (&mx)[16], const unsigned (&mn)[16], int tid,
                                                    bool k_contig, unsigned* rmax, unsigned* rmin) {
  if (k_contig) {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const unsigned w = __reduce_max_sync(0xffffffffu, mx[i]);
      const unsigned v = __reduce_min_sync(0xffffffffu, mn[i]);
      if ((tid & 31) == 0) {
        if (w) atomicMax(&rmax[tid / 64 + 4 * i], w);
        if (v != 0xFFFFFFFFu) atomicMin(&rmin[tid / 64 + 4 * i], v);
      }
    }
  } else {
    unsigned w = 0u, v = 0xFFFFFFFFu;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      w = max(w, mx[i]);
      v = min(v, mn[i]);
    }
    if (w) atomicMax(&rmax[tid % 64], w);
    if (v != 0xFFFFFFFFu) atomicMin(&rmin[tid % 64], v);
  }
}

// Row exponents are stored biased so that zero (what the launch's one
// memset writes) means "no nonzero element seen": e[R] = kExpBias + the
// frexp exponent of the row's largest magnitude, emin[R] = ~(magnitude bits
// of its smallest nonzero element), both combined with atomicMax.
constexpr int kExpBias = 1024;

// One operand's side of a two-operand preparation launch (A's CTAs first,
// then B^T's).
struct ScaleSide {
  const SplitJob* jobs;
  int tiles;
  int* e_out;
  unsigned* emin_out;  // null: no guard
};

// For every arena row R of both operands: e[R] (the row's largest
// magnitude) and, for the AUTO guard, emin[R] (its smallest nonzero one).
// Same tiles as the preparation; magnitudes compared as bit patterns; the
// rows' extremes of a tile combined in shared memory, then atomicMax-ed
// into the encodings above.
__global__ void __launch_bounds__(256) f16_scale_kernel(ScaleSide side_a, ScaleSide side_b, int njobs) {
  constexpr int TK = 64, TR = 64;
  __shared__ unsigned int rmax[TR], rmin[TR];
  __shared__ int sjob;
  const bool on_b = (int)blockIdx.x >= side_a.tiles;
  const ScaleSide sd = on_b ? side_b : side_a;
  const SplitJob* __restrict__ jobs = sd.jobs;
  const int t = (int)blockIdx.x - (on_b ? side_a.tiles : 0), tid = threadIdx.x;
  if (tid == 0) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (jobs[mid].tile_start <= t)
        lo = mid;
      else
        hi = mid - 1;
    }
    sjob = lo;
  }
  if (tid < TR) {
    rmax[tid] = 0u;
    rmin[tid] = 0xFFFFFFFFu;
  }
  __syncthreads();
  const SplitJob& j = jobs[sjob];
  const int local = t - j.tile_start;
  const int64_t r0 = (int64_t)(local / j.tiles_k) * TR, k0 = (int64_t)(local % j.tiles_k) * TK;
  const bool full = r0 + TR <= j.rows && k0 + TK <= j.K;
  const bool al16 = (reinterpret_cast<uintptr_t>(j.src) & 15) == 0;
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  if (al16 && j.cs == 1 && (j.rs & 3) == 0 && (full || (j.K & 3) == 0)) {
    // K contiguous (interior tiles, and edge tiles whose K is a multiple of
    // 4): 128-bit loads, float4 i of a thread in row tid / 16 + 16 i; the 16
    // lanes of a half-warp share that row
    unsigned w[4], v[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int idx = tid + 256 * i;
      const float4 x =
          (full || (r0 + idx / 16 < j.rows && k0 + 4 * (idx % 16) < j.K))
              ? dev::ld_stream(reinterpret_cast<const float4*>(j.src + (r0 + idx / 16) * j.rs + k0 + 4 * (idx % 16)))
              : zero4;
      w[i] = max(max(mag_bits(x.x), mag_bits(x.y)), max(mag_bits(x.z), mag_bits(x.w)));
      v[i] = min(min(nz_bits(x.x), nz_bits(x.y)), min(nz_bits(x.z), nz_bits(x.w)));
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) {
        w[i] = max(w[i], __shfl_xor_sync(0xffffffffu, w[i], o));
        v[i] = min(v[i], __shfl_xor_sync(0xffffffffu, v[i], o));
      }
      if ((tid & 15) == 0) {
        if (w[i]) atomicMax(&rmax[tid / 16 + 16 * i], w[i]);
        if (v[i] != 0xFFFFFFFFu) atomicMin(&rmin[tid / 16 + 16 * i], v[i]);
      }
    }
  } else if (al16 && j.rs == 1 && (j.cs & 3) == 0 && (full || (j.rows & 3) == 0)) {
    // rows contiguous (likewise): 128-bit loads of rows 4 (tid % 16) .. + 3,
    // the same four rows for all of a thread's loads; lanes l and l ^ 16 too
    unsigned w[4] = {0u, 0u, 0u, 0u}, v[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int idx = tid + 256 * i;
      const float4 x =
          (full || (k0 + idx / 16 < j.K && r0 + 4 * (idx % 16) < j.rows))
              ? dev::ld_stream(reinterpret_cast<const float4*>(j.src + (k0 + idx / 16) * j.cs + r0 + 4 * (idx % 16)))
              : zero4;
      w[0] = max(w[0], mag_bits(x.x));
      w[1] = max(w[1], mag_bits(x.y));
      w[2] = max(w[2], mag_bits(x.z));
      w[3] = max(w[3], mag_bits(x.w));
      v[0] = min(v[0], nz_bits(x.x));
      v[1] = min(v[1], nz_bits(x.y));
      v[2] = min(v[2], nz_bits(x.z));
      v[3] = min(v[3], nz_bits(x.w));
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      w[q] = max(w[q], __shfl_xor_sync(0xffffffffu, w[q], 16));
      v[q] = min(v[q], __shfl_xor_sync(0xffffffffu, v[q], 16));
      if ((tid & 31) < 16) {
        if (w[q]) atomicMax(&rmax[4 * (tid % 16) + q], w[q]);
        if (v[q] != 0xFFFFFFFFu) atomicMin(&rmin[4 * (tid % 16) + q], v[q]);
      }
    }
  } else {
    unsigned mx[16], mn[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int idx = tid + 256 * i;
      const int r = j.cs == 1 ? idx / TK : idx % TR, k = j.cs == 1 ? idx % TK : idx / TR;
      const float x = (r0 + r < j.rows && k0 + k < j.K) ? __ldg(j.src + (r0 + r) * j.rs + (k0 + k) * j.cs) : 0.f;
      mx[i] = mag_bits(x);
      mn[i] = nz_bits(x);
    }
    f16_scale_tile_rows(mx, mn, tid, j.cs == 1, rmax, rmin);
  }
  __syncthreads();
  if (tid < TR && r0 + tid < j.rows) {
    if (rmax[tid] != 0u) {
      int e;
      (void)frexpf(__uint_as_float(rmax[tid] >= 0x7F800000u ? 0x7F7FFFFFu : rmax[tid]), &e);  // Inf / NaN: the top exponent
      atomicMax(sd.e_out + j.dst_row + r0 + tid, e + kExpBias);
    }
    if (sd.emin_out && rmin[tid] != 0xFFFFFFFFu) atomicMax(sd.emin_out + j.dst_row + r0 + tid, ~rmin[tid]);
  }
}

// x * 2^n, correctly rounded (what ldexpf gives), by one multiply with a
// normal power of two where n allows it (the common case: one integer add,
// a shift and a multiply) and ldexpf otherwise.
__device__ __forceinline__ float scale_pow2(float x, int n) {
  return (n >= -126 && n <= 127) ? x * __int_as_float((n + 127) << 23) : ldexpf(x, n);
}

__device__ __forceinline__ int f16_row_exp(const int* e, int64_t row) {
  const int v = e[row];
  return v == 0 ? 0 : v - kExpBias;  // all-zero (or padding) rows: scale 2^15
}

// The guard of the FP16 split under GBBLAS_ACCURACY_AUTO, per operand.  An
// element of a row scaled by 2^(15 - e) keeps 22 significant bits while its
// low piece stays a normal FP16 number; below that its absolute error is at
// most 2^-25 of FP16's subnormal step, 2^(e - 40).  In a row whose nonzero
// magnitudes span at most S binades (floor(log2 max) - floor(log2 min)),
// that is at most 2^(S - 39) |a|, so over a K-term dot the FP16 split's
// error stays within 3 * 2^-22 + 2 K eps32 of (|A||B|)_ij - the FP32 GEMM
// rule - when 2^(S - 38) <= K 2^-24, i.e. S <= 14 + floor(log2 K).  Rows (of A,
// and columns of B) beyond that span, or holding Inf or NaN, are "out of
// span": flags[R] = 1 and R goes onto `list`; the GEMM leaves their outputs
// alone and f16_guard_fixup_kernel computes them with FP32 FMAs.
struct F16Guard {
  const unsigned* emin = nullptr;  // ~(smallest nonzero magnitude bits) per arena row (f16_scale_kernel)
  int* flags = nullptr;            // per arena row: 1 = out of span (every row written)
  int* list = nullptr;             // out-of-span arena rows, in no particular order
  int* count = nullptr;            // entries in list
};

// floor(log2 x) + 127 for the magnitude bits of a nonzero float (subnormals
// included).
__device__ __forceinline__ int biased_log2(unsigned bits) {
  return bits >= 0x00800000u ? (int)(bits >> 23) : 9 - __clz(bits);
}

// One operand's side of a two-operand preparation launch (A's CTAs first,
// then B^T's): its jobs, tiles, arena, piece stride, scales and guard.
struct PrepSide {
  const SplitJob* jobs;
  int tiles;
  void* out;
  int64_t piece_stride;
  uint32_t* scales;
  F16Guard guard;
};

// Shared-memory slot of (row r, K element k) of a preparation tile: the
// 16-byte chunks of a row are permuted by the row's group of four (chunk c
// stored at c ^ ((r / 4) & 7)), so the transposing stores of the
// rows-contiguous path meet at most two to a bank (eight with plain rows of
// LD = TK + 4 floats), while every 16-byte read stays whole.
template <int LD>
__device__ __forceinline__ int prep_slot(int r, int k) {
  return r * LD + 4 * ((k >> 2) ^ ((r >> 2) & 7)) + (k & 3);
}

template <int MODE>
__global__ void __launch_bounds__(256) prep_group_kernel(PrepSide side_a, PrepSide side_b, int njobs, int64_t pitch,
                                                         int64_t scale_stride) {
  using PT = PrepTile<MODE>;
  constexpr int TK = PT::TK, TR = PT::TR, LD = PT::LD;
  __shared__ __align__(16) float tile[TR * LD];
  __shared__ int sjob;
  const bool on_b = (int)blockIdx.x >= side_a.tiles;
  const PrepSide sd = on_b ? side_b : side_a;
  const SplitJob* __restrict__ jobs = sd.jobs;
  void* __restrict__ out = sd.out;
  const int64_t piece_stride = sd.piece_stride;
  uint32_t* __restrict__ scales = sd.scales;
  const F16Guard& guard = sd.guard;
  const int t = (int)blockIdx.x - (on_b ? side_a.tiles : 0);
  const int tid = threadIdx.x;
  if (tid == 0) {  // job = last with tile_start <= t
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (jobs[mid].tile_start <= t)
        lo = mid;
      else
        hi = mid - 1;
    }
    sjob = lo;
  }
  __syncthreads();
  const SplitJob& j = jobs[sjob];
  const int local = t - j.tile_start;
  const int64_t r0 = (int64_t)(local / j.tiles_k) * TR, k0 = (int64_t)(local % j.tiles_k) * TK;
  const bool full = r0 + TR <= j.rows && k0 + TK <= j.K;
  const bool al16 = (reinterpret_cast<uintptr_t>(j.src) & 15) == 0;
  // 128-bit loads along the contiguous dimension: on interior tiles, and on
  // edge tiles too where that dimension's extent is a multiple of 4 (each
  // float4 then lies wholly inside or wholly outside the operand)
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  if (al16 && j.cs == 1 && (j.rs & 3) == 0 && (full || (j.K & 3) == 0)) {  // along K
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int idx = tid + 256 * i, r = idx / (TK / 4), k4 = idx % (TK / 4);
      const float4 v = (full || (r0 + r < j.rows && k0 + 4 * k4 < j.K))
                           ? dev::ld_stream(reinterpret_cast<const float4*>(j.src + (r0 + r) * j.rs + k0 + 4 * k4))
                           : zero4;
      *reinterpret_cast<float4*>(&tile[prep_slot<LD>(r, 4 * k4)]) = v;
    }
  } else if (al16 && j.rs == 1 && (j.cs & 3) == 0 && (full || (j.rows & 3) == 0)) {  // along rows
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int idx = tid + 256 * i, k = idx / (TR / 4), r4 = idx % (TR / 4);
      const float4 v = (full || (k0 + k < j.K && r0 + 4 * r4 < j.rows))
                           ? dev::ld_stream(reinterpret_cast<const float4*>(j.src + (k0 + k) * j.cs + r0 + 4 * r4))
                           : zero4;
      tile[prep_slot<LD>(4 * r4 + 0, k)] = v.x;
      tile[prep_slot<LD>(4 * r4 + 1, k)] = v.y;
      tile[prep_slot<LD>(4 * r4 + 2, k)] = v.z;
      tile[prep_slot<LD>(4 * r4 + 3, k)] = v.w;
    }
  } else if (j.cs == 1) {  // K contiguous: consecutive threads along k
#pragma unroll 4
    for (int i = 0; i < 16; ++i) {
      const int idx = tid + 256 * i, r = idx / TK, k = idx % TK;
      tile[prep_slot<LD>(r, k)] = (r0 + r < j.rows && k0 + k < j.K) ? __ldg(j.src + (r0 + r) * j.rs + k0 + k) : 0.f;
    }
  } else {  // rows contiguous (or general): consecutive threads along r
#pragma unroll 4
    for (int i = 0; i < 16; ++i) {
      const int idx = tid + 256 * i, r = idx % TR, k = idx / TR;
      tile[prep_slot<LD>(r, k)] =
          (r0 + r < j.rows && k0 + k < j.K) ? __ldg(j.src + (r0 + r) * j.rs + (k0 + k) * j.cs) : 0.f;
    }
  }
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31;
  if constexpr (MODE == kModeFp8) {
    // warp w: rows 4w..4w+3, lane: 4 consecutive K of the row's 128
    uint8_t* q8 = static_cast<uint8_t*>(out);
#pragma unroll
    for (int rr = 0; rr < 4; ++rr) {
      const int r = warp * 4 + rr;
      const float4 v = *reinterpret_cast<const float4*>(&tile[prep_slot<LD>(r, lane * 4)]);
      float amax = fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w)));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
      int e = 0;
      if (amax > 0.f) {
        int ex;
        const float m = frexpf(amax, &ex);  // amax = m * 2^ex, m in [0.5, 1); 448 = 0.875 * 2^9
        e = ex - 9 + (m > 0.875f ? 1 : 0);
        e = e < -126 ? -126 : (e > 126 ? 126 : e);
      }
      const float inv = __int_as_float((127 - e) << 23);  // 2^-e, a normal float for |e| <= 126
      const __nv_fp8x2_storage_t lo =
          __nv_cvt_float2_to_fp8x2(make_float2(v.x * inv, v.y * inv), __NV_SATFINITE, __NV_E4M3);
      const __nv_fp8x2_storage_t hi =
          __nv_cvt_float2_to_fp8x2(make_float2(v.z * inv, v.w * inv), __NV_SATFINITE, __NV_E4M3);
      const int64_t row = j.dst_row + r0 + r;
      *reinterpret_cast<uint32_t*>(q8 + row * pitch + k0 + lane * 4) = (uint32_t)lo | ((uint32_t)hi << 16);
      if (lane == 0)
        scales[(row >> 7) * scale_stride + k0 + 4 * (row & 31) + ((row >> 5) & 3)] =
            (uint32_t)(127 + e) * 0x01010101u;
    }
  } else if constexpr (MODE == kModeF16) {
    // half-warp per row as below; the row scaled by 2^(15 - e) (exact), then
    // h = fp16_rn(v), l = fp16_rn(v - h) (v - h exact in FP32)
    __half* ph = static_cast<__half*>(out);
    const int* erow = reinterpret_cast<const int*>(scales);
    if (guard.flags && k0 == 0 && tid < TR) {  // the guard: one decision per row, by its first K tile
      const int64_t row = j.dst_row + r0 + tid;
      int out_of_span = 0;
      if (r0 + tid < j.rows) {
        const int e = f16_row_exp(erow, row);  // floor(log2 max) + 1; 128 for Inf / NaN (or >= 2^127)
        const unsigned mn = ~guard.emin[row];  // 0xFFFFFFFF: no nonzero element
        const int span_max = 14 + (63 - __clzll((unsigned long long)(j.K > 0 ? j.K : 1)));  // 14 + floor(log2 K)
        out_of_span = e >= 128 || (mn != 0xFFFFFFFFu && (e - 1) - (biased_log2(mn) - 127) > span_max);
      }
      guard.flags[row] = out_of_span;
      if (out_of_span) guard.list[atomicAdd(guard.count, 1)] = (int)row;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = warp * 8 + 2 * i + (lane >> 4), kk = (lane & 15) * 4;
      const int64_t arow = j.dst_row + r0 + r;
      const int sh = kF16ScaleTop - f16_row_exp(erow, arow);
      float4 v = *reinterpret_cast<const float4*>(&tile[prep_slot<LD>(r, kk)]);
      v = make_float4(scale_pow2(v.x, sh), scale_pow2(v.y, sh), scale_pow2(v.z, sh), scale_pow2(v.w, sh));
      const int64_t base = arow * pitch + k0 + kk;
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        const __half2 h01 = __floats2half2_rn(v.x, v.y);
        const __half2 h23 = __floats2half2_rn(v.z, v.w);
        uint2 w;
        w.x = *reinterpret_cast<const uint32_t*>(&h01);
        w.y = *reinterpret_cast<const uint32_t*>(&h23);
        *reinterpret_cast<uint2*>(ph + p * piece_stride + base) = w;
        const float2 f01 = __half22float2(h01), f23 = __half22float2(h23);
        v.x -= f01.x;
        v.y -= f01.y;
        v.z -= f23.x;
        v.w -= f23.y;
      }
    }
  } else {
    // half-warp per row: rows 8w + 2i + (lane / 16), lane % 16: 4 consecutive K of 64
    __nv_bfloat16* pb = static_cast<__nv_bfloat16*>(out);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = warp * 8 + 2 * i + (lane >> 4), kk = (lane & 15) * 4;
      float4 v = *reinterpret_cast<const float4*>(&tile[prep_slot<LD>(r, kk)]);
      const int64_t base = (j.dst_row + r0 + r) * pitch + k0 + kk;
#pragma unroll
      for (int p = 0; p < MODE; ++p) {
        const __nv_bfloat162 h01 = __floats2bfloat162_rn(v.x, v.y);
        const __nv_bfloat162 h23 = __floats2bfloat162_rn(v.z, v.w);
        uint2 w;
        w.x = *reinterpret_cast<const uint32_t*>(&h01);
        w.y = *reinterpret_cast<const uint32_t*>(&h23);
        *reinterpret_cast<uint2*>(pb + p * piece_stride + base) = w;
        const float2 f01 = __bfloat1622float2(h01), f23 = __bfloat1622float2(h23);
        v.x -= f01.x;  // exact in FP32
        v.y -= f01.y;
        v.z -= f23.x;
        v.w -= f23.y;
      }
    }
  }
}

// Row exponents of the FP16 split for operands whose rows are contiguous
// (row-major B seen as B^T, column-major A): f16_scale_kernel's results by
// a column reduction.  A CTA covers 1024 consecutive rows (4 per thread, as
// one float4) and `kblk` (kColScaleK) of K; each thread keeps 8 loads in flight and
// its rows' extremes in registers, then atomicMax-es them into e[R] and
// emin[R] once.  Conditions (host side, per operand): every job has rows
// contiguous, 16-byte aligned columns and a row count that is a multiple of
// 4 (each float4 wholly inside or outside the operand).
constexpr int kColScaleK = 128;

__global__ void __launch_bounds__(256, 4) f16_col_scale_kernel(ScaleSide side_a, ScaleSide side_b, int njobs,
                                                               int kblk) {
  const bool on_b = (int)blockIdx.x >= side_a.tiles;
  const ScaleSide& sd = on_b ? side_b : side_a;
  const int t = (int)blockIdx.x - (on_b ? side_a.tiles : 0);
  int lo = 0, hi = njobs - 1;  // job: the last whose first CTA is <= t
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (sd.jobs[mid].col_start <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  const SplitJob& j = sd.jobs[lo];
  const int local = t - j.col_start;
  const int kblocks = (int)((j.K + kblk - 1) / kblk);
  const int64_t r = (int64_t)(local / kblocks) * 1024 + 4 * threadIdx.x;  // this thread's first row
  const int64_t k0 = (int64_t)(local % kblocks) * kblk;
  const int64_t k1 = min(k0 + kblk, j.K);
  if (r >= j.rows) return;
  const float* __restrict__ src = j.src + r;
  unsigned w[4] = {0u, 0u, 0u, 0u}, v[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
  for (int64_t k = k0; k < k1; k += 8) {
    float4 x[8];
#pragma unroll
    for (int u = 0; u < 8; ++u)
      x[u] = k + u < k1 ? dev::ld_stream(reinterpret_cast<const float4*>(src + (k + u) * j.cs))
                        : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      w[0] = max(w[0], mag_bits(x[u].x));
      w[1] = max(w[1], mag_bits(x[u].y));
      w[2] = max(w[2], mag_bits(x[u].z));
      w[3] = max(w[3], mag_bits(x[u].w));
      v[0] = min(v[0], nz_bits(x[u].x));
      v[1] = min(v[1], nz_bits(x[u].y));
      v[2] = min(v[2], nz_bits(x[u].z));
      v[3] = min(v[3], nz_bits(x[u].w));
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int64_t row = j.dst_row + r + q;
    if (w[q] != 0u) {
      // frexp's exponent of a positive finite float (subnormals included):
      // floor(log2 x) + 1; Inf / NaN take the top exponent, as elsewhere
      const int e = biased_log2(w[q] >= 0x7F800000u ? 0x7F7FFFFFu : w[q]) - 126;
      atomicMax(sd.e_out + row, e + kExpBias);
    }
    if (sd.emin_out && v[q] != 0xFFFFFFFFu) atomicMax(sd.emin_out + row, ~v[q]);
  }
}

// Split-BF16 preparation of operands whose K is contiguous (row-major A,
// column-major B; 16-byte aligned rows, K a multiple of 4): a warp per
// arena row at a time, each lane 4 consecutive K per 128-bit load (four loads in
// flight), its P pieces written as 8-byte stores - the same pieces as
// prep_group_kernel, without the shared-memory tile or its barriers.
// Padding rows and the K padding get zeros.
struct RowSplitSide {
  const SplitJob* jobs;
  int rows;  // arena rows prepared here (0: this operand takes the tile kernel)
  __nv_bfloat16* out;
  int64_t piece_stride;
};

// A CTA covers `rows_per_cta` consecutive arena rows (8 or 32: a warp
// each, or four each where the launch still has at least four CTAs per SM;
// many small jobs take 32, one large matrix 8).  They lie in one job, since
// every job's rows are padded to a multiple of 128, so thread 0 finds it
// once for all of them.
constexpr int kSplitRowsPerCtaMax = 32;

template <int P>
__global__ void __launch_bounds__(256) split_rows_kernel(RowSplitSide side_a, RowSplitSide side_b, int njobs,
                                                         int64_t pitch, int rows_per_cta) {
  __shared__ int sjob;
  const int a_ctas = side_a.rows / rows_per_cta;
  const bool on_b = (int)blockIdx.x >= a_ctas;
  const RowSplitSide& sd = on_b ? side_b : side_a;
  const int64_t R0 = (int64_t)((int)blockIdx.x - (on_b ? a_ctas : 0)) * rows_per_cta;  // first arena row
  if (threadIdx.x == 0) {
    int lo = 0, hi = njobs - 1;  // job: the last whose first arena row is <= R0
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (sd.jobs[mid].dst_row <= R0)
        lo = mid;
      else
        hi = mid - 1;
    }
    sjob = lo;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const SplitJob& j = sd.jobs[sjob];
  const int per_warp = rows_per_cta / 8;
  for (int rr = 0; rr < per_warp; ++rr) {
  const int64_t R = R0 + (threadIdx.x >> 5) * per_warp + rr;  // arena row
  const int64_t local = R - j.dst_row;
  const int64_t kp = (int64_t)j.tiles_k * PrepTile<P>::TK;  // the job's padded K
  const int64_t K = local < j.rows ? j.K : 0;                // padding rows: all zeros
  const float* __restrict__ src = j.src + (local < j.rows ? local : 0) * j.rs;
  __nv_bfloat16* __restrict__ dst = sd.out + R * pitch;
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t k0 = 4 * lane; k0 < kp; k0 += 4 * 128) {
    float4 x[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t k = k0 + 128 * u;
      x[u] = k < K ? dev::ld_stream(reinterpret_cast<const float4*>(src + k)) : zero4;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t k = k0 + 128 * u;
      if (k >= kp) break;
      float4 v = x[u];
#pragma unroll
      for (int p = 0; p < P; ++p) {
        const __nv_bfloat162 h01 = __floats2bfloat162_rn(v.x, v.y);
        const __nv_bfloat162 h23 = __floats2bfloat162_rn(v.z, v.w);
        uint2 wv;
        wv.x = *reinterpret_cast<const uint32_t*>(&h01);
        wv.y = *reinterpret_cast<const uint32_t*>(&h23);
        *reinterpret_cast<uint2*>(dst + p * sd.piece_stride + k) = wv;
        const float2 f01 = __bfloat1622float2(h01), f23 = __bfloat1622float2(h23);
        v.x -= f01.x;  // exact in FP32
        v.y -= f01.y;
        v.z -= f23.x;
        v.w -= f23.y;
      }
    }
  }
  }
}

// Split-FP16 preparation in one pass for operands whose K is contiguous
// (row-major A, column-major B): one CTA per arena row reads the row once
// into registers (kRowPrepNV float4 per thread), finds its largest and its
// smallest nonzero magnitude (warp shuffles, then the 8 warps' values in
// shared memory), records e[R] (and, under the guard, emin[R] and the
// row's out-of-span decision) exactly as f16_scale_kernel and
// prep_group_kernel do, then scales the row by 2^(15 - e) and writes its two
// FP16 pieces - the same bits as the two-kernel path, from one read of the
// operand instead of two.  Padding rows (beyond the job's rows) get zero
// pieces.  Conditions (host side, per operand): every job K contiguous,
// 16-byte aligned rows, K a multiple of 4 and at most 1024 kRowPrepNV.
constexpr int kRowPrepNV = 8;
constexpr int64_t kRowPrepMinK = 1024;  // shorter rows: the tile kernels (a CTA per row would idle)

struct RowPrepSide {
  const SplitJob* jobs;
  int rows;  // arena rows prepared here (0: this operand takes the tile kernels)
  __half* out;
  int64_t piece_stride;
  int* e_out;
  F16Guard guard;
};

__global__ void __launch_bounds__(256) f16_row_prep_kernel(RowPrepSide side_a, RowPrepSide side_b, int njobs,
                                                           int64_t pitch) {
  constexpr int NV = kRowPrepNV;
  __shared__ unsigned red_max[8], red_min[8];
  __shared__ int sh_shift;
  const bool on_b = (int)blockIdx.x >= side_a.rows;
  const RowPrepSide& sd = on_b ? side_b : side_a;
  const int64_t R = (int64_t)blockIdx.x - (on_b ? side_a.rows : 0);  // arena row
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  int lo = 0, hi = njobs - 1;  // job: the last whose first arena row is <= R
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (sd.jobs[mid].dst_row <= R)
      lo = mid;
    else
      hi = mid - 1;
  }
  const SplitJob& j = sd.jobs[lo];
  const int64_t local = R - j.dst_row;
  const int64_t kp = (int64_t)j.tiles_k * PrepTile<kModeF16>::TK;  // the job's padded K
  __half* __restrict__ ph = sd.out + R * pitch;
  if (local >= j.rows) {  // padding row of the job's last tile
    for (int64_t k = 4 * tid; k < kp; k += 1024) {
      *reinterpret_cast<uint2*>(ph + k) = make_uint2(0u, 0u);
      *reinterpret_cast<uint2*>(ph + sd.piece_stride + k) = make_uint2(0u, 0u);
    }
    if (sd.guard.flags && tid == 0) sd.guard.flags[R] = 0;
    return;
  }
  const float* __restrict__ src = j.src + local * j.rs;
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 x[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const int64_t k = 4 * (tid + 256 * i);
    x[i] = k < j.K ? dev::ld_stream(reinterpret_cast<const float4*>(src + k)) : zero4;
  }
  unsigned mx = 0u, mn = 0xFFFFFFFFu;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    mx = max(mx, max(max(mag_bits(x[i].x), mag_bits(x[i].y)), max(mag_bits(x[i].z), mag_bits(x[i].w))));
    mn = min(mn, min(min(nz_bits(x[i].x), nz_bits(x[i].y)), min(nz_bits(x[i].z), nz_bits(x[i].w))));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
  }
  if (lane == 0) {
    red_max[warp] = mx;
    red_min[warp] = mn;
  }
  __syncthreads();
  if (tid == 0) {
    unsigned w = red_max[0], v = red_min[0];
#pragma unroll
    for (int i = 1; i < 8; ++i) {
      w = max(w, red_max[i]);
      v = min(v, red_min[i]);
    }
    int e_store = 0;  // what f16_scale_kernel leaves: kExpBias + exponent, 0 for an all-zero row
    if (w != 0u) {
      int e;
      (void)frexpf(__uint_as_float(w >= 0x7F800000u ? 0x7F7FFFFFu : w), &e);  // Inf / NaN: the top exponent
      e_store = e + kExpBias;
    }
    sd.e_out[R] = e_store;
    const int e = e_store == 0 ? 0 : e_store - kExpBias;
    if (sd.guard.flags) {
      const_cast<unsigned*>(sd.guard.emin)[R] = v != 0xFFFFFFFFu ? ~v : 0u;
      const int span_max = 14 + (63 - __clzll((unsigned long long)(j.K > 0 ? j.K : 1)));  // 14 + floor(log2 K)
      const int out_of_span = e >= 128 || (v != 0xFFFFFFFFu && (e - 1) - (biased_log2(v) - 127) > span_max);
      sd.guard.flags[R] = out_of_span;
      if (out_of_span) sd.guard.list[atomicAdd(sd.guard.count, 1)] = (int)R;
    }
    sh_shift = kF16ScaleTop - e;
  }
  __syncthreads();
  const int sh = sh_shift;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const int64_t k = 4 * (tid + 256 * i);
    if (k < kp) {
      float4 v = make_float4(scale_pow2(x[i].x, sh), scale_pow2(x[i].y, sh), scale_pow2(x[i].z, sh),
                             scale_pow2(x[i].w, sh));
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        const __half2 h01 = __floats2half2_rn(v.x, v.y);
        const __half2 h23 = __floats2half2_rn(v.z, v.w);
        uint2 w;
        w.x = *reinterpret_cast<const uint32_t*>(&h01);
        w.y = *reinterpret_cast<const uint32_t*>(&h23);
        *reinterpret_cast<uint2*>(ph + p * sd.piece_stride + k) = w;
        const float2 f01 = __half22float2(h01), f23 = __half22float2(h23);
        v.x -= f01.x;
        v.y -= f01.y;
        v.z -= f23.x;
        v.w -= f23.y;
      }
    }
  }
}

// ---------------------------------------------------------------- GEMM
__device__ __forceinline__ int find_problem(const TcProblem* __restrict__ probs, int nprob, int t) {
  int lo = 0, hi = nprob - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (probs[mid].tile_start <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Output tile of global index t (BMT rows x 128 columns): grouped raster
// inside its problem (consecutive tiles walk 8 row-tiles of one column band
// for L2 reuse).
template <int BMT>
__device__ __forceinline__ void tile_coords(const TcProblem& p, int t, int& m0, int& n0) {
  constexpr int kGroup = 8;
  const int local = t - p.tile_start;
  const int group_span = kGroup * p.tiles_n;
  const int g = local / group_span;
  const int first_m = g * kGroup;
  const int gm = min(p.tiles_m - first_m, kGroup);
  const int in_g = local % group_span;
  m0 = (first_m + in_g % gm) * BMT;
  n0 = (in_g / gm) * kBN;
}

// PAIR = false: one CTA per SM computes 128 x 128 tiles (tcgen05 .cta_group::1).
// PAIR = true: clusters of two CTAs compute 256 x 128 tiles with
// .cta_group::2 MMAs issued by the even CTA: each CTA stages its own 128 rows
// of A and 64 of the 128 rows of B^T (so a CTA moves 3/4 of the operand bytes
// per MMA flop of the single form, and fits more stages), both CTAs' copies
// complete on the even CTA's stage barrier, its commits release both CTAs'
// stages and signal both CTAs' epilogues, and both epilogues report drained
// TMEM buffers to it.  Pairs walk tiles in a static order (cluster i takes
// tiles i, i + clusters, ...), so both CTAs see the same sequence.
template <int MODE, bool PAIR>
__global__ void __launch_bounds__(ModeTraits<MODE>::kThreads, 1)
    gemm_split_kernel(const __grid_constant__ CUtensorMap tm_a, const __grid_constant__ CUtensorMap tm_b,
                      const TcProblem* __restrict__ probs, int nprob, int tile_begin, int total_tiles,
                      int64_t sf_stride,
                      int* __restrict__ tile_counter, int* __restrict__ err,
                      const uint32_t* __restrict__ sa, const uint32_t* __restrict__ sb,
                      const int* __restrict__ guard_a, const int* __restrict__ guard_b) {
  using MT = ModeTraits<MODE>;
  using CF = TcCfg<MODE, PAIR>;
  constexpr int P = MT::P;
  constexpr int ST = CF::kStages;
  constexpr int BMT = PAIR ? 2 * kBM : kBM;  // output tile rows (both CTAs of a pair)
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  // stage s: A pieces 0..P-1 (split) or K sub-tiles 0..kSub-1 (FP8), then
  // the same of B, then (FP8) the scale atoms
  constexpr int NT = P * MT::kSub;  // 128-byte-wide tiles per operand and stage
  auto a_tile = [&](int s, int p) { return smem + (size_t)s * CF::kStageBytes + (size_t)p * CF::kABytes; };
  auto b_tile = [&](int s, int p) {
    return smem + (size_t)s * CF::kStageBytes + (size_t)NT * CF::kABytes + (size_t)p * CF::kBBytes;
  };
  // FP8: the stage's scale atoms of A (op 0) / of B^T (op 1), kSub x 512 bytes each
  auto sf_atom = [&](int s, int op) {
    return smem + (size_t)s * CF::kStageBytes + (size_t)NT * (CF::kABytes + CF::kBBytes) +
           (size_t)op * 512 * MT::kSub;
  };
  float* epi_scratch = reinterpret_cast<float*>(smem + (size_t)ST * CF::kStageBytes);  // single CTAs, 1024-aligned
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)ST * CF::kStageBytes + CF::kEpiScratch);
  uint64_t* full = bars;                   // [ST]  TMA -> MMA
  uint64_t* empty = full + ST;             // [ST]  MMA -> TMA
  uint64_t* tfull = empty + ST;            // [kBufs] MMA -> epilogue: chunk in TMEM buffer b
  uint64_t* tempty = tfull + 4;            // [kBufs] epilogue -> MMA: TMEM buffer b drained
  uint64_t* ring_full = tempty + 4;        // [kTileRing] scheduler -> consumers
  uint64_t* ring_empty = ring_full + kTileRing;  // [kTileRing] consumers -> scheduler
  uint64_t* accf = ring_empty + kTileRing;       // [1] every MMA of this CTA finished
  int* ring = reinterpret_cast<int*>(accf + 1);  // [kTileRing] tile ids, -1 = no more work
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(ring + kTileRing);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  volatile int* b_issued_slot = abort_flag + 1;  // single CTAs: K slices the B producer issued (teardown)

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = PAIR ? cluster_ctarank() : 0u;  // 0 = the CTA that issues the MMAs

  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      mbar_init(&full[s], PAIR ? 1 : 2);  // single CTAs: the A and the B producer
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < MT::kBufs; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], MT::kEpiWarps * (PAIR ? 2 : 1));  // one arrival per epilogue warp (of both CTAs)
    }
    for (int r = 0; r < kTileRing; ++r) {
      mbar_init(&ring_full[r], 1);
      mbar_init(&ring_empty[r], 1 + MT::kEpiWarps + (PAIR ? 0 : 1));  // MMA lane, epilogue warps, B producer
    }
    mbar_init(accf, 1);
    *abort_flag = 0;
    *b_issued_slot = 0;
    fence_mbar_init();
    prefetch_tensormap(&tm_a);
    prefetch_tensormap(&tm_b);
  }
  if (warp == 1) {
    if constexpr (PAIR) {
      tmem_alloc2(tmem_slot, CF::kTmemCols);
      tmem_relinquish2();
    } else {
      tmem_alloc(tmem_slot, CF::kTmemCols);
      tmem_relinquish();
    }
  }
  tc_fence_before();
  __syncthreads();
  if constexpr (PAIR) cluster_sync_all();  // the peer's barriers exist before anyone signals them
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  auto fail = [&]() {
    *abort_flag = 1;
    atomicExch(err, (int)GBBLAS_STATUS_TIMEOUT);
  };

  int issued = 0;  // producer: K slices whose copies were issued (all tiles)
  if (warp == 0) {
    if (lane == 0) {
      bool stop = false;
      for (int it = 0; !stop; ++it) {
        const int slot = it % kTileRing, use = it / kTileRing;
        int t;
        // this launch's tiles: tile_begin .. total_tiles - 1
        if constexpr (PAIR)
          t = tile_begin + (int)(blockIdx.x >> 1) + it * (int)(gridDim.x >> 1);
        else
          t = tile_begin + atomicAdd(tile_counter, 1);
        if (t >= total_tiles) t = -1;
        if (use > 0 && !mbar_wait_bounded(&ring_empty[slot], (use - 1) & 1, abort_flag, kWaitLimitNs)) {
          fail();
          break;
        }
        ring[slot] = t;
        mbar_arrive(&ring_full[slot]);  // release: consumers see ring[slot]
        if (t < 0) break;
        const TcProblem& pr = probs[find_problem(probs, nprob, t)];
        int m0, n0;
        tile_coords<BMT>(pr, t, m0, n0);
        const int own_m0 = m0 + (int)rank * kBM;  // this CTA's rows
        for (int kt = 0; kt < pr.num_kt; ++kt) {
          const int s = issued % ST, round = issued / ST;
          if (round > 0 && !mbar_wait_bounded(&empty[s], (round - 1) & 1, abort_flag, kWaitLimitNs)) {
            fail();
            stop = true;
            break;
          }
          const int kx = (pr.kt0 + kt) * MT::kBKe;  // first K element of the stage
          // one 3-D copy per operand brings all P piece planes of the tile
          if constexpr (PAIR) {
            if (rank == 0) {
              mbar_arrive_expect_tx(&full[s], 2 * CF::kStageBytes);  // both CTAs' copies
              tma_load_3d(a_tile(s, 0), &tm_a, &full[s], kx, pr.a_row + own_m0, 0);
              tma_load_3d(b_tile(s, 0), &tm_b, &full[s], kx, pr.b_row + n0, 0);
            } else {
              const uint32_t fb = mapa_shared(smem_u32(&full[s]), 0);
              tma_load_3d_pair(a_tile(s, 0), &tm_a, fb, kx, pr.a_row + own_m0, 0);
              tma_load_3d_pair(b_tile(s, 0), &tm_b, fb, kx, pr.b_row + n0 + kBN / 2, 0);
            }
          } else {
            // A's part of the stage; the B producer warp brings the rest
            mbar_arrive_expect_tx(&full[s], CF::kAStageBytes);
            if constexpr (MT::fp8) {
#pragma unroll
              for (int u = 0; u < MT::kSub; ++u)
                tma_load_3d(a_tile(s, u), &tm_a, &full[s], kx + u * 128, pr.a_row + own_m0, 0);
              // the stage's K-blocks' scale atoms of these 128 rows of A:
              // consecutive in the scale array (one run)
              const int64_t kb0 = kx;  // 128 words per K-block of 128 = one word per K element
              bulk_load(sf_atom(s, 0), sa + (int64_t)((pr.a_row + own_m0) >> 7) * sf_stride + kb0, 512 * MT::kSub,
                        &full[s]);
            } else {
              tma_load_3d(a_tile(s, 0), &tm_a, &full[s], kx, pr.a_row + own_m0, 0);
            }
          }
          ++issued;
        }
      }
    }
  } else if (warp == MT::kBProdWarp) {
    // B producer (single CTAs): follows the tile ring and loads B^T's part
    // of every stage into the same ring slots as the A producer.
    if (lane == 0 && !PAIR) {
      int bissued = 0;
      bool stop = false;
      for (int it = 0; !stop; ++it) {
        const int slot = it % kTileRing, use = it / kTileRing;
        if (!mbar_wait_bounded(&ring_full[slot], use & 1, abort_flag, kWaitLimitNs)) {
          fail();
          break;
        }
        const int t = ring[slot];
        mbar_arrive(&ring_empty[slot]);
        if (t < 0) break;
        const TcProblem& pr = probs[find_problem(probs, nprob, t)];
        int m0, n0;
        tile_coords<BMT>(pr, t, m0, n0);
        for (int kt = 0; kt < pr.num_kt; ++kt) {
          const int s = bissued % ST, round = bissued / ST;
          if (round > 0 && !mbar_wait_bounded(&empty[s], (round - 1) & 1, abort_flag, kWaitLimitNs)) {
            fail();
            stop = true;
            break;
          }
          const int kx = (pr.kt0 + kt) * MT::kBKe;
          mbar_arrive_expect_tx(&full[s], CF::kBStageBytes);
          if constexpr (MT::fp8) {
#pragma unroll
            for (int u = 0; u < MT::kSub; ++u)
              tma_load_3d(b_tile(s, u), &tm_b, &full[s], kx + u * 128, pr.b_row + n0, 0);
            bulk_load(sf_atom(s, 1), sb + (int64_t)((pr.b_row + n0) >> 7) * sf_stride + (int64_t)kx, 512 * MT::kSub,
                      &full[s]);
          } else {
            tma_load_3d(b_tile(s, 0), &tm_b, &full[s], kx, pr.b_row + n0, 0);
          }
          ++bissued;
        }
      }
      *b_issued_slot = bissued;
    }
  } else if (warp == 1) {
    if (lane == 0 && PAIR && rank != 0) {
      // the odd CTA of a pair issues no MMAs: it only keeps its tile ring moving
      for (int it = 0;; ++it) {
        const int slot = it % kTileRing, use = it / kTileRing;
        if (!mbar_wait_bounded(&ring_full[slot], use & 1, abort_flag, kWaitLimitNs)) {
          fail();
          break;
        }
        const int t = ring[slot];
        mbar_arrive(&ring_empty[slot]);
        if (t < 0) break;
      }
    } else if (lane == 0) {
      // split-BF16 (FP16 pieces for kModeF16); M = 256 for a pair
      constexpr uint32_t idesc = MT::f16 ? idesc_f16_f32(BMT, kBN) : idesc_bf16_f32(BMT, kBN);
      // single CTAs: p0*[q0; q1] as one N = 256 MMA - the q0 and q1 tiles of
      // B^T lie back to back in the stage and the main and correction
      // accumulators side by side in TMEM, so A's p0 is read once for both
      constexpr uint32_t idesc_n256 = MT::f16 ? idesc_f16_f32(kBM, 2 * kBN) : idesc_bf16_f32(kBM, 2 * kBN);
      int consumed = 0;  // K slices consumed (all tiles)
      int chunk_g = 0;   // chunks started (all tiles)
      bool stop = false;
      for (int it = 0; !stop; ++it) {
        const int slot = it % kTileRing, use = it / kTileRing;
        if (!mbar_wait_bounded(&ring_full[slot], use & 1, abort_flag, kWaitLimitNs)) {
          fail();
          break;
        }
        const int t = ring[slot];
        mbar_arrive(&ring_empty[slot]);
        if (t < 0) break;
        const int num_kt = probs[find_problem(probs, nprob, t)].num_kt;
        for (int kt = 0; kt < num_kt; ++kt) {
          const int s = consumed % ST, round = consumed / ST;
          const bool chunk_first = (kt % MT::kChunk) == 0;
          const bool chunk_last = ((kt + 1) % MT::kChunk) == 0 || kt + 1 == num_kt;
          if (chunk_first) ++chunk_g;
          const int chunk = chunk_g - 1, b = chunk % MT::kBufs;
          if (chunk_first && chunk >= MT::kBufs) {  // buffer b must have been drained by the epilogue(s)
            if (!mbar_wait_bounded(&tempty[b], ((chunk / MT::kBufs) - 1) & 1, abort_flag, kWaitLimitNs)) {
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
          const uint32_t acc_main = tmem + (uint32_t)b * MT::kBufCols, acc_corr = acc_main + kBN;
          uint32_t a[NT], bb[NT];
#pragma unroll
          for (int p = 0; p < NT; ++p) {
            a[p] = smem_u32(a_tile(s, p));
            bb[p] = smem_u32(b_tile(s, p));
          }
          // FP8: stage s's TMEM scale slot (8 columns per 128-K block: 4 for
          // A's scales, 4 for B's).  Its previous user, the stage's previous
          // round, has finished (the stage came back), so it is free.
          const uint32_t sf_slot = tmem + MT::kSfCol0 + 8u * MT::kSub * (uint32_t)s;
          if constexpr (MT::fp8) {
#pragma unroll
            for (int u = 0; u < MT::kSub; ++u) {
              tmem_cp_scales(sf_slot + 8u * u, smem_u32(sf_atom(s, 0)) + 512u * u);
              tmem_cp_scales(sf_slot + 8u * u + 4u, smem_u32(sf_atom(s, 1)) + 512u * u);
            }
          }
          auto mma = [&](uint32_t d, uint32_t ad, uint32_t bd, uint32_t accumulate) {
            if constexpr (PAIR)
              mma2_f16(d, sw128_kmajor_desc(ad), sw128_kmajor_desc(bd), idesc, accumulate);
            else
              mma_f16(d, sw128_kmajor_desc(ad), sw128_kmajor_desc(bd), idesc, accumulate);
          };
#pragma unroll
          for (int kk = 0; kk < MT::kKSteps; ++kk) {
            // 32 bytes along K per MMA inside the swizzled 128- / 64-byte
            // row: 16 bf16 (kind::f16) or 32 e4m3 (kind::mxf8f6f4)
            const uint32_t off = kk * 32;
            const uint32_t acc = (chunk_first && kk == 0) ? 0u : 1u;
            if constexpr (MT::fp8) {
              // 32-K sub-block kk of each 128-K scale block: byte kk of each scale word
#pragma unroll
              for (int u = 0; u < MT::kSub; ++u)
                mma_mxf8(acc_main, sw128_kmajor_desc(a[u] + off), sw128_kmajor_desc(bb[u] + off),
                         idesc_mxe4m3(kBM, kBN, kk, kk), sf_slot + 8u * u, sf_slot + 8u * u + 4u,
                         u == 0 ? acc : 1u);
            } else {
              // corrections, largest first: p0p1, p1p0 (+ p0p2, p1p1, p2p0)
              if constexpr (PAIR) {
                mma(acc_main, a[0] + off, bb[0] + off, acc);
                mma(acc_corr, a[0] + off, bb[1] + off, acc);
              } else {
                static_assert(CF::kBBytes == kBN * 128, "q1 must follow q0 directly");
                mma_f16(acc_main, sw128_kmajor_desc(a[0] + off), sw128_kmajor_desc(bb[0] + off), idesc_n256, acc);
              }
              mma(acc_corr, a[1] + off, bb[0] + off, 1u);
              if constexpr (P == 3) {
                mma(acc_corr, a[0] + off, bb[2] + off, 1u);
                mma(acc_corr, a[1] + off, bb[1] + off, 1u);
                mma(acc_corr, a[2] + off, bb[0] + off, 1u);
              }
            }
          }
          if constexpr (PAIR) {
            mma_commit2(&empty[s], 3);  // both CTAs' stage s
            if (chunk_last) mma_commit2(&tfull[b], 3);
          } else {
            mma_commit(&empty[s]);
            if (chunk_last) mma_commit(&tfull[b]);
          }
          ++consumed;
        }
      }
      // accf completes once every MMA issued above has finished, on the
      // normal path and after an abort alike, so TMEM (and, for a pair, the
      // peer's shared memory) is never released under a running MMA.
      if constexpr (PAIR)
        mma_commit2(accf, 1);
      else
        mma_commit(accf);
      if (*abort_flag) {
        int never = 0;
        (void)mbar_wait_bounded(accf, 0, &never, kWaitLimitNs);
      }
    }
  } else {
    // epilogue warps 2..: TMEM lane quarter = warp % 4 (the lanes a warp may
    // access), one tile row per thread; column slice (warp - 2) / 4 of kCols.
    constexpr int kCols = MT::kCols;
    const int q = warp & 3;
    const int col0 = ((warp - 2) >> 2) * kCols;
    const uint32_t trow = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)col0;
    int chunk_g = 0;
    for (int it = 0;; ++it) {
      const int slot = it % kTileRing, use = it / kTileRing;
      const bool got =
          __all_sync(0xffffffffu, mbar_wait_bounded(&ring_full[slot], use & 1, abort_flag, kWaitLimitNs));
      if (!got) {
        if (lane == 0) fail();
        break;
      }
      const int t = ring[slot];
      __syncwarp();
      if (lane == 0) mbar_arrive(&ring_empty[slot]);
      if (t < 0) break;
      const TcProblem& pr = probs[find_problem(probs, nprob, t)];
      int m0, n0;
      tile_coords<BMT>(pr, t, m0, n0);
      m0 += (int)rank * kBM;  // this CTA's rows
      const int nchunks = (pr.num_kt + MT::kChunk - 1) / MT::kChunk;
      float acc[kCols];
#pragma unroll
      for (int j = 0; j < kCols; ++j) acc[j] = 0.f;
      bool ok = true;
      for (int c = 0; c < nchunks; ++c, ++chunk_g) {
        const int b = chunk_g % MT::kBufs;
        // tcgen05.ld is warp-collective: make the decision warp-uniform.
        const bool ready =
            __all_sync(0xffffffffu, mbar_wait_bounded(&tfull[b], (chunk_g / MT::kBufs) & 1, abort_flag, kWaitLimitNs));
        if (!ready) {
          if (lane == 0) fail();
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t tb = trow + (uint32_t)b * MT::kBufCols;
        // the fold: FP8 has one accumulator per buffer, the splits two (main,
        // corrections), added with packed round-to-nearest FP32 adds
        if constexpr (MT::fp8) {
#pragma unroll
          for (int c0 = 0; c0 < kCols; c0 += 16) {
            float v0[16];
            tmem_ld16(tb + c0, v0);
            tmem_ld_wait();
#pragma unroll
            for (int j = 0; j < 16; j += 2) {
              const float2 r = __fadd2_rn(make_float2(acc[c0 + j], acc[c0 + j + 1]), make_float2(v0[j], v0[j + 1]));
              acc[c0 + j] = r.x;
              acc[c0 + j + 1] = r.y;
            }
          }
        } else {
#pragma unroll
          for (int c0 = 0; c0 < kCols; c0 += 16) {
            float v0[16], v1[16];
            tmem_ld16(tb + c0, v0);
            tmem_ld16(tb + kBN + c0, v1);
            tmem_ld_wait();
#pragma unroll
            for (int j = 0; j < 16; j += 2) {
              const float2 r = __fadd2_rn(make_float2(v0[j], v0[j + 1]), make_float2(v1[j], v1[j + 1]));
              const float2 q = __fadd2_rn(make_float2(acc[c0 + j], acc[c0 + j + 1]), r);
              acc[c0 + j] = q.x;
              acc[c0 + j + 1] = q.y;
            }
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) {
          if constexpr (PAIR)
            mbar_arrive_cluster(mapa_shared(smem_u32(&tempty[b]), 0));  // the MMA-issuing CTA's barrier
          else
            mbar_arrive(&tempty[b]);
        }
      }
      if (!ok) break;
      const int aborted = __shfl_sync(0xffffffffu, *abort_flag, 0);
      if (aborted) break;
      // FP16 split under the AUTO guard: outputs of out-of-span rows of A /
      // columns of B are left to f16_guard_fixup_kernel (bit c of skip_cols
      // = column col0 + c of the tile)
      bool skip_row = false;
      uint64_t skip_cols = 0;
      if constexpr (MT::f16) {
        // undo the row and column scales: acc * 2^(e_i + f_j - 30)
        const int* ea = reinterpret_cast<const int*>(sa);
        const int* eb = reinterpret_cast<const int*>(sb);
        const int ei = f16_row_exp(ea, (int64_t)pr.a_row + m0 + q * 32 + lane) - 2 * kF16ScaleTop;
#pragma unroll
        for (int c = 0; c < kCols; ++c)
          acc[c] = scale_pow2(acc[c], ei + f16_row_exp(eb, (int64_t)pr.b_row + n0 + col0 + c));
        if (guard_a) {
          skip_row = guard_a[(int64_t)pr.a_row + m0 + q * 32 + lane] != 0;
#pragma unroll
          for (int c = 0; c < kCols; ++c)
            if (__ldg(guard_b + (int64_t)pr.b_row + n0 + col0 + c)) skip_cols |= uint64_t(1) << c;
        }
      }
      if constexpr (CF::kTmaC) {
        if (pr.c_tma) {
          // C += the warp's 32 rows, 32 columns at a time, by TMA reduce-add
          // from a 128-byte-swizzled block (16-byte chunk c of row r at c ^ (r % 8)).
          // The warps hand C's update to the TMA unit and go back to folding
          // the next tile's chunks at once.  Outputs the AUTO guard leaves to
          // its fix-up add -0.0, which leaves every C value (-0.0 included)
          // as it was.
          if constexpr (MT::f16) {
            if (skip_row || skip_cols) {
#pragma unroll
              for (int c = 0; c < kCols; ++c)
                if (skip_row || ((skip_cols >> c) & 1)) acc[c] = -0.0f;
            }
          }
          float* scr = epi_scratch + (warp - 2) * 1024;
#pragma unroll
          for (int cb = 0; cb < kCols; cb += 32) {
#pragma unroll
            for (int c = 0; c < 8; ++c)
              *reinterpret_cast<float4*>(scr + lane * 32 + ((c ^ (lane & 7)) * 4)) =
                  make_float4(acc[cb + 4 * c], acc[cb + 4 * c + 1], acc[cb + 4 * c + 2], acc[cb + 4 * c + 3]);
            fence_proxy_async_shared();
            __syncwarp();
            const int bx = n0 + col0 + cb, by = m0 + q * 32;
            if (lane == 0 && bx < pr.N && by < pr.M) {  // boxes wholly outside C are skipped
              tma_reduce_add_2d(&pr.c_map, smem_u32(scr), bx, by);
              bulk_commit_group();
              bulk_wait_group_read0();  // the block is read before the next one overwrites it
            }
            __syncwarp();
          }
          continue;
        }
      }
      const int row = m0 + q * 32 + lane;
      if (row < pr.M && !skip_row) {
        float* crow = pr.C + (int64_t)row * pr.rsc;
        const bool vec = (pr.csc == 1) && ((pr.rsc & 3) == 0) && ((reinterpret_cast<uintptr_t>(pr.C) & 15) == 0) &&
                         skip_cols == 0;
        const int cn = n0 + col0;
        // C += acc; a split-K partial (overwrite) is stored instead, into
        // dense 16-byte-aligned rows
        const bool add = !pr.overwrite;
        if (vec && cn + kCols <= pr.N) {
          // 64 bytes at a time: four loads in flight before their stores
#pragma unroll
          for (int j0 = 0; j0 < kCols; j0 += 16) {
            float4* p = reinterpret_cast<float4*>(crow + cn + j0);
            float4 cv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) cv[u] = add ? p[u] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const int j = j0 + 4 * u;
              cv[u].x += acc[j];
              cv[u].y += acc[j + 1];
              cv[u].z += acc[j + 2];
              cv[u].w += acc[j + 3];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) p[u] = cv[u];
          }
        } else {
#pragma unroll
          for (int j = 0; j < kCols; ++j)
            if (cn + j < pr.N && !((skip_cols >> j) & 1)) {
              float* q = crow + (int64_t)(cn + j) * pr.csc;
              *q = add ? *q + acc[j] : acc[j];
            }
        }
      }
    }
  }

  // ---- teardown: drain in-flight copies if the pipeline stopped early,
  // make sure every tcgen05 op finished, free TMEM.  (In a pair, every copy of
  // both CTAs completes on the even CTA's stage barriers, so it drains for
  // both, and the odd CTA leaves only after the cluster barrier below.)
  // Single CTAs have two producers, each of which may have stopped at a
  // different slice: after the barrier below neither issues any more, and
  // the slices only one of them issued (at most a ring's worth, since each
  // waits for the consumer that needs both halves) get the missing arrival,
  // so every issued slice's stage completes once its copies have landed.
  if constexpr (!PAIR) __syncthreads();
  if (warp == 0 && lane == 0 && rank == 0 && *abort_flag) {
    int never = 0;
    int hi = issued;
    if constexpr (!PAIR) {
      const int ib = *b_issued_slot;
      const int lo = issued < ib ? issued : ib;
      hi = issued < ib ? ib : issued;
      for (int k = lo; k < hi; ++k) mbar_arrive(&full[k % ST]);
    }
    const int from = hi > ST ? hi - ST : 0;
    for (int k = from; k < hi; ++k) (void)mbar_wait_bounded(&full[k % ST], (k / ST) & 1, &never, kWaitLimitNs / 2);
  }
  if constexpr (PAIR) {
    // after an abort the odd CTA cannot see when its last copies (counted on
    // the even CTA's barriers) land in its shared memory: give them 100 us
    if (warp == 0 && lane == 0 && *abort_flag) {
      const uint64_t t0 = global_timer_ns();
      while (global_timer_ns() - t0 < 100000ull) {
      }
    }
  }
  // the epilogue's TMA reduce-add stores into C have completed
  if constexpr (CF::kTmaC) {
    if (warp >= 2 && warp < 2 + MT::kEpiWarps && lane == 0) bulk_wait_group0();
  }
  tc_fence_before();
  __syncthreads();
  if constexpr (PAIR) cluster_sync_all();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    if constexpr (PAIR)
      tmem_dealloc2(tmem, CF::kTmemCols);
    else
      tmem_dealloc(tmem, CF::kTmemCols);
  }
  if constexpr (PAIR) cluster_sync_all();
}

// The FP16 split's guard, second half: C += A B for the outputs the GEMM
// left alone - every column of each out-of-span row of A, and every row (not
// itself out of span) of each out-of-span column of B - as FP32 FMA dot
// products, one warp per output: lane l sums k = l, l + 32, ... in order,
// then the lanes' sums meet in a fixed shuffle tree.  Error at most
// (K / 32 + 5) eps32 (|A||B|)_ij, order fixed: the same bits on every run.
// CTAs take the listed rows in turn; with empty lists every CTA returns at
// once.  jobs: the A jobs then the B^T jobs of a group without split-K
// (problem i = job i).
__global__ void __launch_bounds__(256) f16_guard_fixup_kernel(const SplitJob* __restrict__ jobs, int njobs,
                                                              const TcProblem* __restrict__ probs,
                                                              const int* __restrict__ list_a,
                                                              const int* __restrict__ list_b,
                                                              const int* __restrict__ counts,
                                                              const int* __restrict__ flags_a) {
  const int na = counts[0], nb = counts[1];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  auto job_of = [&](const SplitJob* js, int64_t row) {  // last job with dst_row <= row
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (js[mid].dst_row <= row)
        lo = mid;
      else
        hi = mid - 1;
    }
    return lo;
  };
  auto dot = [&](const SplitJob& ja, int64_t i, const SplitJob& jb, int64_t jcol) {
    float s = 0.f;
    for (int64_t k = lane; k < ja.K; k += 32) s = fmaf(ja.src[i * ja.rs + k * ja.cs], jb.src[jcol * jb.rs + k * jb.cs], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
  };
  for (int e = blockIdx.x; e < na + nb; e += gridDim.x) {
    const bool row_entry = e < na;
    const int64_t r = row_entry ? list_a[e] : list_b[e - na];
    const int ji = job_of(row_entry ? jobs : jobs + njobs, r);
    const SplitJob& ja = jobs[ji];
    const SplitJob& jb = jobs[njobs + ji];
    const TcProblem& p = probs[ji];
    if (row_entry) {
      const int64_t i = r - ja.dst_row;  // every column of row i
      for (int64_t jc = warp; jc < p.N; jc += nwarps) {
        const float v = dot(ja, i, jb, jc);
        if (lane == 0) p.C[i * p.rsc + jc * p.csc] += v;
      }
    } else {
      const int64_t jc = r - jb.dst_row;  // every row of column jc, but the out-of-span rows' (done above)
      for (int64_t i = warp; i < p.M; i += nwarps) {
        if (flags_a[ja.dst_row + i]) continue;
        const float v = dot(ja, i, jb, jc);
        if (lane == 0) p.C[i * p.rsc + jc * p.csc] += v;
      }
    }
  }
}

// Split-K: C += part[0] + part[1] + ... (in that order) for every element of
// every split problem; blockIdx.y = problem, grid-stride over its elements.
__global__ void __launch_bounds__(256) splitk_reduce_kernel(const SplitReduce* __restrict__ jobs) {
  const SplitReduce j = jobs[blockIdx.y];
  const int64_t total = (int64_t)j.M * j.N, plane = (int64_t)j.M * j.pitch;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / j.N, c = e % j.N;
    const float* p = j.part + r * j.pitch + c;
    float sum = p[0];
    for (int s = 1; s < j.parts; ++s) sum += p[s * plane];
    j.C[r * j.rsc + c * j.csc] += sum;
  }
}

}  // namespace

// ------------------------------------------------------------ host side
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 3-D tensor map over `planes` planes of rows x cols (cols contiguous) BF16
// or 8-bit elements, planes one after another; box of box_rows x row_bytes
// (128 or 64) x all planes, with the swizzle of that row width.
gbblas_status make_map(CUtensorMap* map, const void* base, uint64_t rows, uint64_t cols, uint64_t planes,
                       uint32_t box_rows, bool bytes, uint32_t row_bytes) {
  auto fn = encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return GBBLAS_STATUS_CUDA_ERROR;
  }
  const uint64_t esize = bytes ? 1 : 2;
  cuuint64_t dims[3] = {cols, rows, planes};
  cuuint64_t strides[2] = {cols * esize, rows * cols * esize};
  cuuint32_t box[3] = {(cuuint32_t)(row_bytes / esize), box_rows, (cuuint32_t)planes};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, bytes ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3,
                  const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  row_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d) for %llu x %llu x %llu", (int)r, (unsigned long long)planes,
              (unsigned long long)rows, (unsigned long long)cols);
    return GBBLAS_STATUS_CUDA_ERROR;
  }
  return GBBLAS_STATUS_SUCCESS;
}

namespace {

inline int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

}  // namespace

gbblas_status make_map_f32_2d(CUtensorMap* map, const float* base, uint64_t inner, uint64_t outer,
                              uint64_t row_stride, uint32_t box_inner, uint32_t box_outer, bool swizzle128) {
  auto fn = encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return GBBLAS_STATUS_CUDA_ERROR;
  }
  cuuint64_t dims[2] = {inner, outer};
  cuuint64_t strides[1] = {row_stride * sizeof(float)};
  cuuint32_t box[2] = {box_inner, box_outer};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d) for a %llu x %llu float matrix", (int)r, (unsigned long long)outer,
              (unsigned long long)inner);
    return GBBLAS_STATUS_CUDA_ERROR;
  }
  return GBBLAS_STATUS_SUCCESS;
}

namespace {

// Bytes added to every arena row beyond the padded K.
constexpr int64_t kPitchPadBytes = 0;
inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

// Everything one tensor-core group launch needs: host tables, where they and
// the operand arena live on the device, and the two arena tensor maps.
struct TcGroupPlan {
  int mode = 2;  // 2 / 3 BF16 pieces, kModeFp8
  int nprob = 0;  // tile problems (a split-K problem counts once per part)
  int njobs = 0;  // operand preparations (one per problem of the group)
  int64_t a_rows = 0, b_rows = 0, tiles = 0;
  int64_t kpad = 0;   // longest padded K of the group (elements)
  int64_t pitch = 0;  // arena row pitch in elements (FP8: bytes): kpad + kPitchPadBytes
  int a_tiles = 0, b_tiles = 0;
  std::vector<TcProblem> probs;
  std::vector<SplitJob> ajobs, bjobs;
  std::vector<SplitReduce> reds;     // split-K problems' final sums
  std::vector<int64_t> part_off;     // per tile problem: byte offset of its partial in the workspace, or -1
  std::vector<int64_t> red_off;      // per reduction: byte offset of its first partial
  size_t off_probs = 0, off_jobs = 0, off_red = 0, off_arena = 0, off_sa = 0, off_sb = 0, off_ws = 0, bytes = 0;
  char* base = nullptr;  // device: zeroed header | problems | jobs | reductions | arena | FP8 scales | partials
  bool owned = false;    // base allocated by the plan (graph plans)
  CUtensorMap map_a, map_b;
  bool pair = false;  // CTA pairs computing 256 x 128 tiles (see gemm_split_kernel)
  bool guard = false;  // FP16 split with the AUTO guard (F16Guard, f16_guard_fixup_kernel)
  bool row_prep_a = false, row_prep_b = false;  // FP16 split: operand prepared by f16_row_prep_kernel
  bool col_scale_a = false, col_scale_b = false;  // FP16 split: exponents by f16_col_scale_kernel
  bool row_split_a = false, row_split_b = false;  // BF16 split: operand prepared by split_rows_kernel
  int a_col_ctas = 0, b_col_ctas = 0, col_kblk = 128;
  size_t off_gmin = 0, off_gflag = 0, off_glist = 0;  // guard arrays: A rows then B rows each
  size_t off_init_end = 0;  // the launch clears [kTileCounterOffset, off_init_end)
  std::vector<char> tables;  // host image of [off_probs, off_arena), copied with one memcpy
  bool fp8() const { return mode == kModeFp8; }
  bool f16() const { return mode == kModeF16; }
  int planes() const { return fp8() ? 1 : (f16() ? 2 : mode); }
  int slice_k() const {  // K elements per stage
    return fp8() ? ModeTraits<kModeFp8>::kBKe : (mode == 3 ? ModeTraits<3>::kBKe : ModeTraits<2>::kBKe);
  }
  int pad_k() const { return fp8() ? ModeTraits<kModeFp8>::kBKe : kBK; }  // K padding (multiple of stage and prep tile)
  int row_bytes() const { return mode == 3 ? ModeTraits<3>::kRowBytes : 128; }  // bytes of K per row per sub-tile
  int job_k() const { return fp8() ? 128 : 64; }     // K extent of one preparation tile (PrepTile::TK)
};

namespace {

// Host-side planning (no device work): problem order (largest K first),
// arena rows, tile numbering, split jobs, device layout.  opt.split > 1
// cuts every problem's K into that many parts (at most one per K stage),
// each a tile problem of its own that stores a partial; a reduction then adds
// the parts into C in order.  opt.pair forces the CTA form (-1: the
// GBBLAS_TC_PAIR setting).
gbblas_status plan_group(int mode, const gbblas_gemm_desc* d, int64_t count, TcGroupPlan& pl,
                         const TcLaunchOpts& opt = TcLaunchOpts()) {
  if (mode != 2 && mode != 3 && mode != kModeFp8 && mode != kModeF16 && mode != kModeF16Guard) {
    set_error("tensor-core gemm: unknown mode %d", mode);
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  pl.guard = mode == kModeF16Guard;
  if (pl.guard) mode = kModeF16;
  pl.mode = mode;
  const int64_t sk = pl.slice_k(), pk = pl.pad_k(), jk = pl.job_k(), jr = 4096 / jk;
  std::vector<int64_t> order;
  order.reserve(count);
  for (int64_t i = 0; i < count; ++i) {
    const gbblas_gemm_desc& g = d[i];
    if (g.M > (1 << 29) || g.N > (1 << 29) || g.K > (1 << 30)) {
      set_error("tensor-core gemm: problem %lld too large for the tile grid", (long long)i);
      return GBBLAS_STATUS_NOT_SUPPORTED;
    }
    if (g.M > 0 && g.N > 0 && g.K > 0) order.push_back(i);
  }
  std::stable_sort(order.begin(), order.end(), [&](int64_t x, int64_t y) { return d[x].K > d[y].K; });
  // Single CTAs by default: at 8192^3 CTA pairs measured the same for the
  // three-product split (458 vs 459 TFLOP/s) and +1 % for six products.
  // Pairs (GBBLAS_TC_PAIR=1, or the autotuner's choice for a shape) run the
  // split where padding every problem to 256 rows adds at most 10 % of MMA
  // work (FP8 always runs on single CTAs).
  bool want_pair = opt.pair == 1;
  if (opt.pair < 0)
    if (const char* e = std::getenv("GBBLAS_TC_PAIR"); e && e[0] == '1') want_pair = true;
  if (want_pair && mode != kModeFp8 && mode != kModeF16) {
    double w1 = 0, w2 = 0;
    for (int64_t i : order) {
      const double nk = (double)round_up(d[i].N, kBN) * (double)round_up(d[i].K, pk);
      w1 += (double)round_up(d[i].M, kBM) * nk;
      w2 += (double)round_up(d[i].M, 2 * kBM) * nk;
    }
    pl.pair = w2 <= 1.1 * w1;
  }
  const int64_t bmt = pl.pair ? 2 * kBM : kBM;  // output tile rows
  pl.njobs = (int)order.size();
  pl.ajobs.resize(pl.njobs);
  pl.bjobs.resize(pl.njobs);
  for (int i = 0; i < pl.njobs; ++i) pl.kpad = std::max<int64_t>(pl.kpad, round_up(d[order[i]].K, pk));
  pl.pitch = pl.kpad + kPitchPadBytes / (pl.fp8() ? 1 : (int64_t)sizeof(__nv_bfloat16));
  int64_t ws = 0;  // partial workspace bytes
  for (int i = 0; i < pl.njobs; ++i) {
    const gbblas_gemm_desc& g = d[order[i]];
    const int64_t Mp = round_up(g.M, bmt), Np = round_up(g.N, kBN), Kp = round_up(g.K, pk);
    const int num_kt = (int)(Kp / sk);  // pk is a multiple of sk
    // (the guard's fixup pairs problem i with job i: no split-K under it)
    const int parts = pl.guard ? 1 : std::max(1, std::min(opt.split, num_kt));
    const int64_t ppitch = round_up(g.N, 4);  // partial rows stay 16-byte aligned
    if (parts > 1) {
      pl.reds.push_back({g.C, g.rsc, g.csc, nullptr, (int)g.M, (int)g.N, (int)ppitch, parts});
      pl.red_off.push_back(ws);
    }
    for (int part = 0; part < parts; ++part) {
      TcProblem p;
      p.M = (int)g.M;
      p.N = (int)g.N;
      p.kt0 = (int)((int64_t)num_kt * part / parts);
      p.num_kt = (int)((int64_t)num_kt * (part + 1) / parts) - p.kt0;
      p.a_row = (int)pl.a_rows;
      p.b_row = (int)pl.b_rows;
      p.tiles_m = (int)(Mp / bmt);
      p.tiles_n = (int)(Np / kBN);
      p.tile_start = (int)pl.tiles;
      p.overwrite = parts > 1 ? 1 : 0;
      p.C = parts > 1 ? nullptr : g.C;  // partials: pointed into the workspace when bound
      p.rsc = parts > 1 ? ppitch : g.rsc;
      p.csc = parts > 1 ? 1 : g.csc;
      p.c_tma = 0;
      // single CTAs add their results into C with TMA reduce-add stores
      // where C rows are contiguous, 16-byte aligned and 16-byte-multiple
      // apart (split-K partials are stored by the register path)
      if (!pl.pair && parts == 1 && g.csc == 1 && g.rsc >= g.N && (g.rsc % 4) == 0 &&
          (reinterpret_cast<uintptr_t>(g.C) & 15) == 0 &&
          make_map_f32_2d(&p.c_map, g.C, (uint64_t)g.N, (uint64_t)g.M, (uint64_t)g.rsc, 32, 32, true) ==
              GBBLAS_STATUS_SUCCESS)
        p.c_tma = 1;
      pl.probs.push_back(p);
      pl.part_off.push_back(parts > 1 ? ws : -1);
      if (parts > 1) ws += (int64_t)g.M * ppitch * (int64_t)sizeof(float);
      pl.tiles += (int64_t)p.tiles_m * p.tiles_n;
    }
    pl.ajobs[i] = {g.A, g.M, g.K, g.rsa, g.csa, pl.a_rows, (int)(Mp / jr), (int)(Kp / jk), pl.a_tiles};
    pl.a_tiles += pl.ajobs[i].tiles_r * pl.ajobs[i].tiles_k;
    // B^T: element (n, k) = B[k*rsb + n*csb]
    pl.bjobs[i] = {g.B, g.N, g.K, g.csb, g.rsb, pl.b_rows, (int)(Np / jr), (int)(Kp / jk), pl.b_tiles};
    pl.b_tiles += pl.bjobs[i].tiles_r * pl.bjobs[i].tiles_k;
    pl.a_rows += Mp;
    pl.b_rows += Np;
  }
  pl.nprob = (int)pl.probs.size();
  if (pl.mode == 2 || pl.mode == 3) {
    // the BF16 split's pieces straight from registers where every job of an
    // operand has K contiguous, 16-byte aligned rows and K a multiple of 4
    auto split_ok = [](const SplitJob& j) {
      return j.cs == 1 && (j.rs & 3) == 0 && (reinterpret_cast<uintptr_t>(j.src) & 15) == 0 && (j.K & 3) == 0;
    };
    pl.row_split_a = std::all_of(pl.ajobs.begin(), pl.ajobs.end(), split_ok);
    pl.row_split_b = std::all_of(pl.bjobs.begin(), pl.bjobs.end(), split_ok);
  }
  if (pl.f16()) {
    // one-pass preparation where every job of an operand has K contiguous,
    // 16-byte aligned rows, K a multiple of 4 within the kernel's reach
    auto row_ok = [](const SplitJob& j) {
      return j.cs == 1 && (j.rs & 3) == 0 && (reinterpret_cast<uintptr_t>(j.src) & 15) == 0 && (j.K & 3) == 0 &&
             j.K >= kRowPrepMinK && (int64_t)j.tiles_k * PrepTile<kModeF16>::TK <= 1024 * kRowPrepNV;
    };
    pl.row_prep_a = std::all_of(pl.ajobs.begin(), pl.ajobs.end(), row_ok);
    pl.row_prep_b = std::all_of(pl.bjobs.begin(), pl.bjobs.end(), row_ok);
    // the exponents of an operand whose rows are contiguous by a column
    // reduction (its pieces still come from the tile kernel)
    auto col_ok = [](const SplitJob& j) {
      return j.rs == 1 && (j.cs & 3) == 0 && (reinterpret_cast<uintptr_t>(j.src) & 15) == 0 && (j.rows & 3) == 0;
    };
    auto number = [](std::vector<SplitJob>& jobs, int kblk) {
      int64_t n = 0;
      for (SplitJob& j : jobs) {
        j.col_start = (int)n;
        n += ((j.rows + 1023) / 1024) * ((j.K + kblk - 1) / kblk);
      }
      return n;
    };
    pl.col_scale_a = !pl.row_prep_a && std::all_of(pl.ajobs.begin(), pl.ajobs.end(), col_ok);
    pl.col_scale_b = !pl.row_prep_b && std::all_of(pl.bjobs.begin(), pl.bjobs.end(), col_ok);
    // (shorter K ranges for more CTAs measured slower: 28.6 against 24.5 us
    // for a 4096^2 operand with 16 instead of 128 of K per CTA)
    pl.col_kblk = kColScaleK;
    const int64_t na = pl.col_scale_a ? number(pl.ajobs, pl.col_kblk) : 0,
                  nb = pl.col_scale_b ? number(pl.bjobs, pl.col_kblk) : 0;
    if (na + nb >= (1ll << 31)) pl.col_scale_a = pl.col_scale_b = false;
    pl.a_col_ctas = pl.col_scale_a ? (int)na : 0;
    pl.b_col_ctas = pl.col_scale_b ? (int)nb : 0;
  }
  if ((double)(pl.a_rows + pl.b_rows) * pl.planes() >= 2.0e9 || pl.tiles >= (1ll << 31) ||
      (double)pl.a_tiles >= 2.0e9 || (double)pl.b_tiles >= 2.0e9) {
    set_error("tensor-core gemm: group too large for one launch");
    return GBBLAS_STATUS_NOT_SUPPORTED;
  }
  const size_t esize = pl.fp8() ? 1 : sizeof(__nv_bfloat16);
  const size_t guard_rows = pl.guard ? (size_t)(pl.a_rows + pl.b_rows) : 0;
  // FP16 split: the row exponents (and the guard's minima) right after the
  // zeroed header, so that one memset from the tile counter on clears them
  size_t off = kScratchZeroBytes;
  if (pl.f16()) {
    pl.off_sa = off;
    off += align256((size_t)pl.a_rows * sizeof(int));
    pl.off_sb = off;
    off += align256((size_t)pl.b_rows * sizeof(int));
    pl.off_gmin = off;
    off += align256(guard_rows * sizeof(unsigned));
  }
  pl.off_init_end = off;
  pl.off_probs = off;
  pl.off_jobs = pl.off_probs + align256(sizeof(TcProblem) * pl.nprob);
  pl.off_red = pl.off_jobs + align256(sizeof(SplitJob) * 2 * pl.njobs);
  pl.off_arena = pl.off_red + align256(sizeof(SplitReduce) * pl.reds.size());
  const size_t a_plane = (size_t)(pl.a_rows * pl.pitch), b_plane = (size_t)(pl.b_rows * pl.pitch);
  off = pl.off_arena + align256((size_t)pl.planes() * (a_plane + b_plane) * esize);
  if (pl.fp8()) {  // FP8: one 4-byte scale word per row and K-block
    const size_t kb = (size_t)(pl.kpad / 128);
    pl.off_sa = off;
    off += align256(kb * (size_t)pl.a_rows * sizeof(uint32_t));
    pl.off_sb = off;
    off += align256(kb * (size_t)pl.b_rows * sizeof(uint32_t));
  }
  pl.off_gflag = off;
  pl.off_glist = pl.off_gflag + align256(guard_rows * sizeof(int));
  pl.off_ws = pl.off_glist + align256(guard_rows * sizeof(int));
  pl.bytes = pl.off_ws + align256((size_t)ws);
  return GBBLAS_STATUS_SUCCESS;
}

char* arena_a(const TcGroupPlan& pl) { return pl.base + pl.off_arena; }
char* arena_b(const TcGroupPlan& pl) {
  const size_t esize = pl.fp8() ? 1 : sizeof(__nv_bfloat16);
  return arena_a(pl) + (size_t)pl.planes() * (size_t)(pl.a_rows * pl.pitch) * esize;
}
uint32_t* scales_a(const TcGroupPlan& pl) { return reinterpret_cast<uint32_t*>(pl.base + pl.off_sa); }
uint32_t* scales_b(const TcGroupPlan& pl) { return reinterpret_cast<uint32_t*>(pl.base + pl.off_sb); }

// Point the plan at device memory `base` (>= pl.bytes, header zeroed), copy
// the tables there on `stream`, and encode the arena tensor maps.
gbblas_status bind_group(TcGroupPlan& pl, char* base, cudaStream_t stream) {
  pl.base = base;
  if (pl.nprob == 0) return GBBLAS_STATUS_SUCCESS;
  for (int i = 0; i < pl.nprob; ++i)
    if (pl.part_off[i] >= 0) pl.probs[i].C = reinterpret_cast<float*>(base + pl.off_ws + pl.part_off[i]);
  for (size_t r = 0; r < pl.reds.size(); ++r)
    pl.reds[r].part = reinterpret_cast<const float*>(base + pl.off_ws + pl.red_off[r]);
  // problems, jobs and reductions as one host image and one copy (the image
  // lives in the plan, which outlives the copy)
  pl.tables.assign(pl.off_arena - pl.off_probs, 0);
  char* h = pl.tables.data();
  std::memcpy(h, pl.probs.data(), sizeof(TcProblem) * pl.nprob);
  std::memcpy(h + (pl.off_jobs - pl.off_probs), pl.ajobs.data(), sizeof(SplitJob) * pl.njobs);
  std::memcpy(h + (pl.off_jobs - pl.off_probs) + sizeof(SplitJob) * pl.njobs, pl.bjobs.data(),
              sizeof(SplitJob) * pl.njobs);
  if (!pl.reds.empty())
    std::memcpy(h + (pl.off_red - pl.off_probs), pl.reds.data(), sizeof(SplitReduce) * pl.reds.size());
  GB_CUDA_TRY(cudaMemcpyAsync(base + pl.off_probs, h, pl.tables.size(), cudaMemcpyHostToDevice, stream));
  GB_TRY(make_map(&pl.map_a, arena_a(pl), (uint64_t)pl.a_rows, (uint64_t)pl.pitch, (uint64_t)pl.planes(), kBM,
                  pl.fp8(), pl.row_bytes()));
  GB_TRY(make_map(&pl.map_b, arena_b(pl), (uint64_t)pl.b_rows, (uint64_t)pl.pitch, (uint64_t)pl.planes(),
                  pl.pair ? kBN / 2 : kBN, pl.fp8(), pl.row_bytes()));
  return GBBLAS_STATUS_SUCCESS;
}

// Kernel attributes (dynamic shared memory) and how many CTAs (single) or
// CTA pairs (PAIR) are resident at once on this device; set once per device,
// before any launch or stream capture.
template <int MODE, bool PAIR>
int kernel_setup(DeviceCtx* c) {
  using CF = TcCfg<MODE, PAIR>;
  static std::mutex mu;
  static int resident[64] = {0};
  std::lock_guard<std::mutex> lk(mu);
  int& n = resident[c->device & 63];
  if (n == 0) {
    cudaFuncSetAttribute(gemm_split_kernel<MODE, PAIR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CF::kSmem);
    n = c->num_sms;
    if (PAIR) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(2 * c->num_sms);
      cfg.blockDim = dim3(ModeTraits<MODE>::kThreads);
      cfg.dynamicSmemBytes = CF::kSmem;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = 2;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int k = 0;
      n = (cudaOccupancyMaxActiveClusters(&k, gemm_split_kernel<MODE, PAIR>, &cfg) == cudaSuccess && k > 0)
              ? k
              : c->num_sms / 2;
      cudaGetLastError();  // a refused query leaves no sticky error behind
    }
  }
  return n;
}

template <int MODE, bool PAIR>
gbblas_status launch_gemm_kernel(DeviceCtx* c, const TcGroupPlan& pl, cudaStream_t stream, int max_ctas,
                                 int tile_begin, int tile_end) {
  using CF = TcCfg<MODE, PAIR>;
  int* err = reinterpret_cast<int*>(pl.base + kErrWordOffset);
  int* counter = reinterpret_cast<int*>(pl.base + kTileCounterOffset);
  const auto* dprobs = reinterpret_cast<const TcProblem*>(pl.base + pl.off_probs);
  const int resident = kernel_setup<MODE, PAIR>(c);
  int units = (int)std::min<int64_t>(tile_end - tile_begin, resident);  // CTAs, or CTA pairs
  if (max_ctas > 0) {
    const int cap = PAIR ? std::max(1, max_ctas / 2) : max_ctas;
    if (units > cap) units = cap;
  }
  if constexpr (!PAIR) {
    const int* ga = pl.guard ? reinterpret_cast<const int*>(pl.base + pl.off_gflag) : nullptr;
    gemm_split_kernel<MODE, false><<<units, ModeTraits<MODE>::kThreads, CF::kSmem, stream>>>(
        pl.map_a, pl.map_b, dprobs, pl.nprob, tile_begin, tile_end, pl.kpad, counter, err, scales_a(pl), scales_b(pl), ga,
        ga ? ga + pl.a_rows : nullptr);
    return check_launch("gemm_split_kernel");
  } else {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2 * units);
  cfg.blockDim = dim3(ModeTraits<MODE>::kThreads);
  cfg.dynamicSmemBytes = CF::kSmem;
  cfg.stream = stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 2;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  const cudaError_t e =
      cudaLaunchKernelEx(&cfg, gemm_split_kernel<MODE, true>, pl.map_a, pl.map_b, dprobs, pl.nprob, tile_begin,
                         tile_end, pl.kpad, counter, err, (const uint32_t*)scales_a(pl), (const uint32_t*)scales_b(pl),
                         (const int*)nullptr, (const int*)nullptr);
  if (e != cudaSuccess) {
    count_launch();
    set_error("launch of gemm_split_kernel (CTA pairs) failed: %s", cudaGetErrorString(e));
    return GBBLAS_STATUS_CUDA_ERROR;
  }
  return check_launch("gemm_split_kernel");
  }
}

template <int MODE>
gbblas_status launch_bound(DeviceCtx* c, const TcGroupPlan& pl, cudaStream_t stream, int max_ctas, int slices) {
  if (pl.nprob == 0) return GBBLAS_STATUS_SUCCESS;
  const auto* djobs = reinterpret_cast<const SplitJob*>(pl.base + pl.off_jobs);
  // the tile counter, the guard's counts and (FP16 split) the row exponents
  // and minima: zero, in one memset
  GB_CUDA_TRY(cudaMemsetAsync(pl.base + kTileCounterOffset, 0, pl.off_init_end - kTileCounterOffset, stream));
  F16Guard ga, gb;  // AUTO guard arrays (A rows, then B^T rows)
  int* gcounts = reinterpret_cast<int*>(pl.base + kGuardCountOffset);
  if (pl.guard) {
    unsigned* gmin = reinterpret_cast<unsigned*>(pl.base + pl.off_gmin);
    int* gflag = reinterpret_cast<int*>(pl.base + pl.off_gflag);
    int* glist = reinterpret_cast<int*>(pl.base + pl.off_glist);
    ga = F16Guard{gmin, gflag, glist, gcounts};
    gb = F16Guard{gmin + pl.a_rows, gflag + pl.a_rows, glist + pl.a_rows, gcounts + 1};
  }
  // tiles of the operands the tile kernels prepare (the FP16 split's
  // one-pass operands are done by f16_row_prep_kernel instead)
  const int a_tiles = (pl.row_prep_a || pl.row_split_a) ? 0 : pl.a_tiles,
            b_tiles = (pl.row_prep_b || pl.row_split_b) ? 0 : pl.b_tiles;
  const int prep_ctas = a_tiles + b_tiles;
  if constexpr (MODE == 2 || MODE == 3) {
    if (pl.row_split_a || pl.row_split_b) {
      const RowSplitSide ra{djobs, pl.row_split_a ? (int)pl.a_rows : 0,
                            reinterpret_cast<__nv_bfloat16*>(arena_a(pl)), (int64_t)(pl.a_rows * pl.pitch)};
      const RowSplitSide rb{djobs + pl.njobs, pl.row_split_b ? (int)pl.b_rows : 0,
                            reinterpret_cast<__nv_bfloat16*>(arena_b(pl)), (int64_t)(pl.b_rows * pl.pitch)};
      // arena rows come in multiples of 128 per job: whole CTAs of 8 or 32 rows
      const int64_t rows = (int64_t)ra.rows + rb.rows;
      const int rpc = rows / kSplitRowsPerCtaMax >= 4 * (int64_t)c->num_sms ? kSplitRowsPerCtaMax : 8;
      split_rows_kernel<MODE><<<(unsigned)(rows / rpc), 256, 0, stream>>>(ra, rb, pl.njobs, pl.pitch, rpc);
      GB_TRY(check_launch("split_rows_kernel"));
    }
  }
  if constexpr (MODE == kModeF16) {
    if (pl.row_prep_a || pl.row_prep_b) {
      const RowPrepSide ra{djobs, pl.row_prep_a ? (int)pl.a_rows : 0, reinterpret_cast<__half*>(arena_a(pl)),
                           (int64_t)(pl.a_rows * pl.pitch), reinterpret_cast<int*>(scales_a(pl)), ga};
      const RowPrepSide rb{djobs + pl.njobs, pl.row_prep_b ? (int)pl.b_rows : 0,
                           reinterpret_cast<__half*>(arena_b(pl)), (int64_t)(pl.b_rows * pl.pitch),
                           reinterpret_cast<int*>(scales_b(pl)), gb};
      f16_row_prep_kernel<<<ra.rows + rb.rows, 256, 0, stream>>>(ra, rb, pl.njobs, pl.pitch);
      GB_TRY(check_launch("f16_row_prep_kernel"));
    }
    // per-row exponents of A's and B^T's arena rows (and the guard's
    // minima) for the operands the tile kernel prepares: by the column
    // reduction where the rows are contiguous, else by tiles
    const int a_cols = pl.col_scale_a ? pl.a_col_ctas : 0, b_cols = pl.col_scale_b ? pl.b_col_ctas : 0;
    if (a_cols + b_cols > 0) {
      const ScaleSide sa{djobs, a_cols, reinterpret_cast<int*>(scales_a(pl)), const_cast<unsigned*>(ga.emin)};
      const ScaleSide sb{djobs + pl.njobs, b_cols, reinterpret_cast<int*>(scales_b(pl)),
                         const_cast<unsigned*>(gb.emin)};
      f16_col_scale_kernel<<<a_cols + b_cols, 256, 0, stream>>>(sa, sb, pl.njobs, pl.col_kblk);
      GB_TRY(check_launch("f16_col_scale_kernel"));
    }
    const int a_st = pl.col_scale_a ? 0 : a_tiles, b_st = pl.col_scale_b ? 0 : b_tiles;
    if (a_st + b_st > 0) {
      const ScaleSide sa{djobs, a_st, reinterpret_cast<int*>(scales_a(pl)), const_cast<unsigned*>(ga.emin)};
      const ScaleSide sb{djobs + pl.njobs, b_st, reinterpret_cast<int*>(scales_b(pl)),
                         const_cast<unsigned*>(gb.emin)};
      f16_scale_kernel<<<a_st + b_st, 256, 0, stream>>>(sa, sb, pl.njobs);
      GB_TRY(check_launch("f16_scale_kernel"));
    }
  }
  // the pieces (FP8: values and scale words, 128 per K-block of each 128-row
  // block, i.e. `kpad` per row block) of both operands
  if (prep_ctas > 0) {
    const PrepSide pa{djobs, a_tiles, arena_a(pl), (int64_t)(pl.a_rows * pl.pitch), scales_a(pl), ga};
    const PrepSide pb{djobs + pl.njobs, b_tiles, arena_b(pl), (int64_t)(pl.b_rows * pl.pitch), scales_b(pl), gb};
    prep_group_kernel<MODE><<<prep_ctas, 256, 0, stream>>>(pa, pb, pl.njobs, pl.pitch, pl.kpad);
    GB_TRY(check_launch("prep_group_kernel"));
  }
  // the GEMM, as `slices` launches over consecutive ranges of whole waves of
  // tiles (higher-priority work on other streams gets the SMs between them);
  // each launch restarts the tile counter
  const bool pair = MODE != kModeFp8 && MODE != kModeF16 && pl.pair;
  int64_t wave = std::min<int64_t>(pl.tiles, pair ? c->num_sms / 2 : c->num_sms);
  if (max_ctas > 0) wave = std::min<int64_t>(wave, pair ? std::max(1, max_ctas / 2) : max_ctas);
  wave = std::max<int64_t>(wave, 1);
  const int64_t waves = (pl.tiles + wave - 1) / wave;
  const int64_t nsl = std::max<int64_t>(1, std::min<int64_t>(slices, waves));
  gbblas_status st = GBBLAS_STATUS_SUCCESS;
  for (int64_t sl = 0; sl < nsl && st == GBBLAS_STATUS_SUCCESS; ++sl) {
    const int tb = (int)(wave * (waves * sl / nsl)), te = (int)std::min<int64_t>(pl.tiles, wave * (waves * (sl + 1) / nsl));
    if (sl > 0)
      GB_CUDA_TRY(cudaMemsetAsync(pl.base + kTileCounterOffset, 0, sizeof(int), stream));
    if constexpr (MODE != kModeFp8 && MODE != kModeF16) {
      st = pl.pair ? launch_gemm_kernel<MODE, true>(c, pl, stream, max_ctas, tb, te)
                   : launch_gemm_kernel<MODE, false>(c, pl, stream, max_ctas, tb, te);
    } else {
      st = launch_gemm_kernel<MODE, false>(c, pl, stream, max_ctas, tb, te);
    }
  }
  if (st == GBBLAS_STATUS_SUCCESS && pl.guard) {
    f16_guard_fixup_kernel<<<2 * c->num_sms, 256, 0, stream>>>(
        djobs, pl.njobs, reinterpret_cast<const TcProblem*>(pl.base + pl.off_probs), ga.list, gb.list, gcounts,
        ga.flags);
    st = check_launch("f16_guard_fixup_kernel");
  }
  if (st != GBBLAS_STATUS_SUCCESS || pl.reds.empty()) return st;
  int64_t most = 0;
  for (const SplitReduce& r : pl.reds) most = std::max<int64_t>(most, (int64_t)r.M * r.N);
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((most + 255) / 256, 4 * (int64_t)c->num_sms));
  splitk_reduce_kernel<<<dim3(blocks, (unsigned)pl.reds.size()), 256, 0, stream>>>(
      reinterpret_cast<const SplitReduce*>(pl.base + pl.off_red));
  return check_launch("splitk_reduce_kernel");
}

}  // namespace

int gemm_slices_env() {
  const char* e = std::getenv("GBBLAS_GEMM_SLICES");
  const int v = e ? std::atoi(e) : 1;
  return v > 1 ? v : 1;
}

int tc_stage_k(int mode) {
  if (mode == kModeF16Guard) mode = kModeF16;
  return mode == kModeFp8 ? ModeTraits<kModeFp8>::kBKe : (mode == 3 ? ModeTraits<3>::kBKe : ModeTraits<2>::kBKe);
}

int tc_mode(gbblas_accuracy acc) {
  switch (acc) {
    case GBBLAS_ACCURACY_BF16X3: return 2;
    case GBBLAS_ACCURACY_BF16X6: return 3;
    case GBBLAS_ACCURACY_FP8: return kModeFp8;
    case GBBLAS_ACCURACY_FP16X3: return kModeF16;
    default: return 0;
  }
}

size_t tc_arena_bytes(int mode, int64_t M, int64_t N, int64_t K) {
  const bool guard = mode == kModeF16Guard;
  if (guard) mode = kModeF16;
  const bool fp8 = mode == kModeFp8;
  const int64_t planes = fp8 ? 1 : (mode == kModeF16 ? 2 : mode), sk = fp8 ? ModeTraits<kModeFp8>::kBKe : kBK;
  const int64_t rows = round_up(M, 2 * kBM) + round_up(N, kBN), Kp = round_up(K, sk);
  return (size_t)(rows * (Kp * (fp8 ? 1 : 2) + kPitchPadBytes) * planes + (fp8 ? rows * (Kp / 128) * 4 : 0) +
                  (mode == kModeF16 ? rows * 4 : 0) + (guard ? rows * 12 : 0));
}

void tc_prepare(DeviceCtx* c) {
  sgemm_tma_prepare(c);
  dgemm_digits_prepare(c);
  kernel_setup<2, false>(c);
  kernel_setup<3, false>(c);
  kernel_setup<kModeFp8, false>(c);
  kernel_setup<kModeF16, false>(c);
  kernel_setup<2, true>(c);
  kernel_setup<3, true>(c);
}

gbblas_status tc_group_launch(DeviceCtx* c, const TcGroupPlan* pl, cudaStream_t stream, int max_ctas, int slices) {
  switch (pl->mode) {
    case 3: return launch_bound<3>(c, *pl, stream, max_ctas, slices);
    case kModeFp8: return launch_bound<kModeFp8>(c, *pl, stream, max_ctas, slices);
    case kModeF16: return launch_bound<kModeF16>(c, *pl, stream, max_ctas, slices);
    default: return launch_bound<2>(c, *pl, stream, max_ctas, slices);
  }
}

gbblas_status tc_group_create(DeviceCtx* c, int mode, const gbblas_gemm_desc* descs, int64_t count,
                              TcGroupPlan** out) {
  (void)c;
  TcGroupPlan* pl = new TcGroupPlan();
  gbblas_status st = plan_group(mode, descs, count, *pl);
  if (st != GBBLAS_STATUS_SUCCESS) {
    delete pl;
    return st;
  }
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, pl->bytes);
  if (e != cudaSuccess) {
    delete pl;
    set_error("grouped gemm plan: allocation of %zu bytes failed: %s", pl->bytes, cudaGetErrorString(e));
    return GBBLAS_STATUS_ALLOC_FAILED;
  }
  pl->owned = true;
  e = cudaMemset(p, 0, kScratchZeroBytes);
  if (e == cudaSuccess) {
    st = bind_group(*pl, static_cast<char*>(p), nullptr);
    if (st == GBBLAS_STATUS_SUCCESS && cudaDeviceSynchronize() != cudaSuccess) st = GBBLAS_STATUS_CUDA_ERROR;
  } else {
    st = GBBLAS_STATUS_CUDA_ERROR;
  }
  if (st != GBBLAS_STATUS_SUCCESS) {
    cudaFree(p);
    delete pl;
    return st;
  }
  *out = pl;
  return GBBLAS_STATUS_SUCCESS;
}

void tc_group_destroy(TcGroupPlan* pl) {
  if (!pl) return;
  if (pl->owned && pl->base) cudaFree(pl->base);
  delete pl;
}

int* tc_group_error_word(const TcGroupPlan* pl) {
  return pl->base ? reinterpret_cast<int*>(pl->base + kErrWordOffset) : nullptr;
}

gbblas_status launch_gemm_tc_group(DeviceCtx* c, int mode, const gbblas_gemm_desc* descs, int64_t count,
                                   cudaStream_t stream, int max_ctas, int slices) {
  TcGroupPlan pl;
  GB_TRY(plan_group(mode, descs, count, pl));
  if (pl.nprob == 0) return GBBLAS_STATUS_SUCCESS;
  void* s = nullptr;
  GB_TRY(get_scratch(c, stream, pl.bytes, &s));
  GB_TRY(bind_group(pl, static_cast<char*>(s), stream));
  return tc_group_launch(c, &pl, stream, max_ctas, slices);
}

gbblas_status launch_gemm_tc_opts(DeviceCtx* c, int mode, const gbblas_gemm_desc& d, const TcLaunchOpts& opt,
                                  cudaStream_t stream) {
  TcGroupPlan pl;
  GB_TRY(plan_group(mode, &d, 1, pl, opt));
  if (pl.nprob == 0) return GBBLAS_STATUS_SUCCESS;
  void* s = nullptr;
  GB_TRY(get_scratch(c, stream, pl.bytes, &s));
  GB_TRY(bind_group(pl, static_cast<char*>(s), stream));
  return tc_group_launch(c, &pl, stream, 0, gemm_slices_env());
}

gbblas_status launch_gemm_tc(DeviceCtx* c, int mode, int64_t M, int64_t N, int64_t K, const float* A, int64_t rsa,
                             int64_t csa, const float* B, int64_t rsb, int64_t csb, float* C, int64_t rsc,
                             int64_t csc, cudaStream_t stream) {
  if (M == 0 || N == 0 || K == 0) return GBBLAS_STATUS_SUCCESS;
  gbblas_gemm_desc d{M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc};
  // (the guarded FP16 split runs single CTAs without split-K: nothing to tune)
  return launch_gemm_tc_opts(c, mode, d, mode == kModeF16Guard ? TcLaunchOpts() : tuned_tc_opts(c, mode, M, N, K, stream),
                             stream);
}

}  // namespace gbblas
