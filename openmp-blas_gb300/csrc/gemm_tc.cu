// gemm_tc.cu - FP32-accurate GEMM on the 5th-generation tensor cores
// (split-BF16), single and grouped.  C += A * B for float A, B, C of any
// layout; a group is any number of independent problems of any shapes.
//
//   1. split_group_kernel: every FP32 operand element a becomes P BF16 pieces
//      p0 = bf16_rn(a), p1 = bf16_rn(a - p0), p2 = bf16_rn(a - p0 - p1),
//      written K-major (A as M x K, B as its transpose N x K) into one arena
//      per operand kind: all problems' rows stacked, one common K pitch,
//      piece planes one after another.  One pair of TMA tensor maps then
//      covers every problem of the group.
//   2. gemm_split_kernel (persistent, one CTA per SM): a device-side tile
//      scheduler hands out 128 x 128 output tiles of all problems (largest K
//      first) through an atomic counter.  Per tile: C += sum of the piece
//      products p_i(A) p_j(B) with i + j < P by tcgen05.mma (kind::f16, BF16
//      in, FP32 accumulate) into two TMEM accumulators - p0*p0 alone, and
//      every smaller product together (so small terms are summed at their own
//      scale).  K is walked in chunks of 512: each chunk accumulates in one of
//      two TMEM buffers while the epilogue warps fold the previous chunk into
//      FP32 registers with round-to-nearest adds (the tensor core's own
//      accumulation over long K is measurably less accurate than FP32); the
//      registers go into C once per tile.  The chunk buffers carry over from
//      tile to tile, so a tile's epilogue overlaps the next tile's MMAs.
//        P = 2 ("bf16x3"):  p0p0 + (p0p1 + p1p0)                     3 MMAs
//        P = 3 ("bf16x6"):  p0p0 + (p0p1 + p1p0 + p0p2 + p1p1 + p2p0) 6 MMAs
//      Three pieces hold all 24 significand bits of an FP32 value and the
//      dropped products are below 2^-23 of |a||b|: bf16x6 is at least as
//      accurate as FP32 FMA arithmetic.  bf16x3 keeps about 16 bits.
//
// Warp roles (192 threads):
//   warp 0      tile scheduler + TMA producer: takes the next tile from the
//               global counter, publishes it in a shared-memory tile ring,
//               then streams its K slices (2P tiles of 64 K each) into a
//               stage ring with 2-D tiled bulk copies (128-byte swizzle);
//   warp 1      allocates TMEM and issues the MMAs (one elected lane);
//               tcgen05.commit frees a stage once its MMAs have read it and
//               signals a TMEM chunk buffer as full;
//   warps 2-5   epilogue: tcgen05.ld each finished chunk (warp w reads TMEM
//               lanes 32*(w%4)..+31 = tile rows) into 128 FP32 registers per
//               thread, release the buffer, add the registers into C.
// Every mbarrier wait is bounded (2 s by %globaltimer); a wait that gives up
// records GBBLAS_STATUS_TIMEOUT in the stream's error word, the CTA drains
// its in-flight copies (bounded again), lets its MMAs finish, frees TMEM and
// returns.
//
// Replaces the FP32 path of the reference's mtm (include/mtm.hpp:116-206)
// when the caller asks for GBBLAS_ACCURACY_BF16X3 / BF16X6, and runs the
// batched form of it.  Roofline: tensor pipe; (number of products) *
// 2*M*N*K BF16 flops per problem, reported as 2*M*N*K algorithmic flops.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "tc_ptx.cuh"

namespace gbblas {
namespace {

using namespace tc;

constexpr int kBM = 128;
constexpr int kBN = 128;
constexpr int kBK = 64;  // 64 bf16 = one 128-byte swizzle row
constexpr int kThreads = 192;
constexpr int kChunkTiles = 8;   // K slices folded into registers per chunk (512 of K)
constexpr int kTileRing = 4;     // tiles in flight between scheduler and consumers
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s
constexpr size_t kSmemLimit = 232448;             // 227 KB per CTA

template <int P>
struct TcCfg {
  static constexpr uint32_t kABytes = kBM * kBK * 2;  // one bf16 piece tile of A
  static constexpr uint32_t kBBytes = kBN * kBK * 2;
  static constexpr uint32_t kStageBytes = P * (kABytes + kBBytes);
  static constexpr int kStagesFit = (int)((kSmemLimit - 1024 - 512) / kStageBytes);
  static constexpr int kStages = kStagesFit > 4 ? 4 : kStagesFit;
  static constexpr uint32_t kTmemCols = 4 * kBN;  // two chunk buffers x (main + correction)
  static constexpr size_t kSmem = 1024 /*alignment slack*/ + (size_t)kStages * kStageBytes + 512 /*barriers, ring*/;
  static_assert(kStages >= 2, "need at least a double-buffered stage ring");
  static_assert(kSmem <= kSmemLimit, "exceeds the 227 KB per-CTA shared memory limit");
  static_assert(kStageBytes % 1024 == 0 && kABytes % 1024 == 0 && kBBytes % 1024 == 0,
                "operand tiles must stay 1024-byte aligned for the 128-byte swizzle");
  static_assert(kTmemCols <= 512, "TMEM has 512 columns");
};

// One GEMM of a group, as the kernel sees it (device memory).
struct TcProblem {
  int M, N;
  int num_kt;      // K slices: padded K / 64
  int a_row;       // first row of this problem in the A arena (piece 0)
  int b_row;       // first row in the B^T arena (piece 0)
  int tiles_m, tiles_n;
  int tile_start;  // first global tile index of this problem
  float* C;
  int64_t rsc, csc;
};

// One operand matrix to split (device memory).
struct SplitJob {
  const float* src;
  int64_t rows, K, rs, cs;  // logical rows x K, element (r, k) at src[r*rs + k*cs]
  int64_t dst_row;          // first row in the arena
  int tiles_r, tiles_k;     // 32 x 32 tiles covering padded rows x padded K
  int tile_start;
};

// ---------------------------------------------------------------- split
// For every job, writes P pieces of rows_pad x k_pad into the arena (piece p
// at out + p * piece_stride, row pitch `pitch`), zero outside rows x K.
template <int P>
__global__ void __launch_bounds__(256) split_group_kernel(const SplitJob* __restrict__ jobs, int njobs,
                                                          __nv_bfloat16* __restrict__ out, int64_t piece_stride,
                                                          int64_t pitch) {
  __shared__ float tile[32][33];
  __shared__ int sjob;
  const int t = blockIdx.x;
  if (threadIdx.x == 0 && threadIdx.y == 0) {  // job = last with tile_start <= t
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
  const int64_t r0 = (int64_t)(local / j.tiles_k) * 32, k0 = (int64_t)(local % j.tiles_k) * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  if (j.cs == 1) {  // K contiguous: threads along k
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t r = r0 + ty + 8 * i, k = k0 + tx;
      tile[ty + 8 * i][tx] = (r < j.rows && k < j.K) ? __ldg(j.src + r * j.rs + k) : 0.f;
    }
  } else {  // rows contiguous (or general): threads along r
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t r = r0 + tx, k = k0 + ty + 8 * i;
      tile[tx][ty + 8 * i] = (r < j.rows && k < j.K) ? __ldg(j.src + r * j.rs + k * j.cs) : 0.f;
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t r = j.dst_row + r0 + ty + 8 * i, k = k0 + tx;
    float v = tile[ty + 8 * i][tx];
#pragma unroll
    for (int p = 0; p < P; ++p) {
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      out[p * piece_stride + r * pitch + k] = h;
      v = v - __bfloat162float(h);  // exact in FP32
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

// Output tile of global index t: grouped raster inside its problem
// (consecutive tiles walk 8 row-tiles of one column band for L2 reuse).
__device__ __forceinline__ void tile_coords(const TcProblem& p, int t, int& m0, int& n0) {
  constexpr int kGroup = 8;
  const int local = t - p.tile_start;
  const int group_span = kGroup * p.tiles_n;
  const int g = local / group_span;
  const int first_m = g * kGroup;
  const int gm = min(p.tiles_m - first_m, kGroup);
  const int in_g = local % group_span;
  m0 = (first_m + in_g % gm) * kBM;
  n0 = (in_g / gm) * kBN;
}

template <int P>
__global__ void __launch_bounds__(kThreads, 1)
    gemm_split_kernel(const __grid_constant__ CUtensorMap tm_a, const __grid_constant__ CUtensorMap tm_b,
                      const TcProblem* __restrict__ probs, int nprob, int total_tiles, int a_piece_rows,
                      int b_piece_rows, int* __restrict__ tile_counter, int* __restrict__ err) {
  using CF = TcCfg<P>;
  constexpr int ST = CF::kStages;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  // stage s: A pieces 0..P-1, then B pieces 0..P-1
  auto a_tile = [&](int s, int p) { return smem + (size_t)s * CF::kStageBytes + (size_t)p * CF::kABytes; };
  auto b_tile = [&](int s, int p) {
    return smem + (size_t)s * CF::kStageBytes + (size_t)P * CF::kABytes + (size_t)p * CF::kBBytes;
  };
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)ST * CF::kStageBytes);
  uint64_t* full = bars;                   // [ST]  TMA -> MMA
  uint64_t* empty = full + ST;             // [ST]  MMA -> TMA
  uint64_t* tfull = empty + ST;            // [2]   MMA -> epilogue: chunk in TMEM buffer b
  uint64_t* tempty = tfull + 2;            // [2]   epilogue -> MMA: TMEM buffer b drained
  uint64_t* ring_full = tempty + 2;        // [kTileRing] scheduler -> consumers
  uint64_t* ring_empty = ring_full + kTileRing;  // [kTileRing] consumers -> scheduler
  uint64_t* accf = ring_empty + kTileRing;  // [1] every MMA of this CTA finished
  int* ring = reinterpret_cast<int*>(accf + 1);  // [kTileRing] tile ids, -1 = no more work
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(ring + kTileRing);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 4);  // one arrival per epilogue warp
    }
    for (int r = 0; r < kTileRing; ++r) {
      mbar_init(&ring_full[r], 1);
      mbar_init(&ring_empty[r], 5);  // MMA lane + four epilogue warps
    }
    mbar_init(accf, 1);
    *abort_flag = 0;
    fence_mbar_init();
    prefetch_tensormap(&tm_a);
    prefetch_tensormap(&tm_b);
  }
  if (warp == 1) {
    tmem_alloc(tmem_slot, CF::kTmemCols);
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

  int issued = 0;  // producer: K slices whose copies were issued (all tiles)
  if (warp == 0) {
    if (lane == 0) {
      bool stop = false;
      for (int it = 0; !stop; ++it) {
        const int slot = it % kTileRing, use = it / kTileRing;
        int t = atomicAdd(tile_counter, 1);
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
        tile_coords(pr, t, m0, n0);
        for (int kt = 0; kt < pr.num_kt; ++kt) {
          const int s = issued % ST, round = issued / ST;
          if (round > 0 && !mbar_wait_bounded(&empty[s], (round - 1) & 1, abort_flag, kWaitLimitNs)) {
            fail();
            stop = true;
            break;
          }
          mbar_arrive_expect_tx(&full[s], CF::kStageBytes);
          // piece p of A occupies rows [p*a_piece_rows, (p+1)*a_piece_rows) of the arena map
#pragma unroll
          for (int p = 0; p < P; ++p)
            tma_load_2d(a_tile(s, p), &tm_a, &full[s], kt * kBK, p * a_piece_rows + pr.a_row + m0);
#pragma unroll
          for (int p = 0; p < P; ++p)
            tma_load_2d(b_tile(s, p), &tm_b, &full[s], kt * kBK, p * b_piece_rows + pr.b_row + n0);
          ++issued;
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16_f32(kBM, kBN);
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
          const bool chunk_first = (kt % kChunkTiles) == 0;
          const bool chunk_last = ((kt + 1) % kChunkTiles) == 0 || kt + 1 == num_kt;
          if (chunk_first) ++chunk_g;
          const int chunk = chunk_g - 1, b = chunk & 1;
          if (chunk_first && chunk >= 2) {  // buffer b must have been drained by the epilogue
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
          const uint32_t acc_main = tmem + (uint32_t)(b * 2 * kBN), acc_corr = acc_main + kBN;
          uint32_t a[P], bb[P];
#pragma unroll
          for (int p = 0; p < P; ++p) {
            a[p] = smem_u32(a_tile(s, p));
            bb[p] = smem_u32(b_tile(s, p));
          }
#pragma unroll
          for (int kk = 0; kk < kBK / 16; ++kk) {
            const uint32_t off = kk * 32;  // 16 bf16 along K inside the swizzled row
            const uint32_t acc = (chunk_first && kk == 0) ? 0u : 1u;
            mma_f16(acc_main, sw128_kmajor_desc(a[0] + off), sw128_kmajor_desc(bb[0] + off), idesc, acc);
            // corrections, largest first: p0p1, p1p0 (+ p0p2, p1p1, p2p0)
            mma_f16(acc_corr, sw128_kmajor_desc(a[0] + off), sw128_kmajor_desc(bb[1] + off), idesc, acc);
            mma_f16(acc_corr, sw128_kmajor_desc(a[1] + off), sw128_kmajor_desc(bb[0] + off), idesc, 1u);
            if constexpr (P == 3) {
              mma_f16(acc_corr, sw128_kmajor_desc(a[0] + off), sw128_kmajor_desc(bb[2] + off), idesc, 1u);
              mma_f16(acc_corr, sw128_kmajor_desc(a[1] + off), sw128_kmajor_desc(bb[1] + off), idesc, 1u);
              mma_f16(acc_corr, sw128_kmajor_desc(a[2] + off), sw128_kmajor_desc(bb[0] + off), idesc, 1u);
            }
          }
          mma_commit(&empty[s]);
          if (chunk_last) mma_commit(&tfull[b]);
          ++consumed;
        }
      }
      // accf completes once every MMA issued above has finished, on the
      // normal path and after an abort alike, so TMEM is never freed under a
      // running MMA.
      mma_commit(accf);
      if (*abort_flag) {
        int never = 0;
        (void)mbar_wait_bounded(accf, 0, &never, kWaitLimitNs);
      }
    }
  } else {
    // epilogue warps 2..5: TMEM lane quarter = warp % 4, one tile row per thread.
    const int q = warp & 3;
    const uint32_t trow = tmem + ((uint32_t)(q * 32) << 16);
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
      tile_coords(pr, t, m0, n0);
      const int nchunks = (pr.num_kt + kChunkTiles - 1) / kChunkTiles;
      float acc[kBN];
#pragma unroll
      for (int j = 0; j < kBN; ++j) acc[j] = 0.f;
      bool ok = true;
      for (int c = 0; c < nchunks; ++c, ++chunk_g) {
        const int b = chunk_g & 1;
        // tcgen05.ld is warp-collective: make the decision warp-uniform.
        const bool ready =
            __all_sync(0xffffffffu, mbar_wait_bounded(&tfull[b], (chunk_g >> 1) & 1, abort_flag, kWaitLimitNs));
        if (!ready) {
          if (lane == 0) fail();
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t tb = trow + (uint32_t)(b * 2 * kBN);
#pragma unroll
        for (int c0 = 0; c0 < kBN; c0 += 16) {
          float v0[16], v1[16];
          tmem_ld16(tb + c0, v0);
          tmem_ld16(tb + kBN + c0, v1);
          tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < 16; ++j) acc[c0 + j] += v0[j] + v1[j];
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&tempty[b]);
      }
      if (!ok) break;
      const int aborted = __shfl_sync(0xffffffffu, *abort_flag, 0);
      if (aborted) break;
      const int row = m0 + q * 32 + lane;
      if (row < pr.M) {
        float* crow = pr.C + (int64_t)row * pr.rsc;
        const bool vec =
            (pr.csc == 1) && ((pr.rsc & 3) == 0) && ((reinterpret_cast<uintptr_t>(pr.C) & 15) == 0);
        if (vec && n0 + kBN <= pr.N) {
#pragma unroll
          for (int j = 0; j < kBN; j += 4) {
            float4* p = reinterpret_cast<float4*>(crow + n0 + j);
            float4 cv = *p;
            cv.x += acc[j];
            cv.y += acc[j + 1];
            cv.z += acc[j + 2];
            cv.w += acc[j + 3];
            *p = cv;
          }
        } else {
#pragma unroll
          for (int j = 0; j < kBN; ++j)
            if (n0 + j < pr.N) crow[(int64_t)(n0 + j) * pr.csc] += acc[j];
        }
      }
    }
  }

  // ---- teardown: drain in-flight copies if the pipeline stopped early,
  // make sure every tcgen05 op finished, free TMEM.
  if (warp == 0 && lane == 0 && *abort_flag) {
    int never = 0;
    const int from = issued > ST ? issued - ST : 0;
    for (int k = from; k < issued; ++k) (void)mbar_wait_bounded(&full[k % ST], (k / ST) & 1, &never, kWaitLimitNs / 2);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tmem, CF::kTmemCols);
  }
}

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

// 2-D bf16 tensor map over a rows x cols (cols contiguous) buffer, box of
// box_rows x 64 with 128-byte swizzle.
gbblas_status make_map(CUtensorMap* map, const void* base, uint64_t rows, uint64_t cols, uint32_t box_rows) {
  auto fn = encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return GBBLAS_STATUS_CUDA_ERROR;
  }
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {cols * 2};
  cuuint32_t box[2] = {(cuuint32_t)kBK, box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d) for %llu x %llu", (int)r, (unsigned long long)rows,
              (unsigned long long)cols);
    return GBBLAS_STATUS_CUDA_ERROR;
  }
  return GBBLAS_STATUS_SUCCESS;
}

inline int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }
inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

// Everything one split-BF16 group launch needs: host tables, where they and
// the BF16 arena live on the device, and the two arena tensor maps.
struct TcGroupPlan {
  int pieces = 2;
  int nprob = 0;
  int64_t a_rows = 0, b_rows = 0, pitch = 0, tiles = 0;
  int a_tiles = 0, b_tiles = 0;
  std::vector<TcProblem> probs;
  std::vector<SplitJob> ajobs, bjobs;
  size_t off_probs = 0, off_jobs = 0, off_arena = 0, bytes = 0;
  char* base = nullptr;  // device: zeroed header | problems | jobs | arena
  bool owned = false;    // base allocated by the plan (graph plans)
  CUtensorMap map_a, map_b;
};

namespace {

// Host-side planning (no device work): problem order (largest K first),
// arena rows, tile numbering, split jobs, device layout.
gbblas_status plan_group(int pieces, const gbblas_gemm_desc* d, int64_t count, TcGroupPlan& pl) {
  pl.pieces = pieces;
  std::vector<int64_t> order;
  order.reserve(count);
  for (int64_t i = 0; i < count; ++i) {
    const gbblas_gemm_desc& g = d[i];
    if (g.M > (1 << 29) || g.N > (1 << 29) || g.K > (1 << 30)) {
      set_error("split-bf16 gemm: problem %lld too large for the tile grid", (long long)i);
      return GBBLAS_STATUS_NOT_SUPPORTED;
    }
    if (g.M > 0 && g.N > 0 && g.K > 0) order.push_back(i);
  }
  std::stable_sort(order.begin(), order.end(), [&](int64_t x, int64_t y) { return d[x].K > d[y].K; });
  pl.nprob = (int)order.size();
  pl.probs.resize(pl.nprob);
  pl.ajobs.resize(pl.nprob);
  pl.bjobs.resize(pl.nprob);
  for (int i = 0; i < pl.nprob; ++i) pl.pitch = std::max<int64_t>(pl.pitch, round_up(d[order[i]].K, kBK));
  for (int i = 0; i < pl.nprob; ++i) {
    const gbblas_gemm_desc& g = d[order[i]];
    const int64_t Mp = round_up(g.M, kBM), Np = round_up(g.N, kBN), Kp = round_up(g.K, kBK);
    TcProblem& p = pl.probs[i];
    p.M = (int)g.M;
    p.N = (int)g.N;
    p.num_kt = (int)(Kp / kBK);
    p.a_row = (int)pl.a_rows;
    p.b_row = (int)pl.b_rows;
    p.tiles_m = (int)(Mp / kBM);
    p.tiles_n = (int)(Np / kBN);
    p.tile_start = (int)pl.tiles;
    p.C = g.C;
    p.rsc = g.rsc;
    p.csc = g.csc;
    pl.ajobs[i] = {g.A, g.M, g.K, g.rsa, g.csa, pl.a_rows, (int)(Mp / 32), (int)(Kp / 32), pl.a_tiles};
    pl.a_tiles += pl.ajobs[i].tiles_r * pl.ajobs[i].tiles_k;
    // B^T: element (n, k) = B[k*rsb + n*csb]
    pl.bjobs[i] = {g.B, g.N, g.K, g.csb, g.rsb, pl.b_rows, (int)(Np / 32), (int)(Kp / 32), pl.b_tiles};
    pl.b_tiles += pl.bjobs[i].tiles_r * pl.bjobs[i].tiles_k;
    pl.a_rows += Mp;
    pl.b_rows += Np;
    pl.tiles += (int64_t)p.tiles_m * p.tiles_n;
  }
  if ((double)(pl.a_rows + pl.b_rows) * pieces >= 2.0e9 || pl.tiles >= (1ll << 31) ||
      (double)pl.a_tiles >= 2.0e9 || (double)pl.b_tiles >= 2.0e9) {
    set_error("split-bf16 gemm: group too large for one launch");
    return GBBLAS_STATUS_NOT_SUPPORTED;
  }
  pl.off_probs = kScratchZeroBytes;
  pl.off_jobs = pl.off_probs + align256(sizeof(TcProblem) * pl.nprob);
  pl.off_arena = pl.off_jobs + align256(sizeof(SplitJob) * 2 * pl.nprob);
  const size_t a_piece = (size_t)(pl.a_rows * pl.pitch), b_piece = (size_t)(pl.b_rows * pl.pitch);
  pl.bytes = pl.off_arena + (size_t)pieces * (a_piece + b_piece) * sizeof(__nv_bfloat16);
  return GBBLAS_STATUS_SUCCESS;
}

__nv_bfloat16* arena_a(const TcGroupPlan& pl) { return reinterpret_cast<__nv_bfloat16*>(pl.base + pl.off_arena); }
__nv_bfloat16* arena_b(const TcGroupPlan& pl) {
  return arena_a(pl) + (size_t)pl.pieces * (size_t)(pl.a_rows * pl.pitch);
}

// Point the plan at device memory `base` (>= pl.bytes, header zeroed), copy
// the tables there on `stream`, and encode the arena tensor maps.
gbblas_status bind_group(TcGroupPlan& pl, char* base, cudaStream_t stream) {
  pl.base = base;
  if (pl.nprob == 0) return GBBLAS_STATUS_SUCCESS;
  GB_CUDA_TRY(cudaMemcpyAsync(base + pl.off_probs, pl.probs.data(), sizeof(TcProblem) * pl.nprob,
                              cudaMemcpyHostToDevice, stream));
  GB_CUDA_TRY(cudaMemcpyAsync(base + pl.off_jobs, pl.ajobs.data(), sizeof(SplitJob) * pl.nprob,
                              cudaMemcpyHostToDevice, stream));
  GB_CUDA_TRY(cudaMemcpyAsync(base + pl.off_jobs + sizeof(SplitJob) * pl.nprob, pl.bjobs.data(),
                              sizeof(SplitJob) * pl.nprob, cudaMemcpyHostToDevice, stream));
  GB_TRY(make_map(&pl.map_a, arena_a(pl), (uint64_t)(pl.pieces * pl.a_rows), (uint64_t)pl.pitch, kBM));
  GB_TRY(make_map(&pl.map_b, arena_b(pl), (uint64_t)(pl.pieces * pl.b_rows), (uint64_t)pl.pitch, kBN));
  return GBBLAS_STATUS_SUCCESS;
}

template <int P>
gbblas_status launch_bound(DeviceCtx* c, const TcGroupPlan& pl, cudaStream_t stream, int max_ctas) {
  using CF = TcCfg<P>;
  if (pl.nprob == 0) return GBBLAS_STATUS_SUCCESS;
  int* err = reinterpret_cast<int*>(pl.base + kErrWordOffset);
  int* counter = reinterpret_cast<int*>(pl.base + kTileCounterOffset);
  const auto* dprobs = reinterpret_cast<const TcProblem*>(pl.base + pl.off_probs);
  const auto* djobs = reinterpret_cast<const SplitJob*>(pl.base + pl.off_jobs);
  GB_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(int), stream));
  split_group_kernel<P><<<pl.a_tiles, dim3(32, 8), 0, stream>>>(djobs, pl.nprob, arena_a(pl),
                                                                (int64_t)(pl.a_rows * pl.pitch), pl.pitch);
  GB_TRY(check_launch("split_group_kernel(A)"));
  split_group_kernel<P><<<pl.b_tiles, dim3(32, 8), 0, stream>>>(djobs + pl.nprob, pl.nprob, arena_b(pl),
                                                                (int64_t)(pl.b_rows * pl.pitch), pl.pitch);
  GB_TRY(check_launch("split_group_kernel(B)"));
  static bool attr_set[64] = {false};
  if (!attr_set[c->device & 63]) {
    GB_CUDA_TRY(cudaFuncSetAttribute(gemm_split_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)CF::kSmem));
    attr_set[c->device & 63] = true;
  }
  int grid = (int)std::min<int64_t>(pl.tiles, c->num_sms);
  if (max_ctas > 0 && grid > max_ctas) grid = max_ctas;
  gemm_split_kernel<P><<<grid, kThreads, CF::kSmem, stream>>>(pl.map_a, pl.map_b, dprobs, pl.nprob, (int)pl.tiles,
                                                             (int)pl.a_rows, (int)pl.b_rows, counter, err);
  return check_launch("gemm_split_kernel");
}

}  // namespace

void tc_prepare(DeviceCtx* c) {
  (void)c;
  cudaFuncSetAttribute(gemm_split_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TcCfg<2>::kSmem);
  cudaFuncSetAttribute(gemm_split_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TcCfg<3>::kSmem);
}

gbblas_status tc_group_launch(DeviceCtx* c, const TcGroupPlan* pl, cudaStream_t stream, int max_ctas) {
  return pl->pieces == 3 ? launch_bound<3>(c, *pl, stream, max_ctas) : launch_bound<2>(c, *pl, stream, max_ctas);
}

gbblas_status tc_group_create(DeviceCtx* c, int pieces, const gbblas_gemm_desc* descs, int64_t count,
                              TcGroupPlan** out) {
  (void)c;
  TcGroupPlan* pl = new TcGroupPlan();
  gbblas_status st = plan_group(pieces, descs, count, *pl);
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

gbblas_status launch_gemm_split_bf16_group(DeviceCtx* c, int pieces, const gbblas_gemm_desc* descs, int64_t count,
                                           cudaStream_t stream, int max_ctas) {
  TcGroupPlan pl;
  GB_TRY(plan_group(pieces, descs, count, pl));
  if (pl.nprob == 0) return GBBLAS_STATUS_SUCCESS;
  void* s = nullptr;
  GB_TRY(get_scratch(c, stream, pl.bytes, &s));
  GB_TRY(bind_group(pl, static_cast<char*>(s), stream));
  return tc_group_launch(c, &pl, stream, max_ctas);
}

gbblas_status launch_gemm_split_bf16(DeviceCtx* c, int pieces, int64_t M, int64_t N, int64_t K, const float* A,
                                     int64_t rsa, int64_t csa, const float* B, int64_t rsb, int64_t csb, float* C,
                                     int64_t rsc, int64_t csc, cudaStream_t stream) {
  if (M == 0 || N == 0 || K == 0) return GBBLAS_STATUS_SUCCESS;
  gbblas_gemm_desc d{M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc};
  return launch_gemm_split_bf16_group(c, pieces, &d, 1, stream);
}

}  // namespace gbblas
