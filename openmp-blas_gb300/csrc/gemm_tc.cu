// gemm_tc.cu - FP32-accurate GEMM on the 5th-generation tensor cores
// (split-BF16).  C += A * B for float A, B, C of any layout.
//
//   1. split_bf16_kernel: every FP32 operand element a becomes P BF16 pieces
//      p0 = bf16_rn(a), p1 = bf16_rn(a - p0), p2 = bf16_rn(a - p0 - p1),
//      written K-major (A as M x K, B as its transpose N x K) and zero-padded
//      to the tile grid.
//   2. gemm_split_kernel: C += sum of the piece products p_i(A) p_j(B) with
//      i + j < P, by tcgen05.mma (kind::f16, BF16 in, FP32 accumulate), into
//      two TMEM accumulators - p0*p0 alone, and every smaller product together
//      (so the small terms are summed at their own scale).  K is walked in
//      chunks of 512: each chunk accumulates in one of two TMEM buffers while
//      the epilogue warps fold the previous chunk into FP32 registers with
//      round-to-nearest adds (the tensor core's own accumulation over long K
//      is measurably less accurate than FP32), and the registers are added
//      into C once at the end.
//        P = 2 ("bf16x3"):  p0p0 + (p0p1 + p1p0)                     3 MMAs
//        P = 3 ("bf16x6"):  p0p0 + (p0p1 + p1p0 + p0p2 + p1p1 + p2p0) 6 MMAs
//      Three pieces hold all 24 significand bits of an FP32 value, and the
//      dropped products are below 2^-24 of |a||b|, so bf16x6 is as accurate as
//      FP32 FMA arithmetic; bf16x3 keeps about 16 bits.
//
// Kernel organisation (one 128 x BN output tile per CTA, 192 threads):
//   warp 0      TMA producer: 2-D tiled bulk copies (128-byte swizzle) of the
//               2P operand tiles of a 64-wide K slice into a stage ring;
//   warp 1      allocates TMEM and issues the MMAs (one elected lane);
//               tcgen05.commit frees a stage once its MMAs have read it;
//   warps 2-5   epilogue: tcgen05.ld the accumulators of each finished chunk
//               (warp w reads TMEM lanes 32*(w%4)..+31 = tile rows), fold
//               them into 128 FP32 registers per thread, release the TMEM
//               buffer, and finally add the registers into C.
// Every mbarrier wait is bounded (2 s by %globaltimer); a wait that gives up
// records GBBLAS_STATUS_TIMEOUT in the stream's error word, the CTA drains
// its in-flight copies (bounded again), lets its MMAs finish, frees TMEM and
// returns.
//
// Replaces the FP32 path of the reference's mtm (include/mtm.hpp:116-206)
// when the caller asks for GBBLAS_ACCURACY_BF16X3 / BF16X6.  Roofline:
// tensor pipe; (number of products) * 2*M*N*K BF16 flops per call, reported
// as 2*M*N*K algorithmic flops.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "common.cuh"
#include "tc_ptx.cuh"

namespace gbblas {
namespace {

using namespace tc;

constexpr int kBM = 128;
constexpr int kBK = 64;  // 64 bf16 = one 128-byte swizzle row
constexpr int kThreads = 192;
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s
constexpr size_t kSmemLimit = 232448;             // 227 KB per CTA

// K slices (of kBK) accumulated in TMEM before the epilogue warps fold the
// partial sums into FP32 registers.  The tensor core's accumulation into TMEM
// loses more than FP32 round-to-nearest over long K; folding every 512 keeps
// the result as accurate as FP32 FMA arithmetic at any K.
constexpr int kChunkTiles = 8;

template <int BN, int P>
struct TcCfg {
  static constexpr uint32_t kABytes = kBM * kBK * 2;  // one bf16 piece tile of A
  static constexpr uint32_t kBBytes = BN * kBK * 2;
  static constexpr uint32_t kStageBytes = P * (kABytes + kBBytes);
  static constexpr int kStagesFit = (int)((kSmemLimit - 1024 - 256) / kStageBytes);
  static constexpr int kStages = kStagesFit > 4 ? 4 : kStagesFit;
  // two chunk buffers x (main + correction) accumulators
  static constexpr uint32_t kTmemCols = 4 * BN;
  static constexpr size_t kSmem = 1024 /*alignment slack*/ + (size_t)kStages * kStageBytes + 256 /*barriers*/;
  static constexpr int kProducts = P == 2 ? 3 : 6;
  static_assert(kStages >= 2, "need at least a double-buffered stage ring");
  static_assert(kSmem <= kSmemLimit, "exceeds the 227 KB per-CTA shared memory limit");
  static_assert(kStageBytes % 1024 == 0 && kABytes % 1024 == 0 && kBBytes % 1024 == 0,
                "operand tiles must stay 1024-byte aligned for the 128-byte swizzle");
  static_assert(kTmemCols <= 512, "TMEM has 512 columns");
};

// ---------------------------------------------------------------- split
// Logical matrix X (rows x K), element (r, k) at in[r*rs + k*cs].  Writes P
// pieces, piece i at out + i*piece_stride, each rows_pad x k_pad row-major
// bf16, zero outside rows x K.  Grid covers rows_pad x k_pad in 32 x 32 tiles.
template <int P>
__global__ void __launch_bounds__(256) split_bf16_kernel(const float* __restrict__ in, int64_t rows, int64_t K,
                                                         int64_t rs, int64_t cs, __nv_bfloat16* __restrict__ out,
                                                         int64_t piece_stride, int64_t k_pad) {
  __shared__ float tile[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 32;
  if (cs == 1) {  // K contiguous: threads along k
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t r = r0 + ty + 8 * i, k = k0 + tx;
      tile[ty + 8 * i][tx] = (r < rows && k < K) ? __ldg(in + r * rs + k) : 0.f;
    }
  } else {  // rows contiguous (or general): threads along r
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t r = r0 + tx, k = k0 + ty + 8 * i;
      tile[tx][ty + 8 * i] = (r < rows && k < K) ? __ldg(in + r * rs + k * cs) : 0.f;
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t r = r0 + ty + 8 * i, k = k0 + tx;
    float v = tile[ty + 8 * i][tx];
#pragma unroll
    for (int p = 0; p < P; ++p) {
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      out[p * piece_stride + r * k_pad + k] = h;
      v = v - __bfloat162float(h);  // exact in FP32
    }
  }
}

// ---------------------------------------------------------------- GEMM
template <int BN, int P>
__global__ void __launch_bounds__(kThreads, 1)
    gemm_split_kernel(const __grid_constant__ CUtensorMap tm_a, const __grid_constant__ CUtensorMap tm_b, int M,
                      int N, int num_kt, int tiles_m, int tiles_n, int a_piece_rows, int b_piece_rows,
                      float* __restrict__ C, int64_t rsc, int64_t csc, int* __restrict__ err) {
  using CF = TcCfg<BN, P>;
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
  uint64_t* full = bars;              // [ST]  TMA -> MMA
  uint64_t* empty = bars + ST;        // [ST]  MMA -> TMA
  uint64_t* tfull = bars + 2 * ST;    // [2]   MMA -> epilogue: chunk accumulated in TMEM buffer b
  uint64_t* tempty = tfull + 2;       // [2]   epilogue -> MMA: TMEM buffer b drained
  uint64_t* accf = tempty + 2;        // [1]   every MMA of this CTA finished
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accf + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nchunks = (num_kt + kChunkTiles - 1) / kChunkTiles;

  // Grouped raster: consecutive CTAs walk 8 row-tiles of one column band so
  // a wave shares A and B panels in L2.
  const int bid = blockIdx.x;
  constexpr int kGroup = 8;
  const int group_span = kGroup * tiles_n;
  const int g = bid / group_span;
  const int first_m = g * kGroup;
  const int gm = min(tiles_m - first_m, kGroup);
  const int in_g = bid % group_span;
  const int tile_m = first_m + in_g % gm;
  const int tile_n = in_g / gm;
  const int m0 = tile_m * kBM, n0 = tile_n * BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 4);  // one arrival per epilogue warp
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

  int issued = 0;  // producer: K slices whose copies were issued
  if (warp == 0) {
    if (lane == 0) {
      for (int kt = 0; kt < num_kt; ++kt) {
        const int s = kt % ST, round = kt / ST;
        if (round > 0 && !mbar_wait_bounded(&empty[s], (round - 1) & 1, abort_flag, kWaitLimitNs)) {
          fail();
          break;
        }
        mbar_arrive_expect_tx(&full[s], CF::kStageBytes);
        // piece p of A occupies rows [p*a_piece_rows, (p+1)*a_piece_rows) of one tensor map
#pragma unroll
        for (int p = 0; p < P; ++p) tma_load_2d(a_tile(s, p), &tm_a, &full[s], kt * kBK, p * a_piece_rows + m0);
#pragma unroll
        for (int p = 0; p < P; ++p) tma_load_2d(b_tile(s, p), &tm_b, &full[s], kt * kBK, p * b_piece_rows + n0);
        issued = kt + 1;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16_f32(kBM, BN);
      for (int kt = 0; kt < num_kt; ++kt) {
        const int s = kt % ST, round = kt / ST;
        const int chunk = kt / kChunkTiles, b = chunk & 1;
        const bool chunk_first = (kt % kChunkTiles) == 0;
        const bool chunk_last = ((kt + 1) % kChunkTiles) == 0 || kt + 1 == num_kt;
        if (chunk_first && chunk >= 2) {  // buffer b must have been drained by the epilogue
          if (!mbar_wait_bounded(&tempty[b], ((chunk >> 1) - 1) & 1, abort_flag, kWaitLimitNs)) {
            fail();
            break;
          }
          tc_fence_after();
        }
        if (!mbar_wait_bounded(&full[s], round & 1, abort_flag, kWaitLimitNs)) {
          fail();
          break;
        }
        tc_fence_after();
        const uint32_t acc_main = tmem + (uint32_t)(b * 2 * BN), acc_corr = acc_main + BN;
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
    // Each chunk's TMEM partial sums (main + correction) are folded into FP32
    // registers with round-to-nearest adds, then the buffer is handed back.
    const int q = warp & 3;
    const uint32_t trow = tmem + ((uint32_t)(q * 32) << 16);
    float acc[BN];
#pragma unroll
    for (int j = 0; j < BN; ++j) acc[j] = 0.f;
    bool ok = true;
    for (int chunk = 0; chunk < nchunks; ++chunk) {
      const int b = chunk & 1;
      // tcgen05.ld is warp-collective: make the decision warp-uniform.
      const bool ready =
          __all_sync(0xffffffffu, mbar_wait_bounded(&tfull[b], (chunk >> 1) & 1, abort_flag, kWaitLimitNs));
      if (!ready) {
        if (lane == 0) fail();
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t tb = trow + (uint32_t)(b * 2 * BN);
#pragma unroll
      for (int c0 = 0; c0 < BN; c0 += 16) {
        float v0[16], v1[16];
        tmem_ld16(tb + c0, v0);
        tmem_ld16(tb + BN + c0, v1);
        tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 16; ++j) acc[c0 + j] += v0[j] + v1[j];
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[b]);
    }
    const int aborted = __shfl_sync(0xffffffffu, *abort_flag, 0);
    const int row = m0 + q * 32 + lane;
    if (ok && !aborted && row < M) {
      float* crow = C + (int64_t)row * rsc;
      const bool vec = (csc == 1) && ((rsc & 3) == 0) && ((reinterpret_cast<uintptr_t>(C) & 15) == 0);
      if (vec && n0 + BN <= N) {
#pragma unroll
        for (int j = 0; j < BN; j += 4) {
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
        for (int j = 0; j < BN; ++j)
          if (n0 + j < N) crow[(int64_t)(n0 + j) * csc] += acc[j];
      }
    }
  }

  // ---- teardown: drain in-flight copies if the pipeline stopped early,
  // make sure every tcgen05 op finished, free TMEM.
  if (warp == 0 && lane == 0 && *abort_flag) {
    int never = 0;
    const int from = issued > ST ? issued - ST : 0;
    for (int kt = from; kt < issued; ++kt)
      (void)mbar_wait_bounded(&full[kt % ST], (kt / ST) & 1, &never, kWaitLimitNs / 2);
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

template <int BN, int P>
gbblas_status run_split(DeviceCtx* c, int64_t M, int64_t N, int64_t K, const float* A, int64_t rsa, int64_t csa,
                        const float* B, int64_t rsb, int64_t csb, float* C, int64_t rsc, int64_t csc,
                        cudaStream_t stream) {
  using CF = TcCfg<BN, P>;
  const int64_t Mp = round_up(M, kBM), Np = round_up(N, BN), Kp = round_up(K, kBK);
  const size_t a_elems = (size_t)(Mp * Kp), b_elems = (size_t)(Np * Kp);
  const size_t bytes = kScratchZeroBytes + (size_t)P * (a_elems + b_elems) * sizeof(__nv_bfloat16);
  void* s = nullptr;
  GB_TRY(get_scratch(c, stream, bytes, &s));
  int* err = reinterpret_cast<int*>(static_cast<char*>(s) + kErrWordOffset);
  auto* apieces = reinterpret_cast<__nv_bfloat16*>(static_cast<char*>(s) + kScratchZeroBytes);
  auto* bpieces = apieces + (size_t)P * a_elems;

  dim3 sb(32, 8);
  split_bf16_kernel<P><<<dim3((unsigned)(Kp / 32), (unsigned)(Mp / 32)), sb, 0, stream>>>(A, M, K, rsa, csa, apieces,
                                                                                          (int64_t)a_elems, Kp);
  GB_TRY(check_launch("split_bf16_kernel(A)"));
  // B^T: element (n, k) = B[k*rsb + n*csb]
  split_bf16_kernel<P><<<dim3((unsigned)(Kp / 32), (unsigned)(Np / 32)), sb, 0, stream>>>(B, N, K, csb, rsb, bpieces,
                                                                                          (int64_t)b_elems, Kp);
  GB_TRY(check_launch("split_bf16_kernel(B)"));

  // One map per operand over all P pieces stacked along rows.
  CUtensorMap m_a, m_b;
  GB_TRY(make_map(&m_a, apieces, (uint64_t)(P * Mp), (uint64_t)Kp, kBM));
  GB_TRY(make_map(&m_b, bpieces, (uint64_t)(P * Np), (uint64_t)Kp, BN));

  static bool attr_set[64] = {false};
  if (!attr_set[c->device & 63]) {
    GB_CUDA_TRY(cudaFuncSetAttribute(gemm_split_kernel<BN, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)CF::kSmem));
    attr_set[c->device & 63] = true;
  }
  const int tiles_m = (int)(Mp / kBM), tiles_n = (int)(Np / BN);
  gemm_split_kernel<BN, P><<<tiles_m * tiles_n, kThreads, CF::kSmem, stream>>>(
      m_a, m_b, (int)M, (int)N, (int)(Kp / kBK), tiles_m, tiles_n, (int)Mp, (int)Np, C, rsc, csc, err);
  return check_launch("gemm_split_kernel");
}

}  // namespace

gbblas_status launch_gemm_split_bf16(DeviceCtx* c, int pieces, int64_t M, int64_t N, int64_t K, const float* A,
                                     int64_t rsa, int64_t csa, const float* B, int64_t rsb, int64_t csb, float* C,
                                     int64_t rsc, int64_t csc, cudaStream_t stream) {
  if (M == 0 || N == 0 || K == 0) return GBBLAS_STATUS_SUCCESS;
  if (M > (1 << 29) || N > (1 << 29) || K > (1 << 30)) {
    set_error("split-bf16 gemm: dimension too large for the tile grid");
    return GBBLAS_STATUS_NOT_SUPPORTED;
  }
  if (pieces == 3) return run_split<128, 3>(c, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, stream);
  return run_split<128, 2>(c, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, stream);
}

}  // namespace gbblas
