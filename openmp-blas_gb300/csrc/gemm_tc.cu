// gemm_tc.cu - FP32-accurate GEMM on the 5th-generation tensor cores
// (split-BF16, "bf16x3").  C += A * B for float A, B, C of any layout.
//
//   1. split_bf16_kernel: every FP32 operand element a becomes
//      hi = bf16_rn(a), lo = bf16_rn(a - hi), written K-major (A as M x K,
//      B as its transpose N x K) and zero-padded to the tile grid.
//   2. gemm_bf16x3_kernel: C += hi*hi + (hi*lo + lo*hi) with tcgen05.mma
//      (kind::f16, BF16 in, FP32 accumulate) into two TMEM accumulators - the
//      main product and the correction products are kept apart so the small
//      terms are summed at their own scale - and one FP32 add per element in
//      the epilogue.
//
// Kernel organisation (one 128 x BN output tile per CTA, 192 threads):
//   warp 0      TMA producer: 2-D tiled bulk copies (128-byte swizzle) of the
//               four operand tiles of a 64-wide K slice into a stage ring;
//   warp 1      allocates TMEM and issues the MMAs (one elected lane);
//               tcgen05.commit frees a stage once its MMAs have read it;
//   warps 2-5   epilogue: tcgen05.ld the accumulators (warp w reads TMEM
//               lanes 32*(w%4)..+31 = tile rows), add into C.
// Every mbarrier wait is bounded (2 s by %globaltimer); a wait that gives up
// records GBBLAS_STATUS_TIMEOUT in the stream's error word, the CTA drains
// its in-flight copies (bounded again), frees TMEM and returns.
//
// Replaces the FP32 path of the reference's mtm (include/mtm.hpp:116-206)
// when the caller asks for GBBLAS_ACCURACY_BF16X3.  Roofline: tensor pipe,
// 3 * 2*M*N*K BF16 flops per call (6 * M*N*K), reported as 2*M*N*K
// algorithmic flops.
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

template <int BN>
struct TcCfg {
  static constexpr int kStages = BN == 256 ? 2 : 3;
  static constexpr uint32_t kABytes = kBM * kBK * 2;  // one bf16 tile of A
  static constexpr uint32_t kBBytes = BN * kBK * 2;
  static constexpr uint32_t kStageBytes = 2 * kABytes + 2 * kBBytes;
  static constexpr uint32_t kTmemCols = 2 * BN;  // main + correction accumulators
  static constexpr size_t kSmem = 1024 /*alignment slack*/ + (size_t)kStages * kStageBytes + 256 /*barriers*/;
  static_assert(kSmem <= 232448, "exceeds the 227 KB per-CTA shared memory limit");
  static_assert(kStageBytes % 1024 == 0 && kABytes % 1024 == 0 && kBBytes % 1024 == 0,
                "operand tiles must stay 1024-byte aligned for the 128-byte swizzle");
};

// ---------------------------------------------------------------- split
// Logical matrix X (rows x K), element (r, k) at in[r*rs + k*cs].
// Writes hi/lo as rows_pad x k_pad row-major bf16, zero outside rows x K.
__global__ void __launch_bounds__(256) split_bf16_kernel(const float* __restrict__ in, int64_t rows, int64_t K,
                                                         int64_t rs, int64_t cs, __nv_bfloat16* __restrict__ hi,
                                                         __nv_bfloat16* __restrict__ lo, int64_t k_pad) {
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
    const float v = tile[ty + 8 * i][tx];
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
    hi[r * k_pad + k] = h;
    lo[r * k_pad + k] = l;
  }
}

// ---------------------------------------------------------------- GEMM
template <int BN>
__global__ void __launch_bounds__(kThreads, 1)
    gemm_bf16x3_kernel(const __grid_constant__ CUtensorMap tm_ahi, const __grid_constant__ CUtensorMap tm_alo,
                       const __grid_constant__ CUtensorMap tm_bhi, const __grid_constant__ CUtensorMap tm_blo,
                       int M, int N, int num_kt, int tiles_m, int tiles_n, float* __restrict__ C, int64_t rsc,
                       int64_t csc, int* __restrict__ err) {
  using CF = TcCfg<BN>;
  constexpr int ST = CF::kStages;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  auto stage_base = [&](int s) { return smem + (size_t)s * CF::kStageBytes; };
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)ST * CF::kStageBytes);
  uint64_t* full = bars;           // [ST]
  uint64_t* empty = bars + ST;     // [ST]
  uint64_t* accf = bars + 2 * ST;  // [1]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * ST + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

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
    mbar_init(accf, 1);
    *abort_flag = 0;
    fence_mbar_init();
    prefetch_tensormap(&tm_ahi);
    prefetch_tensormap(&tm_alo);
    prefetch_tensormap(&tm_bhi);
    prefetch_tensormap(&tm_blo);
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
        unsigned char* base = stage_base(s);
        mbar_arrive_expect_tx(&full[s], CF::kStageBytes);
        tma_load_2d(base, &tm_ahi, &full[s], kt * kBK, m0);
        tma_load_2d(base + CF::kABytes, &tm_alo, &full[s], kt * kBK, m0);
        tma_load_2d(base + 2 * CF::kABytes, &tm_bhi, &full[s], kt * kBK, n0);
        tma_load_2d(base + 2 * CF::kABytes + CF::kBBytes, &tm_blo, &full[s], kt * kBK, n0);
        issued = kt + 1;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16_f32(kBM, BN);
      const uint32_t acc_main = tmem, acc_corr = tmem + BN;
      for (int kt = 0; kt < num_kt; ++kt) {
        const int s = kt % ST, round = kt / ST;
        if (!mbar_wait_bounded(&full[s], round & 1, abort_flag, kWaitLimitNs)) {
          fail();
          break;
        }
        tc_fence_after();
        const uint32_t a_hi = smem_u32(stage_base(s));
        const uint32_t a_lo = a_hi + CF::kABytes;
        const uint32_t b_hi = a_hi + 2 * CF::kABytes;
        const uint32_t b_lo = b_hi + CF::kBBytes;
#pragma unroll
        for (int kk = 0; kk < kBK / 16; ++kk) {
          const uint32_t off = kk * 32;  // 16 bf16 along K inside the swizzled row
          const uint32_t first = (kt == 0 && kk == 0) ? 0u : 1u;
          mma_f16(acc_main, sw128_kmajor_desc(a_hi + off), sw128_kmajor_desc(b_hi + off), idesc, first);
          mma_f16(acc_corr, sw128_kmajor_desc(a_hi + off), sw128_kmajor_desc(b_lo + off), idesc, first);
          mma_f16(acc_corr, sw128_kmajor_desc(a_lo + off), sw128_kmajor_desc(b_hi + off), idesc, 1u);
        }
        mma_commit(&empty[s]);
      }
      // Always signal: accf completes once every MMA issued above has
      // finished, on the normal path and after an abort alike, so TMEM is
      // never freed under a running MMA.
      mma_commit(accf);
      if (*abort_flag) {
        int never = 0;
        (void)mbar_wait_bounded(accf, 0, &never, kWaitLimitNs);
      }
    }
  } else {
    // epilogue warps 2..5: TMEM lane quarter = warp % 4
    const int q = warp & 3;
    int never = 0;
    // tcgen05.ld is warp-collective: make the decision warp-uniform.
    const bool ready = __all_sync(0xffffffffu, mbar_wait_bounded(accf, 0, &never, kWaitLimitNs));
    const int aborted = __shfl_sync(0xffffffffu, *abort_flag, 0);
    if (!ready) {
      if (lane == 0) fail();
    } else if (!aborted) {
      tc_fence_after();
      const int row = m0 + q * 32 + lane;
      const uint32_t trow = tmem + ((uint32_t)(q * 32) << 16);
      const bool vec = (csc == 1) && ((rsc & 3) == 0) && ((reinterpret_cast<uintptr_t>(C) & 15) == 0);
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 16) {
        float v0[16], v1[16];
        tmem_ld16(trow + c0, v0);
        tmem_ld16(trow + BN + c0, v1);
        tmem_ld_wait();
        if (row < M) {
          const int col0 = n0 + c0;
          float* crow = C + (int64_t)row * rsc;
          if (vec && col0 + 16 <= N) {
            float4* p = reinterpret_cast<float4*>(crow + col0);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              float4 cv = p[j];
              cv.x += v0[4 * j + 0] + v1[4 * j + 0];
              cv.y += v0[4 * j + 1] + v1[4 * j + 1];
              cv.z += v0[4 * j + 2] + v1[4 * j + 2];
              cv.w += v0[4 * j + 3] + v1[4 * j + 3];
              p[j] = cv;
            }
          } else {
#pragma unroll
            for (int j = 0; j < 16; ++j)
              if (col0 + j < N) crow[(int64_t)(col0 + j) * csc] += v0[j] + v1[j];
          }
        }
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

template <int BN>
gbblas_status run_bf16x3(DeviceCtx* c, int64_t M, int64_t N, int64_t K, const float* A, int64_t rsa, int64_t csa,
                         const float* B, int64_t rsb, int64_t csb, float* C, int64_t rsc, int64_t csc,
                         cudaStream_t stream) {
  using CF = TcCfg<BN>;
  const int64_t Mp = round_up(M, kBM), Np = round_up(N, BN), Kp = round_up(K, kBK);
  const size_t a_elems = (size_t)(Mp * Kp), b_elems = (size_t)(Np * Kp);
  const size_t bytes = kScratchZeroBytes + 2 * (a_elems + b_elems) * sizeof(__nv_bfloat16);
  void* s = nullptr;
  GB_TRY(get_scratch(c, stream, bytes, &s));
  int* err = reinterpret_cast<int*>(static_cast<char*>(s) + kErrWordOffset);
  auto* ahi = reinterpret_cast<__nv_bfloat16*>(static_cast<char*>(s) + kScratchZeroBytes);
  auto* alo = ahi + a_elems;
  auto* bhi = alo + a_elems;
  auto* blo = bhi + b_elems;

  dim3 sb(32, 8);
  split_bf16_kernel<<<dim3((unsigned)(Kp / 32), (unsigned)(Mp / 32)), sb, 0, stream>>>(A, M, K, rsa, csa, ahi, alo,
                                                                                       Kp);
  GB_TRY(check_launch("split_bf16_kernel(A)"));
  // B^T: element (n, k) = B[k*rsb + n*csb]
  split_bf16_kernel<<<dim3((unsigned)(Kp / 32), (unsigned)(Np / 32)), sb, 0, stream>>>(B, N, K, csb, rsb, bhi, blo,
                                                                                       Kp);
  GB_TRY(check_launch("split_bf16_kernel(B)"));

  CUtensorMap m_ahi, m_alo, m_bhi, m_blo;
  GB_TRY(make_map(&m_ahi, ahi, Mp, Kp, kBM));
  GB_TRY(make_map(&m_alo, alo, Mp, Kp, kBM));
  GB_TRY(make_map(&m_bhi, bhi, Np, Kp, BN));
  GB_TRY(make_map(&m_blo, blo, Np, Kp, BN));

  static bool attr_set[64] = {false};
  if (!attr_set[c->device & 63]) {
    GB_CUDA_TRY(cudaFuncSetAttribute(gemm_bf16x3_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)CF::kSmem));
    attr_set[c->device & 63] = true;
  }
  const int tiles_m = (int)(Mp / kBM), tiles_n = (int)(Np / BN);
  gemm_bf16x3_kernel<BN><<<tiles_m * tiles_n, kThreads, CF::kSmem, stream>>>(
      m_ahi, m_alo, m_bhi, m_blo, (int)M, (int)N, (int)(Kp / kBK), tiles_m, tiles_n, C, rsc, csc, err);
  return check_launch("gemm_bf16x3_kernel");
}

}  // namespace

gbblas_status launch_gemm_bf16x3(DeviceCtx* c, int64_t M, int64_t N, int64_t K, const float* A, int64_t rsa,
                                 int64_t csa, const float* B, int64_t rsb, int64_t csb, float* C, int64_t rsc,
                                 int64_t csc, cudaStream_t stream) {
  if (M == 0 || N == 0 || K == 0) return GBBLAS_STATUS_SUCCESS;
  if (M > (1 << 30) || N > (1 << 30) || K > (1 << 30)) {
    set_error("bf16x3 gemm: dimension beyond 2^30");
    return GBBLAS_STATUS_NOT_SUPPORTED;
  }
  if (N <= 128) return run_bf16x3<128>(c, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, stream);
  return run_bf16x3<256>(c, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, stream);
}

}  // namespace gbblas
