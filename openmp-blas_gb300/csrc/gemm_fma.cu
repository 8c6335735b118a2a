// gemm_fma.cu - C += A*B on the CUDA cores (FP32 FMA / FP64 DFMA).
//
// Replaces the reference's Goto/BLIS GEMM (include/mtm.hpp:116-206 with the
// MR x NR micro-kernel include/simd_loop.hpp:80-192).  The GPU keeps the
// same three-level idea with GPU-sized levels:
//   * a CTA owns a BM x BN tile of C (the reference's MB x NB cache block),
//   * K is walked in BK slices staged in shared memory, double-buffered so
//     the next slice's global loads are in flight during the FMAs on the
//     current one (the reference's packed A/B panels, include/utils.hpp:99-141),
//   * each thread owns a TM x TN register tile (the reference's MR x NR
//     `buff`), accumulates over all of K from zero in k order with FMA,
//     and finally adds it into C - like copy_from_buff, C is accumulated.
// Every (C, A, B) layout mix is served: the loaders read A with M or K
// contiguous and B with N or K contiguous using 128-bit loads, and fall back
// to strided element loads for any other strides, always writing shared
// memory in one K-major layout so the inner loop does not change.
#include "common.cuh"

namespace gbblas {
namespace {

enum : int { kVecMN = 0, kVecK = 1, kScalar = 2 };

template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  using t = float4;
  static constexpr int w = 4;
};
template <>
struct Vec16<double> {
  using t = double2;
  static constexpr int w = 2;
};

// 4 consecutive T from shared memory (16-byte aligned).
__device__ __forceinline__ void lds4(const float* p, float (&o)[4]) {
  float4 v = *reinterpret_cast<const float4*>(p);
  o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
}
__device__ __forceinline__ void lds4(const double* p, double (&o)[4]) {
  double2 v0 = reinterpret_cast<const double2*>(p)[0];
  double2 v1 = reinterpret_cast<const double2*>(p)[1];
  o[0] = v0.x; o[1] = v0.y; o[2] = v1.x; o[3] = v1.y;
}

template <typename T, int BM, int BN, int BK, int TM, int TN>
struct Cfg {
  static constexpr int W = Vec16<T>::w;
  static constexpr int NT = (BM / TM) * (BN / TN);
  static constexpr int PAD = W;  // keeps rows 16-byte aligned and spreads banks
  static constexpr int TM4 = TM / 4, TN4 = TN / 4;
  static_assert(TM % 4 == 0 && TN % 4 == 0, "register tile in groups of 4");
  static_assert((BM * BK) % (W * NT) == 0 && (BN * BK) % (W * NT) == 0, "whole vectors per thread");
  static_assert((BM * BK) % NT == 0 && (BN * BK) % NT == 0, "whole elements per thread");
  static constexpr int AV = BM * BK / W / NT;  // vectors of A per thread
  static constexpr int BV = BN * BK / W / NT;
  static constexpr int AS = BM * BK / NT;  // scalars of A per thread
  static constexpr int BS = BN * BK / NT;
  static constexpr int AR = AS > AV * W ? AS : AV * W;  // staging registers
  static constexpr int BR = BS > BV * W ? BS : BV * W;
};

template <typename T, int BM, int BN, int BK, int TM, int TN, int LA, int LB>
__global__ void __launch_bounds__(Cfg<T, BM, BN, BK, TM, TN>::NT, 2)
    gemm_fma_kernel(int64_t M, int64_t N, int64_t K, const T* __restrict__ A, int64_t rsa, int64_t csa,
                    const T* __restrict__ B, int64_t rsb, int64_t csb, T* __restrict__ C, int64_t rsc,
                    int64_t csc, int64_t tiles_n, int64_t ntiles) {
  using CF = Cfg<T, BM, BN, BK, TM, TN>;
  using VT = typename Vec16<T>::t;
  constexpr int W = CF::W, NT = CF::NT, PAD = CF::PAD;
  __shared__ __align__(16) T As[2][BK][BM + PAD];
  __shared__ __align__(16) T Bs[2][BK][BN + PAD];

  const int tid = threadIdx.x;
  const int tx = tid % (BN / TN), ty = tid / (BN / TN);
  int64_t m0 = 0, n0 = 0;  // current output tile (set per tile below)

  T ra[CF::AR], rb[CF::BR];

  // ---- global -> registers for K slice starting at k0 (zero outside bounds)
  auto load_a = [&](int64_t k0) {
    if (LA == kVecMN) {  // A column-major: vectors along M
#pragma unroll
      for (int v = 0; v < CF::AV; ++v) {
        const int q = tid + v * NT, k = q / (BM / W), m = (q % (BM / W)) * W;
        const int64_t gm = m0 + m, gk = k0 + k;
        if (gk < K && gm + W <= M) {
          VT t = __ldg(reinterpret_cast<const VT*>(A + gm + gk * csa));
          const T* tp = reinterpret_cast<const T*>(&t);
#pragma unroll
          for (int e = 0; e < W; ++e) ra[v * W + e] = tp[e];
        } else {
#pragma unroll
          for (int e = 0; e < W; ++e) ra[v * W + e] = (gk < K && gm + e < M) ? A[gm + e + gk * csa] : T(0);
        }
      }
    } else if (LA == kVecK) {  // A row-major: vectors along K
#pragma unroll
      for (int v = 0; v < CF::AV; ++v) {
        const int q = tid + v * NT, m = q / (BK / W), k = (q % (BK / W)) * W;
        const int64_t gm = m0 + m, gk = k0 + k;
        if (gm < M && gk + W <= K) {
          VT t = __ldg(reinterpret_cast<const VT*>(A + gm * rsa + gk));
          const T* tp = reinterpret_cast<const T*>(&t);
#pragma unroll
          for (int e = 0; e < W; ++e) ra[v * W + e] = tp[e];
        } else {
#pragma unroll
          for (int e = 0; e < W; ++e) ra[v * W + e] = (gm < M && gk + e < K) ? A[gm * rsa + gk + e] : T(0);
        }
      }
    } else {
#pragma unroll
      for (int s = 0; s < CF::AS; ++s) {
        const int q = tid + s * NT, k = q / BM, m = q % BM;
        const int64_t gm = m0 + m, gk = k0 + k;
        ra[s] = (gm < M && gk < K) ? A[gm * rsa + gk * csa] : T(0);
      }
    }
  };
  auto store_a = [&](int buf) {
    if (LA == kVecMN) {
#pragma unroll
      for (int v = 0; v < CF::AV; ++v) {
        const int q = tid + v * NT, k = q / (BM / W), m = (q % (BM / W)) * W;
#pragma unroll
        for (int e = 0; e < W; ++e) As[buf][k][m + e] = ra[v * W + e];
      }
    } else if (LA == kVecK) {
#pragma unroll
      for (int v = 0; v < CF::AV; ++v) {
        const int q = tid + v * NT, m = q / (BK / W), k = (q % (BK / W)) * W;
#pragma unroll
        for (int e = 0; e < W; ++e) As[buf][k + e][m] = ra[v * W + e];
      }
    } else {
#pragma unroll
      for (int s = 0; s < CF::AS; ++s) {
        const int q = tid + s * NT, k = q / BM, m = q % BM;
        As[buf][k][m] = ra[s];
      }
    }
  };
  auto load_b = [&](int64_t k0) {
    if (LB == kVecMN) {  // B row-major: vectors along N
#pragma unroll
      for (int v = 0; v < CF::BV; ++v) {
        const int q = tid + v * NT, k = q / (BN / W), n = (q % (BN / W)) * W;
        const int64_t gn = n0 + n, gk = k0 + k;
        if (gk < K && gn + W <= N) {
          VT t = __ldg(reinterpret_cast<const VT*>(B + gk * rsb + gn));
          const T* tp = reinterpret_cast<const T*>(&t);
#pragma unroll
          for (int e = 0; e < W; ++e) rb[v * W + e] = tp[e];
        } else {
#pragma unroll
          for (int e = 0; e < W; ++e) rb[v * W + e] = (gk < K && gn + e < N) ? B[gk * rsb + gn + e] : T(0);
        }
      }
    } else if (LB == kVecK) {  // B column-major: vectors along K
#pragma unroll
      for (int v = 0; v < CF::BV; ++v) {
        const int q = tid + v * NT, n = q / (BK / W), k = (q % (BK / W)) * W;
        const int64_t gn = n0 + n, gk = k0 + k;
        if (gn < N && gk + W <= K) {
          VT t = __ldg(reinterpret_cast<const VT*>(B + gn * csb + gk));
          const T* tp = reinterpret_cast<const T*>(&t);
#pragma unroll
          for (int e = 0; e < W; ++e) rb[v * W + e] = tp[e];
        } else {
#pragma unroll
          for (int e = 0; e < W; ++e) rb[v * W + e] = (gn < N && gk + e < K) ? B[gn * csb + gk + e] : T(0);
        }
      }
    } else {
#pragma unroll
      for (int s = 0; s < CF::BS; ++s) {
        const int q = tid + s * NT, k = q / BN, n = q % BN;
        const int64_t gn = n0 + n, gk = k0 + k;
        rb[s] = (gn < N && gk < K) ? B[gk * rsb + gn * csb] : T(0);
      }
    }
  };
  auto store_b = [&](int buf) {
    if (LB == kVecMN) {
#pragma unroll
      for (int v = 0; v < CF::BV; ++v) {
        const int q = tid + v * NT, k = q / (BN / W), n = (q % (BN / W)) * W;
#pragma unroll
        for (int e = 0; e < W; ++e) Bs[buf][k][n + e] = rb[v * W + e];
      }
    } else if (LB == kVecK) {
#pragma unroll
      for (int v = 0; v < CF::BV; ++v) {
        const int q = tid + v * NT, n = q / (BK / W), k = (q % (BK / W)) * W;
#pragma unroll
        for (int e = 0; e < W; ++e) Bs[buf][k + e][n] = rb[v * W + e];
      }
    } else {
#pragma unroll
      for (int s = 0; s < CF::BS; ++s) {
        const int q = tid + s * NT, k = q / BN, n = q % BN;
        Bs[buf][k][n] = rb[s];
      }
    }
  };

  // Tiles are handed out grid-stride, so a grid capped below the tile count
  // (a caller sharing the GPU with latency-sensitive work) still covers C.
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
  m0 = (tile / tiles_n) * BM;
  n0 = (tile % tiles_n) * BN;
  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = T(0);

  const int64_t ktiles = (K + BK - 1) / BK;
  load_a(0);
  load_b(0);
  store_a(0);
  store_b(0);
  __syncthreads();

  for (int64_t kt = 0; kt < ktiles; ++kt) {
    const int buf = (int)(kt & 1);
    const bool more = kt + 1 < ktiles;
    if (more) {
      load_a((kt + 1) * BK);
      load_b((kt + 1) * BK);
    }
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      T a[TM], b[TN];
#pragma unroll
      for (int g = 0; g < CF::TM4; ++g) {
        T t[4];
        lds4(&As[buf][k][g * (BM / CF::TM4) + ty * 4], t);
#pragma unroll
        for (int i = 0; i < 4; ++i) a[g * 4 + i] = t[i];
      }
#pragma unroll
      for (int g = 0; g < CF::TN4; ++g) {
        T t[4];
        lds4(&Bs[buf][k][g * (BN / CF::TN4) + tx * 4], t);
#pragma unroll
        for (int j = 0; j < 4; ++j) b[g * 4 + j] = t[j];
      }
      if constexpr (sizeof(T) == 4) {
        // packed FP32x2 FMAs: two columns per instruction, each lane an IEEE
        // fmaf (bit-identical to the scalar form), half the issue slots
#pragma unroll
        for (int i = 0; i < TM; ++i) {
          const float2 ai = make_float2(a[i], a[i]);
#pragma unroll
          for (int j = 0; j < TN; j += 2) {
            const float2 r = __ffma2_rn(ai, make_float2(b[j], b[j + 1]), make_float2(acc[i][j], acc[i][j + 1]));
            acc[i][j] = r.x;
            acc[i][j + 1] = r.y;
          }
        }
      } else {
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
      }
    }
    if (more) {
      store_a(buf ^ 1);
      store_b(buf ^ 1);
    }
    __syncthreads();
  }

  // ---- C += acc (the reference's copy_from_buff, include/simd_loop.hpp:160-190);
  // a row's loads are issued before its stores (the compiler cannot see
  // that runtime strides keep the outputs apart)
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int64_t gm = m0 + (i / 4) * (BM / CF::TM4) + ty * 4 + (i % 4);
    if (gm >= M) continue;
    T old[TN];
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int64_t gn = n0 + (j / 4) * (BN / CF::TN4) + tx * 4 + (j % 4);
      old[j] = gn < N ? C[gm * rsc + gn * csc] : T(0);
    }
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int64_t gn = n0 + (j / 4) * (BN / CF::TN4) + tx * 4 + (j % 4);
      if (gn < N) C[gm * rsc + gn * csc] = old[j] + acc[i][j];
    }
  }
  }  // tile loop
}

template <typename T, int BM, int BN, int BK, int TM, int TN>
gbblas_status launch_cfg(int la, int lb, int64_t M, int64_t N, int64_t K, const T* A, int64_t rsa, int64_t csa,
                         const T* B, int64_t rsb, int64_t csb, T* C, int64_t rsc, int64_t csc,
                         cudaStream_t stream, int max_ctas) {
  using CF = Cfg<T, BM, BN, BK, TM, TN>;
  const int64_t tiles_n = (N + BN - 1) / BN, ntiles = tiles_n * ((M + BM - 1) / BM);
  int64_t g = ntiles;
  if (max_ctas > 0 && g > max_ctas) g = max_ctas;
  if (g > 0x7fffffff) g = 0x7fffffff;
  const unsigned grid = (unsigned)g;
#define GB_L(LA_, LB_)                                                                                   \
  gemm_fma_kernel<T, BM, BN, BK, TM, TN, LA_, LB_><<<grid, CF::NT, 0, stream>>>(M, N, K, A, rsa, csa, B, \
                                                                                rsb, csb, C, rsc, csc,  \
                                                                                tiles_n, ntiles)
  if (la == kScalar || lb == kScalar)
    GB_L(kScalar, kScalar);
  else if (la == kVecMN && lb == kVecMN)
    GB_L(kVecMN, kVecMN);
  else if (la == kVecMN && lb == kVecK)
    GB_L(kVecMN, kVecK);
  else if (la == kVecK && lb == kVecMN)
    GB_L(kVecK, kVecMN);
  else
    GB_L(kVecK, kVecK);
#undef GB_L
  return check_launch("gemm_fma_kernel");
}

}  // namespace

template <typename T>
gbblas_status launch_gemm_fma(DeviceCtx* c, int64_t M, int64_t N, int64_t K, const T* A, int64_t rsa,
                              int64_t csa, const T* B, int64_t rsb, int64_t csb, T* C, int64_t rsc, int64_t csc,
                              cudaStream_t stream, int max_ctas, int tile) {
  constexpr int W = Vec16<T>::w;
  // Which loader each operand can use.
  int la = kScalar, lb = kScalar;
  if (aligned16(A)) {
    if (rsa == 1 && csa % W == 0) la = kVecMN;
    else if (csa == 1 && rsa % W == 0) la = kVecK;
  }
  if (aligned16(B)) {
    if (csb == 1 && rsb % W == 0) lb = kVecMN;
    else if (rsb == 1 && csb % W == 0) lb = kVecK;
  }
  if (M == 0 || N == 0 || K == 0) return GBBLAS_STATUS_SUCCESS;
  if constexpr (sizeof(T) == 4) {
    const int64_t big_tiles = ((M + 127) / 128) * ((N + 127) / 128);
    const bool tma = sgemm_tma_eligible(M, N, K, A, rsa, csa, B, rsb, csb);
    // default: TMA-fed where B is row-major (at 8192^3: 63.8 / 58.7 TFLOP/s
    // with A column- / row-major against 58.9 / 57.5 register-staged; with B
    // column-major its FMA pairs need register moves and it trails)
    if (tile < 0)
      tile = (tma && csb == 1 && big_tiles >= (int64_t)c->num_sms) ? 2
                                                                   : (big_tiles >= 2 * (int64_t)c->num_sms ? 1 : 0);
    if (tile == 4 && tma)
      return launch_sgemm_tma(c, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, stream, max_ctas, 2);
    if (tile == 3 && tma)
      return launch_sgemm_tma(c, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, stream, max_ctas, 1);
    if (tile >= 2 && tma)
      return launch_sgemm_tma(c, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, stream, max_ctas);
    if (tile >= 1)
      return launch_cfg<float, 128, 128, 16, 8, 8>(la, lb, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, stream,
                                                   max_ctas);
    return launch_cfg<float, 64, 64, 16, 4, 4>(la, lb, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, stream,
                                               max_ctas);
  } else {
    return launch_cfg<double, 64, 64, 8, 4, 4>(la, lb, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, stream,
                                               max_ctas);
  }
}

template gbblas_status launch_gemm_fma<float>(DeviceCtx*, int64_t, int64_t, int64_t, const float*, int64_t,
                                              int64_t, const float*, int64_t, int64_t, float*, int64_t, int64_t,
                                              cudaStream_t, int, int);
template gbblas_status launch_gemm_fma<double>(DeviceCtx*, int64_t, int64_t, int64_t, const double*, int64_t,
                                               int64_t, const double*, int64_t, int64_t, double*, int64_t,
                                               int64_t, cudaStream_t, int, int);

}  // namespace gbblas
