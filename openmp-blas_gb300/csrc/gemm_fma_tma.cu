// gemm_fma_tma.cu - FP32 C += A*B on the FMA pipes, operands fed by TMA.
//
// The same arithmetic as gemm_fma.cu (each thread accumulates its outputs
// from zero over K in k order with fused multiply-adds, then adds them into
// C, the reference's micro-kernel and copy_from_buff, include/simd_loop.hpp:
// 80-192), so the two give the same bits; what differs is how operands reach
// shared memory.  Here one producer warp streams 128 x 32 tiles of A and
// 32 x 128 tiles of B with cp.async.bulk.tensor into a 6-stage ring
// (mbarrier full / empty per stage, every wait bounded), and eight compute
// warps only read shared memory and issue packed FP32x2 FMAs - no staging
// registers, no block-wide barriers in the K loop.
//
// Tiles land in the operand's own layout:
//   * M- (N-) contiguous operand ("MN-major"): box of 128 x 32, rows of 128
//     floats per k, no swizzle; a thread reads 2 float4 per k.
//   * K-contiguous operand ("K-major"): box of 32 x 128, 128-byte rows with
//     the 128-byte swizzle (16-byte chunk c of row r stored at c ^ (r & 7));
//     a thread reads one float4 = 4 consecutive k of each of its 8 rows.
// Thread (ty, tx) of the 16 x 16 compute grid owns rows ty*4 + {0..3} and
// 64 + ty*4 + {0..3} of an MN-major A (ty + 16 i of a K-major A) and the
// same pattern over tx for B's columns: conflict-free shared-memory reads in
// both layouts.
//
// Persistent: grid = min(tiles, SMs or the caller's cap), tiles in grouped
// raster order (8 tile rows per band) for L2 reuse; the ring carries over
// from tile to tile.  Split-K (parts > 1, for shapes whose tiles leave SMs
// idle): each unit = (tile, K part) stores its K range's sum into that
// part's partial (no other unit writes those elements), then the partials
// are added into C in part order - within the same bound, not the same bits
// as the unsplit kernels.  Roofline: the FMA pipes,
// 2*M*N*K flops.
#include <cuda.h>

#include <mutex>

#include "common.cuh"
#include "tc_ptx.cuh"
#include "tma_map.cuh"

namespace gbblas {
namespace {

using namespace tc;

constexpr int kBM = 128;
constexpr int kBN = 128;
constexpr int kBK = 32;                           // one 128-byte row of a K-major tile
constexpr int kStages = 6;
constexpr uint32_t kTileBytes = kBM * kBK * 4;    // 16 KB, A or B
constexpr uint32_t kStageBytes = 2 * kTileBytes;  // A then B
constexpr int kComputeWarps = 8;
constexpr int kThreads = 32 * (kComputeWarps + 1);
constexpr size_t kSmem = 1024 /*alignment slack*/ + (size_t)kStages * kStageBytes + 256 /*barriers*/;
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s
static_assert(kSmem <= 232448, "exceeds 227 KB of shared memory");
static_assert((2 * kStages) * 8 + 4 <= 256, "barrier area too small");

// The 8 values (one per owned row or column i) of 4 consecutive k (kq*4..+3)
// from a tile: v[i][kk].
template <bool KMAJ>
__device__ __forceinline__ void load_frag(const float* __restrict__ tile, int id, int kq, float (&v)[8][4]) {
  if constexpr (KMAJ) {
    // row r = id + 16 i, 32 floats per row, chunk kq at (kq ^ (r & 7)); r & 7 = id & 7
    const int chunk = (kq ^ (id & 7)) * 4;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const float4 t = *reinterpret_cast<const float4*>(tile + (id + 16 * i) * kBK + chunk);
      v[i][0] = t.x;
      v[i][1] = t.y;
      v[i][2] = t.z;
      v[i][3] = t.w;
    }
  } else {
    // [k][mn], 128 floats per k: rows id*4 + {0..3} and 64 + id*4 + {0..3}
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const float* row = tile + (kq * 4 + kk) * kBM + id * 4;
      const float4 lo = *reinterpret_cast<const float4*>(row);
      const float4 hi = *reinterpret_cast<const float4*>(row + 64);
      v[0][kk] = lo.x;
      v[1][kk] = lo.y;
      v[2][kk] = lo.z;
      v[3][kk] = lo.w;
      v[4][kk] = hi.x;
      v[5][kk] = hi.y;
      v[6][kk] = hi.z;
      v[7][kk] = hi.w;
    }
  }
}

// Tile row / column owned as index i by thread coordinate id.
template <bool KMAJ>
__device__ __forceinline__ int owned(int id, int i) {
  return KMAJ ? id + 16 * i : id * 4 + (i & 3) + 64 * (i >> 2);
}

__device__ __forceinline__ void tile_origin(int t, int tiles_m, int tiles_n, int& m0, int& n0) {
  constexpr int kGroup = 8;
  const int span = kGroup * tiles_n;
  const int g = t / span, first_m = g * kGroup;
  const int gm = min(tiles_m - first_m, kGroup);
  const int in_g = t % span;
  m0 = (first_m + in_g % gm) * kBM;
  n0 = (in_g / gm) * kBN;
}

// A_KMAJ: A row-major (K contiguous), else column-major (M contiguous);
// B_KMAJ: B column-major (K contiguous), else row-major (N contiguous).
template <bool A_KMAJ, bool B_KMAJ>
__global__ void __launch_bounds__(kThreads, 1)
    sgemm_tma_kernel(const __grid_constant__ CUtensorMap tm_a, const __grid_constant__ CUtensorMap tm_b, int M, int N,
                     int K, float* __restrict__ C, int64_t rsc, int64_t csc, int tiles_m, int tiles_n,
                     int parts, float* __restrict__ part_buf, int* __restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)kStages * kStageBytes);
  uint64_t* empty = full + kStages;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(empty + kStages);
  auto a_tile = [&](int s) { return smem + (size_t)s * kStageBytes; };
  auto b_tile = [&](int s) { return smem + (size_t)s * kStageBytes + kTileBytes; };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kComputeWarps);  // one arrival per compute warp
    }
    *abort_flag = 0;
    fence_mbar_init();
    prefetch_tensormap(&tm_a);
    prefetch_tensormap(&tm_b);
  }
  __syncthreads();

  auto fail = [&]() {
    *abort_flag = 1;
    atomicExch(err, (int)GBBLAS_STATUS_TIMEOUT);
  };
  // work unit u = (tile u / parts, K part u % parts); parts > 1 (split-K):
  // each unit adds its K range into its own zeroed M x N partial
  const int nunits = tiles_m * tiles_n * parts;
  const int nk = (K + kBK - 1) / kBK;
  int issued = 0;

  if (warp == kComputeWarps) {
    if (lane == 0) {
      bool stop = false;
      for (int u = blockIdx.x; u < nunits && !stop; u += gridDim.x) {
        const int t = u / parts, pp = u % parts;
        int m0, n0;
        tile_origin(t, tiles_m, tiles_n, m0, n0);
        const int kb = (int)((int64_t)nk * pp / parts), ke = (int)((int64_t)nk * (pp + 1) / parts);
        for (int kt = kb; kt < ke; ++kt) {
          const int s = issued % kStages, round = issued / kStages;
          if (round > 0 && !mbar_wait_bounded(&empty[s], (round - 1) & 1, abort_flag, kWaitLimitNs)) {
            fail();
            stop = true;
            break;
          }
          mbar_arrive_expect_tx(&full[s], kStageBytes);  // out-of-range parts of a box arrive as zeros
          if constexpr (A_KMAJ)
            tma_load_2d(a_tile(s), &tm_a, &full[s], kt * kBK, m0);
          else
            tma_load_2d(a_tile(s), &tm_a, &full[s], m0, kt * kBK);
          if constexpr (B_KMAJ)
            tma_load_2d(b_tile(s), &tm_b, &full[s], kt * kBK, n0);
          else
            tma_load_2d(b_tile(s), &tm_b, &full[s], n0, kt * kBK);
          ++issued;
        }
      }
    }
  } else {
    const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
    int consumed = 0;
    bool ok = true;
    for (int u = blockIdx.x; u < nunits && ok; u += gridDim.x) {
      const int t = u / parts, pp = u % parts;
      int m0, n0;
      tile_origin(t, tiles_m, tiles_n, m0, n0);
      const int kb = (int)((int64_t)nk * pp / parts), ke = (int)((int64_t)nk * (pp + 1) / parts);
      float acc[8][8];
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
      for (int kt = kb; kt < ke; ++kt, ++consumed) {
        const int s = consumed % kStages, round = consumed / kStages;
        // warp-uniform decision: every lane leaves the loop together
        if (!__all_sync(0xffffffffu, mbar_wait_bounded(&full[s], round & 1, abort_flag, kWaitLimitNs))) {
          if (lane == 0) fail();
          ok = false;
          break;
        }
        const float* As = reinterpret_cast<const float*>(a_tile(s));
        const float* Bs = reinterpret_cast<const float*>(b_tile(s));
#pragma unroll
        for (int kq = 0; kq < kBK / 4; ++kq) {
          float a[8][4], b[8][4];
          load_frag<A_KMAJ>(As, ty, kq, a);
          load_frag<B_KMAJ>(Bs, tx, kq, b);
          // Packed FP32x2 FMAs pair two outputs that share one operand value.
          // Pair along the operand whose fragment came in as float4 over
          // rows / columns (an MN-major one), so each pair is a register
          // pair as loaded, with no moves.
          if constexpr (!B_KMAJ || A_KMAJ) {  // pairs along j: (b[j], b[j+1]) x a[i]
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
#pragma unroll
              for (int i = 0; i < 8; ++i) {
                const float2 ai = make_float2(a[i][kk], a[i][kk]);
#pragma unroll
                for (int j = 0; j < 8; j += 2) {
                  const float2 r =
                      __ffma2_rn(ai, make_float2(b[j][kk], b[j + 1][kk]), make_float2(acc[i][j], acc[i][j + 1]));
                  acc[i][j] = r.x;
                  acc[i][j + 1] = r.y;
                }
              }
          } else {  // A MN-major, B K-major: pairs along i, (a[i], a[i+1]) x b[j]
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                const float2 bj = make_float2(b[j][kk], b[j][kk]);
#pragma unroll
                for (int i = 0; i < 8; i += 2) {
                  const float2 r =
                      __ffma2_rn(make_float2(a[i][kk], a[i + 1][kk]), bj, make_float2(acc[i][j], acc[i + 1][j]));
                  acc[i][j] = r.x;
                  acc[i + 1][j] = r.y;
                }
              }
          }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
      }
      if (!ok) break;
      // C += acc (rows / columns outside the matrix dropped).  Split-K: this
      // part's dense partial, which no other unit writes - stored, not added.
      // Loads of C for four rows are issued before their stores (the
      // compiler cannot see that runtime strides keep the rows apart).
      const bool partial = parts > 1;
      float* Ct = partial ? part_buf + (int64_t)pp * M * N : C;
      const int64_t rs = partial ? (int64_t)N : rsc, cs = partial ? 1 : csc;
#pragma unroll
      for (int i0 = 0; i0 < 8; i0 += 4) {
        if constexpr (!B_KMAJ) {
          // columns tx*4 + {0..3} and 64 + tx*4 + {0..3}: two float4 when C rows are contiguous
          const bool vec = cs == 1 && ((rs & 3) == 0) && ((reinterpret_cast<uintptr_t>(Ct) & 15) == 0);
          float4 cv[4][2];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int m = m0 + owned<A_KMAJ>(ty, i0 + i);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const int n = n0 + tx * 4 + 64 * h;
              cv[i][h] = (!partial && vec && m < M && n + 4 <= N)
                             ? *reinterpret_cast<const float4*>(Ct + (int64_t)m * rs + n)
                             : make_float4(0.f, 0.f, 0.f, 0.f);
            }
          }
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int m = m0 + owned<A_KMAJ>(ty, i0 + i);
            if (m >= M) continue;
            float* crow = Ct + (int64_t)m * rs;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const int n = n0 + tx * 4 + 64 * h;
              const float* a4 = &acc[i0 + i][4 * h];
              if (vec && n + 4 <= N) {
                float4 v = cv[i][h];
                v.x += a4[0];
                v.y += a4[1];
                v.z += a4[2];
                v.w += a4[3];
                *reinterpret_cast<float4*>(crow + n) = v;
              } else {
#pragma unroll
                for (int q = 0; q < 4; ++q)
                  if (n + q < N) {
                    float* cq = crow + (int64_t)(n + q) * cs;
                    *cq = partial ? a4[q] : *cq + a4[q];
                  }
              }
            }
          }
        } else {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int m = m0 + owned<A_KMAJ>(ty, i0 + i);
            if (m >= M) continue;
            float* crow = Ct + (int64_t)m * rs;
            float old[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const int n = n0 + owned<true>(tx, j);
              old[j] = (!partial && n < N) ? crow[(int64_t)n * cs] : 0.f;
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const int n = n0 + owned<true>(tx, j);
              if (n < N) crow[(int64_t)n * cs] = old[j] + acc[i0 + i][j];
            }
          }
        }
      }
    }
  }

  // after an abort, let this CTA's copies in flight land before it exits
  if (warp == kComputeWarps && lane == 0 && *abort_flag) {
    int never = 0;
    const int from = issued > kStages ? issued - kStages : 0;
    for (int k = from; k < issued; ++k)
      (void)mbar_wait_bounded(&full[k % kStages], (k / kStages) & 1, &never, kWaitLimitNs / 2);
  }
}

// Split-K: C += part[0] + part[1] + ... (parts in order), grid-stride.
__global__ void __launch_bounds__(256) sgemm_parts_reduce_kernel(float* __restrict__ C, int64_t rsc, int64_t csc,
                                                                 const float* __restrict__ part, int M, int N,
                                                                 int parts) {
  const int64_t total = (int64_t)M * N;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    float s = part[e];
    for (int p = 1; p < parts; ++p) s += part[(int64_t)p * total + e];
    const int64_t r = e / N, c = e % N;
    C[r * rsc + c * csc] += s;
  }
}

// The four kernels' shared-memory attribute, once per device (before any
// stream capture: tc_prepare calls this too).
void set_attributes(DeviceCtx* c) {
  static std::mutex mu;
  static bool done[64] = {false};
  std::lock_guard<std::mutex> lk(mu);
  if (done[c->device & 63]) return;
  cudaFuncSetAttribute(sgemm_tma_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
  cudaFuncSetAttribute(sgemm_tma_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
  cudaFuncSetAttribute(sgemm_tma_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
  cudaFuncSetAttribute(sgemm_tma_kernel<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
  done[c->device & 63] = true;
}

template <bool AK, bool BK>
gbblas_status launch_cfg(DeviceCtx* c, const CUtensorMap& ma, const CUtensorMap& mb, int64_t M, int64_t N,
                         int64_t K, float* C, int64_t rsc, int64_t csc, int* err, cudaStream_t stream, int max_ctas,
                         int parts, float* part_buf) {
  set_attributes(c);
  const int tiles_m = (int)((M + kBM - 1) / kBM), tiles_n = (int)((N + kBN - 1) / kBN);
  int64_t grid = std::min<int64_t>((int64_t)tiles_m * tiles_n * parts, c->num_sms);
  if (max_ctas > 0 && grid > max_ctas) grid = max_ctas;
  sgemm_tma_kernel<AK, BK><<<(unsigned)grid, kThreads, kSmem, stream>>>(ma, mb, (int)M, (int)N, (int)K, C, rsc, csc,
                                                                      tiles_m, tiles_n, parts, part_buf, err);
  return check_launch("sgemm_tma_kernel");
}

}  // namespace

void sgemm_tma_prepare(DeviceCtx* c) { set_attributes(c); }

bool sgemm_tma_eligible(int64_t M, int64_t N, int64_t K, const float* A, int64_t rsa, int64_t csa, const float* B,
                        int64_t rsb, int64_t csb) {
  if (M <= 0 || N <= 0 || K <= 0 || M > (1ll << 31) - 1 || N > (1ll << 31) - 1 || K > (1ll << 31) - 1) return false;
  if ((int64_t)((M + kBM - 1) / kBM) * ((N + kBN - 1) / kBN) > (1ll << 31) - 1) return false;
  if (!aligned16(A) || !aligned16(B)) return false;
  const bool a_ok = (csa == 1 && rsa % 4 == 0 && rsa >= K) || (rsa == 1 && csa % 4 == 0 && csa >= M);
  const bool b_ok = (rsb == 1 && csb % 4 == 0 && csb >= K) || (csb == 1 && rsb % 4 == 0 && rsb >= N);
  return a_ok && b_ok;
}

gbblas_status launch_sgemm_tma(DeviceCtx* c, int64_t M, int64_t N, int64_t K, const float* A, int64_t rsa,
                               int64_t csa, const float* B, int64_t rsb, int64_t csb, float* C, int64_t rsc,
                               int64_t csc, cudaStream_t stream, int max_ctas, int parts) {
  if (M == 0 || N == 0 || K == 0) return GBBLAS_STATUS_SUCCESS;
  if (!sgemm_tma_eligible(M, N, K, A, rsa, csa, B, rsb, csb)) {
    set_error("TMA-fed sgemm: operands not 16-byte aligned with 16-byte-multiple strides");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  const bool ak = csa == 1 && rsa % 4 == 0 && rsa >= K;  // A rows contiguous along K
  const bool bk = rsb == 1 && csb % 4 == 0 && csb >= K;  // B columns contiguous along K
  CUtensorMap ma, mb;
  if (ak)
    GB_TRY(make_map_f32_2d(&ma, A, (uint64_t)K, (uint64_t)M, (uint64_t)rsa, kBK, kBM, true));
  else
    GB_TRY(make_map_f32_2d(&ma, A, (uint64_t)M, (uint64_t)K, (uint64_t)csa, kBM, kBK, false));
  if (bk)
    GB_TRY(make_map_f32_2d(&mb, B, (uint64_t)K, (uint64_t)N, (uint64_t)csb, kBK, kBN, true));
  else
    GB_TRY(make_map_f32_2d(&mb, B, (uint64_t)N, (uint64_t)K, (uint64_t)rsb, kBN, kBK, false));
  const int nk = (int)((K + kBK - 1) / kBK);
  if (parts < 1) parts = 1;
  if (parts > nk) parts = nk;
  const size_t part_bytes = parts > 1 ? sizeof(float) * (size_t)parts * (size_t)M * (size_t)N : 0;
  void* s = nullptr;
  GB_TRY(get_scratch(c, stream, kScratchZeroBytes + part_bytes, &s));
  int* err = reinterpret_cast<int*>(static_cast<char*>(s) + kErrWordOffset);
  float* part_buf = parts > 1 ? reinterpret_cast<float*>(static_cast<char*>(s) + kScratchZeroBytes) : nullptr;
  // (every element of every part is written by exactly one (tile, part) unit: no clearing)
  gbblas_status st;
  if (ak && bk)
    st = launch_cfg<true, true>(c, ma, mb, M, N, K, C, rsc, csc, err, stream, max_ctas, parts, part_buf);
  else if (ak)
    st = launch_cfg<true, false>(c, ma, mb, M, N, K, C, rsc, csc, err, stream, max_ctas, parts, part_buf);
  else if (bk)
    st = launch_cfg<false, true>(c, ma, mb, M, N, K, C, rsc, csc, err, stream, max_ctas, parts, part_buf);
  else
    st = launch_cfg<false, false>(c, ma, mb, M, N, K, C, rsc, csc, err, stream, max_ctas, parts, part_buf);
  if (st != GBBLAS_STATUS_SUCCESS || parts == 1) return st;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((M * N + 255) / 256, 4 * (int64_t)c->num_sms));
  sgemm_parts_reduce_kernel<<<blocks, 256, 0, stream>>>(C, rsc, csc, part_buf, (int)M, (int)N, parts);
  return check_launch("sgemm_parts_reduce_kernel");
}

int sgemm_tma_split_parts(DeviceCtx* c, int64_t M, int64_t N, int64_t K) {
  const int64_t tiles = ((M + kBM - 1) / kBM) * ((N + kBN - 1) / kBN);
  const int64_t nk = (K + kBK - 1) / kBK;
  for (int p = 4; p >= 2; --p)
    if (tiles * p <= (int64_t)c->num_sms && nk >= 8 * p) return p;
  return 1;
}

}  // namespace gbblas
