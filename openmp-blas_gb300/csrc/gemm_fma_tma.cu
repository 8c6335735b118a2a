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
// from tile to tile.  Stream-K (for shapes whose tiles fill the SMs badly,
// e.g. 64 tiles of a 1024^3 product on 152 SMs): the tiles' K blocks, laid
// end to end, are cut into one equal range per CTA, so every SM does the
// same number of FMAs.  A CTA whose range covers a whole tile adds it into C
// as above; a range that covers part of a tile ("segment") stores its sum
// into the segment's slot, and the tile's last segment to finish (an atomic
// count per tile) adds the slots in K order and then that sum into C - a
// fixed order for a given grid, so the bits repeat run to run, within the
// same bound as the unsplit kernels but not their bits.  No second kernel
// and no waiting on other CTAs.  Cluster pairs (for 57-76 tiles: two CTAs
// per tile fill the SMs in one wave): CTA 2t + r of a two-CTA cluster
// computes half r of tile t's K blocks; the even CTA signals (remote
// mbarrier arrive) that its stage ring is free, the odd CTA writes its sums
// into it through distributed shared memory and signals back, the even CTA
// adds them to its own (first half + second half) and updates C.  Every
// wait is bounded, and neither CTA leaves while the other may still touch
// its shared memory.  Roofline: the FMA pipes, 2*M*N*K flops.
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
// Two compute warpgroups (warps 0-7) and one producer warpgroup (warps 8-11,
// of which warp 8 issues the copies).  Registers: the kernel launches with
// 168 per thread (384 x 168 = 64512 of the SM's 65536); at the start the
// producer warpgroup gives back down to 40 and the compute warpgroups take
// 232: 128 x 40 + 256 x 232 = 64512, exactly the launch's total.
constexpr int kThreads = 32 * (kComputeWarps + 4);
constexpr int kLaunchRegs = 168, kProducerRegs = 40, kComputeRegs = 232;
static_assert(kThreads * kLaunchRegs <= 65536, "launch registers exceed the SM's");
static_assert(128 * kProducerRegs + 32 * kComputeWarps * kComputeRegs <= kThreads * kLaunchRegs,
              "register split exceeds what the block launched with");
constexpr size_t kSmem = 1024 /*alignment slack*/ + (size_t)kStages * kStageBytes + 256 /*barriers*/;
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s
static_assert(kSmem <= 232448, "exceeds 227 KB of shared memory");
static_assert((2 * kStages + 4) * 8 + 4 <= 256, "barrier area too small");

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
                     int streamk, int max_seg, float* __restrict__ slots, int* __restrict__ tile_cnt,
                     int* __restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)kStages * kStageBytes);
  uint64_t* empty = full + kStages;
  uint64_t* seg_stored = empty + kStages;   // stream-K: every compute warp stored its part of a segment
  uint64_t* seg_decided = seg_stored + 1;  // stream-K: the tile count was taken
  uint64_t* xfree = seg_decided + 1;       // cluster pairs (odd CTA): the even CTA's ring may be written
  uint64_t* xready = xfree + 1;            // cluster pairs (even CTA): the odd CTA's sums are in its ring
  volatile int* abort_flag = reinterpret_cast<volatile int*>(xready + 1);
  auto a_tile = [&](int s) { return smem + (size_t)s * kStageBytes; };
  auto b_tile = [&](int s) { return smem + (size_t)s * kStageBytes + kTileBytes; };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kComputeWarps);  // one arrival per compute warp
    }
    mbar_init(seg_stored, kComputeWarps);
    mbar_init(seg_decided, 1);
    mbar_init(xfree, 32 * kComputeWarps);  // one arrival per compute thread of the other CTA
    mbar_init(xready, 32 * kComputeWarps);
    *abort_flag = 0;
    fence_mbar_init();
    prefetch_tensormap(&tm_a);
    prefetch_tensormap(&tm_b);
  }
  __syncthreads();
  // cluster pairs: both CTAs' barriers exist before either signals the other
  if (streamk == 2) cluster_sync_all();
  const uint32_t crank = streamk == 2 ? cluster_ctarank() : 0u;

  auto fail = [&]() {
    *abort_flag = 1;
    atomicExch(err, (int)GBBLAS_STATUS_TIMEOUT);
  };
  const int ntiles = tiles_m * tiles_n;
  const int nk = (K + kBK - 1) / kBK;
  // The CTA's segments (tile t, K blocks kb..ke-1), in order: whole tiles
  // t = blockIdx.x, + gridDim.x, ... or, stream-K, its range of the tiles'
  // K blocks laid end to end.  seg(i, t, kb, ke) gives segment i; false when
  // there is none.
  const int64_t kt_total = (int64_t)ntiles * nk;
  const int64_t range_b = streamk == 1 ? kt_total * blockIdx.x / gridDim.x : 0;
  const int64_t range_e = streamk == 1 ? kt_total * (blockIdx.x + 1) / gridDim.x : 0;
  auto seg = [&](int64_t& pos, int& t, int& kb, int& ke) -> bool {
    if (streamk == 0) {
      t = (int)pos;
      if (t >= ntiles) return false;
      kb = 0;
      ke = nk;
      pos += gridDim.x;
      return true;
    }
    if (streamk == 2) {  // cluster pairs: CTA 2t + r computes half r of tile t's K blocks
      if (pos != (int64_t)blockIdx.x) return false;
      t = (int)(blockIdx.x >> 1);
      kb = crank ? nk / 2 : 0;
      ke = crank ? nk : nk / 2;
      ++pos;
      return true;
    }
    if (pos >= range_e) return false;
    t = (int)(pos / nk);
    kb = (int)(pos % nk);
    const int64_t left = range_e - pos;
    ke = left < (int64_t)(nk - kb) ? kb + (int)left : nk;
    pos += ke - kb;
    return true;
  };
  const int64_t pos0 = streamk == 1 ? range_b : blockIdx.x;
  int issued = 0;

  if (warp >= kComputeWarps) {
    // the producer warpgroup: registers back to the pool (warpgroup-wide, one
    // instruction for all four warps), then warp 8 lane 0 streams the tiles
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(kProducerRegs));
    if (warp == kComputeWarps && lane == 0) {
      bool stop = false;
      int t, kb, ke;
      for (int64_t pos = pos0; !stop && seg(pos, t, kb, ke);) {
        int m0, n0;
        tile_origin(t, tiles_m, tiles_n, m0, n0);
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
      // after an abort, let this CTA's copies in flight land before it exits
      if (*abort_flag) {
        int never = 0;
        const int from = issued > kStages ? issued - kStages : 0;
        for (int k = from; k < issued; ++k)
          (void)mbar_wait_bounded(&full[k % kStages], (k / kStages) & 1, &never, kWaitLimitNs / 2);
      }
    }
    return;
  }
  {
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(kComputeRegs));
    const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
    int consumed = 0;
    bool ok = true;
    int t, kb, ke;
    int nparts = 0;              // stream-K segments this CTA finished (phases of the two barriers)
    bool xwaited = false;        // cluster pairs, odd CTA: waited for the even CTA's arrivals
    __shared__ int seg_last;     // stream-K: 1 if this segment is its tile's last to finish
    for (int64_t pos = pos0; ok && seg(pos, t, kb, ke);) {
      int m0, n0;
      tile_origin(t, tiles_m, tiles_n, m0, n0);
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
      if (streamk == 2) {
        // cluster pair: the odd CTA's sums (second half of K) move into the
        // first 64 KB of the even CTA's stage ring - idle once the even CTA's
        // own K loop is done - thread-major (float4 v of thread tid at
        // 256 v + tid), and the even CTA adds them to its own, always in that
        // order, then updates C.  Both waits are bounded.
        // Neither exchange wait gives up early on this CTA's abort flag: a CTA
        // leaves only after the other's accesses to its shared memory landed
        // (or the bound ran out).
        float4* xbuf = reinterpret_cast<float4*>(smem);
        int never = 0;
        if (crank == 0) {
          mbar_arrive_cluster(mapa_shared(smem_u32(xfree), 1));  // release: this CTA is done reading its ring
          if (!__all_sync(0xffffffffu, mbar_wait_cluster_bounded(xready, 0, &never, kWaitLimitNs))) {
            if (lane == 0) fail();
            break;
          }
#pragma unroll
          for (int v = 0; v < 16; ++v) {
            const float4 x = xbuf[256 * v + threadIdx.x];
            float* a = &acc[v / 2][4 * (v % 2)];
            a[0] += x.x;
            a[1] += x.y;
            a[2] += x.z;
            a[3] += x.w;
          }
        } else {
          xwaited = true;
          if (!__all_sync(0xffffffffu, mbar_wait_cluster_bounded(xfree, 0, &never, kWaitLimitNs))) {
            if (lane == 0) fail();
            break;
          }
          const uint32_t base = mapa_shared(smem_u32(xbuf), 0);
#pragma unroll
          for (int v = 0; v < 16; ++v)
            st_cluster_v4(base + 16u * (uint32_t)(256 * v + threadIdx.x),
                          make_float4(acc[v / 2][4 * (v % 2)], acc[v / 2][4 * (v % 2) + 1],
                                      acc[v / 2][4 * (v % 2) + 2], acc[v / 2][4 * (v % 2) + 3]));
          mbar_arrive_cluster(mapa_shared(smem_u32(xready), 0));  // release: the sums are in
          continue;  // the even CTA adds both halves into C
        }
      } else if (kb != 0 || ke != nk) {
        // stream-K segment of tile t: segments are numbered in K order by
        // the CTA that holds their first K block (the largest c with
        // range_b(c) <= x is ((x + 1) G - 1) / T)
        const int64_t G = gridDim.x;
        const int64_t c0 = ((int64_t)t * nk + 1) * G - 1;
        const int first = (int)(c0 / kt_total), last = (int)((((int64_t)t * nk + nk) * G - 1) / kt_total);
        const int sidx = (int)blockIdx.x - first, nseg = last - first + 1;
        // slots are thread-major: float4 v of compute thread tid (its
        // acc[v / 2][4 (v % 2) .. + 3]) at float4 index 256 v + tid, so a
        // warp's 32 lanes store and load 512 contiguous bytes at a time;
        // every segment of a tile uses the same thread-to-output mapping
        float4* slot = reinterpret_cast<float4*>(slots + ((int64_t)t * max_seg + sidx) * (kBM * kBN));
#pragma unroll
        for (int v = 0; v < 16; ++v)
          __stcg(slot + 256 * v + threadIdx.x,
                 make_float4(acc[v / 2][4 * (v % 2)], acc[v / 2][4 * (v % 2) + 1], acc[v / 2][4 * (v % 2) + 2],
                             acc[v / 2][4 * (v % 2) + 3]));
        // every compute warp's slot stores, then one count per segment
        // (bounded waits on two barriers: an aborted warp never leaves the
        // others waiting)
        __threadfence();
        __syncwarp();
        if (lane == 0) mbar_arrive(seg_stored);
        if (!__all_sync(0xffffffffu, mbar_wait_bounded(seg_stored, nparts & 1, abort_flag, kWaitLimitNs))) {
          if (lane == 0) fail();
          break;
        }
        if (threadIdx.x == 0) {
          seg_last = atomicAdd(tile_cnt + t, 1) == nseg - 1;
          __threadfence();
          mbar_arrive(seg_decided);
        }
        if (!__all_sync(0xffffffffu, mbar_wait_bounded(seg_decided, nparts & 1, abort_flag, kWaitLimitNs))) {
          if (lane == 0) fail();
          break;
        }
        ++nparts;
        if (!seg_last) continue;  // another segment of the tile finishes it
        __threadfence();
        // the last segment: the tile's sum over its slots in K order (this
        // segment's own slot included), then into C below
        for (int q = 0; q < nseg; ++q) {
          const float4* sq = reinterpret_cast<const float4*>(slots + ((int64_t)t * max_seg + q) * (kBM * kBN));
#pragma unroll
          for (int v = 0; v < 16; ++v) {
            const float4 x = __ldcg(sq + 256 * v + threadIdx.x);
            float* a = &acc[v / 2][4 * (v % 2)];
            a[0] = q == 0 ? x.x : a[0] + x.x;
            a[1] = q == 0 ? x.y : a[1] + x.y;
            a[2] = q == 0 ? x.z : a[2] + x.z;
            a[3] = q == 0 ? x.w : a[3] + x.w;
          }
        }
      }
      // C += acc (rows / columns outside the matrix dropped).  Loads of C for
      // four rows are issued before their stores (the compiler cannot see
      // that runtime strides keep the rows apart).
      float* Ct = C;
      const int64_t rs = rsc, cs = csc;
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
              cv[i][h] = (vec && m < M && n + 4 <= N)
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
                    *cq += a4[q];
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
              old[j] = n < N ? crow[(int64_t)n * cs] : 0.f;
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
    // cluster pairs, odd CTA that stopped before the exchange: the even CTA
    // may still signal this CTA's barrier; leave only after its arrivals
    // landed (or the bound ran out)
    if (streamk == 2 && crank == 1 && !xwaited) {
      int never = 0;
      (void)mbar_wait_cluster_bounded(xfree, 0, &never, kWaitLimitNs);
    }
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
                         int64_t K, float* C, int64_t rsc, int64_t csc, int* err, cudaStream_t stream, int grid,
                         int streamk, int max_seg, float* slots, int* tile_cnt) {
  set_attributes(c);
  const int tiles_m = (int)((M + kBM - 1) / kBM), tiles_n = (int)((N + kBN - 1) / kBN);
  if (streamk == 2) {  // clusters of two CTAs (one tile per cluster)
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = kSmem;
    cfg.stream = stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    GB_CUDA_TRY(cudaLaunchKernelEx(&cfg, sgemm_tma_kernel<AK, BK>, ma, mb, (int)M, (int)N, (int)K, C, rsc, csc,
                                   tiles_m, tiles_n, streamk, max_seg, slots, tile_cnt, err));
  } else {
    sgemm_tma_kernel<AK, BK><<<(unsigned)grid, kThreads, kSmem, stream>>>(
        ma, mb, (int)M, (int)N, (int)K, C, rsc, csc, tiles_m, tiles_n, streamk, max_seg, slots, tile_cnt, err);
  }
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
                               int64_t csc, cudaStream_t stream, int max_ctas, int streamk) {
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
  const int64_t tiles = ((M + kBM - 1) / kBM) * ((N + kBN - 1) / kBN);
  const int64_t nk = (K + kBK - 1) / kBK;
  int64_t grid = c->num_sms;
  if (max_ctas > 0 && grid > max_ctas) grid = max_ctas;
  // cluster pairs need two CTAs per tile at once and two K blocks per tile;
  // otherwise stream-K
  if (streamk == 2 && (nk < 2 || 2 * tiles > grid)) streamk = 1;
  if (streamk == 2) grid = 2 * tiles;
  if (!streamk) grid = std::min<int64_t>(grid, tiles);
  grid = std::min<int64_t>(grid, tiles * nk);  // stream-K: every CTA gets at least one K block
  // stream-K: a tile meets at most (nk - 1) / L + 2 CTA ranges, L the shortest range
  const int64_t shortest = tiles * nk / grid;
  const int max_seg = streamk == 1 ? (int)((nk - 1) / shortest + 2) : 0;
  const size_t slot_bytes = streamk == 1 ? sizeof(float) * (size_t)kBM * kBN * (size_t)(tiles * max_seg) : 0;
  const size_t cnt_bytes = streamk == 1 ? sizeof(int) * (size_t)tiles : 0;
  void* s = nullptr;
  GB_TRY(get_scratch(c, stream, kScratchZeroBytes + slot_bytes + cnt_bytes, &s));
  int* err = reinterpret_cast<int*>(static_cast<char*>(s) + kErrWordOffset);
  float* slots = streamk == 1 ? reinterpret_cast<float*>(static_cast<char*>(s) + kScratchZeroBytes) : nullptr;
  int* tile_cnt =
      streamk == 1 ? reinterpret_cast<int*>(static_cast<char*>(s) + kScratchZeroBytes + slot_bytes) : nullptr;
  // the per-tile counts start at zero (the scratch is shared with other kernels on this stream)
  if (streamk == 1) GB_CUDA_TRY(cudaMemsetAsync(tile_cnt, 0, cnt_bytes, stream));
  const int g = (int)grid, sk = streamk;
  if (ak && bk) return launch_cfg<true, true>(c, ma, mb, M, N, K, C, rsc, csc, err, stream, g, sk, max_seg, slots, tile_cnt);
  if (ak) return launch_cfg<true, false>(c, ma, mb, M, N, K, C, rsc, csc, err, stream, g, sk, max_seg, slots, tile_cnt);
  if (bk) return launch_cfg<false, true>(c, ma, mb, M, N, K, C, rsc, csc, err, stream, g, sk, max_seg, slots, tile_cnt);
  return launch_cfg<false, false>(c, ma, mb, M, N, K, C, rsc, csc, err, stream, g, sk, max_seg, slots, tile_cnt);
}

bool sgemm_tma_pairs_useful(DeviceCtx* c, int64_t M, int64_t N, int64_t K) {
  const int64_t tiles = ((M + kBM - 1) / kBM) * ((N + kBN - 1) / kBN);
  const int64_t nk = (K + kBK - 1) / kBK;
  // two CTAs per tile fill at least half the SMs and fit in one wave
  return nk >= 8 && 2 * tiles <= c->num_sms && 4 * tiles >= c->num_sms;
}

bool sgemm_tma_streamk_useful(DeviceCtx* c, int64_t M, int64_t N, int64_t K) {
  const int64_t tiles = ((M + kBM - 1) / kBM) * ((N + kBN - 1) / kBN);
  const int64_t nk = (K + kBK - 1) / kBK;
  const int64_t sms = c->num_sms;
  // whole tiles leave part of the last wave idle, and there is K to share
  return nk >= 8 && tiles < 4 * sms && tiles % sms != 0 && tiles % sms < sms * 9 / 10;
}

}  // namespace gbblas
