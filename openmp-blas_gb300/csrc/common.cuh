// common.cuh - shared host/device plumbing for the gbblas CUDA library.
//
// Host side: per-device context (SM count, per-stream scratch for the
// deterministic two-stage reductions, the staging area used by the *_host
// entry points), error bookkeeping and status helpers.
// Device side: cache-hinted vector loads and warp/block reductions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <unordered_map>

#include "../../include/gbblas.h"

namespace gbblas {

// ---------------------------------------------------------------- errors

void set_error(const char* fmt, ...);
const char* last_error();

#define GB_CUDA_TRY(call)                                                                   \
  do {                                                                                      \
    cudaError_t _e = (call);                                                                \
    if (_e != cudaSuccess) {                                                                \
      ::gbblas::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e), __FILE__, \
                          __LINE__);                                                        \
      return GBBLAS_STATUS_CUDA_ERROR;                                                      \
    }                                                                                       \
  } while (0)

#define GB_TRY(expr)                                \
  do {                                              \
    gbblas_status _s = (expr);                      \
    if (_s != GBBLAS_STATUS_SUCCESS) return _s;     \
  } while (0)

// Count of kernels launched by the library (gbblas_kernel_launches()).
void count_launch();

// Check the launch that was just issued (and count it).
inline gbblas_status check_launch(const char* what) {
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("launch of %s failed: %s", what, cudaGetErrorString(e));
    return GBBLAS_STATUS_CUDA_ERROR;
  }
  return GBBLAS_STATUS_SUCCESS;
}

// --------------------------------------------------------------- context

// One per device.  Scratch buffers are per stream so concurrent calls on
// different streams never share one; growth is stream-ordered
// (cudaMallocAsync / cudaFreeAsync on the owning stream).
struct DeviceCtx {
  int device = -1;
  int num_sms = 0;
  int cc_major = 0, cc_minor = 0;
  size_t smem_optin = 0;
  // cudaDevAttrPageableMemoryAccess: the device reads pageable host memory
  // coherently (through the host's page tables on a Grace-coupled GPU)
  int pageable_access = 0;
  std::mutex mu;
  struct Scratch {
    void* ptr = nullptr;
    size_t bytes = 0;
  };
  std::unordered_map<cudaStream_t, Scratch> scratch;
  // *_host staging: one stream, one device arena, guarded by host_mu.
  std::mutex host_mu;
  cudaStream_t host_stream = nullptr;
  void* stage = nullptr;
  size_t stage_bytes = 0;
};

// Context of the current device, created on first use.  Fails with
// GBBLAS_STATUS_NO_DEVICE when no device is visible or it is not sm_103.
gbblas_status get_ctx(DeviceCtx** out);

// Scratch of at least `bytes` for `stream`.  The first kScratchZeroBytes of a
// fresh buffer are zeroed on the stream (reduction kernels keep their
// completion counters there and return them to zero themselves).
constexpr size_t kScratchZeroBytes = 256;
// Byte offset, inside that zeroed header, of the stream's device error word:
// kernels with bounded waits store a gbblas_status there when a wait gives up.
constexpr size_t kErrWordOffset = 64;
// Byte offset of the persistent kernels' tile counter (reset before each launch).
constexpr size_t kTileCounterOffset = 128;
// Byte offset of the FP16 split guard's two list counts (reset before each launch).
constexpr size_t kGuardCountOffset = 136;
gbblas_status get_scratch(DeviceCtx* c, cudaStream_t stream, size_t bytes, void** out);

// Free the scratch of `stream` (stream-ordered) and forget it.
void release_scratch(DeviceCtx* c, cudaStream_t stream);

// Staging arena of at least `bytes` for the *_host paths (caller holds host_mu).
gbblas_status get_stage(DeviceCtx* c, size_t bytes, void** out);

// Address at which this library's kernels may read the host buffer `p`
// directly (over the host link, no staging copy), or nullptr when it must be
// staged: page-locked memory (cudaHostAlloc / cudaHostRegister) through its
// mapped device address, device or managed memory as it is, pageable memory
// only on a device that reads it coherently.  GBBLAS_HOST_DIRECT=0 turns
// direct reads off (every host operand is then staged).
const void* host_read_view(DeviceCtx* c, const void* p);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// ------------------------------------------------------ kernel launchers
// (defined in the kernel translation units; all asynchronous on `stream`)

// y[r] (+)= sum_c A[r*lda + c] * x[c] for r < rows, c < cols
// (every output is a dot of a contiguous row with x).
template <typename T>
gbblas_status launch_gemv_rows(DeviceCtx* c, int64_t rows, int64_t cols, const T* A, int64_t lda,
                               const T* x, T* y, bool accumulate, cudaStream_t stream);

// y[r] (+)= sum_c A[r + c*lda] * x[c] (columns contiguous: axpy form).
template <typename T>
gbblas_status launch_gemv_cols(DeviceCtx* c, int64_t rows, int64_t cols, const T* A, int64_t lda,
                               const T* x, T* y, bool accumulate, cudaStream_t stream);

template <typename T>
gbblas_status launch_dot(DeviceCtx* c, int64_t n, const T* a, const T* b, T* result, cudaStream_t stream);

// max_ctas > 0 caps the grid (the kernel loops over tiles), leaving SMs to
// other streams.
// tile (FP32 only): 3 = TMA-fed, stream-K (K blocks shared out equally among the SMs),
// 2 = TMA-fed 128 x 128 kernel (gemm_fma_tma.cu; where
// sgemm_tma_eligible), 1 = 128 x 128 CTA tiles, 0 = 64 x 64, -1 = by the
// tile count (TMA-fed for a row-major B once the 128 x 128 tiles fill the
// SMs, register-staged 128 x 128 from twice that, else 64 x 64).
template <typename T>
gbblas_status launch_gemm_fma(DeviceCtx* c, int64_t M, int64_t N, int64_t K, const T* A, int64_t rsa,
                              int64_t csa, const T* B, int64_t rsb, int64_t csb, T* C, int64_t rsc,
                              int64_t csc, cudaStream_t stream, int max_ctas = 0, int tile = -1);

// FP32 C += A*B on the FMA pipes with TMA-fed operands (gemm_fma_tma.cu):
// A and B each row- or column-major, 16-byte aligned, row / column pitch a
// multiple of 4 elements.
bool sgemm_tma_eligible(int64_t M, int64_t N, int64_t K, const float* A, int64_t rsa, int64_t csa, const float* B,
                        int64_t rsb, int64_t csb);
void sgemm_tma_prepare(DeviceCtx* c);  // kernel attributes, before any stream capture
// streamk = 1: the tiles' K blocks shared out equally among the CTAs
// (stream-K; sgemm_tma_streamk_useful says where whole tiles fill the SMs
// badly enough for it to be worth trying); 2: clusters of two CTAs, each
// with half of one tile's K blocks, adding through distributed shared
// memory (sgemm_tma_pairs_useful: where two CTAs per tile fill the SMs in
// one wave; stream-K where they cannot).
gbblas_status launch_sgemm_tma(DeviceCtx* c, int64_t M, int64_t N, int64_t K, const float* A, int64_t rsa,
                               int64_t csa, const float* B, int64_t rsb, int64_t csb, float* C, int64_t rsc,
                               int64_t csc, cudaStream_t stream, int max_ctas = 0, int streamk = 0);
bool sgemm_tma_streamk_useful(DeviceCtx* c, int64_t M, int64_t N, int64_t K);
bool sgemm_tma_pairs_useful(DeviceCtx* c, int64_t M, int64_t N, int64_t K);

// C += A*B on the tcgen05 tensor cores (gemm_tc.cu).  mode = tc_mode(acc):
// 2 / 3 = FP32 operands split into that many BF16 pieces, 8 = FP8-E4M3 with
// per-128-K-block power-of-two scales; 0 = not a tensor-core accuracy.
int tc_mode(gbblas_accuracy acc);
// The tensor-core mode GBBLAS_ACCURACY_AUTO takes for a single float GEMM:
// the FP16 split with its guard (rows of A / columns of B whose magnitudes
// span more binades than the split's error bound allows are recomputed with
// FP32 FMAs).
constexpr int kTcModeF16Guard = 13;
// Device bytes of the operand arena one problem needs in `mode`.
size_t tc_arena_bytes(int mode, int64_t M, int64_t N, int64_t K);

// K stage depth of the tensor-core kernel in `mode` (K is padded to it).
int tc_stage_k(int mode);

// Shape of one tensor-core launch: split = K parts per problem (split-K:
// each part a tile problem of its own writing a partial, the parts then
// added into C in order; 1 = none), pair = CTA form for the split-BF16
// modes (-1 = the GBBLAS_TC_PAIR setting, 0 = single CTAs, 1 = CTA pairs).
struct TcLaunchOpts {
  int split = 1;
  int pair = -1;
};

// One problem with the autotuner's launch shape for it.
gbblas_status launch_gemm_tc(DeviceCtx* c, int mode, int64_t M, int64_t N, int64_t K, const float* A, int64_t rsa,
                             int64_t csa, const float* B, int64_t rsb, int64_t csb, float* C, int64_t rsc,
                             int64_t csc, cudaStream_t stream);
// One problem with a given launch shape.
gbblas_status launch_gemm_tc_opts(DeviceCtx* c, int mode, const gbblas_gemm_desc& d, const TcLaunchOpts& opt,
                                  cudaStream_t stream);

// The same for a group of independent problems in one persistent launch
// (tables and operand arena in the stream's scratch).
// slices > 1: the GEMM kernel as that many launches over consecutive ranges
// of whole waves of tiles, so that higher-priority streams get SMs between
// them (the serving loop's heavy requests); the same bits.
gbblas_status launch_gemm_tc_group(DeviceCtx* c, int mode, const gbblas_gemm_desc* descs, int64_t count,
                                   cudaStream_t stream, int max_ctas = 0, int slices = 1);

// A group bound to its own device memory, for repeated (graph-captured)
// launches: create uploads the tables once; launch only enqueues kernels.
struct TcGroupPlan;
gbblas_status tc_group_create(DeviceCtx* c, int mode, const gbblas_gemm_desc* descs, int64_t count,
                              TcGroupPlan** out);
gbblas_status tc_group_launch(DeviceCtx* c, const TcGroupPlan* plan, cudaStream_t stream, int max_ctas = 0,
                              int slices = 1);
// GBBLAS_GEMM_SLICES=n (n > 1): single tensor-core and digit GEMMs run as n
// launches over tile ranges (what the serving loop does with heavy requests).
int gemm_slices_env();
void tc_group_destroy(TcGroupPlan* plan);
int* tc_group_error_word(const TcGroupPlan* plan);

// Set the tensor-core kernels' launch attributes (before any stream capture).
void tc_prepare(DeviceCtx* c);

// Double-precision GEMM on the BF16 tensor cores (Ozaki scheme, 7 or 8
// digits per element; gemm_f64_tc.cu): C += A * B.  guarded (7 digits):
// every 32 x 16 output block whose digit error could exceed the FP64 pipes'
// bound is recomputed on the FP64 pipes.  The digit count of an accuracy (0
// if it is not a digit mode), the longest K a digit count takes, and the
// kernels' launch attributes (set by tc_prepare).
int dgemm_digits_count(gbblas_accuracy acc);
int64_t dgemm_digits_max_k(int digits);
size_t dgemm_digits_scratch_bytes(int digits, bool guarded, int64_t M, int64_t N, int64_t K);
// AUTO for a double GEMM: the guarded digits for this shape (else the FP64 pipes).
bool dgemm_auto_digits(int64_t M, int64_t N, int64_t K, int num_sms);
void dgemm_digits_prepare(DeviceCtx* c);
gbblas_status launch_dgemm_digits(DeviceCtx* c, int digits, bool guarded, int64_t M, int64_t N, int64_t K,
                                  const double* A, int64_t rsa, int64_t csa, const double* B, int64_t rsb,
                                  int64_t csb, double* C, int64_t rsc, int64_t csc, cudaStream_t stream,
                                  int max_ctas = 0, int slices = 1);

// Grouped GEMV: row-streaming problems in one persistent launch, the rest
// per problem (batch.cu).
gbblas_status launch_gemv_group(DeviceCtx* c, const gbblas_gemv_desc* d, int64_t count, cudaStream_t s);

// Autotuner (tune.cu): AUTO accuracy -> 1 = the guarded FP16 split (kTcModeF16Guard), 0 = FMA.
int tuned_gemm_auto(DeviceCtx* c, int64_t M, int64_t N, int64_t K);
// Autotuner: split-K parts and CTA form of one tensor-core GEMM.
TcLaunchOpts tuned_tc_opts(DeviceCtx* c, int mode, int64_t M, int64_t N, int64_t K, cudaStream_t stream);
// Autotuner: FP32 FMA tile (launch_gemm_fma's `tile`).
int tuned_fma_tile(DeviceCtx* c, int64_t M, int64_t N, int64_t K, cudaStream_t stream);

// Streaming operations beside the hot path (stream_ops.cu).
// C[r*ld + l] += u[r] * v[l] (rows of C contiguous).
template <typename T>
gbblas_status launch_outer(DeviceCtx* c, int64_t R, int64_t L, const T* u, const T* v, T* C, int64_t ld,
                           cudaStream_t s);
// C(j, i) = A(i, j): A(i, j) at A[i*rsa + j*csa], C(j, i) at C[j*rsc + i*csc].
template <typename T>
gbblas_status launch_transpose(DeviceCtx* c, int64_t M, int64_t N, const T* A, int64_t rsa, int64_t csa, T* C,
                               int64_t rsc, int64_t csc, cudaStream_t s);
// Square n x n storage transposed in place.
template <typename T>
gbblas_status launch_transpose_square(DeviceCtx* c, int64_t n, T* A, cudaStream_t s);
// out[i] = a[i] op b[i].
template <typename T>
gbblas_status launch_ew(DeviceCtx* c, gbblas_ew_op op, int64_t n, const T* a, const T* b, T* out, cudaStream_t s);

// Synchronise `stream` and report (then clear) any device-side error its
// kernels recorded in the stream's scratch error word.
gbblas_status check_stream_errors(DeviceCtx* c, cudaStream_t stream);

}  // namespace gbblas

// ----------------------------------------------------------- device helpers
#ifdef __CUDACC__
namespace gbblas::dev {

// Streaming loads: read-only path, no L1 allocation (data is used once).
__device__ __forceinline__ float4 ld_stream(const float4* p) {
  float4 r;
  asm volatile("ld.global.nc.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
               : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
               : "l"(p));
  return r;
}
__device__ __forceinline__ double2 ld_stream(const double2* p) {
  double2 r;
  asm volatile("ld.global.nc.L1::no_allocate.v2.f64 {%0,%1}, [%2];" : "=d"(r.x), "=d"(r.y) : "l"(p));
  return r;
}
__device__ __forceinline__ float ld_stream(const float* p) {
  float r;
  asm volatile("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(r) : "l"(p));
  return r;
}
__device__ __forceinline__ double ld_stream(const double* p) {
  double r;
  asm volatile("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(r) : "l"(p));
  return r;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the block in a fixed order (deterministic).  `sh` holds >= 32 T.
// Every thread gets the total.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  T t = lane < nwarps ? sh[lane] : T(0);
  t = warp_sum(t);
  return t;
}

// ---- thread-block clusters (distributed shared memory)
// CTAs in this CTA's cluster (1 for a launch without clusters).
__device__ __forceinline__ unsigned cluster_size() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
// Rank of this CTA in its cluster.
__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// Barrier over every thread of every CTA of the cluster (release / acquire:
// shared-memory writes before it are visible to the cluster's CTAs after).
// Each thread must reach it: kernels that use it exit no thread early.
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// Load the object at shared address `p` of this CTA as it sits in the shared
// memory of CTA `rank` of the cluster.
__device__ __forceinline__ double dsmem_ld(const double* p, unsigned rank) {
  unsigned a = (unsigned)__cvta_generic_to_shared(p), r;
  double v;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(r) : "memory");
  return v;
}
__device__ __forceinline__ float dsmem_ld(const float* p, unsigned rank) {
  unsigned a = (unsigned)__cvta_generic_to_shared(p), r;
  float v;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(r) : "memory");
  return v;
}

}  // namespace gbblas::dev
#endif
