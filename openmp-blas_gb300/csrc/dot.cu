// dot.cu - streaming inner product (replaces amt::dot_prod).
//
// Reference: include/dot.hpp:143-174 picks one of three CPU regimes by size
// (serial SIMD below 2*L1, OpenMP-static L1/2 blocks below L3, L2/2 x L1/2
// two-level blocks above) and combines per-thread partials with an OpenMP
// reduction.  On the GPU one regime fits every size: a grid of
// (SMs x resident CTAs) threads streams both vectors once with 128-bit
// read-only loads, each thread keeps its own partial sums, CTAs reduce with
// warp shuffles, and the last CTA to finish adds the per-CTA partials in
// index order.  The order of every addition is fixed by n and the grid size,
// so results are bit-reproducible run to run.
//
// Accuracy: FP32 partials are Kahan-compensated (products and sums rounded
// with __fmul_rn / __fadd_rn so the compiler cannot contract them into FMAs
// and lose the compensation) and are combined in FP64; FP64 dots use plain
// FMA partials.  Roofline: HBM bandwidth, 2*n*sizeof(T) bytes per call.
#include "common.cuh"

namespace gbblas {
namespace {

constexpr int kDotThreads = 256;
constexpr int kDotCtasPerSm = 4;  // 1024 threads/SM, <= 64 registers each
constexpr int kDotUnroll = 4;

// Per-thread accumulator.  FP32: four Kahan lanes.  FP64: four FMA lanes.
template <typename T>
struct DotAcc;

template <>
struct DotAcc<float> {
  float s[4] = {0.f, 0.f, 0.f, 0.f};
  float c[4] = {0.f, 0.f, 0.f, 0.f};
  __device__ __forceinline__ void add(int lane, float a, float b) {
    float p = __fmul_rn(a, b);
    float y = __fsub_rn(p, c[lane]);
    float t = __fadd_rn(s[lane], y);
    c[lane] = __fsub_rn(__fsub_rn(t, s[lane]), y);
    s[lane] = t;
  }
  __device__ __forceinline__ void add4(float4 a, float4 b) {
    add(0, a.x, b.x);
    add(1, a.y, b.y);
    add(2, a.z, b.z);
    add(3, a.w, b.w);
  }
  __device__ __forceinline__ double total() const {
    return (((double)s[0] - (double)c[0]) + ((double)s[1] - (double)c[1])) +
           (((double)s[2] - (double)c[2]) + ((double)s[3] - (double)c[3]));
  }
};

template <>
struct DotAcc<double> {
  double s[4] = {0., 0., 0., 0.};
  __device__ __forceinline__ void add(int lane, double a, double b) { s[lane] = fma(a, b, s[lane]); }
  __device__ __forceinline__ void add4(double2 a, double2 b, int pair) {
    add(2 * pair, a.x, b.x);
    add(2 * pair + 1, a.y, b.y);
  }
  __device__ __forceinline__ double total() const { return (s[0] + s[1]) + (s[2] + s[3]); }
};

template <typename T>
struct Vec;
template <>
struct Vec<float> {
  using type = float4;
  static constexpr int width = 4;
};
template <>
struct Vec<double> {
  using type = double2;
  static constexpr int width = 2;
};

template <typename T>
__device__ __forceinline__ void acc_vec(DotAcc<T>& acc, typename Vec<T>::type a, typename Vec<T>::type b,
                                        int u);
template <>
__device__ __forceinline__ void acc_vec<float>(DotAcc<float>& acc, float4 a, float4 b, int) {
  acc.add4(a, b);
}
template <>
__device__ __forceinline__ void acc_vec<double>(DotAcc<double>& acc, double2 a, double2 b, int u) {
  acc.add4(a, b, u & 1);
}

// One pass over a[0:n) . b[0:n).  VEC: both pointers 16-byte aligned.
// partials[gridDim.x] (FP64) and *counter live in scratch; with one CTA
// they are not touched.
template <typename T, bool VEC>
__global__ void __launch_bounds__(kDotThreads, kDotCtasPerSm) dot_kernel(const T* __restrict__ a, const T* __restrict__ b,
                                                          int64_t n, double* __restrict__ partials,
                                                          unsigned* __restrict__ counter, T* __restrict__ result) {
  using V = typename Vec<T>::type;
  constexpr int W = Vec<T>::width;
  __shared__ double sh[32];
  __shared__ bool is_last;

  DotAcc<T> acc;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  int64_t tail_start = 0;
  if (VEC) {
    const V* a4 = reinterpret_cast<const V*>(a);
    const V* b4 = reinterpret_cast<const V*>(b);
    const int64_t nv = n / W;
    int64_t i = tid;
    for (; i + (kDotUnroll - 1) * nthr < nv; i += kDotUnroll * nthr) {
      V va[kDotUnroll], vb[kDotUnroll];
#pragma unroll
      for (int u = 0; u < kDotUnroll; ++u) {
        va[u] = dev::ld_stream(a4 + i + u * nthr);
        vb[u] = dev::ld_stream(b4 + i + u * nthr);
      }
#pragma unroll
      for (int u = 0; u < kDotUnroll; ++u) acc_vec<T>(acc, va[u], vb[u], u);
    }
    for (; i < nv; i += nthr) acc_vec<T>(acc, dev::ld_stream(a4 + i), dev::ld_stream(b4 + i), 0);
    tail_start = nv * W;
  }
  for (int64_t i = tail_start + tid; i < n; i += nthr) acc.add(0, dev::ld_stream(a + i), dev::ld_stream(b + i));

  double block_total = dev::block_sum<double>(acc.total(), sh);

  if (gridDim.x == 1) {
    if (threadIdx.x == 0) *result = (T)block_total;
    return;
  }
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = block_total;
    __threadfence();
    unsigned prev = atomicAdd(counter, 1u);
    is_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  double t = 0.0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) t += __ldcg(partials + i);
  t = dev::block_sum<double>(t, sh);
  if (threadIdx.x == 0) {
    *result = (T)t;
    *counter = 0u;  // ready for the next call on this scratch
  }
}

}  // namespace

template <typename T>
gbblas_status launch_dot(DeviceCtx* c, int64_t n, const T* a, const T* b, T* result, cudaStream_t stream) {
  const bool vec = aligned16(a) && aligned16(b);
  const int64_t per_cta = (int64_t)kDotThreads * kDotUnroll * Vec<T>::width;
  int64_t want = (n + per_cta - 1) / per_cta;
  const int64_t full = (int64_t)c->num_sms * kDotCtasPerSm;
  int grid = (int)(want < full ? (want < 1 ? 1 : want) : full);
  double* partials = nullptr;
  unsigned* counter = nullptr;
  if (grid > 1) {
    void* s = nullptr;
    GB_TRY(get_scratch(c, stream, kScratchZeroBytes + sizeof(double) * grid, &s));
    counter = reinterpret_cast<unsigned*>(s);
    partials = reinterpret_cast<double*>(static_cast<char*>(s) + kScratchZeroBytes);
  }
  if (vec)
    dot_kernel<T, true><<<grid, kDotThreads, 0, stream>>>(a, b, n, partials, counter, result);
  else
    dot_kernel<T, false><<<grid, kDotThreads, 0, stream>>>(a, b, n, partials, counter, result);
  return check_launch("dot_kernel");
}

template gbblas_status launch_dot<float>(DeviceCtx*, int64_t, const float*, const float*, float*, cudaStream_t);
template gbblas_status launch_dot<double>(DeviceCtx*, int64_t, const double*, const double*, double*,
                                          cudaStream_t);

}  // namespace gbblas
