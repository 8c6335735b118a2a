// dot.cu - streaming inner product (replaces amt::dot_prod).
//
// Reference: include/dot.hpp:143-174 picks one of three CPU regimes by size
// (serial SIMD below 2*L1, OpenMP-static L1/2 blocks below L3, L2/2 x L1/2
// two-level blocks above) and combines per-thread partials with an OpenMP
// reduction.  On the GPU one regime fits every size: a grid of
// (SMs x resident CTAs) threads streams both vectors once with 128-bit
// read-only loads, each thread keeps its own partial sums, CTAs reduce with
// warp shuffles, the CTAs of each thread-block cluster (kDotCluster CTAs)
// add their totals through distributed shared memory in rank order, and the
// last cluster to finish adds the per-cluster partials in index order.  The
// order of every addition is fixed by n and the grid size, so results are
// bit-reproducible run to run.
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
// CTAs per cluster; the grid is a multiple of it.  Measured at 2^28 elements:
// pairs stream as fast as unclustered CTAs (f32 0.303 ms, f64 0.629 vs 0.623),
// clusters of 4 / 8 lose 15-30 % of the bandwidth.
constexpr int kDotCluster = 2;

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
// partials[gridDim.x / kDotCluster] (FP64) and *counter live in scratch;
// with one cluster they are not touched.  No thread leaves before the two
// cluster barriers.
template <typename T, bool VEC>
__global__ void __launch_bounds__(kDotThreads, kDotCtasPerSm)
    dot_kernel(const T* __restrict__ a, const T* __restrict__ b, int64_t n, double* __restrict__ partials,
               unsigned* __restrict__ counter, T* __restrict__ result) {
  using V = typename Vec<T>::type;
  constexpr int W = Vec<T>::width;
  __shared__ double sh[32];
  __shared__ double cta_total;  // read by the cluster's rank 0
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

  const double block_total = dev::block_sum<double>(acc.total(), sh);

  // cluster step: rank 0 adds the cluster's CTA totals in rank order
  const unsigned csize = dev::cluster_size();
  double cluster_total = block_total;
  unsigned rank = 0;
  if (csize > 1) {
    if (threadIdx.x == 0) cta_total = block_total;
    dev::cluster_sync();
    rank = dev::cluster_rank();
    if (rank == 0 && threadIdx.x == 0) {
      cluster_total = dev::dsmem_ld(&cta_total, 0);
      for (unsigned r = 1; r < csize; ++r) cluster_total += dev::dsmem_ld(&cta_total, r);
    }
    dev::cluster_sync();  // the other CTAs stay resident until rank 0 has read them
    if (rank != 0) return;
  }

  const int nclusters = (int)(gridDim.x / csize);
  if (nclusters == 1) {
    if (threadIdx.x == 0) *result = (T)cluster_total;
    return;
  }
  if (threadIdx.x == 0) {
    partials[blockIdx.x / csize] = cluster_total;
    __threadfence();
    unsigned prev = atomicAdd(counter, 1u);
    is_last = (prev == (unsigned)nclusters - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  double t = 0.0;
  for (int i = threadIdx.x; i < nclusters; i += blockDim.x) t += __ldcg(partials + i);
  t = dev::block_sum<double>(t, sh);
  if (threadIdx.x == 0) {
    *result = (T)t;
    *counter = 0u;  // ready for the next call on this scratch
  }
}

// grid: a multiple of kDotCluster; clusters of kDotCluster CTAs.
template <typename T>
cudaError_t launch_dot_kernel(bool vec, int grid, cudaStream_t stream, const T* a, const T* b, int64_t n,
                              double* partials, unsigned* counter, T* result) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(kDotThreads);
  cfg.stream = stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kDotCluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = kDotCluster > 1 ? 1 : 0;
  return vec ? cudaLaunchKernelEx(&cfg, dot_kernel<T, true>, a, b, n, partials, counter, result)
             : cudaLaunchKernelEx(&cfg, dot_kernel<T, false>, a, b, n, partials, counter, result);
}

}  // namespace

template <typename T>
gbblas_status launch_dot(DeviceCtx* c, int64_t n, const T* a, const T* b, T* result, cudaStream_t stream) {
  const bool vec = aligned16(a) && aligned16(b);
  const int64_t per_cta = (int64_t)kDotThreads * kDotUnroll * Vec<T>::width;
  int64_t want = (n + per_cta - 1) / per_cta;
  const int64_t full = (int64_t)c->num_sms * kDotCtasPerSm;
  int grid = (int)(want < full ? (want < 1 ? 1 : want) : full);
  grid = (grid + kDotCluster - 1) / kDotCluster * kDotCluster;  // whole clusters
  double* partials = nullptr;
  unsigned* counter = nullptr;
  if (grid > kDotCluster) {
    void* s = nullptr;
    GB_TRY(get_scratch(c, stream, kScratchZeroBytes + sizeof(double) * (grid / kDotCluster), &s));
    counter = reinterpret_cast<unsigned*>(s);
    partials = reinterpret_cast<double*>(static_cast<char*>(s) + kScratchZeroBytes);
  }
  GB_CUDA_TRY(launch_dot_kernel<T>(vec, grid, stream, a, b, n, partials, counter, result));
  return check_launch("dot_kernel");
}

template gbblas_status launch_dot<float>(DeviceCtx*, int64_t, const float*, const float*, float*, cudaStream_t);
template gbblas_status launch_dot<double>(DeviceCtx*, int64_t, const double*, const double*, double*,
                                          cudaStream_t);

// ------------------------------------------------------------------------
// Allocation-free single-precision dot (gbblas_sdot_noalloc).
//
// Some callers cannot allocate device memory at call time: code running
// under an allocator that forbids it (a caller-managed memory pool or a
// real-time/serving loop that pre-reserves everything), or a host language
// binding that cannot reach cudaMalloc.  For them the dot's reduction
// scratch - the per-CTA FP64 partials and the completion counter that
// gbblas_sdot takes from its per-stream pool - lives in one fixed device
// array defined in this file instead.  Every GPU that loads the library
// holds this array until the process exits.
namespace {

// Maximum number of per-CTA partials the array holds.  The dot grid is
// (SMs x kDotCtasPerSm) CTAs at most: 608 on a 152-SM GB300.
constexpr int kNoAllocMaxCtas = 4096;
constexpr size_t kNoAllocBytes = kScratchZeroBytes + sizeof(double) * kNoAllocMaxCtas;  // 33,024 bytes

// The scratch itself.  In host code `g_noalloc_scratch` names a host-side
// stand-in, not device memory: its device address comes from
// cudaGetSymbolAddress below and only that address is passed to kernels.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

struct NoAllocDev {
  bool ready = false;
  int num_sms = 0;
  void* scratch = nullptr;  // device address of g_noalloc_scratch on this device
};
constexpr int kNoAllocMaxDevices = 64;
NoAllocDev g_noalloc_dev[kNoAllocMaxDevices];
std::mutex g_noalloc_mu;

// Once per device, with that device current: check it is sm_103 and look up
// the device address of the scratch array.  Allocates nothing.
gbblas_status noalloc_setup(NoAllocDev** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) {
    set_error("gbblas_sdot_noalloc: no usable CUDA device: %s", cudaGetErrorString(e));
    return GBBLAS_STATUS_NO_DEVICE;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  NoAllocDev& d = g_noalloc_dev[dev];
  if (!d.ready) {
    int major = 0, minor = 0, sms = 0;
    GB_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    GB_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    GB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (!(major == 10 && minor == 3)) {
      set_error("gbblas_sdot_noalloc: device %d is sm_%d%d, not sm_103", dev, major, minor);
      return GBBLAS_STATUS_NO_DEVICE;
    }
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || ptr == nullptr) {
      set_error("gbblas_sdot_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return GBBLAS_STATUS_CUDA_ERROR;
    }
    d.num_sms = sms;
    d.scratch = ptr;
    d.ready = true;
  }
  *out = &d;
  return GBBLAS_STATUS_SUCCESS;
}

}  // namespace
}  // namespace gbblas

extern "C" gbblas_status gbblas_sdot_noalloc(int64_t n, const float* a, const float* b, float* result,
                                             void* stream) {
  using namespace gbblas;
  if (n < 0) {
    set_error("gbblas_sdot_noalloc: negative size");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  if (!result || (n > 0 && (!a || !b))) {
    set_error("gbblas_sdot_noalloc: null pointer");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  NoAllocDev* d = nullptr;
  GB_TRY(noalloc_setup(&d));
  cudaStream_t s = as_stream(stream);
  const bool vec = aligned16(a) && aligned16(b);
  const int64_t per_cta = (int64_t)kDotThreads * kDotUnroll * 4;
  const int64_t want = (n + per_cta - 1) / per_cta;
  const int64_t full = (int64_t)d->num_sms * kDotCtasPerSm;
  int64_t grid = want < full ? (want < 1 ? 1 : want) : full;
  grid = (grid + kDotCluster - 1) / kDotCluster * kDotCluster;  // whole clusters
  if (grid > kNoAllocMaxCtas) {
    set_error("gbblas_sdot_noalloc: needs %lld reduction slots, the fixed scratch holds %d",
              (long long)grid, kNoAllocMaxCtas);
    return GBBLAS_STATUS_NOT_SUPPORTED;
  }
  unsigned* counter = static_cast<unsigned*>(d->scratch);
  double* partials = reinterpret_cast<double*>(static_cast<char*>(d->scratch) + kScratchZeroBytes);
  // The counter must start at zero; partials are fully rewritten by each call.
  GB_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned), s));
  GB_CUDA_TRY(launch_dot_kernel<float>(vec, (int)grid, s, a, b, n, partials, counter, result));
  return check_launch("dot_kernel (noalloc)");
}
