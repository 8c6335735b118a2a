// gemv.cu - matrix x vector kernels behind amt::mtv and amt::vtm.
//
// Two access shapes cover both layouts and both products:
//
//   gemv_rows  every output is the dot of one CONTIGUOUS row with x:
//              y[r] (+)= sum_c A[r*lda + c] * x[c].
//              mtv with row-major A (reference include/mtv.hpp:72-98,
//              simd_loop.hpp:21-35, overwrites y) and vtm with column-major
//              A (columns of A are the contiguous rows of A^T).
//   gemv_cols  the axpy form over CONTIGUOUS columns:
//              y[r] (+)= sum_c A[r + c*lda] * x[c].
//              mtv with column-major A (reference include/mtv.hpp:15-70,
//              simd_loop.hpp:52-78, accumulates into y) and vtm with
//              row-major A.
//
// Both stream A from HBM exactly once with 128-bit read-only loads and keep
// x in L1/L2.  When the grid would be too small to fill the 152 SMs the
// reduction dimension is split across CTAs.  Two splits, or up to 8 on a
// small matrix, run as one thread-block cluster per row block: each CTA
// leaves its partials in its shared memory and the cluster's rank 0 adds
// them in split order through distributed shared memory.  Otherwise the
// partials go to per-stream scratch and a second small kernel adds them in
// split order.  Either way
// the additions are in the same order and deterministic (no atomics).
// Roofline: HBM, (rows*cols + rows + cols) * sizeof(T) bytes per call.
#include <utility>

#include "common.cuh"

namespace gbblas {
namespace {

template <typename T>
struct V;
template <>
struct V<float> {
  using t = float4;
  static constexpr int w = 4;
};
template <>
struct V<double> {
  using t = double2;
  static constexpr int w = 2;
};

__device__ __forceinline__ float vdot(float4 a, float4 b, float acc) {
  acc = fmaf(a.x, b.x, acc);
  acc = fmaf(a.y, b.y, acc);
  acc = fmaf(a.z, b.z, acc);
  return fmaf(a.w, b.w, acc);
}
__device__ __forceinline__ double vdot(double2 a, double2 b, double acc) {
  acc = fma(a.x, b.x, acc);
  return fma(a.y, b.y, acc);
}
__device__ __forceinline__ float4 ldg_vec(const float4* p) { return __ldg(p); }
__device__ __forceinline__ double2 ldg_vec(const double2* p) { return __ldg(p); }

constexpr int kRowsThreads = 256;

constexpr int kMaxClusterSplits = 8;  // portable cluster size

// Whether the ksplit CTAs of a row block reduce as one cluster.  Measured on
// split shapes: clusters of two stream as fast as separate CTAs; up to 8 pay
// off while the matrix is small (12-60 MB: 17-24 % faster, the second launch
// saved); on large matrices clusters of 3-4 lose up to 17 % of the bandwidth.
inline bool cluster_splits(int64_t ksplit, int64_t rows, int64_t cols, size_t elem) {
  return ksplit >= 2 && ksplit <= kMaxClusterSplits && (ksplit == 2 || (double)rows * cols * elem <= 64.0e6);
}

// grid = (ceil(rows / R), ksplit); CTA = 8 warps splitting its column range.
// CL: the ksplit CTAs of a row block form a cluster (1, ksplit, 1).
template <typename T, int R, bool VEC, bool CL>
__global__ void __launch_bounds__(kRowsThreads) gemv_rows_kernel(int64_t rows, int64_t cols,
                                                                 const T* __restrict__ A, int64_t lda,
                                                                 const T* __restrict__ x, T* __restrict__ y,
                                                                 bool accumulate, T* __restrict__ partials,
                                                                 int64_t cols_per_split) {
  using VT = typename V<T>::t;
  constexpr int W = V<T>::w;
  __shared__ T red[kRowsThreads / 32][R];
  __shared__ T split_part[R];  // CL: this split's row sums, read by the cluster's rank 0
  const int64_t r0 = (int64_t)blockIdx.x * R;
  const int64_t c0 = (int64_t)blockIdx.y * cols_per_split;
  int64_t c1 = c0 + cols_per_split;
  if (c1 > cols) c1 = cols;
  const int nr = (int)((rows - r0) < R ? (rows - r0) : R);

  T acc[R];
#pragma unroll
  for (int r = 0; r < R; ++r) acc[r] = T(0);

  int64_t scalar_from = c0;
  if (VEC) {
    const int64_t v0 = c0 / W, v1 = c1 / W;  // c0 is a multiple of W
    const VT* xv = reinterpret_cast<const VT*>(x);
    int64_t v = v0 + threadIdx.x;
    if (nr == R) {
      for (; v + kRowsThreads < v1; v += 2 * kRowsThreads) {
        VT xa = ldg_vec(xv + v), xb = ldg_vec(xv + v + kRowsThreads);
        VT aa[R], ab[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const VT* row = reinterpret_cast<const VT*>(A + (r0 + r) * lda);
          aa[r] = dev::ld_stream(row + v);
          ab[r] = dev::ld_stream(row + v + kRowsThreads);
        }
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r] = vdot(ab[r], xb, vdot(aa[r], xa, acc[r]));
      }
    }
    for (; v < v1; v += kRowsThreads) {
      VT xa = ldg_vec(xv + v);
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (r < nr) acc[r] = vdot(dev::ld_stream(reinterpret_cast<const VT*>(A + (r0 + r) * lda) + v), xa, acc[r]);
    }
    scalar_from = v1 * W;
  }
  for (int64_t c = scalar_from + threadIdx.x; c < c1; c += kRowsThreads) {
    T xc = __ldg(x + c);
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (r < nr) acc[r] = fma(dev::ld_stream(A + (r0 + r) * lda + c), xc, acc[r]);
  }

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    T s = dev::warp_sum(acc[r]);
    if (lane == 0) red[warp][r] = s;
  }
  __syncthreads();
  if (threadIdx.x < nr) {
    const int r = threadIdx.x;
    T s = T(0);
#pragma unroll
    for (int w = 0; w < kRowsThreads / 32; ++w) s += red[w][r];
    if (CL) {
      split_part[r] = s;
    } else if (gridDim.y == 1) {
      y[r0 + r] = accumulate ? y[r0 + r] + s : s;
    } else {
      partials[(int64_t)blockIdx.y * rows + r0 + r] = s;
    }
  }
  if constexpr (CL) {
    dev::cluster_sync();
    if (blockIdx.y == 0 && threadIdx.x < nr) {  // rank 0 of the cluster: splits in order
      const int r = threadIdx.x;
      T s = T(0);
      for (unsigned k = 0; k < gridDim.y; ++k) s += dev::dsmem_ld(&split_part[r], k);
      y[r0 + r] = accumulate ? y[r0 + r] + s : s;
    }
    dev::cluster_sync();  // the other splits stay resident until rank 0 has read them
  }
}

// y[r] = (accumulate ? y[r] : 0) + sum_s partials[s*rows + r], s in order.
template <typename T>
__global__ void finish_splits_kernel(int64_t rows, int ksplit, const T* __restrict__ partials, T* __restrict__ y,
                                     bool accumulate) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  T s = T(0);
  for (int k = 0; k < ksplit; ++k) s += partials[(int64_t)k * rows + r];
  y[r] = accumulate ? y[r] + s : s;
}

constexpr int kColsUnroll = 8;

// grid = (ceil(rows / (threads*W)), ksplit).  Each thread owns W (VEC) or 1
// consecutive rows and walks its CTA's column range.  CL: the ksplit CTAs of
// a row block form a cluster (1, ksplit, 1); no thread leaves early then.
template <typename T, bool VEC, bool CL>
__global__ void __launch_bounds__(256) gemv_cols_kernel(int64_t rows, int64_t cols, const T* __restrict__ A,
                                                        int64_t lda, const T* __restrict__ x, T* __restrict__ y,
                                                        bool accumulate, T* __restrict__ partials,
                                                        int64_t cols_per_split) {
  using VT = typename V<T>::t;
  constexpr int W = VEC ? V<T>::w : 1;
  __shared__ T split_part[CL ? 256 * W : 1];
  const int64_t rbase = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * W;
  if (!CL && rbase >= rows) return;
  const int64_t c0 = (int64_t)blockIdx.y * cols_per_split;
  int64_t c1 = c0 + cols_per_split;
  if (c1 > cols) c1 = cols;
  T acc[W];
#pragma unroll
  for (int i = 0; i < W; ++i) acc[i] = T(0);
  const bool full = rbase + W <= rows;
  if (rbase >= rows) {
    // CL only: nothing to add, but the thread still meets the cluster barriers
  } else if (VEC && full) {
    const T* base = A + rbase;
    int64_t c = c0;
    for (; c + kColsUnroll <= c1; c += kColsUnroll) {
      VT a[kColsUnroll];
      T xc[kColsUnroll];
#pragma unroll
      for (int u = 0; u < kColsUnroll; ++u) {
        a[u] = dev::ld_stream(reinterpret_cast<const VT*>(base + (c + u) * lda));
        xc[u] = __ldg(x + c + u);
      }
#pragma unroll
      for (int u = 0; u < kColsUnroll; ++u) {
        const T* av = reinterpret_cast<const T*>(&a[u]);
#pragma unroll
        for (int i = 0; i < W; ++i) acc[i] = fma(av[i], xc[u], acc[i]);
      }
    }
    for (; c < c1; ++c) {
      VT a = dev::ld_stream(reinterpret_cast<const VT*>(base + c * lda));
      T xc = __ldg(x + c);
      const T* av = reinterpret_cast<const T*>(&a);
#pragma unroll
      for (int i = 0; i < W; ++i) acc[i] = fma(av[i], xc, acc[i]);
    }
  } else {
    for (int64_t c = c0; c < c1; ++c) {
      T xc = __ldg(x + c);
#pragma unroll
      for (int i = 0; i < W; ++i)
        if (rbase + i < rows) acc[i] = fma(dev::ld_stream(A + rbase + i + c * lda), xc, acc[i]);
    }
  }
  if constexpr (CL) {
#pragma unroll
    for (int i = 0; i < W; ++i) split_part[threadIdx.x * W + i] = acc[i];
    __syncwarp();  // lanes past the last row rejoin before the aligned cluster barrier
    dev::cluster_sync();
    if (blockIdx.y == 0) {  // rank 0 of the cluster: splits in order
#pragma unroll
      for (int i = 0; i < W; ++i) {
        const int64_t r = rbase + i;
        if (r < rows) {
          T s = T(0);
          for (unsigned k = 0; k < gridDim.y; ++k) s += dev::dsmem_ld(&split_part[threadIdx.x * W + i], k);
          y[r] = accumulate ? y[r] + s : s;
        }
      }
    }
    dev::cluster_sync();  // the other splits stay resident until rank 0 has read them
  } else {
#pragma unroll
    for (int i = 0; i < W; ++i) {
      const int64_t r = rbase + i;
      if (r < rows) {
        if (gridDim.y == 1)
          y[r] = accumulate ? y[r] + acc[i] : acc[i];
        else
          partials[(int64_t)blockIdx.y * rows + r] = acc[i];
      }
    }
  }
}

inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Launch with clusters of (1, grid.y, 1): the splits of one row block.
template <typename... P, typename... A>
cudaError_t launch_split_clusters(void (*kernel)(P...), dim3 grid, int threads, cudaStream_t stream, A&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3((unsigned)threads);
  cfg.stream = stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 1;
  at[0].val.clusterDim.y = grid.y;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

}  // namespace

template <typename T>
gbblas_status launch_gemv_rows(DeviceCtx* c, int64_t rows, int64_t cols, const T* A, int64_t lda, const T* x,
                               T* y, bool accumulate, cudaStream_t stream) {
  if (rows <= 0) return GBBLAS_STATUS_SUCCESS;
  constexpr int W = V<T>::w;
  const bool vec = aligned16(A) && aligned16(x) && (lda % W) == 0;
  const int64_t target = (int64_t)c->num_sms * 8;  // 8 CTAs of 256 threads fill an SM
  const bool use_r4 = rows >= 4 * (int64_t)c->num_sms * 4;
  const int R = use_r4 ? 4 : 1;
  const int64_t groups = cdiv(rows, R);
  int64_t ksplit = 1;
  if (groups < target && cols > 4096) {
    ksplit = cdiv(target, groups);
    int64_t max_split = cdiv(cols, 2048);
    if (ksplit > max_split) ksplit = max_split;
    if (ksplit > 65535) ksplit = 65535;
  }
  int64_t cps = cdiv(cdiv(cols, ksplit), 256) * 256;  // multiple of the vector width
  ksplit = cdiv(cols, cps);
  if (ksplit < 1) ksplit = 1;
  dim3 grid((unsigned)groups, (unsigned)ksplit);
  T* partials = nullptr;
  if (cluster_splits(ksplit, rows, cols, sizeof(T))) {
    cudaError_t e;
    if (R == 4)
      e = vec ? launch_split_clusters(gemv_rows_kernel<T, 4, true, true>, grid, kRowsThreads, stream, rows, cols, A,
                                      lda, x, y, accumulate, partials, cps)
              : launch_split_clusters(gemv_rows_kernel<T, 4, false, true>, grid, kRowsThreads, stream, rows, cols, A,
                                      lda, x, y, accumulate, partials, cps);
    else
      e = vec ? launch_split_clusters(gemv_rows_kernel<T, 1, true, true>, grid, kRowsThreads, stream, rows, cols, A,
                                      lda, x, y, accumulate, partials, cps)
              : launch_split_clusters(gemv_rows_kernel<T, 1, false, true>, grid, kRowsThreads, stream, rows, cols, A,
                                      lda, x, y, accumulate, partials, cps);
    if (e == cudaSuccess) return check_launch("gemv_rows_kernel (split clusters)");
    cudaGetLastError();  // the cluster launch was refused: partials in scratch instead
  }
  if (ksplit > 1) {
    void* s = nullptr;
    GB_TRY(get_scratch(c, stream, kScratchZeroBytes + sizeof(T) * ksplit * rows, &s));
    partials = reinterpret_cast<T*>(static_cast<char*>(s) + kScratchZeroBytes);
  }
  if (R == 4) {
    if (vec)
      gemv_rows_kernel<T, 4, true, false><<<grid, kRowsThreads, 0, stream>>>(rows, cols, A, lda, x, y, accumulate,
                                                                             partials, cps);
    else
      gemv_rows_kernel<T, 4, false, false><<<grid, kRowsThreads, 0, stream>>>(rows, cols, A, lda, x, y, accumulate,
                                                                              partials, cps);
  } else {
    if (vec)
      gemv_rows_kernel<T, 1, true, false><<<grid, kRowsThreads, 0, stream>>>(rows, cols, A, lda, x, y, accumulate,
                                                                             partials, cps);
    else
      gemv_rows_kernel<T, 1, false, false><<<grid, kRowsThreads, 0, stream>>>(rows, cols, A, lda, x, y, accumulate,
                                                                              partials, cps);
  }
  GB_TRY(check_launch("gemv_rows_kernel"));
  if (ksplit > 1) {
    finish_splits_kernel<T><<<(unsigned)cdiv(rows, 256), 256, 0, stream>>>(rows, (int)ksplit, partials, y,
                                                                           accumulate);
    GB_TRY(check_launch("finish_splits_kernel"));
  }
  return GBBLAS_STATUS_SUCCESS;
}

template <typename T>
gbblas_status launch_gemv_cols(DeviceCtx* c, int64_t rows, int64_t cols, const T* A, int64_t lda, const T* x,
                               T* y, bool accumulate, cudaStream_t stream) {
  if (rows <= 0) return GBBLAS_STATUS_SUCCESS;
  constexpr int W = V<T>::w;
  const bool vec = aligned16(A) && (lda % W) == 0;
  const int w = vec ? W : 1;
  int threads = 256;
  const int64_t thr_needed = cdiv(rows, w);
  if (thr_needed < 256) threads = (int)cdiv(thr_needed, 32) * 32;
  const int64_t rblocks = cdiv(thr_needed, threads);
  const int64_t target = (int64_t)c->num_sms * (2048 / threads);
  int64_t ksplit = 1;
  if (rblocks < target && cols > 64) {
    ksplit = cdiv(target, rblocks);
    int64_t max_split = cdiv(cols, 64);
    if (ksplit > max_split) ksplit = max_split;
    if (ksplit > 65535) ksplit = 65535;
  }
  int64_t cps = cdiv(cols, ksplit);
  ksplit = cdiv(cols, cps);
  if (ksplit < 1) ksplit = 1;
  dim3 grid((unsigned)rblocks, (unsigned)ksplit);
  T* partials = nullptr;
  if (cluster_splits(ksplit, rows, cols, sizeof(T))) {
    const cudaError_t e = vec ? launch_split_clusters(gemv_cols_kernel<T, true, true>, grid, threads, stream, rows,
                                                      cols, A, lda, x, y, accumulate, partials, cps)
                              : launch_split_clusters(gemv_cols_kernel<T, false, true>, grid, threads, stream, rows,
                                                      cols, A, lda, x, y, accumulate, partials, cps);
    if (e == cudaSuccess) return check_launch("gemv_cols_kernel (split clusters)");
    cudaGetLastError();  // the cluster launch was refused: partials in scratch instead
  }
  if (ksplit > 1) {
    void* s = nullptr;
    GB_TRY(get_scratch(c, stream, kScratchZeroBytes + sizeof(T) * ksplit * rows, &s));
    partials = reinterpret_cast<T*>(static_cast<char*>(s) + kScratchZeroBytes);
  }
  if (vec)
    gemv_cols_kernel<T, true, false><<<grid, threads, 0, stream>>>(rows, cols, A, lda, x, y, accumulate, partials,
                                                                   cps);
  else
    gemv_cols_kernel<T, false, false><<<grid, threads, 0, stream>>>(rows, cols, A, lda, x, y, accumulate, partials,
                                                                    cps);
  GB_TRY(check_launch("gemv_cols_kernel"));
  if (ksplit > 1) {
    finish_splits_kernel<T><<<(unsigned)cdiv(rows, 256), 256, 0, stream>>>(rows, (int)ksplit, partials, y,
                                                                           accumulate);
    GB_TRY(check_launch("finish_splits_kernel"));
  }
  return GBBLAS_STATUS_SUCCESS;
}

#define GB_INST(T)                                                                                          \
  template gbblas_status launch_gemv_rows<T>(DeviceCtx*, int64_t, int64_t, const T*, int64_t, const T*, T*, \
                                             bool, cudaStream_t);                                            \
  template gbblas_status launch_gemv_cols<T>(DeviceCtx*, int64_t, int64_t, const T*, int64_t, const T*, T*, \
                                             bool, cudaStream_t);
GB_INST(float)
GB_INST(double)
#undef GB_INST

}  // namespace gbblas
