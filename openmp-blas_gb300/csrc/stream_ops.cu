// stream_ops.cu - the HBM-streaming operations beside the hot path:
//
//   outer product   C += a b^T            (reference include/outer.hpp:14-121)
//   transpose       C = A^T, any strides   (reference include/trans.hpp:33-145)
//                   A = A^T in place, square (include/trans.hpp:67-101, 147-169)
//   element-wise    c[i] = a[i] (+ - * /) b[i]  (reference include/el_wise_op.hpp:33-121)
//
// All three move each byte of their operands once; their roofline is HBM
// bandwidth.  Algorithmic bytes: outer 2*M*N*s (read and write C) plus the
// vectors; transpose 2*M*N*s; element-wise 3*n*s.
#include "common.cuh"

namespace gbblas {
namespace {

constexpr int kThreads = 256;

// ---------------------------------------------------------- outer product
// C[r*ld + l] = fma(u[r], v[l], C[r*ld + l]) for r < R, l < L: rows of C are
// contiguous.  Thread (x) owns VEC consecutive columns and keeps their v in
// registers; CTAs stride over rows (y).  The reference's inner loop is the
// same fused update c[i] += a[i] * b_j (include/simd_loop.hpp:42-47), so the
// results agree bit for bit with an FMA-contracting CPU build.
template <typename T, int VEC>
__global__ void __launch_bounds__(kThreads) rank1_kernel(int64_t R, int64_t L, const T* __restrict__ u,
                                                         const T* __restrict__ v, T* __restrict__ C, int64_t ld) {
  const int64_t l = ((int64_t)blockIdx.x * kThreads + threadIdx.x) * VEC;
  if (l >= L) return;
  T vr[VEC];
#pragma unroll
  for (int i = 0; i < VEC; ++i) vr[i] = __ldg(v + l + i);
  for (int64_t r = blockIdx.y; r < R; r += gridDim.y) {
    const T ur = __ldg(u + r);
    T* p = C + r * ld + l;
    if constexpr (VEC == 1) {
      *p = fma(ur, vr[0], *p);
    } else if constexpr (sizeof(T) == 4) {
      float4 c4 = *reinterpret_cast<float4*>(p);
      c4.x = fmaf(ur, vr[0], c4.x);
      c4.y = fmaf(ur, vr[1], c4.y);
      c4.z = fmaf(ur, vr[2], c4.z);
      c4.w = fmaf(ur, vr[3], c4.w);
      *reinterpret_cast<float4*>(p) = c4;
    } else {
      double2 c2 = *reinterpret_cast<double2*>(p);
      c2.x = fma(ur, vr[0], c2.x);
      c2.y = fma(ur, vr[1], c2.y);
      *reinterpret_cast<double2*>(p) = c2;
    }
  }
}

// ---------------------------------------------------------------- transpose
// C(j, i) = A(i, j) for i < M, j < N; A(i, j) at A[i*rsa + j*csa], C(j, i) at
// C[j*rsc + i*csc].  TILE x TILE tiles through shared memory: the tile is read
// with consecutive threads along A's unit-stride index and written with
// consecutive threads along C's, so both sides coalesce for every layout pair.
// Each thread first loads its (TILE/8) x (TILE/32) elements into registers,
// so that many loads are in flight before the first shared-memory store.
template <typename T, int TILE>
__global__ void __launch_bounds__(kThreads, 3) transpose_kernel(int64_t M, int64_t N, const T* __restrict__ A,
                                                                int64_t rsa, int64_t csa, T* __restrict__ C,
                                                                int64_t rsc, int64_t csc, int64_t tiles_n,
                                                                int64_t ntiles) {
  constexpr int KR = TILE / 8, KC = TILE / 32;  // passes of the 32 x 8 thread block
  __shared__ T tile[TILE][TILE + 1];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  const bool a_rows = csa == 1;  // A's j (column) index is contiguous
  const bool c_rows = csc == 1;  // C's i index is contiguous
  // pass (k, h) of the load touches tile element (ai + da, aj + db) ...
  const int ai = a_rows ? ty : tx, aj = a_rows ? tx : ty;
  const int64_t ak = a_rows ? 8 * rsa : 8 * csa, ah = a_rows ? 32 * csa : 32 * rsa;  // ... element steps
  const int ci = c_rows ? tx : ty, cj = c_rows ? ty : tx;
  const int64_t ck = c_rows ? 8 * rsc : 8 * csc, ch = c_rows ? 32 * csc : 32 * rsc;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t i0 = (t / tiles_n) * TILE, j0 = (t % tiles_n) * TILE;
    const bool full = i0 + TILE <= M && j0 + TILE <= N;
    T r[KR][KC];
    const T* pa = A + (i0 + ai) * rsa + (j0 + aj) * csa;
    if (full) {
#pragma unroll
      for (int k = 0; k < KR; ++k)
#pragma unroll
        for (int h = 0; h < KC; ++h) r[k][h] = pa[k * ak + h * ah];
    } else {
#pragma unroll
      for (int k = 0; k < KR; ++k)
#pragma unroll
        for (int h = 0; h < KC; ++h) {
          const int ii = a_rows ? ai + 8 * k : ai + 32 * h, jj = a_rows ? aj + 32 * h : aj + 8 * k;
          r[k][h] = (i0 + ii < M && j0 + jj < N) ? pa[k * ak + h * ah] : T(0);
        }
    }
#pragma unroll
    for (int k = 0; k < KR; ++k)
#pragma unroll
      for (int h = 0; h < KC; ++h) {
        const int ii = a_rows ? ai + 8 * k : ai + 32 * h, jj = a_rows ? aj + 32 * h : aj + 8 * k;
        tile[ii][jj] = r[k][h];
      }
    __syncthreads();
    T* pc = C + (j0 + cj) * rsc + (i0 + ci) * csc;
#pragma unroll
    for (int k = 0; k < KR; ++k)
#pragma unroll
      for (int h = 0; h < KC; ++h) {
        const int ii = c_rows ? ci + 32 * h : ci + 8 * k, jj = c_rows ? cj + 8 * k : cj + 32 * h;
        if (full || (i0 + ii < M && j0 + jj < N)) pc[k * ck + h * ch] = tile[ii][jj];
      }
    __syncthreads();
  }
}

// In place, square n x n: storage element (r, c) = A[r*n + c] swaps with
// (c, r) - the same storage permutation for either layout.  CTA (bj, bi)
// with bj >= bi swaps tile (bi, bj) with tile (bj, bi) through shared memory;
// the others return at once.
template <typename T>
__global__ void __launch_bounds__(kThreads) transpose_square_kernel(int64_t n, T* __restrict__ A) {
  __shared__ T t1[32][33];
  __shared__ T t2[32][33];
  const int64_t bi = blockIdx.y, bj = blockIdx.x;
  if (bj < bi) return;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const bool diag = bi == bj;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int ii = ty + 8 * k;
    const int64_t r1 = bi * 32 + ii, c1 = bj * 32 + tx;
    if (r1 < n && c1 < n) t1[ii][tx] = A[r1 * n + c1];
    const int64_t r2 = bj * 32 + ii, c2 = bi * 32 + tx;
    if (!diag && r2 < n && c2 < n) t2[ii][tx] = A[r2 * n + c2];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int ii = ty + 8 * k;
    // (bi, bj) tile receives the transpose of tile (bj, bi), and vice versa
    const int64_t r1 = bi * 32 + ii, c1 = bj * 32 + tx;
    if (r1 < n && c1 < n) A[r1 * n + c1] = diag ? t1[tx][ii] : t2[tx][ii];
    const int64_t r2 = bj * 32 + ii, c2 = bi * 32 + tx;
    if (!diag && r2 < n && c2 < n) A[r2 * n + c2] = t1[tx][ii];
  }
}

// ------------------------------------------------------------ element-wise
template <int OP, typename T>
__device__ __forceinline__ T ew_apply(T a, T b) {
  if constexpr (OP == GBBLAS_EW_ADD) return a + b;
  if constexpr (OP == GBBLAS_EW_SUB) return a - b;
  if constexpr (OP == GBBLAS_EW_MUL) return a * b;
  return a / b;  // IEEE division (the library is built without fast-math)
}

// c[i] = a[i] op b[i]; 128-bit vectors when all three are 16-byte aligned.
template <typename T, int OP, bool VEC>
__global__ void __launch_bounds__(kThreads) ew_kernel(int64_t n, const T* a, const T* b, T* c) {
  // c may be a or b: element i is read and written by the same thread only.
  const int64_t stride = (int64_t)gridDim.x * kThreads;
  int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if constexpr (VEC) {
    constexpr int W = 16 / sizeof(T);
    const int64_t nv = n / W;
    if constexpr (sizeof(T) == 4) {
      for (int64_t g = i; g < nv; g += stride) {
        const float4 x = dev::ld_stream(reinterpret_cast<const float4*>(a) + g);
        const float4 y = dev::ld_stream(reinterpret_cast<const float4*>(b) + g);
        float4 z;
        z.x = ew_apply<OP>(x.x, y.x);
        z.y = ew_apply<OP>(x.y, y.y);
        z.z = ew_apply<OP>(x.z, y.z);
        z.w = ew_apply<OP>(x.w, y.w);
        reinterpret_cast<float4*>(c)[g] = z;
      }
    } else {
      for (int64_t g = i; g < nv; g += stride) {
        const double2 x = dev::ld_stream(reinterpret_cast<const double2*>(a) + g);
        const double2 y = dev::ld_stream(reinterpret_cast<const double2*>(b) + g);
        double2 z;
        z.x = ew_apply<OP>(x.x, y.x);
        z.y = ew_apply<OP>(x.y, y.y);
        reinterpret_cast<double2*>(c)[g] = z;
      }
    }
    i += nv * W;  // scalar tail
    for (; i < n; i += stride) c[i] = ew_apply<OP>(a[i], b[i]);
  } else {
    for (; i < n; i += stride) c[i] = ew_apply<OP>(a[i], b[i]);
  }
}

template <typename T, int OP>
gbblas_status launch_ew_op(DeviceCtx* c, int64_t n, const T* a, const T* b, T* out, cudaStream_t s) {
  const bool vec = aligned16(a) && aligned16(b) && aligned16(out);
  const int64_t per = vec ? (int64_t)kThreads * (16 / sizeof(T)) : kThreads;
  int64_t grid = (n + per - 1) / per;
  const int64_t cap = (int64_t)c->num_sms * 8;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  if (vec)
    ew_kernel<T, OP, true><<<(unsigned)grid, kThreads, 0, s>>>(n, a, b, out);
  else
    ew_kernel<T, OP, false><<<(unsigned)grid, kThreads, 0, s>>>(n, a, b, out);
  return check_launch("ew_kernel");
}

}  // namespace

template <typename T>
gbblas_status launch_outer(DeviceCtx* c, int64_t R, int64_t L, const T* u, const T* v, T* C, int64_t ld,
                           cudaStream_t s) {
  if (R == 0 || L == 0) return GBBLAS_STATUS_SUCCESS;
  constexpr int W = 16 / sizeof(T);
  const bool vec = aligned16(C) && (ld % W) == 0 && (L % W) == 0;
  const int per = vec ? W : 1;
  const int64_t gx = (L / per + kThreads - 1) / kThreads;
  if (gx > 0x7fffffff) {
    set_error("outer: %lld columns exceed the grid", (long long)L);
    return GBBLAS_STATUS_NOT_SUPPORTED;
  }
  // enough CTAs for about 8 per SM, each walking rows
  int64_t gy = ((int64_t)c->num_sms * 8 + gx - 1) / gx;
  if (gy > R) gy = R;
  if (gy > 65535) gy = 65535;
  if (gy < 1) gy = 1;
  dim3 grid((unsigned)gx, (unsigned)gy);
  if (vec)
    rank1_kernel<T, W><<<grid, kThreads, 0, s>>>(R, L, u, v, C, ld);
  else
    rank1_kernel<T, 1><<<grid, kThreads, 0, s>>>(R, L, u, v, C, ld);
  return check_launch("rank1_kernel");
}

template <typename T>
gbblas_status launch_transpose(DeviceCtx* c, int64_t M, int64_t N, const T* A, int64_t rsa, int64_t csa, T* C,
                               int64_t rsc, int64_t csc, cudaStream_t s) {
  if (M == 0 || N == 0) return GBBLAS_STATUS_SUCCESS;
  constexpr int TILE = 64;  // 16 (f32) / 32 (f64) KB of shared memory per CTA
  const int64_t tm = (M + TILE - 1) / TILE, tn = (N + TILE - 1) / TILE, nt = tm * tn;
  int64_t grid = nt;
  const int64_t cap = (int64_t)c->num_sms * 8;
  if (grid > cap) grid = cap;
  transpose_kernel<T, TILE><<<(unsigned)grid, kThreads, 0, s>>>(M, N, A, rsa, csa, C, rsc, csc, tn, nt);
  return check_launch("transpose_kernel");
}

template <typename T>
gbblas_status launch_transpose_square(DeviceCtx* c, int64_t n, T* A, cudaStream_t s) {
  (void)c;
  if (n == 0) return GBBLAS_STATUS_SUCCESS;
  const int64_t t = (n + 31) / 32;
  if (t > 65535) {
    set_error("transpose in place: n = %lld exceeds the tile grid", (long long)n);
    return GBBLAS_STATUS_NOT_SUPPORTED;
  }
  transpose_square_kernel<T><<<dim3((unsigned)t, (unsigned)t), kThreads, 0, s>>>(n, A);
  return check_launch("transpose_square_kernel");
}

template <typename T>
gbblas_status launch_ew(DeviceCtx* c, gbblas_ew_op op, int64_t n, const T* a, const T* b, T* out, cudaStream_t s) {
  if (n == 0) return GBBLAS_STATUS_SUCCESS;
  switch (op) {
    case GBBLAS_EW_ADD: return launch_ew_op<T, GBBLAS_EW_ADD>(c, n, a, b, out, s);
    case GBBLAS_EW_SUB: return launch_ew_op<T, GBBLAS_EW_SUB>(c, n, a, b, out, s);
    case GBBLAS_EW_MUL: return launch_ew_op<T, GBBLAS_EW_MUL>(c, n, a, b, out, s);
    case GBBLAS_EW_DIV: return launch_ew_op<T, GBBLAS_EW_DIV>(c, n, a, b, out, s);
  }
  set_error("element-wise: unknown operation %d", (int)op);
  return GBBLAS_STATUS_INVALID_VALUE;
}

template gbblas_status launch_outer<float>(DeviceCtx*, int64_t, int64_t, const float*, const float*, float*,
                                           int64_t, cudaStream_t);
template gbblas_status launch_outer<double>(DeviceCtx*, int64_t, int64_t, const double*, const double*, double*,
                                            int64_t, cudaStream_t);
template gbblas_status launch_transpose<float>(DeviceCtx*, int64_t, int64_t, const float*, int64_t, int64_t, float*,
                                               int64_t, int64_t, cudaStream_t);
template gbblas_status launch_transpose<double>(DeviceCtx*, int64_t, int64_t, const double*, int64_t, int64_t,
                                                double*, int64_t, int64_t, cudaStream_t);
template gbblas_status launch_transpose_square<float>(DeviceCtx*, int64_t, float*, cudaStream_t);
template gbblas_status launch_transpose_square<double>(DeviceCtx*, int64_t, double*, cudaStream_t);
template gbblas_status launch_ew<float>(DeviceCtx*, gbblas_ew_op, int64_t, const float*, const float*, float*,
                                        cudaStream_t);
template gbblas_status launch_ew<double>(DeviceCtx*, gbblas_ew_op, int64_t, const double*, const double*, double*,
                                         cudaStream_t);

}  // namespace gbblas
