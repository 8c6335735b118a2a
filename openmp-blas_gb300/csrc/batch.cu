// batch.cu - grouped GEMV, and batches of GEMMs + GEMVs replayed as one
// CUDA graph.
//
// Grouped GEMV ("row-streaming" forms: row-major A, or A^T of column-major A):
// every output element is the dot of one contiguous row with x.  All rows of
// all problems are cut into warp items of R rows; a persistent grid of warps
// walks the items in order (problem by problem, so concurrent warps share
// each problem's x in L1/L2) with 128-bit streaming loads of A.  R is chosen
// per batch by the autotuner.  Column-streaming forms (column-major y = A x,
// row-major y = A^T x) reuse the single-problem kernel per problem.
//
// A batch (gbblas_batch_*) is planned once: the GEMM group's tables and BF16
// arena and the GEMV group's table live in memory the batch owns, and the
// whole thing - grouped tensor-core GEMM on one branch, grouped GEMV on the
// other - is captured into a CUDA graph that each run replays with one
// cudaGraphLaunch.  Roofline: GEMM part tensor pipe, GEMV part HBM
// ((rows*cols + rows + cols) * 4 bytes per problem).
#include <algorithm>
#include <vector>

#include "common.cuh"

namespace gbblas {
namespace {

struct GemvRowsProblem {
  const float* A;
  const float* x;
  float* y;
  int64_t rows, cols, lda;
  int64_t item_start;  // first warp item of this problem
  int accumulate;
};

__device__ __forceinline__ int find_rows_problem(const GemvRowsProblem* __restrict__ p, int lo, int n,
                                                 int64_t item) {
  int hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (p[mid].item_start <= item)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ float dot4(float4 a, float4 b, float acc) {
  acc = fmaf(a.x, b.x, acc);
  acc = fmaf(a.y, b.y, acc);
  acc = fmaf(a.z, b.z, acc);
  return fmaf(a.w, b.w, acc);
}

constexpr int kGroupThreads = 256;
constexpr int kRowUnroll = 4;  // float4 loads of A in flight per lane and row

// Dot of one row (any alignment of its start) with x, summed over the warp.
// The row is split into a head of up to 3 elements that brings it to a
// 16-byte boundary, a body of float4 streaming loads, and a tail.  x is read
// with float4 loads when it shares the body's alignment, element-wise
// (L1 hits) otherwise.
__device__ __forceinline__ float row_dot(const float* __restrict__ row, const float* __restrict__ x, int64_t cols,
                                         int lane) {
  int64_t head = (int64_t)(((16 - (reinterpret_cast<uintptr_t>(row) & 15)) & 15) >> 2);
  if (head > cols) head = cols;
  float acc = 0.f;
  if (lane < head) acc = fmaf(dev::ld_stream(row + lane), __ldg(x + lane), acc);
  const float* rb = row + head;
  const float* xb = x + head;
  const int64_t nv = (cols - head) >> 2;
  const float4* rv = reinterpret_cast<const float4*>(rb);
  const bool xvec = (reinterpret_cast<uintptr_t>(xb) & 15) == 0;
  float acc2 = 0.f;
  int64_t v = lane;
  if (xvec) {
    const float4* xv = reinterpret_cast<const float4*>(xb);
    for (; v + 32 * (kRowUnroll - 1) < nv; v += 32 * kRowUnroll) {
      float4 a[kRowUnroll];
#pragma unroll
      for (int u = 0; u < kRowUnroll; ++u) a[u] = dev::ld_stream(rv + v + 32 * u);
#pragma unroll
      for (int u = 0; u < kRowUnroll; ++u) acc2 = dot4(a[u], __ldg(xv + v + 32 * u), acc2);
    }
    for (; v < nv; v += 32) acc2 = dot4(dev::ld_stream(rv + v), __ldg(xv + v), acc2);
  } else {
    for (; v + 32 * (kRowUnroll - 1) < nv; v += 32 * kRowUnroll) {
      float4 a[kRowUnroll];
#pragma unroll
      for (int u = 0; u < kRowUnroll; ++u) a[u] = dev::ld_stream(rv + v + 32 * u);
#pragma unroll
      for (int u = 0; u < kRowUnroll; ++u) {
        const float* xs = xb + 4 * (v + 32 * u);
        acc2 = dot4(a[u], make_float4(__ldg(xs), __ldg(xs + 1), __ldg(xs + 2), __ldg(xs + 3)), acc2);
      }
    }
    for (; v < nv; v += 32) {
      const float* xs = xb + 4 * v;
      acc2 = dot4(dev::ld_stream(rv + v), make_float4(__ldg(xs), __ldg(xs + 1), __ldg(xs + 2), __ldg(xs + 3)),
                  acc2);
    }
  }
  for (int64_t cidx = head + 4 * nv + lane; cidx < cols; cidx += 32)
    acc = fmaf(dev::ld_stream(row + cidx), __ldg(x + cidx), acc);
  return dev::warp_sum(acc + acc2);
}

// Persistent grid of warps over warp items of R consecutive rows.
template <int R>
__global__ void __launch_bounds__(kGroupThreads, 4)
    gemv_group_rows_kernel(const GemvRowsProblem* __restrict__ probs, int nprob, int64_t total_items) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int p = 0;
  for (int64_t item = w0; item < total_items; item += nw) {
    p = find_rows_problem(probs, p, nprob, item);
    const GemvRowsProblem& pr = probs[p];
    const int64_t r0 = (item - pr.item_start) * R;
    const int nr = (int)((pr.rows - r0) < R ? (pr.rows - r0) : R);
    for (int r = 0; r < nr; ++r) {
      const float s = row_dot(pr.A + (r0 + r) * pr.lda, pr.x, pr.cols, lane);
      if (lane == 0) {
        float* yp = pr.y + r0 + r;
        *yp = pr.accumulate ? *yp + s : s;
      }
    }
  }
}

// Column-streaming GEMV (run per problem with the single-call kernel).
struct GemvColsProblem {
  const float* A;
  const float* x;
  float* y;
  int64_t rows, cols, lda;
  bool accumulate;
};

}  // namespace

// Planned GEMV group: row-streaming table (device) + column-streaming list.
struct GemvGroupPlan {
  int R = 4;
  std::vector<GemvRowsProblem> rows;
  std::vector<GemvColsProblem> cols;
  int64_t total_items = 0;
  GemvRowsProblem* dtable = nullptr;
  bool owned = false;
};

namespace {

gbblas_status plan_gemv_group(const gbblas_gemv_desc* d, int64_t count, int R, GemvGroupPlan& pl) {
  pl.R = R;
  for (int64_t i = 0; i < count; ++i) {
    const gbblas_gemv_desc& g = d[i];
    if ((g.layout != GBBLAS_FIRST_ORDER && g.layout != GBBLAS_LAST_ORDER) || g.M < 0 || g.N < 0) {
      set_error("grouped gemv: descriptor %lld has a bad layout or size", (long long)i);
      return GBBLAS_STATUS_INVALID_VALUE;
    }
    if (g.M == 0 || g.N == 0) continue;
    if (!g.A || !g.x || !g.y) {
      set_error("grouped gemv: descriptor %lld has a null pointer", (long long)i);
      return GBBLAS_STATUS_INVALID_VALUE;
    }
    const bool tr = g.transpose != 0;
    const int64_t out_len = tr ? g.N : g.M, red_len = tr ? g.M : g.N;
    const int64_t lda = g.layout == GBBLAS_LAST_ORDER ? g.N : g.M;
    const bool rows_contig = (g.layout == GBBLAS_LAST_ORDER) != tr;
    if (rows_contig) {
      GemvRowsProblem p;
      p.A = g.A;
      p.x = g.x;
      p.y = g.y;
      p.rows = out_len;
      p.cols = red_len;
      p.lda = lda;
      p.item_start = pl.total_items;
      p.accumulate = g.accumulate != 0;
      pl.total_items += (out_len + R - 1) / R;
      pl.rows.push_back(p);
    } else {
      pl.cols.push_back({g.A, g.x, g.y, out_len, red_len, lda, g.accumulate != 0});
    }
  }
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status launch_gemv_group_plan(DeviceCtx* c, const GemvGroupPlan& pl, cudaStream_t s) {
  if (!pl.rows.empty()) {
    const int nprob = (int)pl.rows.size();
    const int64_t want = (pl.total_items * 32 + kGroupThreads - 1) / kGroupThreads;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)c->num_sms * 4));
    switch (pl.R) {
      case 1:
        gemv_group_rows_kernel<1><<<grid, kGroupThreads, 0, s>>>(pl.dtable, nprob, pl.total_items);
        break;
      case 2:
        gemv_group_rows_kernel<2><<<grid, kGroupThreads, 0, s>>>(pl.dtable, nprob, pl.total_items);
        break;
      case 8:
        gemv_group_rows_kernel<8><<<grid, kGroupThreads, 0, s>>>(pl.dtable, nprob, pl.total_items);
        break;
      default:
        gemv_group_rows_kernel<4><<<grid, kGroupThreads, 0, s>>>(pl.dtable, nprob, pl.total_items);
        break;
    }
    GB_TRY(check_launch("gemv_group_rows_kernel"));
  }
  for (const GemvColsProblem& p : pl.cols)
    GB_TRY(launch_gemv_cols<float>(c, p.rows, p.cols, p.A, p.lda, p.x, p.y, p.accumulate, s));
  return GBBLAS_STATUS_SUCCESS;
}

}  // namespace

// Rows per warp item for a set of GEMVs, from the autotuner.
int tuned_gemv_group_rows(DeviceCtx* c, const gbblas_gemv_desc* d, int64_t count);

gbblas_status launch_gemv_group_rows_fixed(DeviceCtx* c, const gbblas_gemv_desc* d, int64_t count, cudaStream_t s,
                                           int R) {
  GemvGroupPlan pl;
  GB_TRY(plan_gemv_group(d, count, R, pl));
  if (!pl.rows.empty()) {
    void* scratch = nullptr;
    GB_TRY(get_scratch(c, s, kScratchZeroBytes + sizeof(GemvRowsProblem) * pl.rows.size(), &scratch));
    pl.dtable = reinterpret_cast<GemvRowsProblem*>(static_cast<char*>(scratch) + kScratchZeroBytes);
    GB_CUDA_TRY(cudaMemcpyAsync(pl.dtable, pl.rows.data(), sizeof(GemvRowsProblem) * pl.rows.size(),
                                cudaMemcpyHostToDevice, s));
  }
  return launch_gemv_group_plan(c, pl, s);
}

gbblas_status launch_gemv_group(DeviceCtx* c, const gbblas_gemv_desc* d, int64_t count, cudaStream_t s) {
  return launch_gemv_group_rows_fixed(c, d, count, s, tuned_gemv_group_rows(c, d, count));
}

// Time the row-streaming group kernel with R rows per item on the given
// GEMVs (outputs redirected to a scratch vector, so callers' y are
// untouched); used by the autotuner.
gbblas_status time_gemv_group_variant(DeviceCtx* c, const gbblas_gemv_desc* d, int64_t count, int R, float* ms) {
  GemvGroupPlan pl;
  GB_TRY(plan_gemv_group(d, count, R, pl));
  pl.cols.clear();
  if (pl.rows.empty()) {
    *ms = 0.f;
    return GBBLAS_STATUS_SUCCESS;
  }
  int64_t ytotal = 0;
  for (auto& p : pl.rows) ytotal += p.rows;
  cudaStream_t s;
  GB_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  void* mem = nullptr;
  const size_t table_bytes = (sizeof(GemvRowsProblem) * pl.rows.size() + 255) & ~size_t(255);
  cudaError_t e = cudaMallocAsync(&mem, table_bytes + sizeof(float) * ytotal, s);
  if (e != cudaSuccess) {
    cudaStreamDestroy(s);
    set_error("autotune: scratch allocation failed: %s", cudaGetErrorString(e));
    return GBBLAS_STATUS_ALLOC_FAILED;
  }
  float* ybuf = reinterpret_cast<float*>(static_cast<char*>(mem) + table_bytes);
  int64_t off = 0;
  for (auto& p : pl.rows) {
    p.y = ybuf + off;
    p.accumulate = 0;
    off += p.rows;
  }
  pl.dtable = static_cast<GemvRowsProblem*>(mem);
  gbblas_status st = GBBLAS_STATUS_SUCCESS;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  if (cudaMemcpyAsync(pl.dtable, pl.rows.data(), sizeof(GemvRowsProblem) * pl.rows.size(), cudaMemcpyHostToDevice,
                      s) != cudaSuccess)
    st = GBBLAS_STATUS_CUDA_ERROR;
  if (st == GBBLAS_STATUS_SUCCESS) st = launch_gemv_group_plan(c, pl, s);  // warm-up
  if (st == GBBLAS_STATUS_SUCCESS) {
    cudaEventRecord(e0, s);
    for (int i = 0; i < 3 && st == GBBLAS_STATUS_SUCCESS; ++i) st = launch_gemv_group_plan(c, pl, s);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    *ms = t / 3.f;
  }
  cudaFreeAsync(mem, s);
  cudaStreamSynchronize(s);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  return st;
}

}  // namespace gbblas

// ============================================================ batches
using namespace gbblas;

struct gbblas_batch_s {
  DeviceCtx* ctx = nullptr;
  TcGroupPlan* gemm = nullptr;
  GemvGroupPlan gemv;
  std::vector<gbblas_gemm_desc> fma_gemms;  // accuracy FP32: run one by one
  cudaStream_t s0 = nullptr, s1 = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t last = nullptr;
};

namespace {

void batch_free(gbblas_batch b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->gemm) tc_group_destroy(b->gemm);
  if (b->gemv.dtable && b->gemv.owned) cudaFree(b->gemv.dtable);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->join) cudaEventDestroy(b->join);
  if (b->s0) cudaStreamDestroy(b->s0);
  if (b->s1) cudaStreamDestroy(b->s1);
  delete b;
}

}  // namespace

extern "C" {

gbblas_status gbblas_batch_create(const gbblas_gemm_desc* gemms, int64_t ngemm, gbblas_accuracy accuracy,
                                  const gbblas_gemv_desc* gemvs, int64_t ngemv, gbblas_batch* out) {
  if (!out || ngemm < 0 || ngemv < 0 || (ngemm > 0 && !gemms) || (ngemv > 0 && !gemvs)) {
    set_error("gbblas_batch_create: bad arguments");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  if (((int)accuracy < 0 || (int)accuracy > 4) && accuracy != GBBLAS_ACCURACY_FP16X3) {
    set_error("gbblas_batch_create: unknown accuracy %d", (int)accuracy);
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  gbblas_batch b = new gbblas_batch_s();
  b->ctx = c;
  auto fail = [&](gbblas_status st) {
    batch_free(b);
    return st;
  };
  gbblas_status st;
  if (ngemm > 0) {
    if (accuracy == GBBLAS_ACCURACY_FP32) {
      b->fma_gemms.assign(gemms, gemms + ngemm);
    } else {
      // AUTO in a batch: the FP32-accurate split-FP16 GEMM with its guard
      const int mode = accuracy == GBBLAS_ACCURACY_AUTO ? kTcModeF16Guard : tc_mode(accuracy);
      if ((st = tc_group_create(c, mode, gemms, ngemm, &b->gemm)) != GBBLAS_STATUS_SUCCESS) return fail(st);
    }
  }
  if (ngemv > 0) {
    if ((st = plan_gemv_group(gemvs, ngemv, tuned_gemv_group_rows(c, gemvs, ngemv), b->gemv)) !=
        GBBLAS_STATUS_SUCCESS)
      return fail(st);
    if (!b->gemv.rows.empty()) {
      void* p = nullptr;
      if (cudaMalloc(&p, sizeof(GemvRowsProblem) * b->gemv.rows.size()) != cudaSuccess) {
        set_error("gbblas_batch_create: table allocation failed");
        return fail(GBBLAS_STATUS_ALLOC_FAILED);
      }
      b->gemv.dtable = static_cast<GemvRowsProblem*>(p);
      b->gemv.owned = true;
      if (cudaMemcpy(p, b->gemv.rows.data(), sizeof(GemvRowsProblem) * b->gemv.rows.size(),
                     cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(GBBLAS_STATUS_CUDA_ERROR);
    }
  }
  if (cudaStreamCreateWithFlags(&b->s0, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->s1, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming) != cudaSuccess)
    return fail(GBBLAS_STATUS_CUDA_ERROR);
  // Everything a captured launch needs must exist before capture: kernel
  // attributes, and per-stream scratch for the per-problem kernels.
  tc_prepare(c);
  void* scr = nullptr;
  for (cudaStream_t s : {b->s0, b->s1})
    if ((st = get_scratch(c, s, (size_t)64 << 20, &scr)) != GBBLAS_STATUS_SUCCESS) return fail(st);
  if (cudaStreamSynchronize(b->s0) != cudaSuccess || cudaStreamSynchronize(b->s1) != cudaSuccess)
    return fail(GBBLAS_STATUS_CUDA_ERROR);

  // ---- capture: GEMM branch on s0, GEMV branch on s1
  if (cudaStreamBeginCapture(b->s0, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return fail(GBBLAS_STATUS_CUDA_ERROR);
  st = GBBLAS_STATUS_SUCCESS;
  if (cudaEventRecord(b->fork, b->s0) != cudaSuccess || cudaStreamWaitEvent(b->s1, b->fork, 0) != cudaSuccess)
    st = GBBLAS_STATUS_CUDA_ERROR;
  if (st == GBBLAS_STATUS_SUCCESS && b->gemm) st = tc_group_launch(c, b->gemm, b->s0);
  for (const gbblas_gemm_desc& g : b->fma_gemms) {
    if (st != GBBLAS_STATUS_SUCCESS) break;
    st = launch_gemm_fma<float>(c, g.M, g.N, g.K, g.A, g.rsa, g.csa, g.B, g.rsb, g.csb, g.C, g.rsc, g.csc, b->s0);
  }
  if (st == GBBLAS_STATUS_SUCCESS && ngemv > 0) st = launch_gemv_group_plan(c, b->gemv, b->s1);
  if (st == GBBLAS_STATUS_SUCCESS &&
      (cudaEventRecord(b->join, b->s1) != cudaSuccess || cudaStreamWaitEvent(b->s0, b->join, 0) != cudaSuccess))
    st = GBBLAS_STATUS_CUDA_ERROR;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->s0, &g);
  if (st != GBBLAS_STATUS_SUCCESS) {
    if (g) cudaGraphDestroy(g);
    return fail(st);
  }
  if (e != cudaSuccess) {
    set_error("gbblas_batch_create: stream capture failed: %s", cudaGetErrorString(e));
    return fail(GBBLAS_STATUS_CUDA_ERROR);
  }
  b->graph = g;
  if ((e = cudaGraphInstantiate(&b->exec, g, 0)) != cudaSuccess) {
    set_error("gbblas_batch_create: graph instantiation failed: %s", cudaGetErrorString(e));
    return fail(GBBLAS_STATUS_CUDA_ERROR);
  }
  *out = b;
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status gbblas_batch_run(gbblas_batch b, void* stream) {
  if (!b || !b->exec) {
    set_error("gbblas_batch_run: null batch");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  cudaError_t e = cudaGraphLaunch(b->exec, as_stream(stream));
  if (e != cudaSuccess) {
    set_error("gbblas_batch_run: cudaGraphLaunch failed: %s", cudaGetErrorString(e));
    return GBBLAS_STATUS_CUDA_ERROR;
  }
  count_launch();
  b->last = as_stream(stream);
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status gbblas_batch_sync(gbblas_batch b) {
  if (!b) {
    set_error("gbblas_batch_sync: null batch");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  GB_CUDA_TRY(cudaStreamSynchronize(b->last));
  int code = 0;
  if (b->gemm) {
    int* w = tc_group_error_word(b->gemm);
    if (w) {
      GB_CUDA_TRY(cudaMemcpy(&code, w, sizeof(int), cudaMemcpyDeviceToHost));
      if (code) {
        GB_CUDA_TRY(cudaMemset(w, 0, sizeof(int)));
        set_error("a batch kernel gave up a bounded device-side wait");
        return static_cast<gbblas_status>(code);
      }
    }
  }
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status gbblas_batch_destroy(gbblas_batch b) {
  if (!b) return GBBLAS_STATUS_SUCCESS;
  if (b->last) cudaStreamSynchronize(b->last);
  cudaStreamSynchronize(b->s0);
  cudaStreamSynchronize(b->s1);
  batch_free(b);
  return GBBLAS_STATUS_SUCCESS;
}

}  // extern "C"
