// capi.cu - the extern "C" boundary (include/gbblas.h) and the host-side
// runtime behind it: per-device context, per-stream scratch, host staging,
// argument checking and status/error reporting.
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <string>

#include "common.cuh"
#include "tc_ptx.cuh"

namespace gbblas {

// ------------------------------------------------------------------ errors
namespace {
thread_local char g_err[512] = {0};
}

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}

const char* last_error() { return g_err; }

namespace {
std::atomic<uint64_t> g_launches{0};
}
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// ----------------------------------------------------------------- context
namespace {
std::mutex g_ctx_mu;
// Published once per device with a release store after construction; the
// fast path reads it with an acquire load, so two host threads making their
// first call at the same time never see a half-built context.
std::atomic<DeviceCtx*> g_ctx[64] = {};
}  // namespace

gbblas_status get_ctx(DeviceCtx** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) {
    set_error("no CUDA device: %s", cudaGetErrorString(e));
    return GBBLAS_STATUS_NO_DEVICE;
  }
  DeviceCtx* c = g_ctx[dev].load(std::memory_order_acquire);
  if (c) {
    *out = c;
    return GBBLAS_STATUS_SUCCESS;
  }
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  if (!g_ctx[dev].load(std::memory_order_relaxed)) {
    cudaDeviceProp p;
    GB_CUDA_TRY(cudaGetDeviceProperties(&p, dev));
    if (!(p.major == 10 && p.minor == 3)) {
      set_error("device %d is sm_%d%d; this library is built for sm_103a (GB300)", dev, p.major, p.minor);
      return GBBLAS_STATUS_NO_DEVICE;
    }
    DeviceCtx* n = new DeviceCtx();
    n->device = dev;
    n->num_sms = p.multiProcessorCount;
    n->cc_major = p.major;
    n->cc_minor = p.minor;
    n->smem_optin = p.sharedMemPerBlockOptin;
    int pma = 0;
    if (cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) pma = 0;
    n->pageable_access = pma;
    g_ctx[dev].store(n, std::memory_order_release);
  }
  *out = g_ctx[dev].load(std::memory_order_relaxed);
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status get_scratch(DeviceCtx* c, cudaStream_t stream, size_t bytes, void** out) {
  std::lock_guard<std::mutex> lk(c->mu);
  DeviceCtx::Scratch& s = c->scratch[stream];
  if (s.bytes < bytes) {
    size_t want = bytes < (1u << 20) ? (1u << 20) : bytes + bytes / 4;
    void* p = nullptr;
    cudaError_t e = cudaMallocAsync(&p, want, stream);
    if (e != cudaSuccess) {
      set_error("scratch allocation of %zu bytes failed: %s", want, cudaGetErrorString(e));
      return GBBLAS_STATUS_ALLOC_FAILED;
    }
    GB_CUDA_TRY(cudaMemsetAsync(p, 0, kScratchZeroBytes, stream));
    if (s.ptr) {
      // carry a device error status still unread in the old buffer over to
      // the new one, so gbblas_check_stream reports it after the growth
      GB_CUDA_TRY(cudaMemcpyAsync(static_cast<char*>(p) + kErrWordOffset, static_cast<char*>(s.ptr) + kErrWordOffset,
                                  sizeof(int), cudaMemcpyDeviceToDevice, stream));
      GB_CUDA_TRY(cudaFreeAsync(s.ptr, stream));
    }
    s.ptr = p;
    s.bytes = want;
  }
  *out = s.ptr;
  return GBBLAS_STATUS_SUCCESS;
}

void release_scratch(DeviceCtx* c, cudaStream_t stream) {
  std::lock_guard<std::mutex> lk(c->mu);
  auto it = c->scratch.find(stream);
  if (it == c->scratch.end()) return;
  if (it->second.ptr) cudaFreeAsync(it->second.ptr, stream);
  c->scratch.erase(it);
}

gbblas_status check_stream_errors(DeviceCtx* c, cudaStream_t stream) {
  GB_CUDA_TRY(cudaStreamSynchronize(stream));
  void* p = nullptr;
  {
    std::lock_guard<std::mutex> lk(c->mu);
    auto it = c->scratch.find(stream);
    if (it == c->scratch.end() || !it->second.ptr) return GBBLAS_STATUS_SUCCESS;
    p = it->second.ptr;
  }
  int code = 0;
  int* word = reinterpret_cast<int*>(static_cast<char*>(p) + kErrWordOffset);
  GB_CUDA_TRY(cudaMemcpy(&code, word, sizeof(int), cudaMemcpyDeviceToHost));
  if (code != 0) {
    GB_CUDA_TRY(cudaMemset(word, 0, sizeof(int)));
    set_error("a kernel on this stream gave up a bounded device-side wait (status %d)", code);
    return static_cast<gbblas_status>(code);
  }
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status get_stage(DeviceCtx* c, size_t bytes, void** out) {
  if (!c->host_stream) GB_CUDA_TRY(cudaStreamCreateWithFlags(&c->host_stream, cudaStreamNonBlocking));
  if (c->stage_bytes < bytes) {
    if (c->stage) {
      GB_CUDA_TRY(cudaStreamSynchronize(c->host_stream));
      GB_CUDA_TRY(cudaFree(c->stage));
      c->stage = nullptr;
      c->stage_bytes = 0;
    }
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
      set_error("staging allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
      return GBBLAS_STATUS_ALLOC_FAILED;
    }
    c->stage = p;
    c->stage_bytes = bytes;
  }
  *out = c->stage;
  return GBBLAS_STATUS_SUCCESS;
}

const void* host_read_view(DeviceCtx* c, const void* p) {
  const char* e = std::getenv("GBBLAS_HOST_DIRECT");
  if (!p || (e && e[0] == '0')) return nullptr;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();  // not a pointer the runtime knows: stage it
    return nullptr;
  }
  switch (at.type) {
    case cudaMemoryTypeHost:
      return at.devicePointer;  // page-locked: its mapped address (null if not mapped)
    case cudaMemoryTypeDevice:
    case cudaMemoryTypeManaged:
      return at.device == c->device ? p : nullptr;
    default:
      return c->pageable_access ? p : nullptr;
  }
}

namespace {

// ------------------------------------------------------- argument checks
gbblas_status bad(gbblas_status s, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  char buf[512];
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  set_error("%s", buf);
  return s;
}

bool layout_ok(gbblas_layout l) { return l == GBBLAS_FIRST_ORDER || l == GBBLAS_LAST_ORDER; }

// Elements spanned by a rows x cols operand with strides (rs, cs).
int64_t span(int64_t rows, int64_t cols, int64_t rs, int64_t cs) {
  if (rows <= 0 || cols <= 0) return 0;
  return (rows - 1) * rs + (cols - 1) * cs + 1;
}

template <typename T>
gbblas_status check_gemm(int64_t M, int64_t N, int64_t K, const T* A, int64_t rsa, int64_t csa, const T* B,
                         int64_t rsb, int64_t csb, T* C, int64_t rsc, int64_t csc) {
  if (M < 0 || N < 0 || K < 0) return bad(GBBLAS_STATUS_INVALID_VALUE, "gemm: negative size");
  if (rsa < 0 || csa < 0 || rsb < 0 || csb < 0 || rsc < 0 || csc < 0)
    return bad(GBBLAS_STATUS_INVALID_VALUE, "gemm: strides must be non-negative");
  if (M == 0 || N == 0) return GBBLAS_STATUS_SUCCESS;
  if (!C) return bad(GBBLAS_STATUS_INVALID_VALUE, "gemm: C is null");
  if (K > 0 && (!A || !B)) return bad(GBBLAS_STATUS_INVALID_VALUE, "gemm: A or B is null");
  if ((M > 1 && rsc == 0) || (N > 1 && csc == 0))
    return bad(GBBLAS_STATUS_INVALID_VALUE, "gemm: C strides must be non-zero (outputs would alias)");
  return GBBLAS_STATUS_SUCCESS;
}

template <typename T>
gbblas_status check_mv(gbblas_layout la, int64_t M, int64_t N, const T* A, const T* x, T* y) {
  if (!layout_ok(la)) return bad(GBBLAS_STATUS_INVALID_VALUE, "gemv: layout must be 0 or 1");
  if (M < 0 || N < 0) return bad(GBBLAS_STATUS_INVALID_VALUE, "gemv: negative size");
  if ((M > 0 && N > 0) && (!A || !x || !y)) return bad(GBBLAS_STATUS_INVALID_VALUE, "gemv: null pointer");
  return GBBLAS_STATUS_SUCCESS;
}

// y = op(A) x (+ y).  A is M x N dense in layout la.
template <typename T>
gbblas_status gemv_any(DeviceCtx* c, gbblas_layout la, bool transpose, int64_t M, int64_t N, const T* A,
                       const T* x, bool accumulate, T* y, cudaStream_t s) {
  const int64_t out_len = transpose ? N : M;
  const int64_t red_len = transpose ? M : N;
  if (out_len == 0) return GBBLAS_STATUS_SUCCESS;
  if (red_len == 0) {
    if (!accumulate) GB_CUDA_TRY(cudaMemsetAsync(y, 0, sizeof(T) * out_len, s));
    return GBBLAS_STATUS_SUCCESS;
  }
  // Row-major A: rows contiguous (lda = N).  Column-major: columns contiguous (lda = M).
  const bool rows_contig = (la == GBBLAS_LAST_ORDER) != transpose;
  const int64_t lda = la == GBBLAS_LAST_ORDER ? N : M;
  if (rows_contig) return launch_gemv_rows<T>(c, out_len, red_len, A, lda, x, y, accumulate, s);
  return launch_gemv_cols<T>(c, out_len, red_len, A, lda, x, y, accumulate, s);
}

}  // namespace

// Shapes where AUTO takes the guarded tensor-core digits for a double GEMM:
// K of at least 32 (and within the digit kernels' limit) where the digits'
// estimated time is the shorter.  FP64 pipes: about 4000 multiply-adds per
// us per SM (GB300: 2 DFMA per cycle per SM), over as many SMs as there are
// 64 x 64 tiles; measured 0.27 ms at 256^3 (16 tiles).  Digits: about 50 us
// of operand preparation and launches, then ~38 TFLOP/s.
bool dgemm_auto_digits(int64_t M, int64_t N, int64_t K, int num_sms) {
  if (K < 32 || K > dgemm_digits_max_k(7)) return false;
  const double macs = (double)M * (double)N * (double)K;
  const double tiles = (double)((M + 63) / 64) * (double)((N + 63) / 64);
  const double pipes_us = 5.0 + macs / (4000.0 * std::min(tiles, (double)std::max(num_sms, 1)));
  const double digits_us = 50.0 + 2.0 * macs / 38e6;
  return digits_us < pipes_us;
}

namespace {

// The arithmetic of gbblas_dgemm / _host (the reference's double mtm): AUTO,
// or the FP64 pipes throughout when GBBLAS_DGEMM_FP64=1.
gbblas_accuracy dgemm_default_accuracy() {
  const char* e = std::getenv("GBBLAS_DGEMM_FP64");
  return (e && e[0] == '1') ? GBBLAS_ACCURACY_FP64 : GBBLAS_ACCURACY_AUTO;
}

template <typename T>
gbblas_status gemm_any(DeviceCtx* c, int64_t M, int64_t N, int64_t K, const T* A, int64_t rsa, int64_t csa,
                       const T* B, int64_t rsb, int64_t csb, T* C, int64_t rsc, int64_t csc, gbblas_accuracy acc,
                       cudaStream_t s) {
  if (M == 0 || N == 0 || K == 0) return GBBLAS_STATUS_SUCCESS;
  if constexpr (std::is_same_v<T, double>) {
    // FP64_DIGITS7 / 8: the Ozaki scheme on the BF16 tensor cores.  AUTO:
    // its guarded form (the FP64 pipes' error bound, blocks that could miss
    // it recomputed on the pipes) where the shape amortises the operand
    // preparation, the FP64 pipes elsewhere.
    if (const int digits = dgemm_digits_count(acc))
      return launch_dgemm_digits(c, digits, false, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, s, 0,
                                 gemm_slices_env());
    if (acc == GBBLAS_ACCURACY_AUTO && dgemm_auto_digits(M, N, K, c->num_sms)) {
      // a shape beyond the digit kernels' grid, or digit planes that do not
      // fit in device memory, fall back to the FP64 pipes
      const gbblas_status st =
          launch_dgemm_digits(c, 7, true, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, s, 0, gemm_slices_env());
      if (st != GBBLAS_STATUS_ALLOC_FAILED && st != GBBLAS_STATUS_NOT_SUPPORTED) return st;
      cudaGetLastError();  // a failed allocation leaves no sticky error; clear the last one
    }
  }
  if constexpr (std::is_same_v<T, float>) {
    // BF16X3 / BF16X6 / FP16X3 / FP8 always take the tensor cores.  AUTO:
    // whichever FP32-accurate path the autotuner measured faster for this
    // shape bucket (FMA kernel or the guarded FP16 split).
    int mode = tc_mode(acc);
    if (acc == GBBLAS_ACCURACY_AUTO && tuned_gemm_auto(c, M, N, K) == 1) mode = kTcModeF16Guard;
    if (mode != 0) return launch_gemm_tc(c, mode, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, s);
    // FP32 on the FMA pipe: the tile shape the autotuner measured faster
    return launch_gemm_fma<T>(c, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, s, 0,
                              tuned_fma_tile(c, M, N, K, s));
  }
  return launch_gemm_fma<T>(c, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, s);
}

// ----------------------------------------------------------- host staging
size_t round256(size_t b) { return (b + 255) & ~size_t(255); }

struct HostGuard {
  DeviceCtx* c;
  std::unique_lock<std::mutex> lk;
  explicit HostGuard(DeviceCtx* c_) : c(c_), lk(c_->host_mu) {}
};

gbblas_status h2d(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes) GB_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
  return GBBLAS_STATUS_SUCCESS;
}
gbblas_status d2h(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes) GB_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
  return GBBLAS_STATUS_SUCCESS;
}

// The arithmetic choices each element type takes.
template <typename T>
gbblas_status check_accuracy(gbblas_accuracy acc) {
  if constexpr (std::is_same_v<T, float>) {
    if (((int)acc < 0 || (int)acc > 4) && acc != GBBLAS_ACCURACY_FP16X3)
      return bad(GBBLAS_STATUS_INVALID_VALUE, "gemm: unknown accuracy %d", (int)acc);
  } else {
    if (acc != GBBLAS_ACCURACY_FP64 && acc != GBBLAS_ACCURACY_AUTO && !dgemm_digits_count(acc))
      return bad(GBBLAS_STATUS_INVALID_VALUE, "dgemm: accuracy %d is not FP64, AUTO, FP64_DIGITS7 or FP64_DIGITS8",
                 (int)acc);
  }
  return GBBLAS_STATUS_SUCCESS;
}

template <typename T>
gbblas_status gemm_host(int64_t M, int64_t N, int64_t K, const T* A, int64_t rsa, int64_t csa, const T* B,
                        int64_t rsb, int64_t csb, T* C, int64_t rsc, int64_t csc, gbblas_accuracy acc) {
  GB_TRY(check_gemm<T>(M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc));
  GB_TRY(check_accuracy<T>(acc));
  if (M == 0 || N == 0 || K == 0) return GBBLAS_STATUS_SUCCESS;
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  HostGuard g(c);
  const size_t na = span(M, K, rsa, csa), nb = span(K, N, rsb, csb), nc = span(M, N, rsc, csc);
  void* base;
  GB_TRY(get_stage(c, round256(na * sizeof(T)) + round256(nb * sizeof(T)) + round256(nc * sizeof(T)), &base));
  T* dA = static_cast<T*>(base);
  T* dB = reinterpret_cast<T*>(static_cast<char*>(base) + round256(na * sizeof(T)));
  T* dC = reinterpret_cast<T*>(reinterpret_cast<char*>(dB) + round256(nb * sizeof(T)));
  cudaStream_t s = c->host_stream;
  GB_TRY(h2d(dA, A, na * sizeof(T), s));
  GB_TRY(h2d(dB, B, nb * sizeof(T), s));
  GB_TRY(h2d(dC, C, nc * sizeof(T), s));
  GB_TRY(gemm_any<T>(c, M, N, K, dA, rsa, csa, dB, rsb, csb, dC, rsc, csc, acc, s));
  GB_TRY(check_stream_errors(c, s));  // C on the host stays untouched if the GEMM gave up
  GB_TRY(d2h(C, dC, nc * sizeof(T), s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GBBLAS_STATUS_SUCCESS;
}

// The streaming *_host calls read the large operand (the matrix of a GEMV,
// both vectors of a dot) straight from host memory where the device can
// (host_read_view): the kernel's own loads then move the bytes over the host
// link while it computes, with no staging copy and no copy-then-compute
// serialisation; the result is the same bits, since the kernel, grid and
// reduction order are those of the device call.  Small operands (x, y, the
// dot's result) are staged: the kernels read x many times over.
template <typename T>
gbblas_status gemv_host(gbblas_layout la, bool transpose, int64_t M, int64_t N, const T* A, const T* x,
                        bool accumulate, T* y) {
  GB_TRY(check_mv<T>(la, M, N, A, x, y));
  const int64_t out_len = transpose ? N : M, in_len = transpose ? M : N;
  if (out_len == 0) return GBBLAS_STATUS_SUCCESS;
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  HostGuard g(c);
  const size_t na = (size_t)(M * N), nx = (size_t)in_len, ny = (size_t)out_len;
  const T* vA = na ? static_cast<const T*>(host_read_view(c, A)) : nullptr;
  if (vA && !aligned16(vA)) vA = nullptr;  // the staged copy keeps the kernel's 128-bit loads
  const size_t stage_a = vA ? 0 : round256(na * sizeof(T));
  void* base;
  GB_TRY(get_stage(c, stage_a + round256(nx * sizeof(T)) + round256(ny * sizeof(T)), &base));
  T* dA = vA ? const_cast<T*>(vA) : static_cast<T*>(base);
  T* dx = reinterpret_cast<T*>(static_cast<char*>(base) + stage_a);
  T* dy = reinterpret_cast<T*>(reinterpret_cast<char*>(dx) + round256(nx * sizeof(T)));
  cudaStream_t s = c->host_stream;
  if (!vA) GB_TRY(h2d(dA, A, na * sizeof(T), s));
  GB_TRY(h2d(dx, x, nx * sizeof(T), s));
  if (accumulate) GB_TRY(h2d(dy, y, ny * sizeof(T), s));
  GB_TRY(gemv_any<T>(c, la, transpose, M, N, dA, dx, accumulate, dy, s));
  GB_TRY(d2h(y, dy, ny * sizeof(T), s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GBBLAS_STATUS_SUCCESS;
}

template <typename T>
gbblas_status dot_host(int64_t n, const T* a, const T* b, T* result) {
  if (n < 0) return bad(GBBLAS_STATUS_INVALID_VALUE, "dot: negative size");
  if (!result || (n > 0 && (!a || !b))) return bad(GBBLAS_STATUS_INVALID_VALUE, "dot: null pointer");
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  HostGuard g(c);
  const size_t bytes = (size_t)n * sizeof(T);
  const T* va = n ? static_cast<const T*>(host_read_view(c, a)) : nullptr;
  const T* vb = n ? static_cast<const T*>(host_read_view(c, b)) : nullptr;
  if (!va || !vb || !aligned16(va) || !aligned16(vb)) va = vb = nullptr;  // both direct, 128-bit loads, or neither
  const size_t stage_a = va ? 0 : round256(bytes), stage_b = vb ? 0 : round256(bytes);
  void* base;
  GB_TRY(get_stage(c, stage_a + stage_b + 256, &base));
  T* da = va ? const_cast<T*>(va) : static_cast<T*>(base);
  T* db = vb ? const_cast<T*>(vb) : reinterpret_cast<T*>(static_cast<char*>(base) + stage_a);
  T* dr = reinterpret_cast<T*>(static_cast<char*>(base) + stage_a + stage_b);
  cudaStream_t s = c->host_stream;
  if (!va) GB_TRY(h2d(da, a, bytes, s));
  if (!vb) GB_TRY(h2d(db, b, bytes, s));
  GB_TRY(launch_dot<T>(c, n, da, db, dr, s));
  GB_TRY(d2h(result, dr, sizeof(T), s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GBBLAS_STATUS_SUCCESS;
}

template <typename T>
gbblas_status dot_dev(int64_t n, const T* a, const T* b, T* result, void* stream) {
  if (n < 0) return bad(GBBLAS_STATUS_INVALID_VALUE, "dot: negative size");
  if (!result || (n > 0 && (!a || !b))) return bad(GBBLAS_STATUS_INVALID_VALUE, "dot: null pointer");
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  return launch_dot<T>(c, n, a, b, result, as_stream(stream));
}

template <typename T>
gbblas_status gemv_dev(gbblas_layout la, bool transpose, int64_t M, int64_t N, const T* A, const T* x,
                       bool accumulate, T* y, void* stream) {
  GB_TRY(check_mv<T>(la, M, N, A, x, y));
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  return gemv_any<T>(c, la, transpose, M, N, A, x, accumulate, y, as_stream(stream));
}

template <typename T>
gbblas_status gemm_dev(int64_t M, int64_t N, int64_t K, const T* A, int64_t rsa, int64_t csa, const T* B,
                       int64_t rsb, int64_t csb, T* C, int64_t rsc, int64_t csc, gbblas_accuracy acc, void* stream) {
  GB_TRY(check_gemm<T>(M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc));
  GB_TRY(check_accuracy<T>(acc));
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  return gemm_any<T>(c, M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, acc, as_stream(stream));
}

// ---------------------------------------------- outer / transpose / element-wise
template <typename T>
gbblas_status check_outer(gbblas_layout lc, int64_t M, int64_t N, const T* a, const T* b, T* C) {
  if (!layout_ok(lc)) return bad(GBBLAS_STATUS_INVALID_VALUE, "outer: layout must be 0 or 1");
  if (M < 0 || N < 0) return bad(GBBLAS_STATUS_INVALID_VALUE, "outer: negative size");
  if (M > 0 && N > 0 && (!a || !b || !C)) return bad(GBBLAS_STATUS_INVALID_VALUE, "outer: null pointer");
  return GBBLAS_STATUS_SUCCESS;
}

// C (M x N, layout lc) += a b^T as a rank-1 update of contiguous rows:
// row-major C: rows of length N, u = a, v = b; column-major C: columns of
// length M, u = b, v = a (the operand swap of reference include/outer.hpp:110-114).
template <typename T>
gbblas_status outer_any(DeviceCtx* c, gbblas_layout lc, int64_t M, int64_t N, const T* a, const T* b, T* C,
                        cudaStream_t s) {
  if (lc == GBBLAS_LAST_ORDER) return launch_outer<T>(c, M, N, a, b, C, N, s);
  return launch_outer<T>(c, N, M, b, a, C, M, s);
}

template <typename T>
gbblas_status check_transpose(int64_t M, int64_t N, const T* A, int64_t rsa, int64_t csa, T* C, int64_t rsc,
                              int64_t csc) {
  if (M < 0 || N < 0) return bad(GBBLAS_STATUS_INVALID_VALUE, "transpose: negative size");
  if (rsa < 0 || csa < 0 || rsc < 0 || csc < 0)
    return bad(GBBLAS_STATUS_INVALID_VALUE, "transpose: strides must be non-negative");
  if (M == 0 || N == 0) return GBBLAS_STATUS_SUCCESS;
  if (!A || !C) return bad(GBBLAS_STATUS_INVALID_VALUE, "transpose: null pointer");
  if ((N > 1 && rsc == 0) || (M > 1 && csc == 0))
    return bad(GBBLAS_STATUS_INVALID_VALUE, "transpose: C strides must be non-zero (outputs would alias)");
  return GBBLAS_STATUS_SUCCESS;
}

template <typename T>
gbblas_status check_ew(gbblas_ew_op op, int64_t n, const T* a, const T* b, T* c) {
  if ((int)op < 0 || (int)op > 3) return bad(GBBLAS_STATUS_INVALID_VALUE, "element-wise: unknown operation %d", (int)op);
  if (n < 0) return bad(GBBLAS_STATUS_INVALID_VALUE, "element-wise: negative size");
  if (n > 0 && (!a || !b || !c)) return bad(GBBLAS_STATUS_INVALID_VALUE, "element-wise: null pointer");
  return GBBLAS_STATUS_SUCCESS;
}

template <typename T>
gbblas_status outer_dev(gbblas_layout lc, int64_t M, int64_t N, const T* a, const T* b, T* C, void* stream) {
  GB_TRY(check_outer<T>(lc, M, N, a, b, C));
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  return outer_any<T>(c, lc, M, N, a, b, C, as_stream(stream));
}

template <typename T>
gbblas_status transpose_dev(int64_t M, int64_t N, const T* A, int64_t rsa, int64_t csa, T* C, int64_t rsc,
                            int64_t csc, void* stream) {
  GB_TRY(check_transpose<T>(M, N, A, rsa, csa, C, rsc, csc));
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  return launch_transpose<T>(c, M, N, A, rsa, csa, C, rsc, csc, as_stream(stream));
}

template <typename T>
gbblas_status transpose_inplace_dev(int64_t n, T* A, void* stream) {
  if (n < 0) return bad(GBBLAS_STATUS_INVALID_VALUE, "transpose in place: negative size");
  if (n > 0 && !A) return bad(GBBLAS_STATUS_INVALID_VALUE, "transpose in place: null pointer");
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  return launch_transpose_square<T>(c, n, A, as_stream(stream));
}

template <typename T>
gbblas_status ew_dev(gbblas_ew_op op, int64_t n, const T* a, const T* b, T* out, void* stream) {
  GB_TRY(check_ew<T>(op, n, a, b, out));
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  return launch_ew<T>(c, op, n, a, b, out, as_stream(stream));
}

template <typename T>
gbblas_status outer_host(gbblas_layout lc, int64_t M, int64_t N, const T* a, const T* b, T* C) {
  GB_TRY(check_outer<T>(lc, M, N, a, b, C));
  if (M == 0 || N == 0) return GBBLAS_STATUS_SUCCESS;
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  HostGuard g(c);
  const size_t nc = (size_t)(M * N) * sizeof(T), na = (size_t)M * sizeof(T), nb = (size_t)N * sizeof(T);
  void* base;
  GB_TRY(get_stage(c, round256(nc) + round256(na) + round256(nb), &base));
  T* dC = static_cast<T*>(base);
  T* da = reinterpret_cast<T*>(static_cast<char*>(base) + round256(nc));
  T* db = reinterpret_cast<T*>(static_cast<char*>(base) + round256(nc) + round256(na));
  cudaStream_t s = c->host_stream;
  GB_TRY(h2d(dC, C, nc, s));
  GB_TRY(h2d(da, a, na, s));
  GB_TRY(h2d(db, b, nb, s));
  GB_TRY(outer_any<T>(c, lc, M, N, da, db, dC, s));
  GB_TRY(d2h(C, dC, nc, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GBBLAS_STATUS_SUCCESS;
}

template <typename T>
gbblas_status transpose_host(int64_t M, int64_t N, const T* A, int64_t rsa, int64_t csa, T* C, int64_t rsc,
                             int64_t csc) {
  GB_TRY(check_transpose<T>(M, N, A, rsa, csa, C, rsc, csc));
  if (M == 0 || N == 0) return GBBLAS_STATUS_SUCCESS;
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  HostGuard g(c);
  const int64_t sa = span(M, N, rsa, csa), sc = span(N, M, rsc, csc);
  const size_t na = (size_t)sa * sizeof(T), nc = (size_t)sc * sizeof(T);
  void* base;
  GB_TRY(get_stage(c, round256(na) + round256(nc), &base));
  T* dA = static_cast<T*>(base);
  T* dC = reinterpret_cast<T*>(static_cast<char*>(base) + round256(na));
  cudaStream_t s = c->host_stream;
  GB_TRY(h2d(dA, A, na, s));
  // a C with gaps between its elements keeps them: bring it over first
  if (sc != M * N) GB_TRY(h2d(dC, C, nc, s));
  GB_TRY(launch_transpose<T>(c, M, N, dA, rsa, csa, dC, rsc, csc, s));
  GB_TRY(d2h(C, dC, nc, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GBBLAS_STATUS_SUCCESS;
}

template <typename T>
gbblas_status transpose_inplace_host(int64_t n, T* A) {
  if (n < 0) return bad(GBBLAS_STATUS_INVALID_VALUE, "transpose in place: negative size");
  if (n == 0) return GBBLAS_STATUS_SUCCESS;
  if (!A) return bad(GBBLAS_STATUS_INVALID_VALUE, "transpose in place: null pointer");
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  HostGuard g(c);
  const size_t bytes = (size_t)(n * n) * sizeof(T);
  void* base;
  GB_TRY(get_stage(c, round256(bytes), &base));
  T* dA = static_cast<T*>(base);
  cudaStream_t s = c->host_stream;
  GB_TRY(h2d(dA, A, bytes, s));
  GB_TRY(launch_transpose_square<T>(c, n, dA, s));
  GB_TRY(d2h(A, dA, bytes, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GBBLAS_STATUS_SUCCESS;
}

template <typename T>
gbblas_status ew_host(gbblas_ew_op op, int64_t n, const T* a, const T* b, T* out) {
  GB_TRY(check_ew<T>(op, n, a, b, out));
  if (n == 0) return GBBLAS_STATUS_SUCCESS;
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  HostGuard g(c);
  const size_t bytes = (size_t)n * sizeof(T);
  void* base;
  GB_TRY(get_stage(c, 3 * round256(bytes), &base));
  T* da = static_cast<T*>(base);
  T* db = reinterpret_cast<T*>(static_cast<char*>(base) + round256(bytes));
  T* dc = reinterpret_cast<T*>(static_cast<char*>(base) + 2 * round256(bytes));
  cudaStream_t s = c->host_stream;
  GB_TRY(h2d(da, a, bytes, s));
  GB_TRY(h2d(db, b, bytes, s));
  GB_TRY(launch_ew<T>(c, op, n, da, db, dc, s));
  GB_TRY(d2h(out, dc, bytes, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GBBLAS_STATUS_SUCCESS;
}

// Waits on a barrier nothing arrives on, bounded by limit_ns, and records
// GBBLAS_STATUS_TIMEOUT in the stream's error word when the wait gives up.
__global__ void selftest_wait_kernel(uint64_t limit_ns, int* err) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int never = 0;
    if (!tc::mbar_wait_bounded(&bar, 0, &never, limit_ns)) atomicExch(err, (int)GBBLAS_STATUS_TIMEOUT);
  }
}
}  // namespace
}  // namespace gbblas

using namespace gbblas;

extern "C" {

const char* gbblas_status_string(gbblas_status s) {
  switch (s) {
    case GBBLAS_STATUS_SUCCESS: return "GBBLAS_STATUS_SUCCESS";
    case GBBLAS_STATUS_INVALID_VALUE: return "GBBLAS_STATUS_INVALID_VALUE";
    case GBBLAS_STATUS_SHAPE_MISMATCH: return "GBBLAS_STATUS_SHAPE_MISMATCH";
    case GBBLAS_STATUS_ALLOC_FAILED: return "GBBLAS_STATUS_ALLOC_FAILED";
    case GBBLAS_STATUS_CUDA_ERROR: return "GBBLAS_STATUS_CUDA_ERROR";
    case GBBLAS_STATUS_TIMEOUT: return "GBBLAS_STATUS_TIMEOUT";
    case GBBLAS_STATUS_NOT_SUPPORTED: return "GBBLAS_STATUS_NOT_SUPPORTED";
    case GBBLAS_STATUS_NO_DEVICE: return "GBBLAS_STATUS_NO_DEVICE";
    case GBBLAS_STATUS_CANCELLED: return "GBBLAS_STATUS_CANCELLED";
  }
  return "GBBLAS_STATUS_UNKNOWN";
}

const char* gbblas_last_error(void) { return gbblas::last_error(); }

const char* gbblas_version(void) { return "gbblas 0.1 (sm_103a)"; }

uint64_t gbblas_kernel_launches(void) { return gbblas::g_launches.load(); }

gbblas_status gbblas_init(void) {
  DeviceCtx* c;
  return get_ctx(&c);
}

gbblas_status gbblas_check_stream(void* stream) {
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  return check_stream_errors(c, as_stream(stream));
}


gbblas_status gbblas_selftest_bounded_wait(int64_t limit_us, void* stream) {
  if (limit_us < 1 || limit_us > 2000000) return bad(GBBLAS_STATUS_INVALID_VALUE, "selftest: limit out of range");
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  cudaStream_t s = as_stream(stream);
  void* scratch = nullptr;
  GB_TRY(get_scratch(c, s, kScratchZeroBytes, &scratch));
  int* err = reinterpret_cast<int*>(static_cast<char*>(scratch) + kErrWordOffset);
  selftest_wait_kernel<<<1, 32, 0, s>>>((uint64_t)limit_us * 1000ull, err);
  return check_launch("selftest_wait_kernel");
}

gbblas_status gbblas_release_cache(void) {
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  {
    std::lock_guard<std::mutex> lk(c->mu);
    for (auto& kv : c->scratch) {
      if (kv.second.ptr) GB_CUDA_TRY(cudaFreeAsync(kv.second.ptr, kv.first));
    }
    c->scratch.clear();
  }
  std::lock_guard<std::mutex> lk(c->host_mu);
  if (c->stage) {
    GB_CUDA_TRY(cudaStreamSynchronize(c->host_stream));
    GB_CUDA_TRY(cudaFree(c->stage));
    c->stage = nullptr;
    c->stage_bytes = 0;
  }
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status gbblas_sgemm(int64_t M, int64_t N, int64_t K, const float* A, int64_t rsa, int64_t csa, const float* B,
                           int64_t rsb, int64_t csb, float* C, int64_t rsc, int64_t csc, gbblas_accuracy accuracy,
                           void* stream) {
  return gemm_dev<float>(M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, accuracy, stream);
}

gbblas_status gbblas_dgemm(int64_t M, int64_t N, int64_t K, const double* A, int64_t rsa, int64_t csa,
                           const double* B, int64_t rsb, int64_t csb, double* C, int64_t rsc, int64_t csc,
                           void* stream) {
  return gemm_dev<double>(M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, dgemm_default_accuracy(), stream);
}

/* Double-precision GEMM with a choice of arithmetic (FP64 FMA or the
 * tensor-core digit scheme). */
gbblas_status gbblas_dgemm_ex(int64_t M, int64_t N, int64_t K, const double* A, int64_t rsa, int64_t csa,
                              const double* B, int64_t rsb, int64_t csb, double* C, int64_t rsc, int64_t csc,
                              gbblas_accuracy accuracy, void* stream) {
  return gemm_dev<double>(M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, accuracy, stream);
}

gbblas_status gbblas_smtv(gbblas_layout la, int64_t M, int64_t N, const float* A, const float* x, float* y,
                          void* stream) {
  return gemv_dev<float>(la, false, M, N, A, x, la == GBBLAS_FIRST_ORDER, y, stream);
}
gbblas_status gbblas_dmtv(gbblas_layout la, int64_t M, int64_t N, const double* A, const double* x, double* y,
                          void* stream) {
  return gemv_dev<double>(la, false, M, N, A, x, la == GBBLAS_FIRST_ORDER, y, stream);
}
gbblas_status gbblas_svtm(gbblas_layout la, int64_t M, int64_t N, const float* A, const float* v, float* y,
                          void* stream) {
  return gemv_dev<float>(la, true, M, N, A, v, la == GBBLAS_LAST_ORDER, y, stream);
}
gbblas_status gbblas_dvtm(gbblas_layout la, int64_t M, int64_t N, const double* A, const double* v, double* y,
                          void* stream) {
  return gemv_dev<double>(la, true, M, N, A, v, la == GBBLAS_LAST_ORDER, y, stream);
}
gbblas_status gbblas_sgemv(gbblas_layout la, int transpose, int64_t M, int64_t N, const float* A, const float* x,
                           int accumulate, float* y, void* stream) {
  return gemv_dev<float>(la, transpose != 0, M, N, A, x, accumulate != 0, y, stream);
}
gbblas_status gbblas_dgemv(gbblas_layout la, int transpose, int64_t M, int64_t N, const double* A,
                           const double* x, int accumulate, double* y, void* stream) {
  return gemv_dev<double>(la, transpose != 0, M, N, A, x, accumulate != 0, y, stream);
}

gbblas_status gbblas_sdot(int64_t n, const float* a, const float* b, float* result, void* stream) {
  return dot_dev<float>(n, a, b, result, stream);
}
gbblas_status gbblas_ddot(int64_t n, const double* a, const double* b, double* result, void* stream) {
  return dot_dev<double>(n, a, b, result, stream);
}
gbblas_status gbblas_sdot_tuning(int64_t n, const float* a, const float* b, int64_t b1, int64_t b2, int64_t b3,
                                 float* result, void* stream) {
  if (b1 <= 0 || b2 <= 0 || b3 <= 0) return bad(GBBLAS_STATUS_INVALID_VALUE, "dot_tuning: block sizes must be > 0");
  return dot_dev<float>(n, a, b, result, stream);
}
gbblas_status gbblas_ddot_tuning(int64_t n, const double* a, const double* b, int64_t b1, int64_t b2, int64_t b3,
                                 double* result, void* stream) {
  if (b1 <= 0 || b2 <= 0 || b3 <= 0) return bad(GBBLAS_STATUS_INVALID_VALUE, "dot_tuning: block sizes must be > 0");
  return dot_dev<double>(n, a, b, result, stream);
}

gbblas_status gbblas_sgemm_grouped(const gbblas_gemm_desc* descs, int64_t count, gbblas_accuracy accuracy,
                                   void* stream) {
  if (count < 0 || (count > 0 && !descs)) return bad(GBBLAS_STATUS_INVALID_VALUE, "gemm_grouped: bad arguments");
  if (((int)accuracy < 0 || (int)accuracy > 4) && accuracy != GBBLAS_ACCURACY_FP16X3)
    return bad(GBBLAS_STATUS_INVALID_VALUE, "gemm_grouped: unknown accuracy %d", (int)accuracy);
  for (int64_t i = 0; i < count; ++i) {
    const gbblas_gemm_desc& g = descs[i];
    GB_TRY(check_gemm<float>(g.M, g.N, g.K, g.A, g.rsa, g.csa, g.B, g.rsb, g.csb, g.C, g.rsc, g.csc));
  }
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  cudaStream_t s = as_stream(stream);
  if (accuracy == GBBLAS_ACCURACY_FP32) {
    for (int64_t i = 0; i < count; ++i) {
      const gbblas_gemm_desc& g = descs[i];
      GB_TRY(gemm_any<float>(c, g.M, g.N, g.K, g.A, g.rsa, g.csa, g.B, g.rsb, g.csb, g.C, g.rsc, g.csc,
                             GBBLAS_ACCURACY_FP32, s));
    }
    return GBBLAS_STATUS_SUCCESS;
  }
  // AUTO in a group: the split-FP16 GEMM with its guard (FP32-accurate on the tensor cores)
  const int mode = accuracy == GBBLAS_ACCURACY_AUTO ? kTcModeF16Guard : tc_mode(accuracy);
  return launch_gemm_tc_group(c, mode, descs, count, s);
}

gbblas_status gbblas_sgemv_grouped(const gbblas_gemv_desc* descs, int64_t count, void* stream) {
  if (count < 0 || (count > 0 && !descs)) return bad(GBBLAS_STATUS_INVALID_VALUE, "gemv_grouped: bad arguments");
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  return launch_gemv_group(c, descs, count, as_stream(stream));
}

gbblas_status gbblas_sgemm_host(int64_t M, int64_t N, int64_t K, const float* A, int64_t rsa, int64_t csa,
                                const float* B, int64_t rsb, int64_t csb, float* C, int64_t rsc, int64_t csc,
                                gbblas_accuracy accuracy) {
  return gemm_host<float>(M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, accuracy);
}
gbblas_status gbblas_dgemm_host(int64_t M, int64_t N, int64_t K, const double* A, int64_t rsa, int64_t csa,
                                const double* B, int64_t rsb, int64_t csb, double* C, int64_t rsc, int64_t csc) {
  return gemm_host<double>(M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, dgemm_default_accuracy());
}
gbblas_status gbblas_dgemm_ex_host(int64_t M, int64_t N, int64_t K, const double* A, int64_t rsa, int64_t csa,
                                   const double* B, int64_t rsb, int64_t csb, double* C, int64_t rsc, int64_t csc,
                                   gbblas_accuracy accuracy) {
  return gemm_host<double>(M, N, K, A, rsa, csa, B, rsb, csb, C, rsc, csc, accuracy);
}
gbblas_status gbblas_smtv_host(gbblas_layout la, int64_t M, int64_t N, const float* A, const float* x, float* y) {
  return gemv_host<float>(la, false, M, N, A, x, la == GBBLAS_FIRST_ORDER, y);
}
gbblas_status gbblas_dmtv_host(gbblas_layout la, int64_t M, int64_t N, const double* A, const double* x, double* y) {
  return gemv_host<double>(la, false, M, N, A, x, la == GBBLAS_FIRST_ORDER, y);
}
gbblas_status gbblas_svtm_host(gbblas_layout la, int64_t M, int64_t N, const float* A, const float* v, float* y) {
  return gemv_host<float>(la, true, M, N, A, v, la == GBBLAS_LAST_ORDER, y);
}
gbblas_status gbblas_dvtm_host(gbblas_layout la, int64_t M, int64_t N, const double* A, const double* v, double* y) {
  return gemv_host<double>(la, true, M, N, A, v, la == GBBLAS_LAST_ORDER, y);
}
gbblas_status gbblas_sdot_host(int64_t n, const float* a, const float* b, float* result) {
  return dot_host<float>(n, a, b, result);
}
gbblas_status gbblas_ddot_host(int64_t n, const double* a, const double* b, double* result) {
  return dot_host<double>(n, a, b, result);
}

gbblas_status gbblas_souter(gbblas_layout lc, int64_t M, int64_t N, const float* a, const float* b, float* C,
                            void* stream) {
  return outer_dev<float>(lc, M, N, a, b, C, stream);
}
gbblas_status gbblas_douter(gbblas_layout lc, int64_t M, int64_t N, const double* a, const double* b, double* C,
                            void* stream) {
  return outer_dev<double>(lc, M, N, a, b, C, stream);
}
gbblas_status gbblas_stranspose(int64_t M, int64_t N, const float* A, int64_t rsa, int64_t csa, float* C,
                                int64_t rsc, int64_t csc, void* stream) {
  return transpose_dev<float>(M, N, A, rsa, csa, C, rsc, csc, stream);
}
gbblas_status gbblas_dtranspose(int64_t M, int64_t N, const double* A, int64_t rsa, int64_t csa, double* C,
                                int64_t rsc, int64_t csc, void* stream) {
  return transpose_dev<double>(M, N, A, rsa, csa, C, rsc, csc, stream);
}
gbblas_status gbblas_stranspose_inplace(int64_t n, float* A, void* stream) {
  return transpose_inplace_dev<float>(n, A, stream);
}
gbblas_status gbblas_dtranspose_inplace(int64_t n, double* A, void* stream) {
  return transpose_inplace_dev<double>(n, A, stream);
}
gbblas_status gbblas_sew(gbblas_ew_op op, int64_t n, const float* a, const float* b, float* c, void* stream) {
  return ew_dev<float>(op, n, a, b, c, stream);
}
gbblas_status gbblas_dew(gbblas_ew_op op, int64_t n, const double* a, const double* b, double* c, void* stream) {
  return ew_dev<double>(op, n, a, b, c, stream);
}
gbblas_status gbblas_souter_host(gbblas_layout lc, int64_t M, int64_t N, const float* a, const float* b, float* C) {
  return outer_host<float>(lc, M, N, a, b, C);
}
gbblas_status gbblas_douter_host(gbblas_layout lc, int64_t M, int64_t N, const double* a, const double* b,
                                 double* C) {
  return outer_host<double>(lc, M, N, a, b, C);
}
gbblas_status gbblas_stranspose_host(int64_t M, int64_t N, const float* A, int64_t rsa, int64_t csa, float* C,
                                     int64_t rsc, int64_t csc) {
  return transpose_host<float>(M, N, A, rsa, csa, C, rsc, csc);
}
gbblas_status gbblas_dtranspose_host(int64_t M, int64_t N, const double* A, int64_t rsa, int64_t csa, double* C,
                                     int64_t rsc, int64_t csc) {
  return transpose_host<double>(M, N, A, rsa, csa, C, rsc, csc);
}
gbblas_status gbblas_stranspose_inplace_host(int64_t n, float* A) { return transpose_inplace_host<float>(n, A); }
gbblas_status gbblas_dtranspose_inplace_host(int64_t n, double* A) { return transpose_inplace_host<double>(n, A); }
gbblas_status gbblas_sew_host(gbblas_ew_op op, int64_t n, const float* a, const float* b, float* c) {
  return ew_host<float>(op, n, a, b, c);
}
gbblas_status gbblas_dew_host(gbblas_ew_op op, int64_t n, const double* a, const double* b, double* c) {
  return ew_host<double>(op, n, a, b, c);
}

}  // extern "C"
