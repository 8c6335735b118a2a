/*
 * gbblas.h - C ABI of the GB300 (sm_103a) implementation of OpenMP-BLAS's
 * dense hot path: mtm (GEMM), mtv / vtm (GEMV) and dot, plus the streaming
 * operations beside it: outer product, transpose and element-wise ops.
 *
 * The C++ drop-in headers include/mtm.hpp, mtv.hpp, dot.hpp, outer.hpp,
 * trans.hpp and el_wise_op.hpp keep the reference's amt:: templates and call
 * the *_host entry points below; any other language binds these functions
 * directly (ctypes, cgo, JNI...).  No C++ or CUDA type appears in a
 * signature: sizes are int64_t, strides are in elements, streams are
 * `void*` holding a cudaStream_t (NULL = the legacy default stream).
 *
 * Conventions shared by every entry point
 *   - Status codes, never exceptions.  GBBLAS_STATUS_SUCCESS is 0.
 *   - Layouts follow uBLAS: GBBLAS_FIRST_ORDER is column-major (strides
 *     {1, rows}), GBBLAS_LAST_ORDER is row-major (strides {cols, 1}).
 *   - Plain entry points take DEVICE pointers and are asynchronous on the
 *     given stream.  *_host entry points take HOST pointers, stage through a
 *     library-owned device pool, and return after the result is back in host
 *     memory (the reference's "call the lambda and the result is there").
 *   - Sizes are explicit, so the C ABI rejects only what it cannot run
 *     (negative sizes, null pointers, output strides that would alias, an
 *     unknown enum) with GBBLAS_STATUS_INVALID_VALUE.  The reference's shape
 *     rules on tensors (operands are matrices / vectors, inner dimensions
 *     agree: reference include/mtm.hpp:234-250, include/mtv.hpp:126-144 and
 *     189-208, include/dot.hpp:196-214) are checked by the drop-in headers,
 *     which throw std::runtime_error when the callable is created, as the
 *     reference does.  GBBLAS_STATUS_SHAPE_MISMATCH is reserved for
 *     bindings that pass tensor extents through.
 *   - Results are deterministic: reductions use a fixed order, no atomics.
 */
#ifndef GBBLAS_H
#define GBBLAS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBBLAS_VERSION_MAJOR 0
#define GBBLAS_VERSION_MINOR 1

typedef enum gbblas_status {
  GBBLAS_STATUS_SUCCESS = 0,
  GBBLAS_STATUS_INVALID_VALUE = 1,   /* null pointer, negative size, bad enum */
  GBBLAS_STATUS_SHAPE_MISMATCH = 2,  /* operands are not matrices/vectors or dims disagree */
  GBBLAS_STATUS_ALLOC_FAILED = 3,    /* device or pinned-host allocation failed */
  GBBLAS_STATUS_CUDA_ERROR = 4,      /* a CUDA runtime call or launch failed */
  GBBLAS_STATUS_TIMEOUT = 5,         /* a bounded device-side wait gave up */
  GBBLAS_STATUS_NOT_SUPPORTED = 6,   /* combination not provided (e.g. FP8 with double) */
  GBBLAS_STATUS_NO_DEVICE = 7,       /* no sm_103 device visible */
  GBBLAS_STATUS_CANCELLED = 8        /* a served request was cancelled before it ran */
} gbblas_status;

typedef enum gbblas_layout {
  GBBLAS_FIRST_ORDER = 0, /* column-major, uBLAS layout::first_order */
  GBBLAS_LAST_ORDER = 1   /* row-major,    uBLAS layout::last_order  */
} gbblas_layout;

/* Arithmetic used by single-precision GEMM. */
typedef enum gbblas_accuracy {
  GBBLAS_ACCURACY_FP32 = 0,   /* FP32 FMA on the CUDA cores (the reference's arithmetic) */
  GBBLAS_ACCURACY_BF16X3 = 1, /* a = hi + lo in BF16, hi*hi + hi*lo + lo*hi on tcgen05
                                 tensor cores, FP32 accumulation in TMEM: ~16 significand
                                 bits per product, fastest FP32-input path */
  GBBLAS_ACCURACY_FP8 = 2,    /* low accuracy: E4M3 operands with one power-of-two
                                 scale per 128 elements along K (per row of A, per
                                 column of B), kind::f8f6f4 tcgen05 products, FP32
                                 accumulation; ~3 significand bits per operand and
                                 values below 2^-9 of their block's max flush to 0 */
  GBBLAS_ACCURACY_AUTO = 3,   /* FP32-accurate, whichever path the autotuner measured
                                 faster for the shape: FP32, or FP16X3 with a guard -
                                 outputs in a row of A (column of B) whose nonzero
                                 magnitudes span more than 14 + log2(K) binades, or
                                 that holds Inf / NaN, are recomputed with FP32 FMAs,
                                 so the error stays within (2^-19 + 2 K eps32) (|A||B|)_ij.
                                 GBBLAS_GEMM_AUTO=0 / 1 forces the FP32 / FP16X3 choice.
                                 Grouped and batched GEMMs: FP16X3 with the guard; served
                                 GEMMs the same, or one FP32 FMA kernel below 2^26
                                 multiply-adds */
  GBBLAS_ACCURACY_BF16X6 = 4, /* FP32-accurate: a = p0 + p1 + p2 in BF16 (all 24 bits),
                                 the six products p_i*p_j with i + j < 3 on tcgen05 */
  /* Double-precision GEMM (gbblas_dgemm_ex) only: */
  GBBLAS_ACCURACY_FP64 = 5,         /* FP64 FMA on the CUDA cores (the reference's arithmetic) */
  GBBLAS_ACCURACY_FP64_DIGITS7 = 6, /* Ozaki scheme on the BF16 tensor cores: every element
                                       scaled by a power of two per row of A / column of B
                                       and cut into 7 signed 8-bit digits, the 28 digit
                                       products of weight < 7 summed exactly; error at most
                                       about 4 K 2^-53 max_k|a_ik| max_k|b_kj| (the FP64
                                       bound has sum_k |a_ik||b_kj| there); K <= 2^20 */
  GBBLAS_ACCURACY_FP64_DIGITS8 = 7, /* the same with 8 digits (36 products): 2^-8 of that
                                       error; K <= 2^20 */
  /* Single-precision GEMM: */
  GBBLAS_ACCURACY_FP16X3 = 8        /* FP32-accurate, three tcgen05 products: every row of A
                                       and column of B scaled by a power of two into FP16's
                                       range and split a = h + l in FP16 (22 significand
                                       bits), h*h + h*l + l*h with FP32 accumulation */
} gbblas_accuracy;

/* ---------------------------------------------------------------- library */

/* Human-readable name of a status code (static storage). */
const char* gbblas_status_string(gbblas_status s);

/* Message of the last failure on the calling host thread ("" if none). */
const char* gbblas_last_error(void);

/* Version string, e.g. "gbblas 0.1 (sm_103a)". */
const char* gbblas_version(void);

/* Make the library ready on the current device: checks it is sm_103 and
 * creates the device pool.  Optional; every entry point does it lazily. */
gbblas_status gbblas_init(void);

/* Number of kernels this library has launched in this process (all
 * devices).  Benchmarks read it before and after a timed region. */
uint64_t gbblas_kernel_launches(void);

/* Wait for `stream` and report device-side failures of this library's
 * kernels on it: the tensor-core kernels bound every wait on the GPU and, if
 * one gives up, record GBBLAS_STATUS_TIMEOUT instead of hanging.  Returns
 * that status once (and clears it), else SUCCESS.  The *_host entry points
 * do this check themselves. */
gbblas_status gbblas_check_stream(void* stream);

/* Failure-detection self-test: one kernel on `stream` waits, bounded by
 * limit_us microseconds (1 .. 2,000,000), on a device barrier that nothing
 * completes, gives up and records GBBLAS_STATUS_TIMEOUT the way the
 * tensor-core kernels do.  The next gbblas_check_stream(stream) reports it;
 * the context stays usable.  Returns the launch status. */
gbblas_status gbblas_selftest_bounded_wait(int64_t limit_us, void* stream);

/* Release cached device and pinned-host memory held by the library for the
 * current device.  Safe to call at any time no call is in flight. */
gbblas_status gbblas_release_cache(void);

/* --------------------------------------------------------- seeded inputs
 * No counterpart in the reference (its drivers fill operands with ones,
 * src/mtm.cpp:204-205, and its tests with rand() % 100, test/test_utils.hpp:4-8).
 * This is the input recipe of this library's benchmark configurations and
 * parity tests, exported so that any caller can regenerate exactly the
 * operands a published figure was measured on.  Host code only: it needs no
 * GPU and touches no device memory. */

typedef enum gbblas_fill_kind {
  GBBLAS_FILL_UNIFORM = 0, /* U[-1,1): one draw x per value; double (x >> 11) * 2^-52 - 1,
                              float (x >> 40) * 2^-23 - 1 (both exact) */
  GBBLAS_FILL_WIDE = 1     /* s * m * 2^e from two draws d1, d2 per value: s = -1 if bit 63
                              of d1 is set, m = 1 + (d1 bits 11..62) * 2^-52 (double) or
                              1 + (d1 bits 40..62) * 2^-23 (float), e = ((d2 >> 32) mod 21) - 10 */
} gbblas_fill_kind;

/* One std::mt19937_64 seeded with `seed` draws nseg segments one after the
 * other, counts[s] values each; value i of segment s goes to out_f32[s][i]
 * and/or out_f64[s][i] (either array, or any entry of it, may be NULL: the
 * values are drawn and skipped).  The float and the double of one value
 * come from the same draws.  HOST pointers. */
gbblas_status gbblas_seeded_fill(uint64_t seed, int32_t kind, int64_t nseg, const int64_t* counts,
                                 float* const* out_f32, double* const* out_f64);

/* ------------------------------------------------------------------ mtm */

/* C += A * B (single precision).                      replaces amt::mtm,
 * reference include/mtm.hpp:208-267 (lambda body: mtm_helper, 116-206).
 * A is M x K with element strides (rsa, csa), B is K x N with (rsb, csb),
 * C is M x N with (rsc, csc): element (i, j) of C is C[i*rsc + j*csc].
 * Like the reference, C is ACCUMULATED into (zero it first for C = A*B).
 * Any strides are accepted; one unit stride per operand takes the fast
 * path.  `accuracy` picks the arithmetic (GBBLAS_ACCURACY_*). */
gbblas_status gbblas_sgemm(int64_t M, int64_t N, int64_t K, const float* A, int64_t rsa, int64_t csa,
                           const float* B, int64_t rsb, int64_t csb, float* C, int64_t rsc, int64_t csc,
                           gbblas_accuracy accuracy, void* stream);

/* C += A * B (double precision, FP64 arithmetic).      replaces amt::mtm
 * for double tensors, reference include/mtm.hpp:208-267 with
 * include/simd_loop.hpp:132-158. */
gbblas_status gbblas_dgemm(int64_t M, int64_t N, int64_t K, const double* A, int64_t rsa, int64_t csa,
                           const double* B, int64_t rsb, int64_t csb, double* C, int64_t rsc, int64_t csc,
                           void* stream);

/* gbblas_dgemm with a choice of arithmetic: GBBLAS_ACCURACY_FP64 (the same
 * as gbblas_dgemm), GBBLAS_ACCURACY_FP64_DIGITS7 or _DIGITS8 (the tensor-core
 * Ozaki scheme; NOT_SUPPORTED beyond its K limit).  Rows of A or columns of B
 * holding Inf or NaN make their outputs NaN on the digit paths. */
gbblas_status gbblas_dgemm_ex(int64_t M, int64_t N, int64_t K, const double* A, int64_t rsa, int64_t csa,
                              const double* B, int64_t rsb, int64_t csb, double* C, int64_t rsc, int64_t csc,
                              gbblas_accuracy accuracy, void* stream);

/* ------------------------------------------------------------------ mtv */

/* y = A * x for M x N dense A of layout `la`, x of length N, y of length M.
 *                                                   replaces amt::mtv,
 * reference include/mtv.hpp:100-162.  As in the reference, a column-major A
 * ACCUMULATES into y (include/mtv.hpp:15-70, simd_loop.hpp:62,74) and a
 * row-major A OVERWRITES y (include/mtv.hpp:72-98).  A's strides are taken
 * from the layout, not from the caller (reference line 154-156). */
gbblas_status gbblas_smtv(gbblas_layout la, int64_t M, int64_t N, const float* A, const float* x, float* y,
                          void* stream);
gbblas_status gbblas_dmtv(gbblas_layout la, int64_t M, int64_t N, const double* A, const double* x,
                          double* y, void* stream);

/* y = v^T * A for M x N dense A of layout `la`, v of length M, y of length N.
 *                                                   replaces amt::vtm,
 * reference include/mtv.hpp:164-236.  The reference intends this product but
 * builds A^T's strides from the wrong extent (lines 224-227), so it is right
 * only for square column-major A; this function computes y = v^T A for
 * every shape.  Overwrite/accumulate follow the reference's delegation: a
 * column-major A overwrites y, a row-major A accumulates into y. */
gbblas_status gbblas_svtm(gbblas_layout la, int64_t M, int64_t N, const float* A, const float* v, float* y,
                          void* stream);
gbblas_status gbblas_dvtm(gbblas_layout la, int64_t M, int64_t N, const double* A, const double* v,
                          double* y, void* stream);

/* General form behind mtv/vtm: y = op(A) * x (+ y if accumulate != 0),
 * op(A) = A if transpose == 0 else A^T, A M x N dense of layout la. */
gbblas_status gbblas_sgemv(gbblas_layout la, int transpose, int64_t M, int64_t N, const float* A,
                           const float* x, int accumulate, float* y, void* stream);
gbblas_status gbblas_dgemv(gbblas_layout la, int transpose, int64_t M, int64_t N, const double* A,
                           const double* x, int accumulate, double* y, void* stream);

/* ------------------------------------------------------------------ dot */

/* *result = sum_i a[i] * b[i] over n elements; result is a DEVICE pointer.
 *                                             replaces amt::dot_prod,
 * reference include/dot.hpp:176-224 (helper 143-174).  Single precision
 * keeps Kahan-compensated FP32 partials and combines them in FP64, so it is
 * at least as accurate as the reference's blocked OpenMP reduction.
 * n == 0 writes 0. */
gbblas_status gbblas_sdot(int64_t n, const float* a, const float* b, float* result, void* stream);
gbblas_status gbblas_ddot(int64_t n, const double* a, const double* b, double* result, void* stream);

/* Allocation-free form of gbblas_sdot.  No counterpart in the reference: the
 * reference's dot allocates nothing because it runs on the CPU; this entry
 * point exists for GPU callers that cannot allocate device memory when they
 * call (a caller-owned memory pool or a pre-reserved serving loop that must
 * not grow, or a foreign-language binding without access to cudaMalloc).
 * It computes the same result as gbblas_sdot but calls no cudaMalloc,
 * cudaFree or other allocating routine: its reduction scratch is one fixed
 * 33,024-byte device array inside the library (room for 4096 per-CTA
 * partials; a GB300 uses at most 608), which every GPU that loads the
 * library keeps until the process exits.  Inputs and the DEVICE `result`
 * pointer are the caller's, as for gbblas_sdot.
 *   - The first call on each device looks up that array's device address
 *     (cudaGetSymbolAddress); make that first call before any stream capture.
 *     Under CUDA's default lazy module loading, that first call may also be
 *     what loads the library's device code onto the device, and the CUDA
 *     driver allocates the array then.  So the promise "allocates nothing"
 *     holds from the second call on each device: make the first one during
 *     set-up, where allocation is still allowed.
 *   - The address is cached per device for the life of the process; after a
 *     cudaDeviceReset on a device this library must not be used on it again.
 *   - All calls share the one array and it keeps the last call's contents;
 *     the call clears the part that must start at zero.  Calls whose work
 *     overlaps on the GPU (different streams, or different host threads
 *     without ordering) race on the array: serialise them.
 *   - A device whose grid would need more than 4096 partials gets
 *     GBBLAS_STATUS_NOT_SUPPORTED with a message, never a partial result. */
gbblas_status gbblas_sdot_noalloc(int64_t n, const float* a, const float* b, float* result, void* stream);

/* amt::dot_prod_tuning_param (reference include/dot.hpp:92-141): the CPU
 * block sizes b1, b2, b3 have no meaning on the GPU; they are validated
 * (non-zero) and the call computes the same dot as gbblas_?dot. */
gbblas_status gbblas_sdot_tuning(int64_t n, const float* a, const float* b, int64_t b1, int64_t b2,
                                 int64_t b3, float* result, void* stream);
gbblas_status gbblas_ddot_tuning(int64_t n, const double* a, const double* b, int64_t b1, int64_t b2,
                                 int64_t b3, double* result, void* stream);

/* -------------------------------------------------------- outer product */

/* C += a b^T: C is the M x N matrix (dense, layout lc), a has M elements, b
 * has N.  Replaces amt::outer_prod, reference include/outer.hpp:67-119
 * (helper 14-65), which also accumulates into C.  Each element is one fused
 * multiply-add, c = fma(a_i, b_j, c), as in the reference's inner loop
 * (include/simd_loop.hpp:42-47).  DEVICE pointers. */
gbblas_status gbblas_souter(gbblas_layout lc, int64_t M, int64_t N, const float* a, const float* b, float* C,
                            void* stream);
gbblas_status gbblas_douter(gbblas_layout lc, int64_t M, int64_t N, const double* a, const double* b,
                            double* C, void* stream);

/* ------------------------------------------------------------ transpose */

/* C = A^T out of place: A is M x N with element (i, j) at A[i*rsa + j*csa];
 * C is N x M with element (j, i) at C[j*rsc + i*csc].  Any strides (both
 * layouts, padded leading dimensions); C must not overlap A.  Replaces
 * amt::transpose(c, a, num_threads), reference include/trans.hpp:103-145
 * (helper 33-65), which honours both tensors' strides the same way. */
gbblas_status gbblas_stranspose(int64_t M, int64_t N, const float* A, int64_t rsa, int64_t csa, float* C,
                                int64_t rsc, int64_t csc, void* stream);
gbblas_status gbblas_dtranspose(int64_t M, int64_t N, const double* A, int64_t rsa, int64_t csa, double* C,
                                int64_t rsc, int64_t csc, void* stream);

/* In place, square n x n (either layout: the storage is transposed).
 * Replaces amt::transpose(a, num_threads), reference include/trans.hpp:
 * 147-169 (helper 67-101).  The reference's in-place form is only correct
 * for square matrices (it swaps a[i*rows + j] with a[j*cols + i]); the drop-in
 * header rejects other shapes. */
gbblas_status gbblas_stranspose_inplace(int64_t n, float* A, void* stream);
gbblas_status gbblas_dtranspose_inplace(int64_t n, double* A, void* stream);

/* ---------------------------------------------------------- element-wise */

typedef enum gbblas_ew_op {
  GBBLAS_EW_ADD = 0, /* std::plus       */
  GBBLAS_EW_SUB = 1, /* std::minus      */
  GBBLAS_EW_MUL = 2, /* std::multiplies */
  GBBLAS_EW_DIV = 3  /* std::divides (IEEE division) */
} gbblas_ew_op;

/* c[i] = a[i] op b[i] for i < n over the tensors' storage order.  Replaces
 * amt::el_op::add / sub / mul / div / apply / apply_ops, reference
 * include/el_wise_op.hpp:33-121 (which loops over c.size() elements of the
 * three tensors' storage).  DEVICE pointers; c may equal a or b. */
gbblas_status gbblas_sew(gbblas_ew_op op, int64_t n, const float* a, const float* b, float* c, void* stream);
gbblas_status gbblas_dew(gbblas_ew_op op, int64_t n, const double* a, const double* b, double* c, void* stream);

/* ------------------------------------------------------------- batching
 * Many independent problems in one launch.  No counterpart in the reference,
 * which runs one call at a time; these serve callers that would otherwise
 * loop over amt::mtm / amt::mtv (reference src/mtm.cpp:189-214,
 * src/mtv.cpp:173-201 call them once per size). */

/* One GEMM of a group: C += A * B with the strides of gbblas_sgemm
 * (DEVICE pointers). */
typedef struct gbblas_gemm_desc {
  int64_t M, N, K;
  const float* A;
  int64_t rsa, csa;
  const float* B;
  int64_t rsb, csb;
  float* C;
  int64_t rsc, csc;
} gbblas_gemm_desc;

/* One GEMV of a group: y = op(A) x (+ y if accumulate), A dense M x N of
 * layout `layout`, op(A) = A (transpose = 0, y has M entries) or A^T
 * (transpose = 1, y has N entries).  DEVICE pointers. */
typedef struct gbblas_gemv_desc {
  int32_t layout;
  int32_t transpose;
  int32_t accumulate;
  int32_t reserved;
  int64_t M, N;
  const float* A;
  const float* x;
  float* y;
} gbblas_gemv_desc;

/* All GEMMs in one persistent tensor-core launch (accuracy BF16X3, BF16X6,
 * FP16X3, FP8 or AUTO = FP16X3 with its guard; FP32 runs them one by one on
 * the CUDA cores).
 * Problems may not overlap their C. */
gbblas_status gbblas_sgemm_grouped(const gbblas_gemm_desc* descs, int64_t count, gbblas_accuracy accuracy,
                                   void* stream);

/* All GEMVs in one persistent launch (row-streaming forms); column-streaming
 * forms run as per-problem launches on the same stream. */
gbblas_status gbblas_sgemv_grouped(const gbblas_gemv_desc* descs, int64_t count, void* stream);

/* A batch: a fixed set of GEMMs and GEMVs planned once (tables uploaded,
 * tile schedule chosen by the autotuner) and captured into a CUDA graph whose
 * two branches - the grouped tensor-core GEMM and the grouped GEMV - run
 * concurrently.  gbblas_batch_run replays the graph on `stream`; operand
 * pointers are fixed at creation.  Like every GEMM here, each run
 * ACCUMULATES into the C matrices (and into y where accumulate is set). */
typedef struct gbblas_batch_s* gbblas_batch;
gbblas_status gbblas_batch_create(const gbblas_gemm_desc* gemms, int64_t ngemm, gbblas_accuracy accuracy,
                                  const gbblas_gemv_desc* gemvs, int64_t ngemv, gbblas_batch* out);
gbblas_status gbblas_batch_run(gbblas_batch batch, void* stream);
/* Wait for the batch's last run; GBBLAS_STATUS_TIMEOUT if one of its
 * tensor-core kernels gave up a bounded device-side wait. */
gbblas_status gbblas_batch_sync(gbblas_batch batch);
gbblas_status gbblas_batch_destroy(gbblas_batch batch);

/* -------------------------------------------------------------- serving
 * A request loop with continuous batching.  No counterpart in the
 * reference (it has no serving path); it serves callers that issue many
 * mtm / mtv / dot calls of mixed sizes and precisions concurrently.
 *
 * Requests are submitted from any host thread.  A scheduler thread admits
 * them in arrival order while their working set fits the free-HBM budget
 * and a stream slot is free, coalesces everything admitted in one round
 * into grouped launches (split-BF16 GEMMs in one persistent tensor-core
 * launch, float GEMVs in one grouped launch; FP64, FP32-FMA and dot
 * requests as their own kernels) on one of `streams` CUDA streams, so work
 * of successive rounds overlaps on the device.  A host function queued
 * behind each round stamps its requests complete.  Operands and results are
 * DEVICE memory, normally taken from the server's pool (gbblas_server_alloc).
 * Each result is identical whether a request runs alone or in a mix: every
 * kernel used reduces in an order fixed by the request's own shape. */

typedef enum gbblas_op {
  GBBLAS_OP_MTM = 0, /* C += A * B   (A M x K, B K x N, C M x N; all of layout `layout`) */
  GBBLAS_OP_MTV = 1, /* y  = A * x   (amt::mtv semantics; A M x N of layout `layout`) */
  GBBLAS_OP_VTM = 2, /* y  = v^T A   (amt::vtm semantics) */
  GBBLAS_OP_DOT = 3  /* *C = A . B   (n = M elements) */
} gbblas_op;

typedef enum gbblas_dtype { GBBLAS_F32 = 0, GBBLAS_F64 = 1 } gbblas_dtype;

typedef struct gbblas_request {
  int32_t op;       /* gbblas_op */
  int32_t dtype;    /* gbblas_dtype */
  int32_t accuracy; /* gbblas_accuracy of an MTM: float - AUTO = guarded split-FP16
                       (one FP32 FMA kernel below 2^26 multiply-adds);
                       double - FP64 = the FP64 pipes, FP64_DIGITS7 / 8 = unguarded
                       tensor-core digits, any other value gbblas_dgemm's default */
  int32_t layout;   /* gbblas_layout of the matrices */
  int64_t M, N, K;
  const void* A; /* MTM: A;  MTV/VTM: matrix;  DOT: a */
  const void* B; /* MTM: B;  MTV/VTM: x or v;  DOT: b */
  void* C;       /* MTM: C;  MTV/VTM: y;       DOT: 1-element result */
} gbblas_request;

typedef struct gbblas_server_config {
  int32_t streams;       /* light rounds in flight at once (default 16) */
  int32_t max_group;     /* requests per light round (default 256) */
  int64_t budget_bytes;  /* admission budget: operands + results + scratch of
                            requests in flight (default 64 GiB) */
  int64_t scratch_bytes; /* per-stream scratch reserved at start (default 1 GiB) */
  int32_t heavy_streams; /* heavy requests in flight at once (default 2) */
  int32_t heavy_sm_percent; /* share of the SMs the grid of a heavy request that is
                               not sliced may take (1..100; default 75): light
                               rounds keep the rest */
  int64_t heavy_us;      /* estimated GPU time (us) above which a request is
                            heavy: it runs alone on a low-priority stream while
                            light rounds (capped at this much estimated work)
                            run on high-priority streams (default 300) */
  int64_t slice_us;      /* a heavy tensor-core or digit GEMM runs on every SM as
                            launches over tile ranges of about this much estimated
                            work each, so light rounds get SMs between them
                            (default 200; < 0: no slices, the heavy_sm_percent
                            cap instead, which other heavy requests always get) */
} gbblas_server_config;

typedef struct gbblas_server_stats {
  int64_t submitted, completed, rejected, rounds;
  int64_t peak_inflight_bytes;
  double mean_round_size;
} gbblas_server_stats;

typedef struct gbblas_server_s* gbblas_server;

/* cfg may be NULL (defaults).  The server belongs to the current device. */
gbblas_status gbblas_server_create(const gbblas_server_config* cfg, gbblas_server* out);
/* Device memory from the server's pool (stream-ordered, kept resident). */
gbblas_status gbblas_server_alloc(gbblas_server s, int64_t bytes, void** ptr);
gbblas_status gbblas_server_free(gbblas_server s, void* ptr);
/* Enqueue; returns at once with a ticket.  Shape errors are reported here. */
gbblas_status gbblas_server_submit(gbblas_server s, const gbblas_request* r, uint64_t* ticket);
/* Block until the ticket's request is done; latency = completion - submit. */
gbblas_status gbblas_server_wait(gbblas_server s, uint64_t ticket, double* latency_s);
/* Submit reqs[i] at arrival_s[i] seconds after the call (non-decreasing),
 * from a native thread, wait for all, and write each latency (seconds). */
gbblas_status gbblas_server_run_trace(gbblas_server s, const gbblas_request* reqs, const double* arrival_s,
                                      int64_t n, double* latency_s);
gbblas_status gbblas_server_get_stats(gbblas_server s, gbblas_server_stats* out);
/* Where a finished request's latency went (seconds), for tail analysis:
 * times[0] queued (submit -> its round was formed), times[1] host launch
 * (the round's kernels being enqueued), times[2] device and completion
 * (enqueued -> the completion stamp), times[3] requests in its round.
 * A request that never ran (cancelled, rejected launch) reports zeros. */
gbblas_status gbblas_server_request_times(gbblas_server s, uint64_t ticket, double* times);
/* Cancel a request the server has not started: it leaves the queue and its
 * wait returns GBBLAS_STATUS_CANCELLED.  A request already admitted to a
 * round (its work may be on the GPU) or finished cannot be cancelled:
 * GBBLAS_STATUS_NOT_SUPPORTED, and its wait reports how it ended. */
gbblas_status gbblas_server_cancel(gbblas_server s, uint64_t ticket);

/* Host-side failure injection, for testing how a caller (and the server)
 * handle errors: nothing on the GPU is made to fail.  The next `count`
 * events of `kind` fail as if the CUDA call behind them had failed; the
 * server stays usable and later events succeed. */
typedef enum gbblas_inject {
  GBBLAS_INJECT_ALLOC = 0, /* gbblas_server_alloc returns GBBLAS_STATUS_ALLOC_FAILED */
  GBBLAS_INJECT_LAUNCH = 1 /* a round's launch fails before enqueuing anything: its requests
                              complete with GBBLAS_STATUS_CUDA_ERROR */
} gbblas_inject;
gbblas_status gbblas_server_inject(gbblas_server s, int32_t kind, int32_t count);
gbblas_status gbblas_server_destroy(gbblas_server s);

/* ------------------------------------------------ host-buffer entry points
 * Same operations on HOST pointers: inputs are copied to the device, the
 * kernel runs, outputs come back, and the call returns when host memory
 * holds the result.  Page-locked host buffers copy at full link speed;
 * pageable ones are staged.  These are what the amt:: drop-in headers call. */
gbblas_status gbblas_sgemm_host(int64_t M, int64_t N, int64_t K, const float* A, int64_t rsa, int64_t csa,
                                const float* B, int64_t rsb, int64_t csb, float* C, int64_t rsc, int64_t csc,
                                gbblas_accuracy accuracy);
gbblas_status gbblas_dgemm_host(int64_t M, int64_t N, int64_t K, const double* A, int64_t rsa, int64_t csa,
                                const double* B, int64_t rsb, int64_t csb, double* C, int64_t rsc,
                                int64_t csc);
gbblas_status gbblas_dgemm_ex_host(int64_t M, int64_t N, int64_t K, const double* A, int64_t rsa, int64_t csa,
                                   const double* B, int64_t rsb, int64_t csb, double* C, int64_t rsc,
                                   int64_t csc, gbblas_accuracy accuracy);
gbblas_status gbblas_smtv_host(gbblas_layout la, int64_t M, int64_t N, const float* A, const float* x,
                               float* y);
gbblas_status gbblas_dmtv_host(gbblas_layout la, int64_t M, int64_t N, const double* A, const double* x,
                               double* y);
gbblas_status gbblas_svtm_host(gbblas_layout la, int64_t M, int64_t N, const float* A, const float* v,
                               float* y);
gbblas_status gbblas_dvtm_host(gbblas_layout la, int64_t M, int64_t N, const double* A, const double* v,
                               double* y);
gbblas_status gbblas_sdot_host(int64_t n, const float* a, const float* b, float* result);
gbblas_status gbblas_ddot_host(int64_t n, const double* a, const double* b, double* result);
gbblas_status gbblas_souter_host(gbblas_layout lc, int64_t M, int64_t N, const float* a, const float* b,
                                 float* C);
gbblas_status gbblas_douter_host(gbblas_layout lc, int64_t M, int64_t N, const double* a, const double* b,
                                 double* C);
gbblas_status gbblas_stranspose_host(int64_t M, int64_t N, const float* A, int64_t rsa, int64_t csa, float* C,
                                     int64_t rsc, int64_t csc);
gbblas_status gbblas_dtranspose_host(int64_t M, int64_t N, const double* A, int64_t rsa, int64_t csa, double* C,
                                     int64_t rsc, int64_t csc);
gbblas_status gbblas_stranspose_inplace_host(int64_t n, float* A);
gbblas_status gbblas_dtranspose_inplace_host(int64_t n, double* A);
gbblas_status gbblas_sew_host(gbblas_ew_op op, int64_t n, const float* a, const float* b, float* c);
gbblas_status gbblas_dew_host(gbblas_ew_op op, int64_t n, const double* a, const double* b, double* c);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* GBBLAS_H */
