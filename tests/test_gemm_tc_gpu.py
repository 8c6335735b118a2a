"""GEMM on the tcgen05 tensor cores from FP32 operands split into BF16
pieces, through the C ABI: GBBLAS_ACCURACY_BF16X3 (two pieces, three
products) and GBBLAS_ACCURACY_BF16X6 (three pieces, six products).

* integer-valued golden cases of the reference (|x| <= 99 is exact in BF16,
  so hi*hi is exact and every sum below 2^24 is exact): bit equality;
* random U[-1,1) shapes, all layout mixes, ragged sizes, against FP64 with
  the split-BF16 bound written below;
* the 1024^3 plain-mtm config: error reported against plain FP32.
"""
import numpy as np
import pytest

from oracle import oracle as O

import _golden as G

pytestmark = pytest.mark.gpu

BF16X3 = 1
BF16X6 = 4
FP16X3 = 8
MODES = [BF16X3, BF16X6, FP16X3]

# Per-product error of hi*hi + hi*lo + lo*hi: the dropped lo*lo and the split
# residuals are each <= 2^-16 of |a||b| (BF16 keeps 8 significant bits, so
# |a - hi| <= 2^-9 |a| and |a - hi - lo| <= 2^-17 |a|); FP32 accumulation adds
# K * eps32 at most.  Tolerance: 2^-14 + 2 K eps32 times (|A||B|)_ij.
def split_tol(absA, absB, K, mode=BF16X3):
    if mode == FP16X3:
        # rows / columns scaled by 2^(15 - e) into FP16's range; h + l keeps 22
        # bits of a normal element (|a - h - l| <= 2^-22 |a|), and an element's
        # lo in FP16's subnormal range is off by at most 2^-25 of 2^(e - 15);
        # the dropped l*l is below 2^-22 |a||b|
        sa = np.ldexp(1.0, np.frexp(absA.max(axis=1) if absA.shape[1] else np.zeros(absA.shape[0]))[1])
        sb = np.ldexp(1.0, np.frexp(absB.max(axis=0) if absB.shape[0] else np.zeros(absB.shape[1]))[1])
        return ((2.0 ** -19 + 2 * K * np.finfo(np.float32).eps) * (absA @ absB) +
                2.0 ** -38 * max(K, 1) * np.outer(sa, sb))
    if mode == BF16X6:  # all 24 bits kept; dropped products below 2^-23 of |a||b|
        return (2.0 ** -21 + 2 * K * np.finfo(np.float32).eps) * (absA @ absB)
    return (2.0 ** -14 + 2 * K * np.finfo(np.float32).eps) * (absA @ absB)


def run(torch, A, B, C0, la, lb, lc, accuracy=BF16X3):
    import gbblas
    M, K = A.shape
    N = B.shape[1]
    tA = torch.from_numpy(O.to_layout(A, la)).cuda()
    tB = torch.from_numpy(O.to_layout(B, lb)).cuda()
    tC = torch.from_numpy(O.to_layout(C0, lc).copy()).cuda()
    rsa, csa = O.strides(M, K, la)
    rsb, csb = O.strides(K, N, lb)
    rsc, csc = O.strides(M, N, lc)
    gbblas.call("gbblas_sgemm", M, N, K, tA.data_ptr(), rsa, csa, tB.data_ptr(), rsb, csb, tC.data_ptr(),
                rsc, csc, accuracy, None)
    gbblas.call("gbblas_check_stream", None)
    return O.from_layout(tC.cpu().numpy(), M, N, lc)


@pytest.mark.parametrize("mode", MODES)
def test_single_tile_first(cuda, mode):
    """One 128 x 256 x 64 tile: the smallest case the kernel runs."""
    rng = np.random.default_rng(0)
    A = rng.integers(-8, 9, (128, 64)).astype(np.float32)
    B = rng.integers(-8, 9, (64, 256)).astype(np.float32)
    Z = np.zeros((128, 256), np.float32)
    got = run(cuda, A, B, Z, 1, 1, 1, accuracy=mode)
    np.testing.assert_array_equal(got, A @ B)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("name", [n for n in G.names("mtm_float32") if "uniform" not in n])
def test_golden_integer_cases_exact(cuda, name, mode):
    c = G.case(name)
    A, B, C0 = c["A"].astype(np.float32), c["B"].astype(np.float32), c["C0"].astype(np.float32)
    got = run(cuda, A, B, C0, int(c["la"]), int(c["lb"]), int(c["lc"]), accuracy=mode)
    np.testing.assert_array_equal(got, c["C"])


SHAPES = [(1, 1, 1), (5, 7, 3), (100, 200, 300), (128, 256, 64), (129, 257, 65), (300, 100, 1000),
          (256, 512, 2048), (1000, 1000, 1000)]


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("lc,la,lb", [(1, 1, 1), (0, 0, 0), (1, 0, 1), (0, 1, 0)])
def test_random_vs_fp64(cuda, shape, lc, la, lb, mode):
    M, N, K = shape
    rng = np.random.default_rng(M + 3 * N + 7 * K)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    C0 = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    got = run(cuda, A, B, C0, la, lb, lc, accuracy=mode).astype(np.float64)
    exact = A.astype(np.float64) @ B.astype(np.float64) + C0
    tol = split_tol(np.abs(A).astype(np.float64), np.abs(B).astype(np.float64), K, mode) + \
        np.abs(C0) * np.finfo(np.float32).eps * 2
    err = np.abs(got - exact)
    assert np.all(err <= tol), f"max err/tol {np.max(err / tol):.3g}"


@pytest.mark.parametrize("mode", MODES)
def test_wide_range_values(cuda, mode):
    """Entries s * m * 2^e, e uniform in [-10, 10]: relative accuracy holds
    across binades (the split keeps each element's own exponent)."""
    rng = np.random.default_rng(5)
    M = N = K = 384

    def wide(shape):
        s = rng.choice([-1.0, 1.0], shape)
        m = rng.uniform(1, 2, shape)
        e = rng.integers(-10, 11, shape)
        return (s * m * np.exp2(e)).astype(np.float32)

    A, B = wide((M, K)), wide((K, N))
    Z = np.zeros((M, N), np.float32)
    got = run(cuda, A, B, Z, 1, 1, 1, accuracy=mode).astype(np.float64)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    tol = split_tol(np.abs(A).astype(np.float64), np.abs(B).astype(np.float64), K, mode)
    assert np.all(np.abs(got - exact) <= tol)


def test_1024_error_vs_plain_fp32(cuda):
    """M = N = K = 1024, U[-1,1) seed 0, normwise error against FP64:
    six products (all 24 bits) are at least as accurate as plain FP32 (within
    10 %); three products (~16 bits) stay within 8x of it."""
    rng = np.random.default_rng(0)
    A = rng.uniform(-1, 1, (1024, 1024)).astype(np.float32)
    B = rng.uniform(-1, 1, (1024, 1024)).astype(np.float32)
    Z = np.zeros((1024, 1024), np.float32)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64)
    e3 = np.max(np.abs(run(cuda, A, B, Z, 1, 1, 1, accuracy=BF16X3) - exact) / scale)
    e6 = np.max(np.abs(run(cuda, A, B, Z, 1, 1, 1, accuracy=BF16X6) - exact) / scale)
    e_fp32 = np.max(np.abs(run(cuda, A, B, Z, 1, 1, 1, accuracy=0) - exact) / scale)
    print(f"normwise max error: bf16x3 {e3:.3e}  bf16x6 {e6:.3e}  fp32 {e_fp32:.3e}")
    assert e6 <= 1.1 * e_fp32
    assert e3 <= 8 * e_fp32


def test_auto_accuracy_picks_an_fp32_accurate_path(cuda):
    """AUTO runs whichever FP32-accurate path the autotuner measured faster
    for the shape bucket: its result is bit-identical to that path's (on
    U[-1,1) operands at K = 1024 every row and column is within the FP16
    split's span, so its guard changes nothing)."""
    rng = np.random.default_rng(10)
    A = rng.uniform(-1, 1, (1024, 1024)).astype(np.float32)
    B = rng.uniform(-1, 1, (1024, 1024)).astype(np.float32)
    Z = np.zeros((1024, 1024), np.float32)
    auto = run(cuda, A, B, Z, 1, 1, 1, accuracy=3)
    f16 = run(cuda, A, B, Z, 1, 1, 1, accuracy=FP16X3)
    fma = run(cuda, A, B, Z, 1, 1, 1, accuracy=0)
    assert np.array_equal(auto, f16) or np.array_equal(auto, fma)


def _auto_tc(torch, monkeypatch, A, B, C0, la=1, lb=1, lc=1):
    monkeypatch.setenv("GBBLAS_GEMM_AUTO", "1")  # AUTO on the tensor cores: the guarded FP16 split
    return run(torch, A, B, C0, la, lb, lc, accuracy=3)


@pytest.mark.parametrize("K", [512, 2048])
@pytest.mark.parametrize("lc,la,lb", [(1, 1, 1), (0, 0, 0), (1, 0, 1)])
def test_auto_guard_recomputes_out_of_span_rows_and_columns(cuda, monkeypatch, lc, la, lb, K):
    """Rows of A and columns of B mixing magnitudes far apart (one entry of
    2^20 among entries of 2^-20, beyond the FP16 split's span at this K) fall
    back to FP32 FMAs: AUTO meets (2^-19 + 2 K eps32)(|A||B|) everywhere,
    while the plain FP16 split misses it on those rows and columns (the big
    entry meets a zero on the other side, so the small entries, which the
    row's scale pushes into FP16's subnormal range, make the whole result);
    every other output equals the plain FP16 split's bit for bit.  At
    K = 2048 the K-contiguous operands (row-major A, column-major B) take the
    one-pass preparation, which makes the guard's decisions itself."""
    rng = np.random.default_rng(21)
    M, N = 300, 260
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    bad_rows, bad_cols = [3, 150, 299], [0, 77, 259]
    for r in bad_rows:
        A[r] = rng.uniform(-1, 1, K).astype(np.float32) * 2.0 ** -20
        A[r, r % K] = 2.0 ** 20
        B[r % K, :] = 0.0
    for c in bad_cols:
        B[:, c] = rng.uniform(-1, 1, K).astype(np.float32) * 2.0 ** -20
        B[(7 * c) % K, c] = 2.0 ** 20
        A[:, (7 * c) % K] = 0.0
    C0 = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    # the guarded split never cuts K; the plain one must not either for the
    # bit-for-bit comparison below (split-K sums K in parts)
    monkeypatch.setenv("GBBLAS_TC_SPLITK", "1")
    got = _auto_tc(cuda, monkeypatch, A, B, C0, la, lb, lc).astype(np.float64)
    plain = run(cuda, A, B, C0, la, lb, lc, accuracy=FP16X3).astype(np.float64)
    exact = A.astype(np.float64) @ B.astype(np.float64) + C0
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64) + np.abs(C0)
    tol = (2.0 ** -19 + 2 * K * np.finfo(np.float32).eps) * scale
    assert np.all(np.abs(got - exact) <= tol), np.max(np.abs(got - exact) / tol)
    assert np.any(np.abs(plain - exact) > tol)  # the guard was needed
    keep = np.ones((M, N), bool)
    keep[bad_rows, :] = False
    keep[:, bad_cols] = False
    np.testing.assert_array_equal(got[keep], plain[keep])


def test_auto_guard_inf_and_nan_rows(cuda, monkeypatch):
    """Rows holding Inf or NaN are recomputed with FP32 FMAs: their outputs
    are non-finite exactly where the FMA path's are; other rows stay finite
    and within the bound."""
    rng = np.random.default_rng(22)
    M, N, K = 256, 256, 256
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    A[5, 9] = np.inf
    A[200, 0] = np.nan
    Z = np.zeros((M, N), np.float32)
    got = _auto_tc(cuda, monkeypatch, A, B, Z)
    fma = run(cuda, A, B, Z, 1, 1, 1, accuracy=0)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(fma))
    np.testing.assert_array_equal(np.isinf(got), np.isinf(fma))
    ok = np.ones(M, bool)
    ok[[5, 200]] = False
    exact = A[ok].astype(np.float64) @ B.astype(np.float64)
    scale = np.abs(A[ok]).astype(np.float64) @ np.abs(B).astype(np.float64)
    assert np.all(np.abs(got[ok] - exact) <= (2.0 ** -19 + 2 * K * np.finfo(np.float32).eps) * scale)


@pytest.mark.parametrize("K", [16, 1024])
def test_auto_guard_wide_range_operands(cuda, monkeypatch, K):
    """s * m * 2^e operands (e in [-10, 10]: rows span up to 20 binades): at
    K = 16 the FP16 split's span is 14 + 4 = 18 and most rows and columns are
    recomputed with FP32 FMAs; at K = 1024 (span 24) none is and the result
    is the plain FP16 split's.  Both within the bound."""
    rng = np.random.default_rng(23 + K)
    M = N = 320

    def wide(shape):
        return (rng.choice([-1.0, 1.0], shape) * rng.uniform(1, 2, shape) *
                np.exp2(rng.integers(-10, 11, shape))).astype(np.float32)
    A, B = wide((M, K)), wide((K, N))
    Z = np.zeros((M, N), np.float32)
    got = _auto_tc(cuda, monkeypatch, A, B, Z).astype(np.float64)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64)
    assert np.all(np.abs(got - exact) <= (2.0 ** -19 + 2 * K * np.finfo(np.float32).eps) * scale)
    if K == 1024:
        np.testing.assert_array_equal(got, run(cuda, A, B, Z, 1, 1, 1, accuracy=FP16X3))


def test_auto_accuracy_small_uses_fp32_path(cuda):
    rng = np.random.default_rng(9)
    A = rng.uniform(-1, 1, (33, 17)).astype(np.float32)
    B = rng.uniform(-1, 1, (17, 9)).astype(np.float32)
    Z = np.zeros((33, 9), np.float32)
    np.testing.assert_array_equal(run(cuda, A, B, Z, 1, 1, 1, accuracy=3), run(cuda, A, B, Z, 1, 1, 1, accuracy=0))


@pytest.mark.parametrize("mode", [BF16X6, FP16X3])
@pytest.mark.parametrize("dataset", ["uniform", "wide"])
def test_six_products_at_most_fp32_max_relative_error(cuda, dataset, mode):
    """M = N = K = 1024 (seed 12): the six-product BF16 split's and the
    three-product FP16 split's largest elementwise relative error against
    FP64 is no larger than plain FP32's,
    on U[-1,1) and on s * m * 2^e (e in [-10, 10]) operands."""
    rng = np.random.default_rng(12)
    n = 1024
    if dataset == "uniform":
        A = rng.uniform(-1, 1, (n, n)).astype(np.float32)
        B = rng.uniform(-1, 1, (n, n)).astype(np.float32)
    else:
        def wide(shape):
            return (rng.choice([-1.0, 1.0], shape) * rng.uniform(1, 2, shape) *
                    np.exp2(rng.integers(-10, 11, shape))).astype(np.float32)
        A, B = wide((n, n)), wide((n, n))
    Z = np.zeros((n, n), np.float32)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    denom = np.maximum(np.abs(exact), 1e-300)
    r6 = np.max(np.abs(run(cuda, A, B, Z, 1, 1, 1, accuracy=mode) - exact) / denom)
    r32 = np.max(np.abs(run(cuda, A, B, Z, 1, 1, 1, accuracy=0) - exact) / denom)
    print(f"{dataset}: max relative error mode {mode} {r6:.3e}  fp32 {r32:.3e}")
    assert r6 <= r32


@pytest.mark.parametrize("mode", [BF16X3, BF16X6, FP16X3, 3, 2])
def test_sliced_launches_give_the_same_bits(cuda, monkeypatch, mode):
    """GBBLAS_GEMM_SLICES=n runs the GEMM kernel as n launches over
    consecutive tile ranges (what the serving loop does with heavy requests):
    every tile is computed the same way, so the bits do not change."""
    rng = np.random.default_rng(40 + mode)
    M, N, K = 1000, 700, 600
    if mode == 2:  # FP8: small integers, exact
        A = rng.integers(-8, 9, (M, K)).astype(np.float32)
        B = rng.integers(-8, 9, (K, N)).astype(np.float32)
    else:
        A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
        B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    C0 = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    if mode == 3:
        monkeypatch.setenv("GBBLAS_GEMM_AUTO", "1")
        A[17] *= 2.0 ** -30  # one out-of-span row under AUTO's guard
        A[17, 0] = 1.0
    whole = run(cuda, A, B, C0, 1, 1, 1, accuracy=mode)
    for n in (2, 5):
        monkeypatch.setenv("GBBLAS_GEMM_SLICES", str(n))
        np.testing.assert_array_equal(run(cuda, A, B, C0, 1, 1, 1, accuracy=mode), whole)
    monkeypatch.delenv("GBBLAS_GEMM_SLICES")


def _sgemm_strided(torch, A, B, lda, ldb, accuracy):
    """C = A B with A row-major of row stride lda >= K and B column-major of
    column stride ldb >= K (both K contiguous), C row-major, from zero."""
    import gbblas
    M, K = A.shape
    N = B.shape[1]
    hA = np.zeros((M, lda), np.float32)
    hA[:, :K] = A
    hB = np.zeros((N, ldb), np.float32)
    hB[:, :K] = B.T
    tA, tB = torch.from_numpy(hA).cuda(), torch.from_numpy(hB).cuda()
    tC = torch.zeros(M * N, device="cuda")
    gbblas.call("gbblas_sgemm", M, N, K, tA.data_ptr(), lda, 1, tB.data_ptr(), 1, ldb, tC.data_ptr(), N, 1,
                accuracy, None)
    gbblas.call("gbblas_check_stream", None)
    return tC.cpu().numpy().reshape(M, N)


@pytest.mark.parametrize("accuracy", [FP16X3, 3])
@pytest.mark.parametrize("shape", [(192, 320, 1024), (130, 260, 2052), (64, 96, 8192)])
def test_one_pass_preparation_matches_tile_preparation(cuda, monkeypatch, shape, accuracy):
    """The FP16 split prepares operands whose K is contiguous in one pass
    (16-byte aligned rows, K a multiple of 4, 1024 <= K <= 8192: row-major A,
    column-major B).  The same values with a row stride of K + 1 go through
    the scale and tile kernels instead.  Both write the same exponents and
    pieces (and, under AUTO's guard, the same out-of-span decisions: one
    row of A and one column of B are out of span here), so C is the same
    bit for bit."""
    if accuracy == 3:
        monkeypatch.setenv("GBBLAS_GEMM_AUTO", "1")  # AUTO on the tensor cores: the guarded FP16 split
    M, N, K = shape
    rng = np.random.default_rng(M + N + K)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    A[5] *= np.float32(2.0 ** -30)
    A[5, 3] = 2.0 ** 10
    B[:, 7] *= np.float32(2.0 ** -30)
    B[11, 7] = 2.0 ** 10
    one_pass = _sgemm_strided(cuda, A, B, K, K, accuracy)
    tiles = _sgemm_strided(cuda, A, B, K + 1, K + 1, accuracy)
    np.testing.assert_array_equal(one_pass, tiles)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    absA, absB = np.abs(A).astype(np.float64), np.abs(B).astype(np.float64)
    if accuracy == 3:
        tol = (2.0 ** -19 + 2 * K * np.finfo(np.float32).eps) * (absA @ absB)
    else:
        tol = split_tol(absA, absB, K, FP16X3)
        tol[5, :] = np.inf  # out of the plain split's span (the guard's rows)
        tol[:, 7] = np.inf
    assert np.all(np.abs(one_pass - exact) <= tol)


def _sgemm_mn_major(torch, A, B, lda, ldb, accuracy):
    """C = A B with A column-major of column stride lda >= M and B row-major
    of row stride ldb >= N (rows of A and of B^T contiguous), C row-major."""
    import gbblas
    M, K = A.shape
    N = B.shape[1]
    hA = np.zeros((K, lda), np.float32)
    hA[:, :M] = A.T
    hB = np.zeros((K, ldb), np.float32)
    hB[:, :N] = B
    tA, tB = torch.from_numpy(hA).cuda(), torch.from_numpy(hB).cuda()
    tC = torch.zeros(M * N, device="cuda")
    gbblas.call("gbblas_sgemm", M, N, K, tA.data_ptr(), 1, lda, tB.data_ptr(), ldb, 1, tC.data_ptr(), N, 1,
                accuracy, None)
    gbblas.call("gbblas_check_stream", None)
    return tC.cpu().numpy().reshape(M, N)


@pytest.mark.parametrize("accuracy", [FP16X3, 3])
@pytest.mark.parametrize("shape", [(128, 256, 64), (1028, 2052, 300), (96, 4100, 1000)])
def test_column_scale_matches_tile_scale(cuda, monkeypatch, shape, accuracy):
    """The FP16 split finds the row exponents of an operand whose rows are
    contiguous (column-major A, row-major B; 16-byte aligned, row count a
    multiple of 4) by a column reduction; with a leading dimension of
    M + 1 (N + 1) the tile kernel finds them.  Same exponents, same guard
    decisions (one row of A and one column of B out of span), so C is the
    same bit for bit."""
    if accuracy == 3:
        monkeypatch.setenv("GBBLAS_GEMM_AUTO", "1")  # AUTO on the tensor cores: the guarded FP16 split
    M, N, K = shape
    rng = np.random.default_rng(M + 2 * N + 3 * K)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    A[5] *= np.float32(2.0 ** -30)
    A[5, 3] = 2.0 ** 10
    B[:, 7] *= np.float32(2.0 ** -30)
    B[11, 7] = 2.0 ** 10
    col = _sgemm_mn_major(cuda, A, B, M, N, accuracy)
    tiles = _sgemm_mn_major(cuda, A, B, M + 1, N + 1, accuracy)
    np.testing.assert_array_equal(col, tiles)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    absA, absB = np.abs(A).astype(np.float64), np.abs(B).astype(np.float64)
    if accuracy == 3:
        tol = (2.0 ** -19 + 2 * K * np.finfo(np.float32).eps) * (absA @ absB)
    else:
        tol = split_tol(absA, absB, K, FP16X3)
        tol[5, :] = np.inf  # out of the plain split's span (the guard's rows)
        tol[:, 7] = np.inf
    assert np.all(np.abs(col - exact) <= tol)


@pytest.mark.parametrize("mode", [BF16X3, BF16X6])
@pytest.mark.parametrize("shape", [(192, 320, 1024), (130, 260, 2052), (200, 136, 100), (64, 96, 8192), (1, 5, 4)])
def test_row_split_matches_tile_preparation(cuda, shape, mode):
    """The BF16 split writes the pieces of an operand whose K is contiguous
    (16-byte aligned rows, K a multiple of 4) with one warp per row; the
    same values with a row stride of K + 1 go through the tile kernel.
    Same pieces, so C is the same bit for bit, and within the split's bound."""
    M, N, K = shape
    rng = np.random.default_rng(M + 5 * N + K + mode)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    rows = _sgemm_strided(cuda, A, B, K, K, mode)
    tiles = _sgemm_strided(cuda, A, B, K + 1, K + 1, mode)
    np.testing.assert_array_equal(rows, tiles)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    tol = split_tol(np.abs(A).astype(np.float64), np.abs(B).astype(np.float64), K, mode)
    assert np.all(np.abs(rows - exact) <= tol)
