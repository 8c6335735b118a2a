"""Double-precision GEMM on the BF16 tensor cores (Ozaki scheme), through
gbblas_dgemm_ex with GBBLAS_ACCURACY_FP64_DIGITS7 / _DIGITS8.

* integer-valued operands (a few significant bits per row): every digit
  product is kept and every sum is exact, so the result equals the exact
  product bit for bit - including operands whose digits are all +-127, which
  drive each group's 128-K sum in TMEM to its largest magnitude;
* random U[-1,1) shapes, ragged sizes and every layout mix, against the
  oracle's FP64 GEMM (the reference's algorithm) within the digit bound plus
  the FP64 bound;
* Inf / NaN rows and columns give NaN outputs, other outputs stay finite;
* C is accumulated into, like the reference's mtm.

Digit bound (S digits, row scale 2^e_i > max_k |a_ik|, column scale 2^f_j):
|C_ij - exact| <= (S + 1) 2^-8S K 2^(e_i + f_j) + 2 ulp.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

D7 = 6
D8 = 7
MODES = [D7, D8]
NDIG = {D7: 7, D8: 8}


def run(torch, A, B, C0, la, lb, lc, accuracy=D7):
    import gbblas
    M, K = A.shape
    N = B.shape[1]
    tA = torch.from_numpy(O.to_layout(A, la)).cuda()
    tB = torch.from_numpy(O.to_layout(B, lb)).cuda()
    tC = torch.from_numpy(O.to_layout(C0, lc).copy()).cuda()
    rsa, csa = O.strides(M, K, la)
    rsb, csb = O.strides(K, N, lb)
    rsc, csc = O.strides(M, N, lc)
    gbblas.call("gbblas_dgemm_ex", M, N, K, tA.data_ptr(), rsa, csa, tB.data_ptr(), rsb, csb, tC.data_ptr(),
                rsc, csc, accuracy, None)
    gbblas.call("gbblas_check_stream", None)
    return O.from_layout(tC.cpu().numpy(), M, N, lc)


def scales(A, B):
    """2^e_i per row of A and 2^f_j per column of B (frexp exponents of the maxima)."""
    ra = np.abs(A).max(axis=1) if A.shape[1] else np.zeros(A.shape[0])
    cb = np.abs(B).max(axis=0) if B.shape[0] else np.zeros(B.shape[1])
    return np.ldexp(1.0, np.frexp(ra)[1]), np.ldexp(1.0, np.frexp(cb)[1])


def digit_tol(A, B, C0, mode):
    S = NDIG[mode]
    K = A.shape[1]
    sa, sb = scales(A, B)
    eps = np.finfo(np.float64).eps
    fp64 = 2 * max(K, 1) * eps * (np.abs(A) @ np.abs(B) + np.abs(C0))  # the oracle's own error
    digits = (S + 1) * 2.0 ** (-8 * S) * K * np.outer(sa, sb)
    return digits + fp64 + 4 * eps * np.abs(A @ B + C0) + np.finfo(np.float64).tiny


def assert_digit_close(got, A, B, C0, la, lb, lc, mode, what=""):
    ref = O.gemm(A, B, C0, la, lb, lc)
    tol = digit_tol(A, B, C0, mode)
    err = np.abs(got - ref)
    bad = err > tol
    if bad.any():
        i = np.unravel_index(np.argmax(err / tol), err.shape)
        raise AssertionError(f"{what}: {bad.sum()} entries beyond the digit bound; worst at {i}: "
                             f"got {got[i]!r} ref {ref[i]!r} tol {tol[i]:.3g}")


@pytest.mark.parametrize("mode", MODES)
def test_integer_operands_exact(cuda, mode):
    rng = np.random.default_rng(11)
    M, N, K = 200, 70, 300
    A = rng.integers(-1000, 1001, (M, K)).astype(np.float64)
    B = rng.integers(-1000, 1001, (K, N)).astype(np.float64)
    C0 = rng.integers(-5, 6, (M, N)).astype(np.float64)
    got = run(cuda, A, B, C0, 1, 1, 1, accuracy=mode)
    exact = (A.astype(np.int64) @ B.astype(np.int64) + C0.astype(np.int64)).astype(np.float64)
    np.testing.assert_array_equal(got, exact)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("sign", [1.0, -1.0])
def test_largest_digit_sums_exact(cuda, mode, sign):
    """x = 32639 / 32768 has digits 127, 127 (7 digits) or 127, 127, 0, ... :
    every digit product of weight 0..2 is 127^2 with one sign, so each
    group's sum over a 128-K (64-K) chunk is as large as the digits allow;
    x^2 has a 30-bit numerator, so K x^2 is exact in FP64."""
    M, N, K = 128, 64, 4096
    x = 32639.0 / 32768.0
    A = np.full((M, K), sign * x)
    B = np.full((K, N), x)
    Z = np.zeros((M, N))
    got = run(cuda, A, B, Z, 1, 0, 1, accuracy=mode)
    np.testing.assert_array_equal(got, np.full((M, N), sign * K * x * x))


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("la,lb,lc", [(1, 1, 1), (0, 0, 0), (1, 0, 1), (0, 1, 0), (1, 1, 0), (0, 0, 1)])
def test_layouts_ragged_vs_oracle(cuda, mode, la, lb, lc):
    rng = np.random.default_rng(12 + 8 * la + 4 * lb + 2 * lc)
    for (M, N, K) in [(1, 1, 1), (129, 33, 50), (300, 97, 257), (64, 200, 31)]:
        A = rng.uniform(-1, 1, (M, K))
        B = rng.uniform(-1, 1, (K, N))
        C0 = rng.uniform(-1, 1, (M, N))
        got = run(cuda, A, B, C0, la, lb, lc, accuracy=mode)
        assert_digit_close(got, A, B, C0, la, lb, lc, mode, what=f"{M}x{N}x{K} layouts {la}{lb}{lc}")


@pytest.mark.parametrize("mode", MODES)
def test_scaled_rows_and_columns(cuda, mode):
    """Rows and columns of very different magnitudes (2^-300 .. 2^300): the
    per-row / per-column scales keep each output's relative accuracy."""
    rng = np.random.default_rng(13)
    M, N, K = 256, 96, 512
    A = rng.uniform(-1, 1, (M, K)) * np.ldexp(1.0, rng.integers(-300, 301, M))[:, None]
    B = rng.uniform(-1, 1, (K, N)) * np.ldexp(1.0, rng.integers(-300, 301, N))[None, :]
    Z = np.zeros((M, N))
    got = run(cuda, A, B, Z, 1, 1, 1, accuracy=mode)
    assert_digit_close(got, A, B, Z, 1, 1, 1, mode, what="scaled rows and columns")


@pytest.mark.parametrize("mode", MODES)
def test_uniform_1024_matches_fp64_pipes(cuda, mode):
    """1024 x 1024 x 4096 U[-1,1): the digit path against the FP64-FMA path
    on the same inputs (both against the oracle's bound), and its normwise
    error no larger than the FP64 path's."""
    import gbblas
    rng = np.random.default_rng(14)
    M, N, K = 1024, 1024, 4096
    A = rng.uniform(-1, 1, (M, K))
    B = rng.uniform(-1, 1, (K, N))
    Z = np.zeros((M, N))
    got = run(cuda, A, B, Z, 1, 1, 1, accuracy=mode)
    nat = run(cuda, A, B, Z, 1, 1, 1, accuracy=gbblas.ACCURACY_FP64)
    rows = rng.integers(0, M, 64)
    cols = rng.integers(0, N, 64)
    ex = np.array([float(np.dot(A[i].astype(np.longdouble), B[:, j].astype(np.longdouble))) for i, j in zip(rows, cols)])
    e_dig = np.abs(got[rows, cols] - ex).max()
    e_nat = np.abs(nat[rows, cols] - ex).max()
    assert e_dig <= max(e_nat, 1e-15), (e_dig, e_nat)
    sa, sb = scales(A, B)
    S = NDIG[mode]
    bound = (S + 1) * 2.0 ** (-8 * S) * K * np.outer(sa, sb) + 4 * np.finfo(np.float64).eps * np.abs(nat)
    fp64 = 2 * K * np.finfo(np.float64).eps * (np.abs(A) @ np.abs(B))
    assert (np.abs(got - nat) <= bound + fp64).all()


@pytest.mark.parametrize("mode", MODES)
def test_inf_nan_rows_and_columns(cuda, mode):
    rng = np.random.default_rng(15)
    M, N, K = 130, 40, 70
    A = rng.uniform(-1, 1, (M, K))
    B = rng.uniform(-1, 1, (K, N))
    A[3, 5] = np.inf
    A[100, 0] = np.nan
    B[7, 20] = -np.inf
    Z = np.zeros((M, N))
    got = run(cuda, A, B, Z, 1, 1, 1, accuracy=mode)
    bad_r = np.zeros(M, bool)
    bad_r[[3, 100]] = True
    bad_c = np.zeros(N, bool)
    bad_c[20] = True
    mask = bad_r[:, None] | bad_c[None, :]
    assert np.isnan(got[mask]).all()
    assert np.isfinite(got[~mask]).all()
    Ac, Bc = A.copy(), B.copy()
    Ac[bad_r] = 0
    Bc[:, bad_c] = 0
    ref = Ac @ Bc
    tol = digit_tol(Ac, Bc, Z, mode)
    assert (np.abs(got[~mask] - ref[~mask]) <= tol[~mask]).all()


@pytest.mark.parametrize("mode", MODES)
def test_zero_operands_and_general_strides(cuda, mode):
    import gbblas
    rng = np.random.default_rng(16)
    M, N, K = 70, 45, 90
    A = rng.uniform(-1, 1, (M, K))
    A[10] = 0.0  # an all-zero row
    B = rng.uniform(-1, 1, (K, N))
    B[:, 7] = 0.0
    # A with a row pitch of K + 3 (neither stride 1 in the other direction)
    bufA = np.zeros((M, K + 3))
    bufA[:, :K] = A
    tA = cuda.from_numpy(bufA).cuda()
    tB = cuda.from_numpy(np.ascontiguousarray(B)).cuda()
    C0 = rng.uniform(-1, 1, (M, N))
    tC = cuda.from_numpy(C0.copy()).cuda()
    gbblas.call("gbblas_dgemm_ex", M, N, K, tA.data_ptr(), K + 3, 1, tB.data_ptr(), N, 1, tC.data_ptr(), N, 1,
                mode, None)
    gbblas.call("gbblas_check_stream", None)
    got = tC.cpu().numpy()
    assert_digit_close(got, A, B, C0, 1, 1, 1, mode, what="row pitch K+3")
    np.testing.assert_array_equal(got[10], C0[10])
    np.testing.assert_array_equal(got[:, 7], C0[:, 7])


def test_k_limit_and_bad_accuracy(cuda):
    import gbblas
    t = cuda.zeros(8, dtype=cuda.float64, device="cuda")
    p = t.data_ptr()
    # K beyond 2^20: refused before any launch
    with pytest.raises(gbblas.GbblasError):
        gbblas.call("gbblas_dgemm_ex", 1, 1, (1 << 20) + 1, p, 0, 0, p, 0, 0, p, 1, 1, D7, None)
    with pytest.raises(gbblas.GbblasError):
        gbblas.call("gbblas_dgemm_ex", 1, 1, 1, p, 1, 1, p, 1, 1, p, 1, 1, 4, None)


# ------------------------------------------------- guarded form (AUTO, the default)
AUTO = 3
FP64 = 5


def run_any(torch, A, B, C0, accuracy, fn="gbblas_dgemm_ex"):
    import gbblas
    M, K = A.shape
    N = B.shape[1]
    tA = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    tB = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    tC = torch.from_numpy(C0.copy()).cuda()
    args = [M, N, K, tA.data_ptr(), K, 1, tB.data_ptr(), N, 1, tC.data_ptr(), N, 1]
    if fn == "gbblas_dgemm_ex":
        args.append(accuracy)
    gbblas.call(fn, *args, None)
    gbblas.call("gbblas_check_stream", None)
    return tC.cpu().numpy()


def fp64_tol(A, B, C0):
    K = A.shape[1]
    return 2 * max(K, 1) * np.finfo(np.float64).eps * (np.abs(A) @ np.abs(B) + np.abs(C0)) + np.finfo(np.float64).tiny


def test_auto_equals_digits_where_the_guard_passes(cuda):
    """U[-1,1), K >= 32: every block passes, and the guarded result is the
    7-digit result bit for bit (the same digit products in the same order)."""
    rng = np.random.default_rng(21)
    M, N, K = 300, 170, 600  # 2^24.9 multiply-adds: AUTO takes the digits
    A = rng.uniform(-1, 1, (M, K))
    B = rng.uniform(-1, 1, (K, N))
    C0 = rng.uniform(-1, 1, (M, N))
    np.testing.assert_array_equal(run_any(cuda, A, B, C0, AUTO), run_any(cuda, A, B, C0, D7))


def test_guard_recomputes_blocks_the_digits_would_get_wrong(cuda):
    """Rows 0..39 of A carry one huge entry (2^40) against a zero row of B:
    the row scale 2^41 leaves those rows' other entries only their last
    digits, so the unguarded digits miss the FP64 bound there; the guard
    sends exactly those blocks to the FP64 pipes."""
    rng = np.random.default_rng(22)
    M, N, K = 256, 96, 512
    A = rng.uniform(-1, 1, (M, K))
    B = rng.uniform(-1, 1, (K, N))
    A[:40, 0] = 2.0 ** 40
    B[0, :] = 0.0
    C0 = np.zeros((M, N))
    tol = fp64_tol(A, B, C0)
    ref = O.gemm(A, B, C0, 1, 1, 1)
    raw = run_any(cuda, A, B, C0, D7)
    assert (np.abs(raw - ref)[:40] > tol[:40]).any(), "the case must defeat the unguarded digits"
    got = run_any(cuda, A, B, C0, AUTO)
    assert (np.abs(got - ref) <= tol).all()
    # rows 64.. (whole blocks without a huge entry) keep the digit result
    np.testing.assert_array_equal(got[64:], raw[64:])


def test_small_k_and_small_shapes_use_fp64_pipes(cuda):
    rng = np.random.default_rng(23)
    # K < 32, or shapes the FP64 pipes finish before the digit path's ~50 us
    # of preparation (few multiply-adds per 64 x 64 tile)
    for (M, N, K) in [(300, 200, 31), (64, 64, 40), (32, 32, 64), (1, 5, 3)]:
        A = rng.uniform(-1, 1, (M, K))
        B = rng.uniform(-1, 1, (K, N))
        C0 = rng.uniform(-1, 1, (M, N))
        np.testing.assert_array_equal(run_any(cuda, A, B, C0, AUTO), run_any(cuda, A, B, C0, FP64))


def test_dgemm_default_is_auto_and_env_forces_fp64(cuda, monkeypatch):
    rng = np.random.default_rng(24)
    M, N, K = 256, 128, 256
    A = rng.uniform(-1, 1, (M, K))
    B = rng.uniform(-1, 1, (K, N))
    C0 = np.zeros((M, N))
    np.testing.assert_array_equal(run_any(cuda, A, B, C0, None, fn="gbblas_dgemm"), run_any(cuda, A, B, C0, AUTO))
    monkeypatch.setenv("GBBLAS_DGEMM_FP64", "1")
    np.testing.assert_array_equal(run_any(cuda, A, B, C0, None, fn="gbblas_dgemm"), run_any(cuda, A, B, C0, FP64))


@pytest.mark.parametrize("la,lb,lc", [(0, 0, 0), (1, 0, 1), (0, 1, 0)])
def test_auto_layouts_within_fp64_bound(cuda, la, lb, lc):
    rng = np.random.default_rng(25 + la + 2 * lb + 4 * lc)
    M, N, K = 257, 95, 700
    A = rng.uniform(-1, 1, (M, K)) * np.ldexp(1.0, rng.integers(-10, 11, (M, K)))
    B = rng.uniform(-1, 1, (K, N)) * np.ldexp(1.0, rng.integers(-10, 11, (K, N)))
    C0 = rng.uniform(-1, 1, (M, N))
    got = run(cuda, A, B, C0, la, lb, lc, accuracy=AUTO)
    ref = O.gemm(A, B, C0, la, lb, lc)
    assert (np.abs(got - ref) <= fp64_tol(A, B, C0)).all()


# ------------------------------------------------- bit equality with the digit model
from oracle import ozaki as OZ  # noqa: E402


def operands(rng, M, N, K, kind):
    if kind == "uniform":
        return rng.uniform(-1, 1, (M, K)), rng.uniform(-1, 1, (K, N))
    if kind == "wide":
        def w(shape):
            return rng.choice([-1.0, 1.0], shape) * rng.uniform(1, 2, shape) * np.ldexp(1.0, rng.integers(-10, 11, shape))
        return w((M, K)), w((K, N))
    if kind == "scaled":  # rows / columns 2^-300 .. 2^300 apart, one zero row, one Inf row, one NaN column
        A = rng.uniform(-1, 1, (M, K)) * np.ldexp(1.0, rng.integers(-300, 301, M))[:, None]
        B = rng.uniform(-1, 1, (K, N)) * np.ldexp(1.0, rng.integers(-300, 301, N))[None, :]
        A[M // 2] = 0.0
        A[1, K // 3] = np.inf
        B[K // 2, N - 1] = np.nan
        return A, B
    raise ValueError(kind)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("kind", ["uniform", "wide", "scaled"])
def test_bit_exact_against_digit_model(cuda, mode, kind):
    """Unguarded 7 / 8 digits: the GPU result equals the oracle's integer
    model of the scheme (oracle/ozaki.py) bit for bit, NaNs included."""
    rng = np.random.default_rng(31)
    for (M, N, K), (la, lb, lc) in [((129, 33, 300), (1, 1, 1)), ((200, 70, 513), (0, 1, 0)),
                                    ((64, 96, 128), (1, 0, 1)), ((5, 7, 33), (0, 0, 1))]:
        A, B = operands(rng, M, N, K, kind)
        C0 = rng.uniform(-1, 1, (M, N))
        got = run(cuda, A, B, C0, la, lb, lc, accuracy=mode)
        np.testing.assert_array_equal(got, OZ.gemm(A, B, C0, NDIG[mode]), err_msg=f"{M}x{N}x{K} {kind}")


@pytest.mark.parametrize("kind", ["uniform", "wide"])
def test_auto_bit_exact_where_the_guard_keeps_the_digits(cuda, kind):
    """Guarded AUTO: every 32 x 16 block the model's guard keeps equals the
    model bit for bit; the blocks it rejects (rows with a 2^40 entry against
    a zero row of B) are within the FP64 bound."""
    rng = np.random.default_rng(32)
    # wide-range operands pass the guard (which samples a quarter of K) from
    # K of about 4096; below that AUTO sends their blocks to the FP64 pipes
    M, N, K = 256, 96, (640 if kind == "uniform" else 4096)
    A, B = operands(rng, M, N, K, kind)
    A[:40, 0] = 2.0 ** 40
    B[0, :] = 0.0
    C0 = rng.uniform(-1, 1, (M, N))
    got = run_any(cuda, A, B, C0, AUTO)
    keep = OZ.guard_pass(A, B)
    assert keep.any() and (~keep).any()
    want = OZ.gemm(A, B, C0, 7)
    np.testing.assert_array_equal(got[keep], want[keep])
    ref = O.gemm(A, B, C0, 1, 1, 1)
    assert (np.abs(got - ref)[~keep] <= fp64_tol(A, B, C0)[~keep]).all()


@pytest.mark.parametrize("accuracy", [D7, D8, 3])
def test_sliced_launches_give_the_same_bits(cuda, monkeypatch, accuracy):
    """GBBLAS_GEMM_SLICES=n runs the digit GEMM as n launches over
    consecutive ranges of tiles (the serving loop's heavy requests): the
    same bits, the guard's fix-up list included (one row with a 2^40 entry
    against a zero row of B sends blocks to the FP64 pipes under AUTO)."""
    rng = np.random.default_rng(50 + accuracy)
    M, N, K = 1100, 700, 512
    A = rng.uniform(-1, 1, (M, K))
    B = rng.uniform(-1, 1, (K, N))
    C0 = rng.uniform(-1, 1, (M, N))
    if accuracy == 3:
        A[5, 3] = 2.0 ** 40
        B[3, :] = 0.0
    whole = run_any(cuda, A, B, C0, accuracy)
    for n in (2, 7):
        monkeypatch.setenv("GBBLAS_GEMM_SLICES", str(n))
        np.testing.assert_array_equal(run_any(cuda, A, B, C0, accuracy), whole)
    monkeypatch.delenv("GBBLAS_GEMM_SLICES")
