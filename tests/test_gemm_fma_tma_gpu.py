"""The TMA-fed FP32 GEMM on the FMA pipes (GBBLAS_FMA_TILE=2) against the
register-staged kernels and the oracle, through the C ABI.

Both kernels accumulate each output from zero over K in k order with fused
multiply-adds and then add it into C, so they must agree bit for bit; the
TMA-fed one is also checked against the CPU oracle within 2 K eps of
(|A||B| + |C0|).  Layout mixes of A, B and C, ragged and tiny shapes, K not
a multiple of the 32-wide K tile, and operands the TMA cannot take (an
odd pitch, a misaligned base), which fall back to the register-staged path.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

EPS32 = float(np.finfo(np.float32).eps)


def run(torch, A, B, C0, la, lb, lc, tile, monkeypatch, pad_a=0):
    import gbblas
    monkeypatch.setenv("GBBLAS_FMA_TILE", str(tile))
    M, K = A.shape
    N = B.shape[1]
    a_host = O.to_layout(A, la)
    flat = np.zeros(a_host.size + pad_a, np.float32)
    flat[pad_a:] = a_host.ravel()
    tflat = torch.from_numpy(flat).cuda()
    tB = torch.from_numpy(O.to_layout(B, lb)).cuda()
    tC = torch.from_numpy(O.to_layout(C0, lc).copy()).cuda()
    rsa, csa = O.strides(M, K, la)
    rsb, csb = O.strides(K, N, lb)
    rsc, csc = O.strides(M, N, lc)
    gbblas.call("gbblas_sgemm", M, N, K, tflat.data_ptr() + 4 * pad_a, rsa, csa, tB.data_ptr(), rsb, csb,
                tC.data_ptr(), rsc, csc, 0, None)
    gbblas.call("gbblas_check_stream", None)
    return O.from_layout(tC.cpu().numpy(), M, N, lc)


SHAPES = [(1, 1, 1), (7, 5, 3), (128, 128, 32), (129, 257, 65), (300, 200, 1000), (1024, 512, 777), (64, 2000, 96)]
LAYOUTS = [(1, 1, 1), (1, 0, 1), (1, 1, 0), (0, 0, 0), (0, 1, 1), (0, 0, 1)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("la,lb,lc", LAYOUTS)
def test_tma_fed_matches_register_staged_and_oracle(cuda, monkeypatch, shape, la, lb, lc):
    M, N, K = shape
    rng = np.random.default_rng(M + 7 * N + 13 * K + 3 * la + 5 * lb + lc)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    C0 = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    tma = run(cuda, A, B, C0, la, lb, lc, 2, monkeypatch)
    staged = run(cuda, A, B, C0, la, lb, lc, 0, monkeypatch)
    np.testing.assert_array_equal(tma, staged)
    ref = O.gemm(A, B, C0, la, lb, lc)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64) + np.abs(C0)
    assert np.all(np.abs(tma.astype(np.float64) - ref) <= 2 * max(K, 1) * EPS32 * scale)


def test_integer_golden_cases_exact(cuda, monkeypatch):
    import _golden as G
    for name in [n for n in G.names("mtm_float32") if "uniform" not in n]:
        c = G.case(name)
        A, B, C0 = c["A"].astype(np.float32), c["B"].astype(np.float32), c["C0"].astype(np.float32)
        got = run(cuda, A, B, C0, int(c["la"]), int(c["lb"]), int(c["lc"]), 2, monkeypatch)
        np.testing.assert_array_equal(got, c["C"])


@pytest.mark.parametrize("pad_a", [1, 2])
def test_misaligned_operand_falls_back(cuda, monkeypatch, pad_a):
    """A base pointer off the 16-byte grid: the register-staged kernel runs,
    with the same bits."""
    rng = np.random.default_rng(pad_a)
    A = rng.uniform(-1, 1, (200, 300)).astype(np.float32)
    B = rng.uniform(-1, 1, (300, 150)).astype(np.float32)
    C0 = np.zeros((200, 150), np.float32)
    got = run(cuda, A, B, C0, 1, 1, 1, 2, monkeypatch, pad_a=pad_a)
    np.testing.assert_array_equal(got, run(cuda, A, B, C0, 1, 1, 1, 0, monkeypatch))


def test_odd_pitch_falls_back(cuda, monkeypatch):
    """K = 301 row-major: a row pitch of 1204 bytes is no multiple of 16."""
    rng = np.random.default_rng(4)
    A = rng.uniform(-1, 1, (130, 301)).astype(np.float32)
    B = rng.uniform(-1, 1, (301, 140)).astype(np.float32)
    C0 = np.zeros((130, 140), np.float32)
    np.testing.assert_array_equal(run(cuda, A, B, C0, 1, 1, 1, 2, monkeypatch),
                                  run(cuda, A, B, C0, 1, 1, 1, 0, monkeypatch))


def test_large_against_fp64(cuda, monkeypatch):
    import gbblas
    torch = cuda
    monkeypatch.setenv("GBBLAS_FMA_TILE", "2")
    g = torch.Generator(device="cuda").manual_seed(3)
    A = torch.rand(3000, 2500, device="cuda", generator=g) * 2 - 1
    B = torch.rand(2500, 3500, device="cuda", generator=g) * 2 - 1
    C = torch.zeros(3000, 3500, device="cuda")
    gbblas.gemm(A, B, C, accuracy=gbblas.ACCURACY_FP32)
    ref = A.double() @ B.double()
    bound = 2 * 2500 * EPS32 * (A.double().abs() @ B.double().abs())
    assert bool(((C.double() - ref).abs() <= bound).all())


@pytest.mark.parametrize("la,lb", [(1, 1), (0, 0), (1, 0), (0, 1)])
def test_padded_pitch_takes_tma_path(cuda, monkeypatch, la, lb):
    """K = 301 with row / column pitches padded to 304 elements (16-byte
    multiples): the TMA-fed kernel runs; the box's K tail past 301 reads as
    zeros.  Same bits as the register-staged kernel, oracle bound."""
    import gbblas
    torch = cuda
    M, N, K, P = 130, 150, 301, 304
    rng = np.random.default_rng(11 + la + 2 * lb)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    C0 = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    # padding holds NaN: any read past K (or past M, N) would show
    if la == 1:
        abuf = np.full((M, P), np.nan, np.float32); abuf[:, :K] = A; rsa, csa = P, 1
    else:
        PA = 144  # >= M = 130, multiple of 4
        abuf = np.full((K, PA), np.nan, np.float32); abuf[:, :M] = A.T; rsa, csa = 1, PA
    if lb == 1:
        PB = 152  # >= N = 150
        bbuf = np.full((K, PB), np.nan, np.float32); bbuf[:, :N] = B; rsb, csb = PB, 1
    else:
        bbuf = np.full((N, P), np.nan, np.float32); bbuf[:, :K] = B.T; rsb, csb = 1, P
    tA, tB = torch.from_numpy(abuf).cuda(), torch.from_numpy(bbuf).cuda()
    outs = []
    for tile in (2, 0):
        monkeypatch.setenv("GBBLAS_FMA_TILE", str(tile))
        tC = torch.from_numpy(C0.copy()).cuda()
        gbblas.call("gbblas_sgemm", M, N, K, tA.data_ptr(), rsa, csa, tB.data_ptr(), rsb, csb, tC.data_ptr(), N, 1,
                    0, None)
        gbblas.call("gbblas_check_stream", None)
        outs.append(tC.cpu().numpy())
    np.testing.assert_array_equal(outs[0], outs[1])
    exact = A.astype(np.float64) @ B.astype(np.float64) + C0
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64) + np.abs(C0)
    assert np.all(np.abs(outs[0] - exact) <= 2 * K * EPS32 * scale)


@pytest.mark.parametrize("shape", [(1024, 1024, 1024), (300, 200, 4000), (129, 257, 65), (700, 130, 3000),
                                   (128, 128, 8192), (2000, 2000, 512), (1, 1, 4096)])
@pytest.mark.parametrize("la,lb,lc", [(1, 1, 1), (0, 1, 1), (1, 0, 0), (0, 0, 1)])
def test_split_k_within_bound(cuda, monkeypatch, shape, la, lb, lc):
    """GBBLAS_FMA_TILE=3: the TMA-fed kernel in stream-K form (the tiles' K
    blocks shared out equally among the SMs; a tile split between CTAs is
    summed over its segments in K order by the segment that finishes last):
    within the same bound as the unsplit kernels and the same bits on every
    run."""
    M, N, K = shape
    rng = np.random.default_rng(M + N + K + la + 2 * lb + 4 * lc)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    C0 = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    got = run(cuda, A, B, C0, la, lb, lc, 3, monkeypatch)
    np.testing.assert_array_equal(run(cuda, A, B, C0, la, lb, lc, 3, monkeypatch), got)
    exact = A.astype(np.float64) @ B.astype(np.float64) + C0
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64) + np.abs(C0)
    assert np.all(np.abs(got.astype(np.float64) - exact) <= 2 * (K + 4) * EPS32 * scale)


@pytest.mark.parametrize("shape", [(1024, 1024, 1024), (1000, 1000, 1000), (896, 1152, 520), (1100, 900, 4096),
                                   (1024, 1024, 32), (2048, 2048, 512), (129, 257, 65)])
@pytest.mark.parametrize("la,lb,lc", [(1, 1, 1), (0, 1, 1), (1, 0, 0), (0, 0, 1)])
def test_cluster_pairs_within_bound(cuda, monkeypatch, shape, la, lb, lc):
    """GBBLAS_FMA_TILE=4: clusters of two CTAs per tile, each with half of
    the tile's K blocks; the odd CTA's sums move into the even CTA's shared
    memory, which adds them to its own in that order and updates C.  Shapes
    whose two CTAs per tile fit the SMs at once take that form; a single K
    block (K = 32) or more tiles (2048^2) fall back to stream-K.  Within the
    unsplit kernels' bound, and the same bits on every run."""
    M, N, K = shape
    rng = np.random.default_rng(3 * M + N + K + la + 2 * lb + 4 * lc)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    C0 = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    got = run(cuda, A, B, C0, la, lb, lc, 4, monkeypatch)
    np.testing.assert_array_equal(run(cuda, A, B, C0, la, lb, lc, 4, monkeypatch), got)
    exact = A.astype(np.float64) @ B.astype(np.float64) + C0
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64) + np.abs(C0)
    assert np.all(np.abs(got.astype(np.float64) - exact) <= 2 * (K + 4) * EPS32 * scale)


def test_cluster_pairs_integer_exact(cuda, monkeypatch):
    """Small integers: every partial sum is exact, so the two halves' sum
    equals the unsplit kernel's result bit for bit."""
    rng = np.random.default_rng(77)
    M = N = K = 1024
    A = rng.integers(-8, 9, (M, K)).astype(np.float32)
    B = rng.integers(-8, 9, (K, N)).astype(np.float32)
    C0 = rng.integers(-8, 9, (M, N)).astype(np.float32)
    np.testing.assert_array_equal(run(cuda, A, B, C0, 1, 1, 1, 4, monkeypatch),
                                  run(cuda, A, B, C0, 1, 1, 1, 2, monkeypatch))
