"""The CTA-pair form of the tensor-core GEMM (GBBLAS_TC_PAIR=1: clusters of
two CTAs, tcgen05 .cta_group::2 MMAs on 256 x 128 tiles) against FP64 with the
split-BF16 bounds, including ragged shapes, both layouts and a grouped launch.
FP8 always runs on single CTAs: with the setting on it must still be
bit-exact on integer data and follow the quantisation model."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import lowprec as L

from test_gemm_tc_gpu import BF16X3, BF16X6, run, split_tol

pytestmark = pytest.mark.gpu

SHAPES = [(300, 200, 1000), (1000, 1000, 1000), (256, 512, 2048), (513, 129, 700), (2048, 384, 512)]


@pytest.fixture
def pairs(monkeypatch):
    monkeypatch.setenv("GBBLAS_TC_PAIR", "1")


@pytest.mark.parametrize("mode", [BF16X3, BF16X6])
@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("lc,la,lb", [(1, 1, 1), (0, 0, 0), (1, 0, 1)])
def test_pair_split_vs_fp64(cuda, pairs, mode, shape, lc, la, lb):
    M, N, K = shape
    rng = np.random.default_rng(M + 3 * N + 7 * K + mode)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    C0 = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    got = run(cuda, A, B, C0, la, lb, lc, accuracy=mode).astype(np.float64)
    exact = A.astype(np.float64) @ B.astype(np.float64) + C0
    tol = split_tol(np.abs(A).astype(np.float64), np.abs(B).astype(np.float64), K, mode) + \
        np.abs(C0) * np.finfo(np.float32).eps * 2
    assert np.all(np.abs(got - exact) <= tol)


@pytest.mark.parametrize("shape", SHAPES)
def test_fp8_unaffected_by_pair_setting(cuda, pairs, shape):
    M, N, K = shape
    rng = np.random.default_rng(M + N + K)
    A = rng.integers(-8, 9, (M, K)).astype(np.float32)
    B = rng.integers(-8, 9, (K, N)).astype(np.float32)
    Z = np.zeros((M, N), np.float32)
    np.testing.assert_array_equal(run(cuda, A, B, Z, 1, 1, 1, accuracy=2), A.astype(np.float64) @ B)
    U = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    V = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    got = run(cuda, U, V, Z, 1, 1, 1, accuracy=2).astype(np.float64)
    nb = -(-K // 128)
    tol = (2.0 ** -16 + 2 * (nb + 1) * np.finfo(np.float32).eps) * L.gemm_fp8_abs_model(U, V) + 1e-30
    assert np.all(np.abs(got - L.gemm_fp8_model(U, V)) <= tol)


def test_pair_grouped(cuda, pairs):
    import gbblas
    torch = cuda
    rng = np.random.default_rng(9)
    shapes = [(700, 300, 900), (512, 512, 512), (1024, 256, 300)]
    mats, descs = [], []
    for (M, N, K) in shapes:
        A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
        B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
        tA, tB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
        tC = torch.zeros((M, N), dtype=torch.float32, device="cuda")
        mats.append((A, B, tA, tB, tC))
        descs.append(gbblas.gemm_desc(tA, tB, tC))
    gbblas.gemm_grouped(descs, accuracy=BF16X6)
    gbblas.call("gbblas_check_stream", None)
    for (A, B, _, _, tC) in mats:
        exact = A.astype(np.float64) @ B.astype(np.float64)
        tol = split_tol(np.abs(A).astype(np.float64), np.abs(B).astype(np.float64), A.shape[1], BF16X6)
        assert np.all(np.abs(tC.cpu().numpy() - exact) <= tol)
