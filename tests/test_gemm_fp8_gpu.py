"""Low-accuracy GEMM (GBBLAS_ACCURACY_FP8) on the tcgen05 tensor cores:
E4M3 operands with one power-of-two scale per 128-element K-block, through
the C ABI.

* integer data |x| <= 8 survives E4M3 quantisation unchanged: bit equality
  with the exact product, every layout mix, ragged and multi-block shapes;
* random data against the numpy model of the same quantisation
  (oracle/lowprec.py): the kernel may differ from the model's exact block
  dot products only by FP32 rounding, bounded below;
* error against FP64 on both precision input sets is reported (large on the
  wide-range set by design: 2^20 of dynamic range inside a block exceeds
  E4M3's);
* grouped, batched (graph replay) and single calls agree bit for bit.
"""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import lowprec as L

pytestmark = pytest.mark.gpu

FP8 = 2
EPS32 = float(np.finfo(np.float32).eps)


def run(torch, A, B, C0, la, lb, lc, accuracy=FP8):
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


def model_tol(A, B):
    """FP32 rounding of the block sums (inside the tensor core and in the
    epilogue) relative to the block magnitudes: 2^-16 per block sum plus
    one FP32 add per block."""
    K = A.shape[1]
    nb = -(-K // 128)
    return (2.0 ** -16 + 2 * (nb + 1) * EPS32) * L.gemm_fp8_abs_model(A, B) + 1e-30


def test_single_tile_integers_exact(cuda):
    rng = np.random.default_rng(0)
    A = rng.integers(-8, 9, (128, 128)).astype(np.float32)
    B = rng.integers(-8, 9, (128, 128)).astype(np.float32)
    Z = np.zeros((128, 128), np.float32)
    np.testing.assert_array_equal(run(cuda, A, B, Z, 1, 1, 1), A @ B)


INT_SHAPES = [(1, 1, 1), (5, 7, 3), (128, 256, 128), (129, 257, 129), (300, 100, 1000), (256, 384, 2048)]


@pytest.mark.parametrize("shape", INT_SHAPES)
@pytest.mark.parametrize("lc,la,lb", [(1, 1, 1), (0, 0, 0), (1, 0, 1), (0, 1, 0)])
def test_integers_exact_all_layouts(cuda, shape, lc, la, lb):
    M, N, K = shape
    rng = np.random.default_rng(M + 5 * N + 11 * K)
    A = rng.integers(-8, 9, (M, K)).astype(np.float32)
    B = rng.integers(-8, 9, (K, N)).astype(np.float32)
    C0 = rng.integers(-50, 51, (M, N)).astype(np.float32)
    got = run(cuda, A, B, C0, la, lb, lc)
    np.testing.assert_array_equal(got, A.astype(np.float64) @ B + C0)


def test_mixed_block_scales_exact(cuda):
    """Power-of-two magnitudes that differ per row, per column and per
    K-block: each block's own scale keeps the integers exact."""
    rng = np.random.default_rng(3)
    M, N, K = 192, 160, 640
    A = rng.integers(-8, 9, (M, K)).astype(np.float64)
    B = rng.integers(-8, 9, (K, N)).astype(np.float64)
    A *= np.exp2(rng.integers(-20, 20, (M, 1)))
    A[:, 128:256] *= 2.0 ** 9
    B *= np.exp2(rng.integers(-20, 20, (1, N)))
    B[512:, :] *= 2.0 ** -7
    A, B = A.astype(np.float32), B.astype(np.float32)
    Z = np.zeros((M, N), np.float32)
    got = run(cuda, A, B, Z, 1, 1, 1).astype(np.float64)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    # exact per block; only the FP32 sums over blocks and over K round
    tol = 2 * (K / 128 + 1) * EPS32 * (np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64))
    assert np.all(np.abs(got - exact) <= tol)


SHAPES = [(64, 64, 64), (129, 257, 300), (512, 256, 1024), (1000, 1000, 1000)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("lc,la,lb", [(1, 1, 1), (0, 0, 0), (1, 0, 1)])
def test_random_matches_quantisation_model(cuda, shape, lc, la, lb):
    M, N, K = shape
    rng = np.random.default_rng(M + 3 * N + 7 * K)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    Z = np.zeros((M, N), np.float32)
    got = run(cuda, A, B, Z, la, lb, lc).astype(np.float64)
    model = L.gemm_fp8_model(A, B)
    err = np.abs(got - model)
    tol = model_tol(A, B)
    assert np.all(err <= tol), f"max err/tol {np.max(err / tol):.3g}"


def wide(rng, shape):
    s = rng.choice([-1.0, 1.0], shape)
    m = rng.uniform(1, 2, shape)
    e = rng.integers(-10, 11, shape)
    return (s * m * np.exp2(e)).astype(np.float32)


@pytest.mark.parametrize("dataset", ["uniform", "wide"])
def test_error_vs_fp64_reported(cuda, dataset):
    """1024^3 against FP64: the model is followed on both sets; the error
    against FP64 is E4M3's (about 2^-4 per operand on uniform data; much
    larger on the wide set, where small entries of a block flush to zero)."""
    rng = np.random.default_rng(2)
    n = 1024
    if dataset == "uniform":
        A = rng.uniform(-1, 1, (n, n)).astype(np.float32)
        B = rng.uniform(-1, 1, (n, n)).astype(np.float32)
    else:
        A, B = wide(rng, (n, n)), wide(rng, (n, n))
    Z = np.zeros((n, n), np.float32)
    got = run(cuda, A, B, Z, 1, 1, 1).astype(np.float64)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64)
    model = L.gemm_fp8_model(A, B)
    assert np.all(np.abs(got - model) <= model_tol(A, B))
    normwise = np.max(np.abs(got - exact) / scale)
    rel = np.abs(got - exact) / np.maximum(np.abs(exact), 1e-300)
    print(f"fp8 {dataset}: normwise max {normwise:.3e}, relative max {rel.max():.3e} mean {rel.mean():.3e}")
    if dataset == "uniform":
        assert normwise < 2.0 ** -4


def test_grouped_and_batch_match_single(cuda):
    import gbblas
    torch = cuda
    rng = np.random.default_rng(4)
    shapes = [(300, 200, 700), (128, 128, 128), (65, 999, 257), (512, 64, 1536)]
    mats, descs, singles = [], [], []
    for (M, N, K) in shapes:
        A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
        B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
        Z = np.zeros((M, N), np.float32)
        singles.append(run(torch, A, B, Z, 1, 1, 1))
        tA, tB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
        tC = torch.zeros((M, N), dtype=torch.float32, device="cuda")
        mats.append((tA, tB, tC))
        descs.append(gbblas.gemm_desc(tA, tB, tC))
    gbblas.gemm_grouped(descs, accuracy=FP8)
    torch.cuda.synchronize()
    for (tA, tB, tC), ref in zip(mats, singles):
        np.testing.assert_array_equal(tC.cpu().numpy(), ref)
    batch = gbblas.Batch(gemms=descs, accuracy=FP8)
    try:
        for _ in range(2):
            for (_, _, tC) in mats:
                tC.zero_()
            torch.cuda.synchronize()
            batch.run()
            batch.sync()
            for (tA, tB, tC), ref in zip(mats, singles):
                np.testing.assert_array_equal(tC.cpu().numpy(), ref)
    finally:
        batch.close()
