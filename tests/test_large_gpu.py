"""Sizes beyond 2^31 elements: every kernel indexes with 64-bit offsets.

Each case builds its operands on the GPU (about 10-20 GB each, freed
afterwards) with a pattern whose result is exact in floating point and that
only comes out right if elements past index 2^31 are read and written where
they belong.
"""
import pytest

pytestmark = pytest.mark.gpu

BIG = (1 << 31) + 37


def _free(torch):
    torch.cuda.synchronize()
    torch.cuda.empty_cache()


def test_dot_past_2_pow_31(cuda):
    import gbblas
    torch = cuda
    a = torch.zeros(BIG, device="cuda")
    a[1 << 31:] = 1.0  # only the elements past 2^31 count
    b = torch.ones(BIG, device="cuda")
    r = torch.zeros(1, device="cuda")
    gbblas.call("gbblas_sdot", BIG, a.data_ptr(), b.data_ptr(), r.data_ptr(), None)
    assert r.item() == 37.0
    del a, b
    _free(torch)


def test_mtv_rows_past_2_pow_31_elements(cuda):
    import gbblas
    torch = cuda
    M, N = 40000, 60000  # 2.4e9 elements, row-major
    A = torch.zeros(M, N, device="cuda")
    A[:, N - 1000:] = 1.0
    A[M - 1, :] = 2.0
    x = torch.ones(N, device="cuda")
    y = torch.zeros(M, device="cuda")
    gbblas.call("gbblas_smtv", 1, M, N, A.data_ptr(), x.data_ptr(), y.data_ptr(), None)
    torch.cuda.synchronize()
    assert torch.all(y[:-1] == 1000.0)
    assert y[-1].item() == 2.0 * N
    del A
    _free(torch)


def test_transpose_past_2_pow_31_elements(cuda):
    import gbblas
    torch = cuda
    M, N = 50000, 45000  # 2.25e9 elements each side
    A = (torch.arange(M * N, device="cuda", dtype=torch.int64) % (1 << 23)).to(torch.float32).view(M, N)
    C = torch.empty(N, M, device="cuda")
    gbblas.call("gbblas_stranspose", M, N, A.data_ptr(), N, 1, C.data_ptr(), M, 1, None)
    torch.cuda.synchronize()
    for i0, j0 in ((0, 0), (M - 64, N - 64), (M // 2, N // 3), (47721, 44000)):
        assert torch.equal(C[j0:j0 + 64, i0:i0 + 64], A[i0:i0 + 64, j0:j0 + 64].t())
    assert torch.equal(C[:, M - 1], A[M - 1, :])
    del A, C
    _free(torch)


def test_outer_past_2_pow_31_elements(cuda):
    import gbblas
    torch = cuda
    M, N = 50000, 45000
    a = (torch.arange(M, device="cuda") % 1024).float()
    b = (torch.arange(N, device="cuda") % 1000).float()
    C = torch.ones(M, N, device="cuda")
    gbblas.call("gbblas_souter", 1, M, N, a.data_ptr(), b.data_ptr(), C.data_ptr(), None)
    torch.cuda.synchronize()
    for i0 in (0, M // 2, M - 16):
        assert torch.equal(C[i0:i0 + 16], torch.outer(a[i0:i0 + 16], b) + 1.0)
    del C
    _free(torch)


def test_element_wise_past_2_pow_31(cuda):
    import gbblas
    torch = cuda
    x = (torch.arange(BIG, device="cuda", dtype=torch.int64) % 1000).float()
    y = torch.full((BIG,), 3.0, device="cuda")
    z = torch.empty_like(x)
    gbblas.call("gbblas_sew", 2, BIG, x.data_ptr(), y.data_ptr(), z.data_ptr(), None)  # z = 3 x
    torch.cuda.synchronize()
    tail = slice(BIG - (1 << 20), BIG)
    assert torch.equal(z[tail], x[tail] * 3.0)
    assert torch.equal(z[:1 << 20], x[:1 << 20] * 3.0)
    del x, y, z
    _free(torch)


@pytest.mark.parametrize("accuracy", [0, 1, 2, 4])  # FP32, BF16X3, FP8, BF16X6
def test_gemm_operand_past_2_pow_31_elements(cuda, accuracy):
    """A is 40000 x 60000 (2.4e9 elements; its BF16 / FP8 arena is past 2^31
    elements too): C = A * ones, A one only on its last 1000 columns and on
    its last row."""
    import gbblas
    torch = cuda
    M, K, N = 40000, 60000, 128
    A = torch.zeros(M, K, device="cuda")
    A[:, K - 1000:] = 1.0
    A[M - 1, :] = 1.0
    B = torch.ones(K, N, device="cuda")
    C = torch.zeros(M, N, device="cuda")
    gbblas.call("gbblas_sgemm", M, N, K, A.data_ptr(), K, 1, B.data_ptr(), N, 1, C.data_ptr(), N, 1, accuracy, None)
    gbblas.call("gbblas_check_stream", None)
    assert torch.all(C[:-1] == 1000.0)
    assert torch.all(C[-1] == float(K))
    del A, B, C
    _free(torch)
