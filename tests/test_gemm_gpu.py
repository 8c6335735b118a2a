"""mtm on the GPU through the C ABI, against the oracle and the reference's
golden vectors (include/mtm.hpp; test/test.mtm.cpp's eight layout mixes)."""
import numpy as np
import pytest

from oracle import oracle as O

import _golden as G
from _tol import assert_gemm_close

pytestmark = pytest.mark.gpu


def run_gemm(torch, A, B, C0, la, lb, lc, accuracy=0):
    """C0 + A@B through gbblas_?gemm with the operands in the given layouts."""
    import gbblas
    M, K = A.shape
    N = B.shape[1]
    tA = torch.from_numpy(O.to_layout(A, la)).cuda()
    tB = torch.from_numpy(O.to_layout(B, lb)).cuda()
    tC = torch.from_numpy(O.to_layout(C0, lc).copy()).cuda()
    rsa, csa = O.strides(M, K, la)
    rsb, csb = O.strides(K, N, lb)
    rsc, csc = O.strides(M, N, lc)
    p = "s" if A.dtype == np.float32 else "d"
    args = [M, N, K, tA.data_ptr(), rsa, csa, tB.data_ptr(), rsb, csb, tC.data_ptr(), rsc, csc]
    if p == "s":
        args.append(accuracy)
    gbblas.call(f"gbblas_{p}gemm", *args, None)
    torch.cuda.synchronize()
    return O.from_layout(tC.cpu().numpy(), M, N, lc)


@pytest.mark.parametrize("name", G.names("mtm_"))
def test_mtm_golden(cuda, name):
    c = G.case(name)
    dt = c["C"].dtype
    A, B, C0 = c["A"].astype(dt), c["B"].astype(dt), c["C0"].astype(dt)
    got = run_gemm(cuda, A, B, C0, int(c["la"]), int(c["lb"]), int(c["lc"]))
    if int(c["exact"]):
        np.testing.assert_array_equal(got, c["C"])
    else:
        assert_gemm_close(got, c["C"], np.abs(A), np.abs(B), C0, A.shape[1], dt, what=name)


LAYOUTS = [(lc, la, lb) for lc in (0, 1) for la in (0, 1) for lb in (0, 1)]
RAGGED = [1, 2, 3, 5, 8, 13, 17, 31, 33, 64, 127, 129]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("lc,la,lb", LAYOUTS)
def test_mtm_ragged_shapes_vs_oracle(cuda, dt, lc, la, lb):
    rng = np.random.default_rng(lc * 4 + la * 2 + lb)
    for M in RAGGED[::2]:
        for N in RAGGED[1::2]:
            for K in (1, 7, 33, 130):
                A = rng.uniform(-1, 1, (M, K)).astype(dt)
                B = rng.uniform(-1, 1, (K, N)).astype(dt)
                C0 = rng.uniform(-1, 1, (M, N)).astype(dt)
                got = run_gemm(cuda, A, B, C0, la, lb, lc)
                ref = O.gemm(A, B, C0, la, lb, lc)
                assert_gemm_close(got, ref, np.abs(A), np.abs(B), C0, K, dt, what=f"{M}x{N}x{K} {lc}{la}{lb}")


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_mtm_reference_test_sizes_exact(cuda, dt):
    """test/test.mtm.cpp: square sz in [2, 32), integer values in [0, 99],
    C starts at zero; every product and sum is exact, so bit equality."""
    rng = np.random.default_rng(1)
    for (lc, la, lb) in LAYOUTS:
        for sz in range(2, 32, 3):
            A = rng.integers(0, 100, (sz, sz)).astype(dt)
            B = rng.integers(0, 100, (sz, sz)).astype(dt)
            Z = np.zeros((sz, sz), dt)
            np.testing.assert_array_equal(run_gemm(cuda, A, B, Z, la, lb, lc), A @ B)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_mtm_general_strides(cuda, dt):
    """Views with no unit stride (the reference honours any strides)."""
    torch = cuda
    import gbblas
    rng = np.random.default_rng(2)
    M, N, K = 37, 29, 45
    Abig = rng.uniform(-1, 1, (M * 2, K * 3)).astype(dt)
    Bbig = rng.uniform(-1, 1, (K * 2, N * 2)).astype(dt)
    A = Abig[::2, ::3]
    B = Bbig[::2, ::2]
    C0 = rng.uniform(-1, 1, (M, N)).astype(dt)
    tA = torch.from_numpy(Abig).cuda()[::2, ::3]
    tB = torch.from_numpy(Bbig).cuda()[::2, ::2]
    tC = torch.from_numpy(C0.copy()).cuda()
    gbblas.gemm(tA, tB, tC)
    torch.cuda.synchronize()
    ref = O.gemm(np.ascontiguousarray(A), np.ascontiguousarray(B), C0, 1, 1, 1)
    assert_gemm_close(tC.cpu().numpy(), ref, np.abs(A), np.abs(B), C0, K, dt)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_mtm_1024_row_major_vs_oracle(cuda, dt):
    """The plain-mtm config: M = N = K = 1024, row-major, U[-1,1) from
    seed 0 (A drawn first), C zeroed."""
    rng = np.random.default_rng(0)
    A = rng.uniform(-1, 1, (1024, 1024)).astype(dt)
    B = rng.uniform(-1, 1, (1024, 1024)).astype(dt)
    Z = np.zeros((1024, 1024), dt)
    got = run_gemm(cuda, A, B, Z, 1, 1, 1)
    ref = O.gemm(A, B, Z, 1, 1, 1)
    assert_gemm_close(got, ref, np.abs(A), np.abs(B), Z, 1024, dt)


def test_mtm_host_entry_accumulates(cuda):
    import gbblas
    rng = np.random.default_rng(4)
    for dt in (np.float32, np.float64):
        M, N, K = 70, 90, 110
        A = rng.uniform(-1, 1, (M, K)).astype(dt)
        B = rng.uniform(-1, 1, (K, N)).astype(dt)
        C = rng.uniform(-1, 1, (M, N)).astype(dt)
        ref = O.gemm(A, B, C, 0, 1, 0)
        a, b, c = O.to_layout(A, 0), O.to_layout(B, 1), O.to_layout(C, 0).copy()
        gbblas.gemm_host(M, N, K, a, 1, M, b, N, 1, c, 1, M)
        assert_gemm_close(O.from_layout(c, M, N, 0), ref, np.abs(A), np.abs(B), C, K, dt)
