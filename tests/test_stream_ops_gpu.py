"""Outer product, transpose and element-wise ops on the GPU through the C ABI,
against the reference's golden vectors and the oracle: bit equality (each
output element is one fused multiply-add, one copy or one IEEE operation).

Edge cases: empty sizes, 1 x n and n x 1 shapes, sizes that are not
multiples of the vector width or the 32 x 32 tile, operands at unaligned
addresses (scalar paths), padded leading dimensions, in-place element-wise
(c aliasing a), and the host-pointer entry points the drop-in headers call.
Large sizes are checked through size-independent properties.
"""
import numpy as np
import pytest

from oracle import oracle as O

import _golden as G
from _tol import assert_ew_matches_reference

pytestmark = pytest.mark.gpu


def _dt(name):
    return np.float64 if "float64" in name else np.float32


def _pfx(dt):
    return "d" if np.dtype(dt) == np.float64 else "s"


def dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def outer_gpu(torch, a, b, C, lc):
    import gbblas
    M, N = C.shape
    dt = C.dtype
    tC = dev(torch, O.to_layout(C, lc).copy())
    ta, tb = dev(torch, a.astype(dt)), dev(torch, b.astype(dt))
    gbblas.call(f"gbblas_{_pfx(dt)}outer", lc, M, N, ta.data_ptr(), tb.data_ptr(), tC.data_ptr(), None)
    gbblas.call("gbblas_check_stream", None)
    return O.from_layout(tC.cpu().numpy(), M, N, lc)


def transpose_gpu(torch, A, la, lc):
    import gbblas
    M, N = A.shape
    tA = dev(torch, O.to_layout(A, la))
    tC = torch.zeros(M * N, dtype=tA.dtype, device="cuda")
    rsa, csa = O.strides(M, N, la)
    rsc, csc = O.strides(N, M, lc)
    gbblas.call(f"gbblas_{_pfx(A.dtype)}transpose", M, N, tA.data_ptr(), rsa, csa, tC.data_ptr(), rsc, csc, None)
    gbblas.call("gbblas_check_stream", None)
    return O.from_layout(tC.cpu().numpy(), N, M, lc)


def ew_gpu(torch, op, a, b, offset=0):
    """offset > 0 places all three operands `offset` elements into their
    buffers, so none is 16-byte aligned (the scalar path)."""
    import gbblas
    n = a.size
    ta = torch.zeros(n + offset, dtype=torch.float64 if a.dtype == np.float64 else torch.float32, device="cuda")
    tb, tc = torch.zeros_like(ta), torch.zeros_like(ta)
    ta[offset:] = dev(torch, a)
    tb[offset:] = dev(torch, b)
    es = a.itemsize
    gbblas.call(f"gbblas_{_pfx(a.dtype)}ew", op, n, ta.data_ptr() + offset * es, tb.data_ptr() + offset * es,
                tc.data_ptr() + offset * es, None)
    gbblas.call("gbblas_check_stream", None)
    return tc[offset:].cpu().numpy()


# ------------------------------------------------------------ golden vectors

@pytest.mark.parametrize("name", G.names("outer_"))
def test_outer_golden(cuda, name):
    c = G.case(name)
    dt = _dt(name)
    got = outer_gpu(cuda, c["a"].astype(dt), c["b"].astype(dt), c["C0"].astype(dt), int(c["lc"]))
    np.testing.assert_array_equal(got, c["C"])


@pytest.mark.parametrize("name", [n for n in G.names("transpose_") if "inplace" not in n])
def test_transpose_golden(cuda, name):
    c = G.case(name)
    np.testing.assert_array_equal(transpose_gpu(cuda, c["A"], int(c["la"]), int(c["lc"])), c["C"])


@pytest.mark.parametrize("name", G.names("transpose_inplace_"))
def test_transpose_inplace_golden(cuda, name):
    import gbblas
    c = G.case(name)
    t = dev(cuda, c["inp"])
    gbblas.call(f"gbblas_{_pfx(c['inp'].dtype)}transpose_inplace", int(c["n"]), t.data_ptr(), None)
    np.testing.assert_array_equal(t.cpu().numpy(), c["out"])


@pytest.mark.parametrize("name", G.names("ew_"))
def test_ew_golden(cuda, name):
    c = G.case(name)
    assert_ew_matches_reference(ew_gpu(cuda, int(c["op"]), c["a"], c["b"]), c["c"], int(c["op"]))


# -------------------------------------------------------- against the oracle

@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("shape", [(1, 1), (1, 37), (37, 1), (5, 3), (129, 257), (1000, 999), (4096, 1024)])
@pytest.mark.parametrize("lc", [0, 1])
def test_outer_vs_oracle(cuda, dt, shape, lc):
    M, N = shape
    rng = np.random.default_rng(M * 7 + N)
    a, b = rng.uniform(-1, 1, M).astype(dt), rng.uniform(-1, 1, N).astype(dt)
    C = rng.uniform(-1, 1, (M, N)).astype(dt)
    np.testing.assert_array_equal(outer_gpu(cuda, a, b, C, lc), O.outer(a, b, C, lc))


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("shape", [(1, 1), (1, 33), (33, 1), (31, 33), (64, 64), (1000, 999), (4097, 300)])
@pytest.mark.parametrize("la,lc", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_transpose_vs_oracle(cuda, dt, shape, la, lc):
    M, N = shape
    A = np.random.default_rng(M + 3 * N).uniform(-1, 1, (M, N)).astype(dt)
    np.testing.assert_array_equal(transpose_gpu(cuda, A, la, lc), A.T)


def test_transpose_padded_strides(cuda):
    """A with a padded leading dimension into a padded C: gaps untouched."""
    import gbblas
    M, N, lda, ldc = 70, 45, 80, 96
    rng = np.random.default_rng(3)
    Abuf = rng.uniform(-1, 1, M * lda).astype(np.float32)  # row-major, row pitch lda
    Cbuf = np.full(N * ldc, 7.0, np.float32)                # row-major N x M, row pitch ldc
    tA, tC = dev(cuda, Abuf), dev(cuda, Cbuf)
    gbblas.call("gbblas_stranspose", M, N, tA.data_ptr(), lda, 1, tC.data_ptr(), ldc, 1, None)
    got = tC.cpu().numpy()
    want = Cbuf.copy()
    O.transpose_raw(M, N, Abuf, lda, 1, want, ldc, 1)
    np.testing.assert_array_equal(got, want)
    assert np.all(got.reshape(N, ldc)[:, M:] == 7.0)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("n", [1, 2, 31, 32, 33, 100, 1000])
def test_transpose_inplace_vs_oracle(cuda, dt, n):
    import gbblas
    buf = np.random.default_rng(n).uniform(-1, 1, n * n).astype(dt)
    t = dev(cuda, buf)
    gbblas.call(f"gbblas_{_pfx(dt)}transpose_inplace", n, t.data_ptr(), None)
    np.testing.assert_array_equal(t.cpu().numpy(), O.transpose_inplace(buf))


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("n", [0, 1, 3, 4, 1000, 1000003])
@pytest.mark.parametrize("offset", [0, 1])
def test_ew_vs_oracle(cuda, dt, n, offset):
    rng = np.random.default_rng(n + offset)
    a = rng.uniform(-1, 1, n).astype(dt)
    b = (rng.uniform(0.5, 2, n) * rng.choice([-1, 1], n)).astype(dt)
    for op in range(4):
        np.testing.assert_array_equal(ew_gpu(cuda, op, a, b, offset), O.ew(op, a, b))


def test_ew_in_place(cuda):
    import gbblas
    rng = np.random.default_rng(5)
    a = rng.uniform(-1, 1, 100003).astype(np.float32)
    b = rng.uniform(-1, 1, 100003).astype(np.float32)
    ta, tb = dev(cuda, a), dev(cuda, b)
    gbblas.call("gbblas_sew", 0, a.size, ta.data_ptr(), tb.data_ptr(), ta.data_ptr(), None)  # a = a + b
    np.testing.assert_array_equal(ta.cpu().numpy(), O.ew(0, a, b))


# ------------------------------------------------------ host entry points

def test_host_entry_points(cuda):
    import gbblas
    rng = np.random.default_rng(8)
    a = rng.uniform(-1, 1, 300).astype(np.float64)
    b = rng.uniform(-1, 1, 200).astype(np.float64)
    C = rng.uniform(-1, 1, (300, 200))
    for lc in (0, 1):
        buf = O.to_layout(C, lc).copy()
        gbblas.call("gbblas_douter_host", lc, 300, 200, a.ctypes.data, b.ctypes.data, buf.ctypes.data)
        np.testing.assert_array_equal(O.from_layout(buf, 300, 200, lc), O.outer(a, b, C, lc))
    A = rng.uniform(-1, 1, (300, 200)).astype(np.float32)
    out = np.zeros(300 * 200, np.float32)
    gbblas.call("gbblas_stranspose_host", 300, 200, A.ctypes.data, 200, 1, out.ctypes.data, 300, 1)
    np.testing.assert_array_equal(out.reshape(200, 300), A.T)
    sq = rng.uniform(-1, 1, 77 * 77).astype(np.float32)
    want = O.transpose_inplace(sq)
    gbblas.call("gbblas_stranspose_inplace_host", 77, sq.ctypes.data)
    np.testing.assert_array_equal(sq, want)
    x, y = rng.uniform(-1, 1, 999), rng.uniform(1, 2, 999)
    z = np.zeros(999)
    gbblas.call("gbblas_dew_host", 3, 999, x.ctypes.data, y.ctypes.data, z.ctypes.data)
    np.testing.assert_array_equal(z, x / y)


# ------------------------------------------------ large sizes, by property

def test_large_sizes_by_property(cuda):
    """16384 x 8192 f32: transpose twice is the identity; outer of a one-hot
    a adds b to exactly one row; a - b + b recovers a where exact."""
    import gbblas
    torch = cuda
    M, N = 16384, 8192
    g = torch.Generator(device="cuda").manual_seed(1)
    A = torch.rand(M, N, generator=g, device="cuda")
    T = torch.empty(N, M, device="cuda")
    B = torch.empty(M, N, device="cuda")
    gbblas.call("gbblas_stranspose", M, N, A.data_ptr(), N, 1, T.data_ptr(), M, 1, None)
    gbblas.call("gbblas_stranspose", N, M, T.data_ptr(), M, 1, B.data_ptr(), N, 1, None)
    torch.cuda.synchronize()
    assert torch.equal(A, B)
    assert torch.equal(T[:7, :5], A[:5, :7].t())
    u = torch.zeros(M, device="cuda")
    u[12345] = 1.0
    v = torch.rand(N, generator=g, device="cuda")
    C = torch.zeros(M, N, device="cuda")
    gbblas.call("gbblas_souter", 1, M, N, u.data_ptr(), v.data_ptr(), C.data_ptr(), None)
    torch.cuda.synchronize()
    assert torch.equal(C[12345], v)
    assert int((C != 0).sum()) == int((v != 0).sum())
    x = torch.randint(-1000, 1000, (M * 64,), generator=g, device="cuda").float()
    y = torch.randint(-1000, 1000, (M * 64,), generator=g, device="cuda").float()
    z = torch.empty_like(x)
    gbblas.call("gbblas_sew", 1, x.numel(), x.data_ptr(), y.data_ptr(), z.data_ptr(), None)
    gbblas.call("gbblas_sew", 0, x.numel(), z.data_ptr(), y.data_ptr(), z.data_ptr(), None)
    torch.cuda.synchronize()
    assert torch.equal(z, x)
