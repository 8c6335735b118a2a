"""mtv / vtm on the GPU through the C ABI, against the oracle and the
reference's golden vectors (include/mtv.hpp; test/test.mtv.cpp,
test/test.vtm.cpp)."""
import numpy as np
import pytest

from oracle import oracle as O

import _golden as G
from _tol import assert_vec_close

pytestmark = pytest.mark.gpu


def run(torch, op, A, x, y0, layout):
    """Run gbblas mtv/vtm on the dense buffer of A in `layout`; returns y."""
    import gbblas
    M, N = A.shape
    tA = torch.from_numpy(O.to_layout(A, layout)).cuda()
    tx = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    ty = torch.from_numpy(np.ascontiguousarray(y0).copy()).cuda()
    getattr(gbblas, op)(layout, M, N, tA, tx, ty)
    torch.cuda.synchronize()
    return ty.cpu().numpy()


@pytest.mark.parametrize("name", G.names("mtv_"))
def test_mtv_golden(cuda, name):
    c = G.case(name)
    dt = c["y"].dtype
    A, x, y0 = c["A"].astype(dt), c["x"].astype(dt), c["y0"].astype(dt)
    got = run(cuda, "mtv", A, x, y0, int(c["la"]))
    if int(c["exact"]):
        np.testing.assert_array_equal(got, c["y"])
    else:
        assert_vec_close(got, c["y"], np.abs(A) @ np.abs(x) + np.abs(y0), A.shape[1], dt, what=name)


@pytest.mark.parametrize("name", G.names("vtm_"))
def test_vtm_golden(cuda, name):
    c = G.case(name)
    dt = c["y"].dtype
    A, v, y0 = c["A"].astype(dt), c["v"].astype(dt), c["y0"].astype(dt)
    np.testing.assert_array_equal(run(cuda, "vtm", A, v, y0, int(c["la"])), c["y"])


SHAPES = [(2, 2), (3, 7), (7, 3), (17, 33), (33, 17), (64, 1000), (1000, 64), (129, 4097), (4097, 129),
          (2, 300000), (300000, 2), (1024, 1024), (2048, 16384)]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("layout", [0, 1])
def test_mtv_random_vs_oracle(cuda, dt, shape, layout):
    M, N = shape
    rng = np.random.default_rng(M * 31 + N)
    A = rng.uniform(-1, 1, (M, N)).astype(dt)
    x = rng.uniform(-1, 1, N).astype(dt)
    y0 = rng.uniform(-1, 1, M).astype(dt)
    got = run(cuda, "mtv", A, x, y0, layout)
    ref = O.mtv(A, x, y0, layout)
    scale = np.abs(A) @ np.abs(x) + (np.abs(y0) if layout == 0 else 0)
    assert_vec_close(got, ref, scale, N, dt, what=f"mtv {shape} layout {layout}")


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("layout", [0, 1])
def test_vtm_random_vs_oracle(cuda, dt, shape, layout):
    """Every shape and layout computes y = v^T A (the reference's own vtm is
    only right for square column-major A; the oracle and this library are
    right for all)."""
    M, N = shape
    rng = np.random.default_rng(M * 7 + N)
    A = rng.uniform(-1, 1, (M, N)).astype(dt)
    v = rng.uniform(-1, 1, M).astype(dt)
    y0 = rng.uniform(-1, 1, N).astype(dt)
    got = run(cuda, "vtm", A, v, y0, layout)
    ref = O.vtm(A, v, y0, layout)
    scale = np.abs(v) @ np.abs(A) + (np.abs(y0) if layout == 1 else 0)
    assert_vec_close(got, ref, scale, M, dt, what=f"vtm {shape} layout {layout}")


def test_mtv_semantics_overwrite_vs_accumulate(cuda):
    # reference behaviour: y starts at 5, A and x ones (n = 1000):
    # row-major overwrites -> 1000, column-major accumulates -> 1005
    n = 1000
    A = np.ones((n, n), np.float32)
    x = np.ones(n, np.float32)
    y0 = np.full(n, 5, np.float32)
    assert np.all(run(cuda, "mtv", A, x, y0, 1) == 1000)
    assert np.all(run(cuda, "mtv", A, x, y0, 0) == 1005)


def test_mtv_host_entry(cuda):
    import gbblas
    rng = np.random.default_rng(9)
    for dt in (np.float32, np.float64):
        for layout in (0, 1):
            A = rng.uniform(-1, 1, (300, 257)).astype(dt)
            x = rng.uniform(-1, 1, 257).astype(dt)
            y = rng.uniform(-1, 1, 300).astype(dt)
            ref = O.mtv(A, x, y, layout)
            buf = O.to_layout(A, layout)
            gbblas.mtv_host(layout, 300, 257, buf, x, y)
            assert_vec_close(y, ref, np.abs(A) @ np.abs(x) + 1, 257, dt)
            v = rng.uniform(-1, 1, 300).astype(dt)
            z = rng.uniform(-1, 1, 257).astype(dt)
            refz = O.vtm(A, v, z, layout)
            gbblas.vtm_host(layout, 300, 257, buf, v, z)
            assert_vec_close(z, refz, np.abs(v) @ np.abs(A) + 1, 300, dt)


def test_mtv_full_size_properties(cuda):
    """16384 x 16384 row-major float32 (the bandwidth config): linearity
    A(x1 + x2) = Ax1 + Ax2 within tolerance, determinism, and spot rows
    against long-double dots."""
    torch = cuda
    import gbblas
    M = N = 16384
    g = torch.Generator(device="cuda").manual_seed(1)
    A = torch.rand(M, N, device="cuda", generator=g) * 2 - 1
    x1 = torch.rand(N, device="cuda", generator=g) * 2 - 1
    x2 = torch.rand(N, device="cuda", generator=g) * 2 - 1
    y1 = torch.empty(M, device="cuda")
    y2 = torch.empty(M, device="cuda")
    y12 = torch.empty(M, device="cuda")
    gbblas.mtv(1, M, N, A, x1, y1)
    gbblas.mtv(1, M, N, A, x2, y2)
    gbblas.mtv(1, M, N, A, x1 + x2, y12)
    again = torch.empty(M, device="cuda")
    gbblas.mtv(1, M, N, A, x1, again)
    torch.cuda.synchronize()
    assert torch.equal(y1, again)
    scale = (A.abs() @ (x1.abs() + x2.abs())).double()
    err = (y12.double() - y1.double() - y2.double()).abs()
    assert bool((err <= 4 * N * np.finfo(np.float32).eps * scale).all())
    rows = np.random.default_rng(0).integers(0, M, 64)
    An = A[torch.from_numpy(rows).cuda()].cpu().numpy()
    xn = x1.cpu().numpy()
    for i, r in enumerate(rows):
        exact, absdot = O.dot_exact(An[i], xn)
        assert abs(y1[r].item() - exact) <= 2 * N * np.finfo(np.float32).eps * absdot
