"""Full-output parity at the sizes the bandwidth figures are measured on, on
the seeded inputs both benchmark arms use (gbblas_seeded_fill: one
std::mt19937_64(1) draws A, x, a, b in that order; the float32 and float64
sets come from the same draws).

* mtv y = A x, A 16384 x 16384 row-major, float32 and float64: every entry of
  y against the oracle's restatement of the reference's mtv
  (include/mtv.hpp:72-98) within 2 K eps (|A||x|)_i.
* dot of two 2^28 vectors, float32 and float64: against the oracle's
  three-regime dot (include/dot.hpp:143-174) within 2 n eps sum|a_i b_i|, and
  against the exact sum (long double) - the Kahan float32 dot within
  4 eps sum|a_i b_i| + eps |dot|.
* the host-buffer entry points (what the drop-in headers call) give the same
  bits as the device entry points on these inputs.

Then the reference's 32 Ki tests (test/test.mtv.cpp:128-211,
test/test.vtm.cpp:127-211): 32768 x 32768 matrices of both layouts, float and
double, integer entries in [0, 99] as the reference's rand() % 100 rule
(test/test_utils.hpp:4-8), here drawn from the seeded generator; mtv and vtm
against the oracle (double: exact integer sums, so bit for bit).
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from _tol import assert_vec_close

pytestmark = pytest.mark.gpu

M = N = 16384
NDOT = 1 << 28


@pytest.fixture(scope="module")
def bw_inputs(cuda):
    """The bandwidth configuration's inputs on the host, float32 and float64."""
    import gbblas
    O.set_threads(os.cpu_count() or 1)
    f32 = [np.empty(M * N, np.float32), np.empty(N, np.float32), np.empty(NDOT, np.float32),
           np.empty(NDOT, np.float32)]
    f64 = [np.empty(M * N), np.empty(N), np.empty(NDOT), np.empty(NDOT)]
    gbblas.seeded_fill(1, f32, f64)
    return {"f32": f32, "f64": f64}


@pytest.mark.parametrize("tag", ["f32", "f64"])
def test_mtv_16384_full_output(cuda, bw_inputs, tag):
    torch = cuda
    import gbblas
    A, x, _, _ = bw_inputs[tag]
    dt = A.dtype
    tA, tx = torch.from_numpy(A).cuda(), torch.from_numpy(x).cuda()
    ty = torch.full((M,), float("nan"), dtype=tA.dtype, device="cuda")
    gbblas.mtv(1, M, N, tA, tx, ty)
    torch.cuda.synchronize()
    got = ty.cpu().numpy()
    ref = np.zeros(M, dt)
    O.mtv_raw(1, M, N, A, x, ref)
    scale = (tA.view(M, N).abs().double() @ tx.abs().double()).cpu().numpy()
    assert_vec_close(got, ref, scale, N, dt, what=f"mtv {tag} 16384^2 vs oracle")
    # the drop-in's host-buffer call computes the same bits
    yh = np.full(M, np.nan, dt)
    gbblas.mtv_host(1, M, N, A, x, yh)
    np.testing.assert_array_equal(yh, got)
    del tA


@pytest.mark.parametrize("tag", ["f32", "f64"])
def test_dot_2pow28_full(cuda, bw_inputs, tag):
    torch = cuda
    import gbblas
    _, _, a, b = bw_inputs[tag]
    dt = a.dtype
    eps = float(np.finfo(dt).eps)
    ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    out = torch.zeros(1, dtype=ta.dtype, device="cuda")
    gbblas.dot(ta, tb, out)
    torch.cuda.synchronize()
    got = out.item()
    ref = float(O.dot(a, b))
    exact, absdot = O.dot_exact(a, b)
    assert abs(got - ref) <= 2 * NDOT * eps * absdot, (tag, got, ref)
    if tag == "f32":
        assert abs(got - exact) <= 4 * eps * absdot + eps * abs(exact), (got, exact)
    else:
        assert abs(got - exact) <= 2 * NDOT * eps * absdot, (got, exact)
    assert gbblas.dot_host(a, b) == np.asarray(got, dt)
    del ta, tb


@pytest.fixture(scope="module")
def ints_32ki(cuda):
    """32768 x 32768 integer entries in [0, 99] and a 32768 vector, float and
    double from the same draws (seed 32768)."""
    import gbblas
    sz = 32 * 1024
    A32, v32 = np.empty(sz * sz, np.float32), np.empty(sz, np.float32)
    gbblas.seeded_fill(32768, [A32, v32], None)
    for t in (A32, v32):  # U[-1,1) -> floor(50 (u + 1)) in [0, 99], exact in float
        t += 1.0
        t *= 50.0
        np.floor(t, out=t)
    return sz, A32, v32


@pytest.mark.parametrize("dtname", ["float", "double"])
@pytest.mark.parametrize("layout", [0, 1])
@pytest.mark.parametrize("op", ["mtv", "vtm"])
def test_reference_32ki_cases(cuda, ints_32ki, op, layout, dtname):
    torch = cuda
    import gbblas
    sz, A32, v32 = ints_32ki
    dt = np.float32 if dtname == "float" else np.float64
    A = A32 if dt == np.float32 else A32.astype(np.float64)
    v = v32.astype(dt)
    tA, tv = torch.from_numpy(A).cuda(), torch.from_numpy(v).cuda()
    ty = torch.zeros(sz, dtype=tA.dtype, device="cuda")  # both forms give A v (or v A) from zero
    getattr(gbblas, op)(layout, sz, sz, tA, tv, ty)
    torch.cuda.synchronize()
    got = ty.cpu().numpy()
    ref = np.zeros(sz, dt)
    getattr(O.lib(), f"orc_{'s' if dt == np.float32 else 'd'}{op}")(layout, sz, sz, A.ctypes.data, v.ctypes.data,
                                                                     ref.ctypes.data)
    if dt == np.float64:
        np.testing.assert_array_equal(got, ref)  # integer sums below 2^53: exact on both sides
    else:
        # (|A||v|) = A v for non-negative entries; the double result is exact
        ex = np.zeros(sz)
        A64 = A.astype(np.float64)
        getattr(O.lib(), f"orc_d{op}")(layout, sz, sz, A64.ctypes.data, v.astype(np.float64).ctypes.data,
                                       ex.ctypes.data)
        del A64
        assert_vec_close(got, ref, ex, sz, dt, what=f"{op} layout {layout} float 32Ki vs oracle")
    del tA, tv
    torch.cuda.empty_cache()
