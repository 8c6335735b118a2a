"""Pin the CPU oracle (oracle/oracle.c) against the reference.

* the reference's own known answers: the 3x3 pack permutations of
  test/test.pack.cpp:8-83 and the closed-form dot of test/test.dot_prod.cpp
  (iota(1..s) . iota(1..s) = s(s+1)(2s+1)/6);
* golden vectors written by the reference's own compiled headers
  (tests/golden/make_golden.py, oracle/_ref);
* where oracle/_ref is present (this needs the reference sources), fresh
  random cases against the reference directly.
"""
import numpy as np
import pytest

from oracle import oracle as O

import _golden as G
from _tol import assert_ew_matches_reference, assert_gemm_close, assert_vec_close


# ------------------------------------------------------------ known answers

def test_pack_plain_known_answer():
    # test/test.pack.cpp:48-84: in = iota 3x3 column-major, MR = 2
    inp = np.arange(1, 10, dtype=np.float32)
    out = np.arange(1, 10, dtype=np.float32)
    w = (1, 3)
    for i in range(0, 3, 2):
        ib = min(2, 3 - i)
        O.pack(inp, w, ib, ib, 3, out, offset_in=i * w[0], offset_out=i * 3)
    expect_pairs = [(0, 0), (1, 1), (2, 6), (3, 2), (4, 3), (5, 7), (6, 4), (7, 5), (8, 8)]
    for i_in, i_out in expect_pairs:
        assert inp[i_in] == out[i_out]
    np.testing.assert_array_equal(out, G.case("pack_plain_3x3")["out"])


def test_pack_trans_known_answer():
    # test/test.pack.cpp:87-123
    inp = np.arange(1, 10, dtype=np.float32)
    out = np.arange(1, 10, dtype=np.float32)
    w = (1, 3)
    for i in range(0, 3, 2):
        ib = min(2, 3 - i)
        O.pack(inp, w, ib, ib, 3, out, offset_in=i * w[1], offset_out=i * 3, trans=True)
    expect_pairs = [(0, 0), (1, 2), (2, 4), (3, 1), (4, 3), (5, 5), (6, 6), (7, 7), (8, 8)]
    for i_in, i_out in expect_pairs:
        assert inp[i_in] == out[i_out]
    np.testing.assert_array_equal(out, G.case("pack_trans_3x3")["out"])


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_dot_closed_form_iota(dt):
    # test/test.dot_prod.cpp:20-27 runs every s in [2, 2^17+2); a stride of
    # sizes keeps this fast while still crossing all three regimes.
    sizes = list(range(2, 300)) + list(range(300, 1 << 17, 997)) + [(1 << 17) + 1]
    for s in sizes:
        a = np.arange(1, s + 1, dtype=dt)
        exact = s * (s + 1) * (2 * s + 1) // 6
        r = O.dot(a, a)
        # Catch2 Approx default: relative 100 * FLT_EPSILON
        assert abs(r - exact) <= 100 * np.finfo(np.float32).eps * exact, (s, r, exact)


# ------------------------------------------------------------ golden vectors

@pytest.mark.parametrize("name", G.names("mtm_"))
def test_mtm_golden(name):
    c = G.case(name)
    dt = c["C"].dtype
    A, B, C0 = c["A"].astype(dt), c["B"].astype(dt), c["C0"].astype(dt)
    got = O.gemm(A, B, C0, int(c["la"]), int(c["lb"]), int(c["lc"]))
    if int(c["exact"]):
        np.testing.assert_array_equal(got, c["C"])
    else:
        assert_gemm_close(got, c["C"], np.abs(A), np.abs(B), C0, A.shape[1], dt, what=name)


@pytest.mark.parametrize("name", G.names("mtv_"))
def test_mtv_golden(name):
    c = G.case(name)
    dt = c["y"].dtype
    A, x, y0 = c["A"].astype(dt), c["x"].astype(dt), c["y0"].astype(dt)
    got = O.mtv(A, x, y0, int(c["la"]))
    if int(c["exact"]):
        np.testing.assert_array_equal(got, c["y"])
    else:
        assert_vec_close(got, c["y"], np.abs(A) @ np.abs(x) + np.abs(y0), A.shape[1], dt, what=name)


@pytest.mark.parametrize("name", G.names("vtm_"))
def test_vtm_golden(name):
    c = G.case(name)
    dt = c["y"].dtype
    A, v, y0 = c["A"].astype(dt), c["v"].astype(dt), c["y0"].astype(dt)
    got = O.vtm(A, v, y0, int(c["la"]))
    np.testing.assert_array_equal(got, c["y"])


@pytest.mark.parametrize("name", G.names("dot_"))
def test_dot_golden(name):
    c = G.case(name)
    dt = c["r"].dtype
    if "n" in c:
        a = np.arange(1, int(c["n"]) + 1, dtype=dt)
        b = a
    else:
        a, b = c["a"].astype(dt), c["b"].astype(dt)
    got = O.dot(a, b)
    closed = float(c["closed"])
    assert abs(got - closed) <= 100 * np.finfo(np.float32).eps * closed
    if int(c["exact"]):
        assert got == c["r"] == closed


# ------------------------------------------------------------ reference semantics

def test_mtv_overwrite_and_accumulate_semantics():
    # y starts at 5, A and x are ones (n = 1000): row-major overwrites (1000),
    # column-major accumulates (1005) - reference include/mtv.hpp:62,74,95.
    n = 1000
    A = np.ones((n, n), np.float32)
    x = np.ones(n, np.float32)
    y0 = np.full(n, 5, np.float32)
    assert np.all(O.mtv(A, x, y0, O.LAST_ORDER) == 1000)
    assert np.all(O.mtv(A, x, y0, O.FIRST_ORDER) == 1005)


def test_mtm_accumulates_into_c():
    A = np.ones((4, 3), np.float64)
    B = np.ones((3, 5), np.float64)
    C0 = np.full((4, 5), 2.0)
    for lc in (0, 1):
        np.testing.assert_array_equal(O.gemm(A, B, C0, 1, 0, lc), np.full((4, 5), 5.0))


def test_partition_matches_reference_formulas():
    # Register tiles from the Skylake table (include/cpuinfo.hpp):
    # float 16x6, double 8x6, double with row-major C 6x8.
    assert (O.partition(np.float32, 0)["MR"], O.partition(np.float32, 0)["NR"]) == (16, 6)
    assert (O.partition(np.float64, 0)["MR"], O.partition(np.float64, 0)["NR"]) == (8, 6)
    assert (O.partition(np.float64, 1)["MR"], O.partition(np.float64, 1)["NR"]) == (6, 8)


# ------------------------------------------------------------ against the compiled reference

needs_ref = pytest.mark.skipif(not O.ref_available(), reason="oracle/_ref not built (needs the reference sources)")


@needs_ref
def test_cache_geometry_matches_reference():
    assert O.cache_info() == O.ref_cache_info()


@needs_ref
@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("shape", [(2, 2, 2), (33, 17, 65), (100, 37, 513), (300, 200, 1100)])
def test_mtm_bitexact_vs_reference(dt, shape):
    rng = np.random.default_rng(hash(shape) % 1000)
    M, N, K = shape
    A = rng.uniform(-1, 1, (M, K)).astype(dt)
    B = rng.uniform(-1, 1, (K, N)).astype(dt)
    C0 = rng.uniform(-1, 1, (M, N)).astype(dt)
    for lc in (0, 1):
        for la in (0, 1):
            for lb in (0, 1):
                np.testing.assert_array_equal(O.gemm(A, B, C0, la, lb, lc), O.ref_gemm(A, B, C0, la, lb, lc))


@needs_ref
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_mtv_vs_reference(dt):
    rng = np.random.default_rng(7)
    for (M, N) in [(2, 2), (17, 33), (300, 300), (1000, 513)]:
        A = rng.uniform(-1, 1, (M, N)).astype(dt)
        x = rng.uniform(-1, 1, N).astype(dt)
        y0 = rng.uniform(-1, 1, M).astype(dt)
        for la in (0, 1):
            got, ref = O.mtv(A, x, y0, la), O.ref_mtv(A, x, y0, la)
            if la == 1:
                np.testing.assert_array_equal(got, ref)
            else:
                assert_vec_close(got, ref, np.abs(A) @ np.abs(x) + np.abs(y0), N, dt)


@needs_ref
def test_reference_vtm_is_wrong_except_square_column_major():
    """Documents the reference defect the drop-in corrects
    (include/mtv.hpp:224-227): only square column-major A gives v^T A."""
    rng = np.random.default_rng(3)
    for dt in (np.float32, np.float64):
        A = rng.uniform(-1, 1, (64, 64)).astype(dt)
        v = rng.uniform(-1, 1, 64).astype(dt)
        y0 = np.zeros(64, dt)
        np.testing.assert_allclose(O.ref_vtm(A, v, y0, 0), v @ A, rtol=1e-4, atol=1e-4)
        assert np.max(np.abs(O.ref_vtm(A, v, y0, 1) - v @ A)) > 1e-2
        np.testing.assert_allclose(O.vtm(A, v, y0, 1), v @ A, rtol=1e-4, atol=1e-4)
        An = rng.uniform(-1, 1, (60, 40)).astype(dt)
        vn = rng.uniform(-1, 1, 60).astype(dt)
        np.testing.assert_allclose(O.vtm(An, vn, np.zeros(40, dt), 0), vn @ An, rtol=1e-4, atol=1e-4)


@needs_ref
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_dot_vs_reference(dt):
    rng = np.random.default_rng(11)
    for n in (2, 100, 30000, 10 ** 6):
        a = rng.uniform(-1, 1, n).astype(dt)
        b = rng.uniform(-1, 1, n).astype(dt)
        _, absdot = O.dot_exact(a, b)
        assert abs(O.dot(a, b) - O.ref_dot(a, b)) <= 2 * n * np.finfo(dt).eps * absdot
        assert abs(O.dot_tuning(a, b, 64, 32, 1024) - O.ref_dot_tuning(a, b, 64, 32, 1024)) <= 2 * n * np.finfo(dt).eps * absdot


# ------------------------------------------- outer / transpose / element-wise

def _dt(name):
    return np.float64 if "float64" in name else np.float32


@pytest.mark.parametrize("name", G.names("outer_"))
def test_outer_golden_exact(name):
    c = G.case(name)
    dt = _dt(name)
    got = O.outer(c["a"].astype(dt), c["b"].astype(dt), c["C0"].astype(dt), int(c["lc"]))
    np.testing.assert_array_equal(got, c["C"])


@pytest.mark.parametrize("name", [n for n in G.names("transpose_") if "inplace" not in n])
def test_transpose_golden_exact(name):
    c = G.case(name)
    np.testing.assert_array_equal(O.transpose(c["A"], int(c["la"]), int(c["lc"])), c["C"])


@pytest.mark.parametrize("name", G.names("transpose_inplace_"))
def test_transpose_inplace_golden_exact(name):
    c = G.case(name)
    np.testing.assert_array_equal(O.transpose_inplace(c["inp"]), c["out"])


@pytest.mark.parametrize("name", G.names("ew_"))
def test_ew_golden(name):
    c = G.case(name)
    assert_ew_matches_reference(O.ew(int(c["op"]), c["a"], c["b"]), c["c"], int(c["op"]))


def test_ew_division_is_ieee():
    rng = np.random.default_rng(3)
    a = rng.uniform(-1, 1, 10000).astype(np.float32)
    b = rng.uniform(0.5, 3, 10000).astype(np.float32)
    np.testing.assert_array_equal(O.ew(3, a, b), a / b)
    np.testing.assert_array_equal(O.ew(3, a.astype(np.float64), b.astype(np.float64)), a.astype(np.float64) / b)


def test_outer_matches_definition():
    rng = np.random.default_rng(7)
    a = rng.integers(-50, 50, 40).astype(np.float64)
    b = rng.integers(-50, 50, 23).astype(np.float64)
    C = rng.integers(-50, 50, (40, 23)).astype(np.float64)
    for lc in (0, 1):
        np.testing.assert_array_equal(O.outer(a, b, C, lc), C + np.outer(a, b))


@pytest.mark.skipif(not O.ref_available(), reason="reference sources not present")
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_stream_ops_bitexact_vs_reference(dt):
    rng = np.random.default_rng(11)
    for (M, N) in [(3, 2), (65, 129), (300, 7)]:
        a, b = rng.uniform(-1, 1, M).astype(dt), rng.uniform(-1, 1, N).astype(dt)
        C = rng.uniform(-1, 1, (M, N)).astype(dt)
        A = rng.uniform(-1, 1, (M, N)).astype(dt)
        for lc in (0, 1):
            np.testing.assert_array_equal(O.outer(a, b, C, lc), O.ref_outer(a, b, C, lc))
            for la in (0, 1):
                np.testing.assert_array_equal(O.transpose(A, la, lc), O.ref_transpose(A, la, lc))
    s = rng.uniform(-1, 1, 77 * 77).astype(dt)
    np.testing.assert_array_equal(O.transpose_inplace(s), O.ref_transpose_inplace(s))
    x, y = rng.uniform(-1, 1, 4099).astype(dt), rng.uniform(0.25, 4, 4099).astype(dt)
    for op in range(4):
        assert_ew_matches_reference(O.ew(op, x, y), O.ref_ew(op, x, y), op)
