"""CPU checks of the digit model of the double-precision tensor-core GEMM
(oracle/ozaki.py): the digit split is exact and in range, the model stays
within its stated error bound against exact rational arithmetic, the guard
sum is a true lower bound of sum_k |a_ik| |b_kj|, and the largest digit
sums fit the FP32 accumulator exactly."""
from fractions import Fraction

import numpy as np
import pytest

from oracle import ozaki as OZ


def sample(rng, shape, kind):
    if kind == "uniform":
        return rng.uniform(-1, 1, shape)
    if kind == "wide":
        return rng.choice([-1.0, 1.0], shape) * rng.uniform(1, 2, shape) * np.ldexp(1.0, rng.integers(-10, 11, shape))
    if kind == "tiny":  # subnormals and normals near the bottom of the range
        return rng.uniform(-1, 1, shape) * np.ldexp(1.0, rng.integers(-1074, -1000, shape))
    raise ValueError(kind)


@pytest.mark.parametrize("S", [7, 8])
@pytest.mark.parametrize("kind", ["uniform", "wide", "tiny"])
def test_digits_reconstruct_and_stay_in_range(S, kind):
    rng = np.random.default_rng(1)
    X = sample(rng, (40, 50), kind)
    X[3] = 0.0
    e, bad = OZ.row_scales(X)
    assert not bad.any()
    D = OZ.digits(X, e, S)
    assert D[1:].min() >= -128 and D[1:].max() <= 127
    assert np.abs(D[0]).max() <= 128
    # sum_s D_s 2^(-7-8s) approximates x = a / 2^e to within 2^-8S
    for i in range(0, 40, 7):
        for k in range(0, 50, 9):
            rec = sum(Fraction(int(D[s, i, k])) / 2 ** (7 + 8 * s) for s in range(S))
            x = Fraction(float(X[i, k])) / Fraction(2) ** int(e[i])
            assert abs(rec - x) <= Fraction(1, 2 ** (8 * S))


@pytest.mark.parametrize("S", [7, 8])
@pytest.mark.parametrize("kind", ["uniform", "wide"])
def test_model_within_bound_against_exact_arithmetic(S, kind):
    rng = np.random.default_rng(2)
    M, N, K = 6, 5, 300
    A = sample(rng, (M, K), kind)
    B = sample(rng, (K, N), kind)
    C0 = rng.uniform(-1, 1, (M, N))
    got = OZ.gemm(A, B, C0, S)
    bound = OZ.error_bound(A, B, S)
    for i in range(M):
        for j in range(N):
            exact = Fraction(float(C0[i, j])) + sum(Fraction(float(A[i, k])) * Fraction(float(B[k, j]))
                                                     for k in range(K))
            err = abs(Fraction(float(got[i, j])) - exact)
            assert err <= Fraction(float(bound[i, j])) + 2 * abs(exact) * Fraction(2) ** -52


def test_guard_sum_is_a_lower_bound():
    rng = np.random.default_rng(3)
    for kind in ("uniform", "wide"):
        A = sample(rng, (33, 700), kind)
        B = sample(rng, (700, 17), kind)
        ea, _ = OZ.row_scales(A)
        eb, _ = OZ.row_scales(B.T)
        L = OZ.guard_sums(A, B).astype(np.float64)
        scaled = np.ldexp(L, (ea[:, None] + eb[None, :] - 14).astype(np.int32))
        assert (scaled <= np.abs(A) @ np.abs(B) * (1 + 1e-12)).all()


def test_largest_chunk_sums_fit_fp32_exactly():
    """All seven digits +-128 / 127 with one sign: a group's sum over a
    128-K chunk stays below 2^24, the FP32 accumulator's exact range."""
    S = 7
    D = np.full((S, 1, OZ.CHUNK), 127, np.int64)
    D[0] = 128
    G = OZ.groups(D, D)
    assert np.abs(G).max() < 2 ** 24


def test_bad_rows_give_nan():
    A = np.ones((4, 40))
    B = np.ones((40, 3))
    A[1, 2] = np.inf
    B[5, 2] = np.nan
    got = OZ.gemm(A, B, np.zeros((4, 3)))
    assert np.isnan(got[1]).all() and np.isnan(got[:, 2]).all()
    assert (got[[0, 2, 3]][:, [0, 1]] == 40.0).all()
