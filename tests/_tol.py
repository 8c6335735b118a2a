"""Tolerances of the form c * K * eps used throughout the parity tests.

GEMM / GEMV / plain dot: |gpu - oracle| <= 2 * K * eps_T * (|A||B| + |C0|)
elementwise, K = reduction length (both sides round at most K times; the
reference's own error against FP64 stays below 0.33 K eps on the shapes of
its own tests).  Kahan FP32 dot against the exact sum: 4 * eps_f32 * sum|a_i b_i|
plus half an ulp of the result.
"""
import numpy as np

C_GEMM = 2.0
C_KAHAN = 4.0


def eps(dtype) -> float:
    return float(np.finfo(dtype).eps)


def assert_gemm_close(got, ref, absA, absB, C0, K, dtype, c=C_GEMM, what=""):
    scale = np.asarray(absA, np.float64) @ np.asarray(absB, np.float64) + np.abs(np.asarray(C0, np.float64))
    tol = c * max(K, 1) * eps(dtype) * scale + np.finfo(np.float64).tiny
    err = np.abs(np.asarray(got, np.float64) - np.asarray(ref, np.float64))
    bad = err > tol
    if bad.any():
        i = np.unravel_index(np.argmax(err / tol), err.shape)
        raise AssertionError(f"{what}: {bad.sum()} entries beyond c*K*eps (c={c}); worst at {i}: "
                             f"got {got[i]!r} ref {ref[i]!r} tol {tol[i]:.3g}")


def assert_vec_close(got, ref, scale, K, dtype, c=C_GEMM, what=""):
    tol = c * max(K, 1) * eps(dtype) * np.asarray(scale, np.float64) + np.finfo(np.float64).tiny
    err = np.abs(np.asarray(got, np.float64) - np.asarray(ref, np.float64))
    bad = err > tol
    if bad.any():
        i = int(np.argmax(err / tol))
        raise AssertionError(f"{what}: {bad.sum()} entries beyond c*K*eps; worst at {i}: got {got[i]!r} "
                             f"ref {ref[i]!r} tol {tol[i]:.3g}")


# The reference's f32 division under its -ffast-math x86 build is a
# reciprocal estimate refined by one Newton step, up to 3 ulp from the IEEE
# quotient (measured on 10^5 random quotients); this library divides exactly.
REF_F32_DIV_ULP = 4


def ulp_distance(x, y):
    """Distance in units in the last place between same-sign finite floats."""
    x = np.asarray(x)
    y = np.asarray(y)
    it = np.int32 if x.dtype == np.float32 else np.int64
    return np.abs(x.view(it).astype(np.int64) - y.view(it).astype(np.int64))


def assert_ew_matches_reference(got, ref, op):
    """Element-wise results against values the reference produced: bit equality,
    except float division (see REF_F32_DIV_ULP)."""
    got = np.asarray(got)
    ref = np.asarray(ref)
    if op == 3 and got.dtype == np.float32:
        assert np.all(ulp_distance(got, ref) <= REF_F32_DIV_ULP)
    else:
        np.testing.assert_array_equal(got, ref)
