"""numpy model of the low-accuracy GEMM's arithmetic.  TEST INFRASTRUCTURE ONLY.

The reference has no FP8 path (its mtm is FP32/FP64 on the CPU,
include/mtm.hpp:116-206); GBBLAS_ACCURACY_FP8 is this library's own request
for a low-accuracy result.  This module restates that path's published
arithmetic so tests can tell quantisation error (expected, large) from a
wrong kernel (a mismatch against this model):

* E4M3 (OCP FP8, 1 sign, 4 exponent bits with bias 7, 3 mantissa bits, no
  infinities, largest finite 448, smallest subnormal 2^-9), rounding to
  nearest-even with saturation to +-448;
* per 128-element block along K (a row of A, a column of B): scale
  s = 2^e, e the smallest integer with amax * 2^-e <= 448, e clamped to
  [-126, 126], s = 1 for an all-zero block; q = E4M3(v * 2^-e);
* C = sum over blocks of s_a * s_b * (q_a . q_b), the dot products exact
  (E4M3 products are exact in FP32), only the final FP32 sums round.

It also restates the split-FP16 path's operand preparation
(GBBLAS_ACCURACY_FP16X3): a power-of-two scale per row into FP16's range and
the split into FP16 hi + lo pieces, with the truncation bound its GPU tests
use.

Only tests/ and bench.py's precision report import this module.
"""
from __future__ import annotations

import numpy as np

E4M3_MAX = 448.0
BLOCK = 128


def e4m3_round(x: np.ndarray) -> np.ndarray:
    """Round float64 values to the nearest E4M3 value (ties to even),
    saturating to +-448.  Returns float64."""
    x = np.asarray(x, np.float64)
    a = np.abs(x)
    # quantum: 2^(floor(log2 a) - 3) in the normal range (a >= 2^-6), 2^-9 below
    with np.errstate(divide="ignore"):
        e = np.floor(np.log2(np.where(a > 0, a, 1.0)))
    e = np.maximum(e, -6.0)
    q = np.ldexp(1.0, (e - 3).astype(np.int64))
    r = np.rint(a / q) * q  # np.rint rounds half to even
    r = np.minimum(r, E4M3_MAX)
    return np.copysign(r, x)


def block_exponents(amax: np.ndarray) -> np.ndarray:
    """e per block: smallest integer with amax * 2^-e <= 448 (448 = 0.875 * 2^9)."""
    m, ex = np.frexp(np.asarray(amax, np.float64))
    e = ex - 9 + (m > 0.875).astype(np.int64)
    e = np.clip(e, -126, 126)
    return np.where(np.asarray(amax) > 0, e, 0).astype(np.int64)


def quantise_rows(X: np.ndarray):
    """X: rows x K (float32 values).  Returns (q, s): q rows x Kp (float64
    E4M3 values, zero padding to a multiple of 128), s rows x Kp/128 scales."""
    X = np.asarray(X, np.float32).astype(np.float64)
    rows, K = X.shape
    kb = max(1, -(-K // BLOCK))
    Xp = np.zeros((rows, kb * BLOCK))
    Xp[:, :K] = X
    blocks = Xp.reshape(rows, kb, BLOCK)
    amax = np.abs(blocks).max(axis=2)
    e = block_exponents(amax)
    q = e4m3_round(blocks * np.ldexp(1.0, -e)[:, :, None])
    return q.reshape(rows, kb * BLOCK), np.ldexp(1.0, e)


def gemm_fp8_model(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """The FP8 path's product of A (M x K) and B (K x N) with exact block dot
    products (float64).  The kernel differs from it only by FP32 rounding of
    the block sums and their accumulation."""
    qa, sa = quantise_rows(A)
    qb, sb = quantise_rows(np.asarray(B).T)
    kb = sa.shape[1]
    out = np.zeros((A.shape[0], B.shape[1]))
    for b in range(kb):
        sl = slice(b * BLOCK, (b + 1) * BLOCK)
        out += (qa[:, sl] @ qb[:, sl].T) * sa[:, b:b + 1] * sb[:, b][None, :]
    return out


def gemm_fp8_abs_model(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """sum over blocks of s_a s_b (|q_a| . |q_b|): the magnitude that bounds
    the FP32 rounding of the kernel's sums."""
    qa, sa = quantise_rows(A)
    qb, sb = quantise_rows(np.asarray(B).T)
    kb = sa.shape[1]
    out = np.zeros((A.shape[0], B.shape[1]))
    for b in range(kb):
        sl = slice(b * BLOCK, (b + 1) * BLOCK)
        out += (np.abs(qa[:, sl]) @ np.abs(qb[:, sl]).T) * sa[:, b:b + 1] * sb[:, b][None, :]
    return out


# ---------------------------------------------------------------- split-FP16
F16_SCALE_TOP = 15  # a row scaled by 2^(15 - e) lies below 2^15, inside FP16's range


def f16_split_rows(X: np.ndarray):
    """The split-FP16 path's operand preparation for rows of X (float32,
    rows x K): e = the frexp exponent of each row's largest magnitude (0 for
    an all-zero row), v = x 2^(15 - e) (exact), h = fp16_rn(v),
    l = fp16_rn(v - h).  Returns (h, l, e) with h, l in the scaled units."""
    X = np.asarray(X, np.float32)
    amax = np.abs(X).max(axis=1) if X.shape[1] else np.zeros(X.shape[0], np.float32)
    e = np.frexp(amax.astype(np.float64))[1]
    e[amax == 0] = 0
    v = np.ldexp(X.astype(np.float32), (F16_SCALE_TOP - e)[:, None].astype(np.int32)).astype(np.float32)
    h = v.astype(np.float16).astype(np.float32)
    l = (v - h).astype(np.float16).astype(np.float32)
    return h, l, e


def f16_split_error_bound(X: np.ndarray) -> np.ndarray:
    """|x - (h + l) 2^(e - 15)| <= 2^-22 |x| + 2^-25 2^(e - 15) elementwise:
    22 bits of a normal element, and an l in FP16's subnormal range off by
    half its 2^-24 spacing."""
    _, _, e = f16_split_rows(X)
    return 2.0 ** -22 * np.abs(np.asarray(X, np.float64)) + np.ldexp(2.0 ** -25, (e - F16_SCALE_TOP)[:, None])
