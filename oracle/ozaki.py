"""numpy model of the double-precision GEMM as exact BF16 digit products
(the Ozaki scheme).  TEST INFRASTRUCTURE ONLY.

The reference computes double mtm with FP64 FMAs on the CPU
(include/mtm.hpp:116-206, include/simd_loop.hpp:132-158).  This library's
GPU path for it (GBBLAS_ACCURACY_FP64_DIGITS7 / 8, and the guarded form
behind AUTO) rewrites the product into integer products the BF16 tensor
cores compute exactly.  The published method (Ozaki, Ogita, Oishi, Rump:
error-free splitting of floating-point matrix products) is restated here in
integer arithmetic, step for step as the kernels do it, so a test can
demand bit equality between the GPU and this model:

* row scale e_i: the frexp exponent of max_k |a_ik| (column scale f_j of B
  likewise); 0 for an all-zero row; a row holding Inf or NaN is "bad";
* F = round(a / 2^e * 2^(8S-1)) from the FP64 bit pattern (half away from
  zero), written in balanced base 256: S digits, the last S-1 in
  [-128, 127], the first in [-128, 128];
* G_w = sum_k sum_{s+t=w} D_s(a_ik) E_t(b_kj) for w < S (exact integers);
* r = sum_w G_w 2^(8(S-1-w)) (an exact integer; the kernel holds it as
  hi 2^32 + lo in two 64-bit integers) rounded once to the nearest double
  (ties to even) and scaled by 2^(e_i + f_j - 14 - 8(S-1)),
  C_ij = C_ij + r (NaN where the row or column is bad);
* the guard (7 digits): P = max(|D_0| - 1, 0); L_ij = sum over the first
  32 of K of every 128-K chunk of P(a_ik) P(b_kj); a 32 x 16 output block of
  a 128 x 32 tile keeps the digit result when every output in it has
  L >= 2^14, else it is recomputed with FP64 FMAs.

Only tests/ import this module.
"""
from __future__ import annotations

import numpy as np

CHUNK = 128       # K per TMEM chunk (7 digits)
GUARD_K = 32      # K per chunk that the guard planes cover
GUARD_MIN = 1 << 14
TILE_M, TILE_N = 128, 32
BLOCK_M, BLOCK_N = 32, 16


def row_scales(X: np.ndarray):
    """(e, bad) per row of X (rows x K)."""
    X = np.asarray(X, np.float64)
    bad = ~np.isfinite(X).all(axis=1) if X.shape[1] else np.zeros(X.shape[0], bool)
    amax = np.where(np.isfinite(X), np.abs(X), 0.0).max(axis=1) if X.shape[1] else np.zeros(X.shape[0])
    e = np.frexp(amax)[1].astype(np.int64)
    e[amax == 0] = 0
    return e, bad


def digits(X: np.ndarray, e: np.ndarray, S: int) -> np.ndarray:
    """S x rows x K int64 digits of X (rows x K) with row exponents e."""
    X = np.ascontiguousarray(X, np.float64)
    bits = X.view(np.int64)
    ex = (bits >> 52) & 0x7FF
    m = bits & ((1 << 52) - 1)
    m = np.where(ex != 0, m | (1 << 52), m)
    p2 = np.where(ex != 0, ex - 1075, -1074)
    sh = p2 + 8 * S - 1 - e[:, None]
    up = np.clip(sh, 0, 62)
    dn = np.clip(-sh, 1, 62)
    F = np.where(sh >= 0, m << up, np.where(sh > -63, (m + (np.int64(1) << (dn - 1))) >> dn, 0))
    F = np.where(m == 0, 0, F)
    F = np.where(bits < 0, -F, F)
    D = np.zeros((S,) + X.shape, np.int64)
    for s in range(S - 1, 0, -1):
        lo = ((F & 0xFF) ^ 0x80) - 0x80
        D[s] = lo
        F = (F - lo) >> 8
    D[0] = F
    return D


def groups(DA: np.ndarray, DB: np.ndarray) -> np.ndarray:
    """G_w (S x M x N int64) from A's digits (S x M x K) and B^T's (S x N x K)."""
    S = DA.shape[0]
    G = np.zeros((S, DA.shape[1], DB.shape[1]), np.int64)
    for s in range(S):
        for t in range(S - s):
            G[s + t] += DA[s] @ DB[t].T
    return G


def combine(G: np.ndarray, e: np.ndarray, f: np.ndarray) -> np.ndarray:
    """The kernel's epilogue: the exact integer sum_w G_w 2^(8(S-1-w)) (hi 2^32 + lo)
    rounded once to the nearest double (ties to even; Python's int -> float),
    then scaled by the power of two (exact in the normal range)."""
    S = G.shape[0]
    total = np.zeros(G.shape[1:], object)
    for w in range(S):
        total = total + G[w].astype(object) * (1 << (8 * (S - 1 - w)))
    v = np.vectorize(float, otypes=[np.float64])(total) if total.size else np.zeros(total.shape)
    return np.ldexp(v, (e[:, None] + f[None, :] - 14 - 8 * (S - 1)).astype(np.int32))


def gemm(A: np.ndarray, B: np.ndarray, C0: np.ndarray, S: int = 7) -> np.ndarray:
    """C0 + A @ B as the unguarded digit kernels compute it, bit for bit."""
    A = np.asarray(A, np.float64)
    B = np.asarray(B, np.float64)
    ea, bad_a = row_scales(A)
    eb, bad_b = row_scales(B.T)
    DA = digits(np.where(bad_a[:, None], 0.0, A), np.where(bad_a, 0, ea), S)
    DB = digits(np.where(bad_b[:, None], 0.0, B.T), np.where(bad_b, 0, eb), S)
    r = combine(groups(DA, DB), ea, eb)
    r[bad_a, :] = np.nan
    r[:, bad_b] = np.nan
    return np.asarray(C0, np.float64) + r


def guard_sums(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """L_ij: sum over the guarded K positions of P(a) P(b) (7 digits)."""
    A = np.asarray(A, np.float64)
    B = np.asarray(B, np.float64)
    ea, _ = row_scales(A)
    eb, _ = row_scales(B.T)
    K = A.shape[1]
    ks = np.array([k for k in range(K) if k % CHUNK < GUARD_K], np.int64)
    PA = np.maximum(np.abs(digits(A[:, ks], ea, 7)[0]) - 1, 0)
    PB = np.maximum(np.abs(digits(B.T[:, ks], eb, 7)[0]) - 1, 0)
    return PA @ PB.T


def guard_pass(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """Per output: does its 32 x 16 block keep the digit result?"""
    M, N = A.shape[0], B.shape[1]
    ok = guard_sums(A, B) >= GUARD_MIN
    keep = np.zeros((M, N), bool)
    for r0 in range(0, M, BLOCK_M):
        for c0 in range(0, N, BLOCK_N):
            keep[r0:r0 + BLOCK_M, c0:c0 + BLOCK_N] = ok[r0:r0 + BLOCK_M, c0:c0 + BLOCK_N].all()
    return keep


def error_bound(A: np.ndarray, B: np.ndarray, S: int = 7) -> np.ndarray:
    """(S + 1) 2^-8S K 2^(e_i + f_j): the digit truncation bound per output."""
    ea, _ = row_scales(A)
    eb, _ = row_scales(B.T)
    K = A.shape[1]
    return (S + 1) * 2.0 ** (-8 * S) * K * np.ldexp(1.0, (ea[:, None] + eb[None, :]).astype(np.int32))
