"""Write tests/golden/golden.npz from the reference's own compiled hot path.

Run here, where the reference sources exist:

    make -C oracle ref REF_ROOT=<reference checkout> && python tests/golden/make_golden.py

The outputs come from oracle/_ref/libamt_ref.so, i.e. the reference's
include/{mtm,mtv,dot,outer,trans,el_wise_op}.hpp compiled unmodified.  The inputs follow the
reference tests' rule of integer values in [0, 99] (test/test_utils.hpp:4-8),
drawn here from a seeded numpy generator and stored as uint8, so every
product and every partial sum below 2**24 is exact in float32: for those
cases all correct implementations agree bit for bit.  A few cases use
uniform[-1, 1) values (stored as their float bits) to pin rounding
behaviour within a tolerance instead.

Cases:
  mtm   all 8 (C, A, B) layout mixes x {f32, f64} at sizes below one cache
        block (as test/test.mtm.cpp:30-460) plus K = 1100, which crosses the
        reference's K blocking (include/mtm.hpp:163), with C starting at zero
        and at a non-zero value (C += A*B);
  mtv   both layouts with y starting at 5 (column-major accumulates,
        row-major overwrites; include/mtv.hpp:15-98);
  vtm   column-major square A only - the one form the reference computes
        correctly (include/mtv.hpp:224-227);
  dot   the closed form of test/test.dot_prod.cpp (iota . iota) and random
        integer vectors crossing the three size regimes of include/dot.hpp;
  pack  the 3x3 known answers of test/test.pack.cpp:8-83;
  outer C += a b^T, both layouts, integer and uniform values (one fused
        multiply-add per element, so every value is pinned bit for bit),
        sizes as test/test.outer_prod.cpp;
  transpose  out of place for all four layout pairs, and in place for square
        sizes (test/test.trans.cpp);
  ew    c = a op b for the four std functors of include/el_wise_op.hpp.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "golden.npz")


def main() -> None:
    if not O.ref_available():
        raise SystemExit("oracle/_ref/libamt_ref.so missing: run `make -C oracle ref REF_ROOT=<reference checkout>` where the reference is")
    rng = np.random.default_rng(20240601)
    g: dict[str, np.ndarray] = {}
    names = []

    shared: dict[int, str] = {}

    def put(name, **arrs):
        """Store one case; input arrays reused across cases are stored once
        under "in/<n>" and referenced by "<case>/<key>@" entries."""
        names.append(name)
        for k, v in arrs.items():
            v = np.asarray(v)
            if v.size > 64 and k not in ("C", "y", "r", "out", "c"):
                key = shared.get(id(v))
                if key is None:
                    key = f"in/{len(shared)}"
                    shared[id(v)] = key
                    g[key] = v
                g[f"{name}/{k}@"] = np.array(key)
            else:
                g[f"{name}/{k}"] = v

    # ---------------- mtm ----------------
    shapes = [(2, 2, 2), (3, 5, 4), (17, 31, 29), (31, 16, 7), (24, 20, 1100)]
    for dt in (np.float32, np.float64):
        for (M, N, K) in shapes:
            A8 = rng.integers(0, 100, (M, K), dtype=np.uint8)
            B8 = rng.integers(0, 100, (K, N), dtype=np.uint8)
            C8 = rng.integers(0, 100, (M, N), dtype=np.uint8)
            C8z = (np.zeros((M, N), dt), C8.astype(dt))
            for lc in (0, 1):
                for la in (0, 1):
                    for lb in (0, 1):
                        for cinit in (0, 1):
                            if K == 1100 and (lc, la, lb) not in ((0, 0, 0), (1, 1, 1), (1, 0, 1)):
                                continue
                            C0 = C8z[cinit]
                            C = O.ref_gemm(A8.astype(dt), B8.astype(dt), C0, la, lb, lc)
                            put(f"mtm_{np.dtype(dt).name}_{M}x{N}x{K}_c{lc}a{la}b{lb}_i{cinit}",
                                A=A8, B=B8, C0=C0, C=C, lc=lc, la=la, lb=lb, exact=1)
        # uniform values, K crossing the block: rounding pinned within tolerance
        M, N, K = 6, 8, 600
        A = rng.uniform(-1, 1, (M, K)).astype(dt)
        B = rng.uniform(-1, 1, (K, N)).astype(dt)
        for (lc, la, lb) in ((0, 0, 0), (1, 1, 1)):
            C = O.ref_gemm(A, B, np.zeros((M, N), dt), la, lb, lc)
            put(f"mtm_{np.dtype(dt).name}_{M}x{N}x{K}_c{lc}a{la}b{lb}_uniform",
                A=A, B=B, C0=np.zeros((M, N), dt), C=C, lc=lc, la=la, lb=lb, exact=0)

    # ---------------- mtv / vtm ----------------
    for dt in (np.float32, np.float64):
        for (M, N) in [(2, 2), (37, 300), (300, 37), (257, 257)]:
            A8 = rng.integers(0, 100, (M, N), dtype=np.uint8)
            x8 = rng.integers(0, 100, N, dtype=np.uint8)
            y0 = np.full(M, 5, dt)
            for la in (0, 1):
                y = O.ref_mtv(A8.astype(dt), x8.astype(dt), y0, la)
                put(f"mtv_{np.dtype(dt).name}_{M}x{N}_a{la}", A=A8, x=x8, y0=y0, y=y, la=la, exact=1)
        for M in (2, 64, 300):
            A8 = rng.integers(0, 100, (M, M), dtype=np.uint8)
            v8 = rng.integers(0, 100, M, dtype=np.uint8)
            y0 = np.full(M, 5, dt)
            y = O.ref_vtm(A8.astype(dt), v8.astype(dt), y0, 0)
            put(f"vtm_{np.dtype(dt).name}_{M}x{M}_a0", A=A8, v=v8, y0=y0, y=y, la=0, exact=1)
        # uniform-valued mtv (row-major) for rounding behaviour
        A = rng.uniform(-1, 1, (16, 600)).astype(dt)
        x = rng.uniform(-1, 1, 600).astype(dt)
        y = O.ref_mtv(A, x, np.zeros(16, dt), 1)
        put(f"mtv_{np.dtype(dt).name}_16x600_a1_uniform", A=A, x=x, y0=np.zeros(16, dt), y=y, la=1, exact=0)

    # ---------------- dot ----------------
    dot_in = {n: (rng.integers(0, 100, n, dtype=np.uint8), rng.integers(0, 100, n, dtype=np.uint8))
              for n in (2, 17, 24577, 50003)}
    for dt in (np.float32, np.float64):
        for s in (2, 3, 100, 1000, 4097):
            a = np.arange(1, s + 1, dtype=dt)
            r = O.ref_dot(a, a)
            closed = s * (s + 1) * (2 * s + 1) // 6
            put(f"dot_{np.dtype(dt).name}_iota{s}", n=s, r=np.array(r, dt),
                closed=np.array(closed, np.float64), exact=int(closed < 2 ** 24 or dt == np.float64))
        for n, (a8, b8) in dot_in.items():
            r = O.ref_dot(a8.astype(dt), b8.astype(dt))
            exact_sum = int(np.dot(a8.astype(np.int64), b8.astype(np.int64)))
            put(f"dot_{np.dtype(dt).name}_int{n}", a=a8, b=b8, r=np.array(r, dt),
                closed=np.array(exact_sum, np.float64), exact=int(exact_sum < 2 ** 24 or dt == np.float64))

    # ---------------- pack (3x3 known answers) ----------------
    inp = np.arange(1, 10, dtype=np.float32)  # first_order 3x3: strides {1, 3}
    w = (1, 3)
    out = np.arange(1, 10, dtype=np.float32)
    for i in range(0, 3, 2):
        ib = min(2, 3 - i)
        O.ref_pack(inp, w, ib, ib, 3, out, offset_in=i * w[0], offset_out=i * 3)
    put("pack_plain_3x3", inp=inp, out=out)
    out = np.arange(1, 10, dtype=np.float32)
    for i in range(0, 3, 2):
        ib = min(2, 3 - i)
        O.ref_pack(inp, w, ib, ib, 3, out, offset_in=i * w[1], offset_out=i * 3, trans=True)
    put("pack_trans_3x3", inp=inp, out=out)

    # ---------------- outer / transpose / element-wise ----------------
    for dt in (np.float32, np.float64):
        tn = np.dtype(dt).name
        for (M, N) in [(2, 2), (7, 5), (31, 32), (33, 17)]:
            a8 = rng.integers(0, 100, M, dtype=np.uint8)
            b8 = rng.integers(0, 100, N, dtype=np.uint8)
            C8 = rng.integers(0, 100, (M, N), dtype=np.uint8).astype(dt)
            au = rng.uniform(-1, 1, M).astype(dt)
            bu = rng.uniform(-1, 1, N).astype(dt)
            Cu = rng.uniform(-1, 1, (M, N)).astype(dt)
            for lc in (0, 1):
                put(f"outer_{tn}_{M}x{N}_c{lc}_int", a=a8, b=b8, C0=C8,
                    C=O.ref_outer(a8.astype(dt), b8.astype(dt), C8, lc), lc=lc)
                # one fused multiply-add per element: bit-exact for any values
                put(f"outer_{tn}_{M}x{N}_c{lc}_uniform", a=au, b=bu, C0=Cu, C=O.ref_outer(au, bu, Cu, lc), lc=lc)
        for (M, N) in [(2, 2), (5, 7), (32, 31), (40, 3)]:
            A = rng.uniform(-1, 1, (M, N)).astype(dt)
            for la in (0, 1):
                for lc in (0, 1):
                    put(f"transpose_{tn}_{M}x{N}_a{la}c{lc}", A=A, C=O.ref_transpose(A, la, lc), la=la, lc=lc)
        for n in (2, 3, 31, 32, 33):
            buf = rng.uniform(-1, 1, n * n).astype(dt)
            put(f"transpose_inplace_{tn}_{n}", inp=buf, out=O.ref_transpose_inplace(buf), n=n)
        for n in (1, 7, 1000):
            a = rng.uniform(-1, 1, n).astype(dt)
            b = (rng.uniform(0.5, 2, n) * rng.choice([-1, 1], n)).astype(dt)
            for op in range(4):
                put(f"ew_{tn}_{n}_op{op}", a=a, b=b, c=O.ref_ew(op, a, b), op=op)

    g["_names"] = np.array(names)
    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT}: {len(names)} cases, {os.path.getsize(OUT) / 1024:.1f} KiB")


if __name__ == "__main__":
    main()
