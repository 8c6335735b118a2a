"""Grouped GEMM / GEMV and graph-captured batches through the C ABI
(gbblas_sgemm_grouped, gbblas_sgemv_grouped, gbblas_batch_*), checked
problem by problem against the CPU oracle / FP64."""
import os

import numpy as np
import pytest

from oracle import oracle as O

from _tol import assert_vec_close

PKG = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "openmp-blas_gb300")

pytestmark = pytest.mark.gpu

BF16X3, AUTO, BF16X6, FP16X3 = 1, 3, 4, 8


def split_tol(absA, absB, K, mode):
    if mode == BF16X6:
        return (2.0 ** -21 + 2 * K * np.finfo(np.float32).eps) * (absA @ absB)
    if mode == AUTO:  # the guarded FP16 split
        return (2.0 ** -19 + 2 * K * np.finfo(np.float32).eps) * (absA @ absB)
    if mode == FP16X3:  # rows / columns scaled into FP16's range; subnormal low pieces
        sa = np.ldexp(1.0, np.frexp(absA.max(axis=1))[1])
        sb = np.ldexp(1.0, np.frexp(absB.max(axis=0))[1])
        return ((2.0 ** -19 + 2 * K * np.finfo(np.float32).eps) * (absA @ absB) +
                2.0 ** -38 * max(K, 1) * np.outer(sa, sb))
    return (2.0 ** -14 + 2 * K * np.finfo(np.float32).eps) * (absA @ absB)


def make_gemms(torch, rng, shapes):
    """Random problems with assorted layouts; returns (descs, host copies)."""
    import gbblas
    descs, host = [], []
    for i, (M, N, K) in enumerate(shapes):
        A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
        B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
        C0 = rng.uniform(-1, 1, (M, N)).astype(np.float32)
        tA = torch.from_numpy(A).cuda() if i % 2 == 0 else torch.from_numpy(A.T.copy()).cuda().t()
        tB = torch.from_numpy(B).cuda() if i % 3 else torch.from_numpy(B.T.copy()).cuda().t()
        tC = torch.from_numpy(C0.copy()).cuda() if i % 4 else torch.from_numpy(C0.T.copy()).cuda().t()
        descs.append(gbblas.gemm_desc(tA, tB, tC))
        host.append((A, B, C0, tA, tB, tC))
    return descs, host


SHAPES = [(1, 1, 1), (7, 300, 5), (128, 128, 64), (129, 257, 65), (300, 100, 1000), (64, 2048, 96),
          (1000, 33, 517), (512, 512, 512), (40, 800, 1600), (256, 384, 128)]


@pytest.mark.parametrize("mode", [BF16X3, BF16X6, FP16X3, AUTO])
def test_gemm_grouped_vs_fp64(cuda, mode):
    import gbblas
    rng = np.random.default_rng(1)
    descs, host = make_gemms(cuda, rng, SHAPES)
    gbblas.gemm_grouped(descs, accuracy=mode)
    gbblas.call("gbblas_check_stream", None)
    for (A, B, C0, _, _, tC), (M, N, K) in zip(host, SHAPES):
        got = tC.cpu().numpy().astype(np.float64)
        exact = A.astype(np.float64) @ B.astype(np.float64) + C0
        tol = split_tol(np.abs(A).astype(np.float64), np.abs(B).astype(np.float64), K, mode) + 2 * np.finfo(
            np.float32).eps * np.abs(C0)
        assert np.all(np.abs(got - exact) <= tol), (M, N, K)


def test_gemm_grouped_matches_single_calls(cuda):
    """A problem's result does not depend on what else is in the group."""
    import gbblas
    torch = cuda
    rng = np.random.default_rng(2)
    descs, host = make_gemms(torch, rng, SHAPES)
    singles = []
    for (A, B, C0, tA, tB, _), d in zip(host, descs):
        C = torch.from_numpy(C0.copy()).cuda()
        gbblas.gemm(tA, tB, C, accuracy=BF16X6)
        singles.append(C)
    gbblas.gemm_grouped(descs, accuracy=BF16X6)
    torch.cuda.synchronize()
    for (_, _, _, _, _, tC), s in zip(host, singles):
        assert torch.equal(tC.contiguous(), s)


def make_gemvs(torch, rng, specs):
    import gbblas
    descs, host = [], []
    for (layout, tr, M, N, acc) in specs:
        A = rng.uniform(-1, 1, (M, N)).astype(np.float32)
        x = rng.uniform(-1, 1, M if tr else N).astype(np.float32)
        y0 = rng.uniform(-1, 1, N if tr else M).astype(np.float32)
        tA = torch.from_numpy(O.to_layout(A, layout)).cuda()
        tx = torch.from_numpy(x).cuda()
        ty = torch.from_numpy(y0.copy()).cuda()
        descs.append(gbblas.gemv_desc(layout, tr, M, N, tA, tx, ty, acc))
        # keep the device tensors alive: the descriptors hold raw pointers
        host.append((A, x, y0, ty, layout, tr, acc, tA, tx))
    return descs, host


GEMVS = [(1, 0, 300, 257, False), (1, 0, 5, 3, True), (0, 1, 1000, 40, False), (0, 0, 333, 4097, True),
         (1, 1, 64, 2000, True), (1, 0, 4096, 1024, False), (0, 1, 2, 9000, False), (1, 0, 257, 130, True)]


def check_gemvs(host):
    for (A, x, y0, ty, layout, tr, acc, _tA, _tx) in host:
        got = ty.cpu().numpy()
        op = A.T if tr else A
        ref = op.astype(np.float64) @ x.astype(np.float64) + (y0 if acc else 0)
        scale = np.abs(op) @ np.abs(x) + (np.abs(y0) if acc else 0)
        assert_vec_close(got, ref, scale, op.shape[1], np.float32, what=f"gemv {layout}{tr} {A.shape}")


def test_gemv_grouped_all_forms(cuda):
    import gbblas
    rng = np.random.default_rng(3)
    descs, host = make_gemvs(cuda, rng, GEMVS)
    gbblas.gemv_grouped(descs)
    cuda.cuda.synchronize()
    check_gemvs(host)


def test_batch_graph_replay(cuda):
    """A batch replays its CUDA graph: each run adds A*B into C again and
    recomputes y; results equal the immediate grouped calls bit for bit."""
    import gbblas
    torch = cuda
    rng = np.random.default_rng(4)
    gd, gh = make_gemms(torch, rng, SHAPES[:6])
    vd, vh = make_gemvs(torch, rng, [s for s in GEMVS if not s[4]])  # overwrite-only GEMVs
    C_start = [h[5].clone() for h in gh]
    batch = gbblas.Batch(gd, vd, accuracy=BF16X6)
    batch.run()
    batch.sync()
    once = [h[5].clone() for h in gh]
    check_gemvs(vh)
    batch.run()
    batch.sync()
    for (A, B, C0, tA, tB, tC), first, start in zip(gh, once, C_start):
        # second run added the same product again
        delta1 = (first.double() - start.double())
        delta2 = (tC.double() - first.double())
        assert torch.allclose(delta1, delta2, rtol=1e-5, atol=1e-4)
    # same values as the immediate grouped path
    C_imm = [s.clone() for s in C_start]
    imm = [gbblas.gemm_desc(h[3], h[4], c) for h, c in zip(gh, C_imm)]
    gbblas.gemm_grouped(imm, accuracy=BF16X6)
    torch.cuda.synchronize()
    for c, f in zip(C_imm, once):
        assert torch.equal(c, f)
    batch.close()


def test_batch_fp32_accuracy_path(cuda):
    import gbblas
    torch = cuda
    rng = np.random.default_rng(5)
    gd, gh = make_gemms(torch, rng, SHAPES[:4])
    batch = gbblas.Batch(gd, [], accuracy=0)
    batch.run()
    batch.sync()
    for (A, B, C0, _, _, tC), (M, N, K) in zip(gh, SHAPES[:4]):
        ref = O.gemm(A, B, C0, 1, 1, 1)
        got = tC.cpu().numpy()
        scale = np.abs(A) @ np.abs(B) + np.abs(C0)
        assert np.all(np.abs(got - ref) <= 2 * max(K, 1) * np.finfo(np.float32).eps * scale)
    batch.close()


def test_autotune_cache_written(cuda, tmp_path):
    """The autotuner records its GEMV-group choice in the cache file named by
    GBBLAS_TUNE_CACHE (read when the library first tunes in this process, so
    the check runs in a fresh interpreter)."""
    import subprocess
    import sys
    cache = tmp_path / "tune.json"
    code = (
        "import sys, numpy as np, torch; sys.path[:0] = [%r]\n"
        "import gbblas\n"
        "A = torch.rand(3000, 700, device='cuda'); x = torch.rand(700, device='cuda'); y = torch.empty(3000, device='cuda')\n"
        "gbblas.gemv_grouped([gbblas.gemv_desc(1, 0, 3000, 700, A, x, y)])\n"
        "torch.cuda.synchronize()\n"
        "assert torch.allclose(y, A @ x, rtol=1e-4, atol=1e-3)\n" % (PKG,))
    env = dict(os.environ, GBBLAS_TUNE_CACHE=str(cache), GBBLAS_AUTOTUNE="1")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    text = cache.read_text()
    assert "gemv_group_rows|" in text


def test_gemm_grouped_auto_guard_across_problems(cuda):
    """AUTO in a group: out-of-span rows and columns (one entry of 2^20 among
    entries of 2^-20, meeting zeros on the other side) in some problems of the
    group are recomputed with FP32 FMAs - the fixup finds each listed row's
    problem - and every problem meets (2^-19 + 2 K eps32)(|A||B|)."""
    import gbblas
    torch = cuda
    rng = np.random.default_rng(7)
    shapes = [(300, 260, 512), (64, 128, 64), (129, 257, 1000), (500, 40, 300)]
    descs, host = [], []
    for i, (M, N, K) in enumerate(shapes):
        A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
        B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
        if i in (0, 2):  # a few out-of-span rows of A
            for r in (1, M // 2, M - 1):
                A[r] = rng.uniform(-1, 1, K).astype(np.float32) * 2.0 ** -20
                A[r, r % K] = 2.0 ** 20
                B[r % K, :] = 0.0
        if i in (2, 3):  # and columns of B
            for c in (0, N - 1):
                B[:, c] = rng.uniform(-1, 1, K).astype(np.float32) * 2.0 ** -20
                B[(3 * c + 5) % K, c] = 2.0 ** 20
                A[:, (3 * c + 5) % K] = 0.0
        C0 = rng.uniform(-1, 1, (M, N)).astype(np.float32)
        tA, tB, tC = (torch.from_numpy(x.copy()).cuda() for x in (A, B, C0))
        descs.append(gbblas.gemm_desc(tA, tB, tC))
        host.append((A, B, C0, tA, tB, tC))
    gbblas.gemm_grouped(descs, accuracy=AUTO)
    gbblas.call("gbblas_check_stream", None)
    for (A, B, C0, _, _, tC), (M, N, K) in zip(host, shapes):
        got = tC.cpu().numpy().astype(np.float64)
        exact = A.astype(np.float64) @ B.astype(np.float64) + C0
        tol = split_tol(np.abs(A).astype(np.float64), np.abs(B).astype(np.float64), K, AUTO) + \
            2 * np.finfo(np.float32).eps * np.abs(C0)
        assert np.all(np.abs(got - exact) <= tol), (M, N, K, float(np.max(np.abs(got - exact) / tol)))
