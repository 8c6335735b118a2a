"""Split-K on the tensor cores and the tuned launch shapes, through the C ABI.

A single tensor-core GEMM whose K is long against M and N may be cut into
parts along K (GBBLAS_TC_SPLITK=n forces n; otherwise the autotuner picks
1, 2, 4, 8 or 16 per shape bucket): each part is a tile problem of its own
that stores a partial, and the parts are then added into C in part order.

* every forced part count (uneven ones too), all three tensor-core modes,
  against FP64 with the same bounds as unsplit (split-BF16) or the FP8 model,
  C of either layout and accumulated onto;
* integers stay exact whatever the split;
* the result is the same bits on every run (fixed order of the parts);
* the autotuner writes its split-K / CTA-form and FMA-tile choices to its
  cache and the tuned call agrees with the bounds.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import oracle as O
from oracle import lowprec as L

from test_gemm_tc_gpu import BF16X3, BF16X6, run, split_tol

pytestmark = pytest.mark.gpu

FP8 = 2
EPS32 = float(np.finfo(np.float32).eps)
PKG = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "openmp-blas_gb300")

SHAPES = [(256, 256, 8192), (200, 130, 5000), (1, 1, 4096), (129, 257, 3000), (64, 600, 2600)]


def fp8_tol(A, B, extra_adds):
    nb = -(-A.shape[1] // 128)
    return (2.0 ** -16 + 2 * (nb + 1 + extra_adds) * EPS32) * L.gemm_fp8_abs_model(A, B) + 1e-30


@pytest.mark.parametrize("parts", [2, 3, 4, 8, 16])
@pytest.mark.parametrize("mode", [BF16X3, BF16X6, FP8])
@pytest.mark.parametrize("shape", SHAPES)
def test_forced_split_within_bounds(cuda, monkeypatch, parts, mode, shape):
    monkeypatch.setenv("GBBLAS_TC_SPLITK", str(parts))
    M, N, K = shape
    rng = np.random.default_rng(M + 5 * N + 3 * K + parts + 11 * mode)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    C0 = rng.uniform(-1, 1, (M, N)).astype(np.float32)
    lc = parts % 2  # column-major C for odd part counts
    got = run(cuda, A, B, C0, 1, 1, lc, accuracy=mode).astype(np.float64)
    if mode == FP8:
        model = L.gemm_fp8_model(A, B) + C0
        tol = fp8_tol(A, B, parts) + 2 * EPS32 * np.abs(C0)
        assert np.all(np.abs(got - model) <= tol), f"max err/tol {np.max(np.abs(got - model) / tol):.3g}"
    else:
        exact = A.astype(np.float64) @ B.astype(np.float64) + C0
        tol = split_tol(np.abs(A).astype(np.float64), np.abs(B).astype(np.float64), K + parts, mode) + \
            2 * EPS32 * np.abs(C0)
        assert np.all(np.abs(got - exact) <= tol)


@pytest.mark.parametrize("parts", [1, 2, 5, 16])
@pytest.mark.parametrize("mode", [BF16X3, BF16X6, FP8])
def test_split_integers_exact(cuda, monkeypatch, parts, mode):
    monkeypatch.setenv("GBBLAS_TC_SPLITK", str(parts))
    rng = np.random.default_rng(parts + mode)
    M, N, K = 150, 140, 4500
    A = rng.integers(-8, 9, (M, K)).astype(np.float32)
    B = rng.integers(-8, 9, (K, N)).astype(np.float32)
    C0 = rng.integers(-50, 51, (M, N)).astype(np.float32)
    got = run(cuda, A, B, C0, 1, 0, 1, accuracy=mode)
    np.testing.assert_array_equal(got, A.astype(np.float64) @ B + C0)


@pytest.mark.parametrize("mode", [BF16X3, FP8])
def test_split_same_bits_every_run(cuda, monkeypatch, mode):
    monkeypatch.setenv("GBBLAS_TC_SPLITK", "8")
    rng = np.random.default_rng(7)
    A = rng.uniform(-1, 1, (300, 8192)).astype(np.float32)
    B = rng.uniform(-1, 1, (8192, 200)).astype(np.float32)
    Z = np.zeros((300, 200), np.float32)
    first = run(cuda, A, B, Z, 1, 1, 1, accuracy=mode)
    for _ in range(3):
        np.testing.assert_array_equal(run(cuda, A, B, Z, 1, 1, 1, accuracy=mode), first)


def test_tuned_choices_cached_and_within_bounds(cuda, tmp_path):
    """A fresh process with its own cache: an eligible tensor-core shape and a
    large FP32 GEMM are tuned, the choices land in the cache file, and the
    tuned results keep their bounds."""
    cache = tmp_path / "tune.json"
    code = (
        "import sys, numpy as np, torch; sys.path[:0] = [%r]\n"
        "import gbblas\n"
        "g = torch.Generator(device='cuda').manual_seed(1)\n"
        "A = torch.rand(256, 16384, device='cuda', generator=g) * 2 - 1\n"
        "B = torch.rand(16384, 256, device='cuda', generator=g) * 2 - 1\n"
        "C = torch.zeros(256, 256, device='cuda')\n"
        "gbblas.gemm(A, B, C, accuracy=gbblas.ACCURACY_BF16X6)\n"
        "ref = A.double() @ B.double()\n"
        "bound = (2.0 ** -21 + 2 * 16384 * 2.0 ** -23) * (A.double().abs() @ B.double().abs())\n"
        "assert bool(((C.double() - ref).abs() <= bound).all())\n"
        "A2 = torch.rand(2048, 2048, device='cuda', generator=g); B2 = torch.rand(2048, 2048, device='cuda', generator=g)\n"
        "C2 = torch.zeros(2048, 2048, device='cuda')\n"
        "gbblas.gemm(A2, B2, C2, accuracy=gbblas.ACCURACY_FP32)\n"
        "ref2 = A2.double() @ B2.double()\n"
        "assert bool(((C2.double() - ref2).abs() <= 2 * 2048 * 2.0 ** -23 * ref2.abs()).all())\n"
        "torch.cuda.synchronize()\n" % (PKG,))
    env = dict(os.environ, GBBLAS_TUNE_CACHE=str(cache), GBBLAS_AUTOTUNE="1")
    env.pop("GBBLAS_TC_SPLITK", None)
    env.pop("GBBLAS_TC_PAIR", None)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    text = cache.read_text()
    assert "gemm_tc|" in text and "|mode3|" in text
    assert "gemm_fma_tile|" in text
