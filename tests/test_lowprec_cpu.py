"""The low-precision models (oracle/lowprec.py) pinned on the CPU: E4M3
rounding against PyTorch's own float8_e4m3fn cast and hand-checked values,
block scales against their definition, and the split-FP16 preparation
against its truncation bound."""
import numpy as np
import pytest

from oracle import lowprec as L


def test_e4m3_known_values():
    got = L.e4m3_round(np.array([0.1, 448.0, 500.0, 2.0 ** -10, 3 * 2.0 ** -10, -0.3, 0.0, 17.0, 19.0]))
    # 0.1 -> 13 * 2^-7; 2^-10 is half the smallest subnormal (tie -> 0);
    # 17 is a tie between 16 and 18 (even mantissa 16); 19 -> 20
    want = [13 * 2.0 ** -7, 448.0, 448.0, 0.0, 2.0 ** -8, -0.3125, 0.0, 16.0, 20.0]
    np.testing.assert_array_equal(got, want)


def test_e4m3_matches_torch_cast():
    torch = pytest.importorskip("torch")
    if not hasattr(torch, "float8_e4m3fn"):
        pytest.skip("torch without float8_e4m3fn")
    rng = np.random.default_rng(0)
    x = rng.standard_normal(50000) * np.exp2(rng.integers(-14, 9, 50000))
    x = np.clip(x, -448, 448).astype(np.float32)
    t = torch.from_numpy(x).to(torch.float8_e4m3fn).to(torch.float64).numpy()
    np.testing.assert_array_equal(L.e4m3_round(x.astype(np.float64)), t)


def test_block_scale_is_smallest_power_of_two_that_fits():
    rng = np.random.default_rng(1)
    amax = np.concatenate([np.abs(rng.standard_normal(1000)) * np.exp2(rng.integers(-30, 30, 1000)),
                           [448.0, 448.1, 447.9, 1.0, 2.0 ** -140]])
    e = L.block_exponents(amax)
    assert np.all(amax * np.exp2(-e.astype(float)) <= 448.0)
    fits_lower = amax * np.exp2(-(e - 1).astype(float)) <= 448.0
    assert not np.any(fits_lower & (e > -126))
    assert L.block_exponents(np.array([0.0]))[0] == 0


def test_model_exact_on_small_integers():
    """|x| <= 8 integers are E4M3 values after any power-of-two scaling that
    keeps them in range: the model reproduces the exact product."""
    rng = np.random.default_rng(2)
    A = rng.integers(-8, 9, (40, 300)).astype(np.float32)
    B = rng.integers(-8, 9, (300, 24)).astype(np.float32)
    np.testing.assert_array_equal(L.gemm_fp8_model(A, B), A.astype(np.float64) @ B)


@pytest.mark.parametrize("kind", ["uniform", "wide", "tiny"])
def test_f16_split_within_its_bound(kind):
    """The split-FP16 preparation: scaled rows stay inside FP16's range and
    h + l reproduces every element within the bound the GPU tests assume."""
    rng = np.random.default_rng(9)
    shape = (64, 512)
    if kind == "uniform":
        X = rng.uniform(-1, 1, shape)
    elif kind == "wide":
        X = rng.choice([-1.0, 1.0], shape) * rng.uniform(1, 2, shape) * np.ldexp(1.0, rng.integers(-10, 11, shape))
    else:  # magnitudes spread over 2^-40 .. 2^0 within each row
        X = rng.uniform(-1, 1, shape) * np.ldexp(1.0, rng.integers(-40, 1, shape))
    X = X.astype(np.float32)
    X[5] = 0.0
    h, l, e = L.f16_split_rows(X)
    assert np.isfinite(h).all() and np.abs(h).max() <= 2.0 ** 15
    rec = (h.astype(np.float64) + l.astype(np.float64)) * np.ldexp(1.0, (e - L.F16_SCALE_TOP)[:, None])
    assert (np.abs(rec - X.astype(np.float64)) <= L.f16_split_error_bound(X)).all()
    assert (h[5] == 0).all() and (l[5] == 0).all()
