"""dot on the GPU through the C ABI, against the oracle and the golden
vectors of the reference (include/dot.hpp; test/test.dot_prod.cpp)."""
import numpy as np
import pytest

from oracle import oracle as O

import _golden as G
from _tol import C_KAHAN, eps

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def gpu_dot(torch, a, b, offset=0):
    import gbblas
    ta = _dev(torch, np.concatenate([np.zeros(offset, a.dtype), a]))[offset:]
    tb = _dev(torch, np.concatenate([np.zeros(offset, b.dtype), b]))[offset:]
    out = torch.full((1,), float("nan"), dtype=ta.dtype, device="cuda")
    gbblas.dot(ta, tb, out)
    torch.cuda.synchronize()
    return out.item()


@pytest.mark.parametrize("name", G.names("dot_"))
def test_dot_golden(cuda, name):
    c = G.case(name)
    dt = c["r"].dtype
    if "n" in c:
        a = np.arange(1, int(c["n"]) + 1, dtype=dt)
        b = a
    else:
        a, b = c["a"].astype(dt), c["b"].astype(dt)
    got = gpu_dot(cuda, a, b)
    closed = float(c["closed"])
    if int(c["exact"]):
        assert got == closed == float(c["r"])
    else:
        # at least as close to the exact value as the reference's result
        assert abs(got - closed) <= max(abs(float(c["r"]) - closed), eps(dt) * closed)


def test_dot_closed_form_sweep(cuda):
    """test/test.dot_prod.cpp: iota . iota against s(s+1)(2s+1)/6 within
    Catch2's default Approx, over a stride of its size range."""
    for dt in (np.float32, np.float64):
        for s in list(range(2, 130)) + list(range(130, (1 << 17) + 2, 4099)):
            a = np.arange(1, s + 1, dtype=dt)
            exact = s * (s + 1) * (2 * s + 1) // 6
            got = gpu_dot(cuda, a, a)
            assert abs(got - exact) <= 100 * np.finfo(np.float32).eps * exact, (dt, s, got, exact)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("n", [0, 1, 2, 3, 5, 1023, 1024, 4097, 65537, 1 << 20, (1 << 22) + 3])
@pytest.mark.parametrize("offset", [0, 1])
def test_dot_random_vs_oracle(cuda, dt, n, offset):
    rng = np.random.default_rng(n + 17 * offset)
    a = rng.uniform(-1, 1, n).astype(dt)
    b = rng.uniform(-1, 1, n).astype(dt)
    got = gpu_dot(cuda, a, b, offset=offset)
    if n == 0:
        assert got == 0.0
        return
    exact, absdot = O.dot_exact(a, b)
    ref = O.dot(a, b)
    # against the oracle: c * n * eps
    assert abs(got - ref) <= 2 * n * eps(dt) * absdot
    # against the exact sum: Kahan FP32 / FMA FP64 partials combined in FP64
    bound = (C_KAHAN if dt == np.float32 else 2 * np.sqrt(n)) * eps(dt) * absdot + eps(dt) * abs(exact)
    assert abs(got - exact) <= bound, (got, exact, bound)


def test_dot_deterministic_and_large(cuda):
    """2^26 elements: bitwise identical across calls, Kahan-accurate."""
    torch = cuda
    import gbblas
    n = 1 << 26
    g = torch.Generator(device="cuda").manual_seed(1)
    a = torch.rand(n, device="cuda", generator=g, dtype=torch.float32) * 2 - 1
    b = torch.rand(n, device="cuda", generator=g, dtype=torch.float32) * 2 - 1
    outs = []
    for _ in range(3):
        o = torch.zeros(1, device="cuda")
        gbblas.dot(a, b, o)
        outs.append(o.item())
    assert outs[0] == outs[1] == outs[2]
    exact, absdot = O.dot_exact(a.cpu().numpy(), b.cpu().numpy())
    assert abs(outs[0] - exact) <= C_KAHAN * eps(np.float32) * absdot + eps(np.float32) * abs(exact)


def test_dot_host_entry(cuda):
    import gbblas
    rng = np.random.default_rng(5)
    for dt in (np.float32, np.float64):
        a = rng.uniform(-1, 1, 100003).astype(dt)
        b = rng.uniform(-1, 1, 100003).astype(dt)
        exact, absdot = O.dot_exact(a, b)
        got = float(gbblas.dot_host(a, b))
        assert abs(got - exact) <= 4 * eps(dt) * absdot + eps(dt) * abs(exact)
