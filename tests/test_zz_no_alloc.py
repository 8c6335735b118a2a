"""gbblas_sdot_noalloc: the dot for callers that cannot allocate device memory
when they call (a caller-owned pool that must not grow, a serving loop that
reserved everything up front, a binding without cudaMalloc).  Its reduction
scratch is a fixed array inside the library, so this checks, through the
C ABI, that two calls in a row give what gbblas_sdot gives, within the dot
tolerance used elsewhere (4 eps sum|a_i b_i| plus half an ulp).

The file name sorts last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sdot(gbblas, fn, a, b, out):
    gbblas.call(fn, a.numel(), a.data_ptr(), b.data_ptr(), out.data_ptr(), None)


@pytest.mark.parametrize("n", [1, 1000, 65537, 1 << 22, 3 * (1 << 24) + 5])
def test_sdot_noalloc_matches_sdot_twice(cuda, n):
    torch = cuda
    import gbblas
    g = torch.Generator(device="cuda").manual_seed(n)
    a = torch.rand(n, device="cuda", generator=g) * 2 - 1
    b = torch.rand(n, device="cuda", generator=g) * 2 - 1
    ref = torch.zeros(1, device="cuda")
    _sdot(gbblas, "gbblas_sdot", a, b, ref)
    eps = float(np.finfo(np.float32).eps)
    tol = 4 * eps * float((a.double() * b.double()).abs().sum()) + eps * abs(ref.item())
    # the exact sum (long double) from the CPU oracle, with the Kahan dot's bound
    from oracle import oracle as O
    exact, absdot = O.dot_exact(a.cpu().numpy(), b.cpu().numpy())
    tol_exact = 4 * eps * absdot + 0.5 * eps * abs(exact)
    for _ in range(2):
        out = torch.full((1,), float("nan"), device="cuda")
        _sdot(gbblas, "gbblas_sdot_noalloc", a, b, out)
        torch.cuda.synchronize()
        assert abs(out.item() - ref.item()) <= tol, (n, out.item(), ref.item())
        assert abs(out.item() - exact) <= tol_exact, (n, out.item(), exact)


def test_sdot_noalloc_device_memory_unchanged(cuda):
    """After the first call on the device (set-up), further calls take no
    device memory: the free device memory the driver reports does not move
    over many calls of several sizes."""
    torch = cuda
    import gbblas
    g = torch.Generator(device="cuda").manual_seed(11)
    a = torch.rand(1 << 23, device="cuda", generator=g) - 0.5
    b = torch.rand(1 << 23, device="cuda", generator=g) - 0.5
    out = torch.zeros(1, device="cuda")
    _sdot(gbblas, "gbblas_sdot_noalloc", a, b, out)  # set-up call
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for k in range(60):
        n = [7, 4099, 1 << 20, 1 << 23][k % 4]
        gbblas.call("gbblas_sdot_noalloc", n, a.data_ptr(), b.data_ptr(), out.data_ptr(), None)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_sdot_noalloc_alternating_sizes(cuda):
    """The shared scratch keeps the previous call's contents: a large call
    followed by a small one (and back) must not see stale partials."""
    torch = cuda
    import gbblas
    g = torch.Generator(device="cuda").manual_seed(3)
    big_a = torch.rand(1 << 24, device="cuda", generator=g) - 0.5
    big_b = torch.rand(1 << 24, device="cuda", generator=g) - 0.5
    small_a = big_a[: 100000].clone()
    small_b = big_b[: 100000].clone()
    eps = float(np.finfo(np.float32).eps)
    for a, b in ((big_a, big_b), (small_a, small_b), (big_a, big_b), (small_a, small_b)):
        ref = torch.zeros(1, device="cuda")
        out = torch.zeros(1, device="cuda")
        _sdot(gbblas, "gbblas_sdot", a, b, ref)
        _sdot(gbblas, "gbblas_sdot_noalloc", a, b, out)
        torch.cuda.synchronize()
        tol = 4 * eps * float((a.double() * b.double()).abs().sum()) + eps * abs(ref.item())
        assert abs(out.item() - ref.item()) <= tol


def test_sdot_noalloc_rejects_bad_arguments(cuda):
    import gbblas
    assert gbblas.status_of("gbblas_sdot_noalloc", -1, None, None, None, None) == 1
    assert gbblas.status_of("gbblas_sdot_noalloc", 10, None, None, None, None) == 1
