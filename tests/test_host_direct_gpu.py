"""The streaming host-buffer entry points (gbblas_?dot_host, gbblas_?mtv_host,
gbblas_?vtm_host) read large operands straight from host memory where the
device can (page-locked memory through its mapped address; pageable memory
on a device that reads it coherently), and stage them otherwise.  Either
way they must give the device entry points' bits: same kernel, same grid,
same reduction order.  Checked on pinned, pageable and misaligned (staged)
buffers, with direct reads on and off (GBBLAS_HOST_DIRECT=0)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_dot(torch, a, b):
    import gbblas
    out = torch.zeros(1, dtype=torch.from_numpy(a[:1]).dtype, device="cuda")
    gbblas.dot(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), out)
    return out.cpu().numpy()[0]


@pytest.fixture(params=["direct", "staged"])
def host_mode(request, monkeypatch):
    if request.param == "staged":
        monkeypatch.setenv("GBBLAS_HOST_DIRECT", "0")
    else:
        monkeypatch.delenv("GBBLAS_HOST_DIRECT", raising=False)
    return request.param


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("kind", ["pageable", "pinned", "misaligned"])
def test_dot_host_matches_device(cuda, host_mode, dt, kind):
    torch = cuda
    import gbblas
    n = (1 << 22) + 13
    rng = np.random.default_rng(5)
    a = rng.uniform(-1, 1, n + 1).astype(dt)
    b = rng.uniform(-1, 1, n + 1).astype(dt)
    if kind == "pinned":
        ta = torch.from_numpy(a[:n]).pin_memory()
        tb = torch.from_numpy(b[:n]).pin_memory()
        ha, hb = ta.numpy(), tb.numpy()
    elif kind == "misaligned":
        ha, hb = a[1:], b[1:]
    else:
        ha, hb = a[:n], b[:n]
    want = _device_dot(torch, np.ascontiguousarray(ha), np.ascontiguousarray(hb))
    for _ in range(2):  # a misaligned host buffer is staged into aligned device memory: the same kernel again
        got = gbblas.dot_host(ha, hb)
        assert got == want, (kind, host_mode, got, want)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("layout", [0, 1])
@pytest.mark.parametrize("op", ["mtv", "vtm"])
@pytest.mark.parametrize("pinned", [False, True])
def test_gemv_host_matches_device(cuda, host_mode, dt, layout, op, pinned):
    torch = cuda
    import gbblas
    M, N = 3000, 2053
    rng = np.random.default_rng(M + layout)
    A = rng.uniform(-1, 1, M * N).astype(dt)
    if pinned:
        A = torch.from_numpy(A).pin_memory().numpy()
    vin = rng.uniform(-1, 1, N if op == "mtv" else M).astype(dt)
    y0 = rng.uniform(-1, 1, M if op == "mtv" else N).astype(dt)
    ty = torch.from_numpy(y0.copy()).cuda()
    getattr(gbblas, op)(layout, M, N, torch.from_numpy(A).cuda(), torch.from_numpy(vin).cuda(), ty)
    want = ty.cpu().numpy()
    for _ in range(2):
        y = y0.copy()
        getattr(gbblas, f"{op}_host")(layout, M, N, A, vin, y)
        np.testing.assert_array_equal(y, want)
