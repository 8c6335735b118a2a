"""The serving loop (gbblas_server_*): mixed mtm / mtv / vtm / dot requests in
float and double, continuous batching on several streams.

* every result matches the CPU oracle / FP64 within the tolerances of the
  other parity tests;
* every result is bit-identical run alone and run in a concurrent mix
  (the kernels reduce in an order fixed by each request's own shape);
* admission respects the HBM budget; oversize requests are refused.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

AUTO, FP32, BF16X3, BF16X6 = 3, 0, 1, 4


class ReqCase:
    """One request with its device operands and a fresh-output factory."""

    def __init__(self, torch, rng, kind, dtype, layout, dims, accuracy=AUTO):
        import gbblas
        self.kind, self.dtype, self.layout, self.dims, self.accuracy = kind, dtype, layout, dims, accuracy
        npdt = np.float32 if dtype == gbblas.F32 else np.float64
        tdt = torch.float32 if dtype == gbblas.F32 else torch.float64
        self.torch, self.tdt = torch, tdt
        if kind == gbblas.OP_MTM:
            M, N, K = dims
            self.A = rng.uniform(-1, 1, (M, K)).astype(npdt)
            self.B = rng.uniform(-1, 1, (K, N)).astype(npdt)
            self.tA = torch.from_numpy(O.to_layout(self.A, layout)).cuda()
            self.tB = torch.from_numpy(O.to_layout(self.B, layout)).cuda()
            self.out_len = M * N
        elif kind in (gbblas.OP_MTV, gbblas.OP_VTM):
            M, N = dims
            self.A = rng.uniform(-1, 1, (M, N)).astype(npdt)
            self.x = rng.uniform(-1, 1, M if kind == gbblas.OP_VTM else N).astype(npdt)
            self.tA = torch.from_numpy(O.to_layout(self.A, layout)).cuda()
            self.tB = torch.from_numpy(self.x).cuda()
            self.out_len = N if kind == gbblas.OP_VTM else M
        else:
            (n,) = dims
            self.a = rng.uniform(-1, 1, n).astype(npdt)
            self.b = rng.uniform(-1, 1, n).astype(npdt)
            self.tA = torch.from_numpy(self.a).cuda()
            self.tB = torch.from_numpy(self.b).cuda()
            self.out_len = 1

    def request(self):
        """A gbblas_request with a fresh zeroed output (kept on self.outs)."""
        import gbblas
        out = self.torch.zeros(self.out_len, dtype=self.tdt, device="cuda")
        self.outs = getattr(self, "outs", []) + [out]
        d = self.dims
        M, N, K = (d + (0, 0))[:3] if len(d) < 3 else d
        return gbblas.Request(self.kind, self.dtype, self.accuracy, self.layout, M, N, K, self.tA.data_ptr(),
                              self.tB.data_ptr(), out.data_ptr())

    def check(self, out):
        import gbblas
        got = out.cpu().numpy()
        eps = np.finfo(np.float32 if self.dtype == gbblas.F32 else np.float64).eps
        if self.kind == gbblas.OP_MTM:
            M, N, K = self.dims
            C = O.from_layout(got, M, N, self.layout).astype(np.float64)
            exact = self.A.astype(np.float64) @ self.B.astype(np.float64)
            scale = np.abs(self.A).astype(np.float64) @ np.abs(self.B).astype(np.float64)
            c = 2 * K * eps + (2.0 ** -14 if (self.dtype == gbblas.F32 and self.accuracy == BF16X3) else 0)
            assert np.all(np.abs(C - exact) <= c * scale + 1e-30), ("mtm", self.dims)
        elif self.kind in (gbblas.OP_MTV, gbblas.OP_VTM):
            op = self.A.T if self.kind == gbblas.OP_VTM else self.A
            exact = op.astype(np.float64) @ self.x.astype(np.float64)  # y starts at zero
            scale = np.abs(op).astype(np.float64) @ np.abs(self.x).astype(np.float64)
            assert np.all(np.abs(got - exact) <= 2 * op.shape[1] * eps * scale + 1e-30), ("gemv", self.dims)
        else:
            exact, absdot = O.dot_exact(self.a, self.b)
            assert abs(got[0] - exact) <= 4 * eps * absdot + eps * abs(exact), ("dot", self.dims)


def make_cases(torch, seed=0, n=48):
    import gbblas
    rng = np.random.default_rng(seed)
    cases = []
    for i in range(n):
        dtype = gbblas.F64 if i % 5 == 4 else gbblas.F32
        layout = int(rng.integers(0, 2))
        u = rng.random()
        if u < 0.6:
            dims = tuple(int(v) for v in np.exp(rng.uniform(np.log(64), np.log(512), 3)))
            acc = [AUTO, AUTO, BF16X3, FP32][i % 4]
            cases.append(ReqCase(torch, rng, gbblas.OP_MTM, dtype, layout, dims, acc))
        elif u < 0.9:
            dims = tuple(int(v) for v in np.exp(rng.uniform(np.log(64), np.log(2048), 2)))
            kind = gbblas.OP_VTM if i % 2 else gbblas.OP_MTV
            cases.append(ReqCase(torch, rng, kind, dtype, layout, dims))
        else:
            dims = (int(np.exp(rng.uniform(np.log(1000), np.log(1 << 20)))),)
            cases.append(ReqCase(torch, rng, gbblas.OP_DOT, dtype, 1, dims))
    return cases


def test_server_results_vs_oracle_and_alone_equals_mix(cuda):
    import gbblas
    torch = cuda
    cases = make_cases(torch)
    srv = gbblas.Server(streams=4, max_group=16)
    # alone: one request in the system at a time
    for c in cases:
        srv.wait(srv.submit(c.request()))
    alone = [c.outs[-1] for c in cases]
    # mix: all requests arrive within 0.5 ms of each other
    reqs = [c.request() for c in cases]
    arrivals = np.sort(np.random.default_rng(1).uniform(0, 5e-4, len(reqs)))
    lat = srv.run_trace(reqs, arrivals)
    assert np.all(lat > 0)
    st = srv.stats()
    assert st["completed"] == 2 * len(cases)
    for c, a in zip(cases, alone):
        c.check(a)
        assert torch.equal(a, c.outs[-1]), f"alone != mix for {c.kind} {c.dims}"
    srv.close()


def test_server_budget_admission(cuda):
    import gbblas
    torch = cuda
    rng = np.random.default_rng(2)
    # 24 MiB budget; each 1536 x 1536 f32 GEMV holds ~9.4 MiB
    srv = gbblas.Server(streams=4, max_group=8, budget_bytes=24 << 20)
    cases = [ReqCase(torch, rng, gbblas.OP_MTV, gbblas.F32, 1, (1536, 1536)) for _ in range(12)]
    lat = srv.run_trace([c.request() for c in cases], np.zeros(len(cases)))
    assert np.all(lat > 0)
    st = srv.stats()
    assert st["peak_inflight_bytes"] <= 24 << 20
    assert st["rounds"] >= 6  # at most two fit at once
    for c in cases:
        c.check(c.outs[-1])
    # a request larger than the whole budget is refused at submit
    big = ReqCase(torch, rng, gbblas.OP_MTV, gbblas.F32, 1, (4096, 4096))
    with pytest.raises(gbblas.GbblasError) as e:
        srv.submit(big.request())
    assert e.value.status == 3  # GBBLAS_STATUS_ALLOC_FAILED
    srv.close()


def test_server_pool_alloc(cuda):
    import gbblas
    torch = cuda

    class Dev:  # zero-copy torch view of pool memory
        def __init__(self, ptr, n):
            self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f4", "data": (ptr, False), "version": 3}

    srv = gbblas.Server()
    n = 1 << 20
    pa, pb, pr = srv.alloc(4 * n), srv.alloc(4 * n), srv.alloc(4)
    a = torch.as_tensor(Dev(pa, n), device="cuda")
    b = torch.as_tensor(Dev(pb, n), device="cuda")
    r = torch.as_tensor(Dev(pr, 1), device="cuda")
    a.copy_(torch.arange(n, dtype=torch.float32, device="cuda") % 7)
    b.fill_(2.0)
    torch.cuda.synchronize()
    srv.wait(srv.submit(gbblas.Request(gbblas.OP_DOT, gbblas.F32, 0, 1, n, 0, 0, pa, pb, pr)))
    assert r.item() == float(2 * (torch.arange(n) % 7).sum().item())
    for p in (pa, pb, pr):
        srv.free(p)
    srv.close()


def test_server_f64_gemm_on_tensor_core_digits(cuda):
    """float64 GEMMs large enough for the digit scheme (AUTO: guarded, within
    the FP64 bound; FP64_DIGITS7 explicitly) beside float work: the same
    bits alone and in the mix."""
    import gbblas
    torch = cuda
    rng = np.random.default_rng(7)
    cases = [ReqCase(torch, rng, gbblas.OP_MTM, gbblas.F64, 1, (600, 520, 400), AUTO),
             ReqCase(torch, rng, gbblas.OP_MTM, gbblas.F64, 0, (384, 700, 256), AUTO),
             ReqCase(torch, rng, gbblas.OP_MTM, gbblas.F64, 1, (256, 300, 500), gbblas.ACCURACY_FP64_DIGITS7),
             ReqCase(torch, rng, gbblas.OP_MTM, gbblas.F64, 0, (200, 100, 300), gbblas.ACCURACY_FP64),
             ReqCase(torch, rng, gbblas.OP_MTM, gbblas.F32, 1, (300, 200, 500), AUTO),
             ReqCase(torch, rng, gbblas.OP_MTV, gbblas.F64, 1, (700, 900))]
    srv = gbblas.Server(streams=4, max_group=16)
    for c in cases:
        srv.wait(srv.submit(c.request()))
    alone = [c.outs[-1] for c in cases]
    reqs = [c.request() for c in cases]
    srv.run_trace(reqs, np.zeros(len(reqs)))
    for c, a in zip(cases, alone):
        c.check(a)
        assert torch.equal(a, c.outs[-1]), f"alone != mix for {c.kind} {c.dims}"
    srv.close()


# ---------------------------------------------------------------- failure handling
# Every failure below is made on the host (an injected allocation or launch
# failure, a malformed request, a cancellation, an exhausted budget); nothing
# on the GPU faults.  Each must come back as a status, and the same server
# must then serve correct results.

def _healthy(torch, srv, rng):
    """The server still serves: a small GEMM and a dot, checked."""
    import gbblas
    cases = [ReqCase(torch, rng, gbblas.OP_MTM, gbblas.F32, 1, (96, 80, 64), accuracy=FP32),
             ReqCase(torch, rng, gbblas.OP_DOT, gbblas.F64, 1, (5000,))]
    lat = srv.run_trace([c.request() for c in cases], np.zeros(len(cases)))
    assert np.all(lat > 0)
    for c in cases:
        c.check(c.outs[-1])


def test_server_injected_alloc_failure(cuda):
    import gbblas
    torch = cuda
    srv = gbblas.Server(streams=2)
    srv.inject(gbblas.INJECT_ALLOC, 2)
    for _ in range(2):
        with pytest.raises(gbblas.GbblasError) as e:
            srv.alloc(1 << 20)
        assert e.value.status == 3  # GBBLAS_STATUS_ALLOC_FAILED
    p = srv.alloc(1 << 20)  # the injection is used up
    srv.free(p)
    _healthy(torch, srv, np.random.default_rng(31))
    srv.close()


def test_server_injected_launch_failure(cuda):
    """A round whose launch fails reports CUDA_ERROR for its requests; the
    next rounds run normally."""
    import gbblas
    torch = cuda
    rng = np.random.default_rng(32)
    srv = gbblas.Server(streams=1, max_group=1)
    srv.inject(gbblas.INJECT_LAUNCH, 1)
    bad = ReqCase(torch, rng, gbblas.OP_DOT, gbblas.F32, 1, (1000,))
    t = srv.submit(bad.request())
    assert srv.wait_status(t) == 4  # GBBLAS_STATUS_CUDA_ERROR
    assert bad.outs[-1].item() == 0.0  # nothing ran
    _healthy(torch, srv, rng)
    srv.close()


@pytest.mark.parametrize("field,value", [("op", 9), ("dtype", 2), ("layout", 5), ("accuracy", 42), ("M", -1),
                                         ("A", None)])
def test_server_malformed_request(cuda, field, value):
    import gbblas
    torch = cuda
    rng = np.random.default_rng(33)
    srv = gbblas.Server(streams=2)
    req = ReqCase(torch, rng, gbblas.OP_MTV, gbblas.F32, 1, (64, 64)).request()
    setattr(req, field, value)
    with pytest.raises(gbblas.GbblasError) as e:
        srv.submit(req)
    assert e.value.status == 1  # GBBLAS_STATUS_INVALID_VALUE
    assert srv.stats()["submitted"] == 0
    _healthy(torch, srv, rng)
    srv.close()


def test_server_cancel(cuda):
    """Queued requests can be cancelled: their waits return CANCELLED and
    their outputs stay untouched; a request that already ran cannot be; the
    rest complete correctly.  One stream and one request per round: a
    double GEMM on the FP64 pipes (milliseconds) runs first, so the GEMVs
    behind it are still queued when the test cancels them."""
    import gbblas
    torch = cuda
    rng = np.random.default_rng(34)
    srv = gbblas.Server(streams=1, max_group=1, heavy_us=1 << 40)
    first = ReqCase(torch, rng, gbblas.OP_MTM, gbblas.F64, 1, (1536, 1536, 2048), accuracy=5)  # FP64 pipes, ~8 ms
    cases = [ReqCase(torch, rng, gbblas.OP_MTV, gbblas.F32, 1, (1536, 1536)) for _ in range(40)]
    t_first = srv.submit(first.request())
    tickets = [srv.submit(c.request()) for c in cases]
    # from the back of the queue, which the scheduler reaches last
    cancelled = [t for t in reversed(tickets[10:]) if srv.cancel(t) == 0]
    assert len(cancelled) >= 20
    assert srv.wait_status(t_first) == 0
    for c, t in zip(cases, tickets):
        st = srv.wait_status(t)
        if t in cancelled:
            assert st == 8  # GBBLAS_STATUS_CANCELLED
            assert torch.count_nonzero(c.outs[-1]).item() == 0
        else:
            assert st == 0
            c.check(c.outs[-1])
    assert srv.cancel(tickets[0]) == 6  # finished: GBBLAS_STATUS_NOT_SUPPORTED
    assert srv.cancel(10 ** 9) == 1  # unknown ticket
    _healthy(torch, srv, rng)
    srv.close()


def test_server_budget_exhaustion_recovers(cuda):
    """Far more work than the budget holds at once is admitted piece by piece
    as memory frees up; an oversize request is refused and counted; then the
    server serves normally."""
    import gbblas
    torch = cuda
    rng = np.random.default_rng(35)
    srv = gbblas.Server(streams=4, max_group=4, budget_bytes=20 << 20)
    cases = [ReqCase(torch, rng, gbblas.OP_MTV, gbblas.F32, 1, (1536, 1536)) for _ in range(30)]
    lat = srv.run_trace([c.request() for c in cases], np.zeros(len(cases)))
    assert np.all(lat > 0)
    for c in cases:
        c.check(c.outs[-1])
    big = ReqCase(torch, rng, gbblas.OP_MTV, gbblas.F32, 1, (4096, 4096))
    with pytest.raises(gbblas.GbblasError):
        srv.submit(big.request())
    st = srv.stats()
    assert st["rejected"] == 1 and st["peak_inflight_bytes"] <= 20 << 20
    _healthy(torch, srv, rng)
    srv.close()


@pytest.mark.parametrize("slice_us", [-1, 10])
def test_server_heavy_gemms_sliced_or_capped(cuda, slice_us):
    """Heavy GEMMs (estimated beyond heavy_us) run as slices over tile
    ranges on every SM (slice_us > 0) or as one capped launch (slice_us < 0),
    next to light requests: every result matches FP64 / the oracle, and a
    heavy result is the same bits as the same request run alone."""
    import gbblas
    torch = cuda
    rng = np.random.default_rng(36)
    srv = gbblas.Server(streams=4, heavy_us=20, slice_us=slice_us)
    heavy = [ReqCase(torch, rng, gbblas.OP_MTM, gbblas.F64, 1, (1536, 1024, 1024)),
             ReqCase(torch, rng, gbblas.OP_MTM, gbblas.F32, 1, (2048, 2048, 1024)),
             ReqCase(torch, rng, gbblas.OP_MTM, gbblas.F32, 0, (2048, 1536, 1024), accuracy=BF16X6)]
    light = [ReqCase(torch, rng, gbblas.OP_MTV, gbblas.F32, 1, (700, 900)) for _ in range(20)]
    mix = heavy + light
    lat = srv.run_trace([c.request() for c in mix], np.linspace(0, 2e-3, len(mix)))
    assert np.all(lat > 0)
    for c in mix:
        c.check(c.outs[-1])
    for c in heavy:
        in_mix = c.outs[-1].clone()
        srv.wait(srv.submit(c.request()))
        assert torch.equal(c.outs[-1], in_mix)
    srv.close()


def test_server_request_times(cuda):
    """gbblas_server_request_times splits a finished request's latency into
    queued + host launch + device-and-completion, which add up to the latency
    wait() reports; a request that never ran
    (its launch failed) reports zeros; an unfinished or unknown ticket is an
    error."""
    import gbblas
    torch = cuda
    rng = np.random.default_rng(36)
    srv = gbblas.Server(streams=2, max_group=4)
    cases = [ReqCase(torch, rng, gbblas.OP_MTM, gbblas.F32, 1, (256, 192, 320)),
             ReqCase(torch, rng, gbblas.OP_MTV, gbblas.F32, 1, (700, 900)),
             ReqCase(torch, rng, gbblas.OP_DOT, gbblas.F64, 1, (100000,))]
    for c in cases:
        t = srv.submit(c.request())
        lat = srv.wait(t)
        q, launch, dev, size = srv.request_times(t)
        assert q >= 0 and launch >= 0 and dev >= 0 and size >= 1
        # equal, except that the device part is clamped at zero when the
        # completion stamp came a few microseconds before the enqueue stamp
        assert abs((q + launch + dev) - lat) <= 50e-6 + 1e-3 * lat, (q, launch, dev, lat)
        c.check(c.outs[-1])
    srv.inject(gbblas.INJECT_LAUNCH, 1)
    bad = ReqCase(torch, rng, gbblas.OP_DOT, gbblas.F32, 1, (1000,))
    t = srv.submit(bad.request())
    assert srv.wait_status(t) == 4  # GBBLAS_STATUS_CUDA_ERROR
    assert srv.request_times(t) == (0.0, 0.0, 0.0, 0)
    with pytest.raises(gbblas.GbblasError):
        srv.request_times(10 ** 9)
    srv.close()
