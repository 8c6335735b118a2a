"""Failure detection on the GPU without a fault: a kernel waits on a device
barrier that nothing completes, gives up after its limit and records
GBBLAS_STATUS_TIMEOUT in the stream's error word - the mechanism every
bounded wait of the tensor-core and TMA-fed kernels uses.  The status is
reported once by gbblas_check_stream, the wait ends within its limit, and
the context stays usable (a GEMM right after is correct)."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TIMEOUT = 5  # GBBLAS_STATUS_TIMEOUT


def test_bounded_wait_reports_timeout_once_and_context_survives(cuda):
    import gbblas
    torch = cuda
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    assert gbblas.status_of("gbblas_selftest_bounded_wait", 20000, None) == 0  # 20 ms
    assert gbblas.status_of("gbblas_check_stream", None) == TIMEOUT
    elapsed = time.perf_counter() - t0
    assert 0.015 <= elapsed < 1.5, elapsed
    assert gbblas.status_of("gbblas_check_stream", None) == 0  # reported once, then cleared
    A = torch.rand(300, 200, device="cuda")
    B = torch.rand(200, 100, device="cuda")
    C = torch.zeros(300, 100, device="cuda")
    gbblas.gemm(A, B, C, accuracy=gbblas.ACCURACY_BF16X6)
    assert gbblas.status_of("gbblas_check_stream", None) == 0
    ref = A.double() @ B.double()
    assert bool(((C.double() - ref).abs() <= 1e-5 * ref.abs() + 1e-6).all())


def test_timeout_is_per_stream(cuda):
    """A timeout on one stream is reported on that stream only."""
    import gbblas
    torch = cuda
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    assert gbblas.status_of("gbblas_selftest_bounded_wait", 5000, s1.cuda_stream) == 0
    x = torch.rand(1 << 20, device="cuda")
    out = torch.zeros(1, device="cuda")
    torch.cuda.synchronize()  # inputs ready before the other stream reads them
    with torch.cuda.stream(s2):
        gbblas.dot(x, x, out, stream=s2)
    assert gbblas.status_of("gbblas_check_stream", s2.cuda_stream) == 0
    assert gbblas.status_of("gbblas_check_stream", s1.cuda_stream) == TIMEOUT
    assert gbblas.status_of("gbblas_check_stream", s1.cuda_stream) == 0
    assert abs(out.item() - float((x.double() ** 2).sum())) <= 1e-5 * float((x.double() ** 2).sum())
