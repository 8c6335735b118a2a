"""GEMV shapes whose reduction is split across CTAs.

With 2 splits, or up to 8 on a matrix of at most 64 MB, the CTAs of one row
block run as a thread-block cluster and the cluster's rank 0 adds the
splits' partials through distributed shared memory; otherwise the partials
go through scratch and a second kernel.  Both add the splits in order.  The
shapes below take both routes (2 to 8 splits in clusters; 3 to 8 on large
matrices and 10 or more through scratch) on the row-streaming kernel
(row-major mtv) and the column-streaming one (column-major mtv), for both
element types, against the oracle and run to run bit for bit.
"""
import numpy as np
import pytest

from oracle import oracle as O

from _tol import assert_vec_close
from test_gemv_gpu import run

pytestmark = pytest.mark.gpu

ROW_MAJOR_SHAPES = [(700, 6000), (300, 10000), (152, 20000), (2500, 6000), (129, 4097), (100, 20000)]
COL_MAJOR_SHAPES = [(50000, 300), (200000, 1000), (400000, 200), (4097, 129), (20000, 5000)]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("layout,shape", [(1, s) for s in ROW_MAJOR_SHAPES] + [(0, s) for s in COL_MAJOR_SHAPES])
def test_split_gemv_vs_oracle_and_repeatable(cuda, dt, layout, shape):
    M, N = shape
    rng = np.random.default_rng(M + 7 * N + layout)
    A = rng.uniform(-1, 1, (M, N)).astype(dt)
    x = rng.uniform(-1, 1, N).astype(dt)
    y0 = rng.uniform(-1, 1, M).astype(dt)
    got = run(cuda, "mtv", A, x, y0, layout)
    ref = O.mtv(A, x, y0, layout)
    scale = np.abs(A) @ np.abs(x) + (np.abs(y0) if layout == 0 else 0)
    assert_vec_close(got, ref, scale, N, dt, what=f"mtv {shape} layout {layout}")
    np.testing.assert_array_equal(run(cuda, "mtv", A, x, y0, layout), got)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("shape", [(6000, 700), (20000, 152), (300, 50000)])
def test_split_vtm_vs_oracle(cuda, dt, shape):
    """vtm runs the same two kernels on A^T: a column-major A streams rows."""
    M, N = shape
    rng = np.random.default_rng(M + N)
    A = rng.uniform(-1, 1, (M, N)).astype(dt)
    v = rng.uniform(-1, 1, M).astype(dt)
    for layout in (0, 1):
        y0 = rng.uniform(-1, 1, N).astype(dt)
        got = run(cuda, "vtm", A, v, y0, layout)
        ref = O.vtm(A, v, y0, layout)
        scale = np.abs(v) @ np.abs(A) + (np.abs(y0) if layout == 1 else 0)
        assert_vec_close(got, ref, scale, M, dt, what=f"vtm {shape} layout {layout}")
