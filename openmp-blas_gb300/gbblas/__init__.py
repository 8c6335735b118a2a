"""Python binding of libgbblas.so (the C ABI in include/gbblas.h).

This is a thin ctypes layer used by the tests, the benchmark and anyone who
wants the GB300 kernels from Python.  Device operands are torch CUDA tensors
(torch only supplies memory and streams); host operands are numpy arrays and
go through the library's *_host entry points.  There is no CPU fallback: if
the library or a GB300 is missing, calls raise.

Layouts: FIRST_ORDER (0) = column-major, LAST_ORDER (1) = row-major.
"""
from __future__ import annotations

import ctypes
import os

from . import _build

FIRST_ORDER = 0
LAST_ORDER = 1

ACCURACY_FP32 = 0
ACCURACY_BF16X3 = 1
ACCURACY_FP8 = 2
ACCURACY_AUTO = 3
ACCURACY_BF16X6 = 4
ACCURACY_FP64 = 5          # double GEMM on the FP64 pipes
ACCURACY_FP64_DIGITS7 = 6  # double GEMM, Ozaki scheme on the BF16 tensor cores, 7 digits
ACCURACY_FP64_DIGITS8 = 7  # the same with 8 digits
ACCURACY_FP16X3 = 8        # float GEMM: scaled FP16 hi + lo, three tcgen05 products

STATUS = {
    0: "SUCCESS", 1: "INVALID_VALUE", 2: "SHAPE_MISMATCH", 3: "ALLOC_FAILED",
    4: "CUDA_ERROR", 5: "TIMEOUT", 6: "NOT_SUPPORTED", 7: "NO_DEVICE", 8: "CANCELLED",
}

LIB_PATH = _build.LIB

#: every C-ABI symbol include/gbblas.h declares, with (restype, argtypes)
_i64 = ctypes.c_int64
_int = ctypes.c_int
_vp = ctypes.c_void_p
SIGNATURES = {
    "gbblas_status_string": (ctypes.c_char_p, [_int]),
    "gbblas_last_error": (ctypes.c_char_p, []),
    "gbblas_version": (ctypes.c_char_p, []),
    "gbblas_init": (_int, []),
    "gbblas_kernel_launches": (ctypes.c_uint64, []),
    "gbblas_check_stream": (_int, [_vp]),
    "gbblas_selftest_bounded_wait": (_int, [ctypes.c_int64, _vp]),
    "gbblas_release_cache": (_int, []),
    "gbblas_sgemm": (_int, [_i64, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _int, _vp]),
    "gbblas_dgemm": (_int, [_i64, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _vp]),
    "gbblas_dgemm_ex": (_int, [_i64, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _int, _vp]),
    "gbblas_smtv": (_int, [_int, _i64, _i64, _vp, _vp, _vp, _vp]),
    "gbblas_dmtv": (_int, [_int, _i64, _i64, _vp, _vp, _vp, _vp]),
    "gbblas_svtm": (_int, [_int, _i64, _i64, _vp, _vp, _vp, _vp]),
    "gbblas_dvtm": (_int, [_int, _i64, _i64, _vp, _vp, _vp, _vp]),
    "gbblas_sgemv": (_int, [_int, _int, _i64, _i64, _vp, _vp, _int, _vp, _vp]),
    "gbblas_dgemv": (_int, [_int, _int, _i64, _i64, _vp, _vp, _int, _vp, _vp]),
    "gbblas_sdot": (_int, [_i64, _vp, _vp, _vp, _vp]),
    "gbblas_ddot": (_int, [_i64, _vp, _vp, _vp, _vp]),
    "gbblas_sdot_noalloc": (_int, [_i64, _vp, _vp, _vp, _vp]),
    "gbblas_sdot_tuning": (_int, [_i64, _vp, _vp, _i64, _i64, _i64, _vp, _vp]),
    "gbblas_ddot_tuning": (_int, [_i64, _vp, _vp, _i64, _i64, _i64, _vp, _vp]),
    "gbblas_sgemm_grouped": (_int, [_vp, _i64, _int, _vp]),
    "gbblas_sgemv_grouped": (_int, [_vp, _i64, _vp]),
    "gbblas_batch_create": (_int, [_vp, _i64, _int, _vp, _i64, _vp]),
    "gbblas_batch_run": (_int, [_vp, _vp]),
    "gbblas_batch_sync": (_int, [_vp]),
    "gbblas_batch_destroy": (_int, [_vp]),
    "gbblas_server_create": (_int, [_vp, _vp]),
    "gbblas_server_alloc": (_int, [_vp, _i64, _vp]),
    "gbblas_server_free": (_int, [_vp, _vp]),
    "gbblas_server_submit": (_int, [_vp, _vp, _vp]),
    "gbblas_server_wait": (_int, [_vp, ctypes.c_uint64, _vp]),
    "gbblas_server_run_trace": (_int, [_vp, _vp, _vp, _i64, _vp]),
    "gbblas_server_get_stats": (_int, [_vp, _vp]),
    "gbblas_server_request_times": (_int, [_vp, ctypes.c_uint64, _vp]),
    "gbblas_server_destroy": (_int, [_vp]),
    "gbblas_server_cancel": (_int, [_vp, ctypes.c_uint64]),
    "gbblas_server_inject": (_int, [_vp, ctypes.c_int32, ctypes.c_int32]),
    "gbblas_sgemm_host": (_int, [_i64, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _int]),
    "gbblas_dgemm_host": (_int, [_i64, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64]),
    "gbblas_dgemm_ex_host": (_int, [_i64, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _int]),
    "gbblas_smtv_host": (_int, [_int, _i64, _i64, _vp, _vp, _vp]),
    "gbblas_dmtv_host": (_int, [_int, _i64, _i64, _vp, _vp, _vp]),
    "gbblas_svtm_host": (_int, [_int, _i64, _i64, _vp, _vp, _vp]),
    "gbblas_dvtm_host": (_int, [_int, _i64, _i64, _vp, _vp, _vp]),
    "gbblas_sdot_host": (_int, [_i64, _vp, _vp, _vp]),
    "gbblas_ddot_host": (_int, [_i64, _vp, _vp, _vp]),
    "gbblas_souter": (_int, [_int, _i64, _i64, _vp, _vp, _vp, _vp]),
    "gbblas_douter": (_int, [_int, _i64, _i64, _vp, _vp, _vp, _vp]),
    "gbblas_stranspose": (_int, [_i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _vp]),
    "gbblas_dtranspose": (_int, [_i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _vp]),
    "gbblas_stranspose_inplace": (_int, [_i64, _vp, _vp]),
    "gbblas_dtranspose_inplace": (_int, [_i64, _vp, _vp]),
    "gbblas_sew": (_int, [_int, _i64, _vp, _vp, _vp, _vp]),
    "gbblas_dew": (_int, [_int, _i64, _vp, _vp, _vp, _vp]),
    "gbblas_souter_host": (_int, [_int, _i64, _i64, _vp, _vp, _vp]),
    "gbblas_douter_host": (_int, [_int, _i64, _i64, _vp, _vp, _vp]),
    "gbblas_stranspose_host": (_int, [_i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64]),
    "gbblas_dtranspose_host": (_int, [_i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64]),
    "gbblas_stranspose_inplace_host": (_int, [_i64, _vp]),
    "gbblas_dtranspose_inplace_host": (_int, [_i64, _vp]),
    "gbblas_sew_host": (_int, [_int, _i64, _vp, _vp, _vp]),
    "gbblas_dew_host": (_int, [_int, _i64, _vp, _vp, _vp]),
    "gbblas_seeded_fill": (_int, [ctypes.c_uint64, ctypes.c_int32, _i64, _vp, _vp, _vp]),
}

INJECT_ALLOC = 0   # gbblas_server_inject: pool allocations fail
INJECT_LAUNCH = 1  # gbblas_server_inject: round launches fail

FILL_UNIFORM = 0  # U[-1, 1)
FILL_WIDE = 1     # s * m * 2^e, m in [1, 2), e in [-10, 10]

EW_ADD, EW_SUB, EW_MUL, EW_DIV = 0, 1, 2, 3

_lib = None


class GbblasError(RuntimeError):
    def __init__(self, fn: str, status: int, msg: str):
        super().__init__(f"{fn} -> {STATUS.get(status, status)}: {msg}")
        self.status = status


def kernel_launches() -> int:
    """Kernels launched by libgbblas.so so far in this process."""
    return int(lib().gbblas_kernel_launches())


def build(force: bool = False) -> str:
    return _build.build(force=force)


def lib(auto_build: bool = True):
    """Load libgbblas.so (building it first if it is missing or stale)."""
    global _lib
    if _lib is None:
        if auto_build:
            _build.build()
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with gbblas.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(fn: str, status: int) -> None:
    if status != 0:
        raise GbblasError(fn, status, lib().gbblas_last_error().decode())


def call(name: str, *args) -> None:
    """Call a C-ABI function by name and raise GbblasError on a non-zero status."""
    _check(name, getattr(lib(), name)(*args))


def status_of(name: str, *args) -> int:
    """Call a C-ABI function and return its raw status."""
    return getattr(lib(), name)(*args)


# ---------------------------------------------------------------- torch helpers

def _stream_ptr(stream) -> int | None:
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream or None


def _pfx(t) -> str:
    import torch
    if t.dtype == torch.float32:
        return "s"
    if t.dtype == torch.float64:
        return "d"
    raise TypeError(f"unsupported dtype {t.dtype}")


def _dev(t) -> int:
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    return t.data_ptr()


def gemm(A, B, C, accuracy: int = ACCURACY_FP32, stream=None):
    """C += A @ B on device tensors of any strides (2-D torch tensors).
    float32: `accuracy` is one of ACCURACY_FP32 .. ACCURACY_BF16X6; float64:
    ACCURACY_FP32 (gbblas_dgemm, the library default), ACCURACY_AUTO,
    ACCURACY_FP64 (the FP64 pipes) or ACCURACY_FP64_DIGITS7 / 8."""
    M, K = A.shape
    N = B.shape[1]
    p = _pfx(A)
    args = [M, N, K, _dev(A), A.stride(0), A.stride(1), _dev(B), B.stride(0), B.stride(1),
            _dev(C), C.stride(0), C.stride(1)]
    if p == "s":
        call("gbblas_sgemm", *args, accuracy, _stream_ptr(stream))
    elif accuracy == ACCURACY_FP32:
        call("gbblas_dgemm", *args, _stream_ptr(stream))
    else:
        call("gbblas_dgemm_ex", *args, accuracy, _stream_ptr(stream))
    return C


def mtv(layout: int, M: int, N: int, A, x, y, stream=None):
    """amt::mtv on a dense buffer A (M x N in `layout`); see include/gbblas.h."""
    call(f"gbblas_{_pfx(A)}mtv", layout, M, N, _dev(A), _dev(x), _dev(y), _stream_ptr(stream))
    return y


def vtm(layout: int, M: int, N: int, A, v, y, stream=None):
    call(f"gbblas_{_pfx(A)}vtm", layout, M, N, _dev(A), _dev(v), _dev(y), _stream_ptr(stream))
    return y


def gemv(layout: int, transpose: bool, M: int, N: int, A, x, y, accumulate: bool, stream=None):
    call(f"gbblas_{_pfx(A)}gemv", layout, int(transpose), M, N, _dev(A), _dev(x), int(accumulate), _dev(y),
         _stream_ptr(stream))
    return y


def dot(a, b, out, stream=None):
    """out[0] = a . b (out is a 1-element device tensor)."""
    call(f"gbblas_{_pfx(a)}dot", a.numel(), _dev(a), _dev(b), _dev(out), _stream_ptr(stream))
    return out


# ---------------------------------------------------------------- batching

class GemmDesc(ctypes.Structure):
    """gbblas_gemm_desc: C += A*B with element strides (device pointers)."""
    _fields_ = [("M", _i64), ("N", _i64), ("K", _i64), ("A", _vp), ("rsa", _i64), ("csa", _i64),
                ("B", _vp), ("rsb", _i64), ("csb", _i64), ("C", _vp), ("rsc", _i64), ("csc", _i64)]


class GemvDesc(ctypes.Structure):
    """gbblas_gemv_desc: y = op(A) x (+ y); A dense M x N in `layout` (device pointers)."""
    _fields_ = [("layout", ctypes.c_int32), ("transpose", ctypes.c_int32), ("accumulate", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("M", _i64), ("N", _i64), ("A", _vp), ("x", _vp), ("y", _vp)]


def gemm_desc(A, B, C) -> GemmDesc:
    """Descriptor of C += A @ B for 2-D float32 CUDA tensors (any strides)."""
    return GemmDesc(A.shape[0], B.shape[1], A.shape[1], _dev(A), A.stride(0), A.stride(1),
                    _dev(B), B.stride(0), B.stride(1), _dev(C), C.stride(0), C.stride(1))


def gemv_desc(layout, transpose, M, N, A, x, y, accumulate=False) -> GemvDesc:
    return GemvDesc(layout, int(transpose), int(accumulate), 0, M, N, _dev(A), _dev(x), _dev(y))


def gemm_grouped(descs, accuracy: int = ACCURACY_BF16X6, stream=None):
    arr = (GemmDesc * len(descs))(*descs)
    call("gbblas_sgemm_grouped", ctypes.addressof(arr), len(descs), accuracy, _stream_ptr(stream))


def gemv_grouped(descs, stream=None):
    arr = (GemvDesc * len(descs))(*descs)
    call("gbblas_sgemv_grouped", ctypes.addressof(arr), len(descs), _stream_ptr(stream))


class Batch:
    """A batch of GEMMs and GEMVs captured into one CUDA graph
    (gbblas_batch_create / run / sync / destroy)."""

    def __init__(self, gemms=(), gemvs=(), accuracy: int = ACCURACY_BF16X6):
        ga = (GemmDesc * max(1, len(gemms)))(*gemms)
        va = (GemvDesc * max(1, len(gemvs)))(*gemvs)
        h = ctypes.c_void_p()
        call("gbblas_batch_create", ctypes.addressof(ga), len(gemms), accuracy, ctypes.addressof(va), len(gemvs),
             ctypes.byref(h))
        self.handle = h

    def run(self, stream=None):
        call("gbblas_batch_run", self.handle, _stream_ptr(stream))

    def sync(self):
        call("gbblas_batch_sync", self.handle)

    def close(self):
        if self.handle:
            call("gbblas_batch_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- serving

OP_MTM, OP_MTV, OP_VTM, OP_DOT = 0, 1, 2, 3
F32, F64 = 0, 1


class Request(ctypes.Structure):
    """gbblas_request (device pointers)."""
    _fields_ = [("op", ctypes.c_int32), ("dtype", ctypes.c_int32), ("accuracy", ctypes.c_int32),
                ("layout", ctypes.c_int32), ("M", _i64), ("N", _i64), ("K", _i64),
                ("A", _vp), ("B", _vp), ("C", _vp)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("streams", ctypes.c_int32), ("max_group", ctypes.c_int32), ("budget_bytes", _i64),
                ("scratch_bytes", _i64), ("heavy_streams", ctypes.c_int32), ("heavy_sm_percent", ctypes.c_int32),
                ("heavy_us", _i64), ("slice_us", _i64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", _i64), ("completed", _i64), ("rejected", _i64), ("rounds", _i64),
                ("peak_inflight_bytes", _i64), ("mean_round_size", ctypes.c_double)]


class Server:
    """gbblas_server_*: continuous-batching request loop on the current device."""

    def __init__(self, streams=0, max_group=0, budget_bytes=0, scratch_bytes=0, heavy_streams=0, heavy_us=0,
                 heavy_sm_percent=0, slice_us=0):
        cfg = ServerConfig(streams, max_group, budget_bytes, scratch_bytes, heavy_streams, heavy_sm_percent, heavy_us,
                           slice_us)
        h = ctypes.c_void_p()
        call("gbblas_server_create", ctypes.byref(cfg), ctypes.byref(h))
        self.handle = h

    def alloc(self, nbytes: int) -> int:
        p = ctypes.c_void_p()
        call("gbblas_server_alloc", self.handle, nbytes, ctypes.byref(p))
        return p.value

    def free(self, ptr: int) -> None:
        call("gbblas_server_free", self.handle, ptr)

    def submit(self, req: Request) -> int:
        t = ctypes.c_uint64()
        call("gbblas_server_submit", self.handle, ctypes.byref(req), ctypes.byref(t))
        return t.value

    def wait(self, ticket: int) -> float:
        lat = ctypes.c_double()
        call("gbblas_server_wait", self.handle, ticket, ctypes.byref(lat))
        return lat.value

    def run_trace(self, reqs, arrivals):
        import numpy as np
        n = len(reqs)
        arr = (Request * max(1, n))(*reqs)
        t = np.ascontiguousarray(arrivals, dtype=np.float64)
        lat = np.zeros(max(1, n), np.float64)
        call("gbblas_server_run_trace", self.handle, ctypes.addressof(arr), t.ctypes.data, n, lat.ctypes.data)
        return lat[:n]

    def request_times(self, ticket: int):
        """gbblas_server_request_times: (queued, host launch, device and
        completion) seconds and the size of the request's round."""
        import numpy as np
        t = np.zeros(4, np.float64)
        call("gbblas_server_request_times", self.handle, ticket, t.ctypes.data)
        return float(t[0]), float(t[1]), float(t[2]), int(t[3])

    def cancel(self, ticket: int) -> int:
        """gbblas_server_cancel: the raw status (0, or NOT_SUPPORTED when the
        request already runs or ran)."""
        return status_of("gbblas_server_cancel", self.handle, ticket)

    def wait_status(self, ticket: int) -> int:
        """gbblas_server_wait, returning the request's status instead of raising."""
        lat = ctypes.c_double()
        return status_of("gbblas_server_wait", self.handle, ticket, ctypes.byref(lat))

    def inject(self, kind: int, count: int) -> None:
        call("gbblas_server_inject", self.handle, kind, count)

    def stats(self) -> dict:
        st = ServerStats()
        call("gbblas_server_get_stats", self.handle, ctypes.byref(st))
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def close(self):
        if self.handle:
            call("gbblas_server_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- numpy (host) helpers

def _npfx(a) -> str:
    import numpy as np
    if a.dtype == np.float32:
        return "s"
    if a.dtype == np.float64:
        return "d"
    raise TypeError(f"unsupported dtype {a.dtype}")


def gemm_host(M, N, K, a, rsa, csa, b, rsb, csb, c, rsc, csc, accuracy: int = ACCURACY_FP32):
    p = _npfx(a)
    args = [M, N, K, a.ctypes.data, rsa, csa, b.ctypes.data, rsb, csb, c.ctypes.data, rsc, csc]
    if p == "s":
        call("gbblas_sgemm_host", *args, accuracy)
    elif accuracy == ACCURACY_FP32:
        call("gbblas_dgemm_host", *args)
    else:
        call("gbblas_dgemm_ex_host", *args, accuracy)


def mtv_host(layout, M, N, a, x, y):
    call(f"gbblas_{_npfx(a)}mtv_host", layout, M, N, a.ctypes.data, x.ctypes.data, y.ctypes.data)


def vtm_host(layout, M, N, a, v, y):
    call(f"gbblas_{_npfx(a)}vtm_host", layout, M, N, a.ctypes.data, v.ctypes.data, y.ctypes.data)


def dot_host(a, b):
    import numpy as np
    out = np.zeros(1, a.dtype)
    call(f"gbblas_{_npfx(a)}dot_host", a.size, a.ctypes.data, b.ctypes.data, out.ctypes.data)
    return out[0]


# ---------------------------------------------------------------- seeded inputs

def _host_ptr(buf) -> int:
    """Address of a host buffer: a numpy array or a (pinned) CPU torch tensor."""
    if hasattr(buf, "ctypes"):
        return buf.ctypes.data
    if getattr(buf, "is_cuda", False):
        raise ValueError("seeded_fill writes host memory; got a CUDA tensor")
    return buf.data_ptr()


def _numel(buf) -> int:
    return int(buf.size if hasattr(buf, "ctypes") else buf.numel())


def seeded_fill(seed: int, f32=None, f64=None, kind: int = FILL_UNIFORM) -> None:
    """Fill host buffers with the benchmark configurations' seeded inputs
    (gbblas_seeded_fill): one std::mt19937_64(seed) draws the segments in
    order.  `f32` / `f64` are equally long lists of host buffers (numpy arrays
    or CPU torch tensors, contiguous) or None; entry i of either list may be
    None, and segment i's length comes from whichever buffer is given.  An
    int in place of a buffer is a segment of that many values drawn and
    skipped."""
    f32 = list(f32) if f32 is not None else None
    f64 = list(f64) if f64 is not None else None
    nseg = len(f32 if f32 is not None else (f64 or []))
    counts = (ctypes.c_int64 * max(nseg, 1))()
    p32 = (ctypes.c_void_p * max(nseg, 1))()
    p64 = (ctypes.c_void_p * max(nseg, 1))()
    for i in range(nseg):
        a = f32[i] if f32 is not None else None
        b = f64[i] if f64 is not None else None
        if isinstance(a, int) or isinstance(b, int):
            counts[i] = int(a if isinstance(a, int) else b)
            p32[i] = p64[i] = None
            continue
        if a is None and b is None:
            raise ValueError(f"segment {i} has no buffer")
        n = _numel(a) if a is not None else _numel(b)
        if a is not None and b is not None and _numel(b) != n:
            raise ValueError(f"segment {i}: float and double buffers differ in length")
        counts[i] = n
        p32[i] = _host_ptr(a) if a is not None else None
        p64[i] = _host_ptr(b) if b is not None else None
    call("gbblas_seeded_fill", seed, kind, nseg, counts, p32, p64)
