"""ctypes bindings for the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Two libraries are wrapped:

* ``oracle/liboracle.so`` - the C restatement of the reference's hot path
  (oracle/oracle.c, which cites the reference file:line it follows).  It is
  built on every machine (``make -C oracle``).
* ``oracle/_ref/libamt_ref.so`` - the reference's own headers compiled
  unmodified (``make -C oracle ref REF_ROOT=<checkout>``), present only where the reference
  sources are.  ``ref_available()`` says whether it loaded.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg and
reference arm import this module.  The GPU library never does.

Layouts: 0 = first_order (column-major), 1 = last_order (row-major).
All array arguments are numpy arrays; matrices are passed as their dense
buffer in the stated layout (use ``to_layout``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libamt_ref.so")

FIRST_ORDER = 0
LAST_ORDER = 1

_c_size = ctypes.c_size_t
_c_pd = ctypes.c_ssize_t
_vp = ctypes.c_void_p

_lib = None
_ref = None
_ref_tried = False


def build(with_ref: bool = False) -> None:
    """Compile liboracle.so (and, if asked and possible, the reference lib)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    root = os.environ.get("AMT_REFERENCE_ROOT", "")
    if with_ref and root:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_ROOT={root}"], check=False)


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = ctypes.CDLL(ORACLE_SO)
        for s, T in (("s", ctypes.c_float), ("d", ctypes.c_double)):
            f = getattr(L, f"orc_{s}gemm")
            f.argtypes = [_c_size, _c_size, _c_size, _vp, _c_pd, _c_pd, _vp, _c_pd, _c_pd, _vp, _c_pd, _c_pd]
            f.restype = ctypes.c_int
            for nm in ("mtv", "vtm"):
                f = getattr(L, f"orc_{s}{nm}")
                f.argtypes = [ctypes.c_int, _c_size, _c_size, _vp, _vp, _vp]
                f.restype = None
            f = getattr(L, f"orc_{s}dot")
            f.argtypes = [_c_size, _vp, _vp]
            f.restype = T
            f = getattr(L, f"orc_{s}dot_tuning")
            f.argtypes = [_c_size, _vp, _vp, _c_size, _c_size, _c_size]
            f.restype = T
            for nm in ("pack", "pack_trans"):
                f = getattr(L, f"orc_{s}{nm}")
                f.argtypes = [_vp, _c_size, _vp, _vp, _c_size, _c_size]
                f.restype = None
            f = getattr(L, f"orc_{s}dot_exact")
            f.argtypes = [_c_size, _vp, _vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
            f.restype = None
            f = getattr(L, f"orc_{s}outer")
            f.argtypes = [ctypes.c_int, _c_size, _c_size, _vp, _vp, _vp]
            f.restype = None
            f = getattr(L, f"orc_{s}transpose")
            f.argtypes = [_c_size, _c_size, _vp, _c_pd, _c_pd, _vp, _c_pd, _c_pd]
            f.restype = None
            f = getattr(L, f"orc_{s}transpose_inplace")
            f.argtypes = [_c_size, _vp]
            f.restype = None
            f = getattr(L, f"orc_{s}ew")
            f.argtypes = [ctypes.c_int, _c_size, _vp, _vp, _vp]
            f.restype = None
        L.orc_sgemm_sample_exact.argtypes = [_c_size, _vp, _c_pd, _c_pd, _vp, _c_pd, _c_pd, _c_size, _vp, _vp, _vp, _vp]
        L.orc_sgemm_sample_exact.restype = None
        L.orc_dgemm_sample_exact.argtypes = [_c_size, _vp, _c_pd, _c_pd, _vp, _c_pd, _c_pd, _c_size, _vp, _vp, _vp, _vp]
        L.orc_dgemm_sample_exact.restype = None
        L.orc_cache_info.argtypes = [_vp, _vp, _vp]
        L.orc_partition.argtypes = [_c_size, ctypes.c_int, _vp]
        L.orc_max_threads.restype = ctypes.c_int
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_mt64_raw.argtypes = [ctypes.c_uint64, ctypes.c_int64, _vp]
        L.orc_mt64_raw.restype = None
        L.orc_seeded_fill.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int64, _vp, _vp, _vp]
        L.orc_seeded_fill.restype = ctypes.c_int
        _lib = L
    return _lib


def ref():
    """The reference's own compiled hot path, or None where it is absent."""
    global _ref, _ref_tried
    if not _ref_tried:
        _ref_tried = True
        if os.path.exists(REF_SO):
            R = ctypes.CDLL(REF_SO)
            for s, T in (("s", ctypes.c_float), ("d", ctypes.c_double)):
                f = getattr(R, f"ref_{s}gemm")
                f.argtypes = [ctypes.c_int] * 3 + [_c_size] * 3 + [_vp] * 3
                f.restype = ctypes.c_int
                for nm in ("mtv", "vtm"):
                    f = getattr(R, f"ref_{s}{nm}")
                    f.argtypes = [ctypes.c_int, _c_size, _c_size, _vp, _vp, _vp]
                    f.restype = ctypes.c_int
                f = getattr(R, f"ref_{s}dot")
                f.argtypes = [_c_size, _vp, _vp]
                f.restype = T
                f = getattr(R, f"ref_{s}dot_tuning")
                f.argtypes = [_c_size, _vp, _vp, _c_size, _c_size, _c_size]
                f.restype = T
                f = getattr(R, f"ref_{s}outer")
                f.argtypes = [ctypes.c_int, _c_size, _c_size, _vp, _vp, _vp]
                f.restype = ctypes.c_int
                f = getattr(R, f"ref_{s}transpose")
                f.argtypes = [ctypes.c_int, ctypes.c_int, _c_size, _c_size, _vp, _vp]
                f.restype = ctypes.c_int
                f = getattr(R, f"ref_{s}transpose_inplace")
                f.argtypes = [_c_size, _vp]
                f.restype = ctypes.c_int
                f = getattr(R, f"ref_{s}ew")
                f.argtypes = [ctypes.c_int, _c_size, _vp, _vp, _vp]
                f.restype = ctypes.c_int
            R.ref_spack.argtypes = [_vp, _c_size, _vp, _vp, _c_size, _c_size, ctypes.c_int]
            R.ref_cache_info.argtypes = [_vp, _vp, _vp]
            _ref = R
    return _ref


def ref_available() -> bool:
    return ref() is not None


def _sfx(dtype) -> str:
    dt = np.dtype(dtype)
    if dt == np.float32:
        return "s"
    if dt == np.float64:
        return "d"
    raise TypeError(f"unsupported dtype {dt}")


def to_layout(a: np.ndarray, layout: int) -> np.ndarray:
    """Dense buffer of a 2-D logical matrix in the given layout (flat)."""
    return np.ascontiguousarray(a.T if layout == FIRST_ORDER else a).reshape(-1)


def from_layout(buf: np.ndarray, rows: int, cols: int, layout: int) -> np.ndarray:
    """Logical rows x cols matrix from its dense buffer in `layout`."""
    if layout == FIRST_ORDER:
        return buf.reshape(cols, rows).T
    return buf.reshape(rows, cols)


def strides(rows: int, cols: int, layout: int):
    return (1, rows) if layout == FIRST_ORDER else (cols, 1)


# --------------------------------------------------------------------------
# Oracle (C restatement)
# --------------------------------------------------------------------------

def gemm(A: np.ndarray, B: np.ndarray, C: np.ndarray, la: int, lb: int, lc: int) -> np.ndarray:
    """C += A @ B via the oracle; A, B, C are logical 2-D matrices.  Returns new C."""
    M, K = A.shape
    N = B.shape[1]
    dt = A.dtype
    a, b, c = to_layout(A, la), to_layout(B, lb), to_layout(C.astype(dt), lc).copy()
    rsa, csa = strides(M, K, la)
    rsb, csb = strides(K, N, lb)
    rsc, csc = strides(M, N, lc)
    rc = getattr(lib(), f"orc_{_sfx(dt)}gemm")(M, N, K, _ptr(a), rsa, csa, _ptr(b), rsb, csb, _ptr(c), rsc, csc)
    if rc != 0:
        raise RuntimeError("oracle gemm failed")
    return from_layout(c, M, N, lc).copy()


def gemm_raw(M, N, K, a, rsa, csa, b, rsb, csb, c, rsc, csc) -> None:
    """C += A @ B on raw dense buffers with explicit strides (in place on c)."""
    rc = getattr(lib(), f"orc_{_sfx(a.dtype)}gemm")(M, N, K, _ptr(a), rsa, csa, _ptr(b), rsb, csb, _ptr(c), rsc, csc)
    if rc != 0:
        raise RuntimeError("oracle gemm failed")


def mtv(A: np.ndarray, x: np.ndarray, y: np.ndarray, layout: int) -> np.ndarray:
    """Reference mtv semantics: column-major accumulates, row-major overwrites."""
    M, N = A.shape
    a = to_layout(A, layout)
    yy = np.ascontiguousarray(y, dtype=A.dtype).copy()
    xx = np.ascontiguousarray(x, dtype=A.dtype)
    getattr(lib(), f"orc_{_sfx(A.dtype)}mtv")(layout, M, N, _ptr(a), _ptr(xx), _ptr(yy))
    return yy


def mtv_raw(layout, M, N, a, x, y) -> None:
    getattr(lib(), f"orc_{_sfx(a.dtype)}mtv")(layout, M, N, _ptr(a), _ptr(x), _ptr(y))


def vtm(A: np.ndarray, v: np.ndarray, y: np.ndarray, layout: int) -> np.ndarray:
    """y = v^T A (column-major A overwrites y, row-major A accumulates)."""
    M, N = A.shape
    a = to_layout(A, layout)
    yy = np.ascontiguousarray(y, dtype=A.dtype).copy()
    vv = np.ascontiguousarray(v, dtype=A.dtype)
    getattr(lib(), f"orc_{_sfx(A.dtype)}vtm")(layout, M, N, _ptr(a), _ptr(vv), _ptr(yy))
    return yy


def dot(a: np.ndarray, b: np.ndarray):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b, dtype=a.dtype)
    return getattr(lib(), f"orc_{_sfx(a.dtype)}dot")(a.size, _ptr(a), _ptr(b))


def dot_tuning(a: np.ndarray, b: np.ndarray, b1: int, b2: int, b3: int):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b, dtype=a.dtype)
    return getattr(lib(), f"orc_{_sfx(a.dtype)}dot_tuning")(a.size, _ptr(a), _ptr(b), b1, b2, b3)


def dot_exact(a: np.ndarray, b: np.ndarray):
    """(sum a*b, sum |a*b|) in long double."""
    d = ctypes.c_double()
    t = ctypes.c_double()
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b, dtype=a.dtype)
    getattr(lib(), f"orc_{_sfx(a.dtype)}dot_exact")(a.size, _ptr(a), _ptr(b), ctypes.byref(d), ctypes.byref(t))
    return d.value, t.value


def gemm_sample_exact(K, a, rsa, csa, b, rsb, csb, rows, cols):
    """Sampled entries of A@B and |A|@|B| in long double (float or double inputs)."""
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    out = np.empty(rows.size, np.float64)
    aout = np.empty(rows.size, np.float64)
    fn = lib().orc_dgemm_sample_exact if a.dtype == np.float64 else lib().orc_sgemm_sample_exact
    fn(K, _ptr(a), rsa, csa, _ptr(b), rsb, csb, rows.size, _ptr(rows), _ptr(cols), _ptr(out), _ptr(aout))
    return out, aout


def pack(inp: np.ndarray, wi, wo: int, m: int, n: int, out: np.ndarray, offset_in: int = 0,
         offset_out: int = 0, trans: bool = False) -> None:
    """The reference's panel packers on flat buffers (include/utils.hpp:99-141)."""
    w = np.asarray(wi, dtype=np.uintp)
    isz = inp.itemsize
    fn = getattr(lib(), f"orc_{_sfx(inp.dtype)}{'pack_trans' if trans else 'pack'}")
    fn(_ptr(out) + offset_out * isz, wo, _ptr(inp) + offset_in * isz, _ptr(w), m, n)


def cache_info():
    s = np.zeros(3, np.uintp)
    a = np.zeros(3, np.uintp)
    l = np.zeros(3, np.uintp)
    lib().orc_cache_info(_ptr(s), _ptr(a), _ptr(l))
    return s.tolist(), a.tolist(), l.tolist()


def partition(dtype, out_layout: int):
    out = np.zeros(5, np.uintp)
    lib().orc_partition(np.dtype(dtype).itemsize, out_layout, _ptr(out))
    return dict(zip(("MR", "NR", "KB", "MB", "NB"), out.tolist()))


def max_threads() -> int:
    return lib().orc_max_threads()


def set_threads(n: int) -> None:
    lib().orc_set_threads(n)


def outer(a, b, C, layout):
    """C (M x N, logical) += a b^T computed in `layout`; returns the new C."""
    M, N = C.shape
    dt = C.dtype
    c = to_layout(C, layout).copy()
    aa = np.ascontiguousarray(a, dtype=dt)
    bb = np.ascontiguousarray(b, dtype=dt)
    getattr(lib(), f"orc_{_sfx(dt)}outer")(layout, M, N, _ptr(aa), _ptr(bb), _ptr(c))
    return from_layout(c, M, N, layout).copy()


def transpose_raw(M, N, a, rsa, csa, c, rsc, csc) -> None:
    """C(j, i) = A(i, j) on raw buffers with element strides."""
    getattr(lib(), f"orc_{_sfx(a.dtype)}transpose")(M, N, _ptr(a), rsa, csa, _ptr(c), rsc, csc)


def transpose(A, la, lc):
    """A^T of the logical matrix A, computed from A stored in layout la into a
    dense C stored in layout lc; returns the logical N x M result."""
    M, N = A.shape
    a = to_layout(A, la)
    c = np.zeros(M * N, A.dtype)
    rsa, csa = strides(M, N, la)
    rsc, csc = strides(N, M, lc)
    transpose_raw(M, N, a, rsa, csa, c, rsc, csc)
    return from_layout(c, N, M, lc).copy()


def transpose_inplace(buf):
    """Square n x n storage transposed in place (returns a new array)."""
    b = np.ascontiguousarray(buf).copy()
    n = int(round(np.sqrt(b.size)))
    getattr(lib(), f"orc_{_sfx(b.dtype)}transpose_inplace")(n, _ptr(b))
    return b


def ew(op, a, b):
    """a op b element by element: op 0 add, 1 sub, 2 mul, 3 div."""
    aa = np.ascontiguousarray(a)
    bb = np.ascontiguousarray(b, dtype=aa.dtype)
    c = np.empty_like(aa)
    getattr(lib(), f"orc_{_sfx(aa.dtype)}ew")(op, aa.size, _ptr(aa), _ptr(bb), _ptr(c))
    return c


# --------------------------------------------------------------------------
# Reference (compiled from the reference's own headers)
# --------------------------------------------------------------------------

def ref_gemm(A, B, C, la, lb, lc):
    R = ref()
    M, K = A.shape
    N = B.shape[1]
    dt = A.dtype
    a, b, c = to_layout(A, la), to_layout(B, lb), to_layout(C.astype(dt), lc).copy()
    rc = getattr(R, f"ref_{_sfx(dt)}gemm")(lc, la, lb, M, N, K, _ptr(a), _ptr(b), _ptr(c))
    if rc != 0:
        raise RuntimeError("reference mtm threw")
    return from_layout(c, M, N, lc).copy()


def ref_mtv(A, x, y, layout):
    R = ref()
    M, N = A.shape
    a = to_layout(A, layout)
    yy = np.ascontiguousarray(y, dtype=A.dtype).copy()
    xx = np.ascontiguousarray(x, dtype=A.dtype)
    rc = getattr(R, f"ref_{_sfx(A.dtype)}mtv")(layout, M, N, _ptr(a), _ptr(xx), _ptr(yy))
    if rc != 0:
        raise RuntimeError("reference mtv threw")
    return yy


def ref_vtm(A, v, y, layout):
    R = ref()
    M, N = A.shape
    a = to_layout(A, layout)
    yy = np.ascontiguousarray(y, dtype=A.dtype).copy()
    vv = np.ascontiguousarray(v, dtype=A.dtype)
    rc = getattr(R, f"ref_{_sfx(A.dtype)}vtm")(layout, M, N, _ptr(a), _ptr(vv), _ptr(yy))
    if rc != 0:
        raise RuntimeError("reference vtm threw")
    return yy


def ref_dot(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b, dtype=a.dtype)
    return getattr(ref(), f"ref_{_sfx(a.dtype)}dot")(a.size, _ptr(a), _ptr(b))


def ref_dot_tuning(a, b, b1, b2, b3):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b, dtype=a.dtype)
    return getattr(ref(), f"ref_{_sfx(a.dtype)}dot_tuning")(a.size, _ptr(a), _ptr(b), b1, b2, b3)


def ref_cache_info():
    s = np.zeros(3, np.uintp)
    a = np.zeros(3, np.uintp)
    l = np.zeros(3, np.uintp)
    ref().ref_cache_info(_ptr(s), _ptr(a), _ptr(l))
    return s.tolist(), a.tolist(), l.tolist()


def ref_pack(inp, wi, wo, m, n, out, offset_in=0, offset_out=0, trans=False):
    w = np.asarray(wi, dtype=np.uintp)
    isz = inp.itemsize
    ref().ref_spack(_ptr(out) + offset_out * isz, wo, _ptr(inp) + offset_in * isz, _ptr(w), m, n, 1 if trans else 0)


def ref_outer(a, b, C, layout):
    M, N = C.shape
    dt = C.dtype
    c = to_layout(C, layout).copy()
    aa = np.ascontiguousarray(a, dtype=dt)
    bb = np.ascontiguousarray(b, dtype=dt)
    rc = getattr(ref(), f"ref_{_sfx(dt)}outer")(layout, M, N, _ptr(aa), _ptr(bb), _ptr(c))
    if rc != 0:
        raise RuntimeError("reference outer_prod threw")
    return from_layout(c, M, N, layout).copy()


def ref_transpose(A, la, lc):
    M, N = A.shape
    a = to_layout(A, la)
    c = np.zeros(M * N, A.dtype)
    rc = getattr(ref(), f"ref_{_sfx(A.dtype)}transpose")(la, lc, M, N, _ptr(a), _ptr(c))
    if rc != 0:
        raise RuntimeError("reference transpose threw")
    return from_layout(c, N, M, lc).copy()


def ref_transpose_inplace(buf):
    b = np.ascontiguousarray(buf).copy()
    n = int(round(np.sqrt(b.size)))
    if getattr(ref(), f"ref_{_sfx(b.dtype)}transpose_inplace")(n, _ptr(b)) != 0:
        raise RuntimeError("reference transpose threw")
    return b


def ref_ew(op, a, b):
    aa = np.ascontiguousarray(a)
    bb = np.ascontiguousarray(b, dtype=aa.dtype)
    c = np.zeros_like(aa)
    if getattr(ref(), f"ref_{_sfx(aa.dtype)}ew")(op, aa.size, _ptr(aa), _ptr(bb), _ptr(c)) != 0:
        raise RuntimeError("reference element-wise op threw")
    return c


# ---------------------------------------------------------------- seeded inputs

def mt64_raw(seed: int, n: int) -> np.ndarray:
    """The first n outputs of MT19937-64 seeded with `seed` (the oracle's own
    restatement of the engine)."""
    out = np.empty(n, np.uint64)
    lib().orc_mt64_raw(ctypes.c_uint64(seed), n, _ptr(out))
    return out


def seeded_fill(seed: int, counts, f32: bool = True, f64: bool = True, kind: int = 0):
    """Segments of the seeded inputs drawn in order from one MT19937-64(seed):
    returns (list of float32 arrays or None, list of float64 arrays or None)."""
    counts = [int(c) for c in counts]
    n = len(counts)
    a32 = [np.empty(c, np.float32) for c in counts] if f32 else None
    a64 = [np.empty(c, np.float64) for c in counts] if f64 else None
    cc = (ctypes.c_int64 * max(n, 1))(*counts)
    p32 = (ctypes.c_void_p * max(n, 1))(*([a.ctypes.data for a in a32] if f32 else []))
    p64 = (ctypes.c_void_p * max(n, 1))(*([a.ctypes.data for a in a64] if f64 else []))
    rc = lib().orc_seeded_fill(ctypes.c_uint64(seed), kind, n, cc, p32 if f32 else None, p64 if f64 else None)
    if rc != 0:
        raise ValueError(f"orc_seeded_fill: bad kind {kind}")
    return a32, a64
