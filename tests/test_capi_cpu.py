"""The C-ABI library without a GPU: it builds for sm_103a, loads, exports every
symbol include/gbblas.h declares, validates arguments before touching a
device, and fails loudly (GBBLAS_STATUS_NO_DEVICE) rather than computing
anything on the CPU when no GB300 is present."""
import os
import re

import numpy as np
import pytest

import gbblas

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "gbblas.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbblas_[a-z0-9_]+)\s*\(", src)))


def test_library_builds_and_loads():
    path = gbblas.build()
    assert os.path.exists(path)
    assert gbblas.lib().gbblas_version().decode().startswith("gbblas")


def test_every_declared_symbol_is_exported():
    names = declared_symbols()
    assert len(names) >= 20
    L = gbblas.lib()
    for n in names:
        assert hasattr(L, n), n
        assert n in gbblas.SIGNATURES, f"{n} missing from the Python binding"


def test_status_strings():
    L = gbblas.lib()
    for code, name in gbblas.STATUS.items():
        assert L.gbblas_status_string(code).decode() == "GBBLAS_STATUS_" + name


@pytest.mark.parametrize("fn,args", [
    ("gbblas_sgemm", (-1, 2, 2, None, 1, 2, None, 1, 2, None, 1, 2, 0, None)),
    ("gbblas_sgemm", (2, 2, 2, None, -1, 2, None, 1, 2, None, 1, 2, 0, None)),
    ("gbblas_sgemm", (2, 2, 2, 16, 1, 2, 16, 1, 2, None, 1, 2, 0, None)),
    ("gbblas_dgemm", (2, 2, 2, 16, 1, 2, 16, 1, 2, 16, 0, 0, None)),
    ("gbblas_dgemm_ex", (2, 2, 2, 16, 1, 2, 16, 1, 2, 16, 2, 1, 4, None)),  # BF16X6 is float-only
    ("gbblas_dgemm_ex_host", (2, 2, 2, 16, 1, 2, 16, 1, 2, 16, 2, 1, 1)),
    ("gbblas_sgemm_host", (2, 2, 2, 16, 1, 2, 16, 1, 2, 16, 2, 1, 5)),  # FP64 is double-only
    ("gbblas_dgemm_ex", (2, 2, 2, 16, 1, 2, 16, 1, 2, 16, 2, 1, 8, None)),
    ("gbblas_dgemm_ex", (2, -2, 2, 16, 1, 2, 16, 1, 2, 16, 2, 1, 6, None)),
    ("gbblas_smtv", (2, 4, 4, 16, 16, 16, None)),
    ("gbblas_dvtm", (0, -3, 4, 16, 16, 16, None)),
    ("gbblas_sdot", (-5, 16, 16, 16, None)),
    ("gbblas_sdot", (5, None, 16, 16, None)),
    ("gbblas_ddot_tuning", (5, 16, 16, 0, 1, 1, 16, None)),
    ("gbblas_souter", (2, 4, 4, 16, 16, 16, None)),
    ("gbblas_douter", (1, -1, 4, 16, 16, 16, None)),
    ("gbblas_souter", (1, 4, 4, None, 16, 16, None)),
    ("gbblas_stranspose", (4, 4, 16, -1, 1, 16, 4, 1, None)),
    ("gbblas_dtranspose", (4, 4, 16, 4, 1, 16, 0, 1, None)),
    ("gbblas_stranspose", (4, 4, None, 4, 1, 16, 4, 1, None)),
    ("gbblas_stranspose_inplace", (-2, 16, None)),
    ("gbblas_dtranspose_inplace", (3, None, None)),
    ("gbblas_sew", (4, 8, 16, 16, 16, None)),
    ("gbblas_dew", (0, -8, 16, 16, 16, None)),
    ("gbblas_sew_host", (1, 8, None, 16, 16)),
    ("gbblas_selftest_bounded_wait", (0, None)),
    ("gbblas_selftest_bounded_wait", (2000001, None)),
    ("gbblas_server_request_times", (None, 0, 16)),
    ("gbblas_server_request_times", (16, 0, None)),
])
def test_invalid_arguments_rejected_without_device(fn, args):
    assert gbblas.status_of(fn, *args) == 1  # GBBLAS_STATUS_INVALID_VALUE
    assert gbblas.lib().gbblas_last_error().decode()


def test_no_cpu_fallback_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    a = np.ones(64, np.float32)
    out = np.zeros(1, np.float32)
    st = gbblas.status_of("gbblas_sdot_host", 64, a.ctypes.data, a.ctypes.data, out.ctypes.data)
    assert st == 7  # GBBLAS_STATUS_NO_DEVICE
    assert out[0] == 0
    with pytest.raises(gbblas.GbblasError):
        gbblas.dot_host(a, a)


def test_descriptor_structs_match_the_c_layout(tmp_path):
    """The ctypes mirrors of gbblas_gemm_desc / gbblas_gemv_desc have the C
    sizes and field offsets (checked with the C compiler)."""
    import ctypes
    import subprocess
    src = tmp_path / "layout.c"
    fields_g = [f for f, _ in gbblas.GemmDesc._fields_]
    fields_v = [f for f, _ in gbblas.GemvDesc._fields_]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gbblas.h"', "int main(void){",
             'printf("%zu\\n", sizeof(gbblas_gemm_desc));', 'printf("%zu\\n", sizeof(gbblas_gemv_desc));']
    lines += [f'printf("%zu\\n", offsetof(gbblas_gemm_desc, {f}));' for f in fields_g]
    lines += [f'printf("%zu\\n", offsetof(gbblas_gemv_desc, {f}));' for f in fields_v]
    lines += ["return 0;}"]
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [ctypes.sizeof(gbblas.GemmDesc), ctypes.sizeof(gbblas.GemvDesc)]
    want += [getattr(gbblas.GemmDesc, f).offset for f in fields_g]
    want += [getattr(gbblas.GemvDesc, f).offset for f in fields_v]
    assert out == want


def test_accuracy_constants_match_the_header():
    """The binding's ACCURACY_* values are the header's gbblas_accuracy values."""
    import re
    text = open(os.path.join(ROOT, "include", "gbblas.h")).read()
    enum = dict((m.group(1), int(m.group(2))) for m in re.finditer(r"GBBLAS_ACCURACY_(\w+)\s*=\s*(\d+)", text))
    assert {"FP32", "BF16X3", "FP8", "AUTO", "BF16X6", "FP64", "FP64_DIGITS7", "FP64_DIGITS8", "FP16X3"} <= set(enum)
    for name, value in enum.items():
        assert getattr(gbblas, "ACCURACY_" + name) == value, name
    assert len(set(enum.values())) == len(enum)
