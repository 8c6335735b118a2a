"""The C++ drop-in headers (include/mtm.hpp, mtv.hpp, dot.hpp).

CPU: the reference-style test program tests/cpp/test_dropin.cpp compiles
against the headers and the uBLAS compat shim and links against
libgbblas.so, and a caller that mixes value types fails to compile (the
reference's static_assert).
GPU: the program runs the reference's test cases through amt:: on the GB300
and checks them against the CPU oracle.
"""
import os
import subprocess

import pytest

import gbblas

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_dropin.cpp")
BUILD = os.path.join(ROOT, "openmp-blas_gb300", "_build")
EXE = os.path.join(BUILD, "test_dropin")
LIBDIR = os.path.dirname(gbblas.LIB_PATH)
INCLUDES = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "openmp-blas_gb300", "compat")]


def compile_dropin() -> str:
    gbblas.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liboracle.so"], check=True)
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["g++", "-std=c++20", "-O2", "-Wall", "-Wextra", *INCLUDES, SRC, "-o", EXE,
           gbblas.LIB_PATH, os.path.join(ROOT, "oracle", "liboracle.so"),
           "-Wl,-rpath," + LIBDIR, "-Wl,-rpath," + os.path.join(ROOT, "oracle")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return EXE


def test_dropin_compiles_and_links():
    assert os.path.exists(compile_dropin())


def test_mixed_value_types_rejected_at_compile_time(tmp_path):
    src = tmp_path / "bad.cpp"
    src.write_text(
        "#include <mtm.hpp>\n"
        "int main(){ auto a = amt::make_tensor<float>(2,2); auto b = amt::make_tensor<double>(2,2);\n"
        "auto c = amt::make_tensor<float>(2,2); auto f = amt::mtm(c, a, b, std::nullopt); (void)f; }\n")
    r = subprocess.run(["g++", "-std=c++20", "-fsyntax-only", *INCLUDES, str(src)], capture_output=True, text=True)
    assert r.returncode != 0
    assert "same value_type" in r.stderr


@pytest.mark.gpu
def test_dropin_runs_reference_cases_on_gpu(cuda):
    exe = compile_dropin()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 failures" in r.stdout


def test_el_op_rejects_predicates_without_a_device_form(tmp_path):
    src = tmp_path / "bad_pred.cpp"
    src.write_text(
        "#include <el_wise_op.hpp>\n"
        "int main(){ auto a = amt::make_tensor<float>(1,4); auto c = amt::make_tensor<float>(1,4);\n"
        "amt::el_op::apply_ops(c, a, a, std::nullopt, [](float x, float y){ return x > y ? x : y; }); }\n")
    r = subprocess.run(["g++", "-std=c++20", "-fsyntax-only", *INCLUDES, str(src)], capture_output=True, text=True)
    assert r.returncode != 0
    assert "std::plus" in r.stderr
