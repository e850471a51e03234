"""Builds and runs the C++ check of the HCore++-shaped adapter (tests/cpp/test_hcore_gemm.cpp):
every tile combination through hcorepp::api::HCore<double>::Gemm against the reference's pass
rule, then Potrf, Trsm, Syrk and Gemm(aCholesky) against host loops, and a TilePacker round trip.  The compile step runs without a GPU; the run needs one."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_hcore_gemm.cpp")
BIN = os.path.join(ROOT, "hcorepp_gb300", "_build", "test_hcore_gemm")


def build_binary():
    from hcorepp_gb300.build import build, nvcc
    lib = build()
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    cmd = [nvcc(), "-std=c++17", "-O2", "-x", "cu", "-I", os.path.join(ROOT, "include"), SRC, "-o", BIN,
           "-L", os.path.dirname(lib), "-lhcgb", "-Xlinker", "-rpath=" + os.path.dirname(lib)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return BIN


def test_adapter_compiles():
    assert os.path.exists(build_binary())


@pytest.mark.gpu
def test_adapter_all_combinations_pass_reference_rule():
    exe = build_binary()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("Pass") == 31
