"""The GB300 backend at the reference's HCoreKernels / RunContext layer compiles against the
reference's own headers: a temporary copy of the reference tree gets the backend through
hcorepp_gb300/backend/apply_to_reference.py, and the backend sources plus the reference's
operator sources (Compressed.cpp, Dense.cpp, HCore.cpp: the recompression that then runs on
the backend) compile with USE_GB300.  CPU only; skipped where the reference tree is absent."""
import os
import shutil
import subprocess
import sys
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle.build_ref import reference_root  # noqa: E402

REF = reference_root([])
pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "include", "hcorepp")),
                                reason="reference tree not present")


def _cuda_include():
    for c in ("/usr/local/cuda/include",):
        if os.path.exists(os.path.join(c, "cuda_runtime.h")):
            return c
    pytest.skip("CUDA headers not found")


def test_backend_compiles_against_reference_headers():
    sys.path.insert(0, os.path.join(ROOT, "hcorepp_gb300", "backend"))
    from apply_to_reference import apply
    with tempfile.TemporaryDirectory() as tmp:
        tree = os.path.join(tmp, "hcorepp")
        shutil.copytree(os.path.join(REF, "include"), os.path.join(tree, "include"))
        shutil.copytree(os.path.join(REF, "src"), os.path.join(tree, "src"))
        apply(tree)
        apply(tree)  # idempotent
        rc = open(os.path.join(tree, "include/hcorepp/kernels/RunContext.hpp")).read()
        assert rc.count("USE_GB300") == 1
        flags = ["-std=c++17", "-DUSE_GB300", "-fsyntax-only", "-w",
                 "-I", os.path.join(tree, "include"), "-I", os.path.join(ROOT, "include"),
                 "-I", os.path.join(ROOT, "oracle", "shim"), "-I", _cuda_include()]
        sources = ["src/kernels/gb300/kernels.cpp", "src/kernels/gb300/RunContext.cpp",
                   "src/operators/concrete/Compressed.cpp", "src/operators/concrete/Dense.cpp", "src/api/HCore.cpp"]
        for rel in sources:
            r = subprocess.run(["g++", *flags, os.path.join(tree, rel)], capture_output=True, text=True)
            assert r.returncode == 0, f"{rel}:\n{r.stderr[-3000:]}"
