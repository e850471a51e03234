"""Build recipe for oracle/_ref/libhcref.so: the reference's OWN CPU path, compiled
from its sources where they lie, against the BLAS++/LAPACK++ shim in oracle/shim
and SciPy's bundled OpenBLAS.  Test infrastructure only.

Usage: python oracle/build_ref.py [REFERENCE_ROOT]
The reference root is the argument, else the environment variable HCOREPP_REFERENCE_ROOT, else
the read-only checkout this recipe was written against (DEFAULT_REFERENCE_ROOT).
Outputs go to oracle/_ref/ only.  Nothing is copied out of the reference tree.
The reference's own build system (CMake + network fetches) is not used.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
DEFAULT_REFERENCE_ROOT = "/root/reference"


def reference_root(argv=None) -> str:
    """Where the reference sources are read from: argv[1], $HCOREPP_REFERENCE_ROOT, or the default."""
    argv = sys.argv if argv is None else argv
    if len(argv) > 1:
        return argv[1]
    return os.environ.get("HCOREPP_REFERENCE_ROOT", DEFAULT_REFERENCE_ROOT)

# The CPU backend of the TLR GEMM path (and what it links against).
SOURCES = [
    "src/api/HCore.cpp",
    "src/operators/concrete/Compressed.cpp",
    "src/operators/concrete/Dense.cpp",
    "src/operators/helpers/CompressionParameters.cpp",
    "src/data-units/DataHolder.cpp",
    "src/data-units/memory-handlers/on-demand/MemoryHandler.cpp",
    "src/kernels/omp/kernels.cpp",
    "src/kernels/ContextManager.cpp",
    "src/helpers/debugging-timer/IdleTimer.cpp",
]


def openblas_lib() -> str:
    import scipy
    libs = glob.glob(os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs", "libscipy_openblas*.so"))
    if not libs:
        raise RuntimeError("SciPy's bundled OpenBLAS was not found")
    return os.path.realpath(libs[0])


def library_path() -> str:
    return os.path.join(OUT, "libhcref.so")


def build(ref_root: str, verbose: bool = False) -> str:
    if not os.path.isdir(os.path.join(ref_root, "src", "api")):
        raise FileNotFoundError(f"no reference sources under {ref_root}")
    os.makedirs(OUT, exist_ok=True)
    blas = openblas_lib()
    flags = ["-O2", "-fPIC", "-std=c++17", "-fopenmp", "-w",
             "-I", os.path.join(ref_root, "include"), "-I", os.path.join(HERE, "shim")]
    jobs = []
    for rel in SOURCES + [os.path.join(HERE, "ref_driver.cpp")]:
        src = rel if os.path.isabs(rel) else os.path.join(ref_root, rel)
        obj = os.path.join(OUT, os.path.basename(rel).replace(".cpp", ".o"))
        if "on-demand" in rel:
            obj = os.path.join(OUT, "OnDemandMemoryHandler.o")
        jobs.append((src, obj))

    def compile_one(job):
        src, obj = job
        cmd = ["g++", *flags, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
        return obj

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(compile_one, jobs))
    lib = library_path()
    subprocess.run(["g++", "-shared", "-fopenmp", "-o", lib, *objs, blas,
                    "-Wl,-rpath," + os.path.dirname(blas)], check=True)
    return lib


if __name__ == "__main__":
    print(build(reference_root(), verbose=True))
