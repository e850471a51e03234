"""Adds the GB300 backend to a checkout of HCore++ (the reference's source tree):

    python hcorepp_gb300/backend/apply_to_reference.py HCOREPP_ROOT

* copies include/hcorepp/kernels/gb300/ and src/kernels/gb300/ from this directory into the tree;
* adds one `#elif defined(USE_GB300)` branch to each backend selector, beside USE_CUDA:
  include/hcorepp/kernels/RunContext.hpp (RunContext), include/hcorepp/kernels/memory.hpp (memory::),
  include/hcorepp/data-units/memory-handlers/MemoryHandler.hpp (the pool memory handler, as for CUDA),
  and src/kernels/CMakeLists.txt (the backend directory).
Idempotent.  A USE_GB300 build defines USE_GB300, adds hcorepp_gb300/../include (hcgb.h) to the
include path and links libhcgb.so; HCoreKernels<double> then runs on GB300 kernels.
"""
from __future__ import annotations

import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

# (file, the line after which the branch goes, the branch)
SELECTORS = [
    ("include/hcorepp/kernels/RunContext.hpp", '#include "cuda/RunContext.hpp"',
     '#elif defined(USE_GB300)\n#include "gb300/RunContext.hpp"'),
    ("include/hcorepp/kernels/memory.hpp", '#include "cuda/memory.hpp"',
     '#elif defined(USE_GB300)\n#include "gb300/memory.hpp"'),
    ("include/hcorepp/data-units/memory-handlers/MemoryHandler.hpp", '#include "pool/MemoryHandler.hpp"',
     '#elif defined(USE_GB300)\n#include "pool/MemoryHandler.hpp"'),
    ("src/kernels/CMakeLists.txt", "add_subdirectory(${CMAKE_CURRENT_SOURCE_DIR}/cuda)",
     "elseif (${USE_GB300})\n    add_subdirectory(${CMAKE_CURRENT_SOURCE_DIR}/gb300)"),
]


def apply(root: str) -> None:
    for rel in ("include/hcorepp/kernels/gb300", "src/kernels/gb300"):
        dst = os.path.join(root, rel)
        os.makedirs(dst, exist_ok=True)
        src = os.path.join(HERE, rel)
        for name in os.listdir(src):
            shutil.copy2(os.path.join(src, name), os.path.join(dst, name))
    for rel, anchor, branch in SELECTORS:
        path = os.path.join(root, rel)
        text = open(path).read()
        if "USE_GB300" in text:
            continue
        i = text.index(anchor) + len(anchor)
        text = text[:i] + "\n" + branch + text[i:]
        open(path, "w").write(text)


if __name__ == "__main__":
    apply(sys.argv[1])
