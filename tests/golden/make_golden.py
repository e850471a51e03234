"""Extract the known-answer vectors of the reference's own tests into kat.json.

Run in a checkout that has the reference sources (pass their root as argv[1]);
the committed kat.json is what the tests read, so the reference tree is not
needed at test time.  Each entry records the file and line range it came from.
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

# (key, file, first line, last line, array names) -- ranges are 1-based, inclusive.
SOURCES = [
    ("multiply_by_alpha", "tests/kernels/TestKernels.cpp", 122, 156, ["matrix_A", "matrix_C"]),
    ("process_vpointer", "tests/kernels/TestKernels.cpp", 157, 192, ["cv", "b_data", "expected"]),
    ("calculate_uvptr", "tests/kernels/TestKernels.cpp", 239, 265, ["v_new", "expected"]),
    ("calculate_vtnew_no_ungqr", "tests/kernels/TestKernels.cpp", 267, 298, ["vt", "vt_new", "sigma"]),
    ("calculate_vtnew_ungqr", "tests/kernels/TestKernels.cpp", 300, 329, ["vt", "vt_new", "sigma"]),
    ("geqrf", "tests/kernels/TestKernels.cpp", 470, 511, ["matrix_A", "a_expected", "tau_expected"]),
    ("compressed_tile_ddc", "tests/operators/TestCompressedTile.cpp", 124, 260, ["matrix_A", "matrix_B",
                                                                                 "output_matrix"]),
    ("gemm_test9_ccc", "tests/api/TestGemm.cpp", 748, 915, ["matrix_Au", "matrix_Av", "matrix_Bu", "matrix_Bv",
                                                             "output_matrix"]),
    ("gemm_test10_ddc", "tests/api/TestGemm.cpp", 917, 1045, ["matrix_A", "matrix_B", "output_matrix"]),
    ("potrf", "tests/kernels/TestKernels.cpp", 1070, 1124, ["matrix_A", "matrix_Output"]),
    ("trsm", "tests/kernels/TestKernels.cpp", 1126, 1184, ["matrix_A", "matrix_B", "matrix_output"]),
    ("syrk_cross_product", "tests/kernels/TestKernels.cpp", 1185, 1250, ["matrix_A", "matrix_B", "matrix_output"]),
]

NUM = re.compile(r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?")


def extract(text_lines, name):
    src = "\n".join(text_lines)
    m = re.search(r"\b" + re.escape(name) + r"\s*((?:\[[^\]]*\])+)\s*=\s*\{", src)
    if not m:
        raise KeyError(name)
    dims = [d.strip() for d in re.findall(r"\[([^\]]*)\]", m.group(1))]
    depth, i = 0, m.end() - 1
    start = i
    while True:
        ch = src[i]
        if ch == "{":
            depth += 1
        elif ch == "}":
            depth -= 1
            if depth == 0:
                break
        i += 1
    body = src[start:i + 1]
    body = re.sub(r"\b(accuracy|sigma_0)\b", lambda mm: mm.group(1), body)
    return dims, body


def numbers(body):
    return [float(x) for x in NUM.findall(body)]


def main(root: str):
    root = Path(root)
    out = {}
    for key, rel, lo, hi, names in SOURCES:
        lines = (root / rel).read_text().splitlines()[lo - 1:hi]
        entry = {"source": f"{rel}:{lo}-{hi}"}
        for name in names:
            dims, body = extract(lines, name)
            entry[name] = {"dims": dims, "values": numbers(body)}
        out[key] = entry
    dest = Path(__file__).with_name("kat.json")
    dest.write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", dest)


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parents[2]))
    from oracle.build_ref import reference_root
    main(reference_root())
