"""Calibration of the CPU port against the reference's own compiled CPU path (oracle/_ref).

    python -m oracle.calibrate_port [--tiles 64] [--out oracle/port_calibration.json]

The bench's CPU baseline on the GPU host is the numpy port (oracle/cpu_baseline.py): the reference's
sources are not on that host, so its compiled CPU path cannot be built there.  This script runs both
on the machine where oracle/_ref was built, on the same cores and the same seeded sample of C tiles of
the 32 x 32-tile multiply (n = 16384, nb = 512, 1e-8 relative, dense diagonal), each C tile with its
full k-chain in ascending k (examples/matrix_multiplication/omp_main.cpp:112-124), and records both
rates, their ratio and whether the final ranks agree.  TEST / BASELINE INFRASTRUCTURE ONLY.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import time

import numpy as np

from . import cpu_baseline, ref_lib
from . import hcore_oracle as O


def _ref_grid(tiles, nt):
    grid = [[None] * nt for _ in range(nt)]
    for (i, j), t in tiles.items():
        grid[i][j] = ref_lib.RefTile.dense(t[1]) if t[0] == "D" else ref_lib.RefTile.compressed(t[1], t[2], t[3])
    return grid


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--tiles", type=int, default=64)
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)), "port_calibration.json"))
    args = ap.parse_args()
    if not ref_lib.available():
        raise SystemExit("oracle/_ref/libhcref.so is not built on this machine (python oracle/build_ref.py)")
    from hcorepp_gb300.problems import WORKLOADS, build_tiles
    name = "tlr_gemm_n16384_nb512"
    w = WORKLOADS[name]
    cores = os.cpu_count() or 1
    t0 = time.time()
    a = build_tiles(w["n"], w["nb"], w["d"], w["ell"], w["seed_ab"], w["accuracy"], w["dense_diagonal"], cores)
    c = build_tiles(w["n"], w["nb"], w["d"], w["ell"], w["seed_c"], w["accuracy"], w["dense_diagonal"], cores)
    build_s = time.time() - t0
    nt = w["n"] // w["nb"]
    sample = cpu_baseline.sample_tiles(nt, args.tiles)
    params = O.CompressionParameters(w["accuracy"], truncated_svd=True)

    port_results = {}
    port_updates, port_wall = cpu_baseline.run(a, a, c, params, sample, cores, port_results)

    ag, cg = _ref_grid(a, nt), _ref_grid(c, nt)
    c_list = [i + j * nt for (i, j) in sample]
    ref_wall, errors = ref_lib.tlr_gemm(nt, w["nb"], 1.0, 1.0, ag, ag, cg, params, c_list=c_list, nthreads=cores)
    ref_updates = len(sample) * nt

    rank_diff = []
    for (i, j) in sample:
        fin = port_results[(i, j)]["final"]
        port_rank = 0 if fin[0] == "D" else fin[1].shape[1]
        ref_rank = 0 if cg[i][j].kind == 0 else cg[i][j].rank
        rank_diff.append(abs(port_rank - ref_rank))
    out = {
        "machine": platform.machine(), "cores": cores, "workload": name,
        "sample": f"{len(sample)} seeded C tiles x {nt} k-updates = {ref_updates} updates",
        "port_updates_per_s": port_updates / port_wall, "reference_updates_per_s": ref_updates / ref_wall,
        "port_over_reference": (port_updates / port_wall) / (ref_updates / ref_wall),
        "reference_errors": errors, "final_rank_max_abs_diff": int(max(rank_diff)) if rank_diff else 0,
        "input_build_seconds": build_s,
        "note": "both with one BLAS thread per worker and one worker per core; the port in spawned processes, "
                "the reference in OpenMP threads (its driver's own parallelisation)",
    }
    with open(args.out, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
