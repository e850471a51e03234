"""CPU baseline for the TLR multiply: the oracle port (numpy + the host's LAPACK) timed on the
host cores over a bounded, seeded sample of C tiles, each with its full k-chain of updates,
in the style of examples/matrix_multiplication/omp_main.cpp:112-124 (C tiles in parallel, k
sequential per tile, one BLAS thread per worker).

TEST / BASELINE INFRASTRUCTURE ONLY: used by bench.py's cpu_baseline leg and its
``--impl reference`` arm; never by the product.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import time

import numpy as np

_STATE = {}


def _worker_init(a_tiles, b_tiles, c_tiles, params):
    _STATE.update(a=a_tiles, b=b_tiles, c=c_tiles, params=params)


def _to_oracle(t):
    from oracle import hcore_oracle as O
    if t[0] == "D":
        return O.DenseTile(t[1])
    return O.CompressedTile(t[1], t[2], max_rank=t[3])


def _run_chain(ij):
    """One C tile's k-chain in ascending k.  Returns the update count, the chain's time, the rank
    after every update and the final tile (U, V; or the dense tile), the last two for the parity
    check of the GPU result (gathered after the chain, outside its time)."""
    from oracle import hcore_oracle as O
    i, j = ij
    a, b, c, p = _STATE["a"], _STATE["b"], _STATE["c"], _STATE["params"]
    nt = int(round(len(b) ** 0.5))
    ct = _to_oracle(c[(i, j)])
    ranks = []
    t0 = time.monotonic()  # system-wide clock: comparable across the pool's processes
    for k in range(nt):
        info = O.hcore_gemm(1.0, _to_oracle(a[(i, k)]), _to_oracle(b[(k, j)]), 1.0, ct, p)
        ranks.append(info.get("rank"))
    t1 = time.monotonic()
    final = ("D", ct.data) if ct.kind == "dense" else ("C", ct.u, ct.v)
    return nt, (t0, t1), ranks, final


def _ping(_):
    from oracle import hcore_oracle  # noqa: F401  (import LAPACK bindings before timing)
    time.sleep(0.05)
    return os.getpid()


def sample_tiles(nt: int, count: int, seed: int = 1234):
    rng = np.random.default_rng(seed)
    idx = rng.choice(nt * nt, size=min(count, nt * nt), replace=False)
    return [(int(x) % nt, int(x) // nt) for x in idx]


def run(a_tiles, b_tiles, c_tiles, params, sample, processes: int, results: dict | None = None):
    """Returns (updates, wall seconds).  Tiles: dict (i, j) -> ("D", dense) | ("C", u, v, max_rank).
    If `results` is given it receives, per sampled C tile (i, j), the oracle's rank after every
    update (k ascending) and its final tile."""
    # Only ship the tiles the sample touches.
    nt = int(round(len(b_tiles) ** 0.5))
    rows = sorted({i for i, _ in sample})
    cols = sorted({j for _, j in sample})
    a_sub = {(i, k): a_tiles[(i, k)] for i in rows for k in range(nt)}
    c_sub = {ij: c_tiles[ij] for ij in sample}
    b_sub = {(k, j): b_tiles[(k, j)] for k in range(nt) for j in cols}
    # pad b_sub to nt*nt keys' worth of size information
    b_full = dict(b_sub)
    for k in range(nt):
        for j in range(nt):
            b_full.setdefault((k, j), None)
    from hcorepp_gb300.problems import single_threaded_blas_env
    ctx = mp.get_context("spawn")
    with single_threaded_blas_env(), ctx.Pool(processes=processes, initializer=_worker_init,
                                              initargs=(a_sub, b_full, c_sub, params)) as pool:
        pool.map(_ping, range(processes * 2), chunksize=1)
        out = pool.map(_run_chain, sample, chunksize=1)
    # Wall time of the sample: first chain start to last chain end (the results' transfer back to
    # this process is not part of it).
    wall = max(o[1][1] for o in out) - min(o[1][0] for o in out)
    if results is not None:
        for ij, o in zip(sample, out):
            results[ij] = {"ranks": o[2], "final": o[3]}
    return sum(o[0] for o in out), wall
