"""Shared helpers for the parity tests: seeded tile-low-rank inputs and error measures."""
from __future__ import annotations

import numpy as np

from hcorepp_gb300.problems import KernelMatrix
from oracle import hcore_oracle as O


def rel_fro(a, b) -> float:
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def compressed_from_dense(d, accuracy, truncated=True, max_rank=None):
    """Input compression as the reference's dense constructor (Compressed.cpp:75-146), on the CPU."""
    t = O.CompressedTile.from_dense(d, O.CompressionParameters(accuracy, truncated_svd=truncated))
    if max_rank is not None:
        t.max_rank = max_rank
    return t


def kernel_tiles(n, nb, seed, ell=0.1, d=2):
    km = KernelMatrix(n, nb, d, ell, seed)
    return km


def random_lowrank(m, n, r, rng, decay=0.5):
    q1, _ = np.linalg.qr(rng.standard_normal((m, r)))
    q2, _ = np.linalg.qr(rng.standard_normal((n, r)))
    s = decay ** np.arange(r)
    return (q1 * s) @ q2.T


def oracle_tile_grid(km, nt, acc, dense_diagonal):
    """Oracle tiles of a kernel matrix: dense on the diagonal (if asked), else compressed at `acc`
    relative by the reference's dense constructor rule."""
    grid = [[None] * nt for _ in range(nt)]
    for i in range(nt):
        for j in range(nt):
            d = km.tile(i, j)
            grid[i][j] = O.DenseTile(d) if (dense_diagonal and i == j) else compressed_from_dense(d, acc)
    return grid


def load_tile_matrix(T, L, grid, nb, max_rank):
    """A device TileMatrix holding the oracle tiles of `grid`."""
    mt, nt = len(grid), len(grid[0])
    kinds = [[L.DENSE if grid[i][j].kind == "dense" else L.COMPRESSED for j in range(nt)] for i in range(mt)]
    tm = T.TileMatrix(mt, nt, nb, kinds, max_rank)
    for i in range(mt):
        for j in range(nt):
            t = grid[i][j]
            if t.kind == "dense":
                tm.set_tile(i, j, dense=t.data)
            else:
                tm.set_tile(i, j, u=t.u, v=t.v)
    return tm
