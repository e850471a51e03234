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
