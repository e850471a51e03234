"""Synthetic tile-low-rank test matrices: Morton-sorted exponential kernels.

The reference publishes no dataset for its TLR multiply; its drivers build
matrices from LAPACK generators (src/helpers/generators/TileLatmsGenerator.cpp:31-94)
and split them into tiles (src/helpers/TileMatrix.cpp:17-185).  The workloads
measured here use the kernel-matrix family that tile-low-rank codes are built
for instead:

* points ``x_i`` drawn uniformly from ``[0, 1]^d`` with numpy's PCG64 generator
  (``numpy.random.default_rng(seed)``),
* sorted along a Morton (Z-order) curve: each coordinate is quantised to 21 bits
  and the bits are interleaved, coordinate 0 in the lowest bit,
* ``a_ij = exp(-||x_i - x_j||_2 / ell)`` (+ ``diag_shift`` on the diagonal).

Everything here is host-side input preparation; the same arrays feed the GPU
path and the CPU oracle.
"""
from __future__ import annotations

import os

import numpy as np

MORTON_BITS = 21


def morton_codes(x: np.ndarray) -> np.ndarray:
    """Morton code of every point (rows of ``x``), 21 bits per coordinate."""
    n, d = x.shape
    if d * MORTON_BITS > 64:
        raise ValueError("Morton codes support at most 3 coordinates")
    scale = float(1 << MORTON_BITS)
    q = np.minimum((x * scale).astype(np.uint64), np.uint64((1 << MORTON_BITS) - 1))
    code = np.zeros(n, dtype=np.uint64)
    for b in range(MORTON_BITS):
        for c in range(d):
            bit = (q[:, c] >> np.uint64(b)) & np.uint64(1)
            code |= bit << np.uint64(b * d + c)
    return code


def morton_points(n: int, d: int, seed: int) -> np.ndarray:
    """``n`` uniform points in ``[0,1]^d`` from ``seed``, in Morton order."""
    rng = np.random.default_rng(seed)
    x = rng.random((n, d))
    order = np.argsort(morton_codes(x), kind="stable")
    return np.ascontiguousarray(x[order])


def kernel_block(xr: np.ndarray, xc: np.ndarray, ell: float, diag_shift: float = 0.0,
                 same_block: bool = False) -> np.ndarray:
    """Dense block ``exp(-|x_r - x_c| / ell)`` in column-major (Fortran) order."""
    diff = xr[:, None, :] - xc[None, :, :]
    dist = np.sqrt(np.einsum("ijk,ijk->ij", diff, diff))
    a = np.exp(-dist / ell)
    if same_block and diag_shift:
        a[np.diag_indices_from(a)] += diag_shift
    return np.asfortranarray(a)


class KernelMatrix:
    """Lazily tiled exponential-kernel matrix on Morton-sorted points."""

    def __init__(self, n: int, nb: int, d: int, ell: float, seed: int, diag_shift: float = 0.0):
        if n % nb:
            raise ValueError("n must be a multiple of the tile size")
        self.n, self.nb, self.d, self.ell, self.seed = n, nb, d, ell, seed
        self.diag_shift = diag_shift
        self.nt = n // nb
        self.points = morton_points(n, d, seed)

    def tile(self, i: int, j: int) -> np.ndarray:
        nb = self.nb
        xr = self.points[i * nb:(i + 1) * nb]
        xc = self.points[j * nb:(j + 1) * nb]
        return kernel_block(xr, xc, self.ell, self.diag_shift, same_block=(i == j))

    def dense(self) -> np.ndarray:
        return kernel_block(self.points, self.points, self.ell, self.diag_shift, same_block=True)


# Workloads named by what they are (sizes and generator parameters).
WORKLOADS = {
    # 4x4 tiles of 512, every tile compressed (diagonals included), accuracy 1e-8 relative.
    "tlr_gemm_n2048_nb512": dict(n=2048, nb=512, d=2, ell=0.1, seed_ab=1, seed_c=2,
                                 accuracy=1e-8, dense_diagonal=False),
    # 8x8 tiles of 512, dense diagonal tiles: a profiling-size case (inputs above L2, < 1 GB on device).
    "tlr_gemm_n4096_nb512": dict(n=4096, nb=512, d=2, ell=0.1, seed_ab=1, seed_c=2,
                                 accuracy=1e-8, dense_diagonal=True),
    # 32x32 tiles of 512, dense diagonal tiles, accuracy 1e-8 relative: 32^3 tile updates.
    "tlr_gemm_n16384_nb512": dict(n=16384, nb=512, d=2, ell=0.1, seed_ab=1, seed_c=2,
                                  accuracy=1e-8, dense_diagonal=True),
}


# ---------------------------------------------------------------------------------------
# Host-side input compression of the workload tiles (workload preparation, not the measured
# multiply).  Same rule as CompressedTile(dense, params) (src/operators/concrete/Compressed.cpp:
# 75-146): SVD, rank = first i >= 1 with sigma_i below the threshold (relative to sigma_0 when
# truncated), clamped to [1, max(min(m, n) / 3, 1)], V = Sigma_r V_r^T.
# ---------------------------------------------------------------------------------------

def compress_dense(d: np.ndarray, accuracy: float, truncated: bool = True, max_rank: int | None = None):
    m, n = d.shape
    cap = max(min(m, n) // 3, 1) if max_rank is None else max_rank
    u, s, vt = np.linalg.svd(d, full_matrices=False)
    thr = accuracy * s[0] if truncated else accuracy
    small = np.nonzero(s[1:] < thr)[0]
    r = int(small[0]) + 1 if small.size else len(s)
    r = min(max(r, 1), cap)
    return np.asfortranarray(u[:, :r]), np.asfortranarray(s[:r, None] * vt[:r]), cap


def _tile_job(args):
    n, nb, d, ell, seed, diag_shift, i, j, accuracy, dense, max_rank = args
    km = _cached_matrix(n, nb, d, ell, seed, diag_shift)
    blk = km.tile(i, j)
    if dense:
        return (i, j), ("D", blk)
    u, v, cap = compress_dense(blk, accuracy, True, max_rank)
    return (i, j), ("C", u, v, cap)


_KM_CACHE = {}


def _cached_matrix(n, nb, d, ell, seed, diag_shift):
    key = (n, nb, d, ell, seed, diag_shift)
    if key not in _KM_CACHE:
        _KM_CACHE[key] = KernelMatrix(n, nb, d, ell, seed, diag_shift)
    return _KM_CACHE[key]


def build_tiles(n, nb, d, ell, seed, accuracy, dense_diagonal, processes=None, diag_shift=0.0,
                lower_only=False, max_rank=None):
    """All tiles of one matrix (or those with i >= j): dict (i, j) -> ("D", dense) | ("C", u, v,
    max_rank); compressed tiles get capacity max_rank (default the reference's min(m, n) / 3)."""
    import multiprocessing as mp
    nt = n // nb
    jobs = [(n, nb, d, ell, seed, diag_shift, i, j, accuracy, dense_diagonal and i == j, max_rank)
            for j in range(nt) for i in range(nt) if i >= j or not lower_only]
    processes = processes or max(1, min(len(jobs), os.cpu_count() or 1))
    if processes == 1:
        return dict(_tile_job(j) for j in jobs)
    with single_threaded_blas_env(), mp.get_context("spawn").Pool(processes) as pool:
        return dict(pool.map(_tile_job, jobs, chunksize=max(1, len(jobs) // (4 * processes))))


class single_threaded_blas_env:
    """Spawned worker processes inherit one BLAS thread each (no oversubscription)."""
    KEYS = ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")

    def __enter__(self):
        self.saved = {k: os.environ.get(k) for k in self.KEYS}
        for k in self.KEYS:
            os.environ[k] = "1"
        return self

    def __exit__(self, *exc):
        for k, v in self.saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
        return False
