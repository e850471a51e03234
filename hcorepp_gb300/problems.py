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
    # 32x32 tiles of 512, dense diagonal tiles, accuracy 1e-8 relative: 32^3 tile updates.
    "tlr_gemm_n16384_nb512": dict(n=16384, nb=512, d=2, ell=0.1, seed_ab=1, seed_c=2,
                                  accuracy=1e-8, dense_diagonal=True),
}
