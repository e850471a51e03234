"""Incremental recompression (tests/incremental_model.py) against the oracle's restatement of the
reference's algorithm along whole k-chains of the 8 x 8-tile workload (n = 4096, nb = 512,
1e-8 relative): the same rank after every update, the same product error, U orthonormal and V's
rows orthogonal to working precision at the end of each chain.  CPU only."""
import numpy as np

from hcorepp_gb300.problems import WORKLOADS, build_tiles
from oracle import hcore_oracle as O
from tests.incremental_model import incremental_update, operands


def _tile(t):
    if t[0] == "D":
        return O.DenseTile(np.asfortranarray(t[1]))
    return O.CompressedTile(t[1], t[2], max_rank=t[3])


def test_incremental_matches_reference_along_chains():
    w = WORKLOADS["tlr_gemm_n4096_nb512"]
    a_t = build_tiles(w["n"], w["nb"], w["d"], w["ell"], w["seed_ab"], w["accuracy"], w["dense_diagonal"])
    c_t = build_tiles(w["n"], w["nb"], w["d"], w["ell"], w["seed_c"], w["accuracy"], w["dense_diagonal"])
    nt = w["n"] // w["nb"]
    params = O.CompressionParameters(w["accuracy"], truncated_svd=True)
    for (ti, tj) in [(1, 0), (3, 4), (0, 7), (6, 2)]:
        ref = _tile(c_t[(ti, tj)])
        u, v = ref.u.copy(), ref.v.copy()
        exact = ref.to_dense().copy()
        for kx in range(nt):
            a, b = _tile(a_t[(ti, kx)]), _tile(a_t[(kx, tj)])
            exact += (a.to_dense() if a.kind == "compressed" else a.data) @ \
                (b.to_dense() if b.kind == "compressed" else b.data)
            O.hcore_gemm(1.0, a, b, 1.0, ref, params)
            left, right = operands(a, b)
            u, v, rk = incremental_update(u, v, left, right, 1.0, 1.0, w["accuracy"], ref.max_rank)
            assert rk == ref.rank, ((ti, tj), kx, rk, ref.rank)
        nrm = np.linalg.norm(exact)
        e_ref = np.linalg.norm(ref.to_dense() - exact) / nrm
        e_inc = np.linalg.norm(u @ v - exact) / nrm
        assert e_inc <= 1.01 * e_ref + 1e-12, ((ti, tj), e_inc, e_ref)
        assert np.linalg.norm(u.T @ u - np.eye(u.shape[1])) < 1e-10  # Frobenius, ranks up to ~150
        vv = v @ v.T
        off = np.abs(vv - np.diag(np.diag(vv))) / np.sqrt(np.outer(np.diag(vv), np.diag(vv)))
        assert off.max() < 1e-10


def test_incremental_with_the_core_kernels_jacobi():
    """The same with the core kernel's SVD (pivoted QR stopped at 1e-2 x threshold, one-sided
    Jacobi on R^T) and the rotations accumulated for orthonormal left vectors: ranks within 1 of
    the reference's, error within 1 %, U orthonormal to working precision."""
    w = WORKLOADS["tlr_gemm_n4096_nb512"]
    a_t = build_tiles(w["n"], w["nb"], w["d"], w["ell"], w["seed_ab"], w["accuracy"], w["dense_diagonal"])
    c_t = build_tiles(w["n"], w["nb"], w["d"], w["ell"], w["seed_c"], w["accuracy"], w["dense_diagonal"])
    nt = w["n"] // w["nb"]
    params = O.CompressionParameters(w["accuracy"], truncated_svd=True)
    for (ti, tj) in [(1, 0), (0, 7)]:
        ref = _tile(c_t[(ti, tj)])
        u, v = ref.u.copy(), ref.v.copy()
        exact = ref.to_dense().copy()
        for kx in range(nt):
            a, b = _tile(a_t[(ti, kx)]), _tile(a_t[(kx, tj)])
            exact += (a.to_dense() if a.kind == "compressed" else a.data) @ \
                (b.to_dense() if b.kind == "compressed" else b.data)
            O.hcore_gemm(1.0, a, b, 1.0, ref, params)
            left, right = operands(a, b)
            u, v, rk = incremental_update(u, v, left, right, 1.0, 1.0, w["accuracy"], ref.max_rank, core="jacobi")
            assert abs(rk - ref.rank) <= 1, ((ti, tj), kx, rk, ref.rank)
        nrm = np.linalg.norm(exact)
        e_ref = np.linalg.norm(ref.to_dense() - exact) / nrm
        e_inc = np.linalg.norm(u @ v - exact) / nrm
        assert e_inc <= 1.01 * e_ref + 1e-12, ((ti, tj), e_inc, e_ref)
        assert np.linalg.norm(u.T @ u - np.eye(u.shape[1])) < 1e-10  # Frobenius, ranks up to ~150
        vv = v @ v.T
        off = np.abs(vv - np.diag(np.diag(vv))) / np.sqrt(np.outer(np.diag(vv), np.diag(vv)))
        assert off.max() < 1e-10
