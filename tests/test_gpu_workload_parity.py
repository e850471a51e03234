"""GPU parity at the benchmark workloads' own sizes (nb = 512), per update.

* The 4 x 4-tile multiply (n = 2048, nb = 512; Morton-sorted 2-D points, exponential kernel with
  length scale 0.1; A = B from seed 1, C from seed 2; every tile, the diagonal included,
  compressed at 1e-8 relative; alpha = beta = 1), run through hcgb_tlr_gemm in the reference
  driver's k order (examples/matrix_multiplication/omp_main.cpp:112-124) and through the oracle's
  tile loop: after EVERY one of the 64 updates the new rank is within +-1 of the oracle's
  (the rank rule, src/operators/concrete/Compressed.cpp:509-527), and every C tile's relative
  Frobenius error against the exact product of the compressed inputs is within
  2 x max(oracle's error, accuracy).
* The heaviest k-chain of the 32 x 32-tile workload (n = 16384, nb = 512, dense diagonal): C tile
  (13, 12), 32 updates whose stacks reach 216 columns, the same per-update bar.

Both arithmetic forms (plain FP64 and the float-float mixed form) are held to the same bar.
"""
import numpy as np
import pytest

from oracle import hcore_oracle as O
from tests.helpers import rel_fro

pytestmark = pytest.mark.gpu

ACC = 1e-8


@pytest.fixture(scope="module")
def T():
    import torch
    from hcorepp_gb300 import tiles
    assert torch.cuda.is_available()
    return tiles


def _oracle_tile(km, i, j, dense):
    d = km.tile(i, j)
    if dense:
        return O.DenseTile(d)
    return O.CompressedTile.from_dense(d, O.CompressionParameters(ACC, truncated_svd=True))


def _load(T, L, otiles, mt, nt, nb, maxr):
    kinds = [[L.DENSE if otiles[i][j].kind == "dense" else L.COMPRESSED for j in range(nt)] for i in range(mt)]
    tm = T.TileMatrix(mt, nt, nb, kinds, maxr)
    for i in range(mt):
        for j in range(nt):
            t = otiles[i][j]
            if t.kind == "dense":
                tm.set_tile(i, j, dense=t.data)
            else:
                tm.set_tile(i, j, u=t.u, v=t.v)
    return tm


def _run(T, L, a, b, c, mode, n_updates):
    import torch
    info = T.info_buffer(n_updates)
    ctx = T.run_context()
    ctx.set_k_order(0)  # the reference driver's ascending k
    T.tlr_gemm(1.0, a, b, 1.0, c, T.CompressionParameters(ACC, truncated_svd=True, mode=mode), info)
    torch.cuda.synchronize()
    return info.cpu().numpy()


def _check_chain(info, stats, mt, nt):
    """Per update: status OK and the new rank within 1 of the oracle's after the same update."""
    bad = []
    for (i, j, k, _kk, rank, _cl) in stats:
        rec = info[k * mt * nt + i + j * mt]
        assert rec[0] == 0, (i, j, k, rec)
        if abs(int(rec[5]) - int(rank)) > 1:
            bad.append((i, j, k, int(rec[5]), int(rank)))
    assert not bad, bad
    return len(stats)


@pytest.mark.parametrize("mode", [0, 1])
def test_n2048_nb512_all_compressed_per_update_vs_oracle(T, mode):
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300.problems import KernelMatrix
    nt, nb = 4, 512
    maxr = nb // 3
    ka = KernelMatrix(nt * nb, nb, 2, 0.1, 1)
    kc = KernelMatrix(nt * nb, nb, 2, 0.1, 2)
    oa = [[_oracle_tile(ka, i, j, False) for j in range(nt)] for i in range(nt)]
    oc = [[_oracle_tile(kc, i, j, False) for j in range(nt)] for i in range(nt)]
    A = _load(T, L, oa, nt, nt, nb, maxr)
    C = _load(T, L, oc, nt, nt, nb, maxr)
    a_dense = np.block([[t.to_dense() for t in row] for row in oa])
    c_dense = np.block([[t.to_dense() for t in row] for row in oc])
    exact = a_dense @ a_dense + c_dense
    info = _run(T, L, A, A, C, mode, nt ** 3)
    stats = O.tile_matrix_multiply(oa, oa, oc, 1.0, 1.0, O.CompressionParameters(ACC, truncated_svd=True))
    assert _check_chain(info, stats, nt, nt) == 64
    g = C.to_dense()
    for i in range(nt):
        for j in range(nt):
            sl = (slice(i * nb, (i + 1) * nb), slice(j * nb, (j + 1) * nb))
            e_o = rel_fro(oc[i][j].to_dense(), exact[sl])
            e_g = rel_fro(g[sl], exact[sl])
            assert e_g <= 2 * max(e_o, ACC), (i, j, e_g, e_o)
    o_dense = np.block([[t.to_dense() for t in row] for row in oc])
    assert rel_fro(g, exact) <= 2 * max(rel_fro(o_dense, exact), ACC)


@pytest.mark.parametrize("mode", [0, 1])
def test_widest_chain_n16384_nb512_per_update_vs_oracle(T, mode):
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300.problems import KernelMatrix
    nb, kt, ci, cj = 512, 32, 13, 12
    maxr = nb // 3
    ka = KernelMatrix(kt * nb, nb, 2, 0.1, 1)
    kc = KernelMatrix(kt * nb, nb, 2, 0.1, 2)
    arow = [[_oracle_tile(ka, ci, k, k == ci) for k in range(kt)]]
    bcol = [[_oracle_tile(ka, k, cj, k == cj)] for k in range(kt)]
    oc = [[_oracle_tile(kc, ci, cj, False)]]
    A = _load(T, L, arow, 1, kt, nb, maxr)
    B = _load(T, L, bcol, kt, 1, nb, maxr)
    C = _load(T, L, oc, 1, 1, nb, maxr)
    exact = oc[0][0].to_dense() + sum(arow[0][k].to_dense() @ bcol[k][0].to_dense() for k in range(kt))
    info = _run(T, L, A, B, C, mode, kt)
    stats = O.tile_matrix_multiply(arow, bcol, oc, 1.0, 1.0, O.CompressionParameters(ACC, truncated_svd=True))
    assert _check_chain(info, stats, 1, 1) == kt
    assert int(info[:, 4].max()) >= 200  # the stacks this chain recompresses are this wide
    e_o = rel_fro(oc[0][0].to_dense(), exact)
    assert rel_fro(C.to_dense(), exact) <= 2 * max(e_o, ACC)
