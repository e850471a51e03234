"""Pin the numpy oracle against the reference's own CPU code compiled here (oracle/_ref, built by
oracle/build_ref.py from the reference sources).  Skipped where that library is not built
(the GPU host has no reference sources)."""
import numpy as np
import pytest

from oracle import hcore_oracle as O
from oracle import ref_lib as R
from tests.helpers import rel_fro

pytestmark = pytest.mark.skipif(not R.available(), reason="oracle/_ref not built")


def _pair(kind, d, params):
    if kind == "D":
        return O.DenseTile(d), R.RefTile.dense(d)
    o = O.CompressedTile.from_dense(d, params)
    r = R.compress(d, params)
    assert o.rank == r.rank and o.max_rank == r.max_rank
    np.testing.assert_allclose(o.to_dense(), r.to_dense(), atol=1e-13 * np.abs(d).max())
    return o, r


@pytest.mark.parametrize("combo", ["CCC", "DCC", "CDC", "CCD", "DCD", "CDD", "DDD", "DDC"])
@pytest.mark.parametrize("truncated,acc", [(True, 1e-8), (False, 1e-4)])
def test_oracle_matches_compiled_reference(combo, truncated, acc):
    from hcorepp_gb300.problems import KernelMatrix
    nb = 128
    km = KernelMatrix(4 * nb, nb, 2, 0.1, 1)
    kc = KernelMatrix(4 * nb, nb, 2, 0.1, 2)
    params = O.CompressionParameters(acc, truncated_svd=truncated)
    (oa, ra), (ob, rb), (oc, rc) = (_pair(combo[0], km.tile(0, 1), params), _pair(combo[1], km.tile(1, 2), params),
                                    _pair(combo[2], kc.tile(0, 2), params))
    if combo == "DDC":
        u0, v0 = rc.u(), rc.v()
        rc.max_rank = nb  # the reference re-sizes the tile (HCore.cpp:294-298); give the buffer the room
        buf = np.zeros(2 * nb * nb)
        buf[:rc.rows * rc.rank] = u0.ravel(order="F")
        buf[nb * nb:nb * nb + rc.rank * nb] = v0.ravel(order="F")
        rc.buf = buf
    alpha, beta = 3.5, 2.5
    O.hcore_gemm(alpha, oa, ob, beta, oc, params)
    R.tile_gemm(alpha, ra, rb, beta, rc, params)
    if combo == "DDC":
        # U = alpha A B + beta Cu Cv at full rank; V = I.  A caller-owned buffer keeps its old V
        # entries off the diagonal (ReadjustTile only re-sizes owning holders, DataHolder.cpp:66-83),
        # so the U factor is the comparable part.
        assert rc.rank == oc.rank == nb
        assert rel_fro(oc.u, rc.u()) < 1e-12
        return
    if combo[2] == "C":
        assert oc.rank == rc.rank
    assert rel_fro(oc.to_dense(), rc.to_dense()) < 1e-12


def test_tile_loop_matches_compiled_reference():
    """The omp_main.cpp-style tile loop (OpenMP over C tiles) in the compiled reference vs the oracle."""
    from hcorepp_gb300.problems import build_tiles
    nt, nb, acc = 3, 96, 1e-8
    params = O.CompressionParameters(acc, truncated_svd=True)
    a = build_tiles(nt * nb, nb, 2, 0.1, 1, acc, False, processes=1)
    c = build_tiles(nt * nb, nb, 2, 0.1, 2, acc, False, processes=1)
    def grids(t):
        og = [[O.CompressedTile(t[(i, j)][1], t[(i, j)][2], max_rank=t[(i, j)][3]) for j in range(nt)] for i in range(nt)]
        rg = [[R.RefTile.compressed(t[(i, j)][1], t[(i, j)][2], t[(i, j)][3]) for j in range(nt)] for i in range(nt)]
        return og, rg
    oA, rA = grids(a)
    oB, rB = grids(a)
    oC, rC = grids(c)
    O.tile_matrix_multiply(oA, oB, oC, 1.0, 1.0, params)
    secs, errors = R.tlr_gemm(nt, nb, 1.0, 1.0, rA, rB, rC, params, nthreads=2)
    assert errors == 0
    for i in range(nt):
        for j in range(nt):
            assert oC[i][j].rank == rC[i][j].rank
            assert rel_fro(oC[i][j].to_dense(), rC[i][j].to_dense()) < 1e-12
