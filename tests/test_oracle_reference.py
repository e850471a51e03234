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


def _chol_pair(nb, rank, rng, max_rank):
    """The same low-rank tile as an oracle CholeskyTile and a reference buffer holding (U, W)."""
    u = rng.standard_normal((nb, rank)) * 0.5 ** np.arange(rank)
    w = rng.standard_normal((nb, rank))
    return O.CholeskyTile(u, w, max_rank), R.RefTile.cholesky(u, w, max_rank)


@pytest.mark.parametrize("nb,ra,rb,rc", [(60, 7, 9, 5), (96, 20, 12, 0), (128, 30, 30, 30)])
def test_cholesky_gemm_branch_matches_compiled_reference(nb, ra, rb, rc):
    """Gemm(alpha, A, NoTrans, B, Trans, beta, C, aCholesky = true) on compressed A, B, C
    (HCore.cpp:160-174, Compressed.cpp:273-276, :529-595): C = alpha A B^T + beta C with every V
    factor stored as W = V^T."""
    rng = np.random.default_rng(nb + ra)
    mr = nb // 3
    params = O.CompressionParameters(1e-8, truncated_svd=True)
    oa, ra_ = _chol_pair(nb, ra, rng, mr)
    ob, rb_ = _chol_pair(nb, rb, rng, mr)
    oc, rc_ = _chol_pair(nb, max(rc, 1), rng, mr)
    if rc == 0:
        oc.u, oc.w = oc.u[:, :0], oc.w[:, :0]
        rc_.rank = 0
    want = -1.0 * oa.to_dense() @ ob.to_dense().T + 0.5 * oc.to_dense()
    O.hcore_gemm_cholesky(-1.0, oa, ob, 0.5, oc, params)
    R.tile_gemm_ops(-1.0, ra_, 0, rb_, 1, 0.5, rc_, params, cholesky=True)
    got_ref = rc_.u() @ rc_.w().T
    assert abs(rc_.rank - oc.rank) <= 1
    assert rel_fro(got_ref, want) < 1e-7
    assert rel_fro(oc.to_dense(), got_ref) < 1e-7


def test_cholesky_tile_ops_match_compiled_reference():
    """Potrf, Trsm (on W) and Syrk (compressed and dense A) of the oracle against HCore++'s own."""
    rng = np.random.default_rng(11)
    nb = 80
    g = rng.standard_normal((nb, nb))
    spd = g @ g.T + nb * np.eye(nb)
    a = R.RefTile.dense(spd)
    R.potrf(0, a)
    lo, info = O.potrf_lower(spd)
    assert info == 0
    np.testing.assert_allclose(np.tril(a.to_dense()), np.tril(lo), rtol=1e-12, atol=1e-12)
    lkk = np.tril(lo)
    for side, uplo, trans in [(0, 0, 0), (0, 0, 1), (0, 1, 0), (1, 0, 1)]:
        ob, rb = _chol_pair(nb, 9, rng, nb // 3)
        tri = lkk if uplo == 0 else lkk.T
        R.trsm(side, uplo, trans, 0, 1.5, R.RefTile.dense(tri), rb)
        O.hcore_trsm_compressed(side == 0, uplo == 0, trans == 1, False, 1.5, tri, ob)
        np.testing.assert_allclose(rb.w(), ob.w, rtol=1e-10, atol=1e-12)
    oa, ra_ = _chol_pair(nb, 11, rng, nb // 3)
    c0 = rng.standard_normal((nb, nb))
    for uplo in (0, 1):
        rc = R.RefTile.dense(c0)
        oc = O.DenseTile(c0.copy())
        R.syrk(-1.0, ra_, 0, uplo, 0.75, rc)
        O.hcore_syrk(-1.0, oa, uplo == 0, 0.75, oc)
        np.testing.assert_allclose(rc.to_dense(), oc.data, rtol=1e-11, atol=1e-11)
    d = rng.standard_normal((nb, nb))
    for uplo in (0, 1):
        rc = R.RefTile.dense(c0)
        oc = O.DenseTile(c0.copy())
        R.syrk(0.5, R.RefTile.dense(d), 0, uplo, 2.0, rc)
        O.hcore_syrk(0.5, O.DenseTile(d), uplo == 0, 2.0, oc)
        np.testing.assert_allclose(rc.to_dense(), oc.data, rtol=1e-11, atol=1e-11)


def test_tile_cholesky_matches_reference_composition():
    """The oracle's tile-Cholesky driver against the same loop run on HCore++'s own Potrf, Trsm, Syrk
    and Gemm(aCholesky = true), on an SPD exponential-kernel matrix (2-D points, length scale 0.1,
    +1e-2 on the diagonal, 3 x 3 tiles of 96, off-diagonal tiles compressed at 1e-4 relative so that
    no rank reaches the capacity nb/3)."""
    from hcorepp_gb300.problems import KernelMatrix
    nt, nb, acc = 3, 96, 1e-4
    km = KernelMatrix(nt * nb, nb, 2, 0.1, 4, diag_shift=1e-2)
    params = O.CompressionParameters(acc, truncated_svd=True)
    og = [[None] * nt for _ in range(nt)]
    rg = [[None] * nt for _ in range(nt)]
    for i in range(nt):
        for j in range(i + 1):
            blk = km.tile(i, j)
            if i == j:
                og[i][j], rg[i][j] = O.DenseTile(blk.copy()), R.RefTile.dense(blk)
            else:
                t = O.CompressedTile.from_dense(blk, params)
                og[i][j] = O.CholeskyTile(t.u, t.v.T, t.max_rank)
                rg[i][j] = R.RefTile.cholesky(t.u, t.v.T, t.max_rank)
    assert O.tile_cholesky(og, nt, params) == 0
    for k in range(nt):
        R.potrf(0, rg[k][k])
        lkk = R.RefTile.dense(np.tril(rg[k][k].to_dense()))
        for i in range(k + 1, nt):
            R.trsm(0, 0, 0, 0, 1.0, lkk, rg[i][k])
        for i in range(k + 1, nt):
            R.syrk(-1.0, rg[i][k], 0, 0, 1.0, rg[i][i])
            for j in range(k + 1, i):
                R.tile_gemm_ops(-1.0, rg[i][k], 0, rg[j][k], 1, 1.0, rg[i][j], params, cholesky=True)
    a = km.dense()
    for name, get in (("oracle", lambda i, j: og[i][j].to_dense()),
                      ("reference", lambda i, j: rg[i][j].u() @ rg[i][j].w().T if i != j else rg[i][j].to_dense())):
        lf = np.zeros_like(a)
        for i in range(nt):
            for j in range(i + 1):
                blk = get(i, j)
                lf[i * nb:(i + 1) * nb, j * nb:(j + 1) * nb] = np.tril(blk) if i == j else blk
        if name == "oracle":
            l_oracle = lf
        else:
            assert rel_fro(lf, l_oracle) < 1e-9
        assert rel_fro(lf @ lf.T, a) < 10 * acc, name
