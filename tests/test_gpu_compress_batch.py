"""hcgb_compress_tiles: the batched dense -> compressed construction against the per-tile call
hcgb_compress_tile and against the reference's constructor restated in the oracle
(src/operators/concrete/Compressed.cpp:75-146): per tile, the same rank as the per-tile call and
the oracle's rank +-1, reconstruction error at the oracle's level; the Cholesky-flow layout
(compressed_vt) and a capacity of nb included.
"""
import numpy as np
import pytest

from oracle import hcore_oracle as O
from tests.helpers import rel_fro

pytestmark = pytest.mark.gpu

PAIRS = [(0, 1), (0, 3), (1, 2), (2, 2), (3, 0), (3, 1)]


@pytest.fixture(scope="module")
def T():
    import torch
    from hcorepp_gb300 import tiles
    assert torch.cuda.is_available()
    return tiles


def _dense_device(d):
    import torch
    return torch.from_numpy(np.asfortranarray(d).ravel(order="F")).cuda()


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("acc", [1e-8, 1e-4])
def test_batch_matches_per_tile_call_and_oracle(T, mode, acc):
    from hcorepp_gb300.problems import KernelMatrix
    km = KernelMatrix(1024, 256, 2, 0.1, 4)
    params = T.CompressionParameters(acc, truncated_svd=True, mode=mode)
    dense = [km.tile(i, j) for (i, j) in PAIRS]
    cap = 256 // 3
    outs = [T.CompressedTile(256, 256, rank=0, max_rank=cap) for _ in dense]
    ranks = T.CompressedTile.compress_batch([_dense_device(d) for d in dense], outs, params)
    for (i, j), d, g, r in zip(PAIRS, dense, outs, ranks):
        single = T.CompressedTile.from_dense(d, params)
        o = O.CompressedTile.from_dense(d, O.CompressionParameters(acc, truncated_svd=True))
        assert r == g.rank == single.rank, (i, j, r, g.rank, single.rank)
        assert abs(g.rank - o.rank) <= 1, (i, j, g.rank, o.rank)
        assert rel_fro(g.to_dense(), single.to_dense()) <= 1e-12, (i, j)
        assert rel_fro(g.to_dense(), d) <= 2 * max(rel_fro(o.to_dense(), d), 1e-14), (i, j)


def test_batch_into_cholesky_layout_with_capacity_nb(T):
    """Tiles of a vt TileMatrix (tile = U W^T) with capacity nb: the ranks are not clamped at nb/3."""
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300.problems import KernelMatrix
    nb, nt = 256, 4
    km = KernelMatrix(nb * nt, nb, 3, 0.2, 2, diag_shift=1e-2)
    kinds = [[L.DENSE if i == j else L.COMPRESSED if i > j else None for j in range(nt)] for i in range(nt)]
    tm = T.TileMatrix(nt, nt, nb, kinds, nb, vt=True)
    below = [(i, j) for j in range(nt) for i in range(j + 1, nt)]
    params = T.CompressionParameters(1e-8, truncated_svd=True)
    ranks = T.CompressedTile.compress_batch([_dense_device(km.tile(i, j)) for (i, j) in below],
                                            [tm.tile(i, j) for (i, j) in below], params)
    full = tm.to_dense()
    for (i, j), r in zip(below, ranks):
        d = km.tile(i, j)
        ref = O.CompressedTile.from_dense(d, O.CompressionParameters(1e-8, truncated_svd=True), max_rank=nb)
        assert abs(r - ref.rank) <= 1, (i, j, r, ref.rank)
        blk = full[i * nb:(i + 1) * nb, j * nb:(j + 1) * nb]
        assert rel_fro(blk, d) <= 2 * max(rel_fro(ref.to_dense(), d), 1e-14), (i, j)
    assert max(ranks) > nb // 3  # the neighbouring tiles of this kernel need more than the reference's clamp


def test_batch_rejects_mismatched_tiles(T):
    import torch
    params = T.CompressionParameters(1e-8, truncated_svd=True)
    d = torch.zeros(128 * 128, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        T.CompressedTile.compress_batch([d], [T.CompressedTile(128, 64, rank=0, max_rank=8)], params)
    with pytest.raises(ValueError):
        T.CompressedTile.compress_batch([d, d], [T.CompressedTile(128, 128, rank=0, max_rank=8)], params)
