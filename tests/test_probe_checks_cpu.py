"""The tile-by-tile products behind the probe-based accuracy checks of the large benchmarks
(hcorepp_gb300/learned_bench.py: ||C X - (A (A X) + C0 X)||; the factor views they read), on the CPU
with small tile matrices: the tile-by-tile product of a tile matrix (dense and compressed tiles,
both V layouts) with a block of vectors equals the dense matrix's product."""
import numpy as np
import pytest
import torch

from hcorepp_gb300 import _lib as L
from hcorepp_gb300 import tiles as T


def _random_tile_matrix(mt, nt, nb, cap, seed, vt=False):
    rng = np.random.default_rng(seed)
    kinds = [[L.DENSE if (i + j) % 3 == 0 else L.COMPRESSED for j in range(nt)] for i in range(mt)]
    tm = T.TileMatrix(mt, nt, nb, kinds, cap, device="cpu", vt=vt)
    for i in range(mt):
        for j in range(nt):
            if kinds[i][j] == L.DENSE:
                tm.set_tile(i, j, dense=rng.standard_normal((nb, nb)))
            else:
                r = int(rng.integers(1, cap + 1))
                tm.set_tile(i, j, u=rng.standard_normal((nb, r)), v=rng.standard_normal((r, nb)))
                tm.ranks[tm.index(i, j)] = r
    return tm


def test_apply_tlr_matches_the_dense_product():
    from hcorepp_gb300.learned_bench import apply_tlr
    tm = _random_tile_matrix(3, 4, 16, 5, 1)
    x = torch.from_numpy(np.random.default_rng(2).standard_normal((4 * 16, 3)))
    got = apply_tlr(tm, x).numpy()
    want = tm.to_dense() @ x.numpy()
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())


def test_tile_factors_views_match_the_stored_tiles():
    from hcorepp_gb300.learned_bench import tile_factors
    tm = _random_tile_matrix(2, 2, 8, 3, 3)
    dense = tm.to_dense()
    for (i, j), t in tile_factors(tm).items():
        blk = (t[0] @ t[1]) if isinstance(t, tuple) else t
        np.testing.assert_allclose(blk.numpy(), dense[i * 8:(i + 1) * 8, j * 8:(j + 1) * 8], rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("vt", [False, True])
def test_unstored_tiles_hold_no_storage(vt):
    """A kind of None (the upper triangle of a Cholesky factor) takes no arena space and reads as zero."""
    nt, nb = 3, 8
    kinds = [[L.DENSE if i == j else L.COMPRESSED if i > j else None for j in range(nt)] for i in range(nt)]
    tm = T.TileMatrix(nt, nt, nb, kinds, 2, device="cpu", vt=vt)
    assert tm.arena.numel() == 3 * nb * nb + 3 * 2 * nb * 2
    assert not tm.to_dense()[0:nb, nb:].any()
    with pytest.raises(ValueError):
        tm.tile(0, 1)
