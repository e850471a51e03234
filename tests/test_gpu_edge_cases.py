"""Edge cases of the tile update and of the tile-matrix multiply against the oracle: non-square tiles
in every combination the reference handles (HCore.cpp:23-344), alpha = 0 and beta = 0, rank-1 inputs
and a C at full capacity, tiny tiles, and a rectangular tile grid (mt != nt != kt).  Bar as in the
other parity tests: rank within +-1 of the oracle's (Compressed.cpp:509-527), relative Frobenius
error within 2 x max(oracle's error, accuracy) against the exact product of the inputs.
"""
import numpy as np
import pytest

from oracle import hcore_oracle as O
from tests.helpers import compressed_from_dense, rel_fro, random_lowrank

pytestmark = pytest.mark.gpu

COMBOS = ["CCC", "DCC", "CDC", "CCD", "DCD", "CDD", "DDD"]
ACC = 1e-8


@pytest.fixture(scope="module")
def T():
    import torch
    from hcorepp_gb300 import tiles
    assert torch.cuda.is_available()
    return tiles


def _gpu(T, t):
    if t.kind == "dense":
        return T.DenseTile(t.rows, t.cols, t.data)
    return T.CompressedTile(t.rows, t.cols, t.u, t.v, max_rank=t.max_rank)


def _make(kind, d, acc=ACC, max_rank=None):
    return O.DenseTile(d) if kind == "D" else compressed_from_dense(d, acc, True, max_rank)


def _check(oc, gc, exact, acc=ACC):
    e_o = rel_fro(oc.to_dense(), exact)
    e_g = rel_fro(gc.to_dense(), exact)
    assert e_g <= 2 * max(e_o, acc), (e_g, e_o)
    if oc.kind == "compressed":
        assert abs(gc.rank - oc.rank) <= 1, (gc.rank, oc.rank)


def _update(T, alpha, oa, ob, beta, oc, mode, acc=ACC):
    ga, gb, gc = _gpu(T, oa), _gpu(T, ob), _gpu(T, oc)
    exact = alpha * oa.to_dense() @ ob.to_dense() + beta * oc.to_dense()
    O.hcore_gemm(alpha, oa, ob, beta, oc, O.CompressionParameters(acc, truncated_svd=True))
    T.HCore.Gemm(alpha, ga, 0, gb, 0, beta, gc, T.CompressionParameters(acc, truncated_svd=True, mode=mode))
    _check(oc, gc, exact, acc)
    return gc, oc


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("combo", COMBOS)
def test_non_square_tiles(T, combo, mode):
    """A: 96 x 160, B: 160 x 72, C: 96 x 72 (capacities min(m, n) / 3: the update clamps C's rank)."""
    rng = np.random.default_rng(11)
    a = random_lowrank(96, 160, 20, rng, 0.6)
    b = random_lowrank(160, 72, 18, rng, 0.6)
    c = random_lowrank(96, 72, 15, rng, 0.6)
    _update(T, 1.5, _make(combo[0], a), _make(combo[1], b), 0.75, _make(combo[2], c), mode)


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("alpha,beta", [(0.0, 1.25), (2.0, 0.0)])
def test_alpha_or_beta_zero(T, alpha, beta, mode):
    """alpha = 0 recompresses beta C alone; beta = 0 replaces C by the recompressed alpha A B."""
    rng = np.random.default_rng(5)
    a, b, c = (random_lowrank(128, 128, 24, rng, 0.7) for _ in range(3))
    _update(T, alpha, _make("C", a, max_rank=48), _make("C", b, max_rank=48), beta, _make("C", c, max_rank=48), mode)


@pytest.mark.parametrize("mode", [0, 1])
def test_rank_one_inputs_into_a_full_c(T, mode):
    """Rank-1 A and B against a C already at its capacity: the stack is one column wider than C can
    hold, and the new rank is clamped (Compressed.cpp:526-527)."""
    rng = np.random.default_rng(2)
    a = np.outer(rng.standard_normal(128), rng.standard_normal(128))
    b = np.outer(rng.standard_normal(128), rng.standard_normal(128))
    c = random_lowrank(128, 128, 40, rng, 0.9)
    oc = _make("C", c, max_rank=40)
    assert oc.rank == 40
    gc, oc = _update(T, 1.0, _make("C", a, max_rank=40), _make("C", b, max_rank=40), 1.0, oc, mode)
    assert gc.rank == oc.rank == 40


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("combo", ["CCC", "DCC", "CDC"])
def test_tiny_tiles(T, combo, mode):
    """8 x 8 tiles of rank 1 and 2: fewer rows than the lane groups of the QR and Jacobi kernels."""
    rng = np.random.default_rng(9)
    a = random_lowrank(8, 8, 2, rng, 0.5)
    b = random_lowrank(8, 8, 1, rng, 0.5)
    c = random_lowrank(8, 8, 2, rng, 0.5)
    _update(T, 1.0, _make(combo[0], a, max_rank=4), _make(combo[1], b, max_rank=4), 1.0,
            _make(combo[2], c, max_rank=4), mode)


@pytest.mark.parametrize("mode", [0, 1])
def test_rectangular_tile_grid(T, mode):
    """C (2 x 3 tiles) += A (2 x 4 tiles) B (4 x 3 tiles) through hcgb_tlr_gemm in the reference's k
    order, against the oracle's tile loop (examples/matrix_multiplication/omp_main.cpp:112-124)."""
    import torch
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300.problems import KernelMatrix
    nb, mt, nt, kt = 64, 2, 3, 4
    km = KernelMatrix(8 * nb, nb, 2, 0.1, 3)
    kc = KernelMatrix(8 * nb, nb, 2, 0.1, 4)
    oa = [[_make("C", km.tile(i, k)) for k in range(kt)] for i in range(mt)]
    ob = [[_make("C", km.tile(4 + k, j)) for j in range(nt)] for k in range(kt)]
    oc = [[_make("C", kc.tile(i, j)) for j in range(nt)] for i in range(mt)]

    def load(tiles, r, c):
        tm = T.TileMatrix(r, c, nb, [[L.COMPRESSED] * c for _ in range(r)], nb // 3)
        for i in range(r):
            for j in range(c):
                tm.set_tile(i, j, u=tiles[i][j].u, v=tiles[i][j].v)
        return tm

    A, B, C = load(oa, mt, kt), load(ob, kt, nt), load(oc, mt, nt)
    exact = (np.block([[t.to_dense() for t in row] for row in oa]) @ np.block([[t.to_dense() for t in row] for row in ob])
             + np.block([[t.to_dense() for t in row] for row in oc]))
    info = T.info_buffer(mt * nt * kt)
    ctx = T.run_context()
    ctx.set_k_order(0)
    T.tlr_gemm(1.0, A, B, 1.0, C, T.CompressionParameters(ACC, truncated_svd=True, mode=mode), info)
    torch.cuda.synchronize()
    stats = O.tile_matrix_multiply(oa, ob, oc, 1.0, 1.0, O.CompressionParameters(ACC, truncated_svd=True))
    rec = info.cpu().numpy()
    for (i, j, k, _kk, rank, _cl) in stats:
        r = rec[k * mt * nt + i + j * mt]
        assert r[0] == 0 and abs(int(r[5]) - int(rank)) <= 1, (i, j, k, r, rank)
    g = C.to_dense()
    o = np.block([[t.to_dense() for t in row] for row in oc])
    assert rel_fro(g, exact) <= 2 * max(rel_fro(o, exact), ACC)
