"""GPU parity: libhcgb (through its C ABI) against the CPU oracle on the same seeded inputs.

Bar (floating point): truncated ranks within +-1 of the oracle's, and the relative Frobenius
error of the product against the exact FP64 product within the accuracy bound the oracle
itself reaches (factor 2, floor = the requested accuracy).  Known-answer cases use the
reference's comparator (relative 1e-2, tests/helpers/src/testHelpers.cpp:83-88).
"""
import json
import os

import numpy as np
import pytest

from oracle import hcore_oracle as O
from tests.helpers import compressed_from_dense, rel_fro, random_lowrank

pytestmark = pytest.mark.gpu

KAT = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "kat.json")))


@pytest.fixture(scope="module")
def T():
    import torch
    from hcorepp_gb300 import tiles
    assert torch.cuda.is_available()
    return tiles


def _rowmajor(entry, name, r, c):
    return np.array(KAT[entry][name]["values"]).reshape(r, c)


def _gpu_tile(T, t):
    if t.kind == "dense":
        return T.DenseTile(t.rows, t.cols, t.data)
    return T.CompressedTile(t.rows, t.cols, t.u, t.v, max_rank=t.max_rank)


def test_kat_compressed_tile_ddc(T):
    # TestCompressedTile.cpp:124-260 expressed as a CCC update with identity factors.
    a = _rowmajor("compressed_tile_ddc", "matrix_A", 3, 3)
    b = _rowmajor("compressed_tile_ddc", "matrix_B", 3, 2)
    A = T.CompressedTile(3, 3, a, np.eye(3))
    B = T.CompressedTile(3, 2, np.eye(3), b)
    C = T.CompressedTile(3, 2, np.zeros((3, 2)), np.zeros((2, 2)))
    T.HCore.Gemm(1.0, A, 0, B, 0, 1.0, C, T.CompressionParameters(np.finfo(float).eps))
    np.testing.assert_allclose(C.to_dense(), _rowmajor("compressed_tile_ddc", "output_matrix", 3, 2), rtol=1e-2)


def test_kat_gemm_test9_ccc(T):
    # TestGemm.cpp:748-915
    A = T.CompressedTile(5, 4, _rowmajor("gemm_test9_ccc", "matrix_Au", 5, 3),
                         _rowmajor("gemm_test9_ccc", "matrix_Av", 3, 4))
    B = T.CompressedTile(4, 2, _rowmajor("gemm_test9_ccc", "matrix_Bu", 4, 2),
                         _rowmajor("gemm_test9_ccc", "matrix_Bv", 2, 2))
    C = T.CompressedTile(5, 2, np.zeros((5, 1)), np.zeros((1, 2)))
    T.HCore.Gemm(1.0, A, 0, B, 0, 1.0, C, T.CompressionParameters(np.finfo(float).eps))
    assert C.rank == 1
    np.testing.assert_allclose(C.to_dense(), _rowmajor("gemm_test9_ccc", "output_matrix", 5, 2), rtol=1e-2)


def test_kat_gemm_test10_ddc(T):
    # TestGemm.cpp:917-1045: DDC re-sets C at full rank with V = I.
    A = T.DenseTile(5, 3, _rowmajor("gemm_test10_ddc", "matrix_A", 5, 3))
    B = T.DenseTile(3, 4, _rowmajor("gemm_test10_ddc", "matrix_B", 3, 4))
    C = T.CompressedTile(5, 4, np.zeros((5, 4)), np.zeros((4, 4)))
    T.HCore.Gemm(1.0, A, 0, B, 0, 1.0, C, T.CompressionParameters(np.finfo(float).eps))
    np.testing.assert_allclose(C.to_dense(), _rowmajor("gemm_test10_ddc", "output_matrix", 5, 4), rtol=1e-2)
    np.testing.assert_array_equal(C.v(), np.eye(4))


COMBOS = ["CCC", "DCC", "CDC", "CCD", "DCD", "CDD", "DDD"]


def _make(kind, d, acc):
    if kind == "D":
        return O.DenseTile(d)
    return compressed_from_dense(d, acc, truncated=True)


@pytest.mark.parametrize("combo", COMBOS)
@pytest.mark.parametrize("nb", [96, 256])
@pytest.mark.parametrize("mode", [0, 1])
def test_single_update_vs_oracle(T, combo, nb, mode):
    from hcorepp_gb300.problems import KernelMatrix
    acc = 1e-8
    km = KernelMatrix(4 * nb, nb, 2, 0.1, 1)
    kc = KernelMatrix(4 * nb, nb, 2, 0.1, 2)
    da, db, dc = km.tile(0, 1), km.tile(1, 3), kc.tile(0, 3)
    alpha, beta = 3.5, 2.5  # AdvancedGemmTest.cpp:31-32
    oa, ob, oc = _make(combo[0], da, acc), _make(combo[1], db, acc), _make(combo[2], dc, acc)
    ga, gb, gc = _gpu_tile(T, oa), _gpu_tile(T, ob), _gpu_tile(T, oc)
    exact = alpha * oa.to_dense() @ ob.to_dense() + beta * oc.to_dense()
    params = O.CompressionParameters(acc, truncated_svd=True)
    info = O.hcore_gemm(alpha, oa, ob, beta, oc, params)
    T.HCore.Gemm(alpha, ga, 0, gb, 0, beta, gc, T.CompressionParameters(acc, truncated_svd=True, mode=mode))
    e_o = rel_fro(oc.to_dense(), exact)
    e_g = rel_fro(gc.to_dense(), exact)
    assert e_g <= 2 * max(e_o, acc), (e_g, e_o)
    if combo[2] == "C":
        assert abs(gc.rank - oc.rank) <= 1, (gc.rank, oc.rank, info)
    else:
        assert e_g < 1e-13


@pytest.mark.parametrize("accuracy,truncated", [(1e-4, False), (1e-6, True), (1e-10, True)])
@pytest.mark.parametrize("mode", [0, 1])
def test_rank_rule_modes(T, accuracy, truncated, mode):
    rng = np.random.default_rng(7)
    m = n = 128
    a = random_lowrank(m, n, 40, rng, 0.6)
    b = random_lowrank(n, n, 40, rng, 0.6)
    c = random_lowrank(m, n, 40, rng, 0.6)
    p = O.CompressionParameters(accuracy, truncated_svd=truncated)
    oa, ob, oc = (compressed_from_dense(x, 1e-14, True, max_rank=60) for x in (a, b, c))
    ga, gb, gc = (_gpu_tile(T, t) for t in (oa, ob, oc))
    O.hcore_gemm(1.0, oa, ob, 1.0, oc, p)
    T.HCore.Gemm(1.0, ga, 0, gb, 0, 1.0, gc, T.CompressionParameters(accuracy, truncated_svd=truncated, mode=mode))
    assert abs(gc.rank - oc.rank) <= 1
    exact = a @ b + c
    assert rel_fro(gc.to_dense(), exact) <= 2 * max(rel_fro(oc.to_dense(), exact), 1e-15)


@pytest.mark.parametrize("mode", [0, 1])
def test_fixed_rank(T, mode):
    rng = np.random.default_rng(3)
    a, b, c = (random_lowrank(64, 64, 20, rng, 0.7) for _ in range(3))
    oa, ob, oc = (compressed_from_dense(x, 1e-14, True, max_rank=30) for x in (a, b, c))
    ga, gb, gc = (_gpu_tile(T, t) for t in (oa, ob, oc))
    p = O.CompressionParameters(1e-8, fixed_rank=7)
    O.hcore_gemm(1.0, oa, ob, 1.0, oc, p)
    T.HCore.Gemm(1.0, ga, 0, gb, 0, 1.0, gc, T.CompressionParameters(1e-8, fixed_rank=7, mode=mode))
    assert gc.rank == oc.rank == 7
    np.testing.assert_allclose(gc.to_dense(), oc.to_dense(), atol=1e-10 * np.abs(oc.to_dense()).max())


@pytest.mark.parametrize("mode", [0, 1])
def test_rank_clamp_at_capacity(T, mode):
    # Compressed.cpp:526-527: the new rank never exceeds the tile's max rank.
    rng = np.random.default_rng(11)
    a, b, c = (random_lowrank(64, 64, 30, rng, 0.9) for _ in range(3))
    oa, ob = (compressed_from_dense(x, 1e-14, True) for x in (a, b))
    oc = compressed_from_dense(c, 1e-14, True, max_rank=12)
    oc.u, oc.v = oc.u[:, :12], oc.v[:12]
    ga, gb, gc = (_gpu_tile(T, t) for t in (oa, ob, oc))
    p = O.CompressionParameters(1e-12, truncated_svd=True)
    O.hcore_gemm(1.0, oa, ob, 1.0, oc, p)
    T.HCore.Gemm(1.0, ga, 0, gb, 0, 1.0, gc, T.CompressionParameters(1e-12, truncated_svd=True, mode=mode))
    assert gc.rank == oc.rank == 12
    exact_o = oc.to_dense()
    assert rel_fro(gc.to_dense(), exact_o) < 1e-6


@pytest.mark.parametrize("mode", [0, 1])
def test_trans_operands(T, mode):
    # op(A) = A^T, op(B) = B^T (HCore.cpp:73-110 swaps the factor holders); C has room for the full rank.
    rng = np.random.default_rng(5)
    a, b, c = (random_lowrank(48, 48, 12, rng, 0.5) for _ in range(3))
    oa, ob = (compressed_from_dense(x, 1e-14, True) for x in (a, b))
    oc = compressed_from_dense(c, 1e-14, True, max_rank=40)
    ga, gb, gc = (_gpu_tile(T, t) for t in (oa, ob, oc))
    T.HCore.Gemm(1.0, ga, 1, gb, 1, 1.0, gc, T.CompressionParameters(1e-12, truncated_svd=True, mode=mode))
    exact = oa.to_dense().T @ ob.to_dense().T + oc.to_dense()
    assert rel_fro(gc.to_dense(), exact) < 1e-10
    gd = T.DenseTile(48, 48, a)
    gc2 = _gpu_tile(T, compressed_from_dense(c, 1e-14, True, max_rank=40))
    T.HCore.Gemm(2.0, gd, 1, gb, 0, 1.0, gc2, T.CompressionParameters(1e-12, truncated_svd=True, mode=mode))
    exact2 = 2.0 * a.T @ ob.to_dense() + oc.to_dense()
    assert rel_fro(gc2.to_dense(), exact2) < 1e-10


@pytest.mark.parametrize("k_order,oz,mixed", [(0, True, False), (1, True, False), (0, False, False), (1, True, True)])
def test_tlr_multiply_vs_oracle(T, k_order, oz, mixed):
    """A 4x4-tile multiply (nb=128) through hcgb_tlr_gemm against the oracle's tile loop, in the
    reference's k order and in the cost-first order (same sum, other rounding order), with the
    large products and the WY Q application on the tensor cores (oz) and all on the FP64 pipe, and
    with the float-float core Jacobi (mixed)."""
    import torch
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300.problems import KernelMatrix
    nt, nb, acc = 4, 128, 1e-8
    km = KernelMatrix(nt * nb, nb, 2, 0.1, 1)
    kc = KernelMatrix(nt * nb, nb, 2, 0.1, 2)
    maxr = nb // 3
    params = O.CompressionParameters(acc, truncated_svd=True)
    dense_diag = True
    kinds = [[L.DENSE if (dense_diag and i == j) else L.COMPRESSED for j in range(nt)] for i in range(nt)]
    mats = {}
    otiles = {}
    for name, kmat in (("A", km), ("B", km), ("C", kc)):
        tm = T.TileMatrix(nt, nt, nb, kinds, maxr)
        og = [[None] * nt for _ in range(nt)]
        for i in range(nt):
            for j in range(nt):
                d = kmat.tile(i, j)
                if kinds[i][j] == L.DENSE:
                    og[i][j] = O.DenseTile(d)
                    tm.set_tile(i, j, dense=d)
                else:
                    og[i][j] = compressed_from_dense(d, acc)
                    tm.set_tile(i, j, u=og[i][j].u, v=og[i][j].v)
        mats[name], otiles[name] = tm, og
    a_dense, b_dense, c_dense = (mats[x].to_dense() for x in "ABC")
    exact = a_dense @ b_dense + c_dense
    info = T.info_buffer(nt * nt * nt)
    ctx = T.run_context()
    ctx.set_k_order(k_order)
    ctx.set_tensor_products(oz)
    try:
        T.tlr_gemm(1.0, mats["A"], mats["B"], 1.0, mats["C"],
                   T.CompressionParameters(acc, truncated_svd=True, mode=L.MIXED if mixed else L.PLAIN_FP64), info)
        torch.cuda.synchronize()
    finally:
        ctx.set_k_order(0)
        ctx.set_tensor_products(True)
    info = info.cpu().numpy()
    assert int(info[:, 0].max()) == 0, info
    O.tile_matrix_multiply(otiles["A"], otiles["B"], otiles["C"], 1.0, 1.0, params)
    o_dense = np.block([[otiles["C"][i][j].to_dense() for j in range(nt)] for i in range(nt)])
    g_dense = mats["C"].to_dense()
    e_o, e_g = rel_fro(o_dense, exact), rel_fro(g_dense, exact)
    assert e_g <= 2 * max(e_o, acc), (e_g, e_o)
    granks = mats["C"].rank_grid()
    for i in range(nt):
        for j in range(nt):
            if kinds[i][j] == L.COMPRESSED:
                assert abs(granks[i, j] - otiles["C"][i][j].rank) <= 1


def test_tlr_multiply_concurrency_invariant(T):
    """The C-tile grouping (streams) changes the schedule, never the arithmetic: bitwise equal."""
    import torch
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300.problems import KernelMatrix
    nt, nb, acc = 4, 96, 1e-8
    km = KernelMatrix(nt * nb, nb, 2, 0.1, 1)
    kc = KernelMatrix(nt * nb, nb, 2, 0.1, 2)
    kinds = [[L.COMPRESSED] * nt for _ in range(nt)]
    A = T.TileMatrix(nt, nt, nb, kinds, nb // 3)
    C0 = T.TileMatrix(nt, nt, nb, kinds, nb // 3)
    for i in range(nt):
        for j in range(nt):
            ta = compressed_from_dense(km.tile(i, j), acc)
            tc = compressed_from_dense(kc.tile(i, j), acc)
            A.set_tile(i, j, u=ta.u, v=ta.v)
            C0.set_tile(i, j, u=tc.u, v=tc.v)
    ctx = T.run_context()
    outs = []
    for groups in (1, 3, 8):
        ctx.set_concurrency(groups)
        C = T.TileMatrix(nt, nt, nb, kinds, nb // 3)
        C.arena.copy_(C0.arena)
        C.ranks.copy_(C0.ranks)
        T.tlr_gemm(1.0, A, A, 1.0, C, T.CompressionParameters(acc, truncated_svd=True))
        torch.cuda.synchronize()
        outs.append((C.arena.cpu().numpy().copy(), C.ranks.cpu().numpy().copy()))
    ctx.set_concurrency(8)
    for arena, ranks in outs[1:]:
        np.testing.assert_array_equal(ranks, outs[0][1])
        np.testing.assert_array_equal(arena, outs[0][0])


@pytest.mark.parametrize("k_order", [0, 1])
def test_tlr_multiply_graph_replay_bitwise(T, k_order):
    """hcgb_set_graph: the multiply captured as one CUDA graph and replayed gives the same bits as the
    directly launched multiply, call after call, and its launches are counted."""
    import torch
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300.problems import KernelMatrix
    nt, nb, acc = 4, 96, 1e-8
    km = KernelMatrix(nt * nb, nb, 2, 0.1, 1)
    kc = KernelMatrix(nt * nb, nb, 2, 0.1, 2)
    kinds = [[L.DENSE if i == j else L.COMPRESSED for j in range(nt)] for i in range(nt)]
    A = T.TileMatrix(nt, nt, nb, kinds, nb // 3)
    C0 = T.TileMatrix(nt, nt, nb, kinds, nb // 3)
    for i in range(nt):
        for j in range(nt):
            if i == j:
                A.set_tile(i, j, dense=km.tile(i, j))
                C0.set_tile(i, j, dense=kc.tile(i, j))
            else:
                ta = compressed_from_dense(km.tile(i, j), acc)
                tc = compressed_from_dense(kc.tile(i, j), acc)
                A.set_tile(i, j, u=ta.u, v=ta.v)
                C0.set_tile(i, j, u=tc.u, v=tc.v)
    ctx = T.run_context()
    ctx.set_k_order(k_order)
    C = T.TileMatrix(nt, nt, nb, kinds, nb // 3)
    params = T.CompressionParameters(acc, truncated_svd=True)
    outs = []
    try:
        for graph in (False, True, True, True):
            ctx.set_graph(graph)
            C.arena.copy_(C0.arena)
            C.ranks.copy_(C0.ranks)
            l0 = L.kernel_launches()
            T.tlr_gemm(1.0, A, A, 1.0, C, params)
            torch.cuda.synchronize()
            outs.append((C.arena.cpu().numpy().copy(), C.ranks.cpu().numpy().copy(), L.kernel_launches() - l0))
    finally:
        ctx.set_graph(False)
        ctx.set_k_order(0)
    for arena, ranks, launches in outs[1:]:
        np.testing.assert_array_equal(ranks, outs[0][1])
        np.testing.assert_array_equal(arena, outs[0][0])
        # a replay launches the captured kernels; the capturing call also ran the rank gather of the
        # cost-first order before its capture
        assert outs[0][2] > 0 and 0 <= outs[0][2] - launches <= k_order


@pytest.mark.parametrize("combo", ["CCC", "DCC", "CDC"])
def test_mixed_mode_vs_oracle(T, combo):
    """HCGB_MIXED (single-precision Jacobi preconditioning of the core): same ranks (+-1) and
    product accuracy as the plain FP64 form."""
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300.problems import KernelMatrix
    acc, nb = 1e-8, 256
    km = KernelMatrix(4 * nb, nb, 2, 0.1, 1)
    kc = KernelMatrix(4 * nb, nb, 2, 0.1, 2)
    da, db, dc = km.tile(0, 1), km.tile(1, 2), kc.tile(0, 2)
    oa, ob, oc = _make(combo[0], da, acc), _make(combo[1], db, acc), _make(combo[2], dc, acc)
    ga, gb, gc = _gpu_tile(T, oa), _gpu_tile(T, ob), _gpu_tile(T, oc)
    exact = oa.to_dense() @ ob.to_dense() + oc.to_dense()
    O.hcore_gemm(1.0, oa, ob, 1.0, oc, O.CompressionParameters(acc, truncated_svd=True))
    T.HCore.Gemm(1.0, ga, 0, gb, 0, 1.0, gc, T.CompressionParameters(acc, truncated_svd=True, mode=L.MIXED))
    assert abs(gc.rank - oc.rank) <= 1
    assert rel_fro(gc.to_dense(), exact) <= 2 * max(rel_fro(oc.to_dense(), exact), acc)


@pytest.mark.parametrize("truncated,acc", [(True, 1e-8), (False, 1e-6)])
@pytest.mark.parametrize("mode", [0, 1])
def test_compress_tile_vs_oracle(T, truncated, acc, mode):
    """GPU dense -> compressed construction vs the reference's constructor restated in the oracle
    (Compressed.cpp:75-146): rank +-1, reconstruction error at the oracle's level."""
    from hcorepp_gb300.problems import KernelMatrix
    km = KernelMatrix(1024, 256, 2, 0.1, 4)
    for (i, j) in [(0, 1), (0, 3), (2, 2)]:
        d = km.tile(i, j)
        o = O.CompressedTile.from_dense(d, O.CompressionParameters(acc, truncated_svd=truncated))
        g = T.CompressedTile.from_dense(d, T.CompressionParameters(acc, truncated_svd=truncated, mode=mode))
        assert g.max_rank == o.max_rank == 256 // 3
        assert abs(g.rank - o.rank) <= 1, (i, j, g.rank, o.rank)
        e_o = rel_fro(o.to_dense(), d)
        assert rel_fro(g.to_dense(), d) <= 2 * max(e_o, 1e-14), (i, j)


def test_tile_packer_gemm_through_packed_tiles(T):
    """A tile moved as (TileMetadata, device buffer) and re-packed gives a bitwise identical product."""
    rng = np.random.default_rng(9)
    nb = 128
    a = compressed_from_dense(random_lowrank(nb, nb, 20, rng), 1e-10)
    c = compressed_from_dense(random_lowrank(nb, nb, 15, rng), 1e-10)
    bd = rng.standard_normal((nb, nb))
    ga, gb = _gpu_tile(T, a), T.DenseTile(nb, nb, bd)
    outs = []
    for packed in (False, True):
        gc = _gpu_tile(T, c)
        ta, tb = ga, gb
        if packed:
            ta = T.TilePacker.PackTile(*T.TilePacker.UnPackTile(ga))
            tb = T.TilePacker.PackTile(*T.TilePacker.UnPackTile(gb))
        T.HCore.Gemm(1.0, ta, 0, tb, 0, 1.0, gc, T.CompressionParameters(1e-8, truncated_svd=True))
        outs.append((gc.rank, gc.u().copy(), gc.v().copy()))
    assert outs[0][0] == outs[1][0]
    np.testing.assert_array_equal(outs[0][1], outs[1][1])
    np.testing.assert_array_equal(outs[0][2], outs[1][2])


@pytest.mark.parametrize("vt", [False, True])
def test_rank_trimmed_pack_roundtrip(T, vt):
    """hcgb_pack_tiles / hcgb_unpack_tiles: offsets from the device ranks (rank 0 and full capacity
    included), packed bytes equal to the host-side format, and unpacking into a fresh tile matrix
    restores every used value bit for bit."""
    import torch
    from hcorepp_gb300 import _lib as L
    rng = np.random.default_rng(31 + vt)
    mt, nt, nb, mr = 3, 4, 64, 20
    kinds = [[L.DENSE if i == j else L.COMPRESSED for j in range(nt)] for i in range(mt)]
    tm = T.TileMatrix(mt, nt, nb, kinds, mr, vt=vt)
    tm.arena.copy_(torch.from_numpy(rng.standard_normal(tm.arena.numel())))
    ranks = rng.integers(0, mr + 1, size=mt * nt).astype(np.int32)
    ranks[1], ranks[2] = 0, mr
    tm.ranks.copy_(torch.from_numpy(ranks))
    packed = torch.full((tm.arena.numel(),), np.nan, dtype=torch.float64, device="cuda")
    offs = torch.zeros(mt * nt + 1, dtype=torch.int64, device="cuda")
    tm.pack(packed, offs)
    torch.cuda.synchronize()
    want = tm.host_pack(tm.arena.cpu().numpy(), ranks)
    sizes = [nb * nb if kinds[idx % mt][idx // mt] == L.DENSE else 2 * nb * int(ranks[idx]) for idx in range(mt * nt)]
    np.testing.assert_array_equal(offs.cpu().numpy(), np.concatenate([[0], np.cumsum(sizes)]))
    total = int(offs[-1])
    assert total == want.size
    np.testing.assert_array_equal(packed[:total].cpu().numpy(), want)
    tm2 = T.TileMatrix(mt, nt, nb, kinds, mr, vt=vt)
    tm2.ranks.copy_(tm.ranks)
    offs2 = torch.zeros_like(offs)
    tm2.unpack(packed, offs2)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(offs2.cpu().numpy(), offs.cpu().numpy())
    np.testing.assert_array_equal(tm2.host_pack(tm2.arena.cpu().numpy(), ranks), want)


@pytest.mark.parametrize("scaled", [False, True])
def test_tensor_core_products_fp64_accurate(T, scaled):
    """Dense products on the 16-bit tensor cores (error-free splitting) match an extended-precision
    product to FP64 worst-case accuracy, with rows / columns spanning 2^+-40, zero rows and columns
    and mixed signs; the FP64 DMMA path gives the same to rounding."""
    rng = np.random.default_rng(12)
    m, n, k = 96, 40, 200
    a = rng.standard_normal((m, k))
    b = rng.standard_normal((k, n))
    c = rng.standard_normal((m, n))
    if scaled:
        a *= np.exp2(rng.integers(-40, 40, size=(m, 1)))
        b *= np.exp2(rng.integers(-40, 40, size=(1, n)))
        a[5, :] = 0.0
        b[:, 7] = 0.0
        a[:, 3] *= 1e-12
    exact = (a.astype(np.longdouble) @ b.astype(np.longdouble)) * np.longdouble(1.5) + np.longdouble(0.25) * c
    bound = np.abs(a).max(axis=1, keepdims=True) * np.abs(b).max(axis=0, keepdims=True) * 1.5
    ctx = T.run_context()
    out = {}
    for oz in (True, False):
        ctx.set_tensor_products(oz)
        gc = T.DenseTile(m, n, c)
        T.HCore.Gemm(1.5, T.DenseTile(m, k, a), 0, T.DenseTile(k, n, b), 0, 0.25, gc)
        out[oz] = gc.to_dense()
    ctx.set_tensor_products(True)
    for oz, got in out.items():
        err = np.abs(got.astype(np.longdouble) - exact) / (bound + np.abs(0.25 * c))
        assert float(err.max()) < 2e-14, (oz, float(err.max()))


@pytest.mark.parametrize("precond", [1 << 30, 16, 2])
def test_plain_core_preconditioning_changes_rounding_only(T, precond):
    """hcgb_set_precond: with the plain form's FP32 preconditioning sweeps off (the default), from 16
    core columns or on every core of 2 columns and more, the multiply has the same ranks and the
    same product to rounding (the accumulated rotations are orthogonal to ~1e-13), and each is
    within the oracle's accuracy bound."""
    import torch
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300.problems import KernelMatrix
    nt, nb, acc = 4, 256, 1e-8
    km = KernelMatrix(nt * nb, nb, 2, 0.1, 1)
    kc = KernelMatrix(nt * nb, nb, 2, 0.1, 2)
    kinds = [[L.COMPRESSED] * nt for _ in range(nt)]
    oa = [[compressed_from_dense(km.tile(i, j), acc) for j in range(nt)] for i in range(nt)]
    oc = [[compressed_from_dense(kc.tile(i, j), acc) for j in range(nt)] for i in range(nt)]
    A = T.TileMatrix(nt, nt, nb, kinds, nb // 3)
    C0 = T.TileMatrix(nt, nt, nb, kinds, nb // 3)
    for i in range(nt):
        for j in range(nt):
            A.set_tile(i, j, u=oa[i][j].u, v=oa[i][j].v)
            C0.set_tile(i, j, u=oc[i][j].u, v=oc[i][j].v)
    exact = (np.block([[t.to_dense() for t in r] for r in oa]) @ np.block([[t.to_dense() for t in r] for r in oa])
             + np.block([[t.to_dense() for t in r] for r in oc]))
    ctx = T.run_context()
    params = T.CompressionParameters(acc, truncated_svd=True, mode=L.PLAIN_FP64)
    outs = {}
    try:
        for setting in (1 << 30, precond):
            ctx.set_precond(setting)
            C = T.TileMatrix(nt, nt, nb, kinds, nb // 3)
            C.arena.copy_(C0.arena)
            C.ranks.copy_(C0.ranks)
            T.tlr_gemm(1.0, A, A, 1.0, C, params)
            torch.cuda.synchronize()
            outs[setting] = (C.rank_grid(), C.to_dense())
    finally:
        ctx.set_precond(0)
    np.testing.assert_array_equal(outs[precond][0], outs[1 << 30][0])
    assert rel_fro(outs[precond][1], outs[1 << 30][1]) <= 1e-12
    O.tile_matrix_multiply(oa, oa, oc, 1.0, 1.0, O.CompressionParameters(acc, truncated_svd=True))
    e_o = rel_fro(np.block([[t.to_dense() for t in r] for r in oc]), exact)
    assert rel_fro(outs[precond][1], exact) <= 2 * max(e_o, acc)
