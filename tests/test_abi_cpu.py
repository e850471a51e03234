"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, and exports every
entry point include/hcgb.h declares (no compute call: there is no GPU here); and host-side logic
of the Python mirror that needs no kernel (TilePacker)."""
import ctypes

import numpy as np
import pytest

from hcorepp_gb300 import _lib as L
from hcorepp_gb300.build import build


def test_library_builds_and_exports_header_symbols():
    path = build()
    lib = ctypes.CDLL(path)
    names = L.header_functions()
    assert "hcgb_tile_gemm" in names and "hcgb_gemm_batch" in names and "hcgb_tlr_gemm" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_workspace_sizing_is_host_only():
    lib = L.lib()
    small = lib.hcgb_workspace_bytes(1, 64, 64, 21, 21)
    big = lib.hcgb_workspace_bytes(1024, 512, 512, 170, 170)
    assert 0 < small < big
    assert lib.hcgb_workspace_bytes(0, 512, 512, 170, 170) == 0
    # Per update at nb=512: two 512 x 340 stacks dominate (~2.8 MB) plus the core buffers (~8 MB in all).
    per = big / 1024
    assert 2.5e6 < per < 9e6, per


def test_bad_arguments_without_a_device():
    lib = L.lib()
    assert lib.hcgb_sync(None) == L.HCGB_BAD_ARG
    assert lib.hcgb_gemm_batch(None, 1.0, 1.0, 0, None, None, None) == L.HCGB_BAD_ARG


def test_tile_packer_round_trip_on_host():
    """TilePacker.UnPackTile / PackTile (TilePacker.cpp:5-26) on host tensors: metadata fields and a
    tile over the same buffer, no copy."""
    import torch
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300 import tiles as T
    rng = np.random.default_rng(0)
    u, v = rng.standard_normal((40, 5)), rng.standard_normal((5, 30))
    c = T.CompressedTile(40, 30, u, v, max_rank=13, device="cpu")
    meta, buf = T.TilePacker.UnPackTile(c)
    assert (meta.rows, meta.cols, meta.rank, meta.max_rank, meta.leading_dim, meta.type) == (40, 30, 5, 13, 40,
                                                                                              L.COMPRESSED)
    assert buf.data_ptr() == c.buffer.data_ptr()
    p = T.TilePacker.PackTile(meta, buf)
    assert p.buffer.data_ptr() == buf.data_ptr() and p.rank == 5
    np.testing.assert_array_equal(p.to_dense(), u @ v)
    d = T.DenseTile(7, 9, rng.standard_normal((7, 9)), device="cpu")
    md, bd = T.TilePacker.UnPackTile(d)
    assert md.type == L.DENSE and (md.rows, md.cols, md.leading_dim) == (7, 9, 7)
    np.testing.assert_array_equal(T.TilePacker.PackTile(md, bd).to_dense(), d.to_dense())
    with pytest.raises(ValueError):
        T.TilePacker.PackTile(T.TileMetadata(40, 30, 14, 13, 40, "C", L.COMPRESSED), buf)
    with pytest.raises(ValueError):
        T.TilePacker.PackTile(T.TileMetadata(7, 9, 0, 0, 8, "C", L.DENSE), bd)


def test_rank_trimmed_host_pack_layout():
    """TileMatrix.host_pack (the host side of hcgb_pack_tiles' format): tiles in index order
    (i + j * mt), a dense tile whole, a compressed tile's first rank columns of U followed by the
    first rank * nb values of its V region; rank 0 contributes nothing."""
    from hcorepp_gb300 import tiles as T
    mt, nt, nb, mr = 2, 3, 8, 3
    kinds = [[L.DENSE if i == j else L.COMPRESSED for j in range(nt)] for i in range(mt)]
    tm = T.TileMatrix(mt, nt, nb, kinds, mr, device="cpu")
    arena = np.arange(tm.arena.numel(), dtype=np.float64)
    ranks = np.array([0, 2, 3, 0, 1, 1], dtype=np.int32)
    got = tm.host_pack(arena, ranks)
    want = []
    for idx in range(mt * nt):
        i, j = idx % mt, idx // mt
        o = int(tm.offsets[idx])
        if kinds[i][j] == L.DENSE:
            want.append(arena[o:o + nb * nb])
        else:
            r = int(ranks[idx])
            want += [arena[o:o + nb * r], arena[o + nb * mr:o + nb * mr + r * nb]]
    np.testing.assert_array_equal(got, np.concatenate(want))
    assert got.size == 2 * nb * nb + 2 * nb * (2 + 3 + 1 + 1)  # two dense tiles; compressed ranks 2, 3, 1, 1
