"""hcgb_tile_gemm_noalloc: the tile update for callers that may not allocate device memory
(task-runtime workers whose runtime owns the device memory, or real-time callers that forbid
allocation after start-up).  It must give the same result as the allocating entry point
hcgb_tile_gemm, call after call, while using only the library's fixed scratch array, and it
must refuse updates that do not fit that array or the shared-memory limits before touching C.

This file is collected last on purpose: it runs after every other test, and also passes
alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import hcore_oracle as O
from tests.helpers import compressed_from_dense, rel_fro

pytestmark = pytest.mark.gpu

COMBOS = ["CCC", "DCC", "CDC", "CCD", "DCD", "CDD", "DDD"]


def _inputs(seed, combo):
    from hcorepp_gb300.problems import KernelMatrix
    nb, acc = 256, 1e-8
    km = KernelMatrix(4 * nb, nb, 2, 0.1, seed)
    kc = KernelMatrix(4 * nb, nb, 2, 0.1, seed + 1)
    dense = (km.tile(0, 1), km.tile(1, 3), kc.tile(0, 3))
    return [O.DenseTile(d) if kind == "D" else compressed_from_dense(d, acc) for kind, d in zip(combo, dense)]


def _gpu(T, t):
    if t.kind == "dense":
        return T.DenseTile(t.rows, t.cols, t.data)
    return T.CompressedTile(t.rows, t.cols, t.u, t.v, max_rank=t.max_rank)


def _noalloc(L, T, alpha, a, b, beta, c, params, info=None):
    import torch
    ta, tb, tc = a.c_tile(), b.c_tile(), c.c_tile()
    p = params.c()
    stream = torch.cuda.current_stream().cuda_stream
    return L.lib().hcgb_tile_gemm_noalloc(alpha, C.byref(ta), C.byref(tb), beta, C.byref(tc), C.byref(p),
                                          C.c_void_p(stream), C.c_void_p(info.data_ptr() if info is not None else 0))


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("combo", COMBOS)
def test_noalloc_matches_allocating_entry_point_twice(combo, mode):
    import torch
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300 import tiles as T
    assert torch.cuda.is_available()
    acc = 1e-8
    params = T.CompressionParameters(acc, truncated_svd=True, mode=mode)
    info = torch.zeros(len(L.INFO_FIELDS), dtype=torch.int32, device="cuda")
    for call, seed in enumerate((1, 3)):
        oa, ob, oc = _inputs(seed, combo)
        exact = 2.0 * oa.to_dense() @ ob.to_dense() + 0.5 * oc.to_dense()
        # the allocating entry point
        ga, gb, gc = _gpu(T, oa), _gpu(T, ob), _gpu(T, oc)
        T.HCore.Gemm(2.0, ga, 0, gb, 0, 0.5, gc, params)
        # the entry point that allocates nothing (same operands, fresh copy of C)
        na, nb_, nc = _gpu(T, oa), _gpu(T, ob), _gpu(T, oc)
        torch.cuda.synchronize()
        torch_before = torch.cuda.memory_allocated()
        free_before = torch.cuda.mem_get_info()[0]
        rc = _noalloc(L, T, 2.0, na, nb_, 0.5, nc, params, info)
        assert rc == L.HCGB_OK, (combo, call, rc)
        torch.cuda.synchronize()
        if call == 1:  # warmed up (kernels loaded by the first call): the device's free memory is unchanged
            assert torch.cuda.mem_get_info()[0] == free_before
        assert torch.cuda.memory_allocated() == torch_before
        rec = info.cpu().numpy()
        assert rec[0] == L.HCGB_OK
        O.hcore_gemm(2.0, oa, ob, 0.5, oc, O.CompressionParameters(acc, truncated_svd=True))
        if combo[2] == "C":
            assert nc.rank == gc.rank == rec[5], (combo, call, nc.rank, gc.rank, rec)
            assert abs(nc.rank - oc.rank) <= 1
            e_o = rel_fro(oc.to_dense(), exact)
            assert rel_fro(nc.to_dense(), exact) <= 2 * max(e_o, acc)
        else:
            assert rel_fro(nc.to_dense(), exact) < 1e-13
        assert rel_fro(nc.to_dense(), gc.to_dense()) <= 1e-12, (combo, call)


def test_noalloc_rejects_tiles_beyond_its_scratch():
    import torch
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300 import tiles as T
    rng = np.random.default_rng(0)
    # 1024 x 1024 tiles with capacity 341 need far more than the fixed scratch.
    u, v = rng.standard_normal((1024, 4)), rng.standard_normal((4, 1024))
    a = T.CompressedTile(1024, 1024, u, v, max_rank=341)
    b = T.CompressedTile(1024, 1024, u, v, max_rank=341)
    c = T.CompressedTile(1024, 1024, u, v, max_rank=341)
    rc = _noalloc(L, T, 1.0, a, b, 1.0, c, T.CompressionParameters(1e-8, truncated_svd=True))
    torch.cuda.synchronize()
    assert rc == L.HCGB_POOL_TOO_SMALL
    assert c.rank == 4  # untouched


def test_noalloc_rejects_tiles_beyond_shared_memory():
    """2048 x 2048 tiles of capacity 8 fit the scratch array (about 1 MB) but their QR panel does
    not fit a CTA's shared memory: rejected before any launch, C left as it was."""
    import torch
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300 import tiles as T
    rng = np.random.default_rng(1)
    u, v = rng.standard_normal((2048, 3)), rng.standard_normal((3, 2048))
    a = T.CompressedTile(2048, 2048, u, v, max_rank=8)
    b = T.CompressedTile(2048, 2048, u, v, max_rank=8)
    c = T.CompressedTile(2048, 2048, u, v, max_rank=8)
    before_u, before_v = c.u().copy(), c.v().copy()
    rc = _noalloc(L, T, 1.0, a, b, 1.0, c, T.CompressionParameters(1e-8, truncated_svd=True))
    torch.cuda.synchronize()
    assert rc == L.HCGB_POOL_TOO_SMALL
    assert c.rank == 3
    np.testing.assert_array_equal(c.u(), before_u)
    np.testing.assert_array_equal(c.v(), before_v)
