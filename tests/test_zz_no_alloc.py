"""hcgb_tile_gemm_noalloc: the tile update for callers that may not allocate device memory
(task-runtime workers whose runtime owns the device memory, or real-time callers that forbid
allocation after start-up).  It must give the same result as the allocating entry point
hcgb_tile_gemm, call after call, while using only the library's fixed scratch array.

This file is collected last on purpose: it runs after every other test, and also passes
alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import compressed_from_dense, rel_fro

pytestmark = pytest.mark.gpu


def _inputs(seed):
    from hcorepp_gb300.problems import KernelMatrix
    nb, acc = 256, 1e-8
    km = KernelMatrix(4 * nb, nb, 2, 0.1, seed)
    kc = KernelMatrix(4 * nb, nb, 2, 0.1, seed + 1)
    return (compressed_from_dense(km.tile(0, 1), acc), compressed_from_dense(km.tile(1, 3), acc),
            compressed_from_dense(kc.tile(0, 3), acc), km.tile(1, 1))


def _gpu(T, t):
    return T.CompressedTile(t.rows, t.cols, t.u, t.v, max_rank=t.max_rank)


def test_noalloc_matches_allocating_entry_point_twice():
    import torch
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300 import tiles as T
    assert torch.cuda.is_available()
    params = T.CompressionParameters(1e-8, truncated_svd=True)
    lib = L.lib()
    stream = torch.cuda.current_stream().cuda_stream
    for call, (seed, dense_a) in enumerate([(1, False), (3, True)]):
        oa, ob, oc, da = _inputs(seed)
        # existing entry point
        ga = T.DenseTile(da.shape[0], da.shape[1], da) if dense_a else _gpu(T, oa)
        gb, gc = _gpu(T, ob), _gpu(T, oc)
        T.HCore.Gemm(2.0, ga, 0, gb, 0, 0.5, gc, params)
        # the entry point that allocates nothing (same operands, fresh copy of C)
        na = T.DenseTile(da.shape[0], da.shape[1], da) if dense_a else _gpu(T, oa)
        nb_, nc = _gpu(T, ob), _gpu(T, oc)
        ta, tb, tc = na.c_tile(), nb_.c_tile(), nc.c_tile()
        p = params.c()
        info = torch.zeros(len(L.INFO_FIELDS), dtype=torch.int32, device="cuda")
        rc = lib.hcgb_tile_gemm_noalloc(2.0, C.byref(ta), C.byref(tb), 0.5, C.byref(tc), C.byref(p),
                                        C.c_void_p(stream), C.c_void_p(info.data_ptr()))
        assert rc == L.HCGB_OK, (call, rc)
        torch.cuda.synchronize()
        rec = info.cpu().numpy()
        assert rec[0] == L.HCGB_OK
        assert nc.rank == gc.rank == rec[5], (call, nc.rank, gc.rank, rec)
        ref = gc.to_dense()
        assert rel_fro(nc.to_dense(), ref) <= 1e-12, call


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
    ta, tb, tc = a.c_tile(), b.c_tile(), c.c_tile()
    p = T.CompressionParameters(1e-8, truncated_svd=True).c()
    rc = L.lib().hcgb_tile_gemm_noalloc(1.0, C.byref(ta), C.byref(tb), 1.0, C.byref(tc), C.byref(p),
                                        C.c_void_p(torch.cuda.current_stream().cuda_stream), None)
    assert rc == L.HCGB_POOL_TOO_SMALL
    assert c.rank == 4  # untouched
