"""ctypes access to oracle/_ref/libhcref.so (the reference's own CPU path, built by
oracle/build_ref.py).  Test infrastructure only.  ``available()`` is False when the
library has not been built (for example on a machine without the reference sources).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import hcore_oracle as O

_LIB = None
_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "libhcref.so")

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)


def available() -> bool:
    """Built here and loadable on this machine (the x86 build does not load on an Arm host)."""
    if not os.path.exists(_PATH):
        return False
    try:
        lib()
    except OSError:
        return False
    return True


def lib():
    global _LIB
    if _LIB is None:
        L = C.CDLL(_PATH)
        L.hcref_compress.restype = C.c_int
        L.hcref_compress.argtypes = [C.c_int, C.c_int, dp, C.c_double, C.c_int, C.c_int, C.c_int, dp, ip]
        L.hcref_tile_gemm.restype = C.c_int
        L.hcref_tile_gemm.argtypes = ([C.c_double] + [C.c_int] * 5 + [dp] + [C.c_int] * 5 + [dp] + [C.c_double]
                                      + [C.c_int] * 3 + [ip, C.c_int, dp, C.c_double, C.c_int, C.c_int, C.c_int,
                                                         C.POINTER(C.c_ulonglong)])
        L.hcref_tlr_gemm.restype = C.c_double
        L.hcref_tlr_gemm.argtypes = ([C.c_int, C.c_int, C.c_double, C.c_double]
                                     + [ip, ip, ip, C.POINTER(dp)] * 2
                                     + [ip, ip, ip, C.POINTER(dp), ip, C.c_int, C.c_double, C.c_int, C.c_int,
                                        C.c_int, C.c_int, ip])
        L.hcref_tile_gemm_ops.restype = C.c_int
        L.hcref_tile_gemm_ops.argtypes = ([C.c_double] + [C.c_int] * 5 + [dp, C.c_int] + [C.c_int] * 5
                                          + [dp, C.c_int, C.c_double] + [C.c_int] * 3
                                          + [ip, C.c_int, dp, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int])
        L.hcref_potrf.restype = C.c_int
        L.hcref_potrf.argtypes = [C.c_int, C.c_int, dp]
        L.hcref_trsm.restype = C.c_int
        L.hcref_trsm.argtypes = [C.c_int] * 4 + [C.c_double, C.c_int, dp] + [C.c_int] * 4 + [dp]
        L.hcref_syrk.restype = C.c_int
        L.hcref_syrk.argtypes = ([C.c_double] + [C.c_int] * 5 + [dp] + [C.c_int] * 2
                                 + [C.c_double, C.c_int, C.c_int, dp])
        L.hcref_set_blas_threads.argtypes = [C.c_int]
        _LIB = L
    return _LIB


def _ptr(a):
    return a.ctypes.data_as(dp)


class RefTile:
    """A tile in the reference's buffer layout (see ref_driver.cpp)."""

    def __init__(self, kind, rows, cols, rank, max_rank, buf):
        self.kind, self.rows, self.cols, self.rank, self.max_rank = kind, rows, cols, rank, max_rank
        self.buf = buf

    @classmethod
    def dense(cls, a):
        a = np.asfortranarray(a, dtype=np.float64)
        return cls(0, a.shape[0], a.shape[1], 0, 0, a.ravel(order="F").copy())

    @classmethod
    def compressed(cls, u, v, max_rank):
        m, r = u.shape
        n = v.shape[1]
        buf = np.zeros(m * max_rank + max_rank * n)
        buf[:m * r] = np.asarray(u).ravel(order="F")
        buf[m * max_rank:m * max_rank + r * n] = np.asarray(v).ravel(order="F")
        return cls(1, m, n, r, max_rank, buf)

    @classmethod
    def from_oracle(cls, t):
        if t.kind == "dense":
            return cls.dense(t.data)
        return cls.compressed(t.u, t.v, t.max_rank)

    def u(self):
        return self.buf[:self.rows * self.rank].reshape((self.rows, self.rank), order="F")

    def v(self):
        o = self.rows * self.max_rank
        return self.buf[o:o + self.rank * self.cols].reshape((self.rank, self.cols), order="F")

    def w(self):
        """The V region read as HCore++'s Cholesky routines read it: cols x rank, ld cols."""
        o = self.rows * self.max_rank
        return self.buf[o:o + self.rank * self.cols].reshape((self.cols, self.rank), order="F")

    @classmethod
    def cholesky(cls, u, w, max_rank):
        """A compressed tile holding U and W (tile = U W^T) in the buffer."""
        m, r = u.shape
        n = w.shape[0]
        buf = np.zeros(m * max_rank + max_rank * n)
        buf[:m * r] = np.asarray(u).ravel(order="F")
        buf[m * max_rank:m * max_rank + r * n] = np.asarray(w).ravel(order="F")
        return cls(1, m, n, r, max_rank, buf)

    def to_dense(self):
        if self.kind == 0:
            return self.buf.reshape((self.rows, self.cols), order="F").copy()
        return self.u() @ self.v()


def compress(dense, params: O.CompressionParameters) -> RefTile:
    m, n = dense.shape
    maxr = max(min(m, n) // O.MAX_RANK_RATIO, 1)
    out = np.zeros(m * maxr + maxr * n)
    mr = C.c_int(0)
    d = np.asfortranarray(dense, dtype=np.float64).ravel(order="F").copy()
    r = lib().hcref_compress(m, n, _ptr(d), params.accuracy, int(params.truncated_svd), params.fixed_rank,
                             params.op_type, _ptr(out), C.byref(mr))
    if r < 0:
        raise RuntimeError("hcref_compress failed")
    return RefTile(1, m, n, r, mr.value, out)


def tile_gemm(alpha, a: RefTile, b: RefTile, beta, c: RefTile, params: O.CompressionParameters) -> int:
    rk = C.c_int(c.rank)
    fl = C.c_ulonglong(0)
    rc = lib().hcref_tile_gemm(alpha, a.kind, a.rows, a.cols, a.rank, a.max_rank, _ptr(a.buf),
                               b.kind, b.rows, b.cols, b.rank, b.max_rank, _ptr(b.buf), beta,
                               c.kind, c.rows, c.cols, C.byref(rk), c.max_rank, _ptr(c.buf),
                               params.accuracy, int(params.truncated_svd), params.fixed_rank, params.op_type,
                               C.byref(fl))
    if rc != 0:
        raise RuntimeError("hcref_tile_gemm failed")
    c.rank = rk.value
    return fl.value


def tlr_gemm(nt, nb, alpha, beta, a_tiles, b_tiles, c_tiles, params, c_list=None, nthreads=1):
    """Tile grids are dicts/lists indexed [i][j]; returns (seconds, errors).  Updates c_tiles in place."""
    def pack(tiles):
        flat = [tiles[idx % nt][idx // nt] for idx in range(nt * nt)]
        kind = np.array([t.kind for t in flat], dtype=np.int32)
        rank = np.array([t.rank for t in flat], dtype=np.int32)
        maxr = np.array([t.max_rank for t in flat], dtype=np.int32)
        ptrs = (dp * (nt * nt))(*[_ptr(t.buf) for t in flat])
        return flat, kind, rank, maxr, ptrs

    af, ak, ar, am, ap = pack(a_tiles)
    bf, bk, br, bm, bp = pack(b_tiles)
    cf, ck, cr, cm, cp = pack(c_tiles)
    if c_list is None:
        c_list = list(range(nt * nt))
    cl = np.array(c_list, dtype=np.int32)
    err = C.c_int(0)
    L = lib()
    L.hcref_set_blas_threads(1)
    secs = L.hcref_tlr_gemm(nt, nb, alpha, beta,
                            ak.ctypes.data_as(ip), ar.ctypes.data_as(ip), am.ctypes.data_as(ip), ap,
                            bk.ctypes.data_as(ip), br.ctypes.data_as(ip), bm.ctypes.data_as(ip), bp,
                            ck.ctypes.data_as(ip), cr.ctypes.data_as(ip), cm.ctypes.data_as(ip), cp,
                            cl.ctypes.data_as(ip), len(cl), params.accuracy, int(params.truncated_svd),
                            params.fixed_rank, params.op_type, nthreads, C.byref(err))
    for idx in range(nt * nt):
        cf[idx].rank = int(cr[idx])
    return secs, err.value


def tile_gemm_ops(alpha, a: RefTile, op_a, b: RefTile, op_b, beta, c: RefTile, params: O.CompressionParameters,
                  cholesky=False) -> None:
    rk = C.c_int(c.rank)
    rc = lib().hcref_tile_gemm_ops(alpha, a.kind, a.rows, a.cols, a.rank, a.max_rank, _ptr(a.buf), int(op_a),
                                   b.kind, b.rows, b.cols, b.rank, b.max_rank, _ptr(b.buf), int(op_b), beta,
                                   c.kind, c.rows, c.cols, C.byref(rk), c.max_rank, _ptr(c.buf),
                                   params.accuracy, int(params.truncated_svd), params.fixed_rank, params.op_type,
                                   int(cholesky))
    if rc != 0:
        raise RuntimeError("hcref_tile_gemm_ops failed")
    c.rank = rk.value


def potrf(uplo, a: RefTile) -> None:
    if lib().hcref_potrf(int(uplo), a.rows, _ptr(a.buf)) != 0:
        raise RuntimeError("hcref_potrf failed")


def trsm(side, uplo, trans, diag, alpha, a: RefTile, b: RefTile) -> None:
    if lib().hcref_trsm(int(side), int(uplo), int(trans), int(diag), alpha, a.rows, _ptr(a.buf), b.rows, b.cols,
                        b.rank, b.max_rank, _ptr(b.buf)) != 0:
        raise RuntimeError("hcref_trsm failed")


def syrk(alpha, a: RefTile, op_a, uplo, beta, c: RefTile) -> None:
    if lib().hcref_syrk(alpha, a.kind, a.rows, a.cols, a.rank, a.max_rank, _ptr(a.buf), int(op_a), int(uplo), beta,
                        c.rows, c.cols, _ptr(c.buf)) != 0:
        raise RuntimeError("hcref_syrk failed")
