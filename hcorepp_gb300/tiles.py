"""Host-side mirror of HCore++'s operator API for the TLR GEMM, over the C ABI.

Names, argument meaning and error behaviour follow the reference:
  CompressionParameters   include/hcorepp/operators/helpers/CompressionParameters.hpp:44-127
  DenseTile               include/hcorepp/operators/concrete/Dense.hpp:56-91
  CompressedTile          include/hcorepp/operators/concrete/Compressed.hpp:67-151, :169-246
  HCore.gemm              include/hcorepp/api/HCore.hpp:41-63 (src/api/HCore.cpp:23-344)
  TileMatrix              src/helpers/TileMatrix.cpp:17-185 (device-resident tile grid)
Device memory comes from torch (plumbing only); every computation is a libhcgb kernel.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib as L

MAX_RANK_RATIO = 3  # Compressed.hpp:14
GESVD, GESDD = 0, 1


@dataclass(frozen=True)
class CompressionParameters:
    """CompressionParameters(aAccuracy=1e-4, aUseTrmm=false, aUseUngqr=true, aTruncatedSvd=false,
    aFixedRank=0, aOpType=GESDD)."""
    accuracy: float = 1e-4
    use_trmm: bool = False
    use_ungqr: bool = True
    truncated_svd: bool = False
    fixed_rank: int = 0
    op_type: int = GESDD
    mode: int = L.PLAIN_FP64  # GB300 addition: HCGB_PLAIN_FP64, HCGB_MIXED, HCGB_TF32 or HCGB_BF16

    def c(self) -> L.Params:
        return L.make_params(self.accuracy, self.truncated_svd, self.fixed_rank, self.use_trmm, self.use_ungqr,
                             self.op_type, self.mode)


_CONTEXTS = {}


def run_context(device=None) -> L.Context:
    """The per-device context (ContextManager::GetContext's role), bound to torch's current stream."""
    dev = torch.cuda.current_device() if device is None else device
    ctx = _CONTEXTS.get(dev)
    if ctx is None:
        ctx = _CONTEXTS[dev] = L.Context(dev)
    ctx.set_stream(torch.cuda.current_stream(dev).cuda_stream)
    return ctx


def _fortran_flat(a) -> torch.Tensor:
    a = np.asarray(a, dtype=np.float64)
    return torch.from_numpy(np.ascontiguousarray(a.ravel(order="F")))


class DenseTile:
    """A dense rows x cols tile, column-major in device memory."""
    kind = L.DENSE

    def __init__(self, rows: int, cols: int, data=None, buffer: torch.Tensor | None = None, device="cuda"):
        self.rows, self.cols = rows, cols
        if buffer is not None:
            self.buffer = buffer
        else:
            self.buffer = torch.zeros(rows * cols, dtype=torch.float64, device=device)
            if data is not None:
                self.buffer.copy_(_fortran_flat(data))

    def c_tile(self) -> L.Tile:
        return L.Tile(self.buffer.data_ptr(), None, self.rows, self.cols, 0, L.DENSE)

    def to_dense(self) -> np.ndarray:
        return self.buffer.cpu().numpy().reshape((self.rows, self.cols), order="F")

    GetNumOfRows = lambda self: self.rows
    GetNumOfCols = lambda self: self.cols


class CompressedTile:
    """U (rows x rank) . V (rank x cols) in one buffer [U: rows x max_rank | V: max_rank x cols, ld rank].

    CompressedTile(rows, cols, u, v, rank) mirrors the (pointer, rank) constructor
    (Compressed.cpp:50-73): the capacity max_rank defaults to the rank, so the rank can
    never grow.  Pass max_rank to reserve room (the dense constructor uses min(m, n)/3).

    ``vt=True`` marks a tile of a Cholesky flow, whose V region holds W = V^T (cols x rank, ld
    cols) as HCore++'s Trsm, Syrk and Gemm(aCholesky = true) read it; the host accessors
    (``v``, ``w``, ``to_dense``, ``set_factors``) follow the mark, and those calls pass it on.
    """
    kind = L.COMPRESSED

    def __init__(self, rows: int, cols: int, u=None, v=None, rank: int | None = None, max_rank: int | None = None,
                 buffer: torch.Tensor | None = None, rank_buf: torch.Tensor | None = None, device="cuda",
                 vt: bool = False):
        self.rows, self.cols = rows, cols
        self.vt = vt
        if rank is None:
            rank = np.asarray(u).shape[1]
        self.max_rank = max_rank if max_rank is not None else rank
        if rank > self.max_rank:
            raise ValueError("rank exceeds the tile capacity")
        cap = rows * self.max_rank + self.max_rank * cols
        self.buffer = buffer if buffer is not None else torch.zeros(cap, dtype=torch.float64, device=device)
        self.rank_buf = rank_buf if rank_buf is not None else torch.zeros(1, dtype=torch.int32, device=device)
        if u is not None:
            self.set_factors(u, v)

    @classmethod
    def from_dense(cls, dense, params: "CompressionParameters", max_rank: int | None = None, device="cuda"):
        """CompressedTile(rows, cols, data, ld, params, ...) (Compressed.cpp:75-146) on the GPU:
        truncated SVD of the dense tile, rank clamped to max(min(rows, cols)/3, 1) unless
        max_rank is given."""
        d = torch.as_tensor(np.asfortranarray(np.asarray(dense, dtype=np.float64)).ravel(order="F"))
        rows, cols = np.asarray(dense).shape
        cap = max(min(rows, cols) // MAX_RANK_RATIO, 1) if max_rank is None else max_rank
        t = cls(rows, cols, rank=0, max_rank=cap, device=device)
        dd = d.to(device)
        ctx = run_context()
        p = params.c()
        r = C.c_int(0)
        tc = t.c_tile()
        ctx.check(L.lib().hcgb_compress_tile(ctx.handle, C.c_void_p(dd.data_ptr()), rows, cols, C.byref(tc),
                                             C.byref(p), C.byref(r)), allow=(L.HCGB_OK, L.HCGB_NOT_CONVERGED))
        return t

    @staticmethod
    def compress_batch(dense, out, params: "CompressionParameters") -> list:
        """Compress the dense device tiles ``dense`` (float64 tensors of rows x cols values in
        column-major order) into the compressed tiles ``out`` (same shape, their own capacities) with
        hcgb_compress_tiles: one batched pipeline launch per chunk, same rule per tile as from_dense.
        Returns the ranks."""
        n = len(dense)
        if n != len(out):
            raise ValueError("one output tile per dense tile")
        if n == 0:
            return []
        rows, cols = out[0].rows, out[0].cols
        for d, t in zip(dense, out):
            if d.dtype != torch.float64 or not d.is_cuda or d.numel() != rows * cols or not d.is_contiguous():
                raise ValueError("dense tiles: contiguous float64 device tensors of rows x cols values")
        ptrs = (C.c_void_p * n)(*[d.data_ptr() for d in dense])
        tiles = (L.Tile * n)(*[t.c_tile() for t in out])
        ranks = (C.c_int * n)()
        ctx = run_context()
        p = params.c()
        ctx.check(L.lib().hcgb_compress_tiles(ctx.handle, n, ptrs, rows, cols, tiles, C.byref(p), ranks),
                  allow=(L.HCGB_OK, L.HCGB_NOT_CONVERGED))
        return list(ranks)

    def set_factors(self, u, v):
        """Tile = u v (v: rank x cols); stored as W = v^T on a ``vt`` tile."""
        u = np.asarray(u, dtype=np.float64)
        v = np.asarray(v, dtype=np.float64)
        r = u.shape[1]
        if r > self.max_rank:
            raise ValueError("rank exceeds the tile capacity")
        self.buffer[:self.rows * r].copy_(_fortran_flat(u))
        o = self.rows * self.max_rank
        self.buffer[o:o + r * self.cols].copy_(_fortran_flat(v.T if self.vt else v))
        self.rank_buf.fill_(r)

    def c_tile(self, vt: bool | None = None) -> L.Tile:
        vt = self.vt if vt is None else vt
        return L.Tile(self.buffer.data_ptr(), self.rank_buf.data_ptr(), self.rows, self.cols, self.max_rank,
                      L.COMPRESSED_VT if vt else L.COMPRESSED)

    def GetTileRank(self) -> int:
        return int(self.rank_buf.item())

    rank = property(GetTileRank)

    def u(self) -> np.ndarray:
        r = self.rank
        return self.buffer[:self.rows * r].cpu().numpy().reshape((self.rows, r), order="F")

    def v(self) -> np.ndarray:
        """V (rank x cols) of tile = U V."""
        return self.w().T.copy() if self.vt else self._region(self.rank, self.cols)

    def w(self) -> np.ndarray:
        """W = V^T (cols x rank), the Cholesky-flow reading."""
        return self._region(self.cols, self.rank) if self.vt else self.v().T.copy()

    def _region(self, r, c) -> np.ndarray:
        o = self.rows * self.max_rank
        return self.buffer[o:o + r * c].cpu().numpy().reshape((r, c), order="F")

    def to_dense(self) -> np.ndarray:
        return self.u() @ self.v()

    GetNumOfRows = lambda self: self.rows
    GetNumOfCols = lambda self: self.cols


@dataclass(frozen=True)
class TileMetadata:
    """TileMetadata (include/hcorepp/operators/interface/Tile.hpp:30-52): everything a task runtime
    needs to move a tile but its buffer, which stays in device memory."""
    rows: int
    cols: int
    rank: int
    max_rank: int
    leading_dim: int
    layout: str  # "C" = column-major, the only layout of this path
    type: int    # L.DENSE or L.COMPRESSED


class TilePacker:
    """TilePacker<T> (include/hcorepp/operators/interface/TilePacker.hpp:17-60,
    src/operators/TilePacker.cpp:5-26)."""

    @staticmethod
    def UnPackTile(tile):
        """(metadata, buffer) of a tile; the buffer is the tile's own device memory (no copy)."""
        if tile.kind == L.DENSE:
            return TileMetadata(tile.rows, tile.cols, 0, 0, tile.rows, "C", L.DENSE), tile.buffer
        return (TileMetadata(tile.rows, tile.cols, tile.rank, tile.max_rank, tile.rows, "C", L.COMPRESSED),
                tile.buffer)

    @staticmethod
    def PackTile(meta: TileMetadata, buffer: torch.Tensor):
        """A tile over ``buffer`` described by ``meta`` (no copy)."""
        if meta.layout != "C" or meta.leading_dim != meta.rows:
            raise ValueError("PackTile: column-major metadata with leading dimension = rows expected")
        if meta.type == L.DENSE:
            if buffer.numel() < meta.rows * meta.cols:
                raise ValueError("PackTile: buffer smaller than the dense tile")
            return DenseTile(meta.rows, meta.cols, buffer=buffer)
        if meta.rank > meta.max_rank or buffer.numel() < meta.max_rank * (meta.rows + meta.cols):
            raise ValueError("PackTile: rank above capacity or buffer smaller than the compressed tile")
        t = CompressedTile(meta.rows, meta.cols, rank=0, max_rank=meta.max_rank, buffer=buffer, device=buffer.device)
        t.rank_buf.fill_(meta.rank)
        return t

    unpack = UnPackTile
    pack = PackTile


class HCore:
    """HCore<double> (include/hcorepp/api/HCore.hpp:41-63)."""

    @staticmethod
    def Gemm(alpha, a, a_op, b, b_op, beta, c, params: CompressionParameters = CompressionParameters(1e-9),
             cholesky: bool = False):
        """C = alpha op(A) op(B) + beta C; returns the reference's flop count for the update.

        ``cholesky=True`` is the aCholesky branch (HCore.cpp:160-174, Compressed.cpp:273-276,
        :529-595, :669-673): A, B and C compressed with their V regions read and written as W = V^T,
        op(A) = NoTrans, op(B) = Trans.  The reference's branch produces no meaningful result for
        any other combination, so the mirror rejects them."""
        ctx = run_context()
        if cholesky:
            if not (a.kind == b.kind == c.kind == L.COMPRESSED) or a_op != L.NOTRANS or b_op != L.TRANS:
                raise ValueError("Gemm(aCholesky): compressed A, B, C with opA = NoTrans, opB = Trans only")
            ta, tb, tc = a.c_tile(vt=True), b.c_tile(vt=True), c.c_tile(vt=True)
        else:
            ta, tb, tc = a.c_tile(), b.c_tile(), c.c_tile()
        p = params.c()
        nr = C.c_int(0)
        fl = C.c_ulonglong(0)
        rc = L.lib().hcgb_tile_gemm(ctx.handle, float(alpha), C.byref(ta), int(a_op), C.byref(tb), int(b_op),
                                    float(beta), C.byref(tc), C.byref(p), C.byref(nr), C.byref(fl))
        ctx.check(rc, allow=(L.HCGB_OK, L.HCGB_NOT_CONVERGED))
        if c.kind == L.COMPRESSED and ta.kind == L.DENSE and tb.kind == L.DENSE:
            c.max_rank = min(c.rows, c.cols)  # DDC re-sets the tile at full rank (HCore.cpp:294-298)
        return fl.value

    gemm = Gemm


def _dptr(t: torch.Tensor):
    return C.c_void_p(t.data_ptr())


class Blas:
    """Dense per-tile building blocks on the GPU (HCoreKernels<T>::potrf / trsm / syrk)."""

    @staticmethod
    def potrf(uplo: int, n: int, a: torch.Tensor, lda: int) -> int:
        ctx = run_context()
        info = C.c_int(0)
        ctx.check(L.lib().hcgb_potrf(ctx.handle, int(uplo), int(n), _dptr(a), int(lda), C.byref(info)))
        return info.value

    @staticmethod
    def trsm(side, uplo, trans, diag, m, n, alpha, a: torch.Tensor, lda, b: torch.Tensor, ldb):
        ctx = run_context()
        ctx.check(L.lib().hcgb_trsm(ctx.handle, int(side), int(uplo), int(trans), int(diag), int(m), int(n),
                                    float(alpha), _dptr(a), int(lda), _dptr(b), int(ldb)))

    @staticmethod
    def syrk(uplo, trans, n, k, alpha, a: torch.Tensor, lda, beta, c: torch.Tensor, ldc):
        ctx = run_context()
        ctx.check(L.lib().hcgb_syrk(ctx.handle, int(uplo), int(trans), int(n), int(k), float(alpha), _dptr(a),
                                    int(lda), float(beta), _dptr(c), int(ldc)))


def Potrf(a: DenseTile, uplo: int = L.LOWER) -> int:
    """HCore<T>::Potrf (src/api/HCore.cpp:585-621): dense tiles only."""
    if a.kind != L.DENSE:
        raise RuntimeError(" Potrf works only with dense tiles")
    return Blas.potrf(uplo, a.rows, a.buffer, a.rows)


def Trsm(side, uplo, trans, diag, alpha, a: DenseTile, b: CompressedTile):
    """HCore<T>::Trsm (src/api/HCore.cpp:623-647) with the reference's arguments: the solve runs on
    the V buffer of the compressed B viewed as a rows x rank matrix with leading dimension rows."""
    if b.kind != L.COMPRESSED:
        raise RuntimeError(" TRSM: Tile B must be compressed ")
    r = b.rank
    v = b.buffer[b.rows * b.max_rank:]
    Blas.trsm(side, uplo, trans, diag, b.rows, r, alpha, a.buffer, a.rows, v, b.rows)


def Syrk(alpha, a, a_op, uplo, beta, c: DenseTile, params=None):
    """HCore<T>::Syrk (src/api/HCore.cpp:482-583) for a dense C.  Dense A: dsyrk on the uplo
    triangle.  Compressed A, its V region read as W (cols x rank, ld cols) so that A = U W^T:
    C <- beta C - U (W^T W) U^T (the reference hard-codes -1 there), then the other strict triangle
    is set to zero (FillMatrixTriangle, HCore.cpp:555-563)."""
    if c.kind != L.DENSE:
        raise NotImplementedError("Syrk into a compressed C is not provided")
    n = c.rows
    if a.kind == L.DENSE:
        Blas.syrk(uplo, a_op, n, c.cols, alpha, a.buffer, a.rows, beta, c.buffer, n)
        return
    # A = U W^T (Cholesky-flow reading, HCore.cpp:512-545): C <- beta C - A A^T
    ctx = run_context()
    ta, tc = a.c_tile(vt=True), c.c_tile()
    p = (params or CompressionParameters(1e-9)).c()
    ctx.check(L.lib().hcgb_tile_gemm(ctx.handle, -1.0, C.byref(ta), L.NOTRANS, C.byref(ta), L.TRANS, float(beta),
                                     C.byref(tc), C.byref(p), None, None), allow=(L.HCGB_OK, L.HCGB_NOT_CONVERGED))
    other = L.UPPER if uplo == L.LOWER else L.LOWER
    ctx.check(L.lib().hcgb_fill_triangle(ctx.handle, other, n, _dptr(c.buffer), n, 0.0))


def tile_cholesky(a: "TileMatrix", params: CompressionParameters, batched: bool = True,
                  info: torch.Tensor | None = None) -> int:
    """Right-looking tile Cholesky A = L L^T of a symmetric positive definite tile matrix: dense
    diagonal tiles, compressed tiles below the diagonal in the Cholesky-flow layout (TileMatrix with
    ``vt=True``: tile = U W^T), tiles above the diagonal not referenced.

    ``batched=True``: hcgb_tile_cholesky, one panel-solve launch and batched trailing updates per
    step (``info``, optional, from ``info_buffer(nt*(nt*nt-1)//6)``, gets the update records).
    ``batched=False``: the reference's per-tile operations called one by one; the reference provides
    them but no driver, and this loop composes them:
      Potrf(A_kk, Lower)                                                  HCore.cpp:585-621
      Trsm(Left, Lower, NoTrans, NonUnit, 1, A_kk, A_ik): W_ik <- L_kk^-1 W_ik   HCore.cpp:623-647
      Syrk(-1, A_ik, NoTrans, Lower, 1, A_ii)                             HCore.cpp:482-583
      Gemm(-1, A_ik, NoTrans, A_jk, Trans, 1, A_ij, aCholesky = true)     HCore.cpp:23-344
    One call per tile operation, each a GPU kernel sequence on the context stream.
    Returns 0, or k * nb + info of the first failing diagonal tile."""
    if not a.vt:
        raise ValueError("tile_cholesky needs a TileMatrix in the Cholesky-flow layout (vt=True)")
    nt, nb = a.mt, a.nb
    if batched:
        ctx = run_context()
        grid = a.c_grid()
        p = params.c()
        res = C.c_int(0)
        sp = C.c_void_p(info.data_ptr()) if info is not None else None
        ctx.check(L.lib().hcgb_tile_cholesky(ctx.handle, nt, grid, C.byref(p), C.byref(res), sp))
        return res.value
    for k in range(nt):
        akk = a.tile(k, k)
        info = Potrf(akk, L.LOWER)
        if info:
            return k * nb + info
        for i in range(k + 1, nt):
            Trsm(L.LEFT, L.LOWER, L.NOTRANS, L.NONUNIT, 1.0, akk, a.tile(i, k))
        for i in range(k + 1, nt):
            aik = a.tile(i, k)
            Syrk(-1.0, aik, L.NOTRANS, L.LOWER, 1.0, a.tile(i, i), params)
            for j in range(k + 1, i):
                HCore.Gemm(-1.0, aik, L.NOTRANS, a.tile(j, k), L.TRANS, 1.0, a.tile(i, j), params, cholesky=True)
    return 0


class TileMatrix:
    """A grid of mt x nt tiles of nb x nb, resident in one device arena.

    ``kinds[i][j]`` is DENSE or COMPRESSED; compressed tiles get capacity ``max_rank``.
    Ranks live in one device int array (``ranks``), so a whole multiply runs without the host.
    ``vt=True`` lays the compressed tiles out for a Cholesky flow (V region = W = V^T).
    A kind of ``None`` is a tile that is never referenced (the upper triangle of a Cholesky
    factor): it holds no storage and its descriptor has no data pointer.
    """

    def __init__(self, mt: int, nt: int, nb: int, kinds, max_rank: int, device="cuda", vt: bool = False):
        self.mt, self.nt, self.nb, self.max_rank = mt, nt, nb, max_rank
        self.vt = vt
        self.kinds = [[kinds[i][j] for j in range(nt)] for i in range(mt)]
        sizes = []
        for j in range(nt):
            for i in range(mt):
                kind = self.kinds[i][j]
                sizes.append(0 if kind is None else nb * nb if kind == L.DENSE else 2 * nb * max_rank)
        self.offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        self.arena = torch.zeros(int(self.offsets[-1]), dtype=torch.float64, device=device)
        self.ranks = torch.zeros(mt * nt, dtype=torch.int32, device=device)

    def index(self, i, j):
        return i + j * self.mt

    def _view(self, i, j):
        idx = self.index(i, j)
        return self.arena[int(self.offsets[idx]):int(self.offsets[idx + 1])]

    def tile(self, i, j):
        nb = self.nb
        idx = self.index(i, j)
        if self.kinds[i][j] is None:
            raise ValueError(f"tile ({i}, {j}) is not stored")
        if self.kinds[i][j] == L.DENSE:
            return DenseTile(nb, nb, buffer=self._view(i, j))
        return CompressedTile(nb, nb, rank=0, max_rank=self.max_rank, buffer=self._view(i, j),
                              rank_buf=self.ranks[idx:idx + 1], vt=self.vt)

    def c_grid(self):
        """The tile descriptors (device pointers into the arena and the rank array, which never move),
        built once and reused."""
        cached = getattr(self, "_grid", None)
        if cached is not None:
            return cached
        self._grid = self._build_grid()
        return self._grid

    def _build_grid(self):
        nb = self.nb
        arr = (L.Tile * (self.mt * self.nt))()
        base = self.arena.data_ptr()
        rbase = self.ranks.data_ptr()
        for j in range(self.nt):
            for i in range(self.mt):
                idx = self.index(i, j)
                ptr = base + 8 * int(self.offsets[idx])
                if self.kinds[i][j] is None:
                    arr[idx] = L.Tile(None, None, nb, nb, 0, L.DENSE)
                elif self.kinds[i][j] == L.DENSE:
                    arr[idx] = L.Tile(ptr, None, nb, nb, 0, L.DENSE)
                else:
                    arr[idx] = L.Tile(ptr, rbase + 4 * idx, nb, nb, self.max_rank,
                                      L.COMPRESSED_VT if self.vt else L.COMPRESSED)
        return arr

    # ---- rank-trimmed transfer format (hcgb_pack_tiles): tiles in index order (i + j * mt), each
    #      dense tile nb x nb, each compressed tile U (nb x rank) then its V region (rank * nb values)
    def pack(self, packed: torch.Tensor, offsets: torch.Tensor, ctx: L.Context | None = None):
        """Pack the used part of every tile into the device buffer `packed` (float64, at least
        ``self.arena.numel()`` values); `offsets` (int64, mt * nt + 1, device) receives each tile's
        start and the total.  Asynchronous on torch's current stream."""
        ctx = ctx or run_context()
        grid = self.c_grid()
        ctx.check(L.lib().hcgb_pack_tiles(ctx.handle, self.mt * self.nt, grid, _dptr(packed), _dptr(offsets)))

    def unpack(self, packed: torch.Tensor, offsets: torch.Tensor, ctx: L.Context | None = None):
        """Inverse of pack; ``self.ranks`` must already hold the packed tiles' ranks."""
        ctx = ctx or run_context()
        grid = self.c_grid()
        ctx.check(L.lib().hcgb_unpack_tiles(ctx.handle, self.mt * self.nt, grid, _dptr(packed), _dptr(offsets)))

    def host_pack(self, arena: np.ndarray, ranks: np.ndarray) -> np.ndarray:
        """The same format built on the host from a host copy of the arena and the ranks."""
        nb = self.nb
        parts = []
        for idx in range(self.mt * self.nt):
            i, j = idx % self.mt, idx // self.mt
            o = int(self.offsets[idx])
            if self.kinds[i][j] is None:
                continue
            if self.kinds[i][j] == L.DENSE:
                parts.append(arena[o:o + nb * nb])
            else:
                r = int(ranks[idx])
                parts.append(arena[o:o + nb * r])
                vo = o + nb * self.max_rank
                parts.append(arena[vo:vo + r * nb])
        return np.concatenate(parts) if parts else np.zeros(0)

    def set_tile(self, i, j, dense=None, u=None, v=None):
        t = self.tile(i, j)
        if self.kinds[i][j] == L.DENSE:
            t.buffer.copy_(_fortran_flat(dense))
        else:
            t.set_factors(u, v)

    def to_dense(self) -> np.ndarray:
        nb = self.nb
        out = np.zeros((self.mt * nb, self.nt * nb))
        arena = self.arena.cpu().numpy()
        ranks = self.ranks.cpu().numpy()
        for j in range(self.nt):
            for i in range(self.mt):
                idx = self.index(i, j)
                seg = arena[self.offsets[idx]:self.offsets[idx + 1]]
                if self.kinds[i][j] is None:
                    continue
                if self.kinds[i][j] == L.DENSE:
                    blk = seg.reshape((nb, nb), order="F")
                else:
                    r = int(ranks[idx])
                    u = seg[:nb * r].reshape((nb, r), order="F")
                    vreg = seg[nb * self.max_rank:nb * self.max_rank + r * nb]
                    v = vreg.reshape((nb, r), order="F").T if self.vt else vreg.reshape((r, nb), order="F")
                    blk = u @ v
                out[i * nb:(i + 1) * nb, j * nb:(j + 1) * nb] = blk
        return out

    def to_dense_device(self) -> torch.Tensor:
        """The whole matrix as one dense device tensor (U V of every compressed tile), for accuracy
        checks of large grids without a host round trip of the dense matrix."""
        nb = self.nb
        out = torch.zeros((self.mt * nb, self.nt * nb), dtype=torch.float64, device=self.arena.device)
        ranks = self.ranks.cpu().numpy()
        for j in range(self.nt):
            for i in range(self.mt):
                idx = self.index(i, j)
                o = int(self.offsets[idx])
                dst = out[i * nb:(i + 1) * nb, j * nb:(j + 1) * nb]
                if self.kinds[i][j] is None:
                    continue
                if self.kinds[i][j] == L.DENSE:
                    dst.copy_(self.arena[o:o + nb * nb].view(nb, nb).t())
                    continue
                r = int(ranks[idx])
                if r == 0:
                    continue
                u = self.arena[o:o + nb * r].view(r, nb).t()
                vo = o + nb * self.max_rank
                vreg = self.arena[vo:vo + r * nb]
                v = vreg.view(r, nb) if self.vt else vreg.view(nb, r).t()
                dst.copy_(u @ v)
        return out

    def rank_grid(self) -> np.ndarray:
        return self.ranks.cpu().numpy().reshape((self.nt, self.mt)).T.copy()


def info_buffer(n_updates: int, device="cuda") -> torch.Tensor:
    """Device buffer for n hcgb_update_info records (int32, 8 fields each)."""
    return torch.zeros((n_updates, len(L.INFO_FIELDS)), dtype=torch.int32, device=device)


def tlr_gemm(alpha: float, a: TileMatrix, b: TileMatrix, beta: float, c: TileMatrix,
             params: CompressionParameters, info: torch.Tensor | None = None, ctx: L.Context | None = None):
    """C = alpha A B + beta C over tile grids (examples/matrix_multiplication/omp_main.cpp:112-124).

    Asynchronous on torch's current stream.  ``info`` (optional, from ``info_buffer(mt*nt*kt)``)
    receives the per-update records (status, input ranks, k, new rank, sweeps, side); the
    record of update (i, j, k) is row k*mt*nt + i + j*mt."""
    ctx = ctx or run_context()
    if a.nt != b.mt or a.mt != c.mt or b.nt != c.nt:
        raise ValueError("tile grids do not conform")
    ga, gb, gc = a.c_grid(), b.c_grid(), c.c_grid()
    p = params.c()
    sp = C.c_void_p(info.data_ptr()) if info is not None else None
    rc = L.lib().hcgb_tlr_gemm(ctx.handle, c.mt, c.nt, a.nt, float(alpha), ga, gb, float(beta), gc, C.byref(p), sp)
    ctx.check(rc)
