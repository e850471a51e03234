"""CPU oracle: a numpy/LAPACK restatement of HCore++'s CPU path for the TLR GEMM.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this module, and only to check results
(or as the timed CPU baseline); the GPU product never routes through it.

Every function restates one function of the reference's CPU backend
(``src/kernels/omp/kernels.cpp``, which forwards to BLAS++/LAPACK++) or of the
operator/API layers above it, calling the same LAPACK routines (dgeqrf, dorgqr,
dgesdd/dgesvd) through ``scipy.linalg.lapack``.  Matrices are numpy arrays in
their logical shape; the reference's column-major leading-dimension bookkeeping
is kept only where it changes the arithmetic.

Parity pins: ``tests/test_oracle_golden.py`` checks these functions against the
known-answer vectors of the reference's tests (tests/kernels/TestKernels.cpp,
tests/operators/TestCompressedTile.cpp, tests/api/TestGemm.cpp) and, when
``oracle/_ref`` has been built, against the reference's own C++ compiled here.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.linalg.lapack as lapack

MAX_RANK_RATIO = 3  # include/hcorepp/operators/concrete/Compressed.hpp:14

GESVD, GESDD = 0, 1  # include/hcorepp/common/Definitions.hpp CompressionType


@dataclass(frozen=True)
class CompressionParameters:
    """include/hcorepp/operators/helpers/CompressionParameters.hpp:44-46 (defaults kept)."""
    accuracy: float = 1e-4
    use_trmm: bool = False
    use_ungqr: bool = True
    truncated_svd: bool = False
    fixed_rank: int = 0
    op_type: int = GESDD


# ---------------------------------------------------------------------------
# L1 kernels (src/kernels/omp/kernels.cpp)
# ---------------------------------------------------------------------------

def multiply_by_alpha(array: np.ndarray, rows: int, cols: int, m: int, rank: int, alpha: float) -> None:
    """omp/kernels.cpp:22-28: ``array[m*rank + i] *= alpha`` for i < rows*cols (flat, in place)."""
    array[m * rank:m * rank + rows * cols] *= alpha


def process_vpointer(n: int, c_rank: int, ungqr: bool, vm: int, beta: float, cv: np.ndarray,
                     ld_cv: int, v: np.ndarray, a_rank: int, b_data: np.ndarray) -> None:
    """omp/kernels.cpp:31-79 (non-Cholesky branch), flat column-major buffers, in place.

    Writes ``V[j + i*vm] = beta*CV[i + j*ld_cv]`` (i < c_rank) and
    ``V[n*c_rank + j + i*vm] = B[i + j*a_rank]`` (i < a_rank) for j < n.
    """
    for j in range(n):
        for i in range(c_rank):
            v[j + i * vm] = beta * cv[i + j * ld_cv]
    base = n * c_rank
    for j in range(n):
        for i in range(a_rank):
            v[base + j + i * vm] = b_data[i + j * a_rank]


def calculate_new_rank(truncated_svd: bool, sigma: np.ndarray, size_s: int, accuracy: float) -> int:
    """omp/kernels.cpp:82-104: first i >= 1 with sigma_i below the threshold, else size_s."""
    new_rank = size_s
    if truncated_svd:
        thr = accuracy * sigma[0]
    else:
        thr = accuracy
    for i in range(1, size_s):
        if sigma[i] < thr:
            return i
    return new_rank


def calculate_uvptr(rank: int, vm: int, uvptr: np.ndarray, vnew: np.ndarray) -> None:
    """omp/kernels.cpp:106-114: ``UVptr[j + i*rank] = Vnew[i + j*vm]`` (flat, in place)."""
    for j in range(rank):
        for i in range(vm):
            uvptr[j + i * rank] = vnew[i + j * vm]


def calculate_vtnew(rk_new: int, ungqr: bool, min_vm_vn: int, sigma: np.ndarray, vtnew: np.ndarray,
                    size_s: int, vm: int) -> None:
    """omp/kernels.cpp:116-130: scale row i < rk_new of VTnew (ld size_s) by sigma_i (flat, in place).

    With ungqr the row has min_vm_vn entries, otherwise vm entries (conj is a no-op for reals).
    """
    count = min_vm_vn if ungqr else vm
    for i in range(rk_new):
        vtnew[i:i + count * size_s:size_s] *= sigma[i]


def geqrf(a: np.ndarray):
    """omp/kernels.cpp:161-166 -> LAPACK dgeqrf.  Returns (factored a, tau)."""
    qr, tau, _work, info = lapack.dgeqrf(np.asfortranarray(a, dtype=np.float64))
    if info != 0:
        raise RuntimeError(f"dgeqrf info={info}")
    return qr, tau


def svd(a: np.ndarray, op_type: int):
    """omp/kernels.cpp:182-192: gesvd or gesdd with 'S' (economy) vectors."""
    a = np.asfortranarray(a, dtype=np.float64)
    if op_type == GESVD:
        u, s, vt, info = lapack.dgesvd(a, compute_uv=1, full_matrices=0)
    else:
        u, s, vt, info = lapack.dgesdd(a, compute_uv=1, full_matrices=0)
    if info != 0:
        raise RuntimeError(f"svd info={info}")
    return u, s, vt


def ungqr(qr: np.ndarray, tau: np.ndarray, ncols: int) -> np.ndarray:
    """omp/kernels.cpp:218-223 -> LAPACK dorgqr: the first ncols columns of Q."""
    q, _work, info = lapack.dorgqr(np.asfortranarray(qr[:, :ncols]), tau[:ncols])
    if info != 0:
        raise RuntimeError(f"dorgqr info={info}")
    return q


# ---------------------------------------------------------------------------
# L3 operators
# ---------------------------------------------------------------------------

class DenseTile:
    """src/operators/concrete/Dense.cpp: a dense rows x cols tile."""
    kind = "dense"

    def __init__(self, data: np.ndarray):
        self.data = np.array(data, dtype=np.float64, order="F")

    @property
    def rows(self):
        return self.data.shape[0]

    @property
    def cols(self):
        return self.data.shape[1]

    def to_dense(self) -> np.ndarray:
        return self.data.copy()

    def gemm(self, alpha: float, a: np.ndarray, b: np.ndarray, beta: float) -> None:
        """Dense.cpp:46-108 (column-major, no transposes left after HCore's dispatch)."""
        self.data = np.asfortranarray(alpha * (a @ b) + beta * self.data)


class CompressedTile:
    """src/operators/concrete/Compressed.cpp: ``U (rows x rank) . V (rank x cols)``.

    ``max_rank`` is the capacity of the tile buffer; the rank can never grow past it
    (Compressed.cpp:526-527).
    """
    kind = "compressed"

    def __init__(self, u: np.ndarray, v: np.ndarray, max_rank: int | None = None):
        self.u = np.array(u, dtype=np.float64, order="F")
        self.v = np.array(v, dtype=np.float64, order="F")
        self.max_rank = self.rank if max_rank is None else max_rank

    @classmethod
    def from_uv(cls, rows: int, cols: int, uv: np.ndarray, rank: int) -> "CompressedTile":
        """Compressed.cpp:50-73: packed ``[U (rows*rank) | V (rank*cols)]``; max_rank = rank."""
        uv = np.asarray(uv, dtype=np.float64).ravel(order="F")
        u = uv[:rows * rank].reshape((rows, rank), order="F")
        v = uv[rows * rank:rows * rank + rank * cols].reshape((rank, cols), order="F")
        return cls(u, v, max_rank=rank)

    @classmethod
    def from_dense(cls, dense: np.ndarray, params: CompressionParameters,
                   max_rank: int | None = None) -> "CompressedTile":
        """Compressed.cpp:75-146: truncated SVD of a dense tile; max_rank = max(min(m,n)/3, 1) (the
        reference's clamp, Compressed.cpp:83) unless a capacity is given (no counterpart in the
        reference: the capacity-nb runs of a tile Cholesky)."""
        m, n = dense.shape
        if max_rank is None:
            max_rank = max(min(m, n) // MAX_RANK_RATIO, 1)
        min_mn = min(m, n)
        u, s, vt = svd(dense, params.op_type)
        if params.fixed_rank:
            rk = min(params.fixed_rank, min_mn)
        else:
            rk = calculate_new_rank(params.truncated_svd, s, min_mn, params.accuracy)
        rk = min(max(rk, 1), max_rank)
        # CalculateVTnew: VT eats Sigma.
        v = s[:rk, None] * vt[:rk, :]
        return cls(u[:, :rk], v, max_rank=max_rank)

    @property
    def rows(self):
        return self.u.shape[0]

    @property
    def cols(self):
        return self.v.shape[1]

    @property
    def rank(self):
        return self.u.shape[1]

    def to_dense(self) -> np.ndarray:
        return self.u @ self.v

    def gemm(self, alpha: float, a: np.ndarray, b: np.ndarray, beta: float,
             params: CompressionParameters) -> dict:
        """Compressed.cpp:208-694, ungqr / non-trmm / non-Cholesky path (the default).

        ``a`` is the m x ARank left factor and ``b`` the ARank x n right factor that
        HCore::Gemm hands down.  Returns per-stage data for stage-by-stage checks.
        """
        if params.use_trmm or not params.use_ungqr:
            raise NotImplementedError("only the default ungqr/non-trmm recompression is restated")
        m, n = self.rows, self.cols
        crk = self.rank
        arank = a.shape[1]
        k = arank + crk
        um, un, vm, vn = m, k, n, k
        min_um_un = min(um, un)
        min_vm_vn = min(vm, vn)
        size_s = min(m, n, k)
        # LaCpy x2 + MultiplyByAlpha (Compressed.cpp:332-347)
        ustack = np.empty((um, un), order="F")
        ustack[:, :crk] = self.u
        ustack[:, crk:] = alpha * a
        # ProcessVpointer (Compressed.cpp:378-379): V = [beta Cv^T | B^T]
        vstack = np.empty((vm, vn), order="F")
        vstack[:, :crk] = beta * self.v.T
        vstack[:, crk:] = b.T
        # Geqrf x2, R extraction (Compressed.cpp:353-449)
        qu, tau_u = geqrf(ustack)
        ru = np.triu(qu[:min_um_un, :un])
        qv, tau_v = geqrf(vstack)
        rv = np.triu(qv[:min_vm_vn, :vn])
        # RURV = RU * RV^T and its SVD (Compressed.cpp:456-480)
        rurv = ru @ rv.T
        unew, sigma, vtnew = svd(rurv, params.op_type)
        # New rank (Compressed.cpp:509-527)
        if params.fixed_rank:
            rk = min(params.fixed_rank, k)
        else:
            rk = calculate_new_rank(params.truncated_svd, sigma, size_s, params.accuracy)
        rk = max(rk, 1)
        clamped = rk > self.max_rank
        rk = min(rk, self.max_rank)
        # U side: ungqr + Q_U * Unew (Compressed.cpp:549-563)
        q_u = ungqr(qu, tau_u, min_um_un)
        new_u = q_u @ unew[:, :rk]
        # V side: VTnew *= sigma, ungqr, Q_V * VTnew^T, transpose (Compressed.cpp:597-628)
        vts = sigma[:rk, None] * vtnew[:rk, :]
        q_v = ungqr(qv, tau_v, min_vm_vn)
        new_v = (q_v @ vts.T).T
        self.u = np.asfortranarray(new_u)
        self.v = np.asfortranarray(new_v)
        return dict(k=k, sigma=sigma, rank=rk, clamped=clamped, ru=ru, rv=rv)


# ---------------------------------------------------------------------------
# L4 API: HCore<T>::Gemm dispatch (src/api/HCore.cpp:23-344), NoTrans operands
# ---------------------------------------------------------------------------

def hcore_gemm(alpha: float, a, b, beta: float, c, params: CompressionParameters) -> dict:
    """HCore.cpp:23-344 for NoTrans A and B.

    Combination -> temporary dense products -> final ``C.Gemm``:
      CC*: T1 = Av Bu, T2 = T1 Bv, final (Au, T2)         (HCore.cpp:178-264)
      DC*: T = A Bu, final (T, Bv)
      CD*: T = Av B, final (Au, T)
      DD* with dense C: final (A, B)
      DDC: W = A B + beta Cu Cv, C re-set to U = W, V = I at full rank (HCore.cpp:272-299)
    """
    info = {}
    if a.kind == "compressed" and b.kind == "compressed":
        t2 = (a.v @ b.u) @ b.v
        left, right = a.u, t2
    elif a.kind == "dense" and b.kind == "compressed":
        left, right = a.data @ b.u, b.v
    elif a.kind == "compressed" and b.kind == "dense":
        left, right = a.u, a.v @ b.data
    else:
        left, right = a.data, b.data
        if c.kind == "compressed":
            # Dense-dense-compressed: ReadjustTile to full rank with an identity V.
            w = alpha * (left @ right) + beta * (c.u @ c.v)
            r = min(w.shape)
            c.u = np.asfortranarray(w[:, :r]) if w.shape[1] >= r else np.asfortranarray(w)
            c.v = np.eye(r, w.shape[1], order="F")
            c.max_rank = r
            return {"combo": "DDC"}
    if c.kind == "dense":
        c.gemm(alpha, left, right, beta)
    else:
        info = c.gemm(alpha, left, right, beta, params)
    return info


def tile_matrix_multiply(a_tiles, b_tiles, c_tiles, alpha: float, beta: float,
                         params: CompressionParameters, tile_order=None):
    """examples/matrix_multiplication/omp_main.cpp:112-124: for each C tile, k ascending."""
    nt = len(c_tiles)
    kt = len(b_tiles)
    stats = []
    order = tile_order if tile_order is not None else [(i, j) for i in range(nt) for j in range(len(c_tiles[0]))]
    for (i, j) in order:
        for k in range(kt):
            info = hcore_gemm(alpha, a_tiles[i][k], b_tiles[k][j], beta, c_tiles[i][j], params)
            stats.append((i, j, k, info.get("k"), info.get("rank"), info.get("clamped")))
    return stats


# ---------------------------------------------------------------------------
# Tile Cholesky building blocks (src/api/HCore.cpp:482-647, omp/kernels.cpp:234-282)
# ---------------------------------------------------------------------------

def potrf_lower(a: np.ndarray):
    """omp/kernels.cpp:234-243 -> LAPACK dpotrf (lower); returns (L in the lower triangle, info)."""
    c, info = lapack.dpotrf(np.asfortranarray(a), lower=1, clean=0)
    return c, info


def trsm(side_left: bool, lower: bool, trans: bool, unit: bool, alpha: float, a: np.ndarray, b: np.ndarray):
    """BLAS dtrsm: op(A) X = alpha B (left) or X op(A) = alpha B (right).  Like dtrsm, only the
    leading order-m (left) or order-n (right) block of A is referenced."""
    import scipy.linalg as sl
    k = b.shape[0] if side_left else b.shape[1]
    a = np.asarray(a)[:k, :k]
    t = np.tril(a) if lower else np.triu(a)
    if unit:
        t = t - np.diag(np.diag(t)) + np.eye(t.shape[0])
    opt = t.T if trans else t
    if side_left:
        return sl.solve_triangular(opt, alpha * b, lower=(lower != trans))
    return sl.solve_triangular(opt.T, alpha * b.T, lower=not (lower != trans)).T


def hcore_trsm_compressed(side_left, lower, trans, unit, alpha, a: np.ndarray, b) -> None:
    """HCore<T>::Trsm (HCore.cpp:623-647): trsm on the V buffer viewed as rows x rank (ld rows).
    Works on the flat buffer, so it serves a CompressedTile (b.v = V, rank x cols) and a
    CholeskyTile (b.w = W, cols x rank) alike; the buffer keeps its shape."""
    attr = "w" if isinstance(b, CholeskyTile) else "v"
    cur = getattr(b, attr)
    rows, r = b.rows, b.rank
    x = cur.ravel(order="F").copy().reshape((rows, r), order="F")
    x = trsm(side_left, lower, trans, unit, alpha, a, x)
    setattr(b, attr, np.asfortranarray(x.ravel(order="F").reshape(cur.shape, order="F")))


class CholeskyTile:
    """A compressed tile as HCore++'s Cholesky routines read its buffer: U (rows x rank) and
    W (cols x rank, ld cols), tile = U W^T (HCore.cpp:512-545 Syrk, :636-640 Trsm, and the
    aCholesky branch of Gemm, HCore.cpp:160-174, Compressed.cpp:529-595, :669-673)."""
    kind = "compressed"

    def __init__(self, u: np.ndarray, w: np.ndarray, max_rank: int | None = None):
        self.u = np.array(u, dtype=np.float64, order="F")
        self.w = np.array(w, dtype=np.float64, order="F")
        self.max_rank = self.rank if max_rank is None else max_rank

    @property
    def rows(self):
        return self.u.shape[0]

    @property
    def cols(self):
        return self.w.shape[0]

    @property
    def rank(self):
        return self.u.shape[1]

    def to_dense(self) -> np.ndarray:
        return self.u @ self.w.T


def hcore_syrk(alpha: float, a, uplo_lower: bool, beta: float, c: DenseTile) -> None:
    """HCore<T>::Syrk (HCore.cpp:482-583) into a dense C.
    Compressed A = U W^T: C <- beta C - U (W^T W) U^T over the whole tile (the reference uses -1,
    not alpha), then the opposite strict triangle is set to zero (FillMatrixTriangle,
    omp/kernels.cpp:246-264).  Dense A: dsyrk(uplo, NoTrans, n, k = C.cols) on the uplo triangle."""
    if isinstance(a, CholeskyTile):
        prod = (a.u @ (a.w.T @ a.w)) @ a.u.T
        out = beta * c.data - prod
        mask = np.triu(np.ones_like(out, dtype=bool), 1)
        out[mask if uplo_lower else mask.T] = 0.0
        c.data = np.asfortranarray(out)
        return
    tri = np.tril if uplo_lower else np.triu
    full = alpha * (a.data @ a.data.T) + beta * c.data
    c.data = np.asfortranarray(np.where(tri(np.ones_like(full)) > 0, full, c.data))


def hcore_gemm_cholesky(alpha: float, a: CholeskyTile, b: CholeskyTile, beta: float, c: CholeskyTile,
                        params: CompressionParameters) -> dict:
    """HCore<T>::Gemm(alpha, A, NoTrans, B, Trans, beta, C, ..., aCholesky = true) for compressed A, B
    and C (HCore.cpp:160-174; Compressed.cpp:273-276, :468-476, :529-595, :669-673).
    The branch forms T2 = (U_B W_B^T) W_A and recompresses U = [U_C | alpha U_A], W = [beta W_C | T2],
    i.e. alpha A B^T + beta C, with Sigma kept on the W side and every V factor read and written as
    W = V^T.  Restated through the plain recompression on the transposed views
    A = (U_A, W_A^T), B^T = (W_B, U_B^T), C = (U_C, W_C^T)."""
    ca = CompressedTile(a.u, a.w.T, a.max_rank)
    cb = CompressedTile(b.w, b.u.T, b.max_rank)
    cc = CompressedTile(c.u, c.w.T, c.max_rank)
    info = hcore_gemm(alpha, ca, cb, beta, cc, params)
    c.u, c.w = np.asfortranarray(cc.u), np.asfortranarray(cc.v.T)
    return info


def tile_cholesky(a_tiles, nt, params) -> int:
    """Right-looking tile Cholesky A = L L^T composed of the reference's per-tile operations (the
    reference itself has no driver): dense diagonal tiles, CholeskyTile tiles below the diagonal.
      Potrf(A_kk, Lower)                                       HCore.cpp:585-621
      Trsm(Left, Lower, NoTrans, NonUnit, 1, A_kk, A_ik):  W_ik <- L_kk^-1 W_ik   HCore.cpp:623-647
      Syrk(-1, A_ik, NoTrans, Lower, 1, A_ii)                  HCore.cpp:482-583
      Gemm(-1, A_ik, NoTrans, A_jk, Trans, 1, A_ij, aCholesky = true)   HCore.cpp:23-344
    Returns 0, or k * nb + info of the first failing diagonal tile."""
    for k in range(nt):
        c, info = potrf_lower(a_tiles[k][k].data)
        if info:
            return k * a_tiles[k][k].rows + info
        a_tiles[k][k].data = np.asfortranarray(np.where(np.tril(np.ones_like(c)) > 0, c, a_tiles[k][k].data))
        lkk = np.tril(c)
        for i in range(k + 1, nt):
            hcore_trsm_compressed(True, True, False, False, 1.0, lkk, a_tiles[i][k])
        for i in range(k + 1, nt):
            hcore_syrk(-1.0, a_tiles[i][k], True, 1.0, a_tiles[i][i])
            for j in range(k + 1, i):
                hcore_gemm_cholesky(-1.0, a_tiles[i][k], a_tiles[j][k], 1.0, a_tiles[i][j], params)
    return 0
