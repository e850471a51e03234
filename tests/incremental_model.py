"""Numpy model of incremental recompression (test infrastructure, not the reference's algorithm).

A C tile that a recompression produced has U with orthonormal columns and V = Sigma V'^T with
orthogonal rows.  The QR of the U stack [U_C | P] is then
    [U_C | Q_P] [[I, S], [0, R_P]],  S = U_C^T P,  Q_P R_P = qr(P - U_C S)
(block Gram-Schmidt with one re-orthogonalisation), and the V stack [beta V_C^T | R^T] likewise
with the orthonormal V' = beta V_C^T D^-1, D the column norms.  The core M = R_U R_V^T and its
SVD are those of the reference's algorithm (Compressed.cpp:441-527), so are the rank rule and
the new factors U = Q_U U~_r, V = (Q_V V~_r Sigma_r)^T; only the factorisation of the stacks
differs, and only the new columns are factored.
"""
from __future__ import annotations

import numpy as np

from oracle import hcore_oracle as O


def _fast_qr(base: np.ndarray, p: np.ndarray, scale: np.ndarray):
    q1 = base / scale
    s = q1.T @ p
    pr = p - q1 @ s
    s2 = q1.T @ pr  # one re-orthogonalisation pass
    pr -= q1 @ s2
    s += s2
    qp, rp = np.linalg.qr(pr)
    kb, kp = base.shape[1], p.shape[1]
    r = np.zeros((kb + kp, kb + kp))
    r[:kb, :kb] = np.diag(scale)
    r[:kb, kb:] = s
    r[kb:, kb:] = rp
    return np.hstack([q1, qp]), r


def operands(a, b):
    """The (left, right) factors HCore<T>::Gemm hands to CompressedTile<T>::Gemm (HCore.cpp:178-264)."""
    if a.kind == "compressed" and b.kind == "compressed":
        return a.u, (a.v @ b.u) @ b.v
    if a.kind == "dense" and b.kind == "compressed":
        return a.data @ b.u, b.v
    if a.kind == "compressed" and b.kind == "dense":
        return a.u, a.v @ b.data
    raise ValueError("dense-dense updates are not recompressed")


def incremental_update(u: np.ndarray, v: np.ndarray, left: np.ndarray, right: np.ndarray, alpha: float,
                       beta: float, accuracy: float, max_rank: int):
    """One update C <- alpha left right + beta U V with U orthonormal and V's rows orthogonal;
    returns the new (U, V, rank) in the same form.  Relative threshold (truncated SVD)."""
    vt = beta * v.T
    d = np.linalg.norm(vt, axis=0)
    if not np.all(d > 0):
        raise ValueError("V has a zero row: use the full recompression")
    qu, ru = _fast_qr(u, alpha * left, np.ones(u.shape[1]))
    qv, rv = _fast_qr(vt, right.T, d)
    un, sig, vtn = np.linalg.svd(ru @ rv.T)
    rk = O.calculate_new_rank(True, sig, min(ru.shape[0], rv.shape[0]), accuracy)
    rk = min(max(rk, 1), max_rank)
    return qu @ un[:, :rk], (qv @ (vtn[:rk].T * sig[:rk])).T, rk
