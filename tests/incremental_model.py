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
import scipy.linalg as sl

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


def _pair(t: int, pp: int, n2: int):
    """Round-robin pair (i, j) of position pp at step t (the core kernel's ordering)."""
    if pp == 0:
        return 0, 1 + t % (n2 - 1)
    return 1 + (pp + t) % (n2 - 1), 1 + (n2 - 1 - pp + t) % (n2 - 1)


def jacobi_core_svd(m: np.ndarray, accuracy: float, max_sweeps: int = 40):
    """The core kernel's SVD with the rotations accumulated: pivoted QR of M stopped below
    1e-2 x the relative threshold, one-sided Jacobi on X = R^T (X J = W), then
    M ~ (Q_M J) Sigma (P W Sigma^-1)^T.  Returns U (orthonormal, from the accumulated rotations),
    sigma (descending) and V (orthonormal to the sweep tolerance)."""
    q, r, piv = sl.qr(m, pivoting=True)
    d = np.abs(np.diag(r))
    rk = max(int(np.sum(d > 1e-2 * accuracy * d[0])), 1)
    x = r[:rk].T.copy()
    j = np.eye(rk)
    n2 = rk + (rk & 1)
    tol = 8 * np.finfo(float).eps * x.shape[0]
    for _ in range(max_sweeps):
        rotated = False
        for t in range(n2 - 1):
            for pp in range(n2 // 2):
                a_, b_ = _pair(t, pp, n2)
                if a_ >= rk or b_ >= rk:
                    continue
                xa, xb = x[:, a_], x[:, b_]
                aa, bb, c = xa @ xa, xb @ xb, xa @ xb
                if c * c <= tol * tol * aa * bb:
                    continue
                zeta = (bb - aa) / (2 * c)
                tt = np.copysign(1.0, zeta) / (abs(zeta) + np.sqrt(1 + zeta * zeta))
                cs = 1 / np.sqrt(1 + tt * tt)
                sn = cs * tt
                x[:, [a_, b_]] = np.column_stack([cs * xa - sn * xb, sn * xa + cs * xb])
                ja, jb = j[:, a_].copy(), j[:, b_].copy()
                j[:, a_], j[:, b_] = cs * ja - sn * jb, sn * ja + cs * jb
                rotated = True
        if not rotated:
            break
    sig = np.linalg.norm(x, axis=0)
    order = np.argsort(-sig, kind="stable")
    sig = sig[order]
    u = q[:, :rk] @ j[:, order]
    w = np.zeros((m.shape[1], rk))
    w[piv] = x[:, order]  # P W
    v = w / np.where(sig > 0, sig, 1.0)
    return u, sig, v


def incremental_update(u: np.ndarray, v: np.ndarray, left: np.ndarray, right: np.ndarray, alpha: float,
                       beta: float, accuracy: float, max_rank: int, core: str = "svd"):
    """One update C <- alpha left right + beta U V with U orthonormal and V's rows orthogonal;
    returns the new (U, V, rank) in the same form.  Relative threshold (truncated SVD).
    core = "svd": LAPACK SVD of the core; "jacobi": the core kernel's pivoted QR + Jacobi with
    accumulated rotations."""
    vt = beta * v.T
    d = np.linalg.norm(vt, axis=0)
    if not np.all(d > 0):
        raise ValueError("V has a zero row: use the full recompression")
    qu, ru = _fast_qr(u, alpha * left, np.ones(u.shape[1]))
    qv, rv = _fast_qr(vt, right.T, d)
    m = ru @ rv.T
    if core == "svd":
        un, sig, vtn = np.linalg.svd(m)
        vn = vtn.T
    else:
        un, sig, vn = jacobi_core_svd(m, accuracy)
    size_s = min(ru.shape[0], rv.shape[0])
    rk = O.calculate_new_rank(True, sig, min(size_s, sig.size), accuracy)
    rk = min(max(rk, 1), max_rank, sig.size)
    return qu @ un[:, :rk], (qv @ (vn[:, :rk] * sig[:rk])).T, rk
