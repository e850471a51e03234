"""Per-matrix operations behind the HCoreKernels<double> backend (hcgb_d*), against numpy / LAPACK
semantics on the same inputs.  Bars: FP64 rounding level (relative 1e-12 of the operands' scale)
for copies, products and factorisations; orthogonality of computed Q / U / V to 1e-12."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300 import tiles as T
    assert torch.cuda.is_available()
    lib = L.lib()
    vp, ip, dp = C.c_void_p, C.c_int, C.c_double
    lib.hcgb_dgemm.argtypes = [vp, ip, ip, ip, ip, ip, dp, vp, ip, vp, ip, dp, vp, ip]
    lib.hcgb_dcopy2d.argtypes = [vp, ip, ip, ip, dp, vp, ip, vp, ip]
    lib.hcgb_dlacpy.argtypes = [vp, ip, ip, ip, vp, ip, vp, ip]
    lib.hcgb_dlaset.argtypes = [vp, ip, ip, ip, dp, dp, vp, ip]
    lib.hcgb_dscale_rows.argtypes = [vp, ip, ip, vp, vp, ip]
    lib.hcgb_dsymmetrize.argtypes = [vp, ip, ip, vp, ip]
    lib.hcgb_dgeqrf.argtypes = [vp, ip, ip, vp, ip, vp]
    lib.hcgb_dorgqr.argtypes = [vp, ip, ip, ip, vp, ip, vp]
    lib.hcgb_dormqr.argtypes = [vp, ip, ip, ip, ip, ip, vp, ip, vp, vp, ip]
    lib.hcgb_dtrmm.argtypes = [vp, ip, ip, ip, ip, ip, ip, dp, vp, ip, vp, ip]
    lib.hcgb_dgesvd.argtypes = [vp, ip, ip, ip, ip, vp, ip, vp, vp, ip, vp, ip, C.POINTER(C.c_int)]
    return torch, L, T, lib


def dev(torch, a):
    """Column-major device copy of a 2-D array (flat float64 tensor)."""
    a = np.asarray(a, dtype=np.float64)
    return torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()


def host(t, m, n, ld=None):
    ld = ld or m
    return t.cpu().numpy()[:ld * n].reshape((ld, n), order="F")[:m]


def P(t):
    return C.c_void_p(t.data_ptr())


def ok(T, rc):
    ctx = T.run_context()
    ctx.check(rc)


@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_dgemm(env, ta, tb):
    torch, L, T, lib = env
    rng = np.random.default_rng(1)
    m, n, k = 70, 45, 130
    a = rng.standard_normal((k, m) if ta else (m, k))
    b = rng.standard_normal((n, k) if tb else (k, n))
    c = rng.standard_normal((m, n))
    da, db, dc = dev(torch, a), dev(torch, b), dev(torch, c)
    ctx = T.run_context()
    ok(T, lib.hcgb_dgemm(ctx.handle, ta, tb, m, n, k, 1.5, P(da), a.shape[0], P(db), b.shape[0], -0.5, P(dc), m))
    torch.cuda.synchronize()
    want = 1.5 * (a.T if ta else a) @ (b.T if tb else b) - 0.5 * c
    assert np.abs(host(dc, m, n) - want).max() <= 1e-12 * np.abs(want).max()


def test_copies_lacpy_laset_scale_symmetrize(env):
    torch, L, T, lib = env
    rng = np.random.default_rng(2)
    ctx = T.run_context()
    a = rng.standard_normal((9, 6))
    da = dev(torch, a)
    out = torch.zeros(6 * 9, dtype=torch.float64, device="cuda")
    ok(T, lib.hcgb_dcopy2d(ctx.handle, 1, 6, 9, 2.0, P(da), 9, P(out), 6))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(host(out, 6, 9), 2.0 * a.T)
    for part, mask in ((0, np.ones((9, 6), bool)), (1, np.triu(np.ones((9, 6), bool))),
                       (2, np.tril(np.ones((9, 6), bool)))):
        b = torch.full((9 * 6,), 7.0, dtype=torch.float64, device="cuda")
        ok(T, lib.hcgb_dlacpy(ctx.handle, part, 9, 6, P(da), 9, P(b), 9))
        torch.cuda.synchronize()
        np.testing.assert_array_equal(host(b, 9, 6), np.where(mask, a, 7.0))
    for part in (0, 1, 2, 3):
        b = dev(torch, a)
        ok(T, lib.hcgb_dlaset(ctx.handle, part, 9, 6, 0.5, 3.0, P(b), 9))
        torch.cuda.synchronize()
        want = a.copy()
        i, j = np.indices(a.shape)
        off = {0: i != j, 1: i < j, 2: i > j, 3: np.zeros_like(i, bool)}[part]
        want[off] = 0.5
        want[i == j] = 3.0
        np.testing.assert_array_equal(host(b, 9, 6), want)
    s = rng.standard_normal(4)
    b = dev(torch, a)
    ok(T, lib.hcgb_dscale_rows(ctx.handle, 4, 6, P(dev(torch, s[:, None])), P(b), 9))
    torch.cuda.synchronize()
    want = a.copy()
    want[:4] *= s[:, None]
    np.testing.assert_array_equal(host(b, 9, 6), want)
    sq = rng.standard_normal((7, 7))
    for uplo in (0, 1):
        b = dev(torch, sq)
        ok(T, lib.hcgb_dsymmetrize(ctx.handle, uplo, 7, P(b), 7))
        torch.cuda.synchronize()
        tri = np.triu(sq) if uplo == 1 else np.tril(sq)
        np.testing.assert_array_equal(host(b, 7, 7), tri + tri.T - np.diag(np.diag(sq)))


@pytest.mark.parametrize("m,n", [(120, 40), (40, 40), (30, 50)])
def test_geqrf_orgqr_ormqr(env, m, n):
    torch, L, T, lib = env
    import scipy.linalg as sl
    rng = np.random.default_rng(3)
    ctx = T.run_context()
    a = rng.standard_normal((m, n))
    k = min(m, n)
    da = dev(torch, a)
    tau = torch.zeros(k, dtype=torch.float64, device="cuda")
    ok(T, lib.hcgb_dgeqrf(ctx.handle, m, n, P(da), m, P(tau)))
    torch.cuda.synchronize()
    qr = host(da, m, n)
    (qr_ref, tau_ref), _ = sl.qr(a, mode="raw")
    # LAPACK's compact form: same R, reflectors and tau up to rounding
    assert np.abs(np.triu(qr)[:k] - np.triu(qr_ref)[:k]).max() <= 1e-12 * np.abs(a).max() * m
    np.testing.assert_allclose(tau.cpu().numpy(), tau_ref, atol=1e-12)
    # Q C and Q^T C from both sides against the explicit Q
    q = dev(torch, qr[:, :k])
    ok(T, lib.hcgb_dorgqr(ctx.handle, m, k, k, P(q), m, P(tau)))
    torch.cuda.synchronize()
    qh = host(q, m, k)
    assert np.abs(qh.T @ qh - np.eye(k)).max() <= 1e-13 * m
    assert np.abs(qh @ np.triu(qr)[:k] - a).max() <= 1e-12 * np.abs(a).max() * m
    # the full Q (m x m) from the same k reflectors, then Q C, Q^T C, C Q, C Q^T
    qf = np.zeros((m, m))
    qf[:, :k] = qr[:, :k]
    dqf = dev(torch, qf)
    ok(T, lib.hcgb_dorgqr(ctx.handle, m, m, k, P(dqf), m, P(tau)))
    torch.cuda.synchronize()
    qfull = host(dqf, m, m)
    assert np.abs(qfull.T @ qfull - np.eye(m)).max() <= 1e-13 * m
    np.testing.assert_allclose(qfull[:, :k], qh, atol=1e-14)
    for side, trans in ((0, 0), (0, 1), (1, 0), (1, 1)):
        cm, cn = (m, 17) if side == 0 else (17, m)
        c = rng.standard_normal((cm, cn))
        dc = dev(torch, c)
        ok(T, lib.hcgb_dormqr(ctx.handle, side, trans, cm, cn, k, P(da), m, P(tau), P(dc), cm))
        torch.cuda.synchronize()
        qq = qfull.T if trans else qfull
        want = qq @ c if side == 0 else c @ qq
        assert np.abs(host(dc, cm, cn) - want).max() <= 1e-12 * m, (side, trans)


@pytest.mark.parametrize("side,uplo,trans,diag", [(0, 0, 0, 0), (0, 1, 1, 1), (1, 0, 1, 0), (1, 1, 0, 1)])
def test_dtrmm(env, side, uplo, trans, diag):
    torch, L, T, lib = env
    rng = np.random.default_rng(4)
    ctx = T.run_context()
    m, n = 23, 17
    na = m if side == 0 else n
    a = rng.standard_normal((na, na))
    b = rng.standard_normal((m, n))
    tri = np.triu(a) if uplo == 1 else np.tril(a)
    if diag:
        np.fill_diagonal(tri, 1.0)
    op = tri.T if trans else tri
    db = dev(torch, b)
    ok(T, lib.hcgb_dtrmm(ctx.handle, side, uplo, trans, diag, m, n, 0.75, P(dev(torch, a)), na, P(db), m))
    torch.cuda.synchronize()
    want = 0.75 * (op @ b if side == 0 else b @ op)
    assert np.abs(host(db, m, n) - want).max() <= 1e-13 * na


@pytest.mark.parametrize("m,n", [(90, 40), (40, 90), (60, 60)])
def test_dgesvd(env, m, n):
    torch, L, T, lib = env
    rng = np.random.default_rng(5)
    ctx = T.run_context()
    k = min(m, n)
    u0, _ = np.linalg.qr(rng.standard_normal((m, k)))
    v0, _ = np.linalg.qr(rng.standard_normal((n, k)))
    s0 = np.logspace(0, -12, k)
    a = (u0 * s0) @ v0.T
    da = dev(torch, a)
    S = torch.zeros(k, dtype=torch.float64, device="cuda")
    U = torch.zeros(m * k, dtype=torch.float64, device="cuda")
    VT = torch.zeros(k * n, dtype=torch.float64, device="cuda")
    info = C.c_int(-1)
    ok(T, lib.hcgb_dgesvd(ctx.handle, 1, 1, m, n, P(da), m, P(S), P(U), m, P(VT), k, C.byref(info)))
    assert info.value == 0
    s, u, vt = S.cpu().numpy(), host(U, m, k), host(VT, k, n)
    np.testing.assert_allclose(s, np.linalg.svd(a, compute_uv=False), rtol=1e-9, atol=1e-15)
    assert np.all(np.diff(s) <= 0)
    assert np.abs((u * s) @ vt - a).max() <= 1e-13
    assert np.abs(vt @ vt.T - np.eye(k)).max() <= 1e-12
    big = s > 1e-6  # left vectors of well-separated, non-tiny singular values are orthonormal
    assert np.abs(u[:, big].T @ u[:, big] - np.eye(int(big.sum()))).max() <= 1e-10
