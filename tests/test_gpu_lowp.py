"""The low-precision forms (HCGB_TF32 / HCGB_BF16): products on the fifth-generation tensor cores
(tcgen05.mma, FP32 accumulation in tensor memory) after per-row / per-column power-of-two scaling.

Bars (floating point, stated per element): with u the operand unit roundoff (TF32 with
round-to-nearest: 2^-11; BF16: 2^-8), every element of alpha op(A) op(B) + beta C is within
(2 u + 2 K 2^-24) sum_k |A_ik| |B_kj| |alpha| of the exact product plus FP64 rounding of beta C; at
the form level (a whole recompression) the product error against the exact product is bounded by
16 u (operand rounding of the stack products and of the WY Q application), and the rank stays
within the tile capacity.
"""
import numpy as np
import pytest

from oracle import hcore_oracle as O
from tests.helpers import compressed_from_dense, rel_fro

pytestmark = pytest.mark.gpu

UNIT = {2: 2.0 ** -11, 3: 2.0 ** -8}


@pytest.fixture(scope="module")
def T():
    import torch
    from hcorepp_gb300 import tiles
    assert torch.cuda.is_available()
    return tiles


@pytest.mark.parametrize("mode", [2, 3])
@pytest.mark.parametrize("shape,scaled", [((150, 70, 100), False), ((96, 40, 200), True), ((300, 130, 37), False)])
def test_tcgen05_products_within_rounding_bound(T, mode, shape, scaled):
    rng = np.random.default_rng(21)
    m, n, k = shape
    a = rng.standard_normal((m, k))
    b = rng.standard_normal((k, n))
    c = rng.standard_normal((m, n))
    if scaled:  # rows / columns over 2^+-40, a zero row and column (the power-of-two scaling)
        a *= np.exp2(rng.integers(-40, 40, size=(m, 1)))
        b *= np.exp2(rng.integers(-40, 40, size=(1, n)))
        a[5, :] = 0.0
        b[:, 7] = 0.0
    alpha, beta = 1.5, 0.25
    gc = T.DenseTile(m, n, c)
    T.HCore.Gemm(alpha, T.DenseTile(m, k, a), 0, T.DenseTile(k, n, b), 0, beta, gc,
                 T.CompressionParameters(1e-4, mode=mode))
    got = gc.to_dense()
    exact = alpha * (a.astype(np.longdouble) @ b.astype(np.longdouble)) + beta * c
    absprod = np.abs(alpha) * (np.abs(a) @ np.abs(b))
    bound = 1.05 * (2 * UNIT[mode] + 2 * k * 2.0 ** -24) * absprod + 4e-16 * np.abs(beta * c) + 1e-300
    ratio = np.abs(got - exact) / bound
    assert float(ratio.max()) <= 1.0, float(ratio.max())
    # and it is not an FP64 product: the TF32 / BF16 rounding is visible
    assert float((np.abs(got - exact) / (absprod + 1e-300)).max()) > 1e-9


@pytest.mark.parametrize("mode", [2, 3])
@pytest.mark.parametrize("combo", ["CCC", "DCC", "CDC", "CCD"])
def test_lowp_form_single_update(T, mode, combo):
    from hcorepp_gb300.problems import KernelMatrix
    nb, acc = 256, 1e-4
    km = KernelMatrix(4 * nb, nb, 2, 0.1, 1)
    kc = KernelMatrix(4 * nb, nb, 2, 0.1, 2)
    d = (km.tile(0, 1), km.tile(1, 3), kc.tile(0, 3))
    o = [O.DenseTile(x) if kind == "D" else compressed_from_dense(x, acc) for kind, x in zip(combo, d)]
    g = [T.DenseTile(t.rows, t.cols, t.data) if t.kind == "dense" else
         T.CompressedTile(t.rows, t.cols, t.u, t.v, max_rank=t.max_rank) for t in o]
    exact = 2.0 * o[0].to_dense() @ o[1].to_dense() + 0.5 * o[2].to_dense()
    T.HCore.Gemm(2.0, g[0], 0, g[1], 0, 0.5, g[2], T.CompressionParameters(acc, truncated_svd=True, mode=mode))
    err = rel_fro(g[2].to_dense(), exact)
    assert err <= 16 * UNIT[mode], err
    if combo[2] == "C":
        assert 1 <= g[2].rank <= g[2].max_rank
