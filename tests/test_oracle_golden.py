"""Pin the CPU oracle against the reference's own known-answer tests.

Vectors come from tests/golden/kat.json (extracted from the reference's test
sources by tests/golden/make_golden.py; each entry names its file:lines).
Tolerances follow the reference's comparator: relative 1e-2
(tests/helpers/src/testHelpers.cpp:83-88) where the reference uses it, exact
where the reference uses ``==``.
"""
import json
import os

import numpy as np
import pytest

from oracle import hcore_oracle as O

KAT = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "kat.json")))


def arr(entry, name):
    return np.array(KAT[entry][name]["values"], dtype=np.float64)


def rowmajor(entry, name, rows, cols):
    """The reference writes matrices as row-major C arrays and converts to column-major."""
    return arr(entry, name).reshape(rows, cols)


def test_multiply_by_alpha():
    # TestKernels.cpp:122-156: MultiplyByAlpha(A, 3, 4, 0, 1, 2) scales the whole 3x4 array.
    a = arr("multiply_by_alpha", "matrix_A").copy()
    O.multiply_by_alpha(a, 3, 4, 0, 1, 2.0)
    assert np.array_equal(a, arr("multiply_by_alpha", "matrix_C"))


def test_process_vpointer():
    # TestKernels.cpp:157-192 (exact comparison in the reference)
    v = np.zeros(10)
    O.process_vpointer(2, 2, False, 2, 1.0, arr("process_vpointer", "cv"), 2, v, 3, arr("process_vpointer", "b_data"))
    assert np.array_equal(v, arr("process_vpointer", "expected"))


def test_calculate_new_rank_absolute():
    # TestKernels.cpp:194-215: sigma = {acc+1, acc+2, acc, acc-1, acc-2}, acc = 10 -> rank 3
    acc = 10.0
    sigma = np.array([acc + 1, acc + 2, acc, acc - 1, acc - 2])
    assert O.calculate_new_rank(False, sigma, 5, acc) == 3


def test_calculate_new_rank_relative():
    # TestKernels.cpp:217-237: sigma_0 = 2, others around acc*sigma_0 = 20 -> rank 3
    acc, s0 = 10.0, 2.0
    sigma = np.array([s0, acc * s0 + 2, acc * s0, acc * s0 - 1, acc * s0 - 2])
    assert O.calculate_new_rank(True, sigma, 5, acc) == 3


def test_calculate_uvptr():
    # TestKernels.cpp:239-265: rank 3, vm 2
    uv = np.zeros(6)
    O.calculate_uvptr(3, 2, uv, arr("calculate_uvptr", "v_new"))
    assert np.array_equal(uv, arr("calculate_uvptr", "expected"))


@pytest.mark.parametrize("key,ungqr", [("calculate_vtnew_no_ungqr", False), ("calculate_vtnew_ungqr", True)])
def test_calculate_vtnew(key, ungqr):
    # TestKernels.cpp:267-329: vm 4, vn 3, sizeS 3, rank 3
    vt = arr(key, "vt").copy()
    O.calculate_vtnew(3, ungqr, 3, arr(key, "sigma"), vt, 3, 4)
    assert np.array_equal(vt, arr(key, "vt_new"))


def test_geqrf():
    # TestKernels.cpp:470-511: the 2x6 row-major array is read as a 6x2 column-major matrix.
    a = arr("geqrf", "matrix_A").reshape(6, 2, order="F")
    qr, tau = O.geqrf(a)
    np.testing.assert_allclose(qr.ravel(order="F"), arr("geqrf", "a_expected"), rtol=1e-2, atol=1e-6)
    np.testing.assert_allclose(tau, arr("geqrf", "tau_expected"), rtol=1e-2)


def test_compressed_tile_gemm_ddc():
    # TestCompressedTile.cpp:124-260: zero rank-2 C (3x2) += A (3x3) B (3x2), accuracy = eps
    a = rowmajor("compressed_tile_ddc", "matrix_A", 3, 3)
    b = rowmajor("compressed_tile_ddc", "matrix_B", 3, 2)
    c = O.CompressedTile.from_uv(3, 2, np.zeros(3 * 2 + 2 * 2), 2)
    params = O.CompressionParameters(np.finfo(np.float64).eps)
    c.gemm(1.0, a, b, 1.0, params)
    np.testing.assert_allclose(c.to_dense(), rowmajor("compressed_tile_ddc", "output_matrix", 3, 2), rtol=1e-2)


def test_hcore_gemm_ccc_test9():
    # TestGemm.cpp:748-915: CCC into a zero rank-1 C (max rank 1), accuracy = eps
    au = rowmajor("gemm_test9_ccc", "matrix_Au", 5, 3)
    av = rowmajor("gemm_test9_ccc", "matrix_Av", 3, 4)
    bu = rowmajor("gemm_test9_ccc", "matrix_Bu", 4, 2)
    bv = rowmajor("gemm_test9_ccc", "matrix_Bv", 2, 2)
    a = O.CompressedTile(au, av)
    b = O.CompressedTile(bu, bv)
    c = O.CompressedTile.from_uv(5, 2, np.zeros(5 + 2), 1)
    O.hcore_gemm(1.0, a, b, 1.0, c, O.CompressionParameters(np.finfo(np.float64).eps))
    assert c.rank == 1
    np.testing.assert_allclose(c.to_dense(), rowmajor("gemm_test9_ccc", "output_matrix", 5, 2), rtol=1e-2)


def test_hcore_gemm_ddc_test10():
    # TestGemm.cpp:917-1045: DDC re-sets C to full rank (U = A B + C, V = I)
    a = O.DenseTile(rowmajor("gemm_test10_ddc", "matrix_A", 5, 3))
    b = O.DenseTile(rowmajor("gemm_test10_ddc", "matrix_B", 3, 4))
    c = O.CompressedTile.from_uv(5, 4, np.zeros(5 * 4 + 4 * 4), 4)
    O.hcore_gemm(1.0, a, b, 1.0, c, O.CompressionParameters(np.finfo(np.float64).eps))
    np.testing.assert_allclose(c.to_dense(), rowmajor("gemm_test10_ddc", "output_matrix", 5, 4), rtol=1e-2)
    np.testing.assert_array_equal(c.v, np.eye(4))


def test_compress_from_dense_rank_rule():
    # Compressed.cpp:75-146: relative threshold, clamp to max(min(m,n)/3, 1)
    rng = np.random.default_rng(5)
    q1, _ = np.linalg.qr(rng.standard_normal((30, 30)))
    q2, _ = np.linalg.qr(rng.standard_normal((30, 30)))
    s = 10.0 ** -np.arange(30.0)
    a = (q1 * s) @ q2.T
    t = O.CompressedTile.from_dense(a, O.CompressionParameters(3e-6, truncated_svd=True))
    assert t.rank == 6 and t.max_rank == 10
    t = O.CompressedTile.from_dense(a, O.CompressionParameters(1e-14, truncated_svd=True))
    assert t.rank == 10  # clamped at 30 / 3


def test_potrf_kat():
    # TestKernels.cpp:1070-1124: lower Cholesky of [[25,15,5],[15,13,11],[5,11,21]] (the reference
    # prints but does not compare; the lower triangle is the known factor).
    a = rowmajor("potrf", "matrix_A", 3, 3)
    c, info = O.potrf_lower(a)
    assert info == 0
    np.testing.assert_allclose(np.tril(c), rowmajor("potrf", "matrix_Output", 3, 3), rtol=1e-12)


def test_trsm_kat():
    # TestKernels.cpp:1126-1184: Left, Upper, NoTrans, NonUnit, alpha 1
    a = rowmajor("trsm", "matrix_A", 3, 3)
    b = rowmajor("trsm", "matrix_B", 3, 1)
    x = O.trsm(True, False, False, False, 1.0, a, b)
    np.testing.assert_allclose(x, rowmajor("trsm", "matrix_output", 3, 1), rtol=1e-2)


def test_syrk_kat():
    # TestKernels.cpp:1185-1250: C = A A^T on the lower triangle, beta 0; the upper triangle keeps C.
    a = rowmajor("syrk_cross_product", "matrix_A", 4, 4)
    c0 = rowmajor("syrk_cross_product", "matrix_B", 4, 4)
    expected = rowmajor("syrk_cross_product", "matrix_output", 4, 4)
    got = np.where(np.tril(np.ones((4, 4))) > 0, a @ a.T, c0)
    np.testing.assert_allclose(got, expected, rtol=1e-2)
