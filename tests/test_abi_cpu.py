"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, and exports every
entry point include/hcgb.h declares (no compute call: there is no GPU here)."""
import ctypes

from hcorepp_gb300 import _lib as L
from hcorepp_gb300.build import build


def test_library_builds_and_exports_header_symbols():
    path = build()
    lib = ctypes.CDLL(path)
    names = L.header_functions()
    assert "hcgb_tile_gemm" in names and "hcgb_gemm_batch" in names and "hcgb_tlr_gemm" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_workspace_sizing_is_host_only():
    lib = L.lib()
    small = lib.hcgb_workspace_bytes(1, 64, 64, 21, 21)
    big = lib.hcgb_workspace_bytes(1024, 512, 512, 170, 170)
    assert 0 < small < big
    assert lib.hcgb_workspace_bytes(0, 512, 512, 170, 170) == 0
    # Per update at nb=512: two 512 x 340 stacks dominate (~2.8 MB) plus the core buffers (~8 MB in all).
    per = big / 1024
    assert 2.5e6 < per < 9e6, per


def test_bad_arguments_without_a_device():
    lib = L.lib()
    assert lib.hcgb_sync(None) == L.HCGB_BAD_ARG
    assert lib.hcgb_gemm_batch(None, 1.0, 1.0, 0, None, None, None) == L.HCGB_BAD_ARG
