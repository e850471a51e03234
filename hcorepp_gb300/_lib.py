"""ctypes binding of libhcgb.so (include/hcgb.h).

The library is the product: there is no fallback.  Importing a function from here on a
machine without the built library raises immediately.
"""
from __future__ import annotations

import ctypes as C
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libhcgb.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "hcgb.h")

HCGB_OK, HCGB_CUDA_ERROR, HCGB_BAD_ARG, HCGB_POOL_TOO_SMALL = 0, 1, 2, 3
HCGB_RANK_OVERFLOW, HCGB_NOT_CONVERGED, HCGB_UNSUPPORTED = 4, 5, 6
STATUS_NAMES = {0: "OK", 1: "CUDA_ERROR", 2: "BAD_ARG", 3: "POOL_TOO_SMALL", 4: "RANK_OVERFLOW",
                5: "NOT_CONVERGED", 6: "UNSUPPORTED"}
DENSE, COMPRESSED, COMPRESSED_VT = 0, 1, 2  # COMPRESSED_VT: V region holds W = V^T (cols x rank)
LOWER, UPPER = 0, 1
LEFT, RIGHT = 0, 1
NONUNIT, UNIT = 0, 1
NOTRANS, TRANS = 0, 1


class HcgbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class Tile(C.Structure):
    _fields_ = [("data", C.c_void_p), ("rank", C.c_void_p), ("rows", C.c_int), ("cols", C.c_int),
                ("max_rank", C.c_int), ("kind", C.c_int)]


class Update(C.Structure):
    _fields_ = [("a", Tile), ("b", Tile), ("c", Tile)]


class Params(C.Structure):
    _fields_ = [("accuracy", C.c_double), ("truncated_svd", C.c_int), ("fixed_rank", C.c_int),
                ("use_trmm", C.c_int), ("use_ungqr", C.c_int), ("op_type", C.c_int), ("mode", C.c_int)]


class UpdateInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("rank_a", C.c_int), ("rank_b", C.c_int), ("rank_c", C.c_int),
                ("k", C.c_int), ("new_rank", C.c_int), ("sweeps", C.c_int), ("side", C.c_int),
                ("core_cols", C.c_int), ("kc_product", C.c_int), ("kc_qrcp", C.c_int), ("kc_jacobi", C.c_int),
                ("kc_factors", C.c_int), ("sketch_cols", C.c_int), ("sketch_accepted", C.c_int)]


INFO_FIELDS = [f[0] for f in UpdateInfo._fields_]
STAGES = ["plan", "stack", "gemm", "qr", "core_svd", "apply_q", "finalize", "sketch"]

_LIB = None


def header_functions():
    """Names of the functions declared in include/hcgb.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|size_t|long long|const char \*)\s*(hcgb_\w+)\s*\(", text, re.M)))


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is not built; run `python -m hcorepp_gb300.build`")
        L = C.CDLL(LIB_PATH)
        vp, ip = C.c_void_p, C.c_int
        L.hcgb_context_create.argtypes = [ip, vp, C.POINTER(vp)]
        L.hcgb_context_destroy.argtypes = [vp]
        L.hcgb_context_set_stream.argtypes = [vp, vp]
        L.hcgb_sync.argtypes = [vp]
        L.hcgb_last_error.argtypes = [vp]
        L.hcgb_last_error.restype = C.c_char_p
        L.hcgb_workspace_bytes.argtypes = [ip] * 5
        L.hcgb_workspace_bytes.restype = C.c_size_t
        L.hcgb_gemm_batch.argtypes = [vp, C.c_double, C.c_double, ip, C.POINTER(Update), C.POINTER(Params), vp]
        L.hcgb_tlr_gemm.argtypes = [vp, ip, ip, ip, C.c_double, C.POINTER(Tile), C.POINTER(Tile), C.c_double,
                                    C.POINTER(Tile), C.POINTER(Params), vp]
        L.hcgb_tile_gemm.argtypes = [vp, C.c_double, C.POINTER(Tile), ip, C.POINTER(Tile), ip, C.c_double,
                                     C.POINTER(Tile), C.POINTER(Params), C.POINTER(C.c_int),
                                     C.POINTER(C.c_ulonglong)]
        L.hcgb_profile_enable.argtypes = [vp, ip]
        L.hcgb_profile_reset.argtypes = [vp]
        L.hcgb_profile_read.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_longlong), ip]
        L.hcgb_fp64_peak.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.hcgb_set_concurrency.argtypes = [vp, ip]
        L.hcgb_set_k_order.argtypes = [vp, ip]
        L.hcgb_set_tensor_products.argtypes = [vp, ip]
        L.hcgb_set_tensor_products.restype = C.c_int
        L.hcgb_potrf.argtypes = [vp, ip, ip, vp, ip, C.POINTER(C.c_int)]
        L.hcgb_trsm.argtypes = [vp, ip, ip, ip, ip, ip, ip, C.c_double, vp, ip, vp, ip]
        L.hcgb_syrk.argtypes = [vp, ip, ip, ip, ip, C.c_double, vp, ip, C.c_double, vp, ip]
        L.hcgb_fill_triangle.argtypes = [vp, ip, ip, vp, ip, C.c_double]
        L.hcgb_tile_cholesky.argtypes = [vp, ip, C.POINTER(Tile), C.POINTER(Params), C.POINTER(C.c_int), vp]
        for nm in ("hcgb_potrf", "hcgb_trsm", "hcgb_syrk", "hcgb_fill_triangle", "hcgb_tile_cholesky"):
            getattr(L, nm).restype = C.c_int
        L.hcgb_set_k_order.restype = C.c_int
        L.hcgb_compress_tile.argtypes = [vp, vp, ip, ip, C.POINTER(Tile), C.POINTER(Params), C.POINTER(C.c_int)]
        L.hcgb_compress_tile.restype = C.c_int
        L.hcgb_compress_tiles.argtypes = [vp, ip, C.POINTER(vp), ip, ip, C.POINTER(Tile), C.POINTER(Params),
                                          C.POINTER(C.c_int)]
        L.hcgb_compress_tiles.restype = C.c_int
        L.hcgb_tile_gemm_noalloc.argtypes = [C.c_double, C.POINTER(Tile), C.POINTER(Tile), C.c_double,
                                             C.POINTER(Tile), C.POINTER(Params), vp, vp]
        L.hcgb_tile_gemm_noalloc.restype = C.c_int
        L.hcgb_kernel_launches.argtypes = []
        L.hcgb_kernel_launches.restype = C.c_longlong
        L.hcgb_rank_model_create.argtypes = [vp, C.c_ulonglong, C.POINTER(vp)]
        L.hcgb_rank_model_destroy.argtypes = [vp]
        L.hcgb_rank_model_params.argtypes = [vp, vp, vp]
        L.hcgb_rank_model_predict.argtypes = [vp, vp, ip, vp, vp]
        L.hcgb_rank_model_gradient.argtypes = [vp, vp, ip, vp, vp, vp, C.POINTER(C.c_double)]
        L.hcgb_rank_model_train.argtypes = [vp, vp, ip, vp, vp, ip, ip, C.c_float, C.c_ulonglong,
                                            C.POINTER(C.c_double), C.POINTER(C.c_int)]
        L.hcgb_set_rank_model.argtypes = [vp, vp, ip]
        L.hcgb_set_feature_sink.argtypes = [vp, vp]
        L.hcgb_set_graph.argtypes = [vp, ip]
        L.hcgb_set_graph.restype = C.c_int
        L.hcgb_set_tuning.argtypes = [vp, ip, ip]
        L.hcgb_set_tuning.restype = C.c_int
        L.hcgb_set_precond.argtypes = [vp, ip]
        L.hcgb_set_precond.restype = C.c_int
        L.hcgb_set_sketch_limit.argtypes = [vp, ip]
        L.hcgb_set_sketch_limit.restype = C.c_int
        for nm in ("hcgb_rank_model_create", "hcgb_rank_model_destroy", "hcgb_rank_model_params",
                   "hcgb_rank_model_predict", "hcgb_rank_model_gradient", "hcgb_rank_model_train",
                   "hcgb_set_rank_model", "hcgb_set_feature_sink"):
            getattr(L, nm).restype = C.c_int
        for nm in ("hcgb_pack_tiles", "hcgb_unpack_tiles"):
            getattr(L, nm).argtypes = [vp, ip, C.POINTER(Tile), vp, vp]
            getattr(L, nm).restype = C.c_int
        for name in ("hcgb_context_create", "hcgb_context_destroy", "hcgb_context_set_stream", "hcgb_sync",
                     "hcgb_gemm_batch", "hcgb_tlr_gemm", "hcgb_tile_gemm", "hcgb_profile_enable",
                     "hcgb_profile_reset", "hcgb_profile_read", "hcgb_fp64_peak", "hcgb_set_concurrency"):
            getattr(L, name).restype = C.c_int
        _LIB = L
    return _LIB


class Context:
    """One device + stream + workspace (kernels::RunContext's role)."""

    def __init__(self, device: int = 0, stream=None):
        self._h = C.c_void_p()
        rc = lib().hcgb_context_create(device, C.c_void_p(stream or 0), C.byref(self._h))
        if rc:
            raise HcgbError(rc, "hcgb_context_create failed")
        self.device = device

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr: int):
        self.check(lib().hcgb_context_set_stream(self._h, C.c_void_p(stream_ptr)))

    def check(self, rc: int, allow=(HCGB_OK,)):
        if rc not in allow:
            raise HcgbError(rc, lib().hcgb_last_error(self._h).decode())
        return rc

    def sync(self):
        self.check(lib().hcgb_sync(self._h))

    def profile(self, enable: bool):
        self.check(lib().hcgb_profile_enable(self._h, int(enable)))

    def profile_reset(self):
        self.check(lib().hcgb_profile_reset(self._h))

    def profile_read(self):
        n = len(STAGES)
        ms = (C.c_double * n)()
        cnt = (C.c_longlong * n)()
        self.check(lib().hcgb_profile_read(self._h, ms, cnt, n))
        return {STAGES[i]: (ms[i], cnt[i]) for i in range(n)}

    def set_k_order(self, policy: int):
        self.check(lib().hcgb_set_k_order(self._h, int(policy)))

    def set_tensor_products(self, enable: bool):
        """Large factor products on the 16-bit tensor cores (FP64-accurate splitting) or on DMMA."""
        self.check(lib().hcgb_set_tensor_products(self._h, int(bool(enable))))

    def set_graph(self, enable: bool):
        """hcgb_tlr_gemm as a captured CUDA graph, replayed while the call is unchanged."""
        self.check(lib().hcgb_set_graph(self._h, int(bool(enable))))

    def set_tuning(self, oz_min_outputs: int = 2048, wy_min_reflectors: int = 48):
        self.check(lib().hcgb_set_tuning(self._h, int(oz_min_outputs), int(wy_min_reflectors)))

    def set_precond(self, min_cols: int = 0):
        self.check(lib().hcgb_set_precond(self._h, int(min_cols)))

    def set_sketch_limit(self, percent: int = 0):
        self.check(lib().hcgb_set_sketch_limit(self._h, int(percent)))

    def set_concurrency(self, groups: int):
        self.check(lib().hcgb_set_concurrency(self._h, int(groups)))

    def fp64_peak(self):
        d, f = C.c_double(), C.c_double()
        self.check(lib().hcgb_fp64_peak(self._h, C.byref(d), C.byref(f)))
        return d.value, f.value

    def close(self):
        if self._h:
            lib().hcgb_context_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


PLAIN_FP64, MIXED, TF32, BF16 = 0, 1, 2, 3


def kernel_launches() -> int:
    """Kernels libhcgb has launched in this process so far."""
    return int(lib().hcgb_kernel_launches())


def make_params(accuracy=1e-4, truncated_svd=False, fixed_rank=0, use_trmm=False, use_ungqr=True, op_type=1,
                mode=PLAIN_FP64):
    return Params(float(accuracy), int(truncated_svd), int(fixed_rank), int(use_trmm), int(use_ungqr), int(op_type),
                  int(mode))
