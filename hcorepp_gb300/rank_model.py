"""The learned form's rank predictor over the C ABI (hcgb_rank_model_*, hcgb_set_rank_model,
hcgb_set_feature_sink): a device-resident MLP 12 -> 64 -> 64 -> 1 trained by the library's own
kernels on (features, rank) pairs recorded from the plain recompression's own runs.

    model = RankModel(seed=1)
    feats, info = harvest(...)          # features + records of plain multiplies
    model.train(feats, info, epochs=40)
    model.enable()                      # hcgb_tlr_gemm / hcgb_gemm_batch now sketch
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import torch

from . import _lib as L
from . import tiles as T

FEATURES = 12
PARAMS = 5057
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rank_model_weights.npy")


class RankModel:
    def __init__(self, seed: int = 1, ctx: L.Context | None = None):
        self.ctx = ctx or T.run_context()
        self._h = C.c_void_p()
        self.ctx.check(L.lib().hcgb_rank_model_create(self.ctx.handle, C.c_ulonglong(seed), C.byref(self._h)))

    @property
    def handle(self):
        return self._h

    def params(self) -> np.ndarray:
        out = np.zeros(PARAMS, dtype=np.float32)
        rc = L.lib().hcgb_rank_model_params(self._h, out.ctypes.data_as(C.c_void_p), None)
        if rc:
            raise L.HcgbError(rc, "hcgb_rank_model_params")
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(np.asarray(p, dtype=np.float32))
        assert p.size == PARAMS
        rc = L.lib().hcgb_rank_model_params(self._h, None, p.ctypes.data_as(C.c_void_p))
        if rc:
            raise L.HcgbError(rc, "hcgb_rank_model_params")

    def predict(self, feats: torch.Tensor) -> torch.Tensor:
        """Predicted log2(1 + rank) per row of a (n, 12) float32 device tensor."""
        feats = feats.contiguous()
        out = torch.empty(feats.shape[0], dtype=torch.float32, device=feats.device)
        self.ctx.check(L.lib().hcgb_rank_model_predict(self.ctx.handle, self._h, feats.shape[0],
                                                       C.c_void_p(feats.data_ptr()), C.c_void_p(out.data_ptr())))
        return out

    def gradient(self, feats: torch.Tensor, targets: torch.Tensor):
        g = np.zeros(PARAMS, dtype=np.float32)
        loss = C.c_double()
        self.ctx.check(L.lib().hcgb_rank_model_gradient(self.ctx.handle, self._h, feats.shape[0],
                                                        C.c_void_p(feats.contiguous().data_ptr()),
                                                        C.c_void_p(targets.contiguous().data_ptr()),
                                                        g.ctypes.data_as(C.c_void_p), C.byref(loss)))
        return g, loss.value

    def train(self, feats: torch.Tensor, info: torch.Tensor, epochs: int = 40, batch: int = 256, lr: float = 2e-3,
              seed: int = 7):
        """Train on recorded (features, records) pairs; returns (final epoch loss, pairs used)."""
        loss, used = C.c_double(), C.c_int()
        self.ctx.check(L.lib().hcgb_rank_model_train(self.ctx.handle, self._h, feats.shape[0],
                                                     C.c_void_p(feats.contiguous().data_ptr()),
                                                     C.c_void_p(info.contiguous().data_ptr()), epochs, batch,
                                                     C.c_float(lr), C.c_ulonglong(seed), C.byref(loss),
                                                     C.byref(used)))
        return loss.value, used.value

    def enable(self, ctx: L.Context | None = None):
        """The learned form on: sketches sized by this model."""
        ctx = ctx or self.ctx
        ctx.check(L.lib().hcgb_set_rank_model(ctx.handle, self._h, 0))

    def save(self, path: str = WEIGHTS):
        np.save(path, self.params())

    @classmethod
    def load(cls, path: str = WEIGHTS, ctx: L.Context | None = None) -> "RankModel":
        m = cls(0, ctx)
        m.set_params(np.load(path))
        return m

    def close(self):
        if self._h:
            L.lib().hcgb_rank_model_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def learned_off(ctx: L.Context | None = None):
    ctx = ctx or T.run_context()
    ctx.check(L.lib().hcgb_set_rank_model(ctx.handle, None, 0))


def learned_without_network(ctx: L.Context | None = None):
    """The learned form with the sketch sized from the input ranks instead of the predictor."""
    ctx = ctx or T.run_context()
    ctx.check(L.lib().hcgb_set_rank_model(ctx.handle, None, 1))


def feature_sink(feats: torch.Tensor | None, ctx: L.Context | None = None):
    ctx = ctx or T.run_context()
    ctx.check(L.lib().hcgb_set_feature_sink(ctx.handle, C.c_void_p(feats.data_ptr() if feats is not None else 0)))


def harvest_cholesky(a: "T.TileMatrix", params: "T.CompressionParameters", ctx: L.Context | None = None):
    """One tile Cholesky (hcgb_tile_cholesky) of the Cholesky-flow tile matrix `a` in the context's
    current form with the features and records of every trailing update kept: returns (features
    (n, 12) float32, records (n, fields) int32) on the device, n = nt (nt^2 - 1) / 6."""
    ctx = ctx or T.run_context()
    nt = a.mt
    n = max(nt * (nt * nt - 1) // 6, 1)
    feats = torch.zeros((n, FEATURES), dtype=torch.float32, device="cuda")
    info = T.info_buffer(n)
    feature_sink(feats, ctx)
    try:
        res = T.tile_cholesky(a, params, batched=True, info=info)
        torch.cuda.synchronize()
    finally:
        feature_sink(None, ctx)
    if res != 0:
        raise RuntimeError(f"tile Cholesky stopped: not positive definite at {res}")
    return feats, info


def harvest_multiply(a: "T.TileMatrix", b: "T.TileMatrix", c: "T.TileMatrix", params: "T.CompressionParameters",
                     ctx: L.Context | None = None):
    """One multiply C <- A B + C in the context's current form with the features and records of
    every update kept: returns (features (n, 12) float32, records (n, fields) int32) on the device."""
    ctx = ctx or T.run_context()
    n = c.mt * c.nt * a.nt
    feats = torch.zeros((n, FEATURES), dtype=torch.float32, device="cuda")
    info = T.info_buffer(n)
    feature_sink(feats, ctx)
    try:
        T.tlr_gemm(1.0, a, b, 1.0, c, params, info, ctx=ctx)
        torch.cuda.synchronize()
    finally:
        feature_sink(None, ctx)
    return feats, info
