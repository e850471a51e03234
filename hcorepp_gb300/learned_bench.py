"""The 32 x 32-tile multiply at nb = 1024 (n = 32768, 1e-8 relative): the plain FP64, float-float and
learned forms on one GPU, each with its time, error, ranks and sketch counts.

  python -m hcorepp_gb300.learned_bench [--n 32768] [--nb 1024] [--steps 1] [--warmup 1]

Inputs: the kernel family of the nb = 512 workloads (2-D points uniform in [0,1]^2, Morton-sorted,
a_ij = exp(-|x_i - x_j| / 0.1); A = B from seed 1, C from seed 2), diagonal tiles dense, the other tiles
compressed at 1e-8 relative with the reference's capacity nb / 3 by hcgb_compress_tiles (whole tile
columns per call, tiles generated on the GPU).  One step = C <- A A + C from the same C over all 32^3
updates (k order cost-descending), CUDA events around the multiply.

Error: a dense 32768^2 product is 8.6 GB and 7e13 flops of FP64, so the relative error of each form's
C against the exact product of the compressed inputs is measured on 8 seeded Gaussian probe columns X
(||C X - (A (A X) + C0 X)|| / ||A (A X) + C0 X||), every product formed tile by tile from the factors.
"""
from __future__ import annotations

import argparse
import json

import numpy as np
import torch

from . import _lib as L
from . import tiles as T
from .problems import KernelMatrix

FORMS = {"plain_fp64": (L.PLAIN_FP64, False), "mixed_ff48": (L.MIXED, False),
         "learned_ff48": (L.MIXED, True), "learned_plain": (L.PLAIN_FP64, True)}


def kernel_tile(km: KernelMatrix, pts: torch.Tensor, i: int, j: int) -> torch.Tensor:
    nb = km.nb
    xi, xj = pts[i * nb:(i + 1) * nb], pts[j * nb:(j + 1) * nb]
    blk = torch.exp(-torch.cdist(xi, xj, compute_mode="donot_use_mm_for_euclid_dist") / km.ell)
    return blk  # row-major nb x nb


def build(km: KernelMatrix, acc: float, batch_bytes: float = 16e9) -> T.TileMatrix:
    """Dense diagonal tiles; every other tile compressed on the GPU by hcgb_compress_tiles, whole tile
    columns per call up to `batch_bytes` of dense input."""
    nt, nb = km.nt, km.nb
    kinds = [[L.DENSE if i == j else L.COMPRESSED for j in range(nt)] for i in range(nt)]
    tm = T.TileMatrix(nt, nt, nb, kinds, max(nb // 3, 1))
    params = T.CompressionParameters(acc, truncated_svd=True)
    pts = torch.from_numpy(km.points).cuda()
    pending, dense = [], []
    for j in range(nt):
        tm.tile(j, j).buffer.copy_(kernel_tile(km, pts, j, j).t().reshape(-1))
        for i in range(nt):
            if i != j:
                pending.append((i, j))
                dense.append(kernel_tile(km, pts, i, j).t().contiguous().view(-1))
        if len(dense) * nb * nb * 8 >= batch_bytes or j == nt - 1:
            T.CompressedTile.compress_batch(dense, [tm.tile(i, jj) for (i, jj) in pending], params)
            pending, dense = [], []
    torch.cuda.synchronize()
    return tm


def tile_factors(tm: T.TileMatrix):
    """(i, j) -> dense block or (U, V) of the tile, device views."""
    nt, nb = tm.mt, tm.nb
    ranks = tm.ranks.cpu().numpy()
    out = {}
    for j in range(tm.nt):
        for i in range(nt):
            seg = tm._view(i, j)
            if tm.kinds[i][j] == L.DENSE:
                out[(i, j)] = seg.view(nb, nb).t()
            else:
                r = int(ranks[tm.index(i, j)])
                u = seg[:nb * r].view(r, nb).t()
                v = seg[nb * tm.max_rank:nb * tm.max_rank + r * nb].view(nb, r).t()  # r x nb, ld r
                out[(i, j)] = (u, v)
    return out


def apply_tlr(tm: T.TileMatrix, x: torch.Tensor) -> torch.Tensor:
    """The tile matrix times x (n x p), tile by tile."""
    nb = tm.nb
    f = tile_factors(tm)
    y = torch.zeros((tm.mt * nb, x.shape[1]), dtype=x.dtype, device=x.device)
    for (i, j), t in f.items():
        xs = x[j * nb:(j + 1) * nb]
        y[i * nb:(i + 1) * nb] += (t[0] @ (t[1] @ xs)) if isinstance(t, tuple) else t @ xs
    return y


def run(n=32768, nb=1024, acc=1e-8, steps=1, warmup=1, forms=None, probes=8, k_order=1):
    import time
    from . import autotune
    t0 = time.time()
    A = build(KernelMatrix(n, nb, 2, 0.1, 1), acc)
    C0 = build(KernelMatrix(n, nb, 2, 0.1, 2), acc)
    build_s = time.time() - t0
    nt = n // nb
    C = T.TileMatrix(nt, nt, nb, C0.kinds, C0.max_rank)
    g = torch.Generator(device="cpu").manual_seed(5)
    X = torch.randn(n, probes, dtype=torch.float64, generator=g).cuda()
    want = apply_tlr(A, apply_tlr(A, X)) + apply_tlr(C0, X)
    wnorm = float(torch.linalg.norm(want))
    n_upd = nt ** 3
    info = T.info_buffer(n_upd)
    ctx = T.run_context()
    ctx.set_k_order(k_order)
    autotune.apply(ctx, autotune.DEFAULT)
    stream = torch.cuda.current_stream()
    out = {}
    for form in (forms or list(FORMS)):
        mode, learned = FORMS[form]
        params = T.CompressionParameters(acc, truncated_svd=True, mode=mode)
        model = None
        if learned:
            from . import rank_model as RM
            model = RM.RankModel.load(ctx=ctx)
            model.enable(ctx)

        def step(rec=False):
            C.arena.copy_(C0.arena)
            C.ranks.copy_(C0.ranks)
            T.tlr_gemm(1.0, A, A, 1.0, C, params, info if rec else None, ctx=ctx)

        for _ in range(max(warmup, 1)):
            step(True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        rec = info.cpu().numpy()
        err = float(torch.linalg.norm(apply_tlr(C, X) - want)) / wnorm
        comp = rec[:, 4] > 0
        out[form] = {"value": n_upd / (ms * 1e-3), "unit": "tile-updates/s", "ms_per_step": ms,
                     "rel_err_probe": err, "mean_final_rank": float(C.ranks.double().mean()),
                     "mean_k": float(rec[comp, 4].mean()) if comp.any() else 0.0,
                     "max_k": int(rec[:, 4].max()), "updates_at_capacity": int(np.count_nonzero(rec[:, 5] >= C.max_rank)),
                     "updates_sketched": int(np.count_nonzero(rec[:, 13] > 0)),
                     "sketches_accepted": int(np.count_nonzero(rec[:, 14] > 0)),
                     "bad_status": int(np.count_nonzero((rec[:, 0] != 0) & (rec[:, 0] != L.HCGB_NOT_CONVERGED)))}
        if model is not None:
            from . import rank_model as RM
            RM.learned_off(ctx)
            del model
    base = out.get("plain_fp64", {}).get("value")
    for f in out:
        if base:
            out[f]["speedup_over_plain_fp64"] = out[f]["value"] / base
    ctx.set_k_order(0)
    return {"workload": f"tlr_gemm_n{n}_nb{nb}", "n": n, "nb": nb, "tiles": f"{nt}x{nt}", "updates_per_step": n_upd,
            "accuracy": acc, "max_rank": C0.max_rank, "steps": steps, "warmup": warmup,
            "input_build_seconds": build_s, "error": f"relative, on {probes} seeded Gaussian probe columns",
            "forms": out}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=32768)
    ap.add_argument("--nb", type=int, default=1024)
    ap.add_argument("--accuracy", type=float, default=1e-8)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--forms", default=",".join(FORMS))
    args = ap.parse_args()
    print(json.dumps(run(args.n, args.nb, args.accuracy, args.steps, args.warmup, args.forms.split(","))))


if __name__ == "__main__":
    main()
