"""Tile-Cholesky throughput and accuracy on one GPU (hcgb_tile_cholesky).

  python -m hcorepp_gb300.cholesky_bench [--n 16384] [--nb 1024] [--steps 1] [--warmup 1] [--mode mixed]

Matrix: n points uniform in [0,1]^3 (seeded), Morton-sorted; a_ij = exp(-|x_i - x_j| / 0.2) with
1e-2 added to the diagonal (SPD).  Diagonal tiles dense, off-diagonal tiles compressed on the GPU
at 1e-8 relative accuracy with the reference's capacity nb/3, in the Cholesky-flow layout
(tile = U W^T).  One step = one factorization A = L L^T (nt potrf, nt(nt-1)/2 panel solves,
nt(nt^2-1)/6 trailing Syrk/Gemm updates), restarted from the same tiles every step.

Prints one JSON line: trailing updates/s and seconds per factorization (CUDA events around the
driver call), ||L L^T - A||_F / ||A||_F and a seeded random right-hand side's relative solve
residual ||A x - b|| / ||b|| (both evaluated with dense FP64 products on the GPU, outside the
timed region).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import time

import numpy as np
import torch

from . import _lib as L
from . import tiles as T
from .problems import KernelMatrix


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=16384)
    ap.add_argument("--nb", type=int, default=1024)
    ap.add_argument("--d", type=int, default=3)
    ap.add_argument("--ell", type=float, default=0.2)
    ap.add_argument("--shift", type=float, default=1e-2)
    ap.add_argument("--accuracy", type=float, default=1e-8)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--mode", choices=["plain", "mixed"], default="mixed",
                    help="recompression arithmetic of the trailing updates (FP64 or float-float)")
    return ap.parse_args()


def build_matrix(km: KernelMatrix, acc: float) -> T.TileMatrix:
    """Dense diagonal tiles; lower tiles compressed on the GPU straight into the arena (compressed_vt)."""
    nt, nb = km.nt, km.nb
    kinds = [[L.DENSE if i == j else L.COMPRESSED for j in range(nt)] for i in range(nt)]
    tm = T.TileMatrix(nt, nt, nb, kinds, max(nb // 3, 1), vt=True)
    ctx = T.run_context()
    p = T.CompressionParameters(acc, truncated_svd=True).c()
    grid = tm.c_grid()
    r = C.c_int(0)
    for j in range(nt):
        for i in range(j, nt):
            blk = torch.from_numpy(np.asfortranarray(km.tile(i, j)).ravel(order="F")).cuda()
            if i == j:
                tm.tile(i, i).buffer.copy_(blk)
            else:
                ctx.check(L.lib().hcgb_compress_tile(ctx.handle, C.c_void_p(blk.data_ptr()), nb, nb,
                                                     C.byref(grid[tm.index(i, j)]), C.byref(p), C.byref(r)),
                          allow=(L.HCGB_OK, L.HCGB_NOT_CONVERGED))
    torch.cuda.synchronize()
    return tm


def dense_lower_factor(tm: T.TileMatrix) -> torch.Tensor:
    nt, nb = tm.mt, tm.nb
    out = torch.zeros(nt * nb, nt * nb, dtype=torch.float64, device="cuda")
    ranks = tm.ranks.cpu().numpy()
    for j in range(nt):
        for i in range(j, nt):
            seg = tm._view(i, j)
            if i == j:
                blk = torch.tril(seg.view(nb, nb).t())
            else:
                r = int(ranks[tm.index(i, j)])
                u = seg[:nb * r].view(r, nb).t()
                w = seg[nb * tm.max_rank:nb * tm.max_rank + nb * r].view(r, nb).t()
                blk = u @ w.t()
            out[i * nb:(i + 1) * nb, j * nb:(j + 1) * nb] = blk
    return out


def main():
    args = parse()
    torch.cuda.init()
    km = KernelMatrix(args.n, args.nb, args.d, args.ell, args.seed, diag_shift=args.shift)
    nt = km.nt
    t0 = time.time()
    tm = build_matrix(km, args.accuracy)
    build_s = time.time() - t0
    pristine_arena, pristine_ranks = tm.arena.clone(), tm.ranks.clone()
    in_ranks = tm.ranks.cpu().numpy()
    params = T.CompressionParameters(args.accuracy, truncated_svd=True,
                                     mode=L.MIXED if args.mode == "mixed" else L.PLAIN_FP64)
    n_updates = nt * (nt * nt - 1) // 6
    info = T.info_buffer(max(n_updates, 1))
    ctx = T.run_context()
    stream = torch.cuda.current_stream()
    times = []
    for step in range(args.warmup + args.steps):
        tm.arena.copy_(pristine_arena)
        tm.ranks.copy_(pristine_ranks)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        res = T.tile_cholesky(tm, params, batched=True, info=info)
        e1.record(stream)
        torch.cuda.synchronize()
        if res != 0:
            raise RuntimeError(f"tile Cholesky stopped: not positive definite at {res}")
        if step >= args.warmup:
            times.append(e0.elapsed_time(e1) / 1e3)
    secs = float(np.median(times))
    rec = info.cpu().numpy()
    statuses = rec[:, 0]
    # accuracy, outside the timed region
    a = torch.from_numpy(km.dense()).cuda()
    lf = dense_lower_factor(tm)
    anorm = torch.linalg.norm(a)
    fact_res = float(torch.linalg.norm(lf @ lf.t() - a) / anorm)
    g = torch.Generator(device="cpu").manual_seed(7)
    b = torch.randn(args.n, 1, dtype=torch.float64, generator=g).cuda()
    y = torch.linalg.solve_triangular(lf, b, upper=False)
    x = torch.linalg.solve_triangular(lf.t(), y, upper=True)
    solve_res = float(torch.linalg.norm(a @ x - b) / torch.linalg.norm(b))
    off = in_ranks[[tm.index(i, j) for j in range(nt) for i in range(j + 1, nt)]]
    out_ranks = tm.ranks.cpu().numpy()[[tm.index(i, j) for j in range(nt) for i in range(j + 1, nt)]]
    line = {
        "metric": "tile-Cholesky trailing updates/s (Syrk + Gemm(aCholesky), 1e-8 relative)",
        "value": n_updates / secs, "unit": "updates/s", "seconds_per_factorization": secs,
        "steps": args.steps, "warmup": args.warmup, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"tile_cholesky_n{args.n}_nb{args.nb}", "n": args.n, "nb": args.nb, "tiles": nt,
                   "points_dim": args.d, "length_scale": args.ell, "diag_shift": args.shift,
                   "accuracy": args.accuracy, "trailing_updates": n_updates, "mode": args.mode},
        "residual_llt": fact_res, "solve_residual": solve_res,
        "input_rank_mean": float(off.mean()) if off.size else 0.0,
        "input_rank_clamped_frac": float((off >= tm.max_rank).mean()) if off.size else 0.0,
        "factor_rank_mean": float(out_ranks.mean()) if out_ranks.size else 0.0,
        "update_status_max": int(statuses.max()) if statuses.size else 0,
        "mean_sweeps": float(rec[:, 6][rec[:, 4] > 0].mean()) if (rec[:, 4] > 0).any() else 0.0,
        "input_build_seconds": build_s,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
