"""Tile-Cholesky throughput and accuracy on one GPU (hcgb_tile_cholesky).

  python -m hcorepp_gb300.cholesky_bench [--n 16384] [--nb 1024] [--steps 1] [--warmup 1] [--mode mixed]

Matrix: n points uniform in [0,1]^3 (seeded), Morton-sorted; a_ij = exp(-|x_i - x_j| / 0.2) with
1e-2 added to the diagonal (SPD).  Diagonal tiles dense, tiles below the diagonal compressed on the
GPU at 1e-8 relative accuracy with the reference's capacity nb/3 (hcgb_compress_tiles over groups
of tile columns), in the Cholesky-flow layout (tile = U W^T); tiles above the diagonal are not stored.
One step = one factorization A = L L^T (nt potrf, nt(nt-1)/2 panel solves, nt(nt^2-1)/6 trailing
Syrk/Gemm updates), restarted from the same tiles every step.

Prints one JSON line: trailing updates/s and seconds per factorization (CUDA events around the
driver call), ||L L^T - A||_F / ||A||_F and a seeded random right-hand side's relative solve
residual ||A x - b|| / ||b||, outside the timed region.  Up to n = 16384 both use dense FP64
products on the GPU; beyond that (a dense n = 65536 matrix is 34 GB and L L^T 5.6e14 flops) they are
computed tile by tile: A's tiles regenerated on the GPU, ||A||_F exact, ||L L^T - A||_F estimated
from 16 seeded Gaussian probes (E ||E x||^2 = ||E||_F^2), the solve by tile forward / backward
substitution with L's own tiles.

  --inputs host     compress the input tiles on the host cores (the reference's constructor rule,
                    restated in numpy) instead of on the GPU
  --max-rank nb     give compressed tiles room for rank nb instead of the reference's nb / 3
  --learned         the learned form for the trailing updates (hcorepp_gb300/rank_model_weights.npy)
"""
from __future__ import annotations

import argparse
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
    ap.add_argument("--inputs", choices=["gpu", "host"], default="gpu")
    ap.add_argument("--max-rank", choices=["nb3", "nb"], default="nb3")
    ap.add_argument("--learned", action="store_true")
    ap.add_argument("--probes", type=int, default=16)
    return ap.parse_args()


def cholesky_kinds(nt: int):
    """Dense diagonal, compressed below, nothing stored above."""
    return [[L.DENSE if i == j else L.COMPRESSED if i > j else None for j in range(nt)] for i in range(nt)]


def kernel_tile_device(km: KernelMatrix, pts: torch.Tensor, i: int, j: int) -> torch.Tensor:
    """Tile (i, j) of the kernel matrix generated on the GPU (row-major nb x nb), distances formed
    coordinate-wise like the host generator (no |x|^2 + |y|^2 - 2 x.y cancellation)."""
    nb = km.nb
    xi, xj = pts[i * nb:(i + 1) * nb], pts[j * nb:(j + 1) * nb]
    blk = torch.exp(-torch.cdist(xi, xj, compute_mode="donot_use_mm_for_euclid_dist") / km.ell)
    if i == j and km.diag_shift:
        blk = blk + km.diag_shift * torch.eye(nb, dtype=blk.dtype, device=blk.device)
    return blk


def build_matrix(km: KernelMatrix, acc: float, cap: int, batch_bytes: float = 16e9) -> T.TileMatrix:
    """Dense diagonal tiles; the tiles below the diagonal generated on the GPU and compressed straight
    into the arena (compressed_vt) by hcgb_compress_tiles, whole tile columns per call up to
    `batch_bytes` of dense input (the call itself splits its launches to fit the free memory)."""
    nt, nb = km.nt, km.nb
    tm = T.TileMatrix(nt, nt, nb, cholesky_kinds(nt), cap, vt=True)
    params = T.CompressionParameters(acc, truncated_svd=True)
    pts = torch.from_numpy(km.points).cuda()
    pending, dense = [], []

    def flush():
        if pending:
            T.CompressedTile.compress_batch(dense, [tm.tile(i, j) for (i, j) in pending], params)
            pending.clear()
            dense.clear()

    for j in range(nt):
        tm.tile(j, j).buffer.copy_(kernel_tile_device(km, pts, j, j).t().reshape(-1))
        for i in range(j + 1, nt):
            pending.append((i, j))
            dense.append(kernel_tile_device(km, pts, i, j).t().contiguous().view(-1))
        if len(dense) * nb * nb * 8 >= batch_bytes:
            flush()
    flush()
    torch.cuda.synchronize()
    return tm


def build_matrix_host(args, cap: int) -> T.TileMatrix:
    """The lower tiles compressed on the host cores (process pool), loaded in the Cholesky-flow layout."""
    from .problems import build_tiles
    nt, nb = args.n // args.nb, args.nb
    tiles = build_tiles(args.n, nb, args.d, args.ell, args.seed, args.accuracy, True, diag_shift=args.shift,
                        lower_only=True, max_rank=cap)
    tm = T.TileMatrix(nt, nt, nb, cholesky_kinds(nt), cap, vt=True)
    for (i, j), t in tiles.items():
        if t[0] == "D":
            tm.set_tile(i, j, dense=t[1])
        else:
            tm.set_tile(i, j, u=t[1], v=t[2])
    torch.cuda.synchronize()
    return tm


def factor_tiles(tm: T.TileMatrix):
    """L's tiles on the device: dict (i, j) -> dense block (i > j from U W^T, i == j the lower triangle)."""
    nt, nb = tm.mt, tm.nb
    ranks = tm.ranks.cpu().numpy()
    out = {}
    for j in range(nt):
        for i in range(j, nt):
            seg = tm._view(i, j)
            if i == j:
                out[(i, j)] = torch.tril(seg.view(nb, nb).t())
            else:
                r = int(ranks[tm.index(i, j)])
                u = seg[:nb * r].view(r, nb).t()
                w = seg[nb * tm.max_rank:nb * tm.max_rank + nb * r].view(r, nb).t()
                out[(i, j)] = (u, w)  # tile = u w^T, kept factored
    return out


def tiled_checks(km: KernelMatrix, tm: T.TileMatrix, probes: int):
    """||L L^T - A||_F / ||A||_F estimated from Gaussian probes and the random-RHS solve residual, tile by
    tile (A's tiles regenerated on the GPU, never the whole dense matrix)."""
    nt, nb, n = tm.mt, tm.nb, tm.mt * tm.nb
    pts = torch.from_numpy(km.points).cuda()
    lt = factor_tiles(tm)

    def a_tile(i, j):
        return kernel_tile_device(km, pts, i, j)

    def l_mul(i, j, x, trans):  # L_ij x or L_ij^T x
        t = lt[(i, j)]
        if isinstance(t, tuple):
            u, w = t
            return u @ (w.t() @ x) if not trans else w @ (u.t() @ x)
        return (t.t() if trans else t) @ x

    def a_apply(x):
        y = torch.zeros_like(x)
        a_fro2 = 0.0
        for i in range(nt):
            for j in range(nt):
                blk = a_tile(i, j)
                a_fro2 += float((blk * blk).sum())
                y[i * nb:(i + 1) * nb] += blk @ x[j * nb:(j + 1) * nb]
        return y, a_fro2

    def llt_apply(x):
        z = torch.zeros_like(x)  # L^T x
        for i in range(nt):
            for j in range(i, nt):
                z[i * nb:(i + 1) * nb] += l_mul(j, i, x[j * nb:(j + 1) * nb], True)
        y = torch.zeros_like(x)
        for i in range(nt):
            for j in range(i + 1):
                y[i * nb:(i + 1) * nb] += l_mul(i, j, z[j * nb:(j + 1) * nb], False)
        return y

    g = torch.Generator(device="cpu").manual_seed(11)
    xp = torch.randn(n, probes, dtype=torch.float64, generator=g).cuda()
    ax, a_fro2 = a_apply(xp)
    e = llt_apply(xp) - ax
    fact_res = float(torch.sqrt((e * e).sum() / probes)) / a_fro2 ** 0.5
    # solve L L^T x = b by tile substitution
    b = torch.randn(n, 1, dtype=torch.float64, generator=torch.Generator(device="cpu").manual_seed(7)).cuda()
    y = torch.zeros_like(b)
    for i in range(nt):
        r = b[i * nb:(i + 1) * nb].clone()
        for j in range(i):
            r -= l_mul(i, j, y[j * nb:(j + 1) * nb], False)
        y[i * nb:(i + 1) * nb] = torch.linalg.solve_triangular(lt[(i, i)], r, upper=False)
    x = torch.zeros_like(b)
    for i in reversed(range(nt)):
        r = y[i * nb:(i + 1) * nb].clone()
        for j in range(i + 1, nt):
            r -= l_mul(j, i, x[j * nb:(j + 1) * nb], True)
        x[i * nb:(i + 1) * nb] = torch.linalg.solve_triangular(lt[(i, i)].t(), r, upper=True)
    ab, _ = a_apply(x)
    solve_res = float(torch.linalg.norm(ab - b) / torch.linalg.norm(b))
    return fact_res, solve_res


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
    cap = max(args.nb // 3, 1) if args.max_rank == "nb3" else args.nb
    tm = build_matrix_host(args, cap) if args.inputs == "host" else build_matrix(km, args.accuracy, cap)
    build_s = time.time() - t0
    model = None
    if args.learned:
        from . import rank_model as RM
        model = RM.RankModel.load()
        model.enable()
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
    if model is not None:
        from . import rank_model as RM
        RM.learned_off()
    # accuracy, outside the timed region
    if args.n <= 16384:
        a = torch.from_numpy(km.dense()).cuda()
        lf = dense_lower_factor(tm)
        anorm = torch.linalg.norm(a)
        fact_res = float(torch.linalg.norm(lf @ lf.t() - a) / anorm)
        g = torch.Generator(device="cpu").manual_seed(7)
        b = torch.randn(args.n, 1, dtype=torch.float64, generator=g).cuda()
        y = torch.linalg.solve_triangular(lf, b, upper=False)
        x = torch.linalg.solve_triangular(lf.t(), y, upper=True)
        solve_res = float(torch.linalg.norm(a @ x - b) / torch.linalg.norm(b))
        check = "dense FP64 products"
        del a, lf
    else:
        fact_res, solve_res = tiled_checks(km, tm, args.probes)
        check = f"tile by tile; ||L L^T - A||_F from {args.probes} Gaussian probes"
    off = in_ranks[[tm.index(i, j) for j in range(nt) for i in range(j + 1, nt)]]
    out_ranks = tm.ranks.cpu().numpy()[[tm.index(i, j) for j in range(nt) for i in range(j + 1, nt)]]
    line = {
        "metric": "tile-Cholesky trailing updates/s (Syrk + Gemm(aCholesky), 1e-8 relative)",
        "value": n_updates / secs, "unit": "updates/s", "seconds_per_factorization": secs,
        "steps": args.steps, "warmup": args.warmup, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"tile_cholesky_n{args.n}_nb{args.nb}", "n": args.n, "nb": args.nb, "tiles": nt,
                   "points_dim": args.d, "length_scale": args.ell, "diag_shift": args.shift,
                   "accuracy": args.accuracy, "trailing_updates": n_updates, "mode": args.mode,
                   "max_rank": cap, "inputs": args.inputs, "learned": bool(args.learned)},
        "check": check,
        "residual_llt": fact_res, "solve_residual": solve_res,
        "input_rank_mean": float(off.mean()) if off.size else 0.0,
        "input_rank_clamped_frac": float((off >= tm.max_rank).mean()) if off.size else 0.0,
        "factor_rank_mean": float(out_ranks.mean()) if out_ranks.size else 0.0,
        "update_status_max": int(statuses.max()) if statuses.size else 0,
        "mean_sweeps": float(rec[:, 6][rec[:, 4] > 0].mean()) if (rec[:, 4] > 0).any() else 0.0,
        "updates_at_capacity": int(np.count_nonzero(rec[:, 5] >= cap)),
        "updates_sketched": int(np.count_nonzero(rec[:, 13] > 0)),
        "sketches_accepted": int(np.count_nonzero(rec[:, 14] > 0)),
        "input_build_seconds": build_s,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
