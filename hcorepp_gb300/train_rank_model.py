"""Trains the learned form's rank predictor on the plain recompression's own runs.

    python -m hcorepp_gb300.train_rank_model [--out hcorepp_gb300/rank_model_weights.npy]

Training data: (features, new rank) of every recompression in plain FP64 runs over seeds that the
benchmarks do not use (their inputs are seeds 1 and 2), in three families:
  multiply, nb = 512   C <- A B + C of Morton-sorted exponential-kernel matrices (2-D points, length
                       scale 0.1, inputs compressed at 1e-8 relative): n = 8192 (16 x 16 tiles, dense
                       diagonal) and n = 2048 (4 x 4 tiles, every tile compressed), accuracies 1e-8,
                       1e-6, 1e-4
  multiply, nb = 1024  the same family at n = 8192 (8 x 8 tiles, dense diagonal)
  Cholesky, nb = 1024  the trailing updates of a tile Cholesky of the 3-D kernel matrix (length scale
                       0.2, +1e-2 on the diagonal) at n = 16384 (16 x 16 tiles), accuracy 1e-8
The two smaller families are replicated so that each carries about a fifth of the training pairs.  The
features are recorded on the device by the pipeline itself (hcgb_set_feature_sink), the targets come
from the per-update records; training runs the library's own forward / backward / Adam kernels.  The
last seed of every family is held out for the report.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _matrix(T, L, n, nb, seed, acc, dense_diag):
    from hcorepp_gb300.problems import build_tiles
    nt = n // nb
    tiles = build_tiles(n, nb, 2, 0.1, seed, acc, dense_diag)
    kinds = [[L.DENSE if tiles[(i, j)][0] == "D" else L.COMPRESSED for j in range(nt)] for i in range(nt)]
    tm = T.TileMatrix(nt, nt, nb, kinds, nb // 3)
    for (i, j), t in tiles.items():
        if t[0] == "D":
            tm.set_tile(i, j, dense=t[1])
        else:
            tm.set_tile(i, j, u=t[1], v=t[2])
    return tm


def harvest(seeds, accuracies, sizes):
    import torch
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300 import rank_model as RM
    from hcorepp_gb300 import tiles as T
    feats, infos, tags = [], [], []
    ctx = T.run_context()
    RM.learned_off(ctx)
    ctx.set_k_order(0)
    for (n, nb, dense_diag) in sizes:
        for s in seeds:
            A = _matrix(T, L, n, nb, s, 1e-8, dense_diag)
            C0 = _matrix(T, L, n, nb, s + 1, 1e-8, dense_diag)
            for acc in accuracies:
                C = T.TileMatrix(C0.mt, C0.nt, nb, C0.kinds, nb // 3)
                C.arena.copy_(C0.arena)
                C.ranks.copy_(C0.ranks)
                f, i = RM.harvest_multiply(A, A, C, T.CompressionParameters(acc, truncated_svd=True))
                feats.append(f)
                infos.append(i)
                tags.append(torch.full((f.shape[0],), s, dtype=torch.int32, device=f.device))
            del A, C0
            torch.cuda.empty_cache()
    return torch.cat(feats), torch.cat(infos), torch.cat(tags)


def harvest_cholesky(seeds, n=16384, nb=1024, acc=1e-8):
    import torch
    from hcorepp_gb300 import rank_model as RM
    from hcorepp_gb300 import tiles as T
    from hcorepp_gb300.cholesky_bench import build_matrix
    from hcorepp_gb300.problems import KernelMatrix
    feats, infos, tags = [], [], []
    ctx = T.run_context()
    RM.learned_off(ctx)
    for s in seeds:
        km = KernelMatrix(n, nb, 3, 0.2, s, diag_shift=1e-2)
        tm = build_matrix(km, acc, max(nb // 3, 1))
        f, i = RM.harvest_cholesky(tm, T.CompressionParameters(acc, truncated_svd=True))
        feats.append(f)
        infos.append(i)
        tags.append(torch.full((f.shape[0],), s, dtype=torch.int32, device=f.device))
        del tm
        torch.cuda.empty_cache()
    return torch.cat(feats), torch.cat(infos), torch.cat(tags)


def held_out_report(m, feats, info):
    import numpy as np
    hold = info.cpu().numpy()
    keep = (hold[:, 4] > 0) & ((hold[:, 0] == 0) | (hold[:, 0] == 5))
    pred = m.predict(feats).cpu().numpy()[keep]
    true = np.log2(1.0 + hold[keep, 5])
    ra, rb, rc = hold[keep, 1], hold[keep, 2], hold[keep, 3]
    add = np.where((ra > 0) & (rb > 0), np.minimum(ra, rb), np.maximum(ra, rb))
    rule = np.log2(1.0 + np.maximum(rc, add))
    return {"held_out_pairs": int(keep.sum()),
            "held_out_mean_abs_log2rank_error": {"network": float(np.abs(pred - true).mean()),
                                                 "input_rank_rule": float(np.abs(rule - true).mean())},
            "held_out_rank_within_8": {"network": float(np.mean(np.abs(np.exp2(pred) - np.exp2(true)) <= 8)),
                                       "input_rank_rule": float(np.mean(np.abs(np.exp2(rule) - np.exp2(true)) <= 8))},
            "held_out_underpredicted_by_more_than_8": float(np.mean(np.exp2(true) - np.exp2(pred) > 8))}


def main():
    import torch
    from hcorepp_gb300 import rank_model as RM
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=RM.WEIGHTS)
    ap.add_argument("--seeds", default=",".join(str(s) for s in range(3, 35, 2)))
    ap.add_argument("--accuracies", default="1e-8,1e-6,1e-4")
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--report", default=None, help="JSON summary path")
    args = ap.parse_args()
    seeds = [int(s) for s in args.seeds.split(",")]
    accs = [float(a) for a in args.accuracies.split(",")]
    t0 = time.time()
    sizes = [(8192, 512, True), (2048, 512, False)]
    fam = {"multiply_nb512": harvest(seeds, accs, sizes),
           "multiply_nb1024": harvest(seeds[:3] + seeds[-1:], accs, [(8192, 1024, True)]),
           "cholesky_nb1024": harvest_cholesky(seeds[:3] + seeds[-1:])}
    t1 = time.time()
    # the last seed's pairs of every family are held out for the report; the smaller families are
    # replicated to about a quarter of the largest one's training pairs each
    big = int((fam["multiply_nb512"][2] != seeds[-1]).sum())
    tr_f, tr_i = [], []
    for name, (f, i, tag) in fam.items():
        train = tag != seeds[-1]
        reps = max(1, round(big / 4 / max(int(train.sum()), 1))) if name != "multiply_nb512" else 1
        tr_f.append(f[train].repeat(reps, 1))
        tr_i.append(i[train].repeat(reps, 1))
    m = RM.RankModel(seed=1)
    loss, used = m.train(torch.cat(tr_f), torch.cat(tr_i), epochs=args.epochs, batch=args.batch, lr=args.lr)
    t2 = time.time()
    m.save(args.out)
    summary = {"pairs_harvested": {k: int(v[0].shape[0]) for k, v in fam.items()}, "pairs_trained": int(used),
               "final_train_mse_log2rank": loss,
               "held_out": {k: held_out_report(m, f[tag == seeds[-1]], i[tag == seeds[-1]])
                            for k, (f, i, tag) in fam.items()},
               "seconds": {"harvest": t1 - t0, "train": t2 - t1}, "seeds": seeds, "accuracies": accs,
               "sizes": [list(s) for s in sizes]}
    print(json.dumps(summary), flush=True)
    if args.report:
        with open(args.report, "w") as f:
            json.dump(summary, f, indent=1)


if __name__ == "__main__":
    main()
