"""Autotuner of the batched TLR multiply's launch shapes, with a cache keyed by tile size, stack-width
class and arithmetic form.

Knobs (all schedule / routing choices; results are the same up to rounding order):
  groups   independent C-tile groups, one stream each (hcgb_set_concurrency)
  wy_min   reflectors a side needs for the tensor-core WY Q application (plain form; hcgb_set_tuning)
  oz_min   outputs a factor product needs to go to the FP64-accurate tensor-core kernel (hcgb_set_tuning)
  graph    the whole multiply captured once as a CUDA graph and replayed (hcgb_set_graph)
  precond  core columns from which the plain form's core SVD runs FP32 preconditioning sweeps first
           (hcgb_set_precond)

`tune()` times candidates on the caller's own multiply by coordinate descent (one knob at a time,
the others at their current best), restoring C before every trial.  `python -m hcorepp_gb300.autotune`
tunes the benchmark workload on the GPU and writes the cache (tuning_cache.json next to this file),
which `lookup()` reads: the cache key is (nb, the power-of-two class of the mean stack width the
inputs imply, form).
"""
from __future__ import annotations

import json
import os

import numpy as np

CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning_cache.json")
DEFAULT = {"groups": 8, "wy_min": 48, "oz_min": 2048, "graph": 0, "precond": 1 << 30}
CANDIDATES = {"groups": [4, 8, 16], "wy_min": [32, 48, 96, 1 << 30], "oz_min": [512, 1024, 2048, 4096],
              "graph": [0, 1], "precond": [16, 32, 64, 1 << 30]}
ORDER = ["groups", "wy_min", "oz_min", "graph", "precond"]
# The float-float form applies Q in float-float panels on every side (no WY form) and has no FP32
# preconditioning, so wy_min and precond do not act on it.
FORM_KNOBS = {"mixed_ff48": ["groups", "oz_min", "graph"]}


def stack_class(mean_k: float) -> int:
    """Power-of-two class of a mean stack width, 16 .. 1024."""
    c = 16
    while c < mean_k and c < 1024:
        c *= 2
    return c


def cache_key(nb: int, mean_k: float, form: str) -> str:
    return f"nb{nb}-k{stack_class(mean_k)}-{form}"


def mean_stack_width(a_ranks: np.ndarray, c_ranks: np.ndarray, c_compressed: np.ndarray) -> float:
    """The mean width rC + rA of the recompression stacks a multiply starts with (rank grids of A and C;
    dense tiles count with their full size), the quantity the tuning classes are keyed by."""
    rc = c_ranks[c_compressed].astype(float)
    return float(rc.mean() + a_ranks[c_compressed].astype(float).mean()) if rc.size else 0.0


def load(path: str = CACHE) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def lookup(key: str, cache: dict | None = None) -> dict:
    cache = load() if cache is None else cache
    ent = cache.get(key)
    cfg = dict(DEFAULT)
    if ent:
        cfg.update({k: ent["config"][k] for k in DEFAULT if k in ent.get("config", {})})
    return cfg


def store(key: str, config: dict, timings: dict, path: str = CACHE) -> None:
    cache = load(path)
    cache[key] = {"config": {k: config.get(k, DEFAULT[k]) for k in DEFAULT}, "ms_per_multiply": timings}
    with open(path, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
        f.write("\n")


def apply(ctx, config: dict) -> None:
    ctx.set_concurrency(int(config["groups"]))
    ctx.set_tuning(int(config["oz_min"]), int(config["wy_min"]))
    ctx.set_graph(bool(config["graph"]))
    ctx.set_precond(int(config["precond"]))


# A knob moves off its current value only for a gain above the run-to-run noise of a timed multiply.
MIN_GAIN = 0.005


def tune(run_multiply, ctx, steps: int = 2, warmup: int = 1, start: dict | None = None, knobs=None):
    """Coordinate descent over CANDIDATES (the knobs in `knobs`, default all).  run_multiply() restores C
    and runs one multiply on the context's stream.  A candidate replaces the current choice only when it
    is faster by more than MIN_GAIN (relative), so ties keep the defaults (the tensor-core WY Q
    application and product routing among them).  Returns (best config, {config label: ms per
    multiply})."""
    import torch
    best = dict(start or DEFAULT)
    seen = {}

    def time_cfg(cfg):
        label = ",".join(f"{k}={cfg[k]}" for k in ORDER)
        if label in seen:
            return seen[label]
        apply(ctx, cfg)
        for _ in range(warmup):
            run_multiply()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            run_multiply()
        e1.record()
        torch.cuda.synchronize()
        seen[label] = e0.elapsed_time(e1) / steps
        return seen[label]

    best_ms = time_cfg(best)
    for knob in (knobs or ORDER):
        for v in CANDIDATES[knob]:
            cfg = dict(best)
            cfg[knob] = v
            ms = time_cfg(cfg)
            if ms < best_ms * (1.0 - MIN_GAIN):
                best, best_ms = cfg, ms
    apply(ctx, best)
    return best, seen


def main():
    import argparse
    import sys

    import torch
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300 import tiles as T
    from hcorepp_gb300.problems import WORKLOADS, build_tiles
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="tlr_gemm_n16384_nb512", choices=sorted(WORKLOADS))
    ap.add_argument("--forms", default="plain_fp64,mixed_ff48")
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--cache", default=CACHE)
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    nb, nt = w["nb"], w["n"] // w["nb"]
    maxr = nb // 3
    tiles = {}
    for name, seed in (("a", w["seed_ab"]), ("c", w["seed_c"])):
        tiles[name] = build_tiles(w["n"], nb, w["d"], w["ell"], seed, w["accuracy"], w["dense_diagonal"])
    mats = {}
    for name, tl in tiles.items():
        kinds = [[L.DENSE if tl[(i, j)][0] == "D" else L.COMPRESSED for j in range(nt)] for i in range(nt)]
        tm = T.TileMatrix(nt, nt, nb, kinds, maxr)
        for (i, j), t in tl.items():
            if t[0] == "D":
                tm.set_tile(i, j, dense=t[1])
            else:
                tm.set_tile(i, j, u=t[1], v=t[2])
        mats[name] = tm
    A, C0 = mats["a"], mats["c"]
    C = T.TileMatrix(nt, nt, nb, C0.kinds, maxr)
    ctx = T.run_context()
    ctx.set_k_order(1)
    comp = np.array([[C0.kinds[i][j] == L.COMPRESSED for j in range(nt)] for i in range(nt)])
    a_r = np.where(comp, A.rank_grid(), nb)
    mean_k = mean_stack_width(a_r, C0.rank_grid(), comp)
    modes = {"plain_fp64": L.PLAIN_FP64, "mixed_ff48": L.MIXED}
    for form in args.forms.split(","):
        params = T.CompressionParameters(w["accuracy"], truncated_svd=True, mode=modes[form])

        def run():
            C.arena.copy_(C0.arena)
            C.ranks.copy_(C0.ranks)
            T.tlr_gemm(1.0, A, A, 1.0, C, params)

        best, seen = tune(run, ctx, steps=args.steps, knobs=FORM_KNOBS.get(form))
        key = cache_key(nb, mean_k, form)
        store(key, best, seen, args.cache)
        print(json.dumps({"key": key, "best": best, "ms": seen}), flush=True)
    apply(ctx, DEFAULT)


if __name__ == "__main__":
    main()
