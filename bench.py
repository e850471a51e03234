#!/usr/bin/env python
"""TLR-GEMM tile-updates/s at 1e-8 relative accuracy on GB300.

Headline ("value", "e2e", "roofline"): the plain FP64 form -- the stack QR, the core SVD (pivoted
QR + one-sided Jacobi) and the Q application in double precision on the FP64 pipe (DFMA / DMMA);
the factor products FP64-accurate (DMMA, or for the larger ones the 16-bit tensor cores by
error-free splitting, error below FP64's own worst-case bound).

Other forms, each timed in the same process on the same inputs and reported in "forms" with its
own value, e2e, product error and speed-up over the plain form:
  mixed_ff48 : the stack QR, the core's pivoted QR and Jacobi and the Q application in
               float-float arithmetic (two floats, 48-bit significand) on the FP32 pipe.

Workload (default): n = 16384, nb = 512 -> 32 x 32 tiles, Morton-sorted 2-D points,
a_ij = exp(-|x_i - x_j| / 0.1); A = B from seed 1, C from seed 2; diagonal tiles dense,
off-diagonal tiles compressed at 1e-8 relative (ranks ~10-120, capacity nb/3 = 170).
One step = one full multiply C <- A B + C = 32^3 = 32,768 tile updates (beta applied on
every k step, as the reference driver does), starting from the same C every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--forms a,b]

Prints one JSON line (rank 0).  Inputs (A, B, C: ~1.4 GB each) exceed L2, so no flush is
needed between steps.  "value" times the multiply on device-resident tiles; "e2e" times the same
multiply with the host's pinned A and C copied in and C copied out every step, in the
rank-trimmed transfer format (hcgb_pack_tiles: only the factor columns the ranks use), and
checks that the copied-out result equals the device-resident run's.  "parity" runs the plain
form once more in the reference driver's k order and compares every update of the CPU sample's
C tiles with the oracle's (rank within +-1 after each update, final tile error within
2 x max(oracle's error, accuracy)).  The reference arm times the CPU oracle port (numpy +
LAPACK) on the host cores over a seeded sample of C tiles, each with its full 32-update k-chain.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from hcorepp_gb300.problems import WORKLOADS, build_tiles  # noqa: E402
from hcorepp_gb300.replicas import job_throughput  # noqa: E402

METRIC = "TLR-GEMM tile-updates/s at 1e-8 rel err: plain FP64 vs batched mixed+learned"
UNIT = "tile-updates/s"
HEADLINE_FORM = "plain_fp64"
FORM_NOTES = {
    "plain_fp64": "FP64 throughout: stack QR, core SVD (pivoted QR + one-sided Jacobi) and Q application on the "
                  "FP64 pipe; factor products FP64-accurate (DMMA, or 16-bit tensor cores by error-free splitting)",
    "mixed_ff48": "stack QR, core pivoted QR + Jacobi and Q application in float-float (48-bit significand) on the "
                  "FP32 pipe; core product, new factors, truncation test and factor products as in plain_fp64",
    "learned_ff48": "mixed_ff48 with the learned form: an MLP (trained on plain runs of other seeds, "
                    "hcorepp_gb300/rank_model_weights.npy) sizes a Gaussian sketch of each update; the plain "
                    "recompression runs where the a-posteriori residual test fails",
    "learned_plain": "plain_fp64 with the learned form (sketch sized by the MLP, plain fallback)",
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="tlr_gemm_n16384_nb512", choices=sorted(WORKLOADS))
    ap.add_argument("--forms", default="plain_fp64,mixed_ff48,learned_ff48,learned_plain",
                    help="comma-separated forms; plain_fp64 (the headline) always runs first")
    ap.add_argument("--cpu-tiles", type=int, default=256, help="C tiles (each with its full k-chain) in the CPU sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-check", action="store_true", help="skip the dense FP64 accuracy check")
    ap.add_argument("--no-parity", action="store_true", help="skip the per-update parity run against the CPU sample")
    ap.add_argument("--groups", type=int, default=8, help="independent C-tile groups (streams)")
    ap.add_argument("--k-order", type=int, default=1, choices=[0, 1],
                    help="0: ascending k per C tile (reference order); 1: costliest updates first")
    ap.add_argument("--lowp", default="1e-4,1e-6,1e-8",
                    help="accuracies of the TF32 / BF16 low-precision sweep ('' or none to skip)")
    ap.add_argument("--lowp-steps", type=int, default=2, help="timed steps per low-precision run")
    ap.add_argument("--no-config4", action="store_true",
                    help="skip the n = 32768, nb = 1024 multiply (plain, float-float and learned forms; "
                         "hcorepp_gb300/learned_bench.py)")
    ap.add_argument("--no-tuning", action="store_true",
                    help="default launch shapes instead of the autotuner's cache (hcorepp_gb300/tuning_cache.json)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload_inputs(name, processes=None):
    w = WORKLOADS[name]
    a = build_tiles(w["n"], w["nb"], w["d"], w["ell"], w["seed_ab"], w["accuracy"], w["dense_diagonal"], processes)
    c = build_tiles(w["n"], w["nb"], w["d"], w["ell"], w["seed_c"], w["accuracy"], w["dense_diagonal"], processes)
    return w, a, a, c  # A and B come from the same seed


def pasc_flops(ra, rb, rc, nb):
    """The reference's CCC count (tests/api/AdvancedGemmTest.cpp:160-166): 36 nb r^2 + 157 r^3 with
    r = max(rA, rB, rC) -- an upper bound of the work on mixed ranks, reported for continuity only."""
    r = np.maximum(np.maximum(ra, rb), rc).astype(np.float64)
    return 36.0 * nb * r * r + 157.0 * r ** 3


# ----------------------------------------------------------------------------- CPU arm
def cpu_measure(w, a, b, c, n_tiles, processes, results=None):
    from oracle import cpu_baseline
    from oracle.hcore_oracle import CompressionParameters
    nt = w["n"] // w["nb"]
    sample = cpu_baseline.sample_tiles(nt, n_tiles)
    params = CompressionParameters(w["accuracy"], truncated_svd=True)
    updates, wall = cpu_baseline.run(a, b, c, params, sample, processes, results)
    return updates, wall, sample


def port_calibration():
    """The port's speed against the reference's own compiled CPU path on the same cores and sample,
    measured where the reference's sources were available (oracle/calibrate_port.py), or None."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle", "port_calibration.json")
    try:
        with open(path) as f:
            cal = json.load(f)
    except (OSError, ValueError):
        return None
    return {k: cal[k] for k in ("machine", "cores", "sample", "port_updates_per_s", "reference_updates_per_s",
                                "port_over_reference", "final_rank_max_abs_diff") if k in cal}


def reference_arm(args, rank, world):
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    procs = cores
    w, a, b, c = workload_inputs(args.workload, procs)
    n_tiles = args.cpu_tiles or procs
    nt = w["n"] // w["nb"]
    vals = []
    for it in range(args.warmup + args.steps):
        updates, wall, sample = cpu_measure(w, a, b, c, n_tiles, procs)
        if it >= args.warmup:
            vals.append(updates / wall)
    value = statistics.mean(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * nt * n_tiles / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (Morton-sorted exponential kernel, seeded)",
        "config": {"workload": args.workload, "n": w["n"], "nb": w["nb"], "accuracy": w["accuracy"],
                   "updates_per_multiply": nt ** 3},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
                         "sample": f"{n_tiles} seeded C tiles x {nt} k-updates each per step",
                         "calibration": port_calibration()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active," \
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.out = None
        self.lines = []

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line)

    def __enter__(self):
        import threading
        import time
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
            # the sampler is running (first sample read) before the timed region starts
            t0 = time.time()
            while not self.lines and time.time() - t0 < 15 and self.proc.poll() is None:
                time.sleep(0.05)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.reader.join(timeout=5)
            self.out = "".join(self.lines)
        return False

    def summary(self):
        if not self.out:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for row in csv.reader(io.StringIO(self.out)):
            if len(row) < 9:
                continue
            try:
                sm.append(float(row[1]))
                smax = float(row[2])
            except ValueError:
                continue
            for nm, v in zip(names, row[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------- GPU arm
def load_tiles(T, L, tiles, nt, nb, max_rank):
    kinds = [[L.DENSE if tiles[(i, j)][0] == "D" else L.COMPRESSED for j in range(nt)] for i in range(nt)]
    tm = T.TileMatrix(nt, nt, nb, kinds, max_rank)
    host = np.zeros(tm.arena.numel())
    ranks = np.zeros(nt * nt, dtype=np.int32)
    for (i, j), t in tiles.items():
        idx = tm.index(i, j)
        off = int(tm.offsets[idx])
        if t[0] == "D":
            host[off:off + nb * nb] = t[1].ravel(order="F")
        else:
            u, v = t[1], t[2]
            r = u.shape[1]
            host[off:off + nb * r] = u.ravel(order="F")
            host[off + nb * max_rank:off + nb * max_rank + r * nb] = v.ravel(order="F")
            ranks[idx] = r
    return tm, host, ranks


def traffic_from_profiles(kernel_stage, workload, form, updates_per_launch):
    """DRAM bytes per launch of `kernel_stage`: the per-update traffic of an ncu capture on a
    smaller case (profiles/ncu_traffic.json) times the updates one launch processes."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        ent = json.load(open(path)).get(workload, {}).get(form, {}).get(kernel_stage)
        return None if ent is None else float(ent["bytes_per_update"]) * updates_per_launch
    except Exception:
        return None


def stage_algorithmic_flops(info, nb, kinds_of_update):
    """Algorithmic FP64 flops per stage for one multiply, from the per-update records."""
    ra, rb = info[:, 1].astype(float), info[:, 2].astype(float)
    k, r, sw = info[:, 4].astype(float), info[:, 5].astype(float), info[:, 6].astype(float)
    rk = info[:, 8].astype(float)
    comp = k > 0
    m = float(nb)
    kk = np.minimum(k, m)
    out = {}
    # QR of both stacks (Householder, 2 m k^2 - 2 k^3 / 3 each)
    out["qr"] = float(np.sum(np.where(comp, 2 * (2 * m * k * k - 2 * kk ** 3 / 3), 0.0)))
    # Core: triangular product (2 k^3 / 3), pivoted QR stopped at rk rows (sum_s 4 (k-s)^2),
    # Jacobi on rk columns of length k (per sweep rk(rk-1)/2 pairs x 8 k flops: one inner product and
    # one rotation per pair, the squared norms being tracked), U_r = M V_r (2 k^2 r)
    qrcp = 4.0 * (kk ** 3 - np.maximum(kk - rk, 0) ** 3) / 3.0
    out["core_svd"] = float(np.sum(np.where(comp, 2 * kk ** 3 / 3 + qrcp + sw * rk * (rk - 1) / 2 * 8 * kk
                                            + 2 * kk * kk * r, 0.0)))
    # Q application on both sides: 4 m k r - 2 k^2 r each
    out["apply_q"] = float(np.sum(np.where(comp, 2 * (4 * m * k * r - 2 * kk * kk * r), 0.0)))
    g = 0.0
    for i in range(len(info)):
        ak, bk, ck = kinds_of_update[i]
        if ak and bk:  # T1 = Av Bu and one rank-sized product; a dense C adds the nb x nb update
            g += 4 * m * ra[i] * rb[i] + (0.0 if ck else 2 * m * m * min(ra[i], rb[i]))
        elif (not ak) and bk:
            g += 2 * m * m * rb[i] * (1 if ck else 2)
        elif ak and not bk:
            g += 2 * m * m * ra[i] * (1 if ck else 2)
        else:
            g += 2 * m * m * m
    out["gemm"] = g
    return out


class Workbench:
    """The device-resident inputs of one workload and the multiply steps run on them."""

    def __init__(self, args, local):
        import torch
        from hcorepp_gb300 import _lib as L
        from hcorepp_gb300 import tiles as T
        self.torch, self.L, self.T = torch, L, T
        self.args, self.local = args, local
        self.w, self.a_t, self.b_t, self.c_t = workload_inputs(args.workload, None)
        w = self.w
        self.nb = w["nb"]
        self.nt = w["n"] // self.nb
        self.maxr = max(self.nb // 3, 1)
        self.n_updates = self.nt ** 3
        self.ctx = T.run_context(local)
        nt, nb, maxr = self.nt, self.nb, self.maxr
        self.A, self.a_host, self.a_ranks = load_tiles(T, L, self.a_t, nt, nb, maxr)
        self.C0, self.c_host, self.c_ranks = load_tiles(T, L, self.c_t, nt, nb, maxr)
        self.A.arena.copy_(torch.from_numpy(self.a_host))
        self.A.ranks.copy_(torch.from_numpy(self.a_ranks))
        self.C0.arena.copy_(torch.from_numpy(self.c_host))
        self.C0.ranks.copy_(torch.from_numpy(self.c_ranks))
        self.Cw = T.TileMatrix(nt, nt, nb, self.C0.kinds, maxr)
        self.info = T.info_buffer(self.n_updates)
        self.kinds_u = []
        for kk in range(nt):
            for j in range(nt):
                for i in range(nt):
                    self.kinds_u.append((self.a_t[(i, kk)][0] == "C", self.b_t[(kk, j)][0] == "C",
                                         self.c_t[(i, j)][0] == "C"))
        self._e2e = None

    def params(self, mode, accuracy=None):
        return self.T.CompressionParameters(accuracy or self.w["accuracy"], truncated_svd=True, mode=mode)

    def step(self, params, record_info=False):
        """One multiply from the same C: C <- A B + C (B = A: one device copy serves both operands)."""
        self.Cw.arena.copy_(self.C0.arena)
        self.Cw.ranks.copy_(self.C0.ranks)
        self.T.tlr_gemm(1.0, self.A, self.A, 1.0, self.Cw, params, self.info if record_info else None,
                        ctx=self.T.run_context(self.local))

    # ---- end to end through the public API: host (pinned) inputs in, result back to the host.
    #      Tiles travel in the rank-trimmed transfer format (hcgb_pack_tiles): the host holds A and
    #      C packed (only the columns their ranks use); every step copies them in, unpacks them on
    #      the device, multiplies (B = A, as in the device-resident run: one copy serves both
    #      operands), packs C, reads the packed size and copies C and its ranks out.
    def _e2e_buffers(self):
        if self._e2e is None:
            torch, T = self.torch, self.T
            nt, nb, maxr = self.nt, self.nb, self.maxr
            e = {}
            e["Ae"] = T.TileMatrix(nt, nt, nb, self.A.kinds, maxr)
            e["Ce"] = T.TileMatrix(nt, nt, nb, self.C0.kinds, maxr)
            e["a_pk"] = torch.from_numpy(e["Ae"].host_pack(self.a_host, self.a_ranks)).pin_memory()
            e["c_pk"] = torch.from_numpy(e["Ce"].host_pack(self.c_host, self.c_ranks)).pin_memory()
            e["ar_pin"] = torch.from_numpy(self.a_ranks).pin_memory()
            e["cr_pin"] = torch.from_numpy(self.c_ranks).pin_memory()
            e["a_dev"] = torch.empty(e["a_pk"].numel(), dtype=torch.float64, device="cuda")
            e["c_dev"] = torch.empty(e["c_pk"].numel(), dtype=torch.float64, device="cuda")
            e["out_dev"] = torch.empty(e["Ce"].arena.numel(), dtype=torch.float64, device="cuda")
            e["offs"] = [torch.empty(nt * nt + 1, dtype=torch.int64, device="cuda") for _ in range(3)]
            e["out_pin"] = torch.empty(e["Ce"].arena.numel(), dtype=torch.float64).pin_memory()
            e["outr_pin"] = torch.empty_like(e["cr_pin"]).pin_memory()
            e["total_pin"] = torch.empty(1, dtype=torch.int64).pin_memory()
            self._e2e = e
        return self._e2e

    def e2e_step(self, params, moved):
        e = self._e2e_buffers()
        Ae, Ce = e["Ae"], e["Ce"]
        Ae.ranks.copy_(e["ar_pin"], non_blocking=True)
        e["a_dev"].copy_(e["a_pk"], non_blocking=True)
        Ae.unpack(e["a_dev"], e["offs"][0])
        Ce.ranks.copy_(e["cr_pin"], non_blocking=True)
        e["c_dev"].copy_(e["c_pk"], non_blocking=True)
        Ce.unpack(e["c_dev"], e["offs"][1])
        self.T.tlr_gemm(1.0, Ae, Ae, 1.0, Ce, params, ctx=self.T.run_context(self.local))
        Ce.pack(e["out_dev"], e["offs"][2])
        e["outr_pin"].copy_(Ce.ranks, non_blocking=True)
        e["total_pin"].copy_(e["offs"][2][-1:], non_blocking=True)
        self.torch.cuda.current_stream().synchronize()  # the packed size of the result
        total = int(e["total_pin"][0])
        e["out_pin"][:total].copy_(e["out_dev"][:total], non_blocking=True)
        moved["h2d"] = e["a_pk"].numel() * 8 + e["c_pk"].numel() * 8 + 4 * (e["ar_pin"].numel() + e["cr_pin"].numel())
        moved["d2h"] = total * 8 + 4 * e["outr_pin"].numel() + 8
        moved["total"] = total

    def copy_rates(self, moved):
        """The e2e step's host <-> device copies timed alone (CUDA events, same pinned buffers and sizes):
        the part of the e2e gap that is transfer, the rest being the pack / unpack kernels and the one
        host synchronisation that reads the packed size before the device -> host copy."""
        torch = self.torch
        e = self._e2e_buffers()
        stream = torch.cuda.current_stream()
        total = moved["total"]
        out = {}
        for name, fn, nbytes in (
                ("h2d", lambda: (e["a_dev"].copy_(e["a_pk"], non_blocking=True),
                                 e["c_dev"].copy_(e["c_pk"], non_blocking=True)),
                 8 * (e["a_pk"].numel() + e["c_pk"].numel())),
                ("d2h", lambda: e["out_pin"][:total].copy_(e["out_dev"][:total], non_blocking=True), 8 * total)):
            fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(3):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / 3
            out[name] = {"ms": ms, "gb_per_s": nbytes / (ms * 1e-3) / 1e9}
        return out

    def e2e_matches_device_run(self, moved):
        """The host copy of the e2e result against the device-resident run's result (same multiply)."""
        e = self._e2e_buffers()
        want = self.Cw.host_pack(self.Cw.arena.cpu().numpy(), self.Cw.ranks.cpu().numpy())
        return bool(np.array_equal(e["out_pin"][:moved["total"]].numpy(), want))


def timed(torch, stream, steps, fn, world, sampler=None):
    """CUDA-event time (ms per step) of `steps` calls of fn, barrier + synchronize on both sides."""
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    return e0.elapsed_time(e1) / steps


def tuned_config(wb, form, args):
    """The autotuner's launch shapes for this workload's tile size, stack-width class and form."""
    from hcorepp_gb300 import autotune
    cfg = dict(autotune.DEFAULT)
    cfg["groups"] = args.groups
    if args.no_tuning:
        return cfg, None
    comp = np.array([[wb.c_t[(i, j)][0] == "C" for j in range(wb.nt)] for i in range(wb.nt)])
    a_r = np.where(comp, wb.A.rank_grid(), wb.nb)
    key = autotune.cache_key(wb.nb, autotune.mean_stack_width(a_r, wb.C0.rank_grid(), comp), form)
    cache = autotune.load()
    if key in cache:
        cfg = autotune.lookup(key, cache)
    return cfg, key if key in cache else None


def measure_form(wb, form, mode, args, world, with_e2e=True, accuracy=None, steps=None, warmup=None):
    """Device-resident and end-to-end throughput of one form, its serialised stage times and its
    per-update records."""
    torch, L = wb.torch, wb.L
    from hcorepp_gb300 import autotune
    params = wb.params(mode, accuracy)
    steps = steps or args.steps
    warmup = args.warmup if warmup is None else warmup
    ctx = wb.ctx
    cfg, key = tuned_config(wb, form, args)
    autotune.apply(ctx, cfg)
    ctx.set_k_order(args.k_order)
    model = None
    if form.startswith("learned"):
        from hcorepp_gb300 import rank_model as RM
        model = RM.RankModel.load(ctx=ctx)
        model.enable(ctx)
    for _ in range(max(warmup, 1)):
        wb.step(params, record_info=True)
    torch.cuda.synchronize()
    info_h = wb.info.cpu().numpy()
    stream = torch.cuda.current_stream()
    out = {"form": form, "note": FORM_NOTES.get(form, ""), "tuning": {"config": cfg, "cache_key": key}}
    l0 = L.kernel_launches()
    with ClockSampler(wb.local) as clk:
        ms = timed(torch, stream, steps, lambda: wb.step(params), world)
    launches = (L.kernel_launches() - l0) / steps
    value, ms = job_throughput(ms, wb.n_updates, device="cuda")
    out.update(value=value, ms_per_step=ms, gpu_launches_per_step=launches, clocks=clk.summary())
    # One more multiply, serialised on one stream with CUDA events around every stage: the
    # per-kernel durations behind the roofline (not part of the timed region).
    ctx.set_graph(False)
    ctx.set_concurrency(1)
    ctx.profile_reset()
    ctx.profile(True)
    wb.step(params)
    ctx.profile(False)
    out["stages"] = ctx.profile_read()
    autotune.apply(ctx, cfg)
    # the result of this form (same multiply as the timed steps) for the accuracy check
    if not args.no_check:
        out["result_dense"] = wb.Cw.to_dense_device()
    out["ranks_final"] = wb.Cw.rank_grid()
    if with_e2e:
        moved = {}
        wb.e2e_step(params, moved)
        torch.cuda.synchronize()
        e2e_ms = timed(torch, stream, steps, lambda: wb.e2e_step(params, moved), world)
        e2e_value, e2e_ms = job_throughput(e2e_ms, wb.n_updates, device="cuda")
        out["e2e"] = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(moved["h2d"]),
                      "d2h_bytes_per_step": int(moved["d2h"]), "ms_per_step": e2e_ms,
                      "transfer": "rank-trimmed packed tiles (hcgb_pack_tiles / hcgb_unpack_tiles), pinned host "
                                  "buffers",
                      "result_matches_device_run": wb.e2e_matches_device_run(moved),
                      "copies_alone": wb.copy_rates(moved)}
    out["info"] = info_h
    autotune.apply(ctx, autotune.DEFAULT)
    if model is not None:
        from hcorepp_gb300 import rank_model as RM
        RM.learned_off(ctx)
        out["model"] = model  # kept alive while the context may still reference it
    return out


def core_cycle_classes(info_h):
    """Where the core's SM cycles go: per class of core width (columns the Jacobi rotates), the
    updates, their summed core kcycles and the mean kcycles of each core phase."""
    comp = info_h[:, 4] > 0
    cols = info_h[:, 8]
    out = {}
    lo = 0
    for hi in (16, 32, 64, 128, 256, 1 << 30):
        sel = comp & (cols > lo) & (cols <= hi)
        if sel.any():
            kc = info_h[sel, 9:13].astype(np.float64)
            out[f"{lo + 1}-{hi if hi < (1 << 30) else 'max'}"] = {
                "updates": int(sel.sum()), "kcycles_sum": float(kc.sum()),
                "mean_kcycles": {nm: float(kc[:, q].mean()) for q, nm in
                                 enumerate(["product", "qrcp", "jacobi", "factors"])},
                "mean_sweeps": float(info_h[sel, 6].mean())}
        lo = hi
    return out


def roofline_of(wb, res, form, dmma_peak, dfma_peak, args):
    stages = res["stages"]
    info_h = res["info"]
    st_flops = stage_algorithmic_flops(info_h, wb.nb, wb.kinds_u)
    dom = max(stages, key=lambda s: stages[s][0])
    dom_ms_per_launch = stages[dom][0] / max(stages[dom][1], 1)
    dom_flops_per_launch = st_flops.get(dom, 0.0) / max(stages[dom][1], 1)
    tensor_stages = {"gemm"}
    peak = dmma_peak if dom in tensor_stages else dfma_peak
    achieved = dom_flops_per_launch / (dom_ms_per_launch * 1e-3) / 1e12
    comp_updates = int(np.count_nonzero(info_h[:, 4] > 0))
    traffic = traffic_from_profiles(dom, args.workload, form, comp_updates / max(stages[dom][1], 1))
    ff = form == "mixed_ff48" and dom in ("core_svd", "qr", "apply_q")
    roof = {"bound": "fp64_equivalent" if ff else ("tensor" if dom in tensor_stages else "fp64"), "kernel": dom,
            "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "traffic": traffic,
            "peak_source": "measured in this run by hcgb_fp64_peak (FP64 DMMA / DFMA probe kernels); "
                           "MEASURED_PEAKS.json has no FP64 figure",
            "note": ("algorithmic FP64-equivalent flops of the stage; it runs in float-float arithmetic on the "
                     "FP32 pipe and is compared with the FP64 peak it replaces" if ff else
                     "algorithmic FP64 flops of the stage (operation counts of the reference's algorithm) per "
                     "launch / the launch's CUDA-event duration")}
    total_ms = sum(v[0] for v in stages.values())
    extra = {
        "stages_ms_serial_step": {s: stages[s][0] for s in stages},
        "stage_launches_serial_step": {s: stages[s][1] for s in stages},
        "serial_step_ms": total_ms,
        "stage_share": {s: stages[s][0] / total_ms for s in stages},
        "stage_algorithmic_tflops": {s: st_flops[s] / (stages[s][0] * 1e-3) / 1e12 for s in st_flops
                                     if s in stages and stages[s][0] > 0},
    }
    return roof, extra


def parity_block(wb, cpu_results, args, exact):
    """The plain form in the reference driver's k order against the CPU sample's oracle chains.
    `exact`: the FP64 dense product of the compressed inputs (device tensor)."""
    torch, L = wb.torch, wb.L
    ctx = wb.ctx
    ctx.set_k_order(0)
    wb.step(wb.params(L.PLAIN_FP64), record_info=True)
    torch.cuda.synchronize()
    ctx.set_k_order(args.k_order)
    info = wb.info.cpu().numpy()
    nt, nb = wb.nt, wb.nb
    n = nt * nt
    acc = wb.w["accuracy"]
    Cres = wb.Cw
    ranks_bad, updates, worst_dr = 0, 0, 0
    tiles_checked, tiles_bad = 0, 0
    max_ratio = 0.0
    dev_res = Cres.to_dense_device()
    for (i, j), res in cpu_results.items():
        idx = i + j * nt
        for k, r_o in enumerate(res["ranks"]):
            updates += 1
            rec = info[k * n + idx]
            if rec[0] != 0:
                ranks_bad += 1
                continue
            if r_o is None:
                continue
            d = abs(int(rec[5]) - int(r_o))
            worst_dr = max(worst_dr, d)
            ranks_bad += d > 1
        sl = (slice(i * nb, (i + 1) * nb), slice(j * nb, (j + 1) * nb))
        ex = exact[sl]
        fo = res["final"]
        o_dense = torch.from_numpy(np.ascontiguousarray(fo[1] if fo[0] == "D" else fo[1] @ fo[2])).to(ex.device)
        nrm = float(torch.linalg.norm(ex))
        e_o = float(torch.linalg.norm(o_dense - ex)) / nrm
        e_g = float(torch.linalg.norm(dev_res[sl] - ex)) / nrm
        tiles_checked += 1
        bound = 2 * max(e_o, acc)
        tiles_bad += e_g > bound
        max_ratio = max(max_ratio, e_g / bound)
    return {"form": "plain_fp64", "k_order": "ascending (reference driver)", "c_tiles": tiles_checked,
            "updates_compared": updates, "rank_violations": int(ranks_bad), "max_abs_rank_diff": int(worst_dr),
            "tiles_over_error_bound": int(tiles_bad), "max_error_over_bound": float(max_ratio),
            "bar": "rank within +-1 of the oracle after every update; tile rel. Frobenius error vs the exact "
                   "product <= 2 x max(oracle's error, accuracy)"}


def gpu_arm(args, rank, world, local):
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from hcorepp_gb300 import _lib as L

    forms = [f for f in args.forms.split(",") if f]
    forms = [HEADLINE_FORM] + [f for f in forms if f != HEADLINE_FORM]
    modes = {"plain_fp64": L.PLAIN_FP64, "mixed_ff48": L.MIXED, "learned_ff48": L.MIXED,
             "learned_plain": L.PLAIN_FP64}
    from hcorepp_gb300 import rank_model as RM
    if not os.path.exists(RM.WEIGHTS):
        forms = [f for f in forms if not f.startswith("learned")]
    for f in forms:
        if f not in modes:
            raise SystemExit(f"unknown form {f}")
    wb = Workbench(args, local)
    dmma_peak, dfma_peak = wb.ctx.fp64_peak()
    results = {f: measure_form(wb, f, modes[f], args, world) for f in forms}
    # Low-precision forms (TF32 / BF16 products and Q-application products; QR, core SVD and the
    # truncation test in FP64) at several accuracies, each beside the plain FP64 form at the same
    # accuracy: throughput, error against the FP64 dense product, rank growth.
    lowp = {}
    for acc_s in [a for a in args.lowp.split(",") if a and a != "none"]:
        acc = float(acc_s)
        runs = {}
        for name, mode in (("plain_fp64", L.PLAIN_FP64), ("tf32", L.TF32), ("bf16", L.BF16)):
            if name == "plain_fp64" and acc == wb.w["accuracy"]:
                runs[name] = results[HEADLINE_FORM]
                continue
            runs[name] = measure_form(wb, name, mode, args, world, with_e2e=False, accuracy=acc,
                                      steps=args.lowp_steps, warmup=1)
        lowp[acc_s] = runs
    if rank != 0:
        return 0
    head = results[HEADLINE_FORM]
    nb, nt, maxr = wb.nb, wb.nt, wb.maxr
    info_h = head["info"]

    # ---- accuracy against the FP64 dense product of the TLR inputs (cuBLAS, outside the timing)
    exact = None
    if not args.no_check:
        Ad = wb.A.to_dense_device()
        Cd0 = wb.C0.to_dense_device()
        exact = Ad @ Ad + Cd0
        del Ad, Cd0
        nrm = torch.linalg.norm(exact)
        for res in list(results.values()) + [r for runs in lowp.values() for r in runs.values()]:
            if "result_dense" in res:
                res["rel_fro_err_vs_fp64_dense_product"] = float(torch.linalg.norm(res.pop("result_dense") - exact) / nrm)
        torch.cuda.empty_cache()

    roof, extra = roofline_of(wb, head, HEADLINE_FORM, dmma_peak, dfma_peak, args)
    comp_mask = np.array([[wb.c_t[(i, j)][0] == "C" for j in range(nt)] for i in range(nt)])
    rk = head["ranks_final"]
    clamped = int(np.count_nonzero(info_h[:, 5] >= maxr))
    bad = int(np.count_nonzero((info_h[:, 0] != 0) & (info_h[:, 0] != L.HCGB_NOT_CONVERGED)))
    pasc = float(np.sum(pasc_flops(info_h[:, 1], info_h[:, 2], info_h[:, 3], nb)[info_h[:, 4] > 0]))

    # ---- CPU baseline (oracle port) on a bounded sample, host cores; its oracle results feed the
    #      per-update parity check of the plain form
    cpu, parity = None, None
    if not args.no_cpu_baseline:
        procs = os.cpu_count() or 1
        n_tiles = args.cpu_tiles or procs
        cpu_results = {}
        upd, wall, sample = cpu_measure(wb.w, wb.a_t, wb.b_t, wb.c_t, n_tiles, procs, cpu_results)
        cpu = {"value": upd / wall, "unit": UNIT, "cores": procs, "kind": "port",
               "sample": f"{n_tiles} seeded C tiles x {nt} k-updates = {upd} updates, {wall:.1f} s wall",
               "calibration": port_calibration()}
        if not args.no_parity and exact is not None:
            parity = parity_block(wb, cpu_results, args, exact)
    exact = None
    torch.cuda.empty_cache()

    form_blocks = {}
    for f in forms:
        res = results[f]
        blk = {"value": res["value"], "unit": UNIT, "ms_per_step": res["ms_per_step"], "note": res["note"],
               "speedup_over_plain_fp64": res["value"] / head["value"],
               "gpu_launches_per_step": res["gpu_launches_per_step"], "clocks": res["clocks"],
               "tuning": res["tuning"],
               "stages_ms_serial_step": {st: v[0] for st, v in res["stages"].items()},
               "core_kcycles_by_core_cols": core_cycle_classes(res["info"]),
               "updates_sketched": int(np.count_nonzero(res["info"][:, 13] > 0)),
               "sketches_accepted": int(np.count_nonzero(res["info"][:, 14] > 0)),
               "rel_fro_err_vs_fp64_dense_product": res.get("rel_fro_err_vs_fp64_dense_product"),
               "mean_final_rank": float(res["ranks_final"][comp_mask].mean())}
        if "e2e" in res:
            blk["e2e"] = res["e2e"]
        if f != HEADLINE_FORM:
            r2, x2 = roofline_of(wb, res, f, dmma_peak, dfma_peak, args)
            blk["roofline"] = r2
            blk["stage_share"] = x2["stage_share"]
            blk["serial_step_ms"] = x2["serial_step_ms"]
        form_blocks[f] = blk

    lowp_block = {}
    for acc_s, runs in lowp.items():
        base = runs["plain_fp64"]
        ent = {}
        for name, res in runs.items():
            ri = res["info"]
            comp = ri[:, 4] > 0
            ent[name] = {"value": res["value"], "unit": UNIT, "ms_per_step": res["ms_per_step"],
                         "rel_fro_err_vs_fp64_dense_product": res.get("rel_fro_err_vs_fp64_dense_product"),
                         "mean_final_rank": float(res["ranks_final"][comp_mask].mean()),
                         "rank_growth_vs_plain_fp64": float(res["ranks_final"][comp_mask].mean() /
                                                            max(base["ranks_final"][comp_mask].mean(), 1e-9)),
                         "mean_k": float(ri[comp, 4].mean()) if comp.any() else 0.0,
                         "updates_at_capacity": int(np.count_nonzero(ri[:, 5] >= maxr)),
                         "speedup_over_plain_fp64_same_accuracy": res["value"] / base["value"],
                         "gpu_launches_per_step": res["gpu_launches_per_step"]}
        lowp_block[acc_s] = ent

    line = {
        "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (Morton-sorted exponential kernel, seeded)",
        "config": {"workload": args.workload, "n": wb.w["n"], "nb": nb, "tiles": f"{nt}x{nt}",
                   "updates_per_step": wb.n_updates, "accuracy": wb.w["accuracy"], "threshold": "relative",
                   "dense_diagonal": wb.w["dense_diagonal"], "max_rank": maxr, "form": HEADLINE_FORM,
                   "parallelism": "replicas" if world > 1 else "single_gpu",
                   "launch_shapes": head["tuning"],
                   "k_order": "ascending" if args.k_order == 0 else "cost-descending",
                   "l2": "inputs larger than L2 (A, C arenas 1.4 GB each), no flush"},
        "e2e": {k: v for k, v in head["e2e"].items() if k != "ms_per_step"},
        "roofline": roof,
        "fp64": {"dmma_peak_tflops": dmma_peak, "dfma_peak_tflops": dfma_peak,
                 "reference_formula_gflops": pasc / (head["ms_per_step"] * 1e-3) / 1e9,
                 "reference_formula_note": "36 nb r^2 + 157 r^3 with r = max(rA, rB, rC) "
                                           "(tests/api/AdvancedGemmTest.cpp:160-166): overcounts mixed ranks"},
        **extra,
        "gpu_launches": int(round(head["gpu_launches_per_step"] * args.steps)),
        "ranks": {"mean_final": float(rk[comp_mask].mean()), "max_final": int(rk[comp_mask].max()),
                  "updates_at_capacity": clamped, "bad_status": bad,
                  "mean_k": float(info_h[info_h[:, 4] > 0, 4].mean()),
                  "max_sweeps": int(info_h[:, 6].max()),
                  "mean_sweeps": float(info_h[info_h[:, 4] > 0, 6].mean()),
                  "mean_core_cols": float(info_h[info_h[:, 4] > 0, 8].mean())},
        "core_kcycles_mean": {nm: float(info_h[info_h[:, 4] > 0, 9 + q].mean())
                              for q, nm in enumerate(["product", "qrcp", "jacobi", "factors"])},
        "core_kcycles_by_core_cols": core_cycle_classes(info_h),
        "check": {"rel_fro_err_vs_fp64_dense_product": head.get("rel_fro_err_vs_fp64_dense_product")},
        "parity": parity,
        "forms": form_blocks,
        "lowp_forms": {"note": "TF32 / BF16: factor products and the WY Q-application products on tcgen05 "
                               "(FP32 accumulation in tensor memory, per-row / per-column power-of-two scaling); "
                               "stack QR with its T factor, core SVD and truncation test in FP64. Each accuracy "
                               "beside the plain FP64 form at that accuracy; errors against the FP64 dense "
                               "product of the inputs.", "steps": args.lowp_steps, "by_accuracy": lowp_block},
        "cpu_baseline": cpu,
        "clocks": head["clocks"],
    }
    if not args.no_config4 and world == 1:
        from hcorepp_gb300 import learned_bench
        del wb
        torch.cuda.empty_cache()
        c4_forms = ["plain_fp64", "mixed_ff48"] + (["learned_ff48"] if os.path.exists(RM.WEIGHTS) else [])
        line["config4"] = learned_bench.run(steps=1, warmup=1, forms=c4_forms)
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return reference_arm(args, rank, world)
    return gpu_arm(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
