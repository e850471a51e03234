#!/usr/bin/env python
"""TLR-GEMM tile-updates/s at 1e-8 relative accuracy on GB300.

Forms (--mode): "mixed" (default) runs the stack QR, the core's pivoted QR and Jacobi and the Q
application in float-float (48-bit) arithmetic on the FP32 pipe; "plain" keeps them in FP64.  In
both, large factor products run on the 16-bit tensor cores by FP64-accurate error-free splitting.
The product error against the FP64 dense product is the same for both (reported under "check").

Workload (default): n = 16384, nb = 512 -> 32 x 32 tiles, Morton-sorted 2-D points,
a_ij = exp(-|x_i - x_j| / 0.1); A = B from seed 1, C from seed 2; diagonal tiles dense,
off-diagonal tiles compressed at 1e-8 relative (ranks ~10-120, capacity nb/3 = 170).
One step = one full multiply C <- A B + C = 32^3 = 32,768 tile updates (beta applied on
every k step, as the reference driver does), starting from the same C every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  Inputs (A, B, C: ~1.4 GB each) exceed L2, so no flush is
needed between steps.  "value" times the multiply on device-resident tiles; "e2e" times the same
multiply with the host's pinned A and C copied in and C copied out every step, in the
rank-trimmed transfer format (hcgb_pack_tiles: only the factor columns the ranks use), and
checks that the copied-out result equals the device-resident run's.  The reference arm times the
CPU oracle port (numpy + LAPACK) on the host cores over a seeded sample of C tiles, each with its
full 32-update k-chain.
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
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from hcorepp_gb300.problems import WORKLOADS, build_tiles  # noqa: E402
from hcorepp_gb300.replicas import job_throughput  # noqa: E402

METRIC = "TLR-GEMM tile-updates/s at 1e-8 rel err: plain FP64 vs batched mixed+learned"
UNIT = "tile-updates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="tlr_gemm_n16384_nb512", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-tiles", type=int, default=256, help="C tiles (each with its full k-chain) in the CPU sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-check", action="store_true", help="skip the dense FP64 accuracy check")
    ap.add_argument("--groups", type=int, default=8, help="independent C-tile groups (streams)")
    ap.add_argument("--k-order", type=int, default=1, choices=[0, 1],
                    help="0: ascending k per C tile (reference order); 1: costliest updates first")
    ap.add_argument("--mode", default="mixed", choices=["plain", "mixed"],
                    help="plain: FP64 throughout; mixed: float-float (48-bit) stack QR, core pivoted QR and Jacobi, "
                         "and Q application on the FP32 pipe")
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
    """The reference's CCC count (tests/api/AdvancedGemmTest.cpp:160-166): 36 nb r^2 + 157 r^3."""
    r = np.maximum(np.maximum(ra, rb), rc).astype(np.float64)
    return 36.0 * nb * r * r + 157.0 * r ** 3


# ----------------------------------------------------------------------------- CPU arm
def cpu_measure(w, a, b, c, n_tiles, processes):
    from oracle import cpu_baseline
    from oracle.hcore_oracle import CompressionParameters
    nt = w["n"] // w["nb"]
    sample = cpu_baseline.sample_tiles(nt, n_tiles)
    params = CompressionParameters(w["accuracy"], truncated_svd=True)
    updates, wall = cpu_baseline.run(a, b, c, params, sample, processes)
    return updates, wall, sample


def reference_arm(args, rank, world):
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    procs = cores
    w, a, b, c = workload_inputs(args.workload, procs)
    n_tiles = args.cpu_tiles or procs
    vals = []
    for it in range(args.warmup + args.steps):
        updates, wall, sample = cpu_measure(w, a, b, c, n_tiles, procs)
        if it >= args.warmup:
            vals.append(updates / wall)
    value = statistics.mean(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * 32 * n_tiles / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (Morton-sorted exponential kernel, seeded)",
        "config": {"workload": args.workload, "n": w["n"], "nb": w["nb"], "accuracy": w["accuracy"],
                   "updates_per_multiply": (w["n"] // w["nb"]) ** 3},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
                         "sample": f"{n_tiles} seeded C tiles x {w['n'] // w['nb']} k-updates each per step"},
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

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                self.out = ""
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


def traffic_from_profiles(kernel_stage, workload, updates_per_launch):
    """DRAM bytes per launch of `kernel_stage`: the per-update traffic of an ncu capture on a
    smaller case (profiles/ncu_traffic.json) times the updates one launch processes."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        ent = json.load(open(path)).get(workload, {}).get(kernel_stage)
        return None if ent is None else float(ent["bytes_per_update"]) * updates_per_launch
    except Exception:
        return None


def stage_algorithmic_flops(info, nb, kinds_of_update):
    """Algorithmic FP64 flops per stage for one multiply, from the per-update records."""
    ra, rb, rc = info[:, 1].astype(float), info[:, 2].astype(float), info[:, 3].astype(float)
    k, r, sw = info[:, 4].astype(float), info[:, 5].astype(float), info[:, 6].astype(float)
    side = info[:, 7]
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


def gpu_arm(args, rank, world, local):
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from hcorepp_gb300 import _lib as L
    from hcorepp_gb300 import tiles as T

    w, a_t, b_t, c_t = workload_inputs(args.workload, None)
    nb = w["nb"]
    nt = w["n"] // nb
    maxr = max(nb // 3, 1)
    n_updates = nt ** 3

    ctx = T.run_context(local)
    A, a_host, a_ranks = load_tiles(T, L, a_t, nt, nb, maxr)
    B = A  # B = A (same seed and tiles): one device copy serves both operands
    C0, c_host, c_ranks = load_tiles(T, L, c_t, nt, nb, maxr)
    A.arena.copy_(torch.from_numpy(a_host))
    A.ranks.copy_(torch.from_numpy(a_ranks))
    C0.arena.copy_(torch.from_numpy(c_host))
    C0.ranks.copy_(torch.from_numpy(c_ranks))
    Cw = T.TileMatrix(nt, nt, nb, C0.kinds, maxr)
    params = T.CompressionParameters(w["accuracy"], truncated_svd=True,
                                     mode=L.MIXED if args.mode == "mixed" else L.PLAIN_FP64)
    info = T.info_buffer(n_updates)
    dmma_peak, dfma_peak = ctx.fp64_peak()
    ctx.set_concurrency(args.groups)
    ctx.set_k_order(args.k_order)

    def step(record_info=False):
        Cw.arena.copy_(C0.arena)
        Cw.ranks.copy_(C0.ranks)
        T.tlr_gemm(1.0, A, B, 1.0, Cw, params, info if record_info else None, ctx=T.run_context(local))

    for _ in range(max(args.warmup, 1)):
        step(record_info=True)
    torch.cuda.synchronize()
    info_h = info.cpu().numpy()
    bad = int(np.count_nonzero((info_h[:, 0] != 0) & (info_h[:, 0] != L.HCGB_NOT_CONVERGED)))

    # ---- timed region (device-resident inputs)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.profile(False)
    ctx.profile_reset()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = e0.elapsed_time(e1) / args.steps
    launches = int(sum(v[1] for v in ctx.profile_read().values()))
    value, ms = job_throughput(ms, n_updates, device="cuda")

    # ---- one more multiply, serialised on one stream with CUDA events around every stage:
    #      the per-kernel durations behind the roofline (not part of the timed region).
    ctx.set_concurrency(1)
    ctx.profile_reset()
    ctx.profile(True)
    step()
    ctx.profile(False)
    stages = ctx.profile_read()
    ctx.set_concurrency(args.groups)
    serial_ms = sum(v[0] for v in stages.values())

    # ---- end to end through the public API: host (pinned) inputs in, result back to the host.
    #      Tiles travel in the rank-trimmed transfer format (hcgb_pack_tiles): the host holds A and
    #      C packed (only the columns their ranks use); every step copies them in, unpacks them on
    #      the device, multiplies (B = A, as in the device-resident run: one copy serves both
    #      operands), packs C, reads the packed size and copies C and its ranks out.
    Ae = T.TileMatrix(nt, nt, nb, A.kinds, maxr)
    Ce = T.TileMatrix(nt, nt, nb, C0.kinds, maxr)
    a_pk = torch.from_numpy(Ae.host_pack(a_host, a_ranks)).pin_memory()
    c_pk = torch.from_numpy(Ce.host_pack(c_host, c_ranks)).pin_memory()
    ar_pin = torch.from_numpy(a_ranks).pin_memory()
    cr_pin = torch.from_numpy(c_ranks).pin_memory()
    a_dev = torch.empty(a_pk.numel(), dtype=torch.float64, device="cuda")
    c_dev = torch.empty(c_pk.numel(), dtype=torch.float64, device="cuda")
    out_dev = torch.empty(Ce.arena.numel(), dtype=torch.float64, device="cuda")
    offs = [torch.empty(nt * nt + 1, dtype=torch.int64, device="cuda") for _ in range(3)]
    out_pin = torch.empty(Ce.arena.numel(), dtype=torch.float64).pin_memory()
    outr_pin = torch.empty_like(cr_pin).pin_memory()
    total_pin = torch.empty(1, dtype=torch.int64).pin_memory()
    moved = {}

    def e2e_step():
        Ae.ranks.copy_(ar_pin, non_blocking=True)
        a_dev.copy_(a_pk, non_blocking=True)
        Ae.unpack(a_dev, offs[0])
        Ce.ranks.copy_(cr_pin, non_blocking=True)
        c_dev.copy_(c_pk, non_blocking=True)
        Ce.unpack(c_dev, offs[1])
        T.tlr_gemm(1.0, Ae, Ae, 1.0, Ce, params, ctx=T.run_context(local))
        Ce.pack(out_dev, offs[2])
        outr_pin.copy_(Ce.ranks, non_blocking=True)
        total_pin.copy_(offs[2][-1:], non_blocking=True)
        torch.cuda.current_stream().synchronize()  # the packed size of the result
        total = int(total_pin[0])
        out_pin[:total].copy_(out_dev[:total], non_blocking=True)
        moved["h2d"] = a_pk.numel() * 8 + c_pk.numel() * 8 + 4 * (ar_pin.numel() + cr_pin.numel())
        moved["d2h"] = total * 8 + 4 * outr_pin.numel() + 8
        moved["total"] = total

    e2e_step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    e2 = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    e2[0].record(stream)
    for _ in range(args.steps):
        e2e_step()
    e2[1].record(stream)
    torch.cuda.synchronize()
    e2e_ms = e2[0].elapsed_time(e2[1]) / args.steps
    e2e_value, e2e_ms = job_throughput(e2e_ms, n_updates, device="cuda")
    h2d, d2h = moved["h2d"], moved["d2h"]
    # the host copy of the result against the device-resident run's result (same multiply)
    e2e_matches = bool(np.array_equal(out_pin[:moved["total"]].numpy(),
                                      Cw.host_pack(Cw.arena.cpu().numpy(), Cw.ranks.cpu().numpy())))

    if rank != 0:
        return 0

    # ---- accounting: flops, roofline of the dominant stage
    kinds_u = []
    for kk in range(nt):
        for j in range(nt):
            for i in range(nt):
                kinds_u.append((a_t[(i, kk)][0] == "C", b_t[(kk, j)][0] == "C", c_t[(i, j)][0] == "C"))
    pasc = float(np.sum(pasc_flops(info_h[:, 1], info_h[:, 2], info_h[:, 3], nb)[info_h[:, 4] > 0]))
    st_flops = stage_algorithmic_flops(info_h, nb, kinds_u)
    total_stage_ms = sum(v[0] for v in stages.values())
    dom = max(stages, key=lambda s: stages[s][0])
    dom_ms_per_launch = stages[dom][0] / max(stages[dom][1], 1)
    dom_flops_per_launch = st_flops.get(dom, 0.0) / max(stages[dom][1], 1)
    tensor_stages = {"gemm", "qr", "apply_q"}
    peak = dmma_peak if dom in tensor_stages else dfma_peak
    achieved = dom_flops_per_launch / (dom_ms_per_launch * 1e-3) / 1e12
    comp_updates = int(np.count_nonzero(info_h[:, 4] > 0))
    traffic = traffic_from_profiles(dom, args.workload, comp_updates / max(stages[dom][1], 1))

    # ---- accuracy against the FP64 dense product of the TLR inputs (cuBLAS, outside the timing)
    check = {}
    if not args.no_check:
        import torch as th
        Ad = th.from_numpy(A.to_dense()).cuda()
        Cd0 = th.from_numpy(C0.to_dense()).cuda()
        exact = Ad @ Ad + Cd0
        Cres = th.from_numpy(Cw.to_dense()).cuda()
        check["rel_fro_err_vs_fp64_dense_product"] = float(th.linalg.norm(Cres - exact) / th.linalg.norm(exact))
        del Ad, Cd0, exact, Cres
        th.cuda.empty_cache()
    rk = Cw.rank_grid()
    comp_mask = np.array([[c_t[(i, j)][0] == "C" for j in range(nt)] for i in range(nt)])
    clamped = int(np.count_nonzero(info_h[:, 5] >= maxr))

    # ---- CPU baseline (oracle port) on a bounded sample, host cores
    cpu = None
    if not args.no_cpu_baseline:
        procs = os.cpu_count() or 1
        n_tiles = args.cpu_tiles or procs
        upd, wall, sample = cpu_measure(w, a_t, b_t, c_t, n_tiles, procs)
        cpu = {"value": upd / wall, "unit": UNIT, "cores": procs, "kind": "port",
               "sample": f"{n_tiles} seeded C tiles x {nt} k-updates = {upd} updates, {wall:.1f} s wall"}

    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (Morton-sorted exponential kernel, seeded)",
        "config": {"workload": args.workload, "n": w["n"], "nb": w["nb"], "tiles": f"{nt}x{nt}",
                   "updates_per_step": n_updates, "accuracy": w["accuracy"], "threshold": "relative",
                   "dense_diagonal": w["dense_diagonal"], "max_rank": maxr,
                   "form": "plain_fp64" if args.mode == "plain" else "mixed (float-float QR, pivoted QR, Jacobi, Q application)",
                   "parallelism": "replicas" if world > 1 else "single_gpu", "c_tile_groups": args.groups, "k_order": "ascending" if args.k_order == 0 else "cost-descending",
                   "l2": "inputs larger than L2 (A, C arenas 1.4 GB each), no flush"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "transfer": "rank-trimmed packed tiles (hcgb_pack_tiles / hcgb_unpack_tiles), pinned host buffers",
                "result_matches_device_run": e2e_matches},
        "roofline": {"bound": ("fp64_equivalent" if args.mode == "mixed" and dom in ("core_svd", "qr", "apply_q")
                               else ("tensor" if dom in tensor_stages else "fp64_simt")), "kernel": dom,
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                     "traffic": traffic,
                     "peak_source": "measured in this run by hcgb_fp64_peak (FP64 DMMA / DFMA probe); "
                                    "MEASURED_PEAKS.json has no FP64 figure",
                     "note": ("algorithmic FP64-equivalent flops of the stage; in the mixed form it runs in "
                              "float-float arithmetic on the FP32 pipe, so its rate is compared with the FP64 "
                              "peak it replaces" if args.mode == "mixed" else "algorithmic FP64 flops of the stage")},
        "fp64": {"pasc_gflops": pasc / (ms * 1e-3) / 1e9, "pasc_frac_of_dmma_peak": pasc / (ms * 1e-3) / 1e12 / dmma_peak,
                 "dmma_peak_tflops": dmma_peak, "dfma_peak_tflops": dfma_peak},
        "stages_ms_serial_step": {s: stages[s][0] for s in stages},
        "serial_step_ms": serial_ms,
        "stage_share": {s: stages[s][0] / total_stage_ms for s in stages},
        "stage_algorithmic_tflops": {s: st_flops[s] / (stages[s][0] * 1e-3) / 1e12 for s in st_flops
                                     if s in stages and stages[s][0] > 0},
        "gpu_launches": launches,
        "ranks": {"mean_final": float(rk[comp_mask].mean()), "max_final": int(rk[comp_mask].max()),
                  "updates_at_capacity": clamped, "bad_status": bad,
                  "mean_k": float(info_h[info_h[:, 4] > 0, 4].mean()),
                  "max_sweeps": int(info_h[:, 6].max()),
                  "mean_sweeps": float(info_h[info_h[:, 4] > 0, 6].mean()),
                  "mean_core_cols": float(info_h[info_h[:, 4] > 0, 8].mean())},
        "core_kcycles_mean": {nm: float(info_h[info_h[:, 4] > 0, 9 + q].mean())
                              for q, nm in enumerate(["product", "qrcp", "jacobi", "factors"])},
        "check": check,
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
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
