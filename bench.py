#!/usr/bin/env python3
"""Benchmark of the batched db-A* node expansion.

One step = one dpg_expand over a batch of frontier states (car1_v0, 5,000
primitives, 80 obstacles, 100,000 nodes: the batched FP32 workload).  The
metric is checked (node, primitive) expansions per second: every in-ball
pair that went through transform, bounds and collision check.

  value      device-resident inputs and outputs, device time of the expand
             (CUDA events on the library's stream), L2 flushed between steps
  e2e        the C ABI called with page-locked HOST buffers: host->device
             copy of the nodes, expand, device->host copy of all results,
             wall clock per call
  roofline   the exact-check kernel (check_pairs) against the FP32 rate
             measured on this device by an FMA-chain kernel
  cpu_baseline  the oracle's CPU restatement of the reference expand
             (sorted-angle radius query, grid broadphase, per-pair early
             exit, OpenMP over nodes) on a bounded node sample

``--impl reference`` times that CPU restatement alone (the reference's own
C++ cannot be built: its dynobench/nigh/fcl dependencies are absent).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "checked (node,primitive) expansions/s"
UNIT = "pairs/s"
KERNELS_PER_STEP = 6  # prep_nodes nn_mask nn_prefix scan_totals nn_emit check_pairs
L2_FLUSH_BYTES = 512 << 20

# DRAM bytes per check_pairs launch from ncu (dram__bytes_read.sum +
# dram__bytes_write.sum), scaled to the full workload by checked pairs; None
# until a capture exists.
CHECK_TRAFFIC_PER_PAIR = None


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=8.0, help="target CPU time per baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiling runs)")
    ap.add_argument("--nodes", type=int, default=None, help="frontier states per step (default: the workload's)")
    return ap.parse_args()


def dist_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


# ------------------------------------------------------------------ clocks --
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [s.strip() for s in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(s):
            try:
                return float(s)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1])]
        mx = [num(r[2]) for r in rows if num(r[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max([num(r[3]) for r in rows if num(r[3])] or [0])}


# ---------------------------------------------------------- work accounting --
def algorithmic_check_ops(wl, verdict, first_invalid, prim):
    """FP32 operations the exact check must spend, brute force over the
    obstacles, with the reference's order of checks (bounded transform first,
    collision only when every state is in bounds, check_lazy_trajectory at
    src/dbastar/dbastar.cpp:391-490):
      per collision-checked state: parts * (6 pose ops + O * 8 box-test ops)
      (sphere: 10 ops per obstacle), per bounds-checked state: 2 * pos_dim
    States collision-checked: L (valid), first colliding + 1 (collision),
    0 (out of bounds).  States bounds-checked: L, or first invalid + 1."""
    m = wl.robot
    L = wl.prims.length[prim].astype(np.int64)
    fi = first_invalid.astype(np.int64)
    s_col = np.where(verdict == 0, L, np.where(verdict == 1, fi + 1, 0))
    s_bnd = np.where(verdict == 2, fi + 1, L)
    O = len(wl.env.obs_lo)
    parts = m.n_parts
    per_state = parts * (6 + O * (10 if m.kind == 2 else 8))
    pos = 3 if m.kind == 2 else 2
    return int(s_col.sum()) * per_state + int(s_bnd.sum()) * 2 * pos


# ---------------------------------------------------------------- CPU side --
def cpu_rate(wl, threads, seconds, seed=0):
    """Oracle fast expand on a node sample sized to take ~`seconds`."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bind as ob
    n = min(len(wl.nodes), 64)
    while True:
        sample = wl.nodes[:n]
        t0 = time.perf_counter()
        r = ob.expand(wl.robot, wl.prims, wl.env, sample, wl.radius, fast=True, threads=threads)
        dt = time.perf_counter() - t0
        if dt >= 0.25 * seconds or n >= len(wl.nodes):
            break
        n = min(len(wl.nodes), int(n * max(2.0, 0.5 * seconds / max(dt, 1e-3))))
    return r["n_pairs"] / dt, n, dt, r["n_pairs"]


def run_reference(args, rank, world):
    from dynoplan_gb300 import workloads as W
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bind as ob
    wl = W.make_workload(args.config)
    threads = ob.lib().orc_max_threads()
    # size one step to ~`cpu_seconds` / 2 of wall time
    _, n, dt, _ = cpu_rate(wl, threads, max(1.0, args.cpu_seconds / 2))
    sample = wl.nodes[:n]
    for _ in range(args.warmup):
        ob.expand(wl.robot, wl.prims, wl.env, sample[: max(1, n // 8)], wl.radius, fast=True, threads=threads)
    times, pairs = [], 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r = ob.expand(wl.robot, wl.prims, wl.env, sample, wl.radius, fast=True, threads=threads)
        times.append(time.perf_counter() - t0)
        pairs += r["n_pairs"]
    total = sum(times)
    v = pairs / total
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": wl.name, "primitives": wl.prims.P, "nodes_per_step": n,
                   "obstacles": len(wl.env.obs_lo), "delta": wl.delta, "alpha": wl.alpha},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n} of {len(wl.nodes)} frontier states per step"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference expand (oracle/oracle.c orc_expand_fast); the "
                "reference's C++ does not build here (dynobench, nigh, fcl, OMPL absent)",
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local_rank):
    import torch

    from dynoplan_gb300 import _lib
    from dynoplan_gb300 import gpu as G
    from dynoplan_gb300 import workloads as W

    lib = _lib.load()
    dev = local_rank
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    # weak scaling: every rank expands its own frontier batch (replicas; the
    # nodes are independent, no exchange)
    c = W.CONFIGS[args.config]
    wl = W.make_workload(args.config, N=args.nodes)
    if rank > 0:
        wl.nodes = W.make_nodes(wl.robot, wl.env, len(wl.nodes), seed=wl.seed + 13 + 1000 * rank)
    N, nx = wl.nodes.shape
    ctx = G.Context(wl.robot, device=dev)
    ctx.upload_primitives(wl.prims)
    ctx.upload_env(wl.env)
    prec = wl.precision
    es_bytes = 8 if prec == 1 else 4

    # size the outputs from one probing call
    probe = ctx.expand(wl.nodes, wl.radius, precision=prec)
    n_pairs = probe["n_pairs"]
    cap = int(n_pairs * 1.02) + 1024

    # ---------------- device-resident value
    x_d = torch.from_numpy(wl.nodes).to(f"cuda:{dev}")
    outs = {
        "node": torch.empty(cap, dtype=torch.int32, device=dev),
        "prim": torch.empty(cap, dtype=torch.int32, device=dev),
        "verdict": torch.empty(cap, dtype=torch.uint8, device=dev),
        "first_invalid": torch.empty(cap, dtype=torch.int16, device=dev),
        "end_state": torch.empty((cap, nx), dtype=torch.float64 if prec == 1 else torch.float32, device=dev),
        "min_gap": torch.empty(cap, dtype=torch.float32, device=dev),
        "flags": torch.empty(cap, dtype=torch.uint8, device=dev),
    }
    ptrs = {k: v.data_ptr() for k, v in outs.items()}
    for _ in range(args.warmup):
        ctx.expand_device(x_d.data_ptr(), N, wl.radius, ptrs, cap, precision=prec)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = Clocks(dev)
    dev_ms, check_ms, stage, pairs_total, rechecks = [], [], [], 0, 0
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        lib.dpg_bench_flush_l2(dev, L2_FLUSH_BYTES)
        r = ctx.expand_device(x_d.data_ptr(), N, wl.radius, ptrs, cap, precision=prec)
        t = ctx.timings()
        dev_ms.append(sum(t[:4]))
        check_ms.append(t[1])
        stage.append(t)
        pairs_total += r["n_pairs"]
        rechecks += r["n_contact_recheck"]
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    total_s = sum(dev_ms) * 1e-3
    if world > 1:
        tt = torch.tensor([total_s], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        total_s = float(tt.item())
        pp = torch.tensor([pairs_total], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(pp)
        pairs_total = int(pp.item())
    value = pairs_total / total_s

    # work model of the exact check, from the last step's outputs
    verdict = outs["verdict"][:n_pairs].cpu().numpy()
    fi = outs["first_invalid"][:n_pairs].cpu().numpy()
    prim = outs["prim"][:n_pairs].cpu().numpy()
    alg_ops = algorithmic_check_ops(wl, verdict, fi, prim)
    check_s = statistics.mean(check_ms) * 1e-3
    peak = ctypes_peak(lib, dev)
    achieved = alg_ops / check_s / 1e12

    # ---------------- e2e through the C ABI with host buffers
    e2e, pinned = None, []
    if not args.no_e2e:
        e2e, pinned = run_e2e(args, lib, G, ctx, wl, cap, n_pairs, prec, es_bytes, dev)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_bind as ob
        threads = ob.lib().orc_max_threads()
        rate, n, dt, cp = cpu_rate(wl, threads, args.cpu_seconds)
        rate1, n1, dt1, _ = cpu_rate(wl, 1, args.cpu_seconds / 4)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{n} of {N} frontier states ({cp} checked pairs, {dt:.1f} s)",
               "value_1_thread": rate1, "sample_1_thread": f"{n1} frontier states ({dt1:.1f} s)"}

    for h in pinned:
        h.free()
    ctx.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if prec == 0 else "f64",
        "data": "synthetic (seeded: random-control primitives, random boxes, free-space nodes)",
        "config": {"workload": wl.name, "robot": wl.robot.name, "primitives": wl.prims.P,
                   "steps_per_primitive": list(c["steps"]), "obstacles": len(wl.env.obs_lo),
                   "nodes_per_step": N, "delta": wl.delta, "alpha": wl.alpha, "radius": wl.radius,
                   "checked_pairs_per_step": n_pairs, "fp64_rechecks_per_step": rechecks // args.steps,
                   "l2": f"flushed between steps ({L2_FLUSH_BYTES >> 20} MiB write)",
                   "parallelism": f"replicas x{world}", "wall_ms_per_step": 1e3 * wall / args.steps},
        "e2e": e2e,
        "gpu_launches": KERNELS_PER_STEP * args.steps,
        "roofline": {"bound": "fp32", "kernel": "check_pairs", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak,
                     "traffic": (CHECK_TRAFFIC_PER_PAIR * n_pairs) if CHECK_TRAFFIC_PER_PAIR else None,
                     "peak_source": "FMA-chain kernel on this device (dpg_bench_fp32_peak); "
                                    "MEASURED_PEAKS.json holds HBM and bf16 only",
                     "alg_ops_per_launch": alg_ops, "check_ms": 1e3 * check_s},
        "stage_ms": {k: statistics.mean(t[i] for t in stage) for i, k in
                     enumerate(("ball_scan", "check", "fp64_recheck", "copies"))},
        "cpu_baseline": cpu,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def run_e2e(args, lib, G, ctx, wl, cap, n_pairs, prec, es_bytes, dev):
    """The C ABI with page-locked host buffers: H2D of the nodes, the expand,
    D2H of every output; wall clock per call."""
    N, nx = wl.nodes.shape
    xh = G.PinnedArray(wl.nodes.shape, np.float64)
    xh.array[:] = wl.nodes
    hosts = {
        "node": G.PinnedArray(cap, np.uint32), "prim": G.PinnedArray(cap, np.uint32),
        "verdict": G.PinnedArray(cap, np.uint8), "first_invalid": G.PinnedArray(cap, np.int16),
        "end_state": G.PinnedArray((cap, nx), np.float64 if prec == 1 else np.float32),
        "min_gap": G.PinnedArray(cap, np.float32), "flags": G.PinnedArray(cap, np.uint8),
    }
    host_out = {k: v.array for k, v in hosts.items()}
    for _ in range(args.warmup):
        ctx.expand(xh.array, wl.radius, precision=prec, capacity=cap, outputs=host_out)
    e2e_s, e2e_pairs = 0.0, 0
    for _ in range(args.steps):
        lib.dpg_bench_flush_l2(dev, L2_FLUSH_BYTES)
        t0 = time.perf_counter()
        r = ctx.expand(xh.array, wl.radius, precision=prec, capacity=cap, outputs=host_out)
        e2e_s += time.perf_counter() - t0
        e2e_pairs += r["n_pairs"]
    d2h = n_pairs * (4 + 4 + 1 + 2 + es_bytes * nx + 4 + 1)
    e2e = {"value": e2e_pairs / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(N * nx * 8),
           "d2h_bytes_per_step": int(d2h), "ms_per_step": 1e3 * e2e_s / args.steps}
    return e2e, list(hosts.values()) + [xh]


def ctypes_peak(lib, dev):
    import ctypes as C
    v = C.c_double()
    rc = lib.dpg_bench_fp32_peak(dev, 20, C.byref(v))
    return v.value if rc == 0 else float("nan")


def main():
    args = parse()
    rank, world, local_rank = dist_info()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
