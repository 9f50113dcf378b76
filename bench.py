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
# node_tiles nn_prefix cell_scan cell_scatter gather_nodes (spatial order, batches of
# >= 2048 nodes) prep_nodes nn_grid (key-grid ball scan; nn_mask for the quadrotor)
# nn_prefix scan_totals item_positions nn_emit check_pairs (which also restores the node ids)
KERNELS_PER_STEP = 12
# states per culling chunk of check_pairs by robot kind (the kernel's
# Robot<KIND>::CHUNK): unicycle1 0, car1 1, quadrotor 2, quad2d 3
CHUNK_STATES = {0: 8, 1: 8, 2: 16, 3: 16}
L2_FLUSH_BYTES = 512 << 20

# DRAM bytes per checked pair of a check_pairs launch from ncu
# (dram__bytes_read.sum + dram__bytes_write.sum over the pairs of the captured
# launch), per workload; scaled to the bench's launch by its checked pairs.
# Workloads without a capture report traffic null.
# Instruction issue of the check kernel from the same ncu capture
# (profiles/check_pairs_car1_50k.md): sm__inst_executed.avg.per_cycle_active
# over the SM's 4 issue slots per cycle, and warp instructions per pair.
CHECK_ISSUE = {
    2: {"inst_per_cycle": 2.614, "issue_slots": 4, "warp_instructions_per_pair": 879676364 / 4126228,
        "active_lanes_per_instruction": 17.68},
}
CHECK_TRAFFIC_PER_PAIR = {
    2: (37.874944e6 + 51.243264e6) / 4126228,  # ncu capture (grouped slot rounds), car1_v0 with 50,000 nodes
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=8.0, help="target CPU time per baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiling runs)")
    ap.add_argument("--dropin-nodes", type=int, default=2000, help="nodes of the per-node drop-in arm")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch choices (no autotuner)")
    ap.add_argument("--min-gap", action="store_true",
                    help="time the expands with the min_gap output (a clearance diagnostic the reference lacks)")
    ap.add_argument("--tuning", default="", help="launch choices to apply instead of the autotuner, "
                    "e.g. check_variant=0,check_blocks_per_sm=3 (dpg_tuning fields)")
    ap.add_argument("--arm-envs", type=int, default=40, help="training environments of the surrogate arm")
    ap.add_argument("--no-extras", action="store_true",
                    help="headline workload only: no expansion arms, no other workloads (profiling runs)")
    ap.add_argument("--nodes", type=int, default=None, help="frontier states per step (default: the workload's)")
    ap.add_argument("--envs", type=int, default=200, help="--config 4: training environments")
    ap.add_argument("--forward-kernel", type=int, default=2, choices=[0, 1, 2],
                    help="--config 4: surrogate forward kernel (0 per-layer GEMMs, 1 fused, 2 warp-specialised)")
    ap.add_argument("--problems", type=int, default=100, help="--config 5: evaluation problems")
    ap.add_argument("--train-problems", type=int, default=64, help="--config 5: problems the heuristic learns from")
    return ap.parse_args()


def _np_json(o):
    """numpy scalars in the JSON line"""
    if hasattr(o, "item"):
        return o.item()
    raise TypeError(type(o).__name__)


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
        # the sampler is live (its first row written) before the timed region starts
        t_end = time.time() + 5
        while self.p is not None and time.time() < t_end and self.p.poll() is None:
            if os.path.getsize(self.f.name) > 0:
                break
            time.sleep(0.02)

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
F_POSE = 6          # FP32 ops per state and part: shifted centre, axis-aligned extents
F_NARROW = 22       # FP32 ops of one part-vs-obstacle separating-axis test
F_CULL = 4          # FP32 ops of one box-vs-box overlap test
F_AABB = 8          # FP32 ops of the axis-aligned early reject of one part-obstacle test
F_SAT = 14          # FP32 ops of the remaining separating axes
GAP_CAP = 0.05      # min_gap is reported up to this clearance


def canonical_states(wl, p):
    """FP64 canonical states of primitive p as the device tables hold them:
    the stored states (translation robots) or the rollout of the stored
    actions from the stored start (quad2d, quadrotor)."""
    from dynoplan_gb300 import workloads as W
    xs, us = wl.prims.motion(p)
    if wl.robot.kind in (W.QUAD2D, W.QUAD3D):
        out = [xs[0]]
        for u in us:
            out.append(W.step(wl.robot, out[-1][None], u[None])[0])
        return np.array(out)
    return xs


def part_boxes(wl, xs):
    """[L, parts, 2*D] centre and half extent of each collision part"""
    m = wl.robot
    if m.kind == 2:
        c = xs[:, None, 0:3]
        return np.concatenate([c, np.full_like(c, m.radius)], -1)
    a, b = 0.5 * m.box[0], 0.5 * m.box[1]
    parts = [(xs[:, 0], xs[:, 1], xs[:, 2])]
    if m.kind == 1:
        parts.append((xs[:, 0] - m.hitch * np.cos(xs[:, 3]), xs[:, 1] - m.hitch * np.sin(xs[:, 3]), xs[:, 3]))
    out = []
    for cx, cy, th in parts:
        ac, as_ = np.abs(np.cos(th)), np.abs(np.sin(th))
        out.append(np.stack([cx, cy, a * ac + b * as_, a * as_ + b * ac], -1))
    return np.stack(out, 1)


def algorithmic_check_ops(wl, node, verdict, first_invalid, prim, sample=4000, seed=0,
                          chunk=8, band=1e-4, min_gap=False):
    """FP32 operations of the exact check of these pairs, counted for the
    algorithm check_pairs runs (two-level obstacle culling, separating-axis
    narrow phase), without any divergence or idle-lane waste, in the
    reference's order of checks (bounded transform first; collision only when
    every state is in bounds; check_lazy_trajectory, dbastar.cpp:391-490):

      per pair               O * F_CULL         trajectory-box culling
      per chunk of states    |L1| * F_CULL      chunk-box culling of the L1 set
      per collision-checked  parts * F_POSE + |C_chunk| * parts * F_AABB
      state                  + F_SAT per part-obstacle with gap <= band
      per bounds-checked     2 * pos_dim
      state

    collision-checked states: L (valid), first colliding + 1 (collision), 0
    (out of bounds).  The culling margin is band + slack, plus GAP_CAP when
    min_gap is an output.  Also returns the lower bound any axis-aligned-
    broadphase checker needs (F_NARROW per part-obstacle within GAP_CAP with
    min_gap, within the band without; no culling levels).  Exact on a seeded
    sample of `sample` pairs, scaled to all."""
    m = wl.robot
    n = len(verdict)
    if n == 0:
        return 0, 0
    rng = np.random.default_rng(seed)
    idx = rng.choice(n, size=min(sample, n), replace=False)
    oc = 0.5 * (wl.env.obs_lo + wl.env.obs_hi)
    oh = 0.5 * (wl.env.obs_hi - wl.env.obs_lo)
    O, D = len(oc), wl.env.dim
    cap = GAP_CAP if min_gap else band
    M = (GAP_CAP if min_gap else 0.0) + band + 1e-3
    vel = {0: None, 1: None, 3: [3, 4], 2: [7, 8, 9]}[m.kind]
    cache = {}
    total = lower = 0

    def near(cen, hf):  # boxes [.., D] vs obstacles -> [.., O]
        return (np.abs(cen[..., None, :] - oc) <= hf[..., None, :] + oh + M).all(-1)

    for i in idx:
        p, v, fi = int(prim[i]), int(verdict[i]), int(first_invalid[i])
        L = int(wl.prims.length[p])
        s_col = L if v == 0 else (fi + 1 if v == 1 else 0)
        s_bnd = fi + 1 if v == 2 else L
        ops = O * F_CULL + s_bnd * 2 * D
        low = O * F_CULL + s_bnd * 2 * D
        if s_col and O:
            if p not in cache:
                cache[p] = part_boxes(wl, canonical_states(wl, p))
            bx = cache[p].copy()                      # [L, parts, 2D]
            x = wl.nodes[int(node[i])]
            bx[..., :D] += x[:D]
            if vel is not None:
                t = (np.arange(L) * m.dt)[:, None, None]
                bx[..., :D] += t * x[vel][None, None, :]
            lo = (bx[..., :D] - bx[..., D:]).reshape(L, -1, D)
            hi = (bx[..., :D] + bx[..., D:]).reshape(L, -1, D)
            tl, th = lo.min((0, 1)), hi.max((0, 1))
            l1 = near(0.5 * (tl + th), 0.5 * (th - tl))                     # [O]
            gap = (np.abs(bx[:, :, None, :D] - oc) - bx[:, :, None, D:] - oh).max(-1)  # [L, parts, O]
            for c0 in range(0, s_col, chunk):
                c1 = min(L, c0 + chunk)
                cl, ch = lo[c0:c1].min((0, 1)), hi[c0:c1].max((0, 1))
                cand = l1 & near(0.5 * (cl + ch), 0.5 * (ch - cl))
                ops += int(l1.sum()) * F_CULL
                s1 = min(s_col, c1)
                ops += (s1 - c0) * m.n_parts * (F_POSE + int(cand.sum()) * F_AABB)
                ops += F_SAT * int((gap[c0:s1][:, :, cand] <= band).sum())
            low += s_col * m.n_parts * F_POSE + F_NARROW * int((gap[:s_col] <= cap).sum())
        total += ops
        lower += low
    scale = n / len(idx)
    return int(total * scale), int(lower * scale)

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
                   "obstacles": len(wl.env.obs_lo), "delta": wl.delta, "alpha": wl.alpha,
                   "outputs": "node, prim, verdict, first_invalid, end_state, min_gap (FP64)"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n} of {len(wl.nodes)} frontier states per step"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference expand (oracle/oracle.c orc_expand_fast); the "
                "reference's C++ does not build here (dynobench, nigh, fcl, OMPL absent)",
    }
    print(json.dumps(line, default=_np_json), flush=True)


def device_outputs(torch, cap, nx, prec, dev, min_gap=True):
    o = {
        "node": torch.empty(cap, dtype=torch.int32, device=dev),
        "prim": torch.empty(cap, dtype=torch.int32, device=dev),
        "verdict": torch.empty(cap, dtype=torch.uint8, device=dev),
        "first_invalid": torch.empty(cap, dtype=torch.int16, device=dev),
        "end_state": torch.empty((cap, nx), dtype=torch.float64 if prec != 0 else torch.float32, device=dev),
        "min_gap": torch.empty(cap, dtype=torch.float32, device=dev),
        "flags": torch.empty(cap, dtype=torch.uint8, device=dev),
    }
    if not min_gap:
        del o["min_gap"]
    return o


def outputs_named(min_gap):
    """the outputs a timed expand produces: the reference's (neighbour pairs,
    verdict, first invalid state, end state) and the FP64-decision flag;
    min_gap (a clearance diagnostic the reference does not compute) on request"""
    return "node, prim, verdict, first_invalid, end_state, flags" + (", min_gap" if min_gap else "")


def measure_device(args, lib, ctx, wl, dev, steps, warmup, min_gap=None):
    """Device-resident expand of the workload's nodes: `steps` timed calls
    (CUDA events on the library stream, L2 flushed before each).  Returns
    the timing record and the device output tensors of the last step."""
    min_gap = args.min_gap if min_gap is None else min_gap
    import torch
    N, nx = wl.nodes.shape
    prec = wl.precision
    n_pairs = ctx.expand(wl.nodes, wl.radius, precision=prec)["n_pairs"]   # sizes the outputs
    cap = int(n_pairs * 1.02) + 1024
    x_d = torch.from_numpy(wl.nodes).to(f"cuda:{dev}")
    outs = device_outputs(torch, cap, nx, prec, dev, min_gap)
    ptrs = {k: v.data_ptr() for k, v in outs.items()}
    for _ in range(warmup):
        ctx.expand_device(x_d.data_ptr(), N, wl.radius, ptrs, cap, precision=prec)
    torch.cuda.synchronize()
    dev_ms, check_ms, stage, pairs_total, rechecks = [], [], [], 0, 0
    for _ in range(steps):
        lib.dpg_bench_flush_l2(dev, L2_FLUSH_BYTES)
        r = ctx.expand_device(x_d.data_ptr(), N, wl.radius, ptrs, cap, precision=prec)
        t = ctx.timings()
        dev_ms.append(sum(t[:4]))
        check_ms.append(t[1])
        stage.append(t)
        pairs_total += r["n_pairs"]
        rechecks += r["n_contact_recheck"]
    torch.cuda.synchronize()
    return {"dev_s": sum(dev_ms) * 1e-3, "pairs_total": pairs_total, "n_pairs": n_pairs, "cap": cap,
            "check_s": statistics.mean(check_ms) * 1e-3, "rechecks": rechecks, "stage": stage,
            "x_d": x_d, "outs": outs}


def check_roofline(lib, wl, m, dev, cfg):
    """algorithmic FP32 work of the check kernel from the last step's outputs"""
    n = m["n_pairs"]
    outs = m["outs"]
    verdict = outs["verdict"][:n].cpu().numpy()
    fi = outs["first_invalid"][:n].cpu().numpy()
    prim = outs["prim"][:n].cpu().numpy()
    node = outs["node"][:n].cpu().numpy().view(np.uint32)
    alg_ops, alg_lower = algorithmic_check_ops(wl, node, verdict, fi, prim, chunk=CHUNK_STATES[wl.robot.kind],
                                               min_gap="min_gap" in outs)
    peak = ctypes_peak(lib, dev)
    achieved = alg_ops / m["check_s"] / 1e12
    return {"bound": "fp32", "kernel": "check_pairs", "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak,
            "traffic": (CHECK_TRAFFIC_PER_PAIR[cfg] * n) if cfg in CHECK_TRAFFIC_PER_PAIR else None,
            "peak_source": "FMA-chain kernel on this device (dpg_bench_fp32_peak); "
                           "MEASURED_PEAKS.json holds HBM and bf16 only",
            "alg_ops_per_launch": alg_ops, "check_ms": 1e3 * m["check_s"],
            "work_model": "FP32 ops of the culling algorithm as run, no idle-lane waste "
                          "(bench.algorithmic_check_ops; 4000-pair sample, scaled)",
            "lower_bound_ops_per_launch": alg_lower,
            "lower_bound_tflops": alg_lower / m["check_s"] / 1e12,
            **({"issue": {**CHECK_ISSUE[cfg], "frac": CHECK_ISSUE[cfg]["inst_per_cycle"] / CHECK_ISSUE[cfg]["issue_slots"],
                          "source": "ncu capture of the same kernel, profiles/check_pairs_car1_50k.md; the kernel "
                                    "is bound by instruction issue, not by FP32 arithmetic or DRAM"}}
               if cfg in CHECK_ISSUE else {})}


def cpu_baseline(wl, seconds):
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bind as ob
    threads = ob.lib().orc_max_threads()
    N = len(wl.nodes)
    rate, n, dt, cp = cpu_rate(wl, threads, seconds)
    rate1, n1, dt1, _ = cpu_rate(wl, 1, seconds / 4)
    return {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} of {N} frontier states ({cp} checked pairs, {dt:.1f} s)",
            "value_1_thread": rate1, "sample_1_thread": f"{n1} frontier states ({dt1:.1f} s)"}


def other_workload(args, lib, G, cfg, dev):
    """Device-timed expand of another workload (unicycle1 FP64, quadrotor
    FP32) for the same line: value, check time, pairs, CPU baseline."""
    from dynoplan_gb300 import workloads as W
    wl = W.make_workload(cfg)
    with G.Context(wl.robot, device=dev) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        tune = None
        if not args.no_tune:
            import torch
            x_t = torch.from_numpy(wl.nodes).to(f"cuda:{dev}")
            torch.cuda.synchronize()
            tune = ctx.autotune(x_t.data_ptr(), len(wl.nodes), wl.radius, precision=wl.precision)
            del x_t
        m = measure_device(args, lib, ctx, wl, dev, min(args.steps, 10), args.warmup)
        roof = check_roofline(lib, wl, m, dev, cfg)
        # the same nodes with the reference loop's lazy checks (motion order,
        # limit_branching_factor valid motions per node), against the eager
        # expand's verdicts
        n = m["n_pairs"]
        eager = (m["outs"]["node"][:n].cpu().numpy().view(np.uint32),
                 m["outs"]["prim"][:n].cpu().numpy().view(np.uint32), m["outs"]["verdict"][:n].cpu().numpy())
        t_e, _ = timed_wall(lib, dev, min(args.steps, 10), lambda: ctx.expand_device(
            m["x_d"].data_ptr(), len(wl.nodes), wl.radius, {k: v.data_ptr() for k, v in m["outs"].items()},
            m["cap"], precision=wl.precision))
        lazy = LazyArm(lib, ctx, wl, m["x_d"], dev, n, m["cap"], LIMIT_BRANCHING, args.min_gap)
        lz = lazy.measure(min(args.steps, 10), None, eager)
        del lazy
        m.pop("outs")
        m.pop("x_d")
        # the same expand through the C ABI with page-locked host buffers
        e2e = None
        if not args.no_e2e:
            e2e, pinned = run_e2e(args, lib, G, ctx, wl, m["cap"], n, wl.precision, 8 if wl.precision else 4, dev,
                                  steps=min(args.steps, 10))
            for h in pinned:
                h.free()
    rec = {"workload": wl.name, "robot": wl.robot.name, "dtype": "f64" if wl.precision else "f32",
           "precision": {0: "DPG_FP32", 1: "DPG_FP64 (FP32 tests, FP64 band decisions and end states)"}[wl.precision],
           "primitives": wl.prims.P, "obstacles": len(wl.env.obs_lo), "nodes_per_step": len(wl.nodes),
           "checked_pairs_per_step": m["n_pairs"], "outputs": outputs_named(args.min_gap),
           "value": m["pairs_total"] / m["dev_s"], "unit": UNIT,
           "ms_per_step": 1e3 * m["dev_s"] / min(args.steps, 10), "check_ms": 1e3 * m["check_s"],
           "ball_ms": statistics.mean(t[0] for t in m["stage"]),
           "parity": "tests/test_parity_gpu.py::test_full_size_parity (every pair of this workload vs the oracle)",
           "roofline": {k: roof[k] for k in ("achieved", "peak", "unit", "frac")},
           **({"tuning": tune} if tune else {}),
           **({"e2e": e2e} if e2e else {}),
           "lazy_vs_batched": {"limit_branching_factor": LIMIT_BRANCHING,
                               "rate": "in-ball candidate pairs handled per second (wall clock)",
                               "batched": {"value": n / t_e, "ms": 1e3 * t_e}, "batched_lazy": lz}}
    if not args.no_cpu_baseline:
        rec["cpu_baseline"] = cpu_baseline(wl, args.cpu_seconds / 2)
        rec["vs_cpu_all_cores"] = rec["value"] / rec["cpu_baseline"]["value"]
    return rec


def tune_small_set(lib, G, W, dev):
    """The autotuner on car1 with a 400-primitive set (the primitive count of
    the reference's car1 db-A* configuration) over the bench's nodes:
    chosen choice, its check+ball time and the default's."""
    import torch
    wl = W.make_workload(2)
    prims = W.make_primitives(wl.robot, 400, 5, 100, seed=2400)
    with G.Context(wl.robot, device=dev) as ctx:
        ctx.upload_primitives(prims)
        ctx.upload_env(wl.env)
        x = torch.from_numpy(wl.nodes).to(f"cuda:{dev}")
        torch.cuda.synchronize()
        rep = ctx.autotune(x.data_ptr(), len(wl.nodes), wl.radius, precision=0)
    return {"primitives": 400, "nodes": len(wl.nodes), "tuning": rep}


def run_ours(args, rank, world, local_rank):
    import torch

    from dynoplan_gb300 import _lib
    from dynoplan_gb300 import gpu as G
    from dynoplan_gb300 import replicas
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
    es_bytes = 8 if prec != 0 else 4

    # ---------------- launch choices: the project's autotuner on this batch
    tune = None
    if args.tuning:
        ctx.set_tuning(**{k: int(v) for k, v in (kv.split("=") for kv in args.tuning.split(","))})
        tune = {"chosen": ctx.tuning(), "source": "--tuning"}
    elif not args.no_tune:
        x_t = torch.from_numpy(wl.nodes).to(f"cuda:{dev}")
        torch.cuda.synchronize()
        tune = ctx.autotune(x_t.data_ptr(), N, wl.radius, precision=prec)
        del x_t

    # ---------------- device-resident value
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = Clocks(dev)
    t_wall0 = time.perf_counter()
    m = measure_device(args, lib, ctx, wl, dev, args.steps, args.warmup)
    wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    n_pairs, cap, x_d = m["n_pairs"], m["cap"], m["x_d"]
    total_s, pairs_total = replicas.reduce_step(m["dev_s"], m["pairs_total"], device=dev)
    pairs_total = int(pairs_total)
    value = pairs_total / total_s
    roof = check_roofline(lib, wl, m, dev, args.config)
    check_s = m["check_s"]
    stage = m["stage"]
    rechecks = m["rechecks"]
    del m
    # the same expands with the min_gap output as well (not in the timed value above)
    with_mg = None
    if not args.min_gap:
        m2 = measure_device(args, lib, ctx, wl, dev, min(args.steps, 20), args.warmup, min_gap=True)
        with_mg = {"outputs": outputs_named(True), "value": m2["pairs_total"] / m2["dev_s"],
                   "ms_per_step": 1e3 * m2["dev_s"] / min(args.steps, 20), "check_ms": 1e3 * m2["check_s"]}
        del m2

    # ---------------- e2e through the C ABI with host buffers
    e2e, pinned = None, []
    if not args.no_e2e:
        e2e, pinned = run_e2e(args, lib, G, ctx, wl, cap, n_pairs, prec, es_bytes, dev)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(wl, args.cpu_seconds)

    # unicycle1 workload: the same expand with the ball radius = delta (alpha 1), the
    # second reading of the radius the workload's description allows
    variant = None
    if args.config == 1:
        variant = run_radius_variant(args, lib, ctx, wl, x_d, prec, dev)

    # the expansion arms of the metric on this workload, and the other workloads
    arms, others = None, {}
    if rank == 0 and args.config == 2 and not args.no_extras:
        arms = run_arms(args, lib, G, ctx, wl, x_d, dev)
    for h in pinned:
        h.free()
    ctx.close()
    if rank == 0 and args.config == 2 and not args.no_extras:
        for cfg in (1, 3):
            others[W.CONFIGS[cfg]["name"]] = other_workload(args, lib, G, cfg, dev)
        if not args.no_tune:
            others["car1_v0, 400 primitives (autotuner only)"] = tune_small_set(lib, G, W, dev)
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
                   "parallelism": f"replicas x{world}", "wall_ms_per_step": 1e3 * wall / args.steps,
                   "outputs": outputs_named(args.min_gap)},
        "e2e": e2e,
        **({"with_min_gap": with_mg} if with_mg else {}),
        **({"variant_radius_delta": variant} if variant else {}),
        "gpu_launches": KERNELS_PER_STEP * args.steps,
        "roofline": roof,
        "stage_ms": {k: statistics.mean(t[i] for t in stage) for i, k in
                     enumerate(("ball_scan", "check", "fp64_recheck", "copies"))},
        "cpu_baseline": cpu,
        **({"tuning": tune} if tune else {}),
        **({"expansion_arms": arms} if arms else {}),
        **({"other_workloads": others} if others else {}),
        "clocks": clk,
    }
    print(json.dumps(line, default=_np_json), flush=True)


def timed_wall(lib, dev, steps, fn):
    """median wall time of fn() over `steps` calls (2 warm-up calls; L2
    flushed and the device synchronised around each)"""
    import torch
    for _ in range(2):
        fn()
    ts, r = [], None
    for _ in range(steps):
        lib.dpg_bench_flush_l2(dev, L2_FLUSH_BYTES)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts), r


class LazyArm:
    """ball-only dpg_expand + (scores) + dpg_lazy_check on the workload's
    nodes, with device buffers for n_cand candidates"""

    def __init__(self, lib, ctx, wl, x_d, dev, n_cand, cap, limit, min_gap=False):
        import torch
        nx = wl.nodes.shape[1]
        self.lib, self.ctx, self.wl, self.x_d, self.dev = lib, ctx, wl, x_d, dev
        self.n_cand, self.cap, self.limit = n_cand, cap, limit
        self.cand = {"node": torch.empty(cap, dtype=torch.int32, device=dev),
                     "prim": torch.empty(cap, dtype=torch.int32, device=dev)}
        self.cptr = {k: v.data_ptr() for k, v in self.cand.items()}
        es_t = torch.float64 if wl.precision else torch.float32
        self.lz = {"verdict": torch.empty(cap, dtype=torch.uint8, device=dev),
                   "first_invalid": torch.empty(cap, dtype=torch.int16, device=dev),
                   "end_state": torch.empty((cap, nx), dtype=es_t, device=dev),
                   "flags": torch.empty(cap, dtype=torch.uint8, device=dev)}
        if min_gap:
            self.lz["min_gap"] = torch.empty(cap, dtype=torch.float32, device=dev)
        self.lptr = {k: v.data_ptr() for k, v in self.lz.items()}

    def run(self, score_fn=None):
        ctx, wl, N = self.ctx, self.wl, len(self.wl.nodes)
        ctx.expand_device(self.x_d.data_ptr(), N, wl.radius, self.cptr, self.cap, precision=wl.precision,
                          ball_only=True)
        sc = score_fn() if score_fn else None
        return ctx.lazy_check_device(self.x_d.data_ptr(), N, self.n_cand, self.cptr["node"], self.cptr["prim"],
                                     self.lptr, self.limit, score_ptr=sc.data_ptr() if sc is not None else None,
                                     score_stride=2, precision=wl.precision)

    def measure(self, steps, score_fn, eager, score_host=None):
        """rate, exact checks, and the checks against the eager arm's
        verdicts (eager = (node, prim, verdict) host arrays in the same
        candidate order) and the reference loop's accepted sets"""
        from dynoplan_gb300 import _lib
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from lazy_ref import lazy_accept
        t, st = timed_wall(self.lib, self.dev, steps, lambda: self.run(score_fn))
        n = self.n_cand
        node_h, prim_h, v_eager = eager
        v = self.lz["verdict"][:n].cpu().numpy()
        fl = self.lz["flags"][:n].cpu().numpy()
        same_order = (np.array_equal(self.cand["node"][:n].cpu().numpy().view(np.uint32), node_h) and
                      np.array_equal(self.cand["prim"][:n].cpu().numpy().view(np.uint32), prim_h))
        checked = v != _lib.DPG_UNCHECKED
        acc = (fl & _lib.DPG_FLAG_ACCEPTED) != 0
        score = score_host() if score_host else None
        ref_acc, needed = lazy_accept(node_h, prim_h, v_eager == 0, score, self.limit)
        return {"value": n / t, "ms": 1e3 * t, "exact_checks": st["n_checked"],
                "checked_fraction": st["n_checked"] / max(n, 1), "accepted": st["n_accepted"],
                "rounds": st["rounds"],
                "verdicts_identical": bool(same_order and np.array_equal(v[checked], v_eager[checked])),
                "accepted_as_reference_loop": bool(np.array_equal(acc, ref_acc) and checked[needed].all())}


LIMIT_BRANCHING = 20   # limit_branching_factor default (include/dynoplan/dbastar/options.hpp)


def run_arms(args, lib, G, ctx, wl, x_d, dev):
    """The arms of the metric on the headline workload's nodes, each giving
    every node the successors the search takes (its first
    limit_branching_factor valid motions, or all of them):
      plain_gpu_drop_in   one dpg_expand per node (host buffers), in node
                          order: the GPU behind the reference's per-node
                          expand_lazy + check_lazy_trajectory
      batched             one dpg_expand over the batch, every in-ball pair
                          exact-checked (device outputs)
      batched_lazy        ball-only dpg_expand + dpg_lazy_check in motion
                          order: the reference loop's lazy checks, batched
      batched_lazy_surrogate  ball-only dpg_expand + node features + the
                          BF16 surrogate's forward + dpg_lazy_check ranked
                          by its collision logit
    Rate = in-ball candidate pairs handled per second (wall clock with the
    device synchronised, L2 flushed before each step); the lazy arms also
    report how many candidates they exact-checked.  Every accepted motion is
    exact-checked; `verdicts_identical` compares each lazily checked
    candidate with the batched arm's verdict for it, and
    `accepted_as_reference_loop` the accepted sets with the first-`limit`
    valid candidates in the same ranking."""
    import ctypes as C

    import torch

    from dynoplan_gb300 import _lib
    from dynoplan_gb300 import surrogate as SG
    from dynoplan_gb300 import workloads as W
    N, nx = wl.nodes.shape
    limit = LIMIT_BRANCHING
    steps = max(3, min(args.steps, 10))
    out = {"limit_branching_factor": limit, "unit": UNIT, "nodes": N, "steps": steps,
           "rate": "in-ball candidate pairs handled per second (wall clock, device synchronised)"}

    # ---- plain GPU drop-in: one call per node (a node sample)
    nA = min(N, args.dropin_nodes)
    opts = _lib.ExpandOpts(radius=wl.radius, precision=0, x_on_device=0, out_on_device=0, mode=0,
                           contact_band=1e-4, ball_band=1e-5)
    xs = np.ascontiguousarray(wl.nodes[:nA])
    pairs, secs = C.c_int64(), C.c_double()
    _lib.check(lib.dpg_bench_per_node_expand(ctx.h, C.byref(opts), min(nA, 50), nx, xs.ctypes.data,
                                             C.byref(pairs), C.byref(secs)), ctx.h)     # warm-up
    _lib.check(lib.dpg_bench_per_node_expand(ctx.h, C.byref(opts), nA, nx, xs.ctypes.data,
                                             C.byref(pairs), C.byref(secs)), ctx.h)
    out["plain_gpu_drop_in"] = {"value": pairs.value / secs.value, "nodes": nA, "checked_pairs": pairs.value,
                                "ms_per_node": 1e3 * secs.value / nA}

    # ---- candidates (ball only) and the batched eager expand
    n_cand = ctx.expand(wl.nodes, wl.radius, precision=0, ball_only=True)["n_pairs"]
    cap = n_cand + 1024
    eag = device_outputs(torch, cap, nx, 0, dev, args.min_gap)
    eptr = {k: v.data_ptr() for k, v in eag.items()}

    t_b, _ = timed_wall(lib, dev, steps, lambda: ctx.expand_device(x_d.data_ptr(), N, wl.radius, eptr, cap,
                                                                     precision=0))
    out["batched"] = {"value": n_cand / t_b, "ms": 1e3 * t_b, "checked_pairs": n_cand}
    v_eager = eag["verdict"][:n_cand].cpu().numpy()
    node_h = eag["node"][:n_cand].cpu().numpy().view(np.uint32)
    prim_h = eag["prim"][:n_cand].cpu().numpy().view(np.uint32)

    # ---- lazy arms: candidates, (scores), lazy check
    lazy = LazyArm(lib, ctx, wl, x_d, dev, n_cand, cap, limit, args.min_gap)

    out["batched_lazy"] = lazy.measure(steps, None, (node_h, prim_h, v_eager))

    # surrogate: trained first (outside the timing) on exact labels of other
    # environments of the workload's kind; the bench environment is held out
    t0 = time.perf_counter()
    ds = SG.make_dataset(wl, n_envs=args.arm_envs, nodes_per_env=700, pairs_per_env=50000, seed=4, device=dev)
    model = SG.Surrogate(wl.prims.P, max_rows=65536, device=dev, seed=0)
    SG.train(model, ds, epochs=3, batch=65536, lr=2e-3)
    train_s = time.perf_counter() - t0
    logits = torch.empty((cap, 2), dtype=torch.float32, device=dev)

    def score_fn():
        feat = SG.node_features(ctx, x_d)
        return model.forward(feat, lazy.cand["node"][:n_cand], lazy.cand["prim"][:n_cand], logits[:n_cand])

    out["batched_lazy_surrogate"] = lazy.measure(steps, score_fn, (node_h, prim_h, v_eager),
                                                 score_host=lambda: logits[:n_cand, 0].cpu().numpy())
    out["batched_lazy_surrogate"]["forward_ms"] = model.timing()[0]
    score_h = logits[:n_cand, 0].cpu().numpy()
    y = v_eager != 0
    pred = score_h > 0
    tp = int((pred & y).sum())
    out["surrogate"] = {"train_envs": args.arm_envs, "train_labels": len(ds), "train_s": train_s,
                        "held_out_collision_rate": float(y.mean()),
                        "precision": tp / max(int(pred.sum()), 1), "recall": tp / max(int(y.sum()), 1)}
    out["ratio_batched_lazy_surrogate_vs_plain_gpu_drop_in"] = (
        out["batched_lazy_surrogate"]["value"] / out["plain_gpu_drop_in"]["value"])
    out["ratio_batched_vs_plain_gpu_drop_in"] = out["batched"]["value"] / out["plain_gpu_drop_in"]["value"]
    model.close()
    return out


def run_radius_variant(args, lib, ctx, wl, x_d, prec, dev):
    """Device-resident expand with radius = delta, timed like the main line."""
    import torch
    N, nx = wl.nodes.shape
    radius = wl.delta
    n_pairs = ctx.expand(wl.nodes, radius, precision=prec)["n_pairs"]
    cap = int(n_pairs * 1.02) + 1024
    outs = {
        "node": torch.empty(cap, dtype=torch.int32, device=dev),
        "prim": torch.empty(cap, dtype=torch.int32, device=dev),
        "verdict": torch.empty(cap, dtype=torch.uint8, device=dev),
        "first_invalid": torch.empty(cap, dtype=torch.int16, device=dev),
        "end_state": torch.empty((cap, nx), dtype=torch.float64 if prec != 0 else torch.float32, device=dev),
        "flags": torch.empty(cap, dtype=torch.uint8, device=dev),
    }
    if args.min_gap:
        outs["min_gap"] = torch.empty(cap, dtype=torch.float32, device=dev)
    ptrs = {k: v.data_ptr() for k, v in outs.items()}
    for _ in range(args.warmup):
        ctx.expand_device(x_d.data_ptr(), N, radius, ptrs, cap, precision=prec)
    ms, pairs = 0.0, 0
    for _ in range(args.steps):
        lib.dpg_bench_flush_l2(dev, L2_FLUSH_BYTES)
        r = ctx.expand_device(x_d.data_ptr(), N, radius, ptrs, cap, precision=prec)
        ms += sum(ctx.timings()[:4])
        pairs += r["n_pairs"]
    return {"radius": radius, "value": pairs / (ms * 1e-3), "unit": UNIT,
            "checked_pairs_per_step": n_pairs, "ms_per_step": ms / args.steps}


def run_e2e(args, lib, G, ctx, wl, cap, n_pairs, prec, es_bytes, dev, steps=None):
    """The C ABI with page-locked host buffers: H2D of the nodes, the expand,
    D2H of every output; wall clock per call."""
    steps = args.steps if steps is None else steps
    N, nx = wl.nodes.shape
    xh = G.PinnedArray(wl.nodes.shape, np.float64)
    xh.array[:] = wl.nodes
    hosts = {
        "node": G.PinnedArray(cap, np.uint32), "prim": G.PinnedArray(cap, np.uint32),
        "verdict": G.PinnedArray(cap, np.uint8), "first_invalid": G.PinnedArray(cap, np.int16),
        "end_state": G.PinnedArray((cap, nx), np.float64 if prec != 0 else np.float32),
        "flags": G.PinnedArray(cap, np.uint8),
    }
    if args.min_gap:
        hosts["min_gap"] = G.PinnedArray(cap, np.float32)
    host_out = {k: v.array for k, v in hosts.items()}
    for _ in range(args.warmup):
        ctx.expand(xh.array, wl.radius, precision=prec, capacity=cap, outputs=host_out)
    e2e_s, e2e_pairs = 0.0, 0
    for _ in range(steps):
        lib.dpg_bench_flush_l2(dev, L2_FLUSH_BYTES)
        t0 = time.perf_counter()
        r = ctx.expand(xh.array, wl.radius, precision=prec, capacity=cap, outputs=host_out)
        e2e_s += time.perf_counter() - t0
        e2e_pairs += r["n_pairs"]
    d2h = n_pairs * (4 + 4 + 1 + 2 + es_bytes * nx + 1 + (4 if args.min_gap else 0))
    e2e = {"value": e2e_pairs / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(N * nx * 8),
           "d2h_bytes_per_step": int(d2h), "ms_per_step": 1e3 * e2e_s / steps}
    return e2e, list(hosts.values()) + [xh]


# ------------------------------------------------- surrogate (car1_v0 MLP) --
MLP_IN_USED = 96      # 80 node features + 16 primitive embedding (the rest of the 128 is padding)
MLP_HIDDEN = 256
MLP_OUT_USED = 2      # collision logit, cost-to-go
# assemble, 4 forward GEMMs, loss, 4 x (dW GEMM, dX GEMM), 3 bias-gradient sums,
# one Adam launch over every parameter (also the bf16 and transposed copies);
# the activations' transposes and bias gradients come from the producing kernels
MLP_KERNELS_PER_TRAIN_STEP = 18


def mlp_alg_flops(rows):
    """forward FLOPs of the layers' used widths: 96 -> 256 -> 256 -> 256 -> 2"""
    return 2.0 * rows * (MLP_IN_USED * MLP_HIDDEN + 2 * MLP_HIDDEN * MLP_HIDDEN + MLP_HIDDEN * MLP_OUT_USED)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "hbm_gbs": 6800.0}, "fallback"


def lazy_check_counts(node, valid, score, limit=20):
    """Exact checks a lazy loop needs per node to find `limit` valid motions:
    in motion order (the reference) and in ascending predicted-collision
    order; nodes with fewer valid motions check all of theirs."""
    ref = mlp = 0
    order = np.lexsort((score, node))
    for sel_order, acc in ((np.lexsort((np.arange(len(node)), node)), "ref"), (order, "mlp")):
        n_s, v_s = node[sel_order], valid[sel_order]
        starts = np.flatnonzero(np.r_[True, n_s[1:] != n_s[:-1]])
        ends = np.r_[starts[1:], len(n_s)]
        total = 0
        for s, e in zip(starts, ends):
            c = np.cumsum(v_s[s:e])
            hit = np.searchsorted(c, limit)
            total += (hit + 1) if hit < e - s else (e - s)
        if acc == "ref":
            ref = total
        else:
            mlp = total
    return ref, mlp


def run_surrogate(args, rank, world, local_rank):
    """The learned surrogate on car1_v0: BF16 tcgen05 training steps (batch
    65,536) on exact labels of the car1 workload's primitives in seeded
    environments; then inference and label quality on held-out environments."""
    import torch

    from dynoplan_gb300 import _lib
    from dynoplan_gb300 import surrogate as SG
    from dynoplan_gb300 import workloads as W
    if rank > 0:
        return
    lib = _lib.load()
    dev = local_rank
    torch.cuda.set_device(dev)
    wl = W.make_workload(2)
    batch = 65536
    t0 = time.perf_counter()
    ds = SG.make_dataset(wl, n_envs=args.envs, nodes_per_env=700, pairs_per_env=50000, seed=4, device=dev)
    held = SG.make_dataset(wl, n_envs=8, nodes_per_env=2000, pairs_per_env=10 ** 6, seed=5, device=dev)
    build_s = time.perf_counter() - t0
    model = SG.Surrogate(wl.prims.P, max_rows=1 << 20, device=dev, seed=0)
    model.set_fused(args.forward_kernel)
    g = torch.Generator(device=ds.node.device).manual_seed(0)
    n = len(ds)

    def step(i, lr):
        idx = torch.randint(0, n, (batch,), generator=g, device=ds.node.device)
        loss = model.train_step(ds.node_feat, ds.node[idx].contiguous(), ds.prim[idx].contiguous(),
                                ds.target[idx].contiguous(), lr=lr)
        return loss, model.timing()[0]

    for i in range(args.warmup):
        step(i, 2e-3)
    torch.cuda.synchronize()
    clocks = Clocks(dev)
    ms = []
    losses = []
    for i in range(args.steps):
        lib.dpg_bench_flush_l2(dev, L2_FLUSH_BYTES)
        loss, t = step(i, 2e-3)
        ms.append(t)
        losses.append(loss)
    clk = clocks.stop()
    train_s = sum(ms) * 1e-3
    value = args.steps * batch / train_s
    peaks, src = measured_peaks()
    achieved = 3 * mlp_alg_flops(batch) * args.steps / train_s / 1e12
    # a quality pass: train on to ~3 epochs before the held-out metrics
    extra = max(0, int(3 * n / batch) - args.steps - args.warmup)
    for i in range(extra):
        step(i, 2e-3 * 0.5 * (1 + np.cos(np.pi * i / max(extra, 1))))
    # inference: one launch over up to 2^20 held-out pairs
    m = min(len(held), 1 << 20)
    node_h, prim_h = held.node[:m].contiguous(), held.prim[:m].contiguous()
    out = model.forward(held.node_feat, node_h, prim_h)
    inf_ms = []
    for _ in range(5):
        lib.dpg_bench_flush_l2(dev, L2_FLUSH_BYTES)
        model.forward(held.node_feat, node_h, prim_h, out)
        inf_ms.append(model.timing()[0])
    inf_s = statistics.median(inf_ms) * 1e-3
    logit = out[:, 0].float().cpu().numpy()
    y = held.target[:m, 0].cpu().numpy() > 0.5
    pred = logit > 0
    tp = int((pred & y).sum())
    precision = tp / max(int(pred.sum()), 1)
    recall = tp / max(int(y.sum()), 1)
    ref_checks, mlp_checks = lazy_check_counts(node_h.cpu().numpy(), (~y).astype(np.int64), logit)
    line = {
        "metric": "surrogate training samples/s", "value": value, "unit": "samples/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * train_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
        "data": "synthetic (seeded car1_v0 environments, exact GPU labels)",
        "config": {"workload": "car1_v0 surrogate", "batch": batch, "labels": n, "envs": args.envs,
                   "layers": "128(96 used)->256->256->256->16(2 used), GELU, Adam",
                   "dataset_build_s": build_s, "l2": "flushed between steps"},
        "roofline": {"bound": "tensor", "kernel": "train step (tcgen05 GEMMs + epilogues)", "achieved": achieved,
                     "peak": peaks["bf16_tflops_sustained"], "unit": "TFLOP/s",
                     "frac": achieved / peaks["bf16_tflops_sustained"], "traffic": None,
                     "peak_source": f"{src} bf16 sustained",
                     "work_model": "3 x forward FLOPs of the used widths per sample"},
        "inference": {"pairs": m, "kernel": args.forward_kernel, "ms": 1e3 * inf_s, "pairs_per_s": m / inf_s,
                      "tflops": mlp_alg_flops(m) / inf_s / 1e12,
                      "frac": mlp_alg_flops(m) / inf_s / 1e12 / peaks["bf16_tflops"]},
        "quality": {"held_out_pairs": m, "collision_rate": float(y.mean()), "precision": precision,
                    "recall": recall, "loss_last": losses[-1],
                    "lazy_checks_for_20_valid": {"motion_order": ref_checks, "mlp_order": mlp_checks}},
        "gpu_launches": MLP_KERNELS_PER_TRAIN_STEP * args.steps,
        "clocks": clk,
    }
    print(json.dumps(line, default=_np_json), flush=True)


# --------------------------------------------- end-to-end search (quad2d) --
def run_search(args, rank, world, local_rank):
    """db-A* on quad2d_v0 problems (8 x 4 m, 20-60 boxes, start and goal at
    rest in free space), 10,000 primitives of 20-150 steps: the plain time
    lower-bound heuristic against the learned cost-to-go (trained first on
    separate problems from completed plain searches).  Reports
    time-to-first-solution and cost per heuristic."""
    import torch

    from dynoplan_gb300 import gpu as G
    from dynoplan_gb300 import search as S
    from dynoplan_gb300 import surrogate as SG
    from dynoplan_gb300 import workloads as W
    if rank > 0:
        return
    dev = local_rank
    torch.cuda.set_device(dev)
    m = W.robot_model(W.QUAD2D)
    prims = W.make_primitives_hover(m, 10000, 20, 150, seed=1005)
    problem = lambda i: W.make_search_problem(m, (8.0, 4.0), (20, 60), (0.2, 1.0), seed=1005 + 17 * i)
    train_probs = [problem(i) for i in range(args.problems, args.problems + args.train_problems)]
    eval_probs = [problem(i) for i in range(args.problems)]
    delta, batch, limit_ms = 0.5, 32, 5000.0
    t0 = time.perf_counter()
    ds, tr = SG.search_dataset(m, prims, train_probs,
                               S.options(delta, batch=batch, max_expands=10 ** 6, time_limit_ms=limit_ms),
                               device=dev)
    model = SG.Surrogate(prims.P, max_rows=65536, device=dev, seed=0)
    _, train_sps, train_tf = SG.train(model, ds, epochs=8, batch=16384, lr=2e-3)
    setup_s = time.perf_counter() - t0
    clocks = Clocks(dev)
    rows = {}
    with G.Context(m, device=dev) as ctx:
        ctx.upload_primitives(prims)
        for name, heu in (("plain", S.HEU_EUCLIDEAN), ("mlp", S.HEU_MLP)):
            opts = S.options(delta, batch=batch, heuristic=heu, max_expands=10 ** 6, time_limit_ms=limit_ms)
            rows[name] = []
            for env, s, g in eval_probs:
                ctx.upload_env(env)
                r, _, _ = S.search(ctx, s, g, opts, mlp=model if heu == S.HEU_MLP else None)
                rows[name].append(r)
    clk = clocks.stop()

    def summary(rs):
        solved = [r for r in rs if r["solved"]]
        t = [r["time_ms"] for r in solved]
        return {"solved": len(solved), "of": len(rs),
                "median_time_ms": statistics.median(t) if t else None,
                "mean_time_ms": statistics.mean(t) if t else None,
                "median_cost_s": statistics.median([r["cost"] for r in solved]) if solved else None,
                "expands": int(sum(r["expands"] for r in rs)), "checked_pairs": int(sum(r["checked_pairs"] for r in rs)),
                "expand_ms": sum(r["expand_ms"] for r in rs), "novelty_ms": sum(r["novelty_ms"] for r in rs),
                "mlp_ms": sum(r["mlp_ms"] for r in rs), "prepare_ms": sum(r["prepare_ms"] for r in rs),
                "insert_ms": sum(r["insert_ms"] for r in rs), "rounds": sum(r["rounds"] for r in rs),
                "table_ms": sum(r["table_ms"] for r in rs), "query_ms": sum(r["query_ms"] for r in rs),
                "total_ms": sum(r["time_ms"] for r in rs)}
    both = [i for i in range(len(eval_probs)) if rows["plain"][i]["solved"] and rows["mlp"][i]["solved"]]
    ratio = [rows["plain"][i]["time_ms"] / max(rows["mlp"][i]["time_ms"], 1e-3) for i in both]
    cost_ratio = [rows["mlp"][i]["cost"] / max(rows["plain"][i]["cost"], 1e-9) for i in both]
    plain = summary(rows["plain"])
    line = {
        "metric": "db-A* time to first solution (median over solved problems, plain heuristic)",
        "value": plain["median_time_ms"], "unit": "ms", "n_gpus": 1, "steps": len(eval_probs), "warmup": 0,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded quad2d_v0 problems, hover-chaining primitives)",
        "config": {"workload": "quad2d_v0 end-to-end", "primitives": prims.P, "steps_per_primitive": [20, 150],
                   "env": "8 x 4 m, 20-60 boxes of 0.2-1.0 m", "delta": delta, "alpha": 0.5,
                   "batch": batch, "time_limit_ms": limit_ms, "train_problems": len(train_probs),
                   "train_solved": int(sum(r["solved"] for r in tr)), "train_labels": len(ds),
                   "setup_s": setup_s, "train_samples_per_s": train_sps, "train_tflops": train_tf},
        "plain": plain, "mlp": summary(rows["mlp"]),
        "both_solved": len(both),
        "median_speedup_mlp": statistics.median(ratio) if ratio else None,
        "geomean_speedup_mlp": float(np.exp(np.mean(np.log(ratio)))) if ratio else None,
        "median_cost_ratio_mlp": statistics.median(cost_ratio) if cost_ratio else None,
        "clocks": clk,
    }
    print(json.dumps(line, default=_np_json), flush=True)


def ctypes_peak(lib, dev):
    import ctypes as C
    v = C.c_double()
    rc = lib.dpg_bench_fp32_peak(dev, 20, C.byref(v))
    return v.value if rc == 0 else float("nan")


def spawn_ranks(args):
    """`--gpus N` outside torchrun: start N ranks of this script on one node
    (127.0.0.1 rendezvous) and return their exit status."""
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__), *sys.argv[1:]]
    return subprocess.call(cmd)


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(spawn_ranks(args))
    rank, world, local_rank = dist_info()
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.config == 4:
        run_surrogate(args, rank, world, local_rank)
    elif args.config == 5:
        run_search(args, rank, world, local_rank)
    else:
        run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
