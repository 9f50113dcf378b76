"""Generate the golden fixtures in this directory.

Reads the reference's own data (the dynoplan checkout, a required
argument: ``python make_golden.py <dynoplan checkout>``) and writes small
JSON fixtures; it also records the
oracle's outputs on small seeded workloads.  Run it where the reference is
present; the fixtures it writes are committed and the tests only read them.

  reference data used (paths inside the dynoplan project):
    data/motion_primitives/unicycle1_v0/
        unicycle1_v0__ispso__2023_04_03__14_56_57.bin.less.bin.msgpack
    benchmark_initguess/unicycle1_v0/bugtrap_0/delta_10_v0.yaml   (jump annotations)
    benchmark_initguess/unicycle2_v0/bugtrap_0/delta_10_v0.yaml   (jump annotations)
    benchmark_initguess/quad2d/bugtrap/delta_045_v0.yaml          (states + actions)
    benchmark_initguess/quad2d/recovery_wo_obs/delta_03_v0.yaml
    benchmark_initguess/quadrotor_v0/recovery/delta_05_v0.yaml
    benchmark_initguess/quadrotor_v0/recovery/delta_10_v0.yaml
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))


def read_msgpack(path):
    import msgpack  # available where the fixtures are generated
    with open(path, "rb") as f:
        return msgpack.unpackb(f.read(), raw=False)


def read_traj_yaml(path):
    """Top-level scalars, and the `states:` / `actions:` lists of a db-A*
    output file; `# jump from [...] to [...] delta D min time T` comments."""
    out, cur, jumps = {}, None, []
    jre = re.compile(r"#\s*jump from \[([^\]]*)\] to \[([^\]]*)\] delta ([-0-9.e+]+) min time ([-0-9.e+]+)")
    for line in open(path):
        s = line.rstrip("\n")
        m = jre.search(s)
        if m:
            jumps.append(dict(frm=[float(v) for v in m.group(1).split(",")],
                              to=[float(v) for v in m.group(2).split(",")],
                              delta=float(m.group(3)), min_time=float(m.group(4))))
            continue
        t = s.strip()
        if t.startswith("#"):
            continue
        m = re.match(r"^\s*-?\s*([A-Za-z_]+):\s*(.*)$", s)
        if m:
            key, val = m.group(1), m.group(2)
            if val == "":
                cur = key
                out.setdefault(key, [])
            else:
                cur = None
                out[key] = val
            continue
        if cur and t.startswith("- ["):
            out[cur].append([float(v) for v in t[3:t.index("]")].split(",")])
    return out, jumps


def copy_bundled_msgpack(ref):
    """the bundled unicycle1 file itself (81 kB), byte for byte: the reader's
    and writer's format fixture"""
    src = os.path.join(ref, "data/motion_primitives/unicycle1_v0/"
                            "unicycle1_v0__ispso__2023_04_03__14_56_57.bin.less.bin.msgpack")
    with open(src, "rb") as f, open(os.path.join(HERE, "unicycle1_bundled_primitives.msgpack"), "wb") as g:
        g.write(f.read())


def main(ref):
    # 1. bundled unicycle1 primitives
    d = read_msgpack(os.path.join(ref, "data/motion_primitives/unicycle1_v0/"
                                       "unicycle1_v0__ispso__2023_04_03__14_56_57.bin.less.bin.msgpack"))
    json.dump({"source": "data/motion_primitives/unicycle1_v0/unicycle1_v0__ispso__2023_04_03__14_56_57"
                         ".bin.less.bin.msgpack", "data": d["data"]},
              open(os.path.join(HERE, "unicycle1_bundled_primitives.json"), "w"))
    copy_bundled_msgpack(ref)

    # 2. jump annotations (distance and lower_bound_time pins)
    jumps = {}
    for robot, rel in (("unicycle1_v0", "benchmark_initguess/unicycle1_v0/bugtrap_0/delta_10_v0.yaml"),
                       ("unicycle2_v0", "benchmark_initguess/unicycle2_v0/bugtrap_0/delta_10_v0.yaml")):
        _, j = read_traj_yaml(os.path.join(ref, rel))
        jumps[robot] = {"source": rel, "jumps": j}
    json.dump(jumps, open(os.path.join(HERE, "jump_annotations.json"), "w"), indent=1)

    # 3. recorded trajectories (dynamics pins for quad2d and quadrotor)
    trajs = []
    for robot, rel in (("quad2d_v0", "benchmark_initguess/quad2d/bugtrap/delta_045_v0.yaml"),
                       ("quad2d_v0", "benchmark_initguess/quad2d/recovery_wo_obs/delta_03_v0.yaml"),
                       ("quadrotor_v0", "benchmark_initguess/quadrotor_v0/recovery/delta_05_v0.yaml"),
                       ("quadrotor_v0", "benchmark_initguess/quadrotor_v0/recovery/delta_10_v0.yaml"),
                       ("unicycle1_v0", "benchmark_initguess/unicycle1_v0/bugtrap_0/delta_10_v0.yaml")):
        t, _ = read_traj_yaml(os.path.join(ref, rel))
        trajs.append({"robot": robot, "source": rel, "states": t["states"], "actions": t["actions"],
                      "delta": float(t["delta"]) if "delta" in t else None,
                      "max_jump": float(t["max_jump"]) if "max_jump" in t else None})
    json.dump(trajs, open(os.path.join(HERE, "recorded_trajectories.json"), "w"))

    # 4. oracle outputs on small seeded workloads
    import oracle_bind as ob
    from dynoplan_gb300 import workloads as W
    for cfg, scale in ((1, 0.05), (2, 0.01), (3, 0.004), (5, 0.005)):
        wl = W.make_workload(cfg, scale=scale)
        res = ob.expand(wl.robot, wl.prims, wl.env, wl.nodes, wl.radius)
        np.savez_compressed(
            os.path.join(HERE, f"oracle_cfg{cfg}.npz"),
            kind=wl.robot.kind, length=wl.prims.length, states=wl.prims.states, actions=wl.prims.actions,
            env_lo=wl.env.lo, env_hi=wl.env.hi, obs_lo=wl.env.obs_lo, obs_hi=wl.env.obs_hi,
            nodes=wl.nodes, radius=wl.radius, precision=wl.precision,
            node=res["node"], prim=res["prim"], verdict=res["verdict"],
            first_invalid=res["first_invalid"], end_state=res["end_state"], min_gap=res["min_gap"])
        print(f"cfg{cfg}: P={wl.prims.P} N={len(wl.nodes)} pairs={res['n_pairs']}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <path of the dynoplan checkout>")
    main(sys.argv[1])
