"""The C++ layer with the reference's Expander / check_lazy_trajectory
interface (include/dynoplan_gb300/expander.hpp): compiled with g++ against
libdpg.so; its results must equal the oracle's."""
import os
import struct
import subprocess

import numpy as np
import pytest

import oracle_bind as ob
from dynoplan_gb300 import workloads as W
from parity_util import compare

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_expander.cpp")


def build_cpp(tmp):
    exe = os.path.join(tmp, "test_expander")
    libdir = os.path.join(ROOT, "dynoplan_gb300")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), SRC,
                    "-L", libdir, "-ldpg", f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    return exe


def test_cpp_layer_compiles(dpg_lib, tmp_path):
    """Header and test compile and link against the library (no GPU needed)."""
    assert os.path.exists(build_cpp(str(tmp_path)))


def write_input(path, wl):
    m = wl.robot
    with open(path, "wb") as f:
        f.write(struct.pack("<ii", m.kind, wl.prims.P))
        f.write(wl.prims.length.astype("<i4").tobytes())
        f.write(wl.prims.states.astype("<f8").tobytes())
        f.write(wl.prims.actions.astype("<f8").tobytes())
        f.write(struct.pack("<i", wl.env.dim))
        f.write(wl.env.lo.astype("<f8").tobytes())
        f.write(wl.env.hi.astype("<f8").tobytes())
        f.write(struct.pack("<i", len(wl.env.obs_lo)))
        f.write(wl.env.obs_lo.astype("<f8").tobytes())
        f.write(wl.env.obs_hi.astype("<f8").tobytes())
        f.write(struct.pack("<q", len(wl.nodes)))
        f.write(wl.nodes.astype("<f8").tobytes())
        f.write(struct.pack("<d", wl.radius))


def read_output(path, nx):
    raw = open(path, "rb").read()
    (rows,) = struct.unpack_from("<q", raw, 0)
    rec = np.dtype([("node", "<i4"), ("idx", "<i4"), ("verdict", "<i4"), ("fi", "<i4"), ("x", "<f8", (nx,))])
    a = np.frombuffer(raw, dtype=rec, count=rows, offset=8)
    return {"node": a["node"].astype(np.uint32), "prim": a["idx"].astype(np.uint32),
            "verdict": a["verdict"].astype(np.uint8), "first_invalid": a["fi"].astype(np.int16),
            "end_state": a["x"], "n_pairs": rows}


@pytest.mark.gpu
@pytest.mark.parametrize("cfg,scale", [(1, 0.05), (2, 0.01), (5, 0.01)])
def test_cpp_expander_matches_oracle(dpg_lib, tmp_path, cfg, scale):
    wl = W.make_workload(cfg, scale=scale, seed=300 + cfg)
    exe = build_cpp(str(tmp_path))
    inp, outp = os.path.join(tmp_path, "in.bin"), os.path.join(tmp_path, "out.bin")
    write_input(inp, wl)
    r = subprocess.run([exe, inp, outp], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = read_output(outp, wl.robot.nx)
    ora = ob.expand(wl.robot, wl.prims, wl.env, wl.nodes, wl.radius)
    compare(wl.robot.kind, got, ora, 0, min_gap=False)
