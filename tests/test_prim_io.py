"""Motion-primitive files and the loader semantics (include/dpg_prim_io.h),
and the device-side prepend + re-index (dpg_prepend_primitives).

The format fixture is the reference's bundled unicycle1 file, byte for byte
(tests/golden/unicycle1_bundled_primitives.msgpack, copied by
tests/golden/make_golden.py), with the values an independent msgpack
decoder read from it (unicycle1_bundled_primitives.json)."""
import json
import os

import numpy as np
import pytest

from dynoplan_gb300 import primitives_io as PIO
from dynoplan_gb300 import workloads as W

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MSGPACK = os.path.join(GOLD, "unicycle1_bundled_primitives.msgpack")


def _fixture():
    d = json.load(open(os.path.join(GOLD, "unicycle1_bundled_primitives.json")))["data"]
    length = np.array([len(t["states"]) for t in d], np.int32)
    states = np.concatenate([np.array(t["states"], np.float64) for t in d])
    actions = np.concatenate([np.array(t["actions"], np.float64) for t in d])
    return length, states, actions


def test_read_bundled_file_matches_fixture(dpg_lib):
    pr = PIO.read_msgpack(MSGPACK)
    length, states, actions = _fixture()
    assert pr.P == 100
    assert np.array_equal(pr.length, length)
    assert np.array_equal(pr.states, states)      # float32 values, exactly
    assert np.array_equal(pr.actions, actions)


def test_truncation_to_max_motions(dpg_lib):
    full = PIO.read_msgpack(MSGPACK)
    part = PIO.read_msgpack(MSGPACK, max_motions=7)
    assert part.P == 7
    n = int(full.length[:7].sum())
    assert np.array_equal(part.states, full.states[:n])
    assert np.array_equal(part.actions, full.actions[:n - 7])


def test_compact_write_reproduces_the_bundled_bytes(dpg_lib, tmp_path):
    pr = PIO.read_msgpack(MSGPACK)
    out = tmp_path / "w.msgpack"
    PIO.write_msgpack(out, pr, compact=True)
    assert out.read_bytes() == open(MSGPACK, "rb").read()


def test_write_float64_round_trip(dpg_lib, tmp_path):
    pr = W.make_primitives(W.robot_model(W.QUAD3D), 20, 5, 40, seed=3)
    out = tmp_path / "q.msgpack"
    PIO.write_msgpack(out, pr, compact=False)
    back = PIO.read_msgpack(out)
    assert np.array_equal(back.length, pr.length)
    assert np.array_equal(back.states, pr.states) and np.array_equal(back.actions, pr.actions)
    PIO.write_msgpack(out, pr, compact=True)  # lossless too
    back = PIO.read_msgpack(out)
    assert np.array_equal(back.states, pr.states) and np.array_equal(back.actions, pr.actions)


def test_rejects_malformed_files(dpg_lib, tmp_path):
    from dynoplan_gb300._lib import DpgError
    bad = tmp_path / "bad.msgpack"
    bad.write_bytes(b"\x81\xa4data\x91\x82\xa6states\x92\x92\x01\x02\x92\x03\x04\xa7actions\x90")  # 2 states, 0 actions
    with pytest.raises(DpgError):
        PIO.read_msgpack(bad)
    bad.write_bytes(open(MSGPACK, "rb").read()[:-7])  # truncated
    with pytest.raises(DpgError):
        PIO.read_msgpack(bad)
    with pytest.raises(DpgError):
        PIO.read_msgpack(tmp_path / "missing.msgpack")


def test_prepare_noise_and_quaternions(dpg_lib):
    pr = W.make_primitives(W.robot_model(W.QUAD3D), 30, 5, 20, seed=4, noise=0.0)
    pr.states[:, 3:7] *= 1.5  # denormalised quaternions
    out = PIO.prepare(pr, W.QUAD3D, noise=1e-7, seed=9)
    assert np.allclose(np.linalg.norm(out.states[:, 3:7], axis=1), 1.0, atol=1e-15)
    soff = pr.soff()
    last = soff + pr.length - 1
    inner = np.setdiff1d(np.arange(len(pr.states)), np.r_[soff, last])
    base = pr.states.copy()
    base[:, 3:7] /= np.linalg.norm(base[:, 3:7], axis=1, keepdims=True)
    # untouched inner states (after normalisation), bounded noise elsewhere
    assert np.array_equal(out.states[inner], base[inner])
    assert np.abs(out.states[soff][:, [0, 1, 2, 7, 8]] - pr.states[soff][:, [0, 1, 2, 7, 8]]).max() <= 1e-7
    assert np.abs(out.states[soff][:, [0, 1, 2]] - pr.states[soff][:, [0, 1, 2]]).max() > 0
    again = PIO.prepare(pr, W.QUAD3D, noise=1e-7, seed=9)
    assert np.array_equal(again.states, out.states)  # seeded


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", [1, 2, 3, 5])
def test_prepend_equals_upload_of_concatenation(dpg_lib, cfg):
    """prepend(new) after upload(old) == upload(new ++ old), every output"""
    from dynoplan_gb300 import gpu as G
    wl = W.make_workload(cfg, scale=0.02)
    m = wl.robot
    c = W.CONFIGS[cfg]
    new = W.make_primitives(m, 17, c["steps"][0], c["steps"][1], seed=77)
    both = W.Primitives(np.concatenate([new.length, wl.prims.length]).astype(np.int32),
                        np.concatenate([new.states, wl.prims.states]),
                        np.concatenate([new.actions, wl.prims.actions]))
    prec = wl.precision
    with G.Context(m) as a, G.Context(m) as b:
        a.upload_primitives(wl.prims)
        a.prepend_primitives(new)
        b.upload_primitives(both)
        for ctx in (a, b):
            ctx.upload_env(wl.env)
        ra = a.expand(wl.nodes, wl.radius, precision=prec)
        rb = b.expand(wl.nodes, wl.radius, precision=prec)
    assert ra["n_pairs"] == rb["n_pairs"] > 0
    for k in ("node", "prim", "verdict", "first_invalid", "end_state", "flags"):
        assert np.array_equal(ra[k], rb[k]), k
    assert np.array_equal(ra["min_gap"], rb["min_gap"], equal_nan=True)
