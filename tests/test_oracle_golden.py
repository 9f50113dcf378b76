"""The oracle pinned against the reference's own data (CPU only).

Fixtures come from tests/golden/make_golden.py:
  unicycle1_bundled_primitives.json  reference data/motion_primitives/unicycle1_v0
  jump_annotations.json              benchmark_initguess/unicycle{1,2}_v0 "jump" comments
  recorded_trajectories.json         benchmark_initguess quad2d / quadrotor / unicycle1 runs
  oracle_cfg*.npz                    the oracle's own outputs on seeded workloads
"""
import json
import math
import os

import numpy as np
import pytest

import oracle_bind as ob
from dynoplan_gb300 import workloads as W

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def test_unicycle1_bundled_primitives_reproduce():
    """Every step of the 100 bundled primitives is the oracle's unicycle1 step."""
    m = W.robot_model(W.UNICYCLE1)
    data = _load("unicycle1_bundled_primitives.json")["data"]
    assert len(data) == 100
    worst = 0.0
    for t in data:
        xs, us = np.array(t["states"]), np.array(t["actions"])
        assert len(xs) == len(us) + 1
        for k in range(len(us)):
            worst = max(worst, float(np.abs(ob.step(m, xs[k], us[k]) - xs[k + 1]).max()))
        # the rollout helper agrees with step-by-step
        np.testing.assert_allclose(ob.rollout(m, xs[0], us), xs, atol=1e-12)
    assert worst < 1e-12


def test_jump_annotations_pin_unicycle1_metric():
    """'jump from A to B delta D min time T' == distance(A, B), lower_bound_time(A, B)."""
    m = W.robot_model(W.UNICYCLE1)
    jumps = _load("jump_annotations.json")["unicycle1_v0"]["jumps"]
    assert len(jumps) >= 10
    for j in jumps:
        d = ob.distance(m, np.array(j["frm"]), np.array(j["to"]))
        t = ob.lower_bound_time(m, np.array(j["frm"]), np.array(j["to"]))
        # printed with 6 significant digits, from endpoints printed with 6
        # digits (each coordinate is off by up to 5e-6)
        assert d == pytest.approx(j["delta"], rel=2e-5, abs=1e-5)
        assert t == pytest.approx(j["min_time"], rel=2e-5, abs=4e-5)


def test_jump_annotations_pin_sum_of_blocks_rule():
    """unicycle2's 4-block annotations follow the same rule the oracle uses for
    every robot: sum of weighted block distances, SO2 blocks wrapped
    (weights = the __SpaceUni2 ratios 1, 1/2, 1/4, 1/4)."""
    jumps = _load("jump_annotations.json")["unicycle2_v0"]["jumps"]
    assert len(jumps) >= 10

    def so2(a, b):
        d = abs(a - b) % (2 * math.pi)
        return min(d, 2 * math.pi - d)

    for j in jumps:
        a, b = j["frm"], j["to"]
        d = (math.hypot(a[0] - b[0], a[1] - b[1]) + 0.5 * so2(a[2], b[2]) + 0.25 * abs(a[3] - b[3])
             + 0.25 * abs(a[4] - b[4]))
        assert d == pytest.approx(j["delta"], rel=5e-5, abs=1e-5)


@pytest.mark.parametrize("robot,kind,tol", [("quad2d_v0", W.QUAD2D, 2e-5), ("quadrotor_v0", W.QUAD3D, 2e-5),
                                            ("unicycle1_v0", W.UNICYCLE1, 2e-5)])
def test_recorded_trajectories_pin_dynamics(robot, kind, tol):
    """The reference's db-A* outputs are concatenations of transformed
    primitives: inside a primitive every step is the model's step.  With 6
    printed digits a step reproduces to ~1e-5; the few mismatches are the
    primitive boundaries (the discontinuities the search allows)."""
    m = W.robot_model(kind)
    runs = [t for t in _load("recorded_trajectories.json") if t["robot"] == robot]
    assert runs
    for t in runs:
        xs, us = np.array(t["states"]), np.array(t["actions"])
        res = np.array([np.abs(ob.step(m, xs[k], us[k]) - xs[k + 1]).max() for k in range(len(us))])
        scale = 1.0 + np.abs(xs[1:]).max(1)
        ok = res <= tol * scale * 10
        assert ok.mean() > 0.93, (t["source"], ok.mean())
        # the boundaries are a few percent of the steps, as a primitive spans many steps
        assert (~ok).sum() <= 0.07 * len(res)


def test_recorded_unicycle1_jumps_within_delta():
    """Discontinuity bound: every primitive boundary of a solved run jumps by
    at most delta in the robot metric (dbastar.cpp:1021-1031)."""
    m = W.robot_model(W.UNICYCLE1)
    (t,) = [t for t in _load("recorded_trajectories.json") if t["robot"] == "unicycle1_v0"]
    xs, us = np.array(t["states"]), np.array(t["actions"])
    jumps = [ob.distance(m, ob.step(m, xs[k], us[k]), xs[k + 1]) for k in range(len(us))]
    assert max(jumps) <= t["delta"] + 1e-5


@pytest.mark.parametrize("cfg", [1, 2, 3, 5])
def test_oracle_reproduces_committed_outputs(cfg):
    z = np.load(os.path.join(GOLD, f"oracle_cfg{cfg}.npz"))
    m = W.robot_model(int(z["kind"]))
    prims = W.Primitives(z["length"], z["states"], z["actions"])
    env = W.Env(z["env_lo"], z["env_hi"], z["obs_lo"], z["obs_hi"])
    res = ob.expand(m, prims, env, z["nodes"], float(z["radius"]))
    for k in ("node", "prim", "verdict", "first_invalid"):
        np.testing.assert_array_equal(res[k], z[k])
    np.testing.assert_allclose(res["end_state"], z["end_state"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(res["min_gap"], z["min_gap"], rtol=0, atol=1e-9)


@pytest.mark.parametrize("cfg,scale", [(1, 0.05), (2, 0.01), (3, 0.004), (5, 0.005)])
def test_fast_baseline_equals_plain_oracle(cfg, scale):
    """The timed CPU baseline (sorted-angle radius query, grid broadphase,
    OpenMP) gives exactly the plain oracle's pairs, verdicts and states."""
    wl = W.make_workload(cfg, scale=scale)
    a = ob.expand(wl.robot, wl.prims, wl.env, wl.nodes, wl.radius)
    b = ob.expand(wl.robot, wl.prims, wl.env, wl.nodes, wl.radius, fast=True, threads=4)
    assert a["n_pairs"] == b["n_pairs"] > 0
    for k in ("node", "prim", "verdict", "first_invalid", "end_state"):
        np.testing.assert_array_equal(a[k], b[k])


def test_oracle_contact_semantics():
    """Touching counts as contact (gap <= 0); a hair of clearance does not."""
    m = W.robot_model(W.UNICYCLE1)
    env = W.Env(np.zeros(2), np.array([10.0, 10.0]), np.array([[5.0, 4.0]]), np.array([[6.0, 6.0]]))
    e, keep = ob.env_struct(env)
    import ctypes as C
    r = ob.robot(m)
    # box 0.5 x 0.25 heading +x, right face at x + 0.25
    for x, expect in ((4.75, 0.0), (4.75 - 1e-9, 1e-9), (4.8, -0.05)):
        s = np.array([x, 5.0, 0.0])
        g = ob.lib().orc_state_gap(C.byref(r), C.byref(e), s.ctypes.data, 0)
        assert g == pytest.approx(expect, abs=1e-12)


def test_oracle_empty_and_degenerate_inputs():
    m = W.robot_model(W.CAR1)
    prims = W.make_primitives(m, 5, 0, 3, seed=3)   # includes single-state motions
    assert prims.length.min() >= 1
    env = W.Env(np.zeros(2), np.array([4.0, 4.0]), np.zeros((0, 2)), np.zeros((0, 2)))
    nodes = np.zeros((0, 4))
    assert ob.expand(m, prims, env, nodes, 0.15)["n_pairs"] == 0
    nodes = W.make_nodes(m, env, 20, seed=4)
    res = ob.expand(m, prims, env, nodes, 10.0)   # every pair in the ball
    assert res["n_pairs"] == 20 * 5
    assert set(np.unique(res["verdict"])) <= {0, 2}  # no obstacles: never a collision
