"""The tdb-A* restatement (tests/tdb_ref.py) on its own, on the CPU: the
reverse transform of the rollout robots is the same actions rolled out from
the shifted start, and ends at the node's position and velocity."""
import numpy as np
import pytest

import oracle_bind as ob
import tdb_ref
from dynoplan_gb300 import workloads as W


@pytest.mark.parametrize("cfg", [3, 5])
def test_reverse_rollout_robots_are_rollouts_of_the_same_actions(cfg):
    wl = W.make_workload(cfg, scale=0.002, seed=90 + cfg)
    m = wl.robot
    pos, vel = tdb_ref._POS[m.kind], tdb_ref._VEL[m.kind]
    rng = np.random.default_rng(cfg)
    for p in rng.integers(0, wl.prims.P, 6):
        x = wl.nodes[int(rng.integers(0, len(wl.nodes)))]
        st = tdb_ref._states(m, wl.prims, int(p), x, True)
        _, us = wl.prims.motion(int(p))
        again = ob.rollout(m, st[0], us)   # the oracle's FP64 rollout from the shifted start
        np.testing.assert_allclose(again, st, rtol=0, atol=1e-9)
        np.testing.assert_allclose(st[-1][pos], x[pos], rtol=0, atol=1e-12)
        np.testing.assert_allclose(st[-1][vel], x[vel], rtol=0, atol=1e-12)


def test_reverse_translation_robots_end_at_the_node():
    wl = W.make_workload(2, scale=0.002, seed=93)
    for p in range(5):
        x = wl.nodes[p]
        st = tdb_ref._states(wl.robot, wl.prims, p, x, True)
        xs, _ = wl.prims.motion(p)
        np.testing.assert_allclose(st[-1][:2], x[:2], rtol=0, atol=1e-12)
        np.testing.assert_allclose(st[:, 2:], xs[:, 2:], rtol=0, atol=0)   # headings unchanged
