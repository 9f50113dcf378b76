"""The search restatement's rule for a successor's g (its node's g when the
batch was popped) against the reference's (the node's current g): one node
per iteration gives identical searches (CPU, over the oracle's expand)."""
import pytest

import search_ref
from dynoplan_gb300 import workloads as W


@pytest.mark.parametrize("kind,seed", [(W.UNICYCLE1, 11), (W.CAR1, 12)])
def test_g_at_pop_equals_current_g_with_one_node_per_iteration(kind, seed):
    m = W.robot_model(kind)
    prims = W.make_primitives(m, 120, 5, 20, seed=seed)
    env = W.make_env((5.0, 5.0), 12, 0.2, 0.8, seed=seed + 1)
    se = W.make_nodes(m, env, 2, seed=seed + 2, vel_sigma=0.0)
    runs = [search_ref.search(m, prims, env, se[0], se[1], 0.5, batch=1, max_expands=300, g_at_pop=rule)
            for rule in (True, False)]
    a, b = runs
    assert a["expands"] > 100  # searches that explore well beyond the start
    for k in ("status", "expands", "nodes", "solved"):
        assert a[k] == b[k], k
    if a["solved"]:
        assert a["motions"] == b["motions"]
        assert a["cost"] == b["cost"]
