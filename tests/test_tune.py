"""dpg_autotune (include/dpg_tune.h): the launch choices it times give
identical results, the fastest is applied, and a cached key is reused."""
import os

import numpy as np
import pytest

from dynoplan_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cfg,scale", [(2, 0.05), (3, 0.02), (1, 0.5)])
def test_autotune_applies_fastest_and_caches(tmp_path, cfg, scale):
    import torch

    from dynoplan_gb300 import gpu as G
    wl = W.make_workload(cfg, scale=scale, seed=600 + cfg)
    cache = str(tmp_path / "tuning.txt")
    with G.Context(wl.robot) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        before = ctx.expand(wl.nodes, wl.radius, precision=wl.precision)
        x_d = torch.from_numpy(wl.nodes).cuda()
        torch.cuda.synchronize()
        rep = ctx.autotune(x_d.data_ptr(), len(wl.nodes), wl.radius, precision=wl.precision, cache_path=cache)
        assert not rep["from_cache"] and rep["candidates"] >= 6
        assert ctx.tuning() == rep["chosen"]
        assert rep["ms_chosen"] <= rep["ms_initial"] * 1.0 + 1e-9
        after = ctx.expand(wl.nodes, wl.radius, precision=wl.precision)
        for k in ("node", "prim", "verdict", "first_invalid", "end_state", "min_gap", "flags"):
            np.testing.assert_array_equal(before[k], after[k])
        assert os.path.exists(cache) and rep["key"] in open(cache).read()
    with G.Context(wl.robot) as ctx:      # a new context takes the cached choice
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        rep2 = ctx.autotune(x_d.data_ptr(), len(wl.nodes), wl.radius, precision=wl.precision, cache_path=cache)
        assert rep2["from_cache"] and rep2["chosen"] == rep["chosen"] and rep2["key"] == rep["key"]
        assert ctx.tuning() == rep["chosen"]


def test_tune_key_describes_the_workload():
    import ctypes as C

    from dynoplan_gb300 import _lib
    from dynoplan_gb300 import gpu as G
    wl = W.make_workload(2, scale=0.01, seed=3)
    with G.Context(wl.robot) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        buf = C.create_string_buffer(160)
        _lib.check(ctx.lib.dpg_tune_key(ctx.h, 100000, buf, 160), ctx.h)
        key = buf.value.decode()
    assert key.startswith(f"k1_P{wl.prims.P}_Lmax{int(wl.prims.length.max())}_h")
    assert key.endswith(f"_O{len(wl.env.obs_lo)}_N2^17")
