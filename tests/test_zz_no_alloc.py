"""dpg_expand_noalloc, the allocation-free expand (include/dpg.h).

Callers that cannot allocate device memory while they expand -- real-time
planning loops that must not block on the device allocator, host programs
that hand all device memory to their own pool up front -- use this entry
point; its scratch is a fixed 64 MiB device array inside the library instead
of buffers it grows with cudaMalloc.  This file checks,
through the C ABI, that two calls in a row give the results of the regular
entry point (same tolerance as the other parity tests), that device memory
does not change across the calls, and that a batch too large for the
scratch is refused.  It is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from dynoplan_gb300 import workloads as W
from parity_util import compare

pytestmark = pytest.mark.gpu


def _device_out(torch, cap, nx, precision):
    dev = "cuda:0"
    return {
        "node": torch.empty(cap, dtype=torch.int32, device=dev),
        "prim": torch.empty(cap, dtype=torch.int32, device=dev),
        "verdict": torch.empty(cap, dtype=torch.uint8, device=dev),
        "first_invalid": torch.empty(cap, dtype=torch.int16, device=dev),
        "end_state": torch.empty((cap, nx), dtype=torch.float64 if precision else torch.float32, device=dev),
        "min_gap": torch.empty(cap, dtype=torch.float32, device=dev),
        "flags": torch.empty(cap, dtype=torch.uint8, device=dev),
    }


def _call(lib, ctx, x_d, N, outs, cap, radius, precision):
    from dynoplan_gb300._lib import ExpandOpts, ExpandOut
    opts = ExpandOpts(radius=radius, precision=precision, x_on_device=1, out_on_device=1, mode=0,
                      contact_band=1e-4, ball_band=1e-5)
    out = ExpandOut(capacity=cap)
    for k, t in outs.items():
        setattr(out, k, C.c_void_p(t.data_ptr()))
    rc = lib.dpg_expand_noalloc(ctx.h, C.byref(opts), N, C.c_void_p(x_d.data_ptr()), C.byref(out))
    return rc, out


@pytest.mark.parametrize("cfg,scale,precision", [(2, 0.05, 0), (3, 0.01, 0), (1, 0.1, 1)])
def test_noalloc_matches_expand_twice(dpg_lib, cfg, scale, precision):
    torch = pytest.importorskip("torch")
    from dynoplan_gb300 import gpu as G
    wl = W.make_workload(cfg, scale=scale, seed=900 + cfg)
    N, nx = wl.nodes.shape
    with G.Context(wl.robot) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        ref = ctx.expand(wl.nodes, wl.radius, precision=precision)   # the regular entry point
        assert ref["n_pairs"] > 0
        cap = ref["n_pairs"] + 64
        x_d = torch.from_numpy(np.ascontiguousarray(wl.nodes)).to("cuda:0")
        outs = _device_out(torch, cap, nx, precision)
        # run the torch kernels this test uses once, so that their lazy module
        # loading does not fall inside the measured window
        for t in outs.values():
            t.fill_(0x7f if t.dtype in (torch.uint8,) else 123)
            t[:1].cpu()
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        for call in range(2):
            for t in outs.values():          # stale values must not survive
                t.fill_(0x7f if t.dtype in (torch.uint8,) else 123)
            rc, out = _call(dpg_lib, ctx, x_d, N, outs, cap, wl.radius, precision)
            assert rc == 0, dpg_lib.dpg_last_error(ctx.h)
            assert out.n_pairs == ref["n_pairs"]
            n = out.n_pairs
            got = {k: t[:n].cpu().numpy() for k, t in outs.items()}
            got["node"] = got["node"].view(np.uint32)
            got["prim"] = got["prim"].view(np.uint32)
            got["n_pairs"] = n
            compare(wl.robot.kind, got, ref, precision)
            # same pairs, possibly in another order within a primitive (large
            # batches of the regular entry point run in spatial order)
            kg = np.lexsort((got["node"], got["prim"]))
            kr = np.lexsort((ref["node"], ref["prim"]))
            np.testing.assert_array_equal(got["flags"][kg], ref["flags"][kr])
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free_before   # nothing was allocated


def _scratch_need(N, P, keyd, offd):
    """bytes of scratch a call needs: the formula of include/dpg.h"""
    a = lambda v: (v + 255) // 256 * 256
    W = (N + 31) // 32
    Wpad = (W + 31) // 32 * 32
    B = (N + 255) // 256
    return (a(4 * keyd * N) + a(4 * offd * N) + a(4 * Wpad * P) + a(4 * B * P) + a(4 * P) + a(8 * P)
            + 2 * a(8 * (P + 1)) + a(112))


def test_noalloc_refuses_batches_beyond_its_scratch(dpg_lib):
    torch = pytest.importorskip("torch")
    import re

    from dynoplan_gb300 import _lib
    from dynoplan_gb300 import gpu as G
    wl = W.make_workload(2, scale=0.01, seed=77)
    N, P = 100_000, 5000
    assert _scratch_need(92_000, P, 2, 2) <= 64 << 20 < _scratch_need(N, P, 2, 2)
    with G.Context(wl.robot) as ctx:
        ctx.upload_primitives(W.make_primitives(wl.robot, P, 5, 10, seed=3))
        ctx.upload_env(wl.env)
        # x holds all N rows, so that a call that went ahead would still read
        # inside it; the refusal comes on the host before any launch
        x_d = torch.from_numpy(W.make_nodes(wl.robot, wl.env, N, seed=5)).to("cuda:0")
        outs = _device_out(torch, 16, wl.robot.nx, 0)
        rc, _ = _call(dpg_lib, ctx, x_d, N, outs, 16, wl.radius, 0)
        assert rc == _lib.DPG_ERR_ARG
        msg = dpg_lib.dpg_last_error(ctx.h).decode()
        need = int(re.search(r"needs (\d+) bytes", msg).group(1))
        assert need == _scratch_need(N, P, 2, 2), msg   # the header's formula
