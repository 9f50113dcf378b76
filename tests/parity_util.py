"""Comparison of GPU expansion results against the oracle.

Bars (the tolerances every parity test states):
  pairs, verdicts, first_invalid   identical
  end states                      DPG_FP64 and DPG_FP64_STRICT: 1e-9
                                  absolute; DPG_FP32: 1e-5 relative
                                  (|d| <= 1e-5 * max(1, |x|)); wrapped angles
                                  compared modulo 2 pi
  min_gap (FP32 output)           DPG_FP64_STRICT (FP64 tests): 1e-5;
                                  DPG_FP32 and DPG_FP64 (FP32 tests): 2e-4
                                  absolute
"""
import math

import numpy as np

from dynoplan_gb300 import workloads as W

ANGLE_COMPS = {W.UNICYCLE1: [2], W.CAR1: [2, 3], W.QUAD2D: [2], W.QUAD3D: []}
GAP_CAP = 0.05  # min_gap is reported up to this clearance, +inf above


def sort_by_pair(res):
    key = res["node"].astype(np.int64) * (1 << 32) + res["prim"].astype(np.int64)
    order = np.argsort(key, kind="stable")
    return {k: (v[order] if isinstance(v, np.ndarray) and v.shape[:1] == order.shape else v)
            for k, v in res.items()}


def compare(kind, gpu, ora, precision, min_gap=True):
    """Assert parity; returns a dict of residuals for reporting."""
    g = sort_by_pair(gpu)
    o = sort_by_pair(ora)
    assert g["n_pairs"] == o["n_pairs"], (g["n_pairs"], o["n_pairs"])
    np.testing.assert_array_equal(g["node"], o["node"])
    np.testing.assert_array_equal(g["prim"], o["prim"])
    np.testing.assert_array_equal(g["verdict"], o["verdict"])
    np.testing.assert_array_equal(g["first_invalid"], o["first_invalid"])
    ge = g["end_state"].astype(np.float64)
    oe = o["end_state"]
    d = ge - oe
    for c in ANGLE_COMPS[kind]:
        d[:, c] = (d[:, c] + math.pi) % (2 * math.pi) - math.pi
    if precision != 0:   # DPG_FP64, DPG_FP64_STRICT: FP64 end states
        tol = np.full_like(oe, 1e-9)
    else:
        tol = 1e-5 * np.maximum(1.0, np.abs(oe))
    bad = np.abs(d) > tol
    assert not bad.any(), f"end state mismatch at {np.argwhere(bad)[:5].tolist()}: max {np.abs(d).max()}"
    out = {"end_state_max_abs": float(np.abs(d).max()) if len(d) else 0.0}
    if min_gap and len(d):
        tol = 1e-5 if precision == 2 else 2e-4   # FP64 tests only in DPG_FP64_STRICT
        gg, og = g["min_gap"].astype(np.float64), o["min_gap"]
        # NaN (out of bounds) on the same rows
        np.testing.assert_array_equal(np.isnan(gg), np.isnan(og))
        # +inf = clearance above the 5 cm cap; a value within tol of the cap
        # may fall on either side
        near_cap = lambda v: np.isinf(v) | (v >= GAP_CAP - tol)
        both = np.isfinite(gg) & np.isfinite(og)
        close = np.zeros(len(gg), bool)
        close[both] = np.abs(gg[both] - og[both]) <= tol      # differences of finite rows only
        ok = np.where(np.isnan(og), True, np.where(both, close, near_cap(gg) & near_cap(og)))
        assert ok.all(), f"min_gap mismatch at {np.argwhere(~ok)[:5].ravel().tolist()}"
        out["min_gap_max_abs"] = float(np.abs(gg[both] - og[both]).max(initial=0))
    return out
