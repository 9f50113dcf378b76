"""ctypes binding of the C ABI declared in include/dpg.h.

The shared library is built in-tree by ``dynoplan_gb300.build.build_library``
(nvcc, sm_103a).  There is no fallback: if the library cannot be loaded every
entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libdpg.so")

# error codes (dpg.h)
DPG_OK = 0
DPG_ERR_ARG = -1
DPG_ERR_OOM = -2
DPG_ERR_CUDA = -3
DPG_ERR_TIMEOUT = -4
DPG_ERR_ABORTED = -5
DPG_ERR_CAPACITY = -6
DPG_ERR_STATE = -7
DPG_ERR_NODEVICE = -8
DPG_UNCHECKED = 255
DPG_CHECK_LOCKSTEP = 0
DPG_CHECK_SLOTS = 1
DPG_HOST_OUT_PIPELINED = 0
DPG_HOST_OUT_DIRECT = 1
DPG_HOST_OUT_PROGRESS = 2
DPG_FLAG_ACCEPTED = 2

DPG_FP32 = 0
DPG_FP64 = 1
DPG_FLAG_CONTACT_RECHECK = 1


class RobotDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("nx", C.c_int32), ("nu", C.c_int32), ("n_parts", C.c_int32),
        ("dt", C.c_double), ("w", C.c_double * 4), ("box", C.c_double * 2),
        ("hitch", C.c_double), ("wheelbase", C.c_double), ("radius", C.c_double),
        ("mass", C.c_double), ("arm", C.c_double), ("t2t", C.c_double),
        ("inertia", C.c_double * 3), ("ang_gain", C.c_double), ("g", C.c_double),
    ]


class ExpandOpts(C.Structure):
    _fields_ = [
        ("radius", C.c_double), ("precision", C.c_int32), ("x_on_device", C.c_int32),
        ("out_on_device", C.c_int32), ("mode", C.c_int32),
        ("contact_band", C.c_double), ("ball_band", C.c_double),
    ]


class Tuning(C.Structure):
    _fields_ = [("check_variant", C.c_int32), ("check_blocks_per_sm", C.c_int32),
                ("grid_min_nodes", C.c_int32), ("pipe_launches", C.c_int32), ("host_output", C.c_int32)]


class TuneReport(C.Structure):
    _fields_ = [("chosen", Tuning), ("initial", Tuning), ("ms_chosen", C.c_double), ("ms_initial", C.c_double),
                ("seconds", C.c_double), ("candidates", C.c_int32), ("from_cache", C.c_int32),
                ("key", C.c_char * 160)]


class LazyStats(C.Structure):
    _fields_ = [("n_checked", C.c_int64), ("n_valid", C.c_int64), ("n_accepted", C.c_int64),
                ("rounds", C.c_int32), ("max_candidates", C.c_int32)]


class ExpandOut(C.Structure):
    _fields_ = [
        ("capacity", C.c_int64), ("n_pairs", C.c_int64),
        ("node", C.c_void_p), ("prim", C.c_void_p), ("verdict", C.c_void_p),
        ("first_invalid", C.c_void_p), ("end_state", C.c_void_p), ("min_gap", C.c_void_p),
        ("flags", C.c_void_p),
        ("n_scanned", C.c_int64), ("n_contact_recheck", C.c_int64), ("n_ball_recheck", C.c_int64),
    ]


# (name, restype, argtypes) for every function dpg.h declares
SIGNATURES = [
    ("dpg_abi_version", C.c_int, []),
    ("dpg_errstr", C.c_char_p, [C.c_int]),
    ("dpg_robot_default", C.c_int, [C.c_int32, C.POINTER(RobotDesc)]),
    ("dpg_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(RobotDesc)]),
    ("dpg_destroy", None, [C.c_void_p]),
    ("dpg_last_error", C.c_char_p, [C.c_void_p]),
    ("dpg_upload_primitives", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("dpg_prepend_primitives", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("dpg_upload_env", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                                 C.c_void_p, C.c_void_p]),
    ("dpg_expand", C.c_int, [C.c_void_p, C.POINTER(ExpandOpts), C.c_int64, C.c_void_p,
                             C.POINTER(ExpandOut)]),
    ("dpg_expand_noalloc", C.c_int, [C.c_void_p, C.POINTER(ExpandOpts), C.c_int64, C.c_void_p,
                                     C.POINTER(ExpandOut)]),
    ("dpg_check_pairs", C.c_int, [C.c_void_p, C.POINTER(ExpandOpts), C.c_int64, C.c_void_p, C.c_int64,
                                  C.c_void_p, C.c_void_p, C.POINTER(ExpandOut)]),
    ("dpg_lazy_check", C.c_int, [C.c_void_p, C.POINTER(ExpandOpts), C.c_int64, C.c_void_p, C.c_int64,
                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.POINTER(ExpandOut),
                                 C.POINTER(LazyStats)]),
    ("dpg_get_tuning", C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    ("dpg_set_tuning", C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    ("dpg_mlp_wait_selftest", C.c_int, [C.c_int, C.c_uint32]),
    ("dpg_sync", C.c_int, [C.c_void_p]),
    # include/dpg_tune.h
    ("dpg_autotune", C.c_int, [C.c_void_p, C.POINTER(ExpandOpts), C.c_int64, C.c_void_p, C.c_int32, C.c_char_p,
                               C.POINTER(TuneReport)]),
    ("dpg_tune_key", C.c_int, [C.c_void_p, C.c_int64, C.c_char_p, C.c_int32]),
    ("dpg_set_abort", C.c_int, [C.c_void_p, C.c_int32]),
    ("dpg_host_alloc", C.c_void_p, [C.c_size_t]),
    ("dpg_host_free", None, [C.c_void_p]),
    ("dpg_last_timings", C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_int32]),
    # include/dpg_mlp.h
    ("dpg_gemm_bf16", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                C.c_int]),
    ("dpg_mlp_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int64, C.c_uint64]),
    ("dpg_mlp_destroy", None, [C.c_void_p]),
    ("dpg_mlp_param_size", C.c_int64, [C.c_void_p, C.c_int]),
    ("dpg_mlp_get", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    ("dpg_mlp_set", C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    ("dpg_mlp_node_features", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    ("dpg_mlp_forward", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    ("dpg_mlp_train_step", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                     C.c_float, C.c_float, C.POINTER(C.c_float)]),
    ("dpg_mlp_set_fused", C.c_int, [C.c_void_p, C.c_int]),
    ("dpg_mlp_last_timing", C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    # include/dpg_search.h
    ("dpg_search", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                             C.c_void_p, C.c_void_p, C.c_int32]),
    # include/dpg_prim_io.h
    ("dpg_primitives_file_info", C.c_int, [C.c_char_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                                           C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    ("dpg_primitives_file_read", C.c_int, [C.c_char_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("dpg_primitives_file_write", C.c_int, [C.c_char_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                            C.c_int32, C.c_int32]),
    ("dpg_primitives_prepare", C.c_int, [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_double,
                                         C.c_uint64]),
    # include/dpg_roadmap.h
    ("dpg_roadmap_build", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_double, C.c_double,
                                    C.POINTER(C.c_void_p)]),
    ("dpg_roadmap_destroy", None, [C.c_void_p]),
    ("dpg_roadmap_edges", C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.c_void_p, C.c_void_p, C.c_int64]),
    ("dpg_roadmap_distances", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("dpg_roadmap_heuristic", C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]),
    ("dpg_states_valid", C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    # include/dpg_tdb.h
    ("dpg_tdb_check_pairs", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    # include/dpg_bench.h
    ("dpg_bench_fp32_peak", C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_double)]),
    ("dpg_bench_flush_l2", C.c_int, [C.c_int, C.c_size_t]),
    ("dpg_bench_per_node_expand", C.c_int, [C.c_void_p, C.POINTER(ExpandOpts), C.c_int64, C.c_int32, C.c_void_p,
                                            C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
]

_lib = None


class DpgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"dpg error {code}: {msg}")
        self.code = code


def load(path: str = LIB_PATH):
    """Load libdpg.so (once).  Raises if it is missing: no CPU fallback exists."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with dynoplan_gb300.build.build_library() "
            "(the expansion has no CPU fallback)")
    lib = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, ctx=None):
    if rc != DPG_OK:
        lib = load()
        msg = lib.dpg_errstr(rc).decode()
        if ctx:
            detail = lib.dpg_last_error(ctx)
            if detail:
                msg += ": " + detail.decode()
        raise DpgError(rc, msg)
    return rc
