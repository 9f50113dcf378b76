"""The C ABI library loads and exports what include/dpg.h declares (CPU only:
no compute call needs a GPU here)."""
import ctypes as C
import os
import re
import subprocess

import pytest

from dynoplan_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(dpg_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported(dpg_lib):
    from dynoplan_gb300 import _lib
    names = declared_functions()
    assert {"dpg_create", "dpg_expand", "dpg_upload_primitives", "dpg_upload_env"} <= names
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = names - exported
    assert not missing, missing
    # and the Python binding declares a signature for each
    assert names == {s[0] for s in _lib.SIGNATURES}


def test_robot_defaults_match_models(dpg_lib):
    from dynoplan_gb300 import _lib
    for kind in (W.UNICYCLE1, W.CAR1, W.QUAD3D, W.QUAD2D):
        d = _lib.RobotDesc()
        assert dpg_lib.dpg_robot_default(kind, C.byref(d)) == 0
        m = W.robot_model(kind)
        assert (d.nx, d.nu, d.n_parts) == (m.nx, m.nu, m.n_parts)
        assert d.dt == m.dt
        assert list(d.w) == list(m.w)
        assert (d.box[0], d.box[1]) == m.box
        assert (d.hitch, d.wheelbase, d.radius, d.mass, d.arm, d.t2t, d.ang_gain) == (
            m.hitch, m.wheelbase, m.radius, m.mass, m.arm, m.t2t, m.ang_gain)
    d = _lib.RobotDesc()
    assert dpg_lib.dpg_robot_default(17, C.byref(d)) == _lib.DPG_ERR_ARG


def test_error_strings_and_version(dpg_lib):
    assert dpg_lib.dpg_abi_version() == 1
    for code in range(0, -9, -1):
        assert dpg_lib.dpg_errstr(code)
    assert dpg_lib.dpg_errstr(-99) == b"unknown error"


def test_create_rejects_bad_descriptions(dpg_lib):
    from dynoplan_gb300 import _lib
    d = _lib.RobotDesc()
    dpg_lib.dpg_robot_default(W.CAR1, C.byref(d))
    d.nx = 5
    h = C.c_void_p()
    assert dpg_lib.dpg_create(C.byref(h), 0, C.byref(d)) == _lib.DPG_ERR_ARG
    assert not h.value
    # a null description / null out pointer
    assert dpg_lib.dpg_create(None, 0, C.byref(d)) == _lib.DPG_ERR_ARG
    dpg_lib.dpg_destroy(None)   # no-op


def test_no_gpu_is_an_error_not_a_fallback(dpg_lib):
    """Without a device the library refuses: there is no CPU path."""
    from dynoplan_gb300 import _lib
    d = _lib.RobotDesc()
    dpg_lib.dpg_robot_default(W.UNICYCLE1, C.byref(d))
    h = C.c_void_p()
    rc = dpg_lib.dpg_create(C.byref(h), 0, C.byref(d))
    if rc == 0:
        dpg_lib.dpg_destroy(h)
        pytest.skip("a CUDA device is present")
    assert rc == _lib.DPG_ERR_NODEVICE
