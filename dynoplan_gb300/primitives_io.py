"""Motion-primitive files (include/dpg_prim_io.h) from Python: the
reference's msgpack document {"data": [{"states", "actions"}, ...]} read
into and written from the flattened Primitives layout, plus the loader's
noise / quaternion post-processing (load_motion_primitives_new,
src/ompl/robots.cpp:3061-3174).  Host code of the library; no device."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import check
from .workloads import Primitives


def _path(p) -> bytes:
    return os.fsencode(os.fspath(p))


def read_msgpack(path, max_motions: int = 0) -> Primitives:
    """The first `max_motions` motions of a file (0: all), FP64."""
    lib = _lib.load()
    P, nx, nu = C.c_int32(), C.c_int32(), C.c_int32()
    S, A = C.c_int64(), C.c_int64()
    check(lib.dpg_primitives_file_info(_path(path), max_motions, C.byref(P), C.byref(S), C.byref(A), C.byref(nx),
                                       C.byref(nu)))
    length = np.empty(P.value, np.int32)
    states = np.empty((S.value, nx.value), np.float64)
    actions = np.empty((A.value, max(nu.value, 0)), np.float64)
    check(lib.dpg_primitives_file_read(_path(path), max_motions, length.ctypes.data, states.ctypes.data,
                                       actions.ctypes.data if actions.size else None))
    return Primitives(length, states, actions)


def write_msgpack(path, prims: Primitives, compact: bool = True):
    """Write the motions, losslessly: with `compact`, numbers that are exact
    float32 values as float32 and the rest as float64 (the bundled files'
    encoding); otherwise all float64."""
    lib = _lib.load()
    length = np.ascontiguousarray(prims.length, dtype=np.int32)
    states = np.ascontiguousarray(prims.states, dtype=np.float64)
    actions = np.ascontiguousarray(prims.actions, dtype=np.float64)
    nx = states.shape[1]
    nu = actions.shape[1] if actions.ndim == 2 else 0
    check(lib.dpg_primitives_file_write(_path(path), len(length), length.ctypes.data, states.ctypes.data,
                                        actions.ctypes.data if actions.size else None, nx, nu, 1 if compact else 0))


def prepare(prims: Primitives, kind: int, noise: float = 1e-7, seed: int = 0) -> Primitives:
    """A copy with the loader's noise on every motion's first and last state
    (uniform in [-noise, noise], seeded) and, for the quadrotor, normalised
    quaternions."""
    out = Primitives(np.array(prims.length, np.int32), np.array(prims.states, np.float64),
                     np.array(prims.actions, np.float64))
    check(_lib.load().dpg_primitives_prepare(kind, out.P, out.length.ctypes.data, out.states.ctypes.data,
                                             out.states.shape[1], noise, seed))
    return out
