"""Invalid scenes are refused at creation with a status and a message, before any device work
(host-side fault injection: NaN and infinite data, degenerate normals, zero total area, bad enum
values). The reference accepts all of these silently (scene.cuh:264-326) and its walks then
average NaN or zero weights; here wob_scene_create returns WOB_ERR_INVALID_ARGUMENT. Elements of
zero area inside an otherwise valid scene are accepted: they carry no sampling weight and no line
meets them (tests/test_gpu_failure_bounds.py checks that their walks stay finite)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from wobtoolbox_gb300 import workloads as W


def _create(engine, verts, normals, bvals, types, alphas=None):
    lib = engine.load()
    h = C.c_void_p()
    f = lambda a: np.ascontiguousarray(a, np.float32)
    v, n, b = f(verts), f(normals), f(bvals)
    t = np.ascontiguousarray(types, np.int32)
    a = None if alphas is None else f(alphas)
    st = lib.wob_scene_create(v.shape[1], len(v), v.ctypes.data, n.ctypes.data, b.ctypes.data,
                              None if a is None else a.ctypes.data, t.ctypes.data, C.byref(h))
    msg = lib.wob_last_error().decode()
    return st, msg, h


def _star():
    verts, normals = W.star_polygon(64, 3, 0.25)
    return verts, normals, np.ones((64, 2), np.float32), np.zeros(64, np.int32)


@pytest.mark.parametrize("fault,expect", [
    ("nan_data", "boundary values must be finite"),
    ("inf_vertex", "vertices must be finite"),
    ("nan_normal", "normals must be finite"),
    ("zero_normal", "normals must be unit vectors"),
    ("scaled_normal", "normals must be unit vectors"),
    ("nan_alpha", "robin alphas must be finite"),
    ("bad_type", "boundary_types must be"),
])
def test_invalid_scene_is_refused(engine, fault, expect):
    v, n, b, t = _star()
    a = np.ones_like(b)
    if fault == "nan_data":
        b[5, 1] = np.nan
    elif fault == "inf_vertex":
        v[3, 0, 0] = np.inf
    elif fault == "nan_normal":
        n[7, 0] = np.nan
    elif fault == "zero_normal":
        n[9] = 0.0
    elif fault == "scaled_normal":
        n[9] *= 3.0
    elif fault == "nan_alpha":
        a[2, 0] = np.nan
    elif fault == "bad_type":
        t[4] = 7
    st, msg, h = _create(engine, v, n, b, t, a)
    assert st == 1 and expect in msg, (st, msg)
    assert not h.value


def test_zero_total_area_is_refused(engine):
    v = np.zeros((4, 2, 2), np.float32)
    n = np.tile(np.array([[1.0, 0.0]], np.float32), (4, 1))
    st, msg, _ = _create(engine, v, n, np.ones((4, 2)), np.zeros(4))
    assert st == 1 and "total boundary area" in msg, (st, msg)
