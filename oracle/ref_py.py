"""ctypes binding of the reference's own estimator, compiled from the reference tree
(oracle/_ref/libwobref.so, built by `make -C oracle ref` from oracle/ref_driver.cpp).

TEST INFRASTRUCTURE ONLY: used by tests/golden/make_reference_fixtures.py to produce the committed
reference fixtures. The reference tree is only present where the fixtures are generated; nothing
that runs on a GPU machine imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libwobref.so")
REFERENCE = os.environ.get("WOB_REFERENCE_TREE", "/root/reference")


def available() -> bool:
    return os.path.isdir(os.path.join(REFERENCE, "wob", "wob"))


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REFERENCE}"], check=True, capture_output=True)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.wobref_solve_domain.restype = C.c_int
        L.wobref_solve_domain.argtypes = [C.c_int, C.c_uint32, vp, vp, vp, vp, vp, vp, vp, vp, C.c_uint32, C.c_float,
                                          vp, C.c_uint64, vp, C.c_uint32, vp, vp, vp, C.c_uint32]
        L.wobref_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def solve_domain(verts, normals, bvals, types, alphas, params, points, seed: int, n_per_path: int = 0,
                 volume=None):
    """The reference's compute_sample_path_contribution_domain, params.num_sample_paths times per
    point. Returns (sum [n, D+1], sumsq [n, D+1], per_path [n_per_path, n_paths] of u)."""
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    verts, normals, bvals, points = f32(verts), f32(normals), f32(bvals), f32(points)
    types = np.ascontiguousarray(types, dtype=np.int32)
    alphas = None if alphas is None else f32(alphas)
    D = verts.shape[2]
    n = len(points)
    enums = np.array([params.bie_model, params.domain, params.estimator, params.problem], np.int32)
    counts = np.array([params.path_length, params.num_sample_paths, params.num_resampling_candidates,
                       params.num_volume_samples], np.uint32)
    reals = np.array([params.eps, params.first_kind_equation_scaling_constant], np.float32)
    s = np.zeros((n, D + 1))
    q = np.zeros((n, D + 1))
    pp = np.zeros((n_per_path, params.num_sample_paths), np.float32) if n_per_path else None
    vol_res, vol_size, vol_values = 0, 0.0, None
    if volume is not None:
        vol_res, vol_size, vol_values = volume[0], float(volume[1]), f32(volume[2])
    st = lib().wobref_solve_domain(D, len(verts), _p(verts), _p(normals), _p(bvals), _p(types), _p(alphas),
                                   _p(enums), _p(counts), _p(reals), vol_res, vol_size, _p(vol_values), int(seed),
                                   _p(points), n, _p(s), _p(q), _p(pp), n_per_path)
    if st != 0:
        raise RuntimeError(lib().wobref_last_error().decode())
    return s, q, pp
