"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
bench.py, never by the engine. Elements are passed in the engine's storage order.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
HIT_BUFFER = 64


class oracle_params(C.Structure):
    _fields_ = [
        ("bie_model", C.c_int32), ("domain", C.c_int32), ("estimator", C.c_int32), ("problem", C.c_int32),
        ("path_length", C.c_uint32), ("num_sample_paths", C.c_uint32),
        ("num_resampling_candidates", C.c_uint32), ("num_volume_samples", C.c_uint32),
        ("eps", C.c_float), ("first_kind_equation_scaling_constant", C.c_float),
        ("seed", C.c_uint64), ("path_offset", C.c_uint64),
        ("point_offset", C.c_uint32), ("flags", C.c_uint32),
    ]


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True, capture_output=True)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        vp, u32, u64, f32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float
        L.oracle_solve_domain.restype = u64
        L.oracle_solve_domain.argtypes = [C.c_int, u32, vp, vp, vp, vp, vp, u32, f32, vp, C.POINTER(oracle_params),
                                          vp, u32, vp, vp, vp, C.c_int]
        L.oracle_solve_boundary.restype = u64
        L.oracle_solve_boundary.argtypes = [C.c_int, u32, vp, vp, vp, vp, vp, u32, f32, vp,
                                            C.POINTER(oracle_params), vp, vp, vp, vp, vp, vp, u32, vp, vp, vp,
                                            C.c_int]
        L.oracle_solve_domain_cv.restype = u64
        L.oracle_solve_domain_cv.argtypes = [C.c_int, u32, vp, vp, vp, vp, vp, C.POINTER(oracle_params), vp, u32,
                                             u32, vp, u32, vp, vp, vp, C.c_int]
        L.oracle_solve_domain_bcv.restype = u64
        L.oracle_solve_domain_bcv.argtypes = [C.c_int, u32, vp, vp, vp, vp, vp, C.POINTER(oracle_params), vp, u32,
                                              vp, u32, vp, vp, vp, C.c_int]
        L.oracle_lbvh_stats.restype = None
        L.oracle_lbvh_stats.argtypes = [C.c_int, u32, vp, vp, vp, vp, vp, C.POINTER(oracle_params), vp, u32, vp,
                                        C.c_int]
        L.oracle_wos.restype = u64
        L.oracle_wos.argtypes = [u32, vp, vp, vp, vp, C.POINTER(oracle_params), vp, u32, vp, vp, C.c_int]
        L.oracle_closest_point.restype = None
        L.oracle_closest_point.argtypes = [u32, vp, vp, vp, vp, vp, u32, vp, vp, vp]
        L.oracle_vpl_paths.restype = u64
        L.oracle_vpl_paths.argtypes = [C.c_int, u32, vp, vp, vp, vp, vp, C.POINTER(oracle_params), u32, vp, vp,
                                       C.c_int]
        L.oracle_vpl_aggregate.restype = None
        L.oracle_vpl_aggregate.argtypes = [C.c_int, f32, f32, vp, vp, u32, vp, u32, vp, C.c_int]
        L.oracle_solve_unknown.restype = u64
        L.oracle_solve_unknown.argtypes = [C.c_int, u32, vp, vp, vp, vp, vp, C.POINTER(oracle_params), vp, vp, vp,
                                           vp, vp, vp, u32, vp, vp, C.c_int]
        L.oracle_line_query.restype = None
        L.oracle_line_query.argtypes = [C.c_int, u32, vp, vp, vp, vp, vp, vp, u32, vp, vp, vp]
        L.oracle_scene_cdfs.restype = None
        L.oracle_scene_cdfs.argtypes = [C.c_int, u32, vp, vp, vp, vp, vp, vp, vp]
        L.oracle_simple_wob.restype = None
        L.oracle_simple_wob.argtypes = [u32, vp, vp, vp, vp, u64, u32, u32, vp, u32, vp, C.c_int]
        L.oracle_sincospi.argtypes = [vp, vp, vp, u32]
        L.oracle_log.argtypes = [vp, vp, u32]
        L.oracle_philox.argtypes = [vp, u32, u32, vp]
        L.oracle_uniforms.argtypes = [u64, u32, u32, u64, vp, u32]
        L.oracle_green.argtypes = [C.c_int, f32, vp, vp, vp, vp, u32, vp]
        L.oracle_max_threads.restype = C.c_int
        _lib = L
    return _lib


def _f32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a):
    return None if a is None else a.ctypes.data


def params_struct(p, accel: bool = False) -> oracle_params:
    """From any object with the wob_params field names (e.g. wobtoolbox_gb300.EstimatorParams).
    accel: filter line queries through the oracle's padded binary BVH (same results, faster)."""
    s = oracle_params()
    for name, _ in oracle_params._fields_:
        if name == "flags":
            continue
        setattr(s, name, getattr(p, name))
    s.flags = 1 if accel else 0
    return s


class Elements:
    """Element arrays in storage order: verts [n,d,d], normals [n,d], bvals [n,d], types [n], alphas."""

    def __init__(self, verts, normals, bvals, types, alphas=None, volume=None):
        self.verts = _f32(verts)
        self.dim = self.verts.shape[1]
        self.n = self.verts.shape[0]
        self.normals = _f32(normals).reshape(self.n, self.dim)
        self.bvals = _f32(bvals).reshape(self.n, self.dim)
        self.types = np.ascontiguousarray(types, dtype=np.int32)
        self.alphas = None if alphas is None else _f32(alphas).reshape(self.n, self.dim)
        self.volume = volume  # (grid_res, domain_size, values) or None

    def _vol(self):
        if self.volume is None:
            return 0, 0.0, None
        res, size, vals = self.volume
        vals = _f32(vals).reshape(-1)
        return res, float(size), vals


def solve_domain(el: Elements, params, points, per_path: bool = False, n_threads: int = 0, accel: bool = False):
    pts = _f32(points).reshape(-1, el.dim)
    n = len(pts)
    D = el.dim
    s = np.zeros((n, D + 1))
    q = np.zeros((n, D + 1))
    pp = np.zeros((n, params.num_sample_paths, D + 1), dtype=np.float32) if per_path else None
    res, size, vals = el._vol()
    ps = params_struct(params, accel)
    b = lib().oracle_solve_domain(D, el.n, _ptr(el.verts), _ptr(el.normals), _ptr(el.bvals), _ptr(el.alphas),
                                  _ptr(el.types), res, size, _ptr(vals), C.byref(ps), _ptr(pts), n, _ptr(s),
                                  _ptr(q), _ptr(pp), n_threads)
    return s, q, int(b), pp


def solve_boundary(el: Elements, params, p, n, angle, bv, btype, alpha=None, per_path: bool = False,
                   n_threads: int = 0):
    D = el.dim
    p = _f32(p).reshape(-1, D)
    m = len(p)
    n = _f32(n).reshape(m, D)
    angle = _f32(angle).reshape(m)
    bv = _f32(bv).reshape(m)
    btype = np.ascontiguousarray(btype, dtype=np.int32).reshape(m)
    alpha = None if alpha is None else _f32(alpha).reshape(m)
    s = np.zeros(m)
    q = np.zeros(m)
    pp = np.zeros((m, params.num_sample_paths), dtype=np.float32) if per_path else None
    res, size, vals = el._vol()
    ps = params_struct(params)
    b = lib().oracle_solve_boundary(D, el.n, _ptr(el.verts), _ptr(el.normals), _ptr(el.bvals), _ptr(el.alphas),
                                    _ptr(el.types), res, size, _ptr(vals), C.byref(ps), _ptr(p), _ptr(n),
                                    _ptr(angle), _ptr(bv), _ptr(btype), _ptr(alpha), m, _ptr(s), _ptr(q), _ptr(pp),
                                    n_threads)
    return s, q, int(b), pp


def solve_domain_cv(el: Elements, params, sigma_t, n_pot: int, m_ker: int, points, per_path: bool = False,
                    n_threads: int = 0):
    pts = _f32(points).reshape(-1, el.dim)
    n = len(pts)
    D = el.dim
    sg = _f32(sigma_t).reshape(el.n)
    s = np.zeros((n, D + 1))
    q = np.zeros((n, D + 1))
    pp = np.zeros((n, params.num_sample_paths, D + 1), dtype=np.float32) if per_path else None
    ps = params_struct(params)
    b = lib().oracle_solve_domain_cv(D, el.n, _ptr(el.verts), _ptr(el.normals), _ptr(el.bvals), _ptr(el.alphas),
                                     _ptr(el.types), C.byref(ps), _ptr(sg), n_pot, m_ker, _ptr(pts), n, _ptr(s),
                                     _ptr(q), _ptr(pp), n_threads)
    return s, q, int(b), pp


def solve_domain_bcv(el: Elements, params, cv, n_pot: int, points, per_path: bool = False, n_threads: int = 0):
    """Backward estimator with a per-element control variate (storage order) on the unknown
    boundary function; u only."""
    pts = _f32(points).reshape(-1, el.dim)
    n = len(pts)
    c = _f32(cv).reshape(el.n)
    s = np.zeros(n)
    q = np.zeros(n)
    pp = np.zeros((n, params.num_sample_paths), dtype=np.float32) if per_path else None
    ps = params_struct(params)
    b = lib().oracle_solve_domain_bcv(el.dim, el.n, _ptr(el.verts), _ptr(el.normals), _ptr(el.bvals), _ptr(el.alphas),
                                      _ptr(el.types), C.byref(ps), _ptr(c), n_pot, _ptr(pts), n, _ptr(s), _ptr(q),
                                      _ptr(pp), n_threads)
    return s, q, int(b), pp


def lbvh_stats(el: Elements, params, points, n_threads: int = 0):
    """Mean nodes visited and primitives tested per line query of the reference's binary LBVH on the
    line queries the domain estimator makes at these points: (queries, N_node, N_prim)."""
    pts = _f32(points).reshape(-1, el.dim)
    out = np.zeros(3)
    ps = params_struct(params)
    lib().oracle_lbvh_stats(el.dim, el.n, _ptr(el.verts), _ptr(el.normals), _ptr(el.bvals), _ptr(el.alphas),
                            _ptr(el.types), C.byref(ps), _ptr(pts), len(pts), _ptr(out), n_threads)
    q = max(out[0], 1.0)
    return int(out[0]), out[1] / q, out[2] / q


def wos(el: Elements, params, points, per_path: bool = False, n_threads: int = 0):
    """Walk on spheres (2D Dirichlet): (sum [n], per_path [n, paths] or None, closest-point queries)."""
    pts = _f32(points).reshape(-1, 2)
    s = np.zeros(len(pts))
    pp = np.zeros((len(pts), params.num_sample_paths), dtype=np.float32) if per_path else None
    ps = params_struct(params)
    q = lib().oracle_wos(el.n, _ptr(el.verts), _ptr(el.normals), _ptr(el.bvals), _ptr(el.types), C.byref(ps),
                         _ptr(pts), len(pts), _ptr(s), _ptr(pp), n_threads)
    return s, pp, int(q)


def closest_point(el: Elements, points):
    pts = _f32(points).reshape(-1, 2)
    n = len(pts)
    e = np.zeros(n, dtype=np.uint32)
    d = np.zeros(n, dtype=np.float32)
    v = np.zeros(n, dtype=np.float32)
    lib().oracle_closest_point(el.n, _ptr(el.verts), _ptr(el.normals), _ptr(el.bvals), _ptr(el.types), _ptr(pts), n,
                               _ptr(e), _ptr(d), _ptr(v))
    return e, d, v


def vpl_paths(el: Elements, params, n_paths: int, n_threads: int = 0):
    """VPL walks: (points [n, dim], values [n], bounces)."""
    p = np.zeros((n_paths, el.dim), dtype=np.float32)
    mu = np.zeros(n_paths, dtype=np.float32)
    ps = params_struct(params)
    b = lib().oracle_vpl_paths(el.dim, el.n, _ptr(el.verts), _ptr(el.normals), _ptr(el.bvals), _ptr(el.alphas),
                               _ptr(el.types), C.byref(ps), n_paths, _ptr(p), _ptr(mu), n_threads)
    return p, mu, int(b)


def vpl_aggregate(dim: int, area: float, eps: float, vpl_p, vpl_mu, points, n_threads: int = 0):
    vp_ = _f32(vpl_p).reshape(-1, dim)
    mu = _f32(vpl_mu).reshape(-1)
    pts = _f32(points).reshape(-1, dim)
    out = np.zeros((len(pts), dim + 1))
    lib().oracle_vpl_aggregate(dim, float(area), float(eps), _ptr(vp_), _ptr(mu), len(mu), _ptr(pts), len(pts),
                               _ptr(out), n_threads)
    return out


def solve_unknown(el: Elements, params, p, n, angle, bv, btype, alpha=None, per_path: bool = False, n_threads: int = 0):
    D = el.dim
    p = _f32(p).reshape(-1, D)
    m = len(p)
    n = _f32(n).reshape(m, D)
    angle, bv = _f32(angle).reshape(m), _f32(bv).reshape(m)
    btype = np.ascontiguousarray(btype, dtype=np.int32).reshape(m)
    alpha = None if alpha is None else _f32(alpha).reshape(m)
    s = np.zeros(m)
    pp = np.zeros((m, params.num_sample_paths), dtype=np.float32) if per_path else None
    ps = params_struct(params)
    b = lib().oracle_solve_unknown(D, el.n, _ptr(el.verts), _ptr(el.normals), _ptr(el.bvals), _ptr(el.alphas),
                                   _ptr(el.types), C.byref(ps), _ptr(p), _ptr(n), _ptr(angle), _ptr(bv),
                                   _ptr(btype), _ptr(alpha), m, _ptr(s), _ptr(pp), n_threads)
    return s, int(b), pp


def line_query(el: Elements, origins, dirs):
    D = el.dim
    o = _f32(origins).reshape(-1, D)
    d = _f32(dirs).reshape(-1, D)
    n = len(o)
    counts = np.zeros(n, dtype=np.uint32)
    hits = np.zeros((n, HIT_BUFFER), dtype=np.uint32)
    pts = np.zeros((n, HIT_BUFFER, D), dtype=np.float32)
    lib().oracle_line_query(D, el.n, _ptr(el.verts), _ptr(el.normals), _ptr(el.bvals), _ptr(el.types), _ptr(o),
                            _ptr(d), n, _ptr(counts), _ptr(hits), _ptr(pts))
    return counts, hits, pts


def scene_cdfs(el: Elements):
    a = np.zeros(el.n, dtype=np.float32)
    b = np.zeros(el.n, dtype=np.float32)
    t = np.zeros(2, dtype=np.float32)
    lib().oracle_scene_cdfs(el.dim, el.n, _ptr(el.verts), _ptr(el.normals), _ptr(el.bvals), _ptr(el.types),
                            _ptr(a), _ptr(b), _ptr(t))
    return a, b, t


def simple_wob(el: Elements, seed: int, path_length: int, n_paths: int, points, n_threads: int = 0):
    pts = _f32(points).reshape(-1, 2)
    out = np.zeros(len(pts))
    lib().oracle_simple_wob(el.n, _ptr(el.verts), _ptr(el.normals), _ptr(el.bvals), _ptr(el.types), seed,
                            path_length, n_paths, _ptr(pts), len(pts), _ptr(out), n_threads)
    return out


def sincospi(x):
    x = _f32(x).reshape(-1)
    s = np.zeros_like(x)
    c = np.zeros_like(x)
    lib().oracle_sincospi(_ptr(x), _ptr(s), _ptr(c), len(x))
    return s, c


def log(x):
    x = _f32(x).reshape(-1)
    y = np.zeros_like(x)
    lib().oracle_log(_ptr(x), _ptr(y), len(x))
    return y


def philox(ctr, k0: int, k1: int):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().oracle_philox(_ptr(c), k0, k1, _ptr(out))
    return out


def uniforms(seed: int, stream: int, point: int, path: int, n: int):
    out = np.zeros(n, dtype=np.float32)
    lib().oracle_uniforms(seed, stream, point, path, _ptr(out), n)
    return out


def green(dim: int, eps: float, y, x, ny, nx):
    y, x, ny, nx = (_f32(a).reshape(-1, dim) for a in (y, x, ny, nx))
    out = np.zeros((len(y), 7 if dim == 2 else 9), dtype=np.float32)
    lib().oracle_green(dim, eps, _ptr(y), _ptr(x), _ptr(ny), _ptr(nx), len(y), _ptr(out))
    return out


def max_threads() -> int:
    return int(lib().oracle_max_threads())
