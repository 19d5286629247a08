"""Scenes and estimator settings of the reference fixtures (tests/golden/reference_*.npz).

Each case names a workload of the reference (one of its benchmarked configurations, or one of its
shipped data/config_*.json files) at a size the reference's CPU build finishes in seconds. The scene is
rebuilt from seeded generators on both sides; the fixture stores the evaluation points, the
reference's per-point statistics and, for a few points, every path value, plus a checksum of the
scene arrays so that a change of the generators is caught instead of silently compared.
"""
from __future__ import annotations

import hashlib

import numpy as np

from wobtoolbox_gb300 import EstimatorParams
from wobtoolbox_gb300 import workloads as W

F32 = np.float32
FLT_EPS = float(np.finfo(np.float32).eps)


def _three_sources(seed: int, inside: bool):
    rng = np.random.default_rng(seed)
    d = rng.standard_normal((3, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = rng.uniform(0, 0.5, (3, 1)) if inside else rng.uniform(2.0, 4.0, (3, 1))
    return d * r, rng.uniform(-1, 1, 3)


def dl2d_star1024():
    """2D interior Dirichlet, double layer, star r = 1 + 0.3 cos 5t with 1024
    segments, g = e^x cos y, the 7,960 interior points of the 128^2 grid, 8 bounces."""
    sc = W.star_dirichlet_scene()
    params = EstimatorParams(bie_model=1, domain=0, estimator=0, problem=0, path_length=8, eps=FLT_EPS)
    return dict(verts=sc["verts"], normals=sc["normals"], bvals=sc["bvals"], types=sc["types"], alphas=None,
                params=params, volume=None, n_paths=256, n_pp=8, pp_paths=4096)


def robin3d_sphere81920_alpha1():
    """The 3D Robin benchmark's geometry and data with alpha = 1 (the reference's shipped Robin value,
    for which the direct BIE's series converges; at alpha = 2 it diverges): displaced icosphere of
    81,920 triangles, u = 1/(4 pi |x - s|), s = (3, 0.5, 0), direct BIE, backward, 16 bounces."""
    sc = W.robin_sphere_scene(subdiv=6, seed=0, alpha=1.0)
    params = EstimatorParams(bie_model=2, domain=0, estimator=0, problem=2, path_length=16, eps=FLT_EPS)
    return dict(verts=sc["verts"], normals=sc["normals"], bvals=sc["bvals"], types=sc["types"], alphas=sc["alphas"],
                params=params, volume=None, n_paths=1024, n_pp=8, pp_paths=4096)


def fwdsl3d_ext_neumann_sphere5120():
    """The 3D exterior Neumann problem (data/config_general_3d_exterior_Neumann.json): exterior Neumann,
    forward single layer, 4 bounces, Neumann data of three interior point sources, on the displaced
    icosphere at 5,120 triangles."""
    V, F, _ = W.displaced_icosphere(4, 0.15, 4, 0)
    verts, normals = W.mesh_elements(V, F)
    src, q = _three_sources(0, True)
    uv = W.point_sources(verts.reshape(-1, 3), src, q).reshape(len(F), 3, 4)
    g = (uv[..., 1:] * normals[:, None, :].astype(np.float64)).sum(-1).astype(F32)
    params = EstimatorParams(bie_model=0, domain=1, estimator=1, problem=1, path_length=4, eps=FLT_EPS)
    return dict(verts=verts, normals=normals, bvals=g, types=np.ones(len(F), np.int32), alphas=None,
                params=params, volume=None, n_paths=1024, n_pp=8, pp_paths=4096)


def slris3d_mixed_sphere1280():
    """The 3D interior mixed problem (data/config_general_3d_interior_Mixed.json: single layer, backward,
    64 resampling candidates, eps 1e-5, first-kind scaling 2, 4 bounces): Dirichlet on faces whose
    centroid has z > 0, Neumann elsewhere, data of three exterior point sources, icosphere at
    1,280 triangles."""
    V, F, _ = W.displaced_icosphere(3, 0.15, 4, 0)
    verts, normals = W.mesh_elements(V, F)
    types = np.where(verts.astype(np.float64).mean(1)[:, 2] > 0, 0, 1).astype(np.int32)
    src, q = _three_sources(1, False)
    uv = W.point_sources(verts.reshape(-1, 3), src, q).reshape(len(F), 3, 4)
    dudn = (uv[..., 1:] * normals[:, None, :].astype(np.float64)).sum(-1)
    g = np.where(types[:, None] == 0, uv[..., 0], dudn).astype(F32)
    params = EstimatorParams(bie_model=0, domain=0, estimator=0, problem=3, path_length=4, eps=1e-5,
                             num_resampling_candidates=64, first_kind_equation_scaling_constant=2.0)
    return dict(verts=verts, normals=normals, bvals=g, types=types, alphas=None, params=params, volume=None,
                n_paths=512, n_pp=4, pp_paths=4096)


def slris2d_robin_star512():
    """data/config_general_2d_interior_Robin.json's estimator (single layer, backward, 64
    resampling candidates, eps 1e-5, 4 bounces) on a 512-segment star with Robin alpha = 1 and
    g from u = e^x cos y."""
    verts, normals = W.star_polygon(512, 3, 0.25)
    uv = W.exp_cos(verts.reshape(-1, 2)).reshape(len(verts), 2, 3)
    dudn = (uv[..., 1:] * normals[:, None, :].astype(np.float64)).sum(-1)
    g = (uv[..., 0] + dudn).astype(F32)
    params = EstimatorParams(bie_model=0, domain=0, estimator=0, problem=2, path_length=4, eps=1e-5,
                             num_resampling_candidates=64)
    return dict(verts=verts, normals=normals, bvals=g, types=np.full(len(verts), 2, np.int32),
                alphas=np.ones((len(verts), 2), F32), params=params, volume=None, n_paths=512, n_pp=4,
                pp_paths=4096)


def dl2d_poisson_box():
    """apps/poisson_equation.cu with data/config_poisson_equation.json: the box (-1, 1)^2 with
    u = 1 on its sides, the constant source 5 through a volume cache (here 64^2 cells over the
    box), double layer, 4 bounces, 16 volume samples, eps 1e-4."""
    sq = np.array([[[-1, -1], [-1, 1]], [[-1, 1], [1, 1]], [[1, 1], [1, -1]], [[1, -1], [-1, -1]]], F32)
    nrm = np.array([[-1, 0], [0, 1], [1, 0], [0, -1]], F32)
    res = 64
    params = EstimatorParams(bie_model=1, domain=0, estimator=0, problem=0, path_length=4, eps=1e-4,
                             num_volume_samples=16)
    return dict(verts=sq, normals=nrm, bvals=np.ones((4, 2), F32), types=np.zeros(4, np.int32), alphas=None,
                params=params, volume=(res, 2.0, np.full(res * res, 5.0, F32)), n_paths=1024, n_pp=4,
                pp_paths=4096)


def direct2d_int_neumann_star512():
    """The direct BIE's Neumann estimator (line-intersection and |g| sampling,
    estimator.cuh:158-168, 304-334): interior Neumann on a 512-segment star, g = du/dn of
    e^x cos y, 6 bounces."""
    verts, normals = W.star_polygon(512, 3, 0.25)
    uv = W.exp_cos(verts.reshape(-1, 2)).reshape(len(verts), 2, 3)
    g = (uv[..., 1:] * normals[:, None, :].astype(np.float64)).sum(-1).astype(F32)
    params = EstimatorParams(bie_model=2, domain=0, estimator=0, problem=1, path_length=6, eps=FLT_EPS)
    return dict(verts=verts, normals=normals, bvals=g, types=np.ones(len(verts), np.int32), alphas=None,
                params=params, volume=None, n_paths=512, n_pp=4, pp_paths=4096)


CASES = {f.__name__: f for f in [dl2d_star1024, robin3d_sphere81920_alpha1, fwdsl3d_ext_neumann_sphere5120,
                                 slris3d_mixed_sphere1280, slris2d_robin_star512, dl2d_poisson_box,
                                 direct2d_int_neumann_star512]}


def scene_checksum(case: dict) -> str:
    h = hashlib.sha256()
    for k in ("verts", "normals", "bvals", "types", "alphas"):
        a = case[k]
        if a is not None:
            h.update(np.ascontiguousarray(a).tobytes())
    if case["volume"] is not None:
        h.update(np.ascontiguousarray(case["volume"][2]).tobytes())
    return h.hexdigest()[:16]


def fixture_path(name: str) -> str:
    import os
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", f"reference_{name}.npz")
