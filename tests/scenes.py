"""Small seeded scenes shared by the parity tests (2D stars, 3D displaced icospheres), with
closed-form boundary data in the style of apps/general_2d.cu:73-104 / general_3d.cu:75-108."""
from __future__ import annotations

import numpy as np

from wobtoolbox_gb300 import workloads as W

F32 = np.float32


def _u2d(p, exterior):
    """Interior: e^x cos y. Exterior: x/|x|^2 (EXTERIOR_SOLUTION1 of apps/general_2d.cu:78-82)."""
    p = p.astype(np.float64)
    if not exterior:
        return W.exp_cos(p)
    x, y = p[:, 0], p[:, 1]
    r2 = x * x + y * y
    return np.stack([x / r2, 1 / r2 - 2 * x * x / r2 ** 2, -2 * x * y / r2 ** 2], axis=1)


def types_for(problem: int, n: int, seed: int) -> np.ndarray:
    if problem == 3:
        return np.random.default_rng(seed).integers(0, 3, n).astype(np.int32)
    return np.full(n, problem, dtype=np.int32)


def boundary_data(u_at, verts, normals, types, alpha):
    """Per-vertex Dirichlet / Neumann / Robin data from a closed-form u (apps/general_2d.cu:257-269)."""
    n, d = verts.shape[0], verts.shape[1]
    ug = u_at(verts.reshape(-1, d)).reshape(n, d, d + 1)
    dudn = (ug[..., 1:] * normals[:, None, :].astype(np.float64)).sum(-1)
    g = np.where(types[:, None] == 0, ug[..., 0], np.where(types[:, None] == 1, dudn, alpha * ug[..., 0] + dudn))
    return g.astype(F32)


def scene2d(problem: int, exterior: bool, n_seg: int = 96, seed: int = 1, n_points: int = 10):
    verts, normals = W.star_polygon(n_seg, 3, 0.25)
    if exterior:  # apps/general_2d.cu:204-207
        verts = (verts * F32(0.5)).astype(F32)
        verts[..., 1] += F32(0.0625)
        normals = W.segment_normals(verts)
    types = types_for(problem, n_seg, seed)
    alpha = 1.0
    g = boundary_data(lambda p: _u2d(p, exterior), verts, normals, types, alpha)
    alphas = np.full((n_seg, 2), alpha, dtype=F32)
    grid = W.idx_to_domain_point(24, 2.4 if not exterior else 1.6, 2)
    wn = W.winding_number_2d(verts, grid)
    mask = (wn < -0.5) if not exterior else (wn > -0.5)
    pts = grid[mask]
    if exterior:
        pts = pts[np.linalg.norm(pts - np.array([0, 0.0625], F32), axis=1) > 0.15]
    pts = pts[np.random.default_rng(seed).permutation(len(pts))[:n_points]]
    return dict(verts=verts, normals=normals, bvals=g, types=types, alphas=alphas,
                points=np.ascontiguousarray(pts, dtype=F32), u=lambda p: _u2d(p, exterior))


def scene3d(problem: int, exterior: bool, subdiv: int = 2, seed: int = 3, n_points: int = 10):
    V, F, _ = W.displaced_icosphere(subdiv, 0.1, 4, seed)
    verts, normals = W.mesh_elements(V, F)
    types = types_for(problem, len(F), seed)
    alpha = 1.0
    if exterior:
        src, q = np.array([[0.1, 0.2, -0.1]]), np.array([1.0])
    else:
        src, q = np.array([[3.0, 0.5, 0.0]]), np.array([1.0])
    u_at = lambda p: W.point_sources(p, src, q)
    g = boundary_data(u_at, verts, normals, types, alpha)
    alphas = np.full((len(F), 3), alpha, dtype=F32)
    rng = np.random.default_rng(seed)
    dirs = rng.standard_normal((n_points, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    radius = rng.uniform(0.1, 0.5, n_points) if not exterior else rng.uniform(1.8, 2.5, n_points)
    pts = (dirs * radius[:, None]).astype(F32)
    return dict(verts=verts, normals=normals, bvals=g, types=types, alphas=alphas, points=pts, u=u_at)


def boundary_points(sc, k: int = 6, seed: int = 5):
    """Points on element interiors with their normal, angle 1/2, interpolated data, type, alpha."""
    rng = np.random.default_rng(seed)
    verts, normals, g, types = sc["verts"], sc["normals"], sc["bvals"], sc["types"]
    idx = rng.choice(len(verts), k, replace=False)
    d = verts.shape[1]
    if d == 2:
        w = np.stack([np.full(k, 0.5), np.full(k, 0.5)], 1)
    else:
        w = np.full((k, 3), 1.0 / 3.0)
    p = (verts[idx] * w[:, :, None]).sum(1).astype(F32)
    bv = (g[idx] * w).sum(1).astype(F32)
    return dict(p=p, n=normals[idx].astype(F32), angle=np.full(k, 0.5, F32), bv=bv,
                type=types[idx].astype(np.int32), alpha=np.full(k, 1.0, F32))
