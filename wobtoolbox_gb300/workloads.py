"""Synthetic scenes, evaluation points and closed-form solutions of the benchmark workloads.

The reference validates every app against closed-form harmonic solutions (apps/general_2d.cu:73-104,
apps/general_3d.cu:75-108); these generators produce the boundaries and boundary data of the
workloads this engine is measured on, all seeded and reproducible:

* star_polygon: r(theta) = 1 + amp cos(lobes theta), vertices ordered clockwise so that the
  reference's normal rule n = (t_y, -t_x), t = (v1 - v2)/|v1 - v2| (apps/general_2d.cu:245-249)
  points outward, and interior points have winding number -1 (apps/general_2d.cu:279-281).
* displaced_icosphere: a subdivided icosahedron pushed radially by amp * sum_{l<=lmax} c_lm Y_lm,
  c_lm ~ N(0,1) from numpy's default_rng(seed), real orthonormal spherical harmonics without the
  Condon-Shortley phase; faces counter-clockwise seen from outside, normals (b-a)x(c-a)/|.|
  (igl::per_face_normals).
"""
from __future__ import annotations

import math

import numpy as np

F32 = np.float32


# ------------------------------------------------------------------ grids (utils.cuh:68-118)
def idx_to_domain_point(grid_res: int, domain_size: float, dim: int = 2) -> np.ndarray:
    """Cell centres in (-size/2, size/2)^dim, x fastest, evaluated in float32 like the reference."""
    n = grid_res ** dim
    idx = np.arange(n, dtype=np.int64)
    dx = F32(domain_size) / F32(grid_res)
    half = F32(domain_size) / F32(2)
    cols = []
    for k in range(dim):
        c = (idx // (grid_res ** k)) % grid_res
        cols.append((c.astype(F32) + F32(0.5)) * dx - half)
    return np.stack(cols, axis=1).astype(F32)


# ------------------------------------------------------------------ 2D
def star_polygon(n_seg: int = 1024, lobes: int = 5, amp: float = 0.3, radius: float = 1.0, center=(0.0, 0.0)):
    """Closed star polygon, clockwise. Returns segment vertices [n, 2, 2] (float32) and normals [n, 2]."""
    k = np.arange(n_seg, dtype=np.float64)
    theta = -2.0 * np.pi * k / n_seg
    r = radius * (1.0 + amp * np.cos(lobes * theta))
    pts = np.stack([center[0] + r * np.cos(theta), center[1] + r * np.sin(theta)], axis=1).astype(F32)
    v1 = pts
    v2 = np.roll(pts, -1, axis=0)
    verts = np.stack([v1, v2], axis=1)
    return verts, segment_normals(verts)


def segment_normals(verts: np.ndarray) -> np.ndarray:
    """n = (t_y, -t_x), t = (v1 - v2)/|v1 - v2| in float32 (apps/general_2d.cu:245-249)."""
    d = (verts[:, 0, :] - verts[:, 1, :]).astype(F32)
    nn = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]).astype(F32)
    t = d / nn[:, None]
    return np.stack([t[:, 1], -t[:, 0]], axis=1).astype(F32)


def winding_number_2d(verts: np.ndarray, points: np.ndarray, chunk: int = 4096) -> np.ndarray:
    """Generalised winding number of a segment soup at points (signed angle sum / 2 pi)."""
    a = verts[:, 0, :].astype(np.float64)
    b = verts[:, 1, :].astype(np.float64)
    out = np.empty(len(points))
    for s in range(0, len(points), chunk):
        p = points[s:s + chunk].astype(np.float64)[:, None, :]
        va = a[None] - p
        vb = b[None] - p
        cross = va[..., 0] * vb[..., 1] - va[..., 1] * vb[..., 0]
        dot = (va * vb).sum(-1)
        out[s:s + chunk] = np.arctan2(cross, dot).sum(1) / (2 * np.pi)
    return out


def exp_cos(p: np.ndarray) -> np.ndarray:
    """u = e^x cos y and its gradient, [n, 3] (float64)."""
    x, y = p[:, 0].astype(np.float64), p[:, 1].astype(np.float64)
    ex = np.exp(x)
    return np.stack([ex * np.cos(y), ex * np.cos(y), -ex * np.sin(y)], axis=1)


# ------------------------------------------------------------------ 3D meshes
def icosphere(subdiv: int):
    """Unit icosphere: vertices [nv, 3] float64, faces [nf, 3] int64 (CCW seen from outside)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    V = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    for _ in range(subdiv):
        e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]], axis=0)
        e_sorted = np.sort(e, axis=1)
        uniq, inv = np.unique(e_sorted, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = V[uniq[:, 0]] + V[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(V)
        V = np.concatenate([V, mid], axis=0)
        nf = len(F)
        m01 = base + inv[:nf]
        m12 = base + inv[nf:2 * nf]
        m20 = base + inv[2 * nf:]
        a, b, c = F[:, 0], F[:, 1], F[:, 2]
        F = np.concatenate([np.stack([a, m01, m20], 1), np.stack([b, m12, m01], 1), np.stack([c, m20, m12], 1),
                            np.stack([m01, m12, m20], 1)], axis=0)
    return V, F


def real_sph_harm(lmax: int, dirs: np.ndarray) -> np.ndarray:
    """Real orthonormal spherical harmonics Y_lm (l <= lmax, m = -l..l in that order), no
    Condon-Shortley phase; dirs are unit vectors [n, 3]. Returns [n, (lmax+1)^2]."""
    x, y, z = dirs[:, 0], dirs[:, 1], dirs[:, 2]
    ct = np.clip(z, -1.0, 1.0)
    st = np.sqrt(np.maximum(0.0, 1.0 - ct * ct))
    phi = np.arctan2(y, x)
    P = {}
    for m in range(lmax + 1):
        pmm = np.ones_like(ct)
        for i in range(1, m + 1):
            pmm = pmm * (2 * i - 1) * st
        P[(m, m)] = pmm
        if m + 1 <= lmax:
            P[(m + 1, m)] = ct * (2 * m + 1) * pmm
        for l in range(m + 2, lmax + 1):
            P[(l, m)] = ((2 * l - 1) * ct * P[(l - 1, m)] - (l + m - 1) * P[(l - 2, m)]) / (l - m)
    cols = []
    for l in range(lmax + 1):
        for m in range(-l, l + 1):
            am = abs(m)
            k = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
            if m == 0:
                cols.append(k * P[(l, 0)])
            elif m > 0:
                cols.append(math.sqrt(2) * k * np.cos(m * phi) * P[(l, m)])
            else:
                cols.append(math.sqrt(2) * k * np.sin(am * phi) * P[(l, am)])
    return np.stack(cols, axis=1)


def displaced_icosphere(subdiv: int, amp: float = 0.15, lmax: int = 4, seed: int = 0):
    """Icosphere displaced radially by amp * sum c_lm Y_lm. Returns V [nv,3] float64, F, coeffs."""
    V, F = icosphere(subdiv)
    coeffs = np.random.default_rng(seed).standard_normal((lmax + 1) ** 2)
    r = 1.0 + amp * real_sph_harm(lmax, V) @ coeffs
    if r.min() <= 0.05:
        raise ValueError("displacement folds the surface; choose another seed")
    return V * r[:, None], F, coeffs


def face_normals(V: np.ndarray, F: np.ndarray) -> np.ndarray:
    """Unit (b - a) x (c - a) per face (igl::per_face_normals), float32."""
    a, b, c = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    n = np.cross(b - a, c - a)
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    return (n / np.where(ln > 0, ln, 1.0)).astype(F32)


def mesh_elements(V: np.ndarray, F: np.ndarray):
    """Triangle vertices [n, 3, 3] float32 and face normals [n, 3]."""
    Vf = V.astype(F32)
    return np.ascontiguousarray(Vf[F]), face_normals(V.astype(np.float64), F)


def point_sources(p: np.ndarray, sources: np.ndarray, q: np.ndarray) -> np.ndarray:
    """u = sum q_k / (4 pi |x - s_k|) and its gradient, [n, 4] float64."""
    p = p.astype(np.float64)
    out = np.zeros((len(p), 4))
    for s, qq in zip(sources, q):
        d = p - s[None, :]
        r = np.linalg.norm(d, axis=1)
        out[:, 0] += qq / (4 * np.pi * r)
        out[:, 1:] += -qq * d / (4 * np.pi * r[:, None] ** 3)
    return out


# ------------------------------------------------------------------ the benchmark scenes
def star_dirichlet_scene():
    """2D interior Dirichlet star (1024 segments, r = 1 + 0.3 cos 5 theta), g = e^x cos y at the
    vertices, linear along segments; 128^2 grid over [-1.3, 1.3]^2, interior points only."""
    verts, normals = star_polygon(1024, 5, 0.3)
    g = exp_cos(verts.reshape(-1, 2))[:, 0].reshape(-1, 2).astype(F32)
    types = np.zeros(len(verts), dtype=np.int32)
    grid = idx_to_domain_point(128, 2.6, 2)
    wn = winding_number_2d(verts, grid)
    mask = wn < -0.5
    return dict(verts=verts, normals=normals, bvals=g, types=types, alphas=None, grid=grid, mask=mask,
                points=np.ascontiguousarray(grid[mask]))


def robin_sphere_scene(subdiv: int = 6, seed: int = 0, alpha: float = 2.0, source=(3.0, 0.5, 0.0)):
    """3D interior Robin (du/dn + alpha u = h) on a displaced icosphere, u = 1/(4 pi |x - s|)."""
    V, F, coeffs = displaced_icosphere(subdiv, 0.15, 4, seed)
    verts, normals = mesh_elements(V, F)
    s = np.array([source], dtype=np.float64)
    q = np.array([1.0])
    uv = point_sources(verts.reshape(-1, 3), s, q).reshape(len(F), 3, 4)
    h = uv[..., 0] * alpha + (uv[..., 1:] * normals[:, None, :].astype(np.float64)).sum(-1)
    types = np.full(len(F), 2, dtype=np.int32)
    alphas = np.full((len(F), 3), alpha, dtype=F32)
    return dict(verts=verts, normals=normals, bvals=h.astype(F32), types=types, alphas=alphas, coeffs=coeffs,
                source=s, strengths=q)


def slice_points_z0(grid_res: int = 512, domain_size: float = 2.6) -> np.ndarray:
    """Evaluation points (x, y, 0) on a grid_res^2 grid over (-size/2, size/2)^2."""
    g = idx_to_domain_point(grid_res, domain_size, 2)
    return np.ascontiguousarray(np.concatenate([g, np.zeros((len(g), 1), F32)], axis=1))


def inside_by_parity(counts_pos: np.ndarray) -> np.ndarray:
    """Inside a closed surface iff a half-line from the point crosses it an odd number of times."""
    return (counts_pos % 2) == 1


# ------------------------------------------------------------------ batched 2D scenes
def _star_points_inside(rng, lobes, amp, n, margin=0.9):
    th = rng.uniform(0, 2 * np.pi, n)
    rr = margin * (1 + amp * np.cos(lobes * th)) * np.sqrt(rng.uniform(0, 1, n))
    return np.stack([rr * np.cos(th), rr * np.sin(th)], 1).astype(F32)


def _star_points_outside(rng, lobes, amp, scale, n):
    th = rng.uniform(0, 2 * np.pi, n)
    r0 = scale * (1 + amp) * 1.1
    rr = r0 + rng.uniform(0, 1.0, n)
    return np.stack([rr * np.cos(th), rr * np.sin(th)], 1).astype(F32)


def gaussian_source(centers, sigmas, amps, grid_res, domain_size):
    """f = sum_k a_k exp(-|x - c_k|^2 / (2 s_k^2)) on the volume-cache grid (x fastest)."""
    p = idx_to_domain_point(grid_res, domain_size, 2).astype(np.float64)
    f = np.zeros(len(p))
    for c, s, a in zip(centers, sigmas, amps):
        f += a * np.exp(-((p - c) ** 2).sum(1) / (2 * s * s))
    return f.astype(F32)


def batch_scenes(n_scenes=256, seed=0, paths=1024, path_length=8, point_range=(1000, 64000), grid_res=128):
    """Seeded batch of 2D star scenes: lobes U{3..9}, amplitude U[0.1, 0.35], segments log-uniform in
    [64, 16384]; problem types cycle through interior Neumann, exterior Neumann, interior Robin,
    exterior Robin (64 each for 256 scenes). Interior scenes carry a source f = 4 Gaussians
    (sigma U[0.05, 0.2]) on a grid_res^2 volume cache over [-1.3, 1.3]^2; their Neumann data gets the
    constant flux that makes the problem compatible (the flux of g equals the integral of f).
    Neumann: single layer, forward estimator; Robin (alpha = 1): single layer, backward estimator,
    64 resampling candidates, eps 1e-5 (the shipped configs data/config_general_2d_*_{Neumann,Robin}).
    Boundary data from e^x cos y (interior) or x/|x|^2 (exterior). Returns a list of dicts."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_scenes):
        lobes = int(rng.integers(3, 10))
        amp = float(rng.uniform(0.1, 0.35))
        n_seg = int(np.exp(rng.uniform(np.log(64), np.log(16384))))
        kind = i % 4
        exterior = kind in (1, 3)
        robin = kind in (2, 3)
        n_pts = int(rng.integers(point_range[0], point_range[1] + 1))
        verts, normals = star_polygon(n_seg, lobes, amp)
        scale = 1.0
        if exterior:
            scale = 0.5
            verts = (verts * F32(scale)).astype(F32)
            normals = segment_normals(verts)
        flat = verts.reshape(-1, 2).astype(np.float64)
        if exterior:
            r2 = (flat ** 2).sum(1)
            ug = np.stack([flat[:, 0] / r2, 1 / r2 - 2 * flat[:, 0] ** 2 / r2 ** 2, -2 * flat[:, 0] * flat[:, 1] / r2 ** 2], 1)
        else:
            ug = exp_cos(flat)
        ug = ug.reshape(n_seg, 2, 3)
        dudn = (ug[..., 1:] * normals[:, None, :].astype(np.float64)).sum(-1)
        volume = None
        if robin:
            g = ug[..., 0] + dudn
        else:
            g = dudn
        if not exterior:
            cen = _star_points_inside(rng, lobes, amp, 4, 0.5).astype(np.float64)
            sig = rng.uniform(0.05, 0.2, 4)
            a = rng.uniform(-5, 5, 4)
            f = gaussian_source(cen, sig, a, grid_res, 2.6)
            volume = (grid_res, 2.6, f)
            if not robin:
                seg_len = np.linalg.norm(verts[:, 1] - verts[:, 0], axis=1)
                integral = float(np.sum(a * 2 * np.pi * sig ** 2))
                g = g + integral / seg_len.sum()
        pts = _star_points_outside(rng, lobes, amp, scale, n_pts) if exterior else _star_points_inside(rng, lobes, amp, n_pts)
        params = dict(bie_model=0, domain=1 if exterior else 0, estimator=0 if robin else 1,
                      problem=2 if robin else 1, path_length=path_length, num_sample_paths=paths,
                      num_resampling_candidates=64 if robin else 1, num_volume_samples=0 if exterior else 1,
                      eps=float(F32(1e-5)) if robin else float(np.finfo(np.float32).eps))
        out.append(dict(verts=verts, normals=normals, bvals=g.astype(F32), types=np.full(n_seg, 2 if robin else 1, np.int32),
                        alphas=np.full((n_seg, 2), 1.0, F32) if robin else None, volume=volume, points=pts,
                        params=params, lobes=lobes, amp=amp))
    return out


# ------------------------------------------------------------------ VPL potential-flow scene
def vpl_flow_scene():
    """The scene of apps/potential_flow_with_vpl.cu:140-176: the box [-1/2, 1/2]^2 with Neumann data
    -1 / 0 / 1 / 0 on its left / top / right / bottom sides (a unit flow in +x) around four circular
    obstacles (zero flux) of 360, 180, 180 and 90 segments, normals n = (t_y, -t_x) with
    t = (v1 - v2)/|v1 - v2| (float32 like the reference). Returns verts [n, 2, 2], normals [n, 2],
    data [n, 2], types [n] (all Neumann) and the circles (center, radius, segments)."""
    verts = [[[-0.5, -0.5], [-0.5, 0.5]], [[-0.5, 0.5], [0.5, 0.5]], [[0.5, 0.5], [0.5, -0.5]],
             [[0.5, -0.5], [-0.5, -0.5]]]
    normals = [[-1.0, 0.0], [0.0, 1.0], [1.0, 0.0], [0.0, -1.0]]
    data = [[-1.0, -1.0], [0.0, 0.0], [1.0, 1.0], [0.0, 0.0]]
    circles = [((0.2, 0.1), 0.25, 360), ((-0.25, 0.3), 0.15, 180), ((-0.20, -0.25), 0.2, 180), ((0.25, -0.3), 0.05, 90)]
    verts = np.array(verts, F32)
    normals = np.array(normals, F32)
    data = np.array(data, F32)
    vs, ns = [verts], [normals]
    for (cx, cy), r, m in circles:
        c = np.array([cx, cy], F32)
        k = np.arange(m + 1, dtype=np.float64)
        ang = (2 * np.pi) * k / m
        u = np.stack([np.cos(ang), np.sin(ang)], 1).astype(F32)
        p = (c[None, :] + F32(r) * u).astype(F32)
        v = np.stack([p[:-1], p[1:]], 1)
        vs.append(v)
        ns.append(segment_normals(v))
    verts = np.concatenate(vs).astype(F32)
    normals = np.concatenate(ns).astype(F32)
    data = np.concatenate([data, np.zeros((len(verts) - 4, 2), F32)])
    return verts, normals, data, np.ones(len(verts), np.int32), circles


def vpl_flow_points(grid_res: int, circles):
    """Cell centres of the grid over [-1/2, 1/2]^2 outside the circles (apps/potential_flow_with_vpl.cu:178-185)."""
    g = idx_to_domain_point(grid_res, 1.0, 2)
    keep = np.ones(len(g), bool)
    for (cx, cy), r, _ in circles:
        d = g - np.array([cx, cy], F32)
        keep &= ~((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) < F32(r) * F32(r))
    return g, keep
