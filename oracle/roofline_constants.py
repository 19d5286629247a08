"""Measures the roofline constants N_node / N_prim (mean nodes visited and primitives tested per
infinite-line query of the reference's binary LBVH, oracle/lbvh_count.hpp) on the line queries the
walks of the 2D double-layer star workload and of the 3D exterior-Neumann control-variate workload
make. TEST INFRASTRUCTURE ONLY (runs the CPU oracle).

    python oracle/roofline_constants.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import oracle_py as O  # noqa: E402
from wobtoolbox_gb300 import EstimatorParams  # noqa: E402
from wobtoolbox_gb300 import workloads as W  # noqa: E402


def star_dl():
    sc = W.star_dirichlet_scene()
    el = O.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
    p = EstimatorParams(bie_model=1, path_length=8, num_sample_paths=16, seed=0)
    return O.lbvh_stats(el, p, sc["points"])


def exterior_neumann_3d():
    rng = np.random.default_rng(0)
    V, F, _ = W.displaced_icosphere(7, 0.15, 4, 0)
    verts, normals = W.mesh_elements(V, F)
    dirs = rng.standard_normal((3, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    src = dirs * rng.uniform(0, 0.5, (3, 1))
    q = rng.uniform(-1, 1, 3)
    uv = W.point_sources(verts.reshape(-1, 3), src, q).reshape(len(F), 3, 4)
    g = (uv[..., 1:] * normals[:, None, :].astype(np.float64)).sum(-1).astype(np.float32)
    el = O.Elements(verts, normals, g, np.ones(len(F), np.int32))
    cand = W.slice_points_z0(256, 4.0)
    pts = cand[np.linalg.norm(cand, axis=1) > 1.6][::400][:64]
    p = EstimatorParams(bie_model=0, domain=1, estimator=1, problem=1, path_length=4, num_sample_paths=8, seed=0)
    return O.lbvh_stats(el, p, pts)


if __name__ == "__main__":
    for name, fn, f, b in (("2D double-layer star, 1024 segments", star_dl, (8, 14, 30), (16, 44, 8)),
                           ("3D exterior Neumann, 327,680 triangles", exterior_neumann_3d, (18, 30, 40), (32, 76, 12))):
        q, nn, npr = fn()
        print(f"{name}: {q} queries, N_node {nn:.2f}, N_prim {npr:.2f}, "
              f"FLOP/bounce {f[0] * nn + f[1] * npr + f[2]:.0f}, bytes/bounce {b[0] * nn + b[1] * npr + b[2]:.0f}")
