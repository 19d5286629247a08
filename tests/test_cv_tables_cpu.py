"""The float64 restatement of the control-variate tables (oracle/cv_tables.py), which the GPU
tables are checked against: the closed-form potential of a uniformly charged triangle and its
gradient against fine quadrature, at points above, beside, in the plane of and near the triangle."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import cv_tables as T


@pytest.mark.parametrize("x", [(0.3, 0.3, 0.5), (0.3, 0.3, -0.2), (2.0, 1.0, 0.3), (-0.5, 0.2, 0.01),
                               (0.4, 0.2, 0.02), (1.5, -0.3, 0.0)])
def test_closed_form_matches_quadrature(x):
    a, b, c = np.array([0.0, 0, 0]), np.array([1.0, 0.1, 0]), np.array([0.2, 0.9, 0.05])
    x = np.array(x)
    P, G = T.triangle_potential(x[None], a[None], b[None], c[None])
    Pq, Gq = T.quadrature_potential(x, a, b, c, levels=7)
    assert abs(P[0] - Pq) < 2e-4 * abs(Pq)
    assert np.linalg.norm(G[0] - Gq) < 5e-4 * np.linalg.norm(Gq)


def test_split_tends_to_closed_form():
    """The near/far split's error falls as the near radius grows (second-order centroid rule)."""
    from wobtoolbox_gb300 import workloads as W
    V, F, _ = W.displaced_icosphere(2, 0.15, 4, 0)
    verts, normals = W.mesh_elements(V, F)
    cen = verts.astype(np.float64).mean(1)
    sig = 0.05 + 0.02 * np.sin(3 * cen[:, 0])
    exact = T.residual_data(verts, normals, sig, -2.0, 1e9)
    errs = [np.abs(T.residual_data(verts, normals, sig, -2.0, k) - exact).max() for k in (1.0, 2.0, 4.0)]
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < 2e-2 * np.abs(exact).max()


def _median_order(cen, ids=None):
    """Storage order of a median-split hierarchy (spatially compact runs, as the BVH's leaf order)."""
    if ids is None:
        ids = np.arange(len(cen))
    if len(ids) <= 4:
        return list(ids)
    c = cen[ids]
    ax = int(np.argmax(c.max(0) - c.min(0)))
    o = np.argsort(c[:, ax], kind="stable")
    mid = len(ids) // 2
    return _median_order(cen, ids[o[:mid]]) + _median_order(cen, ids[o[mid:]])


def test_cluster_expansion_close_to_pairwise():
    """theta = 0.3: clusters of 32 and groups of 256 and 2048 triangles taken by their quadrupole
    expansion change the residual data and the potential by well under the pairwise split's own
    error; theta = 0 is the pairwise sum."""
    from wobtoolbox_gb300 import workloads as W
    V, F, _ = W.displaced_icosphere(4, 0.15, 4, 0)
    verts, normals = W.mesh_elements(V, F)
    cen = verts.astype(np.float64).mean(1)
    order = np.array(_median_order(cen))
    v, n = verts[order], normals[order]
    c = v.astype(np.float64).mean(1)
    sig = 0.05 + 0.02 * np.sin(3 * c[:, 0]) * np.cos(2 * c[:, 1]) + 0.01 * c[:, 2]
    ref = T.residual_data(v, n, sig, -2.0, 3.0)
    assert np.array_equal(T.residual_data(v, n, sig, -2.0, 3.0, theta=0.0), ref)
    got = T.residual_data(v, n, sig, -2.0, 3.0, theta=0.3)
    assert np.abs(got - ref).max() < 2e-4 * np.abs(ref).max(), np.abs(got - ref).max() / np.abs(ref).max()
    assert not np.array_equal(got, ref)  # clusters were taken
    rng = np.random.default_rng(0)
    d = rng.standard_normal((64, 3))
    pts = d / np.linalg.norm(d, axis=1, keepdims=True) * rng.uniform(1.5, 3.0, (64, 1))
    pr = T.potential(v, sig, pts, 3.0)
    pg = T.potential(v, sig, pts, 3.0, theta=0.3)
    scale = np.abs(pr).max(0)
    assert np.all(np.abs(pg - pr) <= 2e-4 * scale), (np.abs(pg - pr) / scale).max()


def test_treecode_counts_every_source_once():
    """The three-level decisions partition the sources for every target: each source lies in
    exactly one record taken by its expansion or is summed pair by pair (no record taken together
    with an ancestor, none left out). Targets in compact tiles of 32, as the engine takes them:
    the 5,120 centroids of the surface in storage order, a small ball of points just off the
    surface and one far away; several theta."""
    from wobtoolbox_gb300 import workloads as W
    V, F, _ = W.displaced_icosphere(4, 0.15, 4, 0)
    verts, _ = W.mesh_elements(V, F)
    verts = verts[np.array(_median_order(verts.astype(np.float64).mean(1)))]  # spatially compact order
    cen = verts.astype(np.float64).mean(1)
    h2 = np.max(np.stack([((verts[:, 1] - verts[:, 0]) ** 2).sum(1), ((verts[:, 2] - verts[:, 1]) ** 2).sum(1),
                          ((verts[:, 0] - verts[:, 2]) ** 2).sum(1)], 1), 1).astype(np.float64)
    rng = np.random.default_rng(7)
    ball = rng.uniform(-0.05, 0.05, (64, 3))
    tx = np.concatenate([cen, ball + [1.4, 0.0, 0.0], ball + [6.0, 0.0, 0.0]])
    for theta in (0.1, 0.3, 0.6):
        _, _, pair, cover = T._cluster_split(tx, cen, np.ones(len(cen)), 9.0 * h2, theta, return_cover=True)
        assert np.array_equal(cover + pair.sum(1), np.full(len(tx), len(cen))), theta
        assert cover[:len(cen)].max() > 0 and cover[-64:].min() > 2048, (theta, cover.max())
