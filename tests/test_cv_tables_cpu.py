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
