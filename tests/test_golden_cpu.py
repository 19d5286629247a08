"""The oracle against its committed golden outputs (tests/golden/oracle_walks.npz, written by
tests/golden/make_golden.py from seeded inputs stored in the same file): per-path values of a 2D
double-layer walk, a 3D Robin direct-BIE walk, a 2D forward single-layer Neumann walk, a 3D mixed
single-layer walk with resampling, a 3D boundary estimate and walk on spheres, and the hit sets of
200 lines. Bit-exact, so any change to the oracle's arithmetic or random streams is caught here,
on the CPU, while the GPU tests tie the engine to the oracle path for path."""
from __future__ import annotations

import ast
import os

import numpy as np
import pytest

from wobtoolbox_gb300 import EstimatorParams

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_walks.npz")
CASES = ["dl2d", "robin3d", "slfwd2d", "ris3d", "boundary3d", "wos2d"]


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def _same(a, b):
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


@pytest.mark.parametrize("name", CASES)
def test_oracle_walks_match_golden(oracle, golden, name):
    g = {k.split("/", 1)[1]: golden[k] for k in golden.files if k.startswith(name + "/")}
    params = EstimatorParams(**ast.literal_eval(str(g["params"])))
    kind = str(g["kind"])
    el = oracle.Elements(g["verts"], g["normals"], g["bvals"], g["types"], g["alphas"])
    if kind == "domain":
        got = oracle.solve_domain(el, params, g["points"], per_path=True)[3]
    elif kind == "boundary":
        got = oracle.solve_boundary(el, params, g["bp_p"], g["bp_n"], g["bp_angle"], g["bp_bv"], g["bp_type"],
                                    g["bp_alpha"], per_path=True)[3]
    else:
        got = oracle.wos(el, params, g["points"], per_path=True)[1]
    assert _same(got, g["per_path"]), f"{name}: {np.nanmax(np.abs(got - g['per_path']))}"
    assert np.isfinite(g["per_path"]).any()


def test_line_hits_match_golden(oracle, golden):
    g = {k.split("/", 1)[1]: golden[k] for k in golden.files if k.startswith("lines/")}
    el = oracle.Elements(g["verts"], g["normals"], g["bvals"], g["types"])
    c, h, hp = oracle.line_query(el, g["origins"], g["dirs"])
    assert np.array_equal(c, g["counts"]) and c.max() >= 2
    for i in range(len(c)):
        m = min(int(c[i]), h.shape[1])
        assert np.array_equal(h[i, :m], g["hits"][i, :m]) and np.array_equal(hp[i, :m], g["hit_points"][i, :m])
