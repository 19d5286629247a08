"""The 2D line grid (LineGrid in csrc/scene_host.hpp) against brute force over all segments.

A host-built 2D scene answers infinite-line queries from its line grid: the line's direction bin
and offset cell list the candidate segments, each tested with the exact intersection test. The
grid must list every segment the exact test can accept, so the hits, their order and the hit
points are those of the oracle's scan of all segments in storage order. Checked on scenes with
the three bin counts, long and tiny segments, collinear and parallel segments, and on the lines
where conservative bounds are tight: directions on bin boundaries, axis directions, lines through
vertices and along segments, origins far outside the scene, and non-unit directions (which take
the BVH).
"""
from __future__ import annotations

import numpy as np
import pytest

from wobtoolbox_gb300 import workloads as W

pytestmark = pytest.mark.gpu

F32 = np.float32


def _polygon(pts):
    pts = np.asarray(pts, F32)
    segs = np.stack([pts, np.roll(pts, -1, axis=0)], axis=1).astype(F32)
    return segs


def _scene_star(n):
    verts, _ = W.star_polygon(n, 5, 0.3)
    return verts


def _scene_mixed(seed=4):
    """A random star-shaped polygon whose edges range from 1e-4 to about 1 in length."""
    rng = np.random.default_rng(seed)
    ang = np.sort(rng.uniform(0, 2 * np.pi, 400))
    ang = np.concatenate([ang, ang[:40] + 1e-4])  # near-duplicate vertices: tiny edges
    ang = np.sort(ang)
    r = rng.uniform(0.3, 1.2, len(ang))
    return _polygon(np.stack([r * np.cos(ang), r * np.sin(ang)], 1))


def _scene_comb():
    """A closed outline with 200 parallel teeth (many segments share directions and offsets)."""
    pts = [[-1.0, -0.2]]
    for i in range(200):
        x = -1.0 + 2.0 * i / 200
        pts += [[x, 0.5], [x + 0.005, 0.5], [x + 0.005, -0.1], [x + 0.01, -0.1]]
    pts += [[1.0, -0.2]]
    return _polygon(pts)


def _scene_collinear():
    """A square whose bottom edge is split into 64 collinear segments."""
    xs = np.linspace(-1, 1, 65)
    pts = [[x, -1.0] for x in xs[:-1]] + [[1.0, -1.0], [1.0, 1.0], [-1.0, 1.0]]
    return _polygon(pts)


SCENES = {
    "box": lambda: _polygon([[-1, -1], [-1, 1], [1, 1], [1, -1]]),
    "star1024": lambda: _scene_star(1024),
    "star3000": lambda: _scene_star(3000),
    "star10000": lambda: _scene_star(10000),
    "mixed": _scene_mixed,
    "comb": _scene_comb,
    "collinear": _scene_collinear,
}


def _lines(segs, seed):
    rng = np.random.default_rng(seed)
    n = 6000
    o = rng.uniform(-1.4, 1.4, (n, 2)).astype(F32)
    d = rng.standard_normal((n, 2))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(F32)
    # directions on the diamond-angle bin boundaries of every bin count (pa = 2k/K), both signs
    pa = np.concatenate([2.0 * np.arange(K) / K for K in (128, 256, 512)])
    raw = np.where(pa[:, None] <= 1, np.stack([1 - pa, pa], 1), np.stack([1 - pa, 2 - pa], 1))
    bd = (raw / np.linalg.norm(raw, axis=1, keepdims=True)).astype(F32)
    m = min(len(bd), 1500)
    d[:m] = bd[rng.permutation(len(bd))[:m]] * np.where(rng.uniform(size=(m, 1)) < 0.5, 1, -1).astype(F32)
    # axis directions, including a negative zero component
    ax = np.array([[1, 0], [0, 1], [-1, 0], [0, -1], [-1, -0.0], [1, -0.0]], F32)
    d[m:m + 300] = ax[np.arange(300) % len(ax)]
    # lines through vertices, and along segments (origin at a vertex, direction along the edge)
    k = rng.integers(0, len(segs), 600)
    o[m + 300:m + 900] = segs[k, 0]
    e = segs[k[:300], 1] - segs[k[:300], 0]
    ne = np.linalg.norm(e, axis=1, keepdims=True)
    ok = ne[:, 0] > 0
    d[m + 300:m + 600][ok] = (e[ok] / ne[ok]).astype(F32)
    # origins far outside
    o[m + 900:m + 1100] *= F32(40.0)
    # non-unit directions (the BVH answers these)
    d[m + 1100:m + 1200] *= F32(3.0)
    return o, d


@pytest.mark.parametrize("name", list(SCENES))
def test_line_grid_matches_brute_force(engine, oracle, cuda, name):
    torch = cuda
    segs = SCENES[name]()
    nrm = W.segment_normals(segs)
    bv = np.zeros((len(segs), 2), F32)
    scene = engine.SceneHost(segs, nrm, bv, np.zeros(len(segs), np.int32))
    info = scene.info()
    assert info["line_grid_bins"] >= 64 and info["line_grid_cells"] >= 64, info
    o, d = _lines(segs, 7)
    n = len(o)
    counts = torch.zeros(n, dtype=torch.int32, device="cuda")
    hits = torch.zeros(n, 64, dtype=torch.int32, device="cuda")
    hp = torch.zeros(n, 64, 2, dtype=torch.float32, device="cuda")
    scene.line_query(torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda(), n, counts, hits, hp)
    torch.cuda.synchronize()
    assert scene.poll_error() == 0
    v, nn, b, t, a = scene.stored_arrays()
    rc, rh, rp = oracle.line_query(oracle.Elements(v, nn, b, t, a), o, d)
    gc = counts.cpu().numpy().astype(np.uint32)
    bad = np.nonzero(gc != rc)[0]
    assert bad.size == 0, f"{bad.size} lines differ in count, first {bad[:5]}: {gc[bad[:5]]} vs {rc[bad[:5]]}"
    gh, gp = hits.cpu().numpy().astype(np.uint32), hp.cpu().numpy()
    for i in range(n):
        m = min(rc[i], 64)
        assert np.array_equal(gh[i, :m], rh[i, :m]), i
        assert np.array_equal(gp[i, :m], rp[i, :m]), i
    assert rc.max() >= 2
    scene.close()


def test_line_grid_walks_match_oracle(engine, oracle, cuda):
    """The 2D double-layer workload (1024 segments, line grid of 512 x 512 cells) walks exactly
    the oracle's paths."""
    torch = cuda
    sc = W.star_dirichlet_scene()
    scene = engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
    pts = np.ascontiguousarray(sc["points"][::40])
    p = engine.EstimatorParams(bie_model=1, path_length=8, num_sample_paths=64, seed=3)
    vals = torch.full((len(pts), 64, 3), float("nan"), dtype=torch.float32, device="cuda")
    scene.debug_domain_paths(p, torch.from_numpy(pts).cuda(), len(pts), vals)
    torch.cuda.synchronize()
    assert scene.poll_error() == 0
    v, nn, b, t, a = scene.stored_arrays()
    _, _, _, ref = oracle.solve_domain(oracle.Elements(v, nn, b, t, a), p, pts, per_path=True)
    got = vals.cpu().numpy()
    assert np.array_equal(got, ref, equal_nan=True)
    scene.close()
