"""The JSON apps end to end on the GPU: config + OBJ in, raw_data fields and rmse_list.csv out
(apps/general_2d.cu, apps/general_3d.cu), checked against the analytic solution and against the
engine's own API on the same elements and points."""
from __future__ import annotations

import os

import numpy as np
import pytest

from tests import apps_common as A
from wobtoolbox_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _rmse_rows(out):
    return np.loadtxt(os.path.join(out, "rmse_list.csv"), delimiter=",", ndmin=2)


def test_general_2d_matches_api(engine, cuda, tmp_path):
    obj = str(tmp_path / "star.obj")
    pts = A.write_star_obj(obj)
    out = str(tmp_path / "out")
    cfg = str(tmp_path / "cfg.json")
    A.write_config(cfg, obj, out, grid_res=48, num_sample_paths=512, max_iterations=3, path_length=6)
    r = A.run_app("general_2d", cfg)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = _rmse_rows(out)
    assert rows.shape == (3, 5) and np.all(rows[:, 0] == [512, 1024, 1536])
    # cells next to the boundary dominate the RMSE (the double layer's variance grows there); it
    # falls with the sample count
    assert np.all(np.isfinite(rows[:, 2:])) and rows[-1, 2] < rows[0, 2]
    n, u = A.read_field(os.path.join(out, "potential3.scalar"))
    _, ua = A.read_field(os.path.join(out, "potential_analytical.scalar"))
    inside = ~np.isnan(ua)
    assert np.array_equal(~np.isnan(u), inside)
    # the same solve through the API: elements from the same floats, data from the closed form
    segs = np.stack([pts, np.roll(pts, -1, axis=0)], axis=1).astype(np.float32)
    nrm = W.segment_normals(segs)
    sx, sy = segs[..., 0].astype(np.float64), segs[..., 1].astype(np.float64)
    bv = (np.cos(np.pi * sx) * np.sinh(np.pi * sy)).astype(np.float32)
    scene = engine.SceneHost(segs, nrm, bv, np.zeros(len(segs), np.int32))
    grid = W.idx_to_domain_point(48, 1.0, 2)[inside]
    p = engine.EstimatorParams(bie_model=1, path_length=6, num_sample_paths=1536, seed=0)
    s, _, _ = scene.solve_domain_host(p, grid)
    assert np.allclose(u[inside], s[:, 0] / 1536, rtol=1e-4, atol=1e-5)
    scene.close()


def test_general_2d_neumann_shift(engine, cuda, tmp_path):
    """Neumann: the estimate is shifted to the exact value at the grid centre
    (apps/general_2d.cu:106-121, :349-350)."""
    obj = str(tmp_path / "star.obj")
    A.write_star_obj(obj)
    out = str(tmp_path / "out")
    cfg = str(tmp_path / "cfg.json")
    A.write_config(cfg, obj, out, grid_res=32, num_sample_paths=256, max_iterations=2, bie_model="IndirectSingleLayer",
                   estimator="ForwardEstimator", problem="NeumannProblem", eps=1e-5)
    r = A.run_app("general_2d", cfg)
    assert r.returncode == 0, r.stdout + r.stderr
    _, u = A.read_field(os.path.join(out, "potential2.scalar"))
    _, ua = A.read_field(os.path.join(out, "potential_analytical.scalar"))
    ref = 32 * 16 + 16
    assert abs(u[ref] - ua[ref]) <= 1e-5 * max(1.0, abs(ua[ref]))
    assert np.all(np.isfinite(_rmse_rows(out)[:, 2:]))


def test_general_3d_matches_api(engine, cuda, tmp_path):
    obj = str(tmp_path / "sphere.obj")
    V, F = A.write_sphere_obj(obj, subdiv=3)
    out = str(tmp_path / "out")
    cfg = str(tmp_path / "cfg.json")
    A.write_config(cfg, obj, out, grid_res=24, num_sample_paths=256, max_iterations=2, bie_model="Direct",
                   problem="DirichletProblem")
    r = A.run_app("general_3d", cfg)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = _rmse_rows(out)
    assert rows.shape == (2, 6) and np.all(np.isfinite(rows[:, 2:]))
    _, u = A.read_field(os.path.join(out, "potential2.scalar"))
    _, ua = A.read_field(os.path.join(out, "potential_analytical.scalar"))
    _, g = A.read_field(os.path.join(out, "gradient2.vector3"), 3)
    inside = ~np.isnan(ua)
    assert inside.sum() > 100 and np.array_equal(~np.isnan(u), inside) and np.all(np.isfinite(g))
    # the same solve through the API on the normalised mesh (apps/general_3d.cu:204-211)
    mn, mx = V.min(0), V.max(0)
    size = mx - mn
    Vn = ((V - (mn + np.float32(0.5) * size)) * np.float32(1.0 / float(size.max()))).astype(np.float32)
    verts, nrm = W.mesh_elements(Vn, F)
    y1, y2 = verts[..., 1].astype(np.float64), verts[..., 2].astype(np.float64)
    bv = (-np.cos(np.pi * y1) * np.sinh(np.pi * y2)).astype(np.float32)
    scene = engine.SceneHost(verts, nrm, bv, np.zeros(len(F), np.int32))
    g2 = W.idx_to_domain_point(24, 1.0, 2)
    x = np.stack([np.zeros(len(g2), np.float32), g2[:, 1], g2[:, 0]], 1)[inside]
    p = engine.EstimatorParams(bie_model=2, path_length=4, num_sample_paths=512, seed=0)
    s, _, _ = scene.solve_domain_host(p, x)
    assert np.allclose(u[inside], s[:, 0] / 512, rtol=1e-3, atol=1e-4)
    assert np.allclose(g[inside], s[:, 1:] / 512, rtol=1e-3, atol=1e-3)
    scene.close()


def test_potential_flow_vpl_matches_api(engine, cuda, tmp_path):
    """apps/potential_flow_with_vpl.cu: the app's fields equal the engine API's VPL walks and
    aggregation on the same scene and points."""
    import json
    torch = cuda
    out = str(tmp_path / "out")
    cfg = str(tmp_path / "cfg.json")
    with open(cfg, "w") as f:
        json.dump({"output_dir": out, "path_length": 4, "num_sample_paths": 2000, "num_resampling_candidates": 64,
                   "grid_res": 40, "eps": 1e-4, "max_time": 1, "max_iterations": 2}, f)
    r = A.run_app("potential_flow_vpl", cfg)
    assert r.returncode == 0, r.stdout + r.stderr
    n, u = A.read_field(os.path.join(out, "potential2.scalar"))
    _, g = A.read_field(os.path.join(out, "gradient2.vector2"), 2)
    verts, nrm, data, ty, circles = W.vpl_flow_scene()
    grid, keep = W.vpl_flow_points(40, circles)
    assert n == 40 and np.array_equal(~np.isnan(u), keep)
    scene = engine.SceneHost(verts, nrm, data, ty)
    pts = torch.from_numpy(np.ascontiguousarray(grid[keep])).cuda()
    s = torch.zeros(len(pts), 3, dtype=torch.float64, device="cuda")
    vp = torch.zeros(2000, 2, dtype=torch.float32, device="cuda")
    vm = torch.zeros(2000, dtype=torch.float32, device="cuda")
    for it in range(2):
        p = engine.EstimatorParams(bie_model=0, domain=0, estimator=0, problem=1, path_length=4,
                                   num_resampling_candidates=64, eps=1e-4, seed=0, path_offset=it * 2000)
        scene.vpl_paths(p, 2000, vp, vm)
        scene.vpl_aggregate(1e-4, vp, vm, 2000, pts, len(pts), s)
    torch.cuda.synchronize()
    ref = (s / 4000).cpu().numpy().astype(np.float32)
    assert np.array_equal(u[keep], ref[:, 0]) and np.array_equal(g[keep], ref[:, 1:])
    scene.close()
