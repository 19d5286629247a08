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
    # the reference's columns (samples, time, RMSE of u and of the gradient) and two more: the
    # iteration's bounces per second and the cumulative bounce count
    assert rows.shape == (3, 7) and np.all(rows[:, 0] == [512, 1024, 1536])
    assert np.all(rows[:, 5] > 0) and np.all(np.diff(rows[:, 6]) > 0)
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
    assert rows.shape == (2, 8) and np.all(np.isfinite(rows[:, 2:]))
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


def test_poisson_equation_matches_api(engine, cuda, tmp_path):
    """apps/poisson_equation.cu: the box with u = 1 and the constant source 5 through a volume cache;
    the app's fields equal the API's solve, and the centre value matches the series solution of
    Laplace(u) = 5 (the sign the estimator's volume term carries) on (-1, 1)^2."""
    import json
    out = str(tmp_path / "out")
    cfg = str(tmp_path / "cfg.json")
    with open(cfg, "w") as f:
        json.dump({"output_dir": out, "path_length": 4, "num_sample_paths": 256, "num_volume_samples": 4,
                   "grid_res": 32, "eps": 1e-4, "max_time": 1, "max_iterations": 2}, f)
    r = A.run_app("poisson_equation", cfg)
    assert r.returncode == 0, r.stdout + r.stderr
    n, u = A.read_field(os.path.join(out, "potential2.scalar"))
    _, g = A.read_field(os.path.join(out, "gradient2.vector2"), 2)
    assert n == 32 and np.all(np.isfinite(u)) and np.all(np.isfinite(g))
    sq = np.array([[[-1, -1], [-1, 1]], [[-1, 1], [1, 1]], [[1, 1], [1, -1]], [[1, -1], [-1, -1]]], np.float32)
    nrm = np.array([[-1, 0], [0, 1], [1, 0], [0, -1]], np.float32)
    scene = engine.SceneHost(sq, nrm, np.ones((4, 2), np.float32), np.zeros(4, np.int32))
    scene.set_volume_cache(32, 2.0, np.full(32 * 32, 5.0, np.float32))
    grid = W.idx_to_domain_point(32, 2.0, 2)
    p = engine.EstimatorParams(bie_model=1, path_length=4, num_sample_paths=512, num_volume_samples=4, eps=1e-4,
                               seed=0)
    s, _, _ = scene.solve_domain_host(p, grid)
    assert np.allclose(u, s[:, 0] / 512, rtol=1e-4, atol=1e-5)
    assert np.allclose(g, s[:, 1:] / 512, rtol=1e-4, atol=1e-4)
    # u(0) = 1 - 5 * 0.294685 (torsion function of the square of side 2 at its centre)
    N = 1 << 20
    p = engine.EstimatorParams(bie_model=1, path_length=4, num_sample_paths=N, num_volume_samples=16, eps=1e-4,
                               seed=1)
    s, q, _ = scene.solve_domain_host(p, np.zeros((1, 2), np.float32))
    m = s[0, 0] / N
    se = np.sqrt((q[0, 0] / N - m * m) / N)
    assert abs(m - (1.0 - 5.0 * 0.294685)) < 5 * se + 0.01, (m, se)
    scene.close()


def _circle720():
    """The 720-segment circle of apps/boundary_estimate.cu:162-180, vertices in double then float."""
    import math
    v = np.array([[0.5 * math.sin((2 * math.pi) * i / 720), 0.5 * math.cos((2 * math.pi) * i / 720)]
                  for i in range(721)]).astype(np.float32)
    segs = np.stack([v[:-1], v[1:]], axis=1)
    t = segs[:, 0] - segs[:, 1]
    ln = np.sqrt(t[:, 0] * t[:, 0] + t[:, 1] * t[:, 1])
    n_out = np.stack([t[:, 1] / ln, -(t[:, 0] / ln)], 1).astype(np.float32)
    bv = np.zeros((720, 2), np.float32)
    i = np.arange(720)
    bv[(i % 240 == 0) | (i % 240 == 239)] = [1.0, 200.0]
    bv[(i % 240 == 120) | (i % 240 == 119)] = [-1.0, -200.0]
    return segs, n_out, bv


def test_boundary_estimate_matches_api(engine, cuda, tmp_path):
    """apps/boundary_estimate.cu: interior Neumann on the circle, forward single layer; the domain
    fields and the boundary_solution file equal the API's solves on the same elements and points."""
    import json
    torch = cuda
    out = str(tmp_path / "out")
    cfg = str(tmp_path / "cfg.json")
    with open(cfg, "w") as f:
        json.dump({"output_dir": out, "path_length": 4, "num_sample_paths_domain": 128,
                   "num_sample_paths_boundary": 512, "grid_res": 32, "max_time": 1, "max_iterations": 2}, f)
    r = A.run_app("boundary_estimate", cfg)
    assert r.returncode == 0, r.stdout + r.stderr
    n, u = A.read_field(os.path.join(out, "potential2.scalar"))
    _, g = A.read_field(os.path.join(out, "gradient2.vector2"), 2)
    raw = open(os.path.join(out, "boundary_solution2.scalar"), "rb").read()
    assert int(np.frombuffer(raw[:4], np.uint32)[0]) == 720
    ub = np.frombuffer(raw[4:], np.float32)
    assert ub.size == 720 and np.all(np.isfinite(ub))
    grid = W.idx_to_domain_point(32, 1.0, 2)
    inside = np.sqrt(grid[:, 0] * grid[:, 0] + grid[:, 1] * grid[:, 1]) <= np.float32(0.5)
    assert np.array_equal(~np.isnan(u), inside) and np.all(g[~inside] == 0)
    segs, n_out, bv = _circle720()
    scene = engine.SceneHost(segs, -n_out, bv, np.ones(720, np.int32))
    eps = float(np.finfo(np.float32).eps)
    p = engine.EstimatorParams(bie_model=0, estimator=1, problem=1, path_length=4, num_sample_paths=256, eps=eps,
                               seed=0)
    s, _, _ = scene.solve_domain_host(p, grid[inside])
    assert np.allclose(u[inside], s[:, 0] / 256, rtol=1e-4, atol=1e-4)
    assert np.allclose(g[inside], s[:, 1:] / 256, rtol=1e-4, atol=1e-3)
    mid = ((segs[:, 0] + segs[:, 1]) / np.float32(2.0)).astype(np.float32)
    t = lambda a, dt=torch.float32: torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dt)
    sb = torch.zeros(720, dtype=torch.float64, device="cuda")
    p = engine.EstimatorParams(bie_model=0, estimator=1, problem=1, path_length=4, num_sample_paths=1024, eps=eps,
                               seed=0)
    scene.solve_boundary(p, t(mid), t(n_out), t(np.full(720, 0.5)), t(np.zeros(720)), t(np.ones(720), torch.int32),
                         t(np.zeros(720)), 720, sb)
    torch.cuda.synchronize()
    assert np.allclose(ub, sb.cpu().numpy() / 1024, rtol=1e-4, atol=1e-4)
    scene.close()


def _alternating_outline(pts):
    """Segments of a closed outline with the data of apps/simple_wob_and_wos.cu:201-220: -1 / 1 on
    alternate pieces of 1/40 of the length, computed in float like the app."""
    segs = np.stack([pts, np.roll(pts, -1, axis=0)], axis=1).astype(np.float32)
    d = segs[:, 0] - segs[:, 1]
    ln = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]).astype(np.float32)
    total = np.float32(0.0)
    for x in ln:
        total = np.float32(total + x)
    acc = np.float32(0.0)
    bv = np.zeros((len(segs), 2), np.float32)
    for i, x in enumerate(ln):
        sid = int(np.float32(np.float32(acc * np.float32(40.0)) / total))
        bv[i] = 1.0 if sid % 2 == 1 else -1.0
        acc = np.float32(acc + x)
    return segs, W.segment_normals(segs), bv


@pytest.mark.parametrize("is_wos", [False, True])
def test_simple_wob_and_wos_matches_api(engine, cuda, tmp_path, is_wos):
    """apps/simple_wob_and_wos.cu: the double-layer walk or walk on spheres on an outline with
    alternating data; the app's field equals the API's solve on the same elements and points."""
    torch = cuda
    obj = str(tmp_path / "star.obj")
    pts = A.write_star_obj(obj)
    out = str(tmp_path / "out")
    cfg = str(tmp_path / "cfg.json")
    A.write_config(cfg, obj, out, grid_res=32, num_sample_paths=128, max_iterations=2, is_wos=is_wos, eps=1e-4)
    r = A.run_app("simple_wob_and_wos", cfg)
    assert r.returncode == 0, r.stdout + r.stderr
    n, u = A.read_field(os.path.join(out, "potential2.scalar"))
    segs, nrm, bv = _alternating_outline(pts)
    grid = W.idx_to_domain_point(32, 1.0, 2)
    inside = W.winding_number_2d(segs, grid) < -0.5
    assert n == 32 and np.array_equal(~np.isnan(u), inside)
    assert set(np.unique(bv[:, 0])) == {-1.0, 1.0}
    scene = engine.SceneHost(segs, nrm, bv, np.zeros(len(segs), np.int32))
    if is_wos:
        p = engine.EstimatorParams(num_sample_paths=256, eps=1e-4, seed=0)
        s = torch.zeros(int(inside.sum()), dtype=torch.float64, device="cuda")
        scene.solve_wos(p, torch.from_numpy(np.ascontiguousarray(grid[inside])).cuda(), int(inside.sum()), s)
        torch.cuda.synchronize()
        ref = s.cpu().numpy() / 256
    else:
        p = engine.EstimatorParams(bie_model=1, path_length=4, num_sample_paths=256, eps=1e-4, seed=0)
        s, _, _ = scene.solve_domain_host(p, grid[inside])
        ref = s[:, 0] / 256
    assert np.allclose(u[inside], ref, rtol=1e-4, atol=1e-5)
    scene.close()


def test_general_2d_resume_is_exact(engine, cuda, tmp_path):
    """A run stopped after 2 iterations and resumed from its checkpoint to 4 writes the same
    fields, bit for bit, as a run of 4 iterations (the walks are indexed by their path offset)."""
    obj = str(tmp_path / "star.obj")
    A.write_star_obj(obj)
    full, part = str(tmp_path / "full"), str(tmp_path / "part")
    cfg_full, cfg_a, cfg_b = (str(tmp_path / f) for f in ("full.json", "a.json", "b.json"))
    A.write_config(cfg_full, obj, full, grid_res=32, num_sample_paths=256, max_iterations=4, path_length=6)
    A.write_config(cfg_a, obj, part, grid_res=32, num_sample_paths=256, max_iterations=2, path_length=6)
    A.write_config(cfg_b, obj, part, grid_res=32, num_sample_paths=256, max_iterations=4, path_length=6, resume=True)
    for c in (cfg_full, cfg_a, cfg_b):
        r = A.run_app("general_2d", c)
        assert r.returncode == 0, r.stdout + r.stderr
    assert "resuming after 2 iterations" in r.stdout
    for name in ("potential4.scalar", "gradient4.vector2"):
        a = open(os.path.join(full, name), "rb").read()
        b = open(os.path.join(part, name), "rb").read()
        assert a == b, name
    rows = _rmse_rows(part)
    assert rows.shape[0] == 4 and np.all(rows[:, 0] == [256, 512, 768, 1024])
