"""The JSON apps (general_2d / general_3d) up to the solve, on the CPU: config parsing, OBJ
reading, normalisation, the winding-number mask and the analytical raw_data fields
(apps/general_2d.cu:160-292, apps/general_3d.cu:164-309)."""
from __future__ import annotations

import os

import numpy as np
import pytest

from tests import apps_common as A
from wobtoolbox_gb300 import workloads as W


def test_general_2d_setup(tmp_path):
    obj = str(tmp_path / "star.obj")
    pts = A.write_star_obj(obj)
    out = str(tmp_path / "out")
    cfg = str(tmp_path / "cfg.json")
    A.write_config(cfg, obj, out, grid_res=48)
    r = A.run_app("general_2d", cfg, "--setup-only")
    assert r.returncode == 0, r.stderr
    assert "IndirectDoubleLayer" in r.stdout and "( #faces: 200 )" in r.stdout
    n, u = A.read_field(os.path.join(out, "potential_analytical.scalar"))
    _, g = A.read_field(os.path.join(out, "gradient_analytical.vector2"), 2)
    assert n == 48 and os.path.exists(os.path.join(out, "config.json"))
    grid = W.idx_to_domain_point(48, 1.0, 2)
    segs = np.stack([pts, np.roll(pts, -1, axis=0)], axis=1)
    inside = W.winding_number_2d(segs, grid) < -0.5
    assert np.array_equal(~np.isnan(u), inside)
    x, y = grid[inside, 0].astype(np.float64), grid[inside, 1].astype(np.float64)
    assert np.allclose(u[inside], np.cos(np.pi * x) * np.sinh(np.pi * y), rtol=1e-5, atol=1e-6)
    assert np.allclose(g[inside, 1], np.pi * np.cos(np.pi * x) * np.cosh(np.pi * y), rtol=1e-5, atol=1e-6)
    assert np.all(g[~inside] == 0)


def test_general_2d_exterior_transform(tmp_path):
    """Exterior: the boundary is halved and moved up by 1/16 (apps/general_2d.cu:204-207); points
    outside are evaluated against x / |x|^2."""
    obj = str(tmp_path / "star.obj")
    pts = A.write_star_obj(obj)
    out = str(tmp_path / "out")
    cfg = str(tmp_path / "cfg.json")
    A.write_config(cfg, obj, out, grid_res=40, domain="ExteriorDomain")
    assert A.run_app("general_2d", cfg, "--setup-only").returncode == 0
    _, u = A.read_field(os.path.join(out, "potential_analytical.scalar"))
    p2 = (pts * np.float32(0.5)).astype(np.float32)
    p2[:, 1] += np.float32(0.0625)
    grid = W.idx_to_domain_point(40, 1.0, 2)
    segs = np.stack([p2, np.roll(p2, -1, axis=0)], axis=1)
    outside = W.winding_number_2d(segs, grid) >= -0.5
    assert np.array_equal(~np.isnan(u), outside)
    x, y = grid[outside, 0].astype(np.float64), grid[outside, 1].astype(np.float64)
    assert np.allclose(u[outside], x / (x * x + y * y), rtol=1e-5)


def test_general_3d_setup(tmp_path):
    """3D: the mesh is normalised into [-1/2, 1/2]^3, the slice x = 0 is evaluated inside
    (winding number > 1/2)."""
    obj = str(tmp_path / "sphere.obj")
    V, F = A.write_sphere_obj(obj)
    out = str(tmp_path / "out")
    cfg = str(tmp_path / "cfg.json")
    A.write_config(cfg, obj, out, grid_res=24, bie_model="Direct", problem="MixedProblem", seed=3)
    r = A.run_app("general_3d", cfg, "--setup-only")
    assert r.returncode == 0, r.stderr
    n, u = A.read_field(os.path.join(out, "potential_analytical.scalar"))
    _, g = A.read_field(os.path.join(out, "gradient_analytical.vector3"), 3)
    mn, mx = V.min(0), V.max(0)
    size = mx - mn
    Vn = (V - (mn + np.float32(0.5) * size)) * np.float32(1.0 / float(size.max()))
    g2 = W.idx_to_domain_point(24, 1.0, 2)
    x = np.stack([np.zeros(len(g2), np.float32), g2[:, 1], g2[:, 0]], 1)
    inside = A.winding_3d(Vn[F], x) > 0.5
    assert np.array_equal(~np.isnan(u), inside)
    y1, y2 = x[inside, 1].astype(np.float64), x[inside, 2].astype(np.float64)
    assert np.allclose(u[inside], -np.cos(np.pi * y1) * np.sinh(np.pi * y2), rtol=1e-5, atol=1e-6)
    assert np.all(g[inside, 0] == 0)


def test_bad_config_reports_error(tmp_path):
    cfg = str(tmp_path / "cfg.json")
    with open(cfg, "w") as f:
        f.write('{"input_obj_file": "x.obj", "output_dir": "o", "bie_model": "IndirectDoubleLayer"}')
    r = A.run_app("general_2d", cfg, "--setup-only")
    assert r.returncode == 1 and "missing key" in r.stderr
    with open(cfg, "w") as f:
        f.write('{"input_obj_file": "x.obj", ')
    r = A.run_app("general_2d", cfg, "--setup-only")
    assert r.returncode == 1 and "JSON" in r.stderr


@pytest.mark.parametrize("all_points", [False, True])
def test_simple_wob_and_wos_setup(tmp_path, all_points):
    """apps/simple_wob_and_wos.cu up to the solve: the OBJ outline, the winding-number mask (or every
    grid point with evaluate_at_all_points) and the printed configuration."""
    obj = str(tmp_path / "star.obj")
    pts = A.write_star_obj(obj)
    out = str(tmp_path / "out")
    cfg = str(tmp_path / "cfg.json")
    A.write_config(cfg, obj, out, grid_res=40, is_wos=True, evaluate_at_all_points=all_points, eps=1e-4)
    r = A.run_app("simple_wob_and_wos", cfg, "--setup-only")
    assert r.returncode == 0, r.stderr
    assert "( #line segments: 200 )" in r.stdout and "is WoS\t: 1" in r.stdout
    assert "path length" not in r.stdout  # not used by walk on spheres
    segs = np.stack([pts, np.roll(pts, -1, axis=0)], axis=1)
    grid = W.idx_to_domain_point(40, 1.0, 2)
    m = 1600 if all_points else int((W.winding_number_2d(segs, grid) < -0.5).sum())
    assert f"evaluation points\t: {m}\n" in r.stdout
    assert os.path.exists(os.path.join(out, "config.json"))


def test_new_apps_reject_bad_configs(tmp_path):
    cfg = str(tmp_path / "cfg.json")
    with open(cfg, "w") as f:
        f.write('{"input_obj_file": "x.obj", "output_dir": "o", "is_wos": 1}')
    r = A.run_app("simple_wob_and_wos", cfg, "--setup-only")
    assert r.returncode == 1 and "true or false" in r.stderr
    with open(cfg, "w") as f:
        f.write('{"output_dir": "o", "path_length": 4}')
    for app in ("poisson_equation", "boundary_estimate"):
        r = A.run_app(app, cfg)
        assert r.returncode == 1 and "missing key" in r.stderr
