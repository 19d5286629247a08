"""The engine against the reference's own estimator (compiled from the reference tree; committed
fixtures tests/golden/reference_*.npz): per-point estimates at equal sample count, the z-score
distribution against an empirical null, and every path value at a few points
(tests/reference_stats.py). Among the cases: the 2D double-layer star complete (all 7,960
interior points), the 81,920-triangle Robin geometry with the convergent alpha = 1, and the 3D
exterior Neumann and interior mixed problems at reduced mesh size."""
from __future__ import annotations

import dataclasses

import numpy as np
import pytest

from tests import reference_cases as RC
from tests import reference_stats as RS

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", list(RC.CASES))
def test_engine_agrees_with_reference(engine, cuda, name):
    torch = cuda
    case = RC.CASES[name]()
    fix = np.load(RC.fixture_path(name))
    assert str(fix["checksum"]) == RC.scene_checksum(case), "scene generator changed: regenerate the fixture"
    scene = engine.SceneHost(case["verts"], case["normals"], case["bvals"], case["types"], case["alphas"])
    if case["volume"] is not None:
        scene.set_volume_cache(*case["volume"])
    pts = fix["points"]
    D = pts.shape[1]
    d_pts = torch.from_numpy(np.ascontiguousarray(pts)).cuda()

    def run_sums(seed):
        p = dataclasses.replace(case["params"], num_sample_paths=int(fix["n_paths"]), seed=seed)
        s = torch.zeros(len(pts), D + 1, dtype=torch.float64, device="cuda")
        q = torch.zeros_like(s)
        scene.solve_domain(p, d_pts, len(pts), s, q)
        torch.cuda.synchronize()
        assert scene.poll_error() == 0
        return s.cpu().numpy(), q.cpu().numpy()

    def run_per_path(seed):
        n_pp = fix["per_path"].shape[0]
        m = int(fix["pp_paths"])
        p = dataclasses.replace(case["params"], num_sample_paths=m, seed=seed)
        vals = torch.zeros(n_pp, m, D + 1, dtype=torch.float32, device="cuda")
        scene.debug_domain_paths(p, d_pts[:n_pp].contiguous(), n_pp, vals)
        torch.cuda.synchronize()
        return vals[:, :, 0].cpu().numpy()

    rep = RS.check_against_reference(fix, run_sums, run_per_path, name)
    print(name, rep)
    scene.close()
