"""VPL walks and aggregation (apps/potential_flow_with_vpl.cu) against the oracle: the VPL records
bit-identical, the aggregated sums bit-identical (same FP32-per-256 / FP64 blocking)."""
from __future__ import annotations

import numpy as np
import pytest

from tests import scenes as S
from wobtoolbox_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _elems(oracle, scene):
    v, n, b, t, a = scene.stored_arrays()
    return oracle.Elements(v, n, b, t, a)


@pytest.mark.parametrize("dim", [2, 3])
def test_vpl_paths_and_aggregate_match_oracle(engine, oracle, cuda, dim):
    torch = cuda
    if dim == 2:
        verts, nrm, data, ty, circles = W.vpl_flow_scene()
        scene = engine.SceneHost(verts, nrm, data, ty)
        g, keep = W.vpl_flow_points(48, circles)
        pts = np.ascontiguousarray(g[keep][::7])
    else:
        sc = S.scene3d(1, False, subdiv=3)
        scene = engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
        pts = sc["points"]
    p = engine.EstimatorParams(bie_model=0, domain=0, estimator=0, problem=1, path_length=4,
                               num_resampling_candidates=16, eps=1e-4, seed=3, path_offset=1000)
    M = 1500
    vp = torch.zeros(M, dim, dtype=torch.float32, device="cuda")
    vm = torch.zeros(M, dtype=torch.float32, device="cuda")
    b = torch.zeros(1, dtype=torch.int64, device="cuda")
    scene.vpl_paths(p, M, vp, vm, b)
    s = torch.zeros(len(pts), dim + 1, dtype=torch.float64, device="cuda")
    scene.vpl_aggregate(1e-4, vp, vm, M, torch.from_numpy(pts).cuda(), len(pts), s)
    torch.cuda.synchronize()
    el = _elems(oracle, scene)
    op, om, ob = oracle.vpl_paths(el, p, M)
    assert np.array_equal(vp.cpu().numpy(), op) and np.array_equal(vm.cpu().numpy(), om)
    assert int(b.item()) == ob
    area = scene.info()["total_area"]
    ref = oracle.vpl_aggregate(dim, area, 1e-4, op, om, pts)
    assert np.array_equal(s.cpu().numpy(), ref)
    scene.close()


def test_vpl_rejects_other_estimators(engine, cuda):
    torch = cuda
    verts, nrm, data, ty, _ = W.vpl_flow_scene()
    scene = engine.SceneHost(verts, nrm, data, ty)
    vp = torch.zeros(8, 2, dtype=torch.float32, device="cuda")
    vm = torch.zeros(8, dtype=torch.float32, device="cuda")
    for kw in (dict(bie_model=2, problem=1), dict(estimator=1, bie_model=0, problem=1)):
        p = engine.EstimatorParams(path_length=2, **kw)
        with pytest.raises(engine.WobError):
            scene.vpl_paths(p, 8, vp, vm)
    scene.close()
