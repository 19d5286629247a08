"""Edge cases of the entry points: empty inputs do nothing and succeed; paths at large stream
offsets (near 2^40 and 2^63) stay bit-identical to the oracle."""
from __future__ import annotations

import numpy as np
import pytest

from tests import scenes as S

pytestmark = pytest.mark.gpu


def test_empty_inputs_are_noops(engine, cuda):
    torch = cuda
    sc = S.scene2d(0, False)
    scene = engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
    p = engine.EstimatorParams(bie_model=1, path_length=3, num_sample_paths=8)
    d = torch.zeros(1, 3, dtype=torch.float64, device="cuda")
    pts = torch.zeros(1, 2, dtype=torch.float32, device="cuda")
    scene.solve_domain(p, pts, 0, d)
    scene.solve_wos(engine.EstimatorParams(num_sample_paths=8, eps=1e-4), pts, 0, d)
    scene.vpl_aggregate(1e-4, None, None, 0, pts, 1, d)  # no VPLs: adds nothing
    scene.set_rhs(np.zeros((len(sc["verts"]), 2, 2), np.float32))
    scene.solve_domain_multi(engine.EstimatorParams(bie_model=0, path_length=2, num_sample_paths=4), pts, 0, d)
    torch.cuda.synchronize()
    assert torch.count_nonzero(d).item() == 0
    scene.close()


@pytest.mark.parametrize("offset", [(1 << 40) - 16, (1 << 63) - 64])
def test_large_path_offsets(engine, oracle, cuda, offset):
    torch = cuda
    sc = S.scene3d(0, False)
    scene = engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
    p = engine.EstimatorParams(bie_model=2, path_length=3, num_sample_paths=40, seed=(1 << 40) + 3, path_offset=offset,
                               point_offset=(1 << 31) + 5)
    pts = sc["points"][:3]
    vals = torch.zeros((3, 40, 4), dtype=torch.float32, device="cuda")
    scene.debug_domain_paths(p, torch.from_numpy(pts).cuda(), 3, vals)
    torch.cuda.synchronize()
    v, n, b, t, a = scene.stored_arrays()
    _, _, _, ref = oracle.solve_domain(oracle.Elements(v, n, b, t, a), p, pts, per_path=True)
    assert np.array_equal(vals.cpu().numpy(), ref)
    scene.close()
