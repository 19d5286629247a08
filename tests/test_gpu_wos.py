"""Walk on spheres (apps/simple_wob_and_wos.cu) on the GPU against the oracle: closest-point
queries identical to the oracle's scan, paths bit-identical."""
from __future__ import annotations

import numpy as np
import pytest

from tests import scenes as S
from wobtoolbox_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _elems(oracle, scene):
    v, n, b, t, a = scene.stored_arrays()
    return oracle.Elements(v, n, b, t, a)


def test_closest_point_matches_scan(engine, oracle, cuda):
    torch = cuda
    sc = W.star_dirichlet_scene()
    scene = engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
    rng = np.random.default_rng(1)
    x = rng.uniform(-1.4, 1.4, (5000, 2)).astype(np.float32)
    x[:50] = sc["verts"][rng.choice(len(sc["verts"]), 50), 0]  # on vertices: ties between two segments
    e = torch.zeros(len(x), dtype=torch.int32, device="cuda")
    d = torch.zeros(len(x), dtype=torch.float32, device="cuda")
    v = torch.zeros(len(x), dtype=torch.float32, device="cuda")
    scene.closest_point(torch.from_numpy(x).cuda(), len(x), e, d, v)
    torch.cuda.synchronize()
    oe, od, ov = oracle.closest_point(_elems(oracle, scene), x)
    assert np.array_equal(e.cpu().numpy().astype(np.uint32), oe)
    assert np.array_equal(d.cpu().numpy(), od) and np.array_equal(v.cpu().numpy(), ov)
    scene.close()


@pytest.mark.parametrize("which", ["star", "device_built"])
def test_wos_paths_match_oracle(engine, oracle, cuda, which):
    torch = cuda
    sc = S.scene2d(0, False, n_seg=300)
    if which == "star":
        scene = engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
    else:
        t = lambda a, dt=torch.float32: torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dt)
        scene = engine.SceneHost.build_on_device(t(sc["verts"]), t(sc["normals"]), t(sc["bvals"]),
                                                 t(sc["types"], torch.int32))
    pts = sc["points"]
    p = engine.EstimatorParams(num_sample_paths=100, eps=1e-4, seed=5, path_offset=77)
    per = torch.zeros(len(pts), 100, dtype=torch.float32, device="cuda")
    s = torch.zeros(len(pts), dtype=torch.float64, device="cuda")
    q = torch.zeros(1, dtype=torch.int64, device="cuda")
    scene.solve_wos(p, torch.from_numpy(pts).cuda(), len(pts), s, None, q, per)
    torch.cuda.synchronize()
    assert scene.poll_error() == 0
    os_, opp, oq = oracle.wos(_elems(oracle, scene), p, pts, per_path=True)
    assert np.array_equal(per.cpu().numpy(), opp)
    assert int(q.item()) == oq
    assert np.all(np.abs(s.cpu().numpy() - os_) <= 1e-12 * np.abs(opp.astype(np.float64)).sum(1) + 1e-300)
    scene.close()


def test_wos_rejects_non_dirichlet_and_3d(engine, cuda):
    torch = cuda
    sc = S.scene2d(1, False)
    scene = engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
    s = torch.zeros(len(sc["points"]), dtype=torch.float64, device="cuda")
    with pytest.raises(engine.WobError):
        scene.solve_wos(engine.EstimatorParams(num_sample_paths=4, eps=1e-4), torch.from_numpy(sc["points"]).cuda(),
                        len(sc["points"]), s)
    scene.close()
    sc3 = S.scene3d(0, False)
    scene = engine.SceneHost(sc3["verts"], sc3["normals"], sc3["bvals"], sc3["types"])
    with pytest.raises(engine.WobError):
        scene.solve_wos(engine.EstimatorParams(num_sample_paths=4, eps=1e-4), torch.from_numpy(sc3["points"]).cuda(),
                        len(sc3["points"]), s)
    scene.close()
