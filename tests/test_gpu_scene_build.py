"""Scene construction on the GPU (wob_scene_create_device): a different BVH topology and storage
order than the host build, the same hit sets, and sampling tables whose walks are bit-identical to
the oracle's on the device scene's storage order."""
from __future__ import annotations

import numpy as np
import pytest

from tests import scenes as S
from wobtoolbox_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _device_scene(engine, torch, sc):
    t = lambda a, dt=torch.float32: torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dt)
    al = None if sc.get("alphas") is None else t(sc["alphas"])
    return engine.SceneHost.build_on_device(t(sc["verts"]), t(sc["normals"]), t(sc["bvals"]),
                                            t(sc["types"], torch.int32), al)


def _oracle_elems(oracle, scene):
    v, n, b, t, a = scene.stored_arrays()
    return oracle.Elements(v, n, b, t, a)


@pytest.mark.parametrize("case", [("2d", 1, 0, 0, 0), ("2d", 0, 1, 1, 1), ("3d", 2, 0, 0, 2), ("3d", 2, 0, 0, 1),
                                  ("3d", 0, 0, 0, 3), ("3d", 1, 0, 0, 0)])
def test_device_scene_walks_match_oracle(engine, oracle, cuda, case):
    torch = cuda
    d, bie, dom, est, prob = case
    sc = S.scene2d(prob, bool(dom)) if d == "2d" else S.scene3d(prob, bool(dom), subdiv=3)
    scene = _device_scene(engine, torch, sc)
    assert sorted(scene.element_order.tolist()) == list(range(len(sc["verts"])))
    info = scene.info()
    _, _, totals = oracle.scene_cdfs(_oracle_elems(oracle, scene))
    assert info["total_area"] == totals[0]
    p = engine.EstimatorParams(bie_model=bie, domain=dom, estimator=est, problem=prob, path_length=4,
                               num_sample_paths=24, seed=9, num_resampling_candidates=4 if bie == 0 else 1,
                               eps=1e-5 if bie == 0 else float(np.finfo(np.float32).eps),
                               first_kind_equation_scaling_constant=2.0 if prob == 3 else 1.0)
    pts = sc["points"]
    D = pts.shape[1]
    vals = torch.zeros((len(pts), p.num_sample_paths, D + 1), dtype=torch.float32, device="cuda")
    scene.debug_domain_paths(p, torch.from_numpy(pts).cuda(), len(pts), vals)
    torch.cuda.synchronize()
    assert scene.poll_error() == 0
    _, _, _, ref = oracle.solve_domain(_oracle_elems(oracle, scene), p, pts, per_path=True)
    got = vals.cpu().numpy()
    same = (got == ref) | (np.isnan(got) & np.isnan(ref))
    assert same.all(), f"{(~same).sum()} differ"
    scene.close()


@pytest.mark.parametrize("dim", [2, 3])
def test_device_scene_hit_sets_equal_host_scene(engine, cuda, dim):
    torch = cuda
    if dim == 2:
        verts, nrm = W.star_polygon(3000, 7, 0.3)
    else:
        V, F, _ = W.displaced_icosphere(5, 0.15, 4, 1)
        verts, nrm = W.mesh_elements(V, F)
    n = len(verts)
    bv = np.ones((n, dim), np.float32)
    ty = np.zeros(n, np.int32)
    host = engine.SceneHost(verts, nrm, bv, ty)
    dev = _device_scene(engine, torch, dict(verts=verts, normals=nrm, bvals=bv, types=ty))
    assert dev.info()["n_elems"] == n
    rng = np.random.default_rng(dim)
    R = 4096
    o = rng.uniform(-1.2, 1.2, (R, dim)).astype(np.float32)
    dr = rng.standard_normal((R, dim)).astype(np.float32)
    dr /= np.linalg.norm(dr, axis=1, keepdims=True)
    res = []
    for sc in (host, dev):
        c = torch.zeros(R, dtype=torch.int32, device="cuda")
        h = torch.zeros(R, 64, dtype=torch.int32, device="cuda")
        sc.line_query(torch.from_numpy(o).cuda(), torch.from_numpy(dr).cuda(), R, c, h)
        torch.cuda.synchronize()
        res.append((c.cpu().numpy(), h.cpu().numpy(), sc.element_order))
    (ch, hh, oh), (cd, hd, od) = res
    assert np.array_equal(ch, cd) and ch.max() > 2
    for r in range(R):
        m = min(int(ch[r]), 64)
        assert sorted(oh[hh[r, :m]].tolist()) == sorted(od[hd[r, :m]].tolist())
        assert np.all(np.diff(hd[r, :m]) > 0)  # storage order
    host.close()
    dev.close()


def test_device_scene_small_and_degenerate(engine, oracle, cuda):
    """One element, three elements (a single leaf) and many coincident elements (equal Morton
    codes: the radix tree falls back on the caller index)."""
    torch = cuda
    tri = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]]], np.float32)
    for k in (1, 3):
        verts = np.repeat(tri, k, axis=0) + np.arange(k, dtype=np.float32)[:, None, None] * np.float32(0.1)
        nrm = np.tile(np.array([[0, 0, 1]], np.float32), (k, 1))
        sc = dict(verts=verts, normals=nrm, bvals=np.ones((k, 3), np.float32), types=np.zeros(k, np.int32))
        scene = _device_scene(engine, torch, sc)
        assert scene.info()["n_nodes"] == 1
        scene.close()
    V, F, _ = W.displaced_icosphere(2, 0.1, 4, 0)
    verts, nrm = W.mesh_elements(V, F)
    verts = np.concatenate([verts, np.repeat(verts[:1], 40, axis=0)])
    nrm = np.concatenate([nrm, np.repeat(nrm[:1], 40, axis=0)])
    n = len(verts)
    sc = dict(verts=verts, normals=nrm, bvals=np.ones((n, 3), np.float32), types=np.zeros(n, np.int32),
              points=np.array([[0.1, 0.2, 0.0], [-0.3, 0.1, 0.2]], np.float32))
    scene = _device_scene(engine, torch, sc)
    p = engine.EstimatorParams(bie_model=2, problem=0, path_length=3, num_sample_paths=16, seed=1)
    vals = torch.zeros((2, 16, 4), dtype=torch.float32, device="cuda")
    scene.debug_domain_paths(p, torch.from_numpy(sc["points"]).cuda(), 2, vals)
    torch.cuda.synchronize()
    _, _, _, ref = oracle.solve_domain(_oracle_elems(oracle, scene), p, sc["points"], per_path=True)
    assert np.array_equal(vals.cpu().numpy(), ref)
    scene.close()


def test_device_scene_invalid_input(engine, cuda):
    torch = cuda
    sc = S.scene2d(0, False)
    bad = dict(sc)
    bad["verts"] = sc["verts"].copy()
    bad["verts"][3, 0, 0] = np.nan
    with pytest.raises(engine.WobError):
        _device_scene(engine, torch, bad)
    bad = dict(sc)
    bad["types"] = sc["types"].copy()
    bad["types"][0] = 7
    with pytest.raises(engine.WobError):
        _device_scene(engine, torch, bad)
