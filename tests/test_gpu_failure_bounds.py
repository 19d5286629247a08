"""The device-side failure bounds, made to run out without any fault.

- Walk on spheres stops a walk after 4096 jumps (the reference's loop has no bound); lowering the
  bound with wob_scene_set_step_limits makes the walks reach it: the kernel returns, the estimates
  stay finite and the scene's error word carries the step-limit bit.
- BVH traversals stop after a step bound (5 x nodes + 16 by default); lowering it with
  wob_scene_set_step_limits makes the line queries of a forward walk run out: the solve
  returns, the error word carries the traversal bit, the host-buffer entry point returns
  WOB_ERR_DEVICE_LIMIT, and restoring the default gives the unbounded results again.
- Elements of zero area inside a valid scene carry no sampling weight and meet no line: walks on
  such scenes stay finite and bit-identical to the oracle.
- The fused training step's waits on its tensor-core products are bounded: with
  wob_mlp_inject_wait_timeout every block waits on an mbarrier nothing arrives on, the wait runs
  out, the blocks drain and release their tensor memory, the update is skipped (the parameters
  keep their values) and wob_mlp_train returns WOB_ERR_DEVICE_LIMIT; with the injection off the
  same network trains normally afterwards.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from tests import scenes as S

pytestmark = pytest.mark.gpu

ERR_TRAVERSAL_LIMIT = 2
ERR_WOS_STEP_LIMIT = 4
WOB_ERR_DEVICE_LIMIT = 5


def test_wos_step_limit_is_reported(engine, cuda):
    torch = cuda
    sc = S.scene2d(0, False)
    scene = engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
    pts = sc["points"][:4]
    s = torch.zeros(len(pts), dtype=torch.float64, device="cuda")
    q = torch.zeros(1, dtype=torch.int64, device="cuda")
    p = engine.EstimatorParams(num_sample_paths=8, eps=1e-6, seed=3)
    engine.check(engine.load().wob_scene_set_step_limits(scene.handle, 0, 3))
    scene.solve_wos(p, torch.from_numpy(pts).cuda(), len(pts), s, None, q)
    torch.cuda.synchronize()
    assert scene.poll_error() & ERR_WOS_STEP_LIMIT
    assert np.all(np.isfinite(s.cpu().numpy()))
    assert int(q.item()) <= len(pts) * 8 * 3
    assert scene.poll_error() == 0  # polling clears the word
    with pytest.raises(engine.WobError):
        engine.check(engine.load().wob_scene_set_step_limits(scene.handle, 0, 5000))
    engine.check(engine.load().wob_scene_set_step_limits(scene.handle, 0, 0))
    s.zero_()
    scene.solve_wos(p, torch.from_numpy(pts).cuda(), len(pts), s, None, q)
    torch.cuda.synchronize()
    assert scene.poll_error() == 0
    scene.close()


def test_traversal_limit_is_reported_and_reset(engine, cuda):
    torch = cuda
    lib = engine.load()
    sc = S.scene3d(1, True, subdiv=3)
    scene = engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
    pts = sc["points"]
    p = engine.EstimatorParams(bie_model=0, domain=1, estimator=1, problem=1, path_length=4, num_sample_paths=64,
                               seed=5)
    d = torch.from_numpy(pts).cuda()
    ref = torch.zeros(len(pts), 4, dtype=torch.float64, device="cuda")
    scene.solve_domain(p, d, len(pts), ref)
    torch.cuda.synchronize()
    assert scene.poll_error() == 0
    engine.check(lib.wob_scene_set_step_limits(scene.handle, 2, 0))
    s = torch.zeros_like(ref)
    scene.solve_domain(p, d, len(pts), s)
    torch.cuda.synchronize()
    assert scene.poll_error() & ERR_TRAVERSAL_LIMIT
    assert np.all(np.isfinite(s.cpu().numpy()))
    h_s = np.zeros((len(pts), 4))
    b = C.c_uint64(0)
    cp = p.to_c()
    st = lib.wob_solve_domain_host(scene.handle, C.byref(cp), np.ascontiguousarray(pts).ctypes.data, len(pts),
                                   h_s.ctypes.data, None, C.byref(b))
    assert st == WOB_ERR_DEVICE_LIMIT and "bound" in lib.wob_last_error().decode()
    scene.poll_error()
    engine.check(lib.wob_scene_set_step_limits(scene.handle, 0, 0))
    s2 = torch.zeros_like(ref)
    scene.solve_domain(p, d, len(pts), s2)
    torch.cuda.synchronize()
    assert scene.poll_error() == 0
    assert np.allclose(s2.cpu().numpy(), ref.cpu().numpy(), rtol=1e-12, atol=1e-300)
    scene.close()


@pytest.mark.parametrize("dim", [2, 3])
def test_zero_area_elements_walk_finite(engine, oracle, cuda, dim):
    torch = cuda
    if dim == 2:
        sc = S.scene2d(0, False)
        v, n, g, t = sc["verts"], sc["normals"], sc["bvals"], sc["types"]
        extra_v = np.repeat(v[:3, :1, :], 2, axis=1)  # three segments of zero length at vertices
        params = engine.EstimatorParams(bie_model=1, path_length=6, num_sample_paths=64, seed=8)
    else:
        sc = S.scene3d(2, False)
        v, n, g, t = sc["verts"], sc["normals"], sc["bvals"], sc["types"]
        extra_v = np.repeat(v[:3, :1, :], 3, axis=1)  # three triangles collapsed to a point
        params = engine.EstimatorParams(bie_model=2, problem=2, path_length=6, num_sample_paths=64, seed=8)
    verts = np.concatenate([v, extra_v]).astype(np.float32)
    normals = np.concatenate([n, n[:3]]).astype(np.float32)
    bvals = np.concatenate([g, g[:3]]).astype(np.float32)
    types = np.concatenate([t, t[:3]]).astype(np.int32)
    alphas = None if sc["alphas"] is None else np.concatenate([sc["alphas"], sc["alphas"][:3]]).astype(np.float32)
    scene = engine.SceneHost(verts, normals, bvals, types, alphas)
    pts = sc["points"]
    vals = torch.zeros(len(pts), 64, dim + 1, device="cuda")
    scene.debug_domain_paths(params, torch.from_numpy(pts).cuda(), len(pts), vals)
    torch.cuda.synchronize()
    assert scene.poll_error() == 0
    got = vals.cpu().numpy()
    assert np.all(np.isfinite(got))
    sv, sn, sb, st, sa = scene.stored_arrays()
    _, _, _, ref = oracle.solve_domain(oracle.Elements(sv, sn, sb, st, sa), params, pts, per_path=True)
    assert np.array_equal(got, ref)
    scene.close()


def test_training_wait_timeout_is_reported(engine, cuda):
    from wobtoolbox_gb300 import cv
    torch = cuda
    lib = engine.load()
    rng = np.random.default_rng(5)
    n = 4096
    x = rng.uniform(-1, 1, (n, 6)).astype(np.float32)
    t = (np.sin(2 * x[:, 0]) + 0.3 * x[:, 1]).astype(np.float32)
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    mlp = cv.MLP(32, 4, 1, 0.5, seed=1)
    p0 = mlp.params()[0].copy()
    engine.check(lib.wob_mlp_inject_wait_timeout(mlp._h, 1000))
    hist = torch.zeros(5, device="cuda")
    with pytest.raises(engine.WobError) as err:
        mlp.train(dx, dt, n, 5, 1024, 1e-3, seed=3, loss_history=hist)
    assert err.value.status == WOB_ERR_DEVICE_LIMIT and "product" in str(err.value), str(err.value)
    torch.cuda.synchronize()
    assert np.array_equal(mlp.params()[0], p0)  # no update from a step with a missing gradient
    assert not hist.any()
    engine.check(lib.wob_mlp_inject_wait_timeout(mlp._h, 0))
    hist = torch.zeros(50, device="cuda")
    mlp.train(dx, dt, n, 50, 1024, 3e-3, seed=3, loss_history=hist)
    torch.cuda.synchronize()
    h = hist.cpu().numpy()
    assert np.all(h > 0) and h[-5:].mean() < h[:5].mean(), h
    assert not np.array_equal(mlp.params()[0], p0)
    mlp.close()
