"""The residual control variate and the fused training step on the GPU.

- the label clip (wob_clip_magnitude_quantile) against numpy's order statistic, on heavy-tailed
  values with ties, zeros and a quantile of 1;
- the fused training step's gradient (wob_mlp_gradient_fused) against torch float64 autograd and
  against the unfused kernels, for a scalar and a 64-wide head, with a batch that is not a
  multiple of the 64-row tile; device training (wob_mlp_train) is deterministic and lowers the loss;
- the control-variate tables (wob_cv_residual_data, wob_cv_potential) against their float64
  restatement (oracle/cv_tables.py, the same near/far split) and, for the potential, against the
  closed form at every pair;
- the residual scene (wob_scene_clone + wob_scene_add_boundary_offsets, offsets from the device
  or the host) walks bit-identically to the oracle on its stored arrays, leaves its source as it
  was, and outlives it (the shared device buffers are reference counted);
- end to end on the exterior Neumann problem: the trained control variate lowers the per-path
  variance of the forward estimator by more than 5x, and its estimate agrees with the plain
  estimator's.
"""
from __future__ import annotations

import dataclasses

import numpy as np
import pytest

from tests import reference_cases as RC

pytestmark = pytest.mark.gpu


def _torch_grad(params, freqs, x, t, out_dim):
    import torch
    p = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    X = torch.tensor(x, dtype=torch.float64)
    tt = X @ torch.tensor(freqs, dtype=torch.float64).T
    h = torch.cat([torch.sin(2 * np.pi * tt), torch.cos(2 * np.pi * tt)], 1)
    off = 0
    for l in range(5):
        fo = out_dim if l == 4 else 64
        W = p[off:off + fo * 64].reshape(fo, 64)
        off += fo * 64
        b = p[off:off + fo]
        off += fo
        z = h @ W.T + b
        h = z if l == 4 else z * torch.sigmoid(z)
    loss = ((h - torch.tensor(t, dtype=torch.float64).reshape(h.shape)) ** 2).mean()
    loss.backward()
    return p.grad.numpy(), float(loss.item())


@pytest.mark.parametrize("out_dim", [1, 64])
def test_fused_gradient_matches_autograd(engine, cuda, out_dim):
    from wobtoolbox_gb300 import cv
    torch = cuda
    mlp = cv.MLP(32, 4, out_dim, 1.0, seed=5)
    p, f = mlp.params()
    rng = np.random.default_rng(1)
    n = 1000  # 15 full tiles of 64 rows and one partial tile
    x = rng.uniform(-1, 1, (n, 6)).astype(np.float32)
    t = (rng.standard_normal((n, out_dim)) * 0.3).astype(np.float32)
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    g = torch.zeros(mlp.n_params, device="cuda")
    loss = torch.zeros(1, device="cuda")
    engine.check(engine.load().wob_mlp_gradient_fused(mlp._h, dx.data_ptr(), dt.data_ptr(), n, g.data_ptr(),
                                                     loss.data_ptr(), None))
    g2 = torch.zeros_like(g)
    l2 = torch.zeros_like(loss)
    mlp.gradient(dx, dt, n, g2, l2)
    torch.cuda.synchronize()
    ref_g, ref_l = _torch_grad(p, f, x, t, out_dim)
    gg = g.cpu().numpy()
    rel = np.linalg.norm(gg - ref_g) / np.linalg.norm(ref_g)
    cos = float(gg @ ref_g / (np.linalg.norm(gg) * np.linalg.norm(ref_g)))
    assert rel < 5e-2 and cos > 0.998, (rel, cos)
    rel2 = np.linalg.norm(gg - g2.cpu().numpy()) / np.linalg.norm(ref_g)
    assert rel2 < 5e-2, rel2
    assert abs(float(loss.item()) - ref_l) < 2e-2 * ref_l
    mlp.close()


def test_device_training_is_deterministic_and_learns(engine, cuda):
    from wobtoolbox_gb300 import cv
    torch = cuda
    rng = np.random.default_rng(2)
    n = 20000
    x = rng.uniform(-1, 1, (n, 6)).astype(np.float32)
    t = (np.sin(2 * x[:, 0]) * np.cos(x[:, 1]) + 0.3 * x[:, 2]).astype(np.float32)
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    params = []
    for _ in range(2):
        mlp = cv.MLP(32, 4, 1, 0.5, seed=1)
        hist = torch.zeros(400, device="cuda")
        mlp.train(dx, dt, n, 400, 4096, 3e-3, seed=7, loss_history=hist)
        torch.cuda.synchronize()
        h = hist.cpu().numpy()
        assert np.all(np.isfinite(h))
        # the update's last block advances the step counter: every step wrote its own loss slot
        assert np.all(h > 0), np.flatnonzero(h <= 0)[:10]
        assert h[-20:].mean() < 0.5 * h[:5].mean(), (h[:5], h[-20:])
        params.append(mlp.params()[0])
        mlp.close()
    assert np.array_equal(params[0], params[1])


@pytest.mark.parametrize("n,q", [(1, 0.5), (1000, 0.999), (65536, 0.999), (100003, 0.9), (5000, 1.0)])
def test_clip_magnitude_quantile_matches_numpy(engine, cuda, n, q):
    torch = cuda
    rng = np.random.default_rng(n)
    v = (rng.standard_t(1.5, n) * 0.1).astype(np.float32)
    v[: n // 10] = np.round(v[: n // 10], 2)  # ties
    v[n // 10: n // 10 + n // 20] = 0.0
    d = torch.from_numpy(v).cuda()
    t = torch.zeros(1, device="cuda")
    engine.check(engine.load().wob_clip_magnitude_quantile(d.data_ptr(), n, q, t.data_ptr(), None))
    torch.cuda.synchronize()
    k = min(max(int(np.ceil(np.float64(np.float32(q)) * n)), 1), n)
    ref_t = np.sort(np.abs(v))[k - 1]
    assert float(t.item()) == ref_t
    assert np.array_equal(d.cpu().numpy(), np.clip(v, -ref_t, ref_t))
    with pytest.raises(engine.WobError):
        engine.check(engine.load().wob_clip_magnitude_quantile(d.data_ptr(), n, 0.0, None, None))


def _ext_neumann_scene(engine):
    case = RC.fwdsl3d_ext_neumann_sphere5120()
    return case, engine.SceneHost(case["verts"], case["normals"], case["bvals"], case["types"])


@pytest.mark.parametrize("theta", [0.0, 0.3])
def test_cv_tables_match_float64(engine, cuda, theta):
    """Pairwise (theta 0) and with clusters taken by their expansion (theta 0.3, the same cluster
    decisions restated in float64); the 5,120-triangle scene has 160 clusters."""
    from oracle import cv_tables as T
    from wobtoolbox_gb300 import cv
    from wobtoolbox_gb300 import workloads as W
    torch = cuda
    V, F, _ = W.displaced_icosphere(4, 0.15, 4, 0)
    verts, normals = W.mesh_elements(V, F)
    g = np.ones((len(F), 3), np.float32)
    scene = engine.SceneHost(verts, normals, g, np.ones(len(F), np.int32))
    v, n, _, _, _ = scene.stored_arrays()
    cen = v.astype(np.float64).mean(1)
    sig = (0.05 + 0.02 * np.sin(3 * cen[:, 0]) * np.cos(2 * cen[:, 1]) + 0.01 * cen[:, 2]).astype(np.float32)
    d_sig = torch.from_numpy(sig).cuda()
    frames = cv.centroid_inputs(scene).cpu().numpy()
    assert np.abs(frames[:, :3] - cen).max() < 1e-6 and np.array_equal(frames[:, 3:], n)
    for domain, c in ((1, -2.0), (0, 2.0)):
        delta = torch.zeros(len(F), device="cuda")
        engine.check(engine.load().wob_cv_residual_data(scene.handle, d_sig.data_ptr(), domain, 3.0, theta,
                                                        delta.data_ptr(), None))
        torch.cuda.synchronize()
        ref = T.residual_data(v, n, sig, c, 3.0, theta=theta)
        got = delta.cpu().numpy()
        assert np.abs(got - ref).max() < 2e-4 * np.abs(ref).max(), np.abs(got - ref).max()
        if theta > 0:  # and close to the pairwise sum
            dense = T.residual_data(v, n, sig, c, 3.0)
            assert np.abs(got - dense).max() < 4e-4 * np.abs(dense).max()
    # potential at points far from and close to the surface (down to 1e-3 of the radius)
    rng = np.random.default_rng(3)
    dirs = rng.standard_normal((200, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    k = rng.integers(0, len(F), 100)
    near_pts = cen[k] + n[k].astype(np.float64) * rng.uniform(1e-3, 0.05, (100, 1))
    pts = np.concatenate([dirs[:100] * 2.0, near_pts]).astype(np.float32)
    out = cv.control_variate_potential(scene, d_sig, torch.from_numpy(pts).cuda(), len(pts), near_factor=3.0,
                                       theta=theta)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    ref = T.potential(v, sig, pts, 3.0, theta=theta)
    scale = np.abs(ref).max(0)
    assert np.all(np.abs(got - ref) <= 2e-4 * scale + 1e-7), np.abs(got - ref).max(0)
    # the split against the closed form at every pair (the far-field rule's error)
    exact = T.potential(v, sig, pts, 1e9)
    assert np.abs(got[:, 0] - exact[:, 0]).max() < 2e-3 * np.abs(exact[:, 0]).max()
    scene.close()


def test_residual_scene_walks_match_oracle(engine, oracle, cuda):
    """Clones with offsets given on the device and on the host walk bit-identically to the oracle on
    the offset arrays; the source keeps its own data, and the clones (which share the source's BVH
    and tables by reference count) keep working after the source is destroyed."""
    torch = cuda
    case, scene = _ext_neumann_scene(engine)
    rng = np.random.default_rng(4)
    delta = (rng.standard_normal(scene.n_elems) * 0.05).astype(np.float32)
    v0, n0, b0, t0, a0 = scene.stored_arrays()
    clones = [scene.clone_with_offsets(torch.from_numpy(delta).cuda()), scene.clone_with_offsets(delta)]
    p = engine.EstimatorParams(bie_model=0, domain=1, estimator=1, problem=1, path_length=4, num_sample_paths=64,
                               seed=12)
    pts = np.array([[1.8, 0.1, 0.0], [0.0, -1.9, 0.3], [1.2, 1.2, 0.2], [0.3, 0.2, 1.7]], np.float32)
    d = torch.from_numpy(pts).cuda()

    def walk(sc):
        vals = torch.zeros(len(pts), 64, 4, device="cuda")
        sc.debug_domain_paths(p, d, len(pts), vals)
        torch.cuda.synchronize()
        assert sc.poll_error() == 0
        return vals.cpu().numpy()

    def oracle_paths(b):
        return oracle.solve_domain(oracle.Elements(v0, n0, b, t0, a0), p, pts, per_path=True, accel=True)[3]

    src = walk(scene)
    scene.close()
    assert np.array_equal(src, oracle_paths(b0))
    ref = oracle_paths((b0 + delta[:, None]).astype(np.float32))
    for rscene in clones:
        v, n, b, t, a = rscene.stored_arrays()
        assert np.array_equal(v, v0) and np.array_equal(b, (b0 + delta[:, None]).astype(np.float32))
        got = walk(rscene)
        assert np.array_equal(got, ref), np.abs(got - ref).max()
        rscene.close()


def test_trained_residual_control_variate_gains(engine, cuda):
    """Exterior Neumann on the 5,120-triangle sphere: the network trained on the walk's density
    estimates, used as the residual control variate, gives a per-path variance more than 5x below
    the plain forward estimator's, and both estimates agree."""
    from wobtoolbox_gb300 import cv
    from wobtoolbox_gb300 import workloads as W
    torch = cuda
    case, scene = _ext_neumann_scene(engine)
    base = engine.EstimatorParams(bie_model=0, domain=1, estimator=1, problem=1, path_length=4, seed=1)
    mlp, info = cv.train_density_cv(scene, base, n_train=65536, train_paths=256, steps=2000, batch=8192, lr=2e-3)
    rscene, sigma = cv.residual_control_variate(scene, mlp, 1)
    pts = W.slice_points_z0(32, 4.0)
    pts = np.ascontiguousarray(pts[np.linalg.norm(pts, axis=1) > 1.6])
    d = torch.from_numpy(pts).cuda()
    pot = cv.control_variate_potential(scene, sigma, d, len(pts))
    n = 16384
    p = dataclasses.replace(base, num_sample_paths=n)
    s1 = torch.zeros(len(pts), 4, dtype=torch.float64, device="cuda")
    q1 = torch.zeros_like(s1)
    scene.solve_domain(p, d, len(pts), s1, q1)
    s2 = torch.zeros_like(s1)
    q2 = torch.zeros_like(s1)
    rscene.solve_domain(dataclasses.replace(p, seed=2), d, len(pts), s2, q2)
    torch.cuda.synchronize()
    m1 = s1.cpu().numpy()[:, 0] / n
    m2 = s2.cpu().numpy()[:, 0] / n + pot.cpu().numpy()[:, 0]
    v1 = q1.cpu().numpy()[:, 0] / n - (s1.cpu().numpy()[:, 0] / n) ** 2
    v2 = q2.cpu().numpy()[:, 0] / n - (s2.cpu().numpy()[:, 0] / n) ** 2
    ratio = v1.mean() / v2.mean()
    z = (m1 - m2) / np.sqrt((v1 + v2) / n)
    print(f"variance ratio {ratio:.1f}, max |z| {np.abs(z).max():.2f}, training {info['t_train_s']:.3f} s")
    assert ratio > 5.0, ratio
    assert np.abs(z).max() < 5.0 and abs(z.mean()) * np.sqrt(len(z)) < 5.0, z
    mlp.close()
    rscene.close()
    scene.close()
