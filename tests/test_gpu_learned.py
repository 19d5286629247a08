"""The learned control variate on the GPU: the MLP kernels against a float64 CPU evaluation and
torch CPU autograd, the control-variate walk against the CPU oracle (bit-identical paths), the
unknown-boundary solve, and an end-to-end check that the trained network keeps the estimator
unbiased and what it changes in the variance."""
from __future__ import annotations

import numpy as np
import pytest

from tests import scenes as S

pytestmark = pytest.mark.gpu


def _torch_grad(params, freqs, x, t):
    import torch
    p = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    X = torch.tensor(x, dtype=torch.float64)
    tt = X @ torch.tensor(freqs, dtype=torch.float64).T
    h = torch.cat([torch.sin(2 * np.pi * tt), torch.cos(2 * np.pi * tt)], 1)
    off = 0
    for l in range(5):
        fo = 1 if l == 4 else 64
        W = p[off:off + fo * 64].reshape(fo, 64)
        off += fo * 64
        b = p[off:off + fo]
        off += fo
        z = h @ W.T + b
        h = z if l == 4 else z * torch.sigmoid(z)
    loss = ((h[:, 0] - torch.tensor(t, dtype=torch.float64)) ** 2).mean()
    loss.backward()
    return p.grad.numpy(), float(loss.item()), h[:, 0].detach().numpy()


def test_mlp_forward_and_gradient_match_cpu(engine, cuda):
    from wobtoolbox_gb300 import cv
    torch = cuda
    mlp = cv.MLP(32, 4, 1, 1.0, seed=3)
    p, f = mlp.params()
    rng = np.random.default_rng(0)
    n = 1000
    x = rng.uniform(-1, 1, (n, 6)).astype(np.float32)
    t = rng.standard_normal(n).astype(np.float32) * 0.3
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    y = torch.zeros(n, device="cuda")
    mlp.forward(dx, n, y)
    g = torch.zeros(mlp.n_params, device="cuda")
    loss = torch.zeros(1, device="cuda")
    mlp.gradient(dx, dt, n, g, loss)
    torch.cuda.synchronize()
    ref_y = cv.reference_forward(p, f, x)[:, 0]
    gy = y.cpu().numpy()
    # BF16 operands, FP32 accumulation
    assert np.abs(gy - ref_y).max() < 3e-2 * (np.abs(ref_y).max() + 1e-3)
    ref_g, ref_l, _ = _torch_grad(p, f, x, t)
    gg = g.cpu().numpy()
    rel = np.linalg.norm(gg - ref_g) / np.linalg.norm(ref_g)
    cos = float(gg @ ref_g / (np.linalg.norm(gg) * np.linalg.norm(ref_g)))
    assert rel < 5e-2 and cos > 0.998, (rel, cos)
    assert abs(float(loss.item()) - ref_l) < 2e-2 * ref_l
    mlp.close()


def test_mlp_training_reduces_loss(engine, cuda):
    from wobtoolbox_gb300 import cv
    torch = cuda
    mlp = cv.MLP(32, 4, 1, 0.5, seed=1)
    rng = np.random.default_rng(1)
    n = 8192
    x = rng.uniform(-1, 1, (n, 6)).astype(np.float32)
    t = (np.sin(2 * x[:, 0]) * np.cos(x[:, 1]) + 0.3 * x[:, 2]).astype(np.float32)
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    loss = torch.zeros(1, device="cuda")
    first = None
    for it in range(400):
        loss.zero_()
        mlp.adam_step(dx, dt, n, 3e-3, loss)
        if it == 0:
            torch.cuda.synchronize()
            first = float(loss.item())
    torch.cuda.synchronize()
    assert float(loss.item()) < 0.1 * first
    mlp.close()


def _cv_scene(engine):
    sc = S.scene3d(1, True, subdiv=3)
    scene = engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
    return sc, scene


def test_control_variate_walk_matches_oracle(engine, oracle, cuda):
    from wobtoolbox_gb300 import cv
    torch = cuda
    sc, scene = _cv_scene(engine)
    rng = np.random.default_rng(2)
    sig = rng.standard_normal(scene.n_elems).astype(np.float32) * 0.1
    cv.set_control_variate(scene, sig)
    p = engine.EstimatorParams(bie_model=0, domain=1, estimator=1, problem=1, path_length=4, num_sample_paths=32,
                               seed=9)
    pts = sc["points"]
    d = torch.from_numpy(pts).cuda()
    vals = torch.full((len(pts), 32, 4), float("nan"), device="cuda")
    cv.solve_domain_cv(scene, p, d, len(pts), None, per_path=vals, n_potential=5, n_kernel=3)
    torch.cuda.synchronize()
    v, n, b, t, _ = scene.stored_arrays()
    _, _, _, ref = oracle.solve_domain_cv(oracle.Elements(v, n, b, t), p, sig, 5, 3, pts, per_path=True)
    got = vals.cpu().numpy()
    same = (got == ref) | (np.isnan(got) & np.isnan(ref))
    assert same.all(), f"{(~same).sum()} of {same.size} differ"
    scene.close()


def test_unknown_boundary_matches_oracle(engine, oracle, cuda):
    import ctypes as C
    torch = cuda
    sc, scene = _cv_scene(engine)
    bp = S.boundary_points(sc)
    p = engine.EstimatorParams(bie_model=0, domain=1, estimator=0, problem=1, path_length=4, num_sample_paths=64,
                               seed=4)
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in bp.items()}
    k = len(bp["p"])
    s = torch.zeros(k, dtype=torch.float64, device="cuda")
    cp = p.to_c()
    engine.check(engine.load().wob_solve_unknown_boundary(
        scene.handle, C.byref(cp), dev["p"].data_ptr(), dev["n"].data_ptr(), dev["angle"].data_ptr(),
        dev["bv"].data_ptr(), dev["type"].data_ptr(), dev["alpha"].data_ptr(), k, s.data_ptr(), None, None, None))
    torch.cuda.synchronize()
    v, n, b, t, _ = scene.stored_arrays()
    ref, _, pp = oracle.solve_unknown(oracle.Elements(v, n, b, t), p, bp["p"], bp["n"], bp["angle"], bp["bv"],
                                      bp["type"], bp["alpha"], per_path=True)
    assert np.all(np.abs(s.cpu().numpy() - ref) <= 1e-12 * np.abs(pp.astype(np.float64)).sum(1) + 1e-300)
    scene.close()


def test_trained_control_variate_is_unbiased(engine, cuda):
    """Train the network on walk estimates of the density, then compare the control-variate
    estimator with the plain forward estimator at the same points: the means must agree
    (|z| < 5) and the variance ratio is reported."""
    from wobtoolbox_gb300 import cv
    torch = cuda
    sc, scene = _cv_scene(engine)
    base = engine.EstimatorParams(bie_model=0, domain=1, estimator=1, problem=1, path_length=4, seed=1)
    mlp, info = cv.train_density_cv(scene, base, n_train=8192, train_paths=128, steps=300, batch=4096, lr=3e-3)
    table = cv.element_cv_table(mlp, scene)
    assert np.isfinite(table).all()
    cv.set_control_variate(scene, table)
    pts = sc["points"]
    d = torch.from_numpy(pts).cuda()
    n = 20000
    import dataclasses
    p = dataclasses.replace(base, num_sample_paths=n)
    s1 = torch.zeros(len(pts), 4, dtype=torch.float64, device="cuda")
    q1 = torch.zeros_like(s1)
    scene.solve_domain(p, d, len(pts), s1, q1)
    s2 = torch.zeros_like(s1)
    q2 = torch.zeros_like(s1)
    cv.solve_domain_cv(scene, p, d, len(pts), s2, q2, n_potential=16, n_kernel=16)
    torch.cuda.synchronize()
    m1, m2 = s1.cpu().numpy()[:, 0] / n, s2.cpu().numpy()[:, 0] / n
    v1 = q1.cpu().numpy()[:, 0] / n - m1 ** 2
    v2 = q2.cpu().numpy()[:, 0] / n - m2 ** 2
    z = (m1 - m2) / np.sqrt((v1 + v2) / n)
    assert np.abs(z).max() < 5.0, z
    exact = sc["u"](pts)[:, 0]
    print("variance ratio plain/cv per point:", np.round(v1 / v2, 3), "means", m1, m2, "exact", exact)
    mlp.close()
    scene.close()
