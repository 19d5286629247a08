"""Parity of the CUDA walk with the CPU oracle, through the C ABI.

The engine and the oracle draw the same Philox streams and evaluate the same IEEE single-precision
formulas, so every path must come out bit-identical; the per-point FP64 sums may differ only by
FP64 summation order (relative 1e-12 of sum |x|). Covers every (BIE model, domain, estimator,
problem) combination the reference defines, in 2D and 3D, RIS, the first-kind roulette, the
volume source term, the boundary estimator and the line query.
"""
from __future__ import annotations

import itertools

import numpy as np
import pytest

from tests import scenes as S

pytestmark = pytest.mark.gpu

COMBOS = [c for c in itertools.product([0, 1, 2], [0, 1], [0, 1], [0, 1, 2, 3]) if not (c[0] == 1 and c[3] != 0)]


def _ids(c):
    bie, dom, est, prob = c
    return f"{['SL','DL','Direct'][bie]}-{['int','ext'][dom]}-{['bwd','fwd'][est]}-{'DNRM'[prob]}"


def _make(engine, sc):
    return engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])


def _oracle_elems(oracle, scene, volume=None):
    v, n, b, t, a = scene.stored_arrays()
    return oracle.Elements(v, n, b, t, a, volume)


def _params(engine, bie, dom, est, prob, **kw):
    base = dict(bie_model=bie, domain=dom, estimator=est, problem=prob, path_length=5, num_sample_paths=40,
                seed=11, eps=1e-5 if bie == 0 else float(np.finfo(np.float32).eps),
                first_kind_equation_scaling_constant=2.0 if prob == 3 else 1.0)
    base.update(kw)
    return engine.EstimatorParams(**base)


def _check_domain(engine, oracle, cuda, sc, params, volume=None):
    torch = cuda
    scene = _make(engine, sc)
    if volume is not None:
        scene.set_volume_cache(*volume)
    pts = sc["points"]
    D = pts.shape[1]
    d_pts = torch.from_numpy(pts).cuda()
    vals = torch.full((len(pts), params.num_sample_paths, D + 1), float("nan"), dtype=torch.float32, device="cuda")
    scene.debug_domain_paths(params, d_pts, len(pts), vals)
    s = torch.zeros(len(pts), D + 1, dtype=torch.float64, device="cuda")
    q = torch.zeros_like(s)
    b = torch.zeros(1, dtype=torch.int64, device="cuda")
    scene.solve_domain(params, d_pts, len(pts), s, q, b)
    torch.cuda.synchronize()
    assert scene.poll_error() == 0
    os_, oq, ob, ref = oracle.solve_domain(_oracle_elems(oracle, scene, volume), params, pts, per_path=True)
    got = vals.cpu().numpy()
    same = (got == ref) | (np.isnan(got) & np.isnan(ref))
    assert same.all(), f"{(~same).sum()} of {same.size} path values differ; max |diff| {np.nanmax(np.abs(got - ref))}"
    scale = np.abs(ref.astype(np.float64)).sum(1) + 1e-300
    assert np.all(np.abs(s.cpu().numpy() - os_) <= 1e-12 * scale + 1e-300)
    assert np.all(np.abs(q.cpu().numpy() - oq) <= 1e-12 * (ref.astype(np.float64) ** 2).sum(1) + 1e-300)
    assert int(b.item()) == ob
    scene.close()


@pytest.mark.parametrize("combo", COMBOS, ids=_ids)
def test_domain_2d(engine, oracle, cuda, combo):
    bie, dom, est, prob = combo
    sc = S.scene2d(prob, bool(dom))
    _check_domain(engine, oracle, cuda, sc, _params(engine, *combo))


@pytest.mark.parametrize("combo", COMBOS, ids=_ids)
def test_domain_3d(engine, oracle, cuda, combo):
    bie, dom, est, prob = combo
    sc = S.scene3d(prob, bool(dom))
    _check_domain(engine, oracle, cuda, sc, _params(engine, *combo, path_length=4, num_sample_paths=24))


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("prob", [0, 1, 2, 3])
def test_ris(engine, oracle, cuda, dim, prob):
    sc = S.scene2d(prob, False) if dim == 2 else S.scene3d(prob, False)
    p = _params(engine, 0, 0, 0, prob, num_resampling_candidates=8, path_length=4, num_sample_paths=16)
    _check_domain(engine, oracle, cuda, sc, p)


@pytest.mark.parametrize("bie", [1, 2])
def test_volume_source(engine, oracle, cuda, bie):
    # A box with a constant source, as apps/poisson_equation.cu:110-135 (here a Gaussian bump).
    sq = np.array([[[-1, -1], [-1, 1]], [[-1, 1], [1, 1]], [[1, 1], [1, -1]], [[1, -1], [-1, -1]]], np.float32)
    nrm = np.array([[-1, 0], [0, 1], [1, 0], [0, -1]], np.float32)
    sc = dict(verts=sq, normals=nrm, bvals=np.ones((4, 2), np.float32), types=np.zeros(4, np.int32),
              alphas=None, points=np.array([[0.1, 0.2], [-0.5, 0.3], [0.7, -0.6]], np.float32))
    res = 32
    g = np.stack(np.meshgrid(np.arange(res), np.arange(res), indexing="xy"), -1).reshape(-1, 2)
    c = (g + 0.5) * (2.0 / res) - 1.0
    f = (5.0 * np.exp(-8.0 * (c ** 2).sum(1))).astype(np.float32)
    p = _params(engine, bie, 0, 0, 0, num_volume_samples=4, eps=1e-4)
    _check_domain(engine, oracle, cuda, sc, p, volume=(res, 2.0, f))


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("combo", [(0, 0, 1, 1), (0, 0, 0, 3), (1, 0, 0, 0), (2, 0, 0, 1), (2, 1, 0, 2),
                                   (0, 1, 1, 1), (2, 0, 1, 3)], ids=_ids)
def test_boundary_estimator(engine, oracle, cuda, dim, combo):
    torch = cuda
    bie, dom, est, prob = combo
    sc = S.scene2d(prob, bool(dom)) if dim == 2 else S.scene3d(prob, bool(dom))
    bp = S.boundary_points(sc)
    params = _params(engine, *combo, path_length=4, num_sample_paths=32)
    scene = _make(engine, sc)
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in bp.items()}
    k = len(bp["p"])
    vals = torch.full((k, params.num_sample_paths), float("nan"), dtype=torch.float32, device="cuda")
    scene.debug_boundary_paths(params, dev["p"], dev["n"], dev["angle"], dev["bv"], dev["type"], dev["alpha"], k, vals)
    s = torch.zeros(k, dtype=torch.float64, device="cuda")
    scene.solve_boundary(params, dev["p"], dev["n"], dev["angle"], dev["bv"], dev["type"], dev["alpha"], k, s)
    torch.cuda.synchronize()
    os_, _, _, ref = oracle.solve_boundary(_oracle_elems(oracle, scene), params, bp["p"], bp["n"], bp["angle"],
                                           bp["bv"], bp["type"], bp["alpha"], per_path=True)
    got = vals.cpu().numpy()
    same = (got == ref) | (np.isnan(got) & np.isnan(ref))
    assert same.all(), f"{(~same).sum()} differ"
    assert np.all(np.abs(s.cpu().numpy() - os_) <= 1e-12 * np.abs(ref.astype(np.float64)).sum(1) + 1e-300)
    scene.close()


@pytest.mark.parametrize("dim", [2, 3])
def test_line_query_hits(engine, oracle, cuda, dim):
    """Hit sets, their order and the hit points are bit-identical to brute force over all elements."""
    torch = cuda
    sc = S.scene2d(0, False, n_seg=700) if dim == 2 else S.scene3d(0, False, subdiv=4)
    scene = _make(engine, sc)
    rng = np.random.default_rng(21)
    n = 4000
    o = rng.uniform(-1.3, 1.3, (n, dim)).astype(np.float32)
    d = rng.standard_normal((n, dim))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d.astype(np.float32)
    # include axis-aligned directions and rays through element vertices
    d[:50] = np.eye(dim, dtype=np.float32)[np.arange(50) % dim]
    o[50:100] = sc["verts"][:50, 0, :]
    d_o, d_d = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    counts = torch.zeros(n, dtype=torch.int32, device="cuda")
    hits = torch.zeros(n, 64, dtype=torch.int32, device="cuda")
    hp = torch.zeros(n, 64, dim, dtype=torch.float32, device="cuda")
    scene.line_query(d_o, d_d, n, counts, hits, hp)
    torch.cuda.synchronize()
    assert scene.poll_error() == 0
    rc, rh, rp = oracle.line_query(_oracle_elems(oracle, scene), o, d)
    gc = counts.cpu().numpy().astype(np.uint32)
    assert np.array_equal(gc, rc)
    gh, gp = hits.cpu().numpy().astype(np.uint32), hp.cpu().numpy()
    for i in range(n):
        m = min(rc[i], 64)
        assert np.array_equal(gh[i, :m], rh[i, :m])
        assert np.array_equal(gp[i, :m], rp[i, :m])
    assert rc.max() >= 2
    scene.close()


def test_path_offset_resume(engine, oracle, cuda):
    """Two calls with path_offset advanced equal one call with twice the paths (exact resume)."""
    torch = cuda
    sc = S.scene2d(0, False)
    scene = _make(engine, sc)
    pts = sc["points"]
    d_pts = torch.from_numpy(pts).cuda()
    p1 = _params(engine, 1, 0, 0, 0, num_sample_paths=64)
    p2a = _params(engine, 1, 0, 0, 0, num_sample_paths=32)
    p2b = _params(engine, 1, 0, 0, 0, num_sample_paths=32, path_offset=32)
    a = torch.zeros(len(pts), 3, dtype=torch.float64, device="cuda")
    b = torch.zeros_like(a)
    scene.solve_domain(p1, d_pts, len(pts), a)
    scene.solve_domain(p2a, d_pts, len(pts), b)
    scene.solve_domain(p2b, d_pts, len(pts), b)
    torch.cuda.synchronize()
    assert np.allclose(a.cpu().numpy(), b.cpu().numpy(), rtol=1e-12, atol=1e-12)
    scene.close()


def test_host_entry_matches_device_entry(engine, cuda):
    torch = cuda
    sc = S.scene3d(2, False)
    scene = _make(engine, sc)
    pts = sc["points"]
    p = _params(engine, 2, 0, 0, 2, num_sample_paths=64)
    s_h, q_h, b_h = scene.solve_domain_host(p, pts)
    d = torch.zeros(len(pts), 4, dtype=torch.float64, device="cuda")
    scene.solve_domain(p, torch.from_numpy(pts).cuda(), len(pts), d)
    torch.cuda.synchronize()
    assert np.allclose(s_h, d.cpu().numpy(), rtol=1e-12, atol=1e-12)
    assert b_h > 0
    scene.close()


def test_invalid_arguments_raise(engine, cuda):
    sc = S.scene2d(1, False)
    scene = _make(engine, sc)
    pts = sc["points"]
    with pytest.raises(engine.WobError):  # double layer needs Dirichlet elements
        scene.solve_domain_host(_params(engine, 1, 0, 0, 1), pts)
    with pytest.raises(engine.WobError):  # volume samples without a volume cache
        scene.solve_domain_host(_params(engine, 0, 0, 0, 1, num_volume_samples=2), pts)
    with pytest.raises(engine.WobError):
        scene.solve_domain_host(_params(engine, 0, 0, 0, 1, path_length=0), pts)
    scene.close()


@pytest.mark.parametrize("case", ["uniform3d", "li2d", "fwd3d"])
def test_every_tuned_configuration_is_bit_identical(engine, oracle, cuda, case):
    """The configurations the autotuner chooses among (occupancy, paths-per-lane cap and, for the 3D
    forward walk, the lockstep kernel or the split-phase wavefront) give the same paths."""
    import ctypes as C
    lib = engine.load()
    if case == "uniform3d":
        sc = S.scene3d(2, False)
        p = _params(engine, 2, 0, 0, 2, path_length=6, num_sample_paths=64)
    elif case == "fwd3d":
        sc = S.scene3d(1, True, subdiv=3)
        p = _params(engine, 0, 1, 1, 1, path_length=4, num_sample_paths=96)
    else:
        sc = S.scene2d(0, False)
        p = _params(engine, 1, 0, 0, 0, path_length=6, num_sample_paths=64)
    scene = _make(engine, sc)
    v = C.c_int32(-1)
    engine.check(lib.wob_tunable_variant(scene.handle, C.byref(p.to_c()), C.byref(v)))
    assert v.value >= 0
    old = C.c_int32(0)
    engine.check(lib.wob_get_domain_config(v.value, C.byref(old)))
    try:
        chosen, ms = scene.autotune_domain(p, cuda.from_numpy(sc["points"]).cuda(), len(sc["points"]))
        assert 0 <= chosen < len(ms) and len(ms) >= 3 and all(m > 0 for m in ms)
        for cfg in range(len(ms)):
            engine.check(lib.wob_set_domain_config(v.value, cfg))
            _check_domain(engine, oracle, cuda, sc, p)
    finally:
        lib.wob_set_domain_config(v.value, old.value)
    scene.close()


def test_batched_launch_equals_sequential_solves(engine, cuda):
    """One persistent launch over several scenes (mixed models, domains, estimators, sources and
    sizes) gives each scene exactly what wob_solve_domain gives it."""
    from wobtoolbox_gb300 import workloads as W
    torch = cuda
    specs = W.batch_scenes(8, seed=3, paths=64, path_length=4, point_range=(50, 300), grid_res=32)
    scenes, params = [], []
    for sc in specs:
        s = engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
        if sc["volume"] is not None:
            s.set_volume_cache(*sc["volume"])
        scenes.append(s)
        params.append(engine.EstimatorParams(seed=5, **dict(sc["params"], num_resampling_candidates=8
                                                             if sc["params"]["num_resampling_candidates"] > 1 else 1)))
    n_pts = [len(sc["points"]) for sc in specs]
    pts = torch.from_numpy(np.concatenate([sc["points"] for sc in specs])).cuda()
    batch = engine.SceneBatch(scenes, params, n_pts)
    bs = torch.zeros(len(pts), 3, dtype=torch.float64, device="cuda")
    bq = torch.zeros_like(bs)
    bb = torch.zeros(1, dtype=torch.int64, device="cuda")
    batch.solve(pts, bs, bq, bb, path_offset_add=128)
    ss = torch.zeros_like(bs)
    sq = torch.zeros_like(bs)
    sb = torch.zeros_like(bb)
    off = batch.offsets
    for i, (s, p) in enumerate(zip(scenes, params)):
        import dataclasses
        q = dataclasses.replace(p, path_offset=p.path_offset + 128)
        s.solve_domain(q, pts[off[i]:off[i + 1]], n_pts[i], ss[off[i]:off[i + 1]], sq[off[i]:off[i + 1]], sb)
    torch.cuda.synchronize()
    a, b = bs.cpu().numpy(), ss.cpu().numpy()
    scale = np.sqrt(64 * sq.cpu().numpy()) + 1e-300
    assert np.all(np.abs(a - b) <= 1e-12 * scale + 1e-300)
    assert int(bb.item()) == int(sb.item())
    batch.close()
    for s in scenes:
        s.close()
