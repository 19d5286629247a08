"""Multi-RHS walks: several sets of boundary data share one set of paths.

The estimators that may share paths sample without looking at the data, so the value of a path
for RHS r must be bit-identical to the scalar walk on the data of RHS r -- checked here against the
CPU oracle run once per RHS, and against the engine's own scalar walk. Sums are per (point, RHS) in
FP64; the bounce count is that of one scalar solve (the walks are shared).
"""
from __future__ import annotations

import dataclasses

import numpy as np
import pytest

from tests import scenes as S

pytestmark = pytest.mark.gpu

CASES = [  # dim, bie, domain, problem, RIS candidates
    (2, 0, 0, 3, 1), (2, 0, 1, 3, 8), (2, 2, 0, 3, 1), (2, 2, 1, 0, 1), (2, 0, 0, 1, 1),
    (3, 0, 0, 3, 8), (3, 0, 1, 1, 1), (3, 2, 0, 3, 1), (3, 2, 0, 2, 1), (3, 2, 1, 3, 1),
]


def _ids(c):
    d, bie, dom, prob, k = c
    return f"{d}d-{['SL', 'DL', 'Direct'][bie]}-{['int', 'ext'][dom]}-{'DNRM'[prob]}-K{k}"


def _setup(engine, c, n_rhs, seed=0):
    d, bie, dom, prob, k = c
    sc = S.scene2d(prob, bool(dom)) if d == 2 else S.scene3d(prob, bool(dom))
    scene = engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
    rng = np.random.default_rng(seed)
    n = len(sc["verts"])
    rhs = rng.standard_normal((n, d, n_rhs)).astype(np.float32)
    rhs[:, :, 0] = sc["bvals"]  # RHS 0 is the scene's own data
    scene.set_rhs(rhs)
    params = engine.EstimatorParams(bie_model=bie, domain=dom, estimator=0, problem=prob, path_length=4,
                                    num_sample_paths=40, seed=7, num_resampling_candidates=k,
                                    eps=1e-5 if bie == 0 else float(np.finfo(np.float32).eps),
                                    first_kind_equation_scaling_constant=2.0)
    return sc, scene, rhs, params


def _oracle_elems(oracle, scene, rhs_r):
    v, n, _, t, a = scene.stored_arrays()
    return oracle.Elements(v, n, rhs_r[scene.element_order], t, a)


def _compare(got, ref):
    same = (got == ref) | (np.isnan(got) & np.isnan(ref))
    assert same.all(), f"{(~same).sum()} of {same.size} path values differ; max |diff| {np.nanmax(np.abs(got - ref))}"


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_domain_paths_match_scalar_walks(engine, oracle, cuda, case):
    torch = cuda
    R = 5
    sc, scene, rhs, params = _setup(engine, case, R)
    pts = sc["points"]
    P, D = len(pts), pts.shape[1]
    d_pts = torch.from_numpy(pts).cuda()
    per = torch.full((P, params.num_sample_paths, R), float("nan"), dtype=torch.float32, device="cuda")
    s = torch.zeros(P, R, dtype=torch.float64, device="cuda")
    q = torch.zeros_like(s)
    b = torch.zeros(1, dtype=torch.int64, device="cuda")
    scene.solve_domain_multi(params, d_pts, P, s, q, b, per)
    torch.cuda.synchronize()
    assert scene.poll_error() == 0
    got = per.cpu().numpy()
    for r in range(R):
        os_, oq, ob, ref = oracle.solve_domain(_oracle_elems(oracle, scene, rhs[:, :, r]), params, pts, per_path=True)
        _compare(got[:, :, r], ref[:, :, 0])
        scale = np.abs(ref[:, :, 0].astype(np.float64)).sum(1) + 1e-300
        assert np.all(np.abs(s.cpu().numpy()[:, r] - os_[:, 0]) <= 1e-12 * scale)
        assert np.all(np.abs(q.cpu().numpy()[:, r] - oq[:, 0]) <= 1e-12 * (ref[:, :, 0].astype(np.float64) ** 2).sum(1) + 1e-300)
        assert int(b.item()) == ob
    # RHS 0 is the scene's own data: the engine's scalar walk gives the same paths
    vals = torch.zeros((P, params.num_sample_paths, D + 1), dtype=torch.float32, device="cuda")
    scene.debug_domain_paths(params, d_pts, P, vals)
    torch.cuda.synchronize()
    _compare(got[:, :, 0], vals.cpu().numpy()[:, :, 0])
    scene.close()


@pytest.mark.parametrize("case", [CASES[0], CASES[2], CASES[5], CASES[7]], ids=_ids)
def test_unknown_boundary_paths_match_scalar_walks(engine, oracle, cuda, case):
    torch = cuda
    R = 4
    sc, scene, rhs, params = _setup(engine, case, R, seed=1)
    bp = S.boundary_points(sc)
    k = len(bp["p"])
    rng = np.random.default_rng(2)
    bvals = rng.standard_normal((k, R)).astype(np.float32)
    dev = {n: torch.from_numpy(np.ascontiguousarray(v)).cuda() for n, v in bp.items()}
    d_bv = torch.from_numpy(bvals).cuda()
    per = torch.full((k, params.num_sample_paths, R), float("nan"), dtype=torch.float32, device="cuda")
    s = torch.zeros(k, R, dtype=torch.float64, device="cuda")
    scene.solve_unknown_boundary_multi(params, dev["p"], dev["n"], dev["angle"], d_bv, dev["type"], dev["alpha"], k,
                                       s, None, None, per)
    torch.cuda.synchronize()
    got = per.cpu().numpy()
    for r in range(R):
        os_, _, ref = oracle.solve_unknown(_oracle_elems(oracle, scene, rhs[:, :, r]), params, bp["p"], bp["n"],
                                           bp["angle"], bvals[:, r], bp["type"], bp["alpha"], per_path=True)
        _compare(got[:, :, r], ref)
        assert np.all(np.abs(s.cpu().numpy()[:, r] - os_) <= 1e-12 * np.abs(ref.astype(np.float64)).sum(1) + 1e-300)
    scene.close()


@pytest.mark.parametrize("R", [1, 33, 64])
def test_rhs_counts(engine, oracle, cuda, R):
    """One RHS, a ragged count (lanes without an RHS) and the maximum, 64."""
    torch = cuda
    case = (3, 0, 0, 3, 4)
    sc, scene, rhs, params = _setup(engine, case, R, seed=R)
    pts = sc["points"][:4]
    P = len(pts)
    d_pts = torch.from_numpy(pts).cuda()
    per = torch.zeros((P, params.num_sample_paths, R), dtype=torch.float32, device="cuda")
    scene.solve_domain_multi(params, d_pts, P, None, None, None, per)
    torch.cuda.synchronize()
    got = per.cpu().numpy()
    for r in sorted({0, R // 2, R - 1}):
        _, _, _, ref = oracle.solve_domain(_oracle_elems(oracle, scene, rhs[:, :, r]), params, pts, per_path=True)
        _compare(got[:, :, r], ref[:, :, 0])
    scene.close()


def test_many_paths_per_point_accumulate(engine, oracle, cuda):
    """Several warp units per point, accumulated over two calls with a path offset, equal the
    oracle's single run over all paths."""
    torch = cuda
    case = (2, 0, 0, 3, 1)
    sc, scene, rhs, params = _setup(engine, case, 3)
    params.num_sample_paths = 1000
    pts = sc["points"][:3]
    P = len(pts)
    d_pts = torch.from_numpy(pts).cuda()
    s = torch.zeros(P, 3, dtype=torch.float64, device="cuda")
    scene.solve_domain_multi(params, d_pts, P, s)
    params2 = dataclasses.replace(params, path_offset=1000)
    scene.solve_domain_multi(params2, d_pts, P, s)
    torch.cuda.synchronize()
    params_all = dataclasses.replace(params, num_sample_paths=2000)
    for r in range(3):
        os_, _, _, ref = oracle.solve_domain(_oracle_elems(oracle, scene, rhs[:, :, r]), params_all, pts, per_path=True)
        scale = np.abs(ref[:, :, 0].astype(np.float64)).sum(1)
        assert np.all(np.abs(s.cpu().numpy()[:, r] - os_[:, 0]) <= 1e-12 * scale)
    scene.close()


def test_unsupported_and_invalid(engine, cuda):
    torch = cuda
    sc, scene, rhs, params = _setup(engine, (2, 0, 0, 3, 1), 2)
    d_pts = torch.from_numpy(sc["points"]).cuda()
    s = torch.zeros(len(sc["points"]), 2, dtype=torch.float64, device="cuda")
    scene.set_volume_cache(8, 4.0, np.ones(64, np.float32))
    bad = [dict(bie_model=1, problem=0), dict(bie_model=2, problem=1), dict(estimator=1), dict(num_volume_samples=2)]
    for kw in bad:
        p = dataclasses.replace(params, **kw)
        with pytest.raises(engine.WobError) as e:
            scene.solve_domain_multi(p, d_pts, len(sc["points"]), s)
        assert e.value.status == 2  # WOB_ERR_UNSUPPORTED
    with pytest.raises(engine.WobError):
        scene.set_rhs(np.zeros((len(sc["verts"]), 2, 65), np.float32))
    scene.set_rhs(None)
    with pytest.raises(engine.WobError):
        scene.solve_domain_multi(params, d_pts, len(sc["points"]), s)
    scene.close()


@pytest.mark.parametrize("case", [CASES[0], CASES[2], CASES[5], CASES[7]], ids=_ids)
def test_control_variate_paths_match_oracle(engine, oracle, cuda, case):
    """Multi-RHS domain estimate with a per-element control variate per RHS: bit-identical per path
    and RHS to the oracle's backward control-variate estimator on that RHS's data and column."""
    torch = cuda
    R = 3
    sc, scene, rhs, params = _setup(engine, case, R, seed=4)
    cvt = np.random.default_rng(5).uniform(-0.5, 0.5, (scene.n_elems, R)).astype(np.float32)
    scene.set_rhs_control_variate(cvt)
    pts = sc["points"][:6]
    P = len(pts)
    d_pts = torch.from_numpy(pts).cuda()
    per = torch.full((P, params.num_sample_paths, R), float("nan"), dtype=torch.float32, device="cuda")
    s = torch.zeros(P, R, dtype=torch.float64, device="cuda")
    b = torch.zeros(1, dtype=torch.int64, device="cuda")
    scene.solve_domain_multi_cv(params, 3, d_pts, P, s, None, b, per)
    torch.cuda.synchronize()
    got = per.cpu().numpy()
    for r in range(R):
        os_, _, ob, ref = oracle.solve_domain_bcv(_oracle_elems(oracle, scene, rhs[:, :, r]), params, cvt[:, r], 3,
                                                  pts, per_path=True)
        _compare(got[:, :, r], ref)
        assert np.all(np.abs(s.cpu().numpy()[:, r] - os_) <= 1e-12 * np.abs(ref.astype(np.float64)).sum(1) + 1e-300)
        assert int(b.item()) == ob
    # a new RHS table removes the control variate
    scene.set_rhs(rhs)
    with pytest.raises(engine.WobError):
        scene.solve_domain_multi_cv(params, 3, d_pts, P, s)
    scene.close()
