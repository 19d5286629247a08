"""CPU tests of the oracle itself: known-answer vectors, the scalar math it shares with the
engine, and unbiasedness against closed-form harmonic solutions (the reference's own validation,
apps/general_2d.cu:123-154, apps/general_3d.cu): per-point z-scores below 4 at every point, at a
path length and at twice it, with the spread of the z-scores checked against N(0, 1) and the
truncated series' mean shift measured at both lengths (_strict_z)."""
from __future__ import annotations

import numpy as np
import pytest

from tests import scenes as S
from wobtoolbox_gb300 import workloads as W


def test_philox_known_answers(oracle):
    # Known-answer vectors of Philox4x32-10 published with the Random123 library (Salmon et al.).
    kat = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
           ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
           ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
            (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]
    for ctr, key, expect in kat:
        assert [int(x) for x in oracle.philox(ctr, *key)] == list(expect)


def test_uniforms_in_half_open_unit_interval(oracle):
    u = oracle.uniforms(0, 0, 3, 5, 100000)
    assert u.min() > 0.0 and u.max() <= 1.0
    assert abs(u.mean() - 0.5) < 0.005
    # distinct streams per (point, path)
    assert not np.array_equal(u[:8], oracle.uniforms(0, 0, 3, 6, 8))
    assert not np.array_equal(u[:8], oracle.uniforms(0, 1, 3, 5, 8))


def test_sincospi_accuracy(oracle):
    x = np.linspace(0, 2, 400001).astype(np.float32)
    s, c = oracle.sincospi(x)
    xd = x.astype(np.float64) * np.pi
    assert np.abs(s - np.sin(xd)).max() < 2e-7
    assert np.abs(c - np.cos(xd)).max() < 2e-7
    # exact at the quadrant points
    s, c = oracle.sincospi(np.array([0.0, 0.5, 1.0, 1.5, 2.0], np.float32))
    assert np.array_equal(np.abs(s), [0, 1, 0, 1, 0]) and np.array_equal(np.abs(c), [1, 0, 1, 0, 1])


def test_log_accuracy(oracle):
    x = np.concatenate([np.logspace(-44, 38, 200000), np.linspace(1e-6, 4, 200000)]).astype(np.float32)
    x = x[x > 0]
    y = oracle.log(x).astype(np.float64)
    ref = np.log(x.astype(np.float64))
    ulp = np.abs(y - ref) / np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    assert ulp.max() < 4.0
    z = oracle.log(np.array([0.0, -1.0, np.inf, np.nan], np.float32))
    assert z[0] == -np.inf and np.isnan(z[1]) and z[2] == np.inf and np.isnan(z[3])


@pytest.mark.parametrize("dim", [2, 3])
def test_green_functions_closed_form(oracle, dim):
    rng = np.random.default_rng(0)
    y = rng.standard_normal((200, dim))
    x = rng.standard_normal((200, dim))
    ny = rng.standard_normal((200, dim)); ny /= np.linalg.norm(ny, axis=1, keepdims=True)
    nx = rng.standard_normal((200, dim)); nx /= np.linalg.norm(nx, axis=1, keepdims=True)
    out = oracle.green(dim, 1e-7, y, x, ny, nx).astype(np.float64)
    r = y - x
    rn = np.linalg.norm(r, axis=1)
    rh = r / rn[:, None]
    if dim == 2:
        G = -np.log(rn) / (2 * np.pi)
        dGdx = rh / rn[:, None] / (2 * np.pi)
        dGdny = -(rh * ny).sum(1) / rn / (2 * np.pi)
        d2 = (ny - 2 * (rh * ny).sum(1)[:, None] * rh) / (2 * np.pi * rn[:, None] ** 2)
        exp = np.concatenate([G[:, None], dGdx, dGdny[:, None], d2], 1)
        got = out[:, :6]
    else:
        G = 1 / (4 * np.pi * rn)
        dGdx = rh / rn[:, None] ** 2 / (4 * np.pi)
        dGdny = -(rh * ny).sum(1) / rn ** 2 / (4 * np.pi)
        d2 = (ny - 3 * (rh * ny).sum(1)[:, None] * rh) / (4 * np.pi * rn[:, None] ** 3)
        exp = np.concatenate([G[:, None], dGdx, dGdny[:, None], d2], 1)
        got = out[:, :8]
    assert np.allclose(got, exp, rtol=2e-5, atol=1e-6)
    # dG/dx is the gradient of G in x: finite differences
    h = 1e-4
    e0 = np.zeros(dim); e0[0] = h
    Gp = oracle.green(dim, 1e-7, y, x + e0, ny, nx)[:, 0].astype(np.float64)
    Gm = oracle.green(dim, 1e-7, y, x - e0, ny, nx)[:, 0].astype(np.float64)
    fd = (Gp - Gm) / (2 * h)
    assert np.allclose(fd, out[:, 1], rtol=5e-2, atol=5e-3)


def _z_test(mean, ex, var, n):
    se = np.sqrt(np.maximum(var, 1e-300) / n)
    return (mean - ex) / se


def test_double_layer_unbiased_2d(oracle):
    """The 2D star workload's walk: DL interior Dirichlet on a star, g = e^x cos y; z-test per point."""
    sc = W.star_dirichlet_scene()
    el = oracle.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
    import wobtoolbox_gb300 as wob
    pts = sc["points"][::97]
    n = 2048
    p = wob.EstimatorParams(path_length=8, num_sample_paths=n, seed=3)
    s, q, b, _ = oracle.solve_domain(el, p, pts)
    mean = s / n
    var = q / n - mean ** 2
    z = _z_test(mean[:, 0], W.exp_cos(pts)[:, 0], var[:, 0], n)
    assert np.abs(z).max() < 4.5
    assert abs(z.mean()) < 4.0 / np.sqrt(len(z))
    # a line that only grazes the convex hull at its own element has no hit: the path ends early
    assert 0.99 * len(pts) * n * 8 < b <= len(pts) * n * 8


def test_closed_form_walk_matches_estimator(oracle):
    """apps/simple_wob_and_wos.cu:81-108 (closed-form DL walk) vs the general estimator."""
    sc = W.star_dirichlet_scene()
    el = oracle.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
    import wobtoolbox_gb300 as wob
    pts = sc["points"][::301]
    p = wob.EstimatorParams(path_length=6, num_sample_paths=256, seed=1)
    s, _, _, _ = oracle.solve_domain(el, p, pts)
    cf = oracle.simple_wob(el, 1, 6, 256, pts)
    assert np.allclose(cf, s[:, 0], rtol=1e-4, atol=1e-3 * np.abs(s[:, 0]).max())


def _strict_z(z_short, z_long):
    """Acceptance against a closed-form solution, for per-point z-scores at path length L and 2L:
    |z| < 4 at every point at both lengths (no allowance for bias); the z-scores at 2L, shifted by
    their mean, against N(0, 1) (Kolmogorov-Smirnov: the spread, i.e. the variance estimates); and
    the mean shift -- the truncated series' bias in units of the standard error, measured rather
    than allowed for -- at 2L within noise of zero or below the one at L (the series converges)."""
    from scipy import stats
    for z in (z_short, z_long):
        assert np.abs(z).max() < 4.0, z
    assert stats.kstest(z_long - z_long.mean(), "norm").pvalue > 1e-3, z_long
    assert abs(z_long.mean()) < max(4.0 / np.sqrt(len(z_long)), abs(z_short.mean())), (z_short.mean(), z_long.mean())


@pytest.mark.parametrize("combo", [(0, 0, 0, 0), (0, 0, 1, 1), (0, 0, 0, 2), (2, 0, 0, 0), (2, 0, 0, 2),
                                   (0, 1, 1, 1), (2, 1, 0, 0), (0, 0, 0, 3)])
def test_estimators_unbiased_3d(oracle, combo):
    """Backward / forward, SL / Direct, interior / exterior on a 3D displaced sphere (1,280
    triangles) against the point-source solution: 96 points (24 for the forward walks' line
    queries), 4096 paths, path length 6 and 12 (_strict_z)."""
    import wobtoolbox_gb300 as wob
    bie, dom, est, prob = combo
    sc = S.scene3d(prob, bool(dom), subdiv=3, n_points=24 if est == 1 else 96)
    el = oracle.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
    n = 4096
    pts = sc["points"]
    ex = sc["u"](pts)
    # interior Neumann: u is defined up to a constant (apps/general_2d.cu:106-121), test grad u
    comps = [1, 2, 3] if (prob == 1 and dom == 0) else [0]
    zs = []
    for L in (6, 12):
        p = wob.EstimatorParams(bie_model=bie, domain=dom, estimator=est, problem=prob, path_length=L,
                                num_sample_paths=n, seed=5, num_resampling_candidates=1,
                                first_kind_equation_scaling_constant=2.0 if prob == 3 else 1.0)
        s, q, _, _ = oracle.solve_domain(el, p, pts, accel=True)
        mean = s / n
        var = q / n - mean ** 2
        zs.append(np.concatenate([_z_test(mean[:, c], ex[:, c], var[:, c], n) for c in comps]))
    _strict_z(*zs)


@pytest.mark.parametrize("bie", [0, 2])
def test_backward_control_variate_oracle(oracle, bie):
    """Backward estimator with a per-element control variate on the unknown boundary function:
    with cv = 0 it is the plain estimator path for path; with any cv its mean agrees with the plain
    estimator's (the same walks, so the difference of the two per-path values is the CV's
    zero-mean correction)."""
    import wobtoolbox_gb300 as wob
    sc = S.scene3d(3, False, subdiv=2)
    el = oracle.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
    p = wob.EstimatorParams(bie_model=bie, domain=0, estimator=0, problem=3, path_length=4, num_sample_paths=4000,
                            seed=2, first_kind_equation_scaling_constant=2.0,
                            eps=1e-5 if bie == 0 else float(np.finfo(np.float32).eps))
    pts = sc["points"][:3]
    _, _, _, plain = oracle.solve_domain(el, p, pts, per_path=True)
    _, _, _, zero = oracle.solve_domain_bcv(el, p, np.zeros(el.n, np.float32), 4, pts, per_path=True)
    assert np.array_equal(zero, plain[:, :, 0])
    cv = np.random.default_rng(0).uniform(-0.5, 0.5, el.n).astype(np.float32)
    _, _, _, withcv = oracle.solve_domain_bcv(el, p, cv, 4, pts, per_path=True)
    d = withcv.astype(np.float64) - plain[:, :, 0]
    z = d.mean(1) / (d.std(1) / np.sqrt(d.shape[1]))
    assert np.all(np.abs(z) < 4.5), z


def test_walk_on_spheres_oracle_unbiased(oracle):
    """apps/simple_wob_and_wos.cu:111-137 restated: WoS on the star with g = e^x cos y (harmonic)
    is unbiased up to the eps-shell error; per-point z-tests."""
    import wobtoolbox_gb300 as wob
    sc = W.star_dirichlet_scene()
    el = oracle.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
    pts = sc["points"][::397]
    n = 3000
    p = wob.EstimatorParams(num_sample_paths=n, eps=1e-4, seed=2)
    s, pp, q = oracle.wos(el, p, pts, per_path=True)
    mean = s / n
    sd = pp.std(1)
    z = (mean - W.exp_cos(pts)[:, 0]) / (sd / np.sqrt(n))
    assert np.all(np.abs(z) < 4.5), z
    assert 5 < q / (len(pts) * n) < 60


def test_closest_point_oracle_brute_force(oracle):
    sc = W.star_dirichlet_scene()
    el = oracle.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
    rng = np.random.default_rng(0)
    x = rng.uniform(-1.3, 1.3, (200, 2)).astype(np.float32)
    e, d2, v = oracle.closest_point(el, x)
    a, b = el.verts[:, 0].astype(np.float64), el.verts[:, 1].astype(np.float64)
    for i in range(len(x)):
        l = b - a
        t = np.clip(((x[i] - a) * l).sum(1) / (l * l).sum(1), 0, 1)
        dd = (((a + l * t[:, None]) - x[i]) ** 2).sum(1)
        # float32 distances: the closest point is exact to a few ulp of the coordinates
        assert abs(np.sqrt(dd.min()) - np.sqrt(d2[i])) <= 1e-6


def test_lbvh_work_counter(oracle):
    """The binary-LBVH work counter behind the roofline constants: every line query tests at least
    the primitives it hits and visits at least the root; a line far from the scene visits only
    the root."""
    import wobtoolbox_gb300 as wob
    sc = W.star_dirichlet_scene()
    el = oracle.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
    p = wob.EstimatorParams(bie_model=1, path_length=2, num_sample_paths=4, seed=0)
    pts = sc["points"][::50]
    q, nn, npr = oracle.lbvh_stats(el, p, pts)
    assert q == len(pts) * 4 * 3
    assert nn >= 1.0 and npr >= 2.0  # a line through an interior point crosses the closed boundary
    assert nn < 2 * len(el.verts) and npr < len(el.verts)


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_bvh_filter_is_exact(oracle, dim):
    """The oracle's optional BVH filter for line queries (used by the CPU baseline) changes no path."""
    import wobtoolbox_gb300 as wob
    if dim == 2:
        sc = W.star_dirichlet_scene()
        el = oracle.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
        pts = sc["points"][::200]
        p = wob.EstimatorParams(bie_model=1, path_length=6, num_sample_paths=32, seed=3)
    else:
        sc = S.scene3d(1, False, subdiv=3)
        el = oracle.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
        pts = sc["points"]
        p = wob.EstimatorParams(bie_model=2, problem=1, path_length=4, num_sample_paths=32, seed=3)
    _, _, b1, pp1 = oracle.solve_domain(el, p, pts, per_path=True)
    _, _, b2, pp2 = oracle.solve_domain(el, p, pts, per_path=True, accel=True)
    assert b1 == b2 and np.array_equal(pp1, pp2)


@pytest.mark.parametrize("dim", [2, 3])
def test_vpl_aggregate_form_matches_fundamental_solution(oracle, dim):
    """The aggregation's pair form (per-VPL constants, log(max(q, eps^2)) / 2 for log(max(r, eps)),
    one division for the gradient) is the same function as mu G(y, x) A and mu dG/dx(y, x) A of
    equation_kernel.cuh:74-81, 115-121, evaluated here in float64, including points on a VPL and
    within eps of one."""
    rng = np.random.default_rng(dim)
    eps = 1e-4
    area = 3.7
    vp = rng.uniform(-1, 1, (700, dim)).astype(np.float32)
    mu = rng.standard_normal(700).astype(np.float32)
    pts = rng.uniform(-1.2, 1.2, (60, dim)).astype(np.float32)
    pts[0] = vp[5]                                    # on a VPL: that pair adds G(eps) and no gradient
    pts[1] = vp[9] + np.float32(3e-5)                 # within eps of a VPL
    got = oracle.vpl_aggregate(dim, area, eps, vp, mu, pts)
    r = vp[None].astype(np.float64) - pts[:, None].astype(np.float64)
    n = np.linalg.norm(r, axis=2)
    m = np.maximum(n, eps)
    if dim == 2:
        G = -np.log(m) / (2 * np.pi)
        with np.errstate(divide="ignore", invalid="ignore"):
            w = np.where(n > 0, 1.0 / (2 * np.pi * n * m), 0.0)
    else:
        G = 1.0 / (4 * np.pi * m)
        with np.errstate(divide="ignore", invalid="ignore"):
            w = np.where(n > 0, 1.0 / (4 * np.pi * n * np.maximum(n * n, eps)), 0.0)
    ref = np.concatenate([(mu * G * area).sum(1)[:, None], (mu[None, :, None] * w[..., None] * r * area).sum(1)], 1)
    err = np.abs(got - ref)
    assert np.all(err[:, 0] <= 1e-5 * np.abs(mu[None] * G * area).sum(1) + 1e-9)
    assert np.all(err[:, 1:] <= 1e-5 * np.abs(mu[None, :, None] * w[..., None] * r * area).sum(1) + 1e-9)


@pytest.mark.parametrize("combo", [(0, 0, 0, 0, 1), (0, 0, 1, 1, 1), (2, 1, 0, 2, 1), (0, 1, 0, 3, 8), (2, 0, 0, 3, 1)])
def test_estimators_unbiased_2d(oracle, combo):
    """2D counterparts of the 3D z-tests: single layer interior Dirichlet (backward) and Neumann
    (forward), direct exterior Robin, single layer exterior mixed with resampling (8 candidates),
    direct interior mixed -- on a 3-lobed star (200 segments) against e^x cos y / x / |x|^2:
    40 points, 8192 paths, path length 8 and 16 (_strict_z)."""
    import wobtoolbox_gb300 as wob
    bie, dom, est, prob, ris = combo
    sc = S.scene2d(prob, bool(dom), n_seg=200, n_points=40)
    el = oracle.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
    n = 8192
    pts = sc["points"]
    ex = sc["u"](pts)
    comps = [1, 2] if (prob == 1 and dom == 0) else [0]
    zs = []
    for L in (8, 16):
        p = wob.EstimatorParams(bie_model=bie, domain=dom, estimator=est, problem=prob, path_length=L,
                                num_sample_paths=n, seed=21, num_resampling_candidates=ris,
                                eps=1e-5 if bie == 0 else float(np.finfo(np.float32).eps),
                                first_kind_equation_scaling_constant=2.0 if prob == 3 else 1.0)
        s, q, _, _ = oracle.solve_domain(el, p, pts)
        mean = s / n
        var = q / n - mean ** 2
        zs.append(np.concatenate([_z_test(mean[:, c], ex[:, c], var[:, c], n) for c in comps]))
    _strict_z(*zs)


def test_volume_source_box_center(oracle):
    """apps/poisson_equation.cu's problem: u = 1 on the box (-1, 1)^2 and the constant source 5
    through a volume cache; at the centre u = 1 - 5 * 0.294685 (the square's torsion function at
    its centre, with the sign the estimator's volume term carries)."""
    import wobtoolbox_gb300 as wob
    sq = np.array([[[-1, -1], [-1, 1]], [[-1, 1], [1, 1]], [[1, 1], [1, -1]], [[1, -1], [-1, -1]]], np.float32)
    nrm = np.array([[-1, 0], [0, 1], [1, 0], [0, -1]], np.float32)
    res = 128
    el = oracle.Elements(sq, nrm, np.ones((4, 2), np.float32), np.zeros(4, np.int32),
                         volume=(res, 2.0, np.full(res * res, 5.0, np.float32)))
    n = 40000
    p = wob.EstimatorParams(bie_model=1, path_length=4, num_sample_paths=n, num_volume_samples=16, eps=1e-4, seed=2)
    pts = np.zeros((8, 2), np.float32)  # eight independent estimates (point index seeds the stream)
    s, q, _, _ = oracle.solve_domain(el, p, pts)
    mean = s[:, 0] / n
    se = np.sqrt((q[:, 0] / n - mean ** 2) / n)
    m, e = mean.mean(), se.mean() / np.sqrt(len(mean))
    assert abs(m - (1.0 - 5.0 * 0.294685)) < 5 * e + 0.01, (m, e)
