"""Per-path parity with the oracle on the benchmarked scenes themselves, not only on toy scenes.

Three hot-path code paths appear only at these sizes, and each gets a bit-identity check here:

- the 3D interior Robin workload (direct BIE, uniform sampling, 16 bounces) on the real
  81,920-triangle displaced icosphere with Robin alpha = 2 at every vertex: the element records
  then take their alphas from the scene constant instead of the second record array; every
  occupancy build the autotuner chooses among is run;
- the 3D exterior Neumann workload (forward single layer, line-intersection sampling, 4 bounces)
  on the 327,680-triangle icosphere: deep BVH traversals with leaves postponed in batches, in the
  lockstep kernel and in the split-phase wavefront (every trace shape, chunks smaller than the
  launch so that several chunks run);
- a 2D comb whose lines meet far more than 64 segments: the hit buffer overflows and the sample is
  drawn among the first 64 hits with m clamped to 64, as scene.cuh:497 and :801 do.

Every path value must be bit-identical; the per-point FP64 sums may differ only in summation
order (relative 1e-12 of sum |x|)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from wobtoolbox_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _inside_by_oracle(oracle, el, pts, direction):
    """Half-line parity of each point against the scene (brute-force line query of the oracle)."""
    dirs = np.repeat(np.asarray(direction, np.float32)[None, :], len(pts), 0)
    counts, _, hp = oracle.line_query(el, pts, dirs)
    out = np.zeros(len(pts), bool)
    for i in range(len(pts)):
        m = min(int(counts[i]), 64)
        t = ((hp[i, :m] - pts[i]) * dirs[i]).sum(1)
        out[i] = (t > 0).sum() % 2 == 1
    return out


def _run_and_compare(engine, oracle, cuda, scene, params, pts, accel=False):
    torch = cuda
    D = pts.shape[1]
    d_pts = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    vals = torch.full((len(pts), params.num_sample_paths, D + 1), float("nan"), dtype=torch.float32, device="cuda")
    scene.debug_domain_paths(params, d_pts, len(pts), vals)
    s = torch.zeros(len(pts), D + 1, dtype=torch.float64, device="cuda")
    q = torch.zeros_like(s)
    b = torch.zeros(1, dtype=torch.int64, device="cuda")
    scene.solve_domain(params, d_pts, len(pts), s, q, b)
    torch.cuda.synchronize()
    assert scene.poll_error() == 0
    v, n, bv, t, a = scene.stored_arrays()
    el = oracle.Elements(v, n, bv, t, a)
    os_, oq, ob, ref = oracle.solve_domain(el, params, pts, per_path=True, accel=accel)
    got = vals.cpu().numpy()
    same = (got == ref) | (np.isnan(got) & np.isnan(ref))
    assert same.all(), f"{(~same).sum()} of {same.size} path values differ"
    scale = np.abs(ref.astype(np.float64)).sum(1) + 1e-300
    assert np.all(np.abs(s.cpu().numpy() - os_) <= 1e-12 * scale + 1e-300)
    assert np.all(np.abs(q.cpu().numpy() - oq) <= 1e-12 * (ref.astype(np.float64) ** 2).sum(1) + 1e-300)
    assert int(b.item()) == ob
    return ref


def test_robin3d_benchmark_scene_every_tuned_build(engine, oracle, cuda):
    """The headline workload's own scene (81,920 triangles, alpha = 2, 16 bounces), 64 inside
    points of its z = 0 slice including points close to the surface, 1024 paths each."""
    sc = W.robin_sphere_scene(subdiv=6, seed=0, alpha=2.0)
    assert np.all(sc["alphas"] == 2.0)  # one alpha for every vertex: the records' scene-constant path
    scene = engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
    cand = W.slice_points_z0(512, 2.6)
    rng = np.random.default_rng(7)
    r = np.linalg.norm(cand, axis=1)
    near = cand[(r > 0.62) & (r < 1.5)]
    far = cand[r < 0.6]
    pick = np.concatenate([near[rng.choice(len(near), 400, replace=False)], far[rng.choice(len(far), 32, replace=False)]])
    v, n, bv, t, a = scene.stored_arrays()
    el = oracle.Elements(v, n, bv, t, a)
    inside = _inside_by_oracle(oracle, el, pick, (0.36, 0.48, 0.8))
    near_in = pick[:400][inside[:400]][:32]
    pts = np.ascontiguousarray(np.concatenate([near_in, pick[400:]]), dtype=np.float32)
    assert len(pts) == 64
    params = engine.EstimatorParams(bie_model=2, domain=0, estimator=0, problem=2, path_length=16,
                                    num_sample_paths=1024, seed=0)
    lib = engine.load()
    var = C.c_int32(-1)
    engine.check(lib.wob_tunable_variant(scene.handle, C.byref(params.to_c()), C.byref(var)))
    assert var.value == 0
    old = C.c_int32(0)
    engine.check(lib.wob_get_domain_config(var.value, C.byref(old)))
    try:
        for cfg in range(4):
            engine.check(lib.wob_set_domain_config(var.value, cfg))
            _run_and_compare(engine, oracle, cuda, scene, params, pts)
    finally:
        lib.wob_set_domain_config(var.value, old.value)
    scene.close()


def test_exterior_neumann_327680_triangles(engine, oracle, cuda):
    """The learned-CV workload's plain walk: forward single layer on the 327,680-triangle
    icosphere with Neumann data from three interior point sources; 32 exterior slice points
    (several within a few hundredths of the surface), 32 paths, 4 bounces."""
    rng = np.random.default_rng(0)
    V, F, _ = W.displaced_icosphere(7, 0.15, 4, 0)
    verts, normals = W.mesh_elements(V, F)
    dirs = rng.standard_normal((3, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    src = dirs * rng.uniform(0, 0.5, (3, 1))
    q = rng.uniform(-1, 1, 3)
    uv = W.point_sources(verts.reshape(-1, 3), src, q).reshape(len(F), 3, 4)
    g = (uv[..., 1:] * normals[:, None, :].astype(np.float64)).sum(-1).astype(np.float32)
    scene = engine.SceneHost(verts, normals, g, np.ones(len(F), np.int32))
    cand = W.slice_points_z0(256, 4.0)
    r = np.linalg.norm(cand, axis=1)
    ring = cand[(r > 0.6) & (r < 1.6)]
    pick = ring[np.random.default_rng(3).choice(len(ring), 200, replace=False)]
    v, n, bv, t, a = scene.stored_arrays()
    el = oracle.Elements(v, n, bv, t, a)
    inside = _inside_by_oracle(oracle, el, pick, (0.36, 0.48, 0.8))
    outside = pick[~inside][:24]
    far = cand[r > 1.6][:8]
    pts = np.ascontiguousarray(np.concatenate([outside, far]), dtype=np.float32)
    assert len(pts) == 32
    params = engine.EstimatorParams(bie_model=0, domain=1, estimator=1, problem=1, path_length=4,
                                    num_sample_paths=32, seed=0)
    lib = engine.load()
    v = C.c_int32(-1)
    engine.check(lib.wob_tunable_variant(scene.handle, C.byref(params.to_c()), C.byref(v)))
    old = C.c_int32(0)
    engine.check(lib.wob_get_domain_config(v.value, C.byref(old)))
    ref = None
    try:
        # 0: the lockstep kernel; 1-3: the wavefront's trace shapes; 13: shape 1 with the
        # smallest chunk setting
        for cfg in (0, 1, 2, 3, 13):
            engine.check(lib.wob_set_domain_config(v.value, cfg))
            got = _run_and_compare(engine, oracle, cuda, scene, params, pts, accel=True)
            assert ref is None or np.array_equal(got, ref)
            ref = got
    finally:
        lib.wob_set_domain_config(v.value, old.value)
    scene.close()


def test_forward_wavefront_chunks_equal_lockstep(engine, cuda):
    """The wavefront over many chunks (2^19 paths each: 16,384 points x 64 paths = 2 chunks)
    gives every path the lockstep kernel's value, with per-point sums equal up to order."""
    import dataclasses
    torch = cuda
    V, F, _ = W.displaced_icosphere(5, 0.15, 4, 1)
    verts, normals = W.mesh_elements(V, F)
    g = (0.2 + normals[:, None, :2].sum(-1) * np.ones((1, 3))).astype(np.float32)
    scene = engine.SceneHost(verts, normals, g, np.ones(len(F), np.int32))
    pts = W.slice_points_z0(200, 4.0)
    pts = np.ascontiguousarray(pts[np.linalg.norm(pts, axis=1) > 1.6][:16384])
    assert len(pts) == 16384
    d = torch.from_numpy(pts).cuda()
    params = engine.EstimatorParams(bie_model=0, domain=1, estimator=1, problem=1, path_length=5,
                                    num_sample_paths=64, seed=9, path_offset=128)
    lib = engine.load()
    v = C.c_int32(-1)
    engine.check(lib.wob_tunable_variant(scene.handle, C.byref(params.to_c()), C.byref(v)))
    old = C.c_int32(0)
    engine.check(lib.wob_get_domain_config(v.value, C.byref(old)))
    outs = []
    try:
        for cfg in (0, 13):
            engine.check(lib.wob_set_domain_config(v.value, cfg))
            vals = torch.zeros(len(pts), 64, 4, device="cuda")
            scene.debug_domain_paths(params, d, len(pts), vals)
            s = torch.zeros(len(pts), 4, dtype=torch.float64, device="cuda")
            q = torch.zeros_like(s)
            b = torch.zeros(1, dtype=torch.int64, device="cuda")
            scene.solve_domain(dataclasses.replace(params), d, len(pts), s, q, b)
            torch.cuda.synchronize()
            assert scene.poll_error() == 0
            outs.append((vals.cpu().numpy(), s.cpu().numpy(), q.cpu().numpy(), int(b.item())))
    finally:
        lib.wob_set_domain_config(v.value, old.value)
    (va, sa, qa, ba), (vb, sb, qb, bb) = outs
    assert np.array_equal(va, vb)
    scale = np.abs(va.astype(np.float64)).sum(1)
    assert np.all(np.abs(sa - sb) <= 1e-12 * scale + 1e-300)
    assert np.all(np.abs(qa - qb) <= 1e-12 * (va.astype(np.float64) ** 2).sum(1) + 1e-300)
    assert ba == bb == len(pts) * 64 * 5
    scene.close()


def _comb(teeth: int = 200):
    """Closed comb polygon, clockwise (outward normals by the reference's rule): a bar along
    y in [-1, -0.8] with `teeth` thin teeth up to y = 1. A horizontal line through the teeth
    meets 2 * teeth segments."""
    xs = np.linspace(-1.0, 1.0, 2 * teeth + 1)
    pts = [(-1.0, -1.0)]
    for k in range(teeth):
        x0, x1 = xs[2 * k], xs[2 * k + 1]
        pts += [(x0, 1.0), (x1, 1.0), (x1, -0.8), (xs[2 * k + 2], -0.8)] if k < teeth - 1 else [(x0, 1.0), (x1, 1.0)]
    pts += [(1.0, 1.0), (1.0, -1.0)]
    P = np.array(pts, np.float64)
    # drop consecutive duplicates, then orient clockwise
    keep = np.ones(len(P), bool)
    keep[1:] = np.any(np.abs(np.diff(P, axis=0)) > 0, axis=1)
    P = P[keep]
    area = 0.5 * np.sum(P[:, 0] * np.roll(P[:, 1], -1) - np.roll(P[:, 0], -1) * P[:, 1])
    if area > 0:
        P = P[::-1]
    verts = np.stack([P, np.roll(P, -1, axis=0)], 1).astype(np.float32)
    verts = verts[np.linalg.norm(verts[:, 1] - verts[:, 0], axis=1) > 0]
    return verts, W.segment_normals(verts)


def test_comb_more_than_64_hits(engine, oracle, cuda):
    torch = cuda
    verts, normals = _comb(200)
    g = W.exp_cos(verts.reshape(-1, 2))[:, 0].reshape(-1, 2).astype(np.float32)
    scene = engine.SceneHost(verts, normals, g, np.zeros(len(verts), np.int32))
    v, n, bv, t, a = scene.stored_arrays()
    el = oracle.Elements(v, n, bv, t, a)
    # line queries: horizontal and shallow lines through the teeth
    rng = np.random.default_rng(1)
    k = 512
    o = np.stack([rng.uniform(-0.99, 0.99, k), rng.uniform(-0.7, 0.95, k)], 1).astype(np.float32)
    ang = rng.uniform(-0.05, 0.05, k)
    d = np.stack([np.cos(ang), np.sin(ang)], 1).astype(np.float32)
    d_o, d_d = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    counts = torch.zeros(k, dtype=torch.int32, device="cuda")
    hits = torch.zeros(k, 64, dtype=torch.int32, device="cuda")
    hp = torch.zeros(k, 64, 2, dtype=torch.float32, device="cuda")
    scene.line_query(d_o, d_d, k, counts, hits, hp)
    torch.cuda.synchronize()
    assert scene.poll_error() == 0
    rc, rh, rp = oracle.line_query(el, o, d)
    gc = counts.cpu().numpy().astype(np.uint32)
    assert np.array_equal(gc, rc)
    assert (rc > 64).mean() > 0.5, "most lines must overflow the 64-entry hit buffer"
    gh, gp = hits.cpu().numpy().astype(np.uint32), hp.cpu().numpy()
    for i in range(k):
        m = min(int(rc[i]), 64)
        assert np.array_equal(gh[i, :m], rh[i, :m])
        assert np.array_equal(gp[i, :m], rp[i, :m])
    # double-layer walk from points between the teeth: most sampled lines overflow the buffer
    wn = W.winding_number_2d(verts, o)
    pts = np.ascontiguousarray(o[wn < -0.5][:24])
    assert len(pts) >= 8
    params = engine.EstimatorParams(bie_model=1, domain=0, estimator=0, problem=0, path_length=6,
                                    num_sample_paths=64, seed=4)
    _run_and_compare(engine, oracle, cuda, scene, params, pts)
    scene.close()
