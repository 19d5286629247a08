"""The allocation-free host-buffer solve (wob_solve_domain_host_noalloc), for callers that may not
allocate device memory. Called through the C ABI and compared with the allocating host-buffer
entry point (wob_solve_domain_host) on the same inputs, twice in a row: the static device array
it stages through keeps the previous call's contents, so the second call checks that nothing
leaks from the first. Kept in its own file, collected last."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from tests import scenes as S

pytestmark = pytest.mark.gpu


def _noalloc(engine, scene, params, pts, s0=None, q0=None, with_sumsq=True):
    """One call through the C ABI; s0 / q0 are the starting sums it accumulates into."""
    lib = engine.load()
    n = len(pts)
    s = np.zeros((n, scene.dim + 1)) if s0 is None else np.array(s0, dtype=np.float64, copy=True)
    q = (np.zeros((n, scene.dim + 1)) if q0 is None else np.array(q0, dtype=np.float64, copy=True)) if with_sumsq else None
    b = C.c_uint64(0)
    cp = params.to_c()
    st = lib.wob_solve_domain_host_noalloc(scene.handle, C.byref(cp), np.ascontiguousarray(pts).ctypes.data, n,
                                           s.ctypes.data, q.ctypes.data if q is not None else None, C.byref(b), None)
    engine.check(st)
    return s, q, int(b.value)


@pytest.mark.parametrize("dim", [2, 3])
def test_noalloc_matches_allocating_entry(engine, cuda, dim):
    if dim == 2:  # double layer, line-intersection sampling through the BVH
        sc = S.scene2d(0, False, n_seg=400)
        params = engine.EstimatorParams(bie_model=1, path_length=6, num_sample_paths=512, seed=3)
    else:  # direct Robin, uniform sampling
        sc = S.scene3d(2, False, subdiv=3)
        params = engine.EstimatorParams(bie_model=2, problem=2, path_length=6, num_sample_paths=512, seed=3)
    scene = engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
    rng = np.random.default_rng(0)
    pts = np.repeat(sc["points"], 40, axis=0).astype(np.float32)
    pts += rng.uniform(-1e-3, 1e-3, pts.shape).astype(np.float32)
    ref_s, ref_q, ref_b = scene.solve_domain_host(params, pts)
    for _ in range(2):
        s, q, b = _noalloc(engine, scene, params, pts)
        scale = np.sqrt(len(pts) * ref_q) + 1e-300
        assert np.all(np.abs(s - ref_s) <= 1e-12 * scale + 1e-300)
        assert np.all(np.abs(q - ref_q) <= 1e-12 * ref_q + 1e-300)
        assert b == ref_b
    scene.close()


def test_noalloc_accumulates_into_nonzero_sums(engine, cuda):
    """The call adds to the caller's running sums (the reference's cross-iteration +=,
    general_2d.cu:65-67): starting from nonzero sums gives the allocating entry's result plus
    the starting values; without a sumsq array only the sums and the bounce count are produced."""
    sc = S.scene3d(2, False, subdiv=3)
    params = engine.EstimatorParams(bie_model=2, problem=2, path_length=5, num_sample_paths=256, seed=9)
    scene = engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
    pts = np.repeat(sc["points"], 20, axis=0).astype(np.float32)
    ref_s, ref_q, ref_b = scene.solve_domain_host(params, pts)
    rng = np.random.default_rng(1)
    s0 = rng.uniform(-5, 5, ref_s.shape)
    q0 = rng.uniform(0, 5, ref_q.shape)
    scale = np.sqrt(len(pts) * ref_q) + np.abs(s0) + 1e-300
    for _ in range(2):
        s, q, b = _noalloc(engine, scene, params, pts, s0, q0)
        assert np.all(np.abs(s - (ref_s + s0)) <= 1e-12 * scale + 1e-300)
        assert np.all(np.abs(q - (ref_q + q0)) <= 1e-12 * (ref_q + q0) + 1e-300)
        assert b == ref_b
        s, q, b = _noalloc(engine, scene, params, pts, s0, None, with_sumsq=False)
        assert q is None
        assert np.all(np.abs(s - (ref_s + s0)) <= 1e-12 * scale + 1e-300)
        assert b == ref_b
    scene.close()


def test_noalloc_rejects_too_many_points(engine, cuda):
    lib = engine.load()
    m = C.c_uint32(0)
    engine.check(lib.wob_noalloc_max_points(3, C.byref(m)))
    assert 100_000 < m.value < 1_000_000
    sc = S.scene3d(2, False)
    scene = engine.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
    pts = np.zeros((m.value + 1, 3), np.float32)
    params = engine.EstimatorParams(bie_model=2, problem=2, path_length=2, num_sample_paths=1)
    with pytest.raises(engine.WobError, match="no-allocation limit"):
        _noalloc(engine, scene, params, pts)
    scene.close()
