"""The device entry points only enqueue work on the caller's stream, so they can be captured into a
CUDA graph: a captured solve replayed twice adds exactly what two eager calls with the same
parameters add."""
from __future__ import annotations

import numpy as np
import pytest

from tests import scenes as S

pytestmark = pytest.mark.gpu


def test_captured_solves_replay(engine, cuda):
    torch = cuda
    sc2 = S.scene2d(0, False, n_seg=200)
    sc3 = S.scene3d(2, False)
    s2 = engine.SceneHost(sc2["verts"], sc2["normals"], sc2["bvals"], sc2["types"])
    s3 = engine.SceneHost(sc3["verts"], sc3["normals"], sc3["bvals"], sc3["types"], sc3["alphas"])
    s3.set_rhs(np.stack([sc3["bvals"], 2 * sc3["bvals"]], axis=2))
    p2 = torch.from_numpy(sc2["points"]).cuda()
    p3 = torch.from_numpy(sc3["points"]).cuda()
    dl = engine.EstimatorParams(bie_model=1, path_length=4, num_sample_paths=64, seed=2)
    rb = engine.EstimatorParams(bie_model=2, problem=2, path_length=4, num_sample_paths=64, seed=2)
    sl = engine.EstimatorParams(bie_model=0, problem=2, path_length=3, num_sample_paths=64, seed=2,
                                num_resampling_candidates=4, eps=1e-5)
    wos = engine.EstimatorParams(num_sample_paths=64, eps=1e-4, seed=2)
    n2, n3 = len(sc2["points"]), len(sc3["points"])

    def run(bufs, stream):
        a, b, c, d = bufs
        s2.solve_domain(dl, p2, n2, a, None, None, stream)
        s3.solve_domain(rb, p3, n3, b, None, None, stream)
        s3.solve_domain_multi(sl, p3, n3, c, None, None, None, stream)
        s2.solve_wos(wos, p2, n2, d, None, None, None, stream)

    def bufs():
        return (torch.zeros(n2, 3, dtype=torch.float64, device="cuda"), torch.zeros(n3, 4, dtype=torch.float64, device="cuda"),
                torch.zeros(n3, 2, dtype=torch.float64, device="cuda"), torch.zeros(n2, dtype=torch.float64, device="cuda"))

    eager = bufs()
    st = torch.cuda.current_stream()
    run(eager, st)
    run(eager, st)
    torch.cuda.synchronize()
    captured = bufs()
    g = torch.cuda.CUDAGraph()
    gs = torch.cuda.Stream()
    gs.wait_stream(st)
    with torch.cuda.stream(gs):
        with torch.cuda.graph(g, stream=gs):
            run(captured, gs)
    st.wait_stream(gs)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    for e, c in zip(eager, captured):
        e, c = e.cpu().numpy(), c.cpu().numpy()
        assert np.allclose(c, e, rtol=1e-12, atol=1e-300) and np.any(e != 0)
    s2.close()
    s3.close()
