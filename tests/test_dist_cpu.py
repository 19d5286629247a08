"""The multi-rank host logic of bench.py on CPU ranks (gloo, world size 2): process-group setup from
the torchrun environment, barrier, max over ranks (the job's time) and sum over ranks (the units all
ranks processed), and the path sharding: rank r walks the paths r * 2^40 + j of every point, so the
ranks' walks are disjoint Philox streams and their sums add up to the oracle's over both shards."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from oracle import oracle_py as O
    from wobtoolbox_gb300 import EstimatorParams
    from tests import scenes as S

    class A:
        pass
    r, w, _ = bench.dist_init(A())
    bench.barrier(w)
    mx = bench.max_over_ranks(float(r + 1), w)
    sm = bench.sum_over_ranks(float(10 * (r + 1)), w)
    sc = S.scene2d(0, False, n_seg=64)
    el = O.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
    p = EstimatorParams(bie_model=1, path_length=3, num_sample_paths=32, seed=4, path_offset=r * (1 << 40))
    s, _, b, _ = O.solve_domain(el, p, sc["points"][:3], n_threads=1)
    bench.barrier(w)
    q.put((r, w, mx, sm, s, b))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_bench_logic():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=300) for _ in range(2)], key=lambda t: t[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [t[1] for t in res] == [2, 2]
    assert all(t[2] == 2.0 for t in res)       # max over ranks
    assert all(t[3] == 30.0 for t in res)      # sum over ranks
    # disjoint shards: the two ranks' sums differ, and each equals a single-process run of that shard
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle import oracle_py as O
    from wobtoolbox_gb300 import EstimatorParams
    from tests import scenes as S
    sc = S.scene2d(0, False, n_seg=64)
    el = O.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"])
    for r, *_rest in res:
        p = EstimatorParams(bie_model=1, path_length=3, num_sample_paths=32, seed=4, path_offset=r * (1 << 40))
        s, _, b, _ = O.solve_domain(el, p, sc["points"][:3], n_threads=1)
        assert np.array_equal(s, res[r][4]) and b == res[r][5]
    assert not np.array_equal(res[0][4], res[1][4])
