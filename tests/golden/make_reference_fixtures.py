"""Writes tests/golden/reference_<case>.npz: per-point statistics and per-path values of the
REFERENCE's own estimator (wob/wob/*.cuh compiled from the reference tree in its CPU
configuration, oracle/ref_driver.cpp) for the cases of tests/reference_cases.py.

Run where the reference tree is present (it is read, never modified):

    python tests/golden/make_reference_fixtures.py [case ...]

Each fixture holds: the evaluation points; sum and sum of squares of every component of the
reference's path contributions over n_paths paths per point (its random states seeded as
random_states_init does, from std::mt19937_64(5489)); every path's u for the first n_pp points
over pp_paths paths (a second run, seeded from std::mt19937_64(12345)); the estimator settings
and a checksum of the scene arrays. tests/test_reference_parity_cpu.py compares the oracle with
these, tests/test_gpu_reference_parity.py the engine.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle_py as O  # noqa: E402
from oracle import ref_py as R  # noqa: E402
from tests import reference_cases as RC  # noqa: E402
from wobtoolbox_gb300 import workloads as W  # noqa: E402

MAIN_SEED = 5489
PER_PATH_SEED = 12345


def _parity_inside(case, pts):
    """Inside test by half-line parity (exact brute-force line query of the oracle)."""
    el = O.Elements(case["verts"], case["normals"], case["bvals"], case["types"], case["alphas"])
    d = np.array([0.36, 0.48, 0.8], np.float32)[: pts.shape[1]]
    d = (d / np.linalg.norm(d)).astype(np.float32)
    dirs = np.repeat(d[None], len(pts), 0)
    counts, _, hp = O.line_query(el, pts, dirs)
    inside = np.zeros(len(pts), bool)
    for i in range(len(pts)):
        m = min(int(counts[i]), 64)
        t = ((hp[i, :m] - pts[i]) * dirs[i]).sum(1)
        inside[i] = (t > 0).sum() % 2 == 1
    return inside


def points_for(name, case):
    rng = np.random.default_rng(100)
    if name == "dl2d_star1024":
        return W.star_dirichlet_scene()["points"]
    if name == "robin3d_sphere81920_alpha1":
        cand = W.slice_points_z0(512, 2.6)
        cand = cand[rng.choice(len(cand), 2000, replace=False)]
        return np.ascontiguousarray(cand[_parity_inside(case, cand)][:512])
    if name == "fwdsl3d_ext_neumann_sphere5120":
        cand = W.slice_points_z0(256, 4.0)
        cand = cand[rng.choice(len(cand), 1000, replace=False)]
        return np.ascontiguousarray(cand[~_parity_inside(case, cand)][:256])
    if name == "slris3d_mixed_sphere1280":
        cand = rng.uniform(-1.2, 1.2, (1000, 3)).astype(np.float32)
        return np.ascontiguousarray(cand[_parity_inside(case, cand)][:128])
    if name in ("slris2d_robin_star512", "direct2d_int_neumann_star512"):
        cand = rng.uniform(-1.3, 1.3, (2000, 2)).astype(np.float32)
        wn = W.winding_number_2d(case["verts"], cand)
        return np.ascontiguousarray(cand[wn < -0.5][:256])
    if name == "dl2d_poisson_box":
        return rng.uniform(-0.95, 0.95, (128, 2)).astype(np.float32)
    raise KeyError(name)


def make(name):
    case = RC.CASES[name]()
    pts = points_for(name, case).astype(np.float32)
    p = case["params"]
    import dataclasses
    t0 = time.perf_counter()
    s, q, _ = R.solve_domain(case["verts"], case["normals"], case["bvals"], case["types"], case["alphas"],
                             dataclasses.replace(p, num_sample_paths=case["n_paths"]), pts, MAIN_SEED,
                             volume=case["volume"])
    t1 = time.perf_counter()
    pp_pts = pts[: case["n_pp"]]
    _, _, pp = R.solve_domain(case["verts"], case["normals"], case["bvals"], case["types"], case["alphas"],
                              dataclasses.replace(p, num_sample_paths=case["pp_paths"]), pp_pts, PER_PATH_SEED,
                              n_per_path=case["n_pp"], volume=case["volume"])
    t2 = time.perf_counter()
    np.savez_compressed(RC.fixture_path(name), points=pts, sum=s, sumsq=q, per_path=pp,
                        n_paths=case["n_paths"], pp_paths=case["pp_paths"], checksum=RC.scene_checksum(case),
                        params=np.array([p.bie_model, p.domain, p.estimator, p.problem, p.path_length,
                                         p.num_resampling_candidates, p.num_volume_samples], np.int64),
                        reals=np.array([p.eps, p.first_kind_equation_scaling_constant]))
    print(f"{name}: {len(pts)} points x {case['n_paths']} paths ({t1 - t0:.1f} s), "
          f"{case['n_pp']} points x {case['pp_paths']} paths per path ({t2 - t1:.1f} s)")


def main():
    if not R.available():
        raise SystemExit("the reference tree is not present; set WOB_REFERENCE_TREE")
    O.build()
    R.build()
    for name in (sys.argv[1:] or list(RC.CASES)):
        make(name)


if __name__ == "__main__":
    main()
