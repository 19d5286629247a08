"""The oracle against the reference's own estimator (compiled from the reference tree; committed
fixtures tests/golden/reference_*.npz written by tests/golden/make_reference_fixtures.py): the
statistical agreement of tests/reference_stats.py at equal sample count, on the benchmark
workloads (the 2D double-layer star complete: all 7,960 points) and on shipped reference
configurations.
This pins the oracle, and through the engine's bit-identity with the oracle, the engine."""
from __future__ import annotations

import dataclasses

import numpy as np
import pytest

from tests import reference_cases as RC
from tests import reference_stats as RS


@pytest.mark.parametrize("name", list(RC.CASES))
def test_oracle_agrees_with_reference(oracle, name):
    case = RC.CASES[name]()
    fix = np.load(RC.fixture_path(name))
    assert str(fix["checksum"]) == RC.scene_checksum(case), "scene generator changed: regenerate the fixture"
    pts = fix["points"]
    el = oracle.Elements(case["verts"], case["normals"], case["bvals"], case["types"], case["alphas"],
                         case["volume"])
    accel = case["verts"].shape[0] > 64

    def run_sums(seed):
        p = dataclasses.replace(case["params"], num_sample_paths=int(fix["n_paths"]), seed=seed)
        s, q, _, _ = oracle.solve_domain(el, p, pts, accel=accel)
        return s, q

    def run_per_path(seed):
        n_pp = fix["per_path"].shape[0]
        p = dataclasses.replace(case["params"], num_sample_paths=int(fix["pp_paths"]), seed=seed)
        _, _, _, pp = oracle.solve_domain(el, p, pts[:n_pp], per_path=True, accel=accel)
        return pp[:, :, 0]

    rep = RS.check_against_reference(fix, run_sums, run_per_path, name)
    print(name, rep)


@pytest.mark.parametrize("name", list(RC.CASES))
def test_fixture_reproduces_from_reference_tree(name):
    """Where the reference tree is present, its compiled estimator (oracle/_ref) reproduces the
    committed fixture bit for bit: the fixtures are the reference's output, not the oracle's."""
    import dataclasses as dc
    from oracle import ref_py as R
    if not R.available():
        pytest.skip("reference tree not present")
    R.build()
    import sys
    import os
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_reference_fixtures as MK
    case = RC.CASES[name]()
    fix = np.load(RC.fixture_path(name))
    pts = fix["points"]
    p = dc.replace(case["params"], num_sample_paths=int(fix["n_paths"]))
    s, q, _ = R.solve_domain(case["verts"], case["normals"], case["bvals"], case["types"], case["alphas"], p, pts,
                             MK.MAIN_SEED, volume=case["volume"])
    assert np.array_equal(s, fix["sum"]) and np.array_equal(q, fix["sumsq"])
