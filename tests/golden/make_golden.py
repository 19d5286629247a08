"""Writes tests/golden/oracle_walks.npz: seeded inputs and the oracle's per-path outputs for a few
small cases (2D double layer, 3D Robin direct BIE, 2D forward single-layer Neumann with RIS-free
sampling, 3D boundary estimate, walk on spheres, line-query hit sets). tests/test_golden_cpu.py
checks that the oracle still produces them bit for bit, so a change to the oracle that alters any
walk is caught even where no GPU run compares it with the engine.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle_py as O  # noqa: E402
from tests import scenes as S  # noqa: E402
from wobtoolbox_gb300 import EstimatorParams  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_walks.npz")

# (name, scene maker, params, kind)
CASES = [
    ("dl2d", lambda: S.scene2d(0, False), dict(bie_model=1, path_length=6, num_sample_paths=16, seed=5), "domain"),
    ("robin3d", lambda: S.scene3d(2, False, subdiv=2),
     dict(bie_model=2, problem=2, path_length=6, num_sample_paths=16, seed=7), "domain"),
    ("slfwd2d", lambda: S.scene2d(1, False),
     dict(bie_model=0, estimator=1, problem=1, path_length=4, num_sample_paths=16, seed=9, eps=1e-5), "domain"),
    ("ris3d", lambda: S.scene3d(3, False, subdiv=2),
     dict(bie_model=0, problem=3, path_length=4, num_sample_paths=16, num_resampling_candidates=8, seed=11,
          eps=1e-5, first_kind_equation_scaling_constant=2.0), "domain"),
    ("boundary3d", lambda: S.scene3d(0, False, subdiv=2),
     dict(bie_model=2, path_length=4, num_sample_paths=16, seed=13), "boundary"),
    ("wos2d", lambda: S.scene2d(0, False), dict(num_sample_paths=16, eps=1e-4, seed=15), "wos"),
]


def elements(sc):
    return O.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])


def run_case(el, params, kind, arrays):
    p = EstimatorParams(**params)
    if kind == "domain":
        return O.solve_domain(el, p, arrays["points"], per_path=True)[3]
    if kind == "boundary":
        return O.solve_boundary(el, p, arrays["bp_p"], arrays["bp_n"], arrays["bp_angle"], arrays["bp_bv"],
                                arrays["bp_type"], arrays["bp_alpha"], per_path=True)[3]
    return O.wos(el, p, arrays["points"], per_path=True)[1]


def main():
    out = {}
    for name, make, params, kind in CASES:
        sc = make()
        arrays = {k: np.asarray(sc[k]) for k in ("verts", "normals", "bvals", "types", "points")}
        arrays["alphas"] = np.asarray(sc["alphas"]) if sc["alphas"] is not None else np.zeros_like(sc["bvals"])
        if kind == "boundary":
            bp = S.boundary_points(sc)
            for k, v in bp.items():
                arrays["bp_" + k] = np.asarray(v)
        el = O.Elements(arrays["verts"], arrays["normals"], arrays["bvals"], arrays["types"], arrays["alphas"])
        arrays["per_path"] = run_case(el, params, kind, arrays)
        for k, v in arrays.items():
            out[f"{name}/{k}"] = v
        out[f"{name}/params"] = np.array(repr(params))
        out[f"{name}/kind"] = np.array(kind)
    # hit sets of 200 lines on the 2D star (all hits, storage order = element order here)
    sc = S.scene2d(0, False, n_seg=300)
    rng = np.random.default_rng(3)
    o = rng.uniform(-1.3, 1.3, (200, 2)).astype(np.float32)
    d = rng.standard_normal((200, 2))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    c, h, hp = O.line_query(elements(sc), o, d)
    out.update({"lines/verts": sc["verts"], "lines/normals": sc["normals"], "lines/bvals": sc["bvals"],
                "lines/types": sc["types"], "lines/origins": o, "lines/dirs": d, "lines/counts": c, "lines/hits": h,
                "lines/hit_points": hp})
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
