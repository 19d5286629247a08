"""Inputs for the JSON-app tests: configs in the reference's format and OBJ files written from the
seeded generators (coordinates printed exactly, so the apps read the same float32 values)."""
from __future__ import annotations

import json
import os
import subprocess

import numpy as np

from wobtoolbox_gb300 import workloads as W


def _num(x) -> str:
    return f"{float(np.float32(x)):.17g}"


def write_star_obj(path, n_seg=200, scale=0.35):
    verts, _ = W.star_polygon(n_seg, 5, 0.3)
    pts = (verts[:, 0, :] * np.float32(scale)).astype(np.float32)
    with open(path, "w") as f:
        for p in pts:
            f.write(f"v {_num(p[0])} {_num(p[1])} 0.0\n")
        for i in range(n_seg):  # "f a b a" segments, as data/bunny_2d.obj
            a, b = i + 1, (i + 1) % n_seg + 1
            f.write(f"f {a} {b} {a}\n")
    return pts


def write_sphere_obj(path, subdiv=2):
    V, F = W.icosphere(subdiv)
    V = V.astype(np.float32)
    with open(path, "w") as f:
        for p in V:
            f.write(f"v {_num(p[0])} {_num(p[1])} {_num(p[2])}\n")
        for t in F:
            f.write(f"f {t[0] + 1}/{t[0] + 1} {t[1] + 1}/{t[1] + 1} {t[2] + 1}/{t[2] + 1}\n")
    return V, F


def write_config(path, obj, out_dir, **kw):
    cfg = {"input_obj_file": obj, "output_dir": out_dir, "path_length": 4, "num_sample_paths": 64, "grid_res": 32,
           "equation_kernel": "PoissonKernel", "__bie_model_options__": "IndirectSingleLayer, IndirectDoubleLayer, "
           "Direct", "bie_model": "IndirectDoubleLayer", "domain": "InteriorDomain", "estimator": "BackwardEstimator",
           "problem": "DirichletProblem", "max_time": 1}
    cfg.update(kw)
    with open(path, "w") as f:
        json.dump(cfg, f, indent=4)
    return cfg


def run_app(name, cfg_path, *extra, timeout=600):
    from wobtoolbox_gb300 import build
    build.build()
    return subprocess.run([build.app_path(name), cfg_path, *extra], capture_output=True, text=True, timeout=timeout)


def read_field(path, comps=1):
    raw = open(path, "rb").read()
    n = int(np.frombuffer(raw[:4], dtype=np.uint32)[0])
    vals = np.frombuffer(raw[4:], dtype=np.float32)
    assert vals.size == n * n * comps
    return n, vals.reshape(n * n, comps) if comps > 1 else vals


def winding_3d(tri, pts):
    """Generalised winding number of a triangle soup [m, 3, 3] at points [n, 3] (float64)."""
    w = np.zeros(len(pts))
    for k in range(0, len(tri), 512):
        t = tri[None, k:k + 512].astype(np.float64) - pts[:, None, None, :]
        a, b, c = t[:, :, 0], t[:, :, 1], t[:, :, 2]
        la, lb, lc = (np.linalg.norm(x, axis=2) for x in (a, b, c))
        det = np.einsum("nmk,nmk->nm", a, np.cross(b, c))
        den = la * lb * lc + (a * b).sum(2) * lc + (b * c).sum(2) * la + (c * a).sum(2) * lb
        w += 2 * np.arctan2(det, den).sum(1)
    return w / (4 * np.pi)
