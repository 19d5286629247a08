"""The 2D line grid's builder on the CPU: for a million lines over seven scenes (the three bin
counts, long, tiny, collinear and parallel segments), every segment the exact intersection test
accepts is listed, in storage order, in the line's cell (tests/line_grid_check.cpp restates the
device's cell lookup and exact test; the GPU test compares the device queries with the oracle)."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from wobtoolbox_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F32 = np.float32


def _polygon(pts):
    pts = np.asarray(pts, F32)
    return np.stack([pts, np.roll(pts, -1, axis=0)], axis=1).astype(F32)


def _mixed(seed=4):
    rng = np.random.default_rng(seed)
    ang = np.sort(np.concatenate([rng.uniform(0, 2 * np.pi, 400), rng.uniform(0, 2 * np.pi, 40)]))
    ang = np.sort(np.concatenate([ang, ang[:40] + 1e-4]))
    r = rng.uniform(0.3, 1.2, len(ang))
    return _polygon(np.stack([r * np.cos(ang), r * np.sin(ang)], 1))


def _comb():
    pts = [[-1.0, -0.2]]
    for i in range(200):
        x = -1.0 + 2.0 * i / 200
        pts += [[x, 0.5], [x + 0.005, 0.5], [x + 0.005, -0.1], [x + 0.01, -0.1]]
    pts += [[1.0, -0.2]]
    return _polygon(pts)


SCENES = {
    "box": (lambda: _polygon([[-1, -1], [-1, 1], [1, 1], [1, -1]]), 200000),
    "star1024": (lambda: W.star_polygon(1024, 5, 0.3)[0], 200000),
    "star3000": (lambda: W.star_polygon(3000, 5, 0.3)[0], 60000),
    "mixed": (_mixed, 200000),
    "comb": (_comb, 150000),
    "collinear": (lambda: _polygon([[x, -1.0] for x in np.linspace(-1, 1, 65)[:-1]] + [[1, -1], [1, 1], [-1, 1]]),
                  200000),
    "offset_star": (lambda: (W.star_polygon(700, 7, 0.2)[0] * F32(3.0) + F32(50.0)).astype(F32), 150000),
}


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    d = tmp_path_factory.mktemp("line_grid")
    exe = str(d / "line_grid_check")
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-ffp-contract=off", "-pthread",
           os.path.join(ROOT, "tests", "line_grid_check.cpp"),
           os.path.join(ROOT, "wobtoolbox_gb300", "csrc", "scene_build.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe, d


@pytest.mark.parametrize("name", list(SCENES))
def test_line_grid_lists_every_hit(checker, name):
    exe, d = checker
    make, n_lines = SCENES[name]
    segs = np.ascontiguousarray(make(), dtype=F32)
    path = str(d / f"{name}.bin")
    with open(path, "wb") as f:
        f.write(np.uint32(len(segs)).tobytes())
        f.write(segs.reshape(-1, 4).tobytes())
    r = subprocess.run([exe, path, str(n_lines), "7"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    f = r.stdout.split()  # lines L grid K M hits H candidates C missed X unordered U
    stats = {f[i]: f[i + 1] for i in (0, 5, 7, 9, 11)}
    K, M = int(f[3]), int(f[4])
    assert K >= 64 and M >= 64, r.stdout
    assert int(stats["lines"]) > 0.9 * n_lines and int(stats["hits"]) > 0, r.stdout
    assert int(stats["missed"]) == 0, r.stdout
    assert int(stats["unordered"]) == 0, r.stdout
