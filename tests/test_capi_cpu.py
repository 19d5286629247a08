"""CPU checks of the C ABI: the engine library loads without a GPU and exports every entry point
that include/wob_capi.h declares; the Python binding covers the same set; host-side helpers."""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "wob_capi.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+char\s*\*|int)\s*(wob_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(engine):
    lib = C.CDLL(engine._capi.LIB_PATH)
    names = _declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(engine._capi.EXPORTED) == names
    assert engine.load().wob_version() == 1


def test_enum_string_converters(engine):
    wob = engine
    assert wob.string_to_bie_model_type("IndirectDoubleLayer") == 1
    assert wob.bie_model_type_to_string(2) == "Direct"
    assert wob.string_to_problem_type("MixedProblem") == 3
    assert wob.problem_type_to_string(7) == "InvalidProblemType"
    import pytest
    with pytest.raises(ValueError):
        wob.string_to_domain_type("Inside")


def test_params_from_reference_config(engine):
    cfg = {"input_obj_file": "x.obj", "output_dir": "o", "path_length": 4, "num_resampling_candidates": 64,
           "num_sample_paths": 1000, "grid_res": 256, "eps": 1e-5, "equation_kernel": "PoissonKernel",
           "bie_model": "IndirectSingleLayer", "domain": "InteriorDomain", "estimator": "BackwardEstimator",
           "problem": "RobinProblem", "max_time": 1}
    p = engine.EstimatorParams.from_config(cfg)
    assert (p.bie_model, p.domain, p.estimator, p.problem) == (0, 0, 0, 2)
    assert p.num_resampling_candidates == 64 and p.path_length == 4
    assert p.eps == float(np.float32(1e-5)) and p.first_kind_equation_scaling_constant == 1.0
    c = p.to_c()
    assert c.num_sample_paths == 1000 and c.flags == 0


def test_raw_data_roundtrip(tmp_path):
    from wobtoolbox_gb300 import fields
    a = np.arange(12, dtype=np.float32)
    fields.save_field(str(tmp_path / "potential1.scalar"), a, 4)
    raw = open(tmp_path / "potential1.scalar", "rb").read()
    assert raw[:4] == np.uint32(4).tobytes() and len(raw) == 4 + 48
    g, b = fields.load_field(str(tmp_path / "potential1.scalar"))
    assert g == 4 and np.array_equal(a, b)


def test_grid_points_match_reference_formula():
    from wobtoolbox_gb300 import workloads as W
    p = W.idx_to_domain_point(4, 1.0, 2)
    # utils.cuh:92-100: ((x + 0.5) dx - size/2), x = idx % res fastest
    assert np.allclose(p[:4, 0], [-0.375, -0.125, 0.125, 0.375]) and np.all(p[:4, 1] == -0.375)
    assert p.dtype == np.float32


def test_config0_interior_point_count():
    from wobtoolbox_gb300 import workloads as W
    sc = W.star_dirichlet_scene()
    assert sc["mask"].sum() == 7960 and len(sc["verts"]) == 1024
    # clockwise star: outward normals
    mid = sc["verts"].mean(1)
    assert np.all((mid * sc["normals"]).sum(1) > 0)


def test_icosphere_sizes_and_orientation():
    from wobtoolbox_gb300 import workloads as W
    V, F = W.icosphere(3)
    assert len(F) == 20 * 4 ** 3
    n = W.face_normals(V, F)
    assert np.all((n * V[F].mean(1)).sum(1) > 0)
    Vd, Fd, c = W.displaced_icosphere(3, 0.15, 4, 0)
    assert len(c) == 25 and np.linalg.norm(Vd, axis=1).min() > 0.2


def test_cpp_compat_header_compiles_and_links(engine, tmp_path):
    """include/wob_gb300.hpp (the wob:: names of the reference for C++ hosts) compiles against the
    C ABI and links with the library; the enum converters and grid helper run without a GPU."""
    import os
    import subprocess
    from wobtoolbox_gb300 import build as B
    src = tmp_path / "t.cpp"
    src.write_text(r'''
#include "wob_gb300.hpp"
#include <cstdio>
int main() {
    using namespace wob;
    if (string_to_bie_model_type("IndirectDoubleLayer") != IndirectDoubleLayer) return 1;
    if (string_to_problem_type("MixedProblem") != MixedProblem) return 2;
    if (string_to_domain_type("nonsense") != DomainTypeCount) return 3;
    if (bie_model_type_to_string(Direct) != "Direct") return 4;
    if (estimator_type_to_string(ForwardEstimator) != "ForwardEstimator") return 5;
    auto p = utils::idx_to_domain_point<2>(0, 4, 1.0f);
    if (p[0] != -0.375f || p[1] != -0.375f) return 6;
    EstimatorParams prm;
    wob_params c = prm.to_c();
    if (c.bie_model != IndirectDoubleLayer || c.flags != 0) return 7;
    std::printf("%d\n", wob_version());
    return 0;
}
''')
    exe = tmp_path / "t"
    r = subprocess.run(["g++", "-std=c++17", "-I", B.INCLUDE, str(src), "-o", str(exe), "-L", B.OUT, "-lwob_gb300",
                        "-Wl,-rpath," + B.OUT], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == str(engine.load().wob_version())
