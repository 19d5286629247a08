"""GB300 walk-on-boundary (WoB) engine: Python host API.

Mirrors the host-side interface of rsugimoto/WoBToolbox (wob/wob.cuh): the enum names and their
string converters (bie_models.cuh:21-51, estimator.cuh:24-54, equation_kernel.cuh:20-34), a
SceneHost built from boundary elements (scene.cuh:264-326) with an optional volume cache
(scene.cuh:301-306), and estimator parameters matching the Estimator constructor
(estimator.cuh:145-152). The walk itself runs in hand-written sm_103a CUDA behind the C ABI of
include/wob_capi.h; there is no CPU path in this package.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
from typing import Optional

import numpy as np

from . import _capi
from ._capi import WobError, check, load

__all__ = [
    "PoissonKernel", "IndirectSingleLayer", "IndirectDoubleLayer", "Direct", "InteriorDomain", "ExteriorDomain",
    "BackwardEstimator", "ForwardEstimator", "DirichletProblem", "NeumannProblem", "RobinProblem", "MixedProblem",
    "Dirichlet", "Neumann", "Robin", "string_to_bie_model_type", "bie_model_type_to_string",
    "string_to_domain_type", "domain_type_to_string", "string_to_estimator_type", "estimator_type_to_string",
    "string_to_problem_type", "problem_type_to_string", "string_to_equation_kernel_type",
    "EstimatorParams", "SceneHost", "SceneBatch", "WobError", "load",
]

# ---- enums (same values as the reference)
PoissonKernel = 0
IndirectSingleLayer, IndirectDoubleLayer, Direct = 0, 1, 2
InteriorDomain, ExteriorDomain = 0, 1
BackwardEstimator, ForwardEstimator = 0, 1
DirichletProblem, NeumannProblem, RobinProblem, MixedProblem = 0, 1, 2, 3
Dirichlet, Neumann, Robin = 0, 1, 2

_BIE = ["IndirectSingleLayer", "IndirectDoubleLayer", "Direct"]
_DOMAIN = ["InteriorDomain", "ExteriorDomain"]
_EST = ["BackwardEstimator", "ForwardEstimator"]
_PROBLEM = ["DirichletProblem", "NeumannProblem", "RobinProblem", "MixedProblem"]


def _to_enum(names, s: str, kind: str) -> int:
    if s not in names:
        raise ValueError(f"invalid {kind} {s!r}; expected one of {names}")
    return names.index(s)


def string_to_equation_kernel_type(s: str) -> int:
    if s != "PoissonKernel":
        raise ValueError(f"invalid equation kernel {s!r}; expected 'PoissonKernel'")
    return PoissonKernel


def string_to_bie_model_type(s: str) -> int:
    return _to_enum(_BIE, s, "bie_model")


def bie_model_type_to_string(v: int) -> str:
    return _BIE[v] if 0 <= v < len(_BIE) else "InvalidBIEModelType"


def string_to_domain_type(s: str) -> int:
    return _to_enum(_DOMAIN, s, "domain")


def domain_type_to_string(v: int) -> str:
    return _DOMAIN[v] if 0 <= v < len(_DOMAIN) else "InvalidDomainType"


def string_to_estimator_type(s: str) -> int:
    return _to_enum(_EST, s, "estimator")


def estimator_type_to_string(v: int) -> str:
    return _EST[v] if 0 <= v < len(_EST) else "InvalidEstimatorType"


def string_to_problem_type(s: str) -> int:
    return _to_enum(_PROBLEM, s, "problem")


def problem_type_to_string(v: int) -> str:
    return _PROBLEM[v] if 0 <= v < len(_PROBLEM) else "InvalidProblemType"


@dataclasses.dataclass
class EstimatorParams:
    """The reference's Estimator arguments plus the enums run<> dispatches on.

    Defaults follow apps/general_2d.cu:174-195 (num_resampling_candidates 1, eps FLT_EPSILON,
    first_kind_equation_scaling_constant 1).
    """
    bie_model: int = IndirectDoubleLayer
    domain: int = InteriorDomain
    estimator: int = BackwardEstimator
    problem: int = DirichletProblem
    path_length: int = 8
    num_sample_paths: int = 1
    num_resampling_candidates: int = 1
    num_volume_samples: int = 0
    eps: float = float(np.finfo(np.float32).eps)
    first_kind_equation_scaling_constant: float = 1.0
    seed: int = 0
    path_offset: int = 0
    point_offset: int = 0

    def to_c(self) -> _capi.wob_params:
        p = _capi.wob_params()
        for f in dataclasses.fields(self):
            setattr(p, f.name, getattr(self, f.name))
        p.flags = 0
        return p

    @classmethod
    def from_config(cls, cfg: dict, **overrides) -> "EstimatorParams":
        """From a reference JSON config (apps/general_2d.cu:174-195 keys)."""
        string_to_equation_kernel_type(cfg.get("equation_kernel", "PoissonKernel"))
        p = cls(
            bie_model=string_to_bie_model_type(cfg["bie_model"]),
            domain=string_to_domain_type(cfg["domain"]),
            estimator=string_to_estimator_type(cfg["estimator"]),
            problem=string_to_problem_type(cfg["problem"]),
            path_length=int(cfg["path_length"]),
            num_sample_paths=int(cfg["num_sample_paths"]),
            num_resampling_candidates=int(cfg.get("num_resampling_candidates", 1)),
            num_volume_samples=int(cfg.get("num_volume_samples", 0)),
            eps=float(np.float32(cfg.get("eps", np.finfo(np.float32).eps))),
            first_kind_equation_scaling_constant=float(cfg.get("first_kind_equation_scaling_constant", 1.0)),
        )
        return dataclasses.replace(p, **overrides)


def _ptr(x) -> Optional[int]:
    """Device pointer of a torch tensor / int / None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return int(x.data_ptr())


def _stream_ptr(stream) -> Optional[int]:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(stream.cuda_stream)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


class SceneHost:
    """Boundary elements on the GPU with their BVH and sampling tables (wob::SceneHost).

    vertices [n, dim, dim], normals [n, dim], boundary_values [n, dim] (per vertex),
    boundary_types [n], robin_alphas [n, dim] or None. Elements are stored in BVH leaf order;
    `element_order[i]` is the caller index of the i-th stored element.
    """

    def __init__(self, vertices, normals, boundary_values, boundary_types, robin_alphas=None):
        lib = load()
        v = _f32(vertices)
        if v.ndim != 3 or v.shape[1] != v.shape[2] or v.shape[1] not in (2, 3):
            raise ValueError("vertices must have shape [n, dim, dim] with dim 2 or 3")
        self.dim = int(v.shape[1])
        n = int(v.shape[0])
        nrm = _f32(normals).reshape(n, self.dim)
        bv = _f32(boundary_values).reshape(n, self.dim)
        ty = np.ascontiguousarray(boundary_types, dtype=np.int32).reshape(n)
        al = None if robin_alphas is None else _f32(robin_alphas).reshape(n, self.dim)
        h = C.c_void_p()
        check(lib.wob_scene_create(self.dim, n, v.ctypes.data, nrm.ctypes.data, bv.ctypes.data,
                                   None if al is None else al.ctypes.data, ty.ctypes.data, C.byref(h)))
        self._h = h
        self.n_elems = n
        order = np.empty(n, dtype=np.uint32)
        check(lib.wob_scene_get_element_order(h, order.ctypes.data))
        self.element_order = order
        self._host = (v, nrm, bv, ty, al)
        self.n_rhs = 0

    @classmethod
    def build_on_device(cls, vertices, normals, boundary_values, boundary_types, robin_alphas=None, stream=None):
        """The same scene built on the GPU (wob_scene_create_device) from CUDA tensors of the
        constructor's shapes (float32; int32 types)."""
        lib = load()
        obj = cls.__new__(cls)
        obj.dim = int(vertices.shape[1])
        n = int(vertices.shape[0])
        h = C.c_void_p()
        check(lib.wob_scene_create_device(obj.dim, n, _ptr(vertices), _ptr(normals), _ptr(boundary_values),
                                          _ptr(robin_alphas), _ptr(boundary_types), _stream_ptr(stream), C.byref(h)))
        obj._h = h
        obj.n_elems = n
        order = np.empty(n, dtype=np.uint32)
        check(lib.wob_scene_get_element_order(h, order.ctypes.data))
        obj.element_order = order
        cpu = lambda t: None if t is None else t.detach().cpu().numpy()
        obj._host = (cpu(vertices), cpu(normals).reshape(n, obj.dim), cpu(boundary_values).reshape(n, obj.dim),
                     cpu(boundary_types).reshape(n),
                     None if robin_alphas is None else cpu(robin_alphas).reshape(n, obj.dim))
        obj.n_rhs = 0
        return obj

    @property
    def handle(self):
        return self._h

    def stored_arrays(self):
        """Element arrays permuted into the storage order (what the sampling tables refer to)."""
        v, nrm, bv, ty, al = self._host
        o = self.element_order
        return (v[o], nrm[o], bv[o], ty[o], None if al is None else al[o])

    def clone_with_offsets(self, delta, stream=None) -> "SceneHost":
        """An independent copy of this scene whose stored element j has delta[j] added to each of
        its vertex boundary values (delta: device tensor or host array, [n_elems], storage order),
        with the |g| sampling tables rebuilt (wob_scene_clone + wob_scene_add_boundary_offsets).
        The clone's host copy of the element arrays is formed only when first asked for."""
        lib = load()
        h = C.c_void_p()
        check(lib.wob_scene_clone(self._h, C.byref(h)))
        obj = SceneHost.__new__(SceneHost)
        obj._h, obj.dim, obj.n_elems, obj.n_rhs = h, self.dim, self.n_elems, 0
        obj.element_order = self.element_order.copy()
        on_dev = hasattr(delta, "is_cuda") and delta.is_cuda
        if on_dev:
            check(lib.wob_scene_add_boundary_offsets(h, _ptr(delta), self.n_elems, 1, _stream_ptr(stream)))
            kept = delta.detach().reshape(-1).float().clone()  # a later change to delta leaves the clone's view
        else:
            kept = np.ascontiguousarray(np.asarray(delta, dtype=np.float32).reshape(-1))
            check(lib.wob_scene_add_boundary_offsets(h, kept.ctypes.data, self.n_elems, 0, _stream_ptr(stream)))
        parent = self._host

        def host_arrays():
            d_host = kept.cpu().numpy() if on_dev else kept
            v, nrm, bv, ty, al = parent
            bv2 = bv.copy()
            bv2[obj.element_order] = bv[obj.element_order] + d_host[:, None]  # the same float32 adds
            return (v, nrm, bv2, ty, al)

        obj._host_fn = host_arrays
        return obj

    @property
    def _host(self):
        if self.__dict__.get("_host_arrays") is None:
            self._host_arrays = self._host_fn()
        return self._host_arrays

    @_host.setter
    def _host(self, value):
        self._host_arrays = value

    def info(self) -> dict:
        inf = _capi.wob_scene_info()
        check(load().wob_scene_get_info(self._h, C.byref(inf)))
        return {f: getattr(inf, f) for f, _ in inf._fields_}

    def set_volume_cache(self, grid_res: int, domain_size: float, values) -> None:
        vals = _f32(values).reshape(-1)
        if vals.size != grid_res ** self.dim:
            raise ValueError("values must hold grid_res**dim entries")
        check(load().wob_scene_set_volume_cache(self._h, grid_res, float(domain_size), vals.ctypes.data))
        self._volume = (grid_res, float(domain_size), vals.copy())

    def clear_volume_cache(self) -> None:
        check(load().wob_scene_clear_volume_cache(self._h))
        self._volume = None

    def poll_error(self) -> int:
        bits = C.c_uint32()
        check(load().wob_scene_poll_error(self._h, C.byref(bits)))
        return int(bits.value)

    # ---- solves on device buffers (torch CUDA tensors or raw pointers), asynchronous
    def solve_domain(self, params: EstimatorParams, points, n_points: int, sum_, sumsq=None, bounces=None,
                     stream=None) -> None:
        p = params.to_c()
        check(load().wob_solve_domain(self._h, C.byref(p), _ptr(points), int(n_points), _ptr(sum_), _ptr(sumsq),
                                      _ptr(bounces), _stream_ptr(stream)))

    def solve_boundary(self, params: EstimatorParams, p, n, interior_angle, boundary_value, boundary_type,
                       robin_alpha, n_points: int, sum_, sumsq=None, bounces=None, stream=None) -> None:
        pp = params.to_c()
        check(load().wob_solve_boundary(self._h, C.byref(pp), _ptr(p), _ptr(n), _ptr(interior_angle),
                                        _ptr(boundary_value), _ptr(boundary_type), _ptr(robin_alpha),
                                        int(n_points), _ptr(sum_), _ptr(sumsq), _ptr(bounces), _stream_ptr(stream)))

    def debug_domain_paths(self, params: EstimatorParams, points, n_points: int, values, stream=None) -> None:
        p = params.to_c()
        check(load().wob_debug_domain_paths(self._h, C.byref(p), _ptr(points), int(n_points), _ptr(values),
                                            _stream_ptr(stream)))

    def debug_boundary_paths(self, params: EstimatorParams, p, n, interior_angle, boundary_value, boundary_type,
                             robin_alpha, n_points: int, values, stream=None) -> None:
        pp = params.to_c()
        check(load().wob_debug_boundary_paths(self._h, C.byref(pp), _ptr(p), _ptr(n), _ptr(interior_angle),
                                              _ptr(boundary_value), _ptr(boundary_type), _ptr(robin_alpha),
                                              int(n_points), _ptr(values), _stream_ptr(stream)))

    def autotune_domain(self, params: EstimatorParams, points, n_points: int, stream=None):
        """Times the compiled configurations of the kernel these parameters use and keeps the
        fastest. Returns (chosen index or -1, [ms per configuration])."""
        p = params.to_c()
        chosen = C.c_int32(-1)
        n = C.c_int32(0)
        ms = (C.c_float * 64)()
        check(load().wob_autotune_domain(self._h, C.byref(p), _ptr(points), int(n_points), C.byref(chosen), ms,
                                         C.byref(n), _stream_ptr(stream)))
        return int(chosen.value), [float(ms[i]) for i in range(n.value)]

    def line_query(self, origins, dirs, n_rays: int, counts, hits, hit_points=None, stream=None) -> None:
        check(load().wob_line_query(self._h, _ptr(origins), _ptr(dirs), int(n_rays), _ptr(counts), _ptr(hits),
                                    _ptr(hit_points), _stream_ptr(stream)))

    # ---- multi-RHS walks: several sets of boundary data share one set of paths
    def set_rhs(self, values) -> None:
        """values [n_elems, dim, n_rhs] in the caller's element order (n_rhs <= 64); None removes them."""
        if values is None:
            check(load().wob_scene_set_rhs(self._h, None, 0))
            self.n_rhs = 0
            return
        v = _f32(values)
        if v.ndim != 3 or v.shape[0] != self.n_elems or v.shape[1] != self.dim:
            raise ValueError("values must have shape [n_elems, dim, n_rhs]")
        check(load().wob_scene_set_rhs(self._h, v.ctypes.data, int(v.shape[2])))
        self.n_rhs = int(v.shape[2])

    def solve_domain_multi(self, params: EstimatorParams, points, n_points: int, sum_=None, sumsq=None, bounces=None,
                           per_path=None, stream=None) -> None:
        """u at points for every RHS: sum_ / sumsq [n_points, n_rhs] FP64 (accumulated), per_path
        [n_points, paths, n_rhs] (optional)."""
        p = params.to_c()
        check(load().wob_solve_domain_multi(self._h, C.byref(p), _ptr(points), int(n_points), _ptr(sum_),
                                            _ptr(sumsq), _ptr(bounces), _ptr(per_path), _stream_ptr(stream)))

    def solve_unknown_boundary_multi(self, params: EstimatorParams, p, n, interior_angle, boundary_values,
                                     boundary_type, robin_alpha, n_points: int, sum_=None, sumsq=None, bounces=None,
                                     per_path=None, stream=None) -> None:
        """The unknown boundary function at boundary points for every RHS; boundary_values [n_points, n_rhs]."""
        pp = params.to_c()
        check(load().wob_solve_unknown_boundary_multi(self._h, C.byref(pp), _ptr(p), _ptr(n), _ptr(interior_angle),
                                                      _ptr(boundary_values), _ptr(boundary_type), _ptr(robin_alpha),
                                                      int(n_points), _ptr(sum_), _ptr(sumsq), _ptr(bounces),
                                                      _ptr(per_path), _stream_ptr(stream)))

    def set_rhs_control_variate(self, values) -> None:
        """values [n_elems, n_rhs] in storage order (one control-variate column per RHS)."""
        v = _f32(values)
        if v.ndim != 2:
            raise ValueError("values must have shape [n_elems, n_rhs]")
        check(load().wob_scene_set_rhs_control_variate(self._h, v.ctypes.data, int(v.shape[0]), int(v.shape[1])))

    def solve_domain_multi_cv(self, params: EstimatorParams, n_potential: int, points, n_points: int, sum_=None,
                              sumsq=None, bounces=None, per_path=None, stream=None) -> None:
        p = params.to_c()
        check(load().wob_solve_domain_multi_cv(self._h, C.byref(p), int(n_potential), _ptr(points), int(n_points),
                                               _ptr(sum_), _ptr(sumsq), _ptr(bounces), _ptr(per_path),
                                               _stream_ptr(stream)))

    # ---- walk on spheres (apps/simple_wob_and_wos.cu), 2D Dirichlet scenes
    def solve_wos(self, params: EstimatorParams, points, n_points: int, sum_=None, sumsq=None, queries=None,
                  per_path=None, stream=None) -> None:
        p = params.to_c()
        check(load().wob_solve_wos(self._h, C.byref(p), _ptr(points), int(n_points), _ptr(sum_), _ptr(sumsq),
                                   _ptr(queries), _ptr(per_path), _stream_ptr(stream)))

    def closest_point(self, points, n_points: int, elems, dist2, values, stream=None) -> None:
        check(load().wob_closest_point(self._h, _ptr(points), int(n_points), _ptr(elems), _ptr(dist2), _ptr(values),
                                       _stream_ptr(stream)))

    # ---- virtual point lights (apps/potential_flow_with_vpl.cu)
    def vpl_paths(self, params: EstimatorParams, n_paths: int, vpl_points, vpl_values, bounces=None,
                  stream=None) -> None:
        p = params.to_c()
        check(load().wob_vpl_paths(self._h, C.byref(p), int(n_paths), _ptr(vpl_points), _ptr(vpl_values),
                                   _ptr(bounces), _stream_ptr(stream)))

    def vpl_aggregate(self, eps: float, vpl_points, vpl_values, n_vpl: int, points, n_points: int, sum_,
                      stream=None) -> None:
        check(load().wob_vpl_aggregate(self._h, float(eps), _ptr(vpl_points), _ptr(vpl_values), int(n_vpl),
                                       _ptr(points), int(n_points), _ptr(sum_), _stream_ptr(stream)))

    # ---- host-buffer solve (synchronous), the end-to-end entry point
    def solve_domain_host(self, params: EstimatorParams, points: np.ndarray, sum_=None, sumsq=None):
        pts = _f32(points).reshape(-1, self.dim)
        n = pts.shape[0]
        if sum_ is None:
            sum_ = np.zeros((n, self.dim + 1), dtype=np.float64)
        if sumsq is None:
            sumsq = np.zeros((n, self.dim + 1), dtype=np.float64)
        b = C.c_uint64(0)
        p = params.to_c()
        check(load().wob_solve_domain_host(self._h, C.byref(p), pts.ctypes.data, n, sum_.ctypes.data,
                                           sumsq.ctypes.data, C.byref(b)))
        return sum_, sumsq, int(b.value)

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            load().wob_scene_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SceneBatch:
    """Several scenes (same dimension), each with its own parameters and points, solved in one
    persistent launch. Points / sums are concatenated over the scenes in order."""

    def __init__(self, scenes, params, n_points):
        lib = load()
        n = len(scenes)
        arr = (C.c_void_p * n)(*[s.handle.value for s in scenes])
        prm = (_capi.wob_params * n)(*[p.to_c() for p in params])
        npts = (C.c_uint32 * n)(*[int(x) for x in n_points])
        h = C.c_void_p()
        check(lib.wob_batch_create(arr, prm, npts, n, C.byref(h)))
        self._h = h
        self.scenes = list(scenes)  # keep them alive
        self.offsets = np.concatenate([[0], np.cumsum(np.asarray(n_points, dtype=np.int64))])

    def solve(self, points, sum_, sumsq=None, bounces=None, path_offset_add: int = 0, stream=None) -> None:
        check(load().wob_batch_solve(self._h, _ptr(points), _ptr(sum_), _ptr(sumsq), _ptr(bounces),
                                     int(path_offset_add), _stream_ptr(stream)))

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            load().wob_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
