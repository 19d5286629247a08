"""Learned control variate: a Fourier-feature MLP trained on the engine's own boundary estimates.

Pipeline (all GPU work through the C ABI):
1. training points: uniform samples on the boundary (by area), with their normals and data;
2. labels: the walk's estimate of the unknown boundary density at those points
   (wob_solve_unknown_boundary, the value compute_sample_unknown_boundary returns,
   estimator.cuh:232-357), a few hundred paths each;
3. the MLP (x, n) -> sigma is trained with the engine's forward / backward / Adam kernels
   (BF16 tensor-core GEMMs, FP32 accumulation);
4. the trained network is evaluated at every element centroid (one batched inference) and handed
   to the scene as its control-variate density (wob_scene_set_control_variate), which the
   forward single-layer estimator wob_solve_domain_cv uses without bias.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _capi
from ._capi import check, load

F32 = np.float32


class MLP:
    """Handle on a wob_mlp (see include/wob_capi.h)."""

    def __init__(self, n_freq: int = 32, hidden_layers: int = 4, out_dim: int = 1, freq_sigma: float = 1.0,
                 seed: int = 0):
        h = C.c_void_p()
        check(load().wob_mlp_create(n_freq, hidden_layers, out_dim, float(freq_sigma), int(seed), C.byref(h)))
        self._h = h
        self.n_freq, self.hidden, self.out_dim = n_freq, hidden_layers, out_dim
        n = C.c_uint32()
        check(load().wob_mlp_num_params(h, C.byref(n)))
        self.n_params = int(n.value)

    def params(self):
        p = np.zeros(self.n_params, F32)
        f = np.zeros((self.n_freq, 6), F32)
        check(load().wob_mlp_get_params(self._h, p.ctypes.data, f.ctypes.data))
        return p, f

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=F32)
        check(load().wob_mlp_set_params(self._h, p.ctypes.data))

    def forward(self, inputs, n: int, outputs, stream=None) -> None:
        from . import _ptr, _stream_ptr
        check(load().wob_mlp_forward(self._h, _ptr(inputs), int(n), _ptr(outputs), _stream_ptr(stream)))

    def gradient(self, inputs, targets, n: int, grad, loss=None, stream=None) -> None:
        from . import _ptr, _stream_ptr
        check(load().wob_mlp_gradient(self._h, _ptr(inputs), _ptr(targets), int(n), _ptr(grad), _ptr(loss),
                                      _stream_ptr(stream)))

    def adam_step(self, inputs, targets, n: int, lr: float, loss=None, stream=None) -> None:
        from . import _ptr, _stream_ptr
        check(load().wob_mlp_adam_step(self._h, _ptr(inputs), _ptr(targets), int(n), float(lr), _ptr(loss),
                                       _stream_ptr(stream)))

    def train(self, inputs, targets, n: int, steps: int, batch: int, lr: float, seed: int = 0, loss_history=None,
              stream=None) -> None:
        """`steps` Adam steps on the device (wob_mlp_train): cosine learning-rate decay, batches drawn
        on the device, the step replayed as one CUDA graph."""
        from . import _ptr, _stream_ptr
        check(load().wob_mlp_train(self._h, _ptr(inputs), _ptr(targets), int(n), int(steps), int(batch), float(lr),
                                   int(seed), _ptr(loss_history), _stream_ptr(stream)))

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            load().wob_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def reference_forward(params: np.ndarray, freqs: np.ndarray, inputs: np.ndarray, hidden: int = 4, out_dim: int = 1):
    """The same network in numpy float64 (for checks)."""
    t = inputs.astype(np.float64) @ freqs.astype(np.float64).T
    h = np.concatenate([np.sin(2 * np.pi * t), np.cos(2 * np.pi * t)], axis=1)
    off = 0
    for l in range(hidden + 1):
        fo = out_dim if l == hidden else 64
        W = params[off:off + fo * 64].astype(np.float64).reshape(fo, 64)
        off += fo * 64
        b = params[off:off + fo].astype(np.float64)
        off += fo
        z = h @ W.T + b
        h = z if l == hidden else z / (1 + np.exp(-z))
    return h


def sample_boundary_points(verts: np.ndarray, normals: np.ndarray, bvals: np.ndarray, types: np.ndarray, n: int,
                           seed: int = 0):
    """n points uniform over the boundary area: (p, n, interior_angle 1/2, interpolated data, type)."""
    rng = np.random.default_rng(seed)
    D = verts.shape[1]
    v = verts.astype(np.float64)
    if D == 2:
        area = np.linalg.norm(v[:, 1] - v[:, 0], axis=1)
    else:
        area = 0.5 * np.linalg.norm(np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]), axis=1)
    idx = rng.choice(len(v), size=n, p=area / area.sum())
    if D == 2:
        w = rng.uniform(0, 1, n)
        bary = np.stack([1 - w, w], 1)
    else:
        r1, r2 = np.sqrt(rng.uniform(0, 1, n)), rng.uniform(0, 1, n)
        bary = np.stack([1 - r1, r1 * (1 - r2), r1 * r2], 1)
    p = (v[idx] * bary[:, :, None]).sum(1).astype(F32)
    g = (bvals[idx].astype(np.float64) * bary).sum(1).astype(F32)
    return dict(p=p, n=normals[idx].astype(F32), angle=np.full(n, 0.5, F32), bv=g, type=types[idx].astype(np.int32),
                elem=idx, bary=bary)


def train_density_cv(scene, params, n_train: int = 65536, train_paths: int = 256, steps: int = 2000,
                     batch: int = 8192, lr: float = 2e-3, freq_sigma: float = 1.0, seed: int = 0, device=None,
                     log_every: int = 0, clip_quantile: float | None = 0.999):
    """Steps 1-3 of the module docstring. `params` are backward single-layer parameters of the
    problem (the density the forward estimator transports). The labels are clamped to the
    clip_quantile quantile of their magnitude (wob_clip_magnitude_quantile; None: unclipped) --
    the walk's density estimates are heavy-tailed, and the fit only has to be close, not unbiased,
    for the control variate to stay unbiased. Returns (mlp, info)."""
    import dataclasses

    import torch
    dev = device or torch.device("cuda", torch.cuda.current_device())
    D = scene.dim
    d = {"p": torch.empty(n_train, D, device=dev), "n": torch.empty(n_train, D, device=dev),
         "angle": torch.empty(n_train, device=dev), "bv": torch.empty(n_train, device=dev),
         "type": torch.empty(n_train, dtype=torch.int32, device=dev)}
    # training points uniform by area, drawn on the device (wob_scene_sample_boundary)
    check(load().wob_scene_sample_boundary(scene.handle, n_train, int(seed), d["p"].data_ptr(), d["n"].data_ptr(),
                                           d["angle"].data_ptr(), d["bv"].data_ptr(), d["type"].data_ptr(), None,
                                           None))
    s = torch.zeros(n_train, dtype=torch.float64, device=dev)
    q = torch.zeros_like(s)
    b = torch.zeros(1, dtype=torch.int64, device=dev)
    lp = dataclasses.replace(params, num_sample_paths=train_paths, estimator=0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pp = lp.to_c()
    check(load().wob_solve_unknown_boundary(scene.handle, C.byref(pp), d["p"].data_ptr(), d["n"].data_ptr(),
                                            d["angle"].data_ptr(), d["bv"].data_ptr(), d["type"].data_ptr(), None,
                                            n_train, s.data_ptr(), q.data_ptr(), b.data_ptr(), None))
    torch.cuda.synchronize()
    t_labels = time.perf_counter() - t0
    labels = (s / train_paths).float().contiguous()
    label_var = (q / train_paths - (s / train_paths) ** 2).clamp(min=0) / train_paths
    clip_t = torch.zeros(1, dtype=torch.float32, device=dev)
    if clip_quantile is not None:
        check(load().wob_clip_magnitude_quantile(labels.data_ptr(), n_train, float(clip_quantile), clip_t.data_ptr(),
                                                 None))
    x = torch.cat([d["p"], d["n"]], dim=1).contiguous()
    if scene.dim == 2:  # (x, y, 0, nx, ny, 0)
        z = torch.zeros(n_train, 1, device=dev)
        x = torch.cat([d["p"], z, d["n"], z], dim=1).contiguous()
    mlp = MLP(32, 4, 1, freq_sigma, seed)
    loss_hist = torch.zeros(steps, dtype=torch.float32, device=dev)
    labels = labels.contiguous()
    t1 = time.perf_counter()
    mlp.train(x, labels, n_train, steps, batch, lr, seed=seed, loss_history=loss_hist)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    lh = loss_hist.cpu().numpy()
    every = log_every or max(1, steps // 20)
    hist = [(int(i), float(lh[i])) for i in range(0, steps, every)] + [(steps - 1, float(lh[-1]))]
    info = dict(n_train=n_train, train_paths=train_paths, steps=steps, batch=batch, t_labels_s=t_labels,
                t_train_s=t_train, label_noise_var=float(label_var.mean().item()), history=hist,
                label_bounces=int(b.item()), clip_quantile=clip_quantile,
                clip_threshold=float(clip_t.item()) if clip_quantile is not None else None)
    return mlp, info


def train_density_cv_multi(scene, rhs_table: np.ndarray, params, n_train: int = 131072, train_paths: int = 128,
                           steps: int = 2000, batch: int = 8192, lr: float = 2e-3, freq_sigma: float = 1.0,
                           seed: int = 0, device=None):
    """The multi-RHS variant of train_density_cv: one network with an n_rhs-wide head. Labels are the
    unknown boundary function of every RHS at the training points from one set of shared walks
    (wob_solve_unknown_boundary_multi); rhs_table [n_elems, dim, n_rhs] in the caller's element
    order (the table given to scene.set_rhs). Returns (mlp, info)."""
    import dataclasses

    import torch
    dev = device or torch.device("cuda", torch.cuda.current_device())
    v, nrm, bv, ty, _ = scene._host[:5]
    R = rhs_table.shape[2]
    bp = sample_boundary_points(v, nrm, bv, ty, n_train, seed)
    # data of every RHS at the training points: the same barycentric interpolation per RHS
    data = np.einsum("nk,nkr->nr", bp["bary"].astype(np.float64),
                     rhs_table[bp["elem"]].astype(np.float64)).astype(F32)
    d = {k: torch.from_numpy(np.ascontiguousarray(bp[k])).to(dev) for k in ("p", "n", "angle", "type")}
    d_data = torch.from_numpy(np.ascontiguousarray(data)).to(dev)
    s = torch.zeros(n_train, R, dtype=torch.float64, device=dev)
    b = torch.zeros(1, dtype=torch.int64, device=dev)
    lp = dataclasses.replace(params, num_sample_paths=train_paths)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    scene.solve_unknown_boundary_multi(lp, d["p"], d["n"], d["angle"], d_data, d["type"], None, n_train, s, None, b)
    torch.cuda.synchronize()
    t_labels = time.perf_counter() - t0
    labels = (s / train_paths).float().contiguous()
    x = torch.cat([d["p"], d["n"]], dim=1).contiguous()
    if scene.dim == 2:
        z = torch.zeros(n_train, 1, device=dev)
        x = torch.cat([d["p"], z, d["n"], z], dim=1).contiguous()
    mlp = MLP(32, 4, R, freq_sigma, seed)
    loss = torch.zeros(1, dtype=torch.float32, device=dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    t1 = time.perf_counter()
    for it in range(steps):
        idx = torch.randint(0, n_train, (batch,), device=dev, generator=gen)
        cur_lr = lr * 0.5 * (1 + np.cos(np.pi * it / steps))
        mlp.adam_step(x[idx].contiguous(), labels[idx].contiguous(), batch, cur_lr, loss)
        loss.zero_()
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    info = dict(n_train=n_train, train_paths=train_paths, steps=steps, batch=batch, t_labels_s=t_labels,
                t_train_s=t_train, label_bounces=int(b.item()),
                label_mean_abs=float(labels.abs().mean().item()))
    return mlp, info


def element_cv_table(mlp: MLP, scene, device=None) -> np.ndarray:
    """The network at every stored element's centroid (with its normal), storage order:
    [n_elems] for a scalar head, [n_elems, out_dim] otherwise."""
    import torch
    dev = device or torch.device("cuda", torch.cuda.current_device())
    v, nrm, _, _, _ = scene.stored_arrays()
    c = v.astype(np.float64).mean(1).astype(F32)
    if scene.dim == 2:
        z = np.zeros((len(c), 1), F32)
        inp = np.concatenate([c, z, nrm, z], 1)
    else:
        inp = np.concatenate([c, nrm], 1)
    x = torch.from_numpy(np.ascontiguousarray(inp, dtype=F32)).to(dev)
    out = torch.zeros(len(c), mlp.out_dim, dtype=torch.float32, device=dev)
    mlp.forward(x, len(c), out)
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    return o[:, 0].copy() if mlp.out_dim == 1 else o


def centroid_inputs(scene, device=None):
    """(centroid, normal) of every stored element, the network's input there: device tensor [n, 6]
    (2D scenes padded with zeros), storage order (wob_scene_element_frames)."""
    import torch
    from . import _ptr
    dev = device or torch.device("cuda", torch.cuda.current_device())
    out = torch.empty(scene.n_elems, 6, dtype=torch.float32, device=dev)
    check(load().wob_scene_element_frames(scene.handle, _ptr(out), None))
    return out


def residual_control_variate(scene, mlp: MLP, domain: int, near_factor: float = 3.0, theta: float = 0.3,
                             stream=None):
    """The residual control variate of a single-layer Neumann problem (wob_cv_residual_data):
    sigma~ = the network at every stored triangle's centroid, constant on the triangle; returns
    (residual scene, sigma~) where the residual scene is a copy of `scene` whose Neumann data
    carries the offsets delta = (T sigma~ - sigma~) / c. The forward estimator on the residual
    scene plus control_variate_potential(sigma~) estimates u. theta: cluster acceptance of the
    far field (0: every triangle)."""
    import torch
    from . import _ptr, _stream_ptr
    x = centroid_inputs(scene)
    n = scene.n_elems
    sigma = torch.zeros(n, mlp.out_dim, dtype=torch.float32, device=x.device)
    mlp.forward(x, n, sigma, stream)
    sigma = sigma[:, 0].contiguous()
    delta = torch.zeros(n, dtype=torch.float32, device=x.device)
    check(load().wob_cv_residual_data(scene.handle, _ptr(sigma), int(domain), float(near_factor), float(theta),
                                      _ptr(delta), _stream_ptr(stream)))
    return scene.clone_with_offsets(delta, stream), sigma


def control_variate_potential(scene, sigma, points, n_points: int, near_factor: float = 3.0, theta: float = 0.3,
                              stream=None):
    """S sigma~ and its gradient at points (wob_cv_potential): device tensor [n_points, 4]."""
    import torch
    from . import _ptr, _stream_ptr
    out = torch.zeros(n_points, 4, dtype=torch.float32, device=sigma.device)
    check(load().wob_cv_potential(scene.handle, _ptr(sigma), float(near_factor), float(theta), _ptr(points),
                                  int(n_points), _ptr(out), _stream_ptr(stream)))
    return out


def set_control_variate(scene, values: np.ndarray) -> None:
    vals = np.ascontiguousarray(values, dtype=F32)
    check(load().wob_scene_set_control_variate(scene.handle, vals.ctypes.data, len(vals)))


def solve_domain_cv(scene, params, points, n_points: int, sum_, sumsq=None, bounces=None, n_potential: int = 16,
                    n_kernel: int = 16, per_path=None, stream=None) -> None:
    from . import _ptr, _stream_ptr
    p = params.to_c()
    check(load().wob_solve_domain_cv(scene.handle, C.byref(p), int(n_potential), int(n_kernel), _ptr(points),
                                     int(n_points), _ptr(sum_), _ptr(sumsq), _ptr(bounces), _ptr(per_path),
                                     _stream_ptr(stream)))


_ = _capi  # the ctypes declarations live in _capi
