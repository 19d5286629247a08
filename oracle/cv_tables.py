"""Float64 restatement of the control-variate tables (TEST INFRASTRUCTURE ONLY).

The learned control variate of the single-layer Neumann workloads is a density that is constant
on each boundary triangle. Its single-layer potential and the normal derivative of that potential
on the boundary are sums over triangles of the potential of a uniformly charged flat triangle,

    P_T(x) = integral over T of 1 / |x - y| dA(y),

and of its gradient. Both have closed forms (Wilton, Rao, Glisson, Schaubert, Al-Bundak, Butler,
"Potential integrals for uniform and linear source distributions on polygonal and polyhedral
domains", IEEE Trans. Antennas Propag. 32(3), 1984): with h the signed height of x over the
triangle's plane (unit normal n), rho the projection of x onto the plane, and for every edge from
a to b the unit direction s, the in-plane outward normal m = s x n, s- = (a - rho).s,
s+ = (b - rho).s, t = (a - rho).m, R0^2 = t^2 + h^2, R- = |x - a|, R+ = |x - b|,

    f    = ln((R+ + s+) / (R- + s-)),
    beta = atan(t s+ / (R0^2 + |h| R+)) - atan(t s- / (R0^2 + |h| R-)),
    P    = sum over edges (t f - |h| beta),
    grad P = - sum over edges m f - sign(h) n sum over edges beta.

The engine's kernels (csrc/k_cv_tables.cu) evaluate these for triangles near the target and the
one-point (centroid) rule A_T / |x - c_T| far away; residual_data and potential below evaluate the
same split in float64 for the tests, and with near_factor large the closed forms everywhere.
"""
from __future__ import annotations

import numpy as np


def _edge_log(Rp, sp, Rm, sm):
    """ln((R+ + s+)/(R- + s-)) without cancellation when the edge points away from rho."""
    with np.errstate(divide="ignore", invalid="ignore"):
        a = np.log((Rp + sp) / (Rm + sm))
        b = np.log((Rm - sm) / (Rp - sp))
    return np.where(sm + sp >= 0, a, b)


def triangle_potential(x, a, b, c):
    """P_T(x) and grad P_T(x) for points x [n, 3] and triangles (a, b, c) [n, 3] (broadcast)."""
    x, a, b, c = (np.asarray(v, np.float64) for v in (x, a, b, c))
    nrm = np.cross(b - a, c - a)
    n = nrm / np.linalg.norm(nrm, axis=-1, keepdims=True)
    h = ((x - a) * n).sum(-1)
    rho = x - h[..., None] * n
    P = np.zeros(np.broadcast(h, h).shape)
    G = np.zeros(P.shape + (3,))
    beta_sum = np.zeros_like(P)
    ah = np.abs(h)
    for p0, p1 in ((a, b), (b, c), (c, a)):
        e = p1 - p0
        s = e / np.linalg.norm(e, axis=-1, keepdims=True)
        m = np.cross(s, n)
        sm = ((p0 - rho) * s).sum(-1)
        sp = ((p1 - rho) * s).sum(-1)
        t = ((p0 - rho) * m).sum(-1)
        R0sq = t * t + h * h
        Rm = np.linalg.norm(x - p0, axis=-1)
        Rp = np.linalg.norm(x - p1, axis=-1)
        f = _edge_log(Rp, sp, Rm, sm)
        f = np.where(R0sq > 0, f, 0.0)
        with np.errstate(divide="ignore", invalid="ignore"):
            beta = np.arctan(t * sp / (R0sq + ah * Rp)) - np.arctan(t * sm / (R0sq + ah * Rm))
        beta = np.where(R0sq > 0, beta, 0.0)
        P += t * f - ah * beta
        G -= m * f[..., None]
        beta_sum += beta
    G -= (np.sign(h) * beta_sum)[..., None] * n
    return P, G


def quadrature_potential(x, a, b, c, levels: int = 6):
    """The same integrals by the centroid rule on 4^levels sub-triangles (for checking)."""
    x = np.asarray(x, np.float64)
    tris = [(np.asarray(a, np.float64), np.asarray(b, np.float64), np.asarray(c, np.float64))]
    for _ in range(levels):
        nxt = []
        for p, q, r in tris:
            pq, qr, rp = (p + q) / 2, (q + r) / 2, (r + p) / 2
            nxt += [(p, pq, rp), (pq, q, qr), (rp, qr, r), (pq, qr, rp)]
        tris = nxt
    P = 0.0
    G = np.zeros(3)
    for p, q, r in tris:
        A = 0.5 * np.linalg.norm(np.cross(q - p, r - p))
        d = x - (p + q + r) / 3
        R = np.linalg.norm(d)
        P += A / R
        G += -A * d / R ** 3
    return P, G


def _tri_arrays(verts):
    v = np.asarray(verts, np.float64)
    a, b, c = v[:, 0], v[:, 1], v[:, 2]
    cen = (a + b + c) / 3.0
    area = 0.5 * np.linalg.norm(np.cross(b - a, c - a), axis=1)
    h2 = np.max(np.stack([((b - a) ** 2).sum(1), ((c - b) ** 2).sum(1), ((a - c) ** 2).sum(1)], 1), 1)
    return a, b, c, cen, area, h2


def residual_data(verts, normals, sigma, c_coef: float, near_factor: float, chunk: int = 256):
    """delta_j = ((T sigma~)(c_j) - sigma~_j) / c for every triangle j of the stored arrays, with the
    kernel's split: closed form for pairs with |c_j - c_i|^2 < near_factor^2 h_i^2 (h_i the longest
    edge of i), centroid rule otherwise, the triangle's own term zero (k_cv_tables.cu)."""
    a, b, c, cen, area, h2 = _tri_arrays(verts)
    n = np.asarray(normals, np.float64)
    sig = np.asarray(sigma, np.float64)
    near2 = near_factor ** 2 * h2
    out = np.zeros(len(cen))
    for j0 in range(0, len(cen), chunk):
        j1 = min(len(cen), j0 + chunk)
        d = cen[j0:j1, None, :] - cen[None, :, :]
        r2 = (d ** 2).sum(-1)
        near = r2 < near2[None, :]
        with np.errstate(divide="ignore", invalid="ignore"):
            far = np.where(near, 0.0, (d * n[j0:j1, None, :]).sum(-1) / r2 ** 1.5 * (area * sig)[None, :])
        acc = far.sum(1)
        jj, ii = np.nonzero(near)
        jj = jj + j0
        keep = jj != ii
        jj, ii = jj[keep], ii[keep]
        _, G = triangle_potential(cen[jj], a[ii], b[ii], c[ii])
        np.add.at(acc, jj - j0, -sig[ii] * (G * n[jj]).sum(-1))
        tsig = c_coef / (4 * np.pi) * acc
        out[j0:j1] = (tsig - sig[j0:j1]) / c_coef
    return out


def potential(verts, sigma, points, near_factor: float, chunk: int = 128):
    """u~(x) = (1/4 pi) sum_i sigma~_i P_i(x) and its gradient at points ([n, 4]), same split."""
    a, b, c, cen, area, h2 = _tri_arrays(verts)
    sig = np.asarray(sigma, np.float64)
    x = np.asarray(points, np.float64)
    near2 = near_factor ** 2 * h2
    out = np.zeros((len(x), 4))
    for p0 in range(0, len(x), chunk):
        p1 = min(len(x), p0 + chunk)
        d = x[p0:p1, None, :] - cen[None, :, :]
        r2 = (d ** 2).sum(-1)
        near = r2 < near2[None, :]
        w = (area * sig)[None, :]
        with np.errstate(divide="ignore", invalid="ignore"):
            u = np.where(near, 0.0, w / np.sqrt(r2))
            gr = np.where(near[..., None], 0.0, -w[..., None] * d / r2[..., None] ** 1.5)
        acc = np.concatenate([u.sum(1)[:, None], gr.sum(1)], 1)
        pj, ii = np.nonzero(near)
        P, G = triangle_potential(x[p0 + pj], a[ii], b[ii], c[ii])
        np.add.at(acc, pj, np.concatenate([(sig[ii] * P)[:, None], sig[ii][:, None] * G], 1))
        out[p0:p1] = acc / (4 * np.pi)
    return out
