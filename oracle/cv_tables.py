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

With theta > 0 the kernels also take whole clusters (32 consecutive stored triangles) by the
quadrupole expansion of their centroid sources about the cluster's mean centroid z, wherever the
cluster is farther than max(rho / theta, rho + eta) (rho: its radius about z, eta: its largest
near radius) plus omega from the centre W of the 32 consecutive targets of a warp (omega: their
radius about W), the triangles in storage order and the evaluation points in Morton order
(_morton_order). The same test is made first for groups of 8 clusters (256 triangles) and groups of
8 of those (2048 triangles), with records of the same form from their member sources: a far group
is one expansion, a near one is looked into (_hierarchy_split). _cluster_far restates the decision
and _cluster_field the expansion.
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


def _clusters(cen, w, near2, theta, size=32):
    """Per cluster: centre z, far radius, M0, M1, M2 (float64)."""
    nc = (len(cen) + size - 1) // size
    z = np.zeros((nc, 3)); r_far = np.full(nc, np.inf); M0 = np.zeros(nc); M1 = np.zeros((nc, 3))
    M2 = np.zeros((nc, 3, 3))
    for k in range(nc):
        sl = slice(k * size, min(len(cen), (k + 1) * size))
        z[k] = cen[sl].mean(0)
        d = cen[sl] - z[k]
        rho = np.sqrt((d ** 2).sum(1)).max()
        eta = np.sqrt(near2[sl].max())
        if theta > 0:
            r_far[k] = max(rho / theta, rho + eta)
        M0[k] = w[sl].sum()
        M1[k] = (w[sl, None] * d).sum(0)
        M2[k] = np.einsum("i,ij,ik->jk", w[sl], d, d)
    return z, r_far, M0, M1, M2


def _cluster_far(x_group, z, r_far):
    W = x_group.mean(0)
    om = np.sqrt(((x_group - W) ** 2).sum(1)).max()
    return ((W - z) ** 2).sum(1) > (r_far + om) ** 2


def _cluster_field(x, z, M0, M1, M2):
    """sum over the given clusters of the quadrupole expansion of sum w / |x - c| and its gradient,
    for points x [m, 3]: returns phi [m], grad [m, 3]."""
    R = x[:, None, :] - z[None, :, :]
    R2 = (R ** 2).sum(-1)
    Rn = np.sqrt(R2)
    RM1 = (R * M1[None]).sum(-1)
    M2R = np.einsum("kij,mkj->mki", M2, R)
    RM2R = (R * M2R).sum(-1)
    t = np.trace(M2, axis1=1, axis2=2)[None, :]
    Q = 3 * RM2R - R2 * t
    phi = (M0[None] / Rn + RM1 / Rn ** 3 + Q / (2 * Rn ** 5)).sum(1)
    a = -M0[None] / Rn ** 3 - 3 * RM1 / Rn ** 5 - t / Rn ** 5 - 2.5 * Q / Rn ** 7
    g = (a[..., None] * R + M1[None] / Rn[..., None] ** 3 + 3 * M2R / Rn[..., None] ** 5).sum(1)
    return phi, g


def _morton_order(points):
    """The engine's Morton order of evaluation points: 10 bits a coordinate of (p - lo) / (hi - lo)
    in float32 over the points' bounds, codes interleaved x, y, z from the low bit, ties by index."""
    p = np.asarray(points, np.float32)
    lo, hi = p.min(0), p.max(0)
    code = np.zeros(len(p), np.uint64)
    for k in range(3):
        if hi[k] > lo[k]:
            t = (p[:, k] - lo[k]) / np.float32(hi[k] - lo[k])
        else:
            t = np.zeros(len(p), np.float32)
        q = np.minimum(np.maximum(t * np.float32(1024.0), np.float32(0.0)), np.float32(1023.0)).astype(np.uint64)
        for b in range(10):
            code |= ((q >> np.uint64(b)) & np.uint64(1)) << np.uint64(3 * b + k)
    return np.lexsort((np.arange(len(p)), code))


def _cluster_split(tx, cen, w, near2, theta, size=32, order=None, fan=8, return_cover=False):
    """Per target: the far records' expansion (phi, grad) and the mask [targets, sources] of the
    sources still summed pair by pair, for targets tx in warps of 32 consecutive ones. Records of
    three sizes (size, size * fan, size * fan^2 consecutive sources); one is taken when it is far
    and none of its ancestors is (k_cv_tables.cu's cv_sum_kernel). With return_cover, also the
    number of sources inside the records taken for each target (each source must be counted once:
    inside one taken record or summed pair by pair)."""
    levels = [_clusters(cen, w, near2, theta, size * fan ** L) for L in range(3)]
    phi = np.zeros(len(tx)); g = np.zeros((len(tx), 3))
    pair = np.ones((len(tx), len(cen)), bool)
    cover = np.zeros(len(tx), np.int64)
    order = np.arange(len(tx)) if order is None else order
    for g0 in range(0, len(tx), 32):
        grp = order[g0:g0 + 32]
        covered = None  # per level-0 record: inside a record already taken
        for L in (2, 1, 0):
            z, r_far, M0, M1, M2 = levels[L]
            far = _cluster_far(tx[grp], z, r_far)
            if covered is not None:  # ancestors at level L + 1: record k's parent is k // fan
                far &= ~covered[np.arange(len(z)) // fan]
            if far.any():
                ph, gr = _cluster_field(tx[grp], z[far], M0[far], M1[far], M2[far])
                phi[grp] += ph
                g[grp] += gr
                span = size * fan ** L
                for k in np.nonzero(far)[0]:
                    members = np.arange(k * span, min(len(cen), (k + 1) * span))
                    pair[np.ix_(grp, members)] = False
                    cover[grp] += len(members)
            covered = far if covered is None else (far | covered[np.arange(len(z)) // fan])
    if return_cover:
        return phi, g, pair, cover
    return phi, g, pair


def residual_data(verts, normals, sigma, c_coef: float, near_factor: float, chunk: int = 256, theta: float = 0.0):
    """delta_j = ((T sigma~)(c_j) - sigma~_j) / c for every triangle j of the stored arrays, with the
    kernel's split: closed form for pairs with |c_j - c_i|^2 < near_factor^2 h_i^2 (h_i the longest
    edge of i), centroid rule otherwise, the triangle's own term zero (k_cv_tables.cu)."""
    a, b, c, cen, area, h2 = _tri_arrays(verts)
    n = np.asarray(normals, np.float64)
    sig = np.asarray(sigma, np.float64)
    near2 = near_factor ** 2 * h2
    out = np.zeros(len(cen))
    if theta > 0:
        _, cg, pair = _cluster_split(cen, cen, area * sig, near2, theta)
    else:
        cg, pair = np.zeros((len(cen), 3)), None
    for j0 in range(0, len(cen), chunk):
        j1 = min(len(cen), j0 + chunk)
        d = cen[j0:j1, None, :] - cen[None, :, :]
        r2 = (d ** 2).sum(-1)
        take = np.ones(r2.shape, bool) if pair is None else pair[j0:j1]
        near = (r2 < near2[None, :]) & take
        with np.errstate(divide="ignore", invalid="ignore"):
            far = np.where(near | ~take, 0.0, (d * n[j0:j1, None, :]).sum(-1) / r2 ** 1.5 * (area * sig)[None, :])
        acc = far.sum(1) - (cg[j0:j1] * n[j0:j1]).sum(1)
        jj, ii = np.nonzero(near)
        jj = jj + j0
        keep = jj != ii
        jj, ii = jj[keep], ii[keep]
        _, G = triangle_potential(cen[jj], a[ii], b[ii], c[ii])
        np.add.at(acc, jj - j0, -sig[ii] * (G * n[jj]).sum(-1))
        tsig = c_coef / (4 * np.pi) * acc
        out[j0:j1] = (tsig - sig[j0:j1]) / c_coef
    return out


def potential(verts, sigma, points, near_factor: float, chunk: int = 128, theta: float = 0.0):
    """u~(x) = (1/4 pi) sum_i sigma~_i P_i(x) and its gradient at points ([n, 4]), same split."""
    a, b, c, cen, area, h2 = _tri_arrays(verts)
    sig = np.asarray(sigma, np.float64)
    x = np.asarray(points, np.float64)
    near2 = near_factor ** 2 * h2
    out = np.zeros((len(x), 4))
    if theta > 0:
        cphi, cg, pair = _cluster_split(x, cen, area * sig, near2, theta, order=_morton_order(points))
    else:
        cphi, cg, pair = np.zeros(len(x)), np.zeros((len(x), 3)), None
    for p0 in range(0, len(x), chunk):
        p1 = min(len(x), p0 + chunk)
        d = x[p0:p1, None, :] - cen[None, :, :]
        r2 = (d ** 2).sum(-1)
        take = np.ones(r2.shape, bool) if pair is None else pair[p0:p1]
        near = (r2 < near2[None, :]) & take
        w = (area * sig)[None, :]
        with np.errstate(divide="ignore", invalid="ignore"):
            u = np.where(near | ~take, 0.0, w / np.sqrt(r2))
            gr = np.where((near | ~take)[..., None], 0.0, -w[..., None] * d / r2[..., None] ** 1.5)
        acc = np.concatenate([(u.sum(1) + cphi[p0:p1])[:, None], gr.sum(1) + cg[p0:p1]], 1)
        pj, ii = np.nonzero(near)
        P, G = triangle_potential(x[p0 + pj], a[ii], b[ii], c[ii])
        np.add.at(acc, pj, np.concatenate([(sig[ii] * P)[:, None], sig[ii][:, None] * G], 1))
        out[p0:p1] = acc / (4 * np.pi)
    return out
