// C entry points of the CPU oracle (TEST INFRASTRUCTURE ONLY; see wob_oracle.hpp).
// Called through ctypes by tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py.
//
// Elements are passed in the engine's storage order, as SoA arrays with the layout of
// wob_scene_create; the parameter block has the layout of wob_params.
#include "wob_oracle.hpp"
#include "lbvh_count.hpp"

#include <chrono>
#include <cstdint>
#include <cstring>
#include <memory>
#include <type_traits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using namespace wob_oracle;

extern "C" {

struct oracle_params {  // same layout as wob_params
    int32_t bie_model, domain, estimator, problem;
    uint32_t path_length, num_sample_paths, num_resampling_candidates, num_volume_samples;
    float eps, first_kind_equation_scaling_constant;
    uint64_t seed, path_offset;
    uint32_t point_offset, flags;
};

}  // extern "C"

namespace {

template <int D>
void fill_elements(Scene<D> &s, uint32_t n, const float *verts, const float *normals, const float *bvals,
                   const float *alphas, const int32_t *types) {
    s.elems.resize(n);
    for (uint32_t i = 0; i < n; i++) {
        Element<D> &e = s.elems[i];
        for (int j = 0; j < D; j++)
            for (int k = 0; k < D; k++) e.v[j].v[k] = verts[((size_t)i * D + j) * D + k];
        for (int k = 0; k < D; k++) e.n.v[k] = normals[(size_t)i * D + k];
        for (int k = 0; k < D; k++) e.bv[k] = bvals[(size_t)i * D + k];
        for (int k = 0; k < D; k++) e.alpha[k] = alphas ? alphas[(size_t)i * D + k] : 0.0f;
        e.type = types[i];
    }
    s.build();
}

Params to_params(const oracle_params *p) {
    Params r;
    r.bie = p->bie_model;
    r.domain = p->domain;
    r.estimator = p->estimator;
    r.problem = p->problem;
    r.path_length = p->path_length;
    r.num_resampling_candidates = p->num_resampling_candidates;
    r.num_volume_samples = p->num_volume_samples;
    r.eps = p->eps;
    r.fk = p->first_kind_equation_scaling_constant;
    return r;
}

int set_threads(int n_threads) {
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
    return omp_get_max_threads();
#else
    (void)n_threads;
    return 1;
#endif
}

template <int D>
uint64_t solve_domain(const Scene<D> &s, const oracle_params *op, const float *points, uint32_t n_points,
                      double *sum, double *sumsq, float *per_path) {
    const Params prm = to_params(op);
    const uint32_t P = op->num_sample_paths;
    uint64_t total_bounces = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total_bounces)
    for (int64_t ii = 0; ii < (int64_t)n_points; ii++) {
        const uint32_t i = (uint32_t)ii;
        Vec<D> x;
        for (int k = 0; k < D; k++) x.v[k] = points[(size_t)i * D + k];
        double s_[D + 1] = {}, q_[D + 1] = {};
        for (uint32_t j = 0; j < P; j++) {
            Rng rng(op->seed, kStreamDomain, op->point_offset + i, op->path_offset + j);
            Estimator<D> est(&s, prm, &rng);
            float out[D + 1];
            est.domain(x, out);
            total_bounces += est.bounces;
            for (int c = 0; c <= D; c++) {
                s_[c] += (double)out[c];
                q_[c] += (double)out[c] * (double)out[c];
            }
            if (per_path)
                for (int c = 0; c <= D; c++) per_path[((size_t)i * P + j) * (D + 1) + c] = out[c];
        }
        if (sum)
            for (int c = 0; c <= D; c++) sum[(size_t)i * (D + 1) + c] += s_[c];
        if (sumsq)
            for (int c = 0; c <= D; c++) sumsq[(size_t)i * (D + 1) + c] += q_[c];
    }
    return total_bounces;
}

template <int D>
uint64_t solve_boundary(const Scene<D> &s, const oracle_params *op, const float *p, const float *n,
                        const float *angle, const float *bv, const int32_t *type, const float *alpha,
                        uint32_t n_points, double *sum, double *sumsq, float *per_path) {
    const Params prm = to_params(op);
    const uint32_t P = op->num_sample_paths;
    uint64_t total_bounces = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total_bounces)
    for (int64_t ii = 0; ii < (int64_t)n_points; ii++) {
        const uint32_t i = (uint32_t)ii;
        BoundaryPoint<D> x;
        for (int k = 0; k < D; k++) {
            x.p.v[k] = p[(size_t)i * D + k];
            x.n.v[k] = n[(size_t)i * D + k];
        }
        x.interior_angle = angle[i];
        x.boundary_value = bv[i];
        x.boundary_type = type[i];
        x.robin_alpha = alpha ? alpha[i] : 0.0f;
        double s_ = 0.0, q_ = 0.0;
        for (uint32_t j = 0; j < P; j++) {
            Rng rng(op->seed, kStreamBoundary, op->point_offset + i, op->path_offset + j);
            Estimator<D> est(&s, prm, &rng);
            const float v = est.boundary(x);
            total_bounces += est.bounces;
            s_ += (double)v;
            q_ += (double)v * (double)v;
            if (per_path) per_path[(size_t)i * P + j] = v;
        }
        if (sum) sum[i] += s_;
        if (sumsq) sumsq[i] += q_;
    }
    return total_bounces;
}

template <int D>
uint64_t solve_domain_cv(const Scene<D> &s, const oracle_params *op, const float *sigma_t, unsigned n_pot,
                         unsigned m_ker, const float *points, uint32_t n_points, double *sum, double *sumsq,
                         float *per_path) {
    const Params prm = to_params(op);
    const uint32_t P = op->num_sample_paths;
    uint64_t total_bounces = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total_bounces)
    for (int64_t ii = 0; ii < (int64_t)n_points; ii++) {
        const uint32_t i = (uint32_t)ii;
        Vec<D> x;
        for (int k = 0; k < D; k++) x.v[k] = points[(size_t)i * D + k];
        double s_[D + 1] = {}, q_[D + 1] = {};
        for (uint32_t j = 0; j < P; j++) {
            Rng rng(op->seed, kStreamDomain, op->point_offset + i, op->path_offset + j);
            Estimator<D> est(&s, prm, &rng);
            float out[D + 1];
            est.domain_cv(x, sigma_t, n_pot, m_ker, out);
            total_bounces += est.bounces;
            for (int c = 0; c <= D; c++) {
                s_[c] += (double)out[c];
                q_[c] += (double)out[c] * (double)out[c];
            }
            if (per_path)
                for (int c = 0; c <= D; c++) per_path[((size_t)i * P + j) * (D + 1) + c] = out[c];
        }
        if (sum) for (int c = 0; c <= D; c++) sum[(size_t)i * (D + 1) + c] += s_[c];
        if (sumsq) for (int c = 0; c <= D; c++) sumsq[(size_t)i * (D + 1) + c] += q_[c];
    }
    return total_bounces;
}

template <int D>
uint64_t solve_domain_bcv(const Scene<D> &s, const oracle_params *op, const float *cv, unsigned n_pot,
                          const float *points, uint32_t n_points, double *sum, double *sumsq, float *per_path) {
    const Params prm = to_params(op);
    const uint32_t P = op->num_sample_paths;
    uint64_t total_bounces = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total_bounces)
    for (int64_t ii = 0; ii < (int64_t)n_points; ii++) {
        const uint32_t i = (uint32_t)ii;
        Vec<D> x;
        for (int k = 0; k < D; k++) x.v[k] = points[(size_t)i * D + k];
        double s_ = 0.0, q_ = 0.0;
        for (uint32_t j = 0; j < P; j++) {
            Rng rng(op->seed, kStreamDomain, op->point_offset + i, op->path_offset + j);
            Estimator<D> est(&s, prm, &rng);
            const float out = est.domain_bcv(x, cv, n_pot);
            total_bounces += est.bounces;
            s_ += (double)out;
            q_ += (double)out * (double)out;
            if (per_path) per_path[(size_t)i * P + j] = out;
        }
        if (sum) sum[i] += s_;
        if (sumsq) sumsq[i] += q_;
    }
    return total_bounces;
}

template <int D>
uint64_t solve_unknown(const Scene<D> &s, const oracle_params *op, const float *p, const float *n,
                       const float *angle, const float *bv, const int32_t *type, const float *alpha,
                       uint32_t n_points, double *sum, float *per_path) {
    const Params prm = to_params(op);
    const uint32_t P = op->num_sample_paths;
    uint64_t total_bounces = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total_bounces)
    for (int64_t ii = 0; ii < (int64_t)n_points; ii++) {
        const uint32_t i = (uint32_t)ii;
        BoundaryPoint<D> x;
        for (int k = 0; k < D; k++) { x.p.v[k] = p[(size_t)i * D + k]; x.n.v[k] = n[(size_t)i * D + k]; }
        x.interior_angle = angle[i]; x.boundary_value = bv[i]; x.boundary_type = type[i];
        x.robin_alpha = alpha ? alpha[i] : 0.0f;
        double s_ = 0.0;
        for (uint32_t j = 0; j < P; j++) {
            Rng rng(op->seed, kStreamBoundary, op->point_offset + i, op->path_offset + j);
            Estimator<D> est(&s, prm, &rng);
            const float v = est.unknown_boundary(x);
            total_bounces += est.bounces;
            s_ += (double)v;
            if (per_path) per_path[(size_t)i * P + j] = v;
        }
        if (sum) sum[i] += s_;
    }
    return total_bounces;
}

// Box padding of the line-query filter: 1e-5 (extent + max |coordinate|), far above the rounding of
// the box test, so it never drops an element the exact test accepts.
template <int D> float accel_pad(const Scene<D> &s) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY}, mag = 0.0f;
    for (const Element<D> &e : s.elems)
        for (int j = 0; j < D; j++)
            for (int k = 0; k < D; k++) {
                lo[k] = std::min(lo[k], e.v[j].v[k]);
                hi[k] = std::max(hi[k], e.v[j].v[k]);
                mag = std::max(mag, std::fabs(e.v[j].v[k]));
            }
    float ext = 0.0f;
    for (int k = 0; k < D; k++) ext = std::max(ext, hi[k] - lo[k]);
    return 1e-5f * (ext + mag) + 1e-30f;
}

template <int D> struct Holder {
    Scene<D> scene;
    VolumeCache<D> vol;
};

}  // namespace

extern "C" {

// Domain estimator. vol_res == 0: no volume cache. Returns the number of executed bounces.
uint64_t oracle_solve_domain(int dim, uint32_t n_elems, const float *verts, const float *normals, const float *bvals,
                             const float *alphas, const int32_t *types, uint32_t vol_res, float vol_size,
                             const float *vol_values, const oracle_params *params, const float *points,
                             uint32_t n_points, double *sum, double *sumsq, float *per_path, int n_threads) {
    set_threads(n_threads);
    // flags bit 0: filter line queries through a padded binary BVH (same hits, same order; used by
    // the CPU baseline so the host runs the reference's algorithm at a realistic speed)
    const bool accel = (params->flags & 1u) != 0u;
    if (dim == 2) {
        auto h = std::make_unique<Holder<2>>();
        fill_elements<2>(h->scene, n_elems, verts, normals, bvals, alphas, types);
        if (vol_res) { h->vol.build(vol_res, vol_size, vol_values); h->scene.vol = &h->vol; }
        std::unique_ptr<BinaryLbvh<2>> tree;
        if (accel) {
            tree = std::make_unique<BinaryLbvh<2>>(h->scene, accel_pad(h->scene));
            h->scene.accel = tree.get();
            h->scene.accel_candidates = &BinaryLbvh<2>::candidates_cb;
        }
        return solve_domain<2>(h->scene, params, points, n_points, sum, sumsq, per_path);
    }
    auto h = std::make_unique<Holder<3>>();
    fill_elements<3>(h->scene, n_elems, verts, normals, bvals, alphas, types);
    if (vol_res) { h->vol.build(vol_res, vol_size, vol_values); h->scene.vol = &h->vol; }
    std::unique_ptr<BinaryLbvh<3>> tree;
    if (accel) {
        tree = std::make_unique<BinaryLbvh<3>>(h->scene, accel_pad(h->scene));
        h->scene.accel = tree.get();
        h->scene.accel_candidates = &BinaryLbvh<3>::candidates_cb;
    }
    return solve_domain<3>(h->scene, params, points, n_points, sum, sumsq, per_path);
}

uint64_t oracle_solve_boundary(int dim, uint32_t n_elems, const float *verts, const float *normals,
                               const float *bvals, const float *alphas, const int32_t *types, uint32_t vol_res,
                               float vol_size, const float *vol_values, const oracle_params *params,
                               const float *p, const float *n, const float *angle, const float *bv,
                               const int32_t *type, const float *alpha, uint32_t n_points, double *sum,
                               double *sumsq, float *per_path, int n_threads) {
    set_threads(n_threads);
    if (dim == 2) {
        auto h = std::make_unique<Holder<2>>();
        fill_elements<2>(h->scene, n_elems, verts, normals, bvals, alphas, types);
        if (vol_res) { h->vol.build(vol_res, vol_size, vol_values); h->scene.vol = &h->vol; }
        return solve_boundary<2>(h->scene, params, p, n, angle, bv, type, alpha, n_points, sum, sumsq, per_path);
    }
    auto h = std::make_unique<Holder<3>>();
    fill_elements<3>(h->scene, n_elems, verts, normals, bvals, alphas, types);
    if (vol_res) { h->vol.build(vol_res, vol_size, vol_values); h->scene.vol = &h->vol; }
    return solve_boundary<3>(h->scene, params, p, n, angle, bv, type, alpha, n_points, sum, sumsq, per_path);
}

// Forward single-layer Neumann with a per-element control-variate density (storage order).
uint64_t oracle_solve_domain_cv(int dim, uint32_t n_elems, const float *verts, const float *normals,
                                const float *bvals, const float *alphas, const int32_t *types,
                                const oracle_params *params, const float *sigma_t, uint32_t n_pot,
                                uint32_t m_ker, const float *points, uint32_t n_points, double *sum,
                                double *sumsq, float *per_path, int n_threads) {
    set_threads(n_threads);
    if (dim == 2) {
        auto h = std::make_unique<Holder<2>>();
        fill_elements<2>(h->scene, n_elems, verts, normals, bvals, alphas, types);
        return solve_domain_cv<2>(h->scene, params, sigma_t, n_pot, m_ker, points, n_points, sum, sumsq, per_path);
    }
    auto h = std::make_unique<Holder<3>>();
    fill_elements<3>(h->scene, n_elems, verts, normals, bvals, alphas, types);
    return solve_domain_cv<3>(h->scene, params, sigma_t, n_pot, m_ker, points, n_points, sum, sumsq, per_path);
}

// Backward estimator with a per-element control variate on the unknown boundary function (storage
// order); u only: sum [n], sumsq [n], per_path [n][paths].
uint64_t oracle_solve_domain_bcv(int dim, uint32_t n_elems, const float *verts, const float *normals,
                                 const float *bvals, const float *alphas, const int32_t *types,
                                 const oracle_params *params, const float *cv, uint32_t n_pot, const float *points,
                                 uint32_t n_points, double *sum, double *sumsq, float *per_path, int n_threads) {
    set_threads(n_threads);
    if (dim == 2) {
        auto h = std::make_unique<Holder<2>>();
        fill_elements<2>(h->scene, n_elems, verts, normals, bvals, alphas, types);
        return solve_domain_bcv<2>(h->scene, params, cv, n_pot, points, n_points, sum, sumsq, per_path);
    }
    auto h = std::make_unique<Holder<3>>();
    fill_elements<3>(h->scene, n_elems, verts, normals, bvals, alphas, types);
    return solve_domain_bcv<3>(h->scene, params, cv, n_pot, points, n_points, sum, sumsq, per_path);
}

// Roofline constants: runs the domain estimator at the points (params as oracle_solve_domain) and
// measures, for every line query the walks make, the work of the reference's binary LBVH
// (lbvh_count.hpp). out = {queries, nodes visited, primitives tested}.
void oracle_lbvh_stats(int dim, uint32_t n_elems, const float *verts, const float *normals, const float *bvals,
                       const float *alphas, const int32_t *types, const oracle_params *params, const float *points,
                       uint32_t n_points, double *out, int n_threads) {
    set_threads(n_threads);
    auto run = [&](auto &scene, auto dimtag) {
        constexpr int D = decltype(dimtag)::value;
        const BinaryLbvh<D> tree(scene);
        const Params prm = to_params(params);
        double q = 0, nn = 0, np = 0;
#pragma omp parallel reduction(+ : q, nn, np)
        {
            LbvhCounter<D> counter(&tree);
            g_line_observer = &counter;
#pragma omp for schedule(dynamic, 1)
            for (int64_t ii = 0; ii < (int64_t)n_points; ii++) {
                Vec<D> x;
                for (int k = 0; k < D; k++) x.v[k] = points[(size_t)ii * D + k];
                for (uint32_t j = 0; j < params->num_sample_paths; j++) {
                    Rng rng(params->seed, kStreamDomain, params->point_offset + (uint32_t)ii, params->path_offset + j);
                    Estimator<D> est(&scene, prm, &rng);
                    float o[D + 1];
                    est.domain(x, o);
                }
            }
            g_line_observer = nullptr;
            q += (double)counter.queries;
            nn += (double)counter.nodes;
            np += (double)counter.prims;
        }
        out[0] = q;
        out[1] = nn;
        out[2] = np;
    };
    if (dim == 2) {
        auto h = std::make_unique<Holder<2>>();
        fill_elements<2>(h->scene, n_elems, verts, normals, bvals, alphas, types);
        run(h->scene, std::integral_constant<int, 2>());
    } else {
        auto h = std::make_unique<Holder<3>>();
        fill_elements<3>(h->scene, n_elems, verts, normals, bvals, alphas, types);
        run(h->scene, std::integral_constant<int, 3>());
    }
}

// Walk on spheres (2D): per-point sums and per-path values; stream kStreamWos.
uint64_t oracle_wos(uint32_t n_elems, const float *verts, const float *normals, const float *bvals,
                    const int32_t *types, const oracle_params *params, const float *points, uint32_t n_points,
                    double *sum, float *per_path, int n_threads) {
    set_threads(n_threads);
    auto h = std::make_unique<Holder<2>>();
    fill_elements<2>(h->scene, n_elems, verts, normals, bvals, nullptr, types);
    const Scene<2> &scene = h->scene;
    const uint32_t P = params->num_sample_paths;
    uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
    for (int64_t ii = 0; ii < (int64_t)n_points; ii++) {
        Vec<2> x;
        x.v[0] = points[2 * ii];
        x.v[1] = points[2 * ii + 1];
        double acc = 0.0;
        for (uint32_t j = 0; j < P; j++) {
            Rng rng(params->seed, kStreamWos, params->point_offset + (uint32_t)ii, params->path_offset + j);
            unsigned q = 0;
            const float v = wos_path(scene, params->eps, rng, x, q);
            total += q;
            acc += (double)v;
            if (per_path) per_path[(size_t)ii * P + j] = v;
        }
        if (sum) sum[ii] += acc;
    }
    return total;
}

void oracle_closest_point(uint32_t n_elems, const float *verts, const float *normals, const float *bvals,
                          const int32_t *types, const float *points, uint32_t n, uint32_t *elem, float *dist2,
                          float *value) {
    Scene<2> s;
    fill_elements<2>(s, n_elems, verts, normals, bvals, nullptr, types);
    for (uint32_t i = 0; i < n; i++) {
        Vec<2> x;
        x.v[0] = points[2 * i];
        x.v[1] = points[2 * i + 1];
        const ClosestPoint c = closest_point(s, x);
        elem[i] = c.elem;
        dist2[i] = c.d2;
        value[i] = c.elem == 0xFFFFFFFFu ? 0.0f : closest_value(s, c);
    }
}

// VPL walks (apps/potential_flow_with_vpl.cu:77-88): path i from a uniform boundary sample, its
// unknown-boundary estimate; stream kStreamVpl, point 0, path path_offset + i.
uint64_t oracle_vpl_paths(int dim, uint32_t n_elems, const float *verts, const float *normals, const float *bvals,
                          const float *alphas, const int32_t *types, const oracle_params *params, uint32_t n_paths,
                          float *vpl_p, float *vpl_mu, int n_threads) {
    set_threads(n_threads);
    auto run = [&](auto &scene, auto dimtag) -> uint64_t {
        constexpr int D = decltype(dimtag)::value;
        const Params prm = to_params(params);
        uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
        for (int64_t ii = 0; ii < (int64_t)n_paths; ii++) {
            Rng rng(params->seed, kStreamVpl, 0u, params->path_offset + (uint64_t)ii);
            Estimator<D> est(&scene, prm, &rng);
            float ip;
            const BoundaryPoint<D> y = scene.sample_uniform(rng, ip);
            const float mu = est.unknown_boundary(y);
            for (int k = 0; k < D; k++) vpl_p[(size_t)ii * D + k] = y.p.v[k];
            vpl_mu[ii] = mu;
            total += est.bounces;
        }
        return total;
    };
    if (dim == 2) {
        auto h = std::make_unique<Holder<2>>();
        fill_elements<2>(h->scene, n_elems, verts, normals, bvals, alphas, types);
        return run(h->scene, std::integral_constant<int, 2>());
    }
    auto h = std::make_unique<Holder<3>>();
    fill_elements<3>(h->scene, n_elems, verts, normals, bvals, alphas, types);
    return run(h->scene, std::integral_constant<int, 3>());
}

// VPL aggregation (apps/potential_flow_with_vpl.cu:43-75): sum[pt] += sum_i mu_i (G A, dG/dx A),
// the engine's blocking: FP32 partial sums over tiles of 256 VPLs, tile t added in FP64 into split
// t mod 8 (in tile order), the 8 splits added in order. The pair is the engine's form of
// G (equation_kernel.cuh:74-79, 115-121) with per-VPL constants, r = y - x, q = |r|^2:
//   2D: ku = mu (-A/(4 pi)), kw = mu A/(2 pi); mu G A = ku log(max(q, eps^2)) (log(max(|r|, eps))
//       = log(max(q, eps^2)) / 2); mu w = kw / q (q >= eps^2), kw / (|r| eps) (0 < q < eps^2), 0;
//   3D: ku = mu A/(4 pi); mu G A = ku / max(|r|, eps); mu w = ku / (|r| max(q, eps)), 0 at q = 0;
// and mu dG/dx A = mu w (y - x).
void oracle_vpl_aggregate(int dim, float area, float eps, const float *vpl_p, const float *vpl_mu, uint32_t n_vpl,
                          const float *points, uint32_t n_points, double *sum, int n_threads) {
    set_threads(n_threads);
    auto run = [&](auto dimtag) {
        constexpr int D = decltype(dimtag)::value;
        const float cu = D == 2 ? -0x1.45f306p-4f * area : 0x1.45f306p-4f * area;
        const float cw = 0x1.45f306p-3f * area;
        const float eps2 = eps * eps;
#pragma omp parallel for schedule(dynamic, 16)
        for (int64_t ii = 0; ii < (int64_t)n_points; ii++) {
            Vec<D> x;
            for (int k = 0; k < D; k++) x.v[k] = points[(size_t)ii * D + k];
            const uint32_t n_tiles = (n_vpl + 255) / 256;
            double split[8][D + 1] = {};
            for (uint32_t t = 0; t < n_tiles; t++) {
                const uint32_t t0 = t * 256;
                const uint32_t m = std::min<uint32_t>(256u, n_vpl - t0);
                float part[D + 1] = {};
                for (uint32_t j = 0; j < m; j++) {
                    Vec<D> y;
                    for (int k = 0; k < D; k++) y.v[k] = vpl_p[(size_t)(t0 + j) * D + k];
                    const float mu = vpl_mu[t0 + j];
                    const float ku = mu * cu, kw = mu * cw;
                    const Vec<D> r = y - x;
                    float q = 0.0f;
                    for (int k = 0; k < D; k++) q = q + r.v[k] * r.v[k];
                    float g;
                    if (D == 2) {
                        part[0] = part[0] + ku * log_own(fmax_ref(q, eps2));
                        g = q >= eps2 ? kw / q : (q > 0.0f ? kw / (std::sqrt(q) * eps) : 0.0f);
                    } else {
                        const float nr = std::sqrt(q);
                        part[0] = part[0] + ku / fmax_ref(nr, eps);
                        g = q > 0.0f ? ku / (nr * fmax_ref(q, eps)) : 0.0f;
                    }
                    for (int k = 0; k < D; k++) part[1 + k] = part[1 + k] + g * r.v[k];
                }
                for (int c = 0; c <= D; c++) split[t % 8][c] += (double)part[c];
            }
            for (int c = 0; c <= D; c++) {
                double total = split[0][c];
                for (int k = 1; k < 8; k++) total = total + split[k][c];
                sum[(size_t)ii * (D + 1) + c] += total;
            }
        }
    };
    if (dim == 2) run(std::integral_constant<int, 2>());
    else run(std::integral_constant<int, 3>());
}

// compute_sample_unknown_boundary at boundary points (the boundary density / unknown).
uint64_t oracle_solve_unknown(int dim, uint32_t n_elems, const float *verts, const float *normals,
                              const float *bvals, const float *alphas, const int32_t *types,
                              const oracle_params *params, const float *p, const float *n, const float *angle,
                              const float *bv, const int32_t *type, const float *alpha, uint32_t n_points,
                              double *sum, float *per_path, int n_threads) {
    set_threads(n_threads);
    if (dim == 2) {
        auto h = std::make_unique<Holder<2>>();
        fill_elements<2>(h->scene, n_elems, verts, normals, bvals, alphas, types);
        return solve_unknown<2>(h->scene, params, p, n, angle, bv, type, alpha, n_points, sum, per_path);
    }
    auto h = std::make_unique<Holder<3>>();
    fill_elements<3>(h->scene, n_elems, verts, normals, bvals, alphas, types);
    return solve_unknown<3>(h->scene, params, p, n, angle, bv, type, alpha, n_points, sum, per_path);
}

// Brute-force line query: counts[i] = total hits, hits[i][0..63] = element indices in order,
// points[i][k][dim] = hit points.
void oracle_line_query(int dim, uint32_t n_elems, const float *verts, const float *normals, const float *bvals,
                       const int32_t *types, const float *origins, const float *dirs, uint32_t n_rays,
                       uint32_t *counts, uint32_t *hits, float *points) {
    if (dim == 2) {
        Scene<2> s;
        fill_elements<2>(s, n_elems, verts, normals, bvals, nullptr, types);
        for (uint32_t r = 0; r < n_rays; r++) {
            Vec<2> o, d;
            for (int k = 0; k < 2; k++) { o.v[k] = origins[r * 2 + k]; d.v[k] = dirs[r * 2 + k]; }
            counts[r] = s.line_query(o, d, hits + (size_t)r * kHitBuffer);
            const unsigned m = std::min(counts[r], kHitBuffer);
            for (unsigned k = 0; k < m; k++) {
                Vec<2> p = o;
                line_elem_intersect(o, d, s.elems[hits[(size_t)r * kHitBuffer + k]], p);
                for (int j = 0; j < 2; j++) points[((size_t)r * kHitBuffer + k) * 2 + j] = p.v[j];
            }
        }
        return;
    }
    Scene<3> s;
    fill_elements<3>(s, n_elems, verts, normals, bvals, nullptr, types);
    for (uint32_t r = 0; r < n_rays; r++) {
        Vec<3> o, d;
        for (int k = 0; k < 3; k++) { o.v[k] = origins[r * 3 + k]; d.v[k] = dirs[r * 3 + k]; }
        counts[r] = s.line_query(o, d, hits + (size_t)r * kHitBuffer);
        const unsigned m = std::min(counts[r], kHitBuffer);
        for (unsigned k = 0; k < m; k++) {
            Vec<3> p = o;
            line_elem_intersect(o, d, s.elems[hits[(size_t)r * kHitBuffer + k]], p);
            for (int j = 0; j < 3; j++) points[((size_t)r * kHitBuffer + k) * 3 + j] = p.v[j];
        }
    }
}

// Scene CDFs (for comparing with the engine's host build).
void oracle_scene_cdfs(int dim, uint32_t n_elems, const float *verts, const float *normals, const float *bvals,
                       const int32_t *types, float *area_cdf, float *bv_cdf, float *totals) {
    if (dim == 2) {
        Scene<2> s;
        fill_elements<2>(s, n_elems, verts, normals, bvals, nullptr, types);
        std::memcpy(area_cdf, s.area_cdf.data(), n_elems * 4);
        std::memcpy(bv_cdf, s.bv_cdf.data(), n_elems * 4);
        totals[0] = s.total_area;
        totals[1] = s.total_bv;
        return;
    }
    Scene<3> s;
    fill_elements<3>(s, n_elems, verts, normals, bvals, nullptr, types);
    std::memcpy(area_cdf, s.area_cdf.data(), n_elems * 4);
    std::memcpy(bv_cdf, s.bv_cdf.data(), n_elems * 4);
    totals[0] = s.total_area;
    totals[1] = s.total_bv;
}

// Closed-form double-layer walk (apps/simple_wob_and_wos.cu:81-108), 2D interior Dirichlet.
void oracle_simple_wob(uint32_t n_elems, const float *verts, const float *normals, const float *bvals,
                       const int32_t *types, uint64_t seed, uint32_t path_length, uint32_t n_paths,
                       const float *points, uint32_t n_points, double *sum, int n_threads) {
    set_threads(n_threads);
    Scene<2> s;
    fill_elements<2>(s, n_elems, verts, normals, bvals, nullptr, types);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t ii = 0; ii < (int64_t)n_points; ii++) {
        const uint32_t i = (uint32_t)ii;
        Vec<2> x;
        x.v[0] = points[i * 2];
        x.v[1] = points[i * 2 + 1];
        double acc = 0.0;
        for (uint32_t j = 0; j < n_paths; j++) {
            Rng rng(seed, kStreamDomain, i, j);
            acc += (double)simple_wob_path(s, rng, x, path_length);
        }
        sum[i] = acc;
    }
}

// Scalar helpers for unit tests.
void oracle_sincospi(const float *x, float *s, float *c, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) sincospi_own(x[i], s + i, c + i);
}
void oracle_log(const float *x, float *y, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) y[i] = log_own(x[i]);
}
void oracle_philox(const uint32_t *ctr, uint32_t k0, uint32_t k1, uint32_t *out) {
    Philox4x32::generate(ctr, k0, k1, out);
}
void oracle_uniforms(uint64_t seed, uint32_t stream, uint32_t point, uint64_t path, float *out, uint32_t n) {
    Rng r(seed, stream, point, path);
    for (uint32_t i = 0; i < n; i++) out[i] = r.uniform();
}
// Fundamental solutions: out = [G, dG_dx(D), dG_dny, d2G_dxdny(D), d2G_dnxdny] for each (y, x, ny, nx).
void oracle_green(int dim, float eps, const float *y, const float *x, const float *ny, const float *nx, uint32_t n,
                  float *out) {
    for (uint32_t i = 0; i < n; i++) {
        if (dim == 2) {
            EqKernel<2> K{eps};
            Vec<2> Y{{y[2 * i], y[2 * i + 1]}}, X{{x[2 * i], x[2 * i + 1]}}, NY{{ny[2 * i], ny[2 * i + 1]}}, NX{{nx[2 * i], nx[2 * i + 1]}};
            float *o = out + (size_t)i * 7;
            o[0] = K.G(Y, X);
            const Vec<2> g = K.dG_dx(Y, X);
            o[1] = g.v[0]; o[2] = g.v[1];
            o[3] = K.dG_dny(Y, X, NY);
            const Vec<2> h = K.d2G_dxdny(Y, X, NY);
            o[4] = h.v[0]; o[5] = h.v[1];
            o[6] = K.d2G_dnxdny(Y, X, NY, NX);
        } else {
            EqKernel<3> K{eps};
            Vec<3> Y{{y[3 * i], y[3 * i + 1], y[3 * i + 2]}}, X{{x[3 * i], x[3 * i + 1], x[3 * i + 2]}};
            Vec<3> NY{{ny[3 * i], ny[3 * i + 1], ny[3 * i + 2]}}, NX{{nx[3 * i], nx[3 * i + 1], nx[3 * i + 2]}};
            float *o = out + (size_t)i * 9;
            o[0] = K.G(Y, X);
            const Vec<3> g = K.dG_dx(Y, X);
            o[1] = g.v[0]; o[2] = g.v[1]; o[3] = g.v[2];
            o[4] = K.dG_dny(Y, X, NY);
            const Vec<3> h = K.d2G_dxdny(Y, X, NY);
            o[5] = h.v[0]; o[6] = h.v[1]; o[7] = h.v[2];
            o[8] = K.d2G_dnxdny(Y, X, NY, NX);
        }
    }
}

int oracle_max_threads(void) { return set_threads(0); }

}  // extern "C"
