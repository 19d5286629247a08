// The general WoB walk on the device: fundamental solutions, the three BIE models for interior and
// exterior domains, and the backward / forward estimators with every sampling strategy of the
// reference. The BIE model, domain and problem are run-time values (uniform across a launch);
// the dimension is a template parameter.
//
// Restates equation_kernel.cuh:67-145, bie_models.cuh:53-590 and estimator.cuh:113-504.
#pragma once

#include "device_common.cuh"

#include <type_traits>

namespace wobgb {

struct WalkParams {
    int bie, domain, estimator, problem;
    uint32_t path_length, n_paths, n_resampling, n_volume;
    float eps, fk;
    uint64_t seed, path_offset;
    uint32_t point_offset;
    uint32_t ppt;   // paths per lane in one warp unit (set by the launcher, >= 1)
    uint32_t ppt_cap;  // 0: the launcher's choice; else at most this many (an autotuned setting)
    uint32_t no_alloc;  // 1: only kernels that allocate nothing (the allocation-free entry point)
    uint32_t ppt_points;  // 0: paths per lane chosen for the launch's points; else for this many (autotune)
    uint32_t mode;  // boundary kernel: 0 = boundary estimate, 1 = unknown boundary density
    uint32_t n_pot, m_ker;  // control-variate estimator: samples of <G_x, sigma~> and of K sigma~
};

// ------------------------------------------------------------------------------------------
// Fundamental solutions (equation_kernel.cuh:74-100 and 115-142).
// ------------------------------------------------------------------------------------------
template <int D> struct Green;
template <> struct Green<2> {
    float eps;
    __device__ __forceinline__ float G(const V<2> &y, const V<2> &x) const {
        return -0x1.45f306p-3f * log_own(fmax_ref(vnorm(vsub(y, x)), eps));
    }
    __device__ __forceinline__ V<2> dG_dx(const V<2> &y, const V<2> &x) const {
        const V<2> r = vsub(y, x);
        return vdiv(vscale(0x1.45f306p-3f, vnormalized(r)), fmax_ref(vnorm(r), eps));
    }
    __device__ __forceinline__ float dG_dny(const V<2> &y, const V<2> &x, const V<2> &ny) const {
        const V<2> r = vsub(y, x);
        return -0x1.45f306p-3f * vdot(vnormalized(r), ny) / fmax_ref(vnorm(r), eps);
    }
    __device__ __forceinline__ V<2> d2G_dxdny(const V<2> &y, const V<2> &x, const V<2> &ny) const {
        const V<2> r = vsub(y, x);
        const V<2> rh = vnormalized(r);
        const float k = 1.0f / (0x1.921fb6p+2f * fmax_ref(vsqnorm(r), eps));
        return vscale(k, vsub(ny, vscale(2.0f * vdot(rh, ny), rh)));
    }
};
template <> struct Green<3> {
    float eps;
    __device__ __forceinline__ float G(const V<3> &y, const V<3> &x) const {
        return 1.0f / (0x1.921fb6p+3f * fmax_ref(vnorm(vsub(y, x)), eps));
    }
    __device__ __forceinline__ V<3> dG_dx(const V<3> &y, const V<3> &x) const {
        const V<3> r = vsub(y, x);
        return vdiv(vscale(0x1.45f306p-4f, vnormalized(r)), fmax_ref(vsqnorm(r), eps));
    }
    __device__ __forceinline__ float dG_dny(const V<3> &y, const V<3> &x, const V<3> &ny) const {
        const V<3> r = vsub(y, x);
        return -0x1.45f306p-4f * vdot(vnormalized(r), ny) / fmax_ref(vsqnorm(r), eps);
    }
    __device__ __forceinline__ V<3> d2G_dxdny(const V<3> &y, const V<3> &x, const V<3> &ny) const {
        const V<3> r = vsub(y, x);
        const V<3> rh = vnormalized(r);
        const float k = 1.0f / (0x1.921fb6p+3f * fmax_ref(vnorm(r) * vsqnorm(r), eps));
        return vscale(k, vsub(ny, vscale(3.0f * vdot(rh, ny), rh)));
    }
};

// ------------------------------------------------------------------------------------------
// BIE models (bie_models.cuh:53-590); fbu may replace one point by the other (first-kind
// roulette) exactly like the reference's by-reference arguments.
// ------------------------------------------------------------------------------------------
// The BIE models (bie_models.cuh:53-590) are member functions of the walker below: kBie >= 0
// fixes the model at compile time (-1: run-time value), kVol = false drops the source-term code.
// fbu may replace one point by the other (first-kind roulette) exactly like the reference's
// by-reference arguments.

// ------------------------------------------------------------------------------------------
// Estimators (estimator.cuh:113-504).
// ------------------------------------------------------------------------------------------
// Sampling strategies of the estimators (the if-constexpr chains of estimator.cuh:158-168, 255-347,
// 423-427, 445-448). kStrat fixes one at compile time; kStratRuntime picks it from the parameters.
enum : int {
    kStratRuntime = -1,
    kStratLineIntersection = 0,  // backward, double layer + Dirichlet
    kStratDirectNeumann = 1,     // backward, direct + Neumann
    kStratSingleLayer = 2,       // backward, single layer (uniform or RIS)
    kStratUniform = 3,           // backward, every other case: two uniform samples per bounce
    kStratFwdSlNeumann = 4,      // forward, single layer + Neumann
    kStratFwdUniform = 5         // forward, every other case
};

__host__ __device__ __forceinline__ int strategy_of(int bie, int est, int problem) {
    if (est == kBackward) {
        if (bie == kDoubleLayer && problem == kDirichletProblem) return kStratLineIntersection;
        if (bie == kDirect && problem == kNeumannProblem) return kStratDirectNeumann;
        if (bie == kSingleLayer) return kStratSingleLayer;
        return kStratUniform;
    }
    return (bie == kSingleLayer && problem == kNeumannProblem) ? kStratFwdSlNeumann : kStratFwdUniform;
}

// The scene view and parameters are held by value: a kernel parameter whose address is taken
// is copied to local memory, a by-value copy stays in registers / the parameter bank. With
// kByRef the walker holds references instead, for a view and parameters staged in shared memory
// (the batched launch), which cost a shared-memory load per use instead of registers.
template <int D, int kBie = -1, int kStrat = kStratRuntime, bool kVol = true, bool kByRef = false> struct Walker {
    using ViewT = std::conditional_t<kByRef, const SceneView<D> &, const SceneView<D>>;
    using ParamsT = std::conditional_t<kByRef, const WalkParams &, const WalkParams>;
    ViewT s;
    ParamsT p;
    PathRng rng;
    Green<D> K;
    uint32_t bounces;
    bool stayed;  // the last fbu call kept the current point (first-kind roulette)

    __device__ __forceinline__ Walker(const SceneView<D> &s_, const WalkParams &p_, uint32_t stream, uint32_t point, uint64_t path)
        : s(s_), p(p_), rng(p_.seed, stream, point, path), bounces(0), stayed(false) {
        K.eps = p.eps;
    }

    // ---------------- BIE models
    __device__ __forceinline__ int model() const { return kBie >= 0 ? kBie : p.bie; }
    __device__ __forceinline__ float dtc() const { return p.domain == kInterior ? 1.0f : -1.0f; }
    __device__ __forceinline__ float ift(float a) const { return p.domain == kInterior ? a : 1.0f - a; }

    __device__ __forceinline__ float vol_term(const BPoint<D> &b) {
        if (!kVol || p.n_volume == 0) return 0.0f;
        const VSample<D> v = sample_volume<D>(s, rng);
        float r = 0.0f;
        for (uint32_t i = 0; i < p.n_volume; i++) {
            if (b.type == kDirichlet) r = r + K.G(b.p, v.p) * v.value * v.inv_pdf;
            else if (b.type == kNeumann) r = r + K.dG_dny(b.p, v.p, b.n) * v.value * v.inv_pdf;
            else r = r + (K.dG_dny(b.p, v.p, b.n) + b.alpha * K.G(v.p, b.p)) * v.value * v.inv_pdf;
        }
        return r / (float)p.n_volume;
    }
    __device__ __forceinline__ float vol_init_boundary(const BPoint<D> &b) {
        if (!kVol || p.n_volume == 0) return 0.0f;
        const VSample<D> v = sample_volume<D>(s, rng);
        float r = 0.0f;
        for (uint32_t i = 0; i < p.n_volume; i++) r = r - K.G(b.p, v.p) * v.value * v.inv_pdf;
        return r / (float)p.n_volume;
    }
    __device__ __forceinline__ float vol_init_domain(const V<D> &x) {
        if (!kVol || p.n_volume == 0) return 0.0f;
        const VSample<D> v = sample_volume<D>(s, rng);
        float r = 0.0f;
        for (uint32_t i = 0; i < p.n_volume; i++) r = r - K.G(v.p, x) * v.value * v.inv_pdf;
        return r / (float)p.n_volume;
    }
    __device__ __forceinline__ V<D> vol_init_derivative(const V<D> &x) {
        if (!kVol || p.n_volume == 0) return vzero<D>();
        const VSample<D> v = sample_volume<D>(s, rng);
        V<D> r = vzero<D>();
        for (uint32_t i = 0; i < p.n_volume; i++) {
            const V<D> g = K.dG_dx(v.p, x);
#pragma unroll
            for (int j = 0; j < D; j++) r.v[j] = r.v[j] - g.v[j] * v.value * v.inv_pdf;
        }
        return vdiv(r, (float)p.n_volume);
    }

    __device__ __forceinline__ float sdu(const V<D> &x, const BPoint<D> &y, float ip) {
        if (model() == kSingleLayer) return K.G(y.p, x) * ip;
        if (model() == kDoubleLayer) return -K.dG_dny(y.p, x, y.n) * ip;
        if (y.type == kDirichlet) return dtc() * ip * K.G(y.p, x);
        if (y.type == kNeumann) return -dtc() * ip * K.dG_dny(y.p, x, y.n);
        return -dtc() * ip * (K.dG_dny(y.p, x, y.n) + y.alpha * K.G(y.p, x));
    }
    __device__ __forceinline__ float sdk(const V<D> &x, const BPoint<D> &y, float ip) {
        float r = vol_init_domain(x);
        if (model() != kDirect) return r;
        if (y.type == kDirichlet) {
            const float k = -dtc() * ip * K.dG_dny(y.p, x, y.n);
            r = r + k * (y.bv + vol_term(y));
        } else {
            const float k = dtc() * ip * K.G(y.p, x);
            r = r + k * (y.bv + vol_term(y));
        }
        return r;
    }
    __device__ __forceinline__ V<D> gdu(const V<D> &x, const BPoint<D> &y, float ip) {
        V<D> r;
        if (model() == kSingleLayer) {
            const V<D> g = K.dG_dx(y.p, x);
#pragma unroll
            for (int i = 0; i < D; i++) r.v[i] = g.v[i] * ip;
            return r;
        }
        if (model() == kDoubleLayer) {
            const V<D> g = K.d2G_dxdny(y.p, x, y.n);
#pragma unroll
            for (int i = 0; i < D; i++) r.v[i] = -g.v[i] * ip;
            return r;
        }
        if (y.type == kDirichlet) {
            const float c = dtc() * ip;
            const V<D> g = K.dG_dx(y.p, x);
#pragma unroll
            for (int i = 0; i < D; i++) r.v[i] = c * g.v[i];
            return r;
        }
        if (y.type == kNeumann) {
            const float c = -dtc() * ip;
            const V<D> g = K.d2G_dxdny(y.p, x, y.n);
#pragma unroll
            for (int i = 0; i < D; i++) r.v[i] = c * g.v[i];
            return r;
        }
        const float c = -dtc() * ip;
        const V<D> g1 = K.d2G_dxdny(y.p, x, y.n);
        const V<D> g2 = K.dG_dx(y.p, x);
#pragma unroll
        for (int i = 0; i < D; i++) r.v[i] = c * (g1.v[i] + y.alpha * g2.v[i]);
        return r;
    }
    __device__ __forceinline__ V<D> gdk(const V<D> &x, const BPoint<D> &y, float ip) {
        V<D> r = vol_init_derivative(x);
        if (model() != kDirect) return r;
        if (y.type == kDirichlet) {
            const float c = -dtc() * ip;
            const V<D> g = K.d2G_dxdny(y.p, x, y.n);
            const float sv = y.bv + vol_term(y);
#pragma unroll
            for (int i = 0; i < D; i++) r.v[i] = r.v[i] + c * g.v[i] * sv;
        } else {
            const float c = dtc() * ip;
            const V<D> g = K.dG_dx(y.p, x);
            const float sv = y.bv + vol_term(y);
#pragma unroll
            for (int i = 0; i < D; i++) r.v[i] = r.v[i] + c * g.v[i] * sv;
        }
        return r;
    }
    __device__ __forceinline__ float sbu(const BPoint<D> &x, const BPoint<D> &y, float ip) {
        if (model() == kDoubleLayer) return 0.0f;
        if (x.type == kDirichlet) return 0.0f;
        if (model() == kSingleLayer) return K.G(y.p, x.p) * ip;
        if (y.type == kDirichlet) return dtc() / ift(x.angle) * ip * K.G(y.p, x.p);
        if (y.type == kNeumann) return -dtc() / ift(x.angle) * ip * K.dG_dny(y.p, x.p, y.n);
        return -dtc() / ift(x.angle) * ip * (K.dG_dny(y.p, x.p, y.n) + y.alpha * K.G(y.p, x.p));
    }
    __device__ __forceinline__ float sbk(const BPoint<D> &x, const BPoint<D> &y, float ip) {
        if (model() == kDoubleLayer) return x.bv;
        if (x.type == kDirichlet) return x.bv;
        if (model() == kSingleLayer) return vol_init_boundary(x);
        float r = vol_init_boundary(x);
        if (y.type == kDirichlet) {
            const float k = -dtc() / ift(x.angle) * ip * K.dG_dny(y.p, x.p, y.n);
            r = r + k * (y.bv + vol_term(y));
        } else {
            const float k = dtc() / ift(x.angle) * ip * K.G(y.p, x.p);
            r = r + k * (y.bv + vol_term(y));
        }
        return r;
    }
    __device__ __forceinline__ float fbu(BPoint<D> &x, BPoint<D> &y, float ip, bool backward) {
        stayed = false;
        if (model() == kDoubleLayer) return dtc() / (1.0f - ift(x.angle)) * ip * K.dG_dny(y.p, x.p, y.n);
        if (backward && x.type == kDirichlet) {
            if (rng.uniform() * (1.0f + p.fk) < 1.0f) { y = x; stayed = true; return (1.0f + p.fk) * 1.0f; }
            ip = ip * ((1.0f + p.fk) / p.fk);
        } else if (!backward && y.type == kDirichlet) {
            if (rng.uniform() * (1.0f + p.fk) < 1.0f) { x = y; return (1.0f + p.fk) * 1.0f; }
            ip = ip * ((1.0f + p.fk) / p.fk);
        }
        if (model() == kSingleLayer) {
            if (x.type == kDirichlet) return -2.0f * p.fk * ip * K.G(y.p, x.p);
            if (x.type == kNeumann) return -dtc() / ift(x.angle) * ip * K.dG_dny(x.p, y.p, x.n);
            return -dtc() / ift(x.angle) * ip * (K.dG_dny(x.p, y.p, x.n) + x.alpha * K.G(y.p, x.p));
        }
        if (x.type == kDirichlet) {
            if (y.type == kDirichlet) return -p.fk / ift(x.angle) * ip * K.G(y.p, x.p);
            if (y.type == kNeumann) return p.fk / ift(x.angle) * ip * K.dG_dny(y.p, x.p, y.n);
            return p.fk / ift(x.angle) * ip * (K.dG_dny(y.p, x.p, y.n) + y.alpha * K.G(y.p, x.p));
        }
        if (y.type == kDirichlet) return dtc() / ift(x.angle) * ip * K.G(y.p, x.p);
        if (y.type == kNeumann) return -dtc() / ift(x.angle) * ip * K.dG_dny(y.p, x.p, y.n);
        return -dtc() / ift(x.angle) * ip * (K.dG_dny(y.p, x.p, y.n) + y.alpha * K.G(y.p, x.p));
    }
    __device__ __forceinline__ float fbk(const BPoint<D> &x, const BPoint<D> &y, float ip) {
        if (model() == kDoubleLayer) return dtc() * 1.0f / (1.0f - ift(x.angle)) * (x.bv + vol_term(x));
        if (model() == kSingleLayer) {
            if (x.type == kDirichlet) return 2.0f * p.fk * (x.bv + vol_term(x));
            return dtc() / ift(x.angle) * (x.bv + vol_term(x));
        }
        if (x.type == kDirichlet) {
            const float sx = x.bv + vol_term(x);
            if (y.type == kDirichlet) {
                const float k = dtc() / ift(x.angle) * ip * K.dG_dny(y.p, x.p, y.n);
                return dtc() * p.fk * (sx + k * (y.bv + vol_term(y)));
            }
            const float k = dtc() / ift(x.angle) * ip * K.G(y.p, x.p);
            return dtc() * p.fk * (sx - k * (y.bv + vol_term(y)));
        }
        if (y.type == kDirichlet) {
            const float k = -dtc() / ift(x.angle) * ip * K.dG_dny(y.p, x.p, y.n);
            return k * (y.bv + vol_term(y));
        }
        const float k = dtc() / ift(x.angle) * ip * K.G(y.p, x.p);
        return k * (y.bv + vol_term(y));
    }

    // ---------------- estimators
    __device__ __forceinline__ int strat() const { return kStrat != kStratRuntime ? kStrat : strategy_of(model(), p.estimator, p.problem); }
    __device__ __forceinline__ bool backward() const { return strat() <= kStratUniform; }
    __device__ __forceinline__ bool dl_dirichlet() const { return strat() == kStratLineIntersection; }
    __device__ __forceinline__ bool direct_neumann() const { return strat() == kStratDirectNeumann; }
    __device__ __forceinline__ bool sl_neumann() const { return strat() == kStratFwdSlNeumann; }

    __device__ __forceinline__ float ris_target_at(int type, const BPoint<D> &yp, const V<D> &c) const {
        if (type == kDirichlet) return fabsf(K.G(c, yp.p));
        if (type == kNeumann) return fabsf(K.dG_dny(yp.p, c, yp.n));
        return fabsf(K.dG_dny(yp.p, c, yp.n) + yp.alpha * K.G(c, yp.p));
    }
    __device__ __forceinline__ float ris_target(int type, const BPoint<D> &yp, const BPoint<D> &c) const {
        return ris_target_at(type, yp, c.p);
    }
    // Streaming RIS over K uniform candidates (scene.cuh:542-584, 847-889). A candidate's target
    // needs only its position, so the loop reads only the vertices of each candidate's element and
    // keeps the selected candidate's element (sel, 0xFFFFFFFF if none) and draws (su). The draws
    // are taken in the reference's order -- candidate i's D draws, then its selection draw -- but
    // candidate i + 1's draws and guide-table load are issued before candidate i's target is
    // evaluated, so two dependent load chains are in flight instead of one.
    __device__ __forceinline__ void ris_select(const BPoint<D> &yp, uint32_t &sel, float *su, float &w_sum,
                                               uint32_t &M) {
        sel = 0xFFFFFFFFu;
#pragma unroll
        for (int k = 0; k < D; k++) su[k] = 0.0f;
        w_sum = 0.0f;
        M = 0;
        const uint32_t K = p.n_resampling;
        if (K == 0) return;
        float u[D];
#pragma unroll
        for (int k = 0; k < D; k++) u[k] = rng.uniform();
        uint4 g = __ldg(s.area_guide + guide_bin(s.area_G, u[0]));
        for (uint32_t i = 0; i < K; i++) {
            const uint32_t idx = cdf_resolve(s.area_cdf, g, u[0]);
            const V<D> pos = uniform_position<D>(s, idx, u);
            const float r_sel = rng.uniform();
            float un[D];
#pragma unroll
            for (int k = 0; k < D; k++) un[k] = 0.0f;
            if (i + 1 < K) {
#pragma unroll
                for (int k = 0; k < D; k++) un[k] = rng.uniform();
                g = __ldg(s.area_guide + guide_bin(s.area_G, un[0]));
            }
            const float wi = ris_target_at(yp.type, yp, pos) * s.total_area;
            w_sum = w_sum + wi;
            M += 1;
            if (r_sel <= wi / w_sum) {
                sel = idx;
#pragma unroll
                for (int k = 0; k < D; k++) su[k] = u[k];
            }
#pragma unroll
            for (int k = 0; k < D; k++) u[k] = un[k];
        }
    }
    __device__ __forceinline__ BPoint<D> sample_ris(const BPoint<D> &yp, float &inv_pdf) {
        uint32_t sel, M;
        float su[D], w_sum;
        ris_select(yp, sel, su, w_sum, M);
        const BPoint<D> y = sel != 0xFFFFFFFFu ? uniform_point<D>(load_elem<D>(s, sel), su) : bp_zero<D>();
        inv_pdf = w_sum / fmax_ref(ris_target(yp.type, yp, y) * (float)M, kEps10);
        return y;
    }

    // compute_sample_unknown_boundary (estimator.cuh:232-357)
    __device__ __forceinline__ float unknown_boundary(const BPoint<D> &x) {
        float contrib = 0.0f, w = 1.0f;
        BPoint<D> y_prev = x;
        BPoint<D> y = bp_zero<D>();
        float ip = 0.0f;
        const uint32_t L = p.path_length;
        for (uint32_t m = 0; m < L; m++) {
            bounces++;
            if (m == L - 1) w = 0.5f * w;
            // In the last bounce only the known term counts: the transport after it (the next
            // sample and its weight) is never used, so it is skipped; the draws it would take come
            // after every draw that matters, so no path value changes.
            const bool last = m == L - 1;
            if (dl_dirichlet()) {
                y = sample_line_intersection<D>(s, rng, y_prev.p, ip);
                contrib = contrib + w * fbk(y_prev, y, ip);
                if (last) break;
                w = w * fbu(y_prev, y, ip, true);
                y_prev = y;
            } else if (direct_neumann()) {
                y = sample_boundary_value<D>(s, rng, ip);
                contrib = contrib + w * fbk(y_prev, y, ip);
                if (last) break;
                y = sample_line_intersection<D>(s, rng, y_prev.p, ip);
                w = w * fbu(y_prev, y, ip, true);
                y_prev = y;
            } else if (strat() == kStratSingleLayer) {
                contrib = contrib + w * fbk(y_prev, y, ip);
                if (last) break;
                if (p.n_resampling == 1) y = sample_uniform<D>(s, rng, ip);
                else y = sample_ris(y_prev, ip);
                w = w * fbu(y_prev, y, ip, true);
                y_prev = y;
            } else if (!kVol || p.n_volume == 0) {
                // no draw between the two samples (fbk draws only for a source term): take both at
                // once. The last bounce's transport (second sample, fbu) goes unused but is kept:
                // a straight-line loop body measured faster here (the headline workload) than an
                // exit before it, and nothing draws after the walk, so no value changes
                BPoint<D> ya;
                float ipa;
                sample_uniform_pair<D>(s, rng, ya, ipa, y, ip);
                contrib = contrib + w * fbk(y_prev, ya, ipa);
                w = w * fbu(y_prev, y, ip, true);
                y_prev = y;
            } else {
                y = sample_uniform<D>(s, rng, ip);
                contrib = contrib + w * fbk(y_prev, y, ip);
                if (last) break;
                y = sample_uniform<D>(s, rng, ip);
                w = w * fbu(y_prev, y, ip, true);
                y_prev = y;
            }
            if (w == 0.0f) break;
        }
        return contrib;
    }

    // compute_sample_path_contribution_domain (estimator.cuh:154-191 backward, 405-454 forward)
    __device__ __forceinline__ void domain(const V<D> &x, float out[D + 1]) {
        if (backward()) {
            BPoint<D> y, y1;
            float ip, ip1;
            if (dl_dirichlet()) {
                y = sample_line_intersection<D>(s, rng, x, ip);
                y1 = y;
                ip1 = ip;
            } else if (direct_neumann()) {
                y = sample_line_intersection<D>(s, rng, x, ip);
                y1 = sample_boundary_value<D>(s, rng, ip1);
            } else {
                sample_uniform_pair<D>(s, rng, y, ip, y1, ip1);
            }
            out[0] = sdk(x, y1, ip1);
            const V<D> g = gdk(x, y1, ip1);
#pragma unroll
            for (int i = 0; i < D; i++) out[1 + i] = g.v[i];
            const float mu = unknown_boundary(y);
            out[0] = out[0] + mu * sdu(x, y, ip);
            const V<D> gu = gdu(x, y, ip);
#pragma unroll
            for (int i = 0; i < D; i++) out[1 + i] = out[1 + i] + mu * gu.v[i];
            return;
        }
        BPoint<D> y, y2;
        float ip, ip2;
        y = sample_uniform<D>(s, rng, ip);
        out[0] = sdk(x, y, ip);
        const V<D> g = gdk(x, y, ip);
#pragma unroll
        for (int i = 0; i < D; i++) out[1 + i] = g.v[i];
        if (sl_neumann()) y = sample_boundary_value<D>(s, rng, ip);
        else y = sample_uniform<D>(s, rng, ip);
        y2 = sample_uniform<D>(s, rng, ip2);
        float w = ip * fbk(y, y2, ip2);
        BPoint<D> y_prev;
        const uint32_t L = p.path_length;
        for (uint32_t m = 0; m < L; m++) {
            bounces++;
            if (m == L - 1) w = w * 0.5f;
            out[0] = out[0] + w * sdu(x, y, 1.0f);
            const V<D> gu = gdu(x, y, 1.0f);
#pragma unroll
            for (int i = 0; i < D; i++) out[1 + i] = out[1 + i] + w * gu.v[i];
            if (m == L - 1) break;  // the transport after the last bounce is never used
            y_prev = y;
            if (sl_neumann()) y = sample_line_intersection<D>(s, rng, y_prev.p, ip);
            else y = sample_uniform<D>(s, rng, ip);
            w = fbu(y, y_prev, ip, false) * w;
        }
    }

    // Forward single-layer Neumann estimator with a per-element control-variate density sig
    // (storage order; no counterpart in the reference): u(x) = <G_x, sig> + <G_x, r>, r = s_r + K r,
    // s_r = s + K sig - sig. <G_x, sig> from n_pot uniform samples; <G_x, r> by the reference's
    // forward transport (estimator.cuh:433-451) from a uniform source point y0 with weight
    // A (s(y0) + K^ sig(y0) - sig(y0)), K^ sig from m_ker uniform samples.
    __device__ __forceinline__ void domain_cv(const V<D> &x, const float *__restrict__ sig, float out[D + 1]) {
        float p1 = 0.0f;
        V<D> g1 = vzero<D>();
        for (uint32_t k = 0; k < p.n_pot; k++) {
            float ip;
            uint32_t id;
            const BPoint<D> y = sample_uniform_idx<D>(s, rng, ip, id);
            const float c = __ldg(sig + id) * ip;
            p1 = p1 + K.G(y.p, x) * c;
            const V<D> g = K.dG_dx(y.p, x);
#pragma unroll
            for (int i = 0; i < D; i++) g1.v[i] = g1.v[i] + g.v[i] * c;
        }
        if (p.n_pot > 0) {
            p1 = p1 / (float)p.n_pot;
#pragma unroll
            for (int i = 0; i < D; i++) g1.v[i] = g1.v[i] / (float)p.n_pot;
        }
        float ip0;
        uint32_t id0;
        BPoint<D> y = sample_uniform_idx<D>(s, rng, ip0, id0);
        const float s0 = fbk(y, y, ip0);
        float ks = 0.0f;
        for (uint32_t j = 0; j < p.m_ker; j++) {
            float ipz;
            uint32_t idz;
            BPoint<D> z = sample_uniform_idx<D>(s, rng, ipz, idz);
            BPoint<D> yc = y;
            ks = ks + fbu(yc, z, ipz, true) * __ldg(sig + idz);
        }
        if (p.m_ker > 0) ks = ks / (float)p.m_ker;
        float w = ip0 * (s0 + ks - __ldg(sig + id0));
        float res = 0.0f;
        V<D> gres = vzero<D>();
        BPoint<D> y_prev;
        float ip = 0.0f;
        const uint32_t L = p.path_length;
        for (uint32_t m = 0; m < L; m++) {
            bounces++;
            if (m == L - 1) w = w * 0.5f;
            res = res + w * sdu(x, y, 1.0f);
            const V<D> gu = gdu(x, y, 1.0f);
#pragma unroll
            for (int i = 0; i < D; i++) gres.v[i] = gres.v[i] + w * gu.v[i];
            if (m == L - 1) break;  // the transport after the last bounce is never used
            y_prev = y;
            y = sample_line_intersection<D>(s, rng, y_prev.p, ip);
            w = fbu(y, y_prev, ip, false) * w;
        }
        out[0] = p1 + res;
#pragma unroll
        for (int i = 0; i < D; i++) out[1 + i] = g1.v[i] + gres.v[i];
    }

    // compute_sample_path_contribution_boundary (estimator.cuh:193-222 backward, 456-496 forward)
    __device__ __forceinline__ float boundary(const BPoint<D> &x) {
        if (backward()) {
            BPoint<D> y, y1;
            float ip, ip1;
            if (dl_dirichlet()) {
                y = sample_line_intersection<D>(s, rng, x.p, ip);
                y1 = y;
                ip1 = ip;
            } else if (direct_neumann()) {
                y = sample_line_intersection<D>(s, rng, x.p, ip);
                y1 = sample_boundary_value<D>(s, rng, ip1);
            } else {
                y = sample_uniform<D>(s, rng, ip);
                y1 = sample_uniform<D>(s, rng, ip1);
            }
            float r = sbk(x, y1, ip1);
            const float mu = unknown_boundary(y);
            r = r + mu * sbu(x, y, ip);
            return r;
        }
        BPoint<D> y, y2;
        float ip, ip2;
        y = sample_uniform<D>(s, rng, ip);
        float r = sbk(x, y, ip);
        if (sl_neumann()) y = sample_boundary_value<D>(s, rng, ip);
        else y = sample_uniform<D>(s, rng, ip);
        y2 = sample_uniform<D>(s, rng, ip2);
        float w = ip * fbk(y, y2, ip2);
        BPoint<D> y_prev;
        const uint32_t L = p.path_length;
        for (uint32_t m = 0; m < L; m++) {
            bounces++;
            if (m == L - 1) w = w * 0.5f;
            r = r + sbu(x, y, 1.0f) * w;
            if (m == L - 1) break;  // the transport after the last bounce is never used
            y_prev = y;
            if (sl_neumann()) y = sample_line_intersection<D>(s, rng, y_prev.p, ip);
            else y = sample_uniform<D>(s, rng, ip);
            w = fbu(y, y_prev, ip, false) * w;
        }
        return r;
    }
};

// One scene of a batched launch: its view, parameters, first global work unit, first point row
// in the concatenated point / sum arrays, point count and units per point.
template <int D> struct BatchEntry {
    SceneView<D> view;
    WalkParams params;
    uint64_t unit_begin;
    uint32_t point_begin, n_points, slabs;
    uint32_t cls;  // batch_walk_class of the parameters
};

// The specialised walk a batched scene runs: 1 = backward single layer, 2 = forward single-layer
// Neumann (both without a source term), 0 = the general walk.
__host__ __device__ __forceinline__ uint32_t batch_walk_class(const WalkParams &p) {
    if (p.n_volume != 0) return 0u;
    const int st = strategy_of(p.bie, p.estimator, p.problem);
    if (st == kStratSingleLayer) return 1u;
    if (st == kStratFwdSlNeumann) return 2u;
    return 0u;
}

constexpr uint32_t kStreamDomain = 0u;
constexpr uint32_t kStreamBoundary = 1u;

}  // namespace wobgb
