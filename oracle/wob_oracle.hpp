// CPU oracle for the walk-on-boundary (WoB) hot path.
//
// TEST INFRASTRUCTURE ONLY. This header is the checker the CUDA engine is compared with. Only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may link or call it; the engine
// under wobtoolbox_gb300/ never does.
//
// It is a line-by-line CPU restatement of the reference's hot path (rsugimoto/WoBToolbox):
//   equation_kernel.cuh:67-145  fundamental solutions G, dG/dx, dG/dn_y, d2G/dxdn_y
//   bie_models.cuh:53-590       single-layer, double-layer and direct BIE models
//   scene.cuh:30-43,378-937     CDF search, uniform / line-intersection / RIS / |g| sampling
//   estimator.cuh:113-504       backward and forward estimators, the bounce loop
//   utils.cuh:148-166           Kahan summation (used for the area and |g| CDFs)
// with three documented substitutions, all shared with the engine so that the two produce the
// same walk for the same (seed, point, path):
//   * cuRAND XORWOW (utils.cuh:24-40) -> stateless Philox4x32-10 (Salmon et al., SC'11), one
//     counter stream per path, uniforms in (0,1] like curand_uniform;
//   * the lbvh "all hits of an infinite line" query (scene.cuh:483-486, library source absent)
//     -> brute force over every element; hits are kept in element order (the engine stores
//     elements in BVH leaf order, so its depth-first traversal yields the same order);
//   * CUDA sincospi / std::log -> the polynomial sincospi_own / log_own below, so the two sides
//     round identically.
// All arithmetic is IEEE single precision with no contraction (build with -ffp-contract=off);
// fused multiply-adds appear only where written as std::fma.
//
// Parity status: the reference cannot be built here (its Eigen, lbvh, libigl and json
// submodules are empty), and it ships no golden vectors or tests. The oracle is pinned by the
// reference's own validation method: known-answer tests against closed-form harmonic solutions
// (apps/general_2d.cu:73-104, apps/general_3d.cu:75-108) and the closed-form double-layer walk
// of apps/simple_wob_and_wos.cu:81-108. Bit-level parity with Eigen/lbvh is unpinned.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace wob_oracle {

// ------------------------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy as 1, 2, 3").
// ------------------------------------------------------------------------------------------
struct Philox4x32 {
    static constexpr uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    static constexpr uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    static inline void mulhilo(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
        const uint64_t p = (uint64_t)a * (uint64_t)b;
        hi = (uint32_t)(p >> 32);
        lo = (uint32_t)p;
    }
    static inline void round(uint32_t c[4], uint32_t k0, uint32_t k1) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo(M0, c[0], hi0, lo0);
        mulhilo(M1, c[2], hi1, lo1);
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n1 = lo1, n2 = hi0 ^ c[3] ^ k1, n3 = lo0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    }
    static inline void generate(const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
        uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
        for (int r = 0; r < 10; r++) {
            round(c, k0, k1);
            k0 += W0;
            k1 += W1;
        }
        out[0] = c[0]; out[1] = c[1]; out[2] = c[2]; out[3] = c[3];
    }
};

// One random stream per (seed, stream tag, point, path). Counter = (block, path lo, path hi, point),
// key = (seed lo, seed hi + stream tag). Uniforms are ((x >> 8) + 1) * 2^-24, in (0, 1].
struct Rng {
    uint32_t key0, key1, ctr1, ctr2, ctr3, block;
    uint32_t buf[4];
    int used;
    Rng(uint64_t seed, uint32_t stream, uint32_t point, uint64_t path)
        : key0((uint32_t)seed), key1((uint32_t)(seed >> 32) + stream), ctr1((uint32_t)path),
          ctr2((uint32_t)(path >> 32)), ctr3(point), block(0), used(4) {}
    inline float uniform() {
        if (used == 4) {
            const uint32_t c[4] = {block, ctr1, ctr2, ctr3};
            Philox4x32::generate(c, key0, key1, buf);
            block++;
            used = 0;
        }
        const uint32_t x = buf[used++];
        return (float)((x >> 8) + 1u) * 0x1p-24f;
    }
};

// ------------------------------------------------------------------------------------------
// Scalar math restated from first principles (no libm transcendental is used on the walk).
// ------------------------------------------------------------------------------------------
inline float fmax_ref(float a, float b) { return (a < b) ? b : a; }  // std::max semantics
inline float fmin_ref(float a, float b) { return (b < a) ? b : a; }  // std::min semantics

// sin(pi x), cos(pi x): reduce x = q/2 + r with |r| <= 1/4, Taylor polynomials of sin(pi r) and
// cos(pi r) in r^2 (truncation error < 1e-11), then rotate by the quadrant q mod 4.
inline void sincospi_own(float x, float *s_out, float *c_out) {
    const float q = std::nearbyint(x * 2.0f);
    const float r = x - q * 0.5f;
    const float z = r * r;
    float sp = -0x1.e3075p-8f;      // -pi^11/11!
    sp = sp * z + 0x1.507834p-4f;   //  pi^9/9!
    sp = sp * z - 0x1.32d2ccp-1f;   // -pi^7/7!
    sp = sp * z + 0x1.466bc6p+1f;   //  pi^5/5!
    sp = sp * z - 0x1.4abbcep+2f;   // -pi^3/3!
    sp = sp * z + 0x1.921fb6p+1f;   //  pi
    const float s = sp * r;
    float cp = 0x1.f9d38ap-10f;
    cp = cp * z - 0x1.a6d1f2p-6f;
    cp = cp * z + 0x1.e1f506p-3f;
    cp = cp * z - 0x1.55d3c8p+0f;
    cp = cp * z + 0x1.03c1f0p+2f;
    cp = cp * z - 0x1.3bd3ccp+2f;
    const float c = cp * z + 1.0f;
    const int qi = ((int)q) & 3;
    if (qi == 0) { *s_out = s; *c_out = c; }
    else if (qi == 1) { *s_out = c; *c_out = -s; }
    else if (qi == 2) { *s_out = -s; *c_out = -c; }
    else { *s_out = -c; *c_out = s; }
}

// Natural log: x = m 2^e with m in (sqrt(1/2), sqrt(2)], log m = 2 atanh(s), s = (m-1)/(m+1),
// series to s^11 (truncation error < 1e-10), e ln2 added in two parts.
inline float log_own(float x) {
    if (!(x > 0.0f)) return (x == 0.0f) ? -std::numeric_limits<float>::infinity()
                                        : std::numeric_limits<float>::quiet_NaN();
    if (x == std::numeric_limits<float>::infinity()) return x;
    int e_adj = 0;
    if (x < 0x1p-126f) { x = x * 0x1p+23f; e_adj = -23; }
    uint32_t bits;
    std::memcpy(&bits, &x, 4);
    int e = (int)(bits >> 23) - 127 + e_adj;
    const uint32_t mb = (bits & 0x007fffffu) | 0x3f800000u;
    float m;
    std::memcpy(&m, &mb, 4);
    if (m > 0x1.6a09e6p+0f) { m = m * 0.5f; e += 1; }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float z = s * s;
    float p = 0x1.745d18p-4f;      // 1/11
    p = p * z + 0x1.c71c72p-4f;    // 1/9
    p = p * z + 0x1.24924ap-3f;    // 1/7
    p = p * z + 0x1.99999ap-3f;    // 1/5
    p = p * z + 0x1.555556p-2f;    // 1/3
    p = p * z + 1.0f;
    const float logm = (2.0f * s) * p;
    const float fe = (float)e;
    return fe * 0x1.62e4p-1f + (fe * 0x1.7f7d1cp-20f + logm);
}

// ------------------------------------------------------------------------------------------
// Small vectors (no Eigen). Sums are evaluated left to right.
// ------------------------------------------------------------------------------------------
template <int D> struct Vec {
    float v[D];
    float &operator[](int i) { return v[i]; }
    float operator[](int i) const { return v[i]; }
};
template <int D> inline Vec<D> vzero() { Vec<D> r; for (int i = 0; i < D; i++) r.v[i] = 0.0f; return r; }
template <int D> inline Vec<D> operator+(const Vec<D> &a, const Vec<D> &b) { Vec<D> r; for (int i = 0; i < D; i++) r.v[i] = a.v[i] + b.v[i]; return r; }
template <int D> inline Vec<D> operator-(const Vec<D> &a, const Vec<D> &b) { Vec<D> r; for (int i = 0; i < D; i++) r.v[i] = a.v[i] - b.v[i]; return r; }
template <int D> inline Vec<D> operator*(float s, const Vec<D> &a) { Vec<D> r; for (int i = 0; i < D; i++) r.v[i] = s * a.v[i]; return r; }
template <int D> inline Vec<D> operator/(const Vec<D> &a, float s) { Vec<D> r; for (int i = 0; i < D; i++) r.v[i] = a.v[i] / s; return r; }
template <int D> inline float dot(const Vec<D> &a, const Vec<D> &b) {
    float s = a.v[0] * b.v[0];
    for (int i = 1; i < D; i++) s = s + a.v[i] * b.v[i];
    return s;
}
template <int D> inline float sqnorm(const Vec<D> &a) { return dot(a, a); }
template <int D> inline float norm(const Vec<D> &a) { return std::sqrt(sqnorm(a)); }
// Eigen's normalized(): v / sqrt(|v|^2) when |v|^2 > 0, else v unchanged.
template <int D> inline Vec<D> normalized(const Vec<D> &a) {
    const float z = sqnorm(a);
    if (z > 0.0f) return a / std::sqrt(z);
    return a;
}
inline Vec<3> cross(const Vec<3> &a, const Vec<3> &b) {
    Vec<3> r;
    r.v[0] = a.v[1] * b.v[2] - a.v[2] * b.v[1];
    r.v[1] = a.v[2] * b.v[0] - a.v[0] * b.v[2];
    r.v[2] = a.v[0] * b.v[1] - a.v[1] * b.v[0];
    return r;
}

// ------------------------------------------------------------------------------------------
// Enums: same numbering as the reference (bie_models.cuh:21-22, estimator.cuh:24,38, points.hpp:22).
// ------------------------------------------------------------------------------------------
enum BoundaryType { Dirichlet = 0, Neumann = 1, Robin = 2 };
enum BIEModelType { IndirectSingleLayer = 0, IndirectDoubleLayer = 1, Direct = 2 };
enum DomainType { InteriorDomain = 0, ExteriorDomain = 1 };
enum EstimatorType { BackwardEstimator = 0, ForwardEstimator = 1 };
enum ProblemType { DirichletProblem = 0, NeumannProblem = 1, RobinProblem = 2, MixedProblem = 3 };

constexpr float kEps10 = 10.0f * std::numeric_limits<float>::epsilon();  // scene.cuh:418,531
constexpr unsigned kHitBuffer = 64;                                        // scene.cuh:481

// ------------------------------------------------------------------------------------------
// Fundamental solutions of the Laplace equation (equation_kernel.cuh:67-145).
// ------------------------------------------------------------------------------------------
template <int D> struct EqKernel;

template <> struct EqKernel<2> {
    float eps;
    // G = -1/(2pi) log max(|y-x|, eps)                                (equation_kernel.cuh:74-76)
    float G(const Vec<2> &y, const Vec<2> &x) const {
        return -0x1.45f306p-3f * log_own(fmax_ref(norm(y - x), eps));
    }
    // dG/dx = 1/(2pi) r^ / max(|r|, eps)                                 (:78-81)
    Vec<2> dG_dx(const Vec<2> &y, const Vec<2> &x) const {
        const Vec<2> r = y - x;
        return (0x1.45f306p-3f * normalized(r)) / fmax_ref(norm(r), eps);
    }
    // dG/dn_y = -1/(2pi) r^.n_y / max(|r|, eps)                         (:83-86)
    float dG_dny(const Vec<2> &y, const Vec<2> &x, const Vec<2> &ny) const {
        const Vec<2> r = y - x;
        return -0x1.45f306p-3f * dot(normalized(r), ny) / fmax_ref(norm(r), eps);
    }
    // d2G/dx dn_y = 1/(2pi max(|r|^2, eps)) (n_y - 2 (r^.n_y) r^)       (:88-92)
    Vec<2> d2G_dxdny(const Vec<2> &y, const Vec<2> &x, const Vec<2> &ny) const {
        const Vec<2> r = y - x;
        const Vec<2> rh = normalized(r);
        const float k = 1.0f / (0x1.921fb6p+2f * fmax_ref(sqnorm(r), eps));
        return k * (ny - (2.0f * dot(rh, ny)) * rh);
    }
    // d2G/dn_x dn_y                                                       (:94-100)
    float d2G_dnxdny(const Vec<2> &y, const Vec<2> &x, const Vec<2> &ny, const Vec<2> &nx) const {
        const Vec<2> r = y - x;
        const Vec<2> rh = normalized(r);
        const float k = 1.0f / (0x1.921fb6p+2f * fmax_ref(sqnorm(r), eps));
        return k * (dot(nx, ny) - 2.0f * dot(rh, nx) * dot(rh, ny));
    }
};

template <> struct EqKernel<3> {
    float eps;
    // G = 1/(4pi max(|r|, eps))                                          (:115-117)
    float G(const Vec<3> &y, const Vec<3> &x) const {
        return 1.0f / (0x1.921fb6p+3f * fmax_ref(norm(y - x), eps));
    }
    // dG/dx = 1/(4pi) r^ / max(|r|^2, eps)                               (:119-122)
    Vec<3> dG_dx(const Vec<3> &y, const Vec<3> &x) const {
        const Vec<3> r = y - x;
        return (0x1.45f306p-4f * normalized(r)) / fmax_ref(sqnorm(r), eps);
    }
    // dG/dn_y = -1/(4pi) r^.n_y / max(|r|^2, eps)                       (:124-127)
    float dG_dny(const Vec<3> &y, const Vec<3> &x, const Vec<3> &ny) const {
        const Vec<3> r = y - x;
        return -0x1.45f306p-4f * dot(normalized(r), ny) / fmax_ref(sqnorm(r), eps);
    }
    // d2G/dx dn_y = 1/(4pi max(|r|^3, eps)) (n_y - 3 (r^.n_y) r^)        (:129-134)
    Vec<3> d2G_dxdny(const Vec<3> &y, const Vec<3> &x, const Vec<3> &ny) const {
        const Vec<3> r = y - x;
        const Vec<3> rh = normalized(r);
        const float k = 1.0f / (0x1.921fb6p+3f * fmax_ref(norm(r) * sqnorm(r), eps));
        return k * (ny - (3.0f * dot(rh, ny)) * rh);
    }
    float d2G_dnxdny(const Vec<3> &y, const Vec<3> &x, const Vec<3> &ny, const Vec<3> &nx) const {
        const Vec<3> r = y - x;
        const Vec<3> rh = normalized(r);
        const float k = 1.0f / (0x1.921fb6p+3f * fmax_ref(norm(r) * sqnorm(r), eps));
        return k * (dot(nx, ny) - 3.0f * dot(rh, nx) * dot(rh, ny));
    }
};

// ------------------------------------------------------------------------------------------
// Points and elements (points.hpp:32-48, scene.cuh:378-397, 646-678).
// ------------------------------------------------------------------------------------------
template <int D> struct BoundaryPoint {
    Vec<D> p, n;
    float interior_angle;
    float boundary_value;
    int boundary_type;
    float robin_alpha;
};
template <int D> inline BoundaryPoint<D> bp_zero() {
    BoundaryPoint<D> b;
    b.p = vzero<D>(); b.n = vzero<D>();
    b.interior_angle = 0.0f; b.boundary_value = 0.0f; b.boundary_type = Dirichlet; b.robin_alpha = 0.0f;
    return b;
}
// The reference constructs BoundaryPoint{x.p} for domain points: n = 0, other members zero.
template <int D> inline BoundaryPoint<D> bp_from_point(const Vec<D> &p) {
    BoundaryPoint<D> b = bp_zero<D>();
    b.p = p;
    return b;
}

// Element: D vertices, normal, per-vertex boundary value and Robin alpha, one boundary type.
// Sees every line query the oracle makes (used to measure the work of a reference binary BVH on
// the queries of a workload, oracle/lbvh_count.hpp); null except while measuring.
struct LineQueryObserver {
    virtual void on_line(const float *o, const float *d, int dim) = 0;
    virtual ~LineQueryObserver() = default;
};
inline thread_local LineQueryObserver *g_line_observer = nullptr;

template <int D> struct Element {
    Vec<D> v[D];
    Vec<D> n;
    float bv[D];
    float alpha[D];
    int type;
};

// |b-a| (2D), |(c-a) x (b-a)|/2 (3D)                                      (scene.cuh:384,652-654)
inline float elem_area(const Element<2> &e) { return norm(e.v[1] - e.v[0]); }
inline float elem_area(const Element<3> &e) { return norm(cross(e.v[2] - e.v[0], e.v[1] - e.v[0])) / 2.0f; }
// Importance of an element for |g| sampling                              (scene.cuh:386-392,656-663)
inline float elem_boundary_value(const Element<2> &e) {
    return elem_area(e) * (std::fabs(e.bv[0]) + std::fabs(e.bv[1])) / 2.0f;
}
inline float elem_boundary_value(const Element<3> &e) {
    return elem_area(e) * (std::fabs(e.bv[0]) + std::fabs(e.bv[1]) + std::fabs(e.bv[2])) / 3.0f;
}
// val1 + u (val2 - val1)                                                 (scene.cuh:393-396)
inline float interp2(float a, float b, float u) { return a + u * (b - a); }
inline Vec<2> interp2(const Vec<2> &a, const Vec<2> &b, float u) { return a + u * (b - a); }
// (1-sqrt u1) v1 + sqrt u1 (1-u2) v2 + u2 sqrt u1 v3                       (scene.cuh:665-671)
inline float interp3(float a, float b, float c, float u1, float u2) {
    const float s = std::sqrt(u1);
    return (1.0f - s) * a + s * (1.0f - u2) * b + u2 * s * c;
}
inline Vec<3> interp3(const Vec<3> &a, const Vec<3> &b, const Vec<3> &c, float u1, float u2) {
    const float s = std::sqrt(u1);
    const float k1 = 1.0f - s, k2 = s * (1.0f - u2), k3 = u2 * s;
    Vec<3> r;
    for (int i = 0; i < 3; i++) r.v[i] = k1 * a.v[i] + k2 * b.v[i] + k3 * c.v[i];
    return r;
}

// binary_search over a CDF: first i with key <= cdf[i], else n-1          (scene.cuh:30-43)
inline unsigned binary_search(const float *a, unsigned n, float key) {
    unsigned low = 0, high = n - 1;
    while (low < high) {
        const unsigned mid = (high + low) / 2;
        if (key <= a[mid]) high = mid;
        else low = mid + 1;
    }
    return high;
}

// ------------------------------------------------------------------------------------------
// Line / element intersection (scene.cuh:414-436, 707-730), restated with Cramer's rule and a
// division-free inside test. Returns true and the hit point for an accepted hit.
// ------------------------------------------------------------------------------------------
inline bool line_elem_intersect(const Vec<2> &o, const Vec<2> &d, const Element<2> &e, Vec<2> &p) {
    const Vec<2> ed = e.v[0] - e.v[1];          // a - b
    const Vec<2> w = e.v[0] - o;                // a - origin
    const float det = d.v[0] * ed.v[1] - d.v[1] * ed.v[0];
    const float tn = w.v[0] * ed.v[1] - w.v[1] * ed.v[0];
    const float sn = d.v[0] * w.v[1] - d.v[1] * w.v[0];
    bool inside;
    if (det > 0.0f) inside = (sn >= 0.0f) && (sn <= det);
    else if (det < 0.0f) inside = (sn <= 0.0f) && (sn >= det);
    else inside = false;
    if (!inside) return false;
    const float t = tn / det;
    if (!(std::fabs(t) > kEps10)) return false;  // rejects |t| <= 10 eps and NaN
    p = o + t * d;
    return true;
}

inline bool line_elem_intersect(const Vec<3> &o, const Vec<3> &d, const Element<3> &e, Vec<3> &p) {
    const Vec<3> e1 = e.v[0] - e.v[1];          // a - b
    const Vec<3> e2 = e.v[0] - e.v[2];          // a - c
    const Vec<3> q = cross(e1, e2);
    const Vec<3> w = e.v[0] - o;                // a - origin
    const float det = dot(d, q);
    const float tn = dot(w, q);
    const Vec<3> wd = cross(w, d);
    const float bn = -dot(e2, wd);
    const float gn = dot(e1, wd);
    bool inside;
    if (det > 0.0f) inside = (bn >= 0.0f) && (gn >= 0.0f) && (bn + gn <= det);
    else if (det < 0.0f) inside = (bn <= 0.0f) && (gn <= 0.0f) && (bn + gn >= det);
    else inside = false;
    if (!inside) return false;
    const float t = tn / det;
    if (!(std::fabs(t) > kEps10)) return false;
    p = o + t * d;
    return true;
}

// Barycentric coordinates of p in triangle (a, b, c) (scene.cuh:45-69, the libigl formula).
inline void barycentric(const Vec<3> &p, const Vec<3> &a, const Vec<3> &b, const Vec<3> &c, float L[3]) {
    const Vec<3> v0 = b - a, v1 = c - a, v2 = p - a;
    const float d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1);
    const float d20 = dot(v2, v0), d21 = dot(v2, v1);
    const float denom = d00 * d11 - d01 * d01;
    L[1] = (d11 * d20 - d01 * d21) / denom;
    L[2] = (d00 * d21 - d01 * d20) / denom;
    L[0] = 1.0f - (L[1] + L[2]);
}

// ------------------------------------------------------------------------------------------
// Volume cache (scene.cuh:78-120, 206-252): source values on a grid and an |f| CDF.
// The CDF is prefix(|f|) / total, both in double, rounded to float (the reference builds it
// with Thrust reductions of unspecified order).
// ------------------------------------------------------------------------------------------
template <int D> struct VolumeCache {
    unsigned grid_res = 0;
    float domain_size = 0.0f;
    std::vector<float> cache, cdf;
    void build(unsigned res, float size, const float *values) {
        grid_res = res;
        domain_size = size;
        size_t n = 1;
        for (int i = 0; i < D; i++) n *= res;
        cache.assign(values, values + n);
        cdf.resize(n);
        double total = 0.0;
        for (size_t i = 0; i < n; i++) total += std::fabs((double)values[i]);
        if (total == 0.0) {
            for (size_t i = 0; i < n; i++) cdf[i] = (float)((double)(i + 1) / (double)n);
        } else {
            double acc = 0.0;
            for (size_t i = 0; i < n; i++) {
                acc += std::fabs((double)values[i]);
                cdf[i] = (float)(acc / total);
            }
        }
    }
    unsigned count() const { return (unsigned)cache.size(); }
};

// idx -> cell centre in (-size/2, size/2)^D                               (utils.cuh:92-100)
template <int D> inline Vec<D> idx_to_domain_point(unsigned idx, unsigned res, float size) {
    const float dx = size / (float)res;
    unsigned c[3] = {idx % res, (idx / res) % res, idx / (res * res)};
    Vec<D> p;
    for (int i = 0; i < D; i++) p.v[i] = ((float)c[i] + 0.5f) * dx - size / 2.0f;
    return p;
}

template <int D> struct VolumeSample {
    Vec<D> p;
    float value;
    float inv_pdf;
};

// ------------------------------------------------------------------------------------------
// Scene (scene.cuh:264-326 host build, 438-642 / 732-937 device queries).
// ------------------------------------------------------------------------------------------
template <int D> struct Scene {
    std::vector<Element<D>> elems;       // in the engine's storage (BVH leaf) order
    std::vector<float> area_cdf, bv_cdf;
    float total_area = 0.0f, total_bv = 0.0f;
    const VolumeCache<D> *vol = nullptr;

    // scene.cuh:265-299: Kahan prefix sums in float, then each entry divided by the total.
    void build() {
        const size_t n = elems.size();
        area_cdf.resize(n);
        bv_cdf.resize(n);
        {
            float sum = 0.0f, c = 0.0f;
            for (size_t i = 0; i < n; i++) {
                const float y = elem_area(elems[i]) - c;
                const float t = sum + y;
                c = (t - sum) - y;
                sum = t;
                area_cdf[i] = sum;
            }
            total_area = sum;
            for (size_t i = 0; i < n; i++) area_cdf[i] = area_cdf[i] / total_area;
            // Made nondecreasing: after a compensated step a zero-weight element can sit one
            // ulp below its predecessor (shared with the engine, no effect otherwise).
            for (size_t i = 1; i < n; i++) if (area_cdf[i] < area_cdf[i - 1]) area_cdf[i] = area_cdf[i - 1];
        }
        {
            float sum = 0.0f, c = 0.0f;
            for (size_t i = 0; i < n; i++) {
                const float y = elem_boundary_value(elems[i]) - c;
                const float t = sum + y;
                c = (t - sum) - y;
                sum = t;
                bv_cdf[i] = sum;
            }
            total_bv = sum;
            for (size_t i = 0; i < n; i++) bv_cdf[i] = bv_cdf[i] / total_bv;
            for (size_t i = 1; i < n; i++) if (bv_cdf[i] < bv_cdf[i - 1]) bv_cdf[i] = bv_cdf[i - 1];
        }
    }

    // Optional candidate filter for line_query (oracle/lbvh_count.hpp's padded binary BVH): writes
    // the elements whose boxes the line crosses, in any order, and returns their number (or
    // UINT32_MAX when more than cap). The exact test and the storage order stay those below.
    const void *accel = nullptr;
    unsigned (*accel_candidates)(const void *, const float *o, const float *d, unsigned *cand, unsigned cap) = nullptr;

    // "All hits of the infinite line" in element order (brute force, or the exact test on the
    // candidates of the filter, sorted). Returns the full count; at most kHitBuffer element
    // indices are written.
    unsigned line_query(const Vec<D> &o, const Vec<D> &d, unsigned *hits) const {
        if (g_line_observer) g_line_observer->on_line(o.v, d.v, D);
        unsigned count = 0;
        Vec<D> p;
        if (accel) {
            unsigned cand[4096];
            const unsigned nc = accel_candidates(accel, o.v, d.v, cand, 4096);
            if (nc != 0xFFFFFFFFu) {
                std::sort(cand, cand + nc);
                for (unsigned k = 0; k < nc; k++) {
                    if (line_elem_intersect(o, d, elems[cand[k]], p)) {
                        if (count < kHitBuffer) hits[count] = cand[k];
                        count++;
                    }
                }
                return count;
            }
        }
        for (unsigned i = 0; i < (unsigned)elems.size(); i++) {
            if (line_elem_intersect(o, d, elems[i], p)) {
                if (count < kHitBuffer) hits[count] = i;
                count++;
            }
        }
        return count;
    }

    // scene.cuh:441-462 (2D), 734-758 (3D)
    BoundaryPoint<D> sample_uniform(Rng &rng, float &inv_pdf) const {
        const float u1 = rng.uniform();
        const unsigned idx = binary_search(area_cdf.data(), (unsigned)elems.size(), u1);
        const Element<D> &e = elems[idx];
        BoundaryPoint<D> r;
        if constexpr (D == 2) {
            const float u2 = rng.uniform();
            r.p = interp2(e.v[0], e.v[1], u2);
            r.n = e.n;
            r.interior_angle = 0.5f;
            r.boundary_value = interp2(e.bv[0], e.bv[1], u2);
            r.boundary_type = e.type;
            r.robin_alpha = interp2(e.alpha[0], e.alpha[1], u2);
        } else {
            const float u2 = rng.uniform();
            const float u3 = rng.uniform();
            r.p = interp3(e.v[0], e.v[1], e.v[2], u2, u3);
            r.n = e.n;
            r.interior_angle = 0.5f;
            r.boundary_value = interp3(e.bv[0], e.bv[1], e.bv[2], u2, u3);
            r.boundary_type = e.type;
            r.robin_alpha = interp3(e.alpha[0], e.alpha[1], e.alpha[2], u2, u3);
        }
        inv_pdf = total_area;
        return r;
    }

    // scene.cuh:464-516 (2D), 760-821 (3D): random line through x, uniform pick among its hits.
    BoundaryPoint<D> sample_line_intersection2(Rng &rng, const Vec<D> &x, unsigned &m_out) const {
        Vec<D> dir;
        if constexpr (D == 2) {
            const float theta = rng.uniform();
            sincospi_own(theta, &dir.v[0], &dir.v[1]);
        } else {
            dir.v[2] = rng.uniform();
            const float phi = 2.0f * rng.uniform();
            sincospi_own(phi, &dir.v[0], &dir.v[1]);
            const float r = std::sqrt(1.0f - dir.v[2] * dir.v[2]);
            dir.v[0] = dir.v[0] * r;
            dir.v[1] = dir.v[1] * r;
        }
        unsigned hits[kHitBuffer];
        unsigned m = line_query(x, dir, hits);
        if (m == 0) {
            BoundaryPoint<D> z = bp_zero<D>();
            z.interior_angle = 0.5f;
            m_out = 0;
            return z;
        }
        m = std::min(m, kHitBuffer);
        const float u = rng.uniform();
        const unsigned k = std::min(m - 1, (unsigned)((float)m * u));
        const Element<D> &e = elems[hits[k]];
        Vec<D> p = x;  // overwritten: the element is a recorded hit
        line_elem_intersect(x, dir, e, p);
        BoundaryPoint<D> r;
        r.p = p;
        r.n = e.n;
        r.interior_angle = 0.5f;
        r.boundary_type = e.type;
        if constexpr (D == 2) {
            const float t = norm(p - e.v[0]) / elem_area(e);
            r.boundary_value = interp2(e.bv[0], e.bv[1], t);
            r.robin_alpha = interp2(e.alpha[0], e.alpha[1], t);
        } else {
            float L[3];
            barycentric(p, e.v[0], e.v[1], e.v[2], L);
            r.boundary_value = L[0] * e.bv[0] + L[1] * e.bv[1] + L[2] * e.bv[2];
            r.robin_alpha = L[0] * e.alpha[0] + L[1] * e.alpha[1] + L[2] * e.alpha[2];
        }
        m_out = m;
        return r;
    }

    // scene.cuh:524-535 (2D): inv_pdf = m pi |r| / max(|r^.n|, 10 eps);
    // scene.cuh:829-840 (3D): inv_pdf = m 2 pi |r|^2 / max(|r^.n|, 10 eps).
    BoundaryPoint<D> sample_line_intersection(Rng &rng, const Vec<D> &x, float &inv_pdf) const {
        unsigned m;
        BoundaryPoint<D> r = sample_line_intersection2(rng, x, m);
        const Vec<D> rv = r.p - x;
        const float cosv = fmax_ref(std::fabs(dot(normalized(rv), r.n)), kEps10);
        if constexpr (D == 2) inv_pdf = (float)m * 0x1.921fb6p+1f * norm(rv) / cosv;
        else inv_pdf = (float)m * 2.0f * 0x1.921fb6p+1f * sqnorm(rv) / cosv;
        return r;
    }

    // scene.cuh:542-584 / 847-889: streaming RIS over K uniform candidates.
    template <class F>
    BoundaryPoint<D> sample_ris(Rng &rng, F target, unsigned K, float &inv_pdf) const {
        BoundaryPoint<D> y = bp_zero<D>();
        float w_sum = 0.0f;
        unsigned M = 0;
        for (unsigned i = 0; i < K; i++) {
            float ip;
            const BoundaryPoint<D> xi = sample_uniform(rng, ip);
            const float wi = target(xi) * ip;
            w_sum = w_sum + wi;
            M += 1;
            if (rng.uniform() <= wi / w_sum) y = xi;
        }
        inv_pdf = w_sum / fmax_ref(target(y) * (float)M, kEps10);
        return y;
    }

    // scene.cuh:586-622 (2D, linear-density inversion on the element), 891-918 (3D).
    BoundaryPoint<D> sample_boundary_value(Rng &rng, float &inv_pdf) const {
        const float u1 = rng.uniform();
        const unsigned idx = binary_search(bv_cdf.data(), (unsigned)elems.size(), u1);
        const Element<D> &e = elems[idx];
        BoundaryPoint<D> r;
        if constexpr (D == 2) {
            const float u2 = rng.uniform();
            const float ba = std::fabs(e.bv[0]), bb = std::fabs(e.bv[1]);
            float t;
            if (std::fabs(ba - bb) < kEps10) t = u2;
            else t = (-ba + std::sqrt(ba * ba + u2 * (bb * bb - ba * ba))) / (bb - ba);
            r.p = interp2(e.v[0], e.v[1], t);
            r.n = e.n;
            r.interior_angle = 0.5f;
            r.boundary_value = interp2(e.bv[0], e.bv[1], t);
            r.boundary_type = e.type;
            r.robin_alpha = interp2(e.alpha[0], e.alpha[1], t);
            inv_pdf = total_bv / (ba + t * (bb - ba));
        } else {
            const float pmf = idx == 0 ? bv_cdf[idx] : bv_cdf[idx] - bv_cdf[idx - 1];
            const float u2 = rng.uniform();
            const float u3 = rng.uniform();
            r.p = interp3(e.v[0], e.v[1], e.v[2], u2, u3);
            r.n = e.n;
            r.interior_angle = 0.5f;
            r.boundary_value = interp3(e.bv[0], e.bv[1], e.bv[2], u2, u3);
            r.boundary_type = e.type;
            r.robin_alpha = interp3(e.alpha[0], e.alpha[1], e.alpha[2], u2, u3);
            inv_pdf = elem_area(e) / pmf;
        }
        return r;
    }

    // scene.cuh:100-120: source-value sampling of the volume cache.
    VolumeSample<D> sample_volume(Rng &rng) const {
        VolumeSample<D> s;
        const unsigned n = vol->count();
        const float u = rng.uniform();
        const unsigned idx = binary_search(vol->cdf.data(), n, u);
        s.p = idx_to_domain_point<D>(idx, vol->grid_res, vol->domain_size);
        for (int i = 0; i < D; i++) {
            const float uj = rng.uniform();
            s.p.v[i] = s.p.v[i] + (uj - 0.5f) * vol->domain_size / (float)vol->grid_res;
        }
        s.value = vol->cache[idx];
        const float pdf = idx == 0 ? vol->cdf[idx] : vol->cdf[idx] - vol->cdf[idx - 1];
        float cell = 1.0f;
        for (int i = 0; i < D; i++) cell = cell * (vol->domain_size / (float)vol->grid_res);
        s.inv_pdf = cell / pdf;
        return s;
    }
};

// ------------------------------------------------------------------------------------------
// Solver parameters (the reference's Estimator constructor arguments, estimator.cuh:118-152).
// ------------------------------------------------------------------------------------------
struct Params {
    int bie, domain, estimator, problem;
    unsigned path_length;
    unsigned num_resampling_candidates;
    unsigned num_volume_samples;
    float eps;
    float fk;  // first_kind_equation_scaling_constant
};

// ------------------------------------------------------------------------------------------
// BIE models (bie_models.cuh:53-590). One struct, the model selected at run time.
// ------------------------------------------------------------------------------------------
template <int D> struct BIE {
    EqKernel<D> K;
    int bie, domain;
    float fk;
    unsigned nvs;
    const Scene<D> *scene;
    Rng *rng;

    float dtc() const { return domain == InteriorDomain ? 1.0f : -1.0f; }                 // :66-71
    float ift(float a) const { return domain == InteriorDomain ? a : 1.0f - a; }          // :73-78

    VolumeSample<D> draw_volume() const { return scene->sample_volume(*rng); }

    // :79-103 (one volume sample, reused nvs times)
    float vol_term(const BoundaryPoint<D> &b) const {
        if (nvs == 0) return 0.0f;
        const VolumeSample<D> s = draw_volume();
        float r = 0.0f;
        for (unsigned i = 0; i < nvs; i++) {
            if (b.boundary_type == Dirichlet) r = r + K.G(b.p, s.p) * s.value * s.inv_pdf;
            else if (b.boundary_type == Neumann) r = r + K.dG_dny(b.p, s.p, b.n) * s.value * s.inv_pdf;
            else r = r + (K.dG_dny(b.p, s.p, b.n) + b.robin_alpha * K.G(s.p, b.p)) * s.value * s.inv_pdf;
        }
        return r / (float)nvs;
    }
    // :105-119
    float vol_init_boundary(const BoundaryPoint<D> &b) const {
        if (nvs == 0) return 0.0f;
        const VolumeSample<D> s = draw_volume();
        float r = 0.0f;
        for (unsigned i = 0; i < nvs; i++) r = r - K.G(b.p, s.p) * s.value * s.inv_pdf;
        return r / (float)nvs;
    }
    // :121-135
    float vol_init_domain(const Vec<D> &x) const {
        if (nvs == 0) return 0.0f;
        const VolumeSample<D> s = draw_volume();
        float r = 0.0f;
        for (unsigned i = 0; i < nvs; i++) r = r - K.G(s.p, x) * s.value * s.inv_pdf;
        return r / (float)nvs;
    }
    // :137-154
    Vec<D> vol_init_derivative(const Vec<D> &x) const {
        if (nvs == 0) return vzero<D>();
        const VolumeSample<D> s = draw_volume();
        Vec<D> r = vzero<D>();
        for (unsigned i = 0; i < nvs; i++) {
            const Vec<D> g = K.dG_dx(s.p, x);
            for (int j = 0; j < D; j++) r.v[j] = r.v[j] - g.v[j] * s.value * s.inv_pdf;
        }
        return r / (float)nvs;
    }

    // solution_domain_unknown: SL :228-231, DL :341-344, Direct :427-436
    float sdu(const Vec<D> &x, const BoundaryPoint<D> &y, float ip) const {
        if (bie == IndirectSingleLayer) return K.G(y.p, x) * ip;
        if (bie == IndirectDoubleLayer) return -K.dG_dny(y.p, x, y.n) * ip;
        if (y.boundary_type == Dirichlet) return dtc() * ip * K.G(y.p, x);
        if (y.boundary_type == Neumann) return -dtc() * ip * K.dG_dny(y.p, x, y.n);
        return -dtc() * ip * (K.dG_dny(y.p, x, y.n) + y.robin_alpha * K.G(y.p, x));
    }
    // solution_domain_known: SL :232-238, DL :345-351, Direct :437-450
    float sdk(const Vec<D> &x, const BoundaryPoint<D> &y, float ip) const {
        float r = vol_init_domain(x);
        if (bie != Direct) return r;
        if (y.boundary_type == Dirichlet)
            r = r + -dtc() * ip * K.dG_dny(y.p, x, y.n) * (y.boundary_value + vol_term(y));
        else
            r = r + dtc() * ip * K.G(y.p, x) * (y.boundary_value + vol_term(y));
        return r;
    }
    // gradient_domain_unknown: SL :240-243, DL :353-356, Direct :452-462
    Vec<D> gdu(const Vec<D> &x, const BoundaryPoint<D> &y, float ip) const {
        if (bie == IndirectSingleLayer) { const Vec<D> g = K.dG_dx(y.p, x); Vec<D> r; for (int i = 0; i < D; i++) r.v[i] = g.v[i] * ip; return r; }
        if (bie == IndirectDoubleLayer) { const Vec<D> g = K.d2G_dxdny(y.p, x, y.n); Vec<D> r; for (int i = 0; i < D; i++) r.v[i] = -g.v[i] * ip; return r; }
        if (y.boundary_type == Dirichlet) {
            const float c = dtc() * ip;
            const Vec<D> g = K.dG_dx(y.p, x);
            Vec<D> r; for (int i = 0; i < D; i++) r.v[i] = c * g.v[i]; return r;
        }
        if (y.boundary_type == Neumann) {
            const float c = -dtc() * ip;
            const Vec<D> g = K.d2G_dxdny(y.p, x, y.n);
            Vec<D> r; for (int i = 0; i < D; i++) r.v[i] = c * g.v[i]; return r;
        }
        const float c = -dtc() * ip;
        const Vec<D> g1 = K.d2G_dxdny(y.p, x, y.n);
        const Vec<D> g2 = K.dG_dx(y.p, x);
        Vec<D> r; for (int i = 0; i < D; i++) r.v[i] = c * (g1.v[i] + y.robin_alpha * g2.v[i]); return r;
    }
    // gradient_domain_known: SL :244-250, DL :357-363, Direct :463-478
    Vec<D> gdk(const Vec<D> &x, const BoundaryPoint<D> &y, float ip) const {
        Vec<D> r = vol_init_derivative(x);
        if (bie != Direct) return r;
        if (y.boundary_type == Dirichlet) {
            const float c = -dtc() * ip;
            const Vec<D> g = K.d2G_dxdny(y.p, x, y.n);
            const float s = y.boundary_value + vol_term(y);
            for (int i = 0; i < D; i++) r.v[i] = r.v[i] + c * g.v[i] * s;
        } else {
            const float c = dtc() * ip;
            const Vec<D> g = K.dG_dx(y.p, x);
            const float s = y.boundary_value + vol_term(y);
            for (int i = 0; i < D; i++) r.v[i] = r.v[i] + c * g.v[i] * s;
        }
        return r;
    }
    // solution_boundary_unknown: SL :252-257, DL :365-369, Direct :480-493
    float sbu(const BoundaryPoint<D> &x, const BoundaryPoint<D> &y, float ip) const {
        if (bie == IndirectDoubleLayer) return 0.0f;
        if (x.boundary_type == Dirichlet) return 0.0f;
        if (bie == IndirectSingleLayer) return K.G(y.p, x.p) * ip;
        const float c = dtc() / ift(x.interior_angle) * ip;
        if (y.boundary_type == Dirichlet) return c * K.G(y.p, x.p);
        if (y.boundary_type == Neumann) return -dtc() / ift(x.interior_angle) * ip * K.dG_dny(y.p, x.p, y.n);
        return -dtc() / ift(x.interior_angle) * ip * (K.dG_dny(y.p, x.p, y.n) + y.robin_alpha * K.G(y.p, x.p));
    }
    // solution_boundary_known: SL :258-266, DL :370-377, Direct :494-511
    float sbk(const BoundaryPoint<D> &x, const BoundaryPoint<D> &y, float ip) const {
        if (bie == IndirectDoubleLayer) return x.boundary_value;
        if (x.boundary_type == Dirichlet) return x.boundary_value;
        if (bie == IndirectSingleLayer) return vol_init_boundary(x);
        float r = vol_init_boundary(x);
        if (y.boundary_type == Dirichlet)
            r = r + -dtc() / ift(x.interior_angle) * ip * K.dG_dny(y.p, x.p, y.n) * (y.boundary_value + vol_term(y));
        else
            r = r + dtc() / ift(x.interior_angle) * ip * K.G(y.p, x.p) * (y.boundary_value + vol_term(y));
        return r;
    }
    // fredholm_equation_boundary_unknown: SL :268-300, DL :379-388, Direct :513-556.
    // May replace y (backward) or x (forward) by the other point (first-kind roulette).
    float fbu(BoundaryPoint<D> &x, BoundaryPoint<D> &y, float ip, bool backward) const {
        if (bie == IndirectDoubleLayer)
            return dtc() / (1.0f - ift(x.interior_angle)) * ip * K.dG_dny(y.p, x.p, y.n);
        if (backward && x.boundary_type == Dirichlet) {
            if (rng->uniform() * (1.0f + fk) < 1.0f) { y = x; return (1.0f + fk) * 1.0f; }
            ip = ip * ((1.0f + fk) / fk);
        } else if (!backward && y.boundary_type == Dirichlet) {
            if (rng->uniform() * (1.0f + fk) < 1.0f) { x = y; return (1.0f + fk) * 1.0f; }
            ip = ip * ((1.0f + fk) / fk);
        }
        if (bie == IndirectSingleLayer) {
            if (x.boundary_type == Dirichlet) return -2.0f * fk * ip * K.G(y.p, x.p);
            if (x.boundary_type == Neumann) return -dtc() / ift(x.interior_angle) * ip * K.dG_dny(x.p, y.p, x.n);
            return -dtc() / ift(x.interior_angle) * ip * (K.dG_dny(x.p, y.p, x.n) + x.robin_alpha * K.G(y.p, x.p));
        }
        if (x.boundary_type == Dirichlet) {
            if (y.boundary_type == Dirichlet) return -fk / ift(x.interior_angle) * ip * K.G(y.p, x.p);
            if (y.boundary_type == Neumann) return fk / ift(x.interior_angle) * ip * K.dG_dny(y.p, x.p, y.n);
            return fk / ift(x.interior_angle) * ip * (K.dG_dny(y.p, x.p, y.n) + y.robin_alpha * K.G(y.p, x.p));
        }
        if (y.boundary_type == Dirichlet) return dtc() / ift(x.interior_angle) * ip * K.G(y.p, x.p);
        if (y.boundary_type == Neumann) return -dtc() / ift(x.interior_angle) * ip * K.dG_dny(y.p, x.p, y.n);
        return -dtc() / ift(x.interior_angle) * ip * (K.dG_dny(y.p, x.p, y.n) + y.robin_alpha * K.G(y.p, x.p));
    }
    // fredholm_equation_boundary_known: SL :301-316, DL :389-399, Direct :557-587
    float fbk(const BoundaryPoint<D> &x, const BoundaryPoint<D> &y, float ip) const {
        if (bie == IndirectDoubleLayer)
            return dtc() * 1.0f / (1.0f - ift(x.interior_angle)) * (x.boundary_value + vol_term(x));
        if (bie == IndirectSingleLayer) {
            if (x.boundary_type == Dirichlet) return 2.0f * fk * (x.boundary_value + vol_term(x));
            return dtc() / ift(x.interior_angle) * (x.boundary_value + vol_term(x));
        }
        if (x.boundary_type == Dirichlet) {
            const float sx = x.boundary_value + vol_term(x);
            if (y.boundary_type == Dirichlet) {
                const float k = dtc() / ift(x.interior_angle) * ip * K.dG_dny(y.p, x.p, y.n);
                return dtc() * fk * (sx + k * (y.boundary_value + vol_term(y)));
            }
            const float k = dtc() / ift(x.interior_angle) * ip * K.G(y.p, x.p);
            return dtc() * fk * (sx - k * (y.boundary_value + vol_term(y)));
        }
        if (y.boundary_type == Dirichlet)
            return -dtc() / ift(x.interior_angle) * ip * K.dG_dny(y.p, x.p, y.n) * (y.boundary_value + vol_term(y));
        return dtc() / ift(x.interior_angle) * ip * K.G(y.p, x.p) * (y.boundary_value + vol_term(y));
    }
};

// ------------------------------------------------------------------------------------------
// Estimators (estimator.cuh:113-504).
// ------------------------------------------------------------------------------------------
template <int D> struct Estimator {
    const Scene<D> *scene;
    Params prm;
    BIE<D> bie;
    Rng *rng;
    uint64_t bounces = 0;

    Estimator(const Scene<D> *s, const Params &p, Rng *r) : scene(s), prm(p), rng(r) {
        bie.K.eps = p.eps;
        bie.bie = p.bie;
        bie.domain = p.domain;
        bie.fk = p.fk;
        bie.nvs = p.num_volume_samples;
        bie.scene = s;
        bie.rng = r;
    }
    bool dl_dirichlet() const { return prm.bie == IndirectDoubleLayer && prm.problem == DirichletProblem; }
    bool direct_neumann() const { return prm.bie == Direct && prm.problem == NeumannProblem; }
    bool sl_neumann() const { return prm.bie == IndirectSingleLayer && prm.problem == NeumannProblem; }

    // The start samples of the backward estimator (estimator.cuh:158-168, 199-209).
    void backward_start(const Vec<D> &x, BoundaryPoint<D> &y, float &ip, BoundaryPoint<D> &y1, float &ip1) {
        if (dl_dirichlet()) {
            y = scene->sample_line_intersection(*rng, x, ip);
            y1 = y;
            ip1 = ip;
        } else if (direct_neumann()) {
            y = scene->sample_line_intersection(*rng, x, ip);
            y1 = scene->sample_boundary_value(*rng, ip1);
        } else {
            y = scene->sample_uniform(*rng, ip);
            y1 = scene->sample_uniform(*rng, ip1);
        }
    }

    // compute_sample_unknown_boundary (estimator.cuh:232-357): the bounce loop.
    float unknown_boundary(const BoundaryPoint<D> &x) {
        float contrib = 0.0f, w = 1.0f;
        BoundaryPoint<D> y_prev = x;
        BoundaryPoint<D> y = bp_zero<D>();
        float ip = 0.0f;
        const unsigned L = prm.path_length;
        for (unsigned m = 0; m < L; m++) {
            bounces++;
            if (m == L - 1) w = 0.5f * w;
            if (dl_dirichlet()) {
                y = scene->sample_line_intersection(*rng, y_prev.p, ip);
                contrib = contrib + w * bie.fbk(y_prev, y, ip);
                w = w * bie.fbu(y_prev, y, ip, true);
                y_prev = y;
            } else if (direct_neumann()) {
                y = scene->sample_boundary_value(*rng, ip);
                contrib = contrib + w * bie.fbk(y_prev, y, ip);
                y = scene->sample_line_intersection(*rng, y_prev.p, ip);
                w = w * bie.fbu(y_prev, y, ip, true);
                y_prev = y;
            } else if (prm.bie == IndirectSingleLayer) {
                contrib = contrib + w * bie.fbk(y_prev, y, ip);
                if (prm.num_resampling_candidates == 1) {
                    y = scene->sample_uniform(*rng, ip);
                } else {
                    const BoundaryPoint<D> yp = y_prev;
                    const EqKernel<D> &K = bie.K;
                    if (yp.boundary_type == Dirichlet)
                        y = scene->sample_ris(*rng, [&](const BoundaryPoint<D> &c) { return std::fabs(K.G(c.p, yp.p)); },
                                              prm.num_resampling_candidates, ip);
                    else if (yp.boundary_type == Neumann)
                        y = scene->sample_ris(*rng, [&](const BoundaryPoint<D> &c) { return std::fabs(K.dG_dny(yp.p, c.p, yp.n)); },
                                              prm.num_resampling_candidates, ip);
                    else
                        y = scene->sample_ris(*rng, [&](const BoundaryPoint<D> &c) {
                            return std::fabs(K.dG_dny(yp.p, c.p, yp.n) + yp.robin_alpha * K.G(c.p, yp.p));
                        }, prm.num_resampling_candidates, ip);
                }
                w = w * bie.fbu(y_prev, y, ip, true);
                y_prev = y;
            } else {
                y = scene->sample_uniform(*rng, ip);
                contrib = contrib + w * bie.fbk(y_prev, y, ip);
                y = scene->sample_uniform(*rng, ip);
                w = w * bie.fbu(y_prev, y, ip, true);
                y_prev = y;
            }
            if (w == 0.0f) break;
        }
        return contrib;
    }

    // compute_sample_path_contribution_domain: backward (estimator.cuh:154-191),
    // forward (:405-454). out[0] = u, out[1..D] = grad u.
    void domain(const Vec<D> &x, float out[D + 1]) {
        if (prm.estimator == BackwardEstimator) {
            BoundaryPoint<D> y, y1;
            float ip, ip1;
            backward_start(x, y, ip, y1, ip1);
            out[0] = bie.sdk(x, y1, ip1);
            const Vec<D> g = bie.gdk(x, y1, ip1);
            for (int i = 0; i < D; i++) out[1 + i] = g.v[i];
            const float mu = unknown_boundary(y);
            out[0] = out[0] + mu * bie.sdu(x, y, ip);
            const Vec<D> gu = bie.gdu(x, y, ip);
            for (int i = 0; i < D; i++) out[1 + i] = out[1 + i] + mu * gu.v[i];
            return;
        }
        BoundaryPoint<D> y, y2;
        float ip, ip2;
        y = scene->sample_uniform(*rng, ip);
        out[0] = bie.sdk(x, y, ip);
        const Vec<D> g = bie.gdk(x, y, ip);
        for (int i = 0; i < D; i++) out[1 + i] = g.v[i];
        if (sl_neumann()) y = scene->sample_boundary_value(*rng, ip);
        else y = scene->sample_uniform(*rng, ip);
        y2 = scene->sample_uniform(*rng, ip2);
        float w = ip * bie.fbk(y, y2, ip2);
        BoundaryPoint<D> y_prev;
        const unsigned L = prm.path_length;
        for (unsigned m = 0; m < L; m++) {
            bounces++;
            if (m == L - 1) w = w * 0.5f;
            out[0] = out[0] + w * bie.sdu(x, y, 1.0f);
            const Vec<D> gu = bie.gdu(x, y, 1.0f);
            for (int i = 0; i < D; i++) out[1 + i] = out[1 + i] + w * gu.v[i];
            y_prev = y;
            if (sl_neumann()) y = scene->sample_line_intersection(*rng, y_prev.p, ip);
            else y = scene->sample_uniform(*rng, ip);
            w = bie.fbu(y, y_prev, ip, false) * w;
        }
    }

    // Forward single-layer Neumann estimator with a control variate on the density (no counterpart in
    // the reference). sigma_t[i] is the control-variate density on stored element i (piecewise
    // constant). u(x) = <G_x, sigma_t> + <G_x, r>, r solving r = s_r + K r with the residual source
    // s_r = s + K sigma_t - sigma_t. The first term: n_pot uniform samples; the second: the
    // reference's forward transport (estimator.cuh:433-451) started from a uniform point y0 with
    // weight A (s(y0) + K^ sigma_t(y0) - sigma_t(y0)), K^ from m_ker uniform samples.
    BoundaryPoint<D> uniform_idx(float &ip, unsigned &idx) {
        const float u1 = rng->uniform();
        idx = binary_search(scene->area_cdf.data(), (unsigned)scene->elems.size(), u1);
        const Element<D> &e = scene->elems[idx];
        BoundaryPoint<D> r;
        if constexpr (D == 2) {
            const float u2 = rng->uniform();
            r.p = interp2(e.v[0], e.v[1], u2); r.n = e.n; r.interior_angle = 0.5f;
            r.boundary_value = interp2(e.bv[0], e.bv[1], u2); r.boundary_type = e.type;
            r.robin_alpha = interp2(e.alpha[0], e.alpha[1], u2);
        } else {
            const float u2 = rng->uniform();
            const float u3 = rng->uniform();
            r.p = interp3(e.v[0], e.v[1], e.v[2], u2, u3); r.n = e.n; r.interior_angle = 0.5f;
            r.boundary_value = interp3(e.bv[0], e.bv[1], e.bv[2], u2, u3); r.boundary_type = e.type;
            r.robin_alpha = interp3(e.alpha[0], e.alpha[1], e.alpha[2], u2, u3);
        }
        ip = scene->total_area;
        return r;
    }
    void domain_cv(const Vec<D> &x, const float *sigma_t, unsigned n_pot, unsigned m_ker, float out[D + 1]) {
        float p1 = 0.0f;
        Vec<D> g1 = vzero<D>();
        for (unsigned k = 0; k < n_pot; k++) {
            float ip; unsigned id;
            const BoundaryPoint<D> y = uniform_idx(ip, id);
            const float c = sigma_t[id] * ip;
            p1 = p1 + bie.K.G(y.p, x) * c;
            const Vec<D> g = bie.K.dG_dx(y.p, x);
            for (int i = 0; i < D; i++) g1.v[i] = g1.v[i] + g.v[i] * c;
        }
        if (n_pot > 0) {
            p1 = p1 / (float)n_pot;
            for (int i = 0; i < D; i++) g1.v[i] = g1.v[i] / (float)n_pot;
        }
        float ip0; unsigned id0;
        BoundaryPoint<D> y = uniform_idx(ip0, id0);
        const float s0 = bie.fbk(y, y, ip0);
        float ks = 0.0f;
        for (unsigned j = 0; j < m_ker; j++) {
            float ipz; unsigned idz;
            BoundaryPoint<D> z = uniform_idx(ipz, idz);
            BoundaryPoint<D> yc = y;
            ks = ks + bie.fbu(yc, z, ipz, true) * sigma_t[idz];
        }
        if (m_ker > 0) ks = ks / (float)m_ker;
        float w = ip0 * (s0 + ks - sigma_t[id0]);
        float res = 0.0f;
        Vec<D> gres = vzero<D>();
        BoundaryPoint<D> y_prev;
        float ip = 0.0f;
        const unsigned L = prm.path_length;
        for (unsigned m = 0; m < L; m++) {
            bounces++;
            if (m == L - 1) w = w * 0.5f;
            res = res + w * bie.sdu(x, y, 1.0f);
            const Vec<D> gu = bie.gdu(x, y, 1.0f);
            for (int i = 0; i < D; i++) gres.v[i] = gres.v[i] + w * gu.v[i];
            y_prev = y;
            y = scene->sample_line_intersection(*rng, y_prev.p, ip);
            w = bie.fbu(y, y_prev, ip, false) * w;
        }
        out[0] = p1 + res;
        for (int i = 0; i < D; i++) out[1 + i] = g1.v[i] + gres.v[i];
    }

    // Backward estimator with a control variate cv on the unknown boundary function (no
    // counterpart in the reference; uniform start samples: single layer, or direct without
    // NeumannProblem). cv[i] is constant on stored element i. u(x) = sdk(x, y1) +
    // (mu(y0) - cv(y0)) sdu(x, y0) + sum_{i<n} (sdu(x, z_i) / n) cv(z_i): the walk is the plain
    // estimator's (estimator.cuh:154-191, 232-357), the n uniform samples z_i are drawn after it.
    float domain_bcv(const Vec<D> &x, const float *cv, unsigned n_pot) {
        float ip, ip1;
        unsigned id, id1;
        const BoundaryPoint<D> y = uniform_idx(ip, id);
        const BoundaryPoint<D> y1 = uniform_idx(ip1, id1);
        float out = bie.sdk(x, y1, ip1);
        const float mu = unknown_boundary(y);
        out = out + (mu - cv[id]) * bie.sdu(x, y, ip);
        for (unsigned k = 0; k < n_pot; k++) {
            float ipz;
            unsigned idz;
            const BoundaryPoint<D> z = uniform_idx(ipz, idz);
            out = out + (bie.sdu(x, z, ipz) / (float)n_pot) * cv[idz];
        }
        return out;
    }

    // compute_sample_path_contribution_boundary: backward (estimator.cuh:193-222),
    // forward (:456-496).
    float boundary(const BoundaryPoint<D> &x) {
        if (prm.estimator == BackwardEstimator) {
            BoundaryPoint<D> y, y1;
            float ip, ip1;
            if (dl_dirichlet()) {
                y = scene->sample_line_intersection(*rng, x.p, ip);
                y1 = y;
                ip1 = ip;
            } else if (direct_neumann()) {
                y = scene->sample_line_intersection(*rng, x.p, ip);
                y1 = scene->sample_boundary_value(*rng, ip1);
            } else {
                y = scene->sample_uniform(*rng, ip);
                y1 = scene->sample_uniform(*rng, ip1);
            }
            float r = bie.sbk(x, y1, ip1);
            const float mu = unknown_boundary(y);
            r = r + mu * bie.sbu(x, y, ip);
            return r;
        }
        BoundaryPoint<D> y, y2;
        float ip, ip2;
        y = scene->sample_uniform(*rng, ip);
        float r = bie.sbk(x, y, ip);
        if (sl_neumann()) y = scene->sample_boundary_value(*rng, ip);
        else y = scene->sample_uniform(*rng, ip);
        y2 = scene->sample_uniform(*rng, ip2);
        float w = ip * bie.fbk(y, y2, ip2);
        BoundaryPoint<D> y_prev;
        const unsigned L = prm.path_length;
        for (unsigned m = 0; m < L; m++) {
            bounces++;
            if (m == L - 1) w = w * 0.5f;
            r = r + bie.sbu(x, y, 1.0f) * w;
            y_prev = y;
            if (sl_neumann()) y = scene->sample_line_intersection(*rng, y_prev.p, ip);
            else y = scene->sample_uniform(*rng, ip);
            w = bie.fbu(y, y_prev, ip, false) * w;
        }
        return r;
    }
};

// Random stream tags: the domain and boundary estimators use separate Philox keys.
constexpr uint32_t kStreamDomain = 0u;
constexpr uint32_t kStreamBoundary = 1u;
constexpr uint32_t kStreamVpl = 2u;
constexpr uint32_t kStreamWos = 3u;

// The closed-form double-layer interior Dirichlet walk of apps/simple_wob_and_wos.cu:81-108: a
// second, independent oracle for the double-layer estimator. Uses the same line samples; weight
// m sign((y-x).n), then -m sign((y_j - y_{j-1}).n_j) per bounce, the last one halved.
inline float simple_wob_path(const Scene<2> &s, Rng &rng, const Vec<2> &x, unsigned path_length) {
    auto sign = [](float v) { return v > 0.0f ? 1.0f : -1.0f; };
    unsigned m;
    BoundaryPoint<2> y = s.sample_line_intersection2(rng, x, m);
    float weight = (float)m * sign(dot(y.p - x, y.n));
    float contrib = weight * y.boundary_value;
    for (unsigned j = 1; j < path_length; j++) {
        if (j == path_length - 1) weight = weight * 0.5f;
        const Vec<2> yp = y.p;
        y = s.sample_line_intersection2(rng, y.p, m);
        weight = weight * (-(float)m * sign(dot(y.p - yp, y.n)));
        contrib = contrib + weight * y.boundary_value;
    }
    return contrib;
}

// Closest boundary point of a 2D scene (apps/simple_wob_and_wos.cu:49-78 with lbvh's nearest
// query restated as a scan): squared distance to each segment with the clamped parameter
// t = (p - a).l / |l|^2, the smallest distance winning, ties to the smallest storage index.
struct ClosestPoint {
    float d2 = INFINITY;
    unsigned elem = 0xFFFFFFFFu;
    float t = 0.0f;
};
inline ClosestPoint closest_point(const Scene<2> &s, const Vec<2> &p) {
    ClosestPoint best;
    for (unsigned i = 0; i < (unsigned)s.elems.size(); i++) {
        const Element<2> &e = s.elems[i];
        const float ax = e.v[0].v[0], ay = e.v[0].v[1];
        const float lx = e.v[1].v[0] - ax, ly = e.v[1].v[1] - ay;
        float t = ((p.v[0] - ax) * lx + (p.v[1] - ay) * ly) / (lx * lx + ly * ly);
        t = std::min(std::max(t, 0.0f), 1.0f);
        const float cx = (ax + lx * t) - p.v[0], cy = (ay + ly * t) - p.v[1];
        const float d2 = cx * cx + cy * cy;
        if (d2 < best.d2 || (d2 == best.d2 && i < best.elem)) best = ClosestPoint{d2, i, t};
    }
    return best;
}
inline float closest_value(const Scene<2> &s, const ClosestPoint &c) {
    const Element<2> &e = s.elems[c.elem];
    return (e.bv[1] - e.bv[0]) * c.t + e.bv[0];
}

// One walk-on-spheres path (apps/simple_wob_and_wos.cu:111-137): jump to a uniform point on the
// largest empty circle, angle 2 pi u through sincospi_own(2u), until the distance is below eps;
// stopped after max_steps jumps.
inline float wos_path(const Scene<2> &s, float eps, Rng &rng, Vec<2> x, unsigned &queries,
                      unsigned max_steps = 4096) {
    for (unsigned step = 0;; step++) {
        const ClosestPoint c = closest_point(s, x);
        queries++;
        const float R = std::sqrt(c.d2);
        if (R < eps || c.elem == 0xFFFFFFFFu) return c.elem == 0xFFFFFFFFu ? 0.0f : closest_value(s, c);
        if (step + 1 >= max_steps) return closest_value(s, c);
        float sn, cs;
        sincospi_own(2.0f * rng.uniform(), &sn, &cs);
        x.v[0] = x.v[0] + R * cs;
        x.v[1] = x.v[1] + R * sn;
    }
}

}  // namespace wob_oracle
