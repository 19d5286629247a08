// Device building blocks of the GB300 WoB engine: Philox4x32-10 streams, polynomial sin/cos(pi x)
// and log, small vectors, the scene view, CDF lookup through guide tables, the 4-wide BVH
// traversal for "all hits of an infinite line", and the boundary sampling queries.
//
// Every translation unit that includes this header is compiled with -fmad=false: the walk uses
// IEEE single-precision +,-,*,/ and sqrt only (fused multiply-adds only where written as fmaf),
// so a path evaluates to the same bits as a plain IEEE evaluation of the same formulas on a CPU.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace wobgb {

constexpr float kEps10 = 10.0f * 1.1920928955078125e-7f;  // 10 FLT_EPSILON (scene.cuh:418, 531)
constexpr uint32_t kHitBuffer = 64;                         // hit buffer of scene.cuh:481
constexpr uint32_t kStackSize = 64;
constexpr int kWalkBlock = 128;   // threads per block of the walk kernels (and of the shared stack columns)
constexpr int kSharedStack = 24;  // entries of a thread's 3D traversal stack held in shared memory
constexpr int kLeafBatch = 8;     // leaves a 3D line query holds before testing them
constexpr uint32_t kChildEmptyD = 0xFFFFFFFFu;

// Device error word bits (see ErrorWord in capi.cu).
constexpr uint32_t kErrStackOverflow = 1u;
constexpr uint32_t kErrTraversalLimit = 2u;
constexpr uint32_t kErrWosStepLimit = 4u;  // a walk-on-spheres path reached kWosMaxSteps jumps
constexpr uint32_t kWosMaxSteps = 4096;

enum : int { kDirichlet = 0, kNeumann = 1, kRobin = 2 };
enum : int { kSingleLayer = 0, kDoubleLayer = 1, kDirect = 2 };
enum : int { kInterior = 0, kExterior = 1 };
enum : int { kBackward = 0, kForward = 1 };
enum : int { kDirichletProblem = 0, kNeumannProblem = 1, kRobinProblem = 2, kMixedProblem = 3 };

// ------------------------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11). Counter (block, path lo, path hi, point),
// key (seed lo, seed hi + stream); uniforms ((x >> 8) + 1) 2^-24 in (0, 1].
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

struct PathRng {
    uint32_t k0, k1, c1, c2, c3, block;
    uint4 buf;
    int used;
    __device__ __forceinline__ PathRng(uint64_t seed, uint32_t stream, uint32_t point, uint64_t path)
        : k0((uint32_t)seed), k1((uint32_t)(seed >> 32) + stream), c1((uint32_t)path),
          c2((uint32_t)(path >> 32)), c3(point), block(0), buf(make_uint4(0, 0, 0, 0)), used(4) {}
    // Uniforms drawn so far, and the inverse: the stream positioned after d draws (a path whose
    // state is kept in memory between kernels resumes exactly).
    __device__ __forceinline__ uint32_t drawn() const { return used == 4 ? block * 4u : (block - 1u) * 4u + (uint32_t)used; }
    __device__ __forceinline__ void seek(uint32_t d) {
        const uint32_t b = d >> 2, r = d & 3u;
        if (r == 0) {
            block = b;
            used = 4;
        } else {
            buf = philox4x32_10(make_uint4(b, c1, c2, c3), k0, k1);
            block = b + 1u;
            used = (int)r;
        }
    }
    __device__ __forceinline__ float uniform() {
        if (used == 4) {
            buf = philox4x32_10(make_uint4(block, c1, c2, c3), k0, k1);
            block++;
            used = 0;
        }
        const uint32_t x = used == 0 ? buf.x : used == 1 ? buf.y : used == 2 ? buf.z : buf.w;
        used++;
        return (float)((x >> 8) + 1u) * 0x1p-24f;
    }
};

// ------------------------------------------------------------------------------------------
// Scalar math (same polynomials as the CPU oracle; no CUDA transcendental on the walk).
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float fmax_ref(float a, float b) { return (a < b) ? b : a; }

// sin(pi x), cos(pi x): x = q/2 + r, |r| <= 1/4, Taylor polynomials in r^2, quadrant rotation.
__device__ __forceinline__ void sincospi_own(float x, float *s_out, float *c_out) {
    const float q = rintf(x * 2.0f);
    const float r = x - q * 0.5f;
    const float z = r * r;
    float sp = -0x1.e3075p-8f;
    sp = sp * z + 0x1.507834p-4f;
    sp = sp * z - 0x1.32d2ccp-1f;
    sp = sp * z + 0x1.466bc6p+1f;
    sp = sp * z - 0x1.4abbcep+2f;
    sp = sp * z + 0x1.921fb6p+1f;
    const float s = sp * r;
    float cp = 0x1.f9d38ap-10f;
    cp = cp * z - 0x1.a6d1f2p-6f;
    cp = cp * z + 0x1.e1f506p-3f;
    cp = cp * z - 0x1.55d3c8p+0f;
    cp = cp * z + 0x1.03c1f0p+2f;
    cp = cp * z - 0x1.3bd3ccp+2f;
    const float c = cp * z + 1.0f;
    const int qi = ((int)q) & 3;
    float so, co;
    if (qi == 0) { so = s; co = c; }
    else if (qi == 1) { so = c; co = -s; }
    else if (qi == 2) { so = -s; co = -c; }
    else { so = -c; co = s; }
    *s_out = so;
    *c_out = co;
}

// log x = e ln2 + 2 atanh((m-1)/(m+1)), m in (sqrt(1/2), sqrt(2)].
__device__ __forceinline__ float log_own(float x) {
    if (!(x > 0.0f)) return (x == 0.0f) ? __int_as_float(0xff800000) : __int_as_float(0x7fffffff);
    if (x == __int_as_float(0x7f800000)) return x;
    int e_adj = 0;
    if (x < 0x1p-126f) { x = x * 0x1p+23f; e_adj = -23; }
    const uint32_t bits = __float_as_uint(x);
    int e = (int)(bits >> 23) - 127 + e_adj;
    float m = __uint_as_float((bits & 0x007fffffu) | 0x3f800000u);
    if (m > 0x1.6a09e6p+0f) { m = m * 0.5f; e += 1; }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float z = s * s;
    float p = 0x1.745d18p-4f;
    p = p * z + 0x1.c71c72p-4f;
    p = p * z + 0x1.24924ap-3f;
    p = p * z + 0x1.99999ap-3f;
    p = p * z + 0x1.555556p-2f;
    p = p * z + 1.0f;
    const float logm = (2.0f * s) * p;
    const float fe = (float)e;
    return fe * 0x1.62e4p-1f + (fe * 0x1.7f7d1cp-20f + logm);
}

// ------------------------------------------------------------------------------------------
// Vectors: fixed-size, fully unrolled; sums left to right.
// ------------------------------------------------------------------------------------------
template <int D> struct V {
    float v[D];
};
template <int D> __device__ __forceinline__ V<D> vzero() { V<D> r; _Pragma("unroll") for (int i = 0; i < D; i++) r.v[i] = 0.0f; return r; }
template <int D> __device__ __forceinline__ V<D> vadd(const V<D> &a, const V<D> &b) { V<D> r; _Pragma("unroll") for (int i = 0; i < D; i++) r.v[i] = a.v[i] + b.v[i]; return r; }
template <int D> __device__ __forceinline__ V<D> vsub(const V<D> &a, const V<D> &b) { V<D> r; _Pragma("unroll") for (int i = 0; i < D; i++) r.v[i] = a.v[i] - b.v[i]; return r; }
template <int D> __device__ __forceinline__ V<D> vscale(float s, const V<D> &a) { V<D> r; _Pragma("unroll") for (int i = 0; i < D; i++) r.v[i] = s * a.v[i]; return r; }
template <int D> __device__ __forceinline__ V<D> vdiv(const V<D> &a, float s) { V<D> r; _Pragma("unroll") for (int i = 0; i < D; i++) r.v[i] = a.v[i] / s; return r; }
template <int D> __device__ __forceinline__ float vdot(const V<D> &a, const V<D> &b) {
    float s = a.v[0] * b.v[0];
    _Pragma("unroll") for (int i = 1; i < D; i++) s = s + a.v[i] * b.v[i];
    return s;
}
template <int D> __device__ __forceinline__ float vsqnorm(const V<D> &a) { return vdot(a, a); }
template <int D> __device__ __forceinline__ float vnorm(const V<D> &a) { return sqrtf(vsqnorm(a)); }
template <int D> __device__ __forceinline__ V<D> vnormalized(const V<D> &a) {
    const float z = vsqnorm(a);
    if (z > 0.0f) return vdiv(a, sqrtf(z));
    return a;
}
__device__ __forceinline__ V<3> vcross(const V<3> &a, const V<3> &b) {
    V<3> r;
    r.v[0] = a.v[1] * b.v[2] - a.v[2] * b.v[1];
    r.v[1] = a.v[2] * b.v[0] - a.v[0] * b.v[2];
    r.v[2] = a.v[0] * b.v[1] - a.v[1] * b.v[0];
    return r;
}

// ------------------------------------------------------------------------------------------
// Boundary point (points.hpp:32-39).
// ------------------------------------------------------------------------------------------
template <int D> struct BPoint {
    V<D> p, n;
    float angle;  // interior_angle
    float bv;     // boundary_value
    int type;     // boundary_type
    float alpha;  // robin_alpha
};
template <int D> __device__ __forceinline__ BPoint<D> bp_zero() {
    BPoint<D> b;
    b.p = vzero<D>(); b.n = vzero<D>();
    b.angle = 0.0f; b.bv = 0.0f; b.type = kDirichlet; b.alpha = 0.0f;
    return b;
}

// ------------------------------------------------------------------------------------------
// Scene view (device pointers; filled by the host, passed by value to kernels).
// ------------------------------------------------------------------------------------------
template <int D> struct SceneView {
    const float4 *__restrict__ elems;     // 4 float4 / element (2D: the last one padding)
    const float4 *__restrict__ elem_aux;  // D==3: 1 float4 / element (alpha[3], area)
    const float4 *__restrict__ isect;  // D==3: 4 float4 / element (a, a-b, a-c, (a-b)x(a-c), padding)
    const float4 *__restrict__ nodes;  // D==2: 6 float4 / node, D==3: 8 (the last one padding)
    const float *__restrict__ area_cdf;
    const uint4 *__restrict__ area_guide;
    const float *__restrict__ bv_cdf;
    const uint4 *__restrict__ bv_guide;
    const float *__restrict__ vol_values;
    const float *__restrict__ vol_cdf;
    const uint4 *__restrict__ vol_guide;
    const float *__restrict__ cv_table;  // control-variate density per stored element (or null)
    const float4 *__restrict__ lg_bins;  // 2D line grid (LineGrid, scene_host.hpp): K x {cmin, cmax, inv_w, 0}
    const uint32_t *__restrict__ lg_off; // K x (M + 1) list starts
    const uint16_t *__restrict__ lg_ent; // stored element indices
    uint32_t lg_K, lg_M;                 // lg_K == 0: no line grid
    float lg_cx, lg_cy, lg_far;          // offset centre; origins farther (L1) take the BVH
    uint32_t *err;                       // device error word (kErr* bits)
    uint32_t n_elems, n_nodes, area_G, bv_G;
    uint32_t alpha_const;  // D==3: every vertex alpha is alpha_value (elem_aux not read for alphas)
    float alpha_value;
    uint32_t vol_n, vol_G, vol_res, traversal_limit;
    uint32_t wos_step_limit;  // jumps of a walk-on-spheres path (kWosMaxSteps unless overridden)
    float total_area, total_bv, vol_size;
};

template <int D> struct Elem {
    V<D> v[D];
    V<D> n;
    float bv[D], alpha[D];
    float area;
    int type;
};

// 32-byte read-only load (ld.global.nc.v8.f32, sm_100 and later); p must be 32-byte aligned. A
// random gather costs about the same per load instruction for 16 and 32 bytes, so the records are
// laid out for as few 32-byte loads as possible.
struct F8 {
    float4 a, b;
};
__device__ __forceinline__ F8 ldg8(const float4 *p) {
    F8 r;
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(r.a.x), "=f"(r.a.y), "=f"(r.a.z), "=f"(r.a.w), "=f"(r.b.x), "=f"(r.b.y), "=f"(r.b.z), "=f"(r.b.w)
        : "l"(p));
    return r;
}

template <int D> __device__ __forceinline__ Elem<D> load_elem(const SceneView<D> &s, uint32_t i);
template <> __device__ __forceinline__ Elem<2> load_elem<2>(const SceneView<2> &s, uint32_t i) {
    const float4 *p = s.elems + 4 * i;
    const F8 r = ldg8(p);
    const float4 q0 = r.a, q1 = r.b, q2 = __ldg(p + 2);
    Elem<2> e;
    e.v[0].v[0] = q0.x; e.v[0].v[1] = q0.y; e.v[1].v[0] = q0.z; e.v[1].v[1] = q0.w;
    e.n.v[0] = q1.x; e.n.v[1] = q1.y; e.bv[0] = q1.z; e.bv[1] = q1.w;
    e.alpha[0] = q2.x; e.alpha[1] = q2.y; e.area = q2.z; e.type = __float_as_int(q2.w);
    return e;
}
// The 3D record's alphas come from the scene constant when all are equal; the area (used only by
// |g| sampling, which reads it itself) is left NaN.
template <> __device__ __forceinline__ Elem<3> load_elem<3>(const SceneView<3> &s, uint32_t i) {
    const float4 *p = s.elems + 4 * i;
    const F8 r0 = ldg8(p), r1 = ldg8(p + 2);
    const float4 q0 = r0.a, q1 = r0.b, q2 = r1.a, q3 = r1.b;
    float4 q4;
    if (s.alpha_const) q4 = make_float4(s.alpha_value, s.alpha_value, s.alpha_value, __int_as_float(0x7fc00000));
    else q4 = __ldg(s.elem_aux + i);
    Elem<3> e;
    e.v[0].v[0] = q0.x; e.v[0].v[1] = q0.y; e.v[0].v[2] = q0.z;
    e.v[1].v[0] = q0.w; e.v[1].v[1] = q1.x; e.v[1].v[2] = q1.y;
    e.v[2].v[0] = q1.z; e.v[2].v[1] = q1.w; e.v[2].v[2] = q2.x;
    e.n.v[0] = q2.y; e.n.v[1] = q2.z; e.n.v[2] = q2.w;
    e.bv[0] = q3.x; e.bv[1] = q3.y; e.bv[2] = q3.z; e.type = __float_as_int(q3.w);
    e.alpha[0] = q4.x; e.alpha[1] = q4.y; e.alpha[2] = q4.z; e.area = __int_as_float(0x7fc00000);
    return e;
}

// First i in [0, n-1] with key <= cdf[i], else n-1: the reference's binary_search
// (scene.cuh:30-43), started from a guide table. Entry j of the table holds lo = the first index
// whose CDF value reaches (j - 1/2)/G, hi = the lo of entry j + 2 (n - 1 for the last two) and
// the CDF values at lo and lo + 1. For j = floor(key G) every index below lo has a CDF value
// under (j - 1/2)/G < key and cdf[hi] >= (j + 3/2)/G > key, so the answer lies in [lo, hi]; the
// two stored values settle it with one 16-byte load in almost every case, the bisection below
// covers the rest of the sub-range.
__device__ __forceinline__ uint32_t guide_bin(uint32_t G, float key) {
    uint32_t j = (uint32_t)(key * (float)G);
    return j >= G ? G - 1 : j;
}
__device__ __forceinline__ uint32_t cdf_resolve(const float *__restrict__ cdf, const uint4 g, float key) {
    const uint32_t lo = g.x, hi = g.y;
    if (lo >= hi) return hi;
    if (key <= __uint_as_float(g.z)) return lo;
    if (lo + 1 == hi) return hi;
    if (key <= __uint_as_float(g.w)) return lo + 1;
    uint32_t low = lo + 2, high = hi;
    while (low < high) {
        const uint32_t mid = (high + low) / 2;
        if (key <= __ldg(cdf + mid)) high = mid;
        else low = mid + 1;
    }
    return high;
}
__device__ __forceinline__ uint32_t cdf_search(const float *__restrict__ cdf, const uint4 *__restrict__ guide,
                                               uint32_t G, float key) {
    return cdf_resolve(cdf, __ldg(guide + guide_bin(G, key)), key);
}

// val1 + u (val2 - val1) (scene.cuh:393-396)
__device__ __forceinline__ float interp2(float a, float b, float u) { return a + u * (b - a); }
// (1 - sqrt u1) v1 + sqrt u1 (1 - u2) v2 + u2 sqrt u1 v3 (scene.cuh:665-671)
__device__ __forceinline__ float interp3(float a, float b, float c, float k1, float k2, float k3) {
    return k1 * a + k2 * b + k3 * c;
}

// ------------------------------------------------------------------------------------------
// Line / element intersection: Cramer's rule, division-free inside test, t = tn/det, |t| > 10 eps
// (restates scene.cuh:414-436 and 707-730).
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ bool isect_seg(const V<2> &o, const V<2> &d, float ax, float ay, float bx, float by, float &t) {
    const float edx = ax - bx, edy = ay - by;
    const float wx = ax - o.v[0], wy = ay - o.v[1];
    const float det = d.v[0] * edy - d.v[1] * edx;
    const float sn = d.v[0] * wy - d.v[1] * wx;
    bool inside;
    if (det > 0.0f) inside = (sn >= 0.0f) && (sn <= det);
    else if (det < 0.0f) inside = (sn <= 0.0f) && (sn >= det);
    else inside = false;
    if (!inside) return false;
    const float tn = wx * edy - wy * edx;
    t = tn / det;
    return fabsf(t) > kEps10;
}

__device__ __forceinline__ bool isect_tri(const V<3> &o, const V<3> &d, const float4 r0, const float4 r1, const float4 r2, float &t) {
    // r0 = (a.x, a.y, a.z, e1.x), r1 = (e1.y, e1.z, e2.x, e2.y), r2 = (e2.z, q.x, q.y, q.z)
    const float wx = r0.x - o.v[0], wy = r0.y - o.v[1], wz = r0.z - o.v[2];
    float det = d.v[0] * r2.y;
    det = det + d.v[1] * r2.z;
    det = det + d.v[2] * r2.w;
    // w x d
    const float cx = wy * d.v[2] - wz * d.v[1];
    const float cy = wz * d.v[0] - wx * d.v[2];
    const float cz = wx * d.v[1] - wy * d.v[0];
    float bn = r1.z * cx;
    bn = bn + r1.w * cy;
    bn = bn + r2.x * cz;
    bn = -bn;
    float gn = r0.w * cx;
    gn = gn + r1.x * cy;
    gn = gn + r1.y * cz;
    bool inside;
    if (det > 0.0f) inside = (bn >= 0.0f) && (gn >= 0.0f) && (bn + gn <= det);
    else if (det < 0.0f) inside = (bn <= 0.0f) && (gn <= 0.0f) && (bn + gn >= det);
    else inside = false;
    if (!inside) return false;
    float tn = wx * r2.y;
    tn = tn + wy * r2.z;
    tn = tn + wz * r2.w;
    t = tn / det;
    return fabsf(t) > kEps10;
}

template <int D> __device__ __forceinline__ bool isect_elem(const SceneView<D> &s, uint32_t i, const V<D> &o, const V<D> &d, float &t);
template <> __device__ __forceinline__ bool isect_elem<2>(const SceneView<2> &s, uint32_t i, const V<2> &o, const V<2> &d, float &t) {
    const float4 q0 = __ldg(s.elems + 4 * i);
    return isect_seg(o, d, q0.x, q0.y, q0.z, q0.w, t);
}
template <> __device__ __forceinline__ bool isect_elem<3>(const SceneView<3> &s, uint32_t i, const V<3> &o, const V<3> &d, float &t) {
    const float4 *p = s.isect + 4 * i;
    const F8 r = ldg8(p);
    return isect_tri(o, d, r.a, r.b, __ldg(p + 2), t);
}

// Conservative line / box tests against the 4 children of a node; bit k of the result is set
// when child k's (padded) box meets the infinite line.
__device__ __forceinline__ uint32_t node_hits(const SceneView<2> &s, uint32_t node, const V<2> &o, const V<2> &d, float c0, uint4 &child) {
    const float4 *p = s.nodes + 6 * node;
    const F8 r0 = ldg8(p), r1 = ldg8(p + 2);
    const float4 lx = r0.a, ly = r0.b, hx = r1.a, hy = r1.b;
    const float4 cf = __ldg(p + 4);
    child = make_uint4(__float_as_uint(cf.x), __float_as_uint(cf.y), __float_as_uint(cf.z), __float_as_uint(cf.w));
    const float dx = d.v[0], dy = d.v[1];
    // f(p) = dx p.y - dy p.x - c0 takes both signs over the box
    const float lxs[4] = {lx.x, lx.y, lx.z, lx.w}, lys[4] = {ly.x, ly.y, ly.z, ly.w};
    const float hxs[4] = {hx.x, hx.y, hx.z, hx.w}, hys[4] = {hy.x, hy.y, hy.z, hy.w};
    uint32_t mask = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float a1 = dx * lys[k], a2 = dx * hys[k];
        const float b1 = dy * lxs[k], b2 = dy * hxs[k];
        const float fmin_ = fminf(a1, a2) - fmaxf(b1, b2) - c0;
        const float fmax_ = fmaxf(a1, a2) - fminf(b1, b2) - c0;
        if (fmin_ <= 0.0f && fmax_ >= 0.0f) mask |= 1u << k;
    }
    return mask;
}

// The infinite line o + t d in the form the 3D box test uses: per axis the reciprocal direction r
// (|d| clamped to at least 1e-20, so r is finite) and -o r. A slab bound is then one FMA,
// t = fma(b, r, -o r), and no product is infinite or NaN for finite coordinates below 1e18.
struct LineSlab3 {
    float r[3], nor[3];
};
__device__ __forceinline__ LineSlab3 line_slab3(const V<3> &o, const V<3> &d) {
    LineSlab3 L;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const float di = fabsf(d.v[i]) > 1e-20f ? d.v[i] : copysignf(1e-20f, d.v[i]);
        L.r[i] = 1.0f / di;
        L.nor[i] = -(o.v[i] * L.r[i]);
    }
    return L;
}

__device__ __forceinline__ float fmax3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float fmin3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Slab test of the line against the 4 children's boxes. The slab bounds carry an absolute error
// of about one float ulp of |o| along the line (the rounding of o r and of the FMA), while the
// boxes are padded by 1e-5 (extent + max |coordinate|): a line that meets an element of a child
// crosses that child's padded box over a length of at least twice the pad, so the test never
// rejects it, and the hits (decided by the exact element test alone) do not depend on it.
__device__ __forceinline__ uint32_t node_hits(const SceneView<3> &s, uint32_t node, const LineSlab3 &L, uint4 &child) {
    const float4 *p = s.nodes + 8 * node;
    const F8 r0 = ldg8(p), r1 = ldg8(p + 2), r2 = ldg8(p + 4);
    const float4 lx = r0.a, ly = r0.b, lz = r1.a;
    const float4 hx = r1.b, hy = r2.a, hz = r2.b;
    const float4 cf = __ldg(p + 6);
    child = make_uint4(__float_as_uint(cf.x), __float_as_uint(cf.y), __float_as_uint(cf.z), __float_as_uint(cf.w));
    const float lxs[4] = {lx.x, lx.y, lx.z, lx.w}, lys[4] = {ly.x, ly.y, ly.z, ly.w}, lzs[4] = {lz.x, lz.y, lz.z, lz.w};
    const float hxs[4] = {hx.x, hx.y, hx.z, hx.w}, hys[4] = {hy.x, hy.y, hy.z, hy.w}, hzs[4] = {hz.x, hz.y, hz.z, hz.w};
    uint32_t mask = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float tx1 = __fmaf_rn(lxs[k], L.r[0], L.nor[0]), tx2 = __fmaf_rn(hxs[k], L.r[0], L.nor[0]);
        const float ty1 = __fmaf_rn(lys[k], L.r[1], L.nor[1]), ty2 = __fmaf_rn(hys[k], L.r[1], L.nor[1]);
        const float tz1 = __fmaf_rn(lzs[k], L.r[2], L.nor[2]), tz2 = __fmaf_rn(hzs[k], L.r[2], L.nor[2]);
        const float tn = fmax3f(fminf(tx1, tx2), fminf(ty1, ty2), fminf(tz1, tz2));
        const float tf = fmin3f(fmaxf(tx1, tx2), fmaxf(ty1, ty2), fmaxf(tz1, tz2));
        if (tn <= tf) mask |= 1u << k;
    }
    return mask;
}

// 2D line query through the line grid: the line's direction bin (diamond angle of the direction
// taken in the upper half-plane) and offset cell give the candidate segments in storage order,
// each tested exactly. Returns false (nothing done) when d is not a unit vector within 1e-6 or
// the origin lies farther than lg_far from the grid's centre, the preconditions of the grid's
// offset bounds; the caller then traverses the BVH.
__device__ __forceinline__ bool line_grid_query(const SceneView<2> &s, const V<2> &o, const V<2> &d, uint32_t *hits,
                                                uint32_t &count) {
    const float q = d.v[0] * d.v[0] + d.v[1] * d.v[1];
    if (!(fabsf(q - 1.0f) <= 1e-6f)) return false;
    const float ox = o.v[0] - s.lg_cx, oy = o.v[1] - s.lg_cy;
    if (!(fabsf(ox) + fabsf(oy) <= s.lg_far)) return false;
    const bool flip = d.v[1] < 0.0f || (d.v[1] == 0.0f && d.v[0] < 0.0f);
    const float dx = flip ? -d.v[0] : d.v[0], dy = flip ? -d.v[1] : d.v[1];
    const float t = dy / (fabsf(dx) + dy);
    const float pa = dx >= 0.0f ? t : 2.0f - t;
    uint32_t k = (uint32_t)(pa * (0.5f * (float)s.lg_K));
    k = k < s.lg_K ? k : s.lg_K - 1;
    count = 0;
    const float c = -dy * ox + dx * oy;
    const float4 b = __ldg(s.lg_bins + k);
    if (!(c >= b.x && c <= b.y)) return true;
    const float f = (c - b.x) * b.z;
    uint32_t j = f >= (float)s.lg_M ? s.lg_M : (uint32_t)f;
    j = j < s.lg_M ? j : s.lg_M - 1;
    const uint32_t *off = s.lg_off + (size_t)k * (s.lg_M + 1) + j;
    const uint32_t e0 = __ldg(off), e1 = __ldg(off + 1);
    // four candidates per iteration: their index and segment loads in flight together, hits
    // appended in list order
    uint32_t e = e0;
    for (; e + 3 < e1; e += 4) {
        uint32_t id[4];
        float4 q[4];
#pragma unroll
        for (int u = 0; u < 4; u++) id[u] = __ldg(s.lg_ent + e + u);
#pragma unroll
        for (int u = 0; u < 4; u++) q[u] = __ldg(s.elems + 4 * id[u]);
        bool h[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            float tt;
            h[u] = isect_seg(o, d, q[u].x, q[u].y, q[u].z, q[u].w, tt);
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (h[u]) {
                if (count < kHitBuffer) hits[count] = id[u];
                count++;
            }
    }
    for (; e < e1; e++) {
        const uint32_t i = __ldg(s.lg_ent + e);
        float tt;
        if (isect_elem<2>(s, i, o, d, tt)) {
            if (count < kHitBuffer) hits[count] = i;
            count++;
        }
    }
    return true;
}

// All hits of the infinite line o + t d, in storage order (depth-first, children in order, so
// leaves come in increasing element order; or the line grid's cell lists, in storage order).
// Writes the first kHitBuffer element indices to hits and returns the total count. On a stack
// overflow or runaway traversal it flags s.err and returns what it has.
// The hits of one leaf (its elements are consecutive in storage order), appended in order; 3D
// leaves are tested two triangles at a time with both records' loads in flight.
template <int D>
__device__ __forceinline__ uint32_t leaf_hits(const SceneView<D> &s, uint32_t code, const V<D> &o, const V<D> &d,
                                              uint32_t *hits, uint32_t count) {
    const uint32_t first = code & 0x0FFFFFFFu, cnt = ((code >> 28) & 7u) + 1u;
    uint32_t i = first;
    if constexpr (D == 3) {
        for (; i + 1 < first + cnt; i += 2) {
            const float4 *q0 = s.isect + 4 * i, *q1 = q0 + 4;
            const F8 a0 = ldg8(q0), a1 = ldg8(q1);
            const float4 b0 = __ldg(q0 + 2), b1 = __ldg(q1 + 2);
            float t0, t1;
            const bool h0 = isect_tri(o, d, a0.a, a0.b, b0, t0);
            const bool h1 = isect_tri(o, d, a1.a, a1.b, b1, t1);
            if (h0) {
                if (count < kHitBuffer) hits[count] = i;
                count++;
            }
            if (h1) {
                if (count < kHitBuffer) hits[count] = i + 1;
                count++;
            }
        }
    }
    for (; i < first + cnt; i++) {
        float t;
        if (isect_elem<D>(s, i, o, d, t)) {
            if (count < kHitBuffer) hits[count] = i;
            count++;
        }
    }
    return count;
}

// Shared-memory columns of a thread's traversal stack and held leaves (entry-major: lanes at
// different depths still touch distinct banks), for kernels that run nothing but line queries
// (the wavefront's trace kernel). A kernel that references them gets the arrays as static shared
// memory, so walk kernels keep their stacks in local memory instead (line_query3), where the
// shared memory would only take L1 capacity from their gathers.
__device__ __forceinline__ uint32_t *stack_column() {
    __shared__ uint32_t s_stack[kSharedStack * kWalkBlock];
    return s_stack + threadIdx.x;
}
__device__ __forceinline__ uint32_t *leaf_column() {
    __shared__ uint32_t s_leaf[kLeafBatch * kWalkBlock];
    return s_leaf + threadIdx.x;
}

// The 3D line query. Depth-first over the 4-wide BVH, children in order, so the leaves (and the
// hits) come in storage order:
// - the first child a node's test keeps is visited next straight from a register; only its
//   later siblings are pushed (in reverse order), so descending costs no stack traffic;
// - leaves are postponed: a lane takes nodes until it holds kLeafBatch leaves or has nothing
//   left, then tests the held leaves in the order it met them, so the lanes of a warp run node
//   tests together and triangle tests together instead of alternating between them.
__device__ __forceinline__ uint32_t line_query3(const SceneView<3> &s, const V<3> &o, const V<3> &d, uint32_t *hits) {
    uint32_t stack[kStackSize];
    uint32_t leaves[kLeafBatch];
    const LineSlab3 L = line_slab3(o, d);
    int sp = 0;
    uint32_t code = 0u;  // root node
    bool live = true;
    uint32_t steps = 0, count = 0;
    while (live) {
        int nl = 0;
        while (nl < kLeafBatch) {
            if (++steps > s.traversal_limit) {
                atomicOr(s.err, kErrTraversalLimit);
                live = false;
                break;
            }
            if (code & 0x80000000u) {
                leaves[nl++] = code;
            } else {
                uint4 ch;
                uint32_t keep = node_hits(s, code, L, ch);
                const uint32_t cs[4] = {ch.x, ch.y, ch.z, ch.w};
#pragma unroll
                for (int k = 0; k < 4; k++)
                    if (cs[k] == kChildEmptyD) keep &= ~(1u << k);
                if (keep) {
                    if (sp + 3 > (int)kStackSize) {
                        atomicOr(s.err, kErrStackOverflow);
                        live = false;
                        break;
                    }
                    const uint32_t first = (uint32_t)(__ffs(keep) - 1);
#pragma unroll
                    for (int k = 3; k >= 1; k--)
                        if ((uint32_t)k > first && ((keep >> k) & 1u)) stack[sp++] = cs[k];
                    code = cs[first];
                    continue;
                }
            }
            if (sp == 0) {
                live = false;
                break;
            }
            code = stack[--sp];
        }
        for (int l = 0; l < nl; l++) count = leaf_hits<3>(s, leaves[l], o, d, hits, count);
    }
    return count;
}

// The 2D line query: the line grid, else depth-first over the 4-wide BVH.
__device__ __forceinline__ uint32_t line_query2(const SceneView<2> &s, const V<2> &o, const V<2> &d, uint32_t *hits) {
    uint32_t n_grid;
    if (s.lg_K != 0u && line_grid_query(s, o, d, hits, n_grid)) return n_grid;
    uint32_t stack[kStackSize];
    int sp = 0;
    stack[sp++] = 0u;  // root node
    uint32_t count = 0;
    const float c0 = d.v[0] * o.v[1] - d.v[1] * o.v[0];
    uint32_t steps = 0;
    while (sp > 0) {
        if (++steps > s.traversal_limit) { atomicOr(s.err, kErrTraversalLimit); break; }
        const uint32_t code = stack[--sp];
        if (code & 0x80000000u) {
            count = leaf_hits<2>(s, code, o, d, hits, count);
        } else {
            uint4 ch;
            const uint32_t mask = node_hits(s, code, o, d, c0, ch);
            const uint32_t cs[4] = {ch.x, ch.y, ch.z, ch.w};
            if (sp + 4 > (int)kStackSize) { atomicOr(s.err, kErrStackOverflow); break; }
#pragma unroll
            for (int k = 3; k >= 0; k--)
                if ((mask >> k) & 1u)
                    if (cs[k] != kChildEmptyD) stack[sp++] = cs[k];
        }
    }
    return count;
}

template <int D>
__device__ __forceinline__ uint32_t line_query(const SceneView<D> &s, const V<D> &o, const V<D> &d, uint32_t *hits) {
    if constexpr (D == 3) return line_query3(s, o, d, hits);
    else return line_query2(s, o, d, hits);
}

// ------------------------------------------------------------------------------------------
// Boundary sampling queries (scene.cuh:441-622, 734-918).
// ------------------------------------------------------------------------------------------
// The point of a uniform boundary sample on element e from its draws u[0..D-1] (u[0] picked the
// element): linear interpolation in 2D, the sqrt-barycentric map in 3D.
template <int D> __device__ __forceinline__ BPoint<D> uniform_point(const Elem<D> &e, const float *u) {
    BPoint<D> r;
    if constexpr (D == 2) {
        const float u2 = u[1];
        r.p.v[0] = interp2(e.v[0].v[0], e.v[1].v[0], u2);
        r.p.v[1] = interp2(e.v[0].v[1], e.v[1].v[1], u2);
        r.n = e.n;
        r.angle = 0.5f;
        r.bv = interp2(e.bv[0], e.bv[1], u2);
        r.type = e.type;
        r.alpha = interp2(e.alpha[0], e.alpha[1], u2);
    } else {
        const float u2 = u[1], u3 = u[2];
        const float sq = sqrtf(u2);
        const float k1 = 1.0f - sq, k2 = sq * (1.0f - u3), k3 = u3 * sq;
#pragma unroll
        for (int i = 0; i < 3; i++) r.p.v[i] = interp3(e.v[0].v[i], e.v[1].v[i], e.v[2].v[i], k1, k2, k3);
        r.n = e.n;
        r.angle = 0.5f;
        r.bv = interp3(e.bv[0], e.bv[1], e.bv[2], k1, k2, k3);
        r.type = e.type;
        r.alpha = interp3(e.alpha[0], e.alpha[1], e.alpha[2], k1, k2, k3);
    }
    return r;
}

// The position alone of the uniform sample on stored element i with draws u (what a resampling
// candidate's target needs): uniform_point's interpolation, reading only the vertices.
template <int D> __device__ __forceinline__ V<D> uniform_position(const SceneView<D> &s, uint32_t i, const float *u) {
    V<D> r;
    if constexpr (D == 2) {
        const float4 q0 = __ldg(s.elems + 4 * i);
        const float u2 = u[1];
        r.v[0] = interp2(q0.x, q0.z, u2);
        r.v[1] = interp2(q0.y, q0.w, u2);
    } else {
        const float4 *p = s.elems + 4 * i;
        const F8 q = ldg8(p);
        const float cz = __ldg(reinterpret_cast<const float *>(p + 2));
        const float u2 = u[1], u3 = u[2];
        const float sq = sqrtf(u2);
        const float k1 = 1.0f - sq, k2 = sq * (1.0f - u3), k3 = u3 * sq;
        r.v[0] = interp3(q.a.x, q.a.w, q.b.z, k1, k2, k3);
        r.v[1] = interp3(q.a.y, q.b.x, q.b.w, k1, k2, k3);
        r.v[2] = interp3(q.a.z, q.b.y, cz, k1, k2, k3);
    }
    return r;
}

template <int D> __device__ __forceinline__ BPoint<D> sample_uniform(const SceneView<D> &s, PathRng &rng, float &inv_pdf) {
    float u[D];
#pragma unroll
    for (int i = 0; i < D; i++) u[i] = rng.uniform();
    const uint32_t idx = cdf_search(s.area_cdf, s.area_guide, s.area_G, u[0]);
    inv_pdf = s.total_area;
    return uniform_point<D>(load_elem<D>(s, idx), u);
}

// A uniform sample that also returns the stored index of its element.
template <int D> __device__ __forceinline__ BPoint<D> sample_uniform_idx(const SceneView<D> &s, PathRng &rng, float &inv_pdf,
                                                                        uint32_t &idx) {
    float u[D];
#pragma unroll
    for (int i = 0; i < D; i++) u[i] = rng.uniform();
    idx = cdf_search(s.area_cdf, s.area_guide, s.area_G, u[0]);
    inv_pdf = s.total_area;
    return uniform_point<D>(load_elem<D>(s, idx), u);
}

// Two consecutive uniform samples: the draws of both are taken first, in the order two
// sample_uniform calls take them, and both guide and element loads are issued before either is
// used, so the two dependent load chains overlap. Same values as two sample_uniform calls.
template <int D> __device__ __forceinline__ void sample_uniform_pair(const SceneView<D> &s, PathRng &rng, BPoint<D> &ya,
                                                                    float &ipa, BPoint<D> &yb, float &ipb) {
    float ua[D], ub[D];
#pragma unroll
    for (int i = 0; i < D; i++) ua[i] = rng.uniform();
#pragma unroll
    for (int i = 0; i < D; i++) ub[i] = rng.uniform();
    const uint4 ga = __ldg(s.area_guide + guide_bin(s.area_G, ua[0]));
    const uint4 gb = __ldg(s.area_guide + guide_bin(s.area_G, ub[0]));
    const uint32_t ia = cdf_resolve(s.area_cdf, ga, ua[0]);
    const uint32_t ib = cdf_resolve(s.area_cdf, gb, ub[0]);
    const Elem<D> ea = load_elem<D>(s, ia);
    const Elem<D> eb = load_elem<D>(s, ib);
    ya = uniform_point<D>(ea, ua);
    yb = uniform_point<D>(eb, ub);
    ipa = s.total_area;
    ipb = s.total_area;
}

// The random direction of a line-intersection sample (scene.cuh:472-478, 776-784): the upper
// half-circle in 2D, a hemisphere direction in 3D.
template <int D> __device__ __forceinline__ V<D> line_sample_direction(PathRng &rng) {
    V<D> dir;
    if constexpr (D == 2) {
        const float theta = rng.uniform();
        sincospi_own(theta, &dir.v[0], &dir.v[1]);
    } else {
        dir.v[2] = rng.uniform();
        const float phi = 2.0f * rng.uniform();
        sincospi_own(phi, &dir.v[0], &dir.v[1]);
        const float r = sqrtf(1.0f - dir.v[2] * dir.v[2]);
        dir.v[0] = dir.v[0] * r;
        dir.v[1] = dir.v[1] * r;
    }
    return dir;
}

// The sample once the line's hits are known (scene.cuh:488-515, 792-830): none -> the zero point;
// else one of the first min(m, 64) hits chosen uniformly, its point, data and Robin alpha. Split in
// two for kernels that choose the hit where the query ran and form the point elsewhere:
// line_hit_choice takes the choice's draw (only when there is a hit) and returns the element,
// line_hit_point forms the sample on it.
__device__ __forceinline__ uint32_t line_hit_choice(PathRng &rng, const uint32_t *hits, uint32_t &m) {
    if (m == 0) return 0u;
    m = m < kHitBuffer ? m : kHitBuffer;
    const float u = rng.uniform();
    uint32_t k = (uint32_t)((float)m * u);
    k = (m - 1) < k ? (m - 1) : k;
    return hits[k];
}
template <int D> __device__ __forceinline__ BPoint<D> line_hit_point(const SceneView<D> &s, uint32_t ei, uint32_t m,
                                                                    const V<D> &x, const V<D> &dir) {
    if (m == 0) {
        BPoint<D> z = bp_zero<D>();
        z.angle = 0.5f;
        return z;
    }
    const Elem<D> e = load_elem<D>(s, ei);
    float t = 0.0f;
    isect_elem<D>(s, ei, x, dir, t);
    BPoint<D> r;
#pragma unroll
    for (int i = 0; i < D; i++) r.p.v[i] = x.v[i] + t * dir.v[i];
    r.n = e.n;
    r.angle = 0.5f;
    r.type = e.type;
    if constexpr (D == 2) {
        const float tt = vnorm(vsub(r.p, e.v[0])) / e.area;
        r.bv = interp2(e.bv[0], e.bv[1], tt);
        r.alpha = interp2(e.alpha[0], e.alpha[1], tt);
    } else {
        // barycentric coordinates (scene.cuh:45-69)
        const V<3> v0 = vsub(e.v[1], e.v[0]), v1 = vsub(e.v[2], e.v[0]), v2 = vsub(r.p, e.v[0]);
        const float d00 = vdot(v0, v0), d01 = vdot(v0, v1), d11 = vdot(v1, v1);
        const float d20 = vdot(v2, v0), d21 = vdot(v2, v1);
        const float denom = d00 * d11 - d01 * d01;
        const float L1 = (d11 * d20 - d01 * d21) / denom;
        const float L2 = (d00 * d21 - d01 * d20) / denom;
        const float L0 = 1.0f - (L1 + L2);
        r.bv = L0 * e.bv[0] + L1 * e.bv[1] + L2 * e.bv[2];
        r.alpha = L0 * e.alpha[0] + L1 * e.alpha[1] + L2 * e.alpha[2];
    }
    return r;
}
template <int D> __device__ __forceinline__ BPoint<D> line_sample_from_hits(const SceneView<D> &s, PathRng &rng,
                                                                           const V<D> &x, const V<D> &dir,
                                                                           const uint32_t *hits, uint32_t m,
                                                                           uint32_t &m_out) {
    const uint32_t ei = line_hit_choice(rng, hits, m);
    m_out = m;
    return line_hit_point<D>(s, ei, m, x, dir);
}

// inv_pdf of a line-intersection sample r of m hits from x (scene.cuh:519-528, 835-845).
template <int D> __device__ __forceinline__ float line_sample_inv_pdf(const BPoint<D> &r, const V<D> &x, uint32_t m) {
    const V<D> rv = vsub(r.p, x);
    const float cosv = fmax_ref(fabsf(vdot(vnormalized(rv), r.n)), kEps10);
    if constexpr (D == 2) return (float)m * 0x1.921fb6p+1f * vnorm(rv) / cosv;
    else return (float)m * 2.0f * 0x1.921fb6p+1f * vsqnorm(rv) / cosv;
}

template <int D> __device__ __forceinline__ BPoint<D> sample_line_intersection2(const SceneView<D> &s, PathRng &rng, const V<D> &x, uint32_t &m_out) {
    const V<D> dir = line_sample_direction<D>(rng);
    uint32_t hits[kHitBuffer];
    const uint32_t m = line_query<D>(s, x, dir, hits);
    return line_sample_from_hits<D>(s, rng, x, dir, hits, m, m_out);
}

template <int D> __device__ __forceinline__ BPoint<D> sample_line_intersection(const SceneView<D> &s, PathRng &rng, const V<D> &x, float &inv_pdf) {
    uint32_t m;
    const BPoint<D> r = sample_line_intersection2<D>(s, rng, x, m);
    inv_pdf = line_sample_inv_pdf<D>(r, x, m);
    return r;
}

template <int D> __device__ __forceinline__ BPoint<D> sample_boundary_value(const SceneView<D> &s, PathRng &rng, float &inv_pdf) {
    const float u1 = rng.uniform();
    const uint32_t idx = cdf_search(s.bv_cdf, s.bv_guide, s.bv_G, u1);
    const Elem<D> e = load_elem<D>(s, idx);
    BPoint<D> r;
    if constexpr (D == 2) {
        const float u2 = rng.uniform();
        const float ba = fabsf(e.bv[0]), bb = fabsf(e.bv[1]);
        float t;
        if (fabsf(ba - bb) < kEps10) t = u2;
        else t = (-ba + sqrtf(ba * ba + u2 * (bb * bb - ba * ba))) / (bb - ba);
        r.p.v[0] = interp2(e.v[0].v[0], e.v[1].v[0], t);
        r.p.v[1] = interp2(e.v[0].v[1], e.v[1].v[1], t);
        r.n = e.n;
        r.angle = 0.5f;
        r.bv = interp2(e.bv[0], e.bv[1], t);
        r.type = e.type;
        r.alpha = interp2(e.alpha[0], e.alpha[1], t);
        inv_pdf = s.total_bv / (ba + t * (bb - ba));
    } else {
        const float pmf = idx == 0 ? __ldg(s.bv_cdf) : __ldg(s.bv_cdf + idx) - __ldg(s.bv_cdf + idx - 1);
        const float u2 = rng.uniform();
        const float u3 = rng.uniform();
        const float sq = sqrtf(u2);
        const float k1 = 1.0f - sq, k2 = sq * (1.0f - u3), k3 = u3 * sq;
#pragma unroll
        for (int i = 0; i < 3; i++) r.p.v[i] = interp3(e.v[0].v[i], e.v[1].v[i], e.v[2].v[i], k1, k2, k3);
        r.n = e.n;
        r.angle = 0.5f;
        r.bv = interp3(e.bv[0], e.bv[1], e.bv[2], k1, k2, k3);
        r.type = e.type;
        r.alpha = interp3(e.alpha[0], e.alpha[1], e.alpha[2], k1, k2, k3);
        inv_pdf = __ldg(reinterpret_cast<const float *>(s.elem_aux + idx) + 3) / pmf;
    }
    return r;
}

template <int D> struct VSample {
    V<D> p;
    float value, inv_pdf;
};

// Source-value sampling of the volume cache (scene.cuh:100-120).
template <int D> __device__ __forceinline__ VSample<D> sample_volume(const SceneView<D> &s, PathRng &rng) {
    VSample<D> r;
    const float u = rng.uniform();
    const uint32_t idx = cdf_search(s.vol_cdf, s.vol_guide, s.vol_G, u);
    const uint32_t res = s.vol_res;
    const float dx = s.vol_size / (float)res;
    const uint32_t c[3] = {idx % res, (idx / res) % res, idx / (res * res)};
#pragma unroll
    for (int i = 0; i < D; i++) r.p.v[i] = ((float)c[i] + 0.5f) * dx - s.vol_size / 2.0f;
#pragma unroll
    for (int i = 0; i < D; i++) {
        const float uj = rng.uniform();
        r.p.v[i] = r.p.v[i] + (uj - 0.5f) * s.vol_size / (float)res;
    }
    r.value = __ldg(s.vol_values + idx);
    const float pdf = idx == 0 ? __ldg(s.vol_cdf) : __ldg(s.vol_cdf + idx) - __ldg(s.vol_cdf + idx - 1);
    float cell = 1.0f;
#pragma unroll
    for (int i = 0; i < D; i++) cell = cell * (s.vol_size / (float)res);
    r.inv_pdf = cell / pdf;
    return r;
}

}  // namespace wobgb
