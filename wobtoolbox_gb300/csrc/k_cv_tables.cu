// Dense triangle sums of the learned control variate for the single-layer Neumann estimators.
//
// The control variate is a density sigma~ that is constant on every stored triangle (the network
// evaluated at the triangle's centroid). Two sums over all triangles i of the scene use it:
//
//   residual data (targets: the centroids c_j of the triangles, with their normals n_j):
//     (T sigma~)(c_j) = -c / (4 pi) sum_i sigma~_i n_j . grad P_i(c_j),   c = +2 inside, -2 outside,
//     delta_j = ((T sigma~)(c_j) - sigma~_j) / c,
//   where T(x, y) = -c dG/dn_x is the kernel of the single-layer Neumann equation
//   sigma = c g + T sigma (bie_models.cuh:262-316: fredholm_equation_boundary_known / _unknown).
//   Adding delta_j to the Neumann data of triangle j turns the walk's source c g into
//   c g + T sigma~ - sigma~, whose solution is the residual sigma - sigma~;
//
//   potential (targets: evaluation points x): u~(x) = (1/4 pi) sum_i sigma~_i P_i(x) and its
//   gradient, the single-layer potential of sigma~ (solution_domain_unknown, bie_models.cuh:225-240).
//
// P_i(x) is the integral of 1/|x - y| over triangle i. Pairs farther apart than near_factor times
// the triangle's longest edge use the centroid rule A_i / |x - c_i|; nearer pairs use the closed
// form of the potential of a uniformly charged flat triangle and its gradient (Wilton et al.,
// IEEE Trans. Antennas Propag. 32(3), 1984), with coordinates taken relative to the target. A
// triangle's own term in the residual data is zero: n_j is normal to triangle j, so dG/dn_x
// vanishes on it.
//
// Far field by a treecode over consecutive stored triangles (BVH storage order keeps them
// spatially compact): clusters of 32, groups of 8 clusters (256 triangles) and groups of 8 of
// those (2048), each record with its centre z (mean centroid), radius rho, largest near radius eta
// and the moments of its centroid sources about z up to the quadrupole (M0 = sum w, M1 = sum w d,
// M2 = sum w d d^T, w = sigma~ A, d = c - z). A block takes 32 consecutive targets and the
// bounding sphere (W, omega) of their positions; a record with |W - z| > max(rho / theta,
// rho + eta) + omega is far from every target of the block and enters through its quadrupole
// expansion of sum w / |x - c| (one evaluation per target for all its triangles, error of order
// (rho / |x - z|)^3 of its share). The block starts from the largest groups and looks into the
// near ones; a near cluster is taken triangle by triangle as above. theta = 0 takes every
// triangle (the dense sum). The decisions are uniform across the block, so lanes never diverge.
//
// Work decomposition: one block per 32 targets (a lane each); its 8 warps make the same decisions
// and take the work by index (a far group to warp index mod 8, the 8 clusters of a near group one
// each), records read as broadcasts; FP32 partial sums over 32 items, FP64 across them and across
// the warps (in warp order: deterministic).
// This unit is compiled with FMA contraction (it is not part of the bit-exact walk).
#include "device_common.cuh"
#include "launch.hpp"

namespace wobgb {

namespace {

constexpr int kCvBlock = 256;
constexpr int kCvWarps = kCvBlock / 32;
constexpr double kInv4Pi = 0.07957747154594767;

struct TriVerts {
    float a[3], b[3], c[3];
};

__device__ __forceinline__ TriVerts load_tri(const SceneView<3> &s, uint32_t i) {
    const float4 *p = s.elems + 4 * i;
    const float4 q0 = __ldg(p), q1 = __ldg(p + 1), q2 = __ldg(p + 2);
    TriVerts t;
    t.a[0] = q0.x; t.a[1] = q0.y; t.a[2] = q0.z;
    t.b[0] = q0.w; t.b[1] = q1.x; t.b[2] = q1.y;
    t.c[0] = q1.z; t.c[1] = q1.w; t.c[2] = q2.x;
    return t;
}

// ln((R+ + s+) / (R- + s-)), in the form without cancellation for the edge's side of rho.
__device__ __forceinline__ float edge_log(float Rp, float sp, float Rm, float sm) {
    if (sm + sp >= 0.0f) return logf((Rp + sp) / (Rm + sm));
    return logf((Rm - sm) / (Rp - sp));
}

// P(x) = integral over the triangle of 1 / |x - y| dA and grad P(x), closed form (FP32; the
// coordinates are taken relative to x so that near pairs keep their relative precision).
__device__ void triangle_potential(const float x[3], const TriVerts &t, float &P, float G[3]) {
    float a[3], b[3], c[3];
    for (int k = 0; k < 3; k++) { a[k] = t.a[k] - x[k]; b[k] = t.b[k] - x[k]; c[k] = t.c[k] - x[k]; }
    float e1[3], e2[3], n[3];
    for (int k = 0; k < 3; k++) { e1[k] = b[k] - a[k]; e2[k] = c[k] - a[k]; }
    n[0] = e1[1] * e2[2] - e1[2] * e2[1];
    n[1] = e1[2] * e2[0] - e1[0] * e2[2];
    n[2] = e1[0] * e2[1] - e1[1] * e2[0];
    const float nl = sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    P = 0.0f;
    G[0] = G[1] = G[2] = 0.0f;
    if (!(nl > 0.0f)) return;
    for (int k = 0; k < 3; k++) n[k] /= nl;
    const float h = -(a[0] * n[0] + a[1] * n[1] + a[2] * n[2]);  // (x - a) . n with x at the origin
    const float ah = fabsf(h);
    float rho[3];
    for (int k = 0; k < 3; k++) rho[k] = -h * n[k];
    const float *vs[4] = {a, b, c, a};
    float beta_sum = 0.0f;
    for (int e = 0; e < 3; e++) {
        const float *p0 = vs[e], *p1 = vs[e + 1];
        float sv[3], m[3];
        for (int k = 0; k < 3; k++) sv[k] = p1[k] - p0[k];
        const float sl = sqrtf(sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2]);
        for (int k = 0; k < 3; k++) sv[k] /= sl;
        m[0] = sv[1] * n[2] - sv[2] * n[1];
        m[1] = sv[2] * n[0] - sv[0] * n[2];
        m[2] = sv[0] * n[1] - sv[1] * n[0];
        float sm = 0.0f, sp = 0.0f, tt = 0.0f, Rm2 = 0.0f, Rp2 = 0.0f;
        for (int k = 0; k < 3; k++) {
            sm += (p0[k] - rho[k]) * sv[k];
            sp += (p1[k] - rho[k]) * sv[k];
            tt += (p0[k] - rho[k]) * m[k];
            Rm2 += p0[k] * p0[k];
            Rp2 += p1[k] * p1[k];
        }
        const float R0sq = tt * tt + h * h;
        if (!(R0sq > 0.0f)) continue;  // x on the edge's line: no contribution from this edge
        const float Rm = sqrtf(Rm2), Rp = sqrtf(Rp2);
        const float f = edge_log(Rp, sp, Rm, sm);
        const float beta = atanf(tt * sp / (R0sq + ah * Rp)) - atanf(tt * sm / (R0sq + ah * Rm));
        P += tt * f - ah * beta;
        for (int k = 0; k < 3; k++) G[k] -= m[k] * f;
        beta_sum += beta;
    }
    const float sg = h > 0.0f ? 1.0f : (h < 0.0f ? -1.0f : 0.0f);
    for (int k = 0; k < 3; k++) G[k] -= sg * beta_sum * n[k];
}

__device__ __forceinline__ void centroid_of(const TriVerts &t, float c[3]) {
    for (int k = 0; k < 3; k++) c[k] = (t.a[k] + t.b[k] + t.c[k]) / 3.0f;
}

// Per stored triangle: {centroid, sigma~ * area} and the squared near radius.
__global__ void cv_sources_kernel(SceneView<3> s, const float *__restrict__ sigma, float near_factor,
                                  float4 *__restrict__ src, float *__restrict__ near2) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n_elems) return;
    const TriVerts t = load_tri(s, i);
    float c[3];
    centroid_of(t, c);
    float e1[3], e2[3];
    for (int k = 0; k < 3; k++) { e1[k] = t.b[k] - t.a[k]; e2[k] = t.c[k] - t.a[k]; }
    const float cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                cz = e1[0] * e2[1] - e1[1] * e2[0];
    const float area = 0.5f * sqrtf(cx * cx + cy * cy + cz * cz);
    float h2 = 0.0f;
    const float *vs[4] = {t.a, t.b, t.c, t.a};
    for (int e = 0; e < 3; e++) {
        float l2 = 0.0f;
        for (int k = 0; k < 3; k++) l2 += (vs[e + 1][k] - vs[e][k]) * (vs[e + 1][k] - vs[e][k]);
        h2 = fmaxf(h2, l2);
    }
    src[i] = make_float4(c[0], c[1], c[2], sigma[i] * area);
    near2[i] = near_factor * near_factor * h2;
}

constexpr int kClusterSize = 32;

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_max_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Morton order of evaluation points: bounds (order-preserving integer atomics), 30-bit codes (10
// bits a coordinate), a bitonic sort of {code, index} keys padded to a power of two.
__device__ __forceinline__ uint32_t ordered_bits(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float from_ordered_bits(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}
__device__ __forceinline__ uint32_t spread_bits10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
__global__ void bounds_init_kernel(uint32_t *bb) {
    if (threadIdx.x < 6) bb[threadIdx.x] = threadIdx.x < 3 ? 0xffffffffu : 0u;
}
__global__ void pts_bounds_kernel(const float *__restrict__ pts, uint32_t n, uint32_t *__restrict__ bb) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int k = 0; k < 3; k++) {
        const uint32_t o = ordered_bits(pts[(size_t)i * 3 + k]);
        atomicMin(bb + k, o);
        atomicMax(bb + 3 + k, o);
    }
}
__global__ void pts_morton_kernel(const float *__restrict__ pts, uint32_t n, uint32_t n2, const uint32_t *__restrict__ bb,
                                  uint64_t *__restrict__ key) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n2) return;
    if (i >= n) {
        key[i] = ~0ull;
        return;
    }
    uint32_t code = 0;
    for (int k = 0; k < 3; k++) {
        const float lo = from_ordered_bits(bb[k]), hi = from_ordered_bits(bb[3 + k]);
        const float t = hi > lo ? (pts[(size_t)i * 3 + k] - lo) / (hi - lo) : 0.0f;
        const uint32_t q = (uint32_t)fminf(fmaxf(t * 1024.0f, 0.0f), 1023.0f);
        code |= spread_bits10(q) << k;
    }
    key[i] = ((uint64_t)code << 32) | i;
}
__global__ void bitonic_kernel(uint32_t n2, uint32_t j, uint32_t k, uint64_t *__restrict__ key) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n2) return;
    const uint32_t l = i ^ j;
    if (l <= i) return;
    const uint64_t a = key[i], b = key[l];
    if (((i & k) == 0) == (a > b)) {
        key[i] = b;
        key[l] = a;
    }
}

// One warp per cluster: the record {z, r_far}, {M0, M1}, {M2xx, M2yy, M2zz, M2xy}, {M2xz, M2yz,
// trace M2, 0}; r_far = max(rho / theta, rho + eta), infinite for theta = 0.
__global__ void cv_cluster_kernel(uint32_t n, const float4 *__restrict__ src, const float *__restrict__ near2,
                                  float theta, float4 *__restrict__ cl) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_cl = (n + kClusterSize - 1) / kClusterSize;
    if (k >= n_cl) return;
    const uint32_t i = k * kClusterSize + lane;
    const bool valid = i < n;
    const float4 q = valid ? __ldg(src + i) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float e2 = valid ? __ldg(near2 + i) : 0.0f;
    const float cnt = (float)__popc(__ballot_sync(0xffffffffu, valid));
    const float zx = warp_sum_f(q.x) / cnt, zy = warp_sum_f(q.y) / cnt, zz = warp_sum_f(q.z) / cnt;
    const float dx = valid ? q.x - zx : 0.0f, dy = valid ? q.y - zy : 0.0f, dz = valid ? q.z - zz : 0.0f;
    const float rho = sqrtf(warp_max_f(dx * dx + dy * dy + dz * dz));
    const float eta = sqrtf(warp_max_f(e2));
    const float w = q.w;
    const float m0 = warp_sum_f(w);
    const float m1x = warp_sum_f(w * dx), m1y = warp_sum_f(w * dy), m1z = warp_sum_f(w * dz);
    const float mxx = warp_sum_f(w * dx * dx), myy = warp_sum_f(w * dy * dy), mzz = warp_sum_f(w * dz * dz);
    const float mxy = warp_sum_f(w * dx * dy), mxz = warp_sum_f(w * dx * dz), myz = warp_sum_f(w * dy * dz);
    if (lane == 0) {
        const float r_far = theta > 0.0f ? fmaxf(rho / theta, rho + eta) : __int_as_float(0x7f800000);
        cl[4 * k + 0] = make_float4(zx, zy, zz, r_far);
        cl[4 * k + 1] = make_float4(m0, m1x, m1y, m1z);
        cl[4 * k + 2] = make_float4(mxx, myy, mzz, mxy);
        cl[4 * k + 3] = make_float4(mxz, myz, mxx + myy + mzz, 0.0f);
    }
}

// Groups of kGroupFan^L clusters (L = 1, 2: 256 and 2048 consecutive stored triangles), one block
// of 256 threads each: the same record as a cluster's, from the member sources directly (centre =
// mean centroid, exact radius, largest near radius, moments about the centre).
constexpr int kGroupFan = 8;
constexpr int kGroupBlock = 256;
__device__ __forceinline__ float block_reduce(float v, bool is_max, float *red) {
    v = is_max ? warp_max_f(v) : warp_sum_f(v);
    if ((threadIdx.x & 31u) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float t = red[0];
    for (int w = 1; w < kGroupBlock / 32; w++) t = is_max ? fmaxf(t, red[w]) : t + red[w];
    __syncthreads();
    return t;
}
template <uint32_t kSize>
__global__ void __launch_bounds__(kGroupBlock) cv_group_kernel(uint32_t n, const float4 *__restrict__ src,
                                                               const float *__restrict__ near2, float theta,
                                                               float4 *__restrict__ rec) {
    __shared__ float red[kGroupBlock / 32];
    const uint32_t g = blockIdx.x, i0 = g * kSize, i1 = min(n, i0 + kSize);
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    for (uint32_t i = i0 + threadIdx.x; i < i1; i += kGroupBlock) {
        const float4 q = __ldg(src + i);
        sx += q.x;
        sy += q.y;
        sz += q.z;
    }
    const float cnt = (float)(i1 - i0);
    const float zx = block_reduce(sx, false, red) / cnt, zy = block_reduce(sy, false, red) / cnt,
                zz = block_reduce(sz, false, red) / cnt;
    float r2 = 0.0f, e2 = 0.0f, m[10] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    for (uint32_t i = i0 + threadIdx.x; i < i1; i += kGroupBlock) {
        const float4 q = __ldg(src + i);
        const float dx = q.x - zx, dy = q.y - zy, dz = q.z - zz, w = q.w;
        r2 = fmaxf(r2, dx * dx + dy * dy + dz * dz);
        e2 = fmaxf(e2, __ldg(near2 + i));
        m[0] += w;
        m[1] += w * dx; m[2] += w * dy; m[3] += w * dz;
        m[4] += w * dx * dx; m[5] += w * dy * dy; m[6] += w * dz * dz;
        m[7] += w * dx * dy; m[8] += w * dx * dz; m[9] += w * dy * dz;
    }
    const float rho = sqrtf(block_reduce(r2, true, red)), eta = sqrtf(block_reduce(e2, true, red));
#pragma unroll
    for (int k = 0; k < 10; k++) m[k] = block_reduce(m[k], false, red);
    if (threadIdx.x == 0) {
        const float r_far = theta > 0.0f ? fmaxf(rho / theta, rho + eta) : __int_as_float(0x7f800000);
        rec[4 * g + 0] = make_float4(zx, zy, zz, r_far);
        rec[4 * g + 1] = make_float4(m[0], m[1], m[2], m[3]);
        rec[4 * g + 2] = make_float4(m[4], m[5], m[6], m[7]);
        rec[4 * g + 3] = make_float4(m[8], m[9], m[4] + m[5] + m[6], 0.0f);
    }
}

__host__ __device__ __forceinline__ uint32_t div_up(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

// sum w / |x - c| over a cluster by its quadrupole expansion about z (R = x - z):
//   phi = M0 / R + (R . M1) / R^3 + (3 R.M2.R - R^2 tr M2) / (2 R^5),
// and its gradient term by term.
__device__ __forceinline__ void cluster_field(const float x[3], const float4 &q0, const float4 &q1, const float4 &q2,
                                             const float4 &q3, float &phi, float g[3]) {
    const float R[3] = {x[0] - q0.x, x[1] - q0.y, x[2] - q0.z};
    const float R2 = R[0] * R[0] + R[1] * R[1] + R[2] * R[2];
    const float ri = rsqrtf(R2);
    const float ri2 = ri * ri, ri3 = ri * ri2, ri5 = ri3 * ri2;
    const float RM1 = R[0] * q1.y + R[1] * q1.z + R[2] * q1.w;
    const float M2R[3] = {q2.x * R[0] + q2.w * R[1] + q3.x * R[2], q2.w * R[0] + q2.y * R[1] + q3.y * R[2],
                          q3.x * R[0] + q3.y * R[1] + q2.z * R[2]};
    const float RM2R = R[0] * M2R[0] + R[1] * M2R[1] + R[2] * M2R[2];
    const float Q = 3.0f * RM2R - R2 * q3.z;
    phi = q1.x * ri + RM1 * ri3 + 0.5f * Q * ri5;
    const float a = -q1.x * ri3 - 3.0f * RM1 * ri5 - q3.z * ri5 - 2.5f * Q * ri5 * ri2;
    const float m1[3] = {q1.y, q1.z, q1.w};
#pragma unroll
    for (int k = 0; k < 3; k++) g[k] = a * R[k] + m1[k] * ri3 + 3.0f * M2R[k] * ri5;
}

// kMode 0: residual data at the stored triangles' centroids; kMode 1: potential and gradient at
// points (out: [n][4] = u, du/dx, du/dy, du/dz). A block takes 32 consecutive targets (one per
// lane); its kCvWarps warps split the cluster table (warp w takes clusters w, w + kCvWarps, ...)
// and their sums are added in warp order through shared memory at the end.
template <int kMode>
__global__ void __launch_bounds__(kCvBlock) cv_sum_kernel(SceneView<3> s, const float4 *__restrict__ src,
                                                          const float *__restrict__ near2,
                                                          const float *__restrict__ sigma,
                                                          const float4 *__restrict__ cl, const float *__restrict__ pts,
                                                          const uint64_t *__restrict__ order, uint32_t n_targets,
                                                          float c_coef, float *__restrict__ out,
                                                          double *__restrict__ part_sums) {
    __shared__ double s_acc[kCvWarps][4][32];
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t slot = blockIdx.x * 32u + lane;
    const bool active = slot < n_targets;
    // points are taken in Morton order (order: sorted {code, index} keys), so that the 32 targets
    // of a block are close together; triangles are already (BVH storage order)
    const uint32_t tgt = (kMode == 1 && active) ? (uint32_t)__ldg(order + slot) : slot;
    const uint32_t act = __ballot_sync(0xffffffffu, active);
    float xd[3] = {0.0f, 0.0f, 0.0f}, nn[3] = {0.0f, 0.0f, 0.0f};
    if (active) {
        if (kMode == 0) {
            const TriVerts tv = load_tri(s, tgt);
            centroid_of(tv, xd);
            const float4 q2 = __ldg(s.elems + 4 * tgt + 2);
            nn[0] = q2.y; nn[1] = q2.z; nn[2] = q2.w;
        } else {
            for (int k = 0; k < 3; k++) xd[k] = pts[(size_t)tgt * 3 + k];
        }
    }
    // the bounding sphere of the block's targets
    const float cnt = (float)__popc(act);
    const float Wx = warp_sum_f(xd[0]) / cnt, Wy = warp_sum_f(xd[1]) / cnt, Wz = warp_sum_f(xd[2]) / cnt;
    const float ox = xd[0] - Wx, oy = xd[1] - Wy, oz = xd[2] - Wz;
    const float om = sqrtf(warp_max_f(active ? ox * ox + oy * oy + oz * oz : 0.0f));
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const uint32_t n_src = s.n_elems;
    const uint32_t n_cl = div_up(n_src, kClusterSize), n_g1 = div_up(n_cl, kGroupFan), n_g2 = div_up(n_g1, kGroupFan);
    const float4 *g1 = cl + 4 * (size_t)n_cl, *g2 = g1 + 4 * (size_t)n_g1;
    uint32_t taken = 0;
    // far from every target of the block: |W - z| > r_far + omega
    auto is_far = [&](const float4 &q0) {
        const float Dx = Wx - q0.x, Dy = Wy - q0.y, Dz = Wz - q0.z;
        const float thr = q0.w + om;
        return Dx * Dx + Dy * Dy + Dz * Dz > thr * thr;
    };
    // a record's expansion at this lane's target; FP32 partial sums flushed to FP64 every 32 items
    auto expand = [&](const float4 *r, const float4 &q0) {
        const float4 q1 = __ldg(r + 1), q2 = __ldg(r + 2), q3 = __ldg(r + 3);
        float phi, g[3];
        cluster_field(xd, q0, q1, q2, q3, phi, g);
        if (kMode == 0) {
            a[0] -= g[0] * nn[0] + g[1] * nn[1] + g[2] * nn[2];
        } else {
            a[0] += phi;
            a[1] += g[0];
            a[2] += g[1];
            a[3] += g[2];
        }
    };
    auto flush = [&]() {
        if ((++taken & 31u) == 0u) {
#pragma unroll
            for (int c = 0; c < 4; c++) {
                acc[c] += a[c];
                a[c] = 0.0f;
            }
        }
    };
    // Every warp walks the same decisions (uniform across the block); the work is dealt by index:
    // a far group or level-1 group to warp (index mod 8), the clusters of a near level-1 group one
    // per warp, so the near field spreads over the warps as in a flat pass over the clusters.
    // the largest groups are split over gridDim.y blocks of the same targets (part blockIdx.y takes
    // k2 = part, part + gridDim.y, ...), whose sums part_sums holds for cv_parts_kernel
    for (uint32_t k2 = blockIdx.y; k2 < n_g2; k2 += gridDim.y) {
        const float4 h2 = __ldg(g2 + 4 * k2);
        if (is_far(h2)) {
            if (k2 % kCvWarps == wid) {
                expand(g2 + 4 * k2, h2);
                flush();
            }
            continue;
        }
        const uint32_t k1_end = min(n_g1, (k2 + 1) * kGroupFan);
        for (uint32_t k1 = k2 * kGroupFan; k1 < k1_end; k1++) {
            const float4 h1 = __ldg(g1 + 4 * k1);
            if (is_far(h1)) {
                if (k1 % kCvWarps == wid) {
                    expand(g1 + 4 * k1, h1);
                    flush();
                }
                continue;
            }
            const uint32_t k_end = min(n_cl, (k1 + 1) * kGroupFan);
            for (uint32_t k = k1 * kGroupFan + wid; k < k_end; k += kCvWarps) {
                const float4 q0 = __ldg(cl + 4 * k);
                if (is_far(q0)) {
                    expand(cl + 4 * k, q0);
                } else {
                    const uint32_t i0 = k * kClusterSize, i1 = min(n_src, i0 + kClusterSize);
                    for (uint32_t i = i0; i < i1; i++) {
                        const float4 q = __ldg(src + i);
                        const float n2 = __ldg(near2 + i);
                        const float dx = xd[0] - q.x, dy = xd[1] - q.y, dz = xd[2] - q.z;
                        const float r2 = dx * dx + dy * dy + dz * dz;
                        const bool near = r2 < n2;
                        if (!near) {
                            const float rinv = rsqrtf(r2);
                            const float r3 = rinv * rinv * rinv;
                            if (kMode == 0) {
                                a[0] += q.w * (dx * nn[0] + dy * nn[1] + dz * nn[2]) * r3;
                            } else {
                                a[0] += q.w * rinv;
                                const float wr3 = q.w * r3;
                                a[1] -= wr3 * dx;
                                a[2] -= wr3 * dy;
                                a[3] -= wr3 * dz;
                            }
                        }
                        if (__any_sync(0xffffffffu, near && active)) {
                            if (near && active && !(kMode == 0 && i == tgt)) {
                                const TriVerts tri = load_tri(s, i);
                                float P, G[3];
                                triangle_potential(xd, tri, P, G);
                                const float sg = __ldg(sigma + i);
                                if (kMode == 0) {
                                    a[0] -= sg * (G[0] * nn[0] + G[1] * nn[1] + G[2] * nn[2]);
                                } else {
                                    a[0] += sg * P;
                                    a[1] += sg * G[0];
                                    a[2] += sg * G[1];
                                    a[3] += sg * G[2];
                                }
                            }
                        }
                    }
                }
                flush();
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 4; c++) s_acc[wid][c][lane] = acc[c] + a[c];
    __syncthreads();
    if (wid != 0 || !active) return;
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (int w = 0; w < kCvWarps; w++)
#pragma unroll
        for (int c = 0; c < 4; c++) t[c] += s_acc[w][c][lane];
    if (gridDim.y > 1) {
        double *ps = part_sums + ((size_t)blockIdx.y * n_targets + slot) * 4;
        for (int k = 0; k < 4; k++) ps[k] = t[k];
    } else if (kMode == 0) {
        const double c = (double)c_coef;
        const double Tsig = c * kInv4Pi * t[0];
        out[tgt] = (float)((Tsig - (double)__ldg(sigma + tgt)) / c);
    } else {
        for (int k = 0; k < 4; k++) out[(size_t)tgt * 4 + k] = (float)(kInv4Pi * t[k]);
    }
}

// The potential from its parts, added in part order (deterministic): part_sums [parts][slot][4]
// by Morton slot, out [n][4] by point.
__global__ void cv_parts_kernel(const double *__restrict__ part_sums, uint32_t parts, const uint64_t *__restrict__ order,
                                uint32_t n, float *__restrict__ out) {
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= n) return;
    const uint32_t tgt = (uint32_t)__ldg(order + slot);
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (uint32_t p = 0; p < parts; p++)
#pragma unroll
        for (int k = 0; k < 4; k++) t[k] += part_sums[((size_t)p * n + slot) * 4 + k];
#pragma unroll
    for (int k = 0; k < 4; k++) out[(size_t)tgt * 4 + k] = (float)(kInv4Pi * t[k]);
}

// Blocks of the same 32 points the potential's largest groups are split over: with one block per
// 32 points there are too few blocks to fill the GPU for the slice-sized point sets.
constexpr uint32_t kPotentialParts = 8;

// The network's input at every stored element: (centroid, normal), 2D padded with zeros.
template <int D>
__global__ void element_frames_kernel(SceneView<D> s, float *__restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n_elems) return;
    const float4 *p = s.elems + 4 * i;
    float *o = out + (size_t)i * 6;
    if constexpr (D == 2) {
        const float4 q0 = __ldg(p), q1 = __ldg(p + 1);
        o[0] = (q0.x + q0.z) / 2.0f; o[1] = (q0.y + q0.w) / 2.0f; o[2] = 0.0f;
        o[3] = q1.x; o[4] = q1.y; o[5] = 0.0f;
    } else {
        const TriVerts t = load_tri(s, i);
        float c[3];
        centroid_of(t, c);
        const float4 q2 = __ldg(p + 2);
        o[0] = c[0]; o[1] = c[1]; o[2] = c[2];
        o[3] = q2.y; o[4] = q2.z; o[5] = q2.w;
    }
}

// Record i's vertex boundary values (record floats [first, first + dim)) plus delta[i]: the same
// single-precision add as the host copy's update, so the two copies stay identical.
__global__ void add_boundary_offsets_kernel(float *__restrict__ elems, const float *__restrict__ delta, uint32_t n,
                                            uint32_t record_floats, uint32_t first, uint32_t dim) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float d = delta[i];
    float *r = elems + (size_t)i * record_floats + first;
    for (uint32_t k = 0; k < dim; k++) r[k] = r[k] + d;
}

}  // namespace

cudaError_t launch_add_boundary_offsets(float *elems, const float *delta, uint32_t n, uint32_t record_floats,
                                        uint32_t first, uint32_t dim, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    add_boundary_offsets_kernel<<<(n + 255) / 256, 256, 0, stream>>>(elems, delta, n, record_floats, first, dim);
    return cudaGetLastError();
}

template <int D> cudaError_t launch_element_frames(const SceneView<D> &s, float *out, cudaStream_t stream) {
    element_frames_kernel<D><<<(s.n_elems + 255) / 256, 256, 0, stream>>>(s, out);
    return cudaGetLastError();
}
template cudaError_t launch_element_frames<2>(const SceneView<2> &, float *, cudaStream_t);
template cudaError_t launch_element_frames<3>(const SceneView<3> &, float *, cudaStream_t);

cudaError_t launch_cv_sources(const SceneView<3> &s, const float *sigma, float near_factor, float theta, float4 *src,
                              float *near2, float4 *clusters, cudaStream_t stream) {
    cv_sources_kernel<<<(s.n_elems + 255) / 256, 256, 0, stream>>>(s, sigma, near_factor, src, near2);
    const uint32_t n_cl = div_up(s.n_elems, kClusterSize), n_g1 = div_up(n_cl, kGroupFan), n_g2 = div_up(n_g1, kGroupFan);
    cv_cluster_kernel<<<(n_cl * 32 + 255) / 256, 256, 0, stream>>>(s.n_elems, src, near2, theta, clusters);
    cv_group_kernel<kClusterSize * kGroupFan><<<n_g1, kGroupBlock, 0, stream>>>(s.n_elems, src, near2, theta,
                                                                               clusters + 4 * (size_t)n_cl);
    cv_group_kernel<kClusterSize * kGroupFan * kGroupFan><<<n_g2, kGroupBlock, 0, stream>>>(
        s.n_elems, src, near2, theta, clusters + 4 * (size_t)(n_cl + n_g1));
    return cudaGetLastError();
}

uint32_t cv_cluster_records(uint32_t n_elems) {
    const uint32_t n_cl = div_up(n_elems, kClusterSize), n_g1 = div_up(n_cl, kGroupFan);
    return n_cl + n_g1 + div_up(n_g1, kGroupFan);
}

cudaError_t launch_cv_residual(const SceneView<3> &s, const float4 *src, const float *near2, const float4 *clusters,
                               const float *sigma, float c_coef, float *delta, cudaStream_t stream) {
    cv_sum_kernel<0><<<(s.n_elems + 31) / 32, kCvBlock, 0, stream>>>(s, src, near2, sigma, clusters, nullptr, nullptr,
                                                                     s.n_elems, c_coef, delta, nullptr);
    return cudaGetLastError();
}

uint32_t cv_point_order_words(uint32_t n_points) {
    uint32_t n2 = 1;
    while (n2 < n_points) n2 <<= 1;
    // n2 keys of 8 bytes, the 6 bound words (padded to 8), the parts' FP64 sums
    return 2 * n2 + 8 + kPotentialParts * n_points * 8;
}

cudaError_t launch_cv_potential(const SceneView<3> &s, const float4 *src, const float *near2, const float4 *clusters,
                                const float *sigma, const float *pts, uint32_t n_points, uint32_t *scratch,
                                float *out, cudaStream_t stream) {
    if (n_points == 0) return cudaSuccess;
    uint32_t n2 = 1;
    while (n2 < n_points) n2 <<= 1;
    uint64_t *key = (uint64_t *)scratch;
    uint32_t *bb = scratch + 2 * (size_t)n2;
    bounds_init_kernel<<<1, 32, 0, stream>>>(bb);
    pts_bounds_kernel<<<(n_points + 255) / 256, 256, 0, stream>>>(pts, n_points, bb);
    pts_morton_kernel<<<(n2 + 255) / 256, 256, 0, stream>>>(pts, n_points, n2, bb, key);
    for (uint32_t k = 2; k <= n2; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1) bitonic_kernel<<<(n2 + 255) / 256, 256, 0, stream>>>(n2, j, k, key);
    double *part_sums = reinterpret_cast<double *>(scratch + 2 * (size_t)n2 + 8);
    cv_sum_kernel<1><<<dim3((n_points + 31) / 32, kPotentialParts), kCvBlock, 0, stream>>>(
        s, src, near2, sigma, clusters, pts, key, n_points, 0.0f, out, part_sums);
    cv_parts_kernel<<<(n_points + 255) / 256, 256, 0, stream>>>(part_sums, kPotentialParts, key, n_points, out);
    return cudaGetLastError();
}

}  // namespace wobgb
