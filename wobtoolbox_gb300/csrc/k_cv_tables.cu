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
// Work decomposition: two targets per thread (one where two would leave SMs idle), 256 threads per
// block; the sources stream through shared memory in tiles of 256 {centroid, sigma~ A, near
// radius^2}, read as broadcasts. Far pairs
// cost one rsqrt and a dozen FMAs; a warp in which any lane has a near pair takes the closed form
// for those lanes (the targets of a warp and the sources of a tile are both consecutive in BVH
// storage order, so near pairs come in spatial clusters). FP32 partial sums per tile, FP64 across
// tiles. This unit is compiled with FMA contraction (it is not part of the bit-exact walk).
#include "device_common.cuh"
#include "launch.hpp"

namespace wobgb {

namespace {

constexpr int kCvBlock = 256;
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

// kMode 0: residual data at the stored triangles' centroids; kMode 1: potential and gradient at
// points (out: [n][4] = u, du/dx, du/dy, du/dz). Each thread takes kTgt targets (a block covers
// kTgt x 256), so every source read from shared memory serves kTgt pairs; one target per thread
// where two would leave SMs without a block.
template <int kMode, int kTgt>
__global__ void __launch_bounds__(kCvBlock) cv_sum_kernel(SceneView<3> s, const float4 *__restrict__ src,
                                                          const float *__restrict__ near2,
                                                          const float *__restrict__ sigma,
                                                          const float *__restrict__ pts, uint32_t n_targets,
                                                          float c_coef, float *__restrict__ out) {
    __shared__ float4 s_src[kCvBlock];
    __shared__ float s_n2[kCvBlock];
    uint32_t tgt[kTgt];
    bool active[kTgt];
    float xd[kTgt][3], nn[kTgt][3];
    for (int t = 0; t < kTgt; t++) {
        tgt[t] = blockIdx.x * (kCvBlock * kTgt) + t * kCvBlock + threadIdx.x;
        active[t] = tgt[t] < n_targets;
        for (int k = 0; k < 3; k++) xd[t][k] = nn[t][k] = 0.0f;
        if (active[t]) {
            if (kMode == 0) {
                const TriVerts tv = load_tri(s, tgt[t]);
                centroid_of(tv, xd[t]);
                const float4 q2 = __ldg(s.elems + 4 * tgt[t] + 2);
                nn[t][0] = q2.y; nn[t][1] = q2.z; nn[t][2] = q2.w;
            } else {
                for (int k = 0; k < 3; k++) xd[t][k] = pts[(size_t)tgt[t] * 3 + k];
            }
        }
    }
    double acc[kTgt][4];
    for (int t = 0; t < kTgt; t++)
        for (int c = 0; c < 4; c++) acc[t][c] = 0.0;
    const uint32_t n_src = s.n_elems;
    for (uint32_t t0 = 0; t0 < n_src; t0 += kCvBlock) {
        __syncthreads();
        const uint32_t li = t0 + threadIdx.x;
        if (li < n_src) {
            s_src[threadIdx.x] = __ldg(src + li);
            s_n2[threadIdx.x] = __ldg(near2 + li);
        }
        __syncthreads();
        const uint32_t cnt = min((uint32_t)kCvBlock, n_src - t0);
        float a[kTgt][4];
#pragma unroll
        for (int t = 0; t < kTgt; t++)
#pragma unroll
            for (int c = 0; c < 4; c++) a[t][c] = 0.0f;
        for (uint32_t k = 0; k < cnt; k++) {
            const float4 q = s_src[k];
            const float n2 = s_n2[k];
            bool near[kTgt];
            bool any_near = false;
#pragma unroll
            for (int t = 0; t < kTgt; t++) {
                const float dx = xd[t][0] - q.x, dy = xd[t][1] - q.y, dz = xd[t][2] - q.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                near[t] = r2 < n2;
                any_near |= near[t] && active[t];
                if (!near[t]) {
                    const float rinv = rsqrtf(r2);
                    const float r3 = rinv * rinv * rinv;
                    if (kMode == 0) {
                        a[t][0] += q.w * (dx * nn[t][0] + dy * nn[t][1] + dz * nn[t][2]) * r3;
                    } else {
                        a[t][0] += q.w * rinv;
                        const float wr3 = q.w * r3;
                        a[t][1] -= wr3 * dx;
                        a[t][2] -= wr3 * dy;
                        a[t][3] -= wr3 * dz;
                    }
                }
            }
            if (__any_sync(0xffffffffu, any_near)) {
                const uint32_t i = t0 + k;
#pragma unroll
                for (int t = 0; t < kTgt; t++) {
                    if (near[t] && active[t] && !(kMode == 0 && i == tgt[t])) {
                        const TriVerts tri = load_tri(s, i);
                        float P, G[3];
                        triangle_potential(xd[t], tri, P, G);
                        const float sg = __ldg(sigma + i);
                        if (kMode == 0) {
                            a[t][0] -= sg * (G[0] * nn[t][0] + G[1] * nn[t][1] + G[2] * nn[t][2]);
                        } else {
                            a[t][0] += sg * P;
                            a[t][1] += sg * G[0];
                            a[t][2] += sg * G[1];
                            a[t][3] += sg * G[2];
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int t = 0; t < kTgt; t++)
#pragma unroll
            for (int c = 0; c < 4; c++) acc[t][c] += a[t][c];
    }
    for (int t = 0; t < kTgt; t++) {
        if (!active[t]) continue;
        if (kMode == 0) {
            const double c = (double)c_coef;
            const double Tsig = c * kInv4Pi * acc[t][0];
            out[tgt[t]] = (float)((Tsig - (double)__ldg(sigma + tgt[t])) / c);
        } else {
            for (int k = 0; k < 4; k++) out[(size_t)tgt[t] * 4 + k] = (float)(kInv4Pi * acc[t][k]);
        }
    }
}

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

template <int kMode>
void launch_sum(const SceneView<3> &s, const float4 *src, const float *near2, const float *sigma, const float *pts,
                uint32_t n, float c_coef, float *out, cudaStream_t stream) {
    int sms = 152;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t two = (n + 2 * kCvBlock - 1) / (2 * kCvBlock);
    if (two >= 2u * (uint32_t)sms) {
        cv_sum_kernel<kMode, 2><<<two, kCvBlock, 0, stream>>>(s, src, near2, sigma, pts, n, c_coef, out);
    } else {
        cv_sum_kernel<kMode, 1><<<(n + kCvBlock - 1) / kCvBlock, kCvBlock, 0, stream>>>(s, src, near2, sigma, pts, n,
                                                                                       c_coef, out);
    }
}

}  // namespace

template <int D> cudaError_t launch_element_frames(const SceneView<D> &s, float *out, cudaStream_t stream) {
    element_frames_kernel<D><<<(s.n_elems + 255) / 256, 256, 0, stream>>>(s, out);
    return cudaGetLastError();
}
template cudaError_t launch_element_frames<2>(const SceneView<2> &, float *, cudaStream_t);
template cudaError_t launch_element_frames<3>(const SceneView<3> &, float *, cudaStream_t);

cudaError_t launch_cv_sources(const SceneView<3> &s, const float *sigma, float near_factor, float4 *src, float *near2,
                              cudaStream_t stream) {
    cv_sources_kernel<<<(s.n_elems + 255) / 256, 256, 0, stream>>>(s, sigma, near_factor, src, near2);
    return cudaGetLastError();
}

cudaError_t launch_cv_residual(const SceneView<3> &s, const float4 *src, const float *near2, const float *sigma,
                               float c_coef, float *delta, cudaStream_t stream) {
    launch_sum<0>(s, src, near2, sigma, nullptr, s.n_elems, c_coef, delta, stream);
    return cudaGetLastError();
}

cudaError_t launch_cv_potential(const SceneView<3> &s, const float4 *src, const float *near2, const float *sigma,
                                const float *pts, uint32_t n_points, float *out, cudaStream_t stream) {
    if (n_points == 0) return cudaSuccess;
    launch_sum<1>(s, src, near2, sigma, pts, n_points, 0.0f, out, stream);
    return cudaGetLastError();
}

}  // namespace wobgb
