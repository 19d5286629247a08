// Virtual-point-light (VPL) variant of the walk (apps/potential_flow_with_vpl.cu:43-88):
//
// 1. paths (PathComputeFunc, :77-88): path i starts at a uniform boundary sample y_i and its walk
//    returns the unknown boundary estimate mu_i (compute_sample_unknown_boundary) -- one thread per
//    path, Philox stream kStreamVpl, point 0, path index path_offset + i;
// 2. aggregation (AggregateFunc, :43-75): every evaluation point x sums, over all VPLs,
//    mu_i * G(y_i, x) * A and mu_i * dG/dx(y_i, x) * A (the single layer's solution_domain_unknown /
//    gradient_domain_unknown, A = total boundary area) -- an N_points x N_vpl dense sum of kernel
//    evaluations, FP32-issue bound. Partial sums are FP32 per tile of 256 VPLs; tile t goes to
//    split t mod 8, each split adds its tiles in order into FP64, and the 8 split sums of a point
//    are added in split order (the oracle does the same blocking, so the sums are bit-identical).
#include "kernels.cuh"
#include "vpl.hpp"

namespace wobgb {

namespace {

constexpr uint32_t kStreamVpl = 2u;
constexpr int kVplTile = 256;

template <int D>
__global__ void __launch_bounds__(kBlock) vpl_paths_kernel(SceneView<D> s, WalkParams p, uint32_t n_paths,
                                                           float *__restrict__ vpl_p, float *__restrict__ vpl_mu,
                                                           unsigned long long *__restrict__ bounces) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long b = 0;
    if (i < n_paths) {
        Walker<D, kSingleLayer, kStratSingleLayer, false> w(s, p, kStreamVpl, 0u, p.path_offset + i);
        float ip;
        const BPoint<D> y = sample_uniform<D>(s, w.rng, ip);
        const float mu = w.unknown_boundary(y);
        for (int k = 0; k < D; k++) vpl_p[(size_t)i * D + k] = y.p.v[k];
        vpl_mu[i] = mu;
        b = w.bounces;
    }
    if (bounces) {
        const unsigned long long t = warp_sum_u64(b);
        if ((threadIdx.x & 31u) == 0 && t) atomicAdd(bounces, t);
    }
}

// One block serves 32 points with 8 warps; warp w sums the tiles t = w, w + 8, ... (all lanes read
// the same VPL at a time: one shared-memory broadcast), so 8 threads share a point's pairs and the
// grid fills the GPU even for a few ten thousand points. The 8 per-warp FP64 partial sums of a
// point are then added in warp order.
//
// A pair (point x, VPL y with value mu) adds mu G(y, x) A and mu dG/dx(y, x) A = mu w (y - x), with
// r = y - x, q = |r|^2 (equation_kernel.cuh:74-79, 115-121), in this form (the oracle restates it):
//   2D: mu G A = ku log(max(q, eps^2)), ku = mu (-A / (4 pi)) -- log(max(|r|, eps)) / (2 pi)
//       written as log(max(q, eps^2)) / (4 pi); mu w = kw / q for q >= eps^2, kw / (|r| eps) for
//       0 < q < eps^2, 0 at q = 0, kw = mu A / (2 pi);
//   3D: mu G A = ku / max(|r|, eps), mu w = ku / (|r| max(q, eps)) (0 at q = 0), ku = mu A / (4 pi).
// ku and kw are computed once per VPL when its tile is staged in shared memory ({y, ku, kw} in 2D,
// {y, ku} in 3D), so a pair costs one log or one more division and no per-pair scaling.
constexpr int kVplSplit = 8;

template <int D>
__global__ void __launch_bounds__(32 * kVplSplit) vpl_aggregate_kernel(const float *__restrict__ vpl_p,
                                                                       const float *__restrict__ vpl_mu, uint32_t n_vpl,
                                                                       float area, float eps,
                                                                       const float *__restrict__ pts, uint32_t n_points,
                                                                       double *__restrict__ sum) {
    __shared__ float4 tile[kVplSplit][kVplTile];
    __shared__ double red[kVplSplit][32][D + 1];
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    const uint32_t pt = blockIdx.x * 32u + lane;
    const bool active = pt < n_points;
    V<D> x = vzero<D>();
    if (active)
        for (int k = 0; k < D; k++) x.v[k] = __ldg(pts + (size_t)pt * D + k);
    const float cu = D == 2 ? -0x1.45f306p-4f * area : 0x1.45f306p-4f * area;  // -A/(4 pi) or A/(4 pi)
    const float cw = 0x1.45f306p-3f * area;                                      // A/(2 pi)
    const float eps2 = eps * eps;
    double acc[D + 1];
    for (int c = 0; c <= D; c++) acc[c] = 0.0;
    const uint32_t n_tiles = (n_vpl + kVplTile - 1) / kVplTile;
    for (uint32_t t = w; t < n_tiles; t += kVplSplit) {
        const uint32_t t0 = t * kVplTile;
        const uint32_t m = min((uint32_t)kVplTile, n_vpl - t0);
        __syncwarp();
        for (uint32_t j = lane; j < m; j += 32) {
            const float mu = __ldg(vpl_mu + t0 + j);
            float4 e;
            e.x = __ldg(vpl_p + (size_t)(t0 + j) * D);
            e.y = __ldg(vpl_p + (size_t)(t0 + j) * D + 1);
            if constexpr (D == 2) {
                e.z = mu * cu;
                e.w = mu * cw;
            } else {
                e.z = __ldg(vpl_p + (size_t)(t0 + j) * D + 2);
                e.w = mu * cu;
            }
            tile[w][j] = e;
        }
        __syncwarp();
        float part[D + 1];
        for (int c = 0; c <= D; c++) part[c] = 0.0f;
        for (uint32_t j = 0; j < m; j++) {
            const float4 e = tile[w][j];
            V<D> r;
            r.v[0] = e.x - x.v[0];
            r.v[1] = e.y - x.v[1];
            if constexpr (D == 3) r.v[2] = e.z - x.v[2];
            const float q = vsqnorm(r);
            float g;
            if constexpr (D == 2) {
                part[0] = part[0] + e.z * log_own(fmax_ref(q, eps2));
                g = q >= eps2 ? e.w / q : (q > 0.0f ? e.w / (sqrtf(q) * eps) : 0.0f);
            } else {
                const float n = sqrtf(q);
                part[0] = part[0] + e.w / fmax_ref(n, eps);
                g = q > 0.0f ? e.w / (n * fmax_ref(q, eps)) : 0.0f;
            }
            for (int k = 0; k < D; k++) part[1 + k] = part[1 + k] + g * r.v[k];
        }
        for (int c = 0; c <= D; c++) acc[c] += (double)part[c];
    }
    for (int c = 0; c <= D; c++) red[w][lane][c] = acc[c];
    __syncthreads();
    if (w == 0 && active) {
        for (int c = 0; c <= D; c++) {
            double total = red[0][lane][c];
            for (int k = 1; k < kVplSplit; k++) total = total + red[k][lane][c];
            sum[(size_t)pt * (D + 1) + c] += total;
        }
    }
}

template <int D>
cudaError_t paths_impl(const SceneView<D> &s, const WalkParams &p, uint32_t n_paths, float *vpl_p, float *vpl_mu,
                       unsigned long long *bounces, cudaStream_t st) {
    if (n_paths == 0) return cudaSuccess;
    vpl_paths_kernel<D><<<(n_paths + kBlock - 1) / kBlock, kBlock, 0, st>>>(s, p, n_paths, vpl_p, vpl_mu, bounces);
    return cudaGetLastError();
}

template <int D>
cudaError_t aggregate_impl(const float *vpl_p, const float *vpl_mu, uint32_t n_vpl, float area, float eps,
                           const float *pts, uint32_t n_points, double *sum, cudaStream_t st) {
    if (n_points == 0) return cudaSuccess;
    vpl_aggregate_kernel<D><<<(n_points + 31) / 32, 32 * kVplSplit, 0, st>>>(vpl_p, vpl_mu, n_vpl, area, eps, pts,
                                                                            n_points, sum);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_vpl_paths_2d(const SceneView<2> &s, const WalkParams &p, uint32_t n_paths, float *vpl_p,
                                float *vpl_mu, unsigned long long *bounces, cudaStream_t st) {
    return paths_impl<2>(s, p, n_paths, vpl_p, vpl_mu, bounces, st);
}
cudaError_t launch_vpl_paths_3d(const SceneView<3> &s, const WalkParams &p, uint32_t n_paths, float *vpl_p,
                                float *vpl_mu, unsigned long long *bounces, cudaStream_t st) {
    return paths_impl<3>(s, p, n_paths, vpl_p, vpl_mu, bounces, st);
}
cudaError_t launch_vpl_aggregate(int dim, const float *vpl_p, const float *vpl_mu, uint32_t n_vpl, float area,
                                 float eps, const float *pts, uint32_t n_points, double *sum, cudaStream_t st) {
    return dim == 2 ? aggregate_impl<2>(vpl_p, vpl_mu, n_vpl, area, eps, pts, n_points, sum, st)
                    : aggregate_impl<3>(vpl_p, vpl_mu, n_vpl, area, eps, pts, n_points, sum, st);
}

}  // namespace wobgb
