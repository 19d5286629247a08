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

// One (point, VPL) pair: u = G(y, x) A and the factor w of dG/dx(y, x) A = w (y - x), from
// r = y - x, n = |r|, m = max(n, eps) (equation_kernel.cuh:74-79, 115-121):
//   2D: G = -log(m) / (2 pi),  dG/dx = r / (2 pi n m);   3D: G = 1 / (4 pi m),  dG/dx = r / (4 pi n max(n^2, eps)),
// the gradient with one division instead of normalising r and dividing by m (the engine's walk
// kernels evaluate Green<D>::dG_dx literally; the oracle restates this form for the aggregation).
// w = 0 at n = 0, where the normalised direction is the zero vector.
template <int D>
__device__ __forceinline__ void vpl_pair(const V<D> &y, const V<D> &x, float area, float eps, float &u, float &w) {
    const V<D> r = vsub(y, x);
    const float q = vsqnorm(r);
    const float n = sqrtf(q);
    const float m = fmax_ref(n, eps);
    if constexpr (D == 2) {
        u = (-0x1.45f306p-3f * log_own(m)) * area;
        w = n > 0.0f ? (0x1.45f306p-3f * area) / (n * m) : 0.0f;
    } else {
        u = (1.0f / (0x1.921fb6p+3f * m)) * area;
        w = n > 0.0f ? (0x1.45f306p-4f * area) / (n * fmax_ref(q, eps)) : 0.0f;
    }
}

// One block serves 32 points with 8 warps; warp w sums the tiles t = w, w + 8, ... (all lanes read
// the same VPL at a time: one broadcast load), so 8 threads share a point's pairs and the grid
// fills the GPU even for a few ten thousand points. The 8 per-warp FP64 partial sums of a point
// are then added in warp order.
constexpr int kVplSplit = 8;

template <int D>
__global__ void __launch_bounds__(32 * kVplSplit) vpl_aggregate_kernel(const float *__restrict__ vpl_p,
                                                                       const float *__restrict__ vpl_mu, uint32_t n_vpl,
                                                                       float area, float eps,
                                                                       const float *__restrict__ pts, uint32_t n_points,
                                                                       double *__restrict__ sum) {
    __shared__ double red[kVplSplit][32][D + 1];
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    const uint32_t pt = blockIdx.x * 32u + lane;
    const bool active = pt < n_points;
    V<D> x = vzero<D>();
    if (active)
        for (int k = 0; k < D; k++) x.v[k] = __ldg(pts + (size_t)pt * D + k);
    double acc[D + 1];
    for (int c = 0; c <= D; c++) acc[c] = 0.0;
    const uint32_t n_tiles = (n_vpl + kVplTile - 1) / kVplTile;
    for (uint32_t t = w; t < n_tiles; t += kVplSplit) {
        const uint32_t t0 = t * kVplTile;
        const uint32_t m = min((uint32_t)kVplTile, n_vpl - t0);
        float part[D + 1];
        for (int c = 0; c <= D; c++) part[c] = 0.0f;
        for (uint32_t j = 0; j < m; j++) {
            V<D> y;
            for (int k = 0; k < D; k++) y.v[k] = __ldg(vpl_p + (size_t)(t0 + j) * D + k);
            const float mu = __ldg(vpl_mu + t0 + j);
            float u, w;
            vpl_pair<D>(y, x, area, eps, u, w);
            part[0] = part[0] + mu * u;
            for (int k = 0; k < D; k++) part[1 + k] = part[1 + k] + mu * (w * (y.v[k] - x.v[k]));
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
