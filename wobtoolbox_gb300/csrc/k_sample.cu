// Boundary points drawn uniformly by area on the device (the training points of the learned
// control variate): point i is Philox stream 2 of point index i, drawn exactly as the walk's
// uniform boundary sample (sample_uniform, scene.cuh:441-462 / 734-758), with its element's
// normal, the interior angle 1/2, the interpolated boundary value, type and Robin alpha.
#include "device_common.cuh"
#include "launch.hpp"

namespace wobgb {

namespace {

constexpr uint32_t kStreamTraining = 2u;

template <int D>
__global__ void sample_boundary_kernel(SceneView<D> s, uint32_t n, uint64_t seed, float *__restrict__ p,
                                       float *__restrict__ nrm, float *__restrict__ angle, float *__restrict__ bv,
                                       int32_t *__restrict__ type, float *__restrict__ alpha) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    PathRng rng(seed, kStreamTraining, i, 0ull);
    float ip;
    const BPoint<D> y = sample_uniform<D>(s, rng, ip);
#pragma unroll
    for (int k = 0; k < D; k++) {
        p[(size_t)i * D + k] = y.p.v[k];
        nrm[(size_t)i * D + k] = y.n.v[k];
    }
    angle[i] = y.angle;
    bv[i] = y.bv;
    type[i] = y.type;
    if (alpha) alpha[i] = y.alpha;
}

}  // namespace

template <int D>
cudaError_t launch_sample_boundary(const SceneView<D> &s, uint32_t n, uint64_t seed, float *p, float *nrm,
                                   float *angle, float *bv, int32_t *type, float *alpha, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    sample_boundary_kernel<D><<<(n + 255) / 256, 256, 0, stream>>>(s, n, seed, p, nrm, angle, bv, type, alpha);
    return cudaGetLastError();
}
template cudaError_t launch_sample_boundary<2>(const SceneView<2> &, uint32_t, uint64_t, float *, float *, float *,
                                               float *, int32_t *, float *, cudaStream_t);
template cudaError_t launch_sample_boundary<3>(const SceneView<3> &, uint32_t, uint64_t, float *, float *, float *,
                                               float *, int32_t *, float *, cudaStream_t);

}  // namespace wobgb
