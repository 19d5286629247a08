// 3D instantiations of the general walk kernels (see kernels.cuh).
#include "kernels.cuh"

namespace wobgb {

cudaError_t launch_domain_3d(const SceneView<3> &s, const WalkParams &p, const float *pts, uint32_t n_points,
                             double *sum, double *sumsq, unsigned long long *bounces, float *per_path,
                             cudaStream_t stream) {
    return launch_domain_impl<3>(s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
}
cudaError_t launch_boundary_3d(const SceneView<3> &s, const WalkParams &p, const BoundaryInput &bin,
                               uint32_t n_points, double *sum, double *sumsq, unsigned long long *bounces,
                               float *per_path, cudaStream_t stream) {
    return launch_boundary_impl<3>(s, p, bin, n_points, sum, sumsq, bounces, per_path, stream);
}
cudaError_t launch_line_query_3d(const SceneView<3> &s, const float *origins, const float *dirs, uint32_t n,
                                 uint32_t *counts, uint32_t *hits, float *points, cudaStream_t stream) {
    return launch_line_query_impl<3>(s, origins, dirs, n, counts, hits, points, stream);
}

}  // namespace wobgb
