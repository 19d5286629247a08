// Control-variate domain estimator (forward single layer, Neumann) for 2D and 3D scenes.
#include "kernels.cuh"

namespace wobgb {

cudaError_t launch_domain_cv_2d(const SceneView<2> &s, const WalkParams &p, const float *pts, uint32_t n_points,
                                double *sum, double *sumsq, unsigned long long *bounces, float *per_path,
                                cudaStream_t stream) {
    return launch_domain_cv_impl<2>(s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
}
cudaError_t launch_domain_cv_3d(const SceneView<3> &s, const WalkParams &p, const float *pts, uint32_t n_points,
                                double *sum, double *sumsq, unsigned long long *bounces, float *per_path,
                                cudaStream_t stream) {
    return launch_domain_cv_impl<3>(s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
}

}  // namespace wobgb
