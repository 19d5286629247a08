// Routes a solve to the specialised kernel variant for its parameters, or to the general one.
// Variants are instantiated in k2_*.cu / k3_*.cu; every variant is compiled from the same walk
// source (walk_generic.cuh), only with some parameters fixed at compile time.
#include "launch.hpp"
#include "walk_generic.cuh"

namespace wobgb {

cudaError_t launch_domain_2d(const SceneView<2> &s, const WalkParams &p, const float *pts, uint32_t n_points,
                             double *sum, double *sumsq, unsigned long long *bounces, float *per_path,
                             cudaStream_t stream) {
    const int st = strategy_of(p.bie, p.estimator, p.problem);
    if (p.n_volume == 0 && st == kStratLineIntersection)
        return launch_domain_variant<2, kDoubleLayer, kStratLineIntersection, false>(s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
    if (p.n_volume == 0 && st == kStratDirectNeumann)
        return launch_domain_variant<2, kDirect, kStratDirectNeumann, false>(s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
    return launch_domain_variant<2, -1, kStratRuntime, true>(s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
}

cudaError_t launch_domain_3d(const SceneView<3> &s, const WalkParams &p, const float *pts, uint32_t n_points,
                             double *sum, double *sumsq, unsigned long long *bounces, float *per_path,
                             cudaStream_t stream) {
    const int st = strategy_of(p.bie, p.estimator, p.problem);
    if (p.n_volume == 0 && st == kStratUniform && p.bie == kDirect)
        return launch_domain_variant<3, kDirect, kStratUniform, false>(s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
    if (p.n_volume == 0 && st == kStratDirectNeumann)
        return launch_domain_variant<3, kDirect, kStratDirectNeumann, false>(s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
    return launch_domain_variant<3, -1, kStratRuntime, true>(s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
}

cudaError_t launch_boundary_2d(const SceneView<2> &s, const WalkParams &p, const BoundaryInput &bin,
                               uint32_t n_points, double *sum, double *sumsq, unsigned long long *bounces,
                               float *per_path, cudaStream_t stream) {
    return launch_boundary_variant<2, -1, kStratRuntime, true>(s, p, bin, n_points, sum, sumsq, bounces, per_path, stream);
}

cudaError_t launch_boundary_3d(const SceneView<3> &s, const WalkParams &p, const BoundaryInput &bin,
                               uint32_t n_points, double *sum, double *sumsq, unsigned long long *bounces,
                               float *per_path, cudaStream_t stream) {
    const int st = strategy_of(p.bie, p.estimator, p.problem);
    if (p.n_volume == 0 && st == kStratDirectNeumann)
        return launch_boundary_variant<3, kDirect, kStratDirectNeumann, false>(s, p, bin, n_points, sum, sumsq, bounces, per_path, stream);
    return launch_boundary_variant<3, -1, kStratRuntime, true>(s, p, bin, n_points, sum, sumsq, bounces, per_path, stream);
}

cudaError_t launch_line_query_2d(const SceneView<2> &s, const float *origins, const float *dirs, uint32_t n,
                                 uint32_t *counts, uint32_t *hits, float *points, cudaStream_t stream) {
    return launch_line_query_impl<2>(s, origins, dirs, n, counts, hits, points, stream);
}
cudaError_t launch_line_query_3d(const SceneView<3> &s, const float *origins, const float *dirs, uint32_t n,
                                 uint32_t *counts, uint32_t *hits, float *points, cudaStream_t stream) {
    return launch_line_query_impl<3>(s, origins, dirs, n, counts, hits, points, stream);
}

}  // namespace wobgb
