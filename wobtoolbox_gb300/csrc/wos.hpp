// Walk on spheres and the closest-point query (k_wos.cu).
#pragma once

#include "launch.hpp"

namespace wobgb {

cudaError_t launch_wos_2d(const SceneView<2> &s, const WalkParams &p, const float *pts, uint32_t n_points, double *sum,
                          double *sumsq, unsigned long long *queries, float *per_path, cudaStream_t st);
cudaError_t launch_closest_point_2d(const SceneView<2> &s, const float *pts, uint32_t n, uint32_t *elem, float *dist2,
                                    float *value, cudaStream_t st);

}  // namespace wobgb
