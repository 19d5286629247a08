// Virtual-point-light walks and their aggregation (k_vpl.cu).
#pragma once

#include "launch.hpp"

namespace wobgb {

// Single-layer backward walks from uniform boundary samples: vpl_p [n_paths][D], vpl_mu [n_paths].
cudaError_t launch_vpl_paths_2d(const SceneView<2> &s, const WalkParams &p, uint32_t n_paths, float *vpl_p,
                                float *vpl_mu, unsigned long long *bounces, cudaStream_t st);
cudaError_t launch_vpl_paths_3d(const SceneView<3> &s, const WalkParams &p, uint32_t n_paths, float *vpl_p,
                                float *vpl_mu, unsigned long long *bounces, cudaStream_t st);
// sum[pt][0..D] += sum_i mu_i * (G(y_i, x) A, dG/dx(y_i, x) A), FP32 per tile of 256 VPLs, FP64 across.
cudaError_t launch_vpl_aggregate(int dim, const float *vpl_p, const float *vpl_mu, uint32_t n_vpl, float area,
                                 float eps, const float *pts, uint32_t n_points, double *sum, cudaStream_t st);

}  // namespace wobgb
