// Multi-RHS walks (k_multi_rhs.cu): launch entry points shared with the C ABI.
#pragma once

#include "launch.hpp"

namespace wobgb {

constexpr uint32_t kMaxRhs = 64;

// True when the estimator's sampling ignores the boundary data (backward single layer with uniform
// or RIS sampling, backward direct with uniform sampling) and there is no source term.
bool multi_rhs_supported(const WalkParams &p);

// unknown = false: domain estimate u(x) at pts[n_points][D];
// unknown = true: unknown boundary density at the boundary points of bin, whose data per RHS is
// rhs_input[n_points][n_rhs] (bin.bv is not read).
// rhs_table: [n_elems][D][n_rhs] floats in storage order. Outputs sum / sumsq [n_points][n_rhs]
// (FP64, accumulated), per_path [n_points][n_paths][n_rhs] floats (optional).
cudaError_t launch_multi_rhs_2d(const SceneView<2> &s, const WalkParams &p, bool unknown, const float *pts,
                                const BoundaryInput &bin, const float *rhs_table, const float *rhs_input,
                                uint32_t n_rhs, uint32_t n_points, double *sum, double *sumsq,
                                unsigned long long *bounces, float *per_path, cudaStream_t stream);
cudaError_t launch_multi_rhs_3d(const SceneView<3> &s, const WalkParams &p, bool unknown, const float *pts,
                                const BoundaryInput &bin, const float *rhs_table, const float *rhs_input,
                                uint32_t n_rhs, uint32_t n_points, double *sum, double *sumsq,
                                unsigned long long *bounces, float *per_path, cudaStream_t stream);

}  // namespace wobgb
