// Multi-RHS walks (k_multi_rhs.cu): launch entry points shared with the C ABI.
#pragma once

#include "launch.hpp"

namespace wobgb {

constexpr uint32_t kMaxRhs = 64;

// True when the estimator's sampling ignores the boundary data (backward single layer with uniform
// or RIS sampling, backward direct with uniform sampling) and there is no source term.
bool multi_rhs_supported(const WalkParams &p);

// One multi-RHS launch. unknown = false: domain estimate u(x) at points[n_points][D] (with the
// control variate cv_table [n_elems][n_rhs] and n_potential samples when cv_table is set);
// unknown = true: unknown boundary function at the boundary points of bin, whose data per RHS is
// rhs_input[n_points][n_rhs] (bin.bv is not read).
// rhs_table: [n_elems][D][n_rhs] floats in storage order. Outputs sum / sumsq [n_points][n_rhs]
// (FP64, accumulated), per_path [n_points][n_paths][n_rhs] floats (optional).
struct MultiRhsArgs {
    bool unknown;
    const float *points;
    BoundaryInput bin;
    const float *rhs_table, *rhs_input, *cv_table;
    uint32_t n_rhs, n_potential, n_points;
    double *sum, *sumsq;
    unsigned long long *bounces;
    float *per_path;
    cudaStream_t stream;
};
cudaError_t launch_multi_rhs_2d(const SceneView<2> &s, const WalkParams &p, const MultiRhsArgs &a);
cudaError_t launch_multi_rhs_3d(const SceneView<3> &s, const WalkParams &p, const MultiRhsArgs &a);

}  // namespace wobgb
