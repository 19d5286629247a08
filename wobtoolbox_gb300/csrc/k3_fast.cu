// 3D specialisations: direct BIE with two uniform samples per bounce (Dirichlet / Robin / mixed
// data without a Neumann-only problem); direct Neumann with line-intersection sampling.
#include "kernels.cuh"

namespace wobgb {
template cudaError_t launch_domain_variant<3, kDirect, kStratUniform, false, 1>(const SceneView<3> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_domain_variant<3, kDirect, kStratUniform, false, 6>(const SceneView<3> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_domain_variant<3, kDirect, kStratUniform, false, 5>(const SceneView<3> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_domain_variant<3, kDirect, kStratUniform, false, 8>(const SceneView<3> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_domain_variant<3, kDirect, kStratDirectNeumann, false, 1>(const SceneView<3> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_domain_variant<3, kDirect, kStratDirectNeumann, false, 6>(const SceneView<3> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_domain_variant<3, kDirect, kStratDirectNeumann, false, 5>(const SceneView<3> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_domain_variant<3, kDirect, kStratDirectNeumann, false, 8>(const SceneView<3> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_boundary_variant<3, kDirect, kStratDirectNeumann, false>(const SceneView<3> &, const WalkParams &, const BoundaryInput &, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
}  // namespace wobgb
