// Single-layer specialisations without a source term: the backward estimator (uniform or RIS
// sampling, estimator.cuh:276-334) and the forward Neumann estimator (line intersection,
// estimator.cuh:423-451), in 2D and 3D, compiled for at least 5 resident blocks per SM.
#include "kernels.cuh"

namespace wobgb {
template cudaError_t launch_domain_variant<2, kSingleLayer, kStratSingleLayer, false, 5>(const SceneView<2> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_domain_variant<3, kSingleLayer, kStratSingleLayer, false, 5>(const SceneView<3> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_domain_variant<2, kSingleLayer, kStratFwdSlNeumann, false, 5>(const SceneView<2> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_domain_variant<3, kSingleLayer, kStratFwdSlNeumann, false, 5>(const SceneView<3> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
}  // namespace wobgb
