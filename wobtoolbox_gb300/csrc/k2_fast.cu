// 2D specialisations: double-layer Dirichlet with line-intersection sampling; direct Neumann.
#include "kernels.cuh"

namespace wobgb {
template cudaError_t launch_domain_variant<2, kDoubleLayer, kStratLineIntersection, false, 1>(const SceneView<2> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_domain_variant<2, kDoubleLayer, kStratLineIntersection, false, 6>(const SceneView<2> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_domain_variant<2, kDoubleLayer, kStratLineIntersection, false, 5>(const SceneView<2> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_domain_variant<2, kDoubleLayer, kStratLineIntersection, false, 8>(const SceneView<2> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_domain_variant<2, kDirect, kStratDirectNeumann, false>(const SceneView<2> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
}  // namespace wobgb
