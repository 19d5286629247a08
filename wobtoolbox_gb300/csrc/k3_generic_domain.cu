// 3D general domain walk (run-time BIE model and strategy) and the 3D line query.
#include "kernels.cuh"

namespace wobgb {
template cudaError_t launch_domain_variant<3, -1, kStratRuntime, true>(const SceneView<3> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_line_query_impl<3>(const SceneView<3> &, const float *, const float *, uint32_t, uint32_t *, uint32_t *, float *, cudaStream_t);
}  // namespace wobgb
