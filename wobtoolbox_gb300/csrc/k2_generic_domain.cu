// 2D general domain walk (run-time BIE model and strategy) and the 2D line query.
#include "kernels.cuh"

namespace wobgb {
template cudaError_t launch_domain_variant<2, -1, kStratRuntime, true>(const SceneView<2> &, const WalkParams &, const float *, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
template cudaError_t launch_line_query_impl<2>(const SceneView<2> &, const float *, const float *, uint32_t, uint32_t *, uint32_t *, float *, cudaStream_t);
}  // namespace wobgb
