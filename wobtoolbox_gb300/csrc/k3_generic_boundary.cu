// 3D general boundary walk (run-time BIE model and strategy).
#include "kernels.cuh"

namespace wobgb {
template cudaError_t launch_boundary_variant<3, -1, kStratRuntime, true>(const SceneView<3> &, const WalkParams &, const BoundaryInput &, uint32_t, double *, double *, unsigned long long *, float *, cudaStream_t);
}  // namespace wobgb
