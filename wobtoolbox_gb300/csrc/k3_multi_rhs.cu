// Multi-RHS walks for 3D scenes (the kernels are in multi_rhs.cuh).
#include "multi_rhs.cuh"

namespace wobgb {

cudaError_t launch_multi_rhs_3d(const SceneView<3> &s, const WalkParams &p, const MultiRhsArgs &a) {
    return mrhs::launch_multi<3>(s, p, a);
}

}  // namespace wobgb
