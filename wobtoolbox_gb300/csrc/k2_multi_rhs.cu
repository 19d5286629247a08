// Multi-RHS walks for 2D scenes (the kernels are in multi_rhs.cuh).
#include "multi_rhs.cuh"

namespace wobgb {

bool multi_rhs_supported(const WalkParams &p) {
    if (p.estimator != kBackward || p.n_volume != 0) return false;
    const int st = strategy_of(p.bie, p.estimator, p.problem);
    return st == kStratSingleLayer || (p.bie == kDirect && st == kStratUniform);
}

cudaError_t launch_multi_rhs_2d(const SceneView<2> &s, const WalkParams &p, const MultiRhsArgs &a) {
    return mrhs::launch_multi<2>(s, p, a);
}

}  // namespace wobgb
