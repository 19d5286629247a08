// Routes a solve to the specialised kernel variant for its parameters, or to the general one.
// Variants are instantiated in k2_*.cu / k3_*.cu; every variant is compiled from the same walk
// source (walk_generic.cuh), only with some parameters fixed at compile time.
#include "launch.hpp"
#include "walk_generic.cuh"

#include <atomic>

namespace wobgb {

// ---- autotuned variants: 0 = 3D direct uniform, 1 = 2D double-layer line intersection,
// 2 = 3D direct Neumann; configurations = minimum resident blocks {1 (no limit), 5, 6, 8}.
namespace {
std::atomic<int> g_config[kNumTunable] = {{0}, {0}, {0}};
const int kMinBOf[kTuneConfigs] = {1, 5, 6, 8};
const char *kConfigNames[kTuneConfigs] = {"128 threads, no register cap", "128 threads, >=5 blocks/SM",
                                          "128 threads, >=6 blocks/SM", "128 threads, >=8 blocks/SM"};
}  // namespace

int tunable_domain_variant(int dim, const WalkParams &p) {
    if (p.n_volume != 0) return -1;
    const int st = strategy_of(p.bie, p.estimator, p.problem);
    if (dim == 3 && st == kStratUniform && p.bie == kDirect) return 0;
    if (dim == 2 && st == kStratLineIntersection) return 1;
    if (dim == 3 && st == kStratDirectNeumann) return 2;
    return -1;
}
int domain_config(int variant) { return (variant >= 0 && variant < kNumTunable) ? g_config[variant].load() : 0; }
void set_domain_config(int variant, int config) {
    if (variant >= 0 && variant < kNumTunable && config >= 0 && config < kTuneConfigs) g_config[variant].store(config);
}
const char *domain_config_name(int variant, int config) {
    (void)variant;
    return (config >= 0 && config < kTuneConfigs) ? kConfigNames[config] : "";
}

template <int D, int kBie, int kStrat>
static cudaError_t launch_cfg(int config, const SceneView<D> &s, const WalkParams &p, const float *pts, uint32_t n,
                              double *sum, double *sumsq, unsigned long long *b, float *pp, cudaStream_t st) {
    switch (kMinBOf[config]) {
    case 5: return launch_domain_variant<D, kBie, kStrat, false, 5>(s, p, pts, n, sum, sumsq, b, pp, st);
    case 6: return launch_domain_variant<D, kBie, kStrat, false, 6>(s, p, pts, n, sum, sumsq, b, pp, st);
    case 8: return launch_domain_variant<D, kBie, kStrat, false, 8>(s, p, pts, n, sum, sumsq, b, pp, st);
    default: return launch_domain_variant<D, kBie, kStrat, false, 1>(s, p, pts, n, sum, sumsq, b, pp, st);
    }
}

cudaError_t launch_domain_config(int dim, int variant, int config, const void *scene_view, const WalkParams &p,
                                 const float *pts, uint32_t n, double *sum, double *sumsq, unsigned long long *b,
                                 float *pp, cudaStream_t st) {
    if (config < 0 || config >= kTuneConfigs) config = 0;
    if (variant == 0 && dim == 3)
        return launch_cfg<3, kDirect, kStratUniform>(config, *(const SceneView<3> *)scene_view, p, pts, n, sum, sumsq, b, pp, st);
    if (variant == 1 && dim == 2)
        return launch_cfg<2, kDoubleLayer, kStratLineIntersection>(config, *(const SceneView<2> *)scene_view, p, pts, n, sum, sumsq, b, pp, st);
    if (variant == 2 && dim == 3)
        return launch_cfg<3, kDirect, kStratDirectNeumann>(config, *(const SceneView<3> *)scene_view, p, pts, n, sum, sumsq, b, pp, st);
    return cudaErrorInvalidValue;
}

cudaError_t launch_domain_2d(const SceneView<2> &s, const WalkParams &p, const float *pts, uint32_t n_points,
                             double *sum, double *sumsq, unsigned long long *bounces, float *per_path,
                             cudaStream_t stream) {
    const int v = tunable_domain_variant(2, p);
    if (v >= 0) return launch_domain_config(2, v, domain_config(v), &s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
    const int st = strategy_of(p.bie, p.estimator, p.problem);
    if (p.n_volume == 0 && st == kStratDirectNeumann)
        return launch_domain_variant<2, kDirect, kStratDirectNeumann, false>(s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
    if (p.n_volume == 0 && st == kStratSingleLayer)
        return launch_domain_variant<2, kSingleLayer, kStratSingleLayer, false, 5>(s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
    if (p.n_volume == 0 && st == kStratFwdSlNeumann)
        return launch_domain_variant<2, kSingleLayer, kStratFwdSlNeumann, false, 5>(s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
    return launch_domain_variant<2, -1, kStratRuntime, true>(s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
}

cudaError_t launch_domain_3d(const SceneView<3> &s, const WalkParams &p, const float *pts, uint32_t n_points,
                             double *sum, double *sumsq, unsigned long long *bounces, float *per_path,
                             cudaStream_t stream) {
    const int v = tunable_domain_variant(3, p);
    if (v >= 0) return launch_domain_config(3, v, domain_config(v), &s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
    const int st = strategy_of(p.bie, p.estimator, p.problem);
    if (p.n_volume == 0 && st == kStratSingleLayer)
        return launch_domain_variant<3, kSingleLayer, kStratSingleLayer, false, 5>(s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
    if (p.n_volume == 0 && st == kStratFwdSlNeumann)
        return launch_fwd_wavefront_3d(s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
    return launch_domain_variant<3, -1, kStratRuntime, true>(s, p, pts, n_points, sum, sumsq, bounces, per_path, stream);
}

cudaError_t launch_boundary_2d(const SceneView<2> &s, const WalkParams &p, const BoundaryInput &bin,
                               uint32_t n_points, double *sum, double *sumsq, unsigned long long *bounces,
                               float *per_path, cudaStream_t stream) {
    return launch_boundary_variant<2, -1, kStratRuntime, true>(s, p, bin, n_points, sum, sumsq, bounces, per_path, stream);
}

cudaError_t launch_boundary_3d(const SceneView<3> &s, const WalkParams &p, const BoundaryInput &bin,
                               uint32_t n_points, double *sum, double *sumsq, unsigned long long *bounces,
                               float *per_path, cudaStream_t stream) {
    const int st = strategy_of(p.bie, p.estimator, p.problem);
    if (p.n_volume == 0 && st == kStratDirectNeumann)
        return launch_boundary_variant<3, kDirect, kStratDirectNeumann, false>(s, p, bin, n_points, sum, sumsq, bounces, per_path, stream);
    return launch_boundary_variant<3, -1, kStratRuntime, true>(s, p, bin, n_points, sum, sumsq, bounces, per_path, stream);
}

cudaError_t launch_line_query_2d(const SceneView<2> &s, const float *origins, const float *dirs, uint32_t n,
                                 uint32_t *counts, uint32_t *hits, float *points, cudaStream_t stream) {
    return launch_line_query_impl<2>(s, origins, dirs, n, counts, hits, points, stream);
}
cudaError_t launch_line_query_3d(const SceneView<3> &s, const float *origins, const float *dirs, uint32_t n,
                                 uint32_t *counts, uint32_t *hits, float *points, cudaStream_t stream) {
    return launch_line_query_impl<3>(s, origins, dirs, n, counts, hits, points, stream);
}

}  // namespace wobgb
