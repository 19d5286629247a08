// Routes a solve to the specialised kernel variant for its parameters, or to the general one.
// Variants are instantiated in k2_*.cu / k3_*.cu; every variant is compiled from the same walk
// source (walk_generic.cuh), only with some parameters fixed at compile time.
#include "launch.hpp"
#include "walk_generic.cuh"

#include <atomic>
#include <cstdio>

namespace wobgb {

// ---- autotuned variants: 0 = 3D direct uniform, 1 = 2D double-layer line intersection,
// 2 = 3D direct Neumann, 3 = 3D forward single-layer Neumann; configuration c = kernel shape
// (c % 4: for variants 0-2 the minimum resident blocks {1 (no limit), 5, 6, 8}; for variant 3 the
// lockstep kernel at >= 5 blocks/SM or the split-phase wavefront k_fwd_wave.cu in its three trace
// shapes) and c / 4: paths-per-lane cap {launcher's choice (up to 8), 4, 2, 1} for the lockstep
// kernels, paths per wavefront chunk {2^22, 2^21, 2^20, 2^19} for the wavefront.
namespace {
// defaults: the 3D forward walk starts on the wavefront (trace at >= 6 blocks/SM on compressed nodes,
// 2^22-path chunks)
std::atomic<int> g_config[kNumTunable] = {{0}, {0}, {0}, {3}};
const char *kFwdNames[kTuneOccupancies] = {"lockstep walk, >=5 blocks/SM", "wavefront, trace >=8 blocks/SM",
                                           "wavefront, trace >=6 blocks/SM",
                                           "wavefront, trace >=6 blocks/SM, 64-byte compressed nodes"};
const uint32_t kWaveSlotsOf[kTunePptCaps] = {1u << 22, 1u << 21, 1u << 20, 1u << 19};
const int kMinBOf[kTuneOccupancies] = {1, 5, 6, 8};
const uint32_t kPptCapOf[kTunePptCaps] = {0u, 4u, 2u, 1u};
const char *kOccNames[kTuneOccupancies] = {"no register cap", ">=5 blocks/SM", ">=6 blocks/SM", ">=8 blocks/SM"};
const char *kPptNames[kTunePptCaps] = {"paths/lane <= 8", "paths/lane <= 4", "paths/lane <= 2", "paths/lane = 1"};
char g_names[kTuneConfigs][64];
}  // namespace

int tunable_domain_variant(int dim, const WalkParams &p) {
    if (p.n_volume != 0) return -1;
    const int st = strategy_of(p.bie, p.estimator, p.problem);
    if (dim == 3 && st == kStratUniform && p.bie == kDirect) return 0;
    if (dim == 2 && st == kStratLineIntersection) return 1;
    if (dim == 3 && st == kStratDirectNeumann) return 2;
    if (dim == 3 && st == kStratFwdSlNeumann) return 3;
    return -1;
}
int domain_config(int variant) { return (variant >= 0 && variant < kNumTunable) ? g_config[variant].load() : 0; }
void set_domain_config(int variant, int config) {
    if (variant >= 0 && variant < kNumTunable && config >= 0 && config < kTuneConfigs) g_config[variant].store(config);
}
const char *domain_config_name(int variant, int config) {
    (void)variant;
    if (config < 0 || config >= kTuneConfigs) return "";
    static char fwd_names[kTuneConfigs][80];
    if (variant == 3) {
        if (!fwd_names[config][0]) {
            if (config % kTuneOccupancies == 0)
                snprintf(fwd_names[config], sizeof fwd_names[config], "128 threads, %s, %s", kFwdNames[0],
                         kPptNames[config / kTuneOccupancies]);
            else
                snprintf(fwd_names[config], sizeof fwd_names[config], "128 threads, %s, %u paths per chunk",
                         kFwdNames[config % kTuneOccupancies], kWaveSlotsOf[config / kTuneOccupancies]);
        }
        return fwd_names[config];
    }
    if (!g_names[config][0])
        snprintf(g_names[config], sizeof g_names[config], "128 threads, %s, %s", kOccNames[config % kTuneOccupancies],
                 kPptNames[config / kTuneOccupancies]);
    return g_names[config];
}

template <int D, int kBie, int kStrat>
static cudaError_t launch_cfg(int config, const SceneView<D> &s, const WalkParams &p_in, const float *pts, uint32_t n,
                              double *sum, double *sumsq, unsigned long long *b, float *pp, cudaStream_t st) {
    WalkParams p = p_in;
    p.ppt_cap = kPptCapOf[config / kTuneOccupancies];
    switch (kMinBOf[config % kTuneOccupancies]) {
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
    if (variant == 3 && dim == 3) {
        WalkParams q = p;
        q.ppt_cap = kPptCapOf[config / kTuneOccupancies];
        const SceneView<3> &v = *(const SceneView<3> *)scene_view;
        const int shape = config % kTuneOccupancies;
        if (shape == 0 || p.no_alloc)
            return launch_domain_variant<3, kSingleLayer, kStratFwdSlNeumann, false, 5>(v, q, pts, n, sum, sumsq, b, pp, st);
        return launch_fwd_wave_3d(v, p, pts, n, sum, sumsq, b, pp, shape, kWaveSlotsOf[config / kTuneOccupancies], st);
    }
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
