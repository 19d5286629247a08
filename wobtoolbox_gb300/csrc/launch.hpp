// Launch entry points shared between the C ABI (capi.cu) and the per-dimension kernel units.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace wobgb {

template <int D> struct SceneView;
struct WalkParams;

// Boundary points of the boundary estimator (points.hpp:32-39), device pointers.
struct BoundaryInput {
    const float *p, *n, *angle, *bv;
    const int32_t *type;
    const float *alpha;  // may be null
};

// Variants of the walk kernels: kBie / kStrat fix the BIE model and sampling strategy at compile
// time (-1 = run-time), kVol = false drops the source term. Instantiated in the k*_*.cu units.
template <int D, int kBie, int kStrat, bool kVol, int kMinB = 1>
cudaError_t launch_domain_variant(const SceneView<D> &s, const WalkParams &p, const float *pts, uint32_t n_points,
                                  double *sum, double *sumsq, unsigned long long *bounces, float *per_path,
                                  cudaStream_t stream);
template <int D, int kBie, int kStrat, bool kVol>
cudaError_t launch_boundary_variant(const SceneView<D> &s, const WalkParams &p, const BoundaryInput &bin,
                                    uint32_t n_points, double *sum, double *sumsq, unsigned long long *bounces,
                                    float *per_path, cudaStream_t stream);
template <int D>
cudaError_t launch_line_query_impl(const SceneView<D> &s, const float *origins, const float *dirs, uint32_t n,
                                   uint32_t *counts, uint32_t *hits, float *points, cudaStream_t stream);

// Autotuned variants: the hot specialisations are compiled for several occupancy targets.
// tunable_domain_variant() names the tunable variant a solve would use (-1: none);
// set_domain_config() / domain_config() select the compiled configuration used from then on.
// A configuration is (minimum resident blocks per SM, cap on paths per lane of a warp unit).
constexpr int kNumTunable = 4;
constexpr int kTuneOccupancies = 4;
constexpr int kTunePptCaps = 4;
constexpr int kTuneConfigs = kTuneOccupancies * kTunePptCaps;
int tunable_domain_variant(int dim, const WalkParams &p);
int domain_config(int variant);
void set_domain_config(int variant, int config);
const char *domain_config_name(int variant, int config);
cudaError_t launch_domain_config(int dim, int variant, int config, const void *scene_view, const WalkParams &p,
                                 const float *pts, uint32_t n_points, double *sum, double *sumsq,
                                 unsigned long long *bounces, float *per_path, cudaStream_t stream);

// Control-variate domain estimator (k_cv.cu).
cudaError_t launch_domain_cv_2d(const SceneView<2> &s, const WalkParams &p, const float *pts, uint32_t n_points,
                                double *sum, double *sumsq, unsigned long long *bounces, float *per_path,
                                cudaStream_t stream);
cudaError_t launch_domain_cv_3d(const SceneView<3> &s, const WalkParams &p, const float *pts, uint32_t n_points,
                                double *sum, double *sumsq, unsigned long long *bounces, float *per_path,
                                cudaStream_t stream);
// Learned control-variate tables (k_cv_tables.cu): per-triangle sources {centroid, sigma~ area},
// squared near radii and the clusters of 32 stored triangles (4 float4 each: centre and far radius
// for theta, moments to the quadrupole); the residual Neumann data delta_j of each stored triangle;
// the single-layer potential of sigma~ and its gradient at points ([n][4]); the (centroid, normal)
// network input of every stored element ([n][6]).
cudaError_t launch_cv_sources(const SceneView<3> &s, const float *sigma, float near_factor, float theta, float4 *src,
                              float *near2, float4 *clusters, cudaStream_t stream);
// Records (64 bytes each) of the cluster table: clusters of 32 stored triangles, then groups of 8
// clusters, then groups of 8 of those.
uint32_t cv_cluster_records(uint32_t n_elems);
cudaError_t launch_cv_residual(const SceneView<3> &s, const float4 *src, const float *near2, const float4 *clusters,
                               const float *sigma, float c_coef, float *delta, cudaStream_t stream);
// scratch: cv_point_order_words(n_points) 32-bit words (the points' Morton order and bounds).
uint32_t cv_point_order_words(uint32_t n_points);
cudaError_t launch_cv_potential(const SceneView<3> &s, const float4 *src, const float *near2, const float4 *clusters,
                                const float *sigma, const float *pts, uint32_t n_points, uint32_t *scratch,
                                float *out, cudaStream_t stream);
template <int D> cudaError_t launch_element_frames(const SceneView<D> &s, float *out, cudaStream_t stream);
// elems[i * record_floats + first + k] += delta[i] for k < dim (device copy of the element records).
cudaError_t launch_add_boundary_offsets(float *elems, const float *delta, uint32_t n, uint32_t record_floats,
                                        uint32_t first, uint32_t dim, cudaStream_t stream);
// Random-gather ceiling of the uniform-sampling walk (k_probe.cu): samples per second of guide +
// 64-byte record gathers over tables of the given sizes, on the current device.
cudaError_t measure_gather_peak(uint32_t n_rec, uint32_t n_guide, uint32_t iters, int sm_count, double *samples_per_s,
                                float *ms);
// Boundary points uniform by area (k_sample.cu): position, normal, angle, data, type, alpha.
template <int D>
cudaError_t launch_sample_boundary(const SceneView<D> &s, uint32_t n, uint64_t seed, float *p, float *nrm,
                                   float *angle, float *bv, int32_t *type, float *alpha, cudaStream_t stream);
// Clamps device values to [-t, t], t = the ceil(q n)-th smallest |v| (k_sample.cu); t also to
// *threshold when it is not null.
cudaError_t launch_clip_quantile(float *values, uint32_t n, float quantile, float *threshold, cudaStream_t stream);
// Shared error message of the C ABI (capi.cu).
void set_last_error(const char *msg);

// One scene of a batched launch (k_batch.cu). One launch runs the n_scenes scenes of table, all of
// walk class cls (batch_walk_class), whose units are numbered from 0.
template <int D> struct BatchEntry;
cudaError_t launch_batch_2d(const BatchEntry<2> *table, uint32_t n_scenes, uint32_t cls, uint64_t total_units,
                            const float *pts, double *sum, double *sumsq, unsigned long long *bounces,
                            uint64_t path_offset_add, cudaStream_t stream);
cudaError_t launch_batch_3d(const BatchEntry<3> *table, uint32_t n_scenes, uint32_t cls, uint64_t total_units,
                            const float *pts, double *sum, double *sumsq, unsigned long long *bounces,
                            uint64_t path_offset_add, cudaStream_t stream);
// Paths per lane of a warp unit: up to 8, keeping at least 16384 units so the grid-stride loop
// still balances over the persistent grid.
inline uint32_t choose_ppt(uint64_t n_points, uint32_t n_paths) {
    uint32_t ppt = 8;
    while (ppt > 1 && ((uint64_t)n_points * ((n_paths + 32u * ppt - 1) / (32u * ppt)) < 16384u || 32u * ppt > n_paths))
        ppt >>= 1;
    return ppt;
}

// Forward single-layer Neumann walk in 3D as a split-phase wavefront (k_fwd_wave.cu): shape 1
// traces at >= 8 blocks/SM, 2 at >= 6 blocks/SM, 3 at >= 6 blocks/SM on 64-byte compressed nodes
// (built per solve); paths advance in chunks of at most max_slots paths (whole points). Allocates
// its path state stream-ordered (cudaMallocAsync).
cudaError_t launch_fwd_wave_3d(const SceneView<3> &s, const WalkParams &p, const float *pts, uint32_t n_points,
                               double *sum, double *sumsq, unsigned long long *bounces, float *per_path, int shape,
                               uint32_t max_slots, cudaStream_t stream);
// Dispatchers (kernels_dispatch.cu): pick the specialised variant for the parameters.
cudaError_t launch_domain_2d(const SceneView<2> &s, const WalkParams &p, const float *pts, uint32_t n_points,
                             double *sum, double *sumsq, unsigned long long *bounces, float *per_path,
                             cudaStream_t stream);
cudaError_t launch_domain_3d(const SceneView<3> &s, const WalkParams &p, const float *pts, uint32_t n_points,
                             double *sum, double *sumsq, unsigned long long *bounces, float *per_path,
                             cudaStream_t stream);
cudaError_t launch_boundary_2d(const SceneView<2> &s, const WalkParams &p, const BoundaryInput &bin,
                               uint32_t n_points, double *sum, double *sumsq, unsigned long long *bounces,
                               float *per_path, cudaStream_t stream);
cudaError_t launch_boundary_3d(const SceneView<3> &s, const WalkParams &p, const BoundaryInput &bin,
                               uint32_t n_points, double *sum, double *sumsq, unsigned long long *bounces,
                               float *per_path, cudaStream_t stream);
cudaError_t launch_line_query_2d(const SceneView<2> &s, const float *origins, const float *dirs, uint32_t n,
                                 uint32_t *counts, uint32_t *hits, float *points, cudaStream_t stream);
cudaError_t launch_line_query_3d(const SceneView<3> &s, const float *origins, const float *dirs, uint32_t n,
                                 uint32_t *counts, uint32_t *hits, float *points, cudaStream_t stream);

}  // namespace wobgb
