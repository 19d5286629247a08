/*
 * wob_capi.h - C ABI of the GB300 walk-on-boundary (WoB) engine.
 *
 * Plain C types only (no CUDA or torch types in the signatures): streams are passed as void*
 * (a cudaStream_t, or NULL for the legacy default stream), device buffers as plain pointers.
 * Every entry point returns a wob_status; wob_last_error() gives the message of the last failure
 * on the calling thread.
 *
 * Entry points that take device buffers and a stream only enqueue kernels on that stream (no
 * allocation, no synchronisation), so they can be captured into a CUDA graph and replayed; the
 * scene / batch / MLP constructors, the host-buffer solves and the debug entry points synchronise.
 *
 * Each entry point names the reference interface it replaces (rsugimoto/WoBToolbox, path:line).
 * The enums keep the reference's numbering so a caller can pass the values its string
 * converters produce (bie_models.cuh:24-51, estimator.cuh:24-54, points.hpp:22).
 */
#ifndef WOB_CAPI_H
#define WOB_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WOB_CAPI_VERSION 1

typedef enum wob_status {
    WOB_OK = 0,
    WOB_ERR_INVALID_ARGUMENT = 1, /* bad sizes, pointers, enums or geometry */
    WOB_ERR_UNSUPPORTED = 2,      /* a combination the reference does not define */
    WOB_ERR_CUDA = 3,             /* a CUDA runtime call failed */
    WOB_ERR_OUT_OF_MEMORY = 4,
    WOB_ERR_DEVICE_LIMIT = 5      /* a kernel hit an iteration / stack bound and stopped */
} wob_status;

/* wob::BIEModelType (bie_models.cuh:21) */
enum { WOB_INDIRECT_SINGLE_LAYER = 0, WOB_INDIRECT_DOUBLE_LAYER = 1, WOB_DIRECT = 2 };
/* wob::DomainType (bie_models.cuh:22) */
enum { WOB_INTERIOR_DOMAIN = 0, WOB_EXTERIOR_DOMAIN = 1 };
/* wob::EstimatorType (estimator.cuh:24) */
enum { WOB_BACKWARD_ESTIMATOR = 0, WOB_FORWARD_ESTIMATOR = 1 };
/* wob::ProblemType (estimator.cuh:38) */
enum { WOB_DIRICHLET_PROBLEM = 0, WOB_NEUMANN_PROBLEM = 1, WOB_ROBIN_PROBLEM = 2, WOB_MIXED_PROBLEM = 3 };
/* wob::BoundaryType (points.hpp:22) */
enum { WOB_DIRICHLET = 0, WOB_NEUMANN = 1, WOB_ROBIN = 2 };

typedef struct wob_scene_s *wob_scene;
typedef struct wob_batch_s *wob_batch;
typedef struct wob_mlp_s *wob_mlp;

/*
 * Solver parameters: the reference's Estimator constructor arguments (estimator.cuh:145-152)
 * plus the template enums that wob::utils::run<> dispatches on (runtime_utils.cuh:113-153),
 * the sample count of one launch (apps/general_2d.cu:60-61) and the random stream position.
 */
typedef struct wob_params {
    int32_t bie_model;                  /* WOB_INDIRECT_SINGLE_LAYER / _DOUBLE_LAYER / WOB_DIRECT */
    int32_t domain;                     /* WOB_INTERIOR_DOMAIN / WOB_EXTERIOR_DOMAIN */
    int32_t estimator;                  /* WOB_BACKWARD_ESTIMATOR / WOB_FORWARD_ESTIMATOR */
    int32_t problem;                    /* WOB_*_PROBLEM */
    uint32_t path_length;               /* bounces per path, >= 1 */
    uint32_t num_sample_paths;          /* paths per evaluation point in this call, >= 1 */
    uint32_t num_resampling_candidates; /* RIS candidates (1 = plain uniform sampling) */
    uint32_t num_volume_samples;        /* 0 = no source term */
    float eps;                          /* kernel distance clamp (FLT_EPSILON in the reference) */
    float first_kind_equation_scaling_constant; /* 1 in the reference */
    uint64_t seed;                      /* Philox key */
    uint64_t path_offset;               /* index of the first path of this call in each point's stream */
    uint32_t point_offset;              /* stream id of the first evaluation point */
    uint32_t flags;                     /* reserved, must be 0 */
} wob_params;

typedef struct wob_scene_info {
    int32_t dim;
    uint32_t n_elems;
    uint32_t n_nodes;                   /* wide BVH nodes */
    uint32_t bvh_depth;
    float total_area;                   /* Scene::total_boundary_area (scene.cuh:280) */
    float total_boundary_value;         /* Scene::total_boundary_value (scene.cuh:294) */
    int32_t has_volume_cache;
    uint32_t bytes_on_device;
    uint32_t line_grid_bins;            /* 2D host-built scenes: direction bins of the line grid (0: none) */
    uint32_t line_grid_cells;           /* offset cells per direction bin */
} wob_scene_info;

/* Last error message of the calling thread ("" when none). */
const char *wob_last_error(void);
/* WOB_CAPI_VERSION of the loaded library. */
int wob_version(void);
/* Device the library was initialised on and its SM count. */
int wob_device_info(int *device, int *sm_count);

/*
 * Builds a scene from boundary elements on the current CUDA device
 * (replaces wob::SceneHost::SceneHost, scene.cuh:264-299, and the lbvh build it wraps).
 * dim = 2 (segments) or 3 (triangles); host arrays in caller order:
 *   vertices        [n_elems][dim][dim]   a, b (, c)
 *   normals         [n_elems][dim]
 *   boundary_values [n_elems][dim]        per-vertex g (ElementXs::boundary_value_a/b/c)
 *   robin_alphas    [n_elems][dim]        per-vertex alpha; may be NULL (all zero)
 *   boundary_types  [n_elems]             WOB_DIRICHLET / WOB_NEUMANN / WOB_ROBIN
 * The scene stores elements in BVH leaf order (as the reference's CDFs are, scene.cuh:275-279);
 * wob_scene_get_element_order() returns that order. 2D scenes of up to 16384 segments also get a
 * line grid (direction bins x offset cells listing candidate segments in storage order) that
 * answers the walks' infinite-line queries with the same hits as the BVH; its shape is in
 * wob_scene_info, and it uses up to min(16 M, 8192 n) two-byte list entries of device memory.
 */
int wob_scene_create(int dim, uint32_t n_elems, const float *vertices, const float *normals,
                     const float *boundary_values, const float *robin_alphas,
                     const int32_t *boundary_types, wob_scene *out);
int wob_scene_destroy(wob_scene scene);

/*
 * The same scene built on the GPU from DEVICE arrays (same layout as wob_scene_create; no
 * counterpart in the reference, whose SceneHost and lbvh build run on the host, scene.cuh:264-299):
 * Morton codes, a sort, a binary radix tree collapsed into the 4-wide layout, records, Kahan CDFs
 * and guide tables, all on the device. The sampling tables are bit-identical to those of a host
 * build over the same storage order; the BVH topology (and so the storage order) differs, which
 * changes no hit set. Synchronises the stream. WOB_ERR_INVALID_ARGUMENT also when the tree is too
 * deep for the traversal stack (then use wob_scene_create).
 */
int wob_scene_create_device(int dim, uint32_t n_elems, const float *vertices, const float *normals,
                            const float *boundary_values, const float *robin_alphas,
                            const int32_t *boundary_types, void *stream, wob_scene *out);
int wob_scene_get_info(wob_scene scene, wob_scene_info *info);
/* order[i] = caller index of the i-th stored element (n_elems entries, host memory). */
int wob_scene_get_element_order(wob_scene scene, uint32_t *order);
/*
 * Reads and clears the scene's device error word (synchronous): bit 0 = a BVH traversal stack
 * overflowed, bit 1 = a traversal hit its step bound, bit 2 = a walk-on-spheres path was stopped
 * after 4096 jumps. Kernels that set a bit stop that query (or walk) and carry on; the reference
 * has no equivalent (its lbvh query and its WoS loop have no bound).
 */
int wob_scene_poll_error(wob_scene scene, uint32_t *bits);

/*
 * Attaches a source term f on a grid_res^dim cell grid over (-domain_size/2, domain_size/2)^dim,
 * values in host memory, x fastest (replaces SceneHost::set_volume_cache + VolumeCacheHost,
 * scene.cuh:206-252, 301-306). The |f| CDF is built on the host.
 */
int wob_scene_set_volume_cache(wob_scene scene, uint32_t grid_res, float domain_size,
                               const float *values);
int wob_scene_clear_volume_cache(wob_scene scene);

/*
 * Domain estimator over n_points evaluation points, params->num_sample_paths paths each
 * (replaces the per-point DeviceFunctor loop of apps/general_2d.cu:43-71 / general_3d.cu:43-73
 * around Estimator::compute_sample_path_contribution_domain, estimator.cuh:154-191, 405-454,
 * launched by wob::utils::run<>, runtime_utils.cuh:113-153).
 * Device pointers; enqueued on `stream`, asynchronous:
 *   points  [n_points][dim]  float
 *   sum     [n_points][dim+1] double   += sum over paths of [u, grad u]
 *   sumsq   [n_points][dim+1] double   += sum over paths of [u, grad u]^2 (may be NULL)
 *   bounces [1] uint64 += executed bounce-loop iterations (may be NULL)
 * Accumulates into sum/sumsq, so successive calls with path_offset advanced by
 * num_sample_paths continue each point's random stream (the reference's iteration loop,
 * apps/general_2d.cu:327-367, with FP64 running sums instead of FP32 Kahan).
 */
int wob_solve_domain(wob_scene scene, const wob_params *params, const float *points,
                     uint32_t n_points, double *sum, double *sumsq, uint64_t *bounces,
                     void *stream);

/*
 * Same computation with HOST buffers: copies points in, runs, copies sum/sumsq out and
 * synchronises (sum/sumsq are accumulated into, like the device version).
 */
int wob_solve_domain_host(wob_scene scene, const wob_params *params, const float *points,
                          uint32_t n_points, double *sum, double *sumsq, uint64_t *bounces);

/*
 * Autotuner (no counterpart in the reference, whose launch shape is fixed by thrust::for_each):
 * the specialised walk kernels are compiled for several occupancy targets (minimum resident
 * blocks per SM 1, 5, 6, 8) and run with a cap on the paths one lane takes per warp unit (the
 * launcher's choice up to 8, or 4, 2, 1) -- WOB_TUNE_CONFIGS configurations, index = occupancy +
 * 4 x cap; the 3D forward single-layer walk's shapes are the lockstep kernel and the split-phase
 * wavefront's three trace shapes, its second index the wavefront's chunk size. This times each on
 * the first points (device pointer, about 2^23 paths, the paths per lane that a launch over all
 * n_points would take) with the given parameters and makes the fastest the one used for that
 * kernel variant from then on
 * (process-wide). chosen = index of the chosen configuration (-1: these parameters use no
 * tunable kernel), ms_per_config[k] = time of configuration k (room for WOB_TUNE_CONFIGS),
 * n_configs = number of configurations. Allocates a temporary output buffer and synchronises
 * `stream`.
 */
#define WOB_TUNE_CONFIGS 16
int wob_autotune_domain(wob_scene scene, const wob_params *params, const float *points,
                        uint32_t n_points, int32_t *chosen, float *ms_per_config, int32_t *n_configs,
                        void *stream);

/* The tunable kernel variant a solve with these parameters uses (-1: none). */
int wob_tunable_variant(wob_scene scene, const wob_params *params, int32_t *variant);
/* Fix / read the configuration of a tunable variant (e.g. to reuse an earlier tuning result). */
int wob_set_domain_config(int32_t variant, int32_t config);
int wob_get_domain_config(int32_t variant, int32_t *config);

/*
 * Host-buffer domain solve that allocates nothing. No counterpart in the reference: it is for
 * callers that may not allocate device memory (for example a host application that owns the GPU
 * memory budget and forbids plugin allocations, or a real-time loop that must not allocate).
 * Same arguments and accumulate-into semantics as wob_solve_domain_host, plus the stream to run
 * on (NULL = legacy default stream); synchronises that stream before returning.
 *
 * It stages points, running sums and the bounce counter through a 16 MiB static device array
 * that every GPU loading the library holds until the process exits, so n_points is limited to
 * wob_noalloc_max_points(dim) (about 220k points in 3D, 300k in 2D); larger requests fail with
 * WOB_ERR_INVALID_ARGUMENT. It calls no cudaMalloc / cudaFree.
 *
 * Set-up: the first call on a device looks up the array's device address (cudaGetSymbolAddress)
 * and keeps it. Under lazy module loading (the CUDA default) that lookup is also when the runtime
 * loads the module and reserves the array, so make the first call on each device at set-up time,
 * before any stream capture and before a phase that must not allocate. The kept address belongs
 * to the device's context: do not call this entry point for a device after cudaDeviceReset on it.
 *
 * Sharing: each process (each CUDA context) has its own copy of the array. Within a process every
 * call uses the same array, which keeps the previous call's contents (the sums are reloaded from
 * the caller's arrays and the counter cleared on each call); calls that overlapped on the GPU would
 * race on it, so one process-wide lock is held from staging until the call's stream is
 * synchronised. Calls never overlap, and calls for different devices wait for each other.
 */
int wob_solve_domain_host_noalloc(wob_scene scene, const wob_params *params, const float *points,
                                  uint32_t n_points, double *sum, double *sumsq, uint64_t *bounces,
                                  void *stream);
/* Largest n_points wob_solve_domain_host_noalloc accepts for dim 2 or 3. */
int wob_noalloc_max_points(int dim, uint32_t *max_points);

/*
 * Batched domain solves: many scenes, each with its own parameters and evaluation points, in ONE
 * persistent launch (no counterpart in the reference, where each app launches one scene per
 * thrust::for_each, runtime_utils.cuh:146-151). scenes[i] (same dimension and device; they must
 * outlive the batch) is solved with params[i] at n_points[i] points. Points, sums and sums of
 * squares are concatenated over the scenes in order: scene i owns rows
 * [n_points[0] + ... + n_points[i-1], ... + n_points[i]). Each scene's values are exactly those of
 * wob_solve_domain on its rows (same random streams); path_offset_add is added to every scene's
 * path_offset, so repeated solves continue the streams. Asynchronous on `stream`.
 */
int wob_batch_create(const wob_scene *scenes, const wob_params *params, const uint32_t *n_points,
                     uint32_t n_scenes, wob_batch *out);
int wob_batch_solve(wob_batch batch, const float *points, double *sum, double *sumsq,
                    uint64_t *bounces, uint64_t path_offset_add, void *stream);
int wob_batch_destroy(wob_batch batch);

/*
 * Boundary estimator (replaces Estimator::compute_sample_path_contribution_boundary,
 * estimator.cuh:193-222, 456-496, as driven by apps/boundary_estimate.cu:62-95).
 * Device pointers, one boundary point per entry (points.hpp:32-39):
 *   p [n][dim], n [n][dim], interior_angle [n], boundary_value [n], boundary_type [n] int32,
 *   robin_alpha [n] (may be NULL)
 *   sum [n], sumsq [n] (may be NULL) double, accumulated into.
 */
int wob_solve_boundary(wob_scene scene, const wob_params *params, const float *p,
                       const float *n, const float *interior_angle, const float *boundary_value,
                       const int32_t *boundary_type, const float *robin_alpha, uint32_t n_points,
                       double *sum, double *sumsq, uint64_t *bounces, void *stream);

/*
 * The walk's estimate of the unknown boundary function at boundary points: the value
 * Estimator::compute_sample_unknown_boundary returns (estimator.cuh:232-357) -- the density of
 * the indirect models, the missing boundary data of the direct model. Backward estimator only;
 * arguments as wob_solve_boundary (sum / sumsq accumulated over the paths).
 */
int wob_solve_unknown_boundary(wob_scene scene, const wob_params *params, const float *p,
                               const float *n, const float *interior_angle,
                               const float *boundary_value, const int32_t *boundary_type,
                               const float *robin_alpha, uint32_t n_points, double *sum,
                               double *sumsq, uint64_t *bounces, void *stream);

/*
 * Multi-RHS walks (no counterpart in the reference, which solves one set of boundary data per
 * run; the data enter through BoundaryPoint::boundary_value, points.hpp:32-39). Up to
 * WOB_MAX_RHS right-hand sides share one set of paths: the estimator's sampling must not depend
 * on the data -- backward IndirectSingleLayer (uniform or RIS sampling, estimator.cuh:276-334) or
 * backward Direct with uniform sampling (estimator.cuh:335-347, i.e. not NeumannProblem) -- and
 * there is no source term. The value of each path for RHS r is bit-identical to the scalar walk
 * (wob_solve_domain / wob_solve_unknown_boundary) on the data of RHS r.
 *
 * wob_scene_set_rhs: host array values [n_elems][dim][n_rhs] in the caller's element order
 * (per element vertex, as boundary_values of wob_scene_create); n_rhs = 0 removes the table.
 * wob_solve_domain_multi: u(x) only (no gradient) at points [n_points][dim] (device);
 * sum / sumsq [n_points][n_rhs] double, accumulated; per_path [n_points][paths][n_rhs] float
 * (may be NULL; sums may be NULL when per_path is given).
 * wob_solve_unknown_boundary_multi: the unknown boundary function at boundary points (arguments as
 * wob_solve_unknown_boundary) whose data per RHS are boundary_values [n_points][n_rhs] (device).
 */
#define WOB_MAX_RHS 64
int wob_scene_set_rhs(wob_scene scene, const float *values, uint32_t n_rhs);
int wob_solve_domain_multi(wob_scene scene, const wob_params *params, const float *points,
                           uint32_t n_points, double *sum, double *sumsq, uint64_t *bounces,
                           float *per_path, void *stream);
int wob_solve_unknown_boundary_multi(wob_scene scene, const wob_params *params, const float *p,
                                     const float *n, const float *interior_angle,
                                     const float *boundary_values, const int32_t *boundary_type,
                                     const float *robin_alpha, uint32_t n_points, double *sum,
                                     double *sumsq, uint64_t *bounces, float *per_path,
                                     void *stream);

/*
 * Multi-RHS domain estimate with a control variate cv on the unknown boundary function (no
 * counterpart in the reference): host array values [n_elems][n_rhs] in storage order, piecewise
 * constant per element (e.g. the MLP with an n_rhs-wide head at the element centroids). The
 * estimate u(x) = sdk(x, y1) + (mu(y0) - cv(y0)) sdu(x, y0) + sum_{i<n} (sdu(x, z_i) / n) cv(z_i)
 * -- sdk / sdu the known / unknown domain terms of the model (bie_models.cuh), y0, y1 the start
 * samples, z_i n_potential_samples uniform samples drawn after the walk -- is unbiased for any cv;
 * the walk (and mu) is the one wob_solve_domain_multi runs. Setting a new RHS table removes cv.
 */
int wob_scene_set_rhs_control_variate(wob_scene scene, const float *values, uint32_t n_elems,
                                      uint32_t n_rhs);
int wob_solve_domain_multi_cv(wob_scene scene, const wob_params *params,
                              uint32_t n_potential_samples, const float *points, uint32_t n_points,
                              double *sum, double *sumsq, uint64_t *bounces, float *per_path,
                              void *stream);

/*
 * Walk on spheres, the reference's baseline method (apps/simple_wob_and_wos.cu:49-78, 111-137), for
 * 2D scenes with Dirichlet data: each path jumps to a uniform point on the largest empty circle
 * until the distance to the boundary is below params.eps and returns the boundary value at the
 * closest boundary point (BVH closest-point query; ties go to the smallest storage index). Uses
 * num_sample_paths, eps, seed, path_offset and point_offset of params. points [n][2] (device); sum /
 * sumsq [n] double (accumulated), queries = closest-point queries made, per_path [n][paths] float
 * (may be NULL). A path is stopped after 4096 jumps (error-word bit 2).
 * wob_closest_point: the query alone, for points [n][2]: stored element index, squared distance and
 * the boundary value at the closest point (device arrays).
 */
int wob_solve_wos(wob_scene scene, const wob_params *params, const float *points, uint32_t n_points,
                  double *sum, double *sumsq, uint64_t *queries, float *per_path, void *stream);
int wob_closest_point(wob_scene scene, const float *points, uint32_t n_points, uint32_t *elems,
                      float *dist2, float *values, void *stream);

/*
 * Virtual point lights (apps/potential_flow_with_vpl.cu:43-88). wob_vpl_paths runs n_paths
 * backward single-layer walks (PathComputeFunc), path i from a uniform boundary sample y_i, and
 * writes y_i to vpl_points [n_paths][dim] and the unknown-boundary estimate mu_i to vpl_values
 * [n_paths] (device); params.path_offset selects the paths (Philox streams of their own).
 * wob_vpl_aggregate (AggregateFunc) adds, at every point x of points [n_points][dim],
 * sum_i mu_i * (G(y_i, x) A, dG/dx(y_i, x) A) into sum [n_points][dim+1] (double, device), A the
 * scene's total boundary area, eps the kernel's distance clamp; partial sums are FP32 over tiles
 * of 256 VPLs, tile t added in FP64 into split t mod 8, the 8 splits added in order.
 */
int wob_vpl_paths(wob_scene scene, const wob_params *params, uint32_t n_paths, float *vpl_points,
                  float *vpl_values, uint64_t *bounces, void *stream);
int wob_vpl_aggregate(wob_scene scene, float eps, const float *vpl_points, const float *vpl_values,
                      uint32_t n_vpl, const float *points, uint32_t n_points, double *sum, void *stream);

/*
 * Learned control variate (no counterpart in the reference). A control-variate density sigma~
 * is given per stored element (host array, storage order; e.g. the MLP below evaluated at the
 * element centroids). wob_solve_domain_cv then runs the forward single-layer Neumann estimator
 * (estimator.cuh:405-454) on the residual r = sigma - sigma~: u(x) = <G_x, sigma~> + <G_x, r>,
 * where <G_x, sigma~> uses n_potential_samples uniform boundary samples and r is transported by
 * the reference's forward walk from a residual source s + K sigma~ - sigma~ (K sigma~ from
 * n_kernel_samples uniform samples). Unbiased for any sigma~; params must select
 * IndirectSingleLayer / ForwardEstimator / NeumannProblem without a source term. per_path (device,
 * [n_points][paths][dim+1], may be NULL) receives the per-path values instead of the sums.
 */
int wob_scene_set_control_variate(wob_scene scene, const float *values, uint32_t n_elems);
int wob_solve_domain_cv(wob_scene scene, const wob_params *params, uint32_t n_potential_samples,
                        uint32_t n_kernel_samples, const float *points, uint32_t n_points, double *sum,
                        double *sumsq, uint64_t *bounces, float *per_path, void *stream);

/*
 * Step bounds of the scene's device loops (no counterpart in the reference, whose lbvh traversal
 * and walk-on-spheres loop are unbounded). A line or closest-point query that visits more than
 * max_traversal_steps nodes ends there, keeps the hits found so far and sets the scene's error
 * word; a walk-on-spheres path stops after max_wos_jumps jumps with the value at its closest point
 * and sets the error word (wob_scene_poll_error; the host-buffer entry points return
 * WOB_ERR_DEVICE_LIMIT). 0 restores a default: 5 x nodes + 16 steps, which a correct tree never
 * reaches, and 4096 jumps (larger values are refused). Lower values let a caller's error handling
 * be exercised without a faulty scene.
 */
int wob_scene_set_step_limits(wob_scene scene, uint32_t max_traversal_steps, uint32_t max_wos_jumps);

/*
 * Measured ceiling of the uniform-sampling walk's memory access pattern (no counterpart in the
 * reference; the roofline denominator of that walk): samples per second when every thread of a
 * full-occupancy grid issues, with four chains in flight, what one uniform boundary sample reads
 * -- a 16-byte guide-table entry at a random index and the 64-byte record it points to -- over
 * tables of n_records records and n_guide entries (L2-resident at the benchmark's sizes). iters
 * gathers per chain and thread; ms receives the timed launch's duration. Allocates and frees its
 * own tables on the current device.
 */
int wob_measure_gather_peak(uint32_t n_records, uint32_t n_guide, uint32_t iters, double *samples_per_s,
                            float *ms);

/*
 * Residual control variate for the single-layer Neumann estimators (no counterpart in the
 * reference; it reuses the reference's forward walk, estimator.cuh:405-454, unchanged). The
 * control variate is a density sigma~ that is constant on each stored triangle (device array
 * [n_elems], storage order; e.g. the MLP below at the triangle centroids). The single-layer
 * density solves sigma = c g + T sigma with c = +2 inside, -2 outside and T(x, y) = -c dG/dn_x
 * (bie_models.cuh:262-316), so r = sigma - sigma~ solves the same equation with the data
 * g + delta, delta = (T sigma~ - sigma~) / c, and u = S sigma~ + S r.
 *
 * wob_cv_residual_data: delta_j at the centroid of every stored triangle (device [n_elems]).
 * wob_cv_potential: S sigma~ and its gradient at points (device [n][3] in, [n][4] out: u, grad u).
 * Both sum over all triangles: the centroid rule beyond near_factor times a triangle's longest
 * edge, the closed form of a uniformly charged triangle (Wilton et al. 1984) nearer. With
 * theta > 0 the far field of a cluster of 32 consecutive stored triangles is its quadrupole
 * expansion wherever the cluster's radius is below theta times its distance from every target of
 * a warp (and beyond the triangles' near radii); theta = 0 sums every triangle. theta = 0.3 adds
 * about 2e-4 (relative to the largest value) to the centroid rule's own error. 3D scenes.
 * wob_scene_clone: an independent copy of a scene (geometry, records, tables, volume cache): the
 * element records are copied, the device buffers that no entry point writes in place (BVH,
 * intersection records, sampling tables, volume cache, line grid) are shared by reference count,
 * so either scene may be destroyed first and a later change to one leaves the other as it was.
 * Cloning only reads the source scene and may run beside other calls that read it.
 * wob_scene_add_boundary_offsets: adds delta_j to the vertex values of stored element j (delta on
 * the device when delta_on_device != 0, else on the host) and rebuilds the |g| sampling tables;
 * synchronises the stream. The plain forward estimator on such a clone, plus S sigma~ from
 * wob_cv_potential, estimates u; the residual's sampling weight shrinks with |sigma - sigma~|,
 * which is where the variance reduction comes from.
 * wob_scene_element_frames: (centroid, normal) of every stored element, the network's input there:
 * device [n_elems][6] (2D scenes: (x, y, 0, nx, ny, 0)).
 */
int wob_cv_residual_data(wob_scene scene, const float *sigma, int domain, float near_factor, float theta,
                         float *delta, void *stream);
int wob_cv_potential(wob_scene scene, const float *sigma, float near_factor, float theta, const float *points,
                     uint32_t n_points, float *out, void *stream);
int wob_scene_clone(wob_scene scene, wob_scene *out);
int wob_scene_add_boundary_offsets(wob_scene scene, const float *delta, uint32_t n_elems, int delta_on_device,
                                   void *stream);
int wob_scene_element_frames(wob_scene scene, float *out, void *stream);
/* n boundary points uniform by area (the walk's uniform boundary sample, Philox stream 2 of point
 * index i with `seed`): device arrays p, normals [n][dim], interior_angle, boundary_value, type,
 * robin_alpha (may be NULL) [n] -- the training points of the control variate's labels. */
int wob_scene_sample_boundary(wob_scene scene, uint32_t n, uint64_t seed, float *p, float *normals,
                              float *interior_angle, float *boundary_value, int32_t *boundary_type,
                              float *robin_alpha, void *stream);
/* Clamps n device floats in place to [-t, t], where t is the ceil(quantile * n)-th smallest |v|
 * (exact: a radix select on the device), and writes t to *threshold (device, may be NULL). The
 * control variate's labels go through it before training: a mean-squared fit would otherwise
 * chase the few heavy-tailed walk estimates. quantile in (0, 1]. Stream-ordered, no host sync. */
int wob_clip_magnitude_quantile(float *values, uint32_t n, float quantile, float *threshold, void *stream);

/*
 * Fourier-feature MLP trained with the engine's own CUDA kernels: (x, n) in R^6 ->
 * [sin, cos](2 pi B (x, n)) with B n_freq x 6 ~ N(0, freq_sigma^2) -> hidden_layers x (64, SiLU)
 * -> out_dim. 2 n_freq must be 64. Parameters in FP32 (Adam master copy); every GEMM runs on
 * BF16 tensor cores with FP32 accumulation. Device pointers; inputs [n][6], outputs [n][out_dim].
 * wob_mlp_gradient: gradient of mean((y - t)^2) over all n * out_dim entries (grad [n_params],
 * loss [1], device); wob_mlp_adam_step: the same gradient and one Adam update
 * (beta 0.9 / 0.999, eps 1e-8). Parameter layout: per layer W [out][in] row-major, then b [out].
 */
int wob_mlp_create(uint32_t n_freq, uint32_t hidden_layers, uint32_t out_dim, float freq_sigma,
                   uint64_t seed, wob_mlp *out);
int wob_mlp_destroy(wob_mlp mlp);
int wob_mlp_num_params(wob_mlp mlp, uint32_t *n);
int wob_mlp_get_params(wob_mlp mlp, float *params, float *freqs);
int wob_mlp_set_params(wob_mlp mlp, const float *params);
int wob_mlp_forward(wob_mlp mlp, const float *inputs, uint32_t n, float *outputs, void *stream);
int wob_mlp_gradient(wob_mlp mlp, const float *inputs, const float *targets, uint32_t n, float *grad,
                     float *loss, void *stream);
int wob_mlp_adam_step(wob_mlp mlp, const float *inputs, const float *targets, uint32_t n, float lr,
                      float *loss, void *stream);
/*
 * wob_mlp_train: `steps` Adam steps (b1 0.9, b2 0.999, eps 1e-8; learning rate lr with a cosine
 * decay to 0 over the steps) on batches of `batch` rows drawn uniformly with replacement from the
 * n training rows (inputs [n][6], targets [n][out_dim], device) by Philox4x32-10 keyed with
 * `seed`. The loop runs on the device: one step (batch draw, forward, backward, Adam update) is
 * captured once as a CUDA graph and replayed, so no host work happens per step; for 4 hidden
 * layers and 32 frequencies the step is one fused kernel with the network in shared memory and a
 * block-ordered (deterministic) gradient sum. loss_history (device [steps] or NULL) receives each
 * step's batch loss. Ordered after the caller's stream; returns when the last step has run.
 * wob_mlp_gradient_fused: the gradient and loss that one fused step computes, for the given rows
 * in order (no batch draw, no update) -- the fused step's check against wob_mlp_gradient.
 */
int wob_mlp_train(wob_mlp mlp, const float *inputs, const float *targets, uint32_t n, uint32_t steps,
                  uint32_t batch, float lr, uint64_t seed, float *loss_history, void *stream);
int wob_mlp_gradient_fused(wob_mlp mlp, const float *inputs, const float *targets, uint32_t n, float *grad,
                           float *loss, void *stream);
/*
 * wob_mlp_inject_wait_timeout: a test of the fused step's failure path. With polls > 0 every block
 * of the following fused steps waits `polls` polls on an mbarrier nothing arrives on before its
 * first product and takes the timeout as a product that did not complete: the block sets the error
 * word, drains its products, releases its tensor memory and returns; the update is skipped, so the
 * parameters keep their values, and wob_mlp_train returns WOB_ERR_DEVICE_LIMIT. polls = 0 turns it
 * off. No GPU fault or hang is involved.
 */
int wob_mlp_inject_wait_timeout(wob_mlp mlp, uint32_t polls);

/*
 * All hits of the infinite lines origin + t dir (the query of scene.cuh:483-486 / 787-790).
 * Device pointers: origins [n][dim], dirs [n][dim]; counts [n] = number of hits (uncapped);
 * hits [n][64] = stored element indices of the first min(count, 64) hits in storage order;
 * hit_points [n][64][dim] (may be NULL).
 */
int wob_line_query(wob_scene scene, const float *origins, const float *dirs, uint32_t n_rays,
                   uint32_t *counts, uint32_t *hits, float *hit_points, void *stream);

/*
 * Per-path domain contributions for parity checks: values [n_points][num_sample_paths][dim+1]
 * float (device), the exact per-path values whose sums wob_solve_domain accumulates.
 */
int wob_debug_domain_paths(wob_scene scene, const wob_params *params, const float *points,
                           uint32_t n_points, float *values, void *stream);

/* Per-path boundary contributions [n_points][num_sample_paths] float (device). */
int wob_debug_boundary_paths(wob_scene scene, const wob_params *params, const float *p,
                             const float *n, const float *interior_angle,
                             const float *boundary_value, const int32_t *boundary_type,
                             const float *robin_alpha, uint32_t n_points, float *values,
                             void *stream);

#ifdef __cplusplus
}
#endif

#endif /* WOB_CAPI_H */
