// TEST INFRASTRUCTURE ONLY. Runs the reference's own estimator code (wob/wob.cuh and the headers
// it includes, compiled unmodified from the reference tree in the reference's CPU configuration:
// host C++20, OpenMP Thrust back end, std::mt19937 random states, CMakeLists.txt:22-40) on
// caller-given elements and points, and returns per-point statistics of its path contributions.
// Built by oracle/Makefile (target ref) into oracle/_ref/libwobref.so; the stand-ins for the
// reference's absent dependencies (Eigen, lbvh, thrust::optional) are in oracle/ref_shim/.
//
// The per-point functor follows the reference apps' DeviceFunctor (apps/general_2d.cu:40-71,
// apps/general_3d.cu:40-73): one random state per point, an Estimator built with the run's
// parameters, compute_sample_path_contribution_domain once per path. It differs in what it keeps:
// FP64 sums and sums of squares of every component instead of an FP32 Kahan sum, so that the
// tests can form per-point z-scores, and optionally every path's u value for a few points. The
// random states are seeded as random_states_init does (runtime_utils.cuh:84-103): one
// std::mt19937_64 seeded with `seed` draws one seed per point, and each point's std::mt19937 is
// constructed from it. Launch goes through the reference's run<> dispatch
// (runtime_utils.cuh:105-153), i.e. one thrust::for_each over the points.
#include "wob/wob.cuh"

#include <cstdint>
#include <cstring>
#include <exception>
#include <memory>
#include <random>
#include <string>
#include <vector>

namespace {

std::string g_error;

template <unsigned int Dim> struct RefArgs {
    unsigned int path_length, num_sample_paths, num_resampling_candidates, num_volume_samples;
    float eps, first_kind_equation_scaling_constant;
    wob::Scene<float, Dim, false> scene;
    const float *points;
    const std::uint64_t *seeds;
    double *sum, *sumsq;         // [n][Dim + 1]
    float *per_path;             // [n_pp][num_sample_paths] (u only) or null
    unsigned int n_pp;
};

template <unsigned int Dim> struct Functors {
    template <wob::EquationKernelType K, wob::BIEModelType B, wob::DomainType Dm, wob::EstimatorType E,
              wob::ProblemType P>
    struct F {
        inline void operator()(const unsigned int idx, const RefArgs<Dim> &args) {
            wob::randomState_t random_state(static_cast<std::mt19937::result_type>(args.seeds[idx]));
            wob::Estimator<float, Dim, K, B, Dm, E, P> estimator(
                &random_state, args.scene, args.path_length, args.num_resampling_candidates, args.eps,
                args.first_kind_equation_scaling_constant, args.num_volume_samples);
            Eigen::Matrix<float, Dim, 1> x;
            for (unsigned int k = 0; k < Dim; k++) x[k] = args.points[(size_t)idx * Dim + k];
            double s[Dim + 1] = {}, q[Dim + 1] = {};
            for (unsigned int i = 0; i < args.num_sample_paths; i++) {
                const Eigen::Matrix<float, Dim + 1, 1> c =
                    estimator.compute_sample_path_contribution_domain(wob::DomainPoint<float, Dim>{x});
                for (unsigned int k = 0; k <= Dim; k++) {
                    s[k] += (double)c[k];
                    q[k] += (double)c[k] * (double)c[k];
                }
                if (args.per_path && idx < args.n_pp) args.per_path[(size_t)idx * args.num_sample_paths + i] = c[0];
            }
            for (unsigned int k = 0; k <= Dim; k++) {
                args.sum[(size_t)idx * (Dim + 1) + k] = s[k];
                args.sumsq[(size_t)idx * (Dim + 1) + k] = q[k];
            }
        }
    };
};

template <unsigned int Dim>
int solve(unsigned int n_elems, const float *verts, const float *normals, const float *bvals, const std::int32_t *types,
          const float *alphas, const std::int32_t *enums, const std::uint32_t *counts, const float *reals,
          std::uint32_t vol_res, float vol_size, const float *vol_values, std::uint64_t seed, const float *points,
          std::uint32_t n_points, double *sum, double *sumsq, float *per_path, std::uint32_t n_pp) {
    std::vector<wob::ElementXs<float, Dim, false>> elems(n_elems);
    for (unsigned int e = 0; e < n_elems; e++) {
        auto &el = elems[e];
        auto vtx = [&](int j) {
            Eigen::Matrix<float, Dim, 1> v;
            for (unsigned int k = 0; k < Dim; k++) v[k] = verts[((size_t)e * Dim + j) * Dim + k];
            return v;
        };
        for (unsigned int k = 0; k < Dim; k++) el.n[k] = normals[(size_t)e * Dim + k];
        el.a = vtx(0);
        el.b = vtx(1);
        el.boundary_value_a = bvals[(size_t)e * Dim + 0];
        el.boundary_value_b = bvals[(size_t)e * Dim + 1];
        el.robin_alpha_a = alphas ? alphas[(size_t)e * Dim + 0] : 0.0f;
        el.robin_alpha_b = alphas ? alphas[(size_t)e * Dim + 1] : 0.0f;
        if constexpr (Dim == 3) {
            el.c = vtx(2);
            el.boundary_value_c = bvals[(size_t)e * Dim + 2];
            el.robin_alpha_c = alphas ? alphas[(size_t)e * Dim + 2] : 0.0f;
        }
        el.boundary_type = (wob::BoundaryType)types[e];
    }
    wob::SceneHost<float, Dim, false> scene_host(elems);
    thrust::device_vector<float> cache;
    if (vol_res > 0) {
        const size_t cells = Dim == 2 ? (size_t)vol_res * vol_res : (size_t)vol_res * vol_res * vol_res;
        cache.assign(vol_values, vol_values + cells);
        scene_host.set_volume_cache(vol_res, vol_size, cache);
    }
    // random_states_init (runtime_utils.cuh:91-103): one mt19937_64 draws one seed per point
    std::vector<std::uint64_t> seeds(n_points);
    std::mt19937_64 seeder(seed);
    for (auto &s : seeds) s = seeder();

    RefArgs<Dim> args{counts[0], counts[1], counts[2], counts[3], reals[0], reals[1],
                      scene_host.get_device_repr(), points, seeds.data(), sum, sumsq, per_path, n_pp};
    wob::utils::run<Functors<Dim>::template F>(args, n_points, (wob::BIEModelType)enums[0], (wob::DomainType)enums[1],
                                               (wob::EstimatorType)enums[2], (wob::ProblemType)enums[3]);
    return 0;
}

}  // namespace

extern "C" {

const char *wobref_last_error(void) { return g_error.c_str(); }

// enums = {bie, domain, estimator, problem}; counts = {path_length, num_sample_paths,
// num_resampling_candidates, num_volume_samples}; reals = {eps, first_kind_equation_scaling_constant}.
// Elements: verts [n][dim][dim], normals [n][dim], bvals [n][dim], types [n], alphas [n][dim] or
// NULL. Outputs sum / sumsq [n_points][dim + 1]; per_path [n_pp][num_sample_paths] (u) or NULL.
int wobref_solve_domain(int dim, std::uint32_t n_elems, const float *verts, const float *normals, const float *bvals,
                        const std::int32_t *types, const float *alphas, const std::int32_t *enums,
                        const std::uint32_t *counts, const float *reals, std::uint32_t vol_res, float vol_size,
                        const float *vol_values, std::uint64_t seed, const float *points, std::uint32_t n_points,
                        double *sum, double *sumsq, float *per_path, std::uint32_t n_pp) {
    try {
        if (dim == 2)
            return solve<2>(n_elems, verts, normals, bvals, types, alphas, enums, counts, reals, vol_res, vol_size,
                            vol_values, seed, points, n_points, sum, sumsq, per_path, n_pp);
        if (dim == 3)
            return solve<3>(n_elems, verts, normals, bvals, types, alphas, enums, counts, reals, vol_res, vol_size,
                            vol_values, seed, points, n_points, sum, sumsq, per_path, n_pp);
        g_error = "dim must be 2 or 3";
        return 1;
    } catch (const std::exception &ex) {
        g_error = ex.what();
        return 2;
    }
}

}  // extern "C"
