/*
 * C++ layer over the C ABI with the wob:: names a WoBToolbox app uses, so an app's host code ports
 * by swapping includes: the enums and string converters of equation_kernel.cuh:20-35,
 * bie_models.cuh:21-51, estimator.cuh:24-54 and points.hpp:22; ElementXs (scene.cuh:378-397,
 * 646-678) with plain float arrays in place of Eigen vectors; SceneHost (scene.cuh:264-326);
 * the per-point sample loop that an app's DeviceFunctor runs through wob::utils::run<>
 * (runtime_utils.cuh:105-153, apps/general_2d.cu:43-71) as SceneHost::solve_domain; and
 * wob::utils::idx_to_domain_point / save_field (utils.cuh:92-110, runtime_utils.cuh:34-57).
 *
 * Header-only; link libwob_gb300.so. Errors throw wob::Error with wob_last_error()'s message.
 */
#ifndef WOB_GB300_HPP
#define WOB_GB300_HPP

#include "wob_capi.h"

#include <array>
#include <cstdint>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace wob {

enum EquationKernelType { PoissonKernel, EquationKernelTypeCount };
enum BIEModelType { IndirectSingleLayer, IndirectDoubleLayer, Direct, BIEModelTypeCount };
enum DomainType { InteriorDomain, ExteriorDomain, DomainTypeCount };
enum EstimatorType { BackwardEstimator, ForwardEstimator, EstimatorTypeCount };
enum ProblemType { DirichletProblem, NeumannProblem, RobinProblem, MixedProblem, ProblemTypeCount };
enum BoundaryType { Dirichlet, Neumann, Robin };

inline EquationKernelType string_to_equation_kernel_type(const std::string &s) {
    return s == "PoissonKernel" ? PoissonKernel : EquationKernelTypeCount;
}
inline std::string equation_kernel_type_to_string(EquationKernelType t) {
    return t == PoissonKernel ? "PoissonKernel" : "InvalidEquationKernelType";
}
inline BIEModelType string_to_bie_model_type(const std::string &s) {
    if (s == "IndirectSingleLayer") return IndirectSingleLayer;
    if (s == "IndirectDoubleLayer") return IndirectDoubleLayer;
    if (s == "Direct") return Direct;
    return BIEModelTypeCount;
}
inline std::string bie_model_type_to_string(BIEModelType t) {
    switch (t) {
    case IndirectSingleLayer: return "IndirectSingleLayer";
    case IndirectDoubleLayer: return "IndirectDoubleLayer";
    case Direct: return "Direct";
    default: return "InvalidBIEModelType";
    }
}
inline DomainType string_to_domain_type(const std::string &s) {
    if (s == "InteriorDomain") return InteriorDomain;
    if (s == "ExteriorDomain") return ExteriorDomain;
    return DomainTypeCount;
}
inline std::string domain_type_to_string(DomainType t) {
    switch (t) {
    case InteriorDomain: return "InteriorDomain";
    case ExteriorDomain: return "ExteriorDomain";
    default: return "InvalidDomainType";
    }
}
inline EstimatorType string_to_estimator_type(const std::string &s) {
    if (s == "BackwardEstimator") return BackwardEstimator;
    if (s == "ForwardEstimator") return ForwardEstimator;
    return EstimatorTypeCount;
}
inline std::string estimator_type_to_string(EstimatorType t) {
    switch (t) {
    case BackwardEstimator: return "BackwardEstimator";
    case ForwardEstimator: return "ForwardEstimator";
    default: return "InvalidEstimatorType";
    }
}
inline ProblemType string_to_problem_type(const std::string &s) {
    if (s == "DirichletProblem") return DirichletProblem;
    if (s == "NeumannProblem") return NeumannProblem;
    if (s == "RobinProblem") return RobinProblem;
    if (s == "MixedProblem") return MixedProblem;
    return ProblemTypeCount;
}
inline std::string problem_type_to_string(ProblemType t) {
    switch (t) {
    case DirichletProblem: return "DirichletProblem";
    case NeumannProblem: return "NeumannProblem";
    case RobinProblem: return "RobinProblem";
    case MixedProblem: return "MixedProblem";
    default: return "InvalidProblemType";
    }
}

struct Error : std::runtime_error {
    int status;
    Error(int st, const std::string &msg) : std::runtime_error(msg), status(st) {}
};
inline void check(int st) {
    if (st != WOB_OK) throw Error(st, wob_last_error());
}

template <unsigned Dim> struct ElementXs;
template <> struct ElementXs<2> {
    std::array<float, 2> a, b, n;
    float boundary_value_a, boundary_value_b;
    BoundaryType boundary_type;
    float robin_alpha_a = 0.0f, robin_alpha_b = 0.0f;
};
template <> struct ElementXs<3> {
    std::array<float, 3> a, b, c, n;
    float boundary_value_a, boundary_value_b, boundary_value_c;
    BoundaryType boundary_type;
    float robin_alpha_a = 0.0f, robin_alpha_b = 0.0f, robin_alpha_c = 0.0f;
};

// Estimator arguments (estimator.cuh:145-152) plus the enums run<> dispatches on.
struct EstimatorParams {
    BIEModelType bie_model = IndirectDoubleLayer;
    DomainType domain = InteriorDomain;
    EstimatorType estimator = BackwardEstimator;
    ProblemType problem = DirichletProblem;
    unsigned path_length = 8, num_sample_paths = 1, num_resampling_candidates = 1, num_volume_samples = 0;
    float eps = 1.1920928955078125e-7f, first_kind_equation_scaling_constant = 1.0f;
    uint64_t seed = 0, path_offset = 0;
    uint32_t point_offset = 0;

    wob_params to_c() const {
        wob_params p{};
        p.bie_model = bie_model;
        p.domain = domain;
        p.estimator = estimator;
        p.problem = problem;
        p.path_length = path_length;
        p.num_sample_paths = num_sample_paths;
        p.num_resampling_candidates = num_resampling_candidates;
        p.num_volume_samples = num_volume_samples;
        p.eps = eps;
        p.first_kind_equation_scaling_constant = first_kind_equation_scaling_constant;
        p.seed = seed;
        p.path_offset = path_offset;
        p.point_offset = point_offset;
        p.flags = 0;
        return p;
    }
};

template <unsigned Dim> class SceneHost {
  public:
    explicit SceneHost(const std::vector<ElementXs<Dim>> &elems) {
        const size_t n = elems.size();
        std::vector<float> v(n * Dim * Dim), nr(n * Dim), bv(n * Dim), al(n * Dim);
        std::vector<int32_t> ty(n);
        for (size_t i = 0; i < n; i++) {
            const ElementXs<Dim> &e = elems[i];
            for (unsigned k = 0; k < Dim; k++) {
                v[(i * Dim + 0) * Dim + k] = e.a[k];
                v[(i * Dim + 1) * Dim + k] = e.b[k];
                if constexpr (Dim == 3) v[(i * Dim + 2) * Dim + k] = e.c[k];
                nr[i * Dim + k] = e.n[k];
            }
            bv[i * Dim + 0] = e.boundary_value_a;
            bv[i * Dim + 1] = e.boundary_value_b;
            al[i * Dim + 0] = e.robin_alpha_a;
            al[i * Dim + 1] = e.robin_alpha_b;
            if constexpr (Dim == 3) {
                bv[i * Dim + 2] = e.boundary_value_c;
                al[i * Dim + 2] = e.robin_alpha_c;
            }
            ty[i] = (int32_t)e.boundary_type;
        }
        check(wob_scene_create((int)Dim, (uint32_t)n, v.data(), nr.data(), bv.data(), al.data(), ty.data(), &s_));
    }
    ~SceneHost() {
        if (s_) wob_scene_destroy(s_);
    }
    SceneHost(const SceneHost &) = delete;
    SceneHost &operator=(const SceneHost &) = delete;

    // SceneHost::set_volume_cache (scene.cuh:301-306): values [grid_res^Dim] on the grid over
    // (-domain_size/2, domain_size/2)^Dim.
    void set_volume_cache(unsigned grid_res, float domain_size, const std::vector<float> &values) {
        check(wob_scene_set_volume_cache(s_, grid_res, domain_size, values.data()));
    }

    // The per-point loop of an app's DeviceFunctor for one iteration: num_sample_paths paths at each
    // point (host arrays [n][Dim]) accumulated into FP64 sums of [u, grad u] ([n][Dim + 1]) and
    // their squares (may be null). Returns the number of bounces.
    uint64_t solve_domain(const EstimatorParams &prm, const std::vector<float> &points, std::vector<double> &sum,
                          std::vector<double> *sumsq = nullptr) const {
        const uint32_t n = (uint32_t)(points.size() / Dim);
        if (sum.size() < (size_t)n * (Dim + 1)) sum.resize((size_t)n * (Dim + 1), 0.0);
        if (sumsq && sumsq->size() < (size_t)n * (Dim + 1)) sumsq->resize((size_t)n * (Dim + 1), 0.0);
        const wob_params p = prm.to_c();
        uint64_t b = 0;
        check(wob_solve_domain_host(s_, &p, points.data(), n, sum.data(), sumsq ? sumsq->data() : nullptr, &b));
        return b;
    }

    wob_scene handle() const { return s_; }

  private:
    wob_scene s_ = nullptr;
};

namespace utils {

// A point in (-domain_size/2, domain_size/2)^Dim, x fastest (utils.cuh:66-110).
template <unsigned Dim> inline std::array<float, Dim> idx_to_domain_point(unsigned idx, unsigned grid_res, float domain_size) {
    const float dx = domain_size / (float)grid_res;
    std::array<float, Dim> p;
    unsigned r = idx;
    for (unsigned k = 0; k < Dim; k++) {
        p[k] = ((float)(r % grid_res) + 0.5f) * dx - domain_size / 2.0f;
        r /= grid_res;
    }
    return p;
}

// uint32 grid size, then the raw values (runtime_utils.cuh:34-57).
template <typename T> inline void save_field(const std::vector<T> &field, const std::string &filename, unsigned grid_size) {
    std::ofstream out(filename.c_str(), std::ios::out | std::ios::binary);
    if (!out) throw Error(WOB_ERR_INVALID_ARGUMENT, "cannot write " + filename);
    out.write((const char *)&grid_size, sizeof(unsigned));
    out.write((const char *)field.data(), (std::streamsize)(sizeof(T) * field.size()));
}

}  // namespace utils
}  // namespace wob

#endif  // WOB_GB300_HPP
