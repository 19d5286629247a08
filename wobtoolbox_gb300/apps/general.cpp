// The JSON apps general_2d / general_3d (apps/general_2d.cu, apps/general_3d.cu) on the GB300
// engine: same config file, same OBJ input and normalisation, same boundary data from the closed-form
// solutions, same evaluation grid and winding-number mask, same time-budget iteration loop and the
// same raw_data output (potential_analytical.scalar, gradient_analytical.vector<D>,
// potential<N>.scalar, gradient<N>.vector<D>, rmse_list.csv, config.json).
//
//   general_2d <config.json> [--setup-only]      (WOB_APP_DIM = 2; general_3d with 3)
//
// Differences from the reference apps, each deliberate:
// * the optional config keys "seed" (Philox seed of the walks and of the Mixed problem's random
//   boundary types; the reference draws the types from std::random_device) and "max_iterations"
//   (stop after that many iterations even if max_time is not used up);
// * the RMSE is accumulated in double over the normalised estimates (the 3D reference passes the
//   unnormalised sums to compute_rmse, apps/general_3d.cu:367-368);
// * for the Neumann shift, when the reference point (grid centre, or cell 0 outside) is not an
//   evaluated point, the first evaluated point is used instead of propagating NaN;
// * --setup-only stops after the analytical fields are written (no GPU needed);
// * rmse_list.csv carries two more columns after the reference's (sample count, time, RMSE of u
//   and of each gradient component): the iteration's bounces per second and the cumulative bounce
//   count;
// * after every iteration the running FP64 sums, the iteration and sample counts, the elapsed time
//   and the next Philox path offset are written to checkpoint.bin in the output directory; with the
//   optional key "resume": true a run continues from that file. The walks are indexed by their
//   path offset, so a resumed run writes bit for bit the fields an uninterrupted run would.
#include "../../include/wob_gb300.hpp"
#include "app_io.hpp"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <limits>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#ifndef WOB_APP_DIM
#define WOB_APP_DIM 2
#endif

namespace {

constexpr unsigned Dim = WOB_APP_DIM;
using Vec = std::array<float, Dim>;
using VecG = std::array<float, Dim + 1>;  // [u, grad u]

// apps/general_2d.cu:73-95, apps/general_3d.cu:75-98
enum SolutionType { INTERIOR_SOLUTION2, EXTERIOR_SOLUTION1 };

VecG analytical_solution(SolutionType t, const Vec &y) {
    VecG r{};
    const float pi = (float)M_PI;
#if WOB_APP_DIM == 2
    {
        if (t == EXTERIOR_SOLUTION1) {
            const float s = y[0] * y[0] + y[1] * y[1];
            r = {y[0] / s, 1.f / s - 2.f * y[0] * y[0] / (s * s), -2.f * y[0] * y[1] / (s * s)};
        } else {
            r = {std::cos(pi * y[0]) * std::sinh(pi * y[1]), -pi * std::sin(pi * y[0]) * std::sinh(pi * y[1]),
                 pi * std::cos(pi * y[0]) * std::cosh(pi * y[1])};
        }
    }
#else
    {
        if (t == EXTERIOR_SOLUTION1) {
            const float s = y[0] * y[0] + y[1] * y[1] + y[2] * y[2];
            const float n = std::sqrt(s);
            r = {y[2] / (s * n), -3.f * y[2] * y[0] / (s * s * n), -3.f * y[2] * y[1] / (s * s * n),
                 1.f / (s * n) - 3.f * y[2] * y[2] / (s * s * n)};
        } else {
            r = {-std::cos(pi * y[1]) * std::sinh(pi * y[2]), 0.0f, pi * std::sin(pi * y[1]) * std::sinh(pi * y[2]),
                 -pi * std::cos(pi * y[1]) * std::cosh(pi * y[2])};
        }
    }
#endif
    return r;
}
float dirichlet_bc(SolutionType t, const Vec &y) { return analytical_solution(t, y)[0]; }
float neumann_bc(SolutionType t, const Vec &y, const Vec &n) {
    const VecG g = analytical_solution(t, y);
    float d = 0.0f;
    for (unsigned k = 0; k < Dim; k++) d = d + g[1 + k] * n[k];
    return d;
}

// x of grid cell idx: the 2D cell centre, in 3D on the slice x = 0 (apps/general_3d.cu:57-58)
Vec grid_point(unsigned idx, unsigned grid_res) {
    const std::array<float, 2> p = wob::utils::idx_to_domain_point<2>(idx, grid_res, 1.0f);
#if WOB_APP_DIM == 2
    return {p[0], p[1]};
#else
    return {0.0f, p[1], p[0]};
#endif
}

}  // namespace

int main(int argc, char *argv[]) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <config.json> [--setup-only]\n", argv[0]);
        return 2;
    }
    const std::string input_json_file = argv[1];
    const bool setup_only = argc > 2 && std::string(argv[2]) == "--setup-only";
    try {
        const wobapp::Json config = wobapp::read_json_file(input_json_file);
        const std::string input_obj_file = config["input_obj_file"].string();
        const std::string output_dir = config["output_dir"].string();
        wob::EstimatorParams prm;
        prm.path_length = (unsigned)config["path_length"].number();
        prm.num_sample_paths = (unsigned)config["num_sample_paths"].number();
        prm.num_resampling_candidates =
            config.contains("num_resampling_candidates") ? (unsigned)config["num_resampling_candidates"].number() : 1u;
        const unsigned grid_res = (unsigned)config["grid_res"].number();
        prm.eps = config.contains("eps") ? (float)config["eps"].number() : std::numeric_limits<float>::epsilon();
        prm.first_kind_equation_scaling_constant = config.contains("first_kind_equation_scaling_constant")
                                                       ? (float)config["first_kind_equation_scaling_constant"].number()
                                                       : 1.0f;
        prm.seed = config.contains("seed") ? (uint64_t)config["seed"].number() : 0u;
        const unsigned max_iterations =
            config.contains("max_iterations") ? (unsigned)config["max_iterations"].number() : 0u;
        const bool resume = config.contains("resume") && config["resume"].boolean();
        const unsigned num_evaluation_points = grid_res * grid_res;
        const float max_time = (float)config["max_time"].number();
        const wob::EquationKernelType equation_kernel =
            wob::string_to_equation_kernel_type(config["equation_kernel"].string());
        prm.bie_model = wob::string_to_bie_model_type(config["bie_model"].string());
        prm.domain = wob::string_to_domain_type(config["domain"].string());
        prm.estimator = wob::string_to_estimator_type(config["estimator"].string());
        prm.problem = wob::string_to_problem_type(config["problem"].string());
        if (equation_kernel == wob::EquationKernelTypeCount || prm.bie_model == wob::BIEModelTypeCount ||
            prm.domain == wob::DomainTypeCount || prm.estimator == wob::EstimatorTypeCount ||
            prm.problem == wob::ProblemTypeCount)
            throw std::runtime_error("config: unknown equation_kernel / bie_model / domain / estimator / problem");

        // geometry (apps/general_2d.cu:197-207, apps/general_3d.cu:201-216), in float like the reference
        const wobapp::Mesh mesh = wobapp::read_obj(input_obj_file);
        std::vector<Vec> V(mesh.nv());
        for (size_t i = 0; i < mesh.nv(); i++)
            for (unsigned k = 0; k < Dim; k++) V[i][k] = (float)mesh.V[3 * i + k];
#if WOB_APP_DIM == 3
        {
            Vec mn = V[0], mx = V[0];
            for (const Vec &v : V)
                for (unsigned k = 0; k < 3; k++) {
                    mn[k] = std::min(mn[k], v[k]);
                    mx[k] = std::max(mx[k], v[k]);
                }
            Vec size, shift;
            float s = 0.0f;
            for (unsigned k = 0; k < 3; k++) {
                size[k] = mx[k] - mn[k];
                shift[k] = mn[k] + 0.5f * size[k];
                s = std::max(s, size[k]);
            }
            const float inv = (float)(1.0 / (double)s);
            for (Vec &v : V)
                for (unsigned k = 0; k < 3; k++) v[k] = (v[k] - shift[k]) * inv;
        }
#endif
        if (prm.domain == wob::ExteriorDomain)
            for (Vec &v : V) {
                for (unsigned k = 0; k < Dim; k++) v[k] *= 0.5f;
                v[1] += Dim == 2 ? 0.0625f : 0.05f;
            }

        std::cout << "------------------------------------------------------------" << std::endl;
        std::cout << "input json file\t: " << input_json_file << std::endl;
        std::cout << "input obj file\t: " << input_obj_file << std::endl;
        std::cout << " ( #faces: " << mesh.nf() << " )" << std::endl;
        std::cout << "output directory\t: " << output_dir << std::endl;
        std::cout << "path length\t: " << prm.path_length << std::endl;
        std::cout << "#sample paths\t: " << prm.num_sample_paths << std::endl;
        std::cout << "#resampling candidates\t: " << prm.num_resampling_candidates << std::endl;
        std::cout << "grid resolution\t: " << grid_res << std::endl;
        std::cout << "eps\t: " << prm.eps << std::endl;
        std::cout << "first kind equation scaling constant\t: " << prm.first_kind_equation_scaling_constant << std::endl;
        std::cout << "precision\t: float" << std::endl;
        std::cout << "max time\t: " << max_time << " minutes" << std::endl;
        std::cout << "equation type\t: " << wob::equation_kernel_type_to_string(equation_kernel) << std::endl;
        std::cout << "BIE model type\t: " << wob::bie_model_type_to_string(prm.bie_model) << std::endl;
        std::cout << "domain type\t: " << wob::domain_type_to_string(prm.domain) << std::endl;
        std::cout << "estimator type\t: " << wob::estimator_type_to_string(prm.estimator) << std::endl;
        std::cout << "problem type\t: " << wob::problem_type_to_string(prm.problem) << std::endl;
        std::cout << "------------------------------------------------------------" << std::endl;

        std::filesystem::create_directories(output_dir);
        std::filesystem::copy(input_json_file, output_dir + "/config.json",
                              std::filesystem::copy_options::overwrite_existing);

        // elements and boundary data (apps/general_2d.cu:238-270, apps/general_3d.cu:251-288)
        const SolutionType solution_type = prm.domain == wob::InteriorDomain ? INTERIOR_SOLUTION2 : EXTERIOR_SOLUTION1;
        std::mt19937 mt((uint32_t)prm.seed);
        std::uniform_int_distribution<int> dist(0, 2);
        std::vector<wob::ElementXs<Dim>> elems;
        std::vector<double> soup;  // for the winding number
        for (size_t f = 0; f < mesh.nf(); f++) {
            wob::ElementXs<Dim> e;
            const Vec v1 = V[mesh.F[3 * f]], v2 = V[mesh.F[3 * f + 1]];
            Vec n;
#if WOB_APP_DIM == 2
            // n = (t_y, -t_x), t = (v1 - v2) / |v1 - v2| (apps/general_2d.cu:245-249)
            const float tx = v1[0] - v2[0], ty = v1[1] - v2[1];
            const float l = std::sqrt(tx * tx + ty * ty);
            n = {ty / l, -(tx / l)};
            e.a = v1;
            e.b = v2;
            for (unsigned k = 0; k < 2; k++) soup.push_back(v1[k]);
            for (unsigned k = 0; k < 2; k++) soup.push_back(v2[k]);
#else
            // per-face normal (v2 - v1) x (v3 - v1) / |.| (igl::per_face_normals, apps/general_3d.cu:251-252)
            const Vec v3 = V[mesh.F[3 * f + 2]];
            const float e1[3] = {v2[0] - v1[0], v2[1] - v1[1], v2[2] - v1[2]};
            const float e2[3] = {v3[0] - v1[0], v3[1] - v1[1], v3[2] - v1[2]};
            const float c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                e1[0] * e2[1] - e1[1] * e2[0]};
            const float l = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
            n = {c[0] / l, c[1] / l, c[2] / l};
            e.a = v1;
            e.b = v2;
            e.c = v3;
            for (const Vec *v : {&v1, &v2, &v3})
                for (unsigned k = 0; k < 3; k++) soup.push_back((*v)[k]);
#endif
            e.n = n;
            const wob::BoundaryType bt =
                prm.problem == wob::MixedProblem ? (wob::BoundaryType)dist(mt) : (wob::BoundaryType)prm.problem;
            e.boundary_type = bt;
            auto data = [&](const Vec &y) {
                if (bt == wob::Dirichlet) return dirichlet_bc(solution_type, y);
                if (bt == wob::Neumann) return neumann_bc(solution_type, y, n);
                return dirichlet_bc(solution_type, y) + neumann_bc(solution_type, y, n);
            };
            e.boundary_value_a = data(v1);
            e.boundary_value_b = data(v2);
#if WOB_APP_DIM == 3
            e.boundary_value_c = data(v3);
#endif
            if (bt == wob::Robin) {
                e.robin_alpha_a = 1.0f;
                e.robin_alpha_b = 1.0f;
#if WOB_APP_DIM == 3
                e.robin_alpha_c = 1.0f;
#endif
            }
            elems.push_back(e);
        }

        // evaluation grid, winding-number mask, analytical fields (apps/general_2d.cu:272-292)
        std::vector<float> analytical(num_evaluation_points);
        std::vector<Vec> analytical_gradient(num_evaluation_points);
        std::vector<char> evaluate(num_evaluation_points, 0);
#pragma omp parallel for schedule(dynamic, 64)
        for (long long ii = 0; ii < (long long)num_evaluation_points; ii++) {
            const unsigned i = (unsigned)ii;
            const Vec x = grid_point(i, grid_res);
            double xd[3] = {0.0, 0.0, 0.0};
            for (unsigned k = 0; k < Dim; k++) xd[k] = x[k];
            const double w = Dim == 2 ? wobapp::winding_number_2d(soup, xd) : wobapp::winding_number_3d(soup, xd);
            // apps/general_2d.cu:281 (clockwise boundary: -1 inside), apps/general_3d.cu:297
            const bool inside = Dim == 2 ? (prm.domain == wob::InteriorDomain ? w < -0.5 : w >= -0.5)
                                         : (prm.domain == wob::InteriorDomain ? w > 0.5 : w <= 0.5);
            if (inside) {
                const VecG a = analytical_solution(solution_type, x);
                analytical[i] = a[0];
                for (unsigned k = 0; k < Dim; k++) analytical_gradient[i][k] = a[1 + k];
                evaluate[i] = 1;
            } else {
                analytical[i] = std::numeric_limits<float>::quiet_NaN();
                analytical_gradient[i].fill(0.0f);
            }
        }
        const std::string gsuffix = Dim == 2 ? ".vector2" : ".vector3";
        wob::utils::save_field(analytical, output_dir + "/potential_analytical.scalar", grid_res);
        wob::utils::save_field(analytical_gradient, output_dir + "/gradient_analytical" + gsuffix, grid_res);
        std::vector<unsigned> eval_idx;
        for (unsigned i = 0; i < num_evaluation_points; i++)
            if (evaluate[i]) eval_idx.push_back(i);
        std::cout << "evaluation points\t: " << eval_idx.size() << std::endl;
        if (setup_only) return 0;

        wob::SceneHost<Dim> scene(elems);
        const size_t m = eval_idx.size();
        std::vector<float> points(m * Dim);
        for (size_t j = 0; j < m; j++) {
            const Vec x = grid_point(eval_idx[j], grid_res);
            for (unsigned k = 0; k < Dim; k++) points[j * Dim + k] = x[k];
        }
        std::vector<double> sum(m * (Dim + 1), 0.0);

        // the iteration loop (apps/general_2d.cu:327-367)
        unsigned num_iterations = 0, total_sample_count = 0;
        double elapsed_time = 0.0;
        const std::string ckpt_path = output_dir + "/checkpoint.bin";
        struct CkptHeader {
            char magic[8];
            uint32_t dim, grid_res, num_iterations, total_sample_count;
            uint64_t points, path_offset, seed;
            double elapsed_time;
        };
        if (resume) {
            std::ifstream in(ckpt_path, std::ios::binary);
            if (!in) throw std::runtime_error("resume: no " + ckpt_path);
            CkptHeader h{};
            in.read(reinterpret_cast<char *>(&h), sizeof h);
            if (!in || std::string(h.magic, 8) != "WOBCKPT1" || h.dim != Dim || h.grid_res != grid_res ||
                h.points != m || h.seed != prm.seed)
                throw std::runtime_error("resume: " + ckpt_path + " belongs to another run");
            in.read(reinterpret_cast<char *>(sum.data()), (std::streamsize)(sum.size() * sizeof(double)));
            if (!in) throw std::runtime_error("resume: " + ckpt_path + " is truncated");
            num_iterations = h.num_iterations;
            total_sample_count = h.total_sample_count;
            prm.path_offset = h.path_offset;
            elapsed_time = h.elapsed_time;
            std::cout << "resuming after " << num_iterations << " iterations (" << total_sample_count << " samples)"
                      << std::endl;
        }
        std::ofstream rmse_out(output_dir + "/rmse_list.csv", resume ? std::ios::app : std::ios::trunc);
        uint64_t total_bounces = 0;
        std::vector<float> solution(num_evaluation_points);
        std::vector<Vec> gradient(num_evaluation_points);
        while (elapsed_time < max_time * 60.0 && (max_iterations == 0 || num_iterations < max_iterations)) {
            num_iterations += 1;
            total_sample_count += prm.num_sample_paths;
            const auto t0 = std::chrono::steady_clock::now();
            const uint64_t iter_bounces = scene.solve_domain(prm, points, sum);
            const auto t1 = std::chrono::steady_clock::now();
            const double iter_time = std::chrono::duration<double>(t1 - t0).count();
            elapsed_time += iter_time;
            total_bounces += iter_bounces;
            prm.path_offset += prm.num_sample_paths;
            {
                CkptHeader h{};
                std::memcpy(h.magic, "WOBCKPT1", 8);
                h.dim = Dim;
                h.grid_res = grid_res;
                h.num_iterations = num_iterations;
                h.total_sample_count = total_sample_count;
                h.points = m;
                h.path_offset = prm.path_offset;
                h.seed = prm.seed;
                h.elapsed_time = elapsed_time;
                std::ofstream ck(ckpt_path + ".tmp", std::ios::binary | std::ios::trunc);
                ck.write(reinterpret_cast<const char *>(&h), sizeof h);
                ck.write(reinterpret_cast<const char *>(sum.data()), (std::streamsize)(sum.size() * sizeof(double)));
                ck.close();
                std::filesystem::rename(ckpt_path + ".tmp", ckpt_path);
            }

            for (unsigned i = 0; i < num_evaluation_points; i++) {
                solution[i] = std::numeric_limits<float>::quiet_NaN();
                gradient[i].fill(0.0f);
            }
            for (size_t j = 0; j < m; j++) {
                const unsigned i = eval_idx[j];
                solution[i] = (float)(sum[j * (Dim + 1)] / (double)total_sample_count);
                for (unsigned k = 0; k < Dim; k++)
                    gradient[i][k] = (float)(sum[j * (Dim + 1) + 1 + k] / (double)total_sample_count);
            }
            // Neumann problems: shift so the estimate matches the exact value at a reference point
            if (prm.problem == wob::NeumannProblem && m > 0) {
                unsigned ref = prm.domain == wob::InteriorDomain ? grid_res * (grid_res / 2) + grid_res / 2 : 0u;
                if (!evaluate[ref]) ref = eval_idx[0];
                const float offset = solution[ref] - analytical_solution(solution_type, grid_point(ref, grid_res))[0];
                for (size_t j = 0; j < m; j++) solution[eval_idx[j]] -= offset;
            }
            double se[Dim + 1] = {};
            for (size_t j = 0; j < m; j++) {
                const unsigned i = eval_idx[j];
                const VecG a = analytical_solution(solution_type, grid_point(i, grid_res));
                se[0] += std::pow((double)solution[i] - a[0], 2);
                for (unsigned k = 0; k < Dim; k++) se[1 + k] += std::pow((double)gradient[i][k] - a[1 + k], 2);
            }
            std::cout << "\33[2K\rtime " << elapsed_time << " s\t" << num_iterations << " iterations ("
                      << total_sample_count << " samples)\tRMSE :";
            rmse_out << total_sample_count << "," << elapsed_time;
            for (unsigned c = 0; c <= Dim; c++) {
                const double r = m ? std::sqrt(se[c] / (double)m) : 0.0;
                std::cout << " " << r;
                rmse_out << "," << r;
            }
            std::cout << std::flush;
            rmse_out << "," << (iter_time > 0.0 ? (double)iter_bounces / iter_time : 0.0) << "," << total_bounces;
            rmse_out << std::endl;
            wob::utils::save_field(solution, output_dir + "/potential" + std::to_string(num_iterations) + ".scalar",
                                   grid_res);
            wob::utils::save_field(gradient, output_dir + "/gradient" + std::to_string(num_iterations) + gsuffix,
                                   grid_res);
        }
        std::cout << std::endl;
    } catch (const std::exception &ex) {
        std::cerr << "error: " << ex.what() << std::endl;
        return 1;
    }
    return 0;
}
