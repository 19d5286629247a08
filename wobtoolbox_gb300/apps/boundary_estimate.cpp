// The boundary-estimate app (apps/boundary_estimate.cu) on the GB300 engine: an interior Neumann
// problem on a circle of radius 1/2 (720 segments; flux in through two pairs of segments, out through
// two others, in each third), solved with the single-layer forward estimator first on the grid inside
// the circle, then exactly on the boundary at the 720 segment midpoints. Same config keys
// (output_dir, path_length, num_sample_paths_domain, num_sample_paths_boundary,
// num_resampling_candidates, grid_res, eps, max_time), each phase with its own time budget, and the
// same raw_data output (potential<N>.scalar, gradient<N>.vector2 with NaN / 0 outside the circle,
// boundary_solution<N>.scalar: uint32 720 then 720 floats; config.json). As in the reference, the
// estimator runs with one resampling candidate whatever num_resampling_candidates says. The optional
// keys "seed" and "max_iterations" (per phase) are as in the general apps.
//
//   boundary_estimate <config.json>
#include "../../include/wob_gb300.hpp"
#include "app_cuda.hpp"
#include "app_io.hpp"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <limits>
#include <string>
#include <vector>

namespace {

constexpr unsigned kSegments = 720;

// vertex i of the circle, computed in double and stored as float (apps/boundary_estimate.cu:164-169)
std::array<float, 2> circle_vertex(unsigned i) {
    const double r = 0.5f;
    return {(float)(r * std::sin((2 * M_PI) * i / kSegments)), (float)(r * std::cos((2 * M_PI) * i / kSegments))};
}

// n = (t_y, -t_x), t = (v1 - v2) / |v1 - v2| (:170-171): the outward normal of this clockwise circle
std::array<float, 2> outward_normal(const std::array<float, 2> &v1, const std::array<float, 2> &v2) {
    const float tx = v1[0] - v2[0], ty = v1[1] - v2[1];
    const float l = std::sqrt(tx * tx + ty * ty);
    return {ty / l, -(tx / l)};
}

}  // namespace

int main(int argc, char *argv[]) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <config.json>\n", argv[0]);
        return 2;
    }
    try {
        const std::string input_json_file = argv[1];
        const wobapp::Json config = wobapp::read_json_file(input_json_file);
        const std::string output_dir = config["output_dir"].string();
        wob::EstimatorParams prm;
        prm.bie_model = wob::IndirectSingleLayer;
        prm.domain = wob::InteriorDomain;
        prm.estimator = wob::ForwardEstimator;
        prm.problem = wob::NeumannProblem;
        prm.path_length = (unsigned)config["path_length"].number();
        const unsigned num_sample_paths_domain = (unsigned)config["num_sample_paths_domain"].number();
        const unsigned num_sample_paths_boundary = (unsigned)config["num_sample_paths_boundary"].number();
        const unsigned num_resampling_candidates =
            config.contains("num_resampling_candidates") ? (unsigned)config["num_resampling_candidates"].number() : 1u;
        prm.num_resampling_candidates = 1;  // apps/boundary_estimate.cu:49-52, :70-73
        const unsigned grid_res = (unsigned)config["grid_res"].number();
        prm.eps = config.contains("eps") ? (float)config["eps"].number() : std::numeric_limits<float>::epsilon();
        prm.seed = config.contains("seed") ? (uint64_t)config["seed"].number() : 0u;
        const unsigned max_iterations =
            config.contains("max_iterations") ? (unsigned)config["max_iterations"].number() : 0u;
        const unsigned num_evaluation_points = grid_res * grid_res;
        const float max_time = (float)config["max_time"].number();

        std::cout << "------------------------------------------------------------" << std::endl;
        std::cout << "input json file\t: " << input_json_file << std::endl;
        std::cout << "output directory\t: " << output_dir << std::endl;
        std::cout << "path length\t: " << prm.path_length << std::endl;
        std::cout << "#sample paths domain per iteration\t: " << num_sample_paths_domain << std::endl;
        std::cout << "#sample paths boundary per iteration\t: " << num_sample_paths_boundary << std::endl;
        std::cout << "#resampling candidates\t: " << num_resampling_candidates << std::endl;
        std::cout << "grid resolution\t: " << grid_res << std::endl;
        std::cout << "eps\t: " << prm.eps << std::endl;
        std::cout << "precision\t: float" << std::endl;
        std::cout << "max time\t: " << max_time << " minutes" << std::endl;
        std::cout << "------------------------------------------------------------" << std::endl;
        std::filesystem::create_directories(output_dir);
        std::filesystem::copy(input_json_file, output_dir + "/config.json",
                              std::filesystem::copy_options::overwrite_existing);

        // the scene: inward element normals -n; data (1, 200) on segments i mod 240 in {0, 239},
        // (-1, -200) on {119, 120}, 0 elsewhere (:162-180)
        std::vector<wob::ElementXs<2>> elems;
        for (unsigned i = 0; i < kSegments; i++) {
            const std::array<float, 2> v1 = circle_vertex(i), v2 = circle_vertex(i + 1);
            const std::array<float, 2> n = outward_normal(v1, v2);
            wob::ElementXs<2> e;
            e.a = v1;
            e.b = v2;
            e.n = {-n[0], -n[1]};
            e.boundary_type = wob::Neumann;
            const float neumann_boundary_value = 200.0f;
            if (i % 240 == 0 || i % 240 == 239) {
                e.boundary_value_a = 1.0f;
                e.boundary_value_b = neumann_boundary_value;
            } else if (i % 240 == 120 || i % 240 == 119) {
                e.boundary_value_a = -1.0f;
                e.boundary_value_b = -neumann_boundary_value;
            } else {
                e.boundary_value_a = 0.0f;
                e.boundary_value_b = 0.0f;
            }
            elems.push_back(e);
        }
        wob::SceneHost<2> scene(elems);

        // grid points inside the circle (:182-186)
        std::vector<unsigned> eval_idx;
        std::vector<float> points;
        for (unsigned i = 0; i < num_evaluation_points; i++) {
            const std::array<float, 2> x = wob::utils::idx_to_domain_point<2>(i, grid_res, 1.0f);
            if (std::sqrt(x[0] * x[0] + x[1] * x[1]) <= 0.5f) {
                eval_idx.push_back(i);
                points.push_back(x[0]);
                points.push_back(x[1]);
            }
        }
        const size_t m = eval_idx.size();

        // phase 1: the domain (:209-246)
        std::cout << "computing solution in the domain" << std::endl;
        prm.num_sample_paths = num_sample_paths_domain;
        std::vector<double> sum(3 * m, 0.0);
        std::vector<float> solution(num_evaluation_points);
        std::vector<std::array<float, 2>> gradient(num_evaluation_points);
        unsigned num_iterations = 0, total_sample_count = 0;
        double elapsed_time = 0.0;
        while (elapsed_time < max_time * 60.0 && (max_iterations == 0 || num_iterations < max_iterations)) {
            num_iterations += 1;
            total_sample_count += num_sample_paths_domain;
            const auto t0 = std::chrono::steady_clock::now();
            scene.solve_domain(prm, points, sum);
            const auto t1 = std::chrono::steady_clock::now();
            elapsed_time += std::chrono::duration<double>(t1 - t0).count();
            prm.path_offset += num_sample_paths_domain;
            std::cout << "\33[2K\rtime " << elapsed_time << " s\t" << num_iterations << " iterations ("
                      << total_sample_count << " samples)\t" << std::flush;
            for (unsigned i = 0; i < num_evaluation_points; i++) {
                solution[i] = std::numeric_limits<float>::quiet_NaN();
                gradient[i] = {0.0f, 0.0f};
            }
            for (size_t j = 0; j < m; j++) {
                solution[eval_idx[j]] = (float)(sum[3 * j] / (double)total_sample_count);
                gradient[eval_idx[j]] = {(float)(sum[3 * j + 1] / (double)total_sample_count),
                                         (float)(sum[3 * j + 2] / (double)total_sample_count)};
            }
            wob::utils::save_field(solution, output_dir + "/potential" + std::to_string(num_iterations) + ".scalar",
                                   grid_res);
            wob::utils::save_field(gradient, output_dir + "/gradient" + std::to_string(num_iterations) + ".vector2",
                                   grid_res);
        }
        std::cout << std::endl;

        // phase 2: the segment midpoints with the outward normal, interior angle 1/2, Neumann data 0
        // (:65-95, :248-291)
        std::vector<float> bp(2 * kSegments), bn(2 * kSegments), angle(kSegments, 0.5f), bval(kSegments, 0.0f),
            alpha(kSegments, 0.0f);
        std::vector<int32_t> btype(kSegments, (int32_t)wob::Neumann);
        for (unsigned i = 0; i < kSegments; i++) {
            const std::array<float, 2> v1 = circle_vertex(i), v2 = circle_vertex(i + 1);
            const std::array<float, 2> n = outward_normal(v1, v2);
            bp[2 * i] = (v1[0] + v2[0]) / 2.0f;
            bp[2 * i + 1] = (v1[1] + v2[1]) / 2.0f;
            bn[2 * i] = n[0];
            bn[2 * i + 1] = n[1];
        }
        wobapp::DeviceArray<float> d_p(bp), d_n(bn), d_angle(angle), d_bval(bval), d_alpha(alpha);
        wobapp::DeviceArray<int32_t> d_type(btype);
        wobapp::DeviceArray<double> d_sum(kSegments);
        d_sum.zero();
        std::cout << "computing solution on boundary" << std::endl;
        prm.num_sample_paths = num_sample_paths_boundary;
        prm.path_offset = 0;
        std::vector<double> bsum;
        std::vector<float> boundary_solution(kSegments);
        num_iterations = 0;
        total_sample_count = 0;
        elapsed_time = 0.0;
        while (elapsed_time < max_time * 60.0 && (max_iterations == 0 || num_iterations < max_iterations)) {
            num_iterations += 1;
            total_sample_count += num_sample_paths_boundary;
            const auto t0 = std::chrono::steady_clock::now();
            const wob_params p = prm.to_c();
            wob::check(wob_solve_boundary(scene.handle(), &p, d_p.p, d_n.p, d_angle.p, d_bval.p, d_type.p, d_alpha.p,
                                          kSegments, d_sum.p, nullptr, nullptr, nullptr));
            wobapp::cuda_check(cudaDeviceSynchronize(), "running the iteration");
            const auto t1 = std::chrono::steady_clock::now();
            elapsed_time += std::chrono::duration<double>(t1 - t0).count();
            prm.path_offset += num_sample_paths_boundary;
            std::cout << "\33[2K\rtime " << elapsed_time << " s\t" << num_iterations << " iterations ("
                      << total_sample_count << " samples)\t" << std::flush;
            d_sum.download(bsum);
            for (unsigned i = 0; i < kSegments; i++)
                boundary_solution[i] = (float)(bsum[i] / (double)total_sample_count);
            const std::string filename = output_dir + "/boundary_solution" + std::to_string(num_iterations) + ".scalar";
            std::ofstream out(filename.c_str(), std::ios::out | std::ios::binary);
            if (!out) throw std::runtime_error("cannot write " + filename);
            const unsigned count = kSegments;
            out.write((const char *)&count, sizeof(unsigned));
            out.write((const char *)boundary_solution.data(), (std::streamsize)(sizeof(float) * kSegments));
        }
        std::cout << std::endl;
    } catch (const std::exception &ex) {
        std::cerr << "error: " << ex.what() << std::endl;
        return 1;
    }
    return 0;
}
