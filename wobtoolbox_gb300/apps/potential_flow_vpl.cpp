// The VPL potential-flow app (apps/potential_flow_with_vpl.cu) on the GB300 engine: same config
// keys (output_dir, path_length, num_sample_paths, num_resampling_candidates, grid_res, eps,
// max_time), same scene (a unit flow through the box [-1/2, 1/2]^2 around four circular obstacles),
// same two phases per iteration -- num_sample_paths VPL walks, then the aggregation over every
// (grid point, VPL) pair -- and the same raw_data output (potential<N>.scalar, gradient<N>.vector2,
// NaN inside the obstacles; config.json). The optional keys "seed" and "max_iterations" are as in
// the general apps.
//
//   potential_flow_vpl <config.json>
#include "../../include/wob_gb300.hpp"
#include "app_cuda.hpp"
#include "app_io.hpp"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <filesystem>
#include <iostream>
#include <limits>
#include <string>
#include <vector>

namespace {

struct Circle {
    float cx, cy, r;
    unsigned segments;
};

using wobapp::cuda_check;
using wobapp::DeviceArray;

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
        prm.estimator = wob::BackwardEstimator;
        prm.problem = wob::NeumannProblem;
        prm.path_length = (unsigned)config["path_length"].number();
        const unsigned num_sample_paths = (unsigned)config["num_sample_paths"].number();
        prm.num_sample_paths = 1;
        prm.num_resampling_candidates =
            config.contains("num_resampling_candidates") ? (unsigned)config["num_resampling_candidates"].number() : 1u;
        const unsigned grid_res = (unsigned)config["grid_res"].number();
        prm.eps = config.contains("eps") ? (float)config["eps"].number() : std::numeric_limits<float>::epsilon();
        prm.seed = config.contains("seed") ? (uint64_t)config["seed"].number() : 0u;
        const unsigned max_iterations =
            config.contains("max_iterations") ? (unsigned)config["max_iterations"].number() : 0u;
        const float max_time = (float)config["max_time"].number();
        const unsigned num_evaluation_points = grid_res * grid_res;

        std::cout << "------------------------------------------------------------" << std::endl;
        std::cout << "input json file\t: " << input_json_file << std::endl;
        std::cout << "output directory\t: " << output_dir << std::endl;
        std::cout << "path length\t: " << prm.path_length << std::endl;
        std::cout << "#sample paths per iteration\t: " << num_sample_paths << std::endl;
        std::cout << "#resampling candidates\t: " << prm.num_resampling_candidates << std::endl;
        std::cout << "grid resolution\t: " << grid_res << std::endl;
        std::cout << "eps\t: " << prm.eps << std::endl;
        std::cout << "precision\t: float" << std::endl;
        std::cout << "max time\t: " << max_time << " minutes" << std::endl;
        std::cout << "------------------------------------------------------------" << std::endl;
        std::filesystem::create_directories(output_dir);
        std::filesystem::copy(input_json_file, output_dir + "/config.json",
                              std::filesystem::copy_options::overwrite_existing);

        // the scene (apps/potential_flow_with_vpl.cu:140-176)
        std::vector<wob::ElementXs<2>> elems;
        auto add = [&](std::array<float, 2> a, std::array<float, 2> b, std::array<float, 2> n, float g) {
            wob::ElementXs<2> e;
            e.a = a;
            e.b = b;
            e.n = n;
            e.boundary_value_a = g;
            e.boundary_value_b = g;
            e.boundary_type = wob::Neumann;
            elems.push_back(e);
        };
        add({-0.5f, -0.5f}, {-0.5f, 0.5f}, {-1.0f, 0.0f}, -1.0f);
        add({-0.5f, 0.5f}, {0.5f, 0.5f}, {0.0f, 1.0f}, 0.0f);
        add({0.5f, 0.5f}, {0.5f, -0.5f}, {1.0f, 0.0f}, 1.0f);
        add({0.5f, -0.5f}, {-0.5f, -0.5f}, {0.0f, -1.0f}, 0.0f);
        const Circle circles[4] = {{0.2f, 0.1f, 0.25f, 360}, {-0.25f, 0.3f, 0.15f, 180}, {-0.20f, -0.25f, 0.2f, 180},
                                   {0.25f, -0.3f, 0.05f, 90}};
        for (const Circle &c : circles)
            for (unsigned i = 0; i < c.segments; i++) {
                const float c1 = (float)std::cos((2 * M_PI) * i / c.segments), s1 = (float)std::sin((2 * M_PI) * i / c.segments);
                const float c2 = (float)std::cos((2 * M_PI) * (i + 1) / c.segments);
                const float s2 = (float)std::sin((2 * M_PI) * (i + 1) / c.segments);
                const std::array<float, 2> v1 = {c.cx + c.r * c1, c.cy + c.r * s1};
                const std::array<float, 2> v2 = {c.cx + c.r * c2, c.cy + c.r * s2};
                const float tx = v1[0] - v2[0], ty = v1[1] - v2[1];
                const float l = std::sqrt(tx * tx + ty * ty);
                add(v1, v2, {ty / l, -(tx / l)}, 0.0f);
            }

        // evaluation points outside the obstacles (:178-185)
        std::vector<unsigned> eval_idx;
        std::vector<float> points;
        for (unsigned i = 0; i < num_evaluation_points; i++) {
            const std::array<float, 2> x = wob::utils::idx_to_domain_point<2>(i, grid_res, 1.0f);
            bool inside = false;
            for (const Circle &c : circles) {
                const float dx = x[0] - c.cx, dy = x[1] - c.cy;
                if (dx * dx + dy * dy < c.r * c.r) inside = true;
            }
            if (inside) continue;
            eval_idx.push_back(i);
            points.push_back(x[0]);
            points.push_back(x[1]);
        }
        const uint32_t m = (uint32_t)eval_idx.size();

        wob::SceneHost<2> scene(elems);
        DeviceArray<float> d_points(points.size()), d_vp(2 * (size_t)num_sample_paths), d_vm(num_sample_paths);
        DeviceArray<double> d_sum(3 * (size_t)m);
        cuda_check(cudaMemcpy(d_points.p, points.data(), points.size() * 4, cudaMemcpyHostToDevice), "copying points");
        cuda_check(cudaMemset(d_sum.p, 0, 3 * (size_t)m * 8), "clearing sums");

        unsigned num_iterations = 0, total_sample_count = 0;
        double elapsed_time = 0.0;
        std::vector<double> sum(3 * (size_t)m);
        std::vector<float> solution(num_evaluation_points);
        std::vector<std::array<float, 2>> gradient(num_evaluation_points);
        while (elapsed_time < max_time * 60.0 && (max_iterations == 0 || num_iterations < max_iterations)) {
            num_iterations += 1;
            total_sample_count += num_sample_paths;
            const auto t0 = std::chrono::steady_clock::now();
            const wob_params p = prm.to_c();
            wob::check(wob_vpl_paths(scene.handle(), &p, num_sample_paths, d_vp.p, d_vm.p, nullptr, nullptr));
            wob::check(wob_vpl_aggregate(scene.handle(), prm.eps, d_vp.p, d_vm.p, num_sample_paths, d_points.p, m,
                                         d_sum.p, nullptr));
            cuda_check(cudaDeviceSynchronize(), "running the iteration");
            const auto t1 = std::chrono::steady_clock::now();
            elapsed_time += std::chrono::duration<double>(t1 - t0).count();
            prm.path_offset += num_sample_paths;
            std::cout << "\33[2K\rtime " << elapsed_time << " s\t" << num_iterations << " iterations ("
                      << total_sample_count << " samples)\t" << std::flush;
            cuda_check(cudaMemcpy(sum.data(), d_sum.p, sum.size() * 8, cudaMemcpyDeviceToHost), "reading sums");
            for (unsigned i = 0; i < num_evaluation_points; i++) {
                solution[i] = std::numeric_limits<float>::quiet_NaN();
                gradient[i] = {0.0f, 0.0f};
            }
            for (uint32_t j = 0; j < m; j++) {
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
    } catch (const std::exception &ex) {
        std::cerr << "error: " << ex.what() << std::endl;
        return 1;
    }
    return 0;
}
