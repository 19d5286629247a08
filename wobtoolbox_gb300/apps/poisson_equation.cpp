// The Poisson app (apps/poisson_equation.cu) on the GB300 engine: Laplace's operator with the constant
// source 5 on the box (-1, 1)^2 and u = 1 on its four edges, solved with the double-layer backward
// estimator whose volume term samples the source through a volume cache (grid_res^2 cells over the
// box). Same config keys (output_dir, path_length, num_sample_paths, num_volume_samples, grid_res,
// eps, max_time), same evaluation grid (every cell centre of the box), same time-budget iteration
// loop and the same raw_data output (potential<N>.scalar, gradient<N>.vector2, config.json). The
// optional keys "seed" and "max_iterations" are as in the general apps.
//
//   poisson_equation <config.json>
#include "../../include/wob_gb300.hpp"
#include "app_io.hpp"

#include <chrono>
#include <cstdio>
#include <filesystem>
#include <iostream>
#include <limits>
#include <string>
#include <vector>

int main(int argc, char *argv[]) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <config.json>\n", argv[0]);
        return 2;
    }
    try {
        const std::string input_json_file = argv[1];
        const wobapp::Json config = wobapp::read_json_file(input_json_file);
        const std::string output_dir = config["output_dir"].string();
        // Estimator<DL, Interior, Backward, Dirichlet> with one resampling candidate and scaling 1
        // (apps/poisson_equation.cu:43-46)
        wob::EstimatorParams prm;
        prm.bie_model = wob::IndirectDoubleLayer;
        prm.domain = wob::InteriorDomain;
        prm.estimator = wob::BackwardEstimator;
        prm.problem = wob::DirichletProblem;
        prm.path_length = (unsigned)config["path_length"].number();
        prm.num_sample_paths = (unsigned)config["num_sample_paths"].number();
        prm.num_volume_samples = (unsigned)config["num_volume_samples"].number();
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
        std::cout << "#sample paths per iteration\t: " << prm.num_sample_paths << std::endl;
        std::cout << "#num volume samples\t: " << prm.num_volume_samples << std::endl;
        std::cout << "grid resolution\t: " << grid_res << std::endl;
        std::cout << "eps\t: " << prm.eps << std::endl;
        std::cout << "precision\t: float" << std::endl;
        std::cout << "max time\t: " << max_time << " minutes" << std::endl;
        std::cout << "------------------------------------------------------------" << std::endl;
        std::filesystem::create_directories(output_dir);
        std::filesystem::copy(input_json_file, output_dir + "/config.json",
                              std::filesystem::copy_options::overwrite_existing);

        // the box with outward normals and u = 1 (apps/poisson_equation.cu:110-128)
        const float h = 1.0f;
        std::vector<wob::ElementXs<2>> elems;
        auto add = [&](std::array<float, 2> a, std::array<float, 2> b, std::array<float, 2> n) {
            wob::ElementXs<2> e;
            e.a = a;
            e.b = b;
            e.n = n;
            e.boundary_value_a = 1.0f;
            e.boundary_value_b = 1.0f;
            e.boundary_type = wob::Dirichlet;
            elems.push_back(e);
        };
        add({-h, -h}, {-h, h}, {-1.0f, 0.0f});
        add({-h, h}, {h, h}, {0.0f, 1.0f});
        add({h, h}, {h, -h}, {1.0f, 0.0f});
        add({h, -h}, {-h, -h}, {0.0f, -1.0f});
        wob::SceneHost<2> scene(elems);
        // the constant source 5 on the grid over the box (:133-135)
        scene.set_volume_cache(grid_res, 2.0f, std::vector<float>(num_evaluation_points, 5.0f));

        std::vector<float> points(2 * (size_t)num_evaluation_points);
        for (unsigned i = 0; i < num_evaluation_points; i++) {
            const std::array<float, 2> x = wob::utils::idx_to_domain_point<2>(i, grid_res, 2.0f);
            points[2 * (size_t)i] = x[0];
            points[2 * (size_t)i + 1] = x[1];
        }

        // the iteration loop (:151-196)
        std::vector<double> sum(3 * (size_t)num_evaluation_points, 0.0);
        std::vector<float> solution(num_evaluation_points);
        std::vector<std::array<float, 2>> gradient(num_evaluation_points);
        unsigned num_iterations = 0, total_sample_count = 0;
        double elapsed_time = 0.0;
        while (elapsed_time < max_time * 60.0 && (max_iterations == 0 || num_iterations < max_iterations)) {
            num_iterations += 1;
            total_sample_count += prm.num_sample_paths;
            const auto t0 = std::chrono::steady_clock::now();
            scene.solve_domain(prm, points, sum);
            const auto t1 = std::chrono::steady_clock::now();
            elapsed_time += std::chrono::duration<double>(t1 - t0).count();
            prm.path_offset += prm.num_sample_paths;
            std::cout << "\33[2K\rtime " << elapsed_time << " s\t" << num_iterations << " iterations ("
                      << total_sample_count << " samples)\t" << std::flush;
            for (unsigned i = 0; i < num_evaluation_points; i++) {
                solution[i] = (float)(sum[3 * (size_t)i] / (double)total_sample_count);
                gradient[i] = {(float)(sum[3 * (size_t)i + 1] / (double)total_sample_count),
                               (float)(sum[3 * (size_t)i + 2] / (double)total_sample_count)};
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
