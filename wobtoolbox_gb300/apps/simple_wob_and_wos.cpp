// The WoB / WoS comparison app (apps/simple_wob_and_wos.cu) on the GB300 engine: an interior
// Dirichlet problem on a 2D OBJ outline whose boundary data alternate between -1 and 1 over 40
// pieces of equal arc length, solved either with walk on boundary (the double-layer backward
// estimator with line-intersection sampling, :80-107) or with walk on spheres (:110-137). Same config
// keys (input_obj_file, output_dir, is_wos, evaluate_at_all_points, path_length, num_sample_paths,
// grid_res, eps, max_time), same winding-number mask, same time-budget iteration loop and the same
// raw_data output (potential<N>.scalar with NaN at the points not evaluated; config.json). The
// optional keys "seed" and "max_iterations" are as in the general apps.
//
//   simple_wob_and_wos <config.json> [--setup-only]
//
// --setup-only stops after the scene and the evaluation mask are set up (no GPU needed).
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

int main(int argc, char *argv[]) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <config.json> [--setup-only]\n", argv[0]);
        return 2;
    }
    const bool setup_only = argc > 2 && std::string(argv[2]) == "--setup-only";
    try {
        const std::string input_json_file = argv[1];
        const wobapp::Json config = wobapp::read_json_file(input_json_file);
        const std::string input_obj_file = config["input_obj_file"].string();
        const std::string output_dir = config["output_dir"].string();
        const bool is_wos = config["is_wos"].boolean();
        const bool evaluate_at_all_points =
            config.contains("evaluate_at_all_points") ? config["evaluate_at_all_points"].boolean() : false;
        wob::EstimatorParams prm;
        prm.bie_model = wob::IndirectDoubleLayer;
        prm.domain = wob::InteriorDomain;
        prm.estimator = wob::BackwardEstimator;
        prm.problem = wob::DirichletProblem;
        prm.path_length = is_wos ? 1u : (unsigned)config["path_length"].number();
        prm.num_sample_paths = (unsigned)config["num_sample_paths"].number();
        const unsigned grid_res = (unsigned)config["grid_res"].number();
        prm.eps = config.contains("eps") ? (float)config["eps"].number() : std::numeric_limits<float>::epsilon();
        prm.seed = config.contains("seed") ? (uint64_t)config["seed"].number() : 0u;
        const unsigned max_iterations =
            config.contains("max_iterations") ? (unsigned)config["max_iterations"].number() : 0u;
        const unsigned num_evaluation_points = grid_res * grid_res;
        const float max_time = (float)config["max_time"].number();

        // the outline: x and y of the vertices, the first two corners of each face (:171-178)
        const wobapp::Mesh mesh = wobapp::read_obj(input_obj_file);
        std::vector<std::array<float, 2>> V(mesh.nv());
        for (size_t i = 0; i < mesh.nv(); i++) V[i] = {(float)mesh.V[3 * i], (float)mesh.V[3 * i + 1]};

        std::cout << "------------------------------------------------------------" << std::endl;
        std::cout << "input json file\t: " << input_json_file << std::endl;
        std::cout << "input obj file\t: " << input_obj_file << std::endl;
        std::cout << " ( #line segments: " << mesh.nf() << " )" << std::endl;
        std::cout << "output directory\t: " << output_dir << std::endl;
        if (!is_wos) std::cout << "path length\t: " << prm.path_length << std::endl;
        std::cout << "#sample paths per iteration\t: " << prm.num_sample_paths << std::endl;
        std::cout << "grid resolution\t: " << grid_res << std::endl;
        std::cout << "eps\t: " << prm.eps << std::endl;
        std::cout << "precision\t: float" << std::endl;
        std::cout << "max time\t: " << max_time << " minutes" << std::endl;
        std::cout << "is WoS\t: " << is_wos << std::endl;
        std::cout << "evaluate at all points\t: " << evaluate_at_all_points << std::endl;
        std::cout << "------------------------------------------------------------" << std::endl;
        std::filesystem::create_directories(output_dir);
        std::filesystem::copy(input_json_file, output_dir + "/config.json",
                              std::filesystem::copy_options::overwrite_existing);

        // boundary data: piece floor(40 s / L) of the arc length s at the segment's start, -1 on even
        // pieces and 1 on odd ones; n = (t_y, -t_x), t = (v1 - v2) / |v1 - v2| (:201-220), in float
        auto seg_length = [](const std::array<float, 2> &a, const std::array<float, 2> &b) {
            const float dx = a[0] - b[0], dy = a[1] - b[1];
            return std::sqrt(dx * dx + dy * dy);
        };
        float total_boundary_length = 0.0f;
        for (size_t f = 0; f < mesh.nf(); f++)
            total_boundary_length += seg_length(V[mesh.F[3 * f]], V[mesh.F[3 * f + 1]]);
        const unsigned num_segments = 40;
        float boundary_length_sum = 0.0f;
        std::vector<wob::ElementXs<2>> elems;
        std::vector<double> soup;  // for the winding number
        for (size_t f = 0; f < mesh.nf(); f++) {
            const std::array<float, 2> v1 = V[mesh.F[3 * f]], v2 = V[mesh.F[3 * f + 1]];
            const float l = seg_length(v1, v2);
            const float tx = (v1[0] - v2[0]) / l, ty = (v1[1] - v2[1]) / l;
            const int segment_id = (int)(boundary_length_sum * (float)num_segments / total_boundary_length);
            const float boundary_value = segment_id % 2 == 1 ? 1.0f : -1.0f;
            wob::ElementXs<2> e;
            e.a = v1;
            e.b = v2;
            e.n = {ty, -tx};
            e.boundary_value_a = boundary_value;
            e.boundary_value_b = boundary_value;
            e.boundary_type = wob::Dirichlet;
            elems.push_back(e);
            boundary_length_sum += l;
            for (unsigned k = 0; k < 2; k++) soup.push_back(v1[k]);
            for (unsigned k = 0; k < 2; k++) soup.push_back(v2[k]);
        }

        // the points inside (winding number < -1/2 for the clockwise outline), or all (:224-233)
        std::vector<unsigned> eval_idx;
        std::vector<float> points;
        for (unsigned i = 0; i < num_evaluation_points; i++) {
            const std::array<float, 2> x = wob::utils::idx_to_domain_point<2>(i, grid_res, 1.0f);
            const double xd[2] = {x[0], x[1]};
            if (evaluate_at_all_points || wobapp::winding_number_2d(soup, xd) < -0.5) {
                eval_idx.push_back(i);
                points.push_back(x[0]);
                points.push_back(x[1]);
            }
        }
        const uint32_t m = (uint32_t)eval_idx.size();
        std::cout << "evaluation points\t: " << m << std::endl;
        if (setup_only) return 0;

        wob::SceneHost<2> scene(elems);
        wobapp::DeviceArray<float> d_points(points);
        wobapp::DeviceArray<double> d_sum(is_wos ? (size_t)m : 0);
        d_sum.zero();
        std::vector<double> sum(is_wos ? (size_t)m : 3 * (size_t)m, 0.0);
        std::vector<float> solution(num_evaluation_points);

        // the iteration loop (:250-292)
        unsigned num_iterations = 0, total_sample_count = 0;
        double elapsed_time = 0.0;
        while (elapsed_time < max_time * 60.0 && (max_iterations == 0 || num_iterations < max_iterations)) {
            num_iterations += 1;
            total_sample_count += prm.num_sample_paths;
            const auto t0 = std::chrono::steady_clock::now();
            if (is_wos) {
                const wob_params p = prm.to_c();
                wob::check(wob_solve_wos(scene.handle(), &p, d_points.p, m, d_sum.p, nullptr, nullptr, nullptr, nullptr));
                wobapp::cuda_check(cudaDeviceSynchronize(), "running the iteration");
            } else {
                scene.solve_domain(prm, points, sum);
            }
            const auto t1 = std::chrono::steady_clock::now();
            elapsed_time += std::chrono::duration<double>(t1 - t0).count();
            prm.path_offset += prm.num_sample_paths;
            std::cout << "\33[2K\rtime " << elapsed_time << " s\t" << num_iterations << " iterations ("
                      << total_sample_count << " samples)\t" << std::flush;
            if (is_wos) d_sum.download(sum);
            const size_t stride = is_wos ? 1 : 3;
            for (unsigned i = 0; i < num_evaluation_points; i++) solution[i] = std::numeric_limits<float>::quiet_NaN();
            for (uint32_t j = 0; j < m; j++)
                solution[eval_idx[j]] = (float)(sum[stride * j] / (double)total_sample_count);
            wob::utils::save_field(solution, output_dir + "/potential" + std::to_string(num_iterations) + ".scalar",
                                   grid_res);
        }
        std::cout << std::endl;
    } catch (const std::exception &ex) {
        std::cerr << "error: " << ex.what() << std::endl;
        return 1;
    }
    return 0;
}
