// CPU check of the 2D line grid built by build_host_scene (wobtoolbox_gb300/csrc/scene_build.cpp):
// for many lines, every segment the exact intersection test accepts must be listed in the line's
// grid cell. The cell lookup below is the device query's float arithmetic (line_grid_query in
// csrc/device_common.cuh), the exact test is isect_seg's (both built without contraction).
//
//   line_grid_check <scene file> <n_lines> <seed>
// scene file: uint32 n, then n * 4 floats (a.x a.y b.x b.y). Prints
// "lines <L> grid <K> <M> hits <H> candidates <C> missed <X> unordered <U>".
#include "../wobtoolbox_gb300/csrc/scene_host.hpp"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

namespace {

bool isect_seg(float ox, float oy, float dx, float dy, float ax, float ay, float bx, float by) {
    const float edx = ax - bx, edy = ay - by;
    const float wx = ax - ox, wy = ay - oy;
    const float det = dx * edy - dy * edx;
    const float sn = dx * wy - dy * wx;
    bool inside;
    if (det > 0.0f) inside = (sn >= 0.0f) && (sn <= det);
    else if (det < 0.0f) inside = (sn <= 0.0f) && (sn >= det);
    else inside = false;
    if (!inside) return false;
    const float tn = wx * edy - wy * edx;
    const float t = tn / det;
    return std::fabs(t) > 10.0f * 1.1920928955078125e-7f;
}

// The candidate list [b, e) of the line (o, d); false when d is not a unit vector within 1e-6 or
// o is too far from the grid's centre (the device then traverses the BVH).
bool cell_list(const wobgb::LineGrid &g, float ox, float oy, float dx0, float dy0, uint32_t &b, uint32_t &e) {
    const float q = dx0 * dx0 + dy0 * dy0;
    if (!(std::fabs(q - 1.0f) <= 1e-6f)) return false;
    const float px = ox - g.cx, py = oy - g.cy;
    if (!(std::fabs(px) + std::fabs(py) <= g.far)) return false;
    const bool flip = dy0 < 0.0f || (dy0 == 0.0f && dx0 < 0.0f);
    const float dx = flip ? -dx0 : dx0, dy = flip ? -dy0 : dy0;
    const float t = dy / (std::fabs(dx) + dy);
    const float pa = dx >= 0.0f ? t : 2.0f - t;
    uint32_t k = (uint32_t)(pa * (0.5f * (float)g.K));
    k = k < g.K ? k : g.K - 1;
    const float c = -dy * px + dx * py;
    const float *h = g.bins.data() + 4 * (size_t)k;
    b = e = 0;
    if (!(c >= h[0] && c <= h[1])) return true;
    const float f = (c - h[0]) * h[2];
    uint32_t j = f >= (float)g.M ? g.M : (uint32_t)f;
    j = j < g.M ? j : g.M - 1;
    b = g.offsets[(size_t)k * (g.M + 1) + j];
    e = g.offsets[(size_t)k * (g.M + 1) + j + 1];
    return true;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 4) return 2;
    FILE *fp = std::fopen(argv[1], "rb");
    if (!fp) return 2;
    uint32_t n = 0;
    if (std::fread(&n, 4, 1, fp) != 1) return 2;
    std::vector<float> seg((size_t)n * 4);
    if (std::fread(seg.data(), 4, seg.size(), fp) != seg.size()) return 2;
    std::fclose(fp);
    const long n_lines = std::atol(argv[2]);
    std::mt19937_64 rng((uint64_t)std::atol(argv[3]));

    std::vector<float> verts((size_t)n * 4), normals((size_t)n * 2, 0.0f), bvals((size_t)n * 2, 0.0f);
    std::vector<int32_t> types(n, 0);
    for (uint32_t i = 0; i < n; i++) {
        for (int k = 0; k < 4; k++) verts[4 * (size_t)i + k] = seg[4 * (size_t)i + k];
        normals[2 * (size_t)i + 1] = 1.0f;
    }
    wobgb::HostScene s;
    const std::string err = wobgb::build_host_scene(2, n, verts.data(), normals.data(), bvals.data(), nullptr,
                                                    types.data(), s);
    if (!err.empty()) {
        std::printf("error %s\n", err.c_str());
        return 1;
    }
    const wobgb::LineGrid &g = s.line_grid;
    if (g.K == 0) {
        std::printf("lines 0 grid 0 0 hits 0 candidates 0 missed 0 unordered 0\n");
        return 0;
    }
    float lo[2] = {INFINITY, INFINITY}, hi[2] = {-INFINITY, -INFINITY};
    for (size_t i = 0; i < seg.size(); i++) {
        lo[i % 2] = std::fmin(lo[i % 2], seg[i]);
        hi[i % 2] = std::fmax(hi[i % 2], seg[i]);
    }
    std::uniform_real_distribution<double> U(0.0, 1.0);
    const int EF = wobgb::elem_record_floats(2);
    long hits = 0, cands = 0, missed = 0, unordered = 0, lines = 0;
    std::vector<char> listed(n);
    for (long l = 0; l < n_lines; l++) {
        // origins: in and around the scene, on vertices, far outside; directions: random, on the
        // diamond-angle bin boundaries, along axes, along segments
        const int kind = (int)(l % 6);
        float ox, oy, dx, dy;
        const uint32_t si = (uint32_t)(U(rng) * n) % n;
        const float *r = s.elems.data() + (size_t)si * EF;
        if (kind == 1 || kind == 4) {
            ox = r[0];
            oy = r[1];
        } else {
            const double spread = kind == 5 ? 12.0 : 1.2;
            const double cx = 0.5 * ((double)lo[0] + hi[0]), cy = 0.5 * ((double)lo[1] + hi[1]);
            ox = (float)(cx + (U(rng) - 0.5) * spread * (hi[0] - lo[0] + 1e-3));
            oy = (float)(cy + (U(rng) - 0.5) * spread * (hi[1] - lo[1] + 1e-3));
        }
        double ux, uy;
        if (kind == 2) {  // a bin boundary of this grid
            const double pa = 2.0 * (double)(uint32_t)(U(rng) * g.K) / g.K;
            ux = pa <= 1.0 ? 1.0 - pa : 1.0 - pa;
            uy = pa <= 1.0 ? pa : 2.0 - pa;
        } else if (kind == 3) {  // an axis
            const int a = (int)(U(rng) * 4);
            ux = a == 0 ? 1 : a == 2 ? -1 : 0;
            uy = a == 1 ? 1 : a == 3 ? -1 : 0;
        } else if (kind == 4) {  // along the segment starting at the origin
            ux = (double)r[2] - r[0];
            uy = (double)r[3] - r[1];
        } else {
            const double th = U(rng) * 2.0 * M_PI;
            ux = std::cos(th);
            uy = std::sin(th);
        }
        const double nrm = std::hypot(ux, uy);
        if (!(nrm > 0.0)) continue;
        if (U(rng) < 0.5) { ux = -ux; uy = -uy; }
        dx = (float)(ux / nrm);
        dy = (float)(uy / nrm);
        uint32_t b, e;
        if (!cell_list(g, ox, oy, dx, dy, b, e)) continue;
        lines++;
        cands += e - b;
        std::fill(listed.begin(), listed.end(), 0);
        for (uint32_t q = b; q < e; q++) {
            listed[g.entries[q]] = 1;
            if (q > b && g.entries[q] <= g.entries[q - 1]) unordered++;
        }
        for (uint32_t i = 0; i < n; i++) {
            const float *p = s.elems.data() + (size_t)i * EF;
            if (isect_seg(ox, oy, dx, dy, p[0], p[1], p[2], p[3])) {
                hits++;
                if (!listed[i]) missed++;
            }
        }
    }
    std::printf("lines %ld grid %u %u hits %ld candidates %ld missed %ld unordered %ld\n", lines, g.K, g.M, hits,
                cands, missed, unordered);
    return 0;
}
