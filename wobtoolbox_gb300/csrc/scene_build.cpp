// Host-side scene construction (see scene_host.hpp). Built with -ffp-contract=off.
#include "scene_host.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <thread>

namespace wobgb {

namespace {

inline uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// |b - a| in 2D; |(c - a) x (b - a)| / 2 in 3D (scene.cuh:384, 652-654), evaluated left to right.
float area2(const float *a, const float *b) {
    const float dx = b[0] - a[0], dy = b[1] - a[1];
    return std::sqrt(dx * dx + dy * dy);
}
float area3(const float *a, const float *b, const float *c) {
    const float u0 = c[0] - a[0], u1 = c[1] - a[1], u2 = c[2] - a[2];
    const float v0 = b[0] - a[0], v1 = b[1] - a[1], v2 = b[2] - a[2];
    const float x = u1 * v2 - u2 * v1;
    const float y = u2 * v0 - u0 * v2;
    const float z = u0 * v1 - u1 * v0;
    return std::sqrt(x * x + y * y + z * z) / 2.0f;
}

// Kahan prefix sums in float (scene.cuh:274-298 with utils.cuh:148-166), divided by the total,
// then made nondecreasing (a zero-weight element after a compensated step can otherwise sit
// one ulp below its predecessor).
void kahan_cdf(const std::vector<float> &w, std::vector<float> &cdf, float &total) {
    const size_t n = w.size();
    cdf.resize(n);
    float sum = 0.0f, c = 0.0f;
    for (size_t i = 0; i < n; i++) {
        const float y = w[i] - c;
        const float t = sum + y;
        c = (t - sum) - y;
        sum = t;
        cdf[i] = sum;
    }
    total = sum;
    for (size_t i = 0; i < n; i++) cdf[i] = cdf[i] / total;
    for (size_t i = 1; i < n; i++)
        if (cdf[i] < cdf[i - 1]) cdf[i] = cdf[i - 1];
}

struct BvhBuilder {
    int dim;
    uint32_t n;
    std::vector<uint32_t> ids;         // working permutation of caller indices
    std::vector<float> cen, lo, hi;    // per caller element: centroid and padded box (3 each)
    struct Node {
        float lo[4][3], hi[4][3];
        uint32_t child[4];
        uint32_t depth;
    };
    std::vector<Node> nodes;
    uint32_t max_depth = 0;

    void range_box(uint32_t b, uint32_t e, float blo[3], float bhi[3]) const {
        for (int k = 0; k < 3; k++) { blo[k] = std::numeric_limits<float>::infinity(); bhi[k] = -blo[k]; }
        for (uint32_t i = b; i < e; i++) {
            const uint32_t id = ids[i];
            for (int k = 0; k < dim; k++) {
                blo[k] = std::min(blo[k], lo[3 * id + k]);
                bhi[k] = std::max(bhi[k], hi[3 * id + k]);
            }
        }
        for (int k = dim; k < 3; k++) { blo[k] = 0.0f; bhi[k] = 0.0f; }
    }

    // Median split of [b, e) on the longest centroid axis; ties broken by caller index so the
    // partition is fully determined by the input.
    uint32_t split(uint32_t b, uint32_t e) {
        float clo[3], chi[3];
        for (int k = 0; k < 3; k++) { clo[k] = std::numeric_limits<float>::infinity(); chi[k] = -clo[k]; }
        for (uint32_t i = b; i < e; i++)
            for (int k = 0; k < dim; k++) {
                clo[k] = std::min(clo[k], cen[3 * ids[i] + k]);
                chi[k] = std::max(chi[k], cen[3 * ids[i] + k]);
            }
        int axis = 0;
        for (int k = 1; k < dim; k++)
            if (chi[k] - clo[k] > chi[axis] - clo[axis]) axis = k;
        const uint32_t mid = b + (e - b) / 2;
        const float *c = cen.data();
        std::nth_element(ids.begin() + b, ids.begin() + mid, ids.begin() + e, [c, axis](uint32_t x, uint32_t y) {
            const float cx = c[3 * x + axis], cy = c[3 * y + axis];
            return cx < cy || (cx == cy && x < y);
        });
        return mid;
    }

    uint32_t leaf(uint32_t b, uint32_t e) {
        std::sort(ids.begin() + b, ids.begin() + e);
        return make_leaf(b, e - b);
    }

    // Builds the subtree over [b, e) with more than kLeafMax elements; returns its node index.
    uint32_t node(uint32_t b, uint32_t e, uint32_t depth) {
        const uint32_t idx = (uint32_t)nodes.size();
        nodes.emplace_back();
        max_depth = std::max(max_depth, depth);
        uint32_t rb[4], re[4];
        int nr = 0;
        const uint32_t m = split(b, e);
        const uint32_t halves[2][2] = {{b, m}, {m, e}};
        for (int h = 0; h < 2; h++) {
            const uint32_t hb = halves[h][0], he = halves[h][1];
            if (he - hb > kLeafMax) {
                const uint32_t m2 = split(hb, he);
                rb[nr] = hb; re[nr] = m2; nr++;
                rb[nr] = m2; re[nr] = he; nr++;
            } else {
                rb[nr] = hb; re[nr] = he; nr++;
            }
        }
        uint32_t child[4] = {kChildEmpty, kChildEmpty, kChildEmpty, kChildEmpty};
        float clo[4][3] = {}, chi[4][3] = {};
        for (int k = 0; k < nr; k++) {
            child[k] = (re[k] - rb[k] > kLeafMax) ? node(rb[k], re[k], depth + 1) : leaf(rb[k], re[k]);
            range_box(rb[k], re[k], clo[k], chi[k]);
        }
        Node &nd = nodes[idx];
        for (int k = 0; k < 4; k++) {
            nd.child[k] = child[k];
            for (int j = 0; j < 3; j++) { nd.lo[k][j] = clo[k][j]; nd.hi[k][j] = chi[k][j]; }
        }
        nd.depth = depth;
        return idx;
    }
};

bool finite_all(const float *p, size_t n) {
    for (size_t i = 0; i < n; i++)
        if (!std::isfinite(p[i])) return false;
    return true;
}

}  // namespace

std::vector<uint32_t> build_guide(const std::vector<float> &cdf) {
    const uint32_t n = (uint32_t)cdf.size();
    uint32_t G = std::min<uint32_t>(n, 1u << 22);
    if (G == 0) G = 1;
    std::vector<uint32_t> first(G);
    uint32_t i = 0;
    for (uint32_t j = 0; j < G; j++) {
        const double thr = ((double)j - 0.5) / (double)G;
        while (i + 1 < n && (double)cdf[i] < thr) i++;
        first[j] = i;
    }
    std::vector<uint32_t> rec(4 * (size_t)G);
    for (uint32_t j = 0; j < G; j++) {
        const uint32_t lo = first[j];
        const uint32_t hi = (j + 2 < G) ? first[j + 2] : (n ? n - 1 : 0);
        rec[4 * (size_t)j + 0] = lo;
        rec[4 * (size_t)j + 1] = hi;
        rec[4 * (size_t)j + 2] = n ? f2u(cdf[lo]) : 0u;
        rec[4 * (size_t)j + 3] = n ? f2u(cdf[std::min(lo + 1, n - 1)]) : 0u;
    }
    return rec;
}

std::string build_volume_cdf(int dim, uint32_t res, const float *values, std::vector<float> &cdf) {
    size_t n = 1;
    for (int i = 0; i < dim; i++) n *= res;
    if (!finite_all(values, n)) return "volume cache values must be finite";
    cdf.resize(n);
    double total = 0.0;
    for (size_t i = 0; i < n; i++) total += std::fabs((double)values[i]);
    if (total == 0.0) {
        for (size_t i = 0; i < n; i++) cdf[i] = (float)((double)(i + 1) / (double)n);
    } else {
        double acc = 0.0;
        for (size_t i = 0; i < n; i++) {
            acc += std::fabs((double)values[i]);
            cdf[i] = (float)(acc / total);
        }
    }
    return "";
}

namespace {

// Direction angle (radians) of diamond angle pa in [0, 2]: (1 - pa, pa) for pa <= 1, else
// (1 - pa, 2 - pa).
double diamond_to_angle(double pa) {
    return pa <= 1.0 ? std::atan2(pa, 1.0 - pa) : std::atan2(2.0 - pa, 1.0 - pa);
}

float round_down(double x) {
    float f = (float)x;
    if ((double)f > x) f = std::nextafter(f, -std::numeric_limits<float>::infinity());
    return f;
}
float round_up(double x) {
    float f = (float)x;
    if ((double)f < x) f = std::nextafter(f, std::numeric_limits<float>::infinity());
    return f;
}

// The cell of offset c in a bin; the device evaluates the same float expression.
inline uint32_t line_cell(float c, float cmin, float inv_w, uint32_t M) {
    const float f = (c - cmin) * inv_w;
    const uint32_t j = f >= (float)M ? M : (uint32_t)f;
    return j < M ? j : M - 1;
}

}  // namespace

namespace {

// The offset intervals of all segments over direction bin k of K and their cells among M:
// fills c0 / c1 and the bin header {cmin, cmax, inv_w, 0}; returns the number of list entries.
size_t line_bin(const std::vector<float> &elems, uint32_t n, float pad, float cx, float cy, uint32_t K, uint32_t M,
                uint32_t k, std::vector<float> &lo, std::vector<float> &hi, std::vector<uint32_t> &c0,
                std::vector<uint32_t> &c1, float *header) {
    const int EF = elem_record_floats(2);
    const double f0 = diamond_to_angle(2.0 * k / K), f1 = diamond_to_angle(2.0 * (k + 1) / K);
    const double nx0 = -std::sin(f0), ny0 = std::cos(f0), nx1 = -std::sin(f1), ny1 = std::cos(f1);
    const double dphi = f1 - f0;
    const double bend = dphi * dphi / 8.0 + kLineGridAngleSlack;
    float cmin = std::numeric_limits<float>::infinity(), cmax = -cmin;
    for (uint32_t i = 0; i < n; i++) {
        const float *r = elems.data() + (size_t)i * EF;
        const double ax = (double)r[0] - cx, ay = (double)r[1] - cy, bx = (double)r[2] - cx, by = (double)r[3] - cy;
        const double ga0 = nx0 * ax + ny0 * ay, ga1 = nx1 * ax + ny1 * ay;
        const double gb0 = nx0 * bx + ny0 * by, gb1 = nx1 * bx + ny1 * by;
        const double rad = std::max(std::hypot(ax, ay), std::hypot(bx, by)) * bend + (double)pad;
        lo[i] = round_down(std::min(std::min(ga0, ga1), std::min(gb0, gb1)) - rad);
        hi[i] = round_up(std::max(std::max(ga0, ga1), std::max(gb0, gb1)) + rad);
        cmin = std::min(cmin, lo[i]);
        cmax = std::max(cmax, hi[i]);
    }
    float inv_w = cmax > cmin ? (float)M / (cmax - cmin) : 0.0f;
    if (!std::isfinite(inv_w)) inv_w = 0.0f;
    header[0] = cmin;
    header[1] = cmax;
    header[2] = inv_w;
    header[3] = 0.0f;
    size_t listed = 0;
    for (uint32_t i = 0; i < n; i++) {
        c0[i] = line_cell(lo[i], cmin, inv_w, M);
        c1[i] = line_cell(hi[i], cmin, inv_w, M);
        listed += c1[i] - c0[i] + 1;
    }
    return listed;
}

// Estimated list entries of a K x M grid from 16 evenly spaced bins.
double line_grid_estimate(const std::vector<float> &elems, uint32_t n, float pad, float cx, float cy, uint32_t K,
                          uint32_t M) {
    std::vector<float> lo(n), hi(n);
    std::vector<uint32_t> c0(n), c1(n);
    float header[4];
    const uint32_t step = std::max<uint32_t>(1u, K / 16);
    double sum = 0.0;
    uint32_t cnt = 0;
    for (uint32_t k = step / 2; k < K; k += step, cnt++)
        sum += (double)line_bin(elems, n, pad, cx, cy, K, M, k, lo, hi, c0, c1, header);
    return cnt ? sum / cnt * K : 0.0;
}

}  // namespace

// Resolution: K = the power of two >= n in [128, 1024] direction bins and M = the power of two
// >= 2n in [64, 4096] cells (finer grids list fewer non-hits per query; measured on the
// 1024-segment star: K x M = 512 x 512 9.5, 512 x 1024 12.0, 512 x 2048 12.8, 1024 x 2048 14.7 G
// bounces/s). While 16 sample bins predict more list entries than min(kLineGridMaxEntries,
// kLineGridEntriesPerElem x n), M is halved if it exceeds K, else K; scenes where even 64 x 64
// does not fit (long segments: the BVH is the better index) get no grid. Bins are built in
// parallel on the host's cores.
void build_line_grid_2d(const std::vector<float> &elems, uint32_t n, float pad, LineGrid &grid) {
    grid = LineGrid();
    if (n == 0 || n > kLineGridMaxElems) return;
    // offsets about the centre of the scene's box; a line through a point farther than 8 (extent +
    // max |coordinate|) from it takes the BVH, so the query's float offset stays within the
    // padding of the exact one
    const int EF = elem_record_floats(2);
    float bmin[2] = {std::numeric_limits<float>::infinity(), std::numeric_limits<float>::infinity()};
    float bmax[2] = {-bmin[0], -bmin[1]};
    for (uint32_t i = 0; i < n; i++)
        for (int v = 0; v < 2; v++)
            for (int k = 0; k < 2; k++) {
                bmin[k] = std::min(bmin[k], elems[(size_t)i * EF + 2 * v + k]);
                bmax[k] = std::max(bmax[k], elems[(size_t)i * EF + 2 * v + k]);
            }
    const float cx = (float)(0.5 * ((double)bmin[0] + bmax[0])), cy = (float)(0.5 * ((double)bmin[1] + bmax[1]));
    const float ext = std::max(bmax[0] - bmin[0], bmax[1] - bmin[1]);
    const float mag =
        std::max(std::max(std::fabs(bmin[0]), std::fabs(bmax[0])), std::max(std::fabs(bmin[1]), std::fabs(bmax[1])));
    uint32_t K = 128, M = 64;
    while (K < n && K < 1024) K <<= 1;
    while (M < 2 * n && M < 4096) M <<= 1;
    const double budget = std::min((double)kLineGridMaxEntries, (double)kLineGridEntriesPerElem * n);
    while (K >= 64 && M >= 64 && line_grid_estimate(elems, n, pad, cx, cy, K, M) > budget) {
        if (M > K) M >>= 1;
        else K >>= 1;
    }
    if (K < 64 || M < 64) return;
    std::vector<float> bins(4 * (size_t)K);
    std::vector<std::vector<uint32_t>> counts(K);
    std::vector<std::vector<uint16_t>> lists(K);
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const unsigned n_threads = std::min<unsigned>(hw, K);
    std::vector<std::thread> pool;
    std::vector<char> failed(n_threads, 0);
    auto work = [&](unsigned t) {
        try {
            std::vector<float> lo(n), hi(n);
            std::vector<uint32_t> c0(n), c1(n);
            for (uint32_t k = t; k < K; k += n_threads) {
                const size_t listed = line_bin(elems, n, pad, cx, cy, K, M, k, lo, hi, c0, c1,
                                               bins.data() + 4 * (size_t)k);
                std::vector<uint32_t> &count = counts[k];
                count.assign(M + 1, 0u);
                for (uint32_t i = 0; i < n; i++)
                    for (uint32_t j = c0[i]; j <= c1[i]; j++) count[j + 1]++;
                for (uint32_t j = 0; j < M; j++) count[j + 1] += count[j];  // list starts within the bin
                std::vector<uint16_t> &list = lists[k];
                list.resize(listed);
                std::vector<uint32_t> fill(count.begin(), count.end() - 1);
                for (uint32_t i = 0; i < n; i++)
                    for (uint32_t j = c0[i]; j <= c1[i]; j++) list[fill[j]++] = (uint16_t)i;
            }
        } catch (...) {  // out of host memory: this scene does without a grid
            failed[t] = 1;
        }
    };
    try {
        for (unsigned t = 0; t < n_threads; t++) pool.emplace_back(work, t);
    } catch (...) {  // no threads to be had: build the remaining bins here
        for (unsigned t = (unsigned)pool.size(); t < n_threads; t++) work(t);
    }
    for (std::thread &th : pool) th.join();
    for (char f : failed)
        if (f) return;
    size_t total = 0;
    for (uint32_t k = 0; k < K; k++) total += lists[k].size();
    if (total > kLineGridMaxEntries) return;
    grid.K = K;
    grid.M = M;
    grid.cx = cx;
    grid.cy = cy;
    grid.far = 8.0f * (ext + mag);
    grid.bins = std::move(bins);
    grid.offsets.resize((size_t)K * (M + 1));
    grid.entries.resize(total);
    size_t base = 0;
    for (uint32_t k = 0; k < K; k++) {
        for (uint32_t j = 0; j <= M; j++) grid.offsets[(size_t)k * (M + 1) + j] = (uint32_t)(base + counts[k][j]);
        std::copy(lists[k].begin(), lists[k].end(), grid.entries.begin() + base);
        base += lists[k].size();
    }
}

std::string build_host_scene(int dim, uint32_t n, const float *verts, const float *normals,
                             const float *bvals, const float *alphas, const int32_t *types,
                             HostScene &out) {
    if (dim != 2 && dim != 3) return "dim must be 2 or 3";
    if (n == 0) return "a scene needs at least one element";
    if (n > kMaxElements) return "too many elements";
    if (!verts || !normals || !bvals || !types) return "vertices, normals, boundary_values and boundary_types are required";
    const size_t D = (size_t)dim;
    if (!finite_all(verts, n * D * D)) return "vertices must be finite";
    if (!finite_all(normals, n * D)) return "normals must be finite";
    if (!finite_all(bvals, n * D)) return "boundary values must be finite";
    if (alphas && !finite_all(alphas, n * D)) return "robin alphas must be finite";
    for (uint32_t i = 0; i < n; i++)
        if (types[i] < 0 || types[i] > 2) return "boundary_types must be 0 (Dirichlet), 1 (Neumann) or 2 (Robin)";
    // Normals enter every kernel weight (dG/dn); a zero or wildly scaled normal would silently
    // zero or scale the walk's weights, so anything far from unit length is rejected.
    for (uint32_t i = 0; i < n; i++) {
        double q = 0.0;
        for (size_t k = 0; k < D; k++) q += (double)normals[i * D + k] * (double)normals[i * D + k];
        if (!(q >= 0.25 && q <= 4.0))
            return "normals must be unit vectors (element " + std::to_string(i) + " has |n| = " + std::to_string(std::sqrt(q)) + ")";
    }

    // ---- BVH over padded element boxes
    BvhBuilder bb;
    bb.dim = dim;
    bb.n = n;
    bb.ids.resize(n);
    bb.cen.assign(3 * (size_t)n, 0.0f);
    bb.lo.assign(3 * (size_t)n, 0.0f);
    bb.hi.assign(3 * (size_t)n, 0.0f);
    float gmin[3] = {0, 0, 0}, gmax[3] = {0, 0, 0}, mag = 0.0f;
    for (int k = 0; k < dim; k++) { gmin[k] = std::numeric_limits<float>::infinity(); gmax[k] = -gmin[k]; }
    for (uint32_t i = 0; i < n; i++) {
        bb.ids[i] = i;
        const float *v = verts + (size_t)i * D * D;
        for (int k = 0; k < dim; k++) {
            float lo = v[k], hi = v[k], s = v[k];
            for (int j = 1; j < dim; j++) {
                lo = std::min(lo, v[j * D + k]);
                hi = std::max(hi, v[j * D + k]);
                s += v[j * D + k];
            }
            bb.lo[3 * i + k] = lo;
            bb.hi[3 * i + k] = hi;
            bb.cen[3 * i + k] = s / (float)dim;
            gmin[k] = std::min(gmin[k], lo);
            gmax[k] = std::max(gmax[k], hi);
            mag = std::max(mag, std::max(std::fabs(lo), std::fabs(hi)));
        }
    }
    float ext = 0.0f;
    for (int k = 0; k < dim; k++) ext = std::max(ext, gmax[k] - gmin[k]);
    // Boxes are padded far beyond the rounding error of the line/box tests, so culling never
    // removes an element the exact primitive test would accept.
    const float pad = 1e-5f * (ext + mag) + 1e-30f;
    for (size_t i = 0; i < 3 * (size_t)n; i++) { bb.lo[i] -= pad; bb.hi[i] += pad; }

    if (n <= kLeafMax) {
        BvhBuilder::Node root{};
        for (int k = 0; k < 4; k++) root.child[k] = kChildEmpty;
        root.child[0] = bb.leaf(0, n);
        bb.range_box(0, n, root.lo[0], root.hi[0]);
        root.depth = 0;
        bb.nodes.push_back(root);
    } else {
        bb.node(0, n, 0);
    }
    if (3 * (bb.max_depth + 1) + 2 > kTraversalStack) return "BVH too deep for the traversal stack";

    out = HostScene();
    out.dim = dim;
    out.n = n;
    out.order = bb.ids;
    out.n_nodes = (uint32_t)bb.nodes.size();
    out.depth = bb.max_depth + 1;

    // ---- nodes: [lo_x[4], lo_y[4], (lo_z[4]), hi_x[4], hi_y[4], (hi_z[4]), child[4]]
    const int NF = node_record_floats(dim);
    out.nodes.assign((size_t)out.n_nodes * NF, 0.0f);
    for (uint32_t i = 0; i < out.n_nodes; i++) {
        const BvhBuilder::Node &nd = bb.nodes[i];
        float *r = out.nodes.data() + (size_t)i * NF;
        for (int k = 0; k < 4; k++) {
            for (int a = 0; a < dim; a++) {
                r[4 * a + k] = nd.lo[k][a];
                r[4 * (dim + a) + k] = nd.hi[k][a];
            }
            r[4 * (2 * dim) + k] = u2f(nd.child[k]);
        }
    }

    // ---- element records in storage order
    const int EF = elem_record_floats(dim);
    out.elems.assign((size_t)n * EF, 0.0f);
    if (dim == 3) out.isect.assign((size_t)n * kIsect3Floats, 0.0f);
    if (dim == 3) out.elem_aux.assign((size_t)n * kElemAux3Floats, 0.0f);
    std::vector<float> areas(n), bvw(n);
    for (uint32_t s = 0; s < n; s++) {
        const uint32_t i = out.order[s];
        const float *v = verts + (size_t)i * D * D;
        const float *nn = normals + (size_t)i * D;
        const float *bv = bvals + (size_t)i * D;
        float al[3] = {0, 0, 0};
        if (alphas)
            for (int k = 0; k < dim; k++) al[k] = alphas[(size_t)i * D + k];
        float *r = out.elems.data() + (size_t)s * EF;
        if (dim == 2) {
            const float area = area2(v, v + 2);
            r[0] = v[0]; r[1] = v[1]; r[2] = v[2]; r[3] = v[3];
            r[4] = nn[0]; r[5] = nn[1]; r[6] = bv[0]; r[7] = bv[1];
            r[8] = al[0]; r[9] = al[1]; r[10] = area; r[11] = u2f((uint32_t)types[i]);
            areas[s] = area;
            bvw[s] = area * (std::fabs(bv[0]) + std::fabs(bv[1])) / 2.0f;
        } else {
            const float area = area3(v, v + 3, v + 6);
            for (int k = 0; k < 9; k++) r[k] = v[k];
            r[9] = nn[0]; r[10] = nn[1]; r[11] = nn[2];
            r[12] = bv[0]; r[13] = bv[1]; r[14] = bv[2]; r[15] = u2f((uint32_t)types[i]);
            float *x = out.elem_aux.data() + (size_t)s * kElemAux3Floats;
            x[0] = al[0]; x[1] = al[1]; x[2] = al[2]; x[3] = area;
            areas[s] = area;
            bvw[s] = area * (std::fabs(bv[0]) + std::fabs(bv[1]) + std::fabs(bv[2])) / 3.0f;
            // intersection record: a, e1 = a - b, e2 = a - c, q = e1 x e2
            float *q = out.isect.data() + (size_t)s * kIsect3Floats;
            const float e1x = v[0] - v[3], e1y = v[1] - v[4], e1z = v[2] - v[5];
            const float e2x = v[0] - v[6], e2y = v[1] - v[7], e2z = v[2] - v[8];
            q[0] = v[0]; q[1] = v[1]; q[2] = v[2];
            q[3] = e1x; q[4] = e1y; q[5] = e1z;
            q[6] = e2x; q[7] = e2y; q[8] = e2z;
            q[9] = e1y * e2z - e1z * e2y;
            q[10] = e1z * e2x - e1x * e2z;
            q[11] = e1x * e2y - e1y * e2x;
        }
    }

    if (dim == 3) {
        out.alpha_value = alphas ? alphas[0] : 0.0f;
        out.alpha_const = true;
        if (alphas)
            for (size_t i = 0; i < (size_t)n * 3; i++)
                if (f2u(alphas[i]) != f2u(out.alpha_value)) out.alpha_const = false;
    }

    kahan_cdf(areas, out.area_cdf, out.total_area);
    if (!(out.total_area > 0.0f) || !std::isfinite(out.total_area)) return "total boundary area must be positive and finite";
    out.area_guide = build_guide(out.area_cdf);
    kahan_cdf(bvw, out.bv_cdf, out.total_bv);
    out.bv_valid = out.total_bv > 0.0f && std::isfinite(out.total_bv);
    if (out.bv_valid) out.bv_guide = build_guide(out.bv_cdf);
    else out.bv_guide.assign(4, 0u);
    if (dim == 2) build_line_grid_2d(out.elems, n, pad, out.line_grid);
    return "";
}

void rebuild_bv_tables(HostScene &s) {
    const int EF = elem_record_floats(s.dim);
    std::vector<float> bvw(s.n);
    for (uint32_t i = 0; i < s.n; i++) {
        const float *r = s.elems.data() + (size_t)i * EF;
        if (s.dim == 2) {
            bvw[i] = r[10] * (std::fabs(r[6]) + std::fabs(r[7])) / 2.0f;
        } else {
            const float area = s.elem_aux[(size_t)i * kElemAux3Floats + 3];
            bvw[i] = area * (std::fabs(r[12]) + std::fabs(r[13]) + std::fabs(r[14])) / 3.0f;
        }
    }
    kahan_cdf(bvw, s.bv_cdf, s.total_bv);
    s.bv_valid = s.total_bv > 0.0f && std::isfinite(s.total_bv);
    if (s.bv_valid) s.bv_guide = build_guide(s.bv_cdf);
    else s.bv_guide.assign(4, 0u);
}

}  // namespace wobgb
