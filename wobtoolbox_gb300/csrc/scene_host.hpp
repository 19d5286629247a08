// Host-side scene construction for the GB300 WoB engine: validation, the 4-wide BVH, the element
// storage order, the area and |g| CDFs and their guide tables, and the packed device records.
//
// Replaces wob::SceneHost (scene.cuh:264-326) and the lbvh build it wraps (scene.cuh:266).
// All float arithmetic here must be built without contraction (-ffp-contract=off): the CDFs and
// the precomputed intersection records are required to be bit-identical to what a plain IEEE
// single-precision evaluation of the same formulas gives.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace wobgb {

// BVH child codes. Internal children hold the node index (< 2^31). Leaves hold the first stored
// element and the element count (1..kLeafMax) with the top bit set. kChildEmpty marks an unused
// slot of a 4-wide node.
constexpr uint32_t kLeafMax = 4;
constexpr uint32_t kChildEmpty = 0xFFFFFFFFu;
constexpr uint32_t kMaxElements = (1u << 28) - 8u;
constexpr uint32_t kTraversalStack = 64;
inline bool child_is_leaf(uint32_t c) { return (c & 0x80000000u) != 0u; }
inline uint32_t leaf_first(uint32_t c) { return c & 0x0FFFFFFFu; }
inline uint32_t leaf_count(uint32_t c) { return ((c >> 28) & 7u) + 1u; }
inline uint32_t make_leaf(uint32_t first, uint32_t count) {
    return 0x80000000u | ((count - 1u) << 28) | first;
}

// Packed record sizes in floats. Every record starts on a 32-byte boundary so the kernels read it
// with 32-byte loads (ld.global.nc.v8.f32); a random gather costs about the same per load
// instruction whatever its width, so fewer, wider loads per record are faster.
//   element: 2D a, b, n, bv[2], alpha[2], area, type + 16 B padding (64 B);
//            3D a, b, c, n, bv[3], type (64 B), and in a second array alpha[3], area (16 B),
//            read only when the scene's Robin alphas are not all the same value (a sample then
//            costs two 32-byte loads)
//   node: 2D lo_x[4] lo_y[4] hi_x[4] hi_y[4] child[4] + 16 B padding (96 B);
//         3D adds lo_z, hi_z (112 B + 16 B padding)
//   intersection record (3D): a, a - b, a - c, (a - b) x (a - c) + 16 B padding (64 B)
inline int elem_record_floats(int dim) { return dim == 2 ? 16 : 16; }
constexpr int kElemAux3Floats = 4;
inline int node_record_floats(int dim) { return dim == 2 ? 24 : 32; }
constexpr int kIsect3Floats = 16;

// 2D line grid: all segments an infinite line can meet, by direction and offset. The directions
// (half-turn, diamond angle pa in [0, 2]) are cut into K bins; for bin k and a segment, the offsets
// c = n . (p - centre) (n = (-sin phi, cos phi)) its points take over the bin's directions form an interval,
// widened by the curvature of the sinusoids, an angle slack and the scene's padding; the offsets of
// bin k, [cmin, cmax], are cut into M cells, and a cell lists, in storage order, every segment whose
// interval meets it. A line of bin k with offset c can only meet the segments listed in c's cell,
// so testing those exactly gives the same hits, in the same order, as testing all segments.
// Cells come from cell(c) = min((int)((c - cmin) * inv_w), M - 1) on host and device alike (a
// monotone function of c), so a segment is listed in every cell that an offset of its interval
// can fall in.
struct LineGrid {
    uint32_t K = 0, M = 0;             // K == 0: no grid (the BVH answers line queries)
    float cx = 0.0f, cy = 0.0f;        // offsets are taken about this point (the scene's box centre)
    float far = 0.0f;                  // lines through points farther than this (L1 from the centre) take the BVH
    std::vector<float> bins;           // K * 4: cmin, cmax, inv_w, 0
    std::vector<uint32_t> offsets;     // K * (M + 1): start of each cell's list in entries
    std::vector<uint16_t> entries;     // stored element indices
};
constexpr uint32_t kLineGridMaxElems = 16384;   // larger 2D scenes use the BVH alone
constexpr size_t kLineGridMaxEntries = 1u << 24;  // 32 MB of lists at most
constexpr size_t kLineGridEntriesPerElem = 8192;  // 16 KB of lists per segment at most
constexpr double kLineGridAngleSlack = 1e-6;   // rad: rounding of a query's bin and direction

// The line grid of a 2D scene's stored element records (empty if the scene is too large).
void build_line_grid_2d(const std::vector<float> &elems, uint32_t n, float pad, LineGrid &grid);

struct HostScene {
    int dim = 0;
    uint32_t n = 0;
    std::vector<uint32_t> order;           // order[i] = caller index of stored element i
    std::vector<float> elems;              // n * elem_record_floats(dim)
    std::vector<float> elem_aux;           // 3D only: n * kElemAux3Floats (alpha[3], area)
    bool alpha_const = false;              // 3D: every vertex alpha equals alpha_value (bitwise)
    float alpha_value = 0.0f;
    std::vector<float> isect;              // 3D only: n * kIsect3Floats
    std::vector<float> nodes;              // n_nodes * node_record_floats(dim)
    std::vector<float> area_cdf, bv_cdf;   // n each
    std::vector<uint32_t> area_guide, bv_guide;  // packed guide records (4 words each)
    float total_area = 0.0f, total_bv = 0.0f;
    bool bv_valid = false;                 // |g| sampling defined (total |g| finite and > 0)
    uint32_t n_nodes = 0, depth = 0;
    LineGrid line_grid;                    // 2D only
};

// Returns "" on success, else a message. Arrays as documented for wob_scene_create.
std::string build_host_scene(int dim, uint32_t n, const float *verts, const float *normals,
                             const float *bvals, const float *alphas, const int32_t *types,
                             HostScene &out);

// Recomputes the |g| sampling weights, CDF, guide table, total and validity from the boundary
// values in the stored element records (after the values changed).
void rebuild_bv_tables(HostScene &s);

// Guide table of a nondecreasing CDF with G = min(n, 2^22) entries of 4 words each:
// {lo, hi, bits(cdf[lo]), bits(cdf[lo + 1])}, where lo is the first index whose CDF value reaches
// (j - 1/2)/G and hi the lo of entry j + 2 (n - 1 for the last two). See cdf_search in
// device_common.cuh for why the answer for a key in bin j lies in [lo, hi].
std::vector<uint32_t> build_guide(const std::vector<float> &cdf);

// |f| CDF of a volume cache: prefix(|f|) / total in double, rounded to float; uniform if all zero.
std::string build_volume_cdf(int dim, uint32_t res, const float *values, std::vector<float> &cdf);

}  // namespace wobgb
