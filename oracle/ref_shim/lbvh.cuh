// TEST INFRASTRUCTURE ONLY. A stand-in for the lbvh library (the reference's deps/lbvh submodule,
// rsugimoto's fork, no pinned commit and absent here) with the interface the reference's
// scene.cuh uses: bvh / bvh_device over the caller's objects, leaf nodes numbered after the
// n - 1 internal nodes whose object_idx points back into the caller's object order, the AABB and
// Line types over CUDA-style float2 / float4 vectors, and query_device with a line query that
// reports every object the infinite line meets (the callback decides) into a bounded buffer while
// counting all of them.
//
// Own construction: leaves sorted by the Morton code of their box centre within the scene box
// (as lbvh orders its leaves), a balanced binary tree over that order, boxes padded by a relative
// 1e-5 so the box test never drops an object the exact primitive test accepts. Which hits a
// query finds is therefore the brute-force set; their order is the tree's depth-first order.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <numeric>
#include <thrust/host_vector.h>
#include <thrust/pair.h>
#include <vector>

#ifndef WOBREF_VECTOR_TYPES
#define WOBREF_VECTOR_TYPES
struct float2 {
    float x, y;
};
struct float4 {
    float x, y, z, w;
};
struct double2 {
    double x, y;
};
struct double4 {
    double x, y, z, w;
};
inline float2 make_float2(float x, float y) { return float2{x, y}; }
inline float4 make_float4(float x, float y, float z, float w) { return float4{x, y, z, w}; }
inline double2 make_double2(double x, double y) { return double2{x, y}; }
inline double4 make_double4(double x, double y, double z, double w) { return double4{x, y, z, w}; }
#endif

namespace lbvh {

template <typename T, unsigned int Dim> struct vector_of;
template <> struct vector_of<float, 2> { using type = float2; };
template <> struct vector_of<float, 3> { using type = float4; };
template <> struct vector_of<double, 2> { using type = double2; };
template <> struct vector_of<double, 3> { using type = double4; };

template <typename T, unsigned int Dim> struct aabb {
    typename vector_of<T, Dim>::type upper, lower;
};

template <typename T, unsigned int Dim> struct Line {
    typename vector_of<T, Dim>::type origin, dir;
};

template <typename T, unsigned int Dim> struct query_line_intersect {
    explicit query_line_intersect(const Line<T, Dim> &l) : line(l) {}
    Line<T, Dim> line;
};

struct node {
    std::uint32_t parent_idx;
    std::uint32_t left_idx;
    std::uint32_t right_idx;
    std::uint32_t object_idx;  // 0xFFFFFFFF for internal nodes
};

namespace detail {
template <typename V> inline double comp(const V &v, int k) { return k == 0 ? v.x : k == 1 ? v.y : (double)v.z; }
template <> inline double comp<float2>(const float2 &v, int k) { return k == 0 ? v.x : v.y; }
template <> inline double comp<double2>(const double2 &v, int k) { return k == 0 ? v.x : v.y; }

// Infinite line against a box: the line's parameter intervals inside each slab must overlap.
template <typename T, unsigned int Dim> inline bool line_meets_box(const Line<T, Dim> &l, const aabb<T, Dim> &b) {
    double tmin = -std::numeric_limits<double>::infinity(), tmax = std::numeric_limits<double>::infinity();
    for (int k = 0; k < (int)Dim; k++) {
        const double o = comp(l.origin, k), d = comp(l.dir, k);
        const double lo = comp(b.lower, k), hi = comp(b.upper, k);
        if (d == 0.0) {
            if (o < lo || o > hi) return false;
            continue;
        }
        double t1 = (lo - o) / d, t2 = (hi - o) / d;
        if (t1 > t2) std::swap(t1, t2);
        tmin = std::max(tmin, t1);
        tmax = std::min(tmax, t2);
        if (tmin > tmax) return false;
    }
    return true;
}
}  // namespace detail

template <typename T, unsigned int Dim, typename Object> struct bvh_device {
    unsigned int num_nodes;
    unsigned int num_objects;
    const node *nodes;
    const aabb<T, Dim> *aabbs;
    const Object *objects;
};

template <typename T, unsigned int Dim, typename Object, typename AABBGetter> class bvh {
  public:
    template <typename InputIterator> bvh(InputIterator first, InputIterator last, bool = true) : objects_(first, last) {
        build();
    }
    const thrust::host_vector<Object> &objects_host() const { return objects_; }
    const thrust::host_vector<node> &nodes_host() const { return nodes_; }
    bvh_device<T, Dim, Object> get_device_repr() const {
        return bvh_device<T, Dim, Object>{(unsigned int)nodes_.size(), (unsigned int)objects_.size(), nodes_.data(),
                                          aabbs_.data(), objects_.data()};
    }

  private:
    using Box = aabb<T, Dim>;
    using Vec = typename vector_of<T, Dim>::type;

    static void set(Vec &v, int k, double x) {
        if (k == 0) v.x = (T)x;
        else if (k == 1) v.y = (T)x;
        else if constexpr (Dim == 3) v.z = (T)x;
    }
    static Box merge(const Box &a, const Box &b) {
        Box r;
        for (int k = 0; k < (int)Dim; k++) {
            set(r.lower, k, std::min(detail::comp(a.lower, k), detail::comp(b.lower, k)));
            set(r.upper, k, std::max(detail::comp(a.upper, k), detail::comp(b.upper, k)));
        }
        return r;
    }
    static std::uint32_t spread(std::uint32_t x) {  // Dim == 3: 10 bits, two zeros between
        x = (x * 0x00010001u) & 0xFF0000FFu;
        x = (x * 0x00000101u) & 0x0F00F00Fu;
        x = (x * 0x00000011u) & 0xC30C30C3u;
        x = (x * 0x00000005u) & 0x49249249u;
        return x;
    }
    static std::uint32_t spread2(std::uint32_t x) {  // Dim == 2: 16 bits, one zero between
        x &= 0xFFFFu;
        x = (x | (x << 8)) & 0x00FF00FFu;
        x = (x | (x << 4)) & 0x0F0F0F0Fu;
        x = (x | (x << 2)) & 0x33333333u;
        x = (x | (x << 1)) & 0x55555555u;
        return x;
    }

    // Balanced binary tree over the sorted leaves [lo, hi): returns the node index.
    std::uint32_t make(std::uint32_t lo, std::uint32_t hi, std::uint32_t parent, std::uint32_t &next_internal) {
        const std::uint32_t n = (std::uint32_t)objects_.size();
        if (hi - lo == 1) {
            const std::uint32_t leaf = n - 1 + lo;
            nodes_[leaf].parent_idx = parent;
            return leaf;
        }
        const std::uint32_t me = next_internal++;
        const std::uint32_t mid = lo + (hi - lo) / 2;
        nodes_[me].parent_idx = parent;
        nodes_[me].object_idx = 0xFFFFFFFFu;
        nodes_[me].left_idx = make(lo, mid, me, next_internal);
        nodes_[me].right_idx = make(mid, hi, me, next_internal);
        aabbs_[me] = merge(aabbs_[nodes_[me].left_idx], aabbs_[nodes_[me].right_idx]);
        return me;
    }

    void build() {
        const std::uint32_t n = (std::uint32_t)objects_.size();
        AABBGetter get;
        std::vector<Box> boxes(n);
        Box scene;
        for (std::uint32_t i = 0; i < n; i++) {
            Box b = get(objects_[i]);
            double ext = 0.0;
            for (int k = 0; k < (int)Dim; k++)
                ext = std::max(ext, std::max(std::fabs(detail::comp(b.lower, k)), std::fabs(detail::comp(b.upper, k))));
            const double pad = 1e-5 * (ext + 1.0);
            for (int k = 0; k < (int)Dim; k++) {
                set(b.lower, k, detail::comp(b.lower, k) - pad);
                set(b.upper, k, detail::comp(b.upper, k) + pad);
            }
            boxes[i] = b;
            scene = i == 0 ? b : merge(scene, b);
        }
        std::vector<std::uint64_t> key(n);
        for (std::uint32_t i = 0; i < n; i++) {
            std::uint32_t code = 0;
            for (int k = 0; k < (int)Dim; k++) {
                const double lo = detail::comp(scene.lower, k), hi = detail::comp(scene.upper, k);
                const double c = 0.5 * (detail::comp(boxes[i].lower, k) + detail::comp(boxes[i].upper, k));
                const double u = hi > lo ? (c - lo) / (hi - lo) : 0.5;
                const std::uint32_t q = (std::uint32_t)std::min(std::max(u * (Dim == 3 ? 1024.0 : 65536.0), 0.0),
                                                                Dim == 3 ? 1023.0 : 65535.0);
                code |= (Dim == 3 ? spread(q) : spread2(q)) << k;
            }
            key[i] = ((std::uint64_t)code << 32) | i;
        }
        std::sort(key.begin(), key.end());
        nodes_.resize(2 * (size_t)n - 1);
        aabbs_.resize(2 * (size_t)n - 1);
        for (std::uint32_t i = 0; i < n; i++) {
            const std::uint32_t obj = (std::uint32_t)(key[i] & 0xFFFFFFFFu);
            node &leaf = nodes_[n - 1 + i];
            leaf.left_idx = leaf.right_idx = 0xFFFFFFFFu;
            leaf.object_idx = obj;
            aabbs_[n - 1 + i] = boxes[obj];
        }
        std::uint32_t next_internal = 0;
        if (n > 1) make(0, n, 0xFFFFFFFFu, next_internal);
        else nodes_[0].parent_idx = 0xFFFFFFFFu;
    }

    thrust::host_vector<Object> objects_;
    thrust::host_vector<node> nodes_;
    thrust::host_vector<Box> aabbs_;
};

// Every object the query's infinite line meets according to `intersect(line, object)` (a
// pair<bool, point>): the first max_buffer_size go to `out` as (object_idx, point) in depth-first
// order; the return value counts all of them.
template <typename T, unsigned int Dim, typename Object, typename Intersect, typename OutputIterator>
unsigned int query_device(const bvh_device<T, Dim, Object> &tree, const query_line_intersect<T, Dim> &q,
                          Intersect intersect, OutputIterator out, unsigned int max_buffer_size) {
    if (tree.num_objects == 0) return 0;
    std::uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;  // the root: internal node 0, or the single leaf
    unsigned int found = 0;
    while (sp > 0) {
        const std::uint32_t idx = stack[--sp];
        if (!detail::line_meets_box(q.line, tree.aabbs[idx])) continue;
        const node &nd = tree.nodes[idx];
        if (nd.object_idx != 0xFFFFFFFFu) {
            const auto r = intersect(q.line, tree.objects[nd.object_idx]);
            if (r.first) {
                if (found < max_buffer_size) *out++ = thrust::make_pair(nd.object_idx, r.second);
                found++;
            }
            continue;
        }
        if (sp + 2 > 128) break;
        stack[sp++] = nd.right_idx;
        stack[sp++] = nd.left_idx;
    }
    return found;
}

}  // namespace lbvh
