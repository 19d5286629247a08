// Work of the reference's BVH query on a workload, for the roofline constants N_node and N_prim
// (mean nodes visited and primitives tested per line query). TEST INFRASTRUCTURE ONLY.
//
// The reference's BVH is lbvh (scene.cuh:266, query at :483-486 / :787-790), a binary LBVH with one
// object per leaf, queried for every leaf box an infinite line crosses. Its source is absent, so
// this restates the structure it is documented to build: Morton codes of the object centroids
// (10 bits per axis in 3D, 16 in 2D, normalised to the centroid bounds), objects sorted by code, a
// binary radix tree (Karras, HPG 2012) with tight object boxes; the query is a stack traversal
// that pops a node (one node visited), tests both children's boxes against the line, pushes crossed
// internal children and tests the object of every crossed leaf child (one primitive test).
#pragma once

#include "wob_oracle.hpp"

#include <algorithm>
#include <cstdint>
#include <vector>

namespace wob_oracle {

template <int D> struct BinaryLbvh {
    struct Box {
        float lo[3], hi[3];
    };
    int n = 0;
    std::vector<int> left, right;  // child >= 0: internal node; child < 0: leaf -(object + 1)
    std::vector<Box> ibox, lbox;   // internal node boxes, object boxes

    explicit BinaryLbvh(const Scene<D> &s, float pad = 0.0f) {
        n = (int)s.elems.size();
        lbox.resize(n);
        std::vector<float> cen((size_t)n * 3, 0.0f);
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int i = 0; i < n; i++) {
            const Element<D> &e = s.elems[i];
            for (int k = 0; k < 3; k++) {
                lbox[i].lo[k] = 0.0f;
                lbox[i].hi[k] = 0.0f;
            }
            for (int k = 0; k < D; k++) {
                float lo = e.v[0].v[k], hi = e.v[0].v[k], c = 0.0f;
                for (int j = 0; j < D; j++) {
                    lo = std::min(lo, e.v[j].v[k]);
                    hi = std::max(hi, e.v[j].v[k]);
                    c += e.v[j].v[k];
                }
                lbox[i].lo[k] = lo - pad;
                lbox[i].hi[k] = hi + pad;
                cen[3 * i + k] = c / D;
                clo[k] = std::min(clo[k], cen[3 * i + k]);
                chi[k] = std::max(chi[k], cen[3 * i + k]);
            }
        }
        std::vector<std::pair<uint64_t, int>> code((size_t)n);
        const int bits = D == 3 ? 10 : 16;
        for (int i = 0; i < n; i++) {
            uint64_t key = 0;
            uint32_t q[3] = {0, 0, 0};
            for (int k = 0; k < D; k++) {
                const float ext = chi[k] - clo[k];
                const float x = ext > 0.0f ? (cen[3 * i + k] - clo[k]) / ext : 0.0f;
                q[k] = (uint32_t)std::min<float>(std::max(x * (float)((1 << bits) - 1), 0.0f), (float)((1 << bits) - 1));
            }
            for (int b = bits - 1; b >= 0; b--)
                for (int k = 0; k < D; k++) key = (key << 1) | ((q[k] >> b) & 1u);
            code[i] = {key, i};
        }
        std::sort(code.begin(), code.end());
        if (n < 2) return;
        left.assign(n - 1, 0);
        right.assign(n - 1, 0);
        ibox.resize(n - 1);
        auto delta = [&](int a, int b) -> int {
            if (b < 0 || b >= n) return -1;
            const uint64_t ka = code[a].first, kb = code[b].first;
            if (ka != kb) return __builtin_clzll(ka ^ kb);
            return 64 + __builtin_clz((uint32_t)a ^ (uint32_t)b);
        };
        std::vector<int> first(n - 1), last(n - 1);
        for (int i = 0; i < n - 1; i++) {
            const int d = (delta(i, i + 1) - delta(i, i - 1)) >= 0 ? 1 : -1;
            const int dmin = delta(i, i - d);
            int lmax = 2;
            while (delta(i, i + lmax * d) > dmin) lmax *= 2;
            int l = 0;
            for (int t = lmax / 2; t >= 1; t /= 2)
                if (delta(i, i + (l + t) * d) > dmin) l += t;
            const int j = i + l * d;
            const int dn = delta(i, j);
            int sidx = 0, t = l;
            do {
                t = (t + 1) / 2;
                if (delta(i, i + (sidx + t) * d) > dn) sidx += t;
            } while (t > 1);
            const int g = i + sidx * d + std::min(d, 0);
            const int lo = std::min(i, j), hi = std::max(i, j);
            left[i] = (lo == g) ? -(code[g].second + 1) : g;
            right[i] = (hi == g + 1) ? -(code[g + 1].second + 1) : g + 1;
            first[i] = lo;
            last[i] = hi;
        }
        // boxes bottom-up: process internal nodes by increasing range length
        std::vector<int> ord(n - 1);
        for (int i = 0; i < n - 1; i++) ord[i] = i;
        std::sort(ord.begin(), ord.end(), [&](int a, int b) { return last[a] - first[a] < last[b] - first[b]; });
        for (int i : ord) {
            Box b;
            for (int k = 0; k < 3; k++) {
                b.lo[k] = INFINITY;
                b.hi[k] = -INFINITY;
            }
            for (int c : {left[i], right[i]}) {
                const Box &cb = c < 0 ? lbox[-c - 1] : ibox[c];
                for (int k = 0; k < 3; k++) {
                    b.lo[k] = std::min(b.lo[k], cb.lo[k]);
                    b.hi[k] = std::max(b.hi[k], cb.hi[k]);
                }
            }
            ibox[i] = b;
        }
    }

    static bool crosses(const Box &b, const float *o, const float *d) {
        if (D == 2) {
            // the line's implicit function takes both signs over the box corners
            float mn = INFINITY, mx = -INFINITY;
            for (int cx = 0; cx < 2; cx++)
                for (int cy = 0; cy < 2; cy++) {
                    const double px = cx ? b.hi[0] : b.lo[0], py = cy ? b.hi[1] : b.lo[1];
                    const float f = (float)(d[0] * (py - o[1]) - d[1] * (px - o[0]));
                    mn = std::min(mn, f);
                    mx = std::max(mx, f);
                }
            return mn <= 0.0f && mx >= 0.0f;
        }
        double tn = -INFINITY, tf = INFINITY;
        for (int k = 0; k < 3; k++) {
            if (d[k] == 0.0f) {
                if (o[k] < b.lo[k] || o[k] > b.hi[k]) return false;
                continue;
            }
            double t1 = (b.lo[k] - o[k]) / (double)d[k], t2 = (b.hi[k] - o[k]) / (double)d[k];
            if (t1 > t2) std::swap(t1, t2);
            tn = std::max(tn, t1);
            tf = std::min(tf, t2);
        }
        return tn <= tf;
    }

    // the objects whose (padded) boxes the line crosses; UINT32_MAX when more than cap
    unsigned candidates(const float *o, const float *d, unsigned *cand, unsigned cap) const {
        unsigned m = 0;
        if (n < 2) {
            for (int i = 0; i < n; i++) cand[m++] = (unsigned)i;
            return m;
        }
        int stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const int node = stack[--sp];
            for (int c : {left[node], right[node]}) {
                const Box &b = c < 0 ? lbox[-c - 1] : ibox[c];
                if (!crosses(b, o, d)) continue;
                if (c < 0) {
                    if (m == cap) return 0xFFFFFFFFu;
                    cand[m++] = (unsigned)(-c - 1);
                } else if (sp < 128) {
                    stack[sp++] = c;
                } else {
                    return 0xFFFFFFFFu;
                }
            }
        }
        return m;
    }
    static unsigned candidates_cb(const void *self, const float *o, const float *d, unsigned *cand, unsigned cap) {
        return static_cast<const BinaryLbvh *>(self)->candidates(o, d, cand, cap);
    }

    // adds the nodes visited and primitives tested by one infinite-line query
    void count(const float *o, const float *d, uint64_t &nodes, uint64_t &prims) const {
        if (n < 2) {
            prims += (uint64_t)n;
            nodes += 1;
            return;
        }
        int stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const int node = stack[--sp];
            nodes++;
            for (int c : {left[node], right[node]}) {
                const Box &b = c < 0 ? lbox[-c - 1] : ibox[c];
                if (!crosses(b, o, d)) continue;
                if (c < 0) prims++;
                else if (sp < 128) stack[sp++] = c;
            }
        }
    }
};

template <int D> struct LbvhCounter : LineQueryObserver {
    const BinaryLbvh<D> *tree;
    uint64_t queries = 0, nodes = 0, prims = 0;
    explicit LbvhCounter(const BinaryLbvh<D> *t) : tree(t) {}
    void on_line(const float *o, const float *d, int) override {
        queries++;
        tree->count(o, d, nodes, prims);
    }
};

}  // namespace wob_oracle
