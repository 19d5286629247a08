// Scene construction on the GPU from device arrays (no counterpart in the reference, whose
// SceneHost builds on the host, scene.cuh:264-299, with lbvh's build, scene.cuh:266).
//
// Produces the same packed records as build_host_scene (scene_build.cpp) -- element and 3D
// intersection records in storage order, area and |g| CDFs (Kahan prefix sums, normalised, made
// nondecreasing), guide tables, padded boxes -- with a different BVH topology: Morton codes of the
// element centroids, a bitonic sort of (code, caller index), a binary radix tree over the sorted
// codes (Karras, "Maximizing parallelism in the construction of BVHs, octrees, and k-d trees",
// HPG 2012), bottom-up boxes, and a top-down collapse into the 4-wide layout (each wide node takes
// its binary node's two children, each expanded once more when it holds more than kLeafMax
// elements). Storage order is the sorted order, so every leaf is a contiguous range and a
// depth-first traversal with children in order still returns hits in storage order; hit sets do
// not depend on the topology. The CDFs are computed by one thread in storage order with the host
// build's float operations (built with -fmad=false), so the sampling tables are bit-identical to a
// host build over the same storage order.
#include "scene_build_gpu.hpp"

#include "scene_host.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace wobgb {

namespace {

constexpr int kT = 256;

// order-preserving float <-> uint32 map (for atomicMin / atomicMax on floats)
__device__ __forceinline__ uint32_t ord(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ inline float unord(uint32_t u) {
    const uint32_t v = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
    float f;
    std::memcpy(&f, &v, 4);
    return f;
}

struct Bounds {  // ordered-uint encodings
    uint32_t lo[3], hi[3], clo[3], chi[3], mag;
    uint32_t bad;            // bit 0 non-finite vertex, 1 normal, 2 data, 3 alpha, 4 type, 5 normal length
    uint32_t all_dirichlet;  // 1 until a non-Dirichlet element is seen
};

__device__ __forceinline__ bool finite_f(float x) { return isfinite(x); }

template <int D>
__global__ void k_validate(uint32_t n, const float *__restrict__ verts, const float *__restrict__ normals,
                           const float *__restrict__ bvals, const float *__restrict__ alphas,
                           const int32_t *__restrict__ types, float *__restrict__ box, Bounds *b) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t bad = 0;
    const float *v = verts + (size_t)i * D * D;
    for (int k = 0; k < D * D; k++)
        if (!finite_f(v[k])) bad |= 1u;
    for (int k = 0; k < D; k++) {
        if (!finite_f(normals[(size_t)i * D + k])) bad |= 2u;
        if (!finite_f(bvals[(size_t)i * D + k])) bad |= 4u;
        if (alphas && !finite_f(alphas[(size_t)i * D + k])) bad |= 8u;
    }
    float q = 0.0f;
    for (int k = 0; k < D; k++) q += normals[(size_t)i * D + k] * normals[(size_t)i * D + k];
    if (!(q >= 0.25f && q <= 4.0f)) bad |= 32u;  // as the host build: normals far from unit length
    const int t = types[i];
    if (t < 0 || t > 2) bad |= 16u;
    if (bad) atomicOr(&b->bad, bad);
    if (t != 0) atomicAnd(&b->all_dirichlet, 0u);
    // element box, centroid (scene_build.cpp: lo / hi / s / dim, left to right)
    for (int k = D; k < 3; k++) box[(size_t)i * 9 + k] = box[(size_t)i * 9 + 3 + k] = box[(size_t)i * 9 + 6 + k] = 0.0f;
    float mag = 0.0f;
    for (int k = 0; k < D; k++) {
        float lo = v[k], hi = v[k], s = v[k];
        for (int j = 1; j < D; j++) {
            lo = fminf(lo, v[j * D + k]);
            hi = fmaxf(hi, v[j * D + k]);
            s = s + v[j * D + k];
        }
        const float c = s / (float)D;
        box[(size_t)i * 9 + k] = lo;
        box[(size_t)i * 9 + 3 + k] = hi;
        box[(size_t)i * 9 + 6 + k] = c;
        atomicMin(&b->lo[k], ord(lo));
        atomicMax(&b->hi[k], ord(hi));
        atomicMin(&b->clo[k], ord(c));
        atomicMax(&b->chi[k], ord(c));
        mag = fmaxf(mag, fmaxf(fabsf(lo), fabsf(hi)));
    }
    atomicMax(&b->mag, ord(mag));
}

__device__ __forceinline__ uint64_t spread21(uint64_t x) {  // 21 bits -> every third bit
    x &= 0x1FFFFFull;
    x = (x | (x << 32)) & 0x1F00000000FFFFull;
    x = (x | (x << 16)) & 0x1F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}
__device__ __forceinline__ uint64_t spread32(uint64_t x) {  // 32 bits -> every second bit
    x &= 0xFFFFFFFFull;
    x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
    x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
    x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
    x = (x | (x << 2)) & 0x3333333333333333ull;
    x = (x | (x << 1)) & 0x5555555555555555ull;
    return x;
}

template <int D>
__global__ void k_morton(uint32_t n, uint32_t n2, const float *__restrict__ box, const Bounds *b, uint64_t *key,
                         uint32_t *val) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n2) return;
    if (i >= n) {
        key[i] = ~0ull;
        val[i] = 0xFFFFFFFFu;
        return;
    }
    uint64_t q[3] = {0, 0, 0};
    const int bits = D == 3 ? 21 : 32;
    const double scale = (double)((1ull << bits) - 1);
    for (int k = 0; k < D; k++) {
        const double lo = (double)unord(b->clo[k]), hi = (double)unord(b->chi[k]);
        const double ext = hi - lo;
        const double x = ext > 0.0 ? ((double)box[(size_t)i * 9 + 6 + k] - lo) / ext : 0.0;
        q[k] = (uint64_t)fmin(fmax(x * scale, 0.0), scale);
    }
    key[i] = D == 3 ? (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2])
                    : (spread32(q[0]) << 1) | spread32(q[1]);
    val[i] = i;
}

__global__ void k_bitonic(uint32_t n2, uint32_t j, uint32_t k, uint64_t *key, uint32_t *val) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n2) return;
    const uint32_t l = i ^ j;
    if (l <= i) return;
    const uint64_t ka = key[i], kb = key[l];
    const uint32_t va = val[i], vb = val[l];
    const bool greater = ka > kb || (ka == kb && va > vb);
    const bool up = (i & k) == 0;
    if (up == greater) {
        key[i] = kb;
        key[l] = ka;
        val[i] = vb;
        val[l] = va;
    }
}

// common-prefix length of the augmented keys (code, index) at sorted positions a and b
__device__ __forceinline__ int delta(const uint64_t *key, int64_t n, int64_t a, int64_t b) {
    if (b < 0 || b >= n) return -1;
    const uint64_t ka = key[a], kb = key[b];
    if (ka != kb) return __clzll((long long)(ka ^ kb));
    return 64 + __clz((int)((uint32_t)a ^ (uint32_t)b));
}

constexpr uint32_t kLeafBit = 0x80000000u;

// Binary radix tree: internal node i has children child[2i], child[2i+1] (kLeafBit | sorted
// position for leaves) and covers sorted positions [first[i], last[i]].
__global__ void k_radix_tree(uint32_t n, const uint64_t *__restrict__ key, uint32_t *child, uint32_t *first,
                             uint32_t *last, uint32_t *parent_int, uint32_t *parent_leaf) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t N = n;
    if (i >= N - 1) return;
    const int d = (delta(key, N, i, i + 1) - delta(key, N, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(key, N, i, i - d);
    int64_t lmax = 2;
    while (delta(key, N, i, i + lmax * d) > dmin) lmax *= 2;
    int64_t l = 0;
    for (int64_t t = lmax / 2; t >= 1; t /= 2)
        if (delta(key, N, i, i + (l + t) * d) > dmin) l += t;
    const int64_t j = i + l * d;
    const int dnode = delta(key, N, i, j);
    int64_t s = 0, t = l;
    do {
        t = (t + 1) / 2;
        if (delta(key, N, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int64_t g = i + s * d + (d < 0 ? -1 : 0);
    const int64_t lo = i < j ? i : j, hi = i < j ? j : i;
    const uint32_t left = (lo == g) ? (kLeafBit | (uint32_t)g) : (uint32_t)g;
    const uint32_t right = (hi == g + 1) ? (kLeafBit | (uint32_t)(g + 1)) : (uint32_t)(g + 1);
    child[2 * i] = left;
    child[2 * i + 1] = right;
    first[i] = (uint32_t)lo;
    last[i] = (uint32_t)hi;
    if (left & kLeafBit) parent_leaf[left & ~kLeafBit] = (uint32_t)i;
    else parent_int[left] = (uint32_t)i;
    if (right & kLeafBit) parent_leaf[right & ~kLeafBit] = (uint32_t)i;
    else parent_int[right] = (uint32_t)i;
}

// Boxes of the binary nodes, bottom-up: the second child to arrive at a parent writes its box.
// A climb is bounded by the tree height (at most 96 levels for 64-bit codes plus 32 index bits);
// a longer one can only come from a malformed tree and sets bit 5 of the error word.
__global__ void k_boxes(uint32_t n, float pad, const uint32_t *__restrict__ val, const float *__restrict__ ebox,
                        const uint32_t *__restrict__ child, const uint32_t *__restrict__ parent_int,
                        const uint32_t *__restrict__ parent_leaf, uint32_t *flags, float *ibox, uint32_t *err) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n || n < 2) return;
    uint32_t node = parent_leaf[s];
    for (int level = 0;; level++) {
        if (level > 128 || node >= n - 1) {
            atomicOr(err, 32u);
            return;
        }
        __threadfence();
        if (atomicAdd(&flags[node], 1u) == 0u) return;
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int c = 0; c < 2; c++) {
            const uint32_t ch = child[2 * node + c];
            for (int k = 0; k < 3; k++) {
                float a, b;
                if (ch & kLeafBit) {
                    const uint32_t e = val[ch & ~kLeafBit];
                    a = ebox[(size_t)e * 9 + k] - pad;
                    b = ebox[(size_t)e * 9 + 3 + k] + pad;
                } else {
                    a = ((volatile float *)ibox)[(size_t)ch * 6 + k];
                    b = ((volatile float *)ibox)[(size_t)ch * 6 + 3 + k];
                }
                lo[k] = fminf(lo[k], a);
                hi[k] = fmaxf(hi[k], b);
            }
        }
        for (int k = 0; k < 3; k++) {
            ibox[(size_t)node * 6 + k] = lo[k];
            ibox[(size_t)node * 6 + 3 + k] = hi[k];
        }
        if (node == 0) return;
        node = parent_int[node];
    }
}

struct Slot {
    uint32_t code;  // binary child code (kLeafBit | sorted position, or internal index)
};

__device__ __forceinline__ uint32_t range_count(uint32_t code, const uint32_t *first, const uint32_t *last) {
    return (code & kLeafBit) ? 1u : last[code] - first[code] + 1u;
}

// The up to four binary nodes a wide node over binary node b holds, in range order.
__device__ __forceinline__ int wide_children(uint32_t b, const uint32_t *child, const uint32_t *first,
                                             const uint32_t *last, uint32_t out[4]) {
    int m = 0;
    for (int c = 0; c < 2; c++) {
        const uint32_t ch = child[2 * b + c];
        if (!(ch & kLeafBit) && range_count(ch, first, last) > kLeafMax) {
            out[m++] = child[2 * ch];
            out[m++] = child[2 * ch + 1];
        } else {
            out[m++] = ch;
        }
    }
    return m;
}

// per frontier item: how many of its children become wide nodes
__global__ void k_collapse_count(uint32_t cnt, const uint32_t *__restrict__ fb, const uint32_t *child,
                                 const uint32_t *first, const uint32_t *last, uint32_t *ncount) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    uint32_t ch[4];
    const int m = wide_children(fb[t], child, first, last, ch);
    uint32_t c = 0;
    for (int k = 0; k < m; k++)
        if (range_count(ch[k], first, last) > kLeafMax) c++;
    ncount[t] = c;
}

// exclusive scan of cnt values in one block; total written to *total
__global__ void k_scan(uint32_t cnt, const uint32_t *__restrict__ in, uint32_t *out, uint32_t *total) {
    __shared__ uint32_t part[1024];
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    const uint32_t chunk = (cnt + nt - 1) / nt;
    const uint32_t b = tid * chunk, e = min(cnt, b + chunk);
    uint32_t s = 0;
    for (uint32_t i = b; i < e; i++) s += in[i];
    part[tid] = s;
    __syncthreads();
    if (tid == 0) {
        uint32_t acc = 0;
        for (uint32_t k = 0; k < nt; k++) {
            const uint32_t v = part[k];
            part[k] = acc;
            acc += v;
        }
        *total = acc;
    }
    __syncthreads();
    uint32_t acc = part[tid];
    for (uint32_t i = b; i < e; i++) {
        out[i] = acc;
        acc += in[i];
    }
}

// writes the wide node records of one frontier level and the next frontier
template <int D>
__global__ void k_collapse_write(uint32_t cnt, const uint32_t *__restrict__ fw, const uint32_t *__restrict__ fb,
                                 const uint32_t *__restrict__ offs, uint32_t base, const uint32_t *child,
                                 const uint32_t *first, const uint32_t *last, const uint32_t *__restrict__ val,
                                 const float *__restrict__ ebox, const float *__restrict__ ibox, float pad, float *nodes,
                                 uint32_t *nw, uint32_t *nb) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    constexpr int NF = D == 2 ? 24 : 32;
    float *r = nodes + (size_t)fw[t] * NF;
    uint32_t ch[4];
    const int m = wide_children(fb[t], child, first, last, ch);
    uint32_t next = base + offs[t];
    for (int k = 0; k < 4; k++) {
        uint32_t code = kChildEmpty;
        float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
        if (k < m) {
            const uint32_t c = ch[k];
            const uint32_t count = range_count(c, first, last);
            const uint32_t f = (c & kLeafBit) ? (c & ~kLeafBit) : first[c];
            if (count > kLeafMax) {
                code = next;
                nw[next - base] = next;
                nb[next - base] = c;
                next++;
            } else {
                code = 0x80000000u | ((count - 1u) << 28) | f;
            }
            for (int a = 0; a < D; a++) {
                if (c & kLeafBit) {
                    const uint32_t e = val[c & ~kLeafBit];
                    lo[a] = ebox[(size_t)e * 9 + a] - pad;
                    hi[a] = ebox[(size_t)e * 9 + 3 + a] + pad;
                } else {
                    lo[a] = ibox[(size_t)c * 6 + a];
                    hi[a] = ibox[(size_t)c * 6 + 3 + a];
                }
            }
        }
        for (int a = 0; a < D; a++) {
            r[4 * a + k] = lo[a];
            r[4 * (D + a) + k] = hi[a];
        }
        r[4 * (2 * D) + k] = __uint_as_float(code);
        r[4 * (2 * D + 1) + k] = 0.0f;  // padding to a 32-byte multiple
    }
}

// element records, intersection records, area and |g| weights in storage order (scene_build.cpp)
template <int D>
__global__ void k_records(uint32_t n, const uint32_t *__restrict__ val, const float *__restrict__ verts,
                          const float *__restrict__ normals, const float *__restrict__ bvals,
                          const float *__restrict__ alphas, const int32_t *__restrict__ types, float *elems,
                          float *elem_aux, float *isect, float *areas, float *bvw) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t i = val[s];
    const float *v = verts + (size_t)i * D * D;
    const float *nn = normals + (size_t)i * D;
    const float *bv = bvals + (size_t)i * D;
    float al[3] = {0, 0, 0};
    if (alphas)
        for (int k = 0; k < D; k++) al[k] = alphas[(size_t)i * D + k];
    if constexpr (D == 2) {
        float *r = elems + (size_t)s * 16;
        const float dx = v[2] - v[0], dy = v[3] - v[1];
        const float area = sqrtf(dx * dx + dy * dy);
        r[0] = v[0]; r[1] = v[1]; r[2] = v[2]; r[3] = v[3];
        r[4] = nn[0]; r[5] = nn[1]; r[6] = bv[0]; r[7] = bv[1];
        r[8] = al[0]; r[9] = al[1]; r[10] = area; r[11] = __int_as_float(types[i]);
        r[12] = 0.0f; r[13] = 0.0f; r[14] = 0.0f; r[15] = 0.0f;
        areas[s] = area;
        bvw[s] = area * (fabsf(bv[0]) + fabsf(bv[1])) / 2.0f;
    } else {
        float *r = elems + (size_t)s * 16;
        float *aux = elem_aux + (size_t)s * 4;
        const float u0 = v[6] - v[0], u1 = v[7] - v[1], u2 = v[8] - v[2];
        const float w0 = v[3] - v[0], w1 = v[4] - v[1], w2 = v[5] - v[2];
        const float x = u1 * w2 - u2 * w1;
        const float y = u2 * w0 - u0 * w2;
        const float z = u0 * w1 - u1 * w0;
        const float area = sqrtf(x * x + y * y + z * z) / 2.0f;
        for (int k = 0; k < 9; k++) r[k] = v[k];
        r[9] = nn[0]; r[10] = nn[1]; r[11] = nn[2];
        r[12] = bv[0]; r[13] = bv[1]; r[14] = bv[2]; r[15] = __int_as_float(types[i]);
        aux[0] = al[0]; aux[1] = al[1]; aux[2] = al[2]; aux[3] = area;
        areas[s] = area;
        bvw[s] = area * (fabsf(bv[0]) + fabsf(bv[1]) + fabsf(bv[2])) / 3.0f;
        float *q = isect + (size_t)s * 16;
        const float e1x = v[0] - v[3], e1y = v[1] - v[4], e1z = v[2] - v[5];
        const float e2x = v[0] - v[6], e2y = v[1] - v[7], e2z = v[2] - v[8];
        q[0] = v[0]; q[1] = v[1]; q[2] = v[2];
        q[3] = e1x; q[4] = e1y; q[5] = e1z;
        q[6] = e2x; q[7] = e2y; q[8] = e2z;
        q[9] = e1y * e2z - e1z * e2y;
        q[10] = e1z * e2x - e1x * e2z;
        q[11] = e1x * e2y - e1y * e2x;
        q[12] = 0.0f; q[13] = 0.0f; q[14] = 0.0f; q[15] = 0.0f;
    }
}

// Kahan prefix sums, normalisation and the nondecreasing fix-up of scene_build.cpp's kahan_cdf:
// thread 0 builds the area CDF, thread 1 the |g| CDF, each serially in storage order.
__global__ void k_kahan_cdf(uint32_t n, const float *__restrict__ areas, const float *__restrict__ bvw,
                            float *area_cdf, float *bv_cdf, float *totals) {
    const int w = threadIdx.x;
    if (w > 1) return;
    const float *in = w == 0 ? areas : bvw;
    float *cdf = w == 0 ? area_cdf : bv_cdf;
    float sum = 0.0f, c = 0.0f;
    for (uint32_t i = 0; i < n; i++) {
        const float y = in[i] - c;
        const float t = sum + y;
        c = (t - sum) - y;
        sum = t;
        cdf[i] = sum;
    }
    const float total = sum;
    totals[w] = total;
    float prev = -INFINITY;
    for (uint32_t i = 0; i < n; i++) {
        float v = cdf[i] / total;
        if (i > 0 && v < prev) v = prev;
        cdf[i] = v;
        prev = v;
    }
}

// guide table (scene_build.cpp build_guide): first index whose CDF reaches (j - 1/2)/G
__device__ __forceinline__ uint32_t guide_first(const float *cdf, uint32_t n, uint32_t G, uint32_t j) {
    const double thr = ((double)j - 0.5) / (double)G;
    uint32_t lo = 0, hi = n - 1;  // answer in [0, n-1]: first i with cdf[i] >= thr, else n-1
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if ((double)cdf[mid] < thr) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}
__global__ void k_guide(uint32_t n, uint32_t G, const float *__restrict__ cdf, uint32_t *rec) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= G) return;
    const uint32_t lo = guide_first(cdf, n, G, j);
    const uint32_t hi = (j + 2 < G) ? guide_first(cdf, n, G, j + 2) : n - 1;
    rec[4 * (size_t)j + 0] = lo;
    rec[4 * (size_t)j + 1] = hi;
    rec[4 * (size_t)j + 2] = __float_as_uint(cdf[lo]);
    rec[4 * (size_t)j + 3] = __float_as_uint(cdf[min(lo + 1, n - 1)]);
}

struct Tmp {
    std::vector<void *> ptrs;
    ~Tmp() {
        for (void *p : ptrs) cudaFree(p);
    }
    template <class T> cudaError_t alloc(T **p, size_t count) {
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) ptrs.push_back(q);
        *p = (T *)q;
        return e;
    }
};

inline uint32_t blocks(uint64_t n) { return (uint32_t)((n + kT - 1) / kT); }

template <int D>
std::string build_impl(uint32_t n, const float *verts, const float *normals, const float *bvals, const float *alphas,
                       const int32_t *types, cudaStream_t st, DeviceSceneBuild &out, cudaError_t &ce) {
    Tmp tmp;
#define WOB_CK(x)                            \
    do {                                     \
        if ((ce = (x)) != cudaSuccess) return "CUDA error"; \
    } while (0)
    float *box = nullptr;
    Bounds *bd = nullptr;
    WOB_CK(tmp.alloc(&box, (size_t)n * 9));
    WOB_CK(tmp.alloc(&bd, 1));
    Bounds init;
    for (int k = 0; k < 3; k++) {
        init.lo[k] = init.clo[k] = 0xFFFFFFFFu;
        init.hi[k] = init.chi[k] = 0u;
    }
    init.mag = 0u;
    init.bad = 0u;
    init.all_dirichlet = 1u;
    WOB_CK(cudaMemcpyAsync(bd, &init, sizeof(Bounds), cudaMemcpyHostToDevice, st));
    k_validate<D><<<blocks(n), kT, 0, st>>>(n, verts, normals, bvals, alphas, types, box, bd);
    WOB_CK(cudaGetLastError());
    Bounds hb;
    WOB_CK(cudaMemcpyAsync(&hb, bd, sizeof(Bounds), cudaMemcpyDeviceToHost, st));
    WOB_CK(cudaStreamSynchronize(st));
    if (hb.bad & 1u) return "vertices must be finite";
    if (hb.bad & 2u) return "normals must be finite";
    if (hb.bad & 4u) return "boundary values must be finite";
    if (hb.bad & 8u) return "robin alphas must be finite";
    if (hb.bad & 16u) return "boundary_types must be 0 (Dirichlet), 1 (Neumann) or 2 (Robin)";
    if (hb.bad & 32u) return "normals must be unit vectors";
    out.all_dirichlet = hb.all_dirichlet != 0u;
    // padding of the host build: 1e-5 (extent + max |coordinate|)
    float ext = 0.0f;
    for (int k = 0; k < D; k++) ext = std::max(ext, unord(hb.hi[k]) - unord(hb.lo[k]));
    const float pad = 1e-5f * (ext + unord(hb.mag)) + 1e-30f;

    // Morton codes and the sort
    uint32_t n2 = 1;
    while (n2 < n) n2 <<= 1;
    uint64_t *key = nullptr;
    uint32_t *val = nullptr;
    WOB_CK(tmp.alloc(&key, n2));
    WOB_CK(tmp.alloc(&val, n2));
    k_morton<D><<<blocks(n2), kT, 0, st>>>(n, n2, box, bd, key, val);
    for (uint32_t k = 2; k <= n2; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1) k_bitonic<<<blocks(n2), kT, 0, st>>>(n2, j, k, key, val);
    WOB_CK(cudaGetLastError());

    constexpr int NF = D == 2 ? 24 : 32;
    const uint32_t n_int = n > 1 ? n - 1 : 1;
    float *nodes = nullptr;
    WOB_CK(cudaMalloc(&nodes, (size_t)n_int * NF * 4));
    out.nodes = nodes;
    out.nodes_bytes = (size_t)n_int * NF * 4;
    uint32_t n_nodes = 1, depth = 1;
    if (n <= kLeafMax) {
        // one wide node holding one leaf (scene_build.cpp)
        std::vector<float> root(NF, 0.0f);
        std::vector<float> hbox(9 * (size_t)n);
        WOB_CK(cudaMemcpyAsync(hbox.data(), box, hbox.size() * 4, cudaMemcpyDeviceToHost, st));
        WOB_CK(cudaStreamSynchronize(st));
        for (int a = 0; a < D; a++) {
            float lo = INFINITY, hi = -INFINITY;
            for (uint32_t i = 0; i < n; i++) {
                lo = std::min(lo, hbox[9 * i + a] - pad);
                hi = std::max(hi, hbox[9 * i + 3 + a] + pad);
            }
            root[4 * a] = lo;
            root[4 * (D + a)] = hi;
        }
        const uint32_t codes[4] = {make_leaf(0, n), kChildEmpty, kChildEmpty, kChildEmpty};
        for (int k = 0; k < 4; k++) std::memcpy(&root[4 * (2 * D) + k], &codes[k], 4);
        WOB_CK(cudaMemcpyAsync(nodes, root.data(), NF * 4, cudaMemcpyHostToDevice, st));
    } else {
        uint32_t *child, *first, *last, *pint, *pleaf, *flags;
        float *ibox;
        WOB_CK(tmp.alloc(&child, 2 * (size_t)n_int));
        WOB_CK(tmp.alloc(&first, n_int));
        WOB_CK(tmp.alloc(&last, n_int));
        WOB_CK(tmp.alloc(&pint, n_int));
        WOB_CK(tmp.alloc(&pleaf, n));
        WOB_CK(tmp.alloc(&flags, n_int));
        WOB_CK(tmp.alloc(&ibox, 6 * (size_t)n_int));
        WOB_CK(cudaMemsetAsync(flags, 0, (size_t)n_int * 4, st));
        k_radix_tree<<<blocks(n - 1), kT, 0, st>>>(n, key, child, first, last, pint, pleaf);
        k_boxes<<<blocks(n), kT, 0, st>>>(n, pad, val, box, child, pint, pleaf, flags, ibox, &bd->bad);
        WOB_CK(cudaGetLastError());
        // top-down collapse, one level per step
        uint32_t *fw[2], *fb[2], *cnt, *offs, *total;
        for (int b = 0; b < 2; b++) {
            WOB_CK(tmp.alloc(&fw[b], n_int));
            WOB_CK(tmp.alloc(&fb[b], n_int));
        }
        WOB_CK(tmp.alloc(&cnt, n_int));
        WOB_CK(tmp.alloc(&offs, n_int));
        WOB_CK(tmp.alloc(&total, 1));
        const uint32_t zero = 0;
        WOB_CK(cudaMemcpyAsync(fw[0], &zero, 4, cudaMemcpyHostToDevice, st));
        WOB_CK(cudaMemcpyAsync(fb[0], &zero, 4, cudaMemcpyHostToDevice, st));
        uint32_t level_count = 1, cur = 0;
        depth = 0;
        while (level_count > 0) {
            depth++;
            if (3 * depth + 2 > kTraversalStack) return "BVH too deep for the traversal stack";
            k_collapse_count<<<blocks(level_count), kT, 0, st>>>(level_count, fb[cur], child, first, last, cnt);
            k_scan<<<1, 1024, 0, st>>>(level_count, cnt, offs, total);
            k_collapse_write<D><<<blocks(level_count), kT, 0, st>>>(level_count, fw[cur], fb[cur], offs, n_nodes,
                                                                   child, first, last, val, box, ibox, pad, nodes,
                                                                   fw[1 - cur], fb[1 - cur]);
            WOB_CK(cudaGetLastError());
            uint32_t next = 0;
            WOB_CK(cudaMemcpyAsync(&next, total, 4, cudaMemcpyDeviceToHost, st));
            WOB_CK(cudaStreamSynchronize(st));
            n_nodes += next;
            level_count = next;
            cur = 1 - cur;
        }
    }
    out.n_nodes = n_nodes;
    out.depth = depth;

    // records, CDFs, guides
    const int EF = 16;
    float *elems = nullptr, *elem_aux = nullptr, *isect = nullptr, *area_cdf = nullptr, *bv_cdf = nullptr, *areas,
          *bvw, *totals;
    WOB_CK(cudaMalloc(&elems, (size_t)n * EF * 4));
    out.elems = elems;
    out.elems_bytes = (size_t)n * EF * 4;
    if (D == 3) {
        WOB_CK(cudaMalloc(&elem_aux, (size_t)n * 4 * 4));
        out.elem_aux = elem_aux;
        out.elem_aux_bytes = (size_t)n * 4 * 4;
        WOB_CK(cudaMalloc(&isect, (size_t)n * 16 * 4));
        out.isect = isect;
        out.isect_bytes = (size_t)n * 16 * 4;
    }
    WOB_CK(cudaMalloc(&area_cdf, (size_t)n * 4));
    out.area_cdf = area_cdf;
    out.area_cdf_bytes = (size_t)n * 4;
    WOB_CK(cudaMalloc(&bv_cdf, (size_t)n * 4));
    out.bv_cdf = bv_cdf;
    out.bv_cdf_bytes = (size_t)n * 4;
    WOB_CK(tmp.alloc(&areas, n));
    WOB_CK(tmp.alloc(&bvw, n));
    WOB_CK(tmp.alloc(&totals, 2));
    k_records<D><<<blocks(n), kT, 0, st>>>(n, val, verts, normals, bvals, alphas, types, elems, elem_aux, isect, areas,
                                           bvw);
    k_kahan_cdf<<<1, 32, 0, st>>>(n, areas, bvw, area_cdf, bv_cdf, totals);
    WOB_CK(cudaGetLastError());
    float ht[2];
    WOB_CK(cudaMemcpyAsync(ht, totals, 8, cudaMemcpyDeviceToHost, st));
    WOB_CK(cudaMemcpyAsync(&hb, bd, sizeof(Bounds), cudaMemcpyDeviceToHost, st));
    out.order.resize(n);
    WOB_CK(cudaMemcpyAsync(out.order.data(), val, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
    WOB_CK(cudaStreamSynchronize(st));
    if (hb.bad & 32u) return "BVH build failed: malformed radix tree";
    out.total_area = ht[0];
    out.total_bv = ht[1];
    if (!(out.total_area > 0.0f) || !std::isfinite(out.total_area)) return "total boundary area must be positive and finite";
    const uint32_t G = std::max<uint32_t>(1u, std::min<uint32_t>(n, 1u << 22));
    uint32_t *ag = nullptr, *bg = nullptr;
    WOB_CK(cudaMalloc(&ag, (size_t)G * 16));
    out.area_guide = ag;
    out.area_guide_bytes = (size_t)G * 16;
    out.area_G = G;
    k_guide<<<blocks(G), kT, 0, st>>>(n, G, area_cdf, ag);
    out.bv_valid = out.total_bv > 0.0f && std::isfinite(out.total_bv);
    const uint32_t Gb = out.bv_valid ? G : 1u;
    WOB_CK(cudaMalloc(&bg, (size_t)Gb * 16));
    out.bv_guide = bg;
    out.bv_guide_bytes = (size_t)Gb * 16;
    out.bv_G = Gb;
    if (out.bv_valid) k_guide<<<blocks(G), kT, 0, st>>>(n, G, bv_cdf, bg);
    else WOB_CK(cudaMemsetAsync(bg, 0, 16, st));
    WOB_CK(cudaGetLastError());
    WOB_CK(cudaStreamSynchronize(st));
#undef WOB_CK
    return "";
}

}  // namespace

void DeviceSceneBuild::release() {
    for (void **p : {&elems, &elem_aux, &isect, &nodes, &area_cdf, &area_guide, &bv_cdf, &bv_guide}) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
}

std::string build_device_scene(int dim, uint32_t n, const float *verts, const float *normals, const float *bvals,
                               const float *alphas, const int32_t *types, cudaStream_t stream, DeviceSceneBuild &out,
                               cudaError_t &cuda_error) {
    cuda_error = cudaSuccess;
    if (dim != 2 && dim != 3) return "dim must be 2 or 3";
    if (n == 0) return "a scene needs at least one element";
    if (n > kMaxElements) return "too many elements";
    if (!verts || !normals || !bvals || !types) return "vertices, normals, boundary_values and boundary_types are required";
    std::string err = dim == 2 ? build_impl<2>(n, verts, normals, bvals, alphas, types, stream, out, cuda_error)
                               : build_impl<3>(n, verts, normals, bvals, alphas, types, stream, out, cuda_error);
    if (!err.empty()) out.release();
    return err;
}

}  // namespace wobgb
