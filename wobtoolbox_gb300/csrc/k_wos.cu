// Walk on spheres for the 2D interior Dirichlet problem, the baseline method of
// apps/simple_wob_and_wos.cu:49-78 (closest-point query) and :111-137 (WoSFunc).
//
// A walk jumps from x to a uniform point on the largest empty circle around it (radius R = distance
// to the boundary) until R < eps, then takes the boundary value at the closest boundary point. The
// closest-point query runs on the scene's 4-wide BVH: depth-first, children sorted by box distance,
// a subtree pruned when its box is farther than the best distance so far. Among elements at the
// same distance the one with the smallest storage index wins, so the result does not depend on
// the traversal order (the oracle scans all elements in storage order with the same rule).
//
// Work decomposition as the walk kernels (a warp runs the paths of one point, FP64 sums per point),
// with path regeneration inside a warp (see wos_kernel).
// A walk stops after kWosMaxSteps jumps (or the scene's lower test override) at the latest (taking the value at its current closest
// point); such walks are counted in the scene's error word (kErrWosStepLimit).
#include "kernels.cuh"
#include "wos.hpp"

namespace wobgb {

namespace {

constexpr uint32_t kStreamWos = 3u;
constexpr uint32_t kFullMask = 0xffffffffu;

struct Closest {
    float d2;
    uint32_t elem;
    float t;
};

// squared distance from p to segment i and the clamped parameter (apps/simple_wob_and_wos.cu:54-60)
__device__ __forceinline__ float seg_dist2(const SceneView<2> &s, uint32_t i, const V<2> &p, float &t_out) {
    const float4 q0 = __ldg(s.elems + 4 * i);
    const float ax = q0.x, ay = q0.y;
    const float lx = q0.z - ax, ly = q0.w - ay;
    float t = ((p.v[0] - ax) * lx + (p.v[1] - ay) * ly) / (lx * lx + ly * ly);
    t = fminf(fmaxf(t, 0.0f), 1.0f);
    const float cx = (ax + lx * t) - p.v[0], cy = (ay + ly * t) - p.v[1];
    t_out = t;
    return cx * cx + cy * cy;
}

__device__ __forceinline__ float box_dist2(float lx, float ly, float hx, float hy, const V<2> &p) {
    const float dx = fmaxf(fmaxf(lx - p.v[0], 0.0f), p.v[0] - hx);
    const float dy = fmaxf(fmaxf(ly - p.v[1], 0.0f), p.v[1] - hy);
    return dx * dx + dy * dy;
}

__device__ __forceinline__ Closest closest_point(const SceneView<2> &s, const V<2> &p) {
    Closest best{INFINITY, 0xFFFFFFFFu, 0.0f};
    uint32_t stack[kStackSize];
    int sp = 0;
    stack[sp++] = 0u;
    uint32_t steps = 0;
    while (sp > 0) {
        if (++steps > s.traversal_limit) {
            atomicOr(s.err, kErrTraversalLimit);
            break;
        }
        const uint32_t code = stack[--sp];
        if (code & 0x80000000u) {
            const uint32_t first = code & 0x0FFFFFFFu, cnt = ((code >> 28) & 7u) + 1u;
            for (uint32_t i = first; i < first + cnt; i++) {
                float t;
                const float d2 = seg_dist2(s, i, p, t);
                if (d2 < best.d2 || (d2 == best.d2 && i < best.elem)) best = Closest{d2, i, t};
            }
            continue;
        }
        const float4 *q = s.nodes + 6 * code;
        const F8 r0 = ldg8(q), r1 = ldg8(q + 2);
        const float4 lx = r0.a, ly = r0.b, hx = r1.a, hy = r1.b, cf = __ldg(q + 4);
        const float lxs[4] = {lx.x, lx.y, lx.z, lx.w}, lys[4] = {ly.x, ly.y, ly.z, ly.w};
        const float hxs[4] = {hx.x, hx.y, hx.z, hx.w}, hys[4] = {hy.x, hy.y, hy.z, hy.w};
        const uint32_t cs[4] = {__float_as_uint(cf.x), __float_as_uint(cf.y), __float_as_uint(cf.z),
                                __float_as_uint(cf.w)};
        float dk[4];
        int ord[4], m = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            dk[k] = box_dist2(lxs[k], lys[k], hxs[k], hys[k], p);
            if (cs[k] != kChildEmptyD && dk[k] <= best.d2) ord[m++] = k;
        }
        // push the farthest first so the nearest is visited next
        for (int a = 1; a < m; a++)
            for (int b = a; b > 0 && dk[ord[b]] > dk[ord[b - 1]]; b--) {
                const int tmp = ord[b];
                ord[b] = ord[b - 1];
                ord[b - 1] = tmp;
            }
        if (sp + m > (int)kStackSize) {
            atomicOr(s.err, kErrStackOverflow);
            break;
        }
        for (int a = 0; a < m; a++) stack[sp++] = cs[ord[a]];
    }
    return best;
}

// boundary value at the closest point: (g_b - g_a) t + g_a (apps/simple_wob_and_wos.cu:70-73)
__device__ __forceinline__ float closest_value(const SceneView<2> &s, const Closest &c) {
    const float4 q1 = __ldg(s.elems + 4 * c.elem + 1);
    return (q1.w - q1.z) * c.t + q1.z;
}

// A warp runs the 32 * ppt paths of one unit (one point) with path regeneration: when a lane's walk
// ends, the lane takes the next path of the unit, so walks of different lengths do not leave lanes
// idle until the longest one finishes. A path (apps/simple_wob_and_wos.cu:120-133) is its own
// Philox stream: query the closest point, stop below eps (or after kWosMaxSteps jumps) with the
// boundary value there, else jump by the distance in direction 2 pi u; the values do not depend on
// which lane runs a path.
__global__ void __launch_bounds__(kBlock) wos_kernel(SceneView<2> s, WalkParams p, const float *__restrict__ pts,
                                                     uint32_t n_points, double *__restrict__ sum,
                                                     double *__restrict__ sumsq, unsigned long long *__restrict__ queries,
                                                     float *__restrict__ per_path) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t span = 32u * p.ppt;
    const uint32_t slabs = (p.n_paths + span - 1u) / span;
    const uint64_t units = (uint64_t)n_points * slabs;
    unsigned long long my_q = 0;
    for (uint64_t u = warp; u < units; u += n_warps) {
        const uint32_t pt = (uint32_t)(u / slabs);
        const uint32_t first = (uint32_t)(u % slabs) * span;
        const uint32_t end = min(first + span, p.n_paths);
        V<2> x0;
        x0.v[0] = __ldg(pts + 2 * (size_t)pt);
        x0.v[1] = __ldg(pts + 2 * (size_t)pt + 1);
        uint32_t path = first + lane;
        uint32_t next = first + 32u;
        bool active = path < end;
        PathRng rng(p.seed, kStreamWos, p.point_offset + pt, p.path_offset + path);
        V<2> x = x0;
        uint32_t step = 0;
        double acc = 0.0, acc2 = 0.0;
        while (__any_sync(kFullMask, active)) {
            bool done = false;
            if (active) {
                // one step of the path
                const Closest c = closest_point(s, x);
                my_q++;
                const float R = sqrtf(c.d2);
                float out = 0.0f;
                if (R < p.eps || c.elem == 0xFFFFFFFFu) {
                    out = c.elem == 0xFFFFFFFFu ? 0.0f : closest_value(s, c);
                    done = true;
                } else if (step + 1 >= s.wos_step_limit) {
                    atomicOr(s.err, kErrWosStepLimit);
                    out = closest_value(s, c);
                    done = true;
                } else {
                    float sn, cs;
                    sincospi_own(2.0f * rng.uniform(), &sn, &cs);
                    x.v[0] = x.v[0] + R * cs;
                    x.v[1] = x.v[1] + R * sn;
                    step++;
                }
                if (done) {
                    const double v = (double)out;
                    acc += v;
                    acc2 += v * v;
                    if (per_path) per_path[(size_t)pt * p.n_paths + path] = out;
                }
            }
            const uint32_t fin = __ballot_sync(kFullMask, done);
            if (fin) {
                if (done) {
                    path = next + __popc(fin & ((1u << lane) - 1u));
                    active = path < end;
                    if (active) {
                        rng = PathRng(p.seed, kStreamWos, p.point_offset + pt, p.path_offset + path);
                        x = x0;
                        step = 0;
                    }
                }
                next += __popc(fin);
            }
        }
        if (sum) {
            __syncwarp();
            const double sv = warp_sum(acc);
            const double qv = warp_sum(acc2);
            if (lane == 0) {
                atomicAdd(sum + pt, sv);
                if (sumsq) atomicAdd(sumsq + pt, qv);
            }
        }
    }
    if (queries) {
        __syncwarp();
        const unsigned long long b = warp_sum_u64(my_q);
        if (lane == 0 && b) atomicAdd(queries, b);
    }
}

__global__ void closest_point_kernel(SceneView<2> s, const float *__restrict__ pts, uint32_t n, uint32_t *elem,
                                     float *dist2, float *value) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    V<2> x;
    x.v[0] = pts[2 * (size_t)i];
    x.v[1] = pts[2 * (size_t)i + 1];
    const Closest c = closest_point(s, x);
    elem[i] = c.elem;
    dist2[i] = c.d2;
    value[i] = c.elem == 0xFFFFFFFFu ? 0.0f : closest_value(s, c);
}

}  // namespace

cudaError_t launch_wos_2d(const SceneView<2> &s, const WalkParams &p, const float *pts, uint32_t n_points, double *sum,
                          double *sumsq, unsigned long long *queries, float *per_path, cudaStream_t st) {
    if (n_points == 0) return cudaSuccess;
    WalkParams q = p;
    q.ppt = choose_ppt(n_points, p.n_paths);
    const uint64_t units = (uint64_t)n_points * ((p.n_paths + 32u * q.ppt - 1u) / (32u * q.ppt));
    auto k = wos_kernel;
    k<<<persistent_grid(k, units), kBlock, 0, st>>>(s, q, pts, n_points, sum, sumsq, queries, per_path);
    return cudaGetLastError();
}

cudaError_t launch_closest_point_2d(const SceneView<2> &s, const float *pts, uint32_t n, uint32_t *elem, float *dist2,
                                    float *value, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    closest_point_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(s, pts, n, elem, dist2, value);
    return cudaGetLastError();
}

}  // namespace wobgb
