// Forward single-layer Neumann walk in 3D (estimator.cuh:405-454, the exterior Neumann workload's
// estimator) as a per-lane state machine, so that no lane waits for another lane's line query.
//
// In the plain kernel (kernels.cuh) a warp's 32 paths run their bounces in lockstep: every lane
// issues its line query, and the warp moves on only when the longest of the 32 traversals ends,
// while inside a traversal lanes split between node tests and triangle tests. Here every loop
// iteration advances each lane by one traversal step (one node's four boxes or one leaf's
// triangles) of its own current query. A lane whose query ends in that iteration finishes the
// bounce (hit choice, weight, accumulation) and starts its next query, or its next path, at once;
// the warp only waits at the end of a unit of paths. Each lane runs the same operations on its
// path as the plain walk, in the same order, with its own Philox stream, so every path value is
// bit-identical to the plain kernel's and the CPU oracle's; the transport after the last bounce,
// which no output uses, is skipped as in the plain kernel.
//
// Work decomposition as the plain kernel: a persistent grid, a warp takes units of 32 x ppt paths
// of one point, lane l runs paths l, l + 32, ... of the unit one after the other; FP64 running
// sums per lane, reduced over the warp once per unit.
#include "kernels.cuh"

namespace wobgb {

namespace {

constexpr int kFwdBlock = 128;

enum : int { kLaneIdle = 0, kLaneNewPath = 1, kLaneQuery = 2 };

// kBatch: a loop iteration advances a lane by one batch of its traversal (nodes until 8 leaves are
// held, then those leaves: LineTraversal3::step_batch) instead of one stack entry.
template <bool kPerPath, bool kBatch, int kMinB>
__global__ void __launch_bounds__(kFwdBlock, kMinB) fwd_wavefront_kernel(SceneView<3> s, WalkParams p,
                                                                        const float *__restrict__ pts,
                                                                        uint32_t n_points, double *__restrict__ sum,
                                                                        double *__restrict__ sumsq,
                                                                        unsigned long long *__restrict__ bounces,
                                                                        float *__restrict__ per_path) {
    using W = Walker<3, kSingleLayer, kStratFwdSlNeumann, false>;
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t span = 32u * p.ppt;
    const uint32_t slabs = (p.n_paths + span - 1u) / span;
    const uint64_t units = (uint64_t)n_points * slabs;
    const uint32_t L = p.path_length;
    LineTraversal3 tr;
    unsigned long long my_bounces = 0;
    for (uint64_t u = warp; u < units; u += n_warps) {
        const uint32_t pt = (uint32_t)(u / slabs);
        const uint32_t first = (uint32_t)(u % slabs) * span;
        V<3> x;
#pragma unroll
        for (int i = 0; i < 3; i++) x.v[i] = __ldg(pts + (size_t)pt * 3 + i);
        double acc[8];
#pragma unroll
        for (int c = 0; c < 8; c++) acc[c] = 0.0;
        uint32_t k = 0;  // this lane's path within the unit: first + 32 k + lane
        int phase = (first + lane < p.n_paths) ? kLaneNewPath : kLaneIdle;
        W w(s, p, kStreamDomain, p.point_offset + pt, p.path_offset + first + lane);
        float out[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        float wt = 0.0f;
        uint32_t m = 0;
        BPoint<3> y = bp_zero<3>(), y_prev = bp_zero<3>();
        while (__any_sync(0xffffffffu, phase != kLaneIdle)) {
            bool start_bounce = false;
            if (phase == kLaneNewPath) {
                // path start (Walker::domain, forward branch)
                const uint32_t path = first + 32u * k + lane;
                // the walker's per-path state, as a freshly constructed walker has it
                w.rng = PathRng(p.seed, kStreamDomain, p.point_offset + pt, p.path_offset + path);
                w.bounces = 0;
                w.stayed = false;
                float ip, ip2;
                y = sample_uniform<3>(s, w.rng, ip);
                out[0] = w.sdk(x, y, ip);
                const V<3> g = w.gdk(x, y, ip);
#pragma unroll
                for (int i = 0; i < 3; i++) out[1 + i] = g.v[i];
                y = sample_boundary_value<3>(s, w.rng, ip);
                const BPoint<3> y2 = sample_uniform<3>(s, w.rng, ip2);
                wt = ip * w.fbk(y, y2, ip2);
                m = 0;
                start_bounce = true;
            } else if (phase == kLaneQuery) {
                if (kBatch ? tr.step_batch(s) : tr.step(s)) {
                    uint32_t mh;
                    const BPoint<3> yn = line_sample_from_hits<3>(s, w.rng, y_prev.p, tr.d, tr.hits, tr.count, mh);
                    const float ip = line_sample_inv_pdf<3>(yn, y_prev.p, mh);
                    y = yn;
                    wt = w.fbu(y, y_prev, ip, false) * wt;
                    m++;
                    start_bounce = true;
                }
            }
            if (start_bounce) {
                w.bounces++;
                if (m == L - 1) wt = wt * 0.5f;
                out[0] = out[0] + wt * w.sdu(x, y, 1.0f);
                const V<3> gu = w.gdu(x, y, 1.0f);
#pragma unroll
                for (int i = 0; i < 3; i++) out[1 + i] = out[1 + i] + wt * gu.v[i];
                if (m == L - 1) {
                    // path done: record it, then the lane's next path of the unit (next iteration)
                    const uint32_t path = first + 32u * k + lane;
                    if (kPerPath) {
#pragma unroll
                        for (int c = 0; c <= 3; c++) per_path[((size_t)pt * p.n_paths + path) * 4 + c] = out[c];
                    } else {
#pragma unroll
                        for (int c = 0; c <= 3; c++) {
                            const double v = (double)out[c];
                            acc[c] += v;
                            acc[4 + c] += v * v;
                        }
                    }
                    my_bounces += w.bounces;
                    k++;
                    phase = (k < p.ppt && first + 32u * k + lane < p.n_paths) ? kLaneNewPath : kLaneIdle;
                } else {
                    y_prev = y;
                    const V<3> dir = line_sample_direction<3>(w.rng);
                    tr.begin(y_prev.p, dir);
                    phase = kLaneQuery;
                }
            }
        }
        if (!kPerPath) {
            __syncwarp();
#pragma unroll
            for (int c = 0; c <= 3; c++) {
                const double sv = warp_sum(acc[c]);
                const double qv = warp_sum(acc[4 + c]);
                if (lane == 0) {
                    atomicAdd(sum + (size_t)pt * 4 + c, sv);
                    if (sumsq) atomicAdd(sumsq + (size_t)pt * 4 + c, qv);
                }
            }
        }
    }
    if (bounces) {
        __syncwarp();
        const unsigned long long b = warp_sum_u64(my_bounces);
        if (lane == 0 && b) atomicAdd(bounces, b);
    }
}

}  // namespace

template <bool kBatch, int kMinB>
static cudaError_t launch_mode(const SceneView<3> &s, const WalkParams &p, const float *pts, uint32_t n_points,
                               double *sum, double *sumsq, unsigned long long *bounces, float *per_path,
                               uint64_t units, cudaStream_t stream) {
    if (per_path) {
        auto k = fwd_wavefront_kernel<true, kBatch, kMinB>;
        k<<<persistent_grid(k, units), kFwdBlock, 0, stream>>>(s, p, pts, n_points, sum, sumsq, bounces, per_path);
    } else {
        auto k = fwd_wavefront_kernel<false, kBatch, kMinB>;
        k<<<persistent_grid(k, units), kFwdBlock, 0, stream>>>(s, p, pts, n_points, sum, sumsq, bounces, nullptr);
    }
    return cudaGetLastError();
}

cudaError_t launch_fwd_wavefront_3d(const SceneView<3> &s, const WalkParams &p_in, const float *pts, uint32_t n_points,
                                    double *sum, double *sumsq, unsigned long long *bounces, float *per_path,
                                    int mode, cudaStream_t stream) {
    WalkParams p = p_in;
    p.ppt = choose_ppt(n_points, p.n_paths);
    if (p.ppt_cap && p.ppt > p.ppt_cap) p.ppt = p.ppt_cap;
    const uint64_t units = (uint64_t)n_points * ((p.n_paths + 32u * p.ppt - 1u) / (32u * p.ppt));
    switch (mode) {
    case 0: return launch_mode<false, 4>(s, p, pts, n_points, sum, sumsq, bounces, per_path, units, stream);
    case 1: return launch_mode<true, 4>(s, p, pts, n_points, sum, sumsq, bounces, per_path, units, stream);
    default: return launch_mode<true, 1>(s, p, pts, n_points, sum, sumsq, bounces, per_path, units, stream);
    }
}

}  // namespace wobgb
