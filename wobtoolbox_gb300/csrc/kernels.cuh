// Kernels of the general walk: domain estimator, boundary estimator, their per-path debug
// variants and the line query. Instantiated per dimension in kernels_2d.cu / kernels_3d.cu.
//
// Work decomposition: a "unit" is 32 consecutive paths of one evaluation point, run by one warp
// (lane = path). Warps take units in a grid-stride loop over a persistent grid sized from the
// occupancy of the kernel; after a unit the warp reduces its 32 contributions in FP64 with
// shuffles and lane 0 adds them to the point's running sums. Paths are independent Philox
// streams, so the schedule has no influence on any path's value.
#pragma once

#include "launch.hpp"
#include "walk_generic.cuh"

namespace wobgb {

constexpr int kBlock = kWalkBlock;  // threads per block of the walk kernels

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// kMinB: minimum resident blocks per SM requested from the register allocator (1 = no limit);
// the autotuner chooses among the compiled values.
//
// A unit is 32 * ppt consecutive paths of one point: lane l runs paths l, l + 32, ... and keeps
// its running (sum, sum of squares) in FP64, so the FP64 warp reduction and the atomics happen
// once per unit instead of once per 32 paths. For the uniform-sampling and the backward
// single-layer walks the running sums live in shared memory (one slot per thread, touched once
// per path) instead of 16 registers live through the walk (measured: 33.4 -> 34.0 G bounces/s on
// the 3D Robin benchmark, 201 -> 198 ms per iteration of the single-layer walk on 1.3 M
// triangles); the line-query walks keep them in registers, because they rely on L1 hits that the
// shared-memory carve-out would take (the 2D line-grid walk lost 7 %).
template <int D, int kBie, int kStrat, bool kVol, bool kPerPath, int kMinB = 1>
__global__ void __launch_bounds__(kBlock, kMinB) domain_kernel(SceneView<D> s, WalkParams p, const float *__restrict__ pts,
                                                        uint32_t n_points, double *__restrict__ sum,
                                                        double *__restrict__ sumsq,
                                                        unsigned long long *__restrict__ bounces,
                                                        float *__restrict__ per_path) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t span = 32u * p.ppt;
    const uint32_t slabs = (p.n_paths + span - 1u) / span;
    const uint64_t units = (uint64_t)n_points * slabs;
    constexpr bool kSharedSums = kStrat == kStratUniform || kStrat == kStratSingleLayer;
    constexpr int kSlots = kSharedSums ? kBlock : 1;
    __shared__ double acc_s[2 * (D + 1)][kSlots];  // [c]: running sum, [D + 1 + c]: sum of squares
    double acc_r[2 * (D + 1)];
    const uint32_t tid = threadIdx.x;
    auto acc = [&](int c) -> double & {
        if constexpr (kSharedSums) return acc_s[c][tid];
        else return acc_r[c];
    };
    unsigned long long my_bounces = 0;
    for (uint64_t u = warp; u < units; u += n_warps) {
        const uint32_t pt = (uint32_t)(u / slabs);
        const uint32_t first = (uint32_t)(u % slabs) * span;
        V<D> x;
#pragma unroll
        for (int i = 0; i < D; i++) x.v[i] = __ldg(pts + (size_t)pt * D + i);
#pragma unroll
        for (int c = 0; c < 2 * (D + 1); c++) acc(c) = 0.0;
        for (uint32_t k = 0; k < p.ppt; k++) {
            const uint32_t path = first + k * 32u + lane;
            if (path < p.n_paths) {
                float out[D + 1];
                Walker<D, kBie, kStrat, kVol> w(s, p, kStreamDomain, p.point_offset + pt, p.path_offset + path);
                w.domain(x, out);
                my_bounces += w.bounces;
                if (kPerPath) {
#pragma unroll
                    for (int c = 0; c <= D; c++) per_path[((size_t)pt * p.n_paths + path) * (D + 1) + c] = out[c];
                } else {
#pragma unroll
                    for (int c = 0; c <= D; c++) {
                        const double v = (double)out[c];
                        acc(c) += v;
                        acc(D + 1 + c) += v * v;
                    }
                }
            }
        }
        if (!kPerPath) {
            __syncwarp();
#pragma unroll
            for (int c = 0; c <= D; c++) {
                const double sv = warp_sum(acc(c));
                const double qv = warp_sum(acc(D + 1 + c));
                if (lane == 0) {
                    atomicAdd(sum + (size_t)pt * (D + 1) + c, sv);
                    if (sumsq) atomicAdd(sumsq + (size_t)pt * (D + 1) + c, qv);
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

template <int D, int kBie, int kStrat, bool kVol, bool kPerPath>
__global__ void __launch_bounds__(kBlock) boundary_kernel(SceneView<D> s, WalkParams p, BoundaryInput bin,
                                                          uint32_t n_points, double *__restrict__ sum,
                                                          double *__restrict__ sumsq,
                                                          unsigned long long *__restrict__ bounces,
                                                          float *__restrict__ per_path) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t slabs = (p.n_paths + 31u) / 32u;
    const uint64_t units = (uint64_t)n_points * slabs;
    unsigned long long my_bounces = 0;
    for (uint64_t u = warp; u < units; u += n_warps) {
        const uint32_t pt = (uint32_t)(u / slabs);
        const uint32_t path = (uint32_t)(u % slabs) * 32u + lane;
        const bool active = path < p.n_paths;
        float out = 0.0f;
        if (active) {
            BPoint<D> x;
#pragma unroll
            for (int i = 0; i < D; i++) {
                x.p.v[i] = __ldg(bin.p + (size_t)pt * D + i);
                x.n.v[i] = __ldg(bin.n + (size_t)pt * D + i);
            }
            x.angle = __ldg(bin.angle + pt);
            x.bv = __ldg(bin.bv + pt);
            x.type = __ldg(bin.type + pt);
            x.alpha = bin.alpha ? __ldg(bin.alpha + pt) : 0.0f;
            Walker<D, kBie, kStrat, kVol> w(s, p, kStreamBoundary, p.point_offset + pt, p.path_offset + path);
            out = p.mode == 1 ? w.unknown_boundary(x) : w.boundary(x);
            my_bounces += w.bounces;
            if (kPerPath) per_path[(size_t)pt * p.n_paths + path] = out;
        }
        if (!kPerPath) {
            __syncwarp();
            const double v = active ? (double)out : 0.0;
            const double sv = warp_sum(v);
            const double qv = warp_sum(v * v);
            if (lane == 0) {
                atomicAdd(sum + pt, sv);
                if (sumsq) atomicAdd(sumsq + pt, qv);
            }
        }
    }
    if (bounces) {
        __syncwarp();
        const unsigned long long b = warp_sum_u64(my_bounces);
        if (lane == 0 && b) atomicAdd(bounces, b);
    }
}

// Control-variate domain estimator (forward single layer, Neumann): as domain_kernel with
// ppt = 1, the per-path estimate from Walker::domain_cv.
template <int D>
__global__ void __launch_bounds__(kBlock) domain_cv_kernel(SceneView<D> s, WalkParams p, const float *__restrict__ pts,
                                                           uint32_t n_points, double *__restrict__ sum,
                                                           double *__restrict__ sumsq,
                                                           unsigned long long *__restrict__ bounces,
                                                           float *__restrict__ per_path) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t slabs = (p.n_paths + 31u) / 32u;
    const uint64_t units = (uint64_t)n_points * slabs;
    unsigned long long my_bounces = 0;
    for (uint64_t u = warp; u < units; u += n_warps) {
        const uint32_t pt = (uint32_t)(u / slabs);
        const uint32_t path = (uint32_t)(u % slabs) * 32u + lane;
        const bool active = path < p.n_paths;
        float out[D + 1];
#pragma unroll
        for (int c = 0; c <= D; c++) out[c] = 0.0f;
        if (active) {
            V<D> x;
#pragma unroll
            for (int i = 0; i < D; i++) x.v[i] = __ldg(pts + (size_t)pt * D + i);
            Walker<D, kSingleLayer, kStratFwdSlNeumann, false> w(s, p, kStreamDomain, p.point_offset + pt,
                                                                 p.path_offset + path);
            w.domain_cv(x, s.cv_table, out);
            my_bounces += w.bounces;
            if (per_path) {
#pragma unroll
                for (int c = 0; c <= D; c++) per_path[((size_t)pt * p.n_paths + path) * (D + 1) + c] = out[c];
            }
        }
        if (!per_path) {
            __syncwarp();
#pragma unroll
            for (int c = 0; c <= D; c++) {
                const double v = active ? (double)out[c] : 0.0;
                const double sv = warp_sum(v);
                const double qv = warp_sum(v * v);
                if (lane == 0) {
                    atomicAdd(sum + (size_t)pt * (D + 1) + c, sv);
                    if (sumsq) atomicAdd(sumsq + (size_t)pt * (D + 1) + c, qv);
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

template <int D>
cudaError_t launch_domain_cv_impl(const SceneView<D> &s, const WalkParams &p, const float *pts, uint32_t n_points,
                                  double *sum, double *sumsq, unsigned long long *bounces, float *per_path,
                                  cudaStream_t stream) {
    const uint64_t units = (uint64_t)n_points * ((p.n_paths + 31u) / 32u);
    auto k = domain_cv_kernel<D>;
    k<<<persistent_grid(k, units), kBlock, 0, stream>>>(s, p, pts, n_points, sum, sumsq, bounces, per_path);
    return cudaGetLastError();
}

template <int D>
__global__ void __launch_bounds__(kBlock) line_query_kernel(SceneView<D> s, const float *__restrict__ origins,
                                                            const float *__restrict__ dirs, uint32_t n,
                                                            uint32_t *__restrict__ counts,
                                                            uint32_t *__restrict__ hits_out,
                                                            float *__restrict__ points_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    V<D> o, d;
#pragma unroll
    for (int k = 0; k < D; k++) {
        o.v[k] = origins[(size_t)i * D + k];
        d.v[k] = dirs[(size_t)i * D + k];
    }
    uint32_t hits[kHitBuffer];
    const uint32_t c = line_query<D>(s, o, d, hits);
    counts[i] = c;
    const uint32_t m = c < kHitBuffer ? c : kHitBuffer;
    for (uint32_t k = 0; k < m; k++) {
        hits_out[(size_t)i * kHitBuffer + k] = hits[k];
        if (points_out) {
            float t = 0.0f;
            isect_elem<D>(s, hits[k], o, d, t);
#pragma unroll
            for (int j = 0; j < D; j++) points_out[((size_t)i * kHitBuffer + k) * D + j] = o.v[j] + t * d.v[j];
        }
    }
}

template <class K>
inline int persistent_grid(K kernel, uint64_t work_warps) {
    int dev = 0, sm_count = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, 0);
    if (per_sm < 1) per_sm = 1;
    const uint64_t full = (uint64_t)sm_count * (uint64_t)per_sm;
    const uint64_t need = (work_warps + (kBlock / 32) - 1) / (kBlock / 32);
    uint64_t g = need < full ? need : full;
    if (g < 1) g = 1;
    return (int)g;
}

template <int D, int kBie, int kStrat, bool kVol, int kMinB>
cudaError_t launch_domain_variant(const SceneView<D> &s, const WalkParams &p_in, const float *pts, uint32_t n_points,
                                  double *sum, double *sumsq, unsigned long long *bounces, float *per_path,
                                  cudaStream_t stream) {
    WalkParams p = p_in;
    p.ppt = choose_ppt(p.ppt_points ? p.ppt_points : n_points, p.n_paths);
    if (p.ppt_cap && p.ppt > p.ppt_cap) p.ppt = p.ppt_cap;
    const uint64_t units = (uint64_t)n_points * ((p.n_paths + 32u * p.ppt - 1u) / (32u * p.ppt));
    if (per_path) {
        auto k = domain_kernel<D, kBie, kStrat, kVol, true, kMinB>;
        k<<<persistent_grid(k, units), kBlock, 0, stream>>>(s, p, pts, n_points, sum, sumsq, bounces, per_path);
    } else {
        auto k = domain_kernel<D, kBie, kStrat, kVol, false, kMinB>;
        k<<<persistent_grid(k, units), kBlock, 0, stream>>>(s, p, pts, n_points, sum, sumsq, bounces, nullptr);
    }
    return cudaGetLastError();
}

template <int D, int kBie, int kStrat, bool kVol>
cudaError_t launch_boundary_variant(const SceneView<D> &s, const WalkParams &p, const BoundaryInput &bin,
                                    uint32_t n_points, double *sum, double *sumsq, unsigned long long *bounces,
                                    float *per_path, cudaStream_t stream) {
    const uint64_t units = (uint64_t)n_points * ((p.n_paths + 31u) / 32u);
    if (per_path) {
        auto k = boundary_kernel<D, kBie, kStrat, kVol, true>;
        k<<<persistent_grid(k, units), kBlock, 0, stream>>>(s, p, bin, n_points, sum, sumsq, bounces, per_path);
    } else {
        auto k = boundary_kernel<D, kBie, kStrat, kVol, false>;
        k<<<persistent_grid(k, units), kBlock, 0, stream>>>(s, p, bin, n_points, sum, sumsq, bounces, nullptr);
    }
    return cudaGetLastError();
}

template <int D>
cudaError_t launch_line_query_impl(const SceneView<D> &s, const float *origins, const float *dirs, uint32_t n,
                                   uint32_t *counts, uint32_t *hits, float *points, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const uint32_t g = (n + kBlock - 1) / kBlock;
    line_query_kernel<D><<<g, kBlock, 0, stream>>>(s, origins, dirs, n, counts, hits, points);
    return cudaGetLastError();
}

}  // namespace wobgb
