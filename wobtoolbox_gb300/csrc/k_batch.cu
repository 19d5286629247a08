// Batched walk: many scenes, each with its own parameters and evaluation points, in one persistent
// launch per walk class (at most three: backward single layer, forward single-layer Neumann, and
// the general walk). A device table holds, per scene, its scene view, walk parameters and first
// work unit; warps take units in a grid-stride loop and find their scene by bisection over the
// units' prefix. A unit is 32 * ppt paths of one point of one scene, so a warp never mixes scenes,
// and the per-scene work is exactly what a single-scene launch does (same walker variant, same
// paths, same values).
#include "kernels.cuh"

namespace wobgb {

// One unit (32 * ppt paths of one point) of a batched scene with the walker variant W; view and
// p are the scene's view and parameters staged in shared memory by the warp.
template <int D, class W>
__device__ __forceinline__ void batch_unit(const BatchEntry<D> &e, const SceneView<D> &view, const WalkParams &p,
                                           uint32_t lane, uint64_t local, const float *__restrict__ pts,
                                           double *__restrict__ sum, double *__restrict__ sumsq,
                                           uint64_t path_offset_add, unsigned long long &my_bounces) {
    const uint32_t pt = (uint32_t)(local / e.slabs);
    const uint32_t span = 32u * p.ppt;
    const uint32_t first = (uint32_t)(local % e.slabs) * span;
    const uint32_t row = e.point_begin + pt;
    V<D> x;
#pragma unroll
    for (int i = 0; i < D; i++) x.v[i] = __ldg(pts + (size_t)row * D + i);
    double acc[D + 1], acc2[D + 1];
#pragma unroll
    for (int c = 0; c <= D; c++) { acc[c] = 0.0; acc2[c] = 0.0; }
    for (uint32_t k = 0; k < p.ppt; k++) {
        const uint32_t path = first + k * 32u + lane;
        if (path < p.n_paths) {
            float out[D + 1];
            W w(view, p, kStreamDomain, p.point_offset + pt, p.path_offset + path_offset_add + path);
            w.domain(x, out);
            my_bounces += w.bounces;
#pragma unroll
            for (int c = 0; c <= D; c++) {
                const double v = (double)out[c];
                acc[c] += v;
                acc2[c] += v * v;
            }
        }
    }
    __syncwarp();
#pragma unroll
    for (int c = 0; c <= D; c++) {
        const double sv = warp_sum(acc[c]);
        const double qv = warp_sum(acc2[c]);
        if (lane == 0) {
            atomicAdd(sum + (size_t)row * (D + 1) + c, sv);
            if (sumsq) atomicAdd(sumsq + (size_t)row * (D + 1) + c, qv);
        }
    }
}

// One persistent launch per walk class: every scene of the launch runs the same walker variant
// (the specialisation a single-scene launch of that class uses); a warp finds its scene by
// bisection over the units' prefix.
template <int D, class W>
__global__ void __launch_bounds__(kBlock) batch_domain_kernel(const BatchEntry<D> *__restrict__ table,
                                                              uint32_t n_scenes, uint64_t total_units,
                                                              const float *__restrict__ pts, double *__restrict__ sum,
                                                              double *__restrict__ sumsq,
                                                              unsigned long long *__restrict__ bounces,
                                                              uint64_t path_offset_add) {
    __shared__ SceneView<D> s_view[kBlock / 32];
    __shared__ WalkParams s_params[kBlock / 32];
    const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long my_bounces = 0;
    uint32_t staged = 0xFFFFFFFFu;
    for (uint64_t u = warp; u < total_units; u += n_warps) {
        uint32_t lo = 0, hi = n_scenes - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) / 2;
            if (table[mid].unit_begin <= u) lo = mid;
            else hi = mid - 1;
        }
        const BatchEntry<D> &e = table[lo];
        if (lo != staged) {  // the warp's scene changed: stage its view and parameters
            __syncwarp();
            const uint32_t *sv = reinterpret_cast<const uint32_t *>(&e.view);
            uint32_t *dv = reinterpret_cast<uint32_t *>(&s_view[wib]);
            for (uint32_t i = lane; i < sizeof(SceneView<D>) / 4; i += 32) dv[i] = sv[i];
            const uint32_t *sp = reinterpret_cast<const uint32_t *>(&e.params);
            uint32_t *dp = reinterpret_cast<uint32_t *>(&s_params[wib]);
            for (uint32_t i = lane; i < sizeof(WalkParams) / 4; i += 32) dp[i] = sp[i];
            __syncwarp();
            staged = lo;
        }
        batch_unit<D, W>(e, s_view[wib], s_params[wib], lane, u - e.unit_begin, pts, sum, sumsq, path_offset_add,
                         my_bounces);
    }
    if (bounces) {
        __syncwarp();
        const unsigned long long b = warp_sum_u64(my_bounces);
        if (lane == 0 && b) atomicAdd(bounces, b);
    }
}

template <int D, class W>
cudaError_t launch_class(const BatchEntry<D> *table, uint32_t n_scenes, uint64_t total_units, const float *pts,
                         double *sum, double *sumsq, unsigned long long *bounces, uint64_t path_offset_add,
                         cudaStream_t stream) {
    auto k = batch_domain_kernel<D, W>;
    k<<<persistent_grid(k, total_units), kBlock, 0, stream>>>(table, n_scenes, total_units, pts, sum, sumsq, bounces,
                                                                path_offset_add);
    return cudaGetLastError();
}

template <int D>
cudaError_t launch_batch_impl(const BatchEntry<D> *table, uint32_t n_scenes, uint32_t cls, uint64_t total_units,
                              const float *pts, double *sum, double *sumsq, unsigned long long *bounces,
                              uint64_t path_offset_add, cudaStream_t stream) {
    if (total_units == 0 || n_scenes == 0) return cudaSuccess;
    if (cls == 1u)
        return launch_class<D, Walker<D, kSingleLayer, kStratSingleLayer, false, true>>(table, n_scenes, total_units, pts, sum,
                                                                                   sumsq, bounces, path_offset_add, stream);
    if (cls == 2u)
        return launch_class<D, Walker<D, kSingleLayer, kStratFwdSlNeumann, false, true>>(table, n_scenes, total_units, pts,
                                                                                    sum, sumsq, bounces, path_offset_add,
                                                                                    stream);
    return launch_class<D, Walker<D, -1, kStratRuntime, true, true>>(table, n_scenes, total_units, pts, sum, sumsq, bounces,
                                                                path_offset_add, stream);
}

cudaError_t launch_batch_2d(const BatchEntry<2> *table, uint32_t n_scenes, uint32_t cls, uint64_t total_units,
                            const float *pts, double *sum, double *sumsq, unsigned long long *bounces,
                            uint64_t path_offset_add, cudaStream_t stream) {
    return launch_batch_impl<2>(table, n_scenes, cls, total_units, pts, sum, sumsq, bounces, path_offset_add, stream);
}
cudaError_t launch_batch_3d(const BatchEntry<3> *table, uint32_t n_scenes, uint32_t cls, uint64_t total_units,
                            const float *pts, double *sum, double *sumsq, unsigned long long *bounces,
                            uint64_t path_offset_add, cudaStream_t stream) {
    return launch_batch_impl<3>(table, n_scenes, cls, total_units, pts, sum, sumsq, bounces, path_offset_add, stream);
}

}  // namespace wobgb
