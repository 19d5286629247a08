// Training data of the learned control variate, prepared on the device.
//
// Boundary points drawn uniformly by area: point i is Philox stream 2 of point index i, drawn
// exactly as the walk's uniform boundary sample (sample_uniform, scene.cuh:441-462 / 734-758),
// with its element's normal, the interior angle 1/2, the interpolated boundary value, type and
// Robin alpha.
//
// Label clipping: the walk's density estimates have heavy tails (a few paths with grazing line
// intersections carry 1/cos weights), and a mean-squared fit chases those few labels. Values are
// clamped to [-t, t], t = the k-th smallest |v| with k = ceil(q n), found exactly by a radix
// select on the bit pattern of |v| (non-negative floats order as their bits): three histogram
// passes over bits 30-20, 19-10 and 9-0, each followed by a one-block scan that narrows the
// prefix and the remaining rank, all on the caller's stream with no host round trip.
#include "device_common.cuh"
#include "launch.hpp"

#include <algorithm>

namespace wobgb {

namespace {

constexpr uint32_t kStreamTraining = 2u;

template <int D>
__global__ void sample_boundary_kernel(SceneView<D> s, uint32_t n, uint64_t seed, float *__restrict__ p,
                                       float *__restrict__ nrm, float *__restrict__ angle, float *__restrict__ bv,
                                       int32_t *__restrict__ type, float *__restrict__ alpha) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    PathRng rng(seed, kStreamTraining, i, 0ull);
    float ip;
    const BPoint<D> y = sample_uniform<D>(s, rng, ip);
#pragma unroll
    for (int k = 0; k < D; k++) {
        p[(size_t)i * D + k] = y.p.v[k];
        nrm[(size_t)i * D + k] = y.n.v[k];
    }
    angle[i] = y.angle;
    bv[i] = y.bv;
    type[i] = y.type;
    if (alpha) alpha[i] = y.alpha;
}


struct ClipState {
    uint32_t prefix_mask, prefix_value, rank, pad;
};

constexpr int kClipPasses = 3;
__host__ __device__ constexpr int clip_shift(int pass) { return pass == 0 ? 20 : pass == 1 ? 10 : 0; }
__host__ __device__ constexpr int clip_bits(int pass) { return pass == 0 ? 11 : 10; }

__global__ void clip_init_kernel(ClipState *st, uint32_t *hist, uint32_t n, float quantile) {
    const uint32_t i = threadIdx.x;
    for (uint32_t b = i; b < 2048u; b += blockDim.x) hist[b] = 0;
    if (i == 0) {
        double k = ceil((double)quantile * (double)n);
        if (k < 1.0) k = 1.0;
        if (k > (double)n) k = (double)n;
        st->prefix_mask = 0;
        st->prefix_value = 0;
        st->rank = (uint32_t)k;  // 1-based rank among the values still matching the prefix
    }
}

__global__ void clip_hist_kernel(const float *__restrict__ v, uint32_t n, const ClipState *__restrict__ st, int pass,
                                 uint32_t *__restrict__ hist) {
    __shared__ uint32_t sh[2048];
    const int bins = 1 << clip_bits(pass);
    for (int b = threadIdx.x; b < bins; b += blockDim.x) sh[b] = 0;
    __syncthreads();
    const uint32_t mask = st->prefix_mask, val = st->prefix_value;
    const int shift = clip_shift(pass);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t a = __float_as_uint(v[i]) & 0x7fffffffu;
        if ((a & mask) == val) atomicAdd(&sh[(a >> shift) & (uint32_t)(bins - 1)], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < bins; b += blockDim.x)
        if (sh[b]) atomicAdd(&hist[b], sh[b]);
}

// One block: the bin holding the remaining rank, by a running count over the bins in order.
__global__ void clip_select_kernel(ClipState *st, uint32_t *hist, int pass) {
    const int bins = 1 << clip_bits(pass);
    if (threadIdx.x == 0) {
        uint32_t below = 0, rank = st->rank;
        int b = 0;
        for (; b < bins - 1; b++) {
            if (below + hist[b] >= rank) break;
            below += hist[b];
        }
        const int shift = clip_shift(pass);
        st->prefix_mask |= (uint32_t)(bins - 1) << shift;
        st->prefix_value |= (uint32_t)b << shift;
        st->rank = rank - below;
    }
    __syncthreads();
    for (int b = threadIdx.x; b < 2048; b += blockDim.x) hist[b] = 0;
}

__global__ void clip_apply_kernel(float *__restrict__ v, uint32_t n, const ClipState *__restrict__ st,
                                  float *__restrict__ threshold) {
    const float t = __uint_as_float(st->prefix_value);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0 && threshold) *threshold = t;
    if (i < n) v[i] = fminf(fmaxf(v[i], -t), t);
}

}  // namespace

template <int D>
cudaError_t launch_sample_boundary(const SceneView<D> &s, uint32_t n, uint64_t seed, float *p, float *nrm,
                                   float *angle, float *bv, int32_t *type, float *alpha, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    sample_boundary_kernel<D><<<(n + 255) / 256, 256, 0, stream>>>(s, n, seed, p, nrm, angle, bv, type, alpha);
    return cudaGetLastError();
}
template cudaError_t launch_sample_boundary<2>(const SceneView<2> &, uint32_t, uint64_t, float *, float *, float *,
                                               float *, int32_t *, float *, cudaStream_t);
template cudaError_t launch_sample_boundary<3>(const SceneView<3> &, uint32_t, uint64_t, float *, float *, float *,
                                               float *, int32_t *, float *, cudaStream_t);

}  // namespace wobgb

namespace wobgb {

cudaError_t launch_clip_quantile(float *values, uint32_t n, float quantile, float *threshold, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    void *scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&scratch, sizeof(ClipState) + 2048 * sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    ClipState *st = (ClipState *)scratch;
    uint32_t *hist = (uint32_t *)((char *)scratch + sizeof(ClipState));
    clip_init_kernel<<<1, 256, 0, stream>>>(st, hist, n, quantile);
    const uint32_t blocks = (uint32_t)std::min<uint64_t>((n + 255) / 256, 152u * 4u);
    for (int pass = 0; pass < kClipPasses; pass++) {
        clip_hist_kernel<<<blocks, 256, 0, stream>>>(values, n, st, pass, hist);
        clip_select_kernel<<<1, 256, 0, stream>>>(st, hist, pass);
    }
    clip_apply_kernel<<<(n + 255) / 256, 256, 0, stream>>>(values, n, st, threshold);
    e = cudaGetLastError();
    const cudaError_t f = cudaFreeAsync(scratch, stream);
    return e != cudaSuccess ? e : f;
}

}  // namespace wobgb
