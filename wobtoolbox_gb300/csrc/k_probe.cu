// Measured ceiling of the uniform-sampling walk's memory access pattern: random gathers of
// 64-byte records through a guide table, both L2-resident, at full occupancy and with several
// independent gathers in flight per thread.
//
// One "sample" here is what one uniform boundary sample of the walk reads (sample_uniform_pair in
// device_common.cuh): one 16-byte guide-table entry at a random index, then the 64-byte element
// record it points to, as two 32-byte ld.global.nc.v8 loads. The walk issues these as dependent
// chains between its arithmetic; the probe issues kChains chains per thread back to back with no
// other work, so samples per second here bound what the walk's gathers can reach. The table sizes
// are the caller's (the benchmark scene: 81,920 records, 81,920 guide entries).
#include "device_common.cuh"
#include "launch.hpp"

namespace wobgb {

namespace {

constexpr int kChains = 4;

__global__ void probe_fill_kernel(float4 *rec, uint32_t n_rec, uint4 *guide, uint32_t n_guide) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_rec * 4u) rec[i] = make_float4((float)i, 1.0f, 2.0f, 3.0f);
    if (i < n_guide) {
        const uint32_t lo = (uint32_t)(((uint64_t)i * n_rec) / n_guide);
        guide[i] = make_uint4(lo, lo, 0u, 0u);
    }
}

__global__ void __launch_bounds__(256) probe_gather_kernel(const float4 *__restrict__ rec, uint32_t n_rec,
                                                           const uint4 *__restrict__ guide, uint32_t n_guide,
                                                           uint32_t iters, float *__restrict__ sink) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t h[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) h[c] = tid * 0x9E3779B9u + (uint32_t)c * 0x85EBCA6Bu + 1u;
    float acc = 0.0f;
    for (uint32_t it = 0; it < iters; it++) {
        uint4 g[kChains];
#pragma unroll
        for (int c = 0; c < kChains; c++) {
            h[c] ^= h[c] << 13;
            h[c] ^= h[c] >> 17;
            h[c] ^= h[c] << 5;
            g[c] = __ldg(guide + (uint32_t)(((uint64_t)h[c] * n_guide) >> 32));
        }
        F8 a[kChains], b[kChains];
#pragma unroll
        for (int c = 0; c < kChains; c++) {
            const uint32_t r = (g[c].x + (h[c] & 1u)) % n_rec;
            a[c] = ldg8(rec + 4 * r);
            b[c] = ldg8(rec + 4 * r + 2);
        }
#pragma unroll
        for (int c = 0; c < kChains; c++) acc += a[c].a.x + a[c].b.y + b[c].a.z + b[c].b.w;
    }
    if (acc == -1.0f) sink[tid] = acc;  // keeps the loads; never true for this table
}

}  // namespace

cudaError_t measure_gather_peak(uint32_t n_rec, uint32_t n_guide, uint32_t iters, int sm_count, double *samples_per_s,
                                float *ms) {
    float4 *rec = nullptr;
    uint4 *guide = nullptr;
    float *sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const uint32_t blocks = (uint32_t)sm_count * 8u;  // 8 x 256 threads per SM: full occupancy
    cudaError_t e;
    auto done = [&](cudaError_t r) {
        if (rec) cudaFree(rec);
        if (guide) cudaFree(guide);
        if (sink) cudaFree(sink);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        return r;
    };
    if ((e = cudaMalloc(&rec, (size_t)n_rec * 64)) != cudaSuccess ||
        (e = cudaMalloc(&guide, (size_t)n_guide * 16)) != cudaSuccess ||
        (e = cudaMalloc(&sink, (size_t)blocks * 256 * 4)) != cudaSuccess ||
        (e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess)
        return done(e);
    const uint32_t fill = n_rec * 4u > n_guide ? n_rec * 4u : n_guide;
    probe_fill_kernel<<<(fill + 255) / 256, 256>>>(rec, n_rec, guide, n_guide);
    probe_gather_kernel<<<blocks, 256>>>(rec, n_rec, guide, n_guide, iters / 8 + 1, sink);  // warm-up
    cudaEventRecord(e0);
    probe_gather_kernel<<<blocks, 256>>>(rec, n_rec, guide, n_guide, iters, sink);
    cudaEventRecord(e1);
    if ((e = cudaEventSynchronize(e1)) != cudaSuccess) return done(e);
    float t = 0.0f;
    cudaEventElapsedTime(&t, e0, e1);
    *ms = t;
    *samples_per_s = (double)blocks * 256.0 * iters * kChains / (t * 1e-3);
    return done(cudaGetLastError());
}

}  // namespace wobgb
