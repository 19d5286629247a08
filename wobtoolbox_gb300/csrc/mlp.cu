// Fourier-feature MLP for the learned control variate: forward, backward and Adam in CUDA.
//
// Model: v = (x, n) in R^6 -> phi = [sin(2 pi B v), cos(2 pi B v)] (B: n_freq x 6, fixed, seeded)
// -> hidden_layers x (64 -> 64, SiLU) -> 64 -> out_dim. Parameters are kept in FP32 (the Adam
// master copy); every GEMM rounds its operands to BF16 and accumulates in FP32 on the tensor cores
// (mma.sync m16n8k16), so the network computes with BF16 weights and activations.
//
// Parameter layout (FP32): for each layer l: W_l [out][in] row-major, then b_l [out].
#include "../../include/wob_capi.h"

#include "device_common.cuh"
#include "launch.hpp"
#include "mlp_train.hpp"

#include <cuda_bf16.h>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace wobgb {

constexpr int kWidth = 64;
constexpr int kFeatIn = 6;

// ------------------------------------------------------------------------------------------
// GEMM on BF16 tensor cores: C(m, n) = sum_k A(m, k) B(k, n) with arbitrary strides on FP32
// operands (rounded to BF16 when staged in shared memory), FP32 accumulation. A block computes a
// 64 x 64 tile with 4 warps (16 rows each, 8 n8 tiles); grid.z splits K (atomic epilogue).
// ------------------------------------------------------------------------------------------
struct GemmArgs {
    const float *A;
    long sAm, sAk;
    const float *B;
    long sBk, sBn;
    float *C;
    long sCm, sCn;
    int M, N, K;
    const float *bias;  // [N] or null
    float *H;           // epilogue SiLU output (stride as C) or null
    int atomic;         // 1: atomicAdd into C (split-K)
    int k_chunk;        // K range per grid.z slice
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat16 l = __float2bfloat16_rn(lo), h = __float2bfloat16_rn(hi);
    return (uint32_t)__bfloat16_as_ushort(l) | ((uint32_t)__bfloat16_as_ushort(h) << 16);
}

__device__ __forceinline__ void mma_bf16_16816(float c[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = 1.0f / (1.0f + expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

__global__ void __launch_bounds__(128) gemm_bf16_kernel(GemmArgs g) {
    // tiles: As[m][k] (64 x 16), Bs[n][k] (64 x 16), as packed bf16 pairs along k
    __shared__ uint32_t As[64][8 + 1];
    __shared__ uint32_t Bs[64][8 + 1];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, gid = lane >> 2, tig = lane & 3;
    const int m0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
    const int k_begin = blockIdx.z * g.k_chunk;
    const int k_end = min(g.K, k_begin + g.k_chunk);
    float acc[8][4];
#pragma unroll
    for (int j = 0; j < 8; j++)
#pragma unroll
        for (int r = 0; r < 4; r++) acc[j][r] = 0.0f;
    for (int k0 = k_begin; k0 < k_end; k0 += 16) {
        // stage: 64 rows x 8 pairs for A and for B; 128 threads, 4 pairs each
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const int idx = tid * 4 + t;  // 0..511
            const int row = idx >> 3, pr = idx & 7;
            const int k = k0 + 2 * pr;
            float a0 = 0.0f, a1 = 0.0f, b0 = 0.0f, b1 = 0.0f;
            const int m = m0 + row, n = n0 + row;
            if (m < g.M) {
                if (k < k_end) a0 = g.A[m * g.sAm + (long)k * g.sAk];
                if (k + 1 < k_end) a1 = g.A[m * g.sAm + (long)(k + 1) * g.sAk];
            }
            if (n < g.N) {
                if (k < k_end) b0 = g.B[(long)k * g.sBk + n * g.sBn];
                if (k + 1 < k_end) b1 = g.B[(long)(k + 1) * g.sBk + n * g.sBn];
            }
            As[row][pr] = pack_bf16(a0, a1);
            Bs[row][pr] = pack_bf16(b0, b1);
        }
        __syncthreads();
        uint32_t a[4];
        const int r0 = warp * 16 + gid;
        a[0] = As[r0][tig];
        a[1] = As[r0 + 8][tig];
        a[2] = As[r0][tig + 4];
        a[3] = As[r0 + 8][tig + 4];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            uint32_t b[2];
            b[0] = Bs[j * 8 + gid][tig];
            b[1] = Bs[j * 8 + gid][tig + 4];
            mma_bf16_16816(acc[j], a, b);
        }
        __syncthreads();
    }
    // epilogue
#pragma unroll
    for (int j = 0; j < 8; j++) {
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int m = m0 + warp * 16 + gid + (r >= 2 ? 8 : 0);
            const int n = n0 + j * 8 + tig * 2 + (r & 1);
            if (m >= g.M || n >= g.N) continue;
            float v = acc[j][r];
            float *cp = g.C + m * g.sCm + n * g.sCn;
            if (g.atomic) {
                atomicAdd(cp, v);
            } else {
                if (g.bias) v += g.bias[n];
                *cp = v;
                if (g.H) g.H[m * g.sCm + n * g.sCn] = silu(v);
            }
        }
    }
}

static cudaError_t gemm(const GemmArgs &a0, cudaStream_t st) {
    GemmArgs a = a0;
    const int splits = a.atomic ? max(1, min(64, a.K / 256)) : 1;
    a.k_chunk = ((a.K + splits - 1) / splits + 15) / 16 * 16;
    dim3 grid((a.M + 63) / 64, (a.N + 63) / 64, (a.K + a.k_chunk - 1) / a.k_chunk);
    gemm_bf16_kernel<<<grid, 128, 0, st>>>(a);
    return cudaGetLastError();
}

// phi = [sin(2 pi B v), cos(2 pi B v)], v = inputs[i][0..5]
__global__ void fourier_kernel(const float *__restrict__ in, const float *__restrict__ Bf, int n_freq, int n,
                               float *__restrict__ phi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v[kFeatIn];
#pragma unroll
    for (int k = 0; k < kFeatIn; k++) v[k] = in[(long)i * kFeatIn + k];
    for (int f = 0; f < n_freq; f++) {
        float t = 0.0f;
#pragma unroll
        for (int k = 0; k < kFeatIn; k++) t = t + Bf[f * kFeatIn + k] * v[k];
        float s, c;
        sincospi_own(2.0f * t, &s, &c);
        phi[(long)i * (2 * n_freq) + f] = s;
        phi[(long)i * (2 * n_freq) + n_freq + f] = c;
    }
}

// dZ = dH * silu'(Z)
__global__ void silu_backward_kernel(const float *__restrict__ dH, const float *__restrict__ Z, long n,
                                     float *__restrict__ dZ) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dZ[i] = dH[i] * silu_grad(Z[i]);
}

// db[c] += sum_rows dZ[row][c]  (cols <= 64)
__global__ void bias_grad_kernel(const float *__restrict__ dZ, int rows, int cols, float *__restrict__ db) {
    __shared__ float part[64];
    if (threadIdx.x < 64) part[threadIdx.x] = 0.0f;
    __syncthreads();
    const int c = threadIdx.x % cols;
    const int r_step = blockDim.x / cols;
    float s = 0.0f;
    for (int r = blockIdx.x * r_step + threadIdx.x / cols; r < rows && threadIdx.x < r_step * cols; r += gridDim.x * r_step)
        s += dZ[(long)r * cols + c];
    if (threadIdx.x < r_step * cols) atomicAdd(&part[c], s);
    __syncthreads();
    if (threadIdx.x < cols) atomicAdd(&db[threadIdx.x], part[threadIdx.x]);
}

// loss = mean over all entries of (y - t)^2; dY = 2 (y - t) / count
__global__ void mse_kernel(const float *__restrict__ y, const float *__restrict__ t, long count, float *__restrict__ dY,
                           float *__restrict__ loss) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (i < count) {
        const float d = y[i] - t[i];
        dY[i] = 2.0f * d / (float)count;
        l = d * d / (float)count;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, l);
}

__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, long n, float lr, float b1, float b2, float eps, float bc1,
                            float bc2) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// ---- device-driven training loop of networks the fused step does not cover (wob_mlp_train):
// every per-step scalar lives in device memory, so one step is a fixed sequence of launches that
// a CUDA graph replays. sched = {lr, 1 - b1^t, 1 - b2^t, step (as bits)}: the cosine schedule
// and Adam's bias corrections of step s (t = adam_base + s + 1).
__global__ void train_schedule_kernel(uint32_t *step, uint32_t steps, float lr0, uint32_t adam_base, float *sched) {
    const uint32_t s = *step;
    sched[0] = lr0 * 0.5f * (1.0f + cospif((float)s / (float)steps));
    const float t = (float)(adam_base + s + 1u);
    sched[1] = 1.0f - powf(0.9f, t);
    sched[2] = 1.0f - powf(0.999f, t);
    sched[3] = __uint_as_float(s);
    *step = s + 1u;
}

// Batch of the step: indices drawn uniformly from [0, n) by Philox4x32-10 on (row, step, 0,
// "tran") with the seed as key; inputs and targets gathered into xb, tb.
__global__ void train_gather_kernel(const float *__restrict__ in, const float *__restrict__ tg, uint32_t n,
                                    uint32_t out_dim, uint32_t batch, uint64_t seed, const float *__restrict__ sched,
                                    float *__restrict__ xb, float *__restrict__ tb) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= batch) return;
    const uint32_t s = __float_as_uint(sched[3]);
    const uint4 r = philox4x32_10(make_uint4(i, s, 0u, 0x7472616eu), (uint32_t)seed, (uint32_t)(seed >> 32));
    const uint32_t idx = (uint32_t)(((uint64_t)r.x * n) >> 32);
#pragma unroll
    for (int k = 0; k < kFeatIn; k++) xb[(size_t)i * kFeatIn + k] = in[(size_t)idx * kFeatIn + k];
    for (uint32_t k = 0; k < out_dim; k++) tb[(size_t)i * out_dim + k] = tg[(size_t)idx * out_dim + k];
}

__global__ void adam_sched_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                                  float *__restrict__ v, long n, const float *__restrict__ sched, float b1, float b2,
                                  float eps) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float lr = sched[0], bc1 = sched[1], bc2 = sched[2];
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

__global__ void train_record_loss_kernel(const float *__restrict__ loss, const float *__restrict__ sched,
                                         float *__restrict__ hist) {
    hist[__float_as_uint(sched[3])] = *loss;
}

}  // namespace wobgb

// ------------------------------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------------------------------
namespace {
int mfail(int code, const std::string &m) {
    wobgb::set_last_error(m.c_str());
    return code;
}
int mfail_cuda(cudaError_t e, const char *what) {
    wobgb::set_last_error((std::string(what) + ": " + cudaGetErrorString(e)).c_str());
    return e == cudaErrorMemoryAllocation ? WOB_ERR_OUT_OF_MEMORY : WOB_ERR_CUDA;
}
}  // namespace

struct wob_mlp_s {
    int device = 0;
    uint32_t n_freq = 32, hidden = 4, out_dim = 1;
    uint32_t n_params = 0;
    std::vector<uint32_t> w_off, b_off, fan_in, fan_out;  // per layer
    float *params = nullptr, *grad = nullptr, *adam_m = nullptr, *adam_v = nullptr, *freqs = nullptr;
    // activations workspace for `cap` points
    uint32_t cap = 0;
    float *phi = nullptr, *Z = nullptr, *H = nullptr, *Y = nullptr, *dY = nullptr, *dA = nullptr, *dZ = nullptr,
          *loss = nullptr;
    uint64_t adam_steps = 0;
    // training-loop state (wob_mlp_train)
    uint32_t train_cap = 0, partial_blocks = 0;
    float *xb = nullptr, *tb = nullptr, *sched = nullptr, *partial = nullptr, *partial_loss = nullptr;
    uint32_t *step = nullptr;   // [2]: step counter, the fused update's count of finished blocks
    uint32_t *image = nullptr;  // packed BF16 weights of the fused step (zero padding)
    uint32_t *err = nullptr;    // fused step's error word
    uint32_t inject_wait_polls = 0;  // wob_mlp_inject_wait_timeout
    std::mutex mu;

    uint32_t n_layers() const { return hidden + 1; }
    void free_ws() {
        for (float **p : {&phi, &Z, &H, &Y, &dY, &dA, &dZ, &loss, &xb, &tb, &sched, &partial, &partial_loss}) {
            if (*p) cudaFree(*p);
            *p = nullptr;
        }
        for (uint32_t **p : {&step, &image, &err}) {
            if (*p) cudaFree(*p);
            *p = nullptr;
        }
        cap = 0;
        train_cap = 0;
        partial_blocks = 0;
    }
    // workspace of the unfused graph-replayed step
    cudaError_t ensure_train(uint32_t batch) {
        cudaError_t e = ensure(batch);
        if (e != cudaSuccess) return e;
        if (!sched && (e = cudaMalloc(&sched, 16)) != cudaSuccess) return e;
        if (!step && (e = cudaMalloc(&step, 8)) != cudaSuccess) return e;
        if (batch <= train_cap) return cudaSuccess;
        for (float **p : {&xb, &tb}) {
            if (*p) cudaFree(*p);
            *p = nullptr;
        }
        if ((e = cudaMalloc(&xb, (size_t)batch * wobgb::kFeatIn * 4)) != cudaSuccess ||
            (e = cudaMalloc(&tb, (size_t)batch * out_dim * 4)) != cudaSuccess)
            return e;
        train_cap = batch;
        return cudaSuccess;
    }
    // the fused step (mlp_train.cu) covers the 4-hidden-layer, 32-frequency network
    bool fused_ok() const { return hidden == 4 && n_freq == 32 && out_dim <= 64; }
    cudaError_t ensure_fused(uint32_t batch) {
        cudaError_t e;
        if (!step && (e = cudaMalloc(&step, 8)) != cudaSuccess) return e;
        if (!image) {
            const size_t bytes = wobgb::fused_train_image_words() * 4;
            if ((e = cudaMalloc(&image, bytes)) != cudaSuccess || (e = cudaMemset(image, 0, bytes)) != cudaSuccess)
                return e;
        }
        if (!err) {
            if ((e = cudaMalloc(&err, 4)) != cudaSuccess || (e = cudaMemset(err, 0, 4)) != cudaSuccess) return e;
        }
        const uint32_t blocks = wobgb::fused_train_blocks(batch);
        if (blocks <= partial_blocks) return cudaSuccess;
        for (float **p : {&partial, &partial_loss}) {
            if (*p) cudaFree(*p);
            *p = nullptr;
        }
        if ((e = cudaMalloc(&partial, (size_t)blocks * n_params * 4)) != cudaSuccess ||
            (e = cudaMalloc(&partial_loss, (size_t)blocks * 4)) != cudaSuccess)
            return e;
        partial_blocks = blocks;
        return wobgb::prepare_fused_train();
    }
    cudaError_t ensure(uint32_t n) {
        if (n <= cap) return cudaSuccess;
        free_ws();
        const size_t w = (size_t)n * wobgb::kWidth * 4;
        cudaError_t e;
        if ((e = cudaMalloc(&phi, w)) || (e = cudaMalloc(&Z, w * hidden)) || (e = cudaMalloc(&H, w * hidden)) ||
            (e = cudaMalloc(&Y, (size_t)n * out_dim * 4)) || (e = cudaMalloc(&dY, (size_t)n * out_dim * 4)) ||
            (e = cudaMalloc(&dA, w)) || (e = cudaMalloc(&dZ, w)) || (e = cudaMalloc(&loss, 4)))
            return e;
        cap = n;
        return cudaSuccess;
    }
};

namespace {

cudaError_t forward_impl(wob_mlp_s *m, const float *in, uint32_t n, cudaStream_t st) {
    using namespace wobgb;
    fourier_kernel<<<(n + 127) / 128, 128, 0, st>>>(in, m->freqs, (int)m->n_freq, (int)n, m->phi);
    const float *act = m->phi;
    for (uint32_t l = 0; l < m->n_layers(); l++) {
        const bool last = l == m->hidden;
        GemmArgs g{};
        g.A = act; g.sAm = kWidth; g.sAk = 1;
        g.B = m->params + m->w_off[l]; g.sBk = 1; g.sBn = m->fan_in[l];  // B(k, n) = W[n][k]
        g.M = (int)n; g.N = (int)m->fan_out[l]; g.K = (int)m->fan_in[l];
        g.bias = m->params + m->b_off[l];
        if (last) {
            g.C = m->Y; g.sCm = m->out_dim; g.sCn = 1; g.H = nullptr;
        } else {
            g.C = m->Z + (size_t)l * n * kWidth; g.sCm = kWidth; g.sCn = 1;
            g.H = m->H + (size_t)l * n * kWidth;
        }
        cudaError_t e = gemm(g, st);
        if (e != cudaSuccess) return e;
        if (!last) act = m->H + (size_t)l * n * kWidth;
    }
    return cudaGetLastError();
}

// gradient of mean((y - t)^2) into m->grad (zeroed here)
cudaError_t backward_impl(wob_mlp_s *m, const float *in, const float *targets, uint32_t n, cudaStream_t st) {
    using namespace wobgb;
    cudaError_t e = forward_impl(m, in, n, st);
    if (e != cudaSuccess) return e;
    cudaMemsetAsync(m->grad, 0, (size_t)m->n_params * 4, st);
    cudaMemsetAsync(m->loss, 0, 4, st);
    const long cnt = (long)n * m->out_dim;
    mse_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, st>>>(m->Y, targets, cnt, m->dY, m->loss);
    const float *dOut = m->dY;  // gradient wrt the output of layer l (pre-activation for the last)
    int out_stride = (int)m->out_dim;
    for (int l = (int)m->n_layers() - 1; l >= 0; l--) {
        const float *dZl;
        if (l == (int)m->hidden) {
            dZl = dOut;  // linear output layer
        } else {
            silu_backward_kernel<<<(unsigned)(((long)n * kWidth + 255) / 256), 256, 0, st>>>(
                dOut, m->Z + (size_t)l * n * kWidth, (long)n * kWidth, m->dZ);
            dZl = m->dZ;
        }
        const float *act_in = l == 0 ? m->phi : m->H + (size_t)(l - 1) * n * kWidth;
        // dW_l(o, i) = sum_r dZl(r, o) act_in(r, i)
        GemmArgs gw{};
        gw.A = dZl; gw.sAm = 1; gw.sAk = out_stride;
        gw.B = act_in; gw.sBk = kWidth; gw.sBn = 1;
        gw.C = m->grad + m->w_off[l]; gw.sCm = m->fan_in[l]; gw.sCn = 1;
        gw.M = (int)m->fan_out[l]; gw.N = (int)m->fan_in[l]; gw.K = (int)n; gw.atomic = 1;
        if ((e = gemm(gw, st)) != cudaSuccess) return e;
        bias_grad_kernel<<<64, 256, 0, st>>>(dZl, (int)n, (int)m->fan_out[l], m->grad + m->b_off[l]);
        if (l == 0) break;
        // dA_{l-1}(r, i) = sum_o dZl(r, o) W_l(o, i)
        GemmArgs ga{};
        ga.A = dZl; ga.sAm = out_stride; ga.sAk = 1;
        ga.B = m->params + m->w_off[l]; ga.sBk = m->fan_in[l]; ga.sBn = 1;
        ga.C = m->dA; ga.sCm = kWidth; ga.sCn = 1;
        ga.M = (int)n; ga.N = (int)m->fan_in[l]; ga.K = (int)m->fan_out[l];
        if ((e = gemm(ga, st)) != cudaSuccess) return e;
        dOut = m->dA;
        out_stride = kWidth;
        // dZ buffer is reused next iteration: silu_backward reads dA and writes dZ; dA is consumed first
    }
    return cudaGetLastError();
}

}  // namespace

extern "C" {

int wob_mlp_create(uint32_t n_freq, uint32_t hidden_layers, uint32_t out_dim, float freq_sigma, uint64_t seed,
                   wob_mlp *out) {
    if (!out) return mfail(WOB_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (2 * n_freq != (uint32_t)wobgb::kWidth) return mfail(WOB_ERR_UNSUPPORTED, "2 * n_freq must equal the width 64");
    if (hidden_layers < 1 || hidden_layers > 16) return mfail(WOB_ERR_INVALID_ARGUMENT, "hidden_layers must be 1..16");
    if (out_dim < 1 || out_dim > 64) return mfail(WOB_ERR_INVALID_ARGUMENT, "out_dim must be 1..64");
    if (!(freq_sigma > 0.0f)) return mfail(WOB_ERR_INVALID_ARGUMENT, "freq_sigma must be positive");
    wob_mlp_s *m = new wob_mlp_s();
    m->n_freq = n_freq; m->hidden = hidden_layers; m->out_dim = out_dim;
    uint32_t off = 0;
    for (uint32_t l = 0; l <= hidden_layers; l++) {
        const uint32_t fi = wobgb::kWidth, fo = l == hidden_layers ? out_dim : (uint32_t)wobgb::kWidth;
        m->fan_in.push_back(fi); m->fan_out.push_back(fo);
        m->w_off.push_back(off); off += fi * fo;
        m->b_off.push_back(off); off += fo;
    }
    m->n_params = off;
    // deterministic init: splitmix64 -> uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)); Gaussian frequencies
    std::vector<float> p(off, 0.0f), fr(n_freq * wobgb::kFeatIn);
    uint64_t st = seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    auto next = [&]() {
        st += 0x9E3779B97F4A7C15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return (double)((z ^ (z >> 31)) >> 11) * 0x1p-53;
    };
    for (uint32_t l = 0; l <= hidden_layers; l++) {
        const double a = 1.0 / std::sqrt((double)m->fan_in[l]);
        for (uint32_t i = 0; i < m->fan_in[l] * m->fan_out[l]; i++) p[m->w_off[l] + i] = (float)((2.0 * next() - 1.0) * a);
    }
    for (auto &f : fr) {  // Box-Muller
        const double u1 = next() + 1e-300, u2 = next();
        f = (float)(freq_sigma * std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2));
    }
    cudaGetDevice(&m->device);
    cudaError_t e;
    if ((e = cudaMalloc(&m->params, off * 4)) || (e = cudaMalloc(&m->grad, off * 4)) ||
        (e = cudaMalloc(&m->adam_m, off * 4)) || (e = cudaMalloc(&m->adam_v, off * 4)) ||
        (e = cudaMalloc(&m->freqs, fr.size() * 4)) ||
        (e = cudaMemcpy(m->params, p.data(), off * 4, cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(m->freqs, fr.data(), fr.size() * 4, cudaMemcpyHostToDevice)) ||
        (e = cudaMemset(m->adam_m, 0, off * 4)) || (e = cudaMemset(m->adam_v, 0, off * 4))) {
        for (float *q : {m->params, m->grad, m->adam_m, m->adam_v, m->freqs}) if (q) cudaFree(q);
        delete m;
        return mfail_cuda(e, "allocating the MLP");
    }
    *out = m;
    return WOB_OK;
}

int wob_mlp_destroy(wob_mlp m) {
    if (!m) return WOB_OK;
    m->free_ws();
    for (float *q : {m->params, m->grad, m->adam_m, m->adam_v, m->freqs}) if (q) cudaFree(q);
    delete m;
    return WOB_OK;
}

int wob_mlp_num_params(wob_mlp m, uint32_t *n) {
    if (!m || !n) return mfail(WOB_ERR_INVALID_ARGUMENT, "mlp and n are required");
    *n = m->n_params;
    return WOB_OK;
}

int wob_mlp_get_params(wob_mlp m, float *params, float *freqs) {
    if (!m) return mfail(WOB_ERR_INVALID_ARGUMENT, "mlp is NULL");
    cudaError_t e = cudaSuccess;
    if (params) e = cudaMemcpy(params, m->params, m->n_params * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && freqs) e = cudaMemcpy(freqs, m->freqs, m->n_freq * wobgb::kFeatIn * 4, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? WOB_OK : mfail_cuda(e, "reading MLP parameters");
}

int wob_mlp_set_params(wob_mlp m, const float *params) {
    if (!m || !params) return mfail(WOB_ERR_INVALID_ARGUMENT, "mlp and params are required");
    cudaError_t e = cudaMemcpy(m->params, params, m->n_params * 4, cudaMemcpyHostToDevice);
    return e == cudaSuccess ? WOB_OK : mfail_cuda(e, "writing MLP parameters");
}

int wob_mlp_forward(wob_mlp m, const float *inputs, uint32_t n, float *outputs, void *stream) {
    if (!m || (!inputs && n) || (!outputs && n)) return mfail(WOB_ERR_INVALID_ARGUMENT, "mlp, inputs and outputs are required");
    if (n == 0) return WOB_OK;
    std::lock_guard<std::mutex> lock(m->mu);
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = m->ensure(n);
    if (e != cudaSuccess) return mfail_cuda(e, "MLP workspace");
    if ((e = forward_impl(m, inputs, n, st)) != cudaSuccess) return mfail_cuda(e, "MLP forward");
    e = cudaMemcpyAsync(outputs, m->Y, (size_t)n * m->out_dim * 4, cudaMemcpyDeviceToDevice, st);
    return e == cudaSuccess ? WOB_OK : mfail_cuda(e, "MLP forward copy");
}

int wob_mlp_gradient(wob_mlp m, const float *inputs, const float *targets, uint32_t n, float *grad, float *loss,
                     void *stream) {
    if (!m || !inputs || !targets || n == 0) return mfail(WOB_ERR_INVALID_ARGUMENT, "mlp, inputs, targets and n > 0 are required");
    std::lock_guard<std::mutex> lock(m->mu);
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = m->ensure(n);
    if (e != cudaSuccess) return mfail_cuda(e, "MLP workspace");
    if ((e = backward_impl(m, inputs, targets, n, st)) != cudaSuccess) return mfail_cuda(e, "MLP backward");
    if (grad && (e = cudaMemcpyAsync(grad, m->grad, m->n_params * 4, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
        return mfail_cuda(e, "MLP gradient copy");
    if (loss && (e = cudaMemcpyAsync(loss, m->loss, 4, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
        return mfail_cuda(e, "MLP loss copy");
    return WOB_OK;
}

int wob_mlp_adam_step(wob_mlp m, const float *inputs, const float *targets, uint32_t n, float lr, float *loss,
                      void *stream) {
    int st_ = wob_mlp_gradient(m, inputs, targets, n, nullptr, loss, stream);
    if (st_ != WOB_OK) return st_;
    std::lock_guard<std::mutex> lock(m->mu);
    m->adam_steps++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.0f - std::pow(b1, (float)m->adam_steps), bc2 = 1.0f - std::pow(b2, (float)m->adam_steps);
    wobgb::adam_kernel<<<(m->n_params + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
        m->params, m->grad, m->adam_m, m->adam_v, m->n_params, lr, b1, b2, 1e-8f, bc1, bc2);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? WOB_OK : mfail_cuda(e, "Adam step");
}

int wob_mlp_inject_wait_timeout(wob_mlp m, uint32_t polls) {
    if (!m) return mfail(WOB_ERR_INVALID_ARGUMENT, "mlp is NULL");
    std::lock_guard<std::mutex> lock(m->mu);
    m->inject_wait_polls = polls;
    return WOB_OK;
}

int wob_mlp_gradient_fused(wob_mlp m, const float *inputs, const float *targets, uint32_t n, float *grad, float *loss,
                           void *stream) {
    if (!m || !inputs || !targets || !grad || n == 0)
        return mfail(WOB_ERR_INVALID_ARGUMENT, "mlp, inputs, targets, grad and n > 0 are required");
    if (!m->fused_ok()) return mfail(WOB_ERR_UNSUPPORTED, "the fused step needs 4 hidden layers, 32 frequencies and out_dim <= 64");
    std::lock_guard<std::mutex> lock(m->mu);
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = m->ensure_fused(n);
    if (e != cudaSuccess) return mfail_cuda(e, "MLP training workspace");
    if ((e = cudaMemsetAsync(m->step, 0, 8, st)) != cudaSuccess) return mfail_cuda(e, "MLP step counter");
    wobgb::FusedTrainArgs a{m->params, m->freqs, inputs, targets, n, m->out_dim, n, m->n_params, 0u, 0ull, m->step,
                            m->partial, m->partial_loss, m->image, m->err, m->inject_wait_polls};
    e = wobgb::launch_fused_gradient(a, grad, loss, st);
    return e == cudaSuccess ? WOB_OK : mfail_cuda(e, "fused MLP gradient");
}

int wob_mlp_train(wob_mlp m, const float *inputs, const float *targets, uint32_t n, uint32_t steps, uint32_t batch,
                  float lr, uint64_t seed, float *loss_history, void *stream) {
    if (!m || !inputs || !targets || n == 0 || batch == 0)
        return mfail(WOB_ERR_INVALID_ARGUMENT, "mlp, inputs, targets, n > 0 and batch > 0 are required");
    if (!(lr > 0.0f) || !(lr < 1e3f)) return mfail(WOB_ERR_INVALID_ARGUMENT, "lr must be positive");
    if (steps == 0) return WOB_OK;
    std::lock_guard<std::mutex> lock(m->mu);
    using namespace wobgb;
    cudaStream_t user = (cudaStream_t)stream;
    const bool fused = m->fused_ok();
    cudaError_t e = fused ? m->ensure_fused(batch) : m->ensure_train(batch);
    if (e != cudaSuccess) return mfail_cuda(e, "MLP training workspace");
    // kSteps steps are captured once into a CUDA graph on a private stream, ordered after the
    // caller's stream by an event, and the graph replayed; the remaining steps (steps mod kSteps)
    // are launched directly. The fused step's kernels use programmatic dependent launches, which
    // the capture keeps as graph edges.
    const uint32_t kSteps = steps < 16u ? steps : 16u;
    cudaStream_t cs = nullptr;
    cudaEvent_t ev = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    auto cleanup = [&]() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (ev) cudaEventDestroy(ev);
        if (cs) cudaStreamDestroy(cs);
    };
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaMemsetAsync(m->step, 0, 8, user)) != cudaSuccess || (e = cudaEventRecord(ev, user)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(cs, ev, 0)) != cudaSuccess) {
        cleanup();
        return mfail_cuda(e, "preparing the training stream");
    }
    const uint32_t adam_base = (uint32_t)m->adam_steps;
    // the fused step reads the weights from their packed image, which each update keeps current
    if (fused && (e = launch_pack_weights(m->params, m->n_params, m->out_dim, m->image, cs)) != cudaSuccess) {
        cleanup();
        return mfail_cuda(e, "packing the weights");
    }
    if ((e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
        cleanup();
        return mfail_cuda(e, "capturing the training step");
    }
    auto one_step = [&]() -> cudaError_t {
        if (fused) {
            FusedTrainArgs a{m->params, m->freqs, inputs, targets, n, m->out_dim, batch, m->n_params, 1u, seed, m->step,
                             m->partial, m->partial_loss, m->image, m->err, m->inject_wait_polls};
            return launch_fused_train_step(a, m->params, m->adam_m, m->adam_v, steps, lr, adam_base, loss_history, cs);
        }
        train_schedule_kernel<<<1, 1, 0, cs>>>(m->step, steps, lr, adam_base, m->sched);
        train_gather_kernel<<<(batch + 127) / 128, 128, 0, cs>>>(inputs, targets, n, m->out_dim, batch, seed, m->sched,
                                                                 m->xb, m->tb);
        cudaError_t eb = backward_impl(m, m->xb, m->tb, batch, cs);
        adam_sched_kernel<<<(m->n_params + 255) / 256, 256, 0, cs>>>(m->params, m->grad, m->adam_m, m->adam_v,
                                                                     m->n_params, m->sched, 0.9f, 0.999f, 1e-8f);
        if (loss_history) train_record_loss_kernel<<<1, 1, 0, cs>>>(m->loss, m->sched, loss_history);
        return eb != cudaSuccess ? eb : cudaGetLastError();
    };
    cudaError_t e_body = cudaSuccess;
    for (uint32_t i = 0; i < kSteps && e_body == cudaSuccess; i++) e_body = one_step();
    e = cudaStreamEndCapture(cs, &graph);
    if (e_body != cudaSuccess || e != cudaSuccess || (e = cudaGraphInstantiate(&exec, graph, 0)) != cudaSuccess) {
        cleanup();
        return mfail_cuda(e_body != cudaSuccess ? e_body : e, "building the training graph");
    }
    for (uint32_t i = 0; i < steps / kSteps; i++)
        if ((e = cudaGraphLaunch(exec, cs)) != cudaSuccess) {
            cleanup();
            return mfail_cuda(e, "launching the training steps");
        }
    for (uint32_t i = 0; i < steps % kSteps; i++)
        if ((e = one_step()) != cudaSuccess) {
            cleanup();
            return mfail_cuda(e, "launching a training step");
        }
    if ((e = cudaEventRecord(ev, cs)) != cudaSuccess || (e = cudaStreamWaitEvent(user, ev, 0)) != cudaSuccess ||
        (e = cudaStreamSynchronize(cs)) != cudaSuccess) {
        cleanup();
        return mfail_cuda(e, "finishing the training steps");
    }
    // the bias corrections continue from the updates that ran: the step counter (a failed fused
    // step skips its update and stops the count)
    uint32_t ran = steps;
    if ((e = cudaMemcpy(&ran, m->step, 4, cudaMemcpyDeviceToHost)) != cudaSuccess) {
        cleanup();
        return mfail_cuda(e, "reading the step counter");
    }
    m->adam_steps += ran;
    cleanup();
    if (fused) {
        uint32_t bits = 0;
        if ((e = cudaMemcpy(&bits, m->err, 4, cudaMemcpyDeviceToHost)) != cudaSuccess)
            return mfail_cuda(e, "reading the training error word");
        if (bits) {
            cudaMemset(m->err, 0, 4);
            return mfail(WOB_ERR_DEVICE_LIMIT, (bits & 2u) ? "a training block's tensor-core product did not complete within its wait bound"
                                                          : "a training block's weight staging did not complete within its wait bound");
        }
    }
    return WOB_OK;
}

}  // extern "C"
