// Fused training step of the Fourier-feature MLP (mlp.cu's network with 4 hidden layers): one
// kernel runs the batch gather, the forward pass and the backward pass of 64 rows per block (16
// warps, each a 16 x 16 share of every 64 x 64 product) with every weight and activation in shared
// memory and writes the block's gradient; a second kernel sums the blocks' gradients in a fixed
// order (so a step is deterministic), applies Adam, writes the updated weights as a packed BF16
// image in both operand layouts, and its last block advances the step counter. wob_mlp_train
// replays the two as a CUDA graph. Each block of the next step
// stages that image (83 KB) into shared memory with one TMA bulk copy (cp.async.bulk, completion
// on an mbarrier, the wait bounded), instead of every block reading and converting the FP32
// parameters itself.
//
// Network and parameter layout as in mlp.cu: phi = [sin, cos](2 pi B v) (32 frequencies of the
// 6 inputs), 4 hidden layers 64 -> 64 with SiLU, a linear 64 -> out_dim head; FP32 parameters,
// for each layer W [out][in] row-major then b [out]. Every product runs on the BF16 tensor cores
// (mma.sync m16n8k16, FP32 accumulation) with operands rounded to BF16 in shared memory, as in
// mlp.cu; pre-activations are kept as BF16 for the SiLU derivative, bias gradients are summed in
// FP32 from the FP32 products. No atomics: every sum has a fixed order, so training is
// deterministic.
//
// Shared-memory operands are 32-bit words holding two BF16 values adjacent along the reduction
// index (the m16n8k16 fragment layout), rows padded to 36 words so that the 8 rows of 16 bytes an
// ldmatrix / stmatrix phase moves fall in 32 distinct banks. For C[m][n] = sum_k A[m][k] B[k][n] the A operand is
// stored [m][k/2] and the B operand [n][k/2]:
//   forward  Z = A W^T:     A = activation [row][in],   B = W   [out][in]
//   weights  dW = dZ^T A:   A = dZ^T [out][row],        B = A^T [in][row]
//   inputs   dA = dZ W:     A = dZ   [row][out],        B = W^T [in][out]
#include "../../include/wob_capi.h"

#include "device_common.cuh"
#include "launch.hpp"
#include "mlp_train.hpp"

#include <cuda_bf16.h>

namespace wobgb {

namespace {

constexpr int kTM = 64;          // rows per block
constexpr int kW = 64;           // layer width
constexpr int kLd = 36;          // words per shared-memory row (32 pairs + 4 padding)
constexpr int kMat = kW * kLd;   // words per 64 x 64 operand
constexpr int kHidden = 4;
constexpr int kLayers = kHidden + 1;
constexpr int kIn = 6;
// kColSplit x 4 warps: warp w computes rows [16 (w & 3), +16) x columns [kCols (w >> 2), +kCols)
// of every 64 x 64 product; the warps of a row block meet at a named barrier where one reads what
// another wrote
constexpr int kColSplit = 4;
constexpr int kRowBlocks = kTM / 16;
constexpr int kWarps = kRowBlocks * kColSplit;
constexpr int kThreads = kWarps * 32;
constexpr int kCols = kW / kColSplit;  // columns per warp
constexpr int kNT = kCols / 8;         // 8-column tiles per warp
static_assert(kNT % 2 == 0, "fragments move two tiles at a time");
constexpr int kLayerParams = kW * kW + kW;

// operands: Wf (5), Wb (4), act (2: a layer reads one and writes the other), actT (5), Zs (4), dZ, dZT
constexpr size_t kSmemWords = (size_t)(kLayers + kHidden + 2 + kLayers + kHidden + 2) * kMat;
constexpr size_t kSmemFloats = kLayers * kW + kLayers * kRowBlocks * kW + kTM * kIn + kTM * kW + kWarps;

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    const __nv_bfloat16 l = __float2bfloat16_rn(lo), h = __float2bfloat16_rn(hi);
    return (uint32_t)__bfloat16_as_ushort(l) | ((uint32_t)__bfloat16_as_ushort(h) << 16);
}
__device__ __forceinline__ float lo_of(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float hi_of(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Four 8 x 8 BF16 matrices from shared memory in mma fragment layout (lane l gets row l / 4, word
// l % 4 of each); lane l gives the address of row l % 8 of matrix l / 8 (16-byte aligned rows).
__device__ __forceinline__ void ldsm_x4(uint32_t r[4], const uint32_t *row) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_u32(row))
                 : "memory");
}

// acc[j][.] += sum_k A[m0 + .][k] B[k][n0 + 8 j + .] for one warp's 16 rows at m0 and kCols
// columns at n0; K = 64. Fragment c[0..3] of tile j: rows m0 + gid (c0, c1) and m0 + gid + 8 (c2, c3),
// columns n0 + 8 j + 2 tig and n0 + 8 j + 2 tig + 1. The A fragment of a k step is one ldmatrix.x4
// (rows m0..m0+7 and m0+8..m0+15, k words 0-3 and 4-7), the B fragments of two tiles another.
__device__ __forceinline__ void warp_gemm(float acc[kNT][4], const uint32_t *A, const uint32_t *B, int m0, int n0,
                                          int lane) {
    const int r = lane & 7, mi = lane >> 3;
    const uint32_t *a_row = A + (m0 + 8 * (mi & 1) + r) * kLd + 4 * (mi >> 1);
    const uint32_t *b_row = B + (n0 + 8 * (mi >> 1) + r) * kLd + 4 * (mi & 1);
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
        uint32_t a[4];
        ldsm_x4(a, a_row + kk * 8);
#pragma unroll
        for (int j = 0; j < kNT; j += 2) {
            uint32_t b[4];
            ldsm_x4(b, b_row + j * 8 * kLd + kk * 8);
            mma16816(acc[j], a, b);
            mma16816(acc[j + 1], a, b + 2);
        }
    }
}

// Stores a warp's 16 x kCols tile of packed BF16 pairs p[j][h] (fragment layout: row m0 + gid + 8 h,
// columns n0 + 8 j + 2 tig, +1) into M as [row][col / 2] words, or with kTrans as [col][row / 2]
// words (the transposed operand), two tiles per stmatrix.x4.
template <bool kTrans>
__device__ __forceinline__ void store_tile(uint32_t *M, const uint32_t p[kNT][2], int m0, int n0, int lane) {
    const int r = lane & 7, mi = lane >> 3;
#pragma unroll
    for (int j = 0; j < kNT; j += 2) {
        const int row = m0 + 8 * (mi & 1), col = n0 + 8 * (j + (mi >> 1));
        const uint32_t addr = smem_u32(kTrans ? M + (col + r) * kLd + row / 2 : M + (row + r) * kLd + col / 2);
        if (kTrans)
            asm volatile("stmatrix.sync.aligned.m8n8.x4.trans.shared.b16 [%0], {%1,%2,%3,%4};" ::"r"(addr),
                         "r"(p[j][0]), "r"(p[j][1]), "r"(p[j + 1][0]), "r"(p[j + 1][1])
                         : "memory");
        else
            asm volatile("stmatrix.sync.aligned.m8n8.x4.shared.b16 [%0], {%1,%2,%3,%4};" ::"r"(addr), "r"(p[j][0]),
                         "r"(p[j][1]), "r"(p[j + 1][0]), "r"(p[j + 1][1])
                         : "memory");
    }
}

__device__ __forceinline__ void zero_acc(float acc[kNT][4]) {
#pragma unroll
    for (int j = 0; j < kNT; j++)
#pragma unroll
        for (int r = 0; r < 4; r++) acc[j][r] = 0.0f;
}

// The warps of row block rb wait for each other; barrier 0 is __syncthreads'.
__device__ __forceinline__ void row_block_sync(int rb) {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + rb), "r"(kColSplit * 32) : "memory");
}

__device__ __forceinline__ float silu_f(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu_d(float z) {
    const float s = 1.0f / (1.0f + expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

// BF16 value at (row, col) of an operand kept transposed, [col][row / 2] words.
__device__ __forceinline__ void store_t(uint32_t *M, int row, int col, float v) {
    reinterpret_cast<__nv_bfloat16 *>(M)[col * kLd * 2 + row] = __float2bfloat16_rn(v);
}

// Column sums over the warp's 16 rows of the FP32 values in acc (fragment layout of tile j),
// stored to the row block's row dst[n0 + 8 j + 2 tig (+1)] in shared memory (the row blocks' rows
// are added in row-block order later, so the sum does not depend on scheduling).
__device__ __forceinline__ void store_col_sums(float acc[kNT][4], float *dst, int n0, int lane, int tig) {
#pragma unroll
    for (int j = 0; j < kNT; j++) {
        float s0 = acc[j][0] + acc[j][2], s1 = acc[j][1] + acc[j][3];
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) {
            s0 += __shfl_xor_sync(0xffffffffu, s0, o);
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        }
        if (lane < 4) {
            dst[n0 + j * 8 + 2 * tig] = s0;
            dst[n0 + j * 8 + 2 * tig + 1] = s1;
        }
    }
}

constexpr size_t kImageWords = (size_t)(kLayers + kHidden) * kMat;  // Wf then Wb, as in shared memory
constexpr uint32_t kImageBytes = (uint32_t)(kImageWords * 4);
static_assert(kImageBytes % 16 == 0, "bulk copies move multiples of 16 bytes");
// try_wait polls before a block gives up on its staging copy (each poll may suspend the thread
// for a while; the copy normally lands within microseconds).
constexpr uint32_t kStageWaitPolls = 1u << 22;

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
    for (uint32_t i = 0; i < kStageWaitPolls; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__global__ void __launch_bounds__(kThreads, 1) mlp_train_fused_kernel(FusedTrainArgs g) {
    extern __shared__ __align__(128) uint32_t smem[];
    __shared__ __align__(8) uint64_t stage_bar;
    uint32_t *Wf = smem;                      // layer l: [out][in]
    uint32_t *Wb = Wf + kLayers * kMat;       // layer l >= 1: [in][out] at index l - 1
    uint32_t *act = Wb + kHidden * kMat;      // two buffers [row][in]: layer l reads act + (l & 1) kMat
    uint32_t *actT = act + 2 * kMat;          // layer l's input: [in][row]
    uint32_t *Zs = actT + kLayers * kMat;     // hidden layer l's pre-activation: [row][out]
    uint32_t *dZ = Zs + kHidden * kMat;       // [row][out]
    uint32_t *dZT = dZ + kMat;                // [out][row]
    float *bias = reinterpret_cast<float *>(smem + kSmemWords);  // [5][64]
    float *dbias = bias + kLayers * kW;                          // [5][4 row blocks][64]
    float *xin = dbias + kLayers * kRowBlocks * kW;              // [64][6]
    float *tgt = xin + kTM * kIn;                                // [64][64]
    float *red = tgt + kTM * kW;                                 // loss per warp

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, gid = lane >> 2, tig = lane & 3;
    const int rb = warp & (kRowBlocks - 1), m0 = rb * 16, n0 = (warp / kRowBlocks) * kCols;
    const int out_dim = (int)g.out_dim;
    const uint32_t step = *g.step;

    // weights in both layouts: one bulk copy of the packed image (rows of the head beyond out_dim
    // and the row padding are zero there); biases by plain loads meanwhile
    const uint32_t bar = smem_u32(&stage_bar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(kImageBytes) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"(smem_u32(Wf)), "l"(g.image), "r"(kImageBytes), "r"(bar)
                     : "memory");
    }
    for (int l = 0; l < kLayers; l++) {
        const int fo = l == kHidden ? out_dim : kW;
        const float *Wl = g.params + (size_t)l * kLayerParams;
        for (int o = tid; o < kW; o += kThreads) bias[l * kW + o] = o < fo ? Wl[fo * kW + o] : 0.0f;
    }
    // the block's batch rows: Philox4x32-10 on (row, step, 0, "tran") keyed by the seed
    for (int r = tid; r < kTM; r += kThreads) {
        const uint32_t row = blockIdx.x * kTM + r;
        const bool ok = row < g.batch;
        uint32_t idx = row;
        if (ok && g.gather) {
            const uint4 h = philox4x32_10(make_uint4(row, step, 0u, 0x7472616eu), (uint32_t)g.seed,
                                          (uint32_t)(g.seed >> 32));
            idx = (uint32_t)(((uint64_t)h.x * g.n) >> 32);
        }
        for (int k = 0; k < kIn; k++) xin[r * kIn + k] = ok ? g.inputs[(size_t)idx * kIn + k] : 0.0f;
        for (int k = 0; k < out_dim; k++) tgt[r * kW + k] = ok ? g.targets[(size_t)idx * out_dim + k] : 0.0f;
    }
    if (tid < kWarps) red[tid] = 0.0f;
    __syncthreads();  // the barrier's initialisation is visible to every thread from here
    if (!mbar_wait_bounded(bar, 0u)) {
        // the staging copy did not land: flag it, give it one more bounded wait so that it does not
        // write into a later block's shared memory, and leave this block's gradient unwritten
        if (tid == 0) atomicOr(g.err, 1u);
        mbar_wait_bounded(bar, 0u);
        return;
    }
    // Fourier features (mlp.cu's fourier_kernel): phi[r][f] = sin 2 pi t, phi[r][32 + f] = cos 2 pi t
    for (int idx = tid; idx < kTM * 32; idx += kThreads) {
        const int r = idx >> 5, f = idx & 31;
        float t = 0.0f;
#pragma unroll
        for (int k = 0; k < kIn; k++) t = t + g.freqs[f * kIn + k] * xin[r * kIn + k];
        float s, c;
        sincospi_own(2.0f * t, &s, &c);
        reinterpret_cast<__nv_bfloat16 *>(act)[r * kLd * 2 + f] = __float2bfloat16_rn(s);
        reinterpret_cast<__nv_bfloat16 *>(act)[r * kLd * 2 + 32 + f] = __float2bfloat16_rn(c);
        store_t(actT, r, f, s);
        store_t(actT, r, 32 + f, c);
    }
    __syncthreads();

    // ---- forward: a warp reads all 64 columns of its row block's input and writes its kCols
    // columns of the output buffer; the row block's barrier publishes them before the next layer
    float acc[kNT][4];
    for (int l = 0; l < kHidden; l++) {
        const uint32_t *in = act + (l & 1) * kMat;
        uint32_t *out = act + ((l + 1) & 1) * kMat;
        zero_acc(acc);
        warp_gemm(acc, in, Wf + l * kMat, m0, n0, lane);
        uint32_t zp[kNT][2], hp[kNT][2];
#pragma unroll
        for (int j = 0; j < kNT; j++)
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
                const int col = n0 + j * 8 + 2 * tig;
                const float z0 = acc[j][2 * hh] + bias[l * kW + col], z1 = acc[j][2 * hh + 1] + bias[l * kW + col + 1];
                zp[j][hh] = pack2(z0, z1);
                hp[j][hh] = pack2(silu_f(z0), silu_f(z1));
            }
        store_tile<false>(Zs + l * kMat, zp, m0, n0, lane);
        store_tile<false>(out, hp, m0, n0, lane);
        store_tile<true>(actT + (l + 1) * kMat, hp, m0, n0, lane);
        row_block_sync(rb);
    }
    // head: y = act W^T + b; loss sum (y - t)^2 / count; acc becomes dY = 2 (y - t) / count
    {
        zero_acc(acc);
        warp_gemm(acc, act + (kHidden & 1) * kMat, Wf + kHidden * kMat, m0, n0, lane);
        const float count = (float)g.batch * (float)out_dim;
        float ls = 0.0f;
#pragma unroll
        for (int j = 0; j < kNT; j++)
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
                const int row = m0 + gid + 8 * hh, col = n0 + j * 8 + 2 * tig;
                const bool rok = blockIdx.x * kTM + row < g.batch;
                float d0 = 0.0f, d1 = 0.0f;
                if (rok && col < out_dim) d0 = acc[j][2 * hh] + bias[kHidden * kW + col] - tgt[row * kW + col];
                if (rok && col + 1 < out_dim)
                    d1 = acc[j][2 * hh + 1] + bias[kHidden * kW + col + 1] - tgt[row * kW + col + 1];
                ls += d0 * d0 + d1 * d1;
                acc[j][2 * hh] = 2.0f * d0 / count;
                acc[j][2 * hh + 1] = 2.0f * d1 / count;
            }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ls += __shfl_xor_sync(0xffffffffu, ls, o);
        if (lane == 0) red[warp] = ls / count;
    }
    // ---- backward: at the top of each iteration acc holds dL/dZ_l for this warp's rows and
    // columns (FP32)
    for (int l = kHidden; l >= 0; l--) {
        store_col_sums(acc, dbias + (l * kRowBlocks + rb) * kW, n0, lane, tig);
        {
            uint32_t dp[kNT][2];
#pragma unroll
            for (int j = 0; j < kNT; j++)
#pragma unroll
                for (int hh = 0; hh < 2; hh++) dp[j][hh] = pack2(acc[j][2 * hh], acc[j][2 * hh + 1]);
            store_tile<false>(dZ, dp, m0, n0, lane);
            store_tile<true>(dZT, dp, m0, n0, lane);
        }
        __syncthreads();
        const int fo = l == kHidden ? out_dim : kW;
        // weight gradient dW[o][i] = sum_r dZ[r][o] act_l[r][i]: warp w takes o in [m0, m0 + 16),
        // i in [n0, n0 + kCols)
        if (m0 < fo) {
            float wacc[kNT][4];
            zero_acc(wacc);
            warp_gemm(wacc, dZT, actT + l * kMat, m0, n0, lane);
            float *dst = g.partial + (size_t)blockIdx.x * g.n_params + (size_t)l * kLayerParams;
#pragma unroll
            for (int j = 0; j < kNT; j++)
#pragma unroll
                for (int hh = 0; hh < 2; hh++) {
                    const int o = m0 + gid + 8 * hh, i = n0 + j * 8 + 2 * tig;
                    // scalar stores: a block's gradient row starts at block * n_params floats, and
                    // n_params is odd for an odd head width, so pairs are not 8-byte aligned
                    if (o < fo) {
                        dst[o * kW + i] = wacc[j][2 * hh];
                        dst[o * kW + i + 1] = wacc[j][2 * hh + 1];
                    }
                }
        }
        if (l == 0) break;
        // input gradient dA = dZ W_l (this warp's rows and columns), then dZ_{l-1} = dA silu'(Z_{l-1})
        zero_acc(acc);
        warp_gemm(acc, dZ, Wb + (l - 1) * kMat, m0, n0, lane);
#pragma unroll
        for (int j = 0; j < kNT; j++)
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
                const int row = m0 + gid + 8 * hh, col = n0 + j * 8 + 2 * tig;
                const uint32_t zw = Zs[(l - 1) * kMat + row * kLd + (col >> 1)];
                acc[j][2 * hh] *= silu_d(lo_of(zw));
                acc[j][2 * hh + 1] *= silu_d(hi_of(zw));
            }
        __syncthreads();  // every warp is done reading dZ and dZ^T before they are overwritten
    }
    __syncthreads();
    // the block's bias gradients and loss
    float *dst = g.partial + (size_t)blockIdx.x * g.n_params;
    for (int l = 0; l < kLayers; l++) {
        const int fo = l == kHidden ? out_dim : kW;
        for (int o = tid; o < fo; o += kThreads) {
            float b = dbias[(l * kRowBlocks) * kW + o];
            for (int q = 1; q < kRowBlocks; q++) b += dbias[(l * kRowBlocks + q) * kW + o];
            dst[(size_t)l * kLayerParams + fo * kW + o] = b;
        }
    }
    if (tid == 0) {
        float l = red[0];
        for (int q = 1; q < kWarps; q++) l += red[q];
        g.partial_loss[blockIdx.x] = l;
    }
}

// Parameter i's place in the packed image: its BF16 halves in the forward operand W [out][in]
// and, for layers >= 1, in the backward operand W^T [in][out]; biases have none (returns false).
__device__ __forceinline__ bool image_slots(uint32_t i, uint32_t out_dim, uint32_t &f, uint32_t &b) {
    uint32_t l = i / kLayerParams;
    if (l > (uint32_t)kHidden) l = kHidden;
    const uint32_t r = i - l * kLayerParams;
    const uint32_t fo = l == (uint32_t)kHidden ? out_dim : (uint32_t)kW;
    if (r >= fo * kW) return false;
    const uint32_t o = r / kW, in = r % kW;
    f = (l * kMat + o * kLd) * 2u + in;
    b = l >= 1 ? (((uint32_t)kLayers + l - 1u) * kMat + in * kLd) * 2u + o : 0xFFFFFFFFu;
    return true;
}
__device__ __forceinline__ void image_store(uint32_t *image, uint32_t i, uint32_t out_dim, float v) {
    uint32_t f, b;
    if (!image_slots(i, out_dim, f, b)) return;
    __nv_bfloat16 *h = reinterpret_cast<__nv_bfloat16 *>(image);
    const __nv_bfloat16 x = __float2bfloat16_rn(v);
    h[f] = x;
    if (b != 0xFFFFFFFFu) h[b] = x;
}

__global__ void pack_weights_kernel(const float *__restrict__ p, uint32_t n_params, uint32_t out_dim,
                                    uint32_t *__restrict__ image) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_params) image_store(image, i, out_dim, p[i]);
}

// Block-ordered gradient sums: a block of 256 threads takes 32 parameters, 8 threads each summing
// every 8th block gradient in order, the 8 partial sums added in order (a fixed order: the step is
// deterministic).
constexpr int kRedSplit = 8;
__device__ __forceinline__ float ordered_gradient(const float *__restrict__ partial, uint32_t n_blocks,
                                                  uint32_t n_params, uint32_t i, float (*red)[33]) {
    const uint32_t q = threadIdx.x & 31u, sl = threadIdx.x >> 5;
    float s = 0.0f;
    if (i < n_params)
        for (uint32_t b = sl; b < n_blocks; b += kRedSplit) s += partial[(size_t)b * n_params + i];
    red[sl][q] = s;
    __syncthreads();
    float t = 0.0f;
    if (sl == 0)
        for (int k = 0; k < kRedSplit; k++) t += red[k][q];
    return t;
}

// The blocks' losses summed by one warp in a fixed order (lane-strided partial sums, then a
// butterfly that leaves the same value in every lane).
__device__ __forceinline__ float ordered_loss(const float *__restrict__ partial_loss, uint32_t n_blocks) {
    float l = 0.0f;
    for (uint32_t b = threadIdx.x & 31u; b < n_blocks; b += 32u) l += partial_loss[b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    return l;
}

// Sums the blocks' gradients and applies Adam with the cosine schedule of the current step, then
// stores the new weights into the packed image; block 0 records the step's loss. step[0] is the
// step counter, step[1] counts the blocks that are done with it: the last one advances the counter
// (every block has read it by then) and clears the count.
__global__ void __launch_bounds__(256) mlp_reduce_adam_kernel(
    float *__restrict__ p, float *__restrict__ m, float *__restrict__ v, const float *__restrict__ partial,
    const float *__restrict__ partial_loss, uint32_t n_blocks, uint32_t n_params, uint32_t out_dim,
    uint32_t *__restrict__ image, uint32_t *__restrict__ step, uint32_t steps, float lr0, uint32_t adam_base,
    float *__restrict__ loss_hist) {
    __shared__ float red[kRedSplit][33];
    const uint32_t s = *step;
    const uint32_t i = blockIdx.x * 32u + (threadIdx.x & 31u);
    const float gsum = ordered_gradient(partial, n_blocks, n_params, i, red);
    if (threadIdx.x < 32 && i < n_params) {
        const float lr = lr0 * 0.5f * (1.0f + cospif((float)s / (float)steps));
        const float t = (float)(adam_base + s + 1u);
        const float bc1 = 1.0f - powf(0.9f, t), bc2 = 1.0f - powf(0.999f, t);
        const float mi = 0.9f * m[i] + 0.1f * gsum;
        const float vi = 0.999f * v[i] + 0.001f * gsum * gsum;
        m[i] = mi;
        v[i] = vi;
        const float pi = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + 1e-8f);
        p[i] = pi;
        image_store(image, i, out_dim, pi);
    }
    if (loss_hist && blockIdx.x == 0 && threadIdx.x < 32) {
        const float l = ordered_loss(partial_loss, n_blocks);
        if (threadIdx.x == 0) loss_hist[s] = l;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(step + 1, 1u) == gridDim.x - 1u) {
            step[1] = 0u;
            step[0] = s + 1u;
        }
    }
}

__global__ void __launch_bounds__(256) mlp_reduce_grad_kernel(const float *__restrict__ partial,
                                                              const float *__restrict__ partial_loss, uint32_t n_blocks,
                                                              uint32_t n_params, float *__restrict__ grad,
                                                              float *__restrict__ loss) {
    __shared__ float red[kRedSplit][33];
    const uint32_t i = blockIdx.x * 32u + (threadIdx.x & 31u);
    const float gsum = ordered_gradient(partial, n_blocks, n_params, i, red);
    if (threadIdx.x < 32 && i < n_params) grad[i] = gsum;
    if (loss && blockIdx.x == 0 && threadIdx.x < 32) {
        const float l = ordered_loss(partial_loss, n_blocks);
        if (threadIdx.x == 0) *loss = l;
    }
}

}  // namespace

size_t fused_train_smem_bytes() { return kSmemWords * 4 + kSmemFloats * 4; }
size_t fused_train_image_words() { return kImageWords; }
uint32_t fused_train_blocks(uint32_t batch) { return (batch + kTM - 1) / kTM; }

cudaError_t launch_pack_weights(const float *params, uint32_t n_params, uint32_t out_dim, uint32_t *image,
                                cudaStream_t stream) {
    pack_weights_kernel<<<(n_params + 255) / 256, 256, 0, stream>>>(params, n_params, out_dim, image);
    return cudaGetLastError();
}

cudaError_t launch_fused_train_step(const FusedTrainArgs &a, float *params, float *adam_m, float *adam_v,
                                    uint32_t steps, float lr, uint32_t adam_base, float *loss_hist,
                                    cudaStream_t stream) {
    const uint32_t blocks = fused_train_blocks(a.batch);
    mlp_train_fused_kernel<<<blocks, kThreads, fused_train_smem_bytes(), stream>>>(a);
    mlp_reduce_adam_kernel<<<(a.n_params + 31) / 32, 256, 0, stream>>>(
        params, adam_m, adam_v, a.partial, a.partial_loss, blocks, a.n_params, a.out_dim, const_cast<uint32_t *>(a.image),
        a.step, steps, lr, adam_base, loss_hist);
    return cudaGetLastError();
}

cudaError_t launch_fused_gradient(const FusedTrainArgs &a, float *grad, float *loss, cudaStream_t stream) {
    const uint32_t blocks = fused_train_blocks(a.batch);
    cudaError_t e = launch_pack_weights(a.params, a.n_params, a.out_dim, const_cast<uint32_t *>(a.image), stream);
    if (e != cudaSuccess) return e;
    mlp_train_fused_kernel<<<blocks, kThreads, fused_train_smem_bytes(), stream>>>(a);
    mlp_reduce_grad_kernel<<<(a.n_params + 31) / 32, 256, 0, stream>>>(a.partial, a.partial_loss, blocks, a.n_params,
                                                                       grad, loss);
    return cudaGetLastError();
}

cudaError_t prepare_fused_train() {
    return cudaFuncSetAttribute(mlp_train_fused_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)fused_train_smem_bytes());
}

}  // namespace wobgb
