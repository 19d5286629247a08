// Fused training step of the Fourier-feature MLP (mlp.cu's network with 4 hidden layers): one
// kernel runs the batch gather, the forward pass and the backward pass of 64 rows per block with
// every weight and activation in shared memory and writes the block's gradient; a second kernel
// sums the blocks' gradients in a fixed order (so a step is deterministic), applies Adam, writes
// the updated weights as a packed BF16 image in both operand layouts, and its last block advances
// the step counter. Both are programmatic dependent launches (each starts its set-up while the
// previous kernel finishes and waits for it in griddepcontrol.wait); wob_mlp_train captures 16
// steps into a CUDA graph and replays it. Each block of the next step stages that image (74 KB)
// into shared memory with one TMA bulk copy (cp.async.bulk, completion on an mbarrier, the wait
// bounded; the Fourier features are computed meanwhile), instead of every block reading and
// converting the FP32 parameters itself.
//
// Network and parameter layout as in mlp.cu: phi = [sin, cos](2 pi B v) (32 frequencies of the
// 6 inputs), 4 hidden layers 64 -> 64 with SiLU, a linear 64 -> out_dim head; FP32 parameters,
// for each layer W [out][in] row-major then b [out]. Pre-activations are kept as BF16 for the SiLU
// derivative, bias gradients are summed in FP32 from the FP32 products. No atomics: every sum has
// a fixed order, so training is deterministic.
//
// Products: every 64 x 64 x 64 product C[m][n] = sum_k A[m][k] B[n][k] is four tcgen05.mma
// (kind::f16, BF16 operands from shared memory, M = 64, N = 64, K = 16 each) issued by one thread,
// the FP32 accumulator in tensor memory (TMEM), completion signalled on an mbarrier by
// tcgen05.commit. With M = 64 the accumulator's rows 16 q .. 16 q + 15 sit in TMEM lanes 32 q ..
// 32 q + 15, the lane quarter that warps w with w % 4 = q may read: warp w reads rows
// [16 (w % 4), +16) x columns [16 (w / 4), +16) with tcgen05.ld.16x256b (the mma.sync m16n8
// accumulator layout: lane l holds rows l / 4 and l / 4 + 8, columns 2 (l % 4) and + 1 of each
// 8-column tile) and runs the epilogue on them. Both operands are K-major:
//   forward  Z = A W^T:     A = activation [row][in],   B = W   [out][in]
//   weights  dW = dZ^T A:   A = dZ^T [out][row],        B = A^T [in][row]
//   inputs   dA = dZ W:     A = dZ   [row][out],        B = W^T [in][out]
// each stored in the no-swizzle core-matrix layout (cm_index): 8 x 8 BF16 core matrices of 128
// contiguous bytes, K-adjacent ones 128 bytes apart (the descriptor's leading byte offset), 8-row
// groups 1024 bytes apart (its stride byte offset). Epilogues write those layouts with stmatrix
// (.trans for the transposed copies): the 8 rows of a core matrix are one 128-byte line, so a
// phase touches 32 distinct banks.
#include "../../include/wob_capi.h"

#include "device_common.cuh"
#include "launch.hpp"
#include "mlp_train.hpp"

#include <cuda_bf16.h>

namespace wobgb {

namespace {

constexpr int kTM = 64;          // rows per block
constexpr int kW = 64;           // layer width
constexpr int kMatHalves = kW * kW;   // BF16 values per 64 x 64 operand
constexpr int kMat = kMatHalves / 2;  // 32-bit words per operand
constexpr int kHidden = 4;
constexpr int kLayers = kHidden + 1;
constexpr int kIn = 6;
// 16 warps: warp w handles rows [16 (w & 3), +16) x columns [16 (w >> 2), +16) of every product's
// accumulator
constexpr int kRowBlocks = kTM / 16;
constexpr int kColSplit = 4;
constexpr int kWarps = kRowBlocks * kColSplit;
constexpr int kThreads = kWarps * 32;
constexpr int kCols = kW / kColSplit;  // columns per warp
constexpr int kNT = kCols / 8;         // 8-column tiles per warp
static_assert(kNT == 2, "the TMEM loads and the tile stores move two 8-column tiles");
constexpr int kLayerParams = kW * kW + kW;
// TMEM: columns [0, 64) take forward and input-gradient products, [64, 128) and [128, 192) the
// weight gradients of odd and even layers (read out while the next layer's products run)
constexpr uint32_t kTmemCols = 256;

// operands: Wf (5), Wb (4), act, actT (5), Zs (4), dZ, dZT (2: layer l's in dZT + (l & 1) kMat, kept
// until its weight-gradient product has been read out)
constexpr size_t kSmemWords = (size_t)(kLayers + kHidden + 1 + kLayers + kHidden + 3) * kMat;
constexpr size_t kSmemFloats = kLayers * kW + kLayers * kRowBlocks * kW + kTM * kIn + kTM * kW + kWarps;

// BF16 index of element (r, k) of a 64 x 64 K-major operand in the no-swizzle core-matrix layout.
__host__ __device__ constexpr uint32_t cm_index(uint32_t r, uint32_t k) {
    return (r >> 3) * 512u + (k >> 3) * 64u + (r & 7u) * 8u + (k & 7u);
}

// Two floats rounded to BF16 in one word, lo in the low half (one cvt.rn.bf16x2.f32).
__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&v);
}
__device__ __forceinline__ float lo_of(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float hi_of(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ---- tcgen05 helpers
// Shared-memory descriptor of a no-swizzle K-major operand starting at byte address addr:
// start >> 4 (bits 0-13), leading byte offset 128 >> 4 (bits 16-29), stride byte offset
// 1024 >> 4 (bits 32-45), descriptor version 1 (bits 46-47), base offset 0, no swizzle.
__device__ __forceinline__ uint64_t operand_desc(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(1024u >> 4) << 32) |
           (1ull << 46);
}
// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and B (bits 7-9,
// 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kW >> 3) << 17) | ((uint32_t)(kTM >> 4) << 24);

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor cores' reads
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D[tmem] (=|+=) A B^T over K = 64: four K = 16 steps, 256 bytes apart in both operands.
__device__ __forceinline__ void issue_product(uint32_t d_tmem, const uint32_t *A, const uint32_t *B) {
    const uint32_t a = smem_u32(A), b = smem_u32(B);
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
        const uint64_t ad = operand_desc(a + kk * 256u), bd = operand_desc(b + kk * 256u);
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
            "l"(ad), "l"(bd), "r"(kIdesc), "r"(kk));
    }
}
// Arrives on the mbarrier once every tcgen05.mma this thread issued before has completed.
__device__ __forceinline__ void commit_to(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
// Rows [16 q, +16) x 16 columns of a product from TMEM (taddr: lane 32 q, first column) into
// acc[j][.] in the m16n8 accumulator layout of 8-column tile j.
__device__ __forceinline__ void load_acc(float acc[kNT][4], uint32_t taddr) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.16x256b.x2.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < kNT; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[j][q] = __uint_as_float(r[4 * j + q]);
}

// SiLU and its derivative with the fast exponential and division intrinsics (the values are rounded
// to BF16 or multiply BF16-rounded gradients, so their few-ulp error does not show). For z below
// about -88, exp(-z) overflows and __fdividef returns 0 for the huge or infinite denominator, the
// limit of both functions.
__device__ __forceinline__ float silu_f(float z) { return __fdividef(z, 1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_d(float z) {
    const float s = __fdividef(1.0f, 1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

// Stores a warp's 16 x 16 tile of packed BF16 pairs p[j][h] (accumulator layout: row m0 + gid +
// 8 h, columns n0 + 8 j + 2 tig, +1) into operand M at (row, col), or with kTrans at (col, row)
// (the transposed operand): one stmatrix.x4 of four 8 x 8 matrices, each one core matrix.
template <bool kTrans>
__device__ __forceinline__ void store_tile(uint32_t *M, const uint32_t p[kNT][2], int m0, int n0, int lane) {
    const int r = lane & 7, mi = lane >> 3;
    const int row = m0 + 8 * (mi & 1), col = n0 + 8 * (mi >> 1);
    const uint32_t idx = kTrans ? cm_index(col + r, row) : cm_index(row + r, col);
    const uint32_t addr = smem_u32(reinterpret_cast<__nv_bfloat16 *>(M) + idx);
    if (kTrans)
        asm volatile("stmatrix.sync.aligned.m8n8.x4.trans.shared.b16 [%0], {%1,%2,%3,%4};" ::"r"(addr), "r"(p[0][0]),
                     "r"(p[0][1]), "r"(p[1][0]), "r"(p[1][1])
                     : "memory");
    else
        asm volatile("stmatrix.sync.aligned.m8n8.x4.shared.b16 [%0], {%1,%2,%3,%4};" ::"r"(addr), "r"(p[0][0]),
                     "r"(p[0][1]), "r"(p[1][0]), "r"(p[1][1])
                     : "memory");
}

// BF16 value at (r, k) of an operand.
__device__ __forceinline__ void store_bf16(uint32_t *M, int r, int k, float v) {
    reinterpret_cast<__nv_bfloat16 *>(M)[cm_index(r, k)] = __float2bfloat16_rn(v);
}

// Column sums over the warp's 16 rows of the FP32 values in acc (accumulator layout of tile j),
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
// try_wait polls before a block gives up on its staging copy or a product (each poll may suspend
// the thread for a while; either normally completes within microseconds).
constexpr uint32_t kWaitPolls = 1u << 22;

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, uint32_t polls = kWaitPolls) {
    for (uint32_t i = 0; i < polls; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Error bits of FusedTrainArgs::err.
constexpr uint32_t kErrStage = 1u;    // the weight image's bulk copy did not land within the bound
constexpr uint32_t kErrProduct = 2u;  // a product's completion did not arrive within the bound

__global__ void __launch_bounds__(kThreads, 1) mlp_train_fused_kernel(FusedTrainArgs g) {
    extern __shared__ __align__(128) uint32_t smem[];
    // mbarriers: the weight image's staging, forward / input-gradient products, weight-gradient
    // products of even and odd layers (one phase outstanding at a time on each), the teardown drain
    __shared__ __align__(8) uint64_t stage_bar, mma_bar, wgrad_bar[2], drain_bar;
    __shared__ uint32_t tmem_slot;
    uint32_t *Wf = smem;                      // layer l: [out][in]
    uint32_t *Wb = Wf + kLayers * kMat;       // layer l >= 1: [in][out] at index l - 1
    uint32_t *act = Wb + kHidden * kMat;      // [row][in] of the layer being evaluated
    uint32_t *actT = act + kMat;              // layer l's input: [in][row]
    uint32_t *Zs = actT + kLayers * kMat;     // hidden layer l's pre-activation: [row][out]
    uint32_t *dZ = Zs + kHidden * kMat;       // [row][out]
    uint32_t *dZT = dZ + kMat;                // two buffers [out][row]
    float *bias = reinterpret_cast<float *>(smem + kSmemWords);  // [5][64]
    float *dbias = bias + kLayers * kW;                          // [5][4 row blocks][64]
    float *xin = dbias + kLayers * kRowBlocks * kW;              // [64][6]
    float *tgt = xin + kTM * kIn;                                // [64][64]
    float *red = tgt + kTM * kW;                                 // loss per warp

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, gid = lane >> 2, tig = lane & 3;
    const int rb = warp & (kRowBlocks - 1), m0 = rb * 16, n0 = (warp / kRowBlocks) * kCols;
    const int out_dim = (int)g.out_dim;

    // mbarriers and TMEM columns for the accumulators first: they depend on no earlier kernel, so
    // under a programmatic dependent launch they overlap the previous update's tail
    const uint32_t bar = smem_u32(&stage_bar), pbar = smem_u32(&mma_bar), dbar = smem_u32(&drain_bar);
    const uint32_t wbar0 = smem_u32(&wgrad_bar[0]), wbar1 = smem_u32(&wgrad_bar[1]);
    if (tid == 0) {
        for (uint32_t b : {bar, pbar, wbar0, wbar1, dbar})
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // the previous update (weights, image, step counter) complete and visible from here (returns
    // at once without a programmatic dependency); the next kernel may start launching
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;");
    const uint32_t step = *g.step;
    // weights in both layouts: one bulk copy of the packed image (rows of the head beyond out_dim
    // are zero there); biases by plain loads meanwhile
    if (tid == 0) {
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
    tc_fence_before();
    __syncthreads();  // the barriers' initialisation and the TMEM address are visible from here
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t t_lane = tmem + ((uint32_t)(32 * rb) << 16);  // this warp's lane quarter
    // parities of the next completions: mma_bar; wgrad_bar[p] in bit p of wphase
    uint32_t phase = 0, wphase = 0;
    int w_pending = -1;                      // layer whose weight gradient waits in TMEM to be read out
    bool ok = true;
    uint32_t err = 0;
    // Fourier features (mlp.cu's fourier_kernel): phi[r][f] = sin 2 pi t, phi[r][32 + f] = cos 2 pi t,
    // computed while the weight image's copy is in flight (act and actT lie outside its destination)
    for (int idx = tid; idx < kTM * 32; idx += kThreads) {
        const int r = idx >> 5, f = idx & 31;
        float t = 0.0f;
#pragma unroll
        for (int k = 0; k < kIn; k++) t = t + g.freqs[f * kIn + k] * xin[r * kIn + k];
        float s, c;
        sincospi_own(2.0f * t, &s, &c);
        store_bf16(act, r, f, s);
        store_bf16(act, r, 32 + f, c);
        store_bf16(actT, f, r, s);
        store_bf16(actT, 32 + f, r, c);
    }
    fence_async_smem();
    // the barrier of the staging wait also publishes the features to the tensor cores
    if (!__syncthreads_and(mbar_wait_bounded(bar, 0u))) {
        // the staging copy did not land: give it one more bounded wait so that it does not write
        // into a later block's shared memory, release TMEM and leave this block's gradient unwritten
        err = kErrStage;
        mbar_wait_bounded(bar, 0u);
        ok = false;
    }
    if (ok) {
        // injected failure (tests): a bounded wait on drain_bar, on which nothing arrives before the
        // teardown, runs out like a product whose completion never came
        if (g.inject_wait_polls) ok = __syncthreads_and(mbar_wait_bounded(dbar, 0u, g.inject_wait_polls));

        float acc[kNT][4];
        // ---- forward: Z_l = act W_l^T in TMEM columns [0, 64); ok is block-uniform at the top of
        // each layer (the __syncthreads_and that ends the previous one)
        for (int l = 0; l < kHidden && ok; l++) {
            if (tid == 0) {
                tc_fence_after();
                issue_product(tmem, act, Wf + l * kMat);
                commit_to(pbar);
            }
            ok = mbar_wait_bounded(pbar, phase);
            phase ^= 1u;
            tc_fence_after();
            load_acc(acc, t_lane + n0);
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
            // the product has read act (its completion arrived), so act takes the layer's output
            store_tile<false>(Zs + l * kMat, zp, m0, n0, lane);
            store_tile<false>(act, hp, m0, n0, lane);
            store_tile<true>(actT + (l + 1) * kMat, hp, m0, n0, lane);
            fence_async_smem();
            tc_fence_before();
            ok = __syncthreads_and(ok);
        }
        // `run` is the block-wide verdict (a __syncthreads_and), `ok` this thread's own waits since
        bool run = ok;
        // head: y = act W^T + b; loss sum (y - t)^2 / count; acc becomes dY = 2 (y - t) / count
        if (run) {
            if (tid == 0) {
                tc_fence_after();
                issue_product(tmem, act, Wf + kHidden * kMat);
                commit_to(pbar);
            }
            ok = mbar_wait_bounded(pbar, phase);
            phase ^= 1u;
            tc_fence_after();
            load_acc(acc, t_lane + n0);
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
        // columns (FP32). dA = dZ W_l goes to TMEM columns [0, 64) and is committed first (the next
        // layer waits for it); dW_l = dZ^T act_l (dZ^T from buffer l & 1) to columns 64 + 64 (l & 1),
        // committed on wgrad_bar[l & 1] and read out one iteration later, while the next layer's
        // products run. Buffer and columns l & 1 are next written by layer l - 2, after that readout
        // (and the barrier that starts layer l - 1).
        auto drain_wgrad = [&]() {
            // weight gradient dW[o][i] of layer w_pending: warp w takes o in [m0, m0 + 16), i in
            // [n0, n0 + 16)
            const int lw = w_pending, pw = lw & 1;
            ok = mbar_wait_bounded(pw ? wbar1 : wbar0, (wphase >> pw) & 1u) && ok;
            wphase ^= 1u << pw;
            tc_fence_after();
            const int fo = lw == kHidden ? out_dim : kW;
            if (m0 < fo) {
                float wacc[kNT][4];
                load_acc(wacc, t_lane + 64u + 64u * (uint32_t)(lw & 1) + n0);
                float *dst = g.partial + (size_t)blockIdx.x * g.n_params + (size_t)lw * kLayerParams;
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
            w_pending = -1;
        };
        for (int l = kHidden; l >= 0 && run; l--) {
            store_col_sums(acc, dbias + (l * kRowBlocks + rb) * kW, n0, lane, tig);
            {
                uint32_t dp[kNT][2];
#pragma unroll
                for (int j = 0; j < kNT; j++)
#pragma unroll
                    for (int hh = 0; hh < 2; hh++) dp[j][hh] = pack2(acc[j][2 * hh], acc[j][2 * hh + 1]);
                store_tile<false>(dZ, dp, m0, n0, lane);
                store_tile<true>(dZT + (l & 1) * kMat, dp, m0, n0, lane);
            }
            fence_async_smem();
            tc_fence_before();
            run = __syncthreads_and(ok);
            if (!run) break;
            if (tid == 0) {
                tc_fence_after();
                if (l > 0) {
                    issue_product(tmem, dZ, Wb + (l - 1) * kMat);
                    commit_to(pbar);
                }
                issue_product(tmem + 64u + 64u * (uint32_t)(l & 1), dZT + (l & 1) * kMat, actT + l * kMat);
                commit_to((l & 1) ? wbar1 : wbar0);
            }
            if (w_pending >= 0) drain_wgrad();  // the previous layer's dW, in the other columns
            w_pending = l;
            if (l == 0) break;
            // dZ_{l-1} = dA silu'(Z_{l-1}) for this warp's rows and columns (dA has read dZ once
            // mma_bar arrives, so the next iteration may overwrite it)
            ok = mbar_wait_bounded(pbar, phase) && ok;
            phase ^= 1u;
            tc_fence_after();
            load_acc(acc, t_lane + n0);
#pragma unroll
            for (int j = 0; j < kNT; j++)
#pragma unroll
                for (int hh = 0; hh < 2; hh++) {
                    const int row = m0 + gid + 8 * hh, col = n0 + j * 8 + 2 * tig;
                    const uint32_t zw = reinterpret_cast<const uint32_t *>(
                        reinterpret_cast<const __nv_bfloat16 *>(Zs + (l - 1) * kMat) + cm_index(row, col))[0];
                    acc[j][2 * hh] *= silu_d(lo_of(zw));
                    acc[j][2 * hh + 1] *= silu_d(hi_of(zw));
                }
        }
        if (run && w_pending >= 0) drain_wgrad();
        if (!ok) err = kErrProduct;
    }
    // teardown: on an error, one more commit (on drain_bar, bounded wait) covers every product this
    // block issued; every TMEM load has finished; then the TMEM columns are released
    const bool all_ok = __syncthreads_and(err == 0);
    if (!all_ok && tid == 0) {
        commit_to(dbar);
        mbar_wait_bounded(dbar, 0u);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
    if (!all_ok) {
        if (tid == 0) atomicOr(g.err, err ? err : kErrProduct);
        return;
    }
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
    f = l * (uint32_t)kMatHalves + cm_index(o, in);
    b = l >= 1 ? ((uint32_t)kLayers + l - 1u) * (uint32_t)kMatHalves + cm_index(in, o) : 0xFFFFFFFFu;
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
    float *__restrict__ loss_hist, const uint32_t *__restrict__ err) {
    __shared__ float red[kRedSplit][33];
    // the fused step's gradients complete and visible from here; the next step may start launching
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;");
    // a block of the fused step failed (its gradient is missing): no update, no step advance, so the
    // parameters stay those of the last complete step
    if (*err) return;
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

// A launch that may begin while the stream's previous kernel is still running (programmatic
// dependent launch): the kernel waits for that kernel's completion itself (griddepcontrol.wait).
template <typename... Params, typename... Args>
cudaError_t launch_after_previous(void (*kernel)(Params...), uint32_t grid, uint32_t block, size_t smem,
                                  cudaStream_t stream, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

cudaError_t launch_fused_train_step(const FusedTrainArgs &a, float *params, float *adam_m, float *adam_v,
                                    uint32_t steps, float lr, uint32_t adam_base, float *loss_hist,
                                    cudaStream_t stream) {
    const uint32_t blocks = fused_train_blocks(a.batch);
    cudaError_t e = launch_after_previous(mlp_train_fused_kernel, blocks, kThreads, fused_train_smem_bytes(), stream, a);
    if (e != cudaSuccess) return e;
    return launch_after_previous(mlp_reduce_adam_kernel, (a.n_params + 31) / 32, 256, 0, stream, params, adam_m, adam_v,
                                 (const float *)a.partial, (const float *)a.partial_loss, blocks, a.n_params, a.out_dim,
                                 const_cast<uint32_t *>(a.image), a.step, steps, lr, adam_base, loss_hist,
                                 (const uint32_t *)a.err);
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
