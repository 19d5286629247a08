// Fused MLP training step (mlp_train.cu), used by wob_mlp_train for the 4-hidden-layer network.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace wobgb {

struct FusedTrainArgs {
    const float *params;   // [n_params], mlp.cu's layout
    const float *freqs;    // [32][6]
    const float *inputs;   // [n][6] training rows
    const float *targets;  // [n][out_dim]
    uint32_t n, out_dim, batch, n_params;
    uint32_t gather;       // 1: rows drawn by Philox from the n rows; 0: row r of the batch is row r
    uint64_t seed;
    uint32_t *step;        // [2]: step counter (batch draws, learning-rate schedule); blocks done with it
    float *partial;        // [blocks][n_params]: each block's gradient
    float *partial_loss;   // [blocks]
    const uint32_t *image; // packed BF16 weights, both operand layouts (fused_train_image_words words)
    uint32_t *err;         // bit 0: a block's weight staging, bit 1: a product did not complete within its wait bound
    // Nonzero (tests of the failure path): before its first product every block also waits this
    // many polls on an mbarrier nothing arrives on, and takes that as a product whose completion
    // did not arrive.
    uint32_t inject_wait_polls;
};

size_t fused_train_smem_bytes();
size_t fused_train_image_words();
// The packed weight image of params (launch_fused_train_step keeps it current after each update;
// call this before the first step and whenever the parameters were changed by other means). The
// image's padding words must be zero (zero the allocation once).
cudaError_t launch_pack_weights(const float *params, uint32_t n_params, uint32_t out_dim, uint32_t *image,
                                cudaStream_t stream);
uint32_t fused_train_blocks(uint32_t batch);
cudaError_t prepare_fused_train();
// One step: fused forward/backward, block-ordered gradient sum + Adam (cosine learning rate from
// lr over `steps`; bias corrections at step adam_base + s + 1), step counter + 1 (by the update's
// last block; step[1] must be zero before the first step).
cudaError_t launch_fused_train_step(const FusedTrainArgs &a, float *params, float *adam_m, float *adam_v,
                                    uint32_t steps, float lr, uint32_t adam_base, float *loss_hist,
                                    cudaStream_t stream);
// The fused kernel's gradient and loss of one batch, summed over blocks into grad / loss (no update).
cudaError_t launch_fused_gradient(const FusedTrainArgs &a, float *grad, float *loss, cudaStream_t stream);

}  // namespace wobgb
