/*
 * fsph_mlp.cuh -- the warm-start network: a per-particle MLP
 * kFeatures -> 64 -> 64 -> 3 with ReLU, BF16 weights and activations on the
 * tensor cores, FP32 accumulation, FP32 master weights for training.
 *
 * Parameters travel as one FP32 "blob" (FSPH_MLP_BLOB_SIZE floats, layout in
 * include/fsph.h): input normalisation, W1 [kFeatures][64], b1, W2 [64][64], b2,
 * W3 [64][3], b3, output scale.  The device copy used by the kernels
 * (MlpDev) holds every weight matrix in the layouts the mma fragments load
 * from, with padded row strides so the 8 fragment rows of a warp fall in
 * distinct shared-memory banks.
 */
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "fsph_internal.cuh"

namespace fsph {

constexpr int kIn = kFeatures, kHid = 64, kOut = 3;
static_assert(kIn % 16 == 0, "the input is a whole number of 16-wide MMA k-steps");
/* blob offsets (floats) */
constexpr int kBMu = 0;
constexpr int kBSig = kBMu + kIn;
constexpr int kBW1 = kBSig + kIn;
constexpr int kBB1 = kBW1 + kIn * kHid;
constexpr int kBW2 = kBB1 + kHid;
constexpr int kBB2 = kBW2 + kHid * kHid;
constexpr int kBW3 = kBB2 + kHid;
constexpr int kBB3 = kBW3 + kHid * kOut;
constexpr int kBScale = kBB3 + kOut;
constexpr int kBlob = kBScale + 1;
constexpr int kTrainFirst = kBW1;  /* W1 .. b3 are trained; normalisation and scale are fixed */
constexpr int kTrainLast = kBScale;

constexpr int kS1 = kIn + 8;   /* padded strides (bf16 elements) */
constexpr int kS2 = kHid + 8;
constexpr int kS3 = 16;

struct MlpDev {
    __nv_bfloat16 w1t[kHid * kS1];   /* [n = hidden1][k = input]          forward  */
    __nv_bfloat16 w2t[kHid * kS2];   /* [n = hidden2][k = hidden1]        forward  */
    __nv_bfloat16 w3t[8 * kS2];      /* [n = output (pad 8)][k = hidden2] forward  */
    __nv_bfloat16 w2[kHid * kS2];    /* [n = hidden1][k = hidden2]        backward */
    __nv_bfloat16 w3[kHid * kS3];    /* [n = hidden2][k = output (pad 16)] backward */
    float b1[kHid], b2[kHid], b3[8];
    float mu[kIn], isig[kIn];
    float out_scale;
};

/* master FP32 blob -> MlpDev */
void launch_mlp_pack(const float *blob, MlpDev *dev, cudaStream_t s);
/* y[i] = network(x[i]) * out_scale * scale (first 3 components; w = 0);
 * x: n rows of kIn raw features.  If valid != NULL and *valid == 0 the
 * outputs are zero (no features yet).  local_only: read only the first 16
 * inputs (for a network that gives the others no weight). */
void launch_mlp_infer(const MlpDev *m, const float *x, int n, float4 *y, float scale, const unsigned int *valid,
                      cudaStream_t s, bool local_only = false);
/* same network, plain n x 3 output (for training checks) */
void launch_mlp_forward3(const MlpDev *m, const float *x, int n, float *y, cudaStream_t s);
/* the same two on the tcgen05 tensor cores with TMEM accumulators
 * (fsph_mlp_tc.cu); *err |= 1 when a wait on an MMA or a TMA load ran out.
 * tma: a network of the 16 local inputs reads them by TMA boxes
 * (k_mlp_infer_tma), else by per-thread loads (the same results) */
void launch_mlp_infer_tc(const MlpDev *m, const float *x, int n, float4 *y, float scale, const unsigned int *valid,
                         unsigned int *err, cudaStream_t s, bool local_only = false, bool tma = true);
/* looks up the driver entry point the TMA inference needs (outside any
 * stream capture) */
void mlp_tc_prepare();
void launch_mlp_forward3_tc(const MlpDev *m, const float *x, int n, float *y, unsigned int *err, cudaStream_t s);
/* per-block partial gradients of L = mean_i sum_k (y_ik - t_ik / out_scale)^2
 * (blob layout, nblocks rows) and per-block loss sums */
int mlp_grad_blocks(int n);
void launch_mlp_grad(const MlpDev *m, const float *x, const float *t, int n, float *part, float *loss_part,
                     cudaStream_t s);
/* fixed-order sum of the partials into grad[kBlob] and *loss */
void launch_mlp_reduce(const float *part, const float *loss_part, int nblocks, int n, float *grad, float *loss,
                       cudaStream_t s);
/* Adam on the trained range of the blob */
void launch_mlp_adam(float *blob, float *m1, float *m2, const float *grad, float lr, float b1, float b2, float eps,
                     int step, cudaStream_t s);

}  // namespace fsph
