/*
 * fsph_mlp.cu -- BF16 tensor-core kernels of the warm-start network
 * (inference, training gradients, Adam) and the fsph_mlp_* C ABI.
 *
 * Tensor-core use: mma.sync.m16n8k16 BF16 x BF16 -> FP32.  One warp owns
 * 16 particles (the M dimension); layer outputs stay in registers and the
 * FP32 accumulator fragment of one layer is repacked in place as the BF16
 * A fragment of the next (the m16n8k16 C and A layouts line up tile pairs).
 * Training stages each 64-sample chunk's activations and deltas in shared
 * memory, transposed ([feature][sample]), so that the weight-gradient
 * products (K = samples) are tensor-core MMAs as well; every block writes a
 * partial gradient and a fixed-order reduction sums them (deterministic).
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/fsph.h"
#include "fsph_mlp.cuh"

namespace fsph {

static_assert(kBlob == FSPH_MLP_BLOB_SIZE, "blob size in fsph.h");

__device__ __forceinline__ void mma16816(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

/* two floats -> bf16x2, the first in the low half (the lower column) */
__device__ __forceinline__ unsigned pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<unsigned *>(&v);
}
__device__ __forceinline__ unsigned ld32(const __nv_bfloat16 *p) { return *reinterpret_cast<const unsigned *>(p); }

/* --------------------------------------------------------------------- */
__global__ void k_mlp_pack(const float *__restrict__ b, MlpDev *__restrict__ d) {
    const __nv_bfloat16 z = __float2bfloat16(0.0f);
    for (int e = threadIdx.x; e < kHid * kS1; e += blockDim.x) {
        int n = e / kS1, k = e % kS1;
        d->w1t[e] = k < kIn ? __float2bfloat16(b[kBW1 + k * kHid + n]) : z;
    }
    for (int e = threadIdx.x; e < kHid * kS2; e += blockDim.x) {
        int n = e / kS2, k = e % kS2;
        d->w2t[e] = k < kHid ? __float2bfloat16(b[kBW2 + k * kHid + n]) : z;
        d->w2[e] = k < kHid ? __float2bfloat16(b[kBW2 + n * kHid + k]) : z;
    }
    for (int e = threadIdx.x; e < 8 * kS2; e += blockDim.x) {
        int n = e / kS2, k = e % kS2;
        d->w3t[e] = (n < kOut && k < kHid) ? __float2bfloat16(b[kBW3 + k * kOut + n]) : z;
    }
    for (int e = threadIdx.x; e < kHid * kS3; e += blockDim.x) {
        int n = e / kS3, k = e % kS3;
        d->w3[e] = k < kOut ? __float2bfloat16(b[kBW3 + n * kOut + k]) : z;
    }
    for (int e = threadIdx.x; e < kHid; e += blockDim.x) {
        d->b1[e] = b[kBB1 + e];
        d->b2[e] = b[kBB2 + e];
    }
    for (int e = threadIdx.x; e < 8; e += blockDim.x) d->b3[e] = e < kOut ? b[kBB3 + e] : 0.0f;
    for (int e = threadIdx.x; e < kIn; e += blockDim.x) {
        d->mu[e] = b[kBMu + e];
        float s = b[kBSig + e];
        d->isig[e] = s > 1e-20f ? 1.0f / s : 0.0f;
    }
    if (threadIdx.x == 0) d->out_scale = b[kBScale];
}

__device__ __forceinline__ void copy_model(MlpDev &sm, const MlpDev *__restrict__ gm) {
    const unsigned *src = reinterpret_cast<const unsigned *>(gm);
    unsigned *dst = reinterpret_cast<unsigned *>(&sm);
    for (int k = threadIdx.x; k < (int)(sizeof(MlpDev) / 4); k += blockDim.x) dst[k] = src[k];
}

/* Forward pass of one warp's 16 rows starting at base.  Leaves the ReLU'd
 * hidden layers (h1, h2) and the output fragment o (rows g / g+8, columns
 * 2c, 2c+1; columns >= 3 are padding).  Rows >= n read zero features. */
struct Fwd {
    float h1[8][4], h2[8][4], o[4];
    unsigned ax[kIn / 16][4];
    /* normalised inputs of this thread, per 16-column k tile kt:
     * (g, 16kt+2c..+1), (g+8, ..), (g, 16kt+2c+8..+9), (g+8, ..) */
    float xn[kIn / 2];
};

/* KT: the 16-wide input tiles read (inputs past them contribute nothing:
 * a network that gives them no weight runs with KT = 1) */
template <int KT = kIn / 16>
__device__ __forceinline__ void mlp_forward(const MlpDev &sm, const float *__restrict__ x, int n, int base, int g,
                                            int c, Fwd &F) {
    const int r0 = base + g, r1 = base + g + 8;
#pragma unroll
    for (int kt = 0; kt < KT; ++kt) {
        const int cols[4] = {16 * kt + 2 * c, 16 * kt + 2 * c + 1, 16 * kt + 2 * c + 8, 16 * kt + 2 * c + 9};
        float *xn = F.xn + 8 * kt;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int col = cols[q];
            const float v0 = r0 < n ? __ldg(x + (size_t)r0 * kIn + col) : 0.0f;
            const float v1 = r1 < n ? __ldg(x + (size_t)r1 * kIn + col) : 0.0f;
            xn[q] = r0 < n ? (v0 - sm.mu[col]) * sm.isig[col] : 0.0f;       /* row g   */
            xn[4 + q] = r1 < n ? (v1 - sm.mu[col]) * sm.isig[col] : 0.0f;   /* row g+8 */
        }
        F.ax[kt][0] = pack2(xn[0], xn[1]);
        F.ax[kt][1] = pack2(xn[4], xn[5]);
        F.ax[kt][2] = pack2(xn[2], xn[3]);
        F.ax[kt][3] = pack2(xn[6], xn[7]);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float b0v = sm.b1[8 * j + 2 * c], b1v = sm.b1[8 * j + 2 * c + 1];
        F.h1[j][0] = b0v; F.h1[j][1] = b1v; F.h1[j][2] = b0v; F.h1[j][3] = b1v;
#pragma unroll
        for (int kt = 0; kt < KT; ++kt) {
            const __nv_bfloat16 *w = sm.w1t + (8 * j + g) * kS1 + 16 * kt + 2 * c;
            mma16816(F.h1[j], F.ax[kt], ld32(w), ld32(w + 8));
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) F.h1[j][e] = fmaxf(F.h1[j][e], 0.0f);
    }
    unsigned a[4][4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        a[s][0] = pack2(F.h1[2 * s][0], F.h1[2 * s][1]);
        a[s][1] = pack2(F.h1[2 * s][2], F.h1[2 * s][3]);
        a[s][2] = pack2(F.h1[2 * s + 1][0], F.h1[2 * s + 1][1]);
        a[s][3] = pack2(F.h1[2 * s + 1][2], F.h1[2 * s + 1][3]);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float b0v = sm.b2[8 * j + 2 * c], b1v = sm.b2[8 * j + 2 * c + 1];
        F.h2[j][0] = b0v; F.h2[j][1] = b1v; F.h2[j][2] = b0v; F.h2[j][3] = b1v;
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const __nv_bfloat16 *w = sm.w2t + (8 * j + g) * kS2 + 16 * s + 2 * c;
            mma16816(F.h2[j], a[s], ld32(w), ld32(w + 8));
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) F.h2[j][e] = fmaxf(F.h2[j][e], 0.0f);
    }
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        a[s][0] = pack2(F.h2[2 * s][0], F.h2[2 * s][1]);
        a[s][1] = pack2(F.h2[2 * s][2], F.h2[2 * s][3]);
        a[s][2] = pack2(F.h2[2 * s + 1][0], F.h2[2 * s + 1][1]);
        a[s][3] = pack2(F.h2[2 * s + 1][2], F.h2[2 * s + 1][3]);
    }
    F.o[0] = sm.b3[2 * c]; F.o[1] = sm.b3[2 * c + 1]; F.o[2] = F.o[0]; F.o[3] = F.o[1];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const __nv_bfloat16 *w = sm.w3t + g * kS2 + 16 * s + 2 * c;
        mma16816(F.o, a[s], ld32(w), ld32(w + 8));
    }
}

/* y = net(x) * out_scale * scale into float4 rows (inference in the step) or
 * plain rows of 3 (y3). */
template <int KT>
__global__ void __launch_bounds__(128) k_mlp_infer(const MlpDev *__restrict__ gm, const float *__restrict__ x, int n,
                                                   float4 *__restrict__ y, float *__restrict__ y3, float scale,
                                                   const unsigned int *__restrict__ valid) {
    __shared__ __align__(16) MlpDev sm;
    copy_model(sm, gm);
    __syncthreads();
    const bool ok = valid == nullptr || *valid != 0u;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, c = lane & 3;
    const float k = sm.out_scale * scale;
    const int ntiles = (n + 15) / 16;
    for (int tile = blockIdx.x * 4 + warp; tile < ntiles; tile += gridDim.x * 4) {
        const int base = tile * 16, r0 = base + g, r1 = base + g + 8;
        if (!ok) {
            if (c == 0 && y) {
                if (r0 < n) y[r0] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (r1 < n) y[r1] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            continue;
        }
        Fwd F;
        mlp_forward<KT>(sm, x, n, base, g, c, F);
        const float y2a = __shfl_down_sync(0xffffffffu, F.o[0], 1);
        const float y2b = __shfl_down_sync(0xffffffffu, F.o[2], 1);
        if (c == 0) {
            if (y) {
                if (r0 < n) y[r0] = make_float4(F.o[0] * k, F.o[1] * k, y2a * k, 0.0f);
                if (r1 < n) y[r1] = make_float4(F.o[2] * k, F.o[3] * k, y2b * k, 0.0f);
            } else {
                if (r0 < n) { y3[3 * (size_t)r0] = F.o[0] * k; y3[3 * (size_t)r0 + 1] = F.o[1] * k; y3[3 * (size_t)r0 + 2] = y2a * k; }
                if (r1 < n) { y3[3 * (size_t)r1] = F.o[2] * k; y3[3 * (size_t)r1 + 1] = F.o[3] * k; y3[3 * (size_t)r1 + 2] = y2b * k; }
            }
        }
    }
}

/* --------------------------------------------------------------------- */
/* training                                                              */
/* --------------------------------------------------------------------- */
constexpr int kChunk = 64;            /* samples per block iteration (4 warps x 16) */
constexpr int kSS = kChunk + 8;       /* padded stride of the [feature][sample] staging */
constexpr size_t kGradSmem = sizeof(MlpDev) + (size_t)(kIn + 4 * kHid + 8) * kSS * sizeof(__nv_bfloat16) + 64;

int mlp_grad_blocks(int n) {
    int chunks = (n + kChunk - 1) / kChunk;
    return chunks < 304 ? (chunks > 0 ? chunks : 1) : 304;
}

__global__ void __launch_bounds__(128) k_mlp_grad(const MlpDev *__restrict__ gm, const float *__restrict__ x,
                                                  const float *__restrict__ t, int n, float *__restrict__ part,
                                                  float *__restrict__ loss_part) {
    extern __shared__ __align__(16) unsigned char dsm[];
    MlpDev &sm = *reinterpret_cast<MlpDev *>(dsm);
    __nv_bfloat16 *sx = reinterpret_cast<__nv_bfloat16 *>(dsm + ((sizeof(MlpDev) + 15) & ~(size_t)15));
    __nv_bfloat16 *sh1 = sx + kIn * kSS;
    __nv_bfloat16 *sh2 = sh1 + kHid * kSS;
    __nv_bfloat16 *sd1 = sh2 + kHid * kSS;
    __nv_bfloat16 *sd2 = sd1 + kHid * kSS;
    __nv_bfloat16 *sdy = sd2 + kHid * kSS;
    __shared__ float s_loss[4];
    copy_model(sm, gm);
    __syncthreads();
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, g = lane >> 2, c = lane & 3;
    const float inv_scale = sm.out_scale != 0.0f ? 1.0f / sm.out_scale : 0.0f;
    const float gscale = 2.0f / (float)n;
    float acc2[8][4], acc3[4], acc1[kIn / 16][2][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc2[j][0] = acc2[j][1] = acc2[j][2] = acc2[j][3] = 0.f;
    acc3[0] = acc3[1] = acc3[2] = acc3[3] = 0.f;
#pragma unroll
    for (int mt = 0; mt < kIn / 16; ++mt)
#pragma unroll
        for (int jj = 0; jj < 2; ++jj) acc1[mt][jj][0] = acc1[mt][jj][1] = acc1[mt][jj][2] = acc1[mt][jj][3] = 0.f;
    float db1 = 0.f, db2 = 0.f, db3 = 0.f, loss = 0.f;
    const int nchunks = (n + kChunk - 1) / kChunk;
    for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const int base = ch * kChunk + w * 16;
        const int sl0 = w * 16 + g, sl1 = sl0 + 8; /* sample columns in the staging */
        const int r0 = base + g, r1 = base + g + 8;
        Fwd F;
        mlp_forward(sm, x, n, base, g, c, F);
        /* stage x~, h1, h2 transposed */
#pragma unroll
        for (int kt = 0; kt < kIn / 16; ++kt) {
            const int cols[4] = {16 * kt + 2 * c, 16 * kt + 2 * c + 1, 16 * kt + 2 * c + 8, 16 * kt + 2 * c + 9};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                sx[cols[q] * kSS + sl0] = __float2bfloat16(F.xn[8 * kt + q]);
                sx[cols[q] * kSS + sl1] = __float2bfloat16(F.xn[8 * kt + 4 + q]);
            }
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int f0 = 8 * j + 2 * c;
            sh1[f0 * kSS + sl0] = __float2bfloat16(F.h1[j][0]);
            sh1[(f0 + 1) * kSS + sl0] = __float2bfloat16(F.h1[j][1]);
            sh1[f0 * kSS + sl1] = __float2bfloat16(F.h1[j][2]);
            sh1[(f0 + 1) * kSS + sl1] = __float2bfloat16(F.h1[j][3]);
            sh2[f0 * kSS + sl0] = __float2bfloat16(F.h2[j][0]);
            sh2[(f0 + 1) * kSS + sl0] = __float2bfloat16(F.h2[j][1]);
            sh2[f0 * kSS + sl1] = __float2bfloat16(F.h2[j][2]);
            sh2[(f0 + 1) * kSS + sl1] = __float2bfloat16(F.h2[j][3]);
        }
        /* dL/dy = 2 (y - t / out_scale) / n for the 3 real outputs of real rows */
        float dy[4];
        {
            const int c0 = 2 * c, c1 = 2 * c + 1;
            float t00 = (r0 < n && c0 < kOut) ? __ldg(t + 3 * (size_t)r0 + c0) * inv_scale : 0.f;
            float t01 = (r0 < n && c1 < kOut) ? __ldg(t + 3 * (size_t)r0 + c1) * inv_scale : 0.f;
            float t10 = (r1 < n && c0 < kOut) ? __ldg(t + 3 * (size_t)r1 + c0) * inv_scale : 0.f;
            float t11 = (r1 < n && c1 < kOut) ? __ldg(t + 3 * (size_t)r1 + c1) * inv_scale : 0.f;
            float e00 = (r0 < n && c0 < kOut) ? F.o[0] - t00 : 0.f;
            float e01 = (r0 < n && c1 < kOut) ? F.o[1] - t01 : 0.f;
            float e10 = (r1 < n && c0 < kOut) ? F.o[2] - t10 : 0.f;
            float e11 = (r1 < n && c1 < kOut) ? F.o[3] - t11 : 0.f;
            loss += e00 * e00 + e01 * e01 + e10 * e10 + e11 * e11;
            dy[0] = gscale * e00; dy[1] = gscale * e01; dy[2] = gscale * e10; dy[3] = gscale * e11;
            sdy[c0 * kSS + sl0] = __float2bfloat16(dy[0]);
            sdy[c1 * kSS + sl0] = __float2bfloat16(dy[1]);
            sdy[c0 * kSS + sl1] = __float2bfloat16(dy[2]);
            sdy[c1 * kSS + sl1] = __float2bfloat16(dy[3]);
        }
        /* dH2 = (dY W3^T) * relu'(H2); dY padded to K = 16 */
        unsigned ady[4] = {pack2(dy[0], dy[1]), pack2(dy[2], dy[3]), 0u, 0u};
        float d2[8][4];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            d2[j][0] = d2[j][1] = d2[j][2] = d2[j][3] = 0.f;
            const __nv_bfloat16 *wp = sm.w3 + (8 * j + g) * kS3 + 2 * c;
            mma16816(d2[j], ady, ld32(wp), ld32(wp + 8));
#pragma unroll
            for (int e = 0; e < 4; ++e) d2[j][e] = F.h2[j][e] > 0.f ? d2[j][e] : 0.f;
            const int f0 = 8 * j + 2 * c;
            sd2[f0 * kSS + sl0] = __float2bfloat16(d2[j][0]);
            sd2[(f0 + 1) * kSS + sl0] = __float2bfloat16(d2[j][1]);
            sd2[f0 * kSS + sl1] = __float2bfloat16(d2[j][2]);
            sd2[(f0 + 1) * kSS + sl1] = __float2bfloat16(d2[j][3]);
        }
        /* dH1 = (dH2 W2^T) * relu'(H1) */
        {
            unsigned a[4][4];
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                a[s][0] = pack2(d2[2 * s][0], d2[2 * s][1]);
                a[s][1] = pack2(d2[2 * s][2], d2[2 * s][3]);
                a[s][2] = pack2(d2[2 * s + 1][0], d2[2 * s + 1][1]);
                a[s][3] = pack2(d2[2 * s + 1][2], d2[2 * s + 1][3]);
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                float d1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    const __nv_bfloat16 *wp = sm.w2 + (8 * j + g) * kS2 + 16 * s + 2 * c;
                    mma16816(d1, a[s], ld32(wp), ld32(wp + 8));
                }
#pragma unroll
                for (int e = 0; e < 4; ++e) d1[e] = F.h1[j][e] > 0.f ? d1[e] : 0.f;
                const int f0 = 8 * j + 2 * c;
                sd1[f0 * kSS + sl0] = __float2bfloat16(d1[0]);
                sd1[(f0 + 1) * kSS + sl0] = __float2bfloat16(d1[1]);
                sd1[f0 * kSS + sl1] = __float2bfloat16(d1[2]);
                sd1[(f0 + 1) * kSS + sl1] = __float2bfloat16(d1[3]);
            }
        }
        __syncthreads();
        /* weight gradients of the chunk: K = the 64 samples, 4 k-steps.
         * warp w owns dW2 rows 16w..16w+15, dW3 rows 16w.., dW1 columns 16w.. */
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
            const int k0 = 16 * ks + 2 * c;
            unsigned ah1[4] = {ld32(sh1 + (16 * w + g) * kSS + k0), ld32(sh1 + (16 * w + g + 8) * kSS + k0),
                               ld32(sh1 + (16 * w + g) * kSS + k0 + 8), ld32(sh1 + (16 * w + g + 8) * kSS + k0 + 8)};
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const __nv_bfloat16 *bp = sd2 + (8 * j + g) * kSS + k0;
                mma16816(acc2[j], ah1, ld32(bp), ld32(bp + 8));
            }
            unsigned ah2[4] = {ld32(sh2 + (16 * w + g) * kSS + k0), ld32(sh2 + (16 * w + g + 8) * kSS + k0),
                               ld32(sh2 + (16 * w + g) * kSS + k0 + 8), ld32(sh2 + (16 * w + g + 8) * kSS + k0 + 8)};
            {
                const __nv_bfloat16 *bp = sdy + g * kSS + k0;
                mma16816(acc3, ah2, ld32(bp), ld32(bp + 8));
            }
#pragma unroll
            for (int mt = 0; mt < kIn / 16; ++mt) {
                const __nv_bfloat16 *xr = sx + 16 * mt * kSS;
                unsigned axx[4] = {ld32(xr + g * kSS + k0), ld32(xr + (g + 8) * kSS + k0),
                                   ld32(xr + g * kSS + k0 + 8), ld32(xr + (g + 8) * kSS + k0 + 8)};
#pragma unroll
                for (int jj = 0; jj < 2; ++jj) {
                    const __nv_bfloat16 *bp = sd1 + (8 * (2 * w + jj) + g) * kSS + k0;
                    mma16816(acc1[mt][jj], axx, ld32(bp), ld32(bp + 8));
                }
            }
        }
        if (tid < kHid) {
            for (int s = 0; s < kChunk; ++s) {
                db1 += __bfloat162float(sd1[tid * kSS + s]);
                db2 += __bfloat162float(sd2[tid * kSS + s]);
            }
        }
        if (tid < kOut)
            for (int s = 0; s < kChunk; ++s) db3 += __bfloat162float(sdy[tid * kSS + s]);
        __syncthreads();
    }
    /* this block's partial gradient, blob layout */
    float *P = part + (size_t)blockIdx.x * kBlob;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int m0 = 16 * w + g, n0 = 8 * j + 2 * c;
        P[kBW2 + m0 * kHid + n0] = acc2[j][0];
        P[kBW2 + m0 * kHid + n0 + 1] = acc2[j][1];
        P[kBW2 + (m0 + 8) * kHid + n0] = acc2[j][2];
        P[kBW2 + (m0 + 8) * kHid + n0 + 1] = acc2[j][3];
    }
    {
        const int m0 = 16 * w + g, n0 = 2 * c;
        if (n0 < kOut) { P[kBW3 + m0 * kOut + n0] = acc3[0]; P[kBW3 + (m0 + 8) * kOut + n0] = acc3[2]; }
        if (n0 + 1 < kOut) { P[kBW3 + m0 * kOut + n0 + 1] = acc3[1]; P[kBW3 + (m0 + 8) * kOut + n0 + 1] = acc3[3]; }
    }
#pragma unroll
    for (int mt = 0; mt < kIn / 16; ++mt)
#pragma unroll
        for (int jj = 0; jj < 2; ++jj) {
            const int n0 = 8 * (2 * w + jj) + 2 * c, m0 = 16 * mt + g;
            P[kBW1 + m0 * kHid + n0] = acc1[mt][jj][0];
            P[kBW1 + m0 * kHid + n0 + 1] = acc1[mt][jj][1];
            P[kBW1 + (m0 + 8) * kHid + n0] = acc1[mt][jj][2];
            P[kBW1 + (m0 + 8) * kHid + n0 + 1] = acc1[mt][jj][3];
        }
    if (tid < kHid) { P[kBB1 + tid] = db1; P[kBB2 + tid] = db2; }
    if (tid < kOut) P[kBB3 + tid] = db3;
    if (tid < kBW1) P[tid] = 0.0f;
    if (tid == 0) P[kBScale] = 0.0f;
    loss = warp_sum(loss);
    if (lane == 0) s_loss[w] = loss;
    __syncthreads();
    if (tid == 0) loss_part[blockIdx.x] = s_loss[0] + s_loss[1] + s_loss[2] + s_loss[3];
}

__global__ void k_mlp_reduce(const float *__restrict__ part, const float *__restrict__ loss_part, int nblocks, int n,
                             float *__restrict__ grad, float *__restrict__ loss) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < kBlob) {
        float s = 0.f;
        for (int b = 0; b < nblocks; ++b) s += part[(size_t)b * kBlob + e];
        grad[e] = s;
    }
    if (e == 0 && loss) {
        double s = 0.0;
        for (int b = 0; b < nblocks; ++b) s += loss_part[b];
        *loss = (float)(s / (double)(n > 0 ? n : 1));
    }
}

__global__ void k_mlp_adam(float *__restrict__ w, float *__restrict__ m1, float *__restrict__ m2,
                           const float *__restrict__ grad, float lr, float b1, float b2, float eps, float c1,
                           float c2) {
    int e = kTrainFirst + blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kTrainLast) return;
    float gr = grad[e];
    float a = b1 * m1[e] + (1.0f - b1) * gr;
    float v = b2 * m2[e] + (1.0f - b2) * gr * gr;
    m1[e] = a;
    m2[e] = v;
    w[e] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
}

/* --------------------------------------------------------------------- */
void launch_mlp_pack(const float *blob, MlpDev *dev, cudaStream_t s) { k_mlp_pack<<<1, 256, 0, s>>>(blob, dev); }

static unsigned int infer_blocks(int n) {
    unsigned int tiles = (unsigned int)((n + 15) / 16);
    unsigned int b = (tiles + 3) / 4;
    return b < 1216u ? (b > 0 ? b : 1u) : 1216u;
}

void launch_mlp_infer(const MlpDev *m, const float *x, int n, float4 *y, float scale, const unsigned int *valid,
                      cudaStream_t s, bool local_only) {
    auto k = local_only ? k_mlp_infer<1> : k_mlp_infer<kIn / 16>;
    k<<<infer_blocks(n), 128, 0, s>>>(m, x, n, y, nullptr, scale, valid);
}
void launch_mlp_forward3(const MlpDev *m, const float *x, int n, float *y, cudaStream_t s) {
    k_mlp_infer<kIn / 16><<<infer_blocks(n), 128, 0, s>>>(m, x, n, nullptr, y, 1.0f, nullptr);
}
void launch_mlp_grad(const MlpDev *m, const float *x, const float *t, int n, float *part, float *loss_part,
                     cudaStream_t s) {
    static const bool attr = [] { /* set once, thread-safely */
        cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem);
        return true;
    }();
    (void)attr;
    k_mlp_grad<<<mlp_grad_blocks(n), 128, kGradSmem, s>>>(m, x, t, n, part, loss_part);
}
void launch_mlp_reduce(const float *part, const float *loss_part, int nblocks, int n, float *grad, float *loss,
                       cudaStream_t s) {
    k_mlp_reduce<<<(kBlob + 255) / 256, 256, 0, s>>>(part, loss_part, nblocks, n, grad, loss);
}
void launch_mlp_adam(float *blob, float *m1, float *m2, const float *grad, float lr, float b1, float b2, float eps,
                     int step, cudaStream_t s) {
    float c1 = 1.0f - std::pow(b1, (float)step), c2 = 1.0f - std::pow(b2, (float)step);
    int cnt = kTrainLast - kTrainFirst;
    k_mlp_adam<<<(cnt + 255) / 256, 256, 0, s>>>(blob, m1, m2, grad, lr, b1, b2, eps, c1, c2);
}

}  // namespace fsph

/* ======================================================================== */
/* fsph_mlp C ABI                                                           */
/* ======================================================================== */
using namespace fsph;

struct fsph_mlp {
    MlpDev *dev = nullptr;
    float *blob = nullptr, *m1 = nullptr, *m2 = nullptr, *grad = nullptr;
    float *part = nullptr, *loss_part = nullptr, *loss = nullptr;
    int part_blocks = 0;
    int step = 0;
    unsigned int *tc_err = nullptr; /* set by the tcgen05 forward when a wait ran out */
    cudaStream_t stream = nullptr;
    std::string err;
};

namespace {
int mlp_fail(fsph_mlp *m, cudaError_t e, const char *what) {
    if (m) m->err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? FSPH_OOM : FSPH_CUDA_ERROR;
}
#define MLP_CUDA(m, call)                                     \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return mlp_fail(m, e_, #call); \
    } while (0)

int ensure_part(fsph_mlp *m, int n) {
    int nb = mlp_grad_blocks(n);
    if (nb <= m->part_blocks) return FSPH_OK;
    cudaFree(m->part);
    cudaFree(m->loss_part);
    m->part = nullptr;
    m->loss_part = nullptr;
    MLP_CUDA(m, cudaMalloc((void **)&m->part, (size_t)nb * kBlob * sizeof(float)));
    MLP_CUDA(m, cudaMalloc((void **)&m->loss_part, (size_t)nb * sizeof(float)));
    m->part_blocks = nb;
    return FSPH_OK;
}
}  // namespace

extern "C" {

int fsph_mlp_create(fsph_mlp **out) {
    if (!out) return FSPH_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return FSPH_NO_DEVICE;
    }
    fsph_mlp *m = new (std::nothrow) fsph_mlp();
    if (!m) return FSPH_OOM;
    auto bail = [&](int st) { fsph_mlp_destroy(m); return st; };
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(FSPH_CUDA_ERROR);
    if (cudaMalloc((void **)&m->dev, sizeof(MlpDev)) != cudaSuccess) return bail(FSPH_OOM);
    for (float **p : {&m->blob, &m->m1, &m->m2, &m->grad})
        if (cudaMalloc((void **)p, kBlob * sizeof(float)) != cudaSuccess) return bail(FSPH_OOM);
    if (cudaMalloc((void **)&m->loss, sizeof(float)) != cudaSuccess) return bail(FSPH_OOM);
    if (cudaMalloc((void **)&m->tc_err, sizeof(unsigned int)) != cudaSuccess) return bail(FSPH_OOM);
    cudaMemsetAsync(m->tc_err, 0, sizeof(unsigned int), m->stream);
    cudaMemsetAsync(m->blob, 0, kBlob * sizeof(float), m->stream);
    cudaMemsetAsync(m->m1, 0, kBlob * sizeof(float), m->stream);
    cudaMemsetAsync(m->m2, 0, kBlob * sizeof(float), m->stream);
    launch_mlp_pack(m->blob, m->dev, m->stream);
    if (cudaStreamSynchronize(m->stream) != cudaSuccess) return bail(FSPH_CUDA_ERROR);
    *out = m;
    return FSPH_OK;
}

int fsph_mlp_destroy(fsph_mlp *m) {
    if (!m) return FSPH_INVALID_ARG;
    if (m->stream) cudaStreamSynchronize(m->stream);
    cudaFree(m->dev);
    cudaFree(m->blob); cudaFree(m->m1); cudaFree(m->m2); cudaFree(m->grad);
    cudaFree(m->part); cudaFree(m->loss_part); cudaFree(m->loss); cudaFree(m->tc_err);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return FSPH_OK;
}

int fsph_mlp_set_blob(fsph_mlp *m, const float *blob) {
    if (!m || !blob) return FSPH_INVALID_ARG;
    MLP_CUDA(m, cudaMemcpyAsync(m->blob, blob, kBlob * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MLP_CUDA(m, cudaMemsetAsync(m->m1, 0, kBlob * sizeof(float), m->stream));
    MLP_CUDA(m, cudaMemsetAsync(m->m2, 0, kBlob * sizeof(float), m->stream));
    m->step = 0;
    launch_mlp_pack(m->blob, m->dev, m->stream);
    MLP_CUDA(m, cudaStreamSynchronize(m->stream));
    return FSPH_OK;
}

int fsph_mlp_get_blob(fsph_mlp *m, float *blob) {
    if (!m || !blob) return FSPH_INVALID_ARG;
    MLP_CUDA(m, cudaMemcpyAsync(blob, m->blob, kBlob * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MLP_CUDA(m, cudaStreamSynchronize(m->stream));
    return FSPH_OK;
}

int fsph_mlp_forward(fsph_mlp *m, const float *x, int n, float *y, void *stream) {
    if (!m || n < 0 || (n > 0 && (!x || !y))) return FSPH_INVALID_ARG;
    if (n == 0) return FSPH_OK;
    cudaStream_t s = stream ? (cudaStream_t)stream : m->stream;
    launch_mlp_forward3(m->dev, x, n, y, s);
    MLP_CUDA(m, cudaGetLastError());
    if (!stream) MLP_CUDA(m, cudaStreamSynchronize(s));
    return FSPH_OK;
}

int fsph_mlp_forward_tcgen05(fsph_mlp *m, const float *x, int n, float *y) {
    if (!m || n < 0 || (n > 0 && (!x || !y))) return FSPH_INVALID_ARG;
    if (n == 0) return FSPH_OK;
    cudaStream_t s = m->stream;
    MLP_CUDA(m, cudaMemsetAsync(m->tc_err, 0, sizeof(unsigned int), s));
    launch_mlp_forward3_tc(m->dev, x, n, y, m->tc_err, s);
    MLP_CUDA(m, cudaGetLastError());
    unsigned int e = 0;
    MLP_CUDA(m, cudaMemcpyAsync(&e, m->tc_err, sizeof(e), cudaMemcpyDeviceToHost, s));
    MLP_CUDA(m, cudaStreamSynchronize(s));
    if (e) {
        m->err = "tcgen05 forward: a wait on an MMA ran out";
        return FSPH_TIMEOUT;
    }
    return FSPH_OK;
}

int fsph_mlp_gradient(fsph_mlp *m, const float *x, const float *t, int n, float *grad, float *loss) {
    if (!m || n <= 0 || !x || !t || !grad) return FSPH_INVALID_ARG;
    int st = ensure_part(m, n);
    if (st != FSPH_OK) return st;
    int nb = mlp_grad_blocks(n);
    launch_mlp_grad(m->dev, x, t, n, m->part, m->loss_part, m->stream);
    launch_mlp_reduce(m->part, m->loss_part, nb, n, m->grad, m->loss, m->stream);
    MLP_CUDA(m, cudaGetLastError());
    MLP_CUDA(m, cudaMemcpyAsync(grad, m->grad, kBlob * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    float l = 0.f;
    MLP_CUDA(m, cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MLP_CUDA(m, cudaStreamSynchronize(m->stream));
    if (loss) *loss = l;
    return FSPH_OK;
}

int fsph_mlp_train(fsph_mlp *m, const float *x, const float *t, int n, int batch, int epochs, float lr,
                   float *loss_per_epoch) {
    if (!m || !x || !t || n <= 0 || batch <= 0 || epochs <= 0 || !(lr > 0.0f)) return FSPH_INVALID_ARG;
    if (batch > n) batch = n;
    int st = ensure_part(m, batch);
    if (st != FSPH_OK) return st;
    const int nbatches = n / batch;
    std::vector<float> losses((size_t)nbatches);
    float *dloss = nullptr;
    MLP_CUDA(m, cudaMalloc((void **)&dloss, (size_t)nbatches * sizeof(float)));
    for (int ep = 0; ep < epochs; ++ep) {
        for (int b = 0; b < nbatches; ++b) {
            const float *xb = x + (size_t)b * batch * kIn;
            const float *tb = t + (size_t)b * batch * 3;
            const int nb = mlp_grad_blocks(batch);
            launch_mlp_grad(m->dev, xb, tb, batch, m->part, m->loss_part, m->stream);
            launch_mlp_reduce(m->part, m->loss_part, nb, batch, m->grad, dloss + b, m->stream);
            m->step += 1;
            launch_mlp_adam(m->blob, m->m1, m->m2, m->grad, lr, 0.9f, 0.999f, 1e-8f, m->step, m->stream);
            launch_mlp_pack(m->blob, m->dev, m->stream);
        }
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(losses.data(), dloss, (size_t)nbatches * sizeof(float), cudaMemcpyDeviceToHost,
                                m->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
        if (e != cudaSuccess) {
            cudaFree(dloss);
            return mlp_fail(m, e, "training epoch");
        }
        if (loss_per_epoch) {
            double s = 0.0;
            for (float l : losses) s += l;
            loss_per_epoch[ep] = (float)(s / (double)(nbatches > 0 ? nbatches : 1));
        }
    }
    cudaFree(dloss);
    return FSPH_OK;
}

const char *fsph_mlp_last_error(const fsph_mlp *m) { return m ? m->err.c_str() : "null network"; }

}  // extern "C"
