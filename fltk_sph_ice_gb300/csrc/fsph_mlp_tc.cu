/*
 * fsph_mlp_tc.cu -- warm-start network inference on the fifth-generation
 * tensor cores: tcgen05.mma with both operands in shared memory and the FP32
 * accumulators in tensor memory (TMEM), read back with tcgen05.ld for the
 * bias / ReLU / BF16 epilogue that stages the next layer's operand.
 *
 * The same network and rounding points as k_mlp_infer (fsph_mlp.cu): inputs
 * normalised in FP32 and rounded to BF16, each layer accumulated in FP32,
 * hidden activations rounded to BF16; the accumulation order inside an MMA
 * may differ, so results agree to FP32 rounding, not bit for bit.
 *
 * One CTA = one warpgroup (128 threads); a tile = 128 particles = the MMA's
 * M; thread t owns row t of the tile (TMEM lane t).  Per tile:
 *   features -> BF16 A1 [128 x 32]          (smem, all threads)
 *   MMA 1: A1 x W1^T -> TMEM cols [0, 64)    (one thread, 2 x K16)
 *   epilogue 1: +b1, ReLU -> BF16 A2 [128 x 64]
 *   MMA 2: A2 x W2^T -> TMEM cols [64, 128)  (4 x K16)
 *   epilogue 2: +b2, ReLU -> BF16 A2 (A2 free once MMA 2 has completed)
 *   MMA 3: A2 x W3^T (N padded 3 -> 16) -> TMEM cols [0, 16)
 *   epilogue 3: +b3, x out_scale x scale -> y
 * Operands use the canonical K-major layout without swizzle: 8-row x 16-byte
 * core matrices, 128 B apart along K (the leading byte offset) and K / 8 x
 * 128 B apart between 8-row groups (the stride byte offset); all buffers sit
 * in one shared-memory block.  Every wait on an MMA's completion is bounded;
 * a wait that runs out sets *err, the CTA stops, waits (bounded) once more for
 * its MMAs and frees its TMEM.
 */
#include <cuda.h>

#include <cstdint>
#include <cstring>

#include "fsph_mlp.cuh"

namespace fsph {

namespace {

constexpr int kTcRows = 128;
constexpr int kTcThreads = 128;
constexpr uint32_t kTmemCols = 128;
constexpr int kA1Bytes = kTcRows * kIn * 2;   /* 128 x 32 BF16 */
constexpr int kA2Bytes = kTcRows * kHid * 2;  /* 128 x 64 BF16 */
constexpr int kB1Bytes = kHid * kIn * 2;      /* W1^T: 64 x 32 */
constexpr int kB2Bytes = kHid * kHid * 2;     /* W2^T: 64 x 64 */
constexpr int kN3 = 16;                       /* layer 3's N: 3 outputs padded to the MMA minimum */
constexpr int kB3Bytes = kN3 * kHid * 2;      /* W3^T: 16 x 64 */
constexpr uint32_t kSpinLimit = 1u << 22;     /* ~0.1-1 s of polling before an MMA wait gives up */

struct __align__(128) TcSmem {
    unsigned char a1[kA1Bytes];
    unsigned char a2[kA2Bytes];
    unsigned char b1[kB1Bytes];
    unsigned char b2[kB2Bytes];
    unsigned char b3[kB3Bytes];
    float bias1[kHid], bias2[kHid], bias3[8];
    float mu[kIn], isig[kIn];
    unsigned long long mbar;
    uint32_t tmem;
    uint32_t fail;
};

/* byte offset of (row, 8-element chunk kc) in a K-major no-swizzle image with K columns */
__device__ __forceinline__ uint32_t kmaj(int row, int kc, int K) {
    return (uint32_t)((row >> 3) * (K / 8) * 128 + kc * 128 + (row & 7) * 16);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

/* shared-memory matrix descriptor: start, leading and stride byte offsets
 * (each >> 4, 14 bits), the descriptor version 1 at bit 46, no swizzle */
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
           ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}

/* instruction descriptor, kind::f16: D = F32 (bits 4-5), A = B = BF16 (bits
 * 7-9, 10-12), both K-major, N >> 3 at bit 17, M >> 4 at bit 24 */
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

/* bounded wait for the completion of the mbarrier phase with this parity */
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (uint32_t it = 0; it < kSpinLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
        if (it > 32) __nanosleep(64);
    }
    return false;
}

/* 16 consecutive FP32 columns of this thread's TMEM lane */
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ uint32_t bf2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

/* epilogue of a hidden layer: 64 accumulator columns from col0, + bias, ReLU,
 * BF16 into row `row` of the K = 64 operand image */
__device__ __forceinline__ void hidden_epilogue(uint32_t tlane, uint32_t col0, const float *bias, unsigned char *img,
                                                int row) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        float v[16];
        tmem_ld16(tlane + col0 + 16 * q, v);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            uint4 w;
            const float *b = bias + 16 * q + 8 * h;
            const float *x = v + 8 * h;
            w.x = bf2(fmaxf(x[0] + b[0], 0.0f), fmaxf(x[1] + b[1], 0.0f));
            w.y = bf2(fmaxf(x[2] + b[2], 0.0f), fmaxf(x[3] + b[3], 0.0f));
            w.z = bf2(fmaxf(x[4] + b[4], 0.0f), fmaxf(x[5] + b[5], 0.0f));
            w.w = bf2(fmaxf(x[6] + b[6], 0.0f), fmaxf(x[7] + b[7], 0.0f));
            *reinterpret_cast<uint4 *>(img + kmaj(row, 2 * q + h, kHid)) = w;
        }
    }
}

/* KT: the 16-wide input tiles read (1 for a network that weights only the
 * first 16 inputs, whose other inputs the step does not compute) */
template <int KT>
__global__ void __launch_bounds__(kTcThreads) k_mlp_infer_tc(const MlpDev *__restrict__ gm, const float *__restrict__ x,
                                                             int n, float4 *__restrict__ y, float *__restrict__ y3,
                                                             float scale, const unsigned int *__restrict__ valid,
                                                             unsigned int *__restrict__ err) {
    __shared__ TcSmem S;
    const int t = threadIdx.x, warp = t >> 5;
    const int ntiles = (n + kTcRows - 1) / kTcRows;
    const bool ok = valid == nullptr || *valid != 0u;
    if (!ok) { /* no features yet: zero corrections */
        for (int r = blockIdx.x * kTcThreads + t; r < n; r += gridDim.x * kTcThreads) {
            if (y) y[r] = make_float4(0.f, 0.f, 0.f, 0.f);
            else { y3[3 * (size_t)r] = 0.f; y3[3 * (size_t)r + 1] = 0.f; y3[3 * (size_t)r + 2] = 0.f; }
        }
        return;
    }
    /* the weights as K-major operand images, biases and normalisation */
    for (int e = t; e < kHid * (kIn / 8); e += kTcThreads) { /* W1^T: row n = hidden unit, K = inputs */
        const int nr = e / (kIn / 8), kc = e % (kIn / 8);
        *reinterpret_cast<uint4 *>(S.b1 + kmaj(nr, kc, kIn)) =
            *reinterpret_cast<const uint4 *>(gm->w1t + nr * kS1 + 8 * kc);
    }
    for (int e = t; e < kHid * (kHid / 8); e += kTcThreads) {
        const int nr = e / (kHid / 8), kc = e % (kHid / 8);
        *reinterpret_cast<uint4 *>(S.b2 + kmaj(nr, kc, kHid)) =
            *reinterpret_cast<const uint4 *>(gm->w2t + nr * kS2 + 8 * kc);
    }
    for (int e = t; e < kN3 * (kHid / 8); e += kTcThreads) {
        const int nr = e / (kHid / 8), kc = e % (kHid / 8);
        *reinterpret_cast<uint4 *>(S.b3 + kmaj(nr, kc, kHid)) =
            nr < 8 ? *reinterpret_cast<const uint4 *>(gm->w3t + nr * kS2 + 8 * kc) : make_uint4(0u, 0u, 0u, 0u);
    }
    for (int e = t; e < kHid; e += kTcThreads) {
        S.bias1[e] = gm->b1[e];
        S.bias2[e] = gm->b2[e];
    }
    if (t < 8) S.bias3[t] = gm->b3[t];
    if (t < kIn) {
        S.mu[t] = gm->mu[t];
        S.isig[t] = gm->isig[t];
    }
    const uint32_t mbar = smem_u32(&S.mbar);
    if (t == 0) {
        S.fail = 0u;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) { /* 128 TMEM columns for this CTA */
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = S.tmem;
    const uint32_t tlane = tmem + ((uint32_t)(warp * 32) << 16); /* this warp's 32 TMEM lanes */
    const float k = gm->out_scale * scale;
    const uint32_t a1 = smem_u32(S.a1), a2 = smem_u32(S.a2);
    const uint32_t b1 = smem_u32(S.b1), b2 = smem_u32(S.b2), b3 = smem_u32(S.b3);
    uint32_t phase = 0;
    bool failed = false;
    /* this row's raw inputs of the coming tile: loaded while the previous
     * tile's MMAs run */
    float4 in[4 * KT];
    auto fetch = [&](int tile) {
        const int r = tile * kTcRows + t;
#pragma unroll
        for (int q = 0; q < 4 * KT; ++q)
            in[q] = (tile < ntiles && r < n) ? __ldg(reinterpret_cast<const float4 *>(x + (size_t)r * kIn) + q)
                                             : make_float4(0.f, 0.f, 0.f, 0.f);
    };
    fetch(blockIdx.x);
    for (int tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        const int row = tile * kTcRows + t;
        /* layer 1 operand: the normalised inputs of this row, BF16 */
#pragma unroll
        for (int kc = 0; kc < kIn / 8; ++kc) {
            float v[8];
            if (row < n && kc < 2 * KT) {
                const float4 p0 = in[2 * kc], p1 = in[2 * kc + 1];
                const float raw[8] = {p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w};
#pragma unroll
                for (int e = 0; e < 8; ++e) v[e] = (raw[e] - S.mu[8 * kc + e]) * S.isig[8 * kc + e];
            } else {
#pragma unroll
                for (int e = 0; e < 8; ++e) v[e] = 0.0f;
            }
            uint4 w;
            w.x = bf2(v[0], v[1]);
            w.y = bf2(v[2], v[3]);
            w.z = bf2(v[4], v[5]);
            w.w = bf2(v[6], v[7]);
            *reinterpret_cast<uint4 *>(S.a1 + kmaj(t, kc, kIn)) = w;
        }
        fence_proxy_async();
        fence_before();
        __syncthreads();
        fence_after();
        if (t == 0) {
#pragma unroll
            for (int ks = 0; ks < KT; ++ks)
                mma_bf16(tmem, sdesc(a1 + 256 * ks, 128, 128 * (kIn / 8)), sdesc(b1 + 256 * ks, 128, 128 * (kIn / 8)),
                         idesc_bf16(kTcRows, kHid), ks > 0);
            mma_commit(mbar);
        }
        fetch(tile + gridDim.x);
        failed = __syncthreads_or(!mbar_wait(mbar, phase)) != 0;
        phase ^= 1u;
        if (failed) break;
        fence_after();
        hidden_epilogue(tlane, 0, S.bias1, S.a2, t);
        fence_proxy_async();
        fence_before();
        __syncthreads();
        fence_after();
        if (t == 0) {
#pragma unroll
            for (int ks = 0; ks < kHid / 16; ++ks)
                mma_bf16(tmem + 64, sdesc(a2 + 256 * ks, 128, 128 * (kHid / 8)),
                         sdesc(b2 + 256 * ks, 128, 128 * (kHid / 8)), idesc_bf16(kTcRows, kHid), ks > 0);
            mma_commit(mbar);
        }
        failed = __syncthreads_or(!mbar_wait(mbar, phase)) != 0;
        phase ^= 1u;
        if (failed) break;
        fence_after();
        hidden_epilogue(tlane, 64, S.bias2, S.a2, t);
        fence_proxy_async();
        fence_before();
        __syncthreads();
        fence_after();
        if (t == 0) {
#pragma unroll
            for (int ks = 0; ks < kHid / 16; ++ks)
                mma_bf16(tmem, sdesc(a2 + 256 * ks, 128, 128 * (kHid / 8)), sdesc(b3 + 256 * ks, 128, 128 * (kHid / 8)),
                         idesc_bf16(kTcRows, kN3), ks > 0);
            mma_commit(mbar);
        }
        failed = __syncthreads_or(!mbar_wait(mbar, phase)) != 0;
        phase ^= 1u;
        if (failed) break;
        fence_after();
        float o[16];
        tmem_ld16(tlane, o);
        if (row < n) {
            const float r0 = (o[0] + S.bias3[0]) * k, r1 = (o[1] + S.bias3[1]) * k, r2 = (o[2] + S.bias3[2]) * k;
            if (y) y[row] = make_float4(r0, r1, r2, 0.0f);
            else { y3[3 * (size_t)row] = r0; y3[3 * (size_t)row + 1] = r1; y3[3 * (size_t)row + 2] = r2; }
        }
        fence_before();
        __syncthreads(); /* TMEM and A1 / A2 free for the next tile */
        fence_after();
    }
    if (failed) {
        if (t == 0) {
            atomicOr(err, 1u);
            mbar_wait(mbar, phase ^ 1u); /* the phase that did not complete in time, once more */
        }
        __syncthreads();
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

/* ---- the 16 local inputs of a tile by TMA (cp.async.bulk.tensor) ---- */

constexpr int kTmaCols = 16;                                   /* features 0-15: one 64-byte row segment */
constexpr uint32_t kTmaBytes = kTcRows * kTmaCols * 4;         /* one 128 x 16 FP32 box = 8 KB */

__device__ __forceinline__ void mbar_init(uint32_t mbar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
}
/* one thread: expect kTmaBytes on xbar and load the 128 x 16 box at rows
 * [row0, row0 + 128), features [0, 16); rows past n read as zeros */
__device__ __forceinline__ void tma_load_tile(const CUtensorMap *tmap, uint32_t dst, uint32_t xbar, int row0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(xbar), "r"(kTmaBytes) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(tmap)), "r"(0), "r"(row0), "r"(xbar)
        : "memory");
}

/* k_mlp_infer_tc<1> with the tile's inputs brought into shared memory by the
 * tensor-memory accelerator: the next tile's box is requested as soon as the
 * current one has been converted, and lands while this tile's three MMAs and
 * epilogues run.  Each row reads exactly its 64 used bytes (the feature rows
 * are 128 bytes apart).  Same arithmetic as k_mlp_infer_tc<1>, so the same
 * results bit for bit. */
__global__ void __launch_bounds__(kTcThreads) k_mlp_infer_tma(const MlpDev *__restrict__ gm,
                                                              const __grid_constant__ CUtensorMap tmap, int n,
                                                              float4 *__restrict__ y, float scale,
                                                              const unsigned int *__restrict__ valid,
                                                              unsigned int *__restrict__ err) {
    __shared__ TcSmem S;
    __shared__ __align__(128) float xs[kTcRows * kTmaCols];
    __shared__ __align__(8) unsigned long long xbar_word;
    const int t = threadIdx.x, warp = t >> 5;
    const int ntiles = (n + kTcRows - 1) / kTcRows;
    const bool ok = valid == nullptr || *valid != 0u;
    if (!ok) {
        for (int r = blockIdx.x * kTcThreads + t; r < n; r += gridDim.x * kTcThreads)
            y[r] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    for (int e = t; e < kHid * (kIn / 8); e += kTcThreads) {
        const int nr = e / (kIn / 8), kc = e % (kIn / 8);
        *reinterpret_cast<uint4 *>(S.b1 + kmaj(nr, kc, kIn)) =
            *reinterpret_cast<const uint4 *>(gm->w1t + nr * kS1 + 8 * kc);
    }
    for (int e = t; e < kHid * (kHid / 8); e += kTcThreads) {
        const int nr = e / (kHid / 8), kc = e % (kHid / 8);
        *reinterpret_cast<uint4 *>(S.b2 + kmaj(nr, kc, kHid)) =
            *reinterpret_cast<const uint4 *>(gm->w2t + nr * kS2 + 8 * kc);
    }
    for (int e = t; e < kN3 * (kHid / 8); e += kTcThreads) {
        const int nr = e / (kHid / 8), kc = e % (kHid / 8);
        *reinterpret_cast<uint4 *>(S.b3 + kmaj(nr, kc, kHid)) =
            nr < 8 ? *reinterpret_cast<const uint4 *>(gm->w3t + nr * kS2 + 8 * kc) : make_uint4(0u, 0u, 0u, 0u);
    }
    for (int e = t; e < kHid; e += kTcThreads) {
        S.bias1[e] = gm->b1[e];
        S.bias2[e] = gm->b2[e];
    }
    if (t < 8) S.bias3[t] = gm->b3[t];
    if (t < kIn) {
        S.mu[t] = gm->mu[t];
        S.isig[t] = gm->isig[t];
    }
    const uint32_t mbar = smem_u32(&S.mbar), xbar = smem_u32(&xbar_word), xdst = smem_u32(xs);
    if (t == 0) {
        S.fail = 0u;
        mbar_init(mbar);
        mbar_init(xbar);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = S.tmem;
    const uint32_t tlane = tmem + ((uint32_t)(warp * 32) << 16);
    const float k = gm->out_scale * scale;
    const uint32_t a1 = smem_u32(S.a1), a2 = smem_u32(S.a2);
    const uint32_t b1 = smem_u32(S.b1), b2 = smem_u32(S.b2), b3 = smem_u32(S.b3);
    uint32_t phase = 0, xphase = 0;
    bool failed = false, loading = false; /* loading: a box is in flight towards xs */
    if ((int)blockIdx.x < ntiles) {
        if (t == 0) tma_load_tile(&tmap, xdst, xbar, blockIdx.x * kTcRows);
        loading = true;
    }
    for (int tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        const int row = tile * kTcRows + t;
        /* this tile's inputs have landed */
        failed = __syncthreads_or(!mbar_wait(xbar, xphase)) != 0;
        if (failed) break;
        xphase ^= 1u;
        loading = false;
#pragma unroll
        for (int kc = 0; kc < kIn / 8; ++kc) {
            float v[8];
            if (row < n && kc < kTmaCols / 8) {
                const float4 p0 = *reinterpret_cast<const float4 *>(xs + t * kTmaCols + 8 * kc);
                const float4 p1 = *reinterpret_cast<const float4 *>(xs + t * kTmaCols + 8 * kc + 4);
                const float raw[8] = {p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w};
#pragma unroll
                for (int e = 0; e < 8; ++e) v[e] = (raw[e] - S.mu[8 * kc + e]) * S.isig[8 * kc + e];
            } else {
#pragma unroll
                for (int e = 0; e < 8; ++e) v[e] = 0.0f;
            }
            uint4 w;
            w.x = bf2(v[0], v[1]);
            w.y = bf2(v[2], v[3]);
            w.z = bf2(v[4], v[5]);
            w.w = bf2(v[6], v[7]);
            *reinterpret_cast<uint4 *>(S.a1 + kmaj(t, kc, kIn)) = w;
        }
        fence_proxy_async(); /* A1 for the MMA, and xs free for the next box */
        fence_before();
        __syncthreads();
        fence_after();
        const int next = tile + (int)gridDim.x;
        if (t == 0) {
            mma_bf16(tmem, sdesc(a1, 128, 128 * (kIn / 8)), sdesc(b1, 128, 128 * (kIn / 8)), idesc_bf16(kTcRows, kHid),
                     0u);
            mma_commit(mbar);
            if (next < ntiles) tma_load_tile(&tmap, xdst, xbar, next * kTcRows);
        }
        loading = next < ntiles;
        failed = __syncthreads_or(!mbar_wait(mbar, phase)) != 0;
        phase ^= 1u;
        if (failed) break;
        fence_after();
        hidden_epilogue(tlane, 0, S.bias1, S.a2, t);
        fence_proxy_async();
        fence_before();
        __syncthreads();
        fence_after();
        if (t == 0) {
#pragma unroll
            for (int ks = 0; ks < kHid / 16; ++ks)
                mma_bf16(tmem + 64, sdesc(a2 + 256 * ks, 128, 128 * (kHid / 8)),
                         sdesc(b2 + 256 * ks, 128, 128 * (kHid / 8)), idesc_bf16(kTcRows, kHid), ks > 0);
            mma_commit(mbar);
        }
        failed = __syncthreads_or(!mbar_wait(mbar, phase)) != 0;
        phase ^= 1u;
        if (failed) break;
        fence_after();
        hidden_epilogue(tlane, 64, S.bias2, S.a2, t);
        fence_proxy_async();
        fence_before();
        __syncthreads();
        fence_after();
        if (t == 0) {
#pragma unroll
            for (int ks = 0; ks < kHid / 16; ++ks)
                mma_bf16(tmem, sdesc(a2 + 256 * ks, 128, 128 * (kHid / 8)), sdesc(b3 + 256 * ks, 128, 128 * (kHid / 8)),
                         idesc_bf16(kTcRows, kN3), ks > 0);
            mma_commit(mbar);
        }
        failed = __syncthreads_or(!mbar_wait(mbar, phase)) != 0;
        phase ^= 1u;
        if (failed) break;
        fence_after();
        float o[16];
        tmem_ld16(tlane, o);
        if (row < n) {
            const float r0 = (o[0] + S.bias3[0]) * k, r1 = (o[1] + S.bias3[1]) * k, r2 = (o[2] + S.bias3[2]) * k;
            y[row] = make_float4(r0, r1, r2, 0.0f);
        }
        fence_before();
        __syncthreads(); /* TMEM and A1 / A2 free for the next tile */
        fence_after();
    }
    if (failed) {
        if (t == 0) {
            atomicOr(err, 1u);
            mbar_wait(mbar, phase ^ 1u); /* an MMA phase that did not complete in time, once more */
            if (loading) mbar_wait(xbar, xphase); /* a box still in flight towards xs, once more */
        }
        __syncthreads();
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

/* the 2-D map of the feature rows for k_mlp_infer_tma: n rows of kIn floats,
 * 128 bytes apart, read as 128 x 16 boxes; false when the driver entry point
 * is unavailable (the per-thread loads are used then) */
typedef CUresult (*EncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiled encode_tiled() { /* the driver's cuTensorMapEncodeTiled, looked up once, thread-safely */
    static const EncodeTiled encode = []() -> EncodeTiled {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<EncodeTiled>(fn);
        return nullptr;
    }();
    return encode;
}
bool feature_tensor_map(CUtensorMap *m, const float *x, int n) {
    const EncodeTiled encode = encode_tiled();
    if (!encode || n <= 0 || (reinterpret_cast<uintptr_t>(x) & 15u) != 0) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)kIn, (cuuint64_t)n};
    const cuuint64_t strides[1] = {(cuuint64_t)kIn * sizeof(float)};
    const cuuint32_t box[2] = {(cuuint32_t)kTmaCols, (cuuint32_t)kTcRows};
    const cuuint32_t estr[2] = {1u, 1u};
    std::memset(m, 0, sizeof(*m));
    return encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(x), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

unsigned int tc_blocks(int n) {
    const unsigned int tiles = (unsigned int)((n + kTcRows - 1) / kTcRows);
    return tiles < 4u * 152u ? (tiles > 0 ? tiles : 1u) : 4u * 152u; /* four CTAs (512 TMEM columns) per SM */
}

}  // namespace

void mlp_tc_prepare() { encode_tiled(); }

void launch_mlp_infer_tc(const MlpDev *m, const float *x, int n, float4 *y, float scale, const unsigned int *valid,
                         unsigned int *err, cudaStream_t s, bool local_only, bool tma) {
    if (n <= 0) return;
    CUtensorMap map;
    if (local_only && tma && feature_tensor_map(&map, x, n)) {
        k_mlp_infer_tma<<<tc_blocks(n), kTcThreads, 0, s>>>(m, map, n, y, scale, valid, err);
        return;
    }
    auto k = local_only ? k_mlp_infer_tc<1> : k_mlp_infer_tc<kIn / 16>;
    k<<<tc_blocks(n), kTcThreads, 0, s>>>(m, x, n, y, nullptr, scale, valid, err);
}

void launch_mlp_forward3_tc(const MlpDev *m, const float *x, int n, float *y, unsigned int *err, cudaStream_t s) {
    if (n <= 0) return;
    k_mlp_infer_tc<kIn / 16><<<tc_blocks(n), kTcThreads, 0, s>>>(m, x, n, nullptr, y, 1.0f, nullptr, err);
}

}  // namespace fsph
