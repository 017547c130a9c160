/*
 * fsph_passes.cuh -- per-particle bodies of the PBF passes, shared by the
 * single-scene kernels (fsph_kernels.cu, one thread per particle) and the
 * batched persistent kernels (fsph_batch.cu, tiles of one scene per block).
 *
 * A body computes one particle i (a slot in device order) with the constants
 * of its scene, p.  `valid` is false for the padding lanes of a tile: they
 * run the loops on a clamped slot (so warp-wide shuffles stay convergent)
 * and write nothing.  LPP > 1 lets LPP adjacent lanes share one particle's
 * candidates (lane `sub` takes entries sub, sub + LPP, ...); their partial
 * sums are combined with shuffles, and lane 0 of the group writes.
 */
#pragma once
#include "fsph_kernels.cuh"

namespace fsph {

/* ---------------- candidate loop ---------------- */

/* Calls f(j, load(j)) for every candidate slot j of slot i handled by lane
 * `sub` of its LPP-lane group: the list entries sub, sub + LPP, ... or -- for
 * an overflowed list or when lists are off -- every LPP-th slot of the 27
 * cells around the current position.  List entries are taken kBatch at a
 * time: their indices are decoded and their positions loaded before any is
 * used, so each thread keeps kBatch independent loads in flight (the passes
 * are bound by load latency, not by arithmetic).  rs: this thread's 9 row
 * starts in shared memory, strided by the block size.  Load selects the
 * load flavour for x. */
#ifndef FSPH_KBATCH
#define FSPH_KBATCH 4
#endif

/* resident threads per SM the constraint passes are compiled for (single
 * scene and batched): 1536 cap them at 40 registers, 48 warps per SM
 * (measured best) */
#ifndef FSPH_PASS_THREADS
#define FSPH_PASS_THREADS 1536
#endif
#define FSPH_PASS_MINB (FSPH_PASS_THREADS / FSPH_PASS_BLOCK)
constexpr int kBatch = FSPH_KBATCH;

/* FSPH_FOLD 1: the constraint passes keep constant factors out of the pair
 * loop (fewer instructions per candidate; same results to rounding).
 * Measured on the 1M double dam break: lambda 82 -> 80 us, warm step
 * 2.855 -> 2.817 ms, plain step 10.25 -> 10.06 ms; on by default. */
#ifndef FSPH_FOLD
#define FSPH_FOLD 1
#endif
/* FSPH_PERSIST_LAMBDA / FSPH_PERSIST_CORRECTION 1: that single-scene
 * constraint pass runs as many blocks as are resident on the GPU, each warp
 * taking 32-slot chunks round-robin (FSPH_PERSIST sets both).  Measured on
 * the 1M double dam break: lambda 92 -> 82 us with identical results, so on
 * by default; the correction pass gets slower (90 -> 95 us, warm step 2.855
 * -> 2.917 ms), so off. */
#ifdef FSPH_PERSIST
#define FSPH_PERSIST_LAMBDA FSPH_PERSIST
#define FSPH_PERSIST_CORRECTION FSPH_PERSIST
#endif
/* FSPH_DYN_CHUNKS 1 (default): the persistent passes take their last
 * chunks on demand (an atomic counter per pass) instead of round-robin, so
 * warps that finish early take the leftovers; the lambda pass then sums its
 * errors in 64-bit fixed point (units of 2^-32), which is exact and so
 * independent of which warp ran which chunk.  FSPH_DYN_EXTRA whole rounds
 * join the leftovers in the on-demand pool.  Measured on the 1M double dam
 * break (same positions bit for bit): lambda 78.1 -> 75.6 us with the
 * leftovers alone, 73.7 us with one more round (default), 75 / 76 us with
 * two / three, 81 us with every chunk on demand (the counter contends);
 * the correction pass made persistent this way got slower (86 -> 92 us) and
 * stays a plain grid. */
#ifndef FSPH_DYN_CHUNKS
#define FSPH_DYN_CHUNKS 1
#endif
#ifndef FSPH_DYN_EXTRA
#define FSPH_DYN_EXTRA 1
#endif
#ifndef FSPH_PERSIST_LAMBDA
#define FSPH_PERSIST_LAMBDA 1
#endif
#ifndef FSPH_PERSIST_CORRECTION
#define FSPH_PERSIST_CORRECTION 0
#endif

/* Neighbour-list loads do not allocate in L1 (ld.global.nc.L1::no_allocate):
 * a pass streams ≈ 160 B of list per particle once, while the gathered
 * positions (16 B per particle, each read ≈ 40 times per pass) keep L1 to
 * themselves.  FSPH_LIST_HINT 0 gives plain read-only loads. */
#ifndef FSPH_LIST_HINT
#define FSPH_LIST_HINT 1
#endif

__device__ __forceinline__ uint4 load_list_group(const uint4 *a) {
#if FSPH_LIST_HINT == 1
    uint4 r;
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
        : "l"(a));
    return r;
#elif FSPH_LIST_HINT == 2
    /* also first in line for eviction from L2: the streamed lists make room
     * before the gathered positions do */
    uint4 r;
    unsigned long long pol;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
        : "l"(a), "l"(pol));
    return r;
#else
    return __ldg(a);
#endif
}

/* The list groups are prefetched into L2 kListAhead groups ahead of their
 * use (the lists stream from DRAM: they are larger than L2).  Measured at
 * 1 M particles: 2 groups ahead -2.3 % per step; 1, 3 or 4 ahead, or the
 * next group loaded into registers, gain less.  FSPH_LIST_PF 0 turns the
 * prefetch off. */
#ifndef FSPH_LIST_PF
#define FSPH_LIST_PF 1
#endif
constexpr int kListAhead = 2;

__device__ __forceinline__ void prefetch_list_group(const uint4 *a) {
#if FSPH_LIST_PF
    asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
#endif
}

template <int LPP, class Load, class F>
__device__ __forceinline__ void for_each_candidate(const DevParams &p, const unsigned int *__restrict__ cell_start,
                                                   const ListEntry *__restrict__ list,
                                                   const unsigned char *__restrict__ cnt,
                                                   const unsigned int *__restrict__ cellb, int i, float3 xi,
                                                   unsigned int *rs, int sub, Load &&load, F &&f) {
    int k = list ? (int)cnt[i] : (int)kListOverflow;
#if FSPH_DEBUG_BOUNDS
    if (k > kListMax && k != (int)kListOverflow) { /* a count the build never writes: walk the cells */
        if (p.dbg) atomicOr(p.dbg, kBoundCount);
        k = (int)kListOverflow;
    }
#endif
#ifdef FSPH_LIST_GROUPED
    if (LPP == 1 && kBatch == 4 && k != (int)kListOverflow) {
        /* one 16-byte load brings the next four entries (the tail group is
         * padded with a valid slot, so every load stays in bounds) */
        const uint4 *lg = reinterpret_cast<const uint4 *>(list) + i;
#pragma unroll
        for (int g = 1; g < kListAhead; ++g)
            if (4 * g < k) prefetch_list_group(lg + (size_t)g * (size_t)p.n);
        for (int t0 = 0; t0 < k; t0 += 4) {
            if (t0 + 4 * kListAhead < k) prefetch_list_group(lg + (size_t)((t0 >> 2) + kListAhead) * (size_t)p.n);
            const uint4 e = load_list_group(lg + (size_t)(t0 >> 2) * (size_t)p.n);
            const unsigned int j[4] = {bounded(p, e.x, (unsigned int)p.n, kBoundSlot),
                                       bounded(p, e.y, (unsigned int)p.n, kBoundSlot),
                                       bounded(p, e.z, (unsigned int)p.n, kBoundSlot),
                                       bounded(p, e.w, (unsigned int)p.n, kBoundSlot)};
            decltype(load(0u)) xj[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) xj[u] = load(j[u]);
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (t0 + u < k) f(j[u], xj[u]);
        }
    } else
#endif
    if (k != (int)kListOverflow) {
#ifndef FSPH_LIST32
        const int cb = (int)cellb[i];
#pragma unroll
        for (int r = 0; r < 9; ++r) {
            const int base = cb + ((r / 3 - 1) * p.gy + (r % 3 - 1)) * p.gx;
            rs[r * blockDim.x] = cell_row_ok(p, (unsigned int)base) ? __ldg(cell_start + base - 1) : 0u;
        }
#endif
        for (int t0 = sub; t0 < k; t0 += kBatch * LPP) {
            unsigned int j[kBatch];
            decltype(load(0u)) xj[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; ++u) {
                const int t = t0 + u * LPP < k ? t0 + u * LPP : k - 1;
#ifdef FSPH_LIST32
                j[u] = bounded(p, __ldg(list + list_at(t, i, p.n)), (unsigned int)p.n, kBoundSlot);
#else
                const unsigned int e = __ldg(list + list_at(t, i, p.n));
                j[u] = bounded(p, rs[((e >> 12) % 9u) * blockDim.x] + (e & 0xfffu), (unsigned int)p.n, kBoundSlot);
#endif
            }
#pragma unroll
            for (int u = 0; u < kBatch; ++u) xj[u] = load(j[u]);
#pragma unroll
            for (int u = 0; u < kBatch; ++u)
                if (t0 + u * LPP < k) f(j[u], xj[u]);
        }
    } else {
        const int3 c = cell_of(xi, p);
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy) {
                unsigned int s, e;
                row_range(cell_start, c, dy, dz, p, s, e);
                for (unsigned int j = s + (unsigned int)sub; j < e; j += LPP) f(j, load(j));
            }
    }
}

/* Calls f(b, bpos[b]) for every boundary slot b in the 27 cells around the
 * cell of x (nothing when no boundary particle is near that cell).  The
 * boundary is static and sorted by the same cells as the fluid, so a
 * boundary particle within h of x lies in those cells. */
template <class F>
__device__ __forceinline__ void for_each_boundary(const DevParams &p, float3 x, F &&f) {
    const int3 c = cell_of(x, p);
    const unsigned int ci = cell_index(c, p);
    if (!p.bnear[ci]) return;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy) {
            const unsigned int base = ci + (unsigned int)((dz * p.gy + dy) * p.gx);
            if (!cell_row_ok(p, base)) continue;
            const unsigned int s = __ldg(p.bcell + base - 1);
            const unsigned int e = bounded(p, __ldg(p.bcell + base + 2), (unsigned int)p.nb + 1u, kBoundBoundary);
            for (unsigned int j = s; j < e; ++j) f(j, __ldg(p.bpos + j));
        }
}

/* sum over the LPP lanes of a group (every lane of the warp must call it) */
template <int LPP>
__device__ __forceinline__ float group_sum(float v) {
#pragma unroll
    for (int o = LPP / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

/* ---------------- grid build ---------------- */

/* x* = walls(x + dt (v + dt a)), a = gravity when acc == NULL, then the
 * cell key and the slot's rank within the cell. */
__device__ __forceinline__ void predict_body(const DevParams &p, int i, const float4 *__restrict__ pos,
                                             const float4 *__restrict__ vel, const float4 *__restrict__ acc,
                                             float4 *__restrict__ ppos_out, unsigned int *__restrict__ key,
                                             unsigned int *__restrict__ rank, unsigned int *__restrict__ count,
                                             const float4 *__restrict__ dwarm, float4 *__restrict__ xpred_out) {
    float3 x = f3(pos[i]);
    float3 v = f3(vel[i]);
    float3 a = acc ? f3(acc[i]) : p.gravity;
    const float3 x_old = x;
    v = v + p.dt * a;
    x = x + p.dt * v;
    if (p.ntri) polygon_collide(x_old, x, v, p.dt, p);
    x = solid_project(x, p);
    if (xpred_out) xpred_out[i] = make_float4(x.x, x.y, x.z, 0.0f);
    /* warm start: the iterations begin from walls(x* + predicted correction);
     * the grid and lists are then built on that start */
    if (dwarm) x = solid_project(x + f3(dwarm[i]), p);
    ppos_out[i] = make_float4(x.x, x.y, x.z, 0.0f);
    unsigned int c = cell_index(cell_of(x, p), p);
    key[i] = c;
    rank[i] = atomicAdd(count + c, 1u);
}

__device__ __forceinline__ void hash_body(const DevParams &p, int i, float3 x, unsigned int *__restrict__ key,
                                          unsigned int *__restrict__ rank, unsigned int *__restrict__ count) {
    unsigned int c = cell_index(cell_of(x, p), p);
    key[i] = c;
    rank[i] = atomicAdd(count + c, 1u);
}

/* Every slot j within the list radius (= the cell width) of slot i at the
 * build positions xb, self included, as (row << 12) | (j - row_start). */
__device__ __forceinline__ void build_list_body(const DevParams &p, int i, const unsigned int *__restrict__ cell_start,
                                                const float4 *__restrict__ xb, const unsigned int *__restrict__ cellb,
                                                ListEntry *__restrict__ list, unsigned char *__restrict__ cnt) {
    const float3 xi = f3(xb[i]);
    const int cb = (int)cellb[i];
    int k = 0;
    bool ovf = false;
    ListEntry last = 0;
#pragma unroll 1
    for (int r = 0; r < 9; ++r) {
        const int base = cb + ((r / 3 - 1) * p.gy + (r % 3 - 1)) * p.gx;
        if (!cell_row_ok(p, (unsigned int)base)) continue;
        const unsigned int s = __ldg(cell_start + base - 1);
        const unsigned int e = bounded(p, __ldg(cell_start + base + 2), (unsigned int)p.n + 1u, kBoundSlot);
        if (e - s > 4095u) ovf = true;
        /* four candidates' loads in flight before their tests */
        for (unsigned int j0 = s; j0 < e; j0 += 4) {
            float4 xc[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) xc[u] = __ldg(xb + min(j0 + u, e - 1));
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const float3 d = xi - f3(xc[u]);
                if (j0 + u < e && dot3(d, d) < p.rl2) {
#ifdef FSPH_LIST32
                    last = j0 + u;
#else
                    last = (ListEntry)((r << 12) | (j0 + u - s));
#endif
                    if (k < kListMax) list[list_at(k, i, p.n)] = last;
                    ++k;
                }
            }
        }
    }
    const bool overflow = ovf || k > kListMax;
#ifdef FSPH_LIST_GROUPED
    if (!overflow) /* pad the last group (k >= 1: the slot itself is always listed) */
        for (int t = k; (t & 3) != 0; ++t) list[list_at(t, i, p.n)] = last;
#endif
    cnt[i] = overflow ? kListOverflow : (unsigned char)k;
}

/* ---------------- constraint iterations ---------------- */

/* lambda pass of one particle: density, C, sum |grad C|^2 (with the k = i
 * term), lambda into x*.w and rho into dens (lane 0 of a valid group).
 * Returns C (the caller turns it into the error terms). */
template <int LPP, bool KAHAN = false>
__device__ __forceinline__ float lambda_body(const DevParams &p, const unsigned int *__restrict__ cell_start,
                                             float4 *pp, float *__restrict__ dens, DevCtl *ctl,
                                             const ListEntry *__restrict__ list,
                                             const unsigned char *__restrict__ cnt,
                                             const unsigned int *__restrict__ cellb, unsigned int *rs, int i, int sub,
                                             bool valid) {
    const float3 xi = f3(pp[i]);
    float wsum = 0.f, wc = 0.f, sd = 0.f;
    float3 gs = make_float3(0.f, 0.f, 0.f);
    const float agr = p.ag * p.inv_rest_dens;
#if FSPH_FOLD
    /* the pair loop sums g' = (h - r)^2 / r; the coefficient agr (grad W /
     * rho0 = agr g' d) multiplies the sums once after the loop */
    const float agl = 1.0f;
#else
    const float agl = agr;
#endif
    /* plain (L1-cached) loads: only the .w words of pp are written by this
     * pass, and the neighbour loop reads x, y, z */
    for_each_candidate<LPP>(
        p, cell_start, list, cnt, cellb, i, xi, rs, sub, [&](unsigned int j) { return pp[j]; },
        [&](unsigned int, const float4 &xj4) {
            /* branch-free: outside h both q and t clamp to zero; the self
             * pair (d = 0) adds W(0) to the density and nothing else */
            const float3 d = xi - f3(xj4);
            const float r2 = dot3(d, d);
            const float q = fmaxf(p.h2 - r2, 0.0f);
            const float inv_r = pair_rsqrt(r2);
            const float t = fmaxf(p.h - r2 * inv_r, 0.0f);
            const float g = agl * t * t * inv_r; /* grad W / rho0 = (agr / agl) g d */
            if (KAHAN) { /* compensated sum of the density terms */
                const float y = q * q * q - wc;
                const float s = wsum + y;
                wc = (s - wsum) - y;
                wsum = s;
            } else {
                wsum += q * q * q;
            }
            gs = gs + g * d;
            sd += g * g * r2;
        });
    if (LPP > 1) {
        wsum = group_sum<LPP>(wsum);
        sd = group_sum<LPP>(sd);
        gs.x = group_sum<LPP>(gs.x);
        gs.y = group_sum<LPP>(gs.y);
        gs.z = group_sum<LPP>(gs.z);
    }
    float rho = p.mass * p.aw * wsum;
    sd += dot3(gs, gs);
#if FSPH_FOLD
    sd *= agr * agr;
#endif
    if (p.nb) {
        /* boundary particles (rx_sph_pbd.cpp:728-748, 795-818): density
         * rho0 psi_b W and |grad C|^2 terms of (rho0 psi_b / m) grad W / rho0,
         * each boundary neighbour counted once (rx_pbdsph_kernel.cu:577-664);
         * every lane of a group sums them (they are few) */
        float bw = 0.f;
        for_each_boundary(p, xi, [&](unsigned int, const float4 &b4) {
            const float3 d = xi - f3(b4);
            const float r2 = dot3(d, d);
            const float q = fmaxf(p.h2 - r2, 0.0f);
            const float inv_r = pair_rsqrt(r2);
            const float t = fmaxf(p.h - r2 * inv_r, 0.0f);
            const float gb = b4.w * agr * t * t * inv_r;
            bw += b4.w * q * q * q;
            sd += gb * gb * r2;
        });
        rho += p.mass * p.aw * bw;
    }
    float C = rho * p.inv_rest_dens - 1.0f;
    float Cc = (p.clamp_constraint && C < 0.0f) ? 0.0f : C;
    float lam = -Cc / (sd + p.epsilon);
    if (valid && sub == 0) {
        reinterpret_cast<float *>(pp + i)[3] = lam;
        dens[i] = rho;
        if (!(rho == rho)) ctl->nan_flag = 1u;
    }
    return C;
}

/* End of the lambda pass: block partial errors; the last block reduces them
 * in a fixed order, advances the iteration counter and decides whether the
 * device-side loop continues (lp: the loop constants).  Every thread of the
 * block calls it. */
__device__ __forceinline__ void lambda_tail(const DevParams &lp, DevCtl *ctl, ErrPartial *part, float e1, float e2,
                                            float em, cudaGraphConditionalHandle hwhile, int use_graph) {
    __shared__ float sh1[32], sh2[32], shm[32];
    __shared__ double d1[32], d2[32];
    __shared__ int s_last;
    e1 = warp_sum(e1);
    e2 = warp_sum(e2);
    em = warp_max(em);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) { sh1[warp] = e1; sh2[warp] = e2; shm[warp] = em; }
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.f, b = 0.f, m = 0.f;
        for (int w = 0; w < nw; ++w) { a += sh1[w]; b += sh2[w]; m = fmaxf(m, shm[w]); }
        part[blockIdx.x] = ErrPartial{a, b, m, 0.f};
        __threadfence();
        unsigned int t = atomicAdd(&ctl->ticket, 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    /* fixed-order reduction of the block partials (double): strided per
     * thread, a shuffle tree per warp, then the warps in order */
    double a = 0.0, b = 0.0;
    float m = 0.f;
    for (unsigned int k = threadIdx.x; k < gridDim.x; k += blockDim.x) {
        float4 v = __ldcg(reinterpret_cast<const float4 *>(part) + k);
        a += v.x; b += v.y; m = fmaxf(m, v.z);
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    if (lane == 0) { d1[warp] = a; d2[warp] = b; shm[warp] = m; }
    __syncthreads();
    if (threadIdx.x == 0) {
        a = 0.0; b = 0.0; m = 0.f;
        for (int w = 0; w < nw; ++w) { a += d1[w]; b += d2[w]; m = fmaxf(m, shm[w]); }
        float err1 = (float)(a / (double)lp.n);
        float err2 = (float)(b / (double)lp.n);
        ctl->err1 = err1;
        ctl->err2 = err2;
        ctl->errmax = m;
        unsigned int it = ctl->iter + 1u;
        ctl->iter = it;
        float err = lp.error_mode ? err2 : err1;
        int minit = lp.min_iter > 1 ? lp.min_iter : 1;
        int cont = ((int)it < lp.max_iter) && !(err <= lp.eta && (int)it >= minit);
        if (ctl->nan_flag) cont = 0;
        ctl->done = cont ? 0u : 1u;
        ctl->ticket = 0u;
        if (use_graph & 1) cudaGraphSetConditional(hwhile, cont ? 1u : 0u);
    }
}

/* |C| in units of 2^-32, saturating (a diverged step is caught by the NaN
 * flag and the error itself) */
__device__ __forceinline__ unsigned long long err_fix(float x) {
    return (unsigned long long)__float2ll_rn(fminf(x, 1024.0f) * 4294967296.0f);
}
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
/* the next chunk of a persistent pass: round-robin while whole rounds last,
 * then on demand from the pass's counter (warp-uniform) */
__device__ __forceinline__ int next_chunk(int c, int nw, int stat, unsigned int *ctr, int lane) {
    c += nw;
    if (c < stat) return c;
    unsigned int v = 0u;
    if (lane == 0) v = atomicAdd(ctr, 1u);
    return stat + (int)__shfl_sync(0xffffffffu, v, 0);
}
__device__ __forceinline__ int first_chunk(int w, int stat, unsigned int *ctr, int lane) {
    if (w < stat) return w;
    unsigned int v = 0u;
    if (lane == 0) v = atomicAdd(ctr, 1u);
    return stat + (int)__shfl_sync(0xffffffffu, v, 0);
}

/* lambda_tail for fixed-point error sums: integer sums are exact, so the
 * block partials may combine in any order */
__device__ __forceinline__ void lambda_tail_fix(const DevParams &lp, DevCtl *ctl, ErrPartial *part,
                                                unsigned long long q1, unsigned long long q2, float em,
                                                cudaGraphConditionalHandle hwhile, int use_graph) {
    __shared__ unsigned long long sq1[32], sq2[32];
    __shared__ float shm[32];
    __shared__ int s_last;
    ErrPartialFix *pf = reinterpret_cast<ErrPartialFix *>(part);
    q1 = warp_sum_u64(q1);
    q2 = warp_sum_u64(q2);
    em = warp_max(em);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) { sq1[warp] = q1; sq2[warp] = q2; shm[warp] = em; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long a = 0ull, b = 0ull;
        float m = 0.f;
        for (int w = 0; w < nw; ++w) { a += sq1[w]; b += sq2[w]; m = fmaxf(m, shm[w]); }
        pf[blockIdx.x].s1 = a;
        pf[blockIdx.x].s2 = b;
        pf[blockIdx.x].mx = m;
        __threadfence();
        unsigned int t = atomicAdd(&ctl->ticket, 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    unsigned long long a = 0ull, b = 0ull;
    float m = 0.f;
    for (unsigned int k = threadIdx.x; k < gridDim.x; k += blockDim.x) {
        a += __ldcg(&pf[k].s1);
        b += __ldcg(&pf[k].s2);
        m = fmaxf(m, __ldcg(&pf[k].mx));
    }
    a = warp_sum_u64(a);
    b = warp_sum_u64(b);
    m = warp_max(m);
    __syncthreads(); /* every warp has read its shared entries above */
    if (lane == 0) { sq1[warp] = a; sq2[warp] = b; shm[warp] = m; }
    __syncthreads();
    if (threadIdx.x == 0) {
        a = 0ull; b = 0ull; m = 0.f;
        for (int w = 0; w < nw; ++w) { a += sq1[w]; b += sq2[w]; m = fmaxf(m, shm[w]); }
        float err1 = (float)((double)a * 0x1p-32 / (double)lp.n);
        float err2 = (float)((double)b * 0x1p-32 / (double)lp.n);
        ctl->err1 = err1;
        ctl->err2 = err2;
        ctl->errmax = m;
        unsigned int it = ctl->iter + 1u;
        ctl->iter = it;
        float err = lp.error_mode ? err2 : err1;
        int minit = lp.min_iter > 1 ? lp.min_iter : 1;
        int cont = ((int)it < lp.max_iter) && !(err <= lp.eta && (int)it >= minit);
        if (ctl->nan_flag) cont = 0;
        ctl->done = cont ? 0u : 1u;
        ctl->ticket = 0u;
        ctl->grab = 0u; /* every block has passed its loop: the counter is free for the next pass */
        if (use_graph & 1) cudaGraphSetConditional(hwhile, cont ? 1u : 0u);
    }
}

/* correction pass of one particle: dp_i = sum_j (lambda_i + lambda_j + s_corr)
 * grad W_ij / rho0, x*_i <- walls(x*_i + dp_i) into dst (lane 0 of a valid
 * group).  Returns |x*_i - xb_i|^2 (0 for the other lanes). */
template <int LPP>
__device__ __forceinline__ float correction_body(const DevParams &p, const unsigned int *__restrict__ cell_start,
                                                 const float4 *__restrict__ src, float4 *__restrict__ dst,
                                                 const float4 *__restrict__ xb, DevCtl *ctl,
                                                 float4 *__restrict__ dp_out, const ListEntry *__restrict__ list,
                                                 const unsigned char *__restrict__ cnt,
                                                 const unsigned int *__restrict__ cellb, unsigned int *rs, int i,
                                                 int sub, bool valid) {
    const float4 xi4 = src[i];
    const float3 xi = f3(xi4);
    const float li = xi4.w;
    float3 acc = make_float3(0.f, 0.f, 0.f);
    const float k_dt2 = -p.ap_k * p.dt * p.dt;
    const float agr = p.ag * p.inv_rest_dens;
    const float awq = p.aw * p.inv_wq;
#if FSPH_FOLD
    /* agr multiplies the sum once after the loop; for n = 4 the tensile
     * term -k dt^2 (awq q^3)^4 is K q^12 with K = -k dt^2 awq^4 (|K| ~ 1e26
     * for the configured h, well inside FP32) */
    const float agl = 1.0f;
    const float awq2 = awq * awq;
    const float k12 = k_dt2 * (awq2 * awq2);
#else
    const float agl = agr;
#endif
    for_each_candidate<LPP>(
        p, cell_start, list, cnt, cellb, i, xi, rs, sub, [&](unsigned int j) { return __ldg(src + j); },
        [&](unsigned int, const float4 &xj4) {
            /* branch-free: t = 0 outside h and d = 0 for the self pair */
            const float3 d = xi - f3(xj4);
            const float r2 = dot3(d, d);
            const float inv_r = pair_rsqrt(r2);
            const float t = fmaxf(p.h - r2 * inv_r, 0.0f);
            const float g = agl * t * t * inv_r;
            float coef = li + xj4.w;
            if (p.use_ap) {
                const float q = fmaxf(p.h2 - r2, 0.0f);
#if FSPH_FOLD
                if (p.ap_n == 4.0f) {
                    const float q2 = q * q, q4 = q2 * q2;
                    coef = fmaf(k12, (q4 * q4) * q4, coef);
                } else {
                    coef += k_dt2 * __powf(awq * q * q * q, p.ap_n);
                }
#else
                const float ww = awq * q * q * q;
                const float pw = (p.ap_n == 4.0f) ? (ww * ww) * (ww * ww) : __powf(ww, p.ap_n);
                coef += k_dt2 * pw;
#endif
            }
            acc = acc + (coef * g) * d;
        });
    if (LPP > 1) {
        acc.x = group_sum<LPP>(acc.x);
        acc.y = group_sum<LPP>(acc.y);
        acc.z = group_sum<LPP>(acc.z);
    }
#if FSPH_FOLD
    acc = agr * acc;
#endif
    if (p.nb) {
        /* boundary terms (rx_sph_pbd.cpp:977-1019): lambda_b, and s_corr of
         * the (rho0 psi_b / m)-scaled W */
        float3 accb = make_float3(0.f, 0.f, 0.f);
        for_each_boundary(p, xi, [&](unsigned int b, const float4 &b4) {
            const float3 d = xi - f3(b4);
            const float r2 = dot3(d, d);
            const float inv_r = pair_rsqrt(r2);
            const float t = fmaxf(p.h - r2 * inv_r, 0.0f);
            const float g = agr * t * t * inv_r;
            float sc = 0.0f;
            if (p.use_ap) {
                const float q = fmaxf(p.h2 - r2, 0.0f);
                const float ww = b4.w * awq * q * q * q;
                const float pw = (p.ap_n == 4.0f) ? (ww * ww) * (ww * ww) : __powf(ww, p.ap_n);
                sc = k_dt2 * pw;
            }
            accb = accb + ((li + __ldg(p.blam + b) + sc) * g) * d;
        });
        acc = acc + accb;
    }
    if (!valid || sub != 0) return 0.0f;
    if (dp_out) dp_out[i] = make_float4(acc.x, acc.y, acc.z, 0.0f);
    float3 xn = solid_project(xi + acc, p);
    dst[i] = make_float4(xn.x, xn.y, xn.z, 0.0f);
    float3 dd = xn - f3(xb[i]);
    if (!(xn.x == xn.x && xn.y == xn.y && xn.z == xn.z)) ctl->nan_flag = 1u;
    return dot3(dd, dd);
}

/* End of the correction pass: the largest displacement measure of the block;
 * the last block compares the maximum with lp.skin2 (a rebuild is due above
 * it), flips the x* parity and sets the graph's rebuild conditions.  Every
 * thread of the block calls it. */
__device__ __forceinline__ void correction_tail(const DevParams &lp, DevCtl *ctl, float *part, float disp2,
                                                unsigned int par, cudaGraphConditionalHandle hif,
                                                cudaGraphConditionalHandle hif2, int use_graph) {
    __shared__ float shm[32];
    __shared__ int s_last;
    disp2 = warp_max(disp2);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) shm[warp] = disp2;
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = 0.f;
        for (int w = 0; w < nw; ++w) m = fmaxf(m, shm[w]);
        part[blockIdx.x] = m;
        __threadfence();
        unsigned int t = atomicAdd(&ctl->ticket2, 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    float m = 0.f;
    for (unsigned int k = threadIdx.x; k < gridDim.x; k += blockDim.x) m = fmaxf(m, __ldcg(part + k));
    m = warp_max(m);
    __syncthreads(); /* every warp has read its shm entry above */
    if (lane == 0) shm[warp] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        float md = 0.f;
        for (int w = 0; w < nw; ++w) md = fmaxf(md, shm[w]);
        ctl->disp2_bits = __float_as_uint(md);
        unsigned int rb = (md > lp.skin2 || !(md == md)) ? 1u : 0u;
        ctl->rebuild = rb;
        ctl->parity = 1u - par;
        ctl->ticket2 = 0u;
        ctl->grab2 = 0u;
        if (use_graph & 1) {
            unsigned int more = ctl->done ? 0u : 1u;
            cudaGraphSetConditional(hif, rb & more);
            if (use_graph & 2) cudaGraphSetConditional(hif2, rb);
        }
    }
}

/* ---------------- end of step ---------------- */

/* omega_i = sum_j (m / rho_j)(v_j - v_i) x grad_j W_ij (grad_j = -grad_i):
 * the SPH curl of v, each neighbour weighted by its volume m / rho_j as in
 * the XSPH sum and the eta gradient below (Macklin & Mueller 2013, eq. 15,
 * writes the sum without the volume, whose scale their eps absorbs; in
 * SI units that sum is ~1e5 times the curl at h = 0.0457 and the configured
 * eps = 1e-4 then drives the flow unstable).  The XSPH update
 * v_i + c sum_j (m / rho_j)(v_j - v_i) W_ij, and (fo.feat) the warm-start
 * features of the particle. */
/* PRE: m / rho_j comes from mrho (written once per particle by k_finalize,
 * the same correctly rounded quotient) instead of a division per pair, and
 * the pass leaves (|omega_i|, m / rho_i) in wm for vort_apply_body<true>. */
template <bool NBR = true, bool PRE = false>
__device__ __forceinline__ void xsph_vort_body(const DevParams &p, int i, const unsigned int *__restrict__ cell_start,
                                               const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                                               const float *__restrict__ dens, float4 *__restrict__ vel_out,
                                               float4 *__restrict__ vort, const FeatureOut &fo,
                                               const ListEntry *__restrict__ list,
                                               const unsigned char *__restrict__ cnt,
                                               const unsigned int *__restrict__ cellb, unsigned int *rs,
                                               const float *__restrict__ mrho_in = nullptr,
                                               float2 *__restrict__ wm = nullptr) {
    const float3 xi = f3(pos[i]), vi = f3(vel[i]);
    float3 om = make_float3(0.f, 0.f, 0.f), xs = make_float3(0.f, 0.f, 0.f);
    float3 off = make_float3(0.f, 0.f, 0.f), cg = make_float3(0.f, 0.f, 0.f);
    float cntf = 0.f;
    float wpred = 0.f; /* sum q^3 at the next step's predicted relative positions */
    /* poly6-weighted neighbour sums (self excluded) for the features:
     * weights, density, relative velocity, step correction */
    float nw = 0.f, nrho = 0.f;
    float3 nv = make_float3(0.f, 0.f, 0.f), nd = make_float3(0.f, 0.f, 0.f);
    /* branch-free pair terms: q and t clamp to zero outside h, and the self
     * pair (d = 0, v_ij = 0) adds only to the neighbour count */
    for_each_candidate<1>(
        p, cell_start, list, cnt, cellb, i, xi, rs, 0, [&](unsigned int j) { return __ldg(pos + j); },
        [&](unsigned int j, const float4 &xj4) {
            const float3 d = xi - f3(xj4);
            const float r2 = dot3(d, d);
            const float inside = r2 < p.h2 ? 1.0f : 0.0f;
            const float q = fmaxf(p.h2 - r2, 0.0f);
            const float inv_r = pair_rsqrt(r2);
            const float t = fmaxf(p.h - r2 * inv_r, 0.0f);
            const float g = p.ag * t * t * inv_r;
            const float3 vij = f3(__ldg(vel + j)) - vi;
            const float rhoj = (NBR || !PRE) ? __ldg(dens + j) : 0.0f;
            const float mrho = PRE ? __ldg(mrho_in + j) : p.mass / rhoj;
            om = om + cross3(vij, (-g * mrho) * d);
            xs = xs + (p.aw * q * q * q * mrho) * vij;
            cntf += inside;
            off = off - inside * d;
            if (fo.feat) {
                /* the pair at the next step's prediction x + dt v (gravity cancels
                 * in relative positions): poly6 and its spiky gradient there */
                const float3 ds = d - p.dt * vij;
                const float r2s = dot3(ds, ds);
                const float qs = fmaxf(p.h2 - r2s, 0.0f);
                const float inv_rs = pair_rsqrt(r2s);
                const float ts = fmaxf(p.h - r2s * inv_rs, 0.0f);
                wpred += qs * qs * qs;
                cg = cg + (p.ag * ts * ts * inv_rs) * ds;
                if (NBR) {
                    const float w = r2 > 0.0f ? q * q * q : 0.0f;
                    nw += w;
                    nrho += w * rhoj;
                    nv = nv + w * vij;
                    nd = nd + w * f3(__ldg(fo.dstep + j));
                }
            }
        });
    cntf = fmaxf(cntf, 1.0f);
    float3 vn = vi + p.xsph_c * xs;
    vel_out[i] = make_float4(vn.x, vn.y, vn.z, 0.0f);
    vort[i] = make_float4(om.x, om.y, om.z, 0.0f);
    if (PRE) wm[i] = make_float2(sqrtf(dot3(om, om)), mrho_in[i]);
    if (fo.feat) {
        /* warm-start features at the end of the step (dimensionless; see kFeatures) */
        const float inv_h = 1.0f / p.h;
        const float4 *pl = fo.ctl->parity ? fo.ppos0 : fo.ppos1; /* buffer of the last lambda pass */
        const float3 dd = f3(fo.dstep[i]);
        float f[kFeatures];
        f[0] = dens[i] * p.inv_rest_dens - 1.0f;
        f[1] = pl[i].w * p.rest_dens * p.h2;
        f[2] = cntf * (1.0f / 33.0f);
        f[3] = off.x * inv_h / cntf; f[4] = off.y * inv_h / cntf; f[5] = off.z * inv_h / cntf;
        f[6] = vi.x * p.dt * inv_h; f[7] = vi.y * p.dt * inv_h; f[8] = vi.z * p.dt * inv_h;
        f[9] = dd.x * inv_h; f[10] = dd.y * inv_h; f[11] = dd.z * inv_h;
        /* predicted constraint C' = rho' / rho0 - 1 and h grad_i C' at the next prediction */
        const float mr0 = p.mass * p.inv_rest_dens;
        f[12] = mr0 * p.aw * wpred - 1.0f;
        f[13] = mr0 * cg.x * p.h; f[14] = mr0 * cg.y * p.h; f[15] = mr0 * cg.z * p.h;
        /* weighted neighbour means of features 0, 6-8 and 9-11 (zero without neighbours) */
        const float inw = nw > 0.0f ? 1.0f / nw : 0.0f;
        const float vs = p.dt * inv_h;
        f[16] = nw > 0.0f ? nrho * inw * p.inv_rest_dens - 1.0f : 0.0f;
        f[17] = nw > 0.0f ? (vi.x + nv.x * inw) * vs : 0.0f;
        f[18] = nw > 0.0f ? (vi.y + nv.y * inw) * vs : 0.0f;
        f[19] = nw > 0.0f ? (vi.z + nv.z * inw) * vs : 0.0f;
        f[20] = nd.x * inw * inv_h; f[21] = nd.y * inw * inv_h; f[22] = nd.z * inw * inv_h;
#pragma unroll
        for (int k = 23; k < kFeatures; ++k) f[k] = 0.0f;
        float4 *out = reinterpret_cast<float4 *>(fo.feat + (size_t)i * kFeatures);
#pragma unroll
        for (int k = 0; k < kFeatures / 4; ++k) out[k] = make_float4(f[4 * k], f[4 * k + 1], f[4 * k + 2], f[4 * k + 3]);
        if (i == 0) *fo.valid = 1u;
    }
}

/* eta_i = sum_j (m / rho_j)(|w_j| - |w_i|) grad_i W_ij; f = eps (eta/|eta|) x w_i;
 * v_i <- v_i + dt f. */
/* PRE: (|omega_j|, m / rho_j) from wm (one 8-byte gather per pair, no
 * division or square root; the same values xsph_vort_body<.., true> wrote). */
template <bool PRE = false>
__device__ __forceinline__ void vort_apply_body(const DevParams &p, int i, const unsigned int *__restrict__ cell_start,
                                                const float4 *__restrict__ pos, const float4 *__restrict__ vort,
                                                const float *__restrict__ dens, const float4 *__restrict__ vel_in,
                                                float4 *__restrict__ vel_out, const ListEntry *__restrict__ list,
                                                const unsigned char *__restrict__ cnt,
                                                const unsigned int *__restrict__ cellb, unsigned int *rs,
                                                const float2 *__restrict__ wm = nullptr) {
    float4 v4 = vel_in[i];
    if (p.vort_eps != 0.0f) {
        const float3 xi = f3(pos[i]);
        const float3 wi = f3(vort[i]);
        const float wmi = sqrtf(dot3(wi, wi));
        float3 eta = make_float3(0.f, 0.f, 0.f);
        for_each_candidate<1>(
            p, cell_start, list, cnt, cellb, i, xi, rs, 0, [&](unsigned int j) { return __ldg(pos + j); },
            [&](unsigned int j, const float4 &xj4) {
                const float3 d = xi - f3(xj4);
                const float r2 = dot3(d, d);
                const float inv_r = pair_rsqrt(r2);
                const float t = fmaxf(p.h - r2 * inv_r, 0.0f);
                const float g = p.ag * t * t * inv_r;
                float k;
                if (PRE) {
                    const float2 b = __ldg(wm + j); /* (|omega_j|, m / rho_j) */
                    k = b.y * (b.x - wmi) * g;
                } else {
                    const float3 wj = f3(__ldg(vort + j));
                    k = p.mass / __ldg(dens + j) * (sqrtf(dot3(wj, wj)) - wmi) * g;
                }
                eta = eta + k * d;
            });
        float en = sqrtf(dot3(eta, eta));
        if (en > 1e-30f) {
            float3 N = (1.0f / en) * eta;
            float3 f = p.vort_eps * cross3(N, wi);
            v4.x += p.dt * f.x;
            v4.y += p.dt * f.y;
            v4.z += p.dt * f.z;
        }
    }
    vel_out[i] = v4;
}

}  // namespace fsph
