/*
 * fsph_kernels.cu -- sm_103a kernels of the fluid step.
 *
 * One thread per particle in device (cell-sorted) order: the 32 lanes of a
 * warp are 32 consecutive slots, i.e. neighbouring particles of the same few
 * cells, so their nine candidate row ranges mostly coincide and the
 * candidate float4 loads are served by L1 / L2 broadcasts (the whole x*
 * array of a 1M-particle scene is 16 MB and stays resident in the 126 MB L2).
 *
 * Kernel-by-kernel correspondence with the reference:
 *   k_predict_hash     rxPBDSPH::integrate (rx_sph_pbd.cpp:1409-1446) fused with
 *                      calcHashD2 (rx_sph_kernel.cu:54-73)
 *   k_scan / scatter   thrust::sort_by_key + reorderDataAndFindCellStartD
 *                      (rx_cu_funcs.cu:255-260, rx_sph_kernel.cu:108-153)
 *   k_lambda           calScalingFactor (rx_sph_pbd.cpp:699-914) fused with the
 *                      density-error reduction (rx_sph_pbd.cpp:448-454,
 *                      rx_pbdsph_kernel.cu:431-441) and the loop test
 *   k_correction       calPositionCorrection (rx_sph_pbd.cpp:925-1026) fused with
 *                      the position update and wall projection (rx_sph_pbd.cpp:436-445)
 *   k_finalize         velocity / position update (rx_sph_pbd.cpp:464-471)
 *   k_xsph_vort        xsphVisocosity (rx_pbdsph_kernel.cu:1130-1162) + vorticity
 *   k_sph_*            rxSPH::calDensity / calForce / integrate (rx_sph_cpu.cpp:495-1077)
 */
#include "fsph_kernels.cuh"

namespace fsph {

/* ======================================================================== */
/* grid build                                                               */
/* ======================================================================== */

__global__ void k_predict_hash(DevParams p, const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                               const float4 *__restrict__ acc, float4 *__restrict__ ppos_out,
                               unsigned int *__restrict__ key, unsigned int *__restrict__ rank,
                               unsigned int *__restrict__ count, const float4 *__restrict__ dwarm,
                               float4 *__restrict__ xpred_out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    float3 x = f3(pos[i]);
    float3 v = f3(vel[i]);
    float3 a = acc ? f3(acc[i]) : p.gravity;
    v = v + p.dt * a;
    x = x + p.dt * v;
    x = wall_project(x, p);
    if (xpred_out) xpred_out[i] = make_float4(x.x, x.y, x.z, 0.0f);
    /* warm start: the iterations begin from walls(x* + predicted correction);
     * the grid and lists are then built on that start */
    if (dwarm) x = wall_project(x + f3(dwarm[i]), p);
    ppos_out[i] = make_float4(x.x, x.y, x.z, 0.0f);
    unsigned int c = cell_index(cell_of(x, p), p);
    key[i] = c;
    rank[i] = atomicAdd(count + c, 1u);
}

__global__ void k_hash(DevParams p, const float4 *__restrict__ x4, unsigned int *__restrict__ key,
                       unsigned int *__restrict__ rank, unsigned int *__restrict__ count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    unsigned int c = cell_index(cell_of(f3(x4[i]), p), p);
    key[i] = c;
    rank[i] = atomicAdd(count + c, 1u);
}

/* Scan phase 1: each 1024-thread block scans kScanTile = 4096 counts. */
__global__ void __launch_bounds__(1024) k_scan_local(unsigned int *__restrict__ count,
                                                     unsigned int *__restrict__ out,
                                                     unsigned int *__restrict__ block_sums, unsigned int ncells) {
    __shared__ unsigned int warp_tot[32];
    const unsigned int base = blockIdx.x * kScanTile + threadIdx.x * 4;
    unsigned int v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        unsigned int idx = base + k;
        v[k] = idx < ncells ? count[idx] : 0u;
        if (idx < ncells) count[idx] = 0u;
    }
    unsigned int t = v[0] + v[1] + v[2] + v[3];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned int incl = t;
    for (int o = 1; o < 32; o <<= 1) {
        unsigned int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned int w = warp_tot[lane];
        unsigned int wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            unsigned int y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        warp_tot[lane] = wi - w; /* exclusive prefix of the warps */
        if (lane == 31) block_sums[blockIdx.x] = wi;
    }
    __syncthreads();
    unsigned int run = warp_tot[warp] + incl - t;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        unsigned int idx = base + k;
        if (idx < ncells) out[idx] = run;
        run += v[k];
    }
}

/* Scan phase 2: one block scans the block totals; writes the grand total to out[ncells]. */
__global__ void __launch_bounds__(1024) k_scan_top(unsigned int *__restrict__ block_sums, unsigned int nblocks,
                                                   unsigned int *__restrict__ out, unsigned int ncells) {
    __shared__ unsigned int warp_tot[32];
    const int per = (nblocks + 1023) / 1024;
    const unsigned int start = threadIdx.x * per;
    unsigned int t = 0;
    for (int k = 0; k < per; ++k)
        if (start + k < nblocks) t += block_sums[start + k];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned int incl = t;
    for (int o = 1; o < 32; o <<= 1) {
        unsigned int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned int w = warp_tot[lane];
        unsigned int wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            unsigned int y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        warp_tot[lane] = wi - w;
        if (lane == 31) out[ncells] = wi;
    }
    __syncthreads();
    unsigned int run = warp_tot[warp] + incl - t;
    for (int k = 0; k < per; ++k)
        if (start + k < nblocks) {
            unsigned int b = block_sums[start + k];
            block_sums[start + k] = run;
            run += b;
        }
}

__global__ void k_scan_add(unsigned int *__restrict__ out, const unsigned int *__restrict__ block_sums,
                           unsigned int ncells) {
    unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ncells) out[i] += block_sums[i / kScanTile];
}

__global__ void k_scatter(int n, const unsigned int *__restrict__ key, const unsigned int *__restrict__ rank,
                          const unsigned int *__restrict__ cell_start, unsigned int *__restrict__ perm) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    perm[cell_start[key[i]] + rank[i]] = (unsigned int)i;
}

/* The atomic ranks order a cell's slots arbitrarily; sorting each cell's
 * (few) previous-slot indices makes the permutation the stable order of the
 * 64-bit key (cell << 32 | previous slot), identical on every run. */
__global__ void k_cell_sort(const unsigned int *__restrict__ cell_start, unsigned int *__restrict__ perm,
                            unsigned int ncells) {
    unsigned int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    unsigned int s = cell_start[c], e = cell_start[c + 1];
    if (e - s < 2) return;
    for (unsigned int a = s + 1; a < e; ++a) {
        unsigned int v = perm[a];
        unsigned int b = a;
        while (b > s && perm[b - 1] > v) {
            perm[b] = perm[b - 1];
            --b;
        }
        perm[b] = v;
    }
}

__global__ void k_gather(int n, const unsigned int *__restrict__ perm, Gather g, DevCtl *count_build) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d == 0 && count_build) count_build->builds += 1u;
    if (d >= n) return;
    unsigned int s = perm ? perm[d] : (unsigned int)d;
#pragma unroll
    for (int k = 0; k < 6; ++k)
        if (k < g.n4) g.dst4[k][d] = g.src4[k][s];
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (k < g.n1) g.dst1[k][d] = g.src1[k][s];
}

/* In-loop grid rebuild: hash the current x* (the ping-pong buffer named by
 * ctl->parity, which only the device knows inside a captured loop). */
__global__ void k_hash_parity(DevParams p, const float4 *ppos0, const float4 *ppos1, const DevCtl *ctl,
                              unsigned int *__restrict__ key, unsigned int *__restrict__ rank,
                              unsigned int *__restrict__ count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const float4 *x4 = ctl->parity ? ppos1 : ppos0;
    unsigned int c = cell_index(cell_of(f3(x4[i]), p), p);
    key[i] = c;
    rank[i] = atomicAdd(count + c, 1u);
}

/* Gather every array carried through the iterations into temporaries. */
__global__ void k_rebuild_gather(int n, const unsigned int *__restrict__ perm, const DevCtl *ctl,
                                 const float4 *__restrict__ pos, const float4 *ppos0, const float4 *ppos1,
                                 const unsigned int *__restrict__ id, const unsigned int *__restrict__ attr,
                                 const float *__restrict__ dens, float4 *__restrict__ t_pos,
                                 float4 *__restrict__ t_x, unsigned int *__restrict__ t_id,
                                 unsigned int *__restrict__ t_attr, float *__restrict__ t_dens,
                                 const unsigned int *__restrict__ key, unsigned int *__restrict__ cellb,
                                 const float4 *__restrict__ xpred, float4 *__restrict__ t_xpred,
                                 float *__restrict__ t_lam) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    const float4 *x4 = ctl->parity ? ppos1 : ppos0;
    unsigned int s = perm[d];
    if (cellb) cellb[d] = key[s];
    if (xpred) t_xpred[d] = xpred[s];
    /* lambda of the last pass lives in the .w of the other buffer */
    if (t_lam) t_lam[d] = (ctl->parity ? ppos0 : ppos1)[s].w;
    t_pos[d] = pos[s];
    t_x[d] = x4[s];
    t_id[d] = id[s];
    t_attr[d] = attr[s];
    t_dens[d] = dens[s];
}

/* Copy the temporaries back; x* also becomes the new build reference xb. */
__global__ void k_rebuild_copy(int n, DevCtl *ctl, const float4 *__restrict__ t_pos, const float4 *__restrict__ t_x,
                               const unsigned int *__restrict__ t_id, const unsigned int *__restrict__ t_attr,
                               const float *__restrict__ t_dens, float4 *__restrict__ pos, float4 *ppos0,
                               float4 *ppos1, float4 *__restrict__ xb, unsigned int *__restrict__ id,
                               unsigned int *__restrict__ attr, float *__restrict__ dens,
                               const float4 *__restrict__ t_xpred, float4 *__restrict__ xpred,
                               const float *__restrict__ t_lam) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned int par = ctl->parity;
    if (d == 0) {
        ctl->builds += 1u;
        ctl->rebuild = 0u;
    }
    if (d >= n) return;
    if (xpred) xpred[d] = t_xpred[d];
    if (t_lam) (par ? ppos0 : ppos1)[d].w = t_lam[d];
    float4 *x4 = par ? ppos1 : ppos0;
    pos[d] = t_pos[d];
    float4 x = t_x[d];
    x4[d] = x;
    xb[d] = x;
    id[d] = t_id[d];
    attr[d] = t_attr[d];
    dens[d] = t_dens[d];
}

/* ======================================================================== */
/* neighbour lists                                                          */
/* ======================================================================== */

/* Every slot j within the list radius (= the cell width) of slot i at the
 * build positions xb, self included, as (row << 12) | (j - row_start). */
__global__ void k_build_list(DevParams p, const unsigned int *__restrict__ cell_start,
                             const float4 *__restrict__ xb, const unsigned int *__restrict__ cellb,
                             unsigned short *__restrict__ list, unsigned char *__restrict__ cnt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const float3 xi = f3(xb[i]);
    const int cb = (int)cellb[i];
    int k = 0;
    bool ovf = false;
#pragma unroll 1
    for (int r = 0; r < 9; ++r) {
        const int base = cb + ((r / 3 - 1) * p.gy + (r % 3 - 1)) * p.gx;
        const unsigned int s = __ldg(cell_start + base - 1), e = __ldg(cell_start + base + 2);
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
                    if (k < kListMax) list[(size_t)k * p.n + i] = (unsigned short)((r << 12) | (j0 + u - s));
                    ++k;
                }
            }
        }
    }
    cnt[i] = (ovf || k > kListMax) ? kListOverflow : (unsigned char)k;
}

/* Calls f(j, x[j]) for every candidate slot j of slot i: its list entries,
 * or -- for an overflowed list or when lists are off -- every slot of the 27
 * cells around the current position.  List entries are taken kBatch at a
 * time: their indices are decoded and their positions loaded before any is
 * used, so each thread keeps kBatch independent loads in flight (the passes
 * are bound by load latency, not by arithmetic).  rs: this thread's 9 row
 * starts in shared memory, strided by the block size.  Load selects the
 * load flavour for x. */
constexpr int kBatch = 4;

template <class Load, class F>
__device__ __forceinline__ void for_each_candidate(const DevParams &p, const unsigned int *__restrict__ cell_start,
                                                   const unsigned short *__restrict__ list,
                                                   const unsigned char *__restrict__ cnt,
                                                   const unsigned int *__restrict__ cellb, int i, float3 xi,
                                                   unsigned int *rs, Load &&load, F &&f) {
    const int k = list ? (int)cnt[i] : (int)kListOverflow;
    if (k != (int)kListOverflow) {
        const int cb = (int)cellb[i];
#pragma unroll
        for (int r = 0; r < 9; ++r) {
            const int base = cb + ((r / 3 - 1) * p.gy + (r % 3 - 1)) * p.gx;
            rs[r * blockDim.x] = __ldg(cell_start + base - 1);
        }
        for (int t0 = 0; t0 < k; t0 += kBatch) {
            unsigned int j[kBatch];
            float4 xj[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; ++u) {
                const int t = t0 + u < k ? t0 + u : k - 1;
                const unsigned int e = __ldg(list + (size_t)t * p.n + i);
                j[u] = rs[(e >> 12) * blockDim.x] + (e & 0xfffu);
            }
#pragma unroll
            for (int u = 0; u < kBatch; ++u) xj[u] = load(j[u]);
#pragma unroll
            for (int u = 0; u < kBatch; ++u)
                if (t0 + u < k) f(j[u], xj[u]);
        }
    } else {
        const int3 c = cell_of(xi, p);
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy) {
                unsigned int s, e;
                row_range(cell_start, c, dy, dz, p, s, e);
                for (unsigned int j = s; j < e; ++j) f(j, load(j));
            }
    }
}

/* ======================================================================== */
/* PBF                                                                      */
/* ======================================================================== */

/* rho_i = m aw sum_j (h^2 - r^2)^3 over r < h, self included. */
__global__ void k_pbf_density(DevParams p, const unsigned int *__restrict__ cell_start,
                              const float4 *__restrict__ pos, float *__restrict__ dens) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    float3 xi = f3(pos[i]);
    int3 c = cell_of(xi, p);
    float acc = 0.0f;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy) {
            unsigned int s, e;
            row_range(cell_start, c, dy, dz, p, s, e);
            for (unsigned int j = s; j < e; ++j) {
                float3 d = xi - f3(__ldg(pos + j));
                float r2 = dot3(d, d);
                if (r2 < p.h2) {
                    float q = p.h2 - r2;
                    acc += q * q * q;
                }
            }
        }
    dens[i] = p.mass * p.aw * acc;
}

/* a_i = mu sum_{j != i} m (v_j - v_i) / rho_i lapW + g (rx_sph_pbd.cpp:651-689). */
__global__ void k_pbf_visc(DevParams p, const unsigned int *__restrict__ cell_start, const float4 *__restrict__ pos,
                           const float4 *__restrict__ vel, const float *__restrict__ dens,
                           float4 *__restrict__ acc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    float3 xi = f3(pos[i]), vi = f3(vel[i]);
    int3 c = cell_of(xi, p);
    float3 f = make_float3(0.f, 0.f, 0.f);
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy) {
            unsigned int s, e;
            row_range(cell_start, c, dy, dz, p, s, e);
            for (unsigned int j = s; j < e; ++j) {
                if (j == (unsigned int)i) continue;
                float3 d = xi - f3(__ldg(pos + j));
                float r2 = dot3(d, d);
                if (r2 < p.h2 && r2 > 0.0f) {
                    float r = sqrtf(r2);
                    float lw = p.al * (p.h - r);
                    f = f + lw * (f3(__ldg(vel + j)) - vi);
                }
            }
        }
    float k = p.viscosity * p.mass / dens[i];
    float3 a = k * f + p.gravity;
    acc[i] = make_float4(a.x, a.y, a.z, 0.0f);
}

/* lambda pass: density, C, sum |grad C|^2 (with the k = i term), lambda
 * into x*.w, block partial errors; the last block reduces the errors in a
 * fixed order, advances the iteration counter and decides whether the
 * device-side loop continues. */
__global__ void __launch_bounds__(kBlock) k_lambda(DevParams p, const unsigned int *__restrict__ cell_start,
                                                   float4 *ppos0, float4 *ppos1, float *__restrict__ dens,
                                                   DevCtl *ctl, ErrPartial *part,
                                                   cudaGraphConditionalHandle hwhile, int use_graph,
                                                   const unsigned short *__restrict__ list,
                                                   const unsigned char *__restrict__ cnt,
                                                   const unsigned int *__restrict__ cellb) {
    __shared__ float sh1[kBlock / 32], sh2[kBlock / 32], shm[kBlock / 32];
    __shared__ unsigned int s_rs[9 * kBlock];
    __shared__ int s_last;
    const unsigned int par = *((volatile unsigned int *)&ctl->parity);
    float4 *pp = par ? ppos1 : ppos0;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float e1 = 0.f, e2 = 0.f, em = 0.f;
    if (i < p.n) {
        const float3 xi = f3(pp[i]);
        float wsum = 0.f, sd = 0.f;
        float3 gs = make_float3(0.f, 0.f, 0.f);
        const float agr = p.ag * p.inv_rest_dens;
        /* plain (L1-cached) loads: only the .w words of pp are written by this
         * kernel, and the neighbour loop reads x, y, z */
        for_each_candidate(
            p, cell_start, list, cnt, cellb, i, xi, s_rs + threadIdx.x, [&](unsigned int j) { return pp[j]; },
            [&](unsigned int, const float4 &xj4) {
                /* branch-free: outside h both q and t clamp to zero; the self
                 * pair (d = 0) adds W(0) to the density and nothing else */
                const float3 d = xi - f3(xj4);
                const float r2 = dot3(d, d);
                const float q = fmaxf(p.h2 - r2, 0.0f);
                const float inv_r = rsqrtf(fmaxf(r2, 1e-20f));
                const float t = fmaxf(p.h - r2 * inv_r, 0.0f);
                const float g = agr * t * t * inv_r; /* grad W / rho0 = g d */
                wsum += q * q * q;
                gs = gs + g * d;
                sd += g * g * r2;
            });
        float rho = p.mass * p.aw * wsum;
        sd += dot3(gs, gs);
        float C = rho * p.inv_rest_dens - 1.0f;
        float Cc = (p.clamp_constraint && C < 0.0f) ? 0.0f : C;
        float lam = -Cc / (sd + p.epsilon);
        reinterpret_cast<float *>(pp + i)[3] = lam;
        dens[i] = rho;
        e1 = C > 0.0f ? C : 0.0f;
        e2 = fabsf(C);
        em = e2;
        if (!(rho == rho)) ctl->nan_flag = 1u;
    }
    e1 = warp_sum(e1);
    e2 = warp_sum(e2);
    em = warp_max(em);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { sh1[warp] = e1; sh2[warp] = e2; shm[warp] = em; }
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.f, b = 0.f, m = 0.f;
        for (int w = 0; w < kBlock / 32; ++w) { a += sh1[w]; b += sh2[w]; m = fmaxf(m, shm[w]); }
        part[blockIdx.x] = ErrPartial{a, b, m, 0.f};
        __threadfence();
        unsigned int t = atomicAdd(&ctl->ticket, 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    /* fixed-order reduction of the block partials (double) */
    __shared__ double r1[kBlock], r2s[kBlock];
    __shared__ float rm[kBlock];
    double a = 0.0, b = 0.0;
    float m = 0.f;
    for (unsigned int k = threadIdx.x; k < gridDim.x; k += blockDim.x) {
        float4 v = __ldcg(reinterpret_cast<const float4 *>(part) + k);
        a += v.x; b += v.y; m = fmaxf(m, v.z);
    }
    r1[threadIdx.x] = a; r2s[threadIdx.x] = b; rm[threadIdx.x] = m;
    __syncthreads();
    for (int o = kBlock / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            r1[threadIdx.x] += r1[threadIdx.x + o];
            r2s[threadIdx.x] += r2s[threadIdx.x + o];
            rm[threadIdx.x] = fmaxf(rm[threadIdx.x], rm[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        float err1 = (float)(r1[0] / (double)p.n);
        float err2 = (float)(r2s[0] / (double)p.n);
        ctl->err1 = err1;
        ctl->err2 = err2;
        ctl->errmax = rm[0];
        unsigned int it = ctl->iter + 1u;
        ctl->iter = it;
        float err = p.error_mode ? err2 : err1;
        int minit = p.min_iter > 1 ? p.min_iter : 1;
        int cont = ((int)it < p.max_iter) && !(err <= p.eta && (int)it >= minit);
        if (ctl->nan_flag) cont = 0;
        ctl->done = cont ? 0u : 1u;
        ctl->ticket = 0u;
        if (use_graph & 1) cudaGraphSetConditional(hwhile, cont ? 1u : 0u);
    }
}

/* correction pass: dp_i = sum_j (lambda_i + lambda_j + s_corr) grad W_ij / rho0,
 * x*_i <- walls(x*_i + dp_i) into the other ping-pong buffer; the largest
 * displacement since the last grid build decides whether the grid must be
 * rebuilt before the next pass. */
__global__ void __launch_bounds__(kBlock) k_correction(DevParams p, const unsigned int *__restrict__ cell_start,
                                                       float4 *ppos0, float4 *ppos1,
                                                       const float4 *__restrict__ xb, DevCtl *ctl, float *part,
                                                       cudaGraphConditionalHandle hif,
                                                       cudaGraphConditionalHandle hif2, int use_graph,
                                                       float4 *__restrict__ dp_out,
                                                       const unsigned short *__restrict__ list,
                                                       const unsigned char *__restrict__ cnt,
                                                       const unsigned int *__restrict__ cellb) {
    __shared__ float shm[kBlock / 32];
    __shared__ unsigned int s_rs[9 * kBlock];
    __shared__ int s_last;
    const unsigned int par = *((volatile unsigned int *)&ctl->parity);
    const float4 *__restrict__ src = par ? ppos1 : ppos0;
    float4 *__restrict__ dst = par ? ppos0 : ppos1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float disp2 = 0.f;
    if (i < p.n) {
        const float4 xi4 = src[i];
        const float3 xi = f3(xi4);
        const float li = xi4.w;
        float3 acc = make_float3(0.f, 0.f, 0.f);
        const float k_dt2 = -p.ap_k * p.dt * p.dt;
        const float agr = p.ag * p.inv_rest_dens;
        const float awq = p.aw * p.inv_wq;
        for_each_candidate(
            p, cell_start, list, cnt, cellb, i, xi, s_rs + threadIdx.x, [&](unsigned int j) { return __ldg(src + j); },
            [&](unsigned int, const float4 &xj4) {
                /* branch-free: t = 0 outside h and d = 0 for the self pair */
                const float3 d = xi - f3(xj4);
                const float r2 = dot3(d, d);
                const float inv_r = rsqrtf(fmaxf(r2, 1e-20f));
                const float t = fmaxf(p.h - r2 * inv_r, 0.0f);
                const float g = agr * t * t * inv_r;
                float sc = 0.0f;
                if (p.use_ap) {
                    const float q = fmaxf(p.h2 - r2, 0.0f);
                    const float ww = awq * q * q * q;
                    const float pw = (p.ap_n == 4.0f) ? (ww * ww) * (ww * ww) : __powf(ww, p.ap_n);
                    sc = k_dt2 * pw;
                }
                acc = acc + ((li + xj4.w + sc) * g) * d;
            });
        if (dp_out) dp_out[i] = make_float4(acc.x, acc.y, acc.z, 0.0f);
        float3 xn = wall_project(xi + acc, p);
        dst[i] = make_float4(xn.x, xn.y, xn.z, 0.0f);
        float3 dd = xn - f3(xb[i]);
        disp2 = dot3(dd, dd);
        if (!(xn.x == xn.x && xn.y == xn.y && xn.z == xn.z)) ctl->nan_flag = 1u;
    }
    disp2 = warp_max(disp2);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) shm[warp] = disp2;
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = 0.f;
        for (int w = 0; w < kBlock / 32; ++w) m = fmaxf(m, shm[w]);
        part[blockIdx.x] = m;
        __threadfence();
        unsigned int t = atomicAdd(&ctl->ticket2, 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    __shared__ float rm[kBlock];
    float m = 0.f;
    for (unsigned int k = threadIdx.x; k < gridDim.x; k += blockDim.x) m = fmaxf(m, __ldcg(part + k));
    rm[threadIdx.x] = m;
    __syncthreads();
    for (int o = kBlock / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) rm[threadIdx.x] = fmaxf(rm[threadIdx.x], rm[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        float md = rm[0];
        ctl->disp2_bits = __float_as_uint(md);
        unsigned int rb = (md > p.skin2 || !(md == md)) ? 1u : 0u;
        ctl->rebuild = rb;
        ctl->parity = 1u - par;
        ctl->ticket2 = 0u;
        if (use_graph & 1) {
            unsigned int more = ctl->done ? 0u : 1u;
            cudaGraphSetConditional(hif, rb & more);
            if (use_graph & 2) cudaGraphSetConditional(hif2, rb);
        }
    }
}

/* v = (x* - x) / dt, x = x* (rx_sph_pbd.cpp:464-471); also brings id / attr
 * back to the step's home buffers. */
__global__ void k_finalize(DevParams p, const float4 *__restrict__ pos_b, const float4 *ppos0,
                           const float4 *ppos1, const DevCtl *ctl, const unsigned int *__restrict__ id_b,
                           const unsigned int *__restrict__ attr_b, float4 *__restrict__ pos_a,
                           float4 *__restrict__ vel_a, unsigned int *__restrict__ id_a,
                           unsigned int *__restrict__ attr_a, const float4 *__restrict__ xpred,
                           float4 *__restrict__ dstep) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const float4 *pp = ctl->parity ? ppos1 : ppos0;
    float3 xs = f3(pp[i]);
    float3 x = f3(pos_b[i]);
    float3 v = p.inv_dt * (xs - x);
    pos_a[i] = make_float4(xs.x, xs.y, xs.z, 0.0f);
    vel_a[i] = make_float4(v.x, v.y, v.z, 0.0f);
    id_a[i] = id_b[i];
    attr_a[i] = attr_b[i];
    /* total correction of this step, x*_final - x*_predicted */
    if (dstep) {
        float3 dd = xs - f3(xpred[i]);
        dstep[i] = make_float4(dd.x, dd.y, dd.z, 0.0f);
    }
}

/* omega_i = sum_j (v_j - v_i) x grad_j W_ij (grad_j = -grad_i), and the
 * XSPH update v_i + c sum_j (m / rho_j)(v_j - v_i) W_ij. */
__global__ void __launch_bounds__(kBlock) k_xsph_vort(DevParams p, const unsigned int *__restrict__ cell_start,
                                                      const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                                                      const float *__restrict__ dens, float4 *__restrict__ vel_out,
                                                      float4 *__restrict__ vort, FeatureOut fo,
                                                      const unsigned short *__restrict__ list,
                                                      const unsigned char *__restrict__ cnt,
                                                      const unsigned int *__restrict__ cellb) {
    __shared__ unsigned int s_rs[9 * kBlock];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const float3 xi = f3(pos[i]), vi = f3(vel[i]);
    float3 om = make_float3(0.f, 0.f, 0.f), xs = make_float3(0.f, 0.f, 0.f);
    float3 off = make_float3(0.f, 0.f, 0.f), cg = make_float3(0.f, 0.f, 0.f);
    float div = 0.f, cntf = 0.f;
    /* branch-free pair terms: q and t clamp to zero outside h, and the self
     * pair (d = 0, v_ij = 0) adds only to the neighbour count */
    for_each_candidate(
        p, cell_start, list, cnt, cellb, i, xi, s_rs + threadIdx.x, [&](unsigned int j) { return __ldg(pos + j); },
        [&](unsigned int j, const float4 &xj4) {
            const float3 d = xi - f3(xj4);
            const float r2 = dot3(d, d);
            const float inside = r2 < p.h2 ? 1.0f : 0.0f;
            const float q = fmaxf(p.h2 - r2, 0.0f);
            const float inv_r = rsqrtf(fmaxf(r2, 1e-20f));
            const float t = fmaxf(p.h - r2 * inv_r, 0.0f);
            const float g = p.ag * t * t * inv_r;
            const float3 vij = f3(__ldg(vel + j)) - vi;
            const float mrho = p.mass / __ldg(dens + j);
            om = om + cross3(vij, (-g) * d);
            xs = xs + (p.aw * q * q * q * mrho) * vij;
            cntf += inside;
            off = off - inside * d;
            div += mrho * g * dot3(vij, d);
            cg = cg + (mrho * g) * d;
        });
    cntf = fmaxf(cntf, 1.0f);
    float3 vn = vi + p.xsph_c * xs;
    vel_out[i] = make_float4(vn.x, vn.y, vn.z, 0.0f);
    vort[i] = make_float4(om.x, om.y, om.z, 0.0f);
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
        f[12] = div * p.dt;
        f[13] = cg.x * p.h; f[14] = cg.y * p.h; f[15] = cg.z * p.h;
        float4 *out = reinterpret_cast<float4 *>(fo.feat + (size_t)i * kFeatures);
#pragma unroll
        for (int k = 0; k < kFeatures / 4; ++k) out[k] = make_float4(f[4 * k], f[4 * k + 1], f[4 * k + 2], f[4 * k + 3]);
        if (i == 0) *fo.valid = 1u;
    }
}

/* eta_i = sum_j (m / rho_j)(|w_j| - |w_i|) grad_i W_ij; f = eps (eta/|eta|) x w_i;
 * v_i <- v_i + dt f. */
__global__ void __launch_bounds__(kBlock) k_vort_apply(DevParams p, const unsigned int *__restrict__ cell_start,
                                                       const float4 *__restrict__ pos,
                                                       const float4 *__restrict__ vort,
                                                       const float *__restrict__ dens,
                                                       const float4 *__restrict__ vel_in,
                                                       float4 *__restrict__ vel_out,
                                                       const unsigned short *__restrict__ list,
                                                       const unsigned char *__restrict__ cnt,
                                                       const unsigned int *__restrict__ cellb) {
    __shared__ unsigned int s_rs[9 * kBlock];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    float4 v4 = vel_in[i];
    if (p.vort_eps != 0.0f) {
        const float3 xi = f3(pos[i]);
        const float3 wi = f3(vort[i]);
        const float wmi = sqrtf(dot3(wi, wi));
        float3 eta = make_float3(0.f, 0.f, 0.f);
        for_each_candidate(
            p, cell_start, list, cnt, cellb, i, xi, s_rs + threadIdx.x, [&](unsigned int j) { return __ldg(pos + j); },
            [&](unsigned int j, const float4 &xj4) {
                const float3 d = xi - f3(xj4);
                const float r2 = dot3(d, d);
                const float inv_r = rsqrtf(fmaxf(r2, 1e-20f));
                const float t = fmaxf(p.h - r2 * inv_r, 0.0f);
                const float g = p.ag * t * t * inv_r;
                const float3 wj = f3(__ldg(vort + j));
                const float k = p.mass / __ldg(dens + j) * (sqrtf(dot3(wj, wj)) - wmi) * g;
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

/* ======================================================================== */
/* WCSPH                                                                    */
/* ======================================================================== */

__global__ void k_sph_density(DevParams p, const unsigned int *__restrict__ cell_start,
                              const float4 *__restrict__ pos, float *__restrict__ dens, float *__restrict__ pres) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    float3 xi = f3(pos[i]);
    int3 c = cell_of(xi, p);
    float acc = 0.0f;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy) {
            unsigned int s, e;
            row_range(cell_start, c, dy, dz, p, s, e);
            for (unsigned int j = s; j < e; ++j) {
                float3 d = xi - f3(__ldg(pos + j));
                float r2 = dot3(d, d);
                if (r2 < p.h2) {
                    float q = p.h2 - r2;
                    acc += q * q * q;
                }
            }
        }
    float rho = p.mass * p.aw * acc;
    dens[i] = rho;
    pres[i] = p.gas_k * (rho - p.rest_dens);
}

__global__ void k_sph_force(DevParams p, const unsigned int *__restrict__ cell_start, const float4 *__restrict__ pos,
                            const float4 *__restrict__ vel, const float *__restrict__ dens,
                            const float *__restrict__ pres, float4 *__restrict__ acc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    float3 xi = f3(pos[i]), vi = f3(vel[i]);
    float rhoi = dens[i];
    float prsi = pres[i] / (rhoi * rhoi);
    int3 c = cell_of(xi, p);
    float3 fp = make_float3(0.f, 0.f, 0.f), fv = make_float3(0.f, 0.f, 0.f);
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy) {
            unsigned int s, e;
            row_range(cell_start, c, dy, dz, p, s, e);
            for (unsigned int j = s; j < e; ++j) {
                if (j == (unsigned int)i) continue;
                float3 d = xi - f3(__ldg(pos + j));
                float r2 = dot3(d, d);
                if (r2 < p.h2 && r2 > 0.0f) {
                    float r = sqrtf(r2);
                    float t = p.h - r;
                    float rhoj = __ldg(dens + j);
                    float prsj = __ldg(pres + j) / (rhoj * rhoj);
                    float g = p.ag * t * t / r;
                    fp = fp + ((prsi + prsj) * g) * d;
                    float lw = p.al * t / rhoj;
                    fv = fv + lw * (f3(__ldg(vel + j)) - vi);
                }
            }
        }
    float3 a = (-p.mass) * fp + (p.viscosity * p.mass) * fv + p.gravity;
    acc[i] = make_float4(a.x, a.y, a.z, 0.0f);
}

__global__ void k_sph_integrate(DevParams p, const float4 *__restrict__ pos_b, const float4 *__restrict__ vel_b,
                                const float4 *__restrict__ acc, const unsigned int *__restrict__ id_b,
                                const unsigned int *__restrict__ attr_b, float4 *__restrict__ pos_a,
                                float4 *__restrict__ vel_a, unsigned int *__restrict__ id_a,
                                unsigned int *__restrict__ attr_a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    float3 v = f3(vel_b[i]) + p.dt * f3(acc[i]);
    float3 x = f3(pos_b[i]) + p.dt * v;
    x = wall_project(x, p);
    pos_a[i] = make_float4(x.x, x.y, x.z, 0.0f);
    vel_a[i] = make_float4(v.x, v.y, v.z, 0.0f);
    id_a[i] = id_b[i];
    attr_a[i] = attr_b[i];
}

/* ======================================================================== */
/* neighbour sets, reference criterion                                      */
/* ======================================================================== */

/* fl32(|xi - xj|^2 in double) <= fl32(h*h) (rx_nnsearch.h:499-507): a float
 * test decides unless the float distance lies within 1e-5 of h^2, where the
 * double evaluation (separate multiplies and adds, no fusion) decides. */
__device__ inline bool ref_neighbor(float3 xi, float3 xj, float h2) {
    float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
    float d2 = dx * dx + dy * dy + dz * dz;
    if (d2 < h2 * (1.0f - 1e-5f)) return true;
    if (d2 > h2 * (1.0f + 1e-5f)) return false;
    double ex = (double)xi.x - (double)xj.x, ey = (double)xi.y - (double)xj.y, ez = (double)xi.z - (double)xj.z;
    double dd = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
    return __double2float_rn(dd) <= h2;
}

__global__ void k_nb_count(DevParams p, const unsigned int *__restrict__ cell_start, const float4 *__restrict__ pos,
                           unsigned int *__restrict__ cnt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    float3 xi = f3(pos[i]);
    int3 c = cell_of(xi, p);
    unsigned int k = 0;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy) {
            unsigned int s, e;
            row_range(cell_start, c, dy, dz, p, s, e);
            for (unsigned int j = s; j < e; ++j)
                if (ref_neighbor(xi, f3(pos[j]), p.h2)) ++k;
        }
    cnt[i] = k;
}

__global__ void k_nb_fill(DevParams p, const unsigned int *__restrict__ cell_start, const float4 *__restrict__ pos,
                          const unsigned int *__restrict__ id, const unsigned int *__restrict__ offsets,
                          int *__restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    float3 xi = f3(pos[i]);
    int3 c = cell_of(xi, p);
    unsigned int k = offsets[i];
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy) {
            unsigned int s, e;
            row_range(cell_start, c, dy, dz, p, s, e);
            for (unsigned int j = s; j < e; ++j)
                if (ref_neighbor(xi, f3(pos[j]), p.h2)) out[k++] = (int)id[j];
        }
}

/* ======================================================================== */
/* order conversion                                                         */
/* ======================================================================== */

__global__ void k_unsort4(int n, const unsigned int *__restrict__ id, const float4 *__restrict__ src,
                          float4 *__restrict__ dst, int zero_w) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    float4 v = src[d];
    if (zero_w) v.w = 0.0f;
    dst[id[d]] = v;
}
__global__ void k_unsort1(int n, const unsigned int *__restrict__ id, const unsigned int *__restrict__ src,
                          unsigned int *__restrict__ dst) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    dst[id[d]] = src[d];
}
__global__ void k_unsort_w(int n, const unsigned int *__restrict__ id, const float4 *__restrict__ src,
                           float *__restrict__ dst) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    dst[id[d]] = src[d].w;
}
__global__ void k_unsort_rows(int n, const unsigned int *__restrict__ id, const float4 *__restrict__ src,
                              float4 *__restrict__ dst, int k4) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * k4) return;
    int d = e / k4, q = e % k4;
    dst[(size_t)id[d] * k4 + q] = src[e];
}
void launch_unsort_rows(int n, const unsigned int *id, const float4 *src, float4 *dst, int k4, cudaStream_t s) {
    k_unsort_rows<<<blocks_for((long long)n * k4), kBlock, 0, s>>>(n, id, src, dst, k4);
}
__global__ void k_iota(int n, unsigned int *dst) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d < n) dst[d] = (unsigned int)d;
}
__global__ void k_check_finite(int n, const float4 *__restrict__ a, const float4 *__restrict__ b,
                               unsigned int *flag) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    float4 x = a[d];
    bool ok = isfinite(x.x) && isfinite(x.y) && isfinite(x.z);
    if (b) {
        float4 v = b[d];
        ok = ok && isfinite(v.x) && isfinite(v.y) && isfinite(v.z);
    }
    if (!ok) atomicOr(flag, 1u);
}
void launch_check_finite(int n, const float4 *a, const float4 *b, unsigned int *flag, cudaStream_t s) {
    k_check_finite<<<blocks_for(n), kBlock, 0, s>>>(n, a, b, flag);
}
__global__ void k_pack_w(int n, float4 *dst, const float *w) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d < n) dst[d].w = w[d];
}

/* ======================================================================== */
/* launchers                                                                */
/* ======================================================================== */

void launch_predict_hash(const DevParams &p, const float4 *pos, const float4 *vel, const float4 *acc,
                         float4 *ppos_out, unsigned int *key, unsigned int *rank, unsigned int *count,
                         const float4 *dwarm, float4 *xpred_out, cudaStream_t s) {
    k_predict_hash<<<blocks_for(p.n), kBlock, 0, s>>>(p, pos, vel, acc, ppos_out, key, rank, count, dwarm,
                                                      xpred_out);
}
void launch_hash(const DevParams &p, const float4 *x, unsigned int *key, unsigned int *rank, unsigned int *count,
                 cudaStream_t s) {
    k_hash<<<blocks_for(p.n), kBlock, 0, s>>>(p, x, key, rank, count);
}
void launch_scan(unsigned int *count, unsigned int *cell_start, unsigned int *block_sums, unsigned int ncells,
                 cudaStream_t s) {
    unsigned int nb = scan_blocks(ncells);
    k_scan_local<<<nb, 1024, 0, s>>>(count, cell_start, block_sums, ncells);
    k_scan_top<<<1, 1024, 0, s>>>(block_sums, nb, cell_start, ncells);
    k_scan_add<<<blocks_for(ncells, 1024), 1024, 0, s>>>(cell_start, block_sums, ncells);
}
void launch_scatter_sort(const DevParams &p, const unsigned int *key, const unsigned int *rank,
                         const unsigned int *cell_start, unsigned int *perm, unsigned int ncells, cudaStream_t s) {
    k_scatter<<<blocks_for(p.n), kBlock, 0, s>>>(p.n, key, rank, cell_start, perm);
    k_cell_sort<<<blocks_for(ncells), kBlock, 0, s>>>(cell_start, perm, ncells);
}
void launch_gather(int n, const unsigned int *perm, const Gather &g, DevCtl *count_build, cudaStream_t s) {
    k_gather<<<blocks_for(n), kBlock, 0, s>>>(n, perm, g, count_build);
}
void launch_hash_parity(const DevParams &p, const float4 *ppos0, const float4 *ppos1, const DevCtl *ctl,
                        unsigned int *key, unsigned int *rank, unsigned int *count, cudaStream_t s) {
    k_hash_parity<<<blocks_for(p.n), kBlock, 0, s>>>(p, ppos0, ppos1, ctl, key, rank, count);
}
void launch_rebuild_gather(int n, const unsigned int *perm, const DevCtl *ctl, const float4 *pos, const float4 *ppos0,
                           const float4 *ppos1, const unsigned int *id, const unsigned int *attr, const float *dens,
                           float4 *t_pos, float4 *t_x, unsigned int *t_id, unsigned int *t_attr, float *t_dens,
                           const unsigned int *key, unsigned int *cellb, const float4 *xpred, float4 *t_xpred,
                           float *t_lam, cudaStream_t s) {
    k_rebuild_gather<<<blocks_for(n), kBlock, 0, s>>>(n, perm, ctl, pos, ppos0, ppos1, id, attr, dens, t_pos, t_x,
                                                      t_id, t_attr, t_dens, key, cellb, xpred, t_xpred, t_lam);
}
void launch_rebuild_copy(int n, DevCtl *ctl, const float4 *t_pos, const float4 *t_x, const unsigned int *t_id,
                         const unsigned int *t_attr, const float *t_dens, float4 *pos, float4 *ppos0, float4 *ppos1,
                         float4 *xb, unsigned int *id, unsigned int *attr, float *dens, const float4 *t_xpred,
                         float4 *xpred, const float *t_lam, cudaStream_t s) {
    k_rebuild_copy<<<blocks_for(n), kBlock, 0, s>>>(n, ctl, t_pos, t_x, t_id, t_attr, t_dens, pos, ppos0, ppos1, xb,
                                                    id, attr, dens, t_xpred, xpred, t_lam);
}
void launch_pbf_density(const DevParams &p, const unsigned int *cell_start, const float4 *pos, float *dens,
                        cudaStream_t s) {
    k_pbf_density<<<blocks_for(p.n), kBlock, 0, s>>>(p, cell_start, pos, dens);
}
void launch_pbf_visc(const DevParams &p, const unsigned int *cell_start, const float4 *pos, const float4 *vel,
                     const float *dens, float4 *acc, cudaStream_t s) {
    k_pbf_visc<<<blocks_for(p.n), kBlock, 0, s>>>(p, cell_start, pos, vel, dens, acc);
}
void launch_lambda(const DevParams &p, const unsigned int *cell_start, float4 *ppos0, float4 *ppos1, float *dens,
                   DevCtl *ctl, ErrPartial *part, unsigned long long while_handle, int use_graph,
                   const NbrLists &nl, cudaStream_t s) {
    k_lambda<<<blocks_for(p.n), kBlock, 0, s>>>(p, cell_start, ppos0, ppos1, dens, ctl, part,
                                                (cudaGraphConditionalHandle)while_handle, use_graph,
                                                p.use_lists ? nl.list : nullptr, nl.cnt, nl.cellb);
}
void launch_build_list(const DevParams &p, const unsigned int *cell_start, const float4 *xb, const NbrLists &nl,
                       cudaStream_t s) {
    if (!p.use_lists) return;
    k_build_list<<<blocks_for(p.n), kBlock, 0, s>>>(p, cell_start, xb, nl.cellb, nl.list, nl.cnt);
}
void launch_correction(const DevParams &p, const unsigned int *cell_start, float4 *ppos0, float4 *ppos1,
                       const float4 *xb, DevCtl *ctl, float *part, unsigned long long if_handle,
                       unsigned long long if_handle2, int use_graph, float4 *dp_out, const NbrLists &nl,
                       cudaStream_t s) {
    k_correction<<<blocks_for(p.n), kBlock, 0, s>>>(p, cell_start, ppos0, ppos1, xb, ctl, part,
                                                    (cudaGraphConditionalHandle)if_handle,
                                                    (cudaGraphConditionalHandle)if_handle2, use_graph, dp_out,
                                                    p.use_lists ? nl.list : nullptr, nl.cnt, nl.cellb);
}
void launch_finalize(const DevParams &p, const float4 *pos_b, const float4 *ppos0, const float4 *ppos1,
                     const DevCtl *ctl, const unsigned int *id_b, const unsigned int *attr_b, float4 *pos_a,
                     float4 *vel_a, unsigned int *id_a, unsigned int *attr_a, const float4 *xpred, float4 *dstep,
                     cudaStream_t s) {
    k_finalize<<<blocks_for(p.n), kBlock, 0, s>>>(p, pos_b, ppos0, ppos1, ctl, id_b, attr_b, pos_a, vel_a, id_a,
                                                  attr_a, xpred, dstep);
}
void launch_xsph_vort(const DevParams &p, const unsigned int *cell_start, const float4 *pos, const float4 *vel,
                      const float *dens, float4 *vel_out, float4 *vort, const FeatureOut &fo, const NbrLists &nl,
                      cudaStream_t s) {
    k_xsph_vort<<<blocks_for(p.n), kBlock, 0, s>>>(p, cell_start, pos, vel, dens, vel_out, vort, fo,
                                                   p.use_lists ? nl.list : nullptr, nl.cnt, nl.cellb);
}
void launch_vort_apply(const DevParams &p, const unsigned int *cell_start, const float4 *pos, const float4 *vort,
                       const float *dens, const float4 *vel_in, float4 *vel_out, const NbrLists &nl, cudaStream_t s) {
    k_vort_apply<<<blocks_for(p.n), kBlock, 0, s>>>(p, cell_start, pos, vort, dens, vel_in, vel_out,
                                                    p.use_lists ? nl.list : nullptr, nl.cnt, nl.cellb);
}
void launch_sph_density(const DevParams &p, const unsigned int *cell_start, const float4 *pos, float *dens,
                        float *pres, cudaStream_t s) {
    k_sph_density<<<blocks_for(p.n), kBlock, 0, s>>>(p, cell_start, pos, dens, pres);
}
void launch_sph_force(const DevParams &p, const unsigned int *cell_start, const float4 *pos, const float4 *vel,
                      const float *dens, const float *pres, float4 *acc, cudaStream_t s) {
    k_sph_force<<<blocks_for(p.n), kBlock, 0, s>>>(p, cell_start, pos, vel, dens, pres, acc);
}
void launch_sph_integrate(const DevParams &p, const float4 *pos_b, const float4 *vel_b, const float4 *acc,
                          const unsigned int *id_b, const unsigned int *attr_b, float4 *pos_a, float4 *vel_a,
                          unsigned int *id_a, unsigned int *attr_a, cudaStream_t s) {
    k_sph_integrate<<<blocks_for(p.n), kBlock, 0, s>>>(p, pos_b, vel_b, acc, id_b, attr_b, pos_a, vel_a, id_a,
                                                       attr_a);
}
void launch_nb_count(const DevParams &p, const unsigned int *cell_start, const float4 *pos, unsigned int *cnt,
                     cudaStream_t s) {
    k_nb_count<<<blocks_for(p.n), kBlock, 0, s>>>(p, cell_start, pos, cnt);
}
void launch_nb_fill(const DevParams &p, const unsigned int *cell_start, const float4 *pos, const unsigned int *id,
                    const unsigned int *offsets, int *out, cudaStream_t s) {
    k_nb_fill<<<blocks_for(p.n), kBlock, 0, s>>>(p, cell_start, pos, id, offsets, out);
}
void launch_unsort4(int n, const unsigned int *id, const float4 *src, float4 *dst, int zero_w, cudaStream_t s) {
    k_unsort4<<<blocks_for(n), kBlock, 0, s>>>(n, id, src, dst, zero_w);
}
void launch_unsort1(int n, const unsigned int *id, const unsigned int *src, unsigned int *dst, cudaStream_t s) {
    k_unsort1<<<blocks_for(n), kBlock, 0, s>>>(n, id, src, dst);
}
void launch_unsort_w(int n, const unsigned int *id, const float4 *src, float *dst, cudaStream_t s) {
    k_unsort_w<<<blocks_for(n), kBlock, 0, s>>>(n, id, src, dst);
}
void launch_iota(int n, unsigned int *dst, cudaStream_t s) { k_iota<<<blocks_for(n), kBlock, 0, s>>>(n, dst); }
void launch_pack_w(int n, float4 *dst, const float *w, cudaStream_t s) {
    k_pack_w<<<blocks_for(n), kBlock, 0, s>>>(n, dst, w);
}

}  // namespace fsph
