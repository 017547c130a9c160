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
#include <algorithm>
#include <mutex>

#include "fsph_kernels.cuh"
#include "fsph_passes.cuh"

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
    predict_body(p, i, pos, vel, acc, ppos_out, key, rank, count, dwarm, xpred_out);
}

__global__ void k_hash(DevParams p, const float4 *__restrict__ x4, unsigned int *__restrict__ key,
                       unsigned int *__restrict__ rank, unsigned int *__restrict__ count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    hash_body(p, i, f3(x4[i]), key, rank, count);
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
    hash_body(p, i, f3(x4[i]), key, rank, count);
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
                             ListEntry *__restrict__ list, unsigned char *__restrict__ cnt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    build_list_body(p, i, cell_start, xb, cellb, list, cnt);
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
    float rho = p.mass * p.aw * acc;
    if (p.nb) { /* + sum_b rho0 psi_b W (rx_sph_pbd.cpp:624-644) */
        float bw = 0.f;
        for_each_boundary(p, xi, [&](unsigned int, const float4 &b4) {
            const float3 d = xi - f3(b4);
            const float q = fmaxf(p.h2 - dot3(d, d), 0.0f);
            bw += b4.w * q * q * q;
        });
        rho += p.mass * p.aw * bw;
    }
    dens[i] = rho;
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
template <bool KAHAN>
__global__ void __launch_bounds__(kPassBlock, FSPH_PASS_MINB) k_lambda(DevParams p, const unsigned int *__restrict__ cell_start,
                                                   float4 *ppos0, float4 *ppos1, float *__restrict__ dens,
                                                   DevCtl *ctl, ErrPartial *part,
                                                   cudaGraphConditionalHandle hwhile, int use_graph,
                                                   const ListEntry *__restrict__ list,
                                                   const unsigned char *__restrict__ cnt,
                                                   const unsigned int *__restrict__ cellb) {
    __shared__ unsigned int s_rs[9 * kPassBlock];
    const unsigned int par = *((volatile unsigned int *)&ctl->parity);
    float4 *pp = par ? ppos1 : ppos0;
    float e1 = 0.f, e2 = 0.f, em = 0.f;
#if FSPH_PERSIST_LAMBDA && FSPH_DYN_CHUNKS
    /* persistent warps: whole round-robin rounds, then the leftover chunks
     * on demand; the error sums are fixed point, exact in any order */
    unsigned long long q1 = 0ull, q2 = 0ull;
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5, nchunks = (p.n + 31) >> 5;
    const int stat = max(nchunks / nw - FSPH_DYN_EXTRA, 0) * nw;
    for (int c = first_chunk((blockIdx.x * blockDim.x + threadIdx.x) >> 5, stat, &ctl->grab, lane); c < nchunks;
         c = next_chunk(c, nw, stat, &ctl->grab, lane)) {
        const int i = c * 32 + lane;
        if (i < p.n) {
            const float C = lambda_body<1, KAHAN>(p, cell_start, pp, dens, ctl, list, cnt, cellb, s_rs + threadIdx.x,
                                                  i, 0, true);
            q1 += err_fix(C > 0.0f ? C : 0.0f);
            q2 += err_fix(fabsf(C));
            em = fmaxf(em, fabsf(C));
        }
    }
    (void)e1; (void)e2;
    lambda_tail_fix(p, ctl, part, q1, q2, em, hwhile, use_graph);
}
#else
#if FSPH_PERSIST_LAMBDA
    /* persistent warps: warp w takes the 32-slot chunks w, w + W, ... in a
     * fixed order (the error sums stay deterministic) */
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c * 32 < p.n; c += nw) {
        const int i = c * 32 + lane;
#else
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
#endif
        if (i < p.n) {
            const float C = lambda_body<1, KAHAN>(p, cell_start, pp, dens, ctl, list, cnt, cellb, s_rs + threadIdx.x,
                                                  i, 0, true);
            e1 += C > 0.0f ? C : 0.0f;
            e2 += fabsf(C);
            em = fmaxf(em, fabsf(C));
        }
    }
    lambda_tail(p, ctl, part, e1, e2, em, hwhile, use_graph);
}
#endif

/* correction pass: dp_i = sum_j (lambda_i + lambda_j + s_corr) grad W_ij / rho0,
 * x*_i <- walls(x*_i + dp_i) into the other ping-pong buffer; the largest
 * displacement since the last grid build decides whether the grid must be
 * rebuilt before the next pass. */
__global__ void __launch_bounds__(kPassBlock, FSPH_PASS_MINB) k_correction(DevParams p, const unsigned int *__restrict__ cell_start,
                                                       float4 *ppos0, float4 *ppos1,
                                                       const float4 *__restrict__ xb, DevCtl *ctl, float *part,
                                                       cudaGraphConditionalHandle hif,
                                                       cudaGraphConditionalHandle hif2, int use_graph,
                                                       float4 *__restrict__ dp_out,
                                                       const ListEntry *__restrict__ list,
                                                       const unsigned char *__restrict__ cnt,
                                                       const unsigned int *__restrict__ cellb) {
    __shared__ unsigned int s_rs[9 * kPassBlock];
    const unsigned int par = *((volatile unsigned int *)&ctl->parity);
    const float4 *__restrict__ src = par ? ppos1 : ppos0;
    float4 *__restrict__ dst = par ? ppos0 : ppos1;
    float disp2 = 0.f;
#if FSPH_PERSIST_CORRECTION && FSPH_DYN_CHUNKS
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5, nchunks = (p.n + 31) >> 5, stat = (nchunks / nw) * nw;
    for (int c = first_chunk((blockIdx.x * blockDim.x + threadIdx.x) >> 5, stat, &ctl->grab2, lane); c < nchunks;
         c = next_chunk(c, nw, stat, &ctl->grab2, lane)) {
        const int i = c * 32 + lane;
#elif FSPH_PERSIST_CORRECTION
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c * 32 < p.n; c += nw) {
        const int i = c * 32 + lane;
#else
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
#endif
        if (i < p.n)
            disp2 = fmaxf(disp2, correction_body<1>(p, cell_start, src, dst, xb, ctl, dp_out, list, cnt, cellb,
                                                    s_rs + threadIdx.x, i, 0, true));
    }
    correction_tail(p, ctl, part, disp2, par, hif, hif2, use_graph);
}

/* v = (x* - x) / dt, x = x* (rx_sph_pbd.cpp:464-471); also brings id / attr
 * back to the step's home buffers. */
__global__ void k_finalize(DevParams p, const float4 *__restrict__ pos_b, const float4 *ppos0,
                           const float4 *ppos1, const DevCtl *ctl, const unsigned int *__restrict__ id_b,
                           const unsigned int *__restrict__ attr_b, float4 *__restrict__ pos_a,
                           float4 *__restrict__ vel_a, unsigned int *__restrict__ id_a,
                           unsigned int *__restrict__ attr_a, const float4 *__restrict__ xpred,
                           float4 *__restrict__ dstep, const float *__restrict__ dens, float *__restrict__ mrho) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    if (mrho) mrho[i] = p.mass / dens[i]; /* m / rho_i for the XSPH and vorticity passes */
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
template <bool NBR, bool PRE>
__global__ void __launch_bounds__(kBlock) k_xsph_vort(DevParams p, const unsigned int *__restrict__ cell_start,
                                                      const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                                                      const float *__restrict__ dens, float4 *__restrict__ vel_out,
                                                      float4 *__restrict__ vort, FeatureOut fo,
                                                      const ListEntry *__restrict__ list,
                                                      const unsigned char *__restrict__ cnt,
                                                      const unsigned int *__restrict__ cellb,
                                                      const float *__restrict__ mrho, float2 *__restrict__ wm) {
    __shared__ unsigned int s_rs[9 * kBlock];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    xsph_vort_body<NBR, PRE>(p, i, cell_start, pos, vel, dens, vel_out, vort, fo, list, cnt, cellb,
                             s_rs + threadIdx.x, mrho, wm);
}

/* eta_i = sum_j (m / rho_j)(|w_j| - |w_i|) grad_i W_ij; f = eps (eta/|eta|) x w_i;
 * v_i <- v_i + dt f. */
template <bool PRE>
__global__ void __launch_bounds__(kBlock) k_vort_apply(DevParams p, const unsigned int *__restrict__ cell_start,
                                                       const float4 *__restrict__ pos,
                                                       const float4 *__restrict__ vort,
                                                       const float *__restrict__ dens,
                                                       const float4 *__restrict__ vel_in,
                                                       float4 *__restrict__ vel_out,
                                                       const ListEntry *__restrict__ list,
                                                       const unsigned char *__restrict__ cnt,
                                                       const unsigned int *__restrict__ cellb,
                                                       const float2 *__restrict__ wm) {
    __shared__ unsigned int s_rs[9 * kBlock];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    vort_apply_body<PRE>(p, i, cell_start, pos, vort, dens, vel_in, vel_out, list, cnt, cellb, s_rs + threadIdx.x,
                         wm);
}

/* ======================================================================== */
/* static boundary particles                                                */
/* ======================================================================== */
/* p.n = the boundary count in these kernels; p.bpos etc. the sorted boundary */

/* psi_b = m / sum_b' m W(r_bb') (rx_sph_pbd.cpp:1061-1090); bscale[b] = rho0 psi_b / m */
__global__ void k_boundary_volume(DevParams p, float *__restrict__ bscale) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= p.n) return;
    const float3 xb = f3(__ldg(p.bpos + b));
    float wsum = 0.f;
    for_each_boundary(p, xb, [&](unsigned int, const float4 &c4) {
        const float3 d = xb - f3(c4);
        const float q = fmaxf(p.h2 - dot3(d, d), 0.0f);
        wsum += q * q * q;
    });
    const float mw = p.mass * p.aw * wsum; /* sum_b' m W, self included */
    bscale[b] = p.rest_dens / mw;          /* rho0 psi_b / m = rho0 / (sum m W) */
}

/* The boundary-boundary parts of lambda_b, fixed for a static boundary. */
__global__ void k_boundary_static(DevParams p, float2 *__restrict__ bstat) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= p.n) return;
    const float3 xb = f3(__ldg(p.bpos + b));
    const float agr = p.ag * p.inv_rest_dens;
    float bw = 0.f, sd = 0.f;
    for_each_boundary(p, xb, [&](unsigned int, const float4 &c4) {
        const float3 d = xb - f3(c4);
        const float r2 = dot3(d, d);
        const float q = fmaxf(p.h2 - r2, 0.0f);
        const float inv_r = pair_rsqrt(r2);
        const float t = fmaxf(p.h - r2 * inv_r, 0.0f);
        const float gb = c4.w * agr * t * t * inv_r;
        bw += c4.w * q * q * q;
        sd += gb * gb * r2;
    });
    bstat[b] = make_float2(p.mass * p.aw * bw, sd);
}

__global__ void k_boundary_near(DevParams p, unsigned int ncells, unsigned char *__restrict__ bnear) {
    unsigned int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    const int x = (int)(c % (unsigned int)p.gx), y = (int)((c / (unsigned int)p.gx) % (unsigned int)p.gy),
              z = (int)(c / ((unsigned int)p.gx * (unsigned int)p.gy));
    unsigned char any = 0;
    if (x >= 1 && y >= 1 && z >= 1 && x <= p.gx - 2 && y <= p.gy - 2 && z <= p.gz - 2) {
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy) {
                const unsigned int base = c + (unsigned int)((dz * p.gy + dy) * p.gx);
                if (p.bcell[base + 2] > p.bcell[base - 1]) any = 1;
            }
    }
    bnear[c] = any;
}

/* lambda_b = -C_b / (sd_b + eps): rho_b and sd_b from the fluid x* of the
 * current parity plus the static boundary parts (rx_sph_pbd.cpp:825-913,
 * fluid neighbours on the current positions as rx_pbdsph_kernel.cu:666-735). */
__global__ void __launch_bounds__(kBlock) k_boundary_lambda(DevParams p, const unsigned int *__restrict__ cell_start,
                                                            const float4 *ppos0, const float4 *ppos1,
                                                            const DevCtl *ctl, const float2 *__restrict__ bstat,
                                                            float *__restrict__ blam) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= p.nb) return;
    const float4 *pp = ctl->parity ? ppos1 : ppos0;
    const float3 xb = f3(__ldg(p.bpos + b));
    const float agr = p.ag * p.inv_rest_dens;
    float wsum = 0.f, sd = 0.f;
    for_each_candidate<1>(
        p, cell_start, nullptr, nullptr, nullptr, 0, xb, nullptr, 0, [&](unsigned int j) { return pp[j]; },
        [&](unsigned int, const float4 &xj4) {
            const float3 d = xb - f3(xj4);
            const float r2 = dot3(d, d);
            const float q = fmaxf(p.h2 - r2, 0.0f);
            const float inv_r = pair_rsqrt(r2);
            const float t = fmaxf(p.h - r2 * inv_r, 0.0f);
            const float g = agr * t * t * inv_r;
            wsum += q * q * q;
            sd += g * g * r2;
        });
    const float2 st = bstat[b];
    const float rho = p.mass * p.aw * wsum + st.x;
    sd += st.y;
    float C = rho * p.inv_rest_dens - 1.0f;
    if (p.clamp_constraint && C < 0.0f) C = 0.0f;
    blam[b] = -C / (sd + p.epsilon);
}

void launch_boundary_volume(const DevParams &p, float *bscale, cudaStream_t s) {
    k_boundary_volume<<<blocks_for(p.n), kBlock, 0, s>>>(p, bscale);
}
void launch_boundary_static(const DevParams &p, float2 *bstat, cudaStream_t s) {
    k_boundary_static<<<blocks_for(p.n), kBlock, 0, s>>>(p, bstat);
}
void launch_boundary_near(const DevParams &p, unsigned int ncells, unsigned char *bnear, cudaStream_t s) {
    k_boundary_near<<<blocks_for(ncells), kBlock, 0, s>>>(p, ncells, bnear);
}
void launch_boundary_lambda(const DevParams &p, const unsigned int *cell_start, const float4 *ppos0,
                            const float4 *ppos1, const DevCtl *ctl, const float2 *bstat, float *blam, cudaStream_t s) {
    if (p.nb <= 0) return;
    k_boundary_lambda<<<blocks_for(p.nb), kBlock, 0, s>>>(p, cell_start, ppos0, ppos1, ctl, bstat, blam);
}

/* ======================================================================== */
/* WCSPH                                                                    */
/* ======================================================================== */

/* rho_i = m aw sum_j (h^2 - r^2)^3 (r < h, self included) and p_i = k (rho_i -
 * rho0) (rxSPH::calDensity, rx_sph_cpu.cpp:495-552, 569), in the same walk
 * over the 27 cells as the neighbour list of the following force pass
 * (every slot within the list radius, here the cell width h (1 + 1e-3));
 * the force pass's per-neighbour factors ride in the .w words of the sorted
 * copies: pos.w = p / rho^2, vel.w = 1 / rho.  Only .w words are written, so
 * the x, y, z the other threads read stay as they are. */
__global__ void __launch_bounds__(kBlock) k_sph_density(DevParams p, const unsigned int *__restrict__ cell_start,
                                                        float4 *pos, float4 *vel, float *__restrict__ dens,
                                                        float *__restrict__ pres, ListEntry *__restrict__ list,
                                                        unsigned char *__restrict__ cnt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const float3 xi = f3(pos[i]);
    const int3 c = cell_of(xi, p);
    float acc = 0.0f;
    int k = 0;
    bool ovf = false;
    ListEntry last = (ListEntry)i;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy) {
            unsigned int s, e;
            row_range(cell_start, c, dy, dz, p, s, e);
            /* four candidates' loads in flight before their tests */
            for (unsigned int j0 = s; j0 < e; j0 += 4) {
                float4 xc[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) xc[u] = __ldg(pos + min(j0 + u, e - 1));
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (j0 + u >= e) break;
                    const float3 d = xi - f3(xc[u]);
                    const float r2 = dot3(d, d);
                    if (r2 < p.h2) {
                        const float q = p.h2 - r2;
                        acc += q * q * q;
                    }
                    if (list && r2 < p.rl2) {
                        last = (ListEntry)(j0 + u);
                        if (k < kListMax) list[list_at(k, i, p.n)] = last;
                        ++k;
                    }
                }
            }
        }
    if (list) {
        ovf = k > kListMax;
#ifdef FSPH_LIST_GROUPED
        if (!ovf) /* pad the last group (k >= 1: the slot itself is always listed) */
            for (int t = k; (t & 3) != 0; ++t) list[list_at(t, i, p.n)] = last;
#endif
        cnt[i] = ovf ? kListOverflow : (unsigned char)k;
    }
    const float rho = p.mass * p.aw * acc;
    const float prs = p.gas_k * (rho - p.rest_dens);
    dens[i] = rho;
    pres[i] = prs;
    reinterpret_cast<float *>(pos + i)[3] = prs / (rho * rho);
    reinterpret_cast<float *>(vel + i)[3] = 1.0f / rho;
}

/* k_sph_density with LPP lanes per particle, so that small scenes still
 * fill the GPU: the lanes of a group take the candidates of each row in
 * turn (lane s the s-th of every LPP consecutive ones), and each LPP-wide
 * chunk's hits are ranked by a ballot inside the group, so the list holds
 * the same slots in the same order as one thread's walk.  The density is
 * the group's sum of the lanes' partial sums (same terms, other order). */
template <int LPP>
__global__ void __launch_bounds__(kBlock) k_sph_density_lanes(DevParams p, const unsigned int *__restrict__ cell_start,
                                                              float4 *pos, float4 *vel, float *__restrict__ dens,
                                                              float *__restrict__ pres, ListEntry *__restrict__ list,
                                                              unsigned char *__restrict__ cnt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int sub = t % LPP, lane = threadIdx.x & 31;
    const bool valid = t / LPP < p.n;
    const int i = valid ? t / LPP : p.n - 1; /* padding groups walk a real slot and write nothing */
    const unsigned int gmask = ((1u << LPP) - 1u) << (lane & ~(LPP - 1));
    const float3 xi = f3(pos[i]);
    const int3 c = cell_of(xi, p);
    float acc = 0.0f;
    int k = 0;
    unsigned int last = (unsigned int)i;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy) {
            unsigned int s, e;
            row_range(cell_start, c, dy, dz, p, s, e);
            for (unsigned int j0 = s; j0 < e; j0 += LPP) { /* the same trip count for the whole group */
                const unsigned int j = j0 + (unsigned int)sub;
                bool hit = false;
                if (j < e) {
                    const float3 d = xi - f3(__ldg(pos + j));
                    const float r2 = dot3(d, d);
                    if (r2 < p.h2) {
                        const float q = p.h2 - r2;
                        acc += q * q * q;
                    }
                    hit = r2 < p.rl2;
                }
                if (list) {
                    const unsigned int m = __ballot_sync(gmask, hit) & gmask;
                    if (m) {
                        if (hit) {
                            const int at = k + __popc(m & ((1u << lane) - 1u));
                            if (at < kListMax) list[list_at(at, i, p.n)] = (ListEntry)j;
                        }
                        last = __shfl_sync(gmask, j, 31 - __clz(m));
                        k += __popc(m);
                    }
                }
            }
        }
    acc = group_sum<LPP>(acc);
    if (!valid || sub != 0) return;
    if (list) {
        const bool ovf = k > kListMax;
#ifdef FSPH_LIST_GROUPED
        if (!ovf) /* pad the last group (k >= 1: the slot itself is always listed) */
            for (int u = k; (u & 3) != 0; ++u) list[list_at(u, i, p.n)] = (ListEntry)last;
#endif
        cnt[i] = ovf ? kListOverflow : (unsigned char)k;
    }
    const float rho = p.mass * p.aw * acc;
    const float prs = p.gas_k * (rho - p.rest_dens);
    dens[i] = rho;
    pres[i] = prs;
    reinterpret_cast<float *>(pos + i)[3] = prs / (rho * rho);
    reinterpret_cast<float *>(vel + i)[3] = 1.0f / rho;
}

/* a_i = -sum_j m (p_i/rho_i^2 + p_j/rho_j^2) grad W_ij + mu sum_j m (v_j - v_i)
 * lapW_ij / rho_j + g over 0 < r_ij < h (rxSPH::calForce, rx_sph_cpu.cpp:558-656),
 * from the list of the density pass (or the 27 cells when lists are off),
 * with LPP lanes per particle (small scenes then still fill the GPU).
 * Branch-free pair terms: t = max(h - r, 0) is 0 at and beyond h, and at
 * r = 0 too (h - 0 * rsqrt(0) is NaN, which fmaxf maps to 0), so the self
 * pair and coincident particles add nothing, as the reference skips them. */
struct PosVel {
    float4 x, v;
};
template <int LPP>
__global__ void __launch_bounds__(kBlock) k_sph_force(DevParams p, const unsigned int *__restrict__ cell_start,
                                                      const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                                                      float4 *__restrict__ acc, const ListEntry *__restrict__ list,
                                                      const unsigned char *__restrict__ cnt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int sub = t % LPP;
    const bool valid = t / LPP < p.n;
    const int i = valid ? t / LPP : p.n - 1; /* padding lanes run a real slot and write nothing */
    const float4 xi4 = pos[i], vi4 = vel[i];
    const float3 xi = f3(xi4), vi = f3(vi4);
    const float prsi = xi4.w;
    float3 fp = make_float3(0.f, 0.f, 0.f), fv = make_float3(0.f, 0.f, 0.f);
    for_each_candidate<LPP>(
        p, cell_start, list, cnt, nullptr, i, xi, nullptr, sub,
        [&](unsigned int j) { return PosVel{__ldg(pos + j), __ldg(vel + j)}; },
        [&](unsigned int, const PosVel &b) {
            const float3 d = xi - f3(b.x);
            const float r2 = dot3(d, d);
            const float inv_r = rsqrtf(r2);
            const float tt = fmaxf(fmaf(-r2, inv_r, p.h), 0.0f);
            const float g = p.ag * tt * tt * fminf(inv_r, 1e30f);
            fp = fp + ((prsi + b.x.w) * g) * d;
            fv = fv + (p.al * tt * b.v.w) * (f3(b.v) - vi);
        });
    if (LPP > 1) {
        fp.x = group_sum<LPP>(fp.x); fp.y = group_sum<LPP>(fp.y); fp.z = group_sum<LPP>(fp.z);
        fv.x = group_sum<LPP>(fv.x); fv.y = group_sum<LPP>(fv.y); fv.z = group_sum<LPP>(fv.z);
    }
    if (!valid || sub != 0) return;
    const float3 a = (-p.mass) * fp + (p.viscosity * p.mass) * fv + p.gravity;
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
    if (p.ntri) polygon_collide(f3(pos_b[i]), x, v, p.dt, p); /* sphIntegrateWithPolygon, rx_sph_kernel.cu:852-895 */
    x = solid_project(x, p);
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

/* squared distance as the reference's rxNeigh::Dist2: the difference of the
 * float coordinates and its squares summed in double, x + y + z in that
 * order with no fused multiply-add, rounded to float (rx_nnsearch.h:499-507) */
__device__ inline float ref_dist2(float3 xi, float3 xj) {
    double ex = (double)xi.x - (double)xj.x, ey = (double)xi.y - (double)xj.y, ez = (double)xi.z - (double)xj.z;
    return __double2float_rn(__dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez)));
}

__global__ void k_nb_fill(DevParams p, const unsigned int *__restrict__ cell_start, const float4 *__restrict__ pos,
                          const unsigned int *__restrict__ id, const unsigned int *__restrict__ offsets,
                          int *__restrict__ out, float *__restrict__ d2out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    float3 xi = f3(pos[i]);
    int3 c = cell_of(xi, p);
    unsigned int k = offsets[i];
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy) {
            unsigned int s, e;
            row_range(cell_start, c, dy, dz, p, s, e);
            for (unsigned int j = s; j < e; ++j) {
                const float3 xj = f3(pos[j]);
                if (ref_neighbor(xi, xj, p.h2)) {
                    if (d2out) d2out[k] = ref_dist2(xi, xj);
                    out[k++] = (int)id[j];
                }
            }
        }
}

/* ======================================================================== */
/* deletion regions and the active / parked partition                       */
/* ======================================================================== */

/* Particles strictly inside a region [lo, hi] (checkDeletePB,
 * rx_pbdsph_kernel.cu:1171-1187) are deleted: attribute -1, parked at the
 * reference's far point (0, 0, 1e6) with zero velocity. */
__global__ void k_delete_regions(int n, float4 *__restrict__ pos, float4 *__restrict__ vel,
                                 unsigned int *__restrict__ attr, const float4 *__restrict__ reg, int nreg) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n || attr[d] == 0xffffffffu) return;
    const float4 x = pos[d];
    for (int r = 0; r < nreg; ++r) {
        const float4 lo = reg[2 * r], hi = reg[2 * r + 1];
        if (x.x > lo.x && x.x < hi.x && x.y > lo.y && x.y < hi.y && x.z > lo.z && x.z < hi.z) {
            pos[d] = make_float4(0.0f, 0.0f, 1e6f, 0.0f);
            vel[d] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            attr[d] = 0xffffffffu;
            return;
        }
    }
}

/* keep[d] = 1 for a particle that takes part in the steps (attribute != -1) */
__global__ void k_mark_active(int n, const unsigned int *__restrict__ attr, unsigned int *__restrict__ keep) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d < n) keep[d] = attr[d] != 0xffffffffu ? 1u : 0u;
}

/* stable partition, active slots first: perm[new slot] = old slot, from the
 * exclusive scan of the keep flags (scan[n] = the active count) */
__global__ void k_partition_perm(int n, const unsigned int *__restrict__ scan, unsigned int *__restrict__ perm) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    const unsigned int s = scan[d], keep = scan[d + 1] - s, nk = scan[n];
    perm[keep ? s : nk + ((unsigned int)d - s)] = (unsigned int)d;
}

/* rows of k4 float4 per slot: dst[d] = src[perm[d]] */
__global__ void k_gather_rows(int n, const unsigned int *__restrict__ perm, const float4 *__restrict__ src,
                              float4 *__restrict__ dst, int k4) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * k4) return;
    const long long d = t / k4, c = t % k4;
    dst[t] = src[(long long)perm[d] * k4 + c];
}

/* ======================================================================== */
/* density on a lattice (for meshing)                                       */
/* ======================================================================== */

/* The density field at the nodes of an nx x ny x nz lattice (i fastest),
 * node (i, j, k) at minp + (i, j, k) d: 0 outside [lo, hi], else
 * sum_j m W(r_j) over the particles with fl32(|x - x_j|^2 in double) <=
 * fl32(h h), r_j = fl32(sqrt(Dist2)), W in double and the sum in float, as
 * rxPBDSPH::CalColorField (rx_sph_pbd.cpp:2075-2108, the CPU form of
 * pbdsphCalDensityInGrid, rx_pbdsph_kernel.cu:1220-1299).  A float
 * distance test in a 1e-4 band around h^2 skips the double evaluation for
 * the candidates far outside. */
__global__ void __launch_bounds__(kBlock) k_density_grid(DevParams p, const unsigned int *__restrict__ cell_start,
                                                         const float4 *__restrict__ pos, int nx, int ny, int nz,
                                                         double3 minp, double3 dd, double3 lo, double3 hi,
                                                         float *__restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nx * ny * nz) return;
    const int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / ((long long)nx * ny));
    /* minp + Vec3(i, j, k) * d, each product and sum rounded in double */
    const double X = __dadd_rn(minp.x, __dmul_rn((double)i, dd.x));
    const double Y = __dadd_rn(minp.y, __dmul_rn((double)j, dd.y));
    const double Z = __dadd_rn(minp.z, __dmul_rn((double)k, dd.z));
    float acc = 0.0f;
    if (X >= lo.x && X <= hi.x && Y >= lo.y && Y <= hi.y && Z >= lo.z && Z <= hi.z) {
        const float3 xf = make_float3((float)X, (float)Y, (float)Z);
        const int3 c = cell_of(xf, p);
        const float band = p.h2 * (1.0f + 1e-4f);
        const double hd = (double)p.h, aw = (double)p.aw_d, m = (double)p.mass;
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy) {
                unsigned int s, e;
                row_range(cell_start, c, dy, dz, p, s, e);
                for (unsigned int q = s; q < e; ++q) {
                    const float4 xq = __ldg(pos + q);
                    const float3 df = xf - f3(xq);
                    if (dot3(df, df) > band) continue;
                    const double ex = X - (double)xq.x, ey = Y - (double)xq.y, ez = Z - (double)xq.z;
                    const float d2 =
                        __double2float_rn(__dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez)));
                    if (d2 <= p.h2) {
                        const double r = (double)sqrtf(d2);
                        const double qq = __dsub_rn(__dmul_rn(hd, hd), __dmul_rn(r, r));
                        acc = __double2float_rn(__dadd_rn((double)acc, __dmul_rn(m, __dmul_rn(__dmul_rn(__dmul_rn(aw, qq), qq), qq))));
                    }
                }
            }
    }
    out[t] = acc;
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
/* blocks of a constraint-pass launch: one per kPassBlock slots, or (with
 * persistent warps) the resident blocks of the whole GPU, at most that */
static unsigned int pass_blocks(int n, const void *kernel, bool persistent) {
    unsigned int b = blocks_for(n, kPassBlock);
    if (persistent) {
        /* resident blocks of each pass kernel, looked up once (contexts may
         * step from several host threads) */
        static std::mutex mu;
        static const void *known[4] = {nullptr, nullptr, nullptr, nullptr};
        static int resident[4] = {0, 0, 0, 0};
        std::lock_guard<std::mutex> lock(mu);
        int k = 0;
        while (k < 4 && known[k] && known[k] != kernel) ++k;
        if (k == 4) k = 3;
        if (known[k] != kernel) {
            int dev = 0, sms = 0, per = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kPassBlock, 0);
            resident[k] = std::max(1, sms * std::max(per, 1));
            known[k] = kernel;
        }
        b = std::min(b, (unsigned int)resident[k]);
    }
    return b;
}

void launch_lambda(const DevParams &p, const unsigned int *cell_start, float4 *ppos0, float4 *ppos1, float *dens,
                   DevCtl *ctl, ErrPartial *part, unsigned long long while_handle, int use_graph,
                   const NbrLists &nl, cudaStream_t s) {
    auto k = p.compensated ? k_lambda<true> : k_lambda<false>;
    k<<<pass_blocks(p.n, (const void *)k, FSPH_PERSIST_LAMBDA != 0), kPassBlock, 0, s>>>(p, cell_start, ppos0, ppos1, dens, ctl, part,
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
    k_correction<<<pass_blocks(p.n, (const void *)k_correction, FSPH_PERSIST_CORRECTION != 0), kPassBlock, 0, s>>>(p, cell_start, ppos0, ppos1, xb,
                                                                                    ctl, part,
                                                    (cudaGraphConditionalHandle)if_handle,
                                                    (cudaGraphConditionalHandle)if_handle2, use_graph, dp_out,
                                                    p.use_lists ? nl.list : nullptr, nl.cnt, nl.cellb);
}
void launch_finalize(const DevParams &p, const float4 *pos_b, const float4 *ppos0, const float4 *ppos1,
                     const DevCtl *ctl, const unsigned int *id_b, const unsigned int *attr_b, float4 *pos_a,
                     float4 *vel_a, unsigned int *id_a, unsigned int *attr_a, const float4 *xpred, float4 *dstep,
                     cudaStream_t s, const float *dens, float *mrho) {
    k_finalize<<<blocks_for(p.n), kBlock, 0, s>>>(p, pos_b, ppos0, ppos1, ctl, id_b, attr_b, pos_a, vel_a, id_a,
                                                  attr_a, xpred, dstep, dens, mrho);
}
void launch_xsph_vort(const DevParams &p, const unsigned int *cell_start, const float4 *pos, const float4 *vel,
                      const float *dens, float4 *vel_out, float4 *vort, const FeatureOut &fo, const NbrLists &nl,
                      cudaStream_t s, const float *mrho, float2 *wm) {
    /* the neighbour means cost a gather per pair: only when they are used */
    const bool nbr = fo.feat && fo.nbr, pre = mrho && wm;
    auto k = nbr ? (pre ? k_xsph_vort<true, true> : k_xsph_vort<true, false>)
                 : (pre ? k_xsph_vort<false, true> : k_xsph_vort<false, false>);
    k<<<blocks_for(p.n), kBlock, 0, s>>>(p, cell_start, pos, vel, dens, vel_out, vort, fo,
                                         p.use_lists ? nl.list : nullptr, nl.cnt, nl.cellb, mrho, wm);
}
void launch_vort_apply(const DevParams &p, const unsigned int *cell_start, const float4 *pos, const float4 *vort,
                       const float *dens, const float4 *vel_in, float4 *vel_out, const NbrLists &nl, cudaStream_t s,
                       const float2 *wm) {
    auto k = wm ? k_vort_apply<true> : k_vort_apply<false>;
    k<<<blocks_for(p.n), kBlock, 0, s>>>(p, cell_start, pos, vort, dens, vel_in, vel_out,
                                         p.use_lists ? nl.list : nullptr, nl.cnt, nl.cellb, wm);
}
int sph_force_lanes(int n);
void launch_sph_density(const DevParams &p, const unsigned int *cell_start, float4 *pos, float4 *vel, float *dens,
                        float *pres, const NbrLists &nl, cudaStream_t s) {
    ListEntry *l = p.use_lists ? nl.list : nullptr;
    const int lanes = FSPH_SPH_DENSITY_LANES ? sph_force_lanes(p.n) : 1;
    const unsigned int g = blocks_for((long long)p.n * lanes);
    switch (lanes) {
    case 1: k_sph_density<<<g, kBlock, 0, s>>>(p, cell_start, pos, vel, dens, pres, l, nl.cnt); break;
    case 2: k_sph_density_lanes<2><<<g, kBlock, 0, s>>>(p, cell_start, pos, vel, dens, pres, l, nl.cnt); break;
    case 4: k_sph_density_lanes<4><<<g, kBlock, 0, s>>>(p, cell_start, pos, vel, dens, pres, l, nl.cnt); break;
    default: k_sph_density_lanes<8><<<g, kBlock, 0, s>>>(p, cell_start, pos, vel, dens, pres, l, nl.cnt); break;
    }
}
/* lanes per particle of the WCSPH force pass: enough that the launch holds
 * about as many threads as the GPU keeps resident (1536 per SM), at most 8 */
int sph_force_lanes(int n) {
    static const int resident = [] { /* initialised once, thread-safely */
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        return std::max(sms, 1) * 1536;
    }();
#ifdef FSPH_SPH_LANES
    return FSPH_SPH_LANES;
#else
    int lanes = 1;
    while (lanes < 8 && (long long)n * lanes < (long long)resident) lanes *= 2;
    return lanes;
#endif
}
void launch_sph_force(const DevParams &p, const unsigned int *cell_start, const float4 *pos, const float4 *vel,
                      float4 *acc, const NbrLists &nl, cudaStream_t s) {
    const ListEntry *l = p.use_lists ? nl.list : nullptr;
    const int lanes = sph_force_lanes(p.n);
    const unsigned int g = blocks_for((long long)p.n * lanes);
    switch (lanes) {
    case 1: k_sph_force<1><<<g, kBlock, 0, s>>>(p, cell_start, pos, vel, acc, l, nl.cnt); break;
    case 2: k_sph_force<2><<<g, kBlock, 0, s>>>(p, cell_start, pos, vel, acc, l, nl.cnt); break;
    case 4: k_sph_force<4><<<g, kBlock, 0, s>>>(p, cell_start, pos, vel, acc, l, nl.cnt); break;
    default: k_sph_force<8><<<g, kBlock, 0, s>>>(p, cell_start, pos, vel, acc, l, nl.cnt); break;
    }
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
                    const unsigned int *offsets, int *out, float *d2out, cudaStream_t s) {
    k_nb_fill<<<blocks_for(p.n), kBlock, 0, s>>>(p, cell_start, pos, id, offsets, out, d2out);
}
void launch_delete_regions(int n, float4 *pos, float4 *vel, unsigned int *attr, const float4 *reg, int nreg,
                           cudaStream_t s) {
    if (n > 0 && nreg > 0) k_delete_regions<<<blocks_for(n), kBlock, 0, s>>>(n, pos, vel, attr, reg, nreg);
}
void launch_mark_active(int n, const unsigned int *attr, unsigned int *keep, cudaStream_t s) {
    if (n > 0) k_mark_active<<<blocks_for(n), kBlock, 0, s>>>(n, attr, keep);
}
void launch_partition_perm(int n, const unsigned int *scan, unsigned int *perm, cudaStream_t s) {
    if (n > 0) k_partition_perm<<<blocks_for(n), kBlock, 0, s>>>(n, scan, perm);
}
void launch_gather_rows(int n, const unsigned int *perm, const float4 *src, float4 *dst, int k4, cudaStream_t s) {
    if (n > 0) k_gather_rows<<<blocks_for((long long)n * k4), kBlock, 0, s>>>(n, perm, src, dst, k4);
}
void launch_density_grid(const DevParams &p, const unsigned int *cell_start, const float4 *pos, const int nn[3],
                         const double minp[3], const double d[3], const double lo[3], const double hi[3], float *out,
                         cudaStream_t s) {
    const long long tot = (long long)nn[0] * nn[1] * nn[2];
    k_density_grid<<<blocks_for(tot), kBlock, 0, s>>>(p, cell_start, pos, nn[0], nn[1], nn[2],
                                                      make_double3(minp[0], minp[1], minp[2]),
                                                      make_double3(d[0], d[1], d[2]), make_double3(lo[0], lo[1], lo[2]),
                                                      make_double3(hi[0], hi[1], hi[2]), out);
}
/* The reference's cell hash of each position (z Gy Gx + y Gx + x):
 * rule 0 = its CPU grid (rxNNGrid::CalGridHash(Vec3), rx_nnsearch.h:590-599:
 * (p - min) / cw in double, truncated to int, clamped to [0, G-1]);
 * rule 1 = its GPU grid (calcGridPos / calcGridHash, rx_cu_common.cu:121-144:
 * floor((p - origin) / cw) in float, clamped). */
__global__ void __launch_bounds__(kBlock) k_reference_cells(int n, const float4 *__restrict__ pos, int rule,
                                                            double3 org, double cw, int gx, int gy, int gz,
                                                            unsigned int *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 x = pos[i];
    int c[3];
    const int g[3] = {gx, gy, gz};
    const float xf[3] = {x.x, x.y, x.z};
    const double o[3] = {org.x, org.y, org.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int k;
        if (rule == 0) {
            k = (int)__ddiv_rn((double)xf[a] - o[a], cw);
        } else {
            k = (int)floorf(__fdiv_rn(__fsub_rn(xf[a], (float)o[a]), (float)cw));
        }
        c[a] = k < 0 ? 0 : (k >= g[a] ? g[a] - 1 : k);
    }
    out[i] = ((unsigned int)c[2] * (unsigned int)gy + (unsigned int)c[1]) * (unsigned int)gx + (unsigned int)c[0];
}

/* The triangle-mesh collision alone, for parity: x1 and v updated in place
 * from the segments x0 -> x1. */
__global__ void __launch_bounds__(kBlock) k_polygon_collide(DevParams p, int n, const float4 *__restrict__ x0,
                                                            float4 *__restrict__ x1, float4 *__restrict__ v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 x = f3(x1[i]), vv = f3(v[i]);
    polygon_collide(f3(x0[i]), x, vv, p.dt, p);
    x1[i] = make_float4(x.x, x.y, x.z, x1[i].w);
    v[i] = make_float4(vv.x, vv.y, vv.z, v[i].w);
}
void launch_polygon_collide(const DevParams &p, int n, const float4 *x0, float4 *x1, float4 *v, cudaStream_t s) {
    if (n > 0 && p.ntri) k_polygon_collide<<<blocks_for(n), kBlock, 0, s>>>(p, n, x0, x1, v);
}

void launch_reference_cells(int n, const float4 *pos, int rule, const double org[3], double cw, const int g[3],
                            unsigned int *out, cudaStream_t s) {
    if (n > 0)
        k_reference_cells<<<blocks_for(n), kBlock, 0, s>>>(n, pos, rule, make_double3(org[0], org[1], org[2]), cw,
                                                          g[0], g[1], g[2], out);
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
