/*
 * fsph_kernels.cuh -- host-callable launchers of the fluid-step kernels
 * (defined in fsph_kernels.cu).  Every launcher enqueues on `s` and returns
 * without synchronising.
 */
#pragma once
#include "fsph_internal.cuh"

namespace fsph {

constexpr int kBlock = 256;
/* threads per block of the two constraint passes (k_lambda, k_correction);
 * measured at 1 M particles against 256: 128 +6 %, 64 +38 %, 512 -0.8 %
 * per warm step */
#ifndef FSPH_PASS_BLOCK
#define FSPH_PASS_BLOCK 512
#endif
constexpr int kPassBlock = FSPH_PASS_BLOCK;
constexpr int kBlockMax = 512;  /* largest block of the batched persistent kernels */
constexpr int kScanTile = 4096; /* cells per block of the first scan phase */

inline unsigned int blocks_for(long long n, int b = kBlock) { return (unsigned int)((n + b - 1) / b); }
inline unsigned int scan_blocks(unsigned int ncells) { return (ncells + kScanTile - 1) / kScanTile; }

/* ---- grid build: counting sort on the 64-bit key (cell << 32 | previous slot) ---- */
/* x* = walls(x + dt (v + dt a)), a = gravity when acc == NULL; then key + rank.
 * xpred_out (optional) keeps that prediction; dwarm (optional) is a warm-start
 * correction: the iterations then start from walls(x* + dwarm). */
void launch_predict_hash(const DevParams &p, const float4 *pos, const float4 *vel, const float4 *acc,
                         float4 *ppos_out, unsigned int *key, unsigned int *rank, unsigned int *count,
                         const float4 *dwarm, float4 *xpred_out, cudaStream_t s);
void launch_hash(const DevParams &p, const float4 *x, unsigned int *key, unsigned int *rank, unsigned int *count,
                 cudaStream_t s);
/* exclusive scan of count[C] into cell_start[C+1]; zeroes count for the next build */
void launch_scan(unsigned int *count, unsigned int *cell_start, unsigned int *block_sums, unsigned int ncells,
                 cudaStream_t s);
/* perm[cell_start[key] + rank] = slot, then each cell's slots sorted ascending */
void launch_scatter_sort(const DevParams &p, const unsigned int *key, const unsigned int *rank,
                         const unsigned int *cell_start, unsigned int *perm, unsigned int ncells, cudaStream_t s);

/* dst[d] = src[perm[d]] for up to 6 float4 and 4 u32 streams (perm == NULL: plain copy) */
struct Gather {
    const float4 *src4[6];
    float4 *dst4[6];
    const unsigned int *src1[4];
    unsigned int *dst1[4];
    int n4, n1;
};
void launch_gather(int n, const unsigned int *perm, const Gather &g, DevCtl *count_build, cudaStream_t s);

/* in-loop rebuild (the current x* buffer is chosen on the device by ctl->parity) */
void launch_hash_parity(const DevParams &p, const float4 *ppos0, const float4 *ppos1, const DevCtl *ctl,
                        unsigned int *key, unsigned int *rank, unsigned int *count, cudaStream_t s);
void launch_rebuild_gather(int n, const unsigned int *perm, const DevCtl *ctl, const float4 *pos, const float4 *ppos0,
                           const float4 *ppos1, const unsigned int *id, const unsigned int *attr, const float *dens,
                           float4 *t_pos, float4 *t_x, unsigned int *t_id, unsigned int *t_attr, float *t_dens,
                           const unsigned int *key, unsigned int *cellb, const float4 *xpred, float4 *t_xpred,
                           float *t_lam, cudaStream_t s);

/* neighbour lists (see fsph_internal.cuh) */
struct NbrLists {
    ListEntry *list = nullptr;       /* [kListMax][n] */
    unsigned char *cnt = nullptr;    /* [n], kListOverflow = use the cell walk */
    unsigned int *cellb = nullptr;   /* [n] build cell of each slot */
};
/* lists of every slot from the build positions xb (a no-op when p.use_lists == 0) */
void launch_build_list(const DevParams &p, const unsigned int *cell_start, const float4 *xb, const NbrLists &nl,
                       cudaStream_t s);
void launch_rebuild_copy(int n, DevCtl *ctl, const float4 *t_pos, const float4 *t_x, const unsigned int *t_id,
                         const unsigned int *t_attr, const float *t_dens, float4 *pos, float4 *ppos0, float4 *ppos1,
                         float4 *xb, unsigned int *id, unsigned int *attr, float *dens, const float4 *t_xpred,
                         float4 *xpred, const float *t_lam, cudaStream_t s);

/* ---- PBF ---- */
void launch_pbf_density(const DevParams &p, const unsigned int *cell_start, const float4 *pos, float *dens,
                        cudaStream_t s);
void launch_pbf_visc(const DevParams &p, const unsigned int *cell_start, const float4 *pos, const float4 *vel,
                     const float *dens, float4 *acc, cudaStream_t s);
void launch_lambda(const DevParams &p, const unsigned int *cell_start, float4 *ppos0, float4 *ppos1, float *dens,
                   DevCtl *ctl, ErrPartial *part, unsigned long long while_handle, int use_graph,
                   const NbrLists &nl, cudaStream_t s);
void launch_correction(const DevParams &p, const unsigned int *cell_start, float4 *ppos0, float4 *ppos1,
                       const float4 *xb, DevCtl *ctl, float *part, unsigned long long if_handle,
                       unsigned long long if_handle2, int use_graph, float4 *dp_out, const NbrLists &nl,
                       cudaStream_t s);
void launch_finalize(const DevParams &p, const float4 *pos_b, const float4 *ppos0, const float4 *ppos1,
                     const DevCtl *ctl, const unsigned int *id_b, const unsigned int *attr_b, float4 *pos_a,
                     float4 *vel_a, unsigned int *id_a, unsigned int *attr_a, const float4 *xpred, float4 *dstep,
                     cudaStream_t s, const float *dens = nullptr, float *mrho = nullptr);
/* XSPH + vorticity (omega) pass; with fo.feat also the warm-start features.
 * With mrho (m / rho per particle, from launch_finalize) and wm the pass
 * reads m / rho_j instead of dividing per pair and leaves (|omega|, m / rho)
 * in wm, which launch_vort_apply then gathers in place of vort and dens. */
void launch_xsph_vort(const DevParams &p, const unsigned int *cell_start, const float4 *pos, const float4 *vel,
                      const float *dens, float4 *vel_out, float4 *vort, const FeatureOut &fo, const NbrLists &nl,
                      cudaStream_t s, const float *mrho = nullptr, float2 *wm = nullptr);
void launch_vort_apply(const DevParams &p, const unsigned int *cell_start, const float4 *pos, const float4 *vort,
                       const float *dens, const float4 *vel_in, float4 *vel_out, const NbrLists &nl, cudaStream_t s,
                       const float2 *wm = nullptr);

/* ---- static boundary particles (p.bpos / p.bcell / p.bnear of the sorted boundary) ---- */
/* bscale[b] = rho0 psi_b / m with psi_b = m / sum_b' m W(r_bb') (rx_sph_pbd.cpp:1061-1090) */
void launch_boundary_volume(const DevParams &p, float *bscale, cudaStream_t s);
/* bstat[b] = (sum_b' rho0 psi_b' W, sum_b' |(rho0 psi_b' / m) grad W / rho0|^2): the static
 * boundary-boundary parts of lambda_b */
void launch_boundary_static(const DevParams &p, float2 *bstat, cudaStream_t s);
/* bnear[c] = 1 when any boundary slot lies in the 27 cells around cell c */
void launch_boundary_near(const DevParams &p, unsigned int ncells, unsigned char *bnear, cudaStream_t s);
/* lambda_b of every boundary particle from the fluid x* of the current parity (rx_sph_pbd.cpp:825-913) */
void launch_boundary_lambda(const DevParams &p, const unsigned int *cell_start, const float4 *ppos0,
                            const float4 *ppos1, const DevCtl *ctl, const float2 *bstat, float *blam, cudaStream_t s);

/* ---- WCSPH ---- */
/* density + pressure of the sorted positions, the force pass's neighbour
 * lists (nl.list / nl.cnt, when p.use_lists) and its per-neighbour factors
 * in pos.w = p / rho^2 and vel.w = 1 / rho */
void launch_sph_density(const DevParams &p, const unsigned int *cell_start, float4 *pos, float4 *vel, float *dens,
                        float *pres, const NbrLists &nl, cudaStream_t s);
/* acceleration from the lists and .w factors of launch_sph_density */
void launch_sph_force(const DevParams &p, const unsigned int *cell_start, const float4 *pos, const float4 *vel,
                      float4 *acc, const NbrLists &nl, cudaStream_t s);
int sph_force_lanes(int n);
void launch_sph_integrate(const DevParams &p, const float4 *pos_b, const float4 *vel_b, const float4 *acc,
                          const unsigned int *id_b, const unsigned int *attr_b, float4 *pos_a, float4 *vel_a,
                          unsigned int *id_a, unsigned int *attr_a, cudaStream_t s);

/* ---- neighbour sets under the reference criterion ---- */
void launch_nb_count(const DevParams &p, const unsigned int *cell_start, const float4 *pos, unsigned int *cnt,
                     cudaStream_t s);
/* CSR rows from offsets: neighbour slots mapped through id, and (d2out,
 * when given) each pair's squared distance as the reference's Dist2 */
void launch_nb_fill(const DevParams &p, const unsigned int *cell_start, const float4 *pos, const unsigned int *id,
                    const unsigned int *offsets, int *out, float *d2out, cudaStream_t s);

/* ---- deletion regions and the active / parked partition ---- */
/* reg: nreg pairs (lo, hi) of float4 */
void launch_delete_regions(int n, float4 *pos, float4 *vel, unsigned int *attr, const float4 *reg, int nreg,
                           cudaStream_t s);
void launch_mark_active(int n, const unsigned int *attr, unsigned int *keep, cudaStream_t s);
void launch_partition_perm(int n, const unsigned int *scan, unsigned int *perm, cudaStream_t s);
void launch_gather_rows(int n, const unsigned int *perm, const float4 *src, float4 *dst, int k4, cudaStream_t s);

/* ---- density on a lattice (CalImplicitField) ---- */
void launch_density_grid(const DevParams &p, const unsigned int *cell_start, const float4 *pos, const int nn[3],
                         const double minp[3], const double d[3], const double lo[3], const double hi[3], float *out,
                         cudaStream_t s);

/* ---- grid sort as an LSD radix sort of (cell << 32 | slot) keys ---- */
struct RadixBufs {
    unsigned long long *k0 = nullptr, *k1 = nullptr; /* n keys each (ping-pong) */
    unsigned int *hist = nullptr, *offs = nullptr;   /* 256 x tiles (offs: + 1 for the scan's total) */
    unsigned int *bsum = nullptr;                    /* scan_blocks(256 x tiles) */
};
unsigned int radix_tiles(int n);
int radix_passes(unsigned int ncells);
/* perm[d] = the previous slot of the d-th key in (cell, slot) order */
void launch_radix_sort_cells(int n, const unsigned int *cell, unsigned int ncells, const RadixBufs &b,
                             unsigned int *perm, cudaStream_t s);

/* ---- triangle-mesh collision of given segments (parity) ---- */
void launch_polygon_collide(const DevParams &p, int n, const float4 *x0, float4 *x1, float4 *v, cudaStream_t s);

/* ---- the reference's cell hash (rule 0: its CPU grid, 1: its GPU grid) ---- */
void launch_reference_cells(int n, const float4 *pos, int rule, const double org[3], double cw, const int g[3],
                            unsigned int *out, cudaStream_t s);

/* ---- particle order <-> device order ---- */
void launch_unsort4(int n, const unsigned int *id, const float4 *src, float4 *dst, int zero_w, cudaStream_t s);
void launch_unsort1(int n, const unsigned int *id, const unsigned int *src, unsigned int *dst, cudaStream_t s);
void launch_unsort_w(int n, const unsigned int *id, const float4 *src, float *dst, cudaStream_t s);
void launch_iota(int n, unsigned int *dst, cudaStream_t s);
/* rows of k4 float4 per slot: dst[id[d]] = src[d] */
void launch_unsort_rows(int n, const unsigned int *id, const float4 *src, float4 *dst, int k4, cudaStream_t s);
void launch_pack_w(int n, float4 *dst, const float *w, cudaStream_t s);
/* *flag |= 1 when any x/y/z of a (or b, if given) is not finite */
void launch_check_finite(int n, const float4 *a, const float4 *b, unsigned int *flag, cudaStream_t s);

}  // namespace fsph
