/*
 * fsph_internal.cuh -- device-side types shared by the fluid-step kernels.
 *
 * Data layout in HBM (all arrays in DEVICE order, i.e. sorted by grid cell,
 * re-sorted at every grid build and carried sorted across steps):
 *   pos[N], vel[N]      float4  x, v (w unused)
 *   ppos[2][N]          float4  x* ping-pong; .w of the read buffer carries the
 *                               particle's lambda between the lambda and
 *                               correction passes of one iteration
 *   xb[N]               float4  x* at the last grid build (skin test)
 *   dens[N], pres[N]    float
 *   id[N], attr[N]      u32/i32 device slot -> particle index, user tag
 *   cell_start[C+1]     u32     dense grid, cell c holds slots
 *                               [cell_start[c], cell_start[c+1])
 * The grid is a dense cell table over the wall box padded by one cell on
 * every side (cell width h (1 + skin)), linear index (z Gy + y) Gx + x -- the
 * reference's hash (rx_cu_common.cu:121-144) without its clamping -- so the
 * three cells x-1..x+1 of one (y, z) row are one contiguous slot range and a
 * 27-cell neighbourhood is nine ranges.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fsph {

/* An analytic obstacle (the reference's box and sphere obstacles,
 * rx_cu_common.cuh:135-136, at most 10 of each): 128 bytes. */
constexpr int kMaxBoxObstacles = 10, kMaxSphereObstacles = 10;
constexpr int kMaxObstacles = kMaxBoxObstacles + kMaxSphereObstacles;
struct Obstacle {
    float4 cen;              /* centre; w = sphere radius */
    float4 ext;              /* box half extents; w = 0 box, 1 sphere */
    float4 rot[3];           /* box: rows of the world -> local rotation */
    float4 inv[3];           /* box: rows of its inverse */
};

/* Triangle-mesh obstacles (SetPolygonObstacle, rx_ps.h:268): the triangles
 * binned into the cells of the reference's GPU grid (setupCells,
 * rx_sph_pbd_gpu.cpp:1986-2011) that they intersect, as setPolysToCell does
 * (rx_sph_pbd_gpu.cpp:2051-2200); cell c holds idx[start[c], end[c]),
 * start[c] = 0xffffffff when empty. */
struct PolyTable {
    const float4 *vrts;
    const int4 *tris;
    const unsigned int *start, *end, *idx;
    float3 org;                 /* the grid's origin and cell width, as floats */
    float cw;
    int gx, gy, gz;
};

/* Launch-time constants of one solver; passed by value to every kernel. */
struct DevParams {
    int n;
    float h, h2, mass, rest_dens, inv_rest_dens;
    float aw, ag, al;           /* poly6, spiky-gradient, visc-Laplacian coefficients */
    double aw_d;                /* the poly6 coefficient in double (the reference's) */
    float3 wall_lo, wall_hi;    /* box_min + r, box_max - r */
    float3 gravity;
    float viscosity, gas_k;
    float epsilon, eta;
    int min_iter, max_iter, error_mode, clamp_constraint;
    int use_ap;
    float ap_k, ap_n, inv_wq;   /* s_corr = -k (W(r) / W(q h))^n dt^2 */
    float xsph_c, vort_eps;
    float3 grid_origin;
    float inv_cw;
    int gx, gy, gz;
    float skin2;                /* squared displacement since the last build that forces a rebuild */
    float rl2;                  /* squared neighbour-list radius (= cell width) */
    int use_lists;              /* 1: lambda / correction passes read the neighbour lists */
    float dt, inv_dt;
    unsigned int cell_off;      /* first cell of this scene's grid in the cell table (batches; else 0) */
    int compensated;            /* 1: Kahan-compensated density sums in the lambda pass */
    /* static boundary particles (nb = 0: none), sorted by the cells of this grid */
    int nb;
    const float4 *bpos;         /* x, y, z and w = rho0 psi_b / m */
    const float *blam;          /* lambda_b of the current lambda pass */
    const unsigned int *bcell;  /* boundary slots of cell c: [bcell[c], bcell[c + 1]) */
    const unsigned char *bnear; /* 1 when boundary particles lie in the 27 cells around c */
    /* analytic obstacles (nobs = 0: none) */
    int nobs;
    const Obstacle *obs;
    /* triangle-mesh obstacles (ntri = 0: none) */
    int ntri;
    PolyTable poly;
    /* FSPH_DEBUG_BOUNDS builds: where failed index checks are recorded (may be null) */
    unsigned int *dbg;
};

/* FSPH_DEBUG_BOUNDS 1 (a debug build, fltk_sph_ice_gb300.build --debug-bounds):
 * every slot, cell and list index the passes read is checked against its
 * table before it is used; an index out of range is replaced by a valid one
 * (the step's numbers are then wrong, never its memory accesses) and sets a
 * bit of DevParams::dbg, which the step reports in fsph_step_stats.
 * bounds_bits.  Off (0) in the product build: the checks compile away. */
#ifndef FSPH_DEBUG_BOUNDS
#define FSPH_DEBUG_BOUNDS 0
#endif
enum : unsigned int {
    kBoundSlot = 1u,      /* a neighbour slot (list entry or cell walk) >= n */
    kBoundCell = 2u,      /* a cell-table row outside the scene's cells */
    kBoundCount = 8u,     /* a list count above kListMax that is not the overflow mark */
    kBoundBoundary = 16u  /* a boundary slot >= nb */
};
/* v if v < limit, else record `bit` and give 0 */
__device__ __forceinline__ unsigned int bounded(const DevParams &p, unsigned int v, unsigned int limit,
                                                unsigned int bit) {
#if FSPH_DEBUG_BOUNDS
    if (v >= limit) {
        if (p.dbg) atomicOr(p.dbg, bit);
        return 0u;
    }
#else
    (void)p; (void)limit; (void)bit;
#endif
    return v;
}
/* a cell-table row [base - 1, base + 2] inside the scene's cells (the table
 * has one more entry than cells): false (recorded) when not */
__device__ __forceinline__ bool cell_row_ok(const DevParams &p, unsigned int base) {
#if FSPH_DEBUG_BOUNDS
    const unsigned int end = p.cell_off + (unsigned int)p.gx * (unsigned int)p.gy * (unsigned int)p.gz;
    if (base < p.cell_off + 1u || base + 2u > end) {
        if (p.dbg) atomicOr(p.dbg, kBoundCell);
        return false;
    }
#else
    (void)p; (void)base;
#endif
    return true;
}

/* Neighbour lists: up to kListMax entries per particle, transposed (entry
 * k of slot i at list_at(k, i, n)) so a warp's lanes read consecutive
 * words.  An entry is the candidate's slot (32 bits).  Built with
 * FSPH_LIST16 it is (row << 12) | (j - row_start) in 16 bits, row = the
 * (dz, dy) index 0..8 of the 27-cell neighbourhood of the particle's build
 * cell: half the list bytes, but every candidate then pays a shared-memory
 * row-start lookup, and the passes are bound by instruction issue (the
 * 32-bit form measured 14 % faster per step).  A count of kListOverflow
 * sends the particle to the cell walk. */
constexpr int kListMax = 64;
constexpr unsigned char kListOverflow = 255;
#ifndef FSPH_LIST16
#define FSPH_LIST32
#endif
#ifdef FSPH_LIST32
typedef unsigned int ListEntry;   /* the candidate's slot itself */
#else
typedef unsigned short ListEntry; /* (row << 12) | (slot - row start) */
#endif
/* 32-bit entries are stored in groups of four: group g of slot i is the
 * 16-byte word [g * n + i], so a warp reads four entries of its 32 slots
 * with one coalesced 512-byte load; a list's last group is padded with its
 * last entry.  FSPH_LIST_SCALAR keeps one entry per word ([t * n + i]). */
#if defined(FSPH_LIST32) && !defined(FSPH_LIST_SCALAR)
#define FSPH_LIST_GROUPED 1
#endif
__host__ __device__ inline size_t list_at(int t, int i, int n) {
#ifdef FSPH_LIST_GROUPED
    return ((size_t)(t >> 2) * (size_t)n + (size_t)i) * 4 + (size_t)(t & 3);
#else
    return (size_t)t * (size_t)n + (size_t)i;
#endif
}

/* Warm-start features of a particle at the end of a step, all dimensionless:
 *   0 rho/rho0 - 1 of the last lambda pass     1 lambda rho0 h^2
 *   2 neighbour count / 33                     3-5 mean offset to neighbours / h
 *   6-8 v dt / h                               9-11 step correction (x*_final - x*_pred) / h
 *   12 C' = rho'/rho0 - 1 and 13-15 h grad_i C' at the next step's predicted
 *      relative positions x_ij + dt (v_i - v_j) (the constraint the coming
 *      iterations will have to remove, from the same neighbour loop)
 *   16-22 the poly6-weighted means over the neighbours (self excluded) of
 *      features 0, 6-8 and 9-11: what the particle's surroundings do
 *   23-31 zero (the network's input is padded to two 16-wide MMA k-steps)
 * Row-major, kFeatures floats per particle. */
constexpr int kFeatures = 32;
constexpr int kNbrFirst = 16, kNbrLast = 22; /* the neighbour-mean features */
struct DevCtl;
struct FeatureOut {
    float *feat = nullptr;             /* [n][kFeatures]; nullptr: no features */
    const float4 *dstep = nullptr;     /* step correction, home order */
    const float4 *ppos0 = nullptr, *ppos1 = nullptr;
    const DevCtl *ctl = nullptr;
    unsigned int *valid = nullptr;     /* set to 1 once features exist */
    int nbr = 1;                       /* 1: the neighbour means (16-22) too; 0: left zero */
};

/* Device control block of one context: the loop state that the reference
 * kept on the host (rx_sph_pbd_gpu.cpp:874-921). */
struct DevCtl {
    unsigned int iter;          /* iterations executed in this step */
    unsigned int done;          /* 1 when the loop must stop */
    unsigned int rebuild;       /* 1 when the grid must be rebuilt before the next pass */
    unsigned int builds;        /* grid builds in this step */
    unsigned int ticket;        /* last-block-done counter of the reducing kernels */
    unsigned int ticket2;
    unsigned int parity;        /* which ppos buffer holds the current x* */
    unsigned int nan_flag;
    unsigned int disp2_bits;    /* max |x* - xb|^2 of the last correction pass (float bits) */
    unsigned int mlp_err;       /* 1 when a tcgen05 inference gave up waiting on an MMA */
    float err1, err2, errmax;   /* errors of the last lambda pass */
    unsigned int bounds_bits;   /* FSPH_DEBUG_BOUNDS builds: the index checks that failed (kBound*) */
    unsigned int grab, grab2;   /* FSPH_DYN_CHUNKS: chunks handed out on demand (lambda, correction pass) */
};

/* Per-block partial sums of the lambda pass (one-sided, two-sided, max). */
struct ErrPartial {
    float s1, s2, mx, pad;
};
/* The same in fixed point (units of 2^-32, exact and order-free sums) for
 * the lambda pass with chunks handed out on demand; occupies two ErrPartial
 * slots per block. */
struct ErrPartialFix {
    unsigned long long s1, s2;
    float mx, pad[3];
};

__host__ __device__ inline float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ inline float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ inline float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ inline float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
__device__ inline float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

/* FSPH_POST_PRE 1 (default): m / rho is computed once per particle before
 * the XSPH pass (k_finalize, kb_mrho) and the XSPH pass hands (|omega|,
 * m / rho) to the vorticity pass, so neither divides nor takes a square
 * root per pair (0: per pair; the results are the same bit for bit).
 * Measured on the 1M double dam break: warm step 2.790 -> 2.714 ms, plain
 * step 9.758 -> 9.683 ms, positions bit-identical. */
#ifndef FSPH_POST_PRE
#define FSPH_POST_PRE 1
#endif
/* FSPH_SPH_DENSITY_LANES 1: the WCSPH density + list pass runs as many lanes
 * per particle as the force pass (k_sph_density_lanes), so small scenes fill
 * the GPU; 0: one thread per particle. */
#ifndef FSPH_SPH_DENSITY_LANES
#define FSPH_SPH_DENSITY_LANES 1
#endif
/* 1 / sqrt(max(r2, 1e-20)) for the pair loops.  FSPH_RSQRT_FTZ 1 (default)
 * issues rsqrt.approx.ftz.f32: the argument is clamped to a normal number
 * and the result is normal, so the flush-to-zero form, which skips the
 * handling of subnormal inputs, gives the same approximation as rsqrtf.
 * Measured on the 1 M double dam break: the same positions bit for bit,
 * lambda 80.1 -> 79.2 us, correction 88.7 -> 86.6 us, warm step 2.820 ->
 * 2.769 ms, plain step 10.08 -> 9.85 ms (0, rsqrtf, is the other form). */
#ifndef FSPH_RSQRT_FTZ
#define FSPH_RSQRT_FTZ 1
#endif
__device__ __forceinline__ float pair_rsqrt(float r2) {
    const float x = fmaxf(r2, 1e-20f);
#if FSPH_RSQRT_FTZ
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
#else
    return rsqrtf(x);
#endif
}
__device__ inline float3 cross3(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

/* Box-wall projection keeping the particle radius: clamp each axis to
 * [box_min + r, box_max - r].  This is the contact point of the reference's
 * rxSolidBox::GetDistanceR / AABB_point_dist (rx_sph_solid.cpp:44-108,
 * 244-262) for faces, edges and corners alike; velocity is not reflected,
 * as in rx_sph_pbd.cpp:1392. */
__device__ inline float3 wall_project(float3 x, const DevParams &p) {
    x.x = fminf(fmaxf(x.x, p.wall_lo.x), p.wall_hi.x);
    x.y = fminf(fmaxf(x.y, p.wall_lo.y), p.wall_hi.y);
    x.z = fminf(fmaxf(x.z, p.wall_lo.z), p.wall_hi.z);
    return x;
}

/* Obstacle projection: a point inside an obstacle moves to its surface --
 * a box (in its own rotated frame) through the nearest face, ties in x, y,
 * z order; a sphere radially -- as collisionPointBox / collisionPointSphere
 * (rx_cu_common.cu:748-831) with calCollisionSolidPB (rx_pbdsph_kernel.cu:
 * 863-911).  The velocity is left alone, as the CPU path leaves it
 * (rx_sph_pbd.cpp:1384; a PBF step recomputes it from the positions). */
__device__ inline float3 rot3(const float4 *r, float3 v) {
    return make_float3(r[0].x * v.x + r[0].y * v.y + r[0].z * v.z, r[1].x * v.x + r[1].y * v.y + r[1].z * v.z,
                       r[2].x * v.x + r[2].y * v.y + r[2].z * v.z);
}
__device__ inline float3 obstacle_project(float3 x, const DevParams &p) {
    for (int k = 0; k < p.nobs; ++k) {
        const Obstacle &o = p.obs[k];
        const float4 c4 = o.cen, e4 = o.ext;
        const float3 c = make_float3(c4.x, c4.y, c4.z);
        if (e4.w != 0.0f) { /* sphere */
            const float3 l = make_float3(x.x - c.x, x.y - c.y, x.z - c.z);
            const float ll = sqrtf(l.x * l.x + l.y * l.y + l.z * l.z);
            if (ll < c4.w && ll > 0.0f) {
                const float s = c4.w / ll;
                x = make_float3(c.x + s * l.x, c.y + s * l.y, c.z + s * l.z);
            }
        } else { /* box */
            float3 cp = rot3(o.rot, make_float3(x.x - c.x, x.y - c.y, x.z - c.z));
            const float tx = fabsf(cp.x) - e4.x, ty = fabsf(cp.y) - e4.y, tz = fabsf(cp.z) - e4.z;
            if (tx < 0.0f && ty < 0.0f && tz < 0.0f) {
                const float ax = -tx, ay = -ty, az = -tz;
                if (ax <= ay && ax <= az) cp.x = cp.x > 0.0f ? e4.x : -e4.x;
                else if (ay <= ax && ay <= az) cp.y = cp.y > 0.0f ? e4.y : -e4.y;
                else cp.z = cp.z > 0.0f ? e4.z : -e4.z;
                const float3 w = rot3(o.inv, cp);
                x = make_float3(w.x + c.x, w.y + c.y, w.z + c.z);
            }
        }
    }
    return x;
}
/* ---- triangle-mesh obstacles: the reference's GPU rule ---- */
/* IEEE single-precision operations with no fused multiply-add, so that the
 * rule can be restated bit for bit on the CPU; the reference's own build lets
 * the compiler fuse and normalises with an approximate rsqrtf, so it may
 * differ in the last bits. */
__device__ inline float3 psub(float3 a, float3 b) {
    return make_float3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}
__device__ inline float3 padd(float3 a, float3 b) {
    return make_float3(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z));
}
__device__ inline float3 pscale(float3 a, float s) {
    return make_float3(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s));
}
__device__ inline float pdot(float3 a, float3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ inline float3 pcross(float3 a, float3 b) {
    return make_float3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)),
                       __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
                       __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
__device__ inline float plength(float3 a) { return __fsqrt_rn(pdot(a, a)); }
__device__ inline float3 pnormalize(float3 a) {
    const float l = plength(a);
    return make_float3(__fdiv_rn(a.x, l), __fdiv_rn(a.y, l), __fdiv_rn(a.z, l));
}

/* intersectSegmentTriangle (rx_cu_common.cu:891-975): 1 when the segment
 * P0 -> P1 enters the triangle from its front side (I = the crossing point,
 * n = the unit normal), 0 when not, 2 when it lies in the triangle's plane,
 * -1 for a degenerate triangle.  The reference lets a zero-area triangle
 * through its zero-vector test as NaN and reports a hit at a NaN point;
 * here it is -1. */
__device__ inline int seg_triangle(float3 P0, float3 P1, float3 V0, float3 V1, float3 V2, float3 &I, float3 &n) {
    const float3 u = psub(V1, V0), v = psub(V2, V0);
    const float3 c = pcross(u, v);
    if (pdot(c, c) == 0.0f) return -1;
    n = pnormalize(c);
    if (fabsf(n.x) < 1.0e-10 && fabsf(n.y) < 1.0e-10 && fabsf(n.z) < 1.0e-10) return -1;
    const float3 dir = psub(P1, P0);
    const float a = pdot(n, psub(P0, V0));
    const float b = pdot(n, dir);
    if ((double)fabsf(b) < 1e-10) return a == 0.0f ? 2 : 0;
    const float r = __fdiv_rn(-a, b);
    if (r < 0.0f || fabsf(a) > fabsf(b) || b > 0.0f) return 0;
    I = padd(P0, pscale(dir, r));
    const float uu = pdot(u, u), uv = pdot(u, v), vv = pdot(v, v);
    const float3 w = psub(I, V0);
    const float wu = pdot(w, u), wv = pdot(w, v);
    const float D = __fsub_rn(__fmul_rn(uv, uv), __fmul_rn(uu, vv));
    const float sp = __fdiv_rn(__fsub_rn(__fmul_rn(uv, wv), __fmul_rn(vv, wu)), D);
    if (sp < 0.0f || sp > 1.0f) return 0;
    const float tp = __fdiv_rn(__fsub_rn(__fmul_rn(uv, wu), __fmul_rn(uu, wv)), D);
    if (tp < 0.0f || __fadd_rn(sp, tp) > 1.0f) return 0;
    return 1;
}

/* calCollisionPolygonPB (rx_pbdsph_kernel.cu:916-936) with the reference's
 * restitution 0 (rx_sph_pbd_gpu.cpp:103): on a hit, x1 moves back to the
 * crossing point plus the reflected velocity over the remaining part of
 * the step, and v loses its component into the triangle. */
__device__ inline void polygon_hit(float3 x0, float3 &x1, float3 &v, float3 V0, float3 V1, float3 V2, float dt) {
    float3 cp, n;
    if (seg_triangle(x0, x1, V0, V1, V2, cp, n) != 1) return;
    const float d = plength(psub(x1, cp));
    n = pnormalize(n);
    const float3 vr = pscale(pscale(n, -1.0f), pdot(n, v));
    const float l = plength(psub(x1, x0));
    x1 = padd(cp, pscale(vr, __fdiv_rn(__fmul_rn(dt, d), l)));
    v = padd(v, vr);
}

/* calcGridPos / calcGridHash of the reference's GPU grid (float floor, clamped). */
__device__ inline unsigned int poly_cell(float3 x, const PolyTable &t) {
    int c[3];
    const float xs[3] = {x.x, x.y, x.z}, os[3] = {t.org.x, t.org.y, t.org.z};
    const int g[3] = {t.gx, t.gy, t.gz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float f = floorf(__fdiv_rn(__fsub_rn(xs[a], os[a]), t.cw));
        const int k = f != f ? 0 : (int)fminf(fmaxf(f, -1.0f), (float)g[a]);
        c[a] = k < 0 ? 0 : (k >= g[a] ? g[a] - 1 : k);
    }
    return ((unsigned int)c[2] * (unsigned int)t.gy + (unsigned int)c[1]) * (unsigned int)t.gx + (unsigned int)c[0];
}

/* The segment x0 -> x1 (with velocity v) against the triangles of the cells
 * of x0 and of x1, in that order, both visited even when they are the same
 * cell (pbdsphIntegrateWithPolygon, rx_pbdsph_kernel.cu:985-1030). */
__device__ inline void polygon_collide(float3 x0, float3 &x1, float3 &v, float dt, const DevParams &p) {
    const PolyTable &t = p.poly;
    const unsigned int cells[2] = {poly_cell(x0, t), poly_cell(x1, t)};
#pragma unroll 1
    for (int k = 0; k < 2; ++k) {
        const unsigned int s = t.start[cells[k]];
        if (s == 0xffffffffu) continue;
        const unsigned int e = t.end[cells[k]];
        for (unsigned int j = s; j < e; ++j) {
            const int4 tri = t.tris[t.idx[j]];
            polygon_hit(x0, x1, v, f3(t.vrts[tri.x]), f3(t.vrts[tri.y]), f3(t.vrts[tri.z]), dt);
        }
    }
}

/* obstacles, then the box walls (the order of rx_sph_pbd.cpp:1380-1395) */
__device__ inline float3 solid_project(float3 x, const DevParams &p) {
    if (p.nobs) x = obstacle_project(x, p);
    return wall_project(x, p);
}

/* Cell coordinates of a position, clamped to the interior cells [1, G-2] so
 * that every 27-cell neighbourhood stays inside the padded table. */
__device__ inline int3 cell_of(float3 x, const DevParams &p) {
    float fx = (x.x - p.grid_origin.x) * p.inv_cw;
    float fy = (x.y - p.grid_origin.y) * p.inv_cw;
    float fz = (x.z - p.grid_origin.z) * p.inv_cw;
    int cx = (fx == fx) ? (int)floorf(fminf(fmaxf(fx, 1.0f), (float)(p.gx - 2))) : 1;
    int cy = (fy == fy) ? (int)floorf(fminf(fmaxf(fy, 1.0f), (float)(p.gy - 2))) : 1;
    int cz = (fz == fz) ? (int)floorf(fminf(fmaxf(fz, 1.0f), (float)(p.gz - 2))) : 1;
    return make_int3(cx, cy, cz);
}

__device__ inline unsigned int cell_index(int3 c, const DevParams &p) {
    return p.cell_off +
           ((unsigned int)c.z * (unsigned int)p.gy + (unsigned int)c.y) * (unsigned int)p.gx + (unsigned int)c.x;
}

/* Slot range [s, e) of the three cells x-1..x+1 in row (y + dy, z + dz). */
__device__ inline void row_range(const unsigned int *__restrict__ cell_start, int3 c, int dy, int dz,
                                 const DevParams &p, unsigned int &s, unsigned int &e) {
    unsigned int base = p.cell_off +
                        ((unsigned int)(c.z + dz) * (unsigned int)p.gy + (unsigned int)(c.y + dy)) * (unsigned int)p.gx +
                        (unsigned int)c.x;
    if (!cell_row_ok(p, base)) { s = e = 0u; return; }
    s = __ldg(cell_start + base - 1);
    e = bounded(p, __ldg(cell_start + base + 2), (unsigned int)p.n + 1u, kBoundSlot);
}

/* Warp/block reductions. */
__device__ inline float warp_sum(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ inline float warp_max(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

}  // namespace fsph
