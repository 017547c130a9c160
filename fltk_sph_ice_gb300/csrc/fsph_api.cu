/*
 * fsph_api.cu -- the C ABI of include/fsph.h: context, parameters, particle
 * data, the step orchestration and the parity entry points.
 *
 * Step orchestration replaces rxPBDSPH_GPU::Update (rx_sph_pbd_gpu.cpp:790-957)
 * and rxSPH_GPU::Update (rx_sph_gpu.cpp:756-923).  Differences by design:
 *   - no host round trip inside the PBF loop: the lambda kernel reduces the
 *     density error and decides on the device whether to continue; with
 *     use_graph the whole step is one CUDA graph whose iteration loop is a
 *     conditional WHILE node (the reference synchronised and copied the scan
 *     result to the host every iteration, rx_sph.cu:668-691);
 *   - the grid is built once per step on x* (cell width h (1 + skin)) and
 *     rebuilt inside the loop only when a particle has moved more than
 *     skin * h since the build (a conditional IF node), instead of at every
 *     iteration (rx_sph_pbd_gpu.cpp:876); the neighbour criterion is always
 *     evaluated on the current x*, so the neighbour sets are the same;
 *   - particles stay in cell order across steps; getters map back to the
 *     caller's particle order through the device slot -> particle index map;
 *   - no GL buffers and no CPU neighbour mirror (rx_sph_pbd_gpu.cpp:962-1011).
 */
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/fsph.h"
#include "fsph_kernels.cuh"
#include "fsph_mlp.cuh"

using namespace fsph;

namespace {
const double kPi = 3.14159265358979323846;

/* NVTX range for the duration of a scope (seen by ncu / Nsight; free when
 * no tool is attached) */
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

/* device-allocation fault injection (test hook, process-wide): an
 * allocation larger than g_alloc_max_bytes (>= 0), or the allocation
 * numbered g_alloc_fail_at (counted from the last fsph_set_alloc_fault),
 * returns FSPH_OOM without calling cudaMalloc */
std::atomic<long long> g_alloc_max_bytes{-1};
std::atomic<long long> g_alloc_fail_at{-1};
std::atomic<long long> g_alloc_count{0};
bool alloc_faulted(size_t bytes) {
    const long long k = g_alloc_count.fetch_add(1);
    const long long mx = g_alloc_max_bytes.load();
    return (mx >= 0 && (long long)bytes > mx) || k == g_alloc_fail_at.load();
}
}

struct BufSet {
    float4 *pos = nullptr, *vel = nullptr;
    unsigned int *id = nullptr, *attr = nullptr;
};

struct fsph_ctx {
    fsph_params P{};
    DevParams dp{};
    int n = 0;
    int cap = 0;
    int device = 0;
    cudaStream_t stream = nullptr, s2 = nullptr, s3 = nullptr;
    BufSet set[2];
    float4 *ppos[2] = {nullptr, nullptr};
    float4 *xb = nullptr, *acc = nullptr, *vort = nullptr;
    float *mrho = nullptr;  /* m / rho per particle, for the XSPH and vorticity passes */
    float2 *wm = nullptr;   /* (|omega|, m / rho) per particle, from the XSPH pass to the vorticity pass */
    float *dens = nullptr, *pres = nullptr;
    unsigned int *key = nullptr, *rank = nullptr, *perm = nullptr;
    NbrLists nl;
    unsigned int *count = nullptr, *cell_start = nullptr, *block_sums = nullptr;
    unsigned int ncells = 0;
    int gdim[3] = {0, 0, 0};
    DevCtl *ctl = nullptr;
    DevCtl *ctl_host = nullptr;
    unsigned int *flag = nullptr;      /* input-validation flag */
    unsigned int *flag_host = nullptr;
    /* warm start */
    float4 *xpred = nullptr;           /* x* before the iterations, iteration order */
    float4 *dstep = nullptr;           /* x*_final - x*_pred of the last step, home order */
    float4 *dwarm = nullptr;           /* predicted correction for the coming step, home order */
    float4 *tmp4 = nullptr;            /* scratch stream for reorders */
    float *feat = nullptr;             /* [n][kFeatures], home order */
    unsigned int *warm_valid = nullptr;
    MlpDev *mlp_dev = nullptr;
    bool model_loaded = false;
    bool model_nbr = true;          /* the loaded network uses the neighbour-mean features */
    ErrPartial *epart = nullptr;
    float *dpart = nullptr;
    cudaGraphExec_t gexec = nullptr;
    cudaGraph_t graph = nullptr;
    bool graph_valid = false;
    bool home_identity = true;  /* set[0] holds the particles in particle order (id = slot) */
    unsigned int *res_id = nullptr; /* slot order of the last step's results after a SetArrayVBO */
    bool res_in_res_id = false;     /* results are ordered by res_id rather than set[0].id */
    float graph_dt = 0.0f;
    int graph_n = -1;
    /* kernel nodes of the step graph: outside the loop, per iteration, per grid rebuild */
    int k_top = 0, k_iter = 0, k_rebuild = 0;
    /* static boundary particles, sorted by the cells of the fluid grid */
    int nb = 0;
    float4 *b_in = nullptr;            /* as given, input order */
    float4 *b_pos = nullptr;           /* sorted; .w = rho0 psi_b / m */
    float *b_lam = nullptr, *b_scale = nullptr;
    float2 *b_stat = nullptr;
    unsigned int *b_id = nullptr, *b_key = nullptr, *b_rank = nullptr;
    unsigned int *b_count = nullptr, *b_cell = nullptr;
    unsigned char *b_near = nullptr;
    /* dynamic particle count: slots [0, n_active) of the home set take part
     * in the steps, [n_active, n) are deleted particles (attribute -1)
     * parked at the reference's far point */
    int n_active = 0;
    unsigned int *part_scan = nullptr, *part_bsum = nullptr;
    struct Inlet {
        double pos1[3], pos2[3], vel[3], up[3], spacing;
        int accum, span;
    };
    std::vector<Inlet> inlets;
    int inlet_start = -1;
    std::vector<float4> del_regions; /* (lo, hi) pairs */
    float4 *del_dev = nullptr;
    /* analytic obstacles: boxes first, then spheres, as uploaded */
    std::vector<Obstacle> boxes, spheres;
    Obstacle *obs_dev = nullptr;
    int nobs_dev = 0;
    /* triangle-mesh obstacles: vertices (x, y, z floats) and triangles (3
     * vertex indices) as given, and their device copies with the cell table */
    std::vector<float> poly_v;
    std::vector<int> poly_t;
    float4 *poly_vrts = nullptr;
    int4 *poly_tris = nullptr;
    unsigned int *poly_start = nullptr, *poly_end = nullptr, *poly_idx = nullptr;
    PolyTable poly{};
    int ntri_dev = 0;
    bool last_step_graph = false;
    bool stats_pending = false;
    /* per-step JSON-lines record (fsph_set_step_log) */
    FILE *log = nullptr;
    long long steps_done = 0;
    /* set when a reallocation failed part-way: the buffers are incomplete
     * and every call that touches them is refused until fsph_set_params
     * reallocates successfully */
    bool broken = false;
    RadixBufs radix; /* grid_sort 1 */
    std::string err;
};

namespace {

#define FSPH_CUDA(ctx, call)                                                                  \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            (ctx)->err = std::string(#call) + ": " + cudaGetErrorString(e_);                  \
            return e_ == cudaErrorMemoryAllocation ? FSPH_OOM : FSPH_CUDA_ERROR;              \
        }                                                                                     \
    } while (0)

#define FSPH_TRY(expr)             \
    do {                           \
        int st_ = (expr);          \
        if (st_ != FSPH_OK) return st_; \
    } while (0)

int fail(fsph_ctx *c, int st, const std::string &msg) {
    if (c) c->err = msg;
    return st;
}

#define FSPH_USABLE(c)                                                                                       \
    do {                                                                                                     \
        if (!(c)) return FSPH_INVALID_ARG;                                                                   \
        if ((c)->broken)                                                                                     \
            return fail((c), FSPH_OOM, "buffers lost in a failed reallocation; call fsph_set_params again"); \
    } while (0)

/* ---------------- parameters ---------------- */

double poly6_coef(double h) { return 315.0 / (64.0 * kPi * std::pow(h, 9.0)); }

int validate(const fsph_params &p, std::string &why) {
    if (p.solver != FSPH_SOLVER_WCSPH && p.solver != FSPH_SOLVER_PBF) { why = "unknown solver"; return FSPH_INVALID_ARG; }
    if (p.max_particles < 0) { why = "max_particles < 0"; return FSPH_INVALID_ARG; }
    if (!(p.h > 0.0f) || !std::isfinite(p.h)) { why = "h must be positive and finite"; return FSPH_INVALID_ARG; }
    if (!(p.mass > 0.0f)) { why = "mass must be positive"; return FSPH_INVALID_ARG; }
    if (!(p.rest_dens > 0.0f)) { why = "rest_dens must be positive"; return FSPH_INVALID_ARG; }
    if (p.particle_radius < 0.0f) { why = "particle_radius < 0"; return FSPH_INVALID_ARG; }
    for (int a = 0; a < 3; ++a) {
        if (!std::isfinite(p.box_min[a]) || !std::isfinite(p.box_max[a])) { why = "box not finite"; return FSPH_INVALID_ARG; }
        if (!(p.box_max[a] - p.box_min[a] > 2.0 * p.particle_radius)) { why = "box thinner than a particle"; return FSPH_INVALID_ARG; }
    }
    if (p.solver == FSPH_SOLVER_PBF) {
        if (p.max_iter < 1) { why = "max_iter must be >= 1"; return FSPH_INVALID_ARG; }
        if (p.min_iter < 0) { why = "min_iter < 0"; return FSPH_INVALID_ARG; }
        if (!(p.epsilon >= 0.0f)) { why = "epsilon < 0"; return FSPH_INVALID_ARG; }
        if (p.error_mode != FSPH_ERR_ONE_SIDED && p.error_mode != FSPH_ERR_TWO_SIDED) { why = "error_mode"; return FSPH_INVALID_ARG; }
        if (p.use_ap && !(p.ap_q > 0.0f && p.ap_q < 1.0f)) { why = "ap_q must lie in (0, 1)"; return FSPH_INVALID_ARG; }
    }
    if (p.cell_skin < 0.0f || p.cell_skin > 1.0f) { why = "cell_skin must lie in [0, 1]"; return FSPH_INVALID_ARG; }
    if (p.warm_start < 0 || p.warm_start > 1) { why = "warm_start must be 0 or 1"; return FSPH_INVALID_ARG; }
    if (p.grid_sort < 0 || p.grid_sort > 1) { why = "grid_sort must be 0 or 1"; return FSPH_INVALID_ARG; }
    if (p.mlp_tcgen05 < 0 || p.mlp_tcgen05 > 2) { why = "mlp_tcgen05 must be 0, 1 or 2"; return FSPH_INVALID_ARG; }
    return FSPH_OK;
}

/* Grid geometry: cell width h (1 + skin), the box padded by one cell. */
void grid_geometry(const fsph_params &p, double &cw, double org[3], int g[3]) {
    double skin = std::max((double)p.cell_skin, 1e-3);
    cw = (double)p.h * (1.0 + skin);
    for (int a = 0; a < 3; ++a) {
        org[a] = p.box_min[a] - cw;
        g[a] = (int)std::ceil((p.box_max[a] - p.box_min[a]) / cw) + 2;
        if (g[a] < 3) g[a] = 3;
    }
}

DevParams make_dev(const fsph_params &p, int n, float dt) {
    DevParams d{};
    d.n = n;
    d.h = p.h;
    d.h2 = p.h * p.h;
    d.mass = p.mass;
    d.rest_dens = p.rest_dens;
    d.inv_rest_dens = 1.0f / p.rest_dens;
    double h = (double)p.h;
    d.aw = (float)poly6_coef(h);
    d.aw_d = poly6_coef(h);
    d.ag = (float)(-45.0 / (kPi * std::pow(h, 6.0)));
    d.al = (float)(45.0 / (kPi * std::pow(h, 6.0)));
    double r = (double)p.particle_radius;
    d.wall_lo = make_float3((float)(p.box_min[0] + r), (float)(p.box_min[1] + r), (float)(p.box_min[2] + r));
    d.wall_hi = make_float3((float)(p.box_max[0] - r), (float)(p.box_max[1] - r), (float)(p.box_max[2] - r));
    d.gravity = make_float3(p.gravity[0], p.gravity[1], p.gravity[2]);
    d.viscosity = p.viscosity;
    d.gas_k = p.gas_k;
    d.epsilon = p.epsilon;
    d.eta = p.eta;
    d.min_iter = p.min_iter;
    d.max_iter = p.max_iter;
    d.error_mode = p.error_mode;
    d.clamp_constraint = p.clamp_constraint;
    d.use_ap = p.use_ap;
    d.ap_k = p.ap_k;
    d.ap_n = p.ap_n;
    if (p.use_ap) {
        float dq = p.ap_q * p.h;
        double q = h * h - (double)dq * (double)dq;
        double wq = poly6_coef(h) * q * q * q;
        d.inv_wq = (float)(1.0 / wq);
    }
    d.xsph_c = p.xsph_c;
    d.vort_eps = p.vort_eps;
    double cw, org[3];
    int g[3];
    grid_geometry(p, cw, org, g);
    d.grid_origin = make_float3((float)org[0], (float)org[1], (float)org[2]);
    d.inv_cw = (float)(1.0 / cw);
    d.gx = g[0]; d.gy = g[1]; d.gz = g[2];
    /* lists hold every pair within the cell width at the build, so they stay
     * complete while no particle has moved more than half the skin */
    double skin_len = 0.5 * (cw - h) * 0.999;
    d.skin2 = (float)(skin_len * skin_len);
    d.rl2 = (float)(cw * cw);
    d.use_lists = p.walk_cells ? 0 : 1;
    d.compensated = p.compensated_density ? 1 : 0;
    d.dt = dt;
    d.inv_dt = dt != 0.0f ? 1.0f / dt : 0.0f;
    return d;
}

template <class T>
int dalloc(fsph_ctx *c, T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    if (alloc_faulted(count * sizeof(T))) return fail(c, FSPH_OOM, "device allocation refused (injected fault)");
    FSPH_CUDA(c, cudaMalloc((void **)p, count * sizeof(T)));
    return FSPH_OK;
}

void free_particles(fsph_ctx *c) {
    for (int k = 0; k < 2; ++k) {
        cudaFree(c->set[k].pos); cudaFree(c->set[k].vel); cudaFree(c->set[k].id); cudaFree(c->set[k].attr);
        c->set[k] = BufSet{};
        cudaFree(c->ppos[k]); c->ppos[k] = nullptr;
    }
    cudaFree(c->xb); cudaFree(c->acc); cudaFree(c->vort); cudaFree(c->dens); cudaFree(c->pres);
    cudaFree(c->key); cudaFree(c->rank); cudaFree(c->perm); cudaFree(c->epart); cudaFree(c->dpart);
    cudaFree(c->res_id); c->res_id = nullptr;
    cudaFree(c->part_scan); cudaFree(c->part_bsum);
    c->part_scan = c->part_bsum = nullptr;
    cudaFree(c->nl.list); cudaFree(c->nl.cnt); cudaFree(c->nl.cellb);
    c->nl = NbrLists{};
    cudaFree(c->xpred); cudaFree(c->dstep); cudaFree(c->dwarm); cudaFree(c->tmp4); cudaFree(c->feat);
    c->xpred = c->dstep = c->dwarm = c->tmp4 = nullptr;
    c->feat = nullptr;
    c->xb = c->acc = c->vort = nullptr;
    cudaFree(c->mrho); cudaFree(c->wm);
    c->mrho = nullptr;
    c->wm = nullptr;
    c->dens = c->pres = nullptr;
    c->key = c->rank = c->perm = nullptr;
    c->epart = nullptr;
    c->dpart = nullptr;
    cudaFree(c->radix.k0); cudaFree(c->radix.k1);
    cudaFree(c->radix.hist); cudaFree(c->radix.offs); cudaFree(c->radix.bsum);
    c->radix = RadixBufs{};
}

void free_grid(fsph_ctx *c) {
    cudaFree(c->count); cudaFree(c->cell_start); cudaFree(c->block_sums);
    c->count = c->cell_start = c->block_sums = nullptr;
    c->ncells = 0;
}

void free_boundary(fsph_ctx *c) {
    cudaFree(c->b_in); cudaFree(c->b_pos); cudaFree(c->b_lam); cudaFree(c->b_scale); cudaFree(c->b_stat);
    cudaFree(c->b_id); cudaFree(c->b_key); cudaFree(c->b_rank); cudaFree(c->b_count); cudaFree(c->b_cell);
    cudaFree(c->b_near);
    c->b_in = c->b_pos = nullptr;
    c->b_lam = c->b_scale = nullptr;
    c->b_stat = nullptr;
    c->b_id = c->b_key = c->b_rank = c->b_count = c->b_cell = nullptr;
    c->b_near = nullptr;
    c->nb = 0;
}

/* The boundary's fields of the device parameters (none when nb == 0). */
void attach_boundary(const fsph_ctx *c, DevParams &p) {
    p.nb = c->nb;
    p.bpos = c->b_pos;
    p.blam = c->b_lam;
    p.bcell = c->b_cell;
    p.bnear = c->b_near;
}

/* device parameters of the context for n particles */
DevParams dev_for(const fsph_ctx *c, int n, float dt) {
    DevParams p = make_dev(c->P, n, dt);
    attach_boundary(c, p);
    p.nobs = c->nobs_dev;
    p.obs = c->obs_dev;
    p.ntri = c->ntri_dev;
    p.poly = c->poly;
    p.dbg = &c->ctl->bounds_bits;
    return p;
}

/* Rotation of a box obstacle from Euler angles in degrees (pitch, yaw,
 * roll), rows world -> local, as EulerToMatrix (rx_sph_commons.h:185-210),
 * and its inverse (the transpose). */
void box_rotation(const double ang[3], Obstacle &o) {
    const double d2r = kPi / 180.0;
    const double cp = std::cos(ang[0] * d2r), sp = std::sin(ang[0] * d2r);
    const double cy = std::cos(ang[1] * d2r), sy = std::sin(ang[1] * d2r);
    const double cr = std::cos(ang[2] * d2r), sr = std::sin(ang[2] * d2r);
    const double cc = cy * cr, cs = cy * sr, sc = sy * cr, ss = sy * sr;
    const double m[3][3] = {{cc + sp * ss, cs - sp * sc, -sy * cp}, {-cp * sr, cp * cr, -sp},
                            {sc - sp * cs, ss + sp * cc, cy * cp}};
    for (int r = 0; r < 3; ++r) {
        o.rot[r] = make_float4((float)m[r][0], (float)m[r][1], (float)m[r][2], 0.0f);
        o.inv[r] = make_float4((float)m[0][r], (float)m[1][r], (float)m[2][r], 0.0f);
    }
}

/* the obstacle table on the device (boxes, then spheres) */
int upload_obstacles(fsph_ctx *c) {
    std::vector<Obstacle> all(c->boxes);
    all.insert(all.end(), c->spheres.begin(), c->spheres.end());
    if (!c->obs_dev) FSPH_CUDA(c, cudaMalloc((void **)&c->obs_dev, kMaxObstacles * sizeof(Obstacle)));
    if (!all.empty())
        FSPH_CUDA(c, cudaMemcpyAsync(c->obs_dev, all.data(), all.size() * sizeof(Obstacle), cudaMemcpyHostToDevice,
                                     c->stream));
    FSPH_CUDA(c, cudaStreamSynchronize(c->stream));
    if ((int)all.size() != c->nobs_dev) { /* the count is a launch constant of the captured step */
        c->nobs_dev = (int)all.size();
        c->graph_valid = false;
    }
    return FSPH_OK;
}

/* The reference's neighbour-search grid over the simulation range (the box
 * grown by 1 %, rx_sph_pbd.cpp:188-196): cw = L_max / 2^round(log2(L_max/h))
 * for both; the CPU grid (rxNNGrid::Setup, rx_nnsearch.h:174-199) rounds each
 * axis count to a power of two, the GPU grid (setupCells,
 * rx_sph_pbd_gpu.cpp:1986-2011) takes floor(L_axis / cw) + 1.  The same
 * double operations in the same order, so the same bits. */
int reference_grid(const fsph_params &P, int rule, double org[3], double &cw, int g[3]) {
    double lo[3], hi[3], ws[3];
    for (int a = 0; a < 3; ++a) {
        const double size = P.box_max[a] - P.box_min[a];
        lo[a] = P.box_min[a] - 0.5 * 0.01 * size;
        hi[a] = lo[a] + size * (1.0 + 0.01);
    }
    for (int a = 0; a < 3; ++a) ws[a] = hi[a] - lo[a];
    const double h = (double)P.h;
    const double max_axis = std::max(ws[0], std::max(ws[1], ws[2]));
    const int d = (int)(std::log(max_axis / h) / std::log(2.0) + 0.5);
    const int m = (int)(std::pow(2.0, (double)d) + 0.5);
    if (m <= 0) return FSPH_INVALID_ARG;
    cw = max_axis / m;
    for (int a = 0; a < 3; ++a) {
        org[a] = lo[a];
        if (rule == 0) {
            const int da = (int)(std::log(ws[a] / cw) / std::log(2.0) + 0.5);
            g[a] = (int)(std::pow(2.0, (double)da) + 0.5);
        } else {
            g[a] = (int)(ws[a] / cw) + 1;
        }
        if (g[a] < 1) return FSPH_INVALID_ARG;
    }
    if ((double)g[0] * g[1] * g[2] > 4294967295.0) return FSPH_INVALID_ARG;
    return FSPH_OK;
}

/* ---- triangle-mesh obstacles: the cell table ---- */

/* Triangle against the axis-aligned cube [-0.5, 0.5]^3 by separating axes
 * (Akenine-Moeller, "Fast 3D Triangle-Box Overlap Testing", 2001): the three
 * box normals, the triangle's normal and the nine edge cross products.  The
 * reference uses the Green-Hatch test (RXFunc::polygon_intersects_cube) for
 * the same question; the two differ only for triangles that touch a cell
 * without entering it. */
bool tri_cube_overlap(const double v[3][3]) {
    const double hb = 0.5;
    for (int a = 0; a < 3; ++a) { /* box normals: the triangle's extent */
        const double mn = std::min(v[0][a], std::min(v[1][a], v[2][a]));
        const double mx = std::max(v[0][a], std::max(v[1][a], v[2][a]));
        if (mn > hb || mx < -hb) return false;
    }
    double e[3][3];
    for (int k = 0; k < 3; ++k)
        for (int a = 0; a < 3; ++a) e[k][a] = v[(k + 1) % 3][a] - v[k][a];
    for (int k = 0; k < 3; ++k)
        for (int a = 0; a < 3; ++a) { /* axis = unit vector a x edge k */
            double ax[3] = {0.0, 0.0, 0.0};
            const int a1 = (a + 1) % 3, a2 = (a + 2) % 3;
            ax[a1] = -e[k][a2];
            ax[a2] = e[k][a1];
            double mn = 1e300, mx = -1e300;
            for (int j = 0; j < 3; ++j) {
                const double q = ax[0] * v[j][0] + ax[1] * v[j][1] + ax[2] * v[j][2];
                mn = std::min(mn, q);
                mx = std::max(mx, q);
            }
            const double rad = hb * (std::fabs(ax[0]) + std::fabs(ax[1]) + std::fabs(ax[2]));
            if (mn > rad || mx < -rad) return false;
        }
    double nrm[3] = {e[0][1] * e[1][2] - e[0][2] * e[1][1], e[0][2] * e[1][0] - e[0][0] * e[1][2],
                     e[0][0] * e[1][1] - e[0][1] * e[1][0]};
    const double dpl = nrm[0] * v[0][0] + nrm[1] * v[0][1] + nrm[2] * v[0][2];
    const double rad = hb * (std::fabs(nrm[0]) + std::fabs(nrm[1]) + std::fabs(nrm[2]));
    return std::fabs(dpl) <= rad;
}

void free_polygons(fsph_ctx *c) {
    cudaFree(c->poly_vrts); cudaFree(c->poly_tris);
    cudaFree(c->poly_start); cudaFree(c->poly_end); cudaFree(c->poly_idx);
    c->poly_vrts = nullptr; c->poly_tris = nullptr;
    c->poly_start = c->poly_end = c->poly_idx = nullptr;
    c->poly = PolyTable{};
    c->ntri_dev = 0;
}

/* Bin the triangles into the cells of the reference's GPU grid they
 * intersect (setPolysToCell, rx_sph_pbd_gpu.cpp:2051-2200: each triangle's
 * bounding box of cells, (b - origin) / cw truncated and clamped, each cell
 * tested against the triangle), a cell's triangles in ascending index as
 * its stable sort leaves them, and upload the mesh and the table.  The
 * reference never closes the last non-empty cell of its table (its loop
 * compares with the particle count), which drops that cell's triangles;
 * here every cell is closed. */
int polygons_upload(fsph_ctx *c) {
    FSPH_CUDA(c, cudaStreamSynchronize(c->stream));
    free_polygons(c);
    c->graph_valid = false;
    const int nv = (int)c->poly_v.size() / 3, nt = (int)c->poly_t.size() / 3;
    if (nt == 0) return FSPH_OK;
    double org[3], cwd;
    int g[3];
    if (reference_grid(c->P, 1, org, cwd, g) != FSPH_OK)
        return fail(c, FSPH_INVALID_ARG, "degenerate grid for this box and h");
    const float cwf = (float)cwd;
    const double len = (double)cwf;
    const unsigned int ncell = (unsigned int)g[0] * (unsigned int)g[1] * (unsigned int)g[2];
    std::vector<std::pair<unsigned int, unsigned int>> hits; /* (cell, triangle) */
    for (int i = 0; i < nt; ++i) {
        double V[3][3];
        for (int j = 0; j < 3; ++j)
            for (int a = 0; a < 3; ++a) V[j][a] = (double)c->poly_v[3 * (size_t)c->poly_t[3 * i + j] + a];
        int lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            const double bmin = std::min(V[0][a], std::min(V[1][a], V[2][a])) - org[a];
            const double bmax = std::max(V[0][a], std::max(V[1][a], V[2][a])) - org[a];
            const double fl = bmin / len, fh = bmax / len;
            lo[a] = fl < 0.0 ? (int)std::max(fl, -1.0) : (int)std::min(fl, (double)g[a]);
            hi[a] = fh < 0.0 ? (int)std::max(fh, -1.0) : (int)std::min(fh, (double)g[a]);
            lo[a] = std::min(std::max(lo[a], 0), g[a] - 1);
            hi[a] = std::min(std::max(hi[a], 0), g[a] - 1);
        }
        for (int x = lo[0]; x <= hi[0]; ++x)
            for (int y = lo[1]; y <= hi[1]; ++y)
                for (int z = lo[2]; z <= hi[2]; ++z) {
                    const double cen[3] = {org[0] + (x + 0.5) * len, org[1] + (y + 0.5) * len,
                                           org[2] + (z + 0.5) * len};
                    double vc[3][3];
                    for (int j = 0; j < 3; ++j)
                        for (int a = 0; a < 3; ++a) vc[j][a] = (V[j][a] - cen[a]) / len;
                    if (tri_cube_overlap(vc))
                        hits.push_back({((unsigned int)z * (unsigned int)g[1] + (unsigned int)y) * (unsigned int)g[0] +
                                            (unsigned int)x,
                                        (unsigned int)i});
                }
    }
    std::stable_sort(hits.begin(), hits.end(),
                     [](const std::pair<unsigned int, unsigned int> &a, const std::pair<unsigned int, unsigned int> &b) {
                         return a.first < b.first;
                     });
    std::vector<unsigned int> start(ncell, 0xffffffffu), end(ncell, 0u), idx(std::max<size_t>(hits.size(), 1), 0u);
    for (size_t k = 0; k < hits.size(); ++k) {
        idx[k] = hits[k].second;
        if (k == 0 || hits[k].first != hits[k - 1].first) start[hits[k].first] = (unsigned int)k;
        end[hits[k].first] = (unsigned int)k + 1;
    }
    std::vector<float4> hv((size_t)nv);
    for (int v = 0; v < nv; ++v) hv[v] = make_float4(c->poly_v[3 * v], c->poly_v[3 * v + 1], c->poly_v[3 * v + 2], 0.0f);
    std::vector<int4> ht((size_t)nt);
    for (int t = 0; t < nt; ++t) ht[t] = make_int4(c->poly_t[3 * t], c->poly_t[3 * t + 1], c->poly_t[3 * t + 2], 0);
    FSPH_TRY(dalloc(c, &c->poly_vrts, (size_t)nv));
    FSPH_TRY(dalloc(c, &c->poly_tris, (size_t)nt));
    FSPH_TRY(dalloc(c, &c->poly_start, (size_t)ncell));
    FSPH_TRY(dalloc(c, &c->poly_end, (size_t)ncell));
    FSPH_TRY(dalloc(c, &c->poly_idx, idx.size()));
    FSPH_CUDA(c, cudaMemcpy(c->poly_vrts, hv.data(), hv.size() * sizeof(float4), cudaMemcpyHostToDevice));
    FSPH_CUDA(c, cudaMemcpy(c->poly_tris, ht.data(), ht.size() * sizeof(int4), cudaMemcpyHostToDevice));
    FSPH_CUDA(c, cudaMemcpy(c->poly_start, start.data(), start.size() * 4, cudaMemcpyHostToDevice));
    FSPH_CUDA(c, cudaMemcpy(c->poly_end, end.data(), end.size() * 4, cudaMemcpyHostToDevice));
    FSPH_CUDA(c, cudaMemcpy(c->poly_idx, idx.data(), idx.size() * 4, cudaMemcpyHostToDevice));
    PolyTable &t = c->poly;
    t.vrts = c->poly_vrts;
    t.tris = c->poly_tris;
    t.start = c->poly_start;
    t.end = c->poly_end;
    t.idx = c->poly_idx;
    t.org = make_float3((float)org[0], (float)org[1], (float)org[2]);
    t.cw = cwf;
    t.gx = g[0]; t.gy = g[1]; t.gz = g[2];
    c->ntri_dev = nt;
    return FSPH_OK;
}

void drop_graph(fsph_ctx *c) {
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    if (c->graph) cudaGraphDestroy(c->graph);
    c->gexec = nullptr;
    c->graph = nullptr;
    c->graph_valid = false;
}

int alloc_particles(fsph_ctx *c, int cap) {
    free_particles(c);
    size_t n = (size_t)std::max(cap, 1);
    for (int k = 0; k < 2; ++k) {
        FSPH_TRY(dalloc(c, &c->set[k].pos, n)); FSPH_TRY(dalloc(c, &c->set[k].vel, n));
        FSPH_TRY(dalloc(c, &c->set[k].id, n)); FSPH_TRY(dalloc(c, &c->set[k].attr, n));
        FSPH_TRY(dalloc(c, &c->ppos[k], n));
    }
    FSPH_TRY(dalloc(c, &c->xb, n)); FSPH_TRY(dalloc(c, &c->acc, n)); FSPH_TRY(dalloc(c, &c->vort, n));
    FSPH_TRY(dalloc(c, &c->mrho, n)); FSPH_TRY(dalloc(c, &c->wm, n));
    FSPH_TRY(dalloc(c, &c->dens, n)); FSPH_TRY(dalloc(c, &c->pres, n));
    FSPH_TRY(dalloc(c, &c->key, n)); FSPH_TRY(dalloc(c, &c->rank, n)); FSPH_TRY(dalloc(c, &c->perm, n));
    FSPH_TRY(dalloc(c, &c->res_id, n));
    FSPH_TRY(dalloc(c, &c->part_scan, n + 1));
    FSPH_TRY(dalloc(c, &c->part_bsum, scan_blocks((unsigned int)n)));
    FSPH_TRY(dalloc(c, &c->nl.list, n * kListMax)); FSPH_TRY(dalloc(c, &c->nl.cnt, n));
    FSPH_TRY(dalloc(c, &c->nl.cellb, n));
    FSPH_TRY(dalloc(c, &c->xpred, n)); FSPH_TRY(dalloc(c, &c->dstep, n)); FSPH_TRY(dalloc(c, &c->dwarm, n));
    FSPH_TRY(dalloc(c, &c->tmp4, n)); FSPH_TRY(dalloc(c, &c->feat, n * kFeatures));
    FSPH_CUDA(c, cudaMemsetAsync(c->dstep, 0, n * sizeof(float4), c->stream));
    FSPH_CUDA(c, cudaMemsetAsync(c->feat, 0, n * kFeatures * sizeof(float), c->stream));
    {
        const size_t nt = radix_tiles((int)n), nh = nt * 256;
        FSPH_TRY(dalloc(c, &c->radix.k0, n)); FSPH_TRY(dalloc(c, &c->radix.k1, n));
        FSPH_TRY(dalloc(c, &c->radix.hist, nh)); FSPH_TRY(dalloc(c, &c->radix.offs, nh + 1)); /* + the total */
        FSPH_TRY(dalloc(c, &c->radix.bsum, scan_blocks((unsigned int)nh)));
    }
    FSPH_TRY(dalloc(c, &c->epart, 2 * blocks_for((long long)n, kPassBlock))); /* room for ErrPartialFix */
    FSPH_TRY(dalloc(c, &c->dpart, blocks_for((long long)n, kPassBlock)));
    for (int k = 0; k < 2; ++k) {
        FSPH_CUDA(c, cudaMemsetAsync(c->set[k].pos, 0, n * sizeof(float4), c->stream));
        FSPH_CUDA(c, cudaMemsetAsync(c->set[k].vel, 0, n * sizeof(float4), c->stream));
        FSPH_CUDA(c, cudaMemsetAsync(c->set[k].attr, 0, n * sizeof(unsigned int), c->stream));
        FSPH_CUDA(c, cudaMemsetAsync(c->ppos[k], 0, n * sizeof(float4), c->stream));
    }
    FSPH_CUDA(c, cudaMemsetAsync(c->acc, 0, n * sizeof(float4), c->stream));
    FSPH_CUDA(c, cudaMemsetAsync(c->vort, 0, n * sizeof(float4), c->stream));
    FSPH_CUDA(c, cudaMemsetAsync(c->dens, 0, n * sizeof(float), c->stream));
    FSPH_CUDA(c, cudaMemsetAsync(c->pres, 0, n * sizeof(float), c->stream));
    c->cap = cap;
    return FSPH_OK;
}

int alloc_grid(fsph_ctx *c) {
    double cw, org[3];
    int g[3];
    grid_geometry(c->P, cw, org, g);
    double cells = (double)g[0] * g[1] * g[2];
    if (cells > (double)(1u << 28))
        return fail(c, FSPH_INVALID_ARG, "box / h gives more than 2^28 grid cells");
    unsigned int nc = (unsigned int)cells;
    if (nc == c->ncells && c->count) {
        std::memcpy(c->gdim, g, sizeof(g));
        return FSPH_OK;
    }
    free_grid(c);
    FSPH_TRY(dalloc(c, &c->count, nc));
    FSPH_TRY(dalloc(c, &c->cell_start, (size_t)nc + 1));
    FSPH_TRY(dalloc(c, &c->block_sums, scan_blocks(nc)));
    FSPH_CUDA(c, cudaMemsetAsync(c->count, 0, (size_t)nc * sizeof(unsigned int), c->stream));
    c->ncells = nc;
    std::memcpy(c->gdim, g, sizeof(g));
    return FSPH_OK;
}

/* Sort the static boundary by the cells of the current grid and derive its
 * per-cell table, volumes and static lambda_b parts (after every grid
 * (re)allocation). */
int boundary_build(fsph_ctx *c) {
    if (c->nb == 0) return FSPH_OK;
    cudaStream_t s = c->stream;
    cudaFree(c->b_count); cudaFree(c->b_cell); cudaFree(c->b_near);
    c->b_count = c->b_cell = nullptr;
    c->b_near = nullptr;
    FSPH_TRY(dalloc(c, &c->b_count, c->ncells));
    FSPH_TRY(dalloc(c, &c->b_cell, (size_t)c->ncells + 1));
    FSPH_TRY(dalloc(c, &c->b_near, c->ncells));
    FSPH_CUDA(c, cudaMemsetAsync(c->b_count, 0, (size_t)c->ncells * sizeof(unsigned int), s));
    DevParams p = make_dev(c->P, c->nb, 1.0f); /* n = the boundary count */
    launch_hash(p, c->b_in, c->b_key, c->b_rank, c->b_count, s);
    launch_scan(c->b_count, c->b_cell, c->block_sums, c->ncells, s);
    launch_scatter_sort(p, c->b_key, c->b_rank, c->b_cell, c->b_id, c->ncells, s); /* b_id: slot -> input */
    Gather g{};
    g.n4 = 1;
    g.src4[0] = c->b_in;
    g.dst4[0] = c->b_pos;
    launch_gather(c->nb, c->b_id, g, nullptr, s);
    attach_boundary(c, p);
    launch_boundary_near(p, c->ncells, c->b_near, s);
    launch_boundary_volume(p, c->b_scale, s);
    launch_pack_w(c->nb, c->b_pos, c->b_scale, s);
    launch_boundary_static(p, c->b_stat, s);
    FSPH_CUDA(c, cudaMemsetAsync(c->b_lam, 0, (size_t)c->nb * sizeof(float), s));
    FSPH_CUDA(c, cudaGetLastError());
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    return FSPH_OK;
}

/* ---------------- building blocks of a step ---------------- */

/* perm = the slots in (cell, previous slot) order, from the hashed cells:
 * the counting sort (grid_sort 0) or the LSD radix sort (grid_sort 1) */
void sort_cells(fsph_ctx *c, const DevParams &p, cudaStream_t s) {
    if (c->P.grid_sort == 1) launch_radix_sort_cells(p.n, c->key, c->ncells, c->radix, c->perm, s);
    else launch_scatter_sort(p, c->key, c->rank, c->cell_start, c->perm, c->ncells, s);
}

/* sort of the slots of x (device order) by cell: leaves perm */
void enqueue_sort(fsph_ctx *c, const DevParams &p, const float4 *x, cudaStream_t s) {
    launch_hash(p, x, c->key, c->rank, c->count, s);
    launch_scan(c->count, c->cell_start, c->block_sums, c->ncells, s);
    sort_cells(c, p, s);
}

/* the grid rebuild used inside the loop and after it (positions = current x*) */
void enqueue_rebuild(fsph_ctx *c, const DevParams &p, int it, cudaStream_t s) {
    BufSet &I = c->set[it], &O = c->set[1 - it];
    launch_hash_parity(p, c->ppos[0], c->ppos[1], c->ctl, c->key, c->rank, c->count, s);
    launch_scan(c->count, c->cell_start, c->block_sums, c->ncells, s);
    sort_cells(c, p, s);
    const bool ws = c->P.warm_start != 0 || c->P.collect_features != 0;
    float *t_lam = reinterpret_cast<float *>(c->rank); /* free once the scatter has run */
    launch_rebuild_gather(p.n, c->perm, c->ctl, I.pos, c->ppos[0], c->ppos[1], I.id, I.attr, c->dens, O.pos, O.vel,
                          O.id, O.attr, c->pres, c->key, c->nl.cellb, ws ? c->xpred : nullptr, c->tmp4, t_lam, s);
    launch_rebuild_copy(p.n, c->ctl, O.pos, O.vel, O.id, O.attr, c->pres, I.pos, c->ppos[0], c->ppos[1], c->xb, I.id,
                        I.attr, c->dens, c->tmp4, ws ? c->xpred : nullptr, t_lam, s);
    launch_build_list(p, c->cell_start, c->xb, c->nl, s);
}

bool pbf_prepass(const fsph_ctx *c) { return c->P.viscosity != 0.0f; }
/* step corrections and features are produced (warm start on, or collection) */
bool pbf_warm_active(const fsph_ctx *c) { return c->P.warm_start != 0 || c->P.collect_features != 0; }
bool pbf_finalize_ext(const fsph_ctx *c) {
    return c->P.xsph_c != 0.0f || c->P.vort_eps != 0.0f || pbf_warm_active(c);
}

/* PBF: pre-pass, prediction, first grid build; returns the set that carries
 * the particles through the iterations. */
int enqueue_pbf_pre(fsph_ctx *c, const DevParams &p, cudaStream_t s) {
    cudaMemsetAsync(c->ctl, 0, sizeof(DevCtl), s);
    const bool ws = pbf_warm_active(c);
    /* warm-start correction of every particle, home order */
    const float4 *dw = nullptr;
    if (c->P.warm_start == 1) {
        if (c->P.mlp_tcgen05)
            launch_mlp_infer_tc(c->mlp_dev, c->feat, p.n, c->dwarm, p.h, c->warm_valid, &c->ctl->mlp_err, s,
                                !c->model_nbr, c->P.mlp_tcgen05 == 1);
        else
            launch_mlp_infer(c->mlp_dev, c->feat, p.n, c->dwarm, p.h, c->warm_valid, s, !c->model_nbr);
        dw = c->dwarm;
    }
    int src = 0, it = 1;
    const float4 *acc = nullptr;
    if (pbf_prepass(c)) {
        enqueue_sort(c, p, c->set[0].pos, s);
        Gather g{};
        g.n4 = dw ? 3 : 2; g.n1 = 2;
        g.src4[0] = c->set[0].pos; g.dst4[0] = c->set[1].pos;
        g.src4[1] = c->set[0].vel; g.dst4[1] = c->set[1].vel;
        g.src4[2] = dw; g.dst4[2] = c->vort; /* vort is rewritten at the end of the step */
        g.src1[0] = c->set[0].id; g.dst1[0] = c->set[1].id;
        g.src1[1] = c->set[0].attr; g.dst1[1] = c->set[1].attr;
        launch_gather(p.n, c->perm, g, nullptr, s);
        launch_pbf_density(p, c->cell_start, c->set[1].pos, c->dens, s);
        launch_pbf_visc(p, c->cell_start, c->set[1].pos, c->set[1].vel, c->dens, c->acc, s);
        acc = c->acc;
        if (dw) dw = c->vort;
        src = 1; it = 0;
    }
    launch_predict_hash(p, c->set[src].pos, c->set[src].vel, acc, c->ppos[1], c->key, c->rank, c->count, dw,
                        ws ? c->tmp4 : nullptr, s);
    launch_scan(c->count, c->cell_start, c->block_sums, c->ncells, s);
    sort_cells(c, p, s);
    Gather g{};
    g.n4 = ws ? 4 : 3; g.n1 = 3;
    g.src4[0] = c->set[src].pos; g.dst4[0] = c->set[it].pos;
    g.src4[1] = c->ppos[1]; g.dst4[1] = c->ppos[0];
    g.src4[2] = c->ppos[1]; g.dst4[2] = c->xb;
    g.src4[3] = c->tmp4; g.dst4[3] = c->xpred;
    g.src1[0] = c->set[src].id; g.dst1[0] = c->set[it].id;
    g.src1[1] = c->set[src].attr; g.dst1[1] = c->set[it].attr;
    g.src1[2] = c->key; g.dst1[2] = c->nl.cellb;
    launch_gather(p.n, c->perm, g, c->ctl, s);
    launch_build_list(p, c->cell_start, c->xb, c->nl, s);
    return it;
}

void enqueue_pbf_post(fsph_ctx *c, const DevParams &p, int it, cudaStream_t s) {
    const bool ws = pbf_warm_active(c);
    const bool ext = pbf_finalize_ext(c), pre = ext && FSPH_POST_PRE;
    launch_finalize(p, c->set[it].pos, c->ppos[0], c->ppos[1], c->ctl, c->set[it].id, c->set[it].attr,
                    c->set[0].pos, c->set[0].vel, c->set[0].id, c->set[0].attr, ws ? c->xpred : nullptr,
                    ws ? c->dstep : nullptr, s, c->dens, pre ? c->mrho : nullptr);
    if (ext) {
        FeatureOut fo;
        if (ws) {
            fo.feat = c->feat;
            fo.nbr = (c->P.collect_features || c->model_nbr) ? 1 : 0;
            fo.dstep = c->dstep;
            fo.ppos0 = c->ppos[0];
            fo.ppos1 = c->ppos[1];
            fo.ctl = c->ctl;
            fo.valid = c->warm_valid;
        }
        launch_xsph_vort(p, c->cell_start, c->set[0].pos, c->set[0].vel, c->dens, c->set[1].vel, c->vort, fo, c->nl,
                         s, pre ? c->mrho : nullptr, pre ? c->wm : nullptr);
        launch_vort_apply(p, c->cell_start, c->set[0].pos, c->vort, c->dens, c->set[1].vel, c->set[0].vel, c->nl, s,
                          pre ? c->wm : nullptr);
    }
}

int pbf_step_eager(fsph_ctx *c, const DevParams &p) {
    cudaStream_t s = c->stream;
    int it;
    {
        NvtxRange r("pbf_predict_and_grid");
        it = enqueue_pbf_pre(c, p, s);
    }
    NvtxRange r("pbf_constraint_loop");
    for (int k = 0;; ++k) {
        launch_lambda(p, c->cell_start, c->ppos[0], c->ppos[1], c->dens, c->ctl, c->epart, 0ull, 0, c->nl, s);
        launch_boundary_lambda(p, c->cell_start, c->ppos[0], c->ppos[1], c->ctl, c->b_stat, c->b_lam, s);
        launch_correction(p, c->cell_start, c->ppos[0], c->ppos[1], c->xb, c->ctl, c->dpart, 0ull, 0ull, 0,
                          nullptr, c->nl, s);
        FSPH_CUDA(c, cudaMemcpyAsync(c->ctl_host, c->ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, s));
        FSPH_CUDA(c, cudaStreamSynchronize(s));
        if (c->ctl_host->done || k > p.max_iter + 1) break;
        if (c->ctl_host->rebuild) enqueue_rebuild(c, p, it, s);
    }
    if (pbf_finalize_ext(c) && c->ctl_host->rebuild) enqueue_rebuild(c, p, it, s);
    enqueue_pbf_post(c, p, it, s);
    return FSPH_OK;
}

int add_conditional(fsph_ctx *c, cudaGraph_t g, const cudaGraphNode_t *deps, size_t ndeps,
                    cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type, cudaGraphNode_t *node,
                    cudaGraph_t *body) {
    /* the params union has no usable default constructor: zero raw storage */
    alignas(cudaGraphNodeParams) unsigned char raw[sizeof(cudaGraphNodeParams)];
    std::memset(raw, 0, sizeof(raw));
    cudaGraphNodeParams *cp = reinterpret_cast<cudaGraphNodeParams *>(raw);
    cp->type = cudaGraphNodeTypeConditional;
    cp->conditional.handle = h;
    cp->conditional.type = type;
    cp->conditional.size = 1;
    FSPH_CUDA(c, cudaGraphAddNode(node, g, deps, nullptr, ndeps, cp));
    *body = cp->conditional.phGraph_out[0];
    return FSPH_OK;
}

/* kernel nodes directly in g (conditional bodies are separate graphs) */
int kernel_nodes(cudaGraph_t g) {
    size_t n = 0;
    if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess) return 0;
    std::vector<cudaGraphNode_t> v(n);
    if (n && cudaGraphGetNodes(g, v.data(), &n) != cudaSuccess) return 0;
    int k = 0;
    for (cudaGraphNode_t nd : v) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
    }
    return k;
}

/* Capture one PBF step into a graph:
 *   pre-pass -> WHILE(h_while){ IF(h_rb){rebuild}; lambda; correction }
 *            -> [IF(h_rb2){rebuild}] -> finalize (+ XSPH / vorticity)      */
int build_pbf_graph(fsph_ctx *c, const DevParams &p) {
    drop_graph(c);
    cudaStream_t s = c->stream;
    cudaGraph_t g;
    FSPH_CUDA(c, cudaGraphCreate(&g, 0));
    c->graph = g;
    FSPH_CUDA(c, cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    int it = enqueue_pbf_pre(c, p, s);

    cudaStreamCaptureStatus st;
    cudaGraph_t capg;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    FSPH_CUDA(c, cudaStreamGetCaptureInfo(s, &st, nullptr, &capg, &deps, nullptr, &ndeps));
    cudaGraphConditionalHandle hw, hrb, hrb2;
    FSPH_CUDA(c, cudaGraphConditionalHandleCreate(&hw, capg, 1, cudaGraphCondAssignDefault));
    cudaGraphNode_t wnode;
    cudaGraph_t wbody;
    std::vector<cudaGraphNode_t> dv(deps, deps + ndeps);
    FSPH_TRY(add_conditional(c, capg, dv.data(), dv.size(), hw, cudaGraphCondTypeWhile, &wnode, &wbody));

    FSPH_CUDA(c, cudaGraphConditionalHandleCreate(&hrb, wbody, 0, cudaGraphCondAssignDefault));
    cudaGraphNode_t inode;
    cudaGraph_t ibody;
    FSPH_TRY(add_conditional(c, wbody, nullptr, 0, hrb, cudaGraphCondTypeIf, &inode, &ibody));
    FSPH_CUDA(c, cudaStreamBeginCaptureToGraph(c->s3, ibody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    enqueue_rebuild(c, p, it, c->s3);
    FSPH_CUDA(c, cudaStreamEndCapture(c->s3, &ibody));

    const bool ext = pbf_finalize_ext(c);
    hrb2 = 0;
    if (ext) FSPH_CUDA(c, cudaGraphConditionalHandleCreate(&hrb2, capg, 0, cudaGraphCondAssignDefault));
    FSPH_CUDA(c, cudaStreamBeginCaptureToGraph(c->s2, wbody, &inode, nullptr, 1, cudaStreamCaptureModeRelaxed));
    launch_lambda(p, c->cell_start, c->ppos[0], c->ppos[1], c->dens, c->ctl, c->epart, hw, 1, c->nl, c->s2);
    launch_boundary_lambda(p, c->cell_start, c->ppos[0], c->ppos[1], c->ctl, c->b_stat, c->b_lam, c->s2);
    launch_correction(p, c->cell_start, c->ppos[0], c->ppos[1], c->xb, c->ctl, c->dpart, hrb, hrb2, ext ? 3 : 1,
                      nullptr, c->nl, c->s2);
    FSPH_CUDA(c, cudaStreamEndCapture(c->s2, &wbody));
    FSPH_CUDA(c, cudaStreamUpdateCaptureDependencies(s, &wnode, nullptr, 1, cudaStreamSetCaptureDependencies));

    if (ext) {
        cudaGraphNode_t pnode;
        cudaGraph_t pbody;
        FSPH_TRY(add_conditional(c, capg, &wnode, 1, hrb2, cudaGraphCondTypeIf, &pnode, &pbody));
        FSPH_CUDA(c, cudaStreamBeginCaptureToGraph(c->s3, pbody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
        enqueue_rebuild(c, p, it, c->s3);
        FSPH_CUDA(c, cudaStreamEndCapture(c->s3, &pbody));
        FSPH_CUDA(c, cudaStreamUpdateCaptureDependencies(s, &pnode, nullptr, 1, cudaStreamSetCaptureDependencies));
    }
    enqueue_pbf_post(c, p, it, s);
    FSPH_CUDA(c, cudaStreamEndCapture(s, &g));
    c->k_top = kernel_nodes(g);
    c->k_iter = kernel_nodes(wbody);
    c->k_rebuild = kernel_nodes(ibody);
    FSPH_CUDA(c, cudaGraphInstantiate(&c->gexec, g, 0));
    c->graph_valid = true;
    c->graph_dt = p.dt;
    c->graph_n = p.n;
    return FSPH_OK;
}

int sph_step(fsph_ctx *c, const DevParams &p) {
    cudaStream_t s = c->stream;
    FSPH_CUDA(c, cudaMemsetAsync(c->ctl, 0, sizeof(DevCtl), s));
    enqueue_sort(c, p, c->set[0].pos, s);
    Gather g{};
    g.n4 = 2; g.n1 = 2;
    g.src4[0] = c->set[0].pos; g.dst4[0] = c->set[1].pos;
    g.src4[1] = c->set[0].vel; g.dst4[1] = c->set[1].vel;
    g.src1[0] = c->set[0].id; g.dst1[0] = c->set[1].id;
    g.src1[1] = c->set[0].attr; g.dst1[1] = c->set[1].attr;
    launch_gather(p.n, c->perm, g, c->ctl, s);
    launch_sph_density(p, c->cell_start, c->set[1].pos, c->set[1].vel, c->dens, c->pres, c->nl, s);
    launch_sph_force(p, c->cell_start, c->set[1].pos, c->set[1].vel, c->acc, c->nl, s);
    launch_sph_integrate(p, c->set[1].pos, c->set[1].vel, c->acc, c->set[1].id, c->set[1].attr, c->set[0].pos,
                         c->set[0].vel, c->set[0].id, c->set[0].attr, s);
    return FSPH_OK;
}

/* Capture one WCSPH step (grid build, density + lists, forces, integration)
 * into a graph: the step is launch-bound at the configured 32k particles. */
int build_sph_graph(fsph_ctx *c, const DevParams &p) {
    drop_graph(c);
    cudaGraph_t g;
    FSPH_CUDA(c, cudaGraphCreate(&g, 0));
    c->graph = g;
    FSPH_CUDA(c, cudaStreamBeginCaptureToGraph(c->stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    sph_step(c, p);
    FSPH_CUDA(c, cudaStreamEndCapture(c->stream, &g));
    c->k_top = kernel_nodes(g);
    c->k_iter = c->k_rebuild = 0;
    FSPH_CUDA(c, cudaGraphInstantiate(&c->gexec, g, 0));
    c->graph_valid = true;
    c->graph_dt = p.dt;
    c->graph_n = p.n;
    return FSPH_OK;
}

int check_launch(fsph_ctx *c) {
    FSPH_CUDA(c, cudaGetLastError());
    return FSPH_OK;
}

void fill_stats(fsph_ctx *c, fsph_step_stats *st) {
    std::memset(st, 0, sizeof(*st));
    const DevCtl &h = *c->ctl_host;
    st->iterations = (int)h.iter;
    st->grid_builds = (int)h.builds;
    st->density_error_one_sided = h.err1;
    st->density_error_two_sided = h.err2;
    st->density_error_max = h.errmax;
    st->density_error = c->P.error_mode ? h.err2 : h.err1;
    st->status = FSPH_OK;
    st->bounds_bits = (int)h.bounds_bits;
    if (c->last_step_graph) /* every grid build after the first is one run of the rebuild body */
        st->kernels = c->k_top + (int)h.iter * c->k_iter + ((int)h.builds - 1) * c->k_rebuild;
    if (c->P.solver == FSPH_SOLVER_PBF) {
        if (h.nan_flag) st->status = FSPH_NAN_DETECTED;
        else if (h.mlp_err) st->status = FSPH_TIMEOUT; /* the tcgen05 inference gave up on an MMA */
        else if (st->density_error > c->P.eta) st->status = FSPH_NOT_CONVERGED;
    }
    if (h.bounds_bits && st->status != FSPH_NAN_DETECTED)
        st->status = FSPH_CUDA_ERROR; /* a debug build's index check failed */
}

/* Load n host/device float4 positions (and optional velocities) in particle order. */
int load_particles(fsph_ctx *c, const float *pos4, const float *vel4, int n, int where) {
    cudaMemcpyKind k = where == FSPH_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    size_t b = (size_t)n * sizeof(float4);
    if (n > 0) {
        FSPH_CUDA(c, cudaMemcpyAsync(c->set[0].pos, pos4, b, k, c->stream));
        if (vel4) FSPH_CUDA(c, cudaMemcpyAsync(c->set[0].vel, vel4, b, k, c->stream));
        else FSPH_CUDA(c, cudaMemsetAsync(c->set[0].vel, 0, b, c->stream));
        FSPH_CUDA(c, cudaMemsetAsync(c->set[0].attr, 0, (size_t)n * 4, c->stream));
        launch_iota(n, c->set[0].id, c->stream);
        c->home_identity = true;
        c->res_in_res_id = false;
        /* a new state has no step history for the warm start */
        FSPH_CUDA(c, cudaMemsetAsync(c->dstep, 0, b, c->stream));
    }
    FSPH_CUDA(c, cudaMemsetAsync(c->warm_valid, 0, sizeof(unsigned int), c->stream));
    if (n != c->n_active) c->graph_valid = false;
    c->n = n;
    c->n_active = n;
    return check_launch(c);
}

/* Bring the home set to particle order (slot d = particle d), as the
 * setters need it; the last step's results keep its slot order in res_id. */
int home_to_particle_order(fsph_ctx *c) {
    if (c->home_identity) return FSPH_OK;
    cudaStream_t s = c->stream;
    const int n = c->n;
    launch_unsort4(n, c->set[0].id, c->set[0].pos, c->set[1].pos, 0, s);
    launch_unsort4(n, c->set[0].id, c->set[0].vel, c->set[1].vel, 0, s);
    launch_unsort1(n, c->set[0].id, c->set[0].attr, c->set[1].attr, s);
    FSPH_CUDA(c, cudaMemcpyAsync(c->set[0].pos, c->set[1].pos, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));
    FSPH_CUDA(c, cudaMemcpyAsync(c->set[0].vel, c->set[1].vel, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));
    FSPH_CUDA(c, cudaMemcpyAsync(c->set[0].attr, c->set[1].attr, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
    /* the warm-start history (step corrections, features) follows the particles */
    launch_unsort4(n, c->set[0].id, c->dstep, c->tmp4, 0, s);
    FSPH_CUDA(c, cudaMemcpyAsync(c->dstep, c->tmp4, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));
    if (!c->res_in_res_id) {
        /* the last step's other results (density, lambda, forces, ...) stay
         * in its slot order, which res_id keeps for the getters */
        FSPH_CUDA(c, cudaMemcpyAsync(c->res_id, c->set[0].id, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
        c->res_in_res_id = true;
    }
    {
        float4 *tf = reinterpret_cast<float4 *>(c->nl.list); /* lists are rebuilt by every step */
        launch_unsort_rows(n, c->set[0].id, reinterpret_cast<const float4 *>(c->feat), tf, kFeatures / 4, s);
        FSPH_CUDA(c, cudaMemcpyAsync(c->feat, tf, (size_t)n * kFeatures * 4, cudaMemcpyDeviceToDevice, s));
    }
    launch_iota(n, c->set[0].id, s);
    c->home_identity = true;
    return check_launch(c);
}

/* Stable partition of the home set: particles with attribute != -1 first
 * (they take part in the steps), deleted ones after; n_active follows.
 * Synchronises. */
int repartition(fsph_ctx *c) {
    NvtxRange range("fsph_repartition");
    const int n = c->n;
    cudaStream_t s = c->stream;
    if (n > 0) {
        if (!c->res_in_res_id) {
            FSPH_CUDA(c, cudaMemcpyAsync(c->res_id, c->set[0].id, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
            c->res_in_res_id = true;
        }
        launch_mark_active(n, c->set[0].attr, c->key, s);
        launch_scan(c->key, c->part_scan, c->part_bsum, (unsigned int)n, s);
        launch_partition_perm(n, c->part_scan, c->perm, s);
        Gather g{};
        g.n4 = 3; g.n1 = 2;
        g.src4[0] = c->set[0].pos; g.dst4[0] = c->set[1].pos;
        g.src4[1] = c->set[0].vel; g.dst4[1] = c->set[1].vel;
        g.src4[2] = c->dstep; g.dst4[2] = c->tmp4;
        g.src1[0] = c->set[0].id; g.dst1[0] = c->set[1].id;
        g.src1[1] = c->set[0].attr; g.dst1[1] = c->set[1].attr;
        launch_gather(n, c->perm, g, nullptr, s);
        float4 *tf = reinterpret_cast<float4 *>(c->nl.list);
        launch_gather_rows(n, c->perm, reinterpret_cast<const float4 *>(c->feat), tf, kFeatures / 4, s);
        FSPH_CUDA(c, cudaMemcpyAsync(c->set[0].pos, c->set[1].pos, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));
        FSPH_CUDA(c, cudaMemcpyAsync(c->set[0].vel, c->set[1].vel, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));
        FSPH_CUDA(c, cudaMemcpyAsync(c->dstep, c->tmp4, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));
        FSPH_CUDA(c, cudaMemcpyAsync(c->set[0].id, c->set[1].id, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
        FSPH_CUDA(c, cudaMemcpyAsync(c->set[0].attr, c->set[1].attr, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
        FSPH_CUDA(c, cudaMemcpyAsync(c->feat, tf, (size_t)n * kFeatures * 4, cudaMemcpyDeviceToDevice, s));
        unsigned int na = 0;
        FSPH_CUDA(c, cudaMemcpyAsync(&na, c->part_scan + n, 4, cudaMemcpyDeviceToHost, s));
        FSPH_CUDA(c, cudaStreamSynchronize(s));
        FSPH_TRY(check_launch(c));
        if ((int)na != c->n_active) c->graph_valid = false;
        c->n_active = (int)na;
        c->home_identity = false;
    } else {
        c->n_active = 0;
    }
    return FSPH_OK;
}

/* Build the grid on device positions x (length n, current slot order) and
 * gather x (and w) into set[1].pos / ppos[0] / xb, ids into set[1].id. */
int build_on(fsph_ctx *c, const DevParams &p, const float4 *x) {
    cudaStream_t s = c->stream;
    enqueue_sort(c, p, x, s);
    Gather g{};
    g.n4 = 3; g.n1 = 3;
    g.src4[0] = x; g.dst4[0] = c->set[1].pos;
    g.src4[1] = x; g.dst4[1] = c->ppos[0];
    g.src4[2] = x; g.dst4[2] = c->xb;
    g.src1[0] = c->set[0].id; g.dst1[0] = c->set[1].id;
    g.src1[1] = c->set[0].attr; g.dst1[1] = c->set[1].attr;
    g.src1[2] = c->key; g.dst1[2] = c->nl.cellb;
    launch_gather(p.n, c->perm, g, nullptr, s);
    launch_build_list(p, c->cell_start, c->xb, c->nl, s);
    return check_launch(c);
}

int copy_out_scalar(fsph_ctx *c, const float *dev_sorted_src, const unsigned int *id, float *host_dst, int n) {
    float *tmp = reinterpret_cast<float *>(c->key);  /* key is free after a build */
    launch_unsort1(n, id, reinterpret_cast<const unsigned int *>(dev_sorted_src), reinterpret_cast<unsigned int *>(tmp),
                   c->stream);
    FSPH_CUDA(c, cudaMemcpyAsync(host_dst, tmp, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
    return FSPH_OK;
}

}  // namespace

/* ======================================================================== */
/* C ABI                                                                    */
/* ======================================================================== */
extern "C" {

int fsph_abi_version(void) { return FSPH_ABI_VERSION; }

const char *fsph_status_string(int status) {
    switch (status) {
    case FSPH_OK: return "FSPH_OK";
    case FSPH_INVALID_ARG: return "FSPH_INVALID_ARG";
    case FSPH_OOM: return "FSPH_OOM";
    case FSPH_CUDA_ERROR: return "FSPH_CUDA_ERROR";
    case FSPH_NAN_DETECTED: return "FSPH_NAN_DETECTED";
    case FSPH_TIMEOUT: return "FSPH_TIMEOUT";
    case FSPH_NOT_CONVERGED: return "FSPH_NOT_CONVERGED";
    case FSPH_NOT_INITIALIZED: return "FSPH_NOT_INITIALIZED";
    case FSPH_UNSUPPORTED: return "FSPH_UNSUPPORTED";
    case FSPH_NO_DEVICE: return "FSPH_NO_DEVICE";
    }
    return "FSPH_UNKNOWN";
}

const char *fsph_last_error(const fsph_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void fsph_params_default(fsph_params *o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->solver = FSPH_SOLVER_PBF;
    o->max_particles = 0;
    o->h = 0.0457f;
    o->mass = 0.02f;
    o->rest_dens = 998.29f;
    o->particle_radius = 0.01f;
    for (int a = 0; a < 3; ++a) { o->box_min[a] = -0.5; o->box_max[a] = 0.5; }
    o->gravity[1] = -9.82f; /* rxParticleSystemBase constructor, rx_ps.h:165 */
    o->viscosity = 0.0f;
    o->gas_k = 3.0f;
    o->epsilon = 0.001f;  /* rxSPHEnviroment defaults, rx_sph.h:152-160 */
    o->eta = 0.05f;
    o->min_iter = 2;
    o->max_iter = 10;
    o->error_mode = FSPH_ERR_ONE_SIDED;
    o->use_ap = 1;
    o->ap_k = 0.1f;
    o->ap_n = 4.0f;
    o->ap_q = 0.2f;
    o->cell_skin = 0.05f;
    o->use_graph = 1;
    o->mlp_tcgen05 = 1; /* warm-start inference on tcgen05 (same step time as mma.sync, measured) */
}

int fsph_params_from_env(const fsph_env *e, fsph_params *o) {
    if (!e || !o) return FSPH_INVALID_ARG;
    if (!(e->dens > 0) || !(e->mass > 0) || !(e->kernel_particles > 0) || e->max_particles <= 0) return FSPH_INVALID_ARG;
    fsph_params_default(o);
    o->solver = e->solver;
    o->max_particles = e->max_particles;
    /* h = (3 kp m / (4 pi rho))^(1/3), r = (pi / (6 kp))^(1/3) h
     * (rx_sph_pbd.cpp:110-115, rx_sph_cpu.cpp:100-104), in RXREAL storage */
    float volume = (float)e->max_particles * e->mass / e->dens;
    float h = (float)std::pow((3.0 * e->kernel_particles * volume) / (4.0 * e->max_particles * kPi), 1.0 / 3.0);
    float r = (float)(std::pow(kPi / (6.0 * e->kernel_particles), 1.0 / 3.0) * h);
    o->h = h;
    o->particle_radius = r;
    o->mass = e->mass;
    /* rho0 := calRestDensity(h): poly6 sum over a lattice of spacing 2r
     * (rx_sph_pbd.cpp:1035-1049), float accumulation */
    float l = 2.0f * r;
    int nn = (int)std::ceil(h / l) + 1;
    double aw = poly6_coef((double)h);
    float r0 = 0.0f;
    for (int x = -nn; x <= nn; ++x)
        for (int y = -nn; y <= nn; ++y)
            for (int z = -nn; z <= nn; ++z) {
                double dx = (double)(x * l), dy = (double)(y * l), dz = (double)(z * l);
                double rr = std::sqrt(dx * dx + dy * dy + dz * dz);
                double w = (rr <= (double)h) ? aw * std::pow((double)h * h - rr * rr, 3.0) : 0.0;
                r0 = (float)((double)r0 + (double)e->mass * w);
            }
    o->rest_dens = r0;
    for (int a = 0; a < 3; ++a) {
        o->box_min[a] = e->boundary_cen[a] - e->boundary_ext[a];
        o->box_max[a] = e->boundary_cen[a] + e->boundary_ext[a];
    }
    o->gravity[0] = 0.0f; o->gravity[1] = e->gravity_y; o->gravity[2] = 0.0f;
    o->viscosity = e->viscosity;
    o->gas_k = e->gas_k;
    o->epsilon = e->epsilon;
    o->eta = e->eta;
    o->min_iter = e->min_iter;
    o->max_iter = e->max_iter;
    o->error_mode = FSPH_ERR_TWO_SIDED; /* the CPU path's error (rx_sph_pbd.cpp:450) */
    o->use_ap = e->use_ap;
    o->ap_k = e->ap_k; o->ap_n = e->ap_n; o->ap_q = e->ap_q;
    return FSPH_OK;
}

int fsph_create(const fsph_params *params, fsph_ctx **out) {
    if (!params || !out) return FSPH_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return FSPH_NO_DEVICE;
    }
    std::string why;
    int st = validate(*params, why);
    if (st != FSPH_OK) return st;
    fsph_ctx *c = new (std::nothrow) fsph_ctx();
    if (!c) return FSPH_OOM;
    c->P = *params;
    cudaGetDevice(&c->device);
    auto bail = [&](int s) { fsph_destroy(c); return s; };
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(FSPH_CUDA_ERROR);
    if (cudaStreamCreateWithFlags(&c->s2, cudaStreamNonBlocking) != cudaSuccess) return bail(FSPH_CUDA_ERROR);
    if (cudaStreamCreateWithFlags(&c->s3, cudaStreamNonBlocking) != cudaSuccess) return bail(FSPH_CUDA_ERROR);
    if (cudaMalloc((void **)&c->ctl, sizeof(DevCtl)) != cudaSuccess) return bail(FSPH_OOM);
    if (cudaMallocHost((void **)&c->ctl_host, sizeof(DevCtl)) != cudaSuccess) return bail(FSPH_OOM);
    std::memset(c->ctl_host, 0, sizeof(DevCtl));
    if (cudaMalloc((void **)&c->flag, sizeof(unsigned int)) != cudaSuccess) return bail(FSPH_OOM);
    if (cudaMallocHost((void **)&c->flag_host, sizeof(unsigned int)) != cudaSuccess) return bail(FSPH_OOM);
    if (cudaMalloc((void **)&c->warm_valid, sizeof(unsigned int)) != cudaSuccess) return bail(FSPH_OOM);
    if (cudaMalloc((void **)&c->mlp_dev, sizeof(MlpDev)) != cudaSuccess) return bail(FSPH_OOM);
    cudaMemsetAsync(c->warm_valid, 0, sizeof(unsigned int), c->stream);
    cudaMemsetAsync(c->ctl, 0, sizeof(DevCtl), c->stream);
    if ((st = alloc_particles(c, params->max_particles)) != FSPH_OK) return bail(st);
    if ((st = alloc_grid(c)) != FSPH_OK) return bail(st);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return bail(FSPH_CUDA_ERROR);
    *out = c;
    return FSPH_OK;
}

int fsph_destroy(fsph_ctx *c) {
    if (!c) return FSPH_INVALID_ARG;
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->log) std::fclose(c->log);
    drop_graph(c);
    free_particles(c);
    free_grid(c);
    free_boundary(c);
    cudaFree(c->ctl);
    if (c->ctl_host) cudaFreeHost(c->ctl_host);
    cudaFree(c->flag);
    if (c->flag_host) cudaFreeHost(c->flag_host);
    cudaFree(c->warm_valid);
    cudaFree(c->mlp_dev);
    cudaFree(c->obs_dev);
    cudaFree(c->del_dev);
    free_polygons(c);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->s2) cudaStreamDestroy(c->s2);
    if (c->s3) cudaStreamDestroy(c->s3);
    delete c;
    return FSPH_OK;
}

int fsph_set_params(fsph_ctx *c, const fsph_params *p) {
    if (!c || !p) return FSPH_INVALID_ARG;
    std::string why;
    int st = validate(*p, why);
    if (st != FSPH_OK) return fail(c, st, why);
    FSPH_CUDA(c, cudaStreamSynchronize(c->stream));
    const bool rebuild = c->broken; /* a failed reallocation lost the particles */
    if (rebuild) c->n = c->n_active = 0;
    if (!rebuild && p->max_particles != c->P.max_particles && c->n > p->max_particles)
        return fail(c, FSPH_INVALID_ARG, "max_particles below the current particle count");
    const int old_cap = c->P.max_particles;
    const fsph_params old = c->P;
    bool same_box = old.h == p->h;
    for (int a = 0; a < 3; ++a) same_box = same_box && old.box_min[a] == p->box_min[a] && old.box_max[a] == p->box_max[a];
    /* what the boundary's cell table and volumes, and the triangles' table, depend on */
    const bool same_grid = same_box && old.cell_skin == p->cell_skin;
    const bool same_boundary = same_grid && old.mass == p->mass && old.rest_dens == p->rest_dens;
    c->P = *p;
    drop_graph(c);
    if (rebuild || p->max_particles != old_cap) {
        /* keep the particles across the reallocation */
        std::vector<float4> hp((size_t)c->n), hv((size_t)c->n);
        std::vector<int> ha((size_t)c->n);
        if (c->n) {
            FSPH_TRY(fsph_get_array(c, FSPH_POSITION, hp.data(), FSPH_HOST, nullptr));
            FSPH_TRY(fsph_get_array(c, FSPH_VELOCITY, hv.data(), FSPH_HOST, nullptr));
            FSPH_TRY(fsph_get_array(c, FSPH_ATTRIBUTE, ha.data(), FSPH_HOST, nullptr));
        }
        int n = c->n;
        c->broken = true; /* until every buffer is in place again */
        FSPH_TRY(alloc_particles(c, p->max_particles));
        c->n = 0;
        FSPH_TRY(load_particles(c, (const float *)hp.data(), (const float *)hv.data(), n, FSPH_HOST));
        if (n) {
            FSPH_CUDA(c, cudaMemcpyAsync(c->set[0].attr, ha.data(), (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
            FSPH_TRY(repartition(c));
        }
    }
    c->broken = true;
    FSPH_TRY(alloc_grid(c));
    /* the boundary's cell table and volumes follow the grid and the kernel; the
     * triangles' table the reference grid (box and h).  A call that changes
     * neither (gravity, iterations, flags) leaves them */
    if (rebuild || !same_boundary) FSPH_TRY(boundary_build(c));
    if (!c->poly_t.empty() && (rebuild || !same_box)) FSPH_TRY(polygons_upload(c));
    FSPH_CUDA(c, cudaStreamSynchronize(c->stream));
    c->broken = false;
    return FSPH_OK;
}

int fsph_get_params(const fsph_ctx *c, fsph_params *o) {
    if (!c || !o) return FSPH_INVALID_ARG;
    *o = c->P;
    return FSPH_OK;
}

int fsph_num_particles(const fsph_ctx *c) { return c ? c->n : -1; }

int fsph_set_particles(fsph_ctx *c, const float *pos4, const float *vel4, int n, int where) {
    if (!c) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    if (n < 0 || n > c->cap) return fail(c, FSPH_INVALID_ARG, "particle count outside [0, max_particles]");
    if (n > 0 && !pos4) return fail(c, FSPH_INVALID_ARG, "null positions");
    if (where != FSPH_HOST && where != FSPH_DEVICE) return fail(c, FSPH_INVALID_ARG, "where");
    FSPH_TRY(load_particles(c, pos4, vel4, n, where));
    /* finiteness is checked on the device, where the data now is */
    FSPH_CUDA(c, cudaMemsetAsync(c->flag, 0, sizeof(unsigned int), c->stream));
    if (n > 0) launch_check_finite(n, c->set[0].pos, c->set[0].vel, c->flag, c->stream);
    FSPH_CUDA(c, cudaMemcpyAsync(c->flag_host, c->flag, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream));
    FSPH_CUDA(c, cudaStreamSynchronize(c->stream));
    FSPH_TRY(check_launch(c));
    if (*c->flag_host) {
        c->n = 0;
        return fail(c, FSPH_NAN_DETECTED, "non-finite input position or velocity");
    }
    return FSPH_OK;
}

/* dst[slot] = src[p - start] for the slots whose particle p = id[slot] lies
 * in [start, start + count): a range given in particle order lands in the
 * slots of the last step's order, and no other array moves */
__global__ void k_scatter_range4(int n, const unsigned int *__restrict__ id, int start, int count,
                                 const float4 *__restrict__ src, float4 *__restrict__ dst) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    const unsigned int q = id[d] - (unsigned int)start;
    if (q < (unsigned int)count) dst[d] = src[q];
}

int fsph_set_array(fsph_ctx *c, int type, const void *data, int start, int count, int where) {
    if (!c || !data) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    if (start < 0 || count < 0 || count > c->n - start) return fail(c, FSPH_INVALID_ARG, "range outside [0, n)");
    if (type != FSPH_POSITION && type != FSPH_VELOCITY && type != FSPH_ATTRIBUTE)
        return fail(c, FSPH_INVALID_ARG, "settable arrays: POSITION, VELOCITY, ATTRIBUTE");
    if (count == 0) return FSPH_OK; /* nothing to overwrite (and no kernel for an empty range) */
    cudaStream_t s = c->stream;
    int n = c->n;
    /* attributes: bring the home arrays to particle order (once after a
     * step), then overwrite the range; positions and velocities are
     * scattered to their particles' slots without moving anything else */
    if (type == FSPH_ATTRIBUTE) FSPH_TRY(home_to_particle_order(c));
    cudaMemcpyKind k = where == FSPH_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (type == FSPH_POSITION || type == FSPH_VELOCITY) {
        /* staged and checked before it replaces anything: a range with a
         * non-finite value is rejected and the state stays as it was (the
         * same rule as fsph_set_particles) */
        FSPH_CUDA(c, cudaMemcpyAsync(c->tmp4, data, (size_t)count * 16, k, s));
        FSPH_CUDA(c, cudaMemsetAsync(c->flag, 0, sizeof(unsigned int), s));
        launch_check_finite(count, c->tmp4, nullptr, c->flag, s);
        FSPH_CUDA(c, cudaMemcpyAsync(c->flag_host, c->flag, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
        FSPH_TRY(check_launch(c));
        FSPH_CUDA(c, cudaStreamSynchronize(s));
        if (*c->flag_host) return fail(c, FSPH_NAN_DETECTED, "non-finite position or velocity");
        float4 *dst = type == FSPH_POSITION ? c->set[0].pos : c->set[0].vel;
        if (c->home_identity)
            FSPH_CUDA(c, cudaMemcpyAsync(dst + start, c->tmp4, (size_t)count * 16, cudaMemcpyDeviceToDevice, s));
        else
            k_scatter_range4<<<(n + 255) / 256, 256, 0, s>>>(n, c->set[0].id, start, count, c->tmp4, dst);
        /* the caller's buffer was read before the check above returned; the
         * rest is ordered on the context's stream */
        return check_launch(c);
    }
    FSPH_CUDA(c, cudaMemcpyAsync(c->set[0].attr + start, data, (size_t)count * 4, k, s));
    FSPH_TRY(check_launch(c));
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    /* an attribute of -1 deletes a particle, another value revives one */
    if (type == FSPH_ATTRIBUTE) FSPH_TRY(repartition(c));
    return FSPH_OK;
}

int fsph_step(fsph_ctx *c, float dt, void *stream, fsph_step_stats *stats) {
    if (!c) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    NvtxRange range("fsph_step");
    if (c->log && !stats) { /* the record needs the stats of every step */
        fsph_step_stats own;
        return fsph_step(c, dt, stream, &own);
    }
    const auto t_start = std::chrono::steady_clock::now();
    if (c->n <= 0) return fail(c, FSPH_INVALID_ARG, "no particles");
    if (!(dt > 0.0f) || !std::isfinite(dt)) return fail(c, FSPH_INVALID_ARG, "dt must be positive and finite");
    if (c->n_active <= 0) { /* every particle deleted: nothing moves */
        if (stats) std::memset(stats, 0, sizeof(*stats));
        return FSPH_OK;
    }
    cudaStream_t user = (cudaStream_t)stream;
    cudaEvent_t ev = nullptr;
    if (user && user != c->stream) {
        /* order the step after the caller's work on its stream */
        FSPH_CUDA(c, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        FSPH_CUDA(c, cudaEventRecord(ev, user));
        FSPH_CUDA(c, cudaStreamWaitEvent(c->stream, ev, 0));
    }
    if (c->P.solver == FSPH_SOLVER_PBF && c->P.warm_start == 1 && !c->model_loaded)
        return fail(c, FSPH_UNSUPPORTED, "warm_start = 1 needs a network (fsph_set_warm_start_model)");
    DevParams p = dev_for(c, c->n_active, dt);
    c->dp = p;
    c->home_identity = false; /* the step leaves the home set in cell order */
    c->res_in_res_id = false;
    c->last_step_graph = c->P.use_graph != 0;
    if (c->P.solver == FSPH_SOLVER_WCSPH) {
        if (c->P.use_graph) {
            if (!c->graph_valid || c->graph_dt != dt || c->graph_n != c->n_active) FSPH_TRY(build_sph_graph(c, p));
            FSPH_CUDA(c, cudaGraphLaunch(c->gexec, c->stream));
        } else {
            FSPH_TRY(sph_step(c, p));
        }
    } else if (c->P.use_graph) {
        if (!c->graph_valid || c->graph_dt != dt || c->graph_n != c->n_active) FSPH_TRY(build_pbf_graph(c, p));
        FSPH_CUDA(c, cudaGraphLaunch(c->gexec, c->stream));
    } else {
        FSPH_TRY(pbf_step_eager(c, p));
    }
    FSPH_TRY(check_launch(c));
    FSPH_CUDA(c, cudaMemcpyAsync(c->ctl_host, c->ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, c->stream));
    if (!c->del_regions.empty()) {
        /* deletion regions (checkDeletePB after the position update,
         * rx_sph_gpu.cpp:875-890): the deleted particles leave the active part */
        launch_delete_regions(c->n_active, c->set[0].pos, c->set[0].vel, c->set[0].attr, c->del_dev,
                              (int)(c->del_regions.size() / 2), c->stream);
        FSPH_TRY(repartition(c));
    }
    if (ev) {
        FSPH_CUDA(c, cudaEventRecord(ev, c->stream));
        FSPH_CUDA(c, cudaStreamWaitEvent(user, ev, 0));
        cudaEventDestroy(ev);
    }
    ++c->steps_done;
    if (stats) {
        FSPH_CUDA(c, cudaStreamSynchronize(c->stream));
        fill_stats(c, stats);
        if (c->log) {
            const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
            std::fprintf(c->log,
                         "{\"step\": %lld, \"solver\": \"%s\", \"dt\": %.9g, \"n\": %d, \"n_active\": %d, "
                         "\"iterations\": %d, \"grid_builds\": %d, \"density_error\": %.9g, "
                         "\"density_error_one_sided\": %.9g, \"density_error_two_sided\": %.9g, "
                         "\"density_error_max\": %.9g, \"status\": \"%s\", \"host_ms\": %.4f}\n",
                         c->steps_done - 1, c->P.solver == FSPH_SOLVER_PBF ? "pbf" : "wcsph", (double)dt, c->n,
                         c->n_active, stats->iterations, stats->grid_builds, (double)stats->density_error,
                         (double)stats->density_error_one_sided, (double)stats->density_error_two_sided,
                         (double)stats->density_error_max, fsph_status_string(stats->status), ms);
            std::fflush(c->log);
        }
        if (stats->status == FSPH_NAN_DETECTED) return fail(c, FSPH_NAN_DETECTED, "NaN in density or position");
        if (stats->status == FSPH_TIMEOUT) return fail(c, FSPH_TIMEOUT, "warm-start inference: an MMA wait ran out");
        if (stats->bounds_bits)
            return fail(c, FSPH_CUDA_ERROR, "debug bounds check: an index out of range (bits " +
                                                std::to_string(stats->bounds_bits) + ")");
    }
    return FSPH_OK;
}

int fsph_set_step_log(fsph_ctx *c, const char *path) {
    if (!c) return FSPH_INVALID_ARG;
    if (c->log) { std::fclose(c->log); c->log = nullptr; }
    if (!path || !*path) return FSPH_OK;
    c->log = std::fopen(path, "a");
    if (!c->log) return fail(c, FSPH_INVALID_ARG, std::string("cannot open ") + path);
    return FSPH_OK;
}

int fsph_set_alloc_fault(long long max_bytes, long long fail_at) {
    g_alloc_max_bytes = max_bytes;
    g_alloc_fail_at = fail_at;
    g_alloc_count = 0;
    return FSPH_OK;
}

int fsph_last_stats(fsph_ctx *c, fsph_step_stats *stats) {
    if (!c || !stats) return FSPH_INVALID_ARG;
    FSPH_CUDA(c, cudaStreamSynchronize(c->stream));
    fill_stats(c, stats);
    return FSPH_OK;
}

int fsph_sync(fsph_ctx *c) {
    if (!c) return FSPH_INVALID_ARG;
    FSPH_CUDA(c, cudaStreamSynchronize(c->stream));
    return FSPH_OK;
}

int fsph_get_array(fsph_ctx *c, int type, void *dst, int where, void *stream) {
    if (!c || !dst) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    if (where != FSPH_HOST && where != FSPH_DEVICE) return fail(c, FSPH_INVALID_ARG, "where");
    int n = c->n;
    if (n == 0) return FSPH_OK;
    cudaStream_t s = c->stream;
    (void)stream;
    /* the copies below are ordered after the last step on the context's
     * stream; only the types that read the host copy of the control block
     * (which ping-pong buffer holds x*) wait for it first */
    if (type == FSPH_PREDICT_POS || type == FSPH_CORRECTION || type == FSPH_SCALING_FACTOR)
        FSPH_CUDA(c, cudaStreamSynchronize(s));
    const unsigned int *id = c->set[0].id;
    /* the last step's results after a SetArrayVBO keep that step's order */
    const bool result = type == FSPH_FORCE || type == FSPH_VORTICITY || type == FSPH_PREDICT_POS ||
                        type == FSPH_CORRECTION || type == FSPH_DENSITY || type == FSPH_PRESSURE ||
                        type == FSPH_SCALING_FACTOR;
    if (result && c->res_in_res_id) id = c->res_id;
    /* staging in device memory: the rank / key arrays are free between steps */
    float4 *t4 = c->set[1].pos;
    bool vec = true;
    switch (type) {
    case FSPH_POSITION: launch_unsort4(n, id, c->set[0].pos, t4, 1, s); break;
    case FSPH_VELOCITY: launch_unsort4(n, id, c->set[0].vel, t4, 1, s); break;
    case FSPH_FORCE: launch_unsort4(n, id, c->acc, t4, 1, s); break;
    case FSPH_VORTICITY: launch_unsort4(n, id, c->vort, t4, 1, s); break;
    case FSPH_STEP_CORRECTION: launch_unsort4(n, id, c->dstep, t4, 1, s); break;
    case FSPH_FEATURES: {
        /* kFeatures floats per particle, staged in the (free) list storage */
        float4 *tf = reinterpret_cast<float4 *>(c->nl.list);
        launch_unsort_rows(n, id, reinterpret_cast<const float4 *>(c->feat), tf, kFeatures / 4, s);
        FSPH_TRY(check_launch(c));
        FSPH_CUDA(c, cudaMemcpyAsync(dst, tf, (size_t)n * kFeatures * 4,
                                     where == FSPH_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
        FSPH_CUDA(c, cudaStreamSynchronize(s));
        return FSPH_OK;
    }
    case FSPH_PREDICT_POS: launch_unsort4(n, id, c->ppos[c->ctl_host->parity & 1], t4, 1, s); break;
    case FSPH_CORRECTION: {
        /* position change of the last iteration (after wall projection) */
        unsigned int par = c->ctl_host->parity & 1;
        launch_unsort4(n, id, c->ppos[par], t4, 1, s);
        launch_unsort4(n, id, c->ppos[1 - par], c->set[1].vel, 1, s);
        std::vector<float4> a((size_t)n), b((size_t)n);
        FSPH_CUDA(c, cudaMemcpyAsync(a.data(), t4, (size_t)n * 16, cudaMemcpyDeviceToHost, s));
        FSPH_CUDA(c, cudaMemcpyAsync(b.data(), c->set[1].vel, (size_t)n * 16, cudaMemcpyDeviceToHost, s));
        FSPH_CUDA(c, cudaStreamSynchronize(s));
        for (int i = 0; i < n; ++i) { a[i].x -= b[i].x; a[i].y -= b[i].y; a[i].z -= b[i].z; a[i].w = 0.0f; }
        if (where == FSPH_HOST) std::memcpy(dst, a.data(), (size_t)n * 16);
        else FSPH_CUDA(c, cudaMemcpy(dst, a.data(), (size_t)n * 16, cudaMemcpyHostToDevice));
        return FSPH_OK;
    }
    case FSPH_DENSITY:
    case FSPH_PRESSURE:
    case FSPH_ATTRIBUTE: {
        vec = false;
        const unsigned int *src = type == FSPH_DENSITY ? reinterpret_cast<const unsigned int *>(c->dens)
                                  : type == FSPH_PRESSURE ? reinterpret_cast<const unsigned int *>(c->pres)
                                                          : c->set[0].attr;
        launch_unsort1(n, id, src, c->set[1].id, s); /* id = set[0].id for the attribute */
        break;
    }
    case FSPH_SCALING_FACTOR:
        vec = false;
        launch_unsort_w(n, id, c->ppos[1 - (c->ctl_host->parity & 1)], reinterpret_cast<float *>(c->set[1].id), s);
        break;
    case FSPH_SORTED_ID:
        vec = false;
        FSPH_CUDA(c, cudaMemcpyAsync(c->set[1].id, id, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
        break;
    default:
        return fail(c, FSPH_INVALID_ARG, "unknown array type");
    }
    FSPH_TRY(check_launch(c));
    const void *src = vec ? (const void *)t4 : (const void *)c->set[1].id;
    size_t bytes = (size_t)n * (vec ? 16 : 4);
    FSPH_CUDA(c, cudaMemcpyAsync(dst, src, bytes, where == FSPH_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    return FSPH_OK;
}

const void *fsph_device_ptr(fsph_ctx *c, int type) {
    if (!c) return nullptr;
    /* work the context queued without a caller stream (fsph_set_array's
     * scatter) is complete before the caller reads through the pointer */
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
        c->err = "stream synchronisation failed";
        return nullptr;
    }
    switch (type) {
    case FSPH_POSITION: return c->set[0].pos;
    case FSPH_VELOCITY: return c->set[0].vel;
    case FSPH_FORCE: return c->acc;
    case FSPH_DENSITY: return c->dens;
    case FSPH_PRESSURE: return c->pres;
    case FSPH_ATTRIBUTE: return c->set[0].attr;
    case FSPH_VORTICITY: return c->vort;
    case FSPH_SORTED_ID: return c->set[0].id;
    }
    c->err = "no device pointer for this array type";
    return nullptr;
}

int fsph_neighbors_ex(fsph_ctx *c, const float *pos4, int n, float radius, int where, int *offsets, int *indices,
                      float *dist2, long long cap, long long *total) {
    if (!c || !offsets || !total) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    *total = 0;
    if (where != FSPH_HOST && where != FSPH_DEVICE) return fail(c, FSPH_INVALID_ARG, "where");
    const bool given = pos4 != nullptr;
    if (!given) n = c->n;
    if (n < 0 || n > c->cap) return fail(c, FSPH_INVALID_ARG, "n outside [0, max_particles]");
    if (n == 0) { offsets[0] = 0; return FSPH_OK; }
    double cw, org[3];
    int g3[3];
    grid_geometry(c->P, cw, org, g3);
    const float h = radius > 0.0f ? radius : c->P.h;
    if (!std::isfinite(h) || (double)h > cw)
        return fail(c, FSPH_UNSUPPORTED, "radius beyond the grid's cell width h (1 + cell_skin)");
    DevParams p = dev_for(c, n, 1.0f);
    p.h = h;
    p.h2 = h * h;
    cudaStream_t s = c->stream;
    const float4 *x = c->set[0].pos;
    const unsigned int *ids = c->set[0].id;
    if (given) {
        /* the given positions stand in for the particles: scratch copy, ids 0..n-1 */
        FSPH_CUDA(c, cudaMemcpyAsync(c->tmp4, pos4, (size_t)n * 16,
                                     where == FSPH_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
        FSPH_CUDA(c, cudaMemsetAsync(c->flag, 0, sizeof(unsigned int), s));
        launch_check_finite(n, c->tmp4, nullptr, c->flag, s);
        FSPH_CUDA(c, cudaMemcpyAsync(c->flag_host, c->flag, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
        FSPH_CUDA(c, cudaStreamSynchronize(s));
        if (*c->flag_host) return fail(c, FSPH_NAN_DETECTED, "non-finite position");
        launch_iota(n, c->set[1].attr, s);
        x = c->tmp4;
        ids = c->set[1].attr;
    }
    enqueue_sort(c, p, x, s);
    Gather g{};
    g.n4 = 1; g.n1 = 1;
    g.src4[0] = x; g.dst4[0] = c->set[1].pos;
    g.src1[0] = ids; g.dst1[0] = c->set[1].id;
    launch_gather(n, c->perm, g, nullptr, s);
    unsigned int *cnt = c->rank; /* free once the scatter has run */
    launch_nb_count(p, c->cell_start, c->set[1].pos, cnt, s);
    std::vector<unsigned int> hc((size_t)n), ho((size_t)n + 1);
    FSPH_CUDA(c, cudaMemcpyAsync(hc.data(), cnt, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    FSPH_TRY(check_launch(c));
    unsigned long long t = 0;
    for (int i = 0; i < n; ++i) { ho[i] = (unsigned int)t; t += hc[i]; }
    if (t > 0xffffffffull) return fail(c, FSPH_INVALID_ARG, "more than 2^32 neighbour entries");
    ho[n] = (unsigned int)t;
    /* rows in the caller's order, ascending indices within a row */
    std::vector<int> hid((size_t)n);
    FSPH_CUDA(c, cudaMemcpyAsync(hid.data(), c->set[1].id, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    std::vector<unsigned int> cntp((size_t)n + 1, 0);
    for (int d = 0; d < n; ++d) cntp[(size_t)hid[d] + 1] = hc[d];
    for (int i = 0; i < n; ++i) cntp[i + 1] += cntp[i];
    for (int i = 0; i <= n; ++i) offsets[i] = (int)cntp[i];
    *total = (long long)t;
    if (!indices || cap < (long long)t) return FSPH_OK; /* sizes only */
    unsigned int *doff = c->key;
    int *dout = nullptr;
    float *dd2 = nullptr;
    FSPH_CUDA(c, cudaMemcpyAsync(doff, ho.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s));
    FSPH_CUDA(c, cudaMallocAsync((void **)&dout, std::max<size_t>(t, 1) * 4, s));
    if (dist2) FSPH_CUDA(c, cudaMallocAsync((void **)&dd2, std::max<size_t>(t, 1) * 4, s));
    launch_nb_fill(p, c->cell_start, c->set[1].pos, c->set[1].id, doff, dout, dd2, s);
    std::vector<int> hidx((size_t)t);
    std::vector<float> hd2(dist2 ? (size_t)t : 0);
    FSPH_CUDA(c, cudaMemcpyAsync(hidx.data(), dout, (size_t)t * 4, cudaMemcpyDeviceToHost, s));
    if (dist2) FSPH_CUDA(c, cudaMemcpyAsync(hd2.data(), dd2, (size_t)t * 4, cudaMemcpyDeviceToHost, s));
    FSPH_CUDA(c, cudaFreeAsync(dout, s));
    if (dd2) FSPH_CUDA(c, cudaFreeAsync(dd2, s));
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    FSPH_TRY(check_launch(c));
    std::vector<std::pair<int, float> > row;
    for (int d = 0; d < n; ++d) {
        const int pi = hid[d];
        row.clear();
        for (unsigned int k = ho[d]; k < ho[d] + hc[d]; ++k) row.emplace_back(hidx[k], dist2 ? hd2[k] : 0.0f);
        std::sort(row.begin(), row.end());
        for (size_t k = 0; k < row.size(); ++k) {
            indices[cntp[pi] + k] = row[k].first;
            if (dist2) dist2[cntp[pi] + k] = row[k].second;
        }
    }
    return FSPH_OK;
}

int fsph_neighbors(fsph_ctx *c, int *offsets, int *indices, long long cap, long long *total) {
    return fsph_neighbors_ex(c, nullptr, 0, 0.0f, FSPH_HOST, offsets, indices, nullptr, cap, total);
}

int fsph_reference_cell_hash(fsph_ctx *c, int rule, const float *pos4, int n, int where, unsigned int *hash,
                             int *grid, double *cell_width) {
    if (!c || n < 0 || (n > 0 && (!pos4 || !hash))) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    if (rule != 0 && rule != 1) return fail(c, FSPH_INVALID_ARG, "rule: 0 (CPU grid) or 1 (GPU grid)");
    if (where != FSPH_HOST && where != FSPH_DEVICE) return fail(c, FSPH_INVALID_ARG, "where");
    double org[3], cw;
    int g[3];
    if (reference_grid(c->P, rule, org, cw, g) != FSPH_OK)
        return fail(c, FSPH_INVALID_ARG, "degenerate reference grid for this box and h");
    if (grid) std::memcpy(grid, g, sizeof(g));
    if (cell_width) *cell_width = cw;
    if (n == 0) return FSPH_OK;
    cudaStream_t s = c->stream;
    const float4 *dpos = reinterpret_cast<const float4 *>(pos4);
    unsigned int *dout = hash;
    float4 *tpos = nullptr;
    if (where == FSPH_HOST) {
        FSPH_CUDA(c, cudaMallocAsync((void **)&tpos, (size_t)n * sizeof(float4), s));
        FSPH_CUDA(c, cudaMallocAsync((void **)&dout, (size_t)n * sizeof(unsigned int), s));
        FSPH_CUDA(c, cudaMemcpyAsync(tpos, pos4, (size_t)n * sizeof(float4), cudaMemcpyHostToDevice, s));
        dpos = tpos;
    }
    launch_reference_cells(n, dpos, rule, org, cw, g, dout, s);
    cudaError_t e = cudaGetLastError();
    if (where == FSPH_HOST) {
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(hash, dout, (size_t)n * sizeof(unsigned int), cudaMemcpyDeviceToHost, s);
        cudaFreeAsync(tpos, s);
        cudaFreeAsync(dout, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(c, FSPH_CUDA_ERROR, std::string("reference cell hash: ") + cudaGetErrorString(e));
    return FSPH_OK;
}

int fsph_density_grid(fsph_ctx *c, const int *nn, const double *minp, const double *d, float *out, int where) {
    if (!c || !nn || !minp || !d || !out) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    if (where != FSPH_HOST && where != FSPH_DEVICE) return fail(c, FSPH_INVALID_ARG, "where");
    for (int a = 0; a < 3; ++a)
        if (nn[a] <= 0 || !std::isfinite(minp[a]) || !std::isfinite(d[a]))
            return fail(c, FSPH_INVALID_ARG, "lattice: positive node counts, finite origin and spacing");
    const long long tot = (long long)nn[0] * nn[1] * nn[2];
    if (tot > (1ll << 31)) return fail(c, FSPH_INVALID_ARG, "more than 2^31 lattice nodes");
    cudaStream_t s = c->stream;
    float *dout = where == FSPH_DEVICE ? out : nullptr;
    if (c->n_active == 0) { /* no particles: an empty field */
        if (where == FSPH_HOST) std::memset(out, 0, (size_t)tot * sizeof(float));
        else FSPH_CUDA(c, cudaMemsetAsync(out, 0, (size_t)tot * sizeof(float), s));
        FSPH_CUDA(c, cudaStreamSynchronize(s));
        return FSPH_OK;
    }
    /* the simulation range: the box grown by 1 % (rx_sph_pbd.cpp:188-196) */
    double lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        const double size = c->P.box_max[a] - c->P.box_min[a];
        lo[a] = c->P.box_min[a] - 0.5 * 0.01 * size;
        hi[a] = lo[a] + size * (1.0 + 0.01);
    }
    DevParams p = dev_for(c, c->n_active, 1.0f); /* the deleted particles are parked far away */
    FSPH_TRY(build_on(c, p, c->set[0].pos));
    if (!dout) FSPH_CUDA(c, cudaMallocAsync((void **)&dout, (size_t)tot * sizeof(float), s));
    launch_density_grid(p, c->cell_start, c->set[1].pos, nn, minp, d, lo, hi, dout, s);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && where == FSPH_HOST)
        e = cudaMemcpyAsync(out, dout, (size_t)tot * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (where == FSPH_HOST) cudaFreeAsync(dout, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(c, FSPH_CUDA_ERROR, std::string("density grid: ") + cudaGetErrorString(e));
    return FSPH_OK;
}

int fsph_step_fields(fsph_ctx *c, float dt, void *stream) {
    if (!c) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    if (c->n_active <= 0) return fail(c, FSPH_INVALID_ARG, "no particles");
    if (!(dt > 0.0f) || !std::isfinite(dt)) return fail(c, FSPH_INVALID_ARG, "dt must be positive and finite");
    cudaStream_t user = (cudaStream_t)stream;
    if (user && user != c->stream) FSPH_CUDA(c, cudaStreamSynchronize(user));
    DevParams p = dev_for(c, c->n_active, dt);
    cudaStream_t s = c->stream;
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    /* results keep the sorted order of this evaluation (res_id); the
     * particles themselves stay where they are */
    enqueue_sort(c, p, c->set[0].pos, s);
    Gather g{};
    g.n4 = 2; g.n1 = 1;
    g.src4[0] = c->set[0].pos; g.dst4[0] = c->set[1].pos;
    g.src4[1] = c->set[0].vel; g.dst4[1] = c->set[1].vel;
    g.src1[0] = c->set[0].id; g.dst1[0] = c->res_id;
    launch_gather(p.n, c->perm, g, nullptr, s);
    if (c->P.solver == FSPH_SOLVER_WCSPH) {
        launch_sph_density(p, c->cell_start, c->set[1].pos, c->set[1].vel, c->dens, c->pres, c->nl, s);
        launch_sph_force(p, c->cell_start, c->set[1].pos, c->set[1].vel, c->acc, c->nl, s);
    } else {
        launch_pbf_density(p, c->cell_start, c->set[1].pos, c->dens, s);
        launch_pbf_visc(p, c->cell_start, c->set[1].pos, c->set[1].vel, c->dens, c->acc, s);
    }
    FSPH_TRY(check_launch(c));
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    c->res_in_res_id = true;
    return FSPH_OK;
}

/* ---- state file: everything a step reads, in device order ---- */
extern "C++" {
namespace {
const char kStateMagic[8] = {'F', 'S', 'P', 'H', 'S', 'T', 'A', 'T'};
const int kStateVersion = 3;

struct StateHeader {
    char magic[8];
    int version, params_size, n, n_active, nb, inlet_start;
    int n_inlets, n_del, n_boxes, n_spheres;
    int home_identity, model_loaded, model_nbr;
    unsigned int warm_valid;
    int mlp_bytes, features;
    long long steps_done;
    int poly_nv, poly_nt;
    int obstacle_bytes, inlet_bytes; /* layouts of the raw records that follow */
};

template <class T>
bool put(std::FILE *f, const T *v, size_t count) { return count == 0 || std::fwrite(v, sizeof(T), count, f) == count; }
template <class T>
bool get(std::FILE *f, T *v, size_t count) { return count == 0 || std::fread(v, sizeof(T), count, f) == count; }

/* device array <-> file through a host buffer */
template <class T>
int put_dev(fsph_ctx *c, std::FILE *f, const T *d, size_t count) {
    std::vector<T> h(count);
    if (count) FSPH_CUDA(c, cudaMemcpy(h.data(), d, count * sizeof(T), cudaMemcpyDeviceToHost));
    return put(f, h.data(), count) ? FSPH_OK : fail(c, FSPH_INVALID_ARG, "state file: write failed");
}
template <class T>
int get_dev(fsph_ctx *c, std::FILE *f, T *d, size_t count) {
    std::vector<T> h(count);
    if (!get(f, h.data(), count)) return fail(c, FSPH_INVALID_ARG, "state file: truncated");
    if (count) FSPH_CUDA(c, cudaMemcpy(d, h.data(), count * sizeof(T), cudaMemcpyHostToDevice));
    return FSPH_OK;
}
struct FileCloser {
    std::FILE *f;
    ~FileCloser() { if (f) std::fclose(f); }
};
}  // namespace
}  // extern "C++"

int fsph_save_state(fsph_ctx *c, const char *path) {
    if (!c || !path) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    FSPH_CUDA(c, cudaStreamSynchronize(c->stream));
    FileCloser fc{std::fopen(path, "wb")};
    if (!fc.f) return fail(c, FSPH_INVALID_ARG, std::string("cannot write ") + path);
    StateHeader h{};
    std::memcpy(h.magic, kStateMagic, 8);
    h.version = kStateVersion;
    h.params_size = (int)sizeof(fsph_params);
    h.n = c->n; h.n_active = c->n_active; h.nb = c->nb; h.inlet_start = c->inlet_start;
    h.n_inlets = (int)c->inlets.size(); h.n_del = (int)c->del_regions.size();
    h.n_boxes = (int)c->boxes.size(); h.n_spheres = (int)c->spheres.size();
    h.home_identity = c->home_identity ? 1 : 0;
    h.model_loaded = c->model_loaded ? 1 : 0;
    h.model_nbr = c->model_nbr ? 1 : 0;
    FSPH_CUDA(c, cudaMemcpy(&h.warm_valid, c->warm_valid, sizeof(unsigned int), cudaMemcpyDeviceToHost));
    h.mlp_bytes = (int)sizeof(MlpDev);
    h.features = kFeatures;
    h.steps_done = c->steps_done;
    h.poly_nv = (int)(c->poly_v.size() / 3);
    h.poly_nt = (int)(c->poly_t.size() / 3);
    h.obstacle_bytes = (int)sizeof(Obstacle);
    h.inlet_bytes = (int)sizeof(fsph_ctx::Inlet);
    bool ok = put(fc.f, &h, 1) && put(fc.f, &c->P, 1) && put(fc.f, c->inlets.data(), c->inlets.size()) &&
              put(fc.f, c->del_regions.data(), c->del_regions.size()) && put(fc.f, c->boxes.data(), c->boxes.size()) &&
              put(fc.f, c->spheres.data(), c->spheres.size()) && put(fc.f, c->poly_v.data(), c->poly_v.size()) &&
              put(fc.f, c->poly_t.data(), c->poly_t.size());
    if (!ok) return fail(c, FSPH_INVALID_ARG, "state file: write failed");
    const size_t n = (size_t)c->n;
    FSPH_TRY(put_dev(c, fc.f, c->set[0].pos, n));
    FSPH_TRY(put_dev(c, fc.f, c->set[0].vel, n));
    FSPH_TRY(put_dev(c, fc.f, c->set[0].id, n));
    FSPH_TRY(put_dev(c, fc.f, c->set[0].attr, n));
    FSPH_TRY(put_dev(c, fc.f, c->dstep, n));
    FSPH_TRY(put_dev(c, fc.f, c->feat, n * kFeatures));
    FSPH_TRY(put_dev(c, fc.f, c->b_in, (size_t)c->nb));
    if (c->model_loaded)
        FSPH_TRY(put_dev(c, fc.f, reinterpret_cast<const unsigned char *>(c->mlp_dev), sizeof(MlpDev)));
    if (std::fflush(fc.f) != 0) return fail(c, FSPH_INVALID_ARG, "state file: write failed");
    return FSPH_OK;
}

int fsph_load_state(fsph_ctx *c, const char *path) {
    if (!c || !path) return FSPH_INVALID_ARG;
    FileCloser fc{std::fopen(path, "rb")};
    if (!fc.f) return fail(c, FSPH_INVALID_ARG, std::string("cannot read ") + path);
    StateHeader h{};
    if (!get(fc.f, &h, 1) || std::memcmp(h.magic, kStateMagic, 8) != 0)
        return fail(c, FSPH_INVALID_ARG, "not a state file");
    if (h.version != kStateVersion || h.params_size != (int)sizeof(fsph_params) || h.mlp_bytes != (int)sizeof(MlpDev) ||
        h.features != kFeatures || h.obstacle_bytes != (int)sizeof(Obstacle) ||
        h.inlet_bytes != (int)sizeof(fsph_ctx::Inlet))
        return fail(c, FSPH_INVALID_ARG, "state file of another version or build");
    fsph_params P{};
    if (!get(fc.f, &P, 1)) return fail(c, FSPH_INVALID_ARG, "state file: truncated");
    if (h.n < 0 || h.n > P.max_particles || h.n_active < 0 || h.n_active > h.n || h.nb < 0 || h.n_inlets < 0 ||
        h.n_del < 0 || h.n_boxes < 0 || h.n_boxes > kMaxBoxObstacles || h.n_spheres < 0 ||
        h.n_spheres > kMaxSphereObstacles || (h.n_del & 1) || h.n_del > 2 * 64 || h.n_inlets > 4096 ||
        h.poly_nv < 0 || h.poly_nv > (1 << 24) || h.poly_nt < 0 || h.poly_nt > (1 << 24))
        return fail(c, FSPH_INVALID_ARG, "state file: inconsistent counts");
    if (P.solver != c->P.solver) return fail(c, FSPH_INVALID_ARG, "state file of the other solver");
    std::vector<fsph_ctx::Inlet> inlets((size_t)h.n_inlets);
    std::vector<float4> del((size_t)h.n_del);
    std::vector<Obstacle> boxes((size_t)h.n_boxes), spheres((size_t)h.n_spheres);
    std::vector<float> poly_v(3 * (size_t)h.poly_nv);
    std::vector<int> poly_t(3 * (size_t)h.poly_nt);
    if (!get(fc.f, inlets.data(), inlets.size()) || !get(fc.f, del.data(), del.size()) ||
        !get(fc.f, boxes.data(), boxes.size()) || !get(fc.f, spheres.data(), spheres.size()) ||
        !get(fc.f, poly_v.data(), poly_v.size()) || !get(fc.f, poly_t.data(), poly_t.size()))
        return fail(c, FSPH_INVALID_ARG, "state file: truncated");
    for (int k : poly_t)
        if (k < 0 || k >= h.poly_nv) return fail(c, FSPH_INVALID_ARG, "state file: triangle vertex outside the mesh");
    /* the particle arrays are read into host buffers first, so a bad file
     * leaves the context as it was */
    const size_t n = (size_t)h.n;
    std::vector<float4> pos(n), vel(n), dstep(n), bpos((size_t)h.nb);
    std::vector<unsigned int> id(n), attr(n);
    std::vector<float> feat(n * kFeatures);
    std::vector<unsigned char> mlp(h.model_loaded ? sizeof(MlpDev) : 0);
    if (!get(fc.f, pos.data(), n) || !get(fc.f, vel.data(), n) || !get(fc.f, id.data(), n) ||
        !get(fc.f, attr.data(), n) || !get(fc.f, dstep.data(), n) || !get(fc.f, feat.data(), feat.size()) ||
        !get(fc.f, bpos.data(), bpos.size()) || !get(fc.f, mlp.data(), mlp.size()))
        return fail(c, FSPH_INVALID_ARG, "state file: truncated");
    std::vector<unsigned char> seen(n, 0);
    for (size_t k = 0; k < n; ++k) {
        if (id[k] >= n || seen[id[k]]) return fail(c, FSPH_INVALID_ARG, "state file: particle order is not a permutation");
        seen[id[k]] = 1;
    }
    FSPH_TRY(fsph_set_params(c, &P));
    FSPH_TRY(fsph_set_boundary(c, h.nb ? reinterpret_cast<const float *>(bpos.data()) : nullptr, h.nb, FSPH_HOST));
    FSPH_TRY(load_particles(c, reinterpret_cast<const float *>(pos.data()), reinterpret_cast<const float *>(vel.data()),
                            h.n, FSPH_HOST));
    cudaStream_t s = c->stream;
    FSPH_CUDA(c, cudaMemcpyAsync(c->set[0].id, id.data(), n * 4, cudaMemcpyHostToDevice, s));
    FSPH_CUDA(c, cudaMemcpyAsync(c->set[0].attr, attr.data(), n * 4, cudaMemcpyHostToDevice, s));
    FSPH_CUDA(c, cudaMemcpyAsync(c->dstep, dstep.data(), n * 16, cudaMemcpyHostToDevice, s));
    FSPH_CUDA(c, cudaMemcpyAsync(c->feat, feat.data(), feat.size() * 4, cudaMemcpyHostToDevice, s));
    FSPH_CUDA(c, cudaMemcpyAsync(c->warm_valid, &h.warm_valid, sizeof(unsigned int), cudaMemcpyHostToDevice, s));
    if (h.model_loaded) FSPH_CUDA(c, cudaMemcpyAsync(c->mlp_dev, mlp.data(), mlp.size(), cudaMemcpyHostToDevice, s));
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    c->model_loaded = h.model_loaded != 0;
    c->model_nbr = h.model_nbr != 0;
    c->home_identity = h.home_identity != 0;
    c->res_in_res_id = false;
    c->n_active = h.n_active;
    c->inlets = inlets;
    c->inlet_start = h.inlet_start;
    c->del_regions = del;
    c->boxes = boxes;
    c->spheres = spheres;
    c->steps_done = h.steps_done;
    c->poly_v = poly_v;
    c->poly_t = poly_t;
    drop_graph(c);
    FSPH_TRY(upload_obstacles(c));
    FSPH_TRY(polygons_upload(c));
    if (!c->del_regions.empty()) { /* the table fsph_add_delete_region keeps: 64 regions */
        if (!c->del_dev) FSPH_CUDA(c, cudaMalloc((void **)&c->del_dev, 2 * 64 * sizeof(float4)));
        FSPH_CUDA(c, cudaMemcpy(c->del_dev, c->del_regions.data(), c->del_regions.size() * sizeof(float4),
                                cudaMemcpyHostToDevice));
    }
    return FSPH_OK;
}

int fsph_set_warm_start_model(fsph_ctx *c, const float *blob) {
    if (!c || !blob) return FSPH_INVALID_ARG;
    for (int k = 0; k < FSPH_MLP_BLOB_SIZE; ++k)
        if (!std::isfinite(blob[k])) return fail(c, FSPH_INVALID_ARG, "non-finite network parameter");
    mlp_tc_prepare(); /* before any step graph is captured */
    float *d = nullptr;
    FSPH_CUDA(c, cudaMalloc((void **)&d, FSPH_MLP_BLOB_SIZE * sizeof(float)));
    cudaError_t e = cudaMemcpyAsync(d, blob, FSPH_MLP_BLOB_SIZE * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        launch_mlp_pack(d, c->mlp_dev, c->stream);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d);
    if (e != cudaSuccess) return fail(c, FSPH_CUDA_ERROR, std::string("warm-start model: ") + cudaGetErrorString(e));
    c->model_loaded = true;
    /* an input whose spread is given as >= 1e29 carries no weight */
    c->model_nbr = false;
    for (int k = kNbrFirst; k <= kNbrLast; ++k)
        if (blob[FSPH_MLP_FEATURES + k] < 1e29f) c->model_nbr = true;
    return FSPH_OK;
}

int fsph_set_boundary(fsph_ctx *c, const float *bpos4, int nb, int where) {
    if (!c || nb < 0 || (nb > 0 && !bpos4)) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    if (where != FSPH_HOST && where != FSPH_DEVICE) return fail(c, FSPH_INVALID_ARG, "where");
    if (nb > 0 && c->P.solver != FSPH_SOLVER_PBF) return fail(c, FSPH_UNSUPPORTED, "boundary particles: PBF only");
    FSPH_CUDA(c, cudaStreamSynchronize(c->stream));
    free_boundary(c);
    drop_graph(c);
    if (nb == 0) return FSPH_OK;
    const size_t n = (size_t)nb;
    FSPH_TRY(dalloc(c, &c->b_in, n)); FSPH_TRY(dalloc(c, &c->b_pos, n));
    FSPH_TRY(dalloc(c, &c->b_lam, n)); FSPH_TRY(dalloc(c, &c->b_scale, n)); FSPH_TRY(dalloc(c, &c->b_stat, n));
    FSPH_TRY(dalloc(c, &c->b_id, n)); FSPH_TRY(dalloc(c, &c->b_key, n)); FSPH_TRY(dalloc(c, &c->b_rank, n));
    cudaMemcpyKind k = where == FSPH_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    FSPH_CUDA(c, cudaMemcpyAsync(c->b_in, bpos4, n * sizeof(float4), k, c->stream));
    FSPH_CUDA(c, cudaMemsetAsync(c->flag, 0, sizeof(unsigned int), c->stream));
    launch_check_finite(nb, c->b_in, nullptr, c->flag, c->stream);
    FSPH_CUDA(c, cudaMemcpyAsync(c->flag_host, c->flag, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream));
    FSPH_CUDA(c, cudaStreamSynchronize(c->stream));
    if (*c->flag_host) {
        free_boundary(c);
        return fail(c, FSPH_NAN_DETECTED, "non-finite boundary position");
    }
    c->nb = nb;
    const int st = boundary_build(c);
    if (st != FSPH_OK) free_boundary(c);
    return st;
}

int fsph_get_boundary(fsph_ctx *c, int which, float *dst) {
    if (!c || !dst) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    const int nb = c->nb;
    if (nb == 0) return FSPH_OK;
    cudaStream_t s = c->stream;
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    if (which == FSPH_BOUNDARY_POSITION) {
        FSPH_CUDA(c, cudaMemcpyAsync(dst, c->b_in, (size_t)nb * sizeof(float4), cudaMemcpyDeviceToHost, s));
    } else if (which == FSPH_BOUNDARY_VOLUME || which == FSPH_BOUNDARY_LAMBDA) {
        const float *src = which == FSPH_BOUNDARY_VOLUME ? c->b_scale : c->b_lam;
        float *t = reinterpret_cast<float *>(c->b_key); /* free after the boundary build */
        launch_unsort1(nb, c->b_id, reinterpret_cast<const unsigned int *>(src), reinterpret_cast<unsigned int *>(t), s);
        FSPH_CUDA(c, cudaMemcpyAsync(dst, t, (size_t)nb * sizeof(float), cudaMemcpyDeviceToHost, s));
        FSPH_CUDA(c, cudaStreamSynchronize(s));
        if (which == FSPH_BOUNDARY_VOLUME) /* rho0 psi_b / m -> psi_b */
            for (int b = 0; b < nb; ++b) dst[b] = dst[b] * c->P.mass / c->P.rest_dens;
    } else {
        return fail(c, FSPH_INVALID_ARG, "which: FSPH_BOUNDARY_POSITION, _VOLUME or _LAMBDA");
    }
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    FSPH_TRY(check_launch(c));
    return FSPH_OK;
}

int fsph_num_boundary(const fsph_ctx *c) { return c ? c->nb : -1; }

int fsph_set_box_obstacle(fsph_ctx *c, const double *cen, const double *ext, const double *ang,
                          const double *vel, int flg) {
    if (!c || !cen || !ext) return FSPH_INVALID_ARG;
    (void)vel; /* stored by the reference too, and not used by its fluid step */
    if (!flg) return FSPH_OK; /* a disabled obstacle is skipped (rx_pbdsph_kernel.cu:873) */
    if ((int)c->boxes.size() >= kMaxBoxObstacles) return fail(c, FSPH_INVALID_ARG, "at most 10 box obstacles");
    for (int a = 0; a < 3; ++a)
        if (!std::isfinite(cen[a]) || !(ext[a] > 0.0) || !std::isfinite(ext[a]) || (ang && !std::isfinite(ang[a])))
            return fail(c, FSPH_INVALID_ARG, "box obstacle: finite centre and angles, positive extents");
    Obstacle o{};
    o.cen = make_float4((float)cen[0], (float)cen[1], (float)cen[2], 0.0f);
    o.ext = make_float4((float)ext[0], (float)ext[1], (float)ext[2], 0.0f);
    const double zero[3] = {0.0, 0.0, 0.0};
    box_rotation(ang ? ang : zero, o);
    c->boxes.push_back(o);
    return upload_obstacles(c);
}

int fsph_set_sphere_obstacle(fsph_ctx *c, const double *cen, double rad, const double *vel, int flg) {
    if (!c || !cen) return FSPH_INVALID_ARG;
    (void)vel;
    if (!flg) return FSPH_OK;
    if ((int)c->spheres.size() >= kMaxSphereObstacles) return fail(c, FSPH_INVALID_ARG, "at most 10 sphere obstacles");
    if (!(rad > 0.0) || !std::isfinite(rad) || !std::isfinite(cen[0]) || !std::isfinite(cen[1]) ||
        !std::isfinite(cen[2]))
        return fail(c, FSPH_INVALID_ARG, "sphere obstacle: finite centre, positive radius");
    Obstacle o{};
    o.cen = make_float4((float)cen[0], (float)cen[1], (float)cen[2], (float)rad);
    o.ext = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    c->spheres.push_back(o);
    return upload_obstacles(c);
}

int fsph_move_sphere_obstacle(fsph_ctx *c, int b, const double *disp) {
    if (!c || !disp) return FSPH_INVALID_ARG;
    if (b < 0 || b >= (int)c->spheres.size()) return fail(c, FSPH_INVALID_ARG, "no such sphere obstacle");
    float4 &q = c->spheres[(size_t)b].cen;
    q = make_float4((float)(q.x + disp[0]), (float)(q.y + disp[1]), (float)(q.z + disp[2]), q.w);
    FSPH_CUDA(c, cudaStreamSynchronize(c->stream)); /* not under a step that reads the table */
    return upload_obstacles(c);
}

int fsph_get_sphere_obstacle_pos(const fsph_ctx *c, int b, double *pos) {
    if (!c || !pos || b < 0 || b >= (int)c->spheres.size()) return FSPH_INVALID_ARG;
    const float4 q = c->spheres[(size_t)b].cen;
    pos[0] = q.x; pos[1] = q.y; pos[2] = q.z;
    return FSPH_OK;
}

int fsph_clear_obstacles(fsph_ctx *c) {
    if (!c) return FSPH_INVALID_ARG;
    FSPH_CUDA(c, cudaStreamSynchronize(c->stream));
    c->boxes.clear();
    c->spheres.clear();
    return upload_obstacles(c);
}

int fsph_num_obstacles(const fsph_ctx *c) { return c ? (int)(c->boxes.size() + c->spheres.size()) : -1; }

int fsph_set_polygon_obstacle(fsph_ctx *c, const double *vrts, int nv, const int *tris, int nt, const double *vel) {
    if (!c || nv < 0 || nt < 0 || (nv > 0 && !vrts) || (nt > 0 && !tris)) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    (void)vel; /* the reference keeps it unused (its PolyVel lines are commented out) */
    if (nt == 0) return FSPH_OK;
    const long long base = (long long)c->poly_v.size() / 3;
    if (base + nv > (1ll << 24) || (long long)c->poly_t.size() / 3 + nt > (1ll << 24))
        return fail(c, FSPH_INVALID_ARG, "at most 2^24 obstacle vertices and triangles");
    for (long long k = 0; k < 3ll * nv; ++k)
        if (!std::isfinite(vrts[k])) return fail(c, FSPH_INVALID_ARG, "polygon obstacle: non-finite vertex");
    for (long long k = 0; k < 3ll * nt; ++k)
        if (tris[k] < 0 || tris[k] >= nv) return fail(c, FSPH_INVALID_ARG, "polygon obstacle: vertex index outside [0, nv)");
    for (long long k = 0; k < 3ll * nv; ++k) c->poly_v.push_back((float)vrts[k]);
    for (long long k = 0; k < 3ll * nt; ++k) c->poly_t.push_back((int)(tris[k] + base));
    const int st = polygons_upload(c);
    if (st != FSPH_OK) { /* leave no half-added mesh */
        c->poly_v.resize((size_t)base * 3);
        c->poly_t.resize(c->poly_t.size() - 3 * (size_t)nt);
        polygons_upload(c);
    }
    return st;
}

int fsph_clear_polygon_obstacles(fsph_ctx *c) {
    if (!c) return FSPH_INVALID_ARG;
    c->poly_v.clear();
    c->poly_t.clear();
    return polygons_upload(c);
}

int fsph_num_polygon_triangles(const fsph_ctx *c) { return c ? (int)(c->poly_t.size() / 3) : -1; }

int fsph_polygon_collide(fsph_ctx *c, const float *x0_4, float *x1_4, float *v4, int n, float dt, int where) {
    if (!c || n < 0 || (n > 0 && (!x0_4 || !x1_4 || !v4))) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    if (where != FSPH_HOST && where != FSPH_DEVICE) return fail(c, FSPH_INVALID_ARG, "where");
    if (n == 0 || c->ntri_dev == 0) return FSPH_OK;
    cudaStream_t s = c->stream;
    const size_t b = (size_t)n * sizeof(float4);
    const float4 *d0 = reinterpret_cast<const float4 *>(x0_4);
    float4 *d1 = reinterpret_cast<float4 *>(x1_4), *dv = reinterpret_cast<float4 *>(v4);
    float4 *tmp = nullptr;
    if (where == FSPH_HOST) {
        FSPH_CUDA(c, cudaMallocAsync((void **)&tmp, 3 * b, s));
        FSPH_CUDA(c, cudaMemcpyAsync(tmp, x0_4, b, cudaMemcpyHostToDevice, s));
        FSPH_CUDA(c, cudaMemcpyAsync(tmp + n, x1_4, b, cudaMemcpyHostToDevice, s));
        FSPH_CUDA(c, cudaMemcpyAsync(tmp + 2 * (size_t)n, v4, b, cudaMemcpyHostToDevice, s));
        d0 = tmp; d1 = tmp + n; dv = tmp + 2 * (size_t)n;
    }
    launch_polygon_collide(dev_for(c, n, dt), n, d0, d1, dv, s);
    cudaError_t e = cudaGetLastError();
    if (where == FSPH_HOST) {
        if (e == cudaSuccess) e = cudaMemcpyAsync(x1_4, d1, b, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(v4, dv, b, cudaMemcpyDeviceToHost, s);
        cudaFreeAsync(tmp, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(c, FSPH_CUDA_ERROR, std::string("polygon collision: ") + cudaGetErrorString(e));
    return FSPH_OK;
}

int fsph_num_active(const fsph_ctx *c) { return c ? c->n_active : -1; }

int fsph_add_delete_region(fsph_ctx *c, const double *lo, const double *hi) {
    if (!c || !lo || !hi) return FSPH_INVALID_ARG;
    for (int a = 0; a < 3; ++a)
        if (!std::isfinite(lo[a]) || !std::isfinite(hi[a])) return fail(c, FSPH_INVALID_ARG, "region: finite corners");
    if (c->del_regions.size() >= 2 * 64) return fail(c, FSPH_INVALID_ARG, "at most 64 deletion regions");
    c->del_regions.push_back(make_float4((float)lo[0], (float)lo[1], (float)lo[2], 0.0f));
    c->del_regions.push_back(make_float4((float)hi[0], (float)hi[1], (float)hi[2], 0.0f));
    FSPH_CUDA(c, cudaStreamSynchronize(c->stream));
    if (!c->del_dev) FSPH_CUDA(c, cudaMalloc((void **)&c->del_dev, 2 * 64 * sizeof(float4)));
    FSPH_CUDA(c, cudaMemcpy(c->del_dev, c->del_regions.data(), c->del_regions.size() * sizeof(float4),
                            cudaMemcpyHostToDevice));
    return FSPH_OK;
}

int fsph_clear_delete_regions(fsph_ctx *c) {
    if (!c) return FSPH_INVALID_ARG;
    c->del_regions.clear();
    return FSPH_OK;
}

int fsph_add_inlet_line(fsph_ctx *c, const double *pos1, const double *pos2, const double *vel, const double *up,
                        int accum, int span, double spacing) {
    /* the count of lines is returned, so a failure is the negated status */
    if (!c || !pos1 || !pos2 || !vel || !up) return -FSPH_INVALID_ARG;
    if (accum < 1 || span < 0 || !(spacing >= 0.0)) return -fail(c, FSPH_INVALID_ARG, "inlet: accum >= 1, span >= 0");
    fsph_ctx::Inlet q;
    for (int a = 0; a < 3; ++a) {
        q.pos1[a] = pos1[a]; q.pos2[a] = pos2[a]; q.vel[a] = vel[a]; q.up[a] = up[a];
        if (!std::isfinite(pos1[a]) || !std::isfinite(pos2[a]) || !std::isfinite(vel[a]) || !std::isfinite(up[a]))
            return -fail(c, FSPH_INVALID_ARG, "inlet: finite vectors");
    }
    q.accum = accum; q.span = span; q.spacing = spacing;
    c->inlets.push_back(q);
    return (int)c->inlets.size();
}

int fsph_clear_inlets(fsph_ctx *c) {
    if (!c) return FSPH_INVALID_ARG;
    c->inlets.clear();
    c->inlet_start = -1;
    return FSPH_OK;
}

int fsph_num_inlets(const fsph_ctx *c) { return c ? (int)c->inlets.size() : -1; }

namespace {
/* U[0, 1) from (seed, index): the SplitMix64 finaliser */
double inlet_uniform(unsigned long long seed, unsigned long long idx) {
    unsigned long long z = seed * 0x9E3779B97F4A7C15ull + idx * 0xD1B54A32D192ED03ull + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}
}  // namespace

int fsph_emit_inlets(fsph_ctx *c, int step, int *emitted) {
    if (!c) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    NvtxRange range("fsph_emit_inlets");
    if (emitted) *emitted = 0;
    if (c->inlets.empty()) return FSPH_OK;
    /* the particles of every line due at this step, in the reference's
     * placement (addParticles, rx_ps.cpp:444-520): n = l / r along the line,
     * at (i + 1/2) l / n from pos1, jitter 0.01 of the spacing, accum rows
     * stacked along up by spacing * (l / n); attribute = the line's index */
    std::vector<float4> px, pv;
    std::vector<int> pa;
    const double r = (double)c->P.particle_radius;
    for (size_t li = 0; li < c->inlets.size(); ++li) {
        const fsph_ctx::Inlet &q = c->inlets[li];
        if (!(q.span > 0 && step % q.span == 0)) continue;
        double rel[3], l = 0.0;
        for (int a = 0; a < 3; ++a) { rel[a] = q.pos2[a] - q.pos1[a]; l += rel[a] * rel[a]; }
        l = std::sqrt(l);
        const int n = (int)(l / r);
        if (n <= 0 || !(l > 0.0)) continue;
        const double spacing = l / n, jitter = spacing * 0.01;
        double p1[3] = {q.pos1[0], q.pos1[1], q.pos1[2]};
        const unsigned long long seed = (unsigned long long)(li + 1) * 1000003ull + (unsigned long long)step;
        for (int j = 0; j < q.accum; ++j) {
            for (int i = 0; i < n; ++i) {
                float x[3];
                for (int a = 0; a < 3; ++a) {
                    const double u = inlet_uniform(seed, 3ull * (px.size()) + (unsigned long long)a);
                    x[a] = (float)(p1[a] + rel[a] / l * (i + 0.5) * spacing + (u * 2.0 - 1.0) * jitter);
                }
                px.push_back(make_float4(x[0], x[1], x[2], 0.0f));
                pv.push_back(make_float4((float)q.vel[0], (float)q.vel[1], (float)q.vel[2], 0.0f));
                pa.push_back((int)li);
            }
            for (int a = 0; a < 3; ++a) p1[a] += q.up[a] * q.spacing * spacing;
        }
    }
    const int count = (int)px.size();
    if (count == 0) return FSPH_OK;
    /* the new particles go at the inlet index, after the existing ones at
     * first, wrapping to 0 past max_particles (rx_ps.cpp:466-505) */
    FSPH_TRY(home_to_particle_order(c));
    cudaStream_t s = c->stream;
    int index = c->inlet_start < 0 ? c->n : c->inlet_start;
    const int n_old = c->n;
    int n = c->n, done = 0;
    bool over = false;
    while (done < count) {
        if (index >= c->cap) { index = 0; over = true; }
        const int run = std::min(count - done, c->cap - index);
        FSPH_CUDA(c, cudaMemcpyAsync(c->set[0].pos + index, px.data() + done, (size_t)run * 16, cudaMemcpyHostToDevice, s));
        FSPH_CUDA(c, cudaMemcpyAsync(c->set[0].vel + index, pv.data() + done, (size_t)run * 16, cudaMemcpyHostToDevice, s));
        FSPH_CUDA(c, cudaMemcpyAsync(c->set[0].attr + index, pa.data() + done, (size_t)run * 4, cudaMemcpyHostToDevice, s));
        FSPH_CUDA(c, cudaMemsetAsync(c->dstep + index, 0, (size_t)run * 16, s));
        FSPH_CUDA(c, cudaMemsetAsync(c->feat + (size_t)index * kFeatures, 0, (size_t)run * kFeatures * 4, s));
        if (index + run > n) { /* new slots: their ids continue the particle order */
            launch_iota(index + run, c->set[0].id, s);
            n = index + run;
        }
        index += run;
        done += run;
    }
    if (over) n = c->cap;
    if (c->res_in_res_id && n > n_old) {
        /* the results' slot map covers the new particles too (they have no
         * results yet): slot d -> particle d, so it stays a permutation */
        launch_iota(n, c->perm, s);
        FSPH_CUDA(c, cudaMemcpyAsync(c->res_id + n_old, c->perm + n_old, (size_t)(n - n_old) * 4,
                                     cudaMemcpyDeviceToDevice, s));
    }
    c->n = n;
    c->inlet_start = index;
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    FSPH_TRY(check_launch(c));
    FSPH_TRY(repartition(c));
    if (emitted) *emitted = count;
    return FSPH_OK;
}

int fsph_time_pass(fsph_ctx *c, int pass, int reps, float *avg_ms) {
    if (!c || !avg_ms || reps <= 0) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    if (c->n_active <= 0) return fail(c, FSPH_INVALID_ARG, "no particles");
    const bool sph_pass = pass == FSPH_PASS_SPH_DENSITY || pass == FSPH_PASS_SPH_FORCE;
    if (sph_pass != (c->P.solver == FSPH_SOLVER_WCSPH))
        return fail(c, FSPH_UNSUPPORTED, "this pass belongs to the other solver");
    DevParams p = dev_for(c, c->n_active, c->dp.dt > 0.0f ? c->dp.dt : 1e-3f);
    cudaStream_t s = c->stream;
    if (sph_pass) {
        /* the state of a WCSPH step before its passes: grid on x, sorted x, v */
        enqueue_sort(c, p, c->set[0].pos, s);
        Gather g{};
        g.n4 = 2;
        g.src4[0] = c->set[0].pos; g.dst4[0] = c->set[1].pos;
        g.src4[1] = c->set[0].vel; g.dst4[1] = c->set[1].vel;
        launch_gather(p.n, c->perm, g, nullptr, s);
        launch_sph_density(p, c->cell_start, c->set[1].pos, c->set[1].vel, c->dens, c->pres, c->nl, s);
        cudaEvent_t e0, e1;
        FSPH_CUDA(c, cudaEventCreate(&e0));
        FSPH_CUDA(c, cudaEventCreate(&e1));
        FSPH_CUDA(c, cudaEventRecord(e0, s));
        for (int k = 0; k < reps; ++k) {
            if (pass == FSPH_PASS_SPH_DENSITY)
                launch_sph_density(p, c->cell_start, c->set[1].pos, c->set[1].vel, c->dens, c->pres, c->nl, s);
            else
                launch_sph_force(p, c->cell_start, c->set[1].pos, c->set[1].vel, c->acc, c->nl, s);
        }
        FSPH_CUDA(c, cudaEventRecord(e1, s));
        FSPH_CUDA(c, cudaEventSynchronize(e1));
        float ms = 0.0f;
        FSPH_CUDA(c, cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        FSPH_TRY(check_launch(c));
        *avg_ms = ms / (float)reps;
        /* the home set keeps the particles; only scratch arrays were written */
        return FSPH_OK;
    }
    /* the state after a step: x* = x in the home set, already cell-ordered */
    FSPH_TRY(build_on(c, p, c->set[0].pos));
    FSPH_CUDA(c, cudaMemsetAsync(c->ctl, 0, sizeof(DevCtl), s));
    launch_lambda(p, c->cell_start, c->ppos[0], c->ppos[1], c->dens, c->ctl, c->epart, 0ull, 0, c->nl, s);
    cudaEvent_t e0, e1;
    FSPH_CUDA(c, cudaEventCreate(&e0));
    FSPH_CUDA(c, cudaEventCreate(&e1));
    FSPH_CUDA(c, cudaEventRecord(e0, s));
    for (int k = 0; k < reps; ++k) {
        if (pass == FSPH_PASS_LAMBDA) {
            launch_lambda(p, c->cell_start, c->ppos[0], c->ppos[1], c->dens, c->ctl, c->epart, 0ull, 0, c->nl, s);
        } else if (pass == FSPH_PASS_CORRECTION) {
            launch_correction(p, c->cell_start, c->ppos[0], c->ppos[1], c->xb, c->ctl, c->dpart, 0ull, 0ull, 0,
                              nullptr, c->nl, s);
        } else if (pass == FSPH_PASS_GRID) {
            enqueue_sort(c, p, c->set[1].pos, s);
            Gather g{};
            g.n4 = 3; g.n1 = 1;
            g.src4[0] = c->set[1].pos; g.dst4[0] = c->set[1].vel;
            g.src4[1] = c->set[1].pos; g.dst4[1] = c->ppos[1];
            g.src4[2] = c->set[1].pos; g.dst4[2] = c->acc;
            g.src1[0] = c->set[1].id; g.dst1[0] = c->set[1].attr;
            launch_gather(p.n, c->perm, g, nullptr, s);
        } else if (pass == FSPH_PASS_LIST) {
            launch_build_list(p, c->cell_start, c->xb, c->nl, s);
        } else {
            cudaEventDestroy(e0); cudaEventDestroy(e1);
            return fail(c, FSPH_INVALID_ARG, "unknown pass");
        }
    }
    FSPH_CUDA(c, cudaEventRecord(e1, s));
    FSPH_CUDA(c, cudaEventSynchronize(e1));
    float ms = 0.0f;
    FSPH_CUDA(c, cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    FSPH_TRY(check_launch(c));
    *avg_ms = ms / (float)reps;
    return FSPH_OK;
}

int fsph_pbf_eval_lambda(fsph_ctx *c, const float *pos4, int n, float *dens, float *lambda) {
    if (!c || !pos4 || !dens || !lambda) return FSPH_INVALID_ARG;
    FSPH_TRY(fsph_set_particles(c, pos4, nullptr, n, FSPH_HOST));
    if (n == 0) return FSPH_OK;
    DevParams p = dev_for(c, n, 1.0f);
    cudaStream_t s = c->stream;
    FSPH_CUDA(c, cudaMemsetAsync(c->ctl, 0, sizeof(DevCtl), s));
    FSPH_TRY(build_on(c, p, c->set[0].pos));
    launch_lambda(p, c->cell_start, c->ppos[0], c->ppos[1], c->dens, c->ctl, c->epart, 0ull, 0, c->nl, s);
    launch_boundary_lambda(p, c->cell_start, c->ppos[0], c->ppos[1], c->ctl, c->b_stat, c->b_lam, s);
    FSPH_TRY(check_launch(c));
    FSPH_TRY(copy_out_scalar(c, c->dens, c->set[1].id, dens, n));
    launch_unsort_w(n, c->set[1].id, c->ppos[0], reinterpret_cast<float *>(c->key), s);
    FSPH_CUDA(c, cudaMemcpyAsync(lambda, c->key, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    return FSPH_OK;
}

int fsph_pbf_eval_correction(fsph_ctx *c, const float *pos4, const float *lambda, int n, float dt, float *dp4) {
    if (!c || !pos4 || !lambda || !dp4) return FSPH_INVALID_ARG;
    FSPH_TRY(fsph_set_particles(c, pos4, nullptr, n, FSPH_HOST));
    if (n == 0) return FSPH_OK;
    DevParams p = dev_for(c, n, dt);
    cudaStream_t s = c->stream;
    FSPH_CUDA(c, cudaMemsetAsync(c->ctl, 0, sizeof(DevCtl), s));
    /* lambda rides in x*.w, in particle order before the sort */
    float *dl = reinterpret_cast<float *>(c->pres);
    FSPH_CUDA(c, cudaMemcpyAsync(dl, lambda, (size_t)n * 4, cudaMemcpyHostToDevice, s));
    launch_pack_w(n, c->set[0].pos, dl, s);
    FSPH_TRY(build_on(c, p, c->set[0].pos));
    launch_correction(p, c->cell_start, c->ppos[0], c->ppos[1], c->xb, c->ctl, c->dpart, 0ull, 0ull, 0, c->acc, c->nl, s);
    FSPH_TRY(check_launch(c));
    launch_unsort4(n, c->set[1].id, c->acc, c->set[0].vel, 1, s);
    FSPH_CUDA(c, cudaMemcpyAsync(dp4, c->set[0].vel, (size_t)n * 16, cudaMemcpyDeviceToHost, s));
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    /* the context's particles are left at the given positions, zero velocity */
    FSPH_TRY(fsph_set_particles(c, pos4, nullptr, n, FSPH_HOST));
    return FSPH_OK;
}

int fsph_pbf_eval_xsph_vorticity(fsph_ctx *c, const float *pos4, const float *vel4, const float *dens, int n,
                                 float dt, float *vel_out4, float *vort4) {
    if (!c || !pos4 || !vel4 || !dens || !vel_out4 || !vort4) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    if (c->P.solver != FSPH_SOLVER_PBF) return fail(c, FSPH_UNSUPPORTED, "XSPH / vorticity: PBF only");
    if (!(dt > 0.0f) || !std::isfinite(dt)) return fail(c, FSPH_INVALID_ARG, "dt must be positive and finite");
    FSPH_TRY(fsph_set_particles(c, pos4, vel4, n, FSPH_HOST));
    if (n == 0) return FSPH_OK;
    DevParams p = dev_for(c, n, dt);
    cudaStream_t s = c->stream;
    /* densities in particle order ride through the sort as a 32-bit stream */
    unsigned int *dh = reinterpret_cast<unsigned int *>(c->pres);
    float *ds = reinterpret_cast<float *>(c->dens);
    FSPH_CUDA(c, cudaMemcpyAsync(dh, dens, (size_t)n * 4, cudaMemcpyHostToDevice, s));
    enqueue_sort(c, p, c->set[0].pos, s);
    Gather g{};
    g.n4 = 3; g.n1 = 3;
    g.src4[0] = c->set[0].pos; g.dst4[0] = c->set[1].pos;
    g.src4[1] = c->set[0].pos; g.dst4[1] = c->xb;
    g.src4[2] = c->set[0].vel; g.dst4[2] = c->set[1].vel;
    g.src1[0] = c->set[0].id; g.dst1[0] = c->set[1].id;
    g.src1[1] = c->key; g.dst1[1] = c->nl.cellb;
    g.src1[2] = dh; g.dst1[2] = reinterpret_cast<unsigned int *>(ds);
    launch_gather(n, c->perm, g, nullptr, s);
    launch_build_list(p, c->cell_start, c->xb, c->nl, s);
    /* the end-of-step passes of a PBF step, on these inputs */
    launch_xsph_vort(p, c->cell_start, c->set[1].pos, c->set[1].vel, ds, c->acc, c->vort, FeatureOut{}, c->nl, s);
    launch_vort_apply(p, c->cell_start, c->set[1].pos, c->vort, ds, c->acc, c->tmp4, c->nl, s);
    FSPH_TRY(check_launch(c));
    launch_unsort4(n, c->set[1].id, c->tmp4, c->ppos[0], 1, s);
    launch_unsort4(n, c->set[1].id, c->vort, c->ppos[1], 1, s);
    FSPH_CUDA(c, cudaMemcpyAsync(vel_out4, c->ppos[0], (size_t)n * 16, cudaMemcpyDeviceToHost, s));
    FSPH_CUDA(c, cudaMemcpyAsync(vort4, c->ppos[1], (size_t)n * 16, cudaMemcpyDeviceToHost, s));
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    FSPH_TRY(check_launch(c));
    /* the context's particles are left at the given positions and velocities */
    FSPH_TRY(fsph_set_particles(c, pos4, vel4, n, FSPH_HOST));
    return FSPH_OK;
}

int fsph_sph_eval_forces(fsph_ctx *c, const float *pos4, const float *vel4, int n, float *dens, float *pres,
                         float *acc4) {
    if (!c || !pos4 || !dens || !pres || !acc4) return FSPH_INVALID_ARG;
    FSPH_USABLE(c);
    FSPH_TRY(fsph_set_particles(c, pos4, vel4, n, FSPH_HOST));
    if (n == 0) return FSPH_OK;
    DevParams p = dev_for(c, n, 1.0f);
    cudaStream_t s = c->stream;
    enqueue_sort(c, p, c->set[0].pos, s);
    Gather g{};
    g.n4 = 2; g.n1 = 1;
    g.src4[0] = c->set[0].pos; g.dst4[0] = c->set[1].pos;
    g.src4[1] = c->set[0].vel; g.dst4[1] = c->set[1].vel;
    g.src1[0] = c->set[0].id; g.dst1[0] = c->set[1].id;
    launch_gather(n, c->perm, g, nullptr, s);
    launch_sph_density(p, c->cell_start, c->set[1].pos, c->set[1].vel, c->dens, c->pres, c->nl, s);
    launch_sph_force(p, c->cell_start, c->set[1].pos, c->set[1].vel, c->acc, c->nl, s);
    FSPH_TRY(check_launch(c));
    FSPH_TRY(copy_out_scalar(c, c->dens, c->set[1].id, dens, n));
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    FSPH_TRY(copy_out_scalar(c, c->pres, c->set[1].id, pres, n));
    launch_unsort4(n, c->set[1].id, c->acc, c->set[0].vel, 1, s);
    FSPH_CUDA(c, cudaMemcpyAsync(acc4, c->set[0].vel, (size_t)n * 16, cudaMemcpyDeviceToHost, s));
    FSPH_CUDA(c, cudaStreamSynchronize(s));
    FSPH_TRY(fsph_set_particles(c, pos4, vel4, n, FSPH_HOST));
    return FSPH_OK;
}

}  // extern "C"

/* Parameter builders shared with the allocation-free entry point
 * (fsph_noalloc.cu) and the batched scenes (fsph_batch.cu). */
namespace fsph {
DevParams dev_params_for(const fsph_params &p, int n, float dt) { return make_dev(p, n, dt); }
int validate_params(const fsph_params &p, std::string &why) { return validate(p, why); }
void grid_dims_for(const fsph_params &p, int g[3]) {
    double cw, org[3];
    grid_geometry(p, cw, org, g);
}
unsigned long long grid_cells_for(const fsph_params &p) {
    double cw, org[3];
    int g[3];
    grid_geometry(p, cw, org, g);
    return (unsigned long long)g[0] * (unsigned long long)g[1] * (unsigned long long)g[2];
}
}  // namespace fsph
