/*
 * fsph_batch.cu -- many independent PBF scenes advanced together
 * (fsph_batch_* in include/fsph.h).
 *
 * Layout: the scenes' particles are packed back to back in one set of
 * arrays; each scene has its own padded dense grid (cell width h_s (1 +
 * skin)), and the grids are concatenated in one cell table (DevParams::
 * cell_off).  One counting sort over the global cell keys therefore sorts
 * every scene at once and keeps the scenes contiguous and in order, so a
 * scene always owns the slots [off_s, off_s + N_s).
 *
 * Work: a tile is a run of consecutive slots of ONE scene; each pass is one
 * persistent launch (grid = resident blocks x SMs, capped by the tile count)
 * whose blocks walk the tile table, load the tile's scene constants into
 * shared memory and run the same per-particle bodies as the single-scene
 * kernels (fsph_passes.cuh).  A step (prediction, grid build, `iterations`
 * lambda / correction pairs with in-loop grid rebuilds, finalize, XSPH,
 * vorticity) is one CUDA graph with a device-side while loop.
 *
 * Tunables (fsph_batch_config, chosen by fsph_batch_autotune): threads per
 * block, lanes per particle in the constraint passes, and the cell skin.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fsph.h"
#include "fsph_kernels.cuh"
#include "fsph_passes.cuh"

namespace fsph {

DevParams dev_params_for(const fsph_params &p, int n, float dt);
int validate_params(const fsph_params &p, std::string &why);
void grid_dims_for(const fsph_params &p, int g[3]);

/* a run of consecutive slots of one scene */
struct BTile {
    int scene, start, count, pad;
};
struct BatchArgs {
    const DevParams *scenes;
    const BTile *tiles;
    int ntiles;
};

/* The tile's scene constants into shared memory (every thread calls it). */
__device__ __forceinline__ BTile tile_begin(const BatchArgs &b, int t, DevParams &s_p) {
    const BTile tl = b.tiles[t];
    __syncthreads(); /* the previous tile is done with s_p */
    if (threadIdx.x == 0) s_p = b.scenes[tl.scene];
    __syncthreads();
    return tl;
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) kb_predict_hash(BatchArgs b, const float4 *__restrict__ pos,
                                                         const float4 *__restrict__ vel, float4 *__restrict__ ppos_out,
                                                         unsigned int *__restrict__ key, unsigned int *__restrict__ rank,
                                                         unsigned int *__restrict__ count) {
    __shared__ DevParams s_p;
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        const BTile tl = tile_begin(b, t, s_p);
        const DevParams p = s_p;
        if ((int)threadIdx.x < tl.count)
            predict_body(p, tl.start + threadIdx.x, pos, vel, nullptr, ppos_out, key, rank, count, nullptr, nullptr);
    }
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) kb_hash_parity(BatchArgs b, const float4 *ppos0, const float4 *ppos1,
                                                        const DevCtl *ctl, unsigned int *__restrict__ key,
                                                        unsigned int *__restrict__ rank,
                                                        unsigned int *__restrict__ count) {
    __shared__ DevParams s_p;
    const float4 *x4 = ctl->parity ? ppos1 : ppos0;
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        const BTile tl = tile_begin(b, t, s_p);
        const DevParams p = s_p;
        if ((int)threadIdx.x < tl.count) {
            const int i = tl.start + threadIdx.x;
            hash_body(p, i, f3(x4[i]), key, rank, count);
        }
    }
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) kb_build_list(BatchArgs b, const unsigned int *__restrict__ cell_start,
                                                       const float4 *__restrict__ xb,
                                                       const unsigned int *__restrict__ cellb,
                                                       ListEntry *__restrict__ list,
                                                       unsigned char *__restrict__ cnt) {
    __shared__ DevParams s_p;
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        const BTile tl = tile_begin(b, t, s_p);
        const DevParams p = s_p;
        if ((int)threadIdx.x < tl.count) build_list_body(p, tl.start + threadIdx.x, cell_start, xb, cellb, list, cnt);
    }
}

/* lambda pass over all scenes; lp holds the loop constants (n = all
 * particles, min_iter = max_iter = the fixed iteration count). */
template <int BLOCK, int LPP>
__global__ void __launch_bounds__(BLOCK, FSPH_PASS_THREADS / BLOCK)
    kb_lambda(BatchArgs b, DevParams lp, const unsigned int *__restrict__ cell_start,
                                                   float4 *ppos0, float4 *ppos1, float *__restrict__ dens, DevCtl *ctl,
                                                   ErrPartial *part, cudaGraphConditionalHandle hwhile, int use_graph,
                                                   const ListEntry *__restrict__ list,
                                                   const unsigned char *__restrict__ cnt,
                                                   const unsigned int *__restrict__ cellb) {
    __shared__ DevParams s_p;
    __shared__ unsigned int s_rs[9 * BLOCK];
    const unsigned int par = *((volatile unsigned int *)&ctl->parity);
    float4 *pp = par ? ppos1 : ppos0;
    float e1 = 0.f, e2 = 0.f, em = 0.f;
    const int li = threadIdx.x / LPP, sub = threadIdx.x % LPP;
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        const BTile tl = tile_begin(b, t, s_p);
        const DevParams p = s_p;
        const bool valid = li < tl.count;
        const int i = tl.start + (valid ? li : 0);
        const float C = lambda_body<LPP>(p, cell_start, pp, dens, ctl, list, cnt, cellb, s_rs + threadIdx.x, i, sub,
                                         valid);
        if (valid && sub == 0) {
            e1 += C > 0.0f ? C : 0.0f;
            e2 += fabsf(C);
            em = fmaxf(em, fabsf(C));
        }
    }
    lambda_tail(lp, ctl, part, e1, e2, em, hwhile, use_graph);
}

/* correction pass over all scenes; the rebuild measure is the largest
 * |x* - xb|^2 / skin2 of the particle's own scene (lp.skin2 = 1). */
template <int BLOCK, int LPP>
__global__ void __launch_bounds__(BLOCK, FSPH_PASS_THREADS / BLOCK) kb_correction(BatchArgs b, DevParams lp,
                                                       const unsigned int *__restrict__ cell_start, float4 *ppos0,
                                                       float4 *ppos1, const float4 *__restrict__ xb, DevCtl *ctl,
                                                       float *part, cudaGraphConditionalHandle hif,
                                                       cudaGraphConditionalHandle hif2, int use_graph,
                                                       const ListEntry *__restrict__ list,
                                                       const unsigned char *__restrict__ cnt,
                                                       const unsigned int *__restrict__ cellb) {
    __shared__ DevParams s_p;
    __shared__ unsigned int s_rs[9 * BLOCK];
    const unsigned int par = *((volatile unsigned int *)&ctl->parity);
    const float4 *__restrict__ src = par ? ppos1 : ppos0;
    float4 *__restrict__ dst = par ? ppos0 : ppos1;
    float worst = 0.f;
    const int li = threadIdx.x / LPP, sub = threadIdx.x % LPP;
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        const BTile tl = tile_begin(b, t, s_p);
        const DevParams p = s_p;
        const bool valid = li < tl.count;
        const int i = tl.start + (valid ? li : 0);
        const float d2 = correction_body<LPP>(p, cell_start, src, dst, xb, ctl, nullptr, list, cnt, cellb,
                                              s_rs + threadIdx.x, i, sub, valid);
        worst = fmaxf(worst, d2 / p.skin2);
    }
    correction_tail(lp, ctl, part, worst, par, hif, hif2, use_graph);
}

/* m / rho_i of every particle with its scene's mass, for the XSPH and
 * vorticity passes (FSPH_POST_PRE) */
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) kb_mrho(BatchArgs b, const float *__restrict__ dens,
                                                 float *__restrict__ mrho) {
    __shared__ DevParams s_p;
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        const BTile tl = tile_begin(b, t, s_p);
        if ((int)threadIdx.x < tl.count) mrho[tl.start + threadIdx.x] = s_p.mass / dens[tl.start + threadIdx.x];
    }
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) kb_xsph_vort(BatchArgs b, const unsigned int *__restrict__ cell_start,
                                                      const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                                                      const float *__restrict__ dens, float4 *__restrict__ vel_out,
                                                      float4 *__restrict__ vort,
                                                      const ListEntry *__restrict__ list,
                                                      const unsigned char *__restrict__ cnt,
                                                      const unsigned int *__restrict__ cellb,
                                                      const float *__restrict__ mrho, float2 *__restrict__ wm) {
    __shared__ DevParams s_p;
    __shared__ unsigned int s_rs[9 * BLOCK];
    const FeatureOut fo{};
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        const BTile tl = tile_begin(b, t, s_p);
        const DevParams p = s_p;
        if ((int)threadIdx.x < tl.count)
            xsph_vort_body<false, FSPH_POST_PRE != 0>(p, tl.start + threadIdx.x, cell_start, pos, vel, dens, vel_out,
                                                      vort, fo, list, cnt, cellb, s_rs + threadIdx.x, mrho, wm);
    }
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) kb_vort_apply(BatchArgs b, const unsigned int *__restrict__ cell_start,
                                                       const float4 *__restrict__ pos, const float4 *__restrict__ vort,
                                                       const float *__restrict__ dens,
                                                       const float4 *__restrict__ vel_in, float4 *__restrict__ vel_out,
                                                       const ListEntry *__restrict__ list,
                                                       const unsigned char *__restrict__ cnt,
                                                       const unsigned int *__restrict__ cellb,
                                                       const float2 *__restrict__ wm) {
    __shared__ DevParams s_p;
    __shared__ unsigned int s_rs[9 * BLOCK];
    for (int t = blockIdx.x; t < b.ntiles; t += gridDim.x) {
        const BTile tl = tile_begin(b, t, s_p);
        const DevParams p = s_p;
        if ((int)threadIdx.x < tl.count)
            vort_apply_body<FSPH_POST_PRE != 0>(p, tl.start + threadIdx.x, cell_start, pos, vort, dens, vel_in,
                                                vel_out, list, cnt, cellb, s_rs + threadIdx.x, wm);
    }
}

/* Per-scene density errors of the last lambda pass, one block per scene,
 * fixed-order: err[3 s + 0..2] = one-sided mean, two-sided mean, max. */
__global__ void __launch_bounds__(256) kb_scene_errors(const int *__restrict__ offs, const DevParams *__restrict__ scenes,
                                                       const float *__restrict__ dens, float *__restrict__ err) {
    __shared__ double s1[8], s2[8];
    __shared__ float sm[8];
    const int s = blockIdx.x;
    const int a = offs[s], e = offs[s + 1];
    const float inv = scenes[s].inv_rest_dens;
    double e1 = 0.0, e2 = 0.0;
    float m = 0.f;
    for (int i = a + (int)threadIdx.x; i < e; i += blockDim.x) {
        const float C = dens[i] * inv - 1.0f;
        e1 += C > 0.0f ? C : 0.0f;
        e2 += fabsf(C);
        m = fmaxf(m, fabsf(C));
    }
    for (int o = 16; o > 0; o >>= 1) {
        e1 += __shfl_xor_sync(0xffffffffu, e1, o);
        e2 += __shfl_xor_sync(0xffffffffu, e2, o);
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { s1[warp] = e1; s2[warp] = e2; sm[warp] = m; }
    __syncthreads();
    if (threadIdx.x == 0) {
        e1 = 0.0; e2 = 0.0; m = 0.f;
        for (int w = 0; w < 8; ++w) { e1 += s1[w]; e2 += s2[w]; m = fmaxf(m, sm[w]); }
        const double n = (double)(e > a ? e - a : 1);
        err[3 * s + 0] = (float)(e1 / n);
        err[3 * s + 1] = (float)(e2 / n);
        err[3 * s + 2] = m;
    }
}

/* ---------------- launch dispatch over the tunables ---------------- */

/* persistent grid: resident blocks per SM x SMs, capped by the tiles */
template <class K>
unsigned int persistent_grid(K kernel, int block, int ntiles, int sms) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    return (unsigned int)std::max(1, std::min(ntiles, per_sm * sms));
}

struct BLaunch {
    BatchArgs full, cons;  /* tiles of `block` slots; tiles of block / lanes slots (constraint passes) */
    int block, lanes, sms;
};

#define FSPH_BLOCK_SWITCH(BLK, ...)                                  \
    switch (BLK) {                                                   \
    case 128: { constexpr int B_ = 128; __VA_ARGS__; } break;       \
    case 512: { constexpr int B_ = 512; __VA_ARGS__; } break;       \
    default: { constexpr int B_ = 256; __VA_ARGS__; } break;        \
    }
#define FSPH_LANES_SWITCH(LN, ...)                                   \
    switch (LN) {                                                    \
    case 2: { constexpr int L_ = 2; __VA_ARGS__; } break;           \
    case 4: { constexpr int L_ = 4; __VA_ARGS__; } break;           \
    default: { constexpr int L_ = 1; __VA_ARGS__; } break;          \
    }

void blaunch_predict_hash(const BLaunch &L, const float4 *pos, const float4 *vel, float4 *ppos_out,
                          unsigned int *key, unsigned int *rank, unsigned int *count, cudaStream_t s) {
    FSPH_BLOCK_SWITCH(L.block, {
        auto k = kb_predict_hash<B_>;
        k<<<persistent_grid(k, B_, L.full.ntiles, L.sms), B_, 0, s>>>(L.full, pos, vel, ppos_out, key, rank, count);
    })
}
void blaunch_hash_parity(const BLaunch &L, const float4 *p0, const float4 *p1, const DevCtl *ctl, unsigned int *key,
                         unsigned int *rank, unsigned int *count, cudaStream_t s) {
    FSPH_BLOCK_SWITCH(L.block, {
        auto k = kb_hash_parity<B_>;
        k<<<persistent_grid(k, B_, L.full.ntiles, L.sms), B_, 0, s>>>(L.full, p0, p1, ctl, key, rank, count);
    })
}
void blaunch_build_list(const BLaunch &L, const unsigned int *cell_start, const float4 *xb, const NbrLists &nl,
                        cudaStream_t s) {
    FSPH_BLOCK_SWITCH(L.block, {
        auto k = kb_build_list<B_>;
        k<<<persistent_grid(k, B_, L.full.ntiles, L.sms), B_, 0, s>>>(L.full, cell_start, xb, nl.cellb, nl.list,
                                                                       nl.cnt);
    })
}
unsigned int blaunch_lambda(const BLaunch &L, const DevParams &lp, const unsigned int *cell_start, float4 *p0,
                            float4 *p1, float *dens, DevCtl *ctl, ErrPartial *part, unsigned long long hw,
                            int use_graph, const NbrLists &nl, cudaStream_t s) {
    unsigned int g = 0;
    FSPH_BLOCK_SWITCH(L.block, FSPH_LANES_SWITCH(L.lanes, {
        auto k = kb_lambda<B_, L_>;
        g = persistent_grid(k, B_, L.cons.ntiles, L.sms);
        k<<<g, B_, 0, s>>>(L.cons, lp, cell_start, p0, p1, dens, ctl, part, hw, use_graph, nl.list, nl.cnt, nl.cellb);
    }))
    return g;
}
unsigned int blaunch_correction(const BLaunch &L, const DevParams &lp, const unsigned int *cell_start, float4 *p0,
                                float4 *p1, const float4 *xb, DevCtl *ctl, float *part, unsigned long long hif,
                                unsigned long long hif2, int use_graph, const NbrLists &nl, cudaStream_t s) {
    unsigned int g = 0;
    FSPH_BLOCK_SWITCH(L.block, FSPH_LANES_SWITCH(L.lanes, {
        auto k = kb_correction<B_, L_>;
        g = persistent_grid(k, B_, L.cons.ntiles, L.sms);
        k<<<g, B_, 0, s>>>(L.cons, lp, cell_start, p0, p1, xb, ctl, part, hif, hif2, use_graph, nl.list, nl.cnt,
                           nl.cellb);
    }))
    return g;
}
void blaunch_xsph_vort(const BLaunch &L, const unsigned int *cell_start, const float4 *pos, const float4 *vel,
                       const float *dens, float4 *vel_out, float4 *vort, const NbrLists &nl, cudaStream_t s,
                       float *mrho, float2 *wm) {
    FSPH_BLOCK_SWITCH(L.block, {
        if (FSPH_POST_PRE) {
            auto km = kb_mrho<B_>;
            km<<<persistent_grid(km, B_, L.full.ntiles, L.sms), B_, 0, s>>>(L.full, dens, mrho);
        }
        auto k = kb_xsph_vort<B_>;
        k<<<persistent_grid(k, B_, L.full.ntiles, L.sms), B_, 0, s>>>(L.full, cell_start, pos, vel, dens, vel_out, vort,
                                                                       nl.list, nl.cnt, nl.cellb, mrho, wm);
    })
}
void blaunch_vort_apply(const BLaunch &L, const unsigned int *cell_start, const float4 *pos, const float4 *vort,
                        const float *dens, const float4 *vel_in, float4 *vel_out, const NbrLists &nl, cudaStream_t s,
                        const float2 *wm) {
    FSPH_BLOCK_SWITCH(L.block, {
        auto k = kb_vort_apply<B_>;
        k<<<persistent_grid(k, B_, L.full.ntiles, L.sms), B_, 0, s>>>(L.full, cell_start, pos, vort, dens, vel_in,
                                                                       vel_out, nl.list, nl.cnt, nl.cellb, wm);
    })
}

}  // namespace fsph

/* ======================================================================== */
/* host side                                                                */
/* ======================================================================== */
using namespace fsph;

struct fsph_batch {
    int nscenes = 0, n = 0, iters = 4;
    std::vector<fsph_params> P;
    std::vector<int> counts, offs;
    fsph_batch_config cfg{256, 1, 0.05f, 0};
    int sms = 1;
    cudaStream_t stream = nullptr, s2 = nullptr, s3 = nullptr;
    /* particles: set 0 = home (step start / end), set 1 = through the iterations */
    float4 *pos[2] = {nullptr, nullptr}, *vel[2] = {nullptr, nullptr};
    unsigned int *id[2] = {nullptr, nullptr}, *attr[2] = {nullptr, nullptr};
    float4 *ppos[2] = {nullptr, nullptr};
    float4 *xb = nullptr, *vort = nullptr, *tmp4 = nullptr;
    float *dens = nullptr, *tdens = nullptr;
    float *mrho = nullptr;  /* m / rho per particle (XSPH and vorticity passes) */
    float2 *wm = nullptr;   /* (|omega|, m / rho) per particle */
    unsigned int *key = nullptr, *rank = nullptr, *perm = nullptr;
    NbrLists nl;
    /* grid */
    unsigned int *count = nullptr, *cell_start = nullptr, *block_sums = nullptr;
    unsigned int ncells = 0, cap_cells = 0;
    /* scenes and tiles of the current configuration */
    DevParams *d_scenes = nullptr;
    int *d_offs = nullptr;
    BTile *d_tiles_full = nullptr, *d_tiles_cons = nullptr;
    int nt_full = 0, nt_cons = 0, cap_tiles_full = 0, cap_tiles_cons = 0;
    DevCtl *ctl = nullptr, *ctl_host = nullptr;
    ErrPartial *epart = nullptr;
    float *dpart = nullptr;
    int cap_part = 0;
    float *d_err = nullptr, *h_err = nullptr;
    /* step graph */
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    bool graph_valid = false;
    float graph_dt = 0.0f;
    bool loaded = false;
    std::string err;
};

namespace {

#define FB_CUDA(b, call)                                                             \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            (b)->err = std::string(#call) + ": " + cudaGetErrorString(e_);           \
            return e_ == cudaErrorMemoryAllocation ? FSPH_OOM : FSPH_CUDA_ERROR;     \
        }                                                                            \
    } while (0)
#define FB_TRY(expr)                     \
    do {                                 \
        int st_ = (expr);                \
        if (st_ != FSPH_OK) return st_;  \
    } while (0)

int bfail(fsph_batch *b, int st, const std::string &m) {
    if (b) b->err = m;
    return st;
}

template <class T>
int balloc(fsph_batch *b, T **p, size_t count) {
    *p = nullptr;
    FB_CUDA(b, cudaMalloc((void **)p, std::max<size_t>(count, 1) * sizeof(T)));
    return FSPH_OK;
}

void bdrop_graph(fsph_batch *b) {
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->gexec = nullptr;
    b->graph = nullptr;
    b->graph_valid = false;
}

void bfree(fsph_batch *b) {
    for (int k = 0; k < 2; ++k) {
        cudaFree(b->pos[k]); cudaFree(b->vel[k]); cudaFree(b->id[k]); cudaFree(b->attr[k]); cudaFree(b->ppos[k]);
    }
    cudaFree(b->xb); cudaFree(b->vort); cudaFree(b->tmp4); cudaFree(b->dens); cudaFree(b->tdens);
    cudaFree(b->mrho); cudaFree(b->wm);
    cudaFree(b->key); cudaFree(b->rank); cudaFree(b->perm);
    cudaFree(b->nl.list); cudaFree(b->nl.cnt); cudaFree(b->nl.cellb);
    cudaFree(b->count); cudaFree(b->cell_start); cudaFree(b->block_sums);
    cudaFree(b->d_scenes); cudaFree(b->d_offs); cudaFree(b->d_tiles_full); cudaFree(b->d_tiles_cons);
    cudaFree(b->ctl); cudaFree(b->epart); cudaFree(b->dpart); cudaFree(b->d_err);
    if (b->ctl_host) cudaFreeHost(b->ctl_host);
    if (b->h_err) cudaFreeHost(b->h_err);
}

/* tiles of `per` consecutive slots, never straddling a scene */
std::vector<BTile> make_tiles(const fsph_batch *b, int per) {
    std::vector<BTile> t;
    for (int s = 0; s < b->nscenes; ++s)
        for (int a = 0; a < b->counts[s]; a += per) t.push_back(BTile{s, b->offs[s] + a, std::min(per, b->counts[s] - a), 0});
    return t;
}

/* Scene constants, cell table and tiles for cfg; the step graph is rebuilt
 * at the next step. */
int apply_config(fsph_batch *b, const fsph_batch_config &cfg, float dt) {
    if (cfg.block != 128 && cfg.block != 256 && cfg.block != 512) return bfail(b, FSPH_INVALID_ARG, "block must be 128, 256 or 512");
    if (cfg.lanes != 1 && cfg.lanes != 2 && cfg.lanes != 4) return bfail(b, FSPH_INVALID_ARG, "lanes must be 1, 2 or 4");
    if (!(cfg.cell_skin >= 0.02f && cfg.cell_skin <= 0.5f)) return bfail(b, FSPH_INVALID_ARG, "cell_skin must lie in [0.02, 0.5]");
    FB_CUDA(b, cudaStreamSynchronize(b->stream));
    std::vector<DevParams> h(b->nscenes);
    unsigned long long cells = 0;
    for (int s = 0; s < b->nscenes; ++s) {
        fsph_params q = b->P[s];
        q.cell_skin = cfg.cell_skin;
        q.walk_cells = 0;
        h[s] = dev_params_for(q, b->n, dt);
        h[s].cell_off = (unsigned int)cells;
        h[s].dbg = &b->ctl->bounds_bits;
        cells += (unsigned long long)h[s].gx * h[s].gy * h[s].gz;
    }
    if (cells > (1ull << 30)) return bfail(b, FSPH_INVALID_ARG, "the scenes' grids exceed 2^30 cells");
    const unsigned int nc = (unsigned int)cells;
    if (nc > b->cap_cells) {
        cudaFree(b->count); cudaFree(b->cell_start); cudaFree(b->block_sums);
        b->count = b->cell_start = b->block_sums = nullptr;
        FB_TRY(balloc(b, &b->count, nc));
        FB_TRY(balloc(b, &b->cell_start, (size_t)nc + 1));
        FB_TRY(balloc(b, &b->block_sums, scan_blocks(nc)));
        b->cap_cells = nc;
    }
    FB_CUDA(b, cudaMemsetAsync(b->count, 0, (size_t)nc * sizeof(unsigned int), b->stream));
    b->ncells = nc;
    FB_CUDA(b, cudaMemcpyAsync(b->d_scenes, h.data(), h.size() * sizeof(DevParams), cudaMemcpyHostToDevice, b->stream));
    std::vector<BTile> tf = make_tiles(b, cfg.block), tc = make_tiles(b, cfg.block / cfg.lanes);
    if ((int)tf.size() > b->cap_tiles_full) {
        cudaFree(b->d_tiles_full);
        FB_TRY(balloc(b, &b->d_tiles_full, tf.size()));
        b->cap_tiles_full = (int)tf.size();
    }
    if ((int)tc.size() > b->cap_tiles_cons) {
        cudaFree(b->d_tiles_cons);
        FB_TRY(balloc(b, &b->d_tiles_cons, tc.size()));
        b->cap_tiles_cons = (int)tc.size();
    }
    FB_CUDA(b, cudaMemcpyAsync(b->d_tiles_full, tf.data(), tf.size() * sizeof(BTile), cudaMemcpyHostToDevice, b->stream));
    FB_CUDA(b, cudaMemcpyAsync(b->d_tiles_cons, tc.data(), tc.size() * sizeof(BTile), cudaMemcpyHostToDevice, b->stream));
    b->nt_full = (int)tf.size();
    b->nt_cons = (int)tc.size();
    /* block partials: one per block of the largest persistent launch */
    const int need = std::max(b->nt_full, b->nt_cons);
    if (need > b->cap_part) {
        cudaFree(b->epart); cudaFree(b->dpart);
        b->epart = nullptr; b->dpart = nullptr;
        FB_TRY(balloc(b, &b->epart, need));
        FB_TRY(balloc(b, &b->dpart, need));
        b->cap_part = need;
    }
    FB_CUDA(b, cudaStreamSynchronize(b->stream));
    b->cfg = cfg;
    bdrop_graph(b);
    return FSPH_OK;
}

BLaunch launch_of(const fsph_batch *b) {
    BLaunch L;
    L.full = BatchArgs{b->d_scenes, b->d_tiles_full, b->nt_full};
    L.cons = BatchArgs{b->d_scenes, b->d_tiles_cons, b->nt_cons};
    L.block = b->cfg.block;
    L.lanes = b->cfg.lanes;
    L.sms = b->sms;
    return L;
}

/* loop constants: every scene runs exactly `iters` iterations */
DevParams loop_params(const fsph_batch *b, float dt) {
    DevParams lp{};
    lp.n = b->n;
    lp.dbg = &b->ctl->bounds_bits;
    lp.min_iter = b->iters;
    lp.max_iter = b->iters;
    lp.eta = -1.0f;
    lp.error_mode = FSPH_ERR_ONE_SIDED;
    lp.skin2 = 1.0f; /* the correction pass reduces |x* - xb|^2 / skin2 of each scene */
    lp.dt = dt;
    lp.inv_dt = 1.0f / dt;
    return lp;
}

void benqueue_sort_tail(fsph_batch *b, cudaStream_t s) {
    launch_scan(b->count, b->cell_start, b->block_sums, b->ncells, s);
    DevParams q{};
    q.n = b->n;
    launch_scatter_sort(q, b->key, b->rank, b->cell_start, b->perm, b->ncells, s);
}

/* in-loop / post-loop rebuild: re-sort every scene on the current x* */
void benqueue_rebuild(fsph_batch *b, const BLaunch &L, cudaStream_t s) {
    blaunch_hash_parity(L, b->ppos[0], b->ppos[1], b->ctl, b->key, b->rank, b->count, s);
    benqueue_sort_tail(b, s);
    float *t_lam = reinterpret_cast<float *>(b->rank); /* free once the scatter has run */
    launch_rebuild_gather(b->n, b->perm, b->ctl, b->pos[1], b->ppos[0], b->ppos[1], b->id[1], b->attr[1], b->dens,
                          b->pos[0], b->vel[0], b->id[0], b->attr[0], b->tdens, b->key, b->nl.cellb, nullptr, nullptr,
                          t_lam, s);
    launch_rebuild_copy(b->n, b->ctl, b->pos[0], b->vel[0], b->id[0], b->attr[0], b->tdens, b->pos[1], b->ppos[0],
                        b->ppos[1], b->xb, b->id[1], b->attr[1], b->dens, nullptr, nullptr, t_lam, s);
    blaunch_build_list(L, b->cell_start, b->xb, b->nl, s);
}

void benqueue_pre(fsph_batch *b, const BLaunch &L, cudaStream_t s) {
    cudaMemsetAsync(b->ctl, 0, sizeof(DevCtl), s);
    blaunch_predict_hash(L, b->pos[0], b->vel[0], b->ppos[1], b->key, b->rank, b->count, s);
    benqueue_sort_tail(b, s);
    Gather g{};
    g.n4 = 3; g.n1 = 3;
    g.src4[0] = b->pos[0]; g.dst4[0] = b->pos[1];
    g.src4[1] = b->ppos[1]; g.dst4[1] = b->ppos[0];
    g.src4[2] = b->ppos[1]; g.dst4[2] = b->xb;
    g.src1[0] = b->id[0]; g.dst1[0] = b->id[1];
    g.src1[1] = b->attr[0]; g.dst1[1] = b->attr[1];
    g.src1[2] = b->key; g.dst1[2] = b->nl.cellb;
    launch_gather(b->n, b->perm, g, b->ctl, s);
    blaunch_build_list(L, b->cell_start, b->xb, b->nl, s);
}

void benqueue_post(fsph_batch *b, const BLaunch &L, const DevParams &lp, cudaStream_t s) {
    launch_finalize(lp, b->pos[1], b->ppos[0], b->ppos[1], b->ctl, b->id[1], b->attr[1], b->pos[0], b->vel[0],
                    b->id[0], b->attr[0], nullptr, nullptr, s);
    blaunch_xsph_vort(L, b->cell_start, b->pos[0], b->vel[0], b->dens, b->vel[1], b->vort, b->nl, s, b->mrho, b->wm);
    blaunch_vort_apply(L, b->cell_start, b->pos[0], b->vort, b->dens, b->vel[1], b->vel[0], b->nl, s, b->wm);
    kb_scene_errors<<<b->nscenes, 256, 0, s>>>(b->d_offs, b->d_scenes, b->dens, b->d_err);
}

int badd_conditional(fsph_batch *b, cudaGraph_t g, const cudaGraphNode_t *deps, size_t ndeps,
                     cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type, cudaGraphNode_t *node,
                     cudaGraph_t *body) {
    alignas(cudaGraphNodeParams) unsigned char raw[sizeof(cudaGraphNodeParams)];
    std::memset(raw, 0, sizeof(raw));
    cudaGraphNodeParams *cp = reinterpret_cast<cudaGraphNodeParams *>(raw);
    cp->type = cudaGraphNodeTypeConditional;
    cp->conditional.handle = h;
    cp->conditional.type = type;
    cp->conditional.size = 1;
    FB_CUDA(b, cudaGraphAddNode(node, g, deps, nullptr, ndeps, cp));
    *body = cp->conditional.phGraph_out[0];
    return FSPH_OK;
}

/* pre -> WHILE{ IF(rebuild){rebuild}; lambda; correction } -> IF(rebuild){rebuild} -> post */
int bbuild_graph(fsph_batch *b, float dt) {
    bdrop_graph(b);
    const BLaunch L = launch_of(b);
    const DevParams lp = loop_params(b, dt);
    cudaStream_t s = b->stream;
    cudaGraph_t g;
    FB_CUDA(b, cudaGraphCreate(&g, 0));
    b->graph = g;
    FB_CUDA(b, cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    benqueue_pre(b, L, s);
    cudaStreamCaptureStatus st;
    cudaGraph_t capg;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    FB_CUDA(b, cudaStreamGetCaptureInfo(s, &st, nullptr, &capg, &deps, nullptr, &ndeps));
    cudaGraphConditionalHandle hw, hrb, hrb2;
    FB_CUDA(b, cudaGraphConditionalHandleCreate(&hw, capg, 1, cudaGraphCondAssignDefault));
    cudaGraphNode_t wnode, inode, pnode;
    cudaGraph_t wbody, ibody, pbody;
    std::vector<cudaGraphNode_t> dv(deps, deps + ndeps);
    FB_TRY(badd_conditional(b, capg, dv.data(), dv.size(), hw, cudaGraphCondTypeWhile, &wnode, &wbody));
    FB_CUDA(b, cudaGraphConditionalHandleCreate(&hrb, wbody, 0, cudaGraphCondAssignDefault));
    FB_TRY(badd_conditional(b, wbody, nullptr, 0, hrb, cudaGraphCondTypeIf, &inode, &ibody));
    FB_CUDA(b, cudaStreamBeginCaptureToGraph(b->s3, ibody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    benqueue_rebuild(b, L, b->s3);
    FB_CUDA(b, cudaStreamEndCapture(b->s3, &ibody));
    FB_CUDA(b, cudaGraphConditionalHandleCreate(&hrb2, capg, 0, cudaGraphCondAssignDefault));
    FB_CUDA(b, cudaStreamBeginCaptureToGraph(b->s2, wbody, &inode, nullptr, 1, cudaStreamCaptureModeRelaxed));
    blaunch_lambda(L, lp, b->cell_start, b->ppos[0], b->ppos[1], b->dens, b->ctl, b->epart, hw, 1, b->nl, b->s2);
    blaunch_correction(L, lp, b->cell_start, b->ppos[0], b->ppos[1], b->xb, b->ctl, b->dpart, hrb, hrb2, 3, b->nl,
                       b->s2);
    FB_CUDA(b, cudaStreamEndCapture(b->s2, &wbody));
    FB_CUDA(b, cudaStreamUpdateCaptureDependencies(s, &wnode, nullptr, 1, cudaStreamSetCaptureDependencies));
    FB_TRY(badd_conditional(b, capg, &wnode, 1, hrb2, cudaGraphCondTypeIf, &pnode, &pbody));
    FB_CUDA(b, cudaStreamBeginCaptureToGraph(b->s3, pbody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    benqueue_rebuild(b, L, b->s3);
    FB_CUDA(b, cudaStreamEndCapture(b->s3, &pbody));
    FB_CUDA(b, cudaStreamUpdateCaptureDependencies(s, &pnode, nullptr, 1, cudaStreamSetCaptureDependencies));
    benqueue_post(b, L, lp, s);
    FB_CUDA(b, cudaStreamEndCapture(s, &g));
    FB_CUDA(b, cudaGraphInstantiate(&b->gexec, g, 0));
    b->graph_valid = true;
    b->graph_dt = dt;
    return FSPH_OK;
}

/* the same launches with the loop on the host (no conditional nodes, so
 * profilers can see every kernel) */
int bstep_eager(fsph_batch *b, float dt) {
    if (b->graph_dt != dt) {
        fsph_batch_config c = b->cfg;
        FB_TRY(apply_config(b, c, dt));
        b->graph_dt = dt;
    }
    const BLaunch L = launch_of(b);
    const DevParams lp = loop_params(b, dt);
    cudaStream_t s = b->stream;
    benqueue_pre(b, L, s);
    for (int k = 0;; ++k) {
        blaunch_lambda(L, lp, b->cell_start, b->ppos[0], b->ppos[1], b->dens, b->ctl, b->epart, 0ull, 0, b->nl, s);
        blaunch_correction(L, lp, b->cell_start, b->ppos[0], b->ppos[1], b->xb, b->ctl, b->dpart, 0ull, 0ull, 0,
                           b->nl, s);
        FB_CUDA(b, cudaMemcpyAsync(b->ctl_host, b->ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, s));
        FB_CUDA(b, cudaStreamSynchronize(s));
        if (b->ctl_host->rebuild) benqueue_rebuild(b, L, s);
        if (b->ctl_host->done || k > b->iters + 1) break;
    }
    benqueue_post(b, L, lp, s);
    return FSPH_OK;
}

int bstep(fsph_batch *b, float dt) {
    if (b->cfg.eager) {
        FB_TRY(bstep_eager(b, dt));
        FB_CUDA(b, cudaGetLastError());
        FB_CUDA(b, cudaMemcpyAsync(b->ctl_host, b->ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, b->stream));
        FB_CUDA(b, cudaMemcpyAsync(b->h_err, b->d_err, 3 * sizeof(float) * b->nscenes, cudaMemcpyDeviceToHost,
                                   b->stream));
        return FSPH_OK;
    }
    if (!b->graph_valid || b->graph_dt != dt) {
        fsph_batch_config c = b->cfg;
        FB_TRY(apply_config(b, c, dt));
        FB_TRY(bbuild_graph(b, dt));
    }
    FB_CUDA(b, cudaGraphLaunch(b->gexec, b->stream));
    FB_CUDA(b, cudaGetLastError());
    FB_CUDA(b, cudaMemcpyAsync(b->ctl_host, b->ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, b->stream));
    FB_CUDA(b, cudaMemcpyAsync(b->h_err, b->d_err, 3 * sizeof(float) * b->nscenes, cudaMemcpyDeviceToHost, b->stream));
    return FSPH_OK;
}

/* process-wide autotuner cache: scene-set signature -> configuration */
std::mutex g_tune_mu;
std::map<std::string, fsph_batch_config> g_tune_cache;

std::string signature(const fsph_batch *b, float dt) {
    std::string s(reinterpret_cast<const char *>(&dt), sizeof(dt));
    s.append(reinterpret_cast<const char *>(&b->iters), sizeof(int));
    s.append(reinterpret_cast<const char *>(b->counts.data()), b->counts.size() * sizeof(int));
    s.append(reinterpret_cast<const char *>(b->P.data()), b->P.size() * sizeof(fsph_params));
    return s;
}

/* home-state copies the autotuner restores after each trial */
struct Saved {
    float4 *pos = nullptr, *vel = nullptr;
    unsigned int *id = nullptr, *attr = nullptr;
    ~Saved() { cudaFree(pos); cudaFree(vel); cudaFree(id); cudaFree(attr); }
};

int save_state(fsph_batch *b, Saved &sv) {
    const size_t n = (size_t)b->n;
    FB_TRY(balloc(b, &sv.pos, n)); FB_TRY(balloc(b, &sv.vel, n));
    FB_TRY(balloc(b, &sv.id, n)); FB_TRY(balloc(b, &sv.attr, n));
    FB_CUDA(b, cudaMemcpyAsync(sv.pos, b->pos[0], n * 16, cudaMemcpyDeviceToDevice, b->stream));
    FB_CUDA(b, cudaMemcpyAsync(sv.vel, b->vel[0], n * 16, cudaMemcpyDeviceToDevice, b->stream));
    FB_CUDA(b, cudaMemcpyAsync(sv.id, b->id[0], n * 4, cudaMemcpyDeviceToDevice, b->stream));
    FB_CUDA(b, cudaMemcpyAsync(sv.attr, b->attr[0], n * 4, cudaMemcpyDeviceToDevice, b->stream));
    return FSPH_OK;
}

int restore_state(fsph_batch *b, const Saved &sv) {
    const size_t n = (size_t)b->n;
    FB_CUDA(b, cudaMemcpyAsync(b->pos[0], sv.pos, n * 16, cudaMemcpyDeviceToDevice, b->stream));
    FB_CUDA(b, cudaMemcpyAsync(b->vel[0], sv.vel, n * 16, cudaMemcpyDeviceToDevice, b->stream));
    FB_CUDA(b, cudaMemcpyAsync(b->id[0], sv.id, n * 4, cudaMemcpyDeviceToDevice, b->stream));
    FB_CUDA(b, cudaMemcpyAsync(b->attr[0], sv.attr, n * 4, cudaMemcpyDeviceToDevice, b->stream));
    return FSPH_OK;
}

}  // namespace

/* ======================================================================== */
/* C ABI                                                                    */
/* ======================================================================== */
extern "C" {

int fsph_batch_create(const fsph_params *params, const int *counts, int nscenes, int iterations, fsph_batch **out) {
    if (!params || !counts || !out || nscenes <= 0 || iterations < 1) return FSPH_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return FSPH_NO_DEVICE;
    }
    long long total = 0;
    for (int s = 0; s < nscenes; ++s) {
        std::string why;
        if (params[s].solver != FSPH_SOLVER_PBF) return FSPH_INVALID_ARG;
        if (validate_params(params[s], why) != FSPH_OK) return FSPH_INVALID_ARG;
        if (counts[s] < 0) return FSPH_INVALID_ARG;
        total += counts[s];
    }
    /* 32-bit slots and list entries: keep the batch well below 2^31 particles */
    if (total > (1ll << 30)) return FSPH_INVALID_ARG;
    fsph_batch *b = new (std::nothrow) fsph_batch();
    if (!b) return FSPH_OOM;
    auto bail = [&](int st) { fsph_batch_destroy(b); return st; };
    b->nscenes = nscenes;
    b->iters = iterations;
    b->P.assign(params, params + nscenes);
    b->counts.assign(counts, counts + nscenes);
    b->offs.assign(nscenes + 1, 0);
    for (int s = 0; s < nscenes; ++s) b->offs[s + 1] = b->offs[s] + counts[s];
    b->n = b->offs[nscenes];
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(FSPH_CUDA_ERROR);
    if (cudaStreamCreateWithFlags(&b->s2, cudaStreamNonBlocking) != cudaSuccess) return bail(FSPH_CUDA_ERROR);
    if (cudaStreamCreateWithFlags(&b->s3, cudaStreamNonBlocking) != cudaSuccess) return bail(FSPH_CUDA_ERROR);
    const size_t n = (size_t)std::max(b->n, 1);
    int st = FSPH_OK;
    auto A = [&](auto **p, size_t c) { if (st == FSPH_OK) st = balloc(b, p, c); };
    for (int k = 0; k < 2; ++k) {
        A(&b->pos[k], n); A(&b->vel[k], n); A(&b->id[k], n); A(&b->attr[k], n); A(&b->ppos[k], n);
    }
    A(&b->xb, n); A(&b->vort, n); A(&b->tmp4, n); A(&b->dens, n); A(&b->tdens, n);
    A(&b->mrho, n); A(&b->wm, n);
    A(&b->key, n); A(&b->rank, n); A(&b->perm, n);
    A(&b->nl.list, n * kListMax); A(&b->nl.cnt, n); A(&b->nl.cellb, n);
    A(&b->d_scenes, (size_t)nscenes); A(&b->d_offs, (size_t)nscenes + 1); A(&b->d_err, 3 * (size_t)nscenes);
    A(&b->ctl, 1);
    if (st != FSPH_OK) return bail(st);
    if (cudaMallocHost((void **)&b->ctl_host, sizeof(DevCtl)) != cudaSuccess) return bail(FSPH_OOM);
    if (cudaMallocHost((void **)&b->h_err, 3 * sizeof(float) * nscenes) != cudaSuccess) return bail(FSPH_OOM);
    std::memset(b->ctl_host, 0, sizeof(DevCtl));
    std::memset(b->h_err, 0, 3 * sizeof(float) * nscenes);
    cudaMemcpyAsync(b->d_offs, b->offs.data(), (nscenes + 1) * sizeof(int), cudaMemcpyHostToDevice, b->stream);
    cudaMemsetAsync(b->ctl, 0, sizeof(DevCtl), b->stream);
    cudaMemsetAsync(b->vort, 0, n * sizeof(float4), b->stream);
    cudaMemsetAsync(b->dens, 0, n * sizeof(float), b->stream);
    for (int k = 0; k < 2; ++k) {
        cudaMemsetAsync(b->ppos[k], 0, n * sizeof(float4), b->stream);
        cudaMemsetAsync(b->attr[k], 0, n * sizeof(unsigned int), b->stream);
    }
    if ((st = apply_config(b, b->cfg, 0.0016f)) != FSPH_OK) return bail(st);
    *out = b;
    return FSPH_OK;
}

int fsph_batch_destroy(fsph_batch *b) {
    if (!b) return FSPH_INVALID_ARG;
    if (b->stream) cudaStreamSynchronize(b->stream);
    bdrop_graph(b);
    bfree(b);
    if (b->stream) cudaStreamDestroy(b->stream);
    if (b->s2) cudaStreamDestroy(b->s2);
    if (b->s3) cudaStreamDestroy(b->s3);
    delete b;
    return FSPH_OK;
}

const char *fsph_batch_last_error(const fsph_batch *b) { return b ? b->err.c_str() : "null batch"; }

int fsph_batch_num_particles(const fsph_batch *b) { return b ? b->n : -1; }

int fsph_batch_offsets(const fsph_batch *b, int *offsets) {
    if (!b || !offsets) return FSPH_INVALID_ARG;
    std::memcpy(offsets, b->offs.data(), b->offs.size() * sizeof(int));
    return FSPH_OK;
}

int fsph_batch_set_particles(fsph_batch *b, const float *pos4, const float *vel4, int where) {
    if (!b || !pos4) return FSPH_INVALID_ARG;
    if (where != FSPH_HOST && where != FSPH_DEVICE) return bfail(b, FSPH_INVALID_ARG, "where");
    cudaMemcpyKind k = where == FSPH_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const size_t bytes = (size_t)b->n * sizeof(float4);
    cudaStream_t s = b->stream;
    FB_CUDA(b, cudaMemcpyAsync(b->pos[0], pos4, bytes, k, s));
    if (vel4) FB_CUDA(b, cudaMemcpyAsync(b->vel[0], vel4, bytes, k, s));
    else FB_CUDA(b, cudaMemsetAsync(b->vel[0], 0, bytes, s));
    FB_CUDA(b, cudaMemsetAsync(b->attr[0], 0, (size_t)b->n * 4, s));
    launch_iota(b->n, b->id[0], s);
    unsigned int *flag = b->rank; /* scratch between steps */
    FB_CUDA(b, cudaMemsetAsync(flag, 0, sizeof(unsigned int), s));
    launch_check_finite(b->n, b->pos[0], b->vel[0], flag, s);
    unsigned int hflag = 0;
    FB_CUDA(b, cudaMemcpyAsync(&hflag, flag, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    FB_CUDA(b, cudaStreamSynchronize(s));
    FB_CUDA(b, cudaGetLastError());
    if (hflag) return bfail(b, FSPH_NAN_DETECTED, "non-finite input position or velocity");
    b->loaded = true;
    return FSPH_OK;
}

int fsph_batch_step(fsph_batch *b, float dt, void *stream) {
    if (!b) return FSPH_INVALID_ARG;
    if (!b->loaded) return bfail(b, FSPH_NOT_INITIALIZED, "no particles (fsph_batch_set_particles)");
    if (!(dt > 0.0f) || !std::isfinite(dt)) return bfail(b, FSPH_INVALID_ARG, "dt must be positive and finite");
    cudaStream_t user = (cudaStream_t)stream;
    cudaEvent_t ev = nullptr;
    if (user && user != b->stream) {
        FB_CUDA(b, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        FB_CUDA(b, cudaEventRecord(ev, user));
        FB_CUDA(b, cudaStreamWaitEvent(b->stream, ev, 0));
    }
    int st = bstep(b, dt);
    if (ev) {
        cudaEventRecord(ev, b->stream);
        cudaStreamWaitEvent(user, ev, 0);
        cudaEventDestroy(ev);
    }
    return st;
}

int fsph_batch_get_array(fsph_batch *b, int type, void *dst, int where) {
    if (!b || !dst) return FSPH_INVALID_ARG;
    if (where != FSPH_HOST && where != FSPH_DEVICE) return bfail(b, FSPH_INVALID_ARG, "where");
    cudaStream_t s = b->stream;
    const int n = b->n;
    cudaMemcpyKind k = where == FSPH_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (type == FSPH_POSITION || type == FSPH_VELOCITY) {
        launch_unsort4(n, b->id[0], type == FSPH_POSITION ? b->pos[0] : b->vel[0], b->tmp4, 1, s);
        FB_CUDA(b, cudaMemcpyAsync(dst, b->tmp4, (size_t)n * 16, k, s));
    } else if (type == FSPH_DENSITY) {
        float *t = reinterpret_cast<float *>(b->key);
        launch_unsort1(n, b->id[0], reinterpret_cast<const unsigned int *>(b->dens), reinterpret_cast<unsigned int *>(t), s);
        FB_CUDA(b, cudaMemcpyAsync(dst, t, (size_t)n * 4, k, s));
    } else {
        return bfail(b, FSPH_INVALID_ARG, "batched arrays: POSITION, VELOCITY, DENSITY");
    }
    FB_CUDA(b, cudaStreamSynchronize(s));
    FB_CUDA(b, cudaGetLastError());
    return FSPH_OK;
}

int fsph_batch_scene_stats(fsph_batch *b, int scene, fsph_step_stats *st) {
    if (!b || !st || scene < 0 || scene >= b->nscenes) return FSPH_INVALID_ARG;
    FB_CUDA(b, cudaStreamSynchronize(b->stream));
    std::memset(st, 0, sizeof(*st));
    st->iterations = (int)b->ctl_host->iter;
    st->grid_builds = (int)b->ctl_host->builds;
    st->density_error_one_sided = b->h_err[3 * scene];
    st->density_error_two_sided = b->h_err[3 * scene + 1];
    st->density_error_max = b->h_err[3 * scene + 2];
    st->density_error = b->P[scene].error_mode ? st->density_error_two_sided : st->density_error_one_sided;
    st->bounds_bits = (int)b->ctl_host->bounds_bits;
    st->status = b->ctl_host->nan_flag ? FSPH_NAN_DETECTED : st->bounds_bits ? FSPH_CUDA_ERROR : FSPH_OK;
    return FSPH_OK;
}

int fsph_batch_set_config(fsph_batch *b, const fsph_batch_config *cfg) {
    if (!b || !cfg) return FSPH_INVALID_ARG;
    return apply_config(b, *cfg, b->graph_dt > 0.0f ? b->graph_dt : 0.0016f);
}

int fsph_batch_get_config(const fsph_batch *b, fsph_batch_config *cfg) {
    if (!b || !cfg) return FSPH_INVALID_ARG;
    *cfg = b->cfg;
    return FSPH_OK;
}

int fsph_batch_autotune(fsph_batch *b, float dt, int steps, fsph_batch_config *best, float *best_ms) {
    if (!b || steps < 1 || !(dt > 0.0f)) return FSPH_INVALID_ARG;
    if (!b->loaded) return bfail(b, FSPH_NOT_INITIALIZED, "no particles (fsph_batch_set_particles)");
    const std::string sig = signature(b, dt);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(sig);
        if (it != g_tune_cache.end()) {
            FB_TRY(apply_config(b, it->second, dt));
            if (best) *best = it->second;
            if (best_ms) *best_ms = -1.0f; /* cached: not timed */
            return FSPH_OK;
        }
    }
    Saved sv;
    FB_TRY(save_state(b, sv));
    cudaEvent_t e0, e1;
    FB_CUDA(b, cudaEventCreate(&e0));
    FB_CUDA(b, cudaEventCreate(&e1));
    fsph_batch_config win = b->cfg;
    float win_ms = 1e30f;
    int st = FSPH_OK;
    const int blocks[3] = {128, 256, 512}, lanes[3] = {1, 2, 4};
    const float skins[3] = {0.05f, 0.1f, 0.2f};
    for (int bi = 0; bi < 3 && st == FSPH_OK; ++bi)
        for (int li = 0; li < 3 && st == FSPH_OK; ++li)
            for (int si = 0; si < 3 && st == FSPH_OK; ++si) {
                fsph_batch_config c{blocks[bi], lanes[li], skins[si], 0};
                if ((st = apply_config(b, c, dt)) != FSPH_OK) break;
                if ((st = restore_state(b, sv)) != FSPH_OK) break;
                if ((st = bstep(b, dt)) != FSPH_OK) break; /* builds the graph; warm-up */
                if (cudaEventRecord(e0, b->stream) != cudaSuccess) { st = FSPH_CUDA_ERROR; break; }
                for (int k = 0; k < steps && st == FSPH_OK; ++k) st = bstep(b, dt);
                if (st != FSPH_OK) break;
                if (cudaEventRecord(e1, b->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
                    st = FSPH_CUDA_ERROR;
                    break;
                }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                ms /= (float)steps;
                if (ms < win_ms) { win_ms = ms; win = c; }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    FB_TRY(st);
    FB_TRY(apply_config(b, win, dt));
    FB_TRY(restore_state(b, sv));
    FB_CUDA(b, cudaStreamSynchronize(b->stream));
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[sig] = win;
    }
    if (best) *best = win;
    if (best_ms) *best_ms = win_ms;
    return FSPH_OK;
}

}  // extern "C"
