/*
 * fsph_noalloc.cu -- fsph_pbf_eval_lambda_noalloc: the lambda pass for
 * callers that cannot allocate device memory (see include/fsph.h).
 *
 * All working memory lives in one file-scope __device__ array, carved into
 * the grid tables and sorted copies the pass needs.  Host code only ever
 * holds that array's device address, looked up with cudaGetSymbolAddress
 * once per device; the array's name in host code is a host-side stand-in,
 * not a device address, and is never passed to a kernel.  The kernels are
 * the ones the context-based path launches, so the results are the same.
 */
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/fsph.h"
#include "fsph_kernels.cuh"

namespace fsph {
/* parameter builders of the context-based path (fsph_api.cu) */
DevParams dev_params_for(const fsph_params &p, int n, float dt);
unsigned long long grid_cells_for(const fsph_params &p);
}  // namespace fsph

using namespace fsph;

namespace {

constexpr size_t kMaxP = FSPH_NOALLOC_MAX_PARTICLES;
constexpr size_t kMaxC = FSPH_NOALLOC_MAX_CELLS;
constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

constexpr size_t kOffCount = 0;                                             /* u32[kMaxC]   */
constexpr size_t kOffStart = align256(kOffCount + kMaxC * 4);               /* u32[kMaxC+1] */
constexpr size_t kOffBsum = align256(kOffStart + (kMaxC + 1) * 4);          /* scan blocks  */
constexpr size_t kOffKey = align256(kOffBsum + ((kMaxC + kScanTile - 1) / kScanTile) * 4);
constexpr size_t kOffRank = align256(kOffKey + kMaxP * 4);
constexpr size_t kOffPerm = align256(kOffRank + kMaxP * 4);
constexpr size_t kOffX = align256(kOffPerm + kMaxP * 4);                    /* float4[kMaxP] */
constexpr size_t kOffDens = align256(kOffX + kMaxP * 16);
constexpr size_t kOffCtl = align256(kOffDens + kMaxP * 4);
constexpr size_t kOffPart = align256(kOffCtl + sizeof(DevCtl));
/* two ErrPartial slots per block: room for the fixed-point partials (ErrPartialFix) */
constexpr size_t kScratchBytes = align256(kOffPart + 2 * ((kMaxP + kPassBlock - 1) / kPassBlock) * sizeof(ErrPartial));

constexpr int kMaxDevices = 64;

}  // namespace

/* The fixed working memory (about 10.3 MB per device). */
static __device__ __align__(256) unsigned char g_fsph_noalloc_scratch[kScratchBytes];

namespace {

std::mutex g_mu;
unsigned char *g_addr[kMaxDevices] = {};

/* Device address of the scratch array on the current device; looked up once
 * per device (the first call on a device does this set-up). */
int scratch_address(unsigned char **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FSPH_CUDA_ERROR;
    if (dev < 0 || dev >= kMaxDevices) return FSPH_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_fsph_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return FSPH_CUDA_ERROR;
        }
        g_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_addr[dev];
    return FSPH_OK;
}

}  // namespace

extern "C" int fsph_pbf_eval_lambda_noalloc(const fsph_params *params, const float *pos4, int n, float *dens,
                                            float *lambda, void *stream) {
    if (!params) return FSPH_INVALID_ARG;
    if (n < 0 || (size_t)n > kMaxP) return FSPH_INVALID_ARG;
    if (n == 0) return FSPH_OK;
    if (!pos4 || !dens || !lambda) return FSPH_INVALID_ARG;
    const fsph_params &P = *params;
    if (!(P.h > 0.0f) || !std::isfinite(P.h) || !(P.mass > 0.0f) || !(P.rest_dens > 0.0f)) return FSPH_INVALID_ARG;
    if (P.cell_skin < 0.0f || P.cell_skin > 1.0f) return FSPH_INVALID_ARG;
    for (int a = 0; a < 3; ++a)
        if (!std::isfinite(P.box_min[a]) || !std::isfinite(P.box_max[a]) || !(P.box_max[a] > P.box_min[a]))
            return FSPH_INVALID_ARG;
    const unsigned long long cells = grid_cells_for(P);
    if (cells == 0 || cells > kMaxC) return FSPH_INVALID_ARG;

    unsigned char *base = nullptr;
    int st = scratch_address(&base);
    if (st != FSPH_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned int *count = reinterpret_cast<unsigned int *>(base + kOffCount);
    unsigned int *cell_start = reinterpret_cast<unsigned int *>(base + kOffStart);
    unsigned int *bsum = reinterpret_cast<unsigned int *>(base + kOffBsum);
    unsigned int *key = reinterpret_cast<unsigned int *>(base + kOffKey);
    unsigned int *rank = reinterpret_cast<unsigned int *>(base + kOffRank);
    unsigned int *perm = reinterpret_cast<unsigned int *>(base + kOffPerm);
    float4 *x = reinterpret_cast<float4 *>(base + kOffX);
    float *d_sorted = reinterpret_cast<float *>(base + kOffDens);
    DevCtl *ctl = reinterpret_cast<DevCtl *>(base + kOffCtl);
    ErrPartial *part = reinterpret_cast<ErrPartial *>(base + kOffPart);

    const DevParams p = dev_params_for(P, n, 1.0f);
    const unsigned int nc = (unsigned int)cells;
    /* the array keeps the previous call's contents: clear what must start at zero */
    if (cudaMemsetAsync(count, 0, (size_t)nc * sizeof(unsigned int), s) != cudaSuccess) return FSPH_CUDA_ERROR;
    if (cudaMemsetAsync(ctl, 0, sizeof(DevCtl), s) != cudaSuccess) return FSPH_CUDA_ERROR;
    launch_hash(p, reinterpret_cast<const float4 *>(pos4), key, rank, count, s);
    launch_scan(count, cell_start, bsum, nc, s);
    launch_scatter_sort(p, key, rank, cell_start, perm, nc, s);
    Gather g{};
    g.n4 = 1;
    g.n1 = 0;
    g.src4[0] = reinterpret_cast<const float4 *>(pos4);
    g.dst4[0] = x;
    launch_gather(n, perm, g, nullptr, s);
    launch_lambda(p, cell_start, x, x, d_sorted, ctl, part, 0ull, 0, NbrLists{}, s);
    launch_unsort1(n, perm, reinterpret_cast<const unsigned int *>(d_sorted), reinterpret_cast<unsigned int *>(dens), s);
    launch_unsort_w(n, perm, x, lambda, s);
    if (cudaGetLastError() != cudaSuccess) return FSPH_CUDA_ERROR;
    return FSPH_OK;
}
