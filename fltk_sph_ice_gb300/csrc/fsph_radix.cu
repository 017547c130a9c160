/*
 * fsph_radix.cu -- the grid build's sort as an LSD radix sort of 64-bit keys
 * (cell << 32 | previous slot), the alternative (fsph_params.grid_sort = 1)
 * to the counting sort with per-cell ordering.  Both give the same
 * permutation: the keys are formed in previous-slot order, so a stable sort
 * on the cell bits alone orders them as the full 64-bit key; only the
 * significant cell bits are sorted, 8 per pass.
 *
 * Replaces the reference's thrust::sort_by_key of (hash, index) pairs
 * (CuSort, rx_cu_funcs.cu:250-260; called from calcHash ->
 * reorderDataAndFindCellStart, rx_sph.cu:75-120).
 *
 * One pass: a per-tile digit histogram (digit-major table, so an exclusive
 * scan of the table gives every (digit, tile) its output offset), the scan,
 * then a scatter that ranks each key stably inside its tile (warp-private
 * counters in shared memory, __match_any_sync groups of equal digits within
 * each 32-key round) and writes it to its offset.  The last pass writes the
 * slot (the low 32 bits) straight into the permutation.
 */
#include "fsph_kernels.cuh"

namespace fsph {

namespace {
constexpr int kRadixThreads = 256;
constexpr int kRadixWarps = kRadixThreads / 32;
constexpr int kRadixIpt = 8;                             /* keys per thread */
constexpr int kRadixTile = kRadixThreads * kRadixIpt;   /* keys per block */
constexpr int kRadixBins = 256;
static_assert(kRadixBins == kRadixThreads, "one digit per thread in the offset pass");

__device__ __forceinline__ unsigned long long radix_key(const unsigned int *__restrict__ cell,
                                                        const unsigned long long *__restrict__ key_in, int i) {
    return key_in ? key_in[i] : ((unsigned long long)cell[i] << 32) | (unsigned int)i;
}

__global__ void __launch_bounds__(kRadixThreads)
    k_radix_hist(int n, const unsigned int *__restrict__ cell, const unsigned long long *__restrict__ key_in,
                 int shift, unsigned int ntiles, unsigned int *__restrict__ hist) {
    __shared__ unsigned int h[kRadixBins];
    h[threadIdx.x] = 0u;
    __syncthreads();
    const int base = blockIdx.x * kRadixTile;
    for (int k = threadIdx.x; k < kRadixTile; k += kRadixThreads) {
        const int i = base + k;
        if (i >= n) break;
        atomicAdd(&h[(unsigned int)(radix_key(cell, key_in, i) >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kRadixThreads)
    k_radix_scatter(int n, const unsigned int *__restrict__ cell, const unsigned long long *__restrict__ key_in,
                    int shift, unsigned int ntiles, const unsigned int *__restrict__ offs,
                    unsigned long long *__restrict__ key_out, unsigned int *__restrict__ perm_out) {
    __shared__ unsigned int cnt[kRadixWarps][kRadixBins];
    for (int k = threadIdx.x; k < kRadixWarps * kRadixBins; k += kRadixThreads) (&cnt[0][0])[k] = 0u;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned int below = (1u << lane) - 1u;
    /* warp w owns the contiguous keys [w * 32 * kRadixIpt, (w + 1) * 32 * kRadixIpt) of the tile */
    const int wbase = blockIdx.x * kRadixTile + warp * 32 * kRadixIpt;
    unsigned long long key[kRadixIpt];
    unsigned int dig[kRadixIpt], loc[kRadixIpt];
#pragma unroll
    for (int r = 0; r < kRadixIpt; ++r) {
        const int i = wbase + r * 32 + lane;
        const bool ok = i < n;
        const unsigned long long kk = ok ? radix_key(cell, key_in, i) : 0ull;
        const unsigned int d = ok ? (unsigned int)(kk >> shift) & 255u : (unsigned int)kRadixBins;
        const unsigned int peers = __match_any_sync(0xffffffffu, d);
        const int leader = __ffs(peers) - 1;
        unsigned int pre = 0u;
        if (lane == leader && ok) {
            pre = cnt[warp][d];
            cnt[warp][d] = pre + (unsigned int)__popc(peers);
        }
        pre = __shfl_sync(0xffffffffu, pre, leader);
        __syncwarp();
        key[r] = kk;
        dig[r] = d;
        loc[r] = pre + (unsigned int)__popc(peers & below);
    }
    __syncthreads();
    {   /* digit d: the tile's global offset, then the warps before */
        const unsigned int d = threadIdx.x;
        unsigned int run = offs[d * ntiles + blockIdx.x];
        for (int w = 0; w < kRadixWarps; ++w) {
            const unsigned int t = cnt[w][d];
            cnt[w][d] = run;
            run += t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRadixIpt; ++r) {
        if (dig[r] >= (unsigned int)kRadixBins) continue;
        const unsigned int dst = cnt[warp][dig[r]] + loc[r];
        if (perm_out) perm_out[dst] = (unsigned int)key[r];
        else key_out[dst] = key[r];
    }
}
}  // namespace

unsigned int radix_tiles(int n) { return (unsigned int)((n + kRadixTile - 1) / kRadixTile); }

int radix_passes(unsigned int ncells) {
    int bits = 0;
    while (bits < 32 && (1ull << bits) < (unsigned long long)ncells) ++bits;
    return bits < 8 ? 1 : (bits + 7) / 8;
}

void launch_radix_sort_cells(int n, const unsigned int *cell, unsigned int ncells, const RadixBufs &b,
                             unsigned int *perm, cudaStream_t s) {
    if (n <= 0) return;
    const unsigned int nt = radix_tiles(n);
    const int passes = radix_passes(ncells);
    const unsigned long long *in = nullptr;
    unsigned long long *out = b.k0;
    for (int ps = 0; ps < passes; ++ps) {
        const int shift = 32 + 8 * ps;
        const bool last = ps == passes - 1;
        k_radix_hist<<<nt, kRadixThreads, 0, s>>>(n, cell, in, shift, nt, b.hist);
        launch_scan(b.hist, b.offs, b.bsum, (unsigned int)kRadixBins * nt, s);
        k_radix_scatter<<<nt, kRadixThreads, 0, s>>>(n, cell, in, shift, nt, b.offs, last ? nullptr : out,
                                                     last ? perm : nullptr);
        in = out;
        out = out == b.k0 ? b.k1 : b.k0;
    }
}

}  // namespace fsph
