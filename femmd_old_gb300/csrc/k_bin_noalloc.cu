// k_bin_noalloc.cu -- cell binning that allocates nothing.
//
// Some callers cannot call cudaMalloc at the point where they need particles
// binned into cells.  Two examples: a simulation loop that is being recorded
// into a CUDA graph, and a host framework that hands out all device memory
// from its own pool.  cudaMalloc and cudaFree synchronise the whole device,
// are not permitted while a stream is being captured, and would bypass the
// framework's memory accounting.  femmd_bin_cells_noalloc serves those
// callers: the caller passes device pointers for the positions and for both
// outputs, and the working memory the counting sort needs lives in one
// file-scope __device__ array of fixed size, which only device code names.
// Every GPU that loads this library holds that array until the process
// exits.
//
// The sort is the same counting sort as the context's rebuild: each particle
// gets the reference's cell id, the counts are histogrammed with
// warp-aggregated atomics, an exclusive scan turns them into cell_start, the
// particles are scattered into their cells, and each cell is sorted by
// particle id.  The output order is the reference CPU's order (ascending id
// inside a cell), so it equals femmd_get_cells after a context build.
#include <cuda_runtime.h>

#include "femmd.h"
#include "femmd_internal.h"
#include "device_common.cuh"

namespace {

using namespace femmd;

constexpr int kNaMaxParticles = FEMMD_NOALLOC_MAX_PARTICLES;
constexpr int kNaMaxCells = FEMMD_NOALLOC_MAX_CELLS;
constexpr int kNaScan = 1024;
constexpr int kNaMaxScanBlocks = (kNaMaxCells + kNaScan - 1) / kNaScan;
// layout of the scratch array, in ints
constexpr size_t kOffCell = 0;
constexpr size_t kOffRank = kOffCell + kNaMaxParticles;
constexpr size_t kOffCount = kOffRank + kNaMaxParticles;
constexpr size_t kOffBlock = kOffCount + kNaMaxCells;
constexpr size_t kScratchInts = kOffBlock + kNaMaxScanBlocks;

// The scratch: per-particle cell and rank, per-cell counts, per-block sums.
// Only device code names it, so every launch uses the array of the module
// and context it runs in (nothing about it is cached on the host, and a
// device reset leaves nothing stale behind).
static __device__ __align__(256) int g_bin_scratch[kScratchInts];

// The counts start at zero; the array keeps the previous call's contents.
__global__ void __launch_bounds__(kBlock) na_clear(int ncells) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < ncells) g_bin_scratch[kOffCount + c] = 0;
}

__global__ void __launch_bounds__(kBlock) na_count(const float2 *pos, int n, int ncx, int ncy, float Lx, float Ly) {
    int *scratch = g_bin_scratch;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool act = i < n;
    unsigned active = __ballot_sync(0xffffffffu, act);
    if (!act) return;
    float2 p = pos[i];
    int c = cell_of(p.x, p.y, ncx, ncy, Lx, Ly);
    scratch[kOffCell + i] = c;
    unsigned peers = __match_any_sync(active, c);
    int lane = threadIdx.x & 31;
    int leader = __ffs(peers) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(scratch + kOffCount + c, __popc(peers));
    base = __shfl_sync(peers, base, leader);
    scratch[kOffRank + i] = base + __popc(peers & ((1u << lane) - 1u));
}

__global__ void __launch_bounds__(kNaScan) na_block_sums(int ncells) {
    const int *scratch = g_bin_scratch;
    int *block_sums = g_bin_scratch + kOffBlock;
    __shared__ int red[32];
    int c = blockIdx.x * kNaScan + threadIdx.x;
    int v = c < ncells ? scratch[kOffCount + c] : 0;
    v = warp_sum_int(v);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        int w = warp_sum_int(red[threadIdx.x]);
        if (threadIdx.x == 0) block_sums[blockIdx.x] = w;
    }
}

__global__ void __launch_bounds__(kNaScan) na_scan(int ncells, int n, int *cell_start) {
    const int *scratch = g_bin_scratch;
    const int *block_sums = g_bin_scratch + kOffBlock;
    __shared__ int wsum[32];
    __shared__ int prefix;
    int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    int acc = 0;
    for (int b = t; b < (int)blockIdx.x; b += kNaScan) acc += block_sums[b];
    acc = warp_sum_int(acc);
    if (lane == 0) wsum[warp] = acc;
    __syncthreads();
    if (t == 0) {
        int p = 0;
        for (int w = 0; w < kNaScan / 32; w++) p += wsum[w];
        prefix = p;
    }
    __syncthreads();
    int c = blockIdx.x * kNaScan + t;
    int v = c < ncells ? scratch[kOffCount + c] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __syncthreads();
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = wsum[lane], z = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, z, o);
            if (lane >= o) z += y;
        }
        wsum[lane] = z - w;
    }
    __syncthreads();
    if (c < ncells) cell_start[c] = prefix + wsum[warp] + x - v;
    if (blockIdx.x == gridDim.x - 1 && t == 0) cell_start[ncells] = n;
}

__global__ void __launch_bounds__(kBlock) na_scatter(int n, const int *cell_start, int *cell_ids) {
    const int *scratch = g_bin_scratch;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int slot = cell_start[scratch[kOffCell + i]] + scratch[kOffRank + i];
    if (slot >= 0 && slot < n) cell_ids[slot] = i;
}

__global__ void __launch_bounds__(kBlock) na_sort(int ncells, const int *cell_start, int *cell_ids) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    int b = cell_start[c], n = cell_start[c + 1] - b;
    int *ids = cell_ids + b;
    int gap = 1;
    while (gap < n / 3) gap = 3 * gap + 1;
    for (; gap > 0; gap /= 3)
        for (int k = gap; k < n; k++) {
            int v = ids[k], m = k - gap;
            while (m >= 0 && ids[m] > v) {
                ids[m + gap] = ids[m];
                m -= gap;
            }
            ids[m + gap] = v;
        }
}

}  // namespace

extern "C" femmd_status femmd_bin_cells_noalloc(const float *d_pos, int n, double Lx, double Ly, int ncx, int ncy,
                                                int *d_cell_start, int *d_cell_ids, void *stream) {
    if (n < 0 || ncx < 1 || ncy < 1 || !(Lx > 0) || !(Ly > 0)) return FEMMD_INVALID_ARG;
    long long ncells = (long long)ncx * ncy;
    if (n > kNaMaxParticles || ncells > kNaMaxCells) return FEMMD_CAPACITY_OVERFLOW;
    if (!d_cell_start || (n > 0 && (!d_pos || !d_cell_ids))) return FEMMD_INVALID_ARG;
    // an error an earlier, unrelated call left pending stays in place for
    // its owner; only an error this call's launches raise is reported (and
    // cleared)
    const cudaError_t prior = cudaPeekAtLastError();
    cudaStream_t s = (cudaStream_t)stream;
    const int nc = (int)ncells;
    const int pb = (n + kBlock - 1) / kBlock, sb = (nc + kNaScan - 1) / kNaScan, cb = (nc + kBlock - 1) / kBlock;
    na_clear<<<cb, kBlock, 0, s>>>(nc);
    if (pb > 0) na_count<<<pb, kBlock, 0, s>>>((const float2 *)d_pos, n, ncx, ncy, (float)Lx, (float)Ly);
    na_block_sums<<<sb, kNaScan, 0, s>>>(nc);
    na_scan<<<sb, kNaScan, 0, s>>>(nc, n, d_cell_start);
    if (pb > 0) na_scatter<<<pb, kBlock, 0, s>>>(n, d_cell_start, d_cell_ids);
    na_sort<<<cb, kBlock, 0, s>>>(nc, d_cell_start, d_cell_ids);
    const cudaError_t now = cudaPeekAtLastError();
    if (now == cudaSuccess || now == prior) return FEMMD_OK;
    cudaGetLastError();
    return FEMMD_CUDA_ERROR;
}
