// k_nn.cu -- cell binning and Verlet neighbour lists on the GPU.
//
// Reference path: updateCellsCPU / updateCellsGPU (femmd2D/src/nn.cpp:8-20,
// nnCuda.cu:69-82) and buildNNCPUSerial / buildNNGPUKernel (nn.cpp:22-62,
// nnCuda.cu:84-135), driven by NeighborList::update (nn.cpp:114-134).
//
// Binning is an integer counting sort: warp-aggregated atomic histogram
// (one atomicAdd per distinct cell in a warp, found with __match_any_sync),
// exclusive scan of the counts into cellStart, scatter to the slots, then a
// per-cell sort by particle id.  The result is deterministic and is the
// reference CPU's order (ascending id inside a cell), and it has no per-cell
// capacity (the reference's cellContent[c*maxPPC+k] has one and never checks
// it).  Each cell's particles are also copied into cellSorted as
// (x, y, id|type<<27, excl) so the list build streams contiguous float4s.
//
// The list build visits the 3x3 cells in the reference's order (cx outer,
// cy inner, both axes wrapped as applyCellBC does, nnCuda.cu:26-36), keeps
// j != i outside i's exclusion group with the reference's float
// dr2 <= (rc+skin)^2, and writes the packed layout of nbr_at (16-byte
// groups of four entries, coalesced for the force kernel).  Counts beyond the capacity raise an
// overflow flag; the host grows the list and repeats the steps.
#include "femmd_internal.h"
#include "launch.h"
#include "device_common.cuh"
#include "nn_body.cuh"

namespace femmd {

// Integrator::run start: NeighborList::update(1) (nn.cpp:114-134) forces a
// rebuild and leaves totalUpdates = 1, dispHi = 0; k_rebuild_begin of the
// forced rebuild does the counting.
__global__ void k_run_start(DevSys s) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        DevScalars *c = s.sc;
        c->rebuild = 1;
        c->dispHi = 0.0f;
        c->totalUpdates = 0;
        c->obsRow = 0;
        c->ticket = 0;
        c->triTicket = 0;
        c->accU = c->accW = c->accK = 0ull;
        c->vvMaxBits = 0u;
        c->stepNow = s.stepBase;
    }
}

// The taken branch of NeighborList::update (nn.cpp:118-124): count the update
// and restart the displacement accumulator.
__global__ void k_rebuild_begin(DevSys s) {
    if (threadIdx.x == 0 && blockIdx.x == 0 && s.sc->rebuild) {
        s.sc->totalUpdates += 1;
        s.sc->dispHi = 0.0f;
        if (s.trace) {
            int row = s.sc->obsRow - 1;
            if (row >= 0 && row < s.obsCap) s.trace[(size_t)row * kTraceCols + 4] = global_ns();
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_cells_count(DevSys s, int parity, int check) {
    if (check && !s.sc->rebuild) return;
    const float2 *pos = parity ? s.pos1 : s.pos0;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool act = i < s.N;
    unsigned active = __ballot_sync(0xffffffffu, act);
    if (!act) return;
    float2 p = pos[i];
    // a non-finite position would land in a clamped edge cell; flag it so the
    // in-cell placement and the list build (quadratic in a cell's size) are skipped
    if (!(isfinite(p.x) && isfinite(p.y))) atomicOr(&s.sc->nonfinite, 1);
    if (outside_box(s, p)) atomicOr(&s.sc->outside, 1);
    int c = cell_col(p.x, p.y, s.ncx, s.ncy, s.Lx, s.Ly);
    s.cellOf[i] = c;
    unsigned peers = __match_any_sync(active, c);
    int lane = threadIdx.x & 31;
    int leader = __ffs(peers) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&s.cellCount[c], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    s.rank[i] = base + __popc(peers & ((1u << lane) - 1u));
}

// per-block totals of kScanBlock cell counts
__global__ void __launch_bounds__(kScanBlock) k_scan_blocks(DevSys s, int check) {
    if (check && !s.sc->rebuild) return;
    __shared__ int red[32];
    int c = blockIdx.x * kScanBlock + threadIdx.x;
    int v = c < s.ncells ? s.cellCount[c] : 0;
    v = warp_sum_int(v);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        int w = red[threadIdx.x];
        w = warp_sum_int(w);
        if (threadIdx.x == 0) s.blockSums[blockIdx.x] = w;
    }
}

// exclusive scan -> cellStart; counts are cleared for the next binning
__global__ void __launch_bounds__(kScanBlock) k_scan_apply(DevSys s, int nblocks, int check) {
    if (check && !s.sc->rebuild) return;
    __shared__ int wsum[32];
    __shared__ int prefix;
    int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    // prefix of earlier blocks (fixed order)
    int acc = 0;
    for (int b = t; b < blockIdx.x; b += kScanBlock) acc += s.blockSums[b];
    acc = warp_sum_int(acc);
    if (lane == 0) wsum[warp] = acc;
    __syncthreads();
    if (t == 0) {
        int p = 0;
        for (int w = 0; w < kScanBlock / 32; w++) p += wsum[w];
        prefix = p;
    }
    __syncthreads();
    int c = blockIdx.x * kScanBlock + t;
    int v = c < s.ncells ? s.cellCount[c] : 0;
    // inclusive warp scan
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
        int w = wsum[lane];
        int z = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, z, o);
            if (lane >= o) z += y;
        }
        wsum[lane] = z - w;  // exclusive warp offsets
    }
    __syncthreads();
    if (c < s.ncells) {
        s.cellStart[c] = prefix + wsum[warp] + x - v;
        s.cellCount[c] = 0;
    }
    if (blockIdx.x == nblocks - 1 && t == 0) {
        s.cellStart[s.ncells] = s.N;
        s.sc->nbrSum = 0ull;
        s.sc->maxCount = 0;
    }
}

__global__ void __launch_bounds__(kBlock) k_scatter(DevSys s, int check) {
    if (check && !s.sc->rebuild) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.N) return;
    int slot = s.cellStart[s.cellOf[i]] + s.rank[i];
    if (slot >= 0 && slot < s.N)
        s.unsorted[slot] = i;
    else
        atomicOr(&s.sc->overflow, 2);  // inconsistent counts: never write outside the array
}

// ascending id inside each cell + the cell-ordered float4 copy, one thread
// per particle
__global__ void __launch_bounds__(kBlock) k_cell_place(DevSys s, int parity, int check) {
    if ((check && !s.sc->rebuild) || s.sc->nonfinite || (s.sc->overflow & 2)) return;
    const float2 *pos = parity ? s.pos1 : s.pos0;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < s.N) place_one<true>(s, pos, i, &s.sc->overflow);
}

// One thread per particle, writing its list straight to HBM (staging the
// lists in shared memory for coalesced stores measured slower).  Threads
// take the particles in cell order (slot t of cellSorted), so the lanes of a
// warp sit in the same or adjacent cells of one column and walk nearly the
// same candidate ranges; each particle's list is still its own column.
//
// A warp whose 32 slots lie in one cell column, away from the y edges,
// first copies the candidates of its three stencil columns (one contiguous
// slot window per column) into shared memory with coalesced loads; its lanes
// then walk their own ranges there, in the same order.  Other warps walk
// cellSorted directly.
constexpr int kWinCap = 256;  // staged candidates per warp (16 bytes each)

__global__ void __launch_bounds__(kNnBlock) k_build_nn(DevSys s, int parity, int check) {
    if ((check && !s.sc->rebuild) || s.sc->nonfinite || (s.sc->overflow & 2)) return;
    __shared__ float4 win[kNnBlock / 32][kWinCap];
    const float2 *pos = parity ? s.pos1 : s.pos0;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool fast = fast_walk_ok(s);  // the same for the whole grid
    int k = 0;
    if (fast) {
        const bool valid = t < s.N;
        const float4 me = valid ? __ldg(s.cellSorted + t) : make_float4(0.f, 0.f, 0.f, 0.f);
        const int i = __float_as_int(me.z) & kIdMask;
        // the cell the binning gave the particle, from the same position
        int ix, iy;
        cell_xy(me.x, me.y, s.ncx, s.ncy, s.Lx, s.Ly, ix, iy);
        const int ncy = s.ncy;
        int qb[3] = {0, 0, 0}, qe[3] = {0, 0, 0};
        float sx[3] = {0.f, 0.f, 0.f};
        if (valid && iy >= 1 && iy <= ncy - 2) stencil_columns(s, ix, iy, qb, qe, sx);
        // slots are in cell order: ix and iy do not decrease along the warp,
        // so lane 0's range starts and lane 31's range ends bound the windows
        const unsigned all = __ballot_sync(0xffffffffu, valid);
        const int ixa = __shfl_sync(0xffffffffu, ix, 0), ixb = __shfl_sync(0xffffffffu, ix, 31);
        const int iya = __shfl_sync(0xffffffffu, iy, 0), iyb = __shfl_sync(0xffffffffu, iy, 31);
        bool staged = all == 0xffffffffu && ixa == ixb && iya >= 1 && iyb <= ncy - 2;
        int wb[3], wo[3], wl[3];
        if (staged) {
            int tot = 0;
#pragma unroll
            for (int d = 0; d < 3; d++) {
                wb[d] = __shfl_sync(0xffffffffu, qb[d], 0);
                wl[d] = __shfl_sync(0xffffffffu, qe[d], 31) - wb[d];
                wo[d] = tot;
                tot += wl[d];
            }
            staged = tot <= kWinCap;  // the same on every lane
        }
        if (staged) {
            float4 *w = win[threadIdx.x >> 5];
            const int lane = threadIdx.x & 31;
#pragma unroll
            for (int d = 0; d < 3; d++)
                for (int q = lane; q < wl[d]; q += 32) w[wo[d] + q] = __ldg(s.cellSorted + wb[d] + q);
            __syncwarp();
            ListOut o = list_out(s, i);
            k = build_fast_staged(s, i, make_float2(me.x, me.y), __float_as_int(me.w), w, qb, qe, sx, wb, wo, o);
            o.finish(k, s.nbrCap);
        } else if (valid) {
            ListOut o = list_out(s, i);
            k = build_fast_at<true>(s, i, ix * ncy + iy, make_float2(me.x, me.y), __float_as_int(me.w), o);
            o.finish(k, s.nbrCap);
        }
        if (valid) s.nbrCount[i] = k;
    } else if (t < s.N) {
        const int i = t;
        ListOut o = list_out(s, i);
        k = build_general<true>(s, pos, i, o);
        o.finish(k, s.nbrCap);
        s.nbrCount[i] = k;
    }
    // build statistics and overflow
    int kmax = warp_max_int(k);
    int ksum = warp_sum_int(k);
    if ((threadIdx.x & 31) == 0) {
        if (ksum) atomicAdd(&s.sc->nbrSum, (unsigned long long)ksum);
        if (kmax > 0) atomicMax(&s.sc->maxCount, kmax);
        if (kmax > s.nbrCap) atomicOr(&s.sc->overflow, 1);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&s.sc->builds, 1ull);
    if (s.trace && (threadIdx.x & 31) == 0) {
        int row = s.sc->obsRow - 1;
        if (row >= 0 && row < s.obsCap) atomicMax(&s.trace[(size_t)row * kTraceCols + 5], global_ns());
    }
}

int scan_blocks(int ncells) { return (ncells + kScanBlock - 1) / kScanBlock; }

cudaError_t enqueue_bin(Launch &L, const DevSys &s, int parity, int check) {
    cudaError_t e;
    int pb = (s.N + kBlock - 1) / kBlock;
    int nsb = scan_blocks(s.ncells);
    if (check && (e = L.kernel(k_rebuild_begin, dim3(1), dim3(32), 0, s))) return e;
    if ((e = L.kernel(k_cells_count, dim3(pb), dim3(kBlock), 0, s, parity, check))) return e;
    if ((e = L.kernel(k_scan_blocks, dim3(nsb), dim3(kScanBlock), 0, s, check))) return e;
    if ((e = L.kernel(k_scan_apply, dim3(nsb), dim3(kScanBlock), 0, s, nsb, check))) return e;
    return L.kernel(k_scatter, dim3(pb), dim3(kBlock), 0, s, check);
}

cudaError_t enqueue_rebuild(Launch &L, const DevSys &s, int parity, int check) {
    if (s.fast) return enqueue_rebuild_fast(L, s, parity, check);
    cudaError_t e;
    int pb = (s.N + kBlock - 1) / kBlock;
    if ((e = enqueue_bin(L, s, parity, check))) return e;
    if ((e = L.kernel(k_cell_place, dim3(pb), dim3(kBlock), 0, s, parity, check))) return e;
    const int nb = (s.N + kNnBlock - 1) / kNnBlock;
    if ((e = L.kernel(k_build_nn, dim3(nb), dim3(kNnBlock), 0, s, parity, check))) return e;
    return cudaSuccess;
}

cudaError_t enqueue_run_start(Launch &L, const DevSys &s) {
    return L.kernel(k_run_start, dim3(1), dim3(32), 0, s);
}

}  // namespace femmd
