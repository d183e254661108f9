// k_fast.cu -- the fast force mode of the femmd2D timestep.
//
// The reference-exact mode (k_force.cu, k_nn.cu) reproduces the reference's
// float operations and list order so that trajectories match it bit for bit.
// The fast mode keeps what the contract fixes -- the same cell and neighbour
// SETS, forces, energies and virial within 1e-5 of FP64 -- and drops what only
// the bit-exact trajectory needs:
//   * storage order: every rebuild stores the free particles [nBonded, N) in
//     cell order (column-major cells, ascending id inside a cell), so a
//     warp's particles are neighbours in space and a block's neighbours lie
//     in a few contiguous cell-slot ranges; perm[s] keeps the id of the
//     particle at slot s (bonded particles never move, so bonds, triangles
//     and area springs keep their indices);
//   * windows: a step block of free particles inside one cell column stages
//     the current positions of its stencil window in shared memory once per
//     step, and its lists name window entries, so the pair loop gathers from
//     shared memory;
//   * pair arithmetic: fused multiply-adds, the hardware reciprocal
//     (rcp.approx, 1 ulp) for 1/r^2, and energies summed per particle as
//     sum s6^2, sum s6 and the number of pairs inside the cutoff (one type);
//   * minimum image: a warp whose particles all lie at least imgD inside every
//     periodic edge has no interacting pair across the boundary and does no
//     image work; the warps at an edge take the image per pair, with the
//     difference rounded once from its exact value (TwoSum), as the exact
//     image mode of the reference-exact path.
// Cutoff decisions of the list (dr^2 <= (rc + skin)^2) use the reference's
// own float expression (this file, like the others, is compiled without
// contraction; the pair loop asks for its fused multiply-adds explicitly).
//
// Reference: pairForce/ljforce (femmd2D/src/interactionsCuda.cu:43-100),
// calcPairForcesNN (interactions.cpp:347-389), updateCellsCPU / buildNNCPUSerial
// (nn.cpp:8-62), NeighborList::update (nn.cpp:114-134), the leapfrog of
// Integrator::doStep (integrator.cpp:8-29, 100-135).
#include <cuda_runtime.h>
#include <algorithm>
#include <mutex>
#include <vector>
#include "femmd_internal.h"
#include "launch.h"
#include "device_common.cuh"
#include "nn_body.cuh"
#include "step_body.cuh"

namespace femmd {

constexpr int kPermBlock = 1024;  // cell slots per block of the storage reorder

// A kernel's dynamic shared-memory limit raised to at least 'smem', and the
// blocks of 'threads' threads it keeps resident on the whole GPU at that
// size, queried once per device, kernel, block size and size: the attribute
// call and the occupancy query would cost host time at every launch
// otherwise.  The limit only grows (it is one value per kernel, and launches
// of one kernel take different sizes).
static cudaError_t kernel_setup(const void *fn, int threads, size_t smem, int *resident) {
    struct Occ {
        int dev;
        const void *fn;
        int threads;
        size_t smem;
        int resident;
    };
    struct Limit {
        int dev;
        const void *fn;
        size_t smem;
    };
    static std::mutex mu;
    static std::vector<Occ> occ;
    static std::vector<Limit> limits;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return e;
    std::lock_guard<std::mutex> g(mu);
    Limit *lim = nullptr;
    for (Limit &l : limits)
        if (l.dev == dev && l.fn == fn) lim = &l;
    if (!lim || lim->smem < smem) {
        if ((e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem))) return e;
        if (lim) lim->smem = smem;
        else limits.push_back(Limit{dev, fn, smem});
    }
    for (const Occ &c : occ)
        if (c.dev == dev && c.fn == fn && c.threads == threads && c.smem == smem) {
            *resident = c.resident;
            return cudaSuccess;
        }
    int sms = 0, per = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev))) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, smem))) return e;
    *resident = per * sms;
    occ.push_back(Occ{dev, fn, threads, smem, *resident});
    return cudaSuccess;
}

// ================================================================ rebuild

// Placement inside the cell by ascending particle id (the counting sort's
// atomics gave arbitrary ranks): sortedIds[t] = old slot.  The new storage
// order is then a function of the positions and ids alone -- the reference's
// cell order -- whatever order the particles were stored in before.
__global__ void __launch_bounds__(kBlock) k_fplace(DevSys s, int parity, int check) {
    if ((check && !s.sc->rebuild) || s.sc->nonfinite || (s.sc->overflow & 2)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.N) return;
    const int c = s.cellOf[i];
    const int b = s.cellStart[c], e = s.cellStart[c + 1];
    const int id = s.perm[i];
    int r = 0;
    for (int q = b; q < e; q++) r += __ldg(s.perm + __ldg(s.unsorted + q)) < id;
    const int slot = b + r;
    if (slot >= e) {  // inconsistent cell contents: never write outside the cell
        atomicOr(&s.sc->overflow, 2);
        return;
    }
    if (s.nBonded == 0) {
        // no bonded particles: the new storage slot is the cell slot, so the
        // reorder (k_fperm's work) is written from here, reads by particle
        const float2 *pos = parity ? s.pos1 : s.pos0;
        const float2 pp = pos[i];
        const int tag = slot | (s.numTypes > 1 ? (s.typeId[i] << kIdBits) : 0);
        s.cellSorted[slot] = make_float4(pp.x, pp.y, __int_as_float(tag), __int_as_float(s.excl[i]));
        s.sortedIds[slot] = slot;
        s.newCell[slot] = c;
        s.sPos[slot] = pp;
        s.sVel[slot] = s.vel[i];
        s.sAcc[slot] = s.acc[i];
        s.sPerm[slot] = id;
        return;
    }
    s.sortedIds[slot] = i;
}

// The binning and in-cell placement of a small system without bonded
// particles and with one particle kind, in one block: what k_rebuild_begin,
// k_cells_count, k_scan_blocks, k_scan_apply, k_scatter and k_fplace do as
// six launches, with the cell counts, their exclusive scan and the ids of
// each cell's particles in shared memory.  The outputs are theirs (cellStart,
// the cell-ordered candidate copy, sortedIds, newCell and the state in the
// new order in the scratch arrays); the placement inside a cell is by id, so
// the order of the counting atomics leaves no trace.
constexpr int kSmallBinThreads = 1024;
constexpr int kSmallBinMaxN = kSmallMaxTiles * kFastBlock;
constexpr int kSmallBinPer = kSmallBinMaxN / kSmallBinThreads;  // particles per thread at most
constexpr size_t kSmallBinMaxSmem = 200 * 1024;

static size_t small_bin_smem(const DevSys &s) { return (size_t)(s.ncells + 1 + 3 * (size_t)s.N + 8) * sizeof(int); }

static bool small_bin_fits(const DevSys &s) {
    return s.nBonded == 0 && s.numTypes == 1 && !s.trace && s.N > 0 && s.N <= kSmallBinMaxN &&
           small_bin_smem(s) <= kSmallBinMaxSmem;
}

__global__ void __launch_bounds__(kSmallBinThreads, 1) k_fbin_small(DevSys s, int parity, int check) {
    extern __shared__ int ism[];
    __shared__ int wsum[kSmallBinThreads / 32];
    __shared__ int skip;
    DevScalars *sc = s.sc;
    if (check && !sc->rebuild) return;
    int *start = ism;                  // counts, then cell starts (ncells + 1)
    int *cof = start + s.ncells + 1;   // cell of each slot
    int *rk = cof + s.N;               // rank among the cell's particles (atomic order)
    int *ids = rk + s.N;               // ids in cell-slot order, unsorted inside a cell
    const int tid = threadIdx.x, T = blockDim.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        // the placement is skipped after a non-finite position or inconsistent counts
        skip = (sc->nonfinite || (sc->overflow & 2)) ? 1 : 0;
        if (check) {  // k_rebuild_begin: the taken branch of NeighborList::update
            sc->totalUpdates += 1;
            sc->dispHi = 0.0f;
        }
    }
    for (int c = tid; c < s.ncells; c += T) start[c] = 0;
    __syncthreads();
    const float2 *pos = parity ? s.pos1 : s.pos0;
    bool bad = false;
    // the thread's particles i = tid + u T (at most kSmallBinPer): every
    // position loaded before the first is binned, so the loads overlap
    float2 pp[kSmallBinPer];
#pragma unroll
    for (int u = 0; u < kSmallBinPer; u++) {
        const int i = tid + u * T;
        if (i < s.N) pp[u] = pos[i];
    }
#pragma unroll
    for (int u = 0; u < kSmallBinPer; u++) {
        const int i = tid + u * T;
        if (i >= s.N) break;
        const float2 p = pp[u];
        if (!(isfinite(p.x) && isfinite(p.y))) {
            atomicOr(&sc->nonfinite, 1);
            bad = true;
        }
        if (outside_box(s, p)) atomicOr(&sc->outside, 1);
        const int c = cell_col(p.x, p.y, s.ncx, s.ncy, s.Lx, s.Ly);
        cof[i] = c;
        rk[i] = atomicAdd(&start[c], 1);
    }
    if (bad) skip = 1;
    __syncthreads();
    // exclusive scan of the counts: a contiguous run of cells per thread
    const int per = (s.ncells + T - 1) / T;
    const int c0 = min(tid * per, s.ncells), c1 = min(c0 + per, s.ncells);
    int tot = 0;
    for (int c = c0; c < c1; c++) tot += start[c];
    int x = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const int w = lane < T / 32 ? wsum[lane] : 0;
        int z = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, z, o);
            if (lane >= o) z += y;
        }
        if (lane < T / 32) wsum[lane] = z - w;
    }
    __syncthreads();
    int run = wsum[warp] + x - tot;
    for (int c = c0; c < c1; c++) {
        const int v = start[c];
        start[c] = run;
        run += v;
    }
    if (tid == 0) {
        start[s.ncells] = s.N;
        sc->nbrSum = 0ull;
        sc->maxCount = 0;
    }
    __syncthreads();
    for (int c = tid; c <= s.ncells; c += T) s.cellStart[c] = start[c];
    int pid[kSmallBinPer];
#pragma unroll
    for (int u = 0; u < kSmallBinPer; u++) {
        const int i = tid + u * T;
        pid[u] = i < s.N ? __ldg(s.perm + i) : 0;
    }
#pragma unroll
    for (int u = 0; u < kSmallBinPer; u++) {
        const int i = tid + u * T;
        if (i >= s.N) break;
        const int slot = start[cof[i]] + rk[i];
        rk[i] = pid[u];  // the rank is spent: the slot's id from here on
        if (slot >= 0 && slot < s.N) {
            ids[slot] = pid[u];
        } else {  // inconsistent counts: never write outside the array
            atomicOr(&sc->overflow, 2);
            skip = 1;
        }
    }
    __syncthreads();
    if (skip) return;
#pragma unroll 4
    for (int i = tid; i < s.N; i += T) {
        const int c = cof[i];
        const int b = start[c], e = start[c + 1];
        const int id = rk[i];
        int r = 0;
        for (int q = b; q < e; q++) r += ids[q] < id;
        const int slot = b + r;
        if (slot >= e) {  // inconsistent cell contents: never write outside the cell
            atomicOr(&sc->overflow, 2);
            continue;
        }
        const float2 x = __ldg(pos + i);
        s.cellSorted[slot] = make_float4(x.x, x.y, __int_as_float(slot), __int_as_float(__ldg(s.excl + i)));
        s.sortedIds[slot] = slot;
        s.newCell[slot] = c;
        s.sPos[slot] = x;
        s.sVel[slot] = __ldg(s.vel + i);
        s.sAcc[slot] = __ldg(s.acc + i);
        s.sPerm[slot] = id;
    }
}

// Free particles among each block's cell slots (only with bonded particles).
__global__ void __launch_bounds__(kPermBlock) k_ffree_count(DevSys s, int check) {
    if ((check && !s.sc->rebuild) || s.sc->nonfinite || (s.sc->overflow & 2)) return;
    __shared__ int red[kPermBlock / 32];
    const int t = blockIdx.x * kPermBlock + threadIdx.x;
    int v = (t < s.N && __ldg(s.sortedIds + t) >= s.nBonded) ? 1 : 0;
    v = warp_sum_int(v);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        int w = red[threadIdx.x];
        w = warp_sum_int(w);
        if (threadIdx.x == 0) s.fBlockSums[blockIdx.x] = w;
    }
}

// New storage slot of every particle: bonded ones keep theirs, free ones take
// nBonded + their rank among the free particles in cell order.  Writes the
// cell-ordered candidate copy (tags are the new slots), the new slots in
// cell order (sortedIds), the cell of each new slot, and the free particles'
// state in the new order into the scratch arrays.
__global__ void __launch_bounds__(kPermBlock) k_fperm(DevSys s, int parity, int check) {
    if ((check && !s.sc->rebuild) || s.sc->nonfinite || (s.sc->overflow & 2)) return;
    __shared__ int wsum[kPermBlock / 32];
    __shared__ int prefix;
    const float2 *pos = parity ? s.pos1 : s.pos0;
    const int t = blockIdx.x * kPermBlock + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int old = t < s.N ? __ldg(s.sortedIds + t) : -1;
    const bool fr = old >= s.nBonded;
    int ns = t;
    if (s.nBonded > 0) {
        // prefix of the earlier blocks (fixed order), then the block's own scan
        int acc = 0;
        for (int b = threadIdx.x; b < (int)blockIdx.x; b += kPermBlock) acc += s.fBlockSums[b];
        acc = warp_sum_int(acc);
        if (lane == 0) wsum[warp] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            int p = 0;
            for (int w = 0; w < kPermBlock / 32; w++) p += wsum[w];
            prefix = p;
        }
        __syncthreads();
        const unsigned bal = __ballot_sync(0xffffffffu, fr);
        const int before = __popc(bal & ((1u << lane) - 1u));
        if (lane == 0) wsum[warp] = __popc(bal);
        __syncthreads();
        if (warp == 0) {
            const int w = wsum[lane];
            int z = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, z, o);
                if (lane >= o) z += y;
            }
            wsum[lane] = z - w;
        }
        __syncthreads();
        ns = fr ? s.nBonded + prefix + wsum[warp] + before : old;
    }
    if (t >= s.N) return;
    const float2 p = pos[old];
    const int tag = ns | (s.numTypes > 1 ? (s.typeId[old] << kIdBits) : 0);
    s.cellSorted[t] = make_float4(p.x, p.y, __int_as_float(tag), __int_as_float(s.excl[old]));
    s.sortedIds[t] = ns;
    s.newCell[ns] = s.cellOf[old];
    if (s.cslot) {
        // the cell-ordered mirror of the positions the next step reads
        (parity ? s.cpos1 : s.cpos0)[t] = p;
        s.cslot[ns] = t;
    }
    if (fr) {
        s.sPos[ns] = p;
        s.sVel[ns] = s.vel[old];
        s.sAcc[ns] = s.acc[old];
        s.sPerm[ns] = s.perm[old];
    }
}

// The window of every step-kernel block (one thread per block).  A block of
// free particles whose cell slots lie in one cell column (rows r0 .. r1 of
// column ix) takes, per stencil column ix - 1 .. ix + 1, the rows r0 - 1 ..
// r1 + 1 (piece 2d) and the row across the y edge when the block touches it
// (piece 2d + 1).  A block reaching from the lower rows r0 .. of column ix
// into the upper rows .. r1 of column ix + 1 takes, per column ix - 1 + w
// (w = 0 .. 3), the upper range (piece 2w + 1: rows r0 - 1 .. ncy - 1, only
// the last row for w = 3) and the lower range (piece 2w: rows 0 .. r1 + 1,
// only row 0 for w = 0): the lower column's particles find their stencil
// rows in the upper ranges and their row across the edge in the lower ones,
// the upper column's the other way round.  A piece starting at cell slot a
// takes window entries from an even base, with a & 1 entries before it and
// its end padded to an even count, so that its positions can be copied
// straight from the storage array in 16-byte units when cell slots and
// storage slots coincide.  Other blocks (bonded particles, blocks over more
// cells, windows too large, grids the fast walk does not cover) keep global
// storage slots.  The block's longest list (in groups) is gathered by the
// list build.
// (walk_ok: fast_walk_ok; cs(c): the start of cell c; nc(q): the cell of
// cell slot q.)
template <class CS, class NC>
__device__ __forceinline__ void fwindow_record_t(const DevSys &s, int b, bool walk_ok, CS cs, NC nc) {
    int *out = s.blockWin + kWinInts * (size_t)b;
    const int f = b * kFastBlock, l = min(f + kFastBlock, s.N) - 1;
    const int ncy = s.ncy, ncx = s.ncx;
    bool ok = f >= s.nBonded && walk_ok && ncy >= 3;
    int st[kWinPieces], off[kWinPieces], cnt[kWinPieces];
#pragma unroll
    for (int p = 0; p < kWinPieces; p++) st[p] = off[p] = cnt[p] = 0;
    int acc = 0, ix = 0, two = 0;
    int rs[kWinPieces], re[kWinPieces];
#pragma unroll
    for (int p = 0; p < kWinPieces; p++) rs[p] = 0, re[p] = -1;
    if (ok) {
        const int cf = nc(f), cl = nc(l);
        ix = cf / ncy;
        const int ixl = cl / ncy, r0 = cf - ix * ncy, r1 = cl - ixl * ncy;
        // row ranges [ra, rb] per piece and window column (rb < ra: empty)
        int ra[kWinPieces], rb[kWinPieces];
#pragma unroll
        for (int p = 0; p < kWinPieces; p++) ra[p] = 0, rb[p] = -1;
        if (ixl == ix && !(r0 == 0 && r1 == ncy - 1)) {
            const int lo = max(r0 - 1, 0), hi = min(r1 + 1, ncy - 1);
#pragma unroll
            for (int d = 0; d < 3; d++) {
                ra[2 * d] = lo;
                rb[2 * d] = hi;
                if (r0 == 0) ra[2 * d + 1] = rb[2 * d + 1] = ncy - 1;
                else if (r1 == ncy - 1) ra[2 * d + 1] = rb[2 * d + 1] = 0;
            }
        } else if (ixl == ix + 1 && r0 >= 1 && r1 <= ncy - 2) {
            two = 1;
#pragma unroll
            for (int w = 0; w < 4; w++) {
                ra[2 * w] = 0;
                rb[2 * w] = w == 0 ? 0 : r1 + 1;
                ra[2 * w + 1] = w == 3 ? ncy - 1 : r0 - 1;
                rb[2 * w + 1] = ncy - 1;
            }
        } else {
            ok = false;
        }
        if (ok) {
#pragma unroll
            for (int p = 0; p < kWinPieces; p++) {
                rs[p] = ra[p];
                re[p] = rb[p];
                if (rb[p] < ra[p]) continue;
                int nx = ix + (p >> 1) - 1;
                if (nx < 0) nx += ncx;
                else if (nx >= ncx) nx -= ncx;
                const int col = nx * ncy;
                const int a = cs(col + ra[p]), e = cs(col + rb[p] + 1);
                st[p] = a;
                cnt[p] = e - a;
                off[p] = acc + (a & 1);
                if (cnt[p] > 0) acc += ((e + 1) & ~1) - (a & ~1);
            }
            ok = acc <= kWinMax - 1;  // the last entry is the ghost's
        }
    }
    out[kWLen] = ok ? acc : -1;
#pragma unroll
    for (int p = 0; p < kWinPieces; p++) {
        out[kWStart + p] = st[p];
        out[kWOff + p] = off[p];
        out[kWCount + p] = cnt[p];
    }
    out[kWGroups] = 0;
    out[kWCol0] = ix;
    out[kWTwo] = two;
#pragma unroll
    for (int p = 0; p < kWinPieces; p++) {
        out[kWRow0 + p] = ok ? rs[p] : 0;
        out[kWRow1 + p] = ok ? re[p] : -1;
    }
}

__device__ __forceinline__ void fwindow_record(const DevSys &s, int b) {
    fwindow_record_t(s, b, fast_walk_ok(s), [&](int c) { return s.cellStart[c]; },
                     [&](int q) { return s.newCell[q]; });
}

__global__ void __launch_bounds__(kBlock) k_fwindows(DevSys s, int check) {
    if ((check && !s.sc->rebuild) || s.sc->nonfinite || (s.sc->overflow & 2)) return;
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < (s.N + kFastBlock - 1) / kFastBlock) fwindow_record(s, b);
}

// The list build of the fast mode.  One thread per cell slot t builds the
// list of the particle stored there (storage slot = its tag).  An entry is
// the neighbour's storage slot, or -- for a particle of a windowed step
// block -- the neighbour's index in that block's window.  Every candidate
// writes the lane's column of a per-warp shared-memory stage ([entry][lane]:
// conflict-free whatever the entry index): at its next entry when it is a
// hit, in a spare row when it is not, so the candidate loop has no branch.
// At the end the warp copies the stage to the list one 16-byte group of
// every lane per store (the force kernel's own read pattern).  A lane whose
// list outgrows the stage walks again and writes the rest directly.  Unused
// words of a list's last group name the ghost (slot N, or the window's last
// entry), whose position lies far outside the box, so the force loop needs
// no count test per entry.
constexpr int kLBlock = 128;  // threads per block of the list build
constexpr int kLWin = 256;    // staged candidates per warp
constexpr int kLStage = 48;   // list entries per lane staged in shared memory (a multiple of 8)
static_assert(kLStage % 8 == 0, "whole 16-bit groups in the stage");

struct StagePut {
    int (*st)[32];  // [kLStage + 1][32]; row kLStage takes the misses
    int lane;
    __device__ __forceinline__ void put(bool hit, int val, int &k) const {
        st[(hit && k < kLStage) ? k : kLStage][lane] = val;
        k += hit ? 1 : 0;
    }
};

// Entries from kLStage on, written straight to the list.
struct DirectPut {
    int *nbr;
    int slot, cap, Ncap;
    __device__ __forceinline__ void put(bool hit, int val, int &k) const {
        if (hit) {
            if (k >= kLStage && k < cap) nbr[nbr_at(k, slot, Ncap)] = val;
            k++;
        }
    }
};

// Entries from kLStage on, straight to a list of 16-bit window entries.
struct DirectPut16 {
    unsigned short *nbr16;
    int slot, cap, Ncap;
    __device__ __forceinline__ void put(bool hit, int val, int &k) const {
        if (hit) {
            if (k >= kLStage && k < cap) nbr16[nbr16_at(k, slot, Ncap)] = (unsigned short)val;
            k++;
        }
    }
};

// Every entry written straight to the list (up to the capacity).
struct ListPut {
    int *nbr;
    int slot, cap, Ncap;
    __device__ __forceinline__ void put(bool hit, int val, int &k) const {
        if (hit) {
            if (k < cap) nbr[nbr_at(k, slot, Ncap)] = val;
            k++;
        }
    }
};

// Candidate e (position, tag, group) of the particle at p (group gi) with
// the column's image shift (sx, sy): inside the list radius by the
// reference's float dr^2 (no contraction), not the particle itself (cell
// slot q != self) and not in its exclusion group.
template <bool EX>
__device__ __forceinline__ bool fhit(float4 e, float sx, float sy, float2 p, int gi, float R2, int q, int self) {
    const float dx = (p.x - e.x) - sx;
    const float dy = (p.y - e.y) - sy;
    const float dr2 = dx * dx + dy * dy;
    return dr2 <= R2 && q != self && (!EX || gi == -1 || gi != __float_as_int(e.w));
}

// Candidates [qb, qe) of cand (cell slots qbase + q).  The entry written is
// the candidate's tag, or q + dv with win (its window index).
template <bool EX, bool SX, bool RO, class Put>
__device__ __forceinline__ void fwalk(const float4 *cand, int qb, int qe, int qbase, float sx, float sy, float2 p,
                                      int gi, float R2, int self, bool win, int dv, const Put &out, int &k) {
    int q = qb;
#pragma unroll 1
    for (; q + 4 <= qe; q += 4) {
        float4 e[4];
#pragma unroll
        for (int u = 0; u < 4; u++) e[u] = RO ? __ldg(cand + q + u) : cand[q + u];
#pragma unroll
        for (int u = 0; u < 4; u++)
            out.put(fhit<EX>(e[u], SX ? sx : 0.0f, sy, p, gi, R2, qbase + q + u, self),
                    win ? ((q + u + dv) | (__float_as_int(e[u].z) & ~kIdMask)) : __float_as_int(e[u].z), k);
    }
#pragma unroll 1
    for (; q < qe; q++) {
        const float4 e = RO ? __ldg(cand + q) : cand[q];
        out.put(fhit<EX>(e, SX ? sx : 0.0f, sy, p, gi, R2, qbase + q, self),
                win ? ((q + dv) | (__float_as_int(e.z) & ~kIdMask)) : __float_as_int(e.z), k);
    }
}

// The window deltas of a lane: entry = cell slot + dm[d] for the main rows
// of stencil column d, + dw[d] for the row across the y edge.  In a block
// over two columns a lane of the lower column (j = 0) finds its main rows in
// the upper ranges of window columns d and its edge row in their lower
// ranges; a lane of the upper column (j = 1) the other way round, in window
// columns d + 1.
struct WinDelta {
    bool win;
    int len;
    int dm[3], dw[3];
};

__device__ __forceinline__ WinDelta win_delta(const DevSys &s, int slot) {
    WinDelta w;
    const int *bw = s.blockWin + kWinInts * (size_t)(slot / kFastBlock);
    w.len = bw[kWLen];
    w.win = w.len >= 0;
    const bool two = bw[kWTwo] != 0;
    const int j = two && s.newCell[slot] / s.ncy != bw[kWCol0] ? 1 : 0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const int pm = !two ? 2 * d : (j == 0 ? 2 * d + 1 : 2 * d + 2);
        const int pw = !two ? 2 * d + 1 : (j == 0 ? 2 * d : 2 * d + 3);
        w.dm[d] = bw[kWOff + pm] - bw[kWStart + pm];
        w.dw[d] = bw[kWOff + pw] - bw[kWStart + pw];
    }
    return w;
}

// The particle at cell slot t over the column ranges of its stencil (every
// periodic axis with >= 5 cells, every position inside the box:
// fast_walk_ok), straight from cellSorted.  Cell indices wrap on every axis
// as applyCellBC does (nnCuda.cu:26-36); the image shift only where the box
// is periodic.
template <bool EX, class Put>
__device__ __forceinline__ void flist_columns(const DevSys &s, int ix, int iy, float2 p, int gi, int t,
                                              const WinDelta &wd, const Put &out, int &k) {
    const int ncx = s.ncx, ncy = s.ncy;
    const float R2 = s.nnRadiusSq;
    const float Lx = s.wrapx ? s.Lx : 0.0f, Ly = s.wrapy ? s.Ly : 0.0f;
    const int *cs = s.cellStart;
    const float4 *cand = s.cellSorted;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        int nx = ix + d - 1;
        float sx = 0.0f;
        if (nx < 0) {
            nx = ncx - 1;
            sx = -Lx;
        } else if (nx == ncx) {
            nx = 0;
            sx = Lx;
        }
        const int col = nx * ncy;
        const bool w = wd.win;
        if (iy > 0 && iy < ncy - 1) {
            fwalk<EX, true, true>(cand, __ldg(cs + col + iy - 1), __ldg(cs + col + iy + 2), 0, sx, 0.0f, p, gi, R2,
                                  t, w, wd.dm[d], out, k);
        } else if (iy == 0) {
            fwalk<EX, true, true>(cand, __ldg(cs + col + ncy - 1), __ldg(cs + col + ncy), 0, sx, -Ly, p, gi, R2, t,
                                  w, wd.dw[d], out, k);
            fwalk<EX, true, true>(cand, __ldg(cs + col), __ldg(cs + col + 2), 0, sx, 0.0f, p, gi, R2, t, w,
                                  wd.dm[d], out, k);
        } else {
            fwalk<EX, true, true>(cand, __ldg(cs + col + ncy - 2), __ldg(cs + col + ncy), 0, sx, 0.0f, p, gi, R2, t,
                                  w, wd.dm[d], out, k);
            fwalk<EX, true, true>(cand, __ldg(cs + col), __ldg(cs + col + 1), 0, sx, Ly, p, gi, R2, t, w, wd.dw[d],
                                  out, k);
        }
    }
}

// Any grid and any position: the reference's 3x3 walk with both axes
// wrapped (a grid of one or two cells along an axis visits a cell more than
// once, as the reference does) and the float minimum image per candidate.
// Blocks are never windowed here: entries are storage slots.
template <class Put>
__device__ __forceinline__ void flist_general(const DevSys &s, int ix, int iy, float2 p, int gi, int t,
                                              const Put &out, int &k) {
    const int ncx = s.ncx, ncy = s.ncy;
    const float R2 = s.nnRadiusSq;
    for (int dx = -1; dx <= 1; dx++) {
        int nx = ix + dx;
        if (nx < 0) nx = ncx - 1; else if (nx == ncx) nx = 0;
        for (int dy = -1; dy <= 1; dy++) {
            int ny = iy + dy;
            if (ny < 0) ny = ncy - 1; else if (ny == ncy) ny = 0;
            const int nc = nx * ncy + ny;
            const int qb = __ldg(s.cellStart + nc), qe = __ldg(s.cellStart + nc + 1);
            for (int q = qb; q < qe; q++) {
                const float4 e = __ldg(s.cellSorted + q);
                const int gj = __float_as_int(e.w);
                float dxr, dxo, dyr, dyo;
                image_axis(p.x, e.x, s.Lx, s.wrapx, false, dxr, dxo);
                image_axis(p.y, e.y, s.Ly, s.wrapy, false, dyr, dyo);
                const float dr2 = dxr * dxr + dyr * dyr;
                out.put(q != t && (gi == -1 || gj == -1 || gi != gj) && dr2 <= R2, __float_as_int(e.z), k);
            }
        }
    }
}

// The whole walk of one lane through a Put.  staged: the warp's candidates
// are in w (build window offsets wo, cell slots wb) and the lane's ranges
// are qb..qe; otherwise the column walk or the general walk.
template <class Put>
__device__ __forceinline__ void flist_walk(const DevSys &s, bool fastw, bool staged, bool valid, bool ex, int ix,
                                           int iy, float2 p, int gi, int t, const WinDelta &wd, const float4 *w,
                                           const int *qb, const int *qe, const float *sx, const int *wb,
                                           const int *wo, const Put &out, int &k) {
    if (fastw) {
        if (staged) {
            const float R2 = s.nnRadiusSq;
#pragma unroll
            for (int d = 0; d < 3; d++) {
                // window index q is cell slot q - wo[d] + wb[d] of column d;
                // the staged rows never cross a y edge (main rows only)
                const int lb = wo[d] + qb[d] - wb[d], le = wo[d] + qe[d] - wb[d];
                const int qbase = wb[d] - wo[d];
                const int dv = qbase + wd.dm[d];
                // the same shift on every lane: one cell column
                if (sx[d] != 0.0f) {
                    if (ex) fwalk<true, true, false>(w, lb, le, qbase, sx[d], 0.0f, p, gi, R2, t, wd.win, dv, out, k);
                    else fwalk<false, true, false>(w, lb, le, qbase, sx[d], 0.0f, p, gi, R2, t, wd.win, dv, out, k);
                } else {
                    if (ex) fwalk<true, false, false>(w, lb, le, qbase, 0.0f, 0.0f, p, gi, R2, t, wd.win, dv, out, k);
                    else fwalk<false, false, false>(w, lb, le, qbase, 0.0f, 0.0f, p, gi, R2, t, wd.win, dv, out, k);
                }
            }
        } else if (valid) {
            if (ex) flist_columns<true>(s, ix, iy, p, gi, t, wd, out, k);
            else flist_columns<false>(s, ix, iy, p, gi, t, wd, out, k);
        }
    } else if (valid) {
        flist_general(s, ix, iy, p, gi, t, out, k);
    }
}

// One thread per cell slot t: the Verlet list of the particle stored there,
// written to its storage column.  A warp whose 32 slots lie in one cell
// column away from the y edges stages its three stencil column windows in
// shared memory first.  The free particles' state then moves from the
// scratch arrays to their new slots, with the constant arrays gathered from
// the id-order originals.
__global__ void __launch_bounds__(kLBlock) k_flist(DevSys s, int parity, int check, int skip_windowed) {
    if ((check && !s.sc->rebuild) || s.sc->nonfinite || (s.sc->overflow & 2)) return;
    // skip_windowed: k_flist_p builds the windowed blocks (block = step
    // block: cell slots are storage slots without bonded particles)
    if (skip_windowed && s.blockWin[kWinInts * (size_t)blockIdx.x + kWLen] >= 0) return;
    __shared__ float4 win[kLBlock / 32][kLWin];
    __shared__ int stage[kLBlock / 32][kLStage + 1][32];
    float2 *pos = parity ? s.pos1 : s.pos0;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const bool valid = t < s.N;
    const float4 me = valid ? __ldg(s.cellSorted + t) : make_float4(0.f, 0.f, 0.f, 0.f);
    const int gi = __float_as_int(me.w);
    const int ns = valid ? (__float_as_int(me.z) & kIdMask) : 0;
    const float2 p = make_float2(me.x, me.y);
    int ix, iy;
    cell_xy(me.x, me.y, s.ncx, s.ncy, s.Lx, s.Ly, ix, iy);
    const bool ex = __any_sync(0xffffffffu, valid && gi != -1);
    const bool fastw = fast_walk_ok(s);
    const WinDelta wd = win_delta(s, ns);
    int qb[3] = {0, 0, 0}, qe[3] = {0, 0, 0}, wb[3] = {0, 0, 0}, wo[3] = {0, 0, 0}, wl[3] = {0, 0, 0};
    float sx[3] = {0.f, 0.f, 0.f};
    bool staged = false;
    if (fastw) {
        const int ncy = s.ncy;
        if (valid && iy >= 1 && iy <= ncy - 2) stencil_columns(s, ix, iy, qb, qe, sx);
        const unsigned all = __ballot_sync(0xffffffffu, valid);
        const int ixa = __shfl_sync(0xffffffffu, ix, 0), ixb = __shfl_sync(0xffffffffu, ix, 31);
        const int iya = __shfl_sync(0xffffffffu, iy, 0), iyb = __shfl_sync(0xffffffffu, iy, 31);
        staged = all == 0xffffffffu && ixa == ixb && iya >= 1 && iyb <= ncy - 2;
        if (staged) {
            int tot = 0;
#pragma unroll
            for (int d = 0; d < 3; d++) {
                wb[d] = __shfl_sync(0xffffffffu, qb[d], 0);
                wl[d] = __shfl_sync(0xffffffffu, qe[d], 31) - wb[d];
                wo[d] = tot;
                tot += wl[d];
            }
            staged = tot <= kLWin;
        }
        if (staged) {
            float4 *w = win[wid];
#pragma unroll
            for (int d = 0; d < 3; d++)
                for (int q = lane; q < wl[d]; q += 32) w[wo[d] + q] = __ldg(s.cellSorted + wb[d] + q);
            __syncwarp();
        }
    }
    StagePut sp;
    sp.st = stage[wid];
    sp.lane = lane;
    int k = 0;
    flist_walk(s, fastw, staged, valid, ex, ix, iy, p, gi, t, wd, win[wid], qb, qe, sx, wb, wo, sp, k);
    const int cap = s.nbrCap;
    if (__any_sync(0xffffffffu, valid && k > kLStage && cap > kLStage)) {
        // the rest of an outgrown stage, straight to the list
        DirectPut dp;
        dp.nbr = s.nbr;
        dp.slot = ns;
        dp.cap = cap;
        dp.Ncap = s.Ncap;
        int k2 = 0;
        flist_walk(s, fastw, staged, valid && k > kLStage, ex, ix, iy, p, gi, t, wd, win[wid], qb, qe, sx, wb, wo, dp,
                   k2);
    }
    // the stage to the list: group g of every lane in one store per g; the
    // unused words of the last group name the ghost
    const int ghost = wd.win ? kWinGhost : s.N;
    const int kk = valid ? min(k, cap) : 0;
    const int ng = (kk + 3) >> 2;
    const int ngs = min(ng, kLStage / 4);
    const int gmax = __reduce_max_sync(0xffffffffu, ngs);
    __syncwarp();
    int4 *out = reinterpret_cast<int4 *>(s.nbr) + ns;
    for (int g = 0; g < gmax; g++) {
        if (g < ngs) {
            int v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] = 4 * g + u < kk ? stage[wid][4 * g + u][lane] : ghost;
            out[(size_t)g * s.Ncap] = make_int4(v[0], v[1], v[2], v[3]);
        }
    }
    if (valid && kk > kLStage && (kk & 3)) {
        // a last group past the stage: its unused words
        for (int q = kk; q < 4 * ng; q++) s.nbr[nbr_at(q, ns, s.Ncap)] = ghost;
    }
    if (valid) {
        s.nbrCount[ns] = k;

        if (ns >= s.nBonded) {
            const int id = s.sPerm[ns];
            pos[ns] = s.sPos[ns];
            s.vel[ns] = s.sVel[ns];
            s.acc[ns] = s.sAcc[ns];
            s.perm[ns] = id;
            const_cast<float *>(s.mass)[ns] = __ldg(s.idMass + id);
            if (s.numTypes > 1) const_cast<int *>(s.typeId)[ns] = __ldg(s.idType + id);
            if (!s.sigmaByType) const_cast<float *>(s.sigma)[ns] = __ldg(s.idSigma + id);
            if (s.wallDelta) const_cast<float *>(s.wallDelta)[ns] = __ldg(s.idWallDelta + id);
            if (s.wallSig) const_cast<float *>(s.wallSig)[ns] = __ldg(s.idWallSig + id);
        }
    }
    {
        // the longest list of each step block, one atomic per block a warp touches
        const int blk = valid ? ns / kFastBlock : -1;
        const unsigned peers = __match_any_sync(0xffffffffu, blk);
        const int gm = __reduce_max_sync(peers, ng);
        if (valid && lane == __ffs(peers) - 1) atomicMax(&s.blockWin[kWinInts * (size_t)blk + kWGroups], gm);
    }
    const int kmax = __reduce_max_sync(0xffffffffu, valid ? k : 0);
    const int ksum = __reduce_add_sync(0xffffffffu, valid ? k : 0);
    if (lane == 0) {
        if (ksum) atomicAdd(&s.sc->nbrSum, (unsigned long long)ksum);
        if (kmax > 0) atomicMax(&s.sc->maxCount, kmax);
        if (kmax > s.nbrCap) atomicOr(&s.sc->overflow, 1);
    }
    if (!skip_windowed && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&s.sc->builds, 1ull);
    if (s.trace && lane == 0) {
        const int row = s.sc->obsRow - 1;
        if (row >= 0 && row < s.obsCap) atomicMax(&s.trace[(size_t)row * kTraceCols + 5], global_ns());
    }
}

static cudaError_t launch_flist_p(Launch &L, const DevSys &s, int parity, int check);

cudaError_t enqueue_rebuild_fast(Launch &L, const DevSys &s, int parity, int check) {
    cudaError_t e;
    if (small_bin_fits(s)) {
        // a small system: binning and placement in one block, then the lists
        const size_t smem = small_bin_smem(s);
        int resident = 0;
        if ((e = kernel_setup((const void *)k_fbin_small, kSmallBinThreads, smem, &resident))) return e;
        if ((e = L.kernel(k_fbin_small, dim3(1), dim3(kSmallBinThreads), smem, s, parity, check))) return e;
        return launch_flist_p(L, s, parity, check);
    }
    if ((e = enqueue_bin(L, s, parity, check))) return e;
    const int pb = (s.N + kBlock - 1) / kBlock;
    const int permb = (s.N + kPermBlock - 1) / kPermBlock;
    if ((e = L.kernel(k_fplace, dim3(pb), dim3(kBlock), 0, s, parity, check))) return e;
    if (s.nBonded > 0) {
        if ((e = L.kernel(k_ffree_count, dim3(permb), dim3(kPermBlock), 0, s, check))) return e;
        if ((e = L.kernel(k_fperm, dim3(permb), dim3(kPermBlock), 0, s, parity, check))) return e;
    }
    // without bonded particles the persistent build makes the windows and
    // every list itself
    if (s.nBonded == 0 && s.numTypes == 1) return launch_flist_p(L, s, parity, check);
    const int fb = (s.N + kFastBlock - 1) / kFastBlock;
    if ((e = L.kernel(k_fwindows, dim3((fb + kBlock - 1) / kBlock), dim3(kBlock), 0, s, check))) return e;
    const int nb = (s.N + kLBlock - 1) / kLBlock;
    return L.kernel(k_flist, dim3(nb), dim3(kLBlock), 0, s, parity, check, 0);
}

// ============================================================ step kernel

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// The pair difference on one axis.  IMG: the particle lies within imgD of
// a periodic edge, so an interacting pair may cross it: a difference of
// more than half the box is moved by one box length, rounded once from its
// exact value.
template <bool WRAP, bool IMG>
__device__ __forceinline__ float fdiff(float a, float b, float L) {
    float d = a - b;
    if (WRAP && IMG && fabsf(d) > 0.5f * L) {
        const float sh = d > 0.0f ? L : -L;
        d = (d - sh) + two_sum_err(a, -b, d);
    }
    return d;
}

// One Lennard-Jones pair of particle i (type ti, sigma si) with neighbour
// position q, tag/type tj and sigma sj, added into the running sums.  The
// cutoff test selects the terms (no branch per pair).  One type with sigma
// from the table: A += s6^2, B += s6, n += 1 inside the cutoff; otherwise
// the doubled energy u2 and virial w2 per pair.
template <bool MT, bool SG, bool SIG1, bool WX, bool WY, bool IMG>
__device__ __forceinline__ void fpair(const DevSys &s, const PairEntry *tab, const PairEntry &pe0, int ti, float si,
                                      float2 pi, float qx, float qy, int tj, float sj, float &fx, float &fy, float &A,
                                      float &B, float &n, float &u2, float &w2) {
    const float dx = fdiff<WX, IMG>(pi.x, qx, s.Lx);
    const float dy = fdiff<WY, IMG>(pi.y, qy, s.Ly);
    const float r2 = __fmaf_rn(dx, dx, __fmul_rn(dy, dy));
    float rcut2, c, sig2, eps4, us;
    {
        const PairEntry pe = MT ? tab[ti * s.numTypes + tj] : pe0;
        eps4 = pe.eps4;
        us = pe.us;
        if (SG) {
            const float sij = (si + sj) * 0.5f;
            sig2 = sij * sij;
            rcut2 = pe.rc * pe.rc * sig2;
            c = pe.eps48 * rcp_approx(sig2);
        } else {
            rcut2 = pe.rcut2;
            c = pe.c;
            sig2 = pe.sig2;
        }
    }
    const bool in = r2 < rcut2;
    const float ir2 = in ? ((SIG1 && !SG) ? rcp_approx(r2) : sig2 * rcp_approx(r2)) : 0.0f;
    const float ir4 = ir2 * ir2, ir6 = ir4 * ir2, ir8 = ir4 * ir4;
    const float fc = ir8 * __fmaf_rn(c, ir6, -0.5f * c);
    fx = __fmaf_rn(fc, dx, fx);
    fy = __fmaf_rn(fc, dy, fy);
    if (MT || SG) {
        u2 += in ? __fmaf_rn(eps4, __fmaf_rn(ir6, ir6, -ir6), us) : 0.0f;
        w2 = __fmaf_rn(fc, r2, w2);
    } else {
        A = __fmaf_rn(ir6, ir6, A);
        B += ir6;
        n += in ? 1.0f : 0.0f;
    }
}

// Lennard-Jones forces of particle i over its list (cnt entries).  The
// list's 16-byte groups come from the block's shared copy (slist: its first
// srows groups, one row of kFastBlock groups per group index; the rest from
// global memory) or, with srows = 0, from global memory with the group two
// ahead in flight.  WIN: the entries index the block's staged
// window (wpos, wtyp, wsig); otherwise they are storage slots gathered from
// pin.  Unused words of the last group name the ghost, so no entry needs a
// count test.  Energy and virial come back doubled (per ordered pair), as
// the reference-exact kernel's.
// NC: the positions stay unchanged for the whole launch, so their gathers
// may take the non-coherent path; otherwise (the small-system run, where
// other blocks write them between steps) they are read from L2.
template <bool MT, bool SG, bool SIG1, bool WX, bool WY, bool IMG, bool WIN, bool NC = true>
__device__ __forceinline__ void fast_pairs(const DevSys &s, const PairEntry *tab, int i, float2 pi, int cnt,
                                           const int4 *slist, int srows, const float2 *__restrict__ pin,
                                           const float2 *wpos,
                                           const int *wtyp, const float *wsig, float &fx, float &fy, float &ue2,
                                           float &we2) {
    const int ng = (cnt + 3) >> 2;
    const size_t row = (size_t)s.Ncap;
    const int4 *__restrict__ lst = reinterpret_cast<const int4 *>(s.nbr) + i;
    const int ti = MT ? s.typeId[i] : 0;
    const float si = SG ? s.sigma[i] : 0.0f;
    const PairEntry pe0 = tab[0];
    float A = 0.0f, B = 0.0f, n = 0.0f, u2 = 0.0f, w2 = 0.0f;
    const int4 zero4 = make_int4(0, 0, 0, 0);
    int4 g1 = zero4, g2 = zero4;
    if (srows == 0) {
        g1 = ng > 0 ? __ldg(lst) : zero4;
        g2 = ng > 1 ? __ldg(lst + row) : zero4;
    }
#pragma unroll 1
    for (int gi = 0; gi < ng; gi++) {
        int4 g0;
        if (srows > 0) {
            g0 = gi < srows ? slist[gi * kFastBlock + (threadIdx.x & (kFastBlock - 1))] : __ldg(lst + gi * row);
        } else {
            g0 = g1;
            g1 = g2;
            g2 = gi + 2 < ng ? __ldg(lst + (gi + 2) * row) : zero4;
        }
        int e[4] = {g0.x, g0.y, g0.z, g0.w};
        float2 q[4];
        int tj[4] = {0, 0, 0, 0};
        float sj[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (WIN) {
                // masked to the window: a stray entry can name a wrong
                // window slot but never one outside the shared arrays; the
                // type travels in the entry's high bits
                const int w = (int)min((unsigned)e[u] & (unsigned)kIdMask, (unsigned)(kWinMax - 1));
                q[u] = wpos[w];
                if (MT) tj[u] = (unsigned)e[u] >> kIdBits;
                if (SG) sj[u] = wsig[w];
            } else {
                const int j = MT ? (e[u] & kIdMask) : e[u];
                q[u] = NC ? __ldg(pin + j) : __ldcg(pin + j);
                if (MT) tj[u] = (unsigned)e[u] >> kIdBits;
                if (SG) sj[u] = __ldg(s.sigma + j);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
            fpair<MT, SG, SIG1, WX, WY, IMG>(s, tab, pe0, ti, si, pi, q[u].x, q[u].y, tj[u], sj[u], fx, fy, A, B, n,
                                             u2, w2);
    }
    if (MT || SG) {
        ue2 += u2;
        we2 += w2;
    } else {
        ue2 += __fmaf_rn(pe0.eps4, A - B, pe0.us * n);
        we2 += pe0.eps48 * __fmaf_rn(-0.5f, B, A);
    }
}

// The pair loop of the persistent kernel for a warp with no image work (one
// particle type): the four pairs of a list group are worked two at a time in
// packed float2 arithmetic (lane x of every float2 is one pair, lane y the
// other), the x and y differences in separate float2s.  The pairs inside
// the cutoff are counted as sum ir2 r2 (each term 1 to within the
// reciprocal's rounding, 0 outside the cutoff), the energy shift's weight.
// The exact minimum image of two packed differences d = a - q (one axis, box
// length L): a lane whose |d| exceeds L/2 moves by one box length, rounded
// once from its exact value, (d -+ L) + the TwoSum error of a - q (the
// scalar fdiff's arithmetic, operation for operation); other lanes keep d.
__device__ __forceinline__ float2 img2(float2 d, float2 q, float2 a, float L) {
    const float h = 0.5f * L;
    const bool cx = fabsf(d.x) > h, cy = fabsf(d.y) > h;
    if (!(cx || cy)) return d;
    const float2 m1 = make_float2(-1.0f, -1.0f);
    const float2 bb = __ffma2_rn(a, m1, d);     // d - a
    const float2 t = __ffma2_rn(bb, m1, d);     // d - bb
    const float2 e1 = __ffma2_rn(t, m1, a);     // a - t
    const float2 e2n = __fadd2_rn(q, bb);       // -((-q) - bb)
    const float2 err = __ffma2_rn(e2n, m1, e1); // (a - t) + ((-q) - bb)
    float2 r = d;
    if (cx) r.x = (d.x - (d.x > 0.0f ? L : -L)) + err.x;
    if (cy) r.y = (d.y - (d.y > 0.0f ? L : -L)) + err.y;
    return r;
}

// IMG: a warp at a periodic edge (WX, WY): the packed exact image per pair.
template <bool SIG1, bool WIN, bool W16, bool NC = true, bool IMG = false, bool WX = false, bool WY = false>
__device__ __forceinline__ void fast_pairs_x2(const DevSys &s, const PairEntry &pe, int i, float2 pi, int cnt,
                                              const int4 *slist, int srows, const float2 *__restrict__ pin,
                                              const float2 *wpos, float &fx, float &fy, float &ue2, float &we2) {
    // W16: the group holds eight 16-bit window entries, worked as two halves
    const int ng = W16 ? (cnt + 7) >> 3 : (cnt + 3) >> 2;
    const size_t row = (size_t)s.Ncap;
    const int4 *__restrict__ lst = reinterpret_cast<const int4 *>(s.nbr) + i;
    const float rc2 = pe.rcut2;
    const float2 cv = make_float2(pe.c, pe.c), hcv = make_float2(-0.5f * pe.c, -0.5f * pe.c);
    const float2 sv = make_float2(pe.sig2, pe.sig2), m1 = make_float2(-1.0f, -1.0f);
    const float2 xv = make_float2(pi.x, pi.x), yv = make_float2(pi.y, pi.y);
    const float2 z = make_float2(0.0f, 0.0f);
    float2 FX = z, FY = z, Av = z, Bv = z, Nv = z;
    // four neighbours, two pairs at a time
    auto quad = [&](const float2 *q) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const float2 qa = q[2 * h], qb = q[2 * h + 1];
            const float2 qx = make_float2(qa.x, qb.x), qy = make_float2(qa.y, qb.y);
            float2 dx = __ffma2_rn(qx, m1, xv);
            float2 dy = __ffma2_rn(qy, m1, yv);
            if (IMG && WX) dx = img2(dx, qx, xv, s.Lx);
            if (IMG && WY) dy = img2(dy, qy, yv, s.Ly);
            const float2 r2 = __ffma2_rn(dx, dx, __fmul2_rn(dy, dy));
            float2 ir2 = make_float2(r2.x < rc2 ? rcp_approx(r2.x) : 0.0f, r2.y < rc2 ? rcp_approx(r2.y) : 0.0f);
            if (!SIG1) ir2 = __fmul2_rn(ir2, sv);
            const float2 ir4 = __fmul2_rn(ir2, ir2), ir6 = __fmul2_rn(ir4, ir2), ir8 = __fmul2_rn(ir4, ir4);
            const float2 fc = __fmul2_rn(ir8, __ffma2_rn(cv, ir6, hcv));
            FX = __ffma2_rn(fc, dx, FX);
            FY = __ffma2_rn(fc, dy, FY);
            Av = __ffma2_rn(ir6, ir6, Av);
            Bv = __fadd2_rn(Bv, ir6);
            Nv = __ffma2_rn(ir2, r2, Nv);
        }
    };
#pragma unroll 1
    for (int gi = 0; gi < ng; gi++) {
        const int4 g =
            gi < srows ? slist[gi * kFastBlock + (threadIdx.x & (kFastBlock - 1))] : __ldg(lst + gi * row);
        if (W16) {
            const unsigned wd[4] = {(unsigned)g.x, (unsigned)g.y, (unsigned)g.z, (unsigned)g.w};
#pragma unroll
            for (int hf = 0; hf < 2; hf++) {
                const unsigned e[4] = {wd[2 * hf] & 0xffffu, wd[2 * hf] >> 16, wd[2 * hf + 1] & 0xffffu,
                                       wd[2 * hf + 1] >> 16};
                float2 q[4];
#pragma unroll
                for (int u = 0; u < 4; u++) q[u] = wpos[min(e[u], (unsigned)kWinGhost)];
                quad(q);
            }
        } else {
            const int e[4] = {g.x, g.y, g.z, g.w};
            float2 q[4];
#pragma unroll
            for (int u = 0; u < 4; u++)
                q[u] = WIN ? wpos[min((unsigned)e[u], (unsigned)kWinGhost)]
                           : (NC ? __ldg(pin + e[u]) : __ldcg(pin + e[u]));
            quad(q);
        }
    }
    fx += FX.x + FX.y;
    fy += FY.x + FY.y;
    const float A = Av.x + Av.y, B = Bv.x + Bv.y;
    const float n = SIG1 ? Nv.x + Nv.y : (Nv.x + Nv.y) / pe.sig2;
    ue2 += __fmaf_rn(pe.eps4, A - B, pe.us * n);
    we2 += pe.eps48 * __fmaf_rn(-0.5f, B, A);
}

// x wrapped into [0, L): one box length added or taken away, the reference's
// r - floor(r/L) L for every |r| < 2L (the same single rounding), the full
// expression beyond.
__device__ __forceinline__ float fast_wrap(float x, float L) {
    if (x < 0.0f) x += L;
    else if (x >= L) x -= L;
    if (!(x >= 0.0f && x < L)) x = wrap_coord(x, L);
    return x;
}

// The rest of particle i's step in the fast mode: finish_particle with the
// divisions replaced by the hardware reciprocal (a = f / m), the one-box
// wrap, and the mass and velocity loaded by the caller.
template <bool WX, bool WY>
__device__ __forceinline__ void fast_finish(const DevSys &s, int i, int mode, float2 pi, float m, float2 v,
                                            float2 *pout, float2 *cpout, float fx, float fy, float ue, float we,
                                            float utri,
                                            float uwall, float &ue_out, float &we_out, float &ke, float &vvm,
                                            bool &bad, float2 *xo = nullptr, float2 *vo = nullptr) {
    ue *= 0.5f;
    we *= 0.5f;
    ue += uwall;
    if (s.wallOn) {
        const float yw = wall_y(s, s.sc->stepNow);
        const float dl = s.wallDelta[i];
        const float ht = (pi.y + dl) - yw;
        if (ht > 0.0f) {
            fy -= s.wallK * ht;
            ue += 0.5f * s.wallK * ht * ht;
        }
        const float hb = dl - pi.y;
        if (hb > 0.0f) {
            fy += s.wallK * hb;
            ue += 0.5f * s.wallK * hb * hb;
        }
    }
    bad = bad || !(isfinite(fx) && isfinite(fy));
    const float im = rcp_approx(m);
    const float ax = fx * im, ay = fy * im;
    const float dt = s.dt, hdt = s.hdt;
    if (mode == MODE_FORCES) {
        s.forceOut[i] = make_float2(fx, fy);
        s.energyOut[i] = ue + utri;
    } else if (mode == MODE_INIT) {
        s.acc[i] = make_float2(ax, ay);
        s.forceOut[i] = make_float2(fx, fy);
    } else {
        if (mode == MODE_MID || mode == MODE_LAST) {
            v.x = __fmaf_rn(hdt, ax, v.x);
            v.y = __fmaf_rn(hdt, ay, v.y);
            const float vv = __fmaf_rn(v.x, v.x, __fmul_rn(v.y, v.y));
            vvm = fmaxf(vvm, vv);
            ke = __fmaf_rn(m, vv, ke);
        }
        if (mode == MODE_LAST) {
            s.vel[i] = v;
            s.acc[i] = make_float2(ax, ay);
            s.forceOut[i] = make_float2(fx, fy);
        } else {
            v.x = __fmaf_rn(hdt, ax, v.x);
            v.y = __fmaf_rn(hdt, ay, v.y);
            float2 x = make_float2(__fmaf_rn(dt, v.x, pi.x), __fmaf_rn(dt, v.y, pi.y));
            if (WX) x.x = fast_wrap(x.x, s.Lx);
            if (WY) x.y = fast_wrap(x.y, s.Ly);
            pout[i] = x;
            if (cpout) cpout[s.cslot[i]] = x;  // the cell-ordered mirror
            s.vel[i] = v;
            if (xo) *xo = x;
            if (vo) *vo = v;
        }
    }
    ue_out += ue;
    we_out += we;
}

// ---- asynchronous bulk copies global -> shared (the untiled TMA form) on an
// mbarrier.  Both addresses and the size are multiples of 16 bytes.
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// A wait that gives up: false after 'limit' polls (each of which may itself
// block for a short, hardware-bounded time).
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity, int limit) {
    for (int k = 0; k < limit; k++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// A poll that may suspend the thread in hardware until the phase completes,
// for at most about hint_ns nanoseconds: a waiting thread takes no issue
// slots from the warps that work.
__device__ __forceinline__ bool mbar_try_wait_sleep(unsigned long long *bar, unsigned parity, unsigned hint_ns) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity), "r"(hint_ns)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_sleep(unsigned long long *bar, unsigned parity, int limit,
                                                unsigned hint_ns) {
    for (int k = 0; k < limit; k++)
        if (mbar_try_wait_sleep(bar, parity, hint_ns)) return true;
    return false;
}

constexpr int kWaitLimit = 1 << 22;   // polls before a step block reports a stuck copy
constexpr int kSleepLimit = 1 << 22;  // suspending polls (of at most kSleepNs each) before it does
constexpr unsigned kSleepNs = 256;
constexpr int kFlagTimeout = 8;      // DevScalars::overflow bit: a bounded wait expired

// Resident blocks per SM the register allocation must allow (kFastBlock
// threads each).
#ifndef FEMMD_FAST_MINB
#define FEMMD_FAST_MINB 8
#endif
constexpr int kFastMinBlocks = FEMMD_FAST_MINB;

// The step kernel of the fast mode, one thread per storage slot.  One thread
// of each block starts asynchronous bulk copies of the block's list groups
// (rows > 0: 'rows' rows of kFastBlock groups reserved in shared memory) and,
// for a windowed block of one particle kind whose cell slots are storage
// slots, of its window pieces; the other threads meanwhile load their own
// particle and, where the window was not copied, gather it.  The pair loop
// then reads shared memory only.
template <bool MT, bool SG, bool SIG1, bool WX, bool WY>
__global__ void __launch_bounds__(kFastBlock, kFastMinBlocks) k_fstep(DevSys s, int mode, int parity,
                                                                     cudaGraphConditionalHandle h, int use_h,
                                                                     int rows) {
    const float2 *__restrict__ pin = parity ? s.pos1 : s.pos0;
    float2 *__restrict__ pout = parity ? s.pos0 : s.pos1;
    float2 *cpout = s.cposOn ? (parity ? s.cpos0 : s.cpos1) : nullptr;
    extern __shared__ float4 smem_f4[];
    const int nt = s.numTypes;
    const int ntab = MT ? nt * nt : 1;
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(smem_f4);
    PairEntry *tab = reinterpret_cast<PairEntry *>(smem_f4 + 1);
    int4 *slist = reinterpret_cast<int4 *>(tab + ntab);
    float2 *wpos = reinterpret_cast<float2 *>(slist + (size_t)rows * kFastBlock);
    int *wtyp = reinterpret_cast<int *>(wpos + kWinMax);
    float *wsig = reinterpret_cast<float *>(wtyp + (MT ? kWinMax : 0));
    const int *bw = s.blockWin + kWinInts * (size_t)blockIdx.x;
    const int len = bw[kWLen];
    const int b0 = blockIdx.x * kFastBlock;
    // the window is copied straight from the positions when cell slots are
    // storage slots, else from their cell-ordered mirror
    const bool tmaWin = !SG && len >= 0 && (s.nBonded == 0 || s.cposOn);
    const float2 *wsrc = s.nBonded == 0 ? pin : (parity ? s.cpos1 : s.cpos0);
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        const int G = rows > 0 ? min(bw[kWGroups], rows) : 0;
        const unsigned rowBytes = (unsigned)min(kFastBlock, s.Ncap - b0) * 16u;
        unsigned total = (unsigned)G * rowBytes;
        if (tmaWin)
            for (int p = 0; p < kWinPieces; p++) {
                const int a = bw[kWStart + p], c = bw[kWCount + p];
                if (c > 0) total += (unsigned)(((a + c + 1) & ~1) - (a & ~1)) * 8u;
            }
        mbar_expect_tx(bar, total);
        const int4 *lsrc = reinterpret_cast<const int4 *>(s.nbr) + b0;
        for (int g = 0; g < G; g++) bulk_copy_g2s(slist + g * kFastBlock, lsrc + (size_t)g * s.Ncap, rowBytes, bar);
        if (tmaWin)
            for (int p = 0; p < kWinPieces; p++) {
                const int a = bw[kWStart + p], c = bw[kWCount + p];
                if (c > 0) {
                    const int a0 = a & ~1, e0 = (a + c + 1) & ~1;
                    bulk_copy_g2s(wpos + bw[kWOff + p] - (a & 1), wsrc + a0, (unsigned)(e0 - a0) * 8u, bar);
                }
            }
    }
    // the particle's own data meanwhile
    const int i = b0 + threadIdx.x;
    const bool act = i < s.N;
    const int ic = act ? i : 0;
    const float2 pi = pin[ic];
    const int cnt = act ? min(s.nbrCount[ic], s.nbrCap) : 0;
    const float m = s.mass[ic];
    const float2 v = (mode != MODE_FORCES && mode != MODE_INIT) ? s.vel[ic] : make_float2(0.0f, 0.0f);
    if (MT) {
        for (int q = threadIdx.x; q < nt * nt; q += blockDim.x) tab[q] = s.pair[q];
    } else if (threadIdx.x == 0) {
        tab[0] = s.pair[0];
    }
    if (s.trace && blockIdx.x == 0 && threadIdx.x == 0) {
        const int row = s.sc->obsRow;
        if (row < s.obsCap) s.trace[(size_t)row * kTraceCols + 2] = global_ns();
    }
    if (len >= 0) {
        if (!tmaWin) {
            // the window gathered: cell slots are not storage slots
            for (int p = 0; p < kWinPieces; p++) {
                const int st = bw[kWStart + p], off = bw[kWOff + p], c = bw[kWCount + p];
                for (int w = threadIdx.x; w < c; w += kFastBlock) {
                    const int j = __ldg(s.sortedIds + st + w);
                    wpos[off + w] = __ldg(pin + j);
                    if (SG) wsig[off + w] = s.sigma[j];
                }
            }
        }
        if (threadIdx.x == 0) {
            wpos[kWinGhost] = __ldg(pin + s.N);  // the ghost slot's far position
            if (SG) wsig[kWinGhost] = 1.0f;
        }
    }
    __syncthreads();
    bool ok = mbar_wait_bounded(bar, 0, kWaitLimit);
    if (!ok) {
        // a copy that never completed: report it, give the copies in flight
        // one more bounded wait before the block leaves, skip the pair terms
        atomicOr(&s.sc->overflow, kFlagTimeout);
        mbar_wait_bounded(bar, 0, kWaitLimit);
    }
    float ue = 0.0f, we = 0.0f, ke = 0.0f, vvm = 0.0f;
    bool bad = false;
    float fx = 0.0f, fy = 0.0f, ue2 = 0.0f, we2 = 0.0f, utri = 0.0f, uwall = 0.0f;
    if (act) bonded_forces<WX, WY, true>(s, i, mode, pin, pi, fx, fy, ue2, utri, uwall);
    const float D = s.imgD;
    const bool near = act && ((WX && (pi.x < D || pi.x > s.Lx - D)) || (WY && (pi.y < D || pi.y > s.Ly - D)));
    const bool img = __any_sync(0xffffffffu, near);
    const int srows = rows > 0 ? rows : 0;
    if (act && ok) {
        if (len >= 0) {
            if (img)
                fast_pairs<MT, SG, SIG1, WX, WY, true, true>(s, tab, i, pi, cnt, slist, srows, pin, wpos, wtyp, wsig, fx, fy,
                                                             ue2, we2);
            else
                fast_pairs<MT, SG, SIG1, WX, WY, false, true>(s, tab, i, pi, cnt, slist, srows, pin, wpos, wtyp, wsig, fx, fy,
                                                              ue2, we2);
        } else {
            if (img)
                fast_pairs<MT, SG, SIG1, WX, WY, true, false>(s, tab, i, pi, cnt, slist, srows, pin, wpos, wtyp, wsig, fx, fy,
                                                              ue2, we2);
            else
                fast_pairs<MT, SG, SIG1, WX, WY, false, false>(s, tab, i, pi, cnt, slist, srows, pin, wpos, wtyp, wsig, fx,
                                                               fy, ue2, we2);
        }
    }
    if (act) fast_finish<WX, WY>(s, i, mode, pi, m, v, pout, cpout, fx, fy, ue2, we2, utri, uwall, ue, we, ke, vvm, bad);
    step_reduce<kFastBlock>(s, mode, ue, we, ke, vvm, bad, h, use_h);
}

// Shared memory of a step block: the mbarrier, the pair table, 'rows' rows
// of list groups, the window (positions; types and sigmas where needed).
static size_t fstep_smem(const DevSys &s, bool mt, bool sg, int rows) {
    return 16 + sizeof(PairEntry) * (size_t)(mt ? s.numTypes * s.numTypes : 1) +
           (size_t)rows * kFastBlock * sizeof(int4) +
           (size_t)kWinMax * (sizeof(float2) + (mt ? sizeof(int) : 0) + (sg ? sizeof(float) : 0));
}

constexpr size_t kFastSmemMax = 200 * 1024;  // the list rows stay in global memory beyond this

template <bool MT, bool SG, bool SIG1, bool WX, bool WY>
static cudaError_t launch_fstep(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h,
                                int use_h) {
    const dim3 g((s.N + kFastBlock - 1) / kFastBlock), b(kFastBlock);
    int rows = s.nbrCap / 4;
    if (fstep_smem(s, MT, SG, rows) > kFastSmemMax) rows = 0;
    const size_t smem = fstep_smem(s, MT, SG, rows);
    int resident = 0;
    cudaError_t e = kernel_setup((const void *)k_fstep<MT, SG, SIG1, WX, WY>, kFastBlock, smem, &resident);
    if (e) return e;
    return L.kernel(k_fstep<MT, SG, SIG1, WX, WY>, g, b, smem, s, mode, parity, h, use_h, rows);
}

// ---- the persistent step kernel (one particle kind, no bonded particles).
// Each block holds kFastBlock consumer threads and one producer warp and
// works the tiles (step blocks of kFastBlock storage slots) blockIdx.x,
// blockIdx.x + gridDim.x, ... through two shared-memory stages.  The
// producer's lane 0 copies a tile's list rows and window pieces into a stage
// with asynchronous bulk copies while the consumers work the other stage;
// 'full' barriers carry the copied bytes to the consumers, 'empty' barriers
// (one arrival per consumer warp) hand a stage back.  The consumers load
// their next tile's own particle data while they work the current one, and
// the energies, the largest speed and the finiteness flag are reduced once
// per block.  Every wait is bounded: a wait that gives up sets kFlagTimeout,
// the consumers skip the pair terms from then on, and the producer issues no
// further copy and waits (bounded) for those in flight before it leaves.
constexpr int kPBlock = kFastBlock + 32;  // consumer threads + the producer warp
constexpr int kPRows = 8;                 // list rows staged per tile (the rest read from global memory)
#ifndef FEMMD_FAST_PROWS16
#define FEMMD_FAST_PROWS16 5
#endif
constexpr int kPRows16 = FEMMD_FAST_PROWS16;  // the same with 16-bit entries (8 per row)
#ifndef FEMMD_FAST_PMINB
#define FEMMD_FAST_PMINB 5
#endif
constexpr int kPMinBlocks = FEMMD_FAST_PMINB;
#ifndef FEMMD_FAST_PSTAGES
#define FEMMD_FAST_PSTAGES 2
#endif
constexpr int kPStages = FEMMD_FAST_PSTAGES;  // stages per block: tiles copied ahead of the one worked + 1
static_assert(kPStages >= 2 && kPStages <= 4, "persistent step stages");

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Shared memory of a persistent block: full[kPStages], empty[kPStages], the
// pair table entry, then per stage 'rows' list rows and the window.
__host__ __device__ constexpr size_t pstage_bytes(int rows) {
    return (size_t)rows * kFastBlock * sizeof(int4) + (size_t)kWinMax * sizeof(float2);
}
constexpr size_t kPBarBytes = 2 * kPStages * sizeof(unsigned long long);
__host__ __device__ constexpr size_t pstage_base(int ntab) {
    return ((kPBarBytes + 31) & ~(size_t)31) + (size_t)ntab * sizeof(PairEntry);
}
static size_t pstep_smem(int rows, int ntab) { return pstage_base(ntab) + kPStages * pstage_bytes(rows); }

// A consumer's own particle data of one tile, loaded a tile ahead.
struct PTile {
    float2 p, v;
    float m;
    int cnt, len;
};

__device__ __forceinline__ PTile ptile_load(const DevSys &s, const float2 *__restrict__ pin, int t, int mode) {
    PTile r;
    const int i = t * kFastBlock + (int)threadIdx.x;
    const bool act = i < s.N;
    const int ic = act ? i : 0;
    r.p = __ldg(pin + ic);
    r.cnt = act ? min(__ldg(s.nbrCount + ic), s.nbrCap) : 0;
    r.m = __ldg(s.mass + ic);
    r.v = (mode != MODE_FORCES && mode != MODE_INIT) ? s.vel[ic] : make_float2(0.0f, 0.0f);
    r.len = __ldg(s.blockWin + kWinInts * (size_t)t + kWLen);
    return r;
}

template <bool MT, bool SIG1, bool WX, bool WY>
__global__ void __launch_bounds__(kPBlock, kPMinBlocks) k_fstep_p(DevSys s, int mode, int parity,
                                                                 cudaGraphConditionalHandle h, int use_h, int rows) {
    const float2 *__restrict__ pin = parity ? s.pos1 : s.pos0;
    float2 *__restrict__ pout = parity ? s.pos0 : s.pos1;
    float2 *cpout = s.cposOn ? (parity ? s.cpos0 : s.cpos1) : nullptr;
    extern __shared__ float4 smem_f4[];
    unsigned char *sm = reinterpret_cast<unsigned char *>(smem_f4);
    unsigned long long *full = reinterpret_cast<unsigned long long *>(sm);
    unsigned long long *empty = full + kPStages;
    PairEntry *tab = reinterpret_cast<PairEntry *>(sm + ((kPBarBytes + 31) & ~(size_t)31));
    const int ntab = MT ? s.numTypes * s.numTypes : 1;
    // window source: the positions when cell slots are storage slots, else
    // their cell-ordered mirror
    const float2 *wsrc = s.nBonded == 0 ? pin : (parity ? s.cpos1 : s.cpos0);
    const size_t sb = pstage_bytes(rows);
    // stage q's list rows and window (computed, not indexed from an array:
    // an array indexed by the stage number would live in local memory)
    const size_t base = pstage_base(ntab);
    auto slist_of = [&](int q) { return reinterpret_cast<int4 *>(sm + base + q * sb); };
    auto wpos_of = [&](int q) {
        return reinterpret_cast<float2 *>(sm + base + q * sb + (size_t)rows * kFastBlock * sizeof(int4));
    };
    const int ntiles = (s.N + kFastBlock - 1) / kFastBlock;
    if (threadIdx.x == 0) {
        const float2 g = __ldg(pin + s.N);  // the ghost slot's far position
        for (int q = 0; q < kPStages; q++) {
            mbar_init(&full[q], 1);
            mbar_init(&empty[q], kFastBlock / 32);
            wpos_of(q)[kWinGhost] = g;
        }
        if (!MT) tab[0] = s.pair[0];
        if (s.trace && blockIdx.x == 0) {
            const int row = s.sc->obsRow;
            if (row < s.obsCap) s.trace[(size_t)row * kTraceCols + 2] = global_ns();
        }
    }
    if (MT)
        for (int q = threadIdx.x; q < ntab; q += blockDim.x) tab[q] = s.pair[q];
    __syncthreads();
    float ue = 0.0f, we = 0.0f, ke = 0.0f, vvm = 0.0f;
    bool bad = false;
    if (threadIdx.x >= kFastBlock) {
        // the producer; the window record of its next tile is loaded an
        // iteration ahead, so its latency passes while the producer waits
        // for a free stage
        if (threadIdx.x == kFastBlock) {
            int k = 0;
            bool live = true;
            int wv[kWGroups + 1];
            if (blockIdx.x < ntiles) {
                const int *bw = s.blockWin + kWinInts * (size_t)blockIdx.x;
#pragma unroll
                for (int q = 0; q <= kWGroups; q++) wv[q] = bw[q];
            }
            for (int t = blockIdx.x; t < ntiles; t += gridDim.x, k++) {
                const int st = k % kPStages, use = k / kPStages;
                if (use > 0) {
                    // the stage's last tile: consumed, and its copies landed
                    live = mbar_wait_sleep(&empty[st], (use - 1) & 1, kSleepLimit, kSleepNs) &&
                           mbar_wait_sleep(&full[st], (use - 1) & 1, kSleepLimit, kSleepNs);
                    if (!live) {
                        atomicOr(&s.sc->overflow, kFlagTimeout);
                        break;
                    }
                }
                const int len = wv[kWLen];
                const int b0 = t * kFastBlock;
                const int G = min(wv[kWGroups], rows);
                const unsigned rowBytes = (unsigned)min(kFastBlock, s.Ncap - b0) * 16u;
                unsigned total = (unsigned)G * rowBytes;
                if (len >= 0)
#pragma unroll
                    for (int p = 0; p < kWinPieces; p++) {
                        const int a = wv[kWStart + p], c = wv[kWCount + p];
                        if (c > 0) total += (unsigned)(((a + c + 1) & ~1) - (a & ~1)) * 8u;
                    }
                mbar_expect_tx(&full[st], total);
                const int4 *lsrc = reinterpret_cast<const int4 *>(s.nbr) + b0;
                for (int g = 0; g < G; g++)
                    bulk_copy_g2s(slist_of(st) + g * kFastBlock, lsrc + (size_t)g * s.Ncap, rowBytes, &full[st]);
                if (len >= 0)
#pragma unroll
                    for (int p = 0; p < kWinPieces; p++) {
                        const int a = wv[kWStart + p], c = wv[kWCount + p];
                        if (c > 0) {
                            const int a0 = a & ~1, e0 = (a + c + 1) & ~1;
                            bulk_copy_g2s(wpos_of(st) + wv[kWOff + p] - (a & 1), wsrc + a0, (unsigned)(e0 - a0) * 8u,
                                          &full[st]);
                        }
                    }
                const int tn = t + gridDim.x;
                if (tn < ntiles) {
                    const int *bw = s.blockWin + kWinInts * (size_t)tn;
#pragma unroll
                    for (int q = 0; q <= kWGroups; q++) wv[q] = bw[q];
                }
            }
            if (!live) {
                // copies of the last kPStages tiles issued may still be in
                // flight: a bounded wait each
                for (int kl = k - kPStages; kl < k; kl++)
                    if (kl >= 0)
                        mbar_wait_sleep(&full[kl % kPStages], (kl / kPStages) & 1, kSleepLimit, kSleepNs);
            }
        }
        __syncwarp();
    } else {
        // the consumers
        const int lane = threadIdx.x & 31;
        const float D = s.imgD;
        bool dead = false;
        int t = blockIdx.x;
        PTile nx;
        if (t < ntiles) nx = ptile_load(s, pin, t, mode);
        for (int k = 0; t < ntiles; k++) {
            const PTile cur = nx;
            const int tn = t + gridDim.x;
            if (tn < ntiles) nx = ptile_load(s, pin, tn, mode);
            const int st = k % kPStages;
            bool ok = false;
            if (!dead) {
                ok = mbar_wait_bounded(&full[st], (k / kPStages) & 1, kWaitLimit);
                if (!ok) {
                    dead = true;
                    atomicOr(&s.sc->overflow, kFlagTimeout);
                }
            }
            const int i = t * kFastBlock + threadIdx.x;
            const bool act = i < s.N;
            float fx = 0.0f, fy = 0.0f, ue2 = 0.0f, we2 = 0.0f, utri = 0.0f, uwall = 0.0f;
            if (act) bonded_forces<WX, WY, true>(s, i, mode, pin, cur.p, fx, fy, ue2, utri, uwall);
            const bool near = act && ((WX && (cur.p.x < D || cur.p.x > s.Lx - D)) ||
                                      (WY && (cur.p.y < D || cur.p.y > s.Ly - D)));
            const bool img = __any_sync(0xffffffffu, near);
            if (act && ok) {
                if (MT) {
                    // several types: the scalar loop, each pair's type from its entry
                    if (cur.len >= 0) {
                        if (img)
                            fast_pairs<true, false, false, WX, WY, true, true>(s, tab, i, cur.p, cur.cnt, slist_of(st),
                                                                               rows, pin, wpos_of(st), nullptr,
                                                                               nullptr, fx, fy, ue2, we2);
                        else
                            fast_pairs<true, false, false, WX, WY, false, true>(s, tab, i, cur.p, cur.cnt,
                                                                                slist_of(st), rows, pin, wpos_of(st),
                                                                                nullptr, nullptr, fx, fy, ue2, we2);
                    } else {
                        if (img)
                            fast_pairs<true, false, false, WX, WY, true, false>(s, tab, i, cur.p, cur.cnt,
                                                                                slist_of(st), rows, pin, wpos_of(st),
                                                                                nullptr, nullptr, fx, fy, ue2, we2);
                        else
                            fast_pairs<true, false, false, WX, WY, false, false>(s, tab, i, cur.p, cur.cnt,
                                                                                 slist_of(st), rows, pin,
                                                                                 wpos_of(st), nullptr, nullptr, fx, fy,
                                                                                 ue2, we2);
                    }
                } else if (cur.len >= 0 && s.win16) {
                    if (img)
                        fast_pairs_x2<SIG1, true, true, true, true, WX, WY>(s, tab[0], i, cur.p, cur.cnt,
                                                                            slist_of(st), rows, pin, wpos_of(st), fx,
                                                                            fy, ue2, we2);
                    else
                        fast_pairs_x2<SIG1, true, true>(s, tab[0], i, cur.p, cur.cnt, slist_of(st), rows, pin,
                                                        wpos_of(st), fx, fy, ue2, we2);
                } else if (cur.len >= 0) {
                    if (img)
                        fast_pairs_x2<SIG1, true, false, true, true, WX, WY>(s, tab[0], i, cur.p, cur.cnt,
                                                                             slist_of(st), rows, pin, wpos_of(st), fx,
                                                                             fy, ue2, we2);
                    else
                        fast_pairs_x2<SIG1, true, false>(s, tab[0], i, cur.p, cur.cnt, slist_of(st), rows, pin,
                                                         wpos_of(st), fx, fy, ue2, we2);
                } else {
                    if (img)
                        fast_pairs_x2<SIG1, false, false, true, true, WX, WY>(s, tab[0], i, cur.p, cur.cnt,
                                                                              slist_of(st), rows, pin, wpos_of(st),
                                                                              fx, fy, ue2, we2);
                    else
                        fast_pairs_x2<SIG1, false, false>(s, tab[0], i, cur.p, cur.cnt, slist_of(st), rows, pin,
                                                          wpos_of(st), fx, fy, ue2, we2);
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[st]);
            if (act)
                fast_finish<WX, WY>(s, i, mode, cur.p, cur.m, cur.v, pout, cpout, fx, fy, ue2, we2, utri, uwall, ue, we, ke,
                                    vvm, bad);
            t = tn;
        }
    }
    step_reduce<kPBlock>(s, mode, ue, we, ke, vvm, bad, h, use_h);
}

template <bool MT, bool SIG1, bool WX, bool WY>
static cudaError_t launch_fstep_p(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h,
                                  int use_h) {
    // staged list rows: 16-byte groups of eight 16-bit entries (win16) or
    // four 32-bit ones; longer lists read their last groups from global memory
    const int rows = s.win16 ? std::max(1, std::min((s.nbrCap + 7) / 8, kPRows16))
                             : std::max(1, std::min(s.nbrCap / 4, kPRows));
    const size_t smem = pstep_smem(rows, MT ? s.numTypes * s.numTypes : 1);
    auto kern = k_fstep_p<MT, SIG1, WX, WY>;
    int resident = 0;
    cudaError_t e = kernel_setup((const void *)kern, kPBlock, smem, &resident);
    if (e) return e;
    const int ntiles = (s.N + kFastBlock - 1) / kFastBlock;
    const int grid = std::max(1, std::min(ntiles, std::max(1, resident)));
    return L.kernel(kern, dim3(grid), dim3(kPBlock), smem, s, mode, parity, h, use_h, rows);
}

template <bool MT, bool SIG1>
static cudaError_t fstep_p_image(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h,
                                 int use_h) {
    if (s.wrapx && s.wrapy) return launch_fstep_p<MT, SIG1, true, true>(L, s, mode, parity, h, use_h);
    if (s.wrapx) return launch_fstep_p<MT, SIG1, true, false>(L, s, mode, parity, h, use_h);
    return launch_fstep_p<MT, SIG1, false, false>(L, s, mode, parity, h, use_h);
}

// ---- the persistent list build (systems without bonded particles).
// The windowed step blocks' lists (k_fwindows) are built here, k_flist
// builds the others.  A block holds kFastBlock consumer threads, one per
// slot of a tile, and a producer warp; tiles blockIdx.x, blockIdx.x +
// gridDim.x, ... pass through two shared-memory stages.  The producer's lane
// 0 copies, with asynchronous bulk copies, a tile's window pieces of
// cellSorted and the cell starts of the rows those pieces cover into a stage,
// with a header (tile, window deltas, where each piece's cell starts sit).
// A consumer finds its own particle in the window, walks its stencil
// ranges there (the reference's float dr^2 <= (rc + skin)^2, as k_flist),
// stages its entries (window indices) in its own column of a per-block
// [entry][slot] array, stores them as 16-byte groups and copies the
// reordered state of its slot back from the scratch arrays.  Waits are
// bounded as in k_fstep_p.
constexpr int kLPMinBlocks = 5;
constexpr int kLPCs = 512;   // cell-start words per stage
constexpr int kLPHdr = 32;   // header words per stage
// header word offsets
constexpr int kHT = 0, kHLen = 1, kHTwo = 2, kHCol0 = 3, kHCsOk = 4, kHDelta = 5, kHCsb = kHDelta + kWinPieces,
              kHColp = kHCsb + kWinPieces;
static_assert(kHColp + kWinPieces <= kLPHdr, "list-build stage header");

__host__ __device__ constexpr size_t lp_stage_bytes() {
    return (size_t)kLPHdr * 4 + (size_t)kLPCs * 4 + (size_t)kWinMax * sizeof(float4);
}
static size_t lp_smem() {
    return 32 + 2 * lp_stage_bytes() + (size_t)(kLStage + 1) * kFastBlock * sizeof(unsigned short);
}

// the consumers' entry stage (window indices fit 16 bits): column = the
// thread's slot in the tile
struct TileStagePut {
    unsigned short (*st)[kFastBlock];  // [kLStage + 1][kFastBlock]
    int col;
    __device__ __forceinline__ void put(bool hit, int val, int &k) const {
        if (hit) st[min(k, kLStage)][col] = (unsigned short)val;
        k += hit ? 1 : 0;
    }
};

// Window candidates [wb, we) of a lane at p whose own window entry is self,
// with the image shift (sx, sy) where SX / SY; the entry is the window
// index.  The lane's own particle appears once among its ranges (no stencil
// row of the lane repeats its own row), at entry self.
template <bool SX, bool SY, class Put>
__device__ __forceinline__ void lp_walk(const float4 *wc, int wb, int we, float sx, float sy, float2 p, int self,
                                        float R2, const Put &out, int &k) {
    wb = min(max(wb, 0), kWinMax);
    we = min(max(we, wb), kWinMax);
    auto one = [&](int w) {
        const float4 e = wc[w];
        const float dx = SX ? (p.x - e.x) - sx : p.x - e.x;
        const float dy = SY ? (p.y - e.y) - sy : p.y - e.y;
        const float dr2 = dx * dx + dy * dy;
        out.put(dr2 <= R2 && w != self, w, k);
    };
    int w = wb;
#pragma unroll 1
    for (; w + 1 < we; w += 2) {
        one(w);
        one(w + 1);
    }
    if (w < we) one(w);
}

template <class Put>
__device__ __forceinline__ void lp_range(const float4 *wc, int wb, int we, float sx, float sy, float2 p, int self,
                                         float R2, const Put &out, int &k) {
    if (sx == 0.0f && sy == 0.0f) lp_walk<false, false>(wc, wb, we, 0.0f, 0.0f, p, self, R2, out, k);
    else lp_walk<true, true>(wc, wb, we, sx, sy, p, self, R2, out, k);
}

// The ranges of stencil column d (cell column ix + d - 1) of a lane (cell
// (ix, iy), own column j of the tile).
template <class Put>
__device__ __forceinline__ void lp_stencil_col(const DevSys &s, const int *hd, const int *csm, const float4 *wc,
                                               int ix, int iy, int j, float2 p, int self, int d, const Put &out,
                                               int &k) {
    const int ncx = s.ncx, ncy = s.ncy;
    const float R2 = s.nnRadiusSq;
    const float Lx = s.wrapx ? s.Lx : 0.0f, Ly = s.wrapy ? s.Ly : 0.0f;
    const bool two = hd[kHTwo] != 0, csok = hd[kHCsOk] != 0;
    // the cell start of row r of piece q's column
    // (indices clamped to the staged words: a record that disagreed with the
    // cells could give wrong entries, never an access outside the stage)
    auto cs = [&](int q, int r) {
        return csok ? csm[min(max(hd[kHCsb + q] + hd[kHColp + q] + r, 0), kLPCs - 1)]
                    : __ldg(s.cellStart + hd[kHColp + q] + r);
    };
    const int pm = !two ? 2 * d : (j == 0 ? 2 * d + 1 : 2 * d + 2);
    const int pw = !two ? 2 * d + 1 : (j == 0 ? 2 * d : 2 * d + 3);
    const int nx = ix + d - 1;
    const float sx = nx < 0 ? -Lx : (nx == ncx ? Lx : 0.0f);
    const int dm = hd[kHDelta + pm], dw = hd[kHDelta + pw];
    if (iy > 0 && iy < ncy - 1) {
        lp_range(wc, cs(pm, iy - 1) + dm, cs(pm, iy + 2) + dm, sx, 0.0f, p, self, R2, out, k);
    } else if (iy == 0) {
        lp_range(wc, cs(pw, ncy - 1) + dw, cs(pw, ncy) + dw, sx, -Ly, p, self, R2, out, k);
        lp_range(wc, cs(pm, 0) + dm, cs(pm, 2) + dm, sx, 0.0f, p, self, R2, out, k);
    } else {
        lp_range(wc, cs(pm, ncy - 2) + dm, cs(pm, ncy) + dm, sx, 0.0f, p, self, R2, out, k);
        lp_range(wc, cs(pw, 0) + dw, cs(pw, 1) + dw, sx, Ly, p, self, R2, out, k);
    }
}

// All stencil ranges of a lane, column by column.
template <class Put>
__device__ __forceinline__ void lp_stencil(const DevSys &s, const int *hd, const int *csm, const float4 *wc, int ix,
                                           int iy, int j, float2 p, int self, const Put &out, int &k) {
#pragma unroll
    for (int d = 0; d < 3; d++) lp_stencil_col(s, hd, csm, wc, ix, iy, j, p, self, d, out, k);
}

// The cell-start words a windowed tile's stage takes (window record bw): a
// stage holds them when they are at most kLPCs.
__device__ __forceinline__ int lp_cs_words(const DevSys &s, const int *bw) {
    int used = 0;
#pragma unroll
    for (int p = 0; p < kWinPieces; p++) {
        const int ra = bw[kWRow0 + p], rb = bw[kWRow1 + p];
        if (rb >= ra) {
            int nx = bw[kWCol0] + (p >> 1) - 1;
            if (nx < 0) nx += s.ncx;
            else if (nx >= s.ncx) nx -= s.ncx;
            const int colp = nx * s.ncy;
            used += ((colp + rb + 2 + 3) & ~3) - ((colp + ra) & ~3);
        }
    }
    return used;
}

// The stage of a windowed tile (window record bw, len >= 0): the header
// rest (the caller wrote kHT and kHLen), then, on bar, bulk copies of the
// window pieces of cellSorted and of the cell starts of the rows they cover.
__device__ __forceinline__ void lp_issue(const DevSys &s, const int *bw, int *hd, int *csm, float4 *wc,
                                         unsigned long long *bar) {
    const int ncx = s.ncx, ncy = s.ncy;
    const int col0 = bw[kWCol0];
    hd[kHTwo] = bw[kWTwo];
    hd[kHCol0] = col0;
    // first pass: sizes, where each piece's cell starts go
    int used = 0;
    unsigned total = 0;
    int a0s[kWinPieces], nws[kWinPieces];
#pragma unroll
    for (int p = 0; p < kWinPieces; p++) {
        int nx = col0 + (p >> 1) - 1;
        if (nx < 0) nx += ncx;
        else if (nx >= ncx) nx -= ncx;
        const int colp = nx * ncy;
        const int ra = bw[kWRow0 + p], rb = bw[kWRow1 + p];
        hd[kHColp + p] = colp;
        hd[kHDelta + p] = bw[kWOff + p] - bw[kWStart + p];
        a0s[p] = 0;
        nws[p] = 0;
        if (rb >= ra) {
            const int a0 = (colp + ra) & ~3, e0 = (colp + rb + 2 + 3) & ~3;
            a0s[p] = a0;
            nws[p] = e0 - a0;
            hd[kHCsb + p] = used - a0;
            used += e0 - a0;
        }
        total += (unsigned)bw[kWCount + p] * 16u;
    }
    const bool csok = used <= kLPCs;
    hd[kHCsOk] = csok ? 1 : 0;
    if (csok) total += (unsigned)used * 4u;
    mbar_expect_tx(bar, total);
#pragma unroll
    for (int p = 0; p < kWinPieces; p++) {
        const int c = bw[kWCount + p];
        if (c > 0) bulk_copy_g2s(wc + bw[kWOff + p], s.cellSorted + bw[kWStart + p], (unsigned)c * 16u, bar);
        if (csok && nws[p] > 0)
            bulk_copy_g2s(csm + (hd[kHCsb + p] + a0s[p]), s.cellStart + a0s[p], (unsigned)nws[p] * 4u, bar);
    }
}

__global__ void __launch_bounds__(kPBlock, kLPMinBlocks) k_flist_p(DevSys s, int parity, int check) {
    if ((check && !s.sc->rebuild) || s.sc->nonfinite || (s.sc->overflow & 2)) return;
    float2 *pos = parity ? s.pos1 : s.pos0;
    extern __shared__ float4 smem_f4[];
    unsigned char *sm = reinterpret_cast<unsigned char *>(smem_f4);
    unsigned long long *full = reinterpret_cast<unsigned long long *>(sm);
    unsigned long long *empty = full + 2;
    auto hdr_of = [&](int q) { return reinterpret_cast<int *>(sm + 32 + q * lp_stage_bytes()); };
    auto cs_of = [&](int q) { return reinterpret_cast<int *>(sm + 32 + q * lp_stage_bytes() + kLPHdr * 4); };
    auto wc_of = [&](int q) {
        return reinterpret_cast<float4 *>(sm + 32 + q * lp_stage_bytes() + kLPHdr * 4 + kLPCs * 4);
    };
    unsigned short(*ost)[kFastBlock] =
        reinterpret_cast<unsigned short(*)[kFastBlock]>(sm + 32 + 2 * lp_stage_bytes());
    const int ntiles = (s.N + kFastBlock - 1) / kFastBlock;
    if (threadIdx.x == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        mbar_init(&empty[0], kFastBlock / 32);
        mbar_init(&empty[1], kFastBlock / 32);
        if (blockIdx.x == 0) atomicAdd(&s.sc->builds, 1ull);
    }
    __syncthreads();
    if (threadIdx.x >= kFastBlock) {
        // the producer
        if (threadIdx.x == kFastBlock) {
            // the window record of a tile is made (fwindow_record) an
            // iteration before its copies are issued, so its loads pass
            // while the producer waits for a free stage
            int k = 0;
            bool live = true;
            if (blockIdx.x < ntiles) fwindow_record(s, blockIdx.x);
            for (int t = blockIdx.x; t < ntiles; t += gridDim.x, k++) {
                const int st = k & 1, use = k >> 1;
                if (use > 0) {
                    live = mbar_wait_sleep(&empty[st], (use - 1) & 1, kSleepLimit, kSleepNs) &&
                           mbar_wait_sleep(&full[st], (use - 1) & 1, kSleepLimit, kSleepNs);
                    if (!live) {
                        atomicOr(&s.sc->overflow, kFlagTimeout);
                        break;
                    }
                }
                const int *bw = s.blockWin + kWinInts * (size_t)t;
                int *hd = hdr_of(st);
                const int len = bw[kWLen];
                hd[kHT] = t;
                hd[kHLen] = len;
                const int tn = t + gridDim.x;
                if (len < 0) {
                    mbar_expect_tx(&full[st], 0u);  // a block the consumers walk in global memory
                    if (tn < ntiles) fwindow_record(s, tn);
                    continue;
                }
                lp_issue(s, bw, hd, cs_of(st), wc_of(st), &full[st]);
                if (tn < ntiles) fwindow_record(s, tn);
            }
            if (!live) {
                for (int kl = k - 2; kl < k; kl++)
                    if (kl >= 0) mbar_wait_sleep(&full[kl & 1], (kl >> 1) & 1, kSleepLimit, kSleepNs);
            }
        }
        __syncwarp();
        return;
    }
    // the consumers
    const int lane = threadIdx.x & 31;
    const int cap = s.nbrCap;
    TileStagePut sp;
    sp.st = ost;
    sp.col = threadIdx.x;
    for (int t = blockIdx.x, k = 0; t < ntiles; t += gridDim.x, k++) {
        const int st = k & 1;
        if (!mbar_wait_sleep(&full[st], (k >> 1) & 1, kSleepLimit, kSleepNs)) {
            atomicOr(&s.sc->overflow, kFlagTimeout);
            break;
        }
        const int *hd = hdr_of(st);
        const bool win = hd[kHLen] >= 0;
        const int slot = t * kFastBlock + threadIdx.x;
        const bool valid = slot < s.N;
        // the reordered state of the slot, back from the scratch arrays
        // (loaded now, stored at the end)
        const int sl = valid ? slot : 0;
        const int id = __ldg(s.sPerm + sl);
        const float2 np = __ldg(s.sPos + sl), nv = __ldg(s.sVel + sl), na = __ldg(s.sAcc + sl);
        const int *csm = cs_of(st);
        const float4 *wc = wc_of(st);
        const bool two = win && hd[kHTwo] != 0;
        // the lane's cell column in the tile: the upper column's slots
        // start at row 0 of window column 2 (piece 4)
        int j = 0;
        if (two) {
            const int bnd = hd[kHCsOk] ? csm[min(max(hd[kHCsb + 4] + hd[kHColp + 4], 0), kLPCs - 1)]
                                       : __ldg(s.cellStart + hd[kHColp + 4]);
            j = slot >= bnd ? 1 : 0;
        }
        const int pown = !two ? 2 : (j == 0 ? 3 : 4);
        int kk = 0;
        if (!win) {
            // no window: the lane's stencil straight from global memory,
            // entries (storage slots) written straight to the list
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[st]);
            if (valid) {
                const float4 me = __ldg(s.cellSorted + slot);
                int ix, iy;
                cell_xy(me.x, me.y, s.ncx, s.ncy, s.Lx, s.Ly, ix, iy);
                const float2 p = make_float2(me.x, me.y);
                ListPut lp;
                lp.nbr = s.nbr;
                lp.slot = slot;
                lp.cap = cap;
                lp.Ncap = s.Ncap;
                if (fast_walk_ok(s)) {
                    WinDelta wd;
                    wd.win = false;
                    wd.len = -1;
#pragma unroll
                    for (int d = 0; d < 3; d++) wd.dm[d] = wd.dw[d] = 0;
                    flist_columns<false>(s, ix, iy, p, -1, slot, wd, lp, kk);
                } else {
                    flist_general(s, ix, iy, p, -1, slot, lp, kk);
                }
            }
        } else if (valid) {
            const int self = min(max(slot + hd[kHDelta + pown], 0), kWinMax - 1);
            const float4 me = wc[self];
            int ix, iy;
            cell_xy(me.x, me.y, s.ncx, s.ncy, s.Lx, s.Ly, ix, iy);
            const float2 p = make_float2(me.x, me.y);
            lp_stencil(s, hd, csm, wc, ix, iy, j, p, self, sp, kk);
            if (kk > kLStage && cap > kLStage) {
                int k2 = 0;
                if (s.win16) {
                    DirectPut16 dp;
                    dp.nbr16 = reinterpret_cast<unsigned short *>(s.nbr);
                    dp.slot = slot;
                    dp.cap = cap;
                    dp.Ncap = s.Ncap;
                    lp_stencil(s, hd, csm, wc, ix, iy, j, p, self, dp, k2);
                } else {
                    DirectPut dp;
                    dp.nbr = s.nbr;
                    dp.slot = slot;
                    dp.cap = cap;
                    dp.Ncap = s.Ncap;
                    lp_stencil(s, hd, csm, wc, ix, iy, j, p, self, dp, k2);
                }
            }
        }
        const int kc = valid ? min(kk, cap) : 0;
        // groups of the list: eight 16-bit window entries with win16, else
        // four 32-bit entries
        const bool w16 = win && s.win16;
        const int ng = w16 ? (kc + 7) >> 3 : (kc + 3) >> 2;
        if (w16) {
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[st]);
            const int ngs = min(ng, kLStage / 8);
            const int gmax = __reduce_max_sync(0xffffffffu, ngs);
            int4 *out = reinterpret_cast<int4 *>(s.nbr) + slot;
            for (int g = 0; g < gmax; g++) {
                if (g < ngs) {
                    int v[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int k0 = 8 * g + 2 * u;
                        const unsigned lo = k0 < kc ? ost[k0][threadIdx.x] : kWinGhost;
                        const unsigned hi = k0 + 1 < kc ? ost[k0 + 1][threadIdx.x] : kWinGhost;
                        v[u] = (int)(lo | hi << 16);
                    }
                    out[(size_t)g * s.Ncap] = make_int4(v[0], v[1], v[2], v[3]);
                }
            }
            if (valid && kc > kLStage && (kc & 7)) {
                unsigned short *n16 = reinterpret_cast<unsigned short *>(s.nbr);
                for (int q = kc; q < 8 * ng; q++) n16[nbr16_at(q, slot, s.Ncap)] = (unsigned short)kWinGhost;
            }
        } else if (win) {
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[st]);
            // the stage to the list: group g of every lane in one store per g
            const int ngs = min(ng, kLStage / 4);
            const int gmax = __reduce_max_sync(0xffffffffu, ngs);
            int4 *out = reinterpret_cast<int4 *>(s.nbr) + slot;
            for (int g = 0; g < gmax; g++) {
                if (g < ngs) {
                    int v[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) v[u] = 4 * g + u < kc ? (int)ost[4 * g + u][threadIdx.x] : kWinGhost;
                    out[(size_t)g * s.Ncap] = make_int4(v[0], v[1], v[2], v[3]);
                }
            }
            if (valid && kc > kLStage && (kc & 3))
                for (int q = kc; q < 4 * ng; q++) s.nbr[nbr_at(q, slot, s.Ncap)] = kWinGhost;
        } else if (valid) {
            // unused words of the last group name the ghost slot
            for (int q = kc; q < 4 * ng; q++) s.nbr[nbr_at(q, slot, s.Ncap)] = s.N;
        }
        if (valid) {
            s.nbrCount[slot] = kk;
            pos[slot] = np;
            s.vel[slot] = nv;
            s.acc[slot] = na;
            s.perm[slot] = id;
            const_cast<float *>(s.mass)[slot] = __ldg(s.idMass + id);
            if (s.numTypes > 1) const_cast<int *>(s.typeId)[slot] = __ldg(s.idType + id);
            if (!s.sigmaByType) const_cast<float *>(s.sigma)[slot] = __ldg(s.idSigma + id);
            if (s.wallDelta) const_cast<float *>(s.wallDelta)[slot] = __ldg(s.idWallDelta + id);
            if (s.wallSig) const_cast<float *>(s.wallSig)[slot] = __ldg(s.idWallSig + id);
        }
        const int gm = __reduce_max_sync(0xffffffffu, ng);
        const int kmax = __reduce_max_sync(0xffffffffu, valid ? kk : 0);
        const int ksum = __reduce_add_sync(0xffffffffu, valid ? kk : 0);
        if (lane == 0) {
            atomicMax(&s.blockWin[kWinInts * (size_t)t + kWGroups], gm);
            if (ksum) atomicAdd(&s.sc->nbrSum, (unsigned long long)ksum);
            if (kmax > 0) atomicMax(&s.sc->maxCount, kmax);
            if (kmax > cap) atomicOr(&s.sc->overflow, 1);
            if (s.trace) {
                const int row = s.sc->obsRow - 1;
                if (row >= 0 && row < s.obsCap) atomicMax(&s.trace[(size_t)row * kTraceCols + 5], global_ns());
            }
        }
    }
}

static cudaError_t launch_flist_p(Launch &L, const DevSys &s, int parity, int check) {
    const size_t smem = lp_smem();
    int resident = 0;
    cudaError_t e = kernel_setup((const void *)k_flist_p, kPBlock, smem, &resident);
    if (e) return e;
    const int ntiles = (s.N + kFastBlock - 1) / kFastBlock;
    const int grid = std::max(1, std::min(ntiles, std::max(1, resident)));
    return L.kernel(k_flist_p, dim3(grid), dim3(kPBlock), smem, s, parity, check);
}

template <bool MT, bool SG, bool SIG1>
static cudaError_t fstep_image(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h,
                               int use_h) {
    if (s.wrapx && s.wrapy) return launch_fstep<MT, SG, SIG1, true, true>(L, s, mode, parity, h, use_h);
    if (s.wrapx) return launch_fstep<MT, SG, SIG1, true, false>(L, s, mode, parity, h, use_h);
    return launch_fstep<MT, SG, SIG1, false, false>(L, s, mode, parity, h, use_h);
}

// ---- the small-system run (one particle kind, sigma by type, no bonded
// particles, walls, gravity or area springs; a few step blocks).  At this
// size a step kernel lasts a few microseconds and a graph node or a launch
// costs as much again, so k_fsmall advances a run's middle steps in one
// cooperative launch: one block per step block (tile), the tile's list rows
// kept in shared memory, per step the window copied in, the pair terms and
// the leapfrog of k_fstep_p, then a bounded grid-wide exchange after which
// every block takes the same rebuild decision from the same maximum.  A
// rebuild happens inside the launch too (small_rebuild: the binning, the
// in-cell placement, the window records and the lists of k_fbin_small and
// k_flist_p, in four exchanges).  Where that cannot be done (a tile without
// a window, or one whose cell starts overflow a stage) the launch ends with
// the rebuild pending and the rebuild kernels run; a neighbour-list overflow
// or a non-finite position ends it too (the run is then repeated or fails).
// The number of steps done goes to DevScalars::smallDone.
//
// The exchange: each block writes a record {tag << 32 | word, U, W, K} (word:
// its max v^2 bits after a step, flag bits during a rebuild; U, W, K: its
// fixed-point energy sums) into one of three record sets, the tag word last
// with release semantics, and warp 0 of every block waits until all tag
// words carry the exchange's tag (acquire), taking the largest word as a
// float and the OR of the words.  Block 0 sums a step's fixed-point records
// (exact integer sums: the same totals as the step kernels' atomics) during
// the next exchange, while it waits.  Set j is written again at exchange
// j + 3, which no block reaches before block 0 has published exchange j + 2,
// after those sums.  Tags grow by one per exchange (DevScalars::gbTag holds
// the next launch's base).
constexpr int kGridSpin = 1 << 20;  // polls of one record (about 0.5 us each) before an exchange gives up

__device__ __forceinline__ void st_release_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// This block's record of exchange 'tag' (record set par), then the wait of
// warp 0 for every block's: xsh[0] = 1 (0 when a wait gave up), xsh[1] = the
// OR of the words, xsh[2] = their maximum as a float.  withhold: the record
// is not written (femmd_test_expire_next_exchange: every wait gives up).
// Call after a __syncthreads that follows the block's stores.
__device__ __forceinline__ void small_exchange(const DevSys &s, unsigned tag, int par, unsigned long long qu,
                                               unsigned long long qw, unsigned long long qk, unsigned word,
                                               unsigned *xsh, bool withhold) {
    unsigned long long *set = s.smallRec + (size_t)par * kSmallMaxTiles * 4;
    const int lane = threadIdx.x & 31;
    if (threadIdx.x == 0 && !withhold) {
        unsigned long long *r = set + 4 * (size_t)blockIdx.x;
        r[1] = qu;
        r[2] = qw;
        r[3] = qk;
        st_release_u64(r, ((unsigned long long)tag << 32) | word);
    }
    if (threadIdx.x < 32) {
        float m = 0.0f;
        unsigned orw = 0u;
        int ok = 1;
        for (int b = lane; b < (int)gridDim.x && ok; b += 32) {
            const unsigned long long *w = set + 4 * (size_t)b;
            unsigned long long x = ld_acquire_u64(w);
            int it = 0;
            while ((unsigned)(x >> 32) != tag) {
                if (++it > kGridSpin) {
                    ok = 0;
                    break;
                }
                __nanosleep(32);
                x = ld_acquire_u64(w);
            }
            if (ok) {
                m = fmaxf(m, __uint_as_float((unsigned)x));
                orw |= (unsigned)x;
            }
        }
        ok = __all_sync(0xffffffffu, ok);
        m = warp_max(m);
        orw = __reduce_or_sync(0xffffffffu, orw);
        if (lane == 0) {
            xsh[0] = (unsigned)ok;
            xsh[1] = orw;
            xsh[2] = __float_as_uint(m);
        }
    }
}

// Block 0, warp 1: the totals of an earlier step's records (set par), into
// the scalars and the observable row of that step.
__device__ __forceinline__ void small_totals(const DevSys &s, int par, float vm2, float d, int r, int row) {
    const unsigned long long *set = s.smallRec + (size_t)par * kSmallMaxTiles * 4;
    const int lane = threadIdx.x & 31;
    unsigned long long su = 0ull, sw = 0ull, sk = 0ull;
    for (int b = lane; b < (int)gridDim.x; b += 32) {
        su += __ldcg(set + 4 * (size_t)b + 1);
        sw += __ldcg(set + 4 * (size_t)b + 2);
        sk += __ldcg(set + 4 * (size_t)b + 3);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        su += __shfl_down_sync(0xffffffffu, su, o);
        sw += __shfl_down_sync(0xffffffffu, sw, o);
        sk += __shfl_down_sync(0xffffffffu, sk, o);
    }
    if (lane == 0) {
        DevScalars *sc = s.sc;
        const double U = from_fixed(su), W = from_fixed(sw), KE = from_fixed(sk);
        sc->U = U;
        sc->W = W;
        sc->KE = KE;
        sc->vvMax = vm2;
        if (s.obs && row < s.obsCap) {
            double *o = s.obs + (size_t)row * kObsCols;
            o[0] = U;
            o[1] = W;
            o[2] = KE;
            o[3] = (double)vm2;
            o[4] = (double)d;
            o[5] = (double)r;
        }
    }
}

// k_fsmall's threads: one per storage slot of the tile for the steps; three
// per slot (one per stencil column) for the list walk of a rebuild
constexpr int kSmallThreads = 3 * kFastBlock;

// Shared memory of k_fsmall: scalars, the list rows, the step window, the
// list build's stage (header, cell starts, window of cellSorted), an entry
// stage and a count per stencil column, and the cell starts of the binning.
constexpr size_t kSmHdr = 512;
__host__ __device__ constexpr size_t small_smem(int rows, int ncells) {
    return kSmHdr + (size_t)rows * kFastBlock * sizeof(int4) + (size_t)kWinMax * sizeof(float2) +
           lp_stage_bytes() + 3 * (size_t)(kLStage + 1) * kFastBlock * sizeof(unsigned short) +
           3 * (size_t)kFastBlock * sizeof(int) + (((size_t)ncells + 1 + 3) & ~(size_t)3) * sizeof(int);
}

// Rebuild outcomes inside the small run
constexpr int kSmallRebuilt = 0, kSmallStop = 1, kSmallPending = 2;

// The state a thread of k_fsmall carries between steps and rebuilds.
struct SmallSlot {
    float2 pi, v;   // position and velocity of the thread's storage slot
    float m;        // its mass
    int id, excl;   // its particle id and exclusion group
    int cnt;        // its list length
};

// The tile's list rows and window record (from the global list and
// blockWin; the L2 copy, since this launch may have written them).
__device__ __forceinline__ void small_load_tile(const DevSys &s, int rows, int4 *slist, int *wrec, int &G) {
    const int t = blockIdx.x;
    const int *bw = s.blockWin + kWinInts * (size_t)t;
    for (int q = threadIdx.x; q < kWinInts; q += blockDim.x) wrec[q] = __ldcg(bw + q);
    __syncthreads();
    G = min(wrec[kWGroups], rows);
    const int i = t * kFastBlock + threadIdx.x;
    const int4 *lrow = reinterpret_cast<const int4 *>(s.nbr) + (size_t)t * kFastBlock + threadIdx.x;
    if (threadIdx.x < kFastBlock && i < s.Ncap)
        for (int g = 0; g < G; g++) slist[g * kFastBlock + threadIdx.x] = __ldcg(lrow + (size_t)g * s.Ncap);
}

// Window bytes a step copies (16-byte spans of the record's pieces).
__device__ __forceinline__ unsigned small_win_bytes(const int *wrec) {
    unsigned b = 0;
    if (wrec[kWLen] >= 0)
        for (int q = 0; q < kWinPieces; q++) {
            const int a = wrec[kWStart + q], c = wrec[kWCount + q];
            if (c > 0) b += (unsigned)(((a + c + 1) & ~1) - (a & ~1)) * 8u;
        }
    return b;
}

// Steps come from DevScalars::smallLeft and the start parity from
// DevScalars::smallPar; a launch ends with the positions in pos0 (parity 0),
// so that a rebuild that may follow it has a fixed parity.  use_h: inside the run graph, set its WHILE (steps left) and
// IF (rebuild pending) conditions.
template <bool SIG1, bool WX, bool WY>
__global__ void __launch_bounds__(kSmallThreads, 1) k_fsmall(DevSys s, int rows, cudaGraphConditionalHandle hw,
                                                             cudaGraphConditionalHandle hif, int use_h) {
    extern __shared__ float4 smem_f4[];
    unsigned char *sm = reinterpret_cast<unsigned char *>(smem_f4);
    PairEntry *tab = reinterpret_cast<PairEntry *>(sm);
    unsigned *xsh = reinterpret_cast<unsigned *>(sm + 32);  // the exchange's ok, OR, max
    int *bsh = reinterpret_cast<int *>(sm + 44);             // [0] block flags, [1] block max groups
    float *red = reinterpret_cast<float *>(sm + 52);         // [warp][4]
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(sm + 120);  // the window copies
    unsigned long long *lbar = bar + 1;                                          // the list build's copies
    int *wrec = reinterpret_cast<int *>(sm + 136);                               // the tile's window record
    int *hd = wrec + kWinInts;                                                   // the list build's header
    int4 *slist = reinterpret_cast<int4 *>(sm + kSmHdr);
    float2 *wpos = reinterpret_cast<float2 *>(slist + (size_t)rows * kFastBlock);
    int *csm = reinterpret_cast<int *>(wpos + kWinMax);
    float4 *wc = reinterpret_cast<float4 *>(csm + kLPCs);
    unsigned short(*ost)[kFastBlock] = reinterpret_cast<unsigned short(*)[kFastBlock]>(wc + kWinMax);
    int *kcol = reinterpret_cast<int *>(ost + 3 * (kLStage + 1));  // [stencil column][slot] entry counts
    int *cst = kcol + 3 * kFastBlock;
    static_assert(136 + (kWinInts + kLPHdr) * 4 <= kSmHdr, "small-run shared header");
    DevScalars *sc = s.sc;
    const int t = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // threads below kFastBlock own the tile's storage slots
    const bool worker = threadIdx.x < kFastBlock;
    const int i = t * kFastBlock + (threadIdx.x & (kFastBlock - 1));
    const bool act = worker && i < s.N;
    const int ic = act ? i : 0;
    if (threadIdx.x == 0) {
        tab[0] = s.pair[0];
        mbar_init(bar, 1);
        mbar_init(lbar, 1);
        wpos[kWinGhost] = s.pos0[s.N];  // the ghost slot's far position, never moved
    }
    int G = 0;
    small_load_tile(s, rows, slist, wrec, G);
    unsigned wbytes = small_win_bytes(wrec);
    int p = sc->smallPar;  // the parity of the current positions
    SmallSlot me;
    me.pi = (p ? s.pos1 : s.pos0)[ic];
    me.v = s.vel[ic];
    me.m = s.mass[ic];
    me.id = s.perm[ic];
    me.excl = s.excl[ic];
    me.cnt = act ? min(s.nbrCount[ic], s.nbrCap) : 0;
    const float D = s.imgD;
    const bool outside0 = sc->outside != 0;
    float dispHi = sc->dispHi;  // every block follows the same recurrence
    int row = sc->obsRow, stepNow = sc->stepNow;
    const int steps = sc->smallLeft;
    const unsigned base = sc->gbTag;
    const bool withhold = sc->testWithhold != 0;
    unsigned xi = 0, wuse = 0, luse = 0;  // exchanges, window copies and list-build copies so far
    // a step's totals that block 0 has still to sum (record set pset)
    int pset = -1, prow = 0, pr = 0;
    float pvm = 0.0f, pd = 0.0f;
    int k = 0;
    bool pending = false, stop = false, failed = false;
    __syncthreads();
    // one exchange: true unless a wait gave up
    auto xchg = [&](unsigned long long qa, unsigned long long qb, unsigned long long qc, unsigned word) {
        small_exchange(s, base + xi + 1u, (int)(xi % 3u), qa, qb, qc, word, xsh,
                       withhold && xi == 0 && blockIdx.x == 0);
        if (blockIdx.x == 0 && warp == 1 && pset >= 0) small_totals(s, pset, pvm, pd, pr, prow);
        __syncthreads();
        pset = -1;
        xi++;
        if (xsh[0]) return true;
        if (threadIdx.x == 0) atomicOr(&sc->overflow, kFlagTimeout);
        failed = true;
        return false;
    };
    // a bounded wait for a copy phase, the same verdict on every thread; a
    // copy that never completed is reported and given one more bounded wait
    auto copies_done = [&](unsigned long long *b, unsigned par) {
        const bool ok = mbar_wait_bounded(b, par, kWaitLimit);
        if (!__syncthreads_or(!ok)) return true;
        if (threadIdx.x == 0) atomicOr(&sc->overflow, kFlagTimeout);
        mbar_wait_bounded(b, par, kWaitLimit);
        failed = true;
        return false;
    };
    // block 0 clears the cell counts for the next binning (every block has
    // added to them or read them)
    auto clear_counts = [&]() {
        if (blockIdx.x == 0)
            for (int q = threadIdx.x; q < s.ncells; q += kSmallThreads) s.cellCount[q] = 0;
    };
    // the rebuild of the positions in pos (parity p), inside the launch
    auto small_rebuild = [&](float2 *pos) -> int {
        // 1: cells and ranks among the cell's particles (counting atomics)
        int c = 0, rk = 0;
        unsigned fl = 0;
        if (act) {
            if (!(isfinite(me.pi.x) && isfinite(me.pi.y))) {
                atomicOr(&sc->nonfinite, 1);
                fl |= 1u;
            }
            if (outside_box(s, me.pi)) {
                atomicOr(&sc->outside, 1);
                fl |= 2u;
            }
            c = cell_col(me.pi.x, me.pi.y, s.ncx, s.ncy, s.Lx, s.Ly);
            rk = atomicAdd(&s.cellCount[c], 1);
        }
        fl = (__syncthreads_or(fl & 1u) ? 1u : 0u) | (__syncthreads_or(fl & 2u) ? 2u : 0u);
        if (!xchg(0ull, 0ull, 0ull, fl)) return kSmallStop;
        const unsigned f1 = xsh[1];
        if (f1 & 1u) {  // a non-finite position: the run fails
            clear_counts();
            return kSmallStop;
        }
        const bool walk_ok = (s.wrapx ? s.ncx >= 5 : s.ncx >= 3) && (s.wrapy ? s.ncy >= 5 : s.ncy >= 3) &&
                             !outside0 && !(f1 & 2u);
        // 2: every block scans the counts into cell starts (block 0 also
        // writes them out), then the ids go to their cells
        const int nc = s.ncells;
        for (int q = threadIdx.x; q < nc; q += kSmallThreads) cst[q] = __ldcg(s.cellCount + q);
        __syncthreads();
        {
            // a run of cells per slot thread: its total, the scan of the
            // totals (warps, then the kFastBlock / 32 warp sums), its run
            const int per = (nc + kFastBlock - 1) / kFastBlock;
            const int c0 = worker ? min((int)threadIdx.x * per, nc) : nc, c1 = min(c0 + per, nc);
            int tot = 0;
            for (int q = c0; q < c1; q++) tot += cst[q];
            int x = tot;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            int *ws = reinterpret_cast<int *>(red);  // the slot warps' totals
            if (worker && lane == 31) ws[warp] = x;
            __syncthreads();
            int before = 0;
            if (worker)
                for (int w = 0; w < warp; w++) before += ws[w];
            int run = before + x - tot;
            for (int q = c0; q < c1; q++) {
                const int v = cst[q];
                cst[q] = run;
                run += v;
            }
            if (threadIdx.x == 0) cst[nc] = s.N;
        }
        __syncthreads();
        if (blockIdx.x == 0) {
            for (int q = threadIdx.x; q <= nc; q += kSmallThreads) s.cellStart[q] = cst[q];
            if (threadIdx.x == 0) {
                sc->nbrSum = 0ull;
                sc->maxCount = 0;
            }
        }
        unsigned f2 = 0;
        if (act) {
            const int slot0 = cst[c] + rk;
            if (slot0 >= 0 && slot0 < s.N) s.unsorted[slot0] = me.id;
            else f2 = 1u;  // inconsistent counts: never write outside the array
        }
        f2 = __syncthreads_or(f2) ? 1u : 0u;
        if (f2 && threadIdx.x == 0) atomicOr(&sc->overflow, 2);
        if (!xchg(0ull, 0ull, 0ull, f2)) return kSmallStop;
        clear_counts();
        if (xsh[1]) return kSmallStop;
        // 3: the placement inside the cell by id (k_fplace), and the tile's
        // window record from the cell starts here
        unsigned f3 = 0;
        if (act) {
            const int b = cst[c], e = cst[c + 1];
            int r = 0;
            for (int q = b; q < e; q++) r += __ldcg(s.unsorted + q) < me.id;
            const int ns = b + r;
            if (ns < e) {
                s.cellSorted[ns] = make_float4(me.pi.x, me.pi.y, __int_as_float(ns), __int_as_float(me.excl));
                s.sortedIds[ns] = ns;
                s.newCell[ns] = c;
                s.sPos[ns] = me.pi;
                s.sVel[ns] = me.v;
                s.sAcc[ns] = s.acc[i];
                s.sPerm[ns] = me.id;
            } else {
                f3 |= 1u;
            }
        }
        if (threadIdx.x == 0) {
            auto cell_of = [&](int q) {
                int lo = 0, hi = nc - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (cst[mid] <= q) lo = mid;
                    else hi = mid - 1;
                }
                return lo;
            };
            fwindow_record_t(s, t, walk_ok, [&](int q) { return cst[q]; }, cell_of);
            bsh[0] = 0;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            // the record just written (this thread's own stores)
            const int *bw = s.blockWin + kWinInts * (size_t)t;
            for (int q = 0; q < kWinInts; q++) wrec[q] = bw[q];
            if (wrec[kWLen] < 0 || lp_cs_words(s, wrec) > kLPCs) bsh[0] = 2;  // no stage for this tile
        }
        __syncthreads();
        f3 = (__syncthreads_or(f3) ? 1u : 0u) | (unsigned)bsh[0];
        if ((f3 & 1u) && threadIdx.x == 0) atomicOr(&sc->overflow, 2);
        if (!xchg(0ull, 0ull, 0ull, f3)) return kSmallStop;
        if (xsh[1] & 1u) return kSmallStop;
        if (xsh[1] & 2u) return kSmallPending;  // a tile without a stage: the rebuild kernels
        // 4: the tile's lists (k_flist_p's walk), then the slot's new
        // particle from the scratch arrays
        if (threadIdx.x == 0) {
            if (blockIdx.x == 0) {
                sc->totalUpdates += 1;  // k_rebuild_begin
                atomicAdd(&sc->builds, 1ull);
            }
            hd[kHT] = t;
            hd[kHLen] = wrec[kWLen];
            asm volatile("fence.proxy.async.global;" ::: "memory");
            lp_issue(s, wrec, hd, csm, wc, lbar);
        }
        __syncthreads();
        if (!copies_done(lbar, luse & 1u)) return kSmallStop;
        luse++;
        const int cap = s.nbrCap;
        const int slot = i;
        // three threads per slot walk the three stencil columns, each into
        // its own entry stage; the slot's thread then joins them in column
        // order (the order of k_flist_p's walk)
        const int sub = threadIdx.x / kFastBlock;
        int kd = 0, ix = 0, iy = 0, j = 0, self = 0;
        float2 q = make_float2(0.0f, 0.0f);
        if (slot < s.N) {
            const bool two = hd[kHTwo] != 0;
            if (two) {
                const int bnd = csm[min(max(hd[kHCsb + 4] + hd[kHColp + 4], 0), kLPCs - 1)];
                j = slot >= bnd ? 1 : 0;
            }
            const int pown = !two ? 2 : (j == 0 ? 3 : 4);
            self = min(max(slot + hd[kHDelta + pown], 0), kWinMax - 1);
            const float4 e = wc[self];
            cell_xy(e.x, e.y, s.ncx, s.ncy, s.Lx, s.Ly, ix, iy);
            q = make_float2(e.x, e.y);
            TileStagePut sp;
            sp.st = ost + sub * (kLStage + 1);
            sp.col = threadIdx.x & (kFastBlock - 1);
            lp_stencil_col(s, hd, csm, wc, ix, iy, j, q, self, sub, sp, kd);
        }
        kcol[threadIdx.x] = kd;
        __syncthreads();
        int k0 = 0, k1 = 0, kk = 0;
        if (act) {
            k0 = kcol[threadIdx.x];
            k1 = kcol[kFastBlock + threadIdx.x];
            kk = k0 + k1 + kcol[2 * kFastBlock + threadIdx.x];
            if (kk > kLStage && cap > kLStage) {
                // entries past the stage: the whole walk again, straight to the list
                int k2 = 0;
                DirectPut16 dp;
                dp.nbr16 = reinterpret_cast<unsigned short *>(s.nbr);
                dp.slot = slot;
                dp.cap = cap;
                dp.Ncap = s.Ncap;
                lp_stencil(s, hd, csm, wc, ix, iy, j, q, self, dp, k2);
            }
        }
        // entry k of the joined list (k < kLStage: every column's first kLStage entries are staged)
        auto entry = [&](int k) -> unsigned {
            const int d = k < k0 ? 0 : (k < k0 + k1 ? 1 : 2);
            const int r = k - (d == 0 ? 0 : (d == 1 ? k0 : k0 + k1));
            return ost[d * (kLStage + 1) + r][threadIdx.x];
        };
        const int kc = act ? min(kk, cap) : 0;
        const int ng = (kc + 7) >> 3;
        if (worker) {
            const int ngs = min(ng, kLStage / 8);
            const int gmax = __reduce_max_sync(0xffffffffu, ngs);
            int4 *out = reinterpret_cast<int4 *>(s.nbr) + slot;
            for (int g = 0; g < gmax; g++) {
                if (g < ngs) {
                    int v[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int e0 = 8 * g + 2 * u;
                        const unsigned lo = e0 < kc ? entry(e0) : kWinGhost;
                        const unsigned hi = e0 + 1 < kc ? entry(e0 + 1) : kWinGhost;
                        v[u] = (int)(lo | hi << 16);
                    }
                    out[(size_t)g * s.Ncap] = make_int4(v[0], v[1], v[2], v[3]);
                }
            }
            if (act && kc > kLStage && (kc & 7)) {
                unsigned short *n16 = reinterpret_cast<unsigned short *>(s.nbr);
                for (int q = kc; q < 8 * ng; q++) n16[nbr16_at(q, slot, s.Ncap)] = (unsigned short)kWinGhost;
            }
        }
        if (act) {
            const int id = __ldcg(s.sPerm + slot);
            me.pi = __ldcg(s.sPos + slot);
            me.v = __ldcg(s.sVel + slot);
            const float2 na = __ldcg(s.sAcc + slot);
            me.id = id;
            me.m = __ldg(s.idMass + id);
            me.cnt = kc;
            s.nbrCount[slot] = kk;
            pos[slot] = me.pi;
            s.vel[slot] = me.v;
            s.acc[slot] = na;
            s.perm[slot] = id;
            const_cast<float *>(s.mass)[slot] = me.m;
        }
        const int gm = __reduce_max_sync(0xffffffffu, ng);
        const int kmax = __reduce_max_sync(0xffffffffu, act ? kk : 0);
        const int ksum = __reduce_add_sync(0xffffffffu, act ? kk : 0);
        if (threadIdx.x == 0) bsh[1] = 0;
        __syncthreads();
        unsigned f4 = 0;
        if (lane == 0) {
            atomicMax(&bsh[1], gm);
            if (ksum) atomicAdd(&sc->nbrSum, (unsigned long long)ksum);
            if (kmax > 0) atomicMax(&sc->maxCount, kmax);
            if (kmax > cap) {
                atomicOr(&sc->overflow, 1);
                f4 = 1u;
            }
        }
        f4 = __syncthreads_or(f4) ? 1u : 0u;
        if (threadIdx.x == 0) {
            s.blockWin[kWinInts * (size_t)t + kWGroups] = bsh[1];
            wrec[kWGroups] = bsh[1];
        }
        __syncthreads();
        // the tile's rows into shared memory (this block wrote them)
        G = min(wrec[kWGroups], rows);
        if (worker && i < s.Ncap)
            for (int g = 0; g < G; g++)
                slist[g * kFastBlock + threadIdx.x] =
                    __ldcg(reinterpret_cast<const int4 *>(s.nbr) + (size_t)g * s.Ncap + i);
        wbytes = small_win_bytes(wrec);
        if (!xchg(0ull, 0ull, 0ull, f4)) return kSmallStop;
        if (xsh[1]) return kSmallStop;  // a list overflow: the run is repeated with longer lists
        return kSmallRebuilt;
    };
    for (; k < steps;) {
        const float2 *pin = p ? s.pos1 : s.pos0;
        float2 *pout = p ? s.pos0 : s.pos1;
        const int len = wrec[kWLen];
        // the window by bulk copies (other blocks wrote it before the last
        // exchange; the proxy fence orders their release before the copies)
        if (len >= 0) {
            if (threadIdx.x == 0) {
                asm volatile("fence.proxy.async.global;" ::: "memory");
                mbar_expect_tx(bar, wbytes);
                for (int q = 0; q < kWinPieces; q++) {
                    const int a = wrec[kWStart + q], c = wrec[kWCount + q];
                    if (c > 0) {
                        const int a0 = a & ~1, e0 = (a + c + 1) & ~1;
                        bulk_copy_g2s(wpos + wrec[kWOff + q] - (a & 1), pin + a0, (unsigned)(e0 - a0) * 8u, bar);
                    }
                }
            }
            if (!copies_done(bar, wuse & 1u)) break;
            wuse++;
        }
        const float2 pi = me.pi;
        const int cnt = me.cnt;
        float fx = 0.0f, fy = 0.0f, ue2 = 0.0f, we2 = 0.0f;
        const bool near = act && ((WX && (pi.x < D || pi.x > s.Lx - D)) || (WY && (pi.y < D || pi.y > s.Ly - D)));
        const bool img = __any_sync(0xffffffffu, near);
        if (act) {
            if (len >= 0 && s.win16) {
                if (img) fast_pairs_x2<SIG1, true, true, false, true, WX, WY>(s, tab[0], i, pi, cnt, slist, rows, pin,
                                                                            wpos, fx, fy, ue2, we2);
                else fast_pairs_x2<SIG1, true, true, false>(s, tab[0], i, pi, cnt, slist, rows, pin, wpos, fx, fy,
                                                            ue2, we2);
            } else if (len >= 0) {
                if (img) fast_pairs_x2<SIG1, true, false, false, true, WX, WY>(s, tab[0], i, pi, cnt, slist, rows, pin,
                                                                             wpos, fx, fy, ue2, we2);
                else fast_pairs_x2<SIG1, true, false, false>(s, tab[0], i, pi, cnt, slist, rows, pin, wpos, fx, fy,
                                                             ue2, we2);
            } else {
                if (img) fast_pairs_x2<SIG1, false, false, false, true, WX, WY>(s, tab[0], i, pi, cnt, slist, rows,
                                                                              pin, wpos, fx, fy, ue2, we2);
                else fast_pairs_x2<SIG1, false, false, false>(s, tab[0], i, pi, cnt, slist, rows, pin, wpos, fx, fy,
                                                              ue2, we2);
            }
        }
        float ue = 0.0f, we = 0.0f, ke = 0.0f, vvm = 0.0f;
        bool bad = false;
        if (act)
            fast_finish<WX, WY>(s, i, MODE_MID, pi, me.m, me.v, pout, nullptr, fx, fy, ue2, we2, 0.0f, 0.0f, ue, we,
                                ke, vvm, bad, &me.pi, &me.v);
        // the block's sums
        const float su = warp_sum_f(ue), sw = warp_sum_f(we), sk = warp_sum_f(ke), mx = warp_max(vvm);
        const unsigned anybad = __ballot_sync(0xffffffffu, bad);
        if (worker && lane == 0) {
            red[4 * warp + 0] = su;
            red[4 * warp + 1] = sw;
            red[4 * warp + 2] = sk;
            red[4 * warp + 3] = mx;
            if (anybad) atomicOr(&sc->nonfinite, 1);
        }
        __syncthreads();
        unsigned long long qa = 0ull, qb = 0ull, qc = 0ull;
        float mm = 0.0f;
        if (threadIdx.x == 0) {
            float a = 0.0f, b = 0.0f, c = 0.0f;
            for (int w = 0; w < kFastBlock / 32; w++) {
                a += red[4 * w];
                b += red[4 * w + 1];
                c += red[4 * w + 2];
                mm = fmaxf(mm, red[4 * w + 3]);
            }
            bool ob = false;
            qa = to_fixed(a, ob);
            qb = to_fixed(b, ob);
            qc = to_fixed(c, ob);
            if (ob) atomicOr(&sc->nonfinite, 2);
        }
        const int stepSet = (int)(xi % 3u);
        if (!xchg(qa, qb, qc, __float_as_uint(mm))) break;
        // the step's totals, the same on every block: the rebuild rule of
        // evalProps / NeighborList::update (md3dsystem.cpp:177, nn.cpp:118)
        const float vm2 = __uint_as_float(xsh[2]);
        const float d = dispHi + sqrtf(vm2) * s.dt;
        const int r = (double)d > s.halfSkin;
        pset = stepSet;
        pvm = vm2;
        pd = d;
        pr = r;
        prow = row;
        dispHi = d;
        row++;
        stepNow++;
        p ^= 1;
        k++;
        if (r) {
            const int o = small_rebuild(p ? s.pos1 : s.pos0);
            if (o == kSmallRebuilt) {
                dispHi = 0.0f;  // k_rebuild_begin
                continue;
            }
            if (o == kSmallPending) pending = true;
            else stop = true;
            break;
        }
    }
    // back to parity 0 (each thread its own slot), then one more exchange so
    // that every block has finished before the rebuild kernels or the next
    // launch read the positions
    if (p == 1 && act) s.pos0[i] = me.pi;
    __syncthreads();
    bool fin = false;
    if (!failed) fin = xchg(0ull, 0ull, 0ull, 0u);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (!fin) atomicOr(&sc->overflow, kFlagTimeout);
        // an exchange that gave up, a non-finite position or a list
        // overflow ends the run's loop
        const int left = (k > 0 && fin && !stop) ? steps - k : 0;
        sc->dispHi = dispHi;
        sc->rebuild = pending ? 1 : 0;
        sc->obsRow = row;
        sc->stepNow = stepNow;
        sc->smallDone = k;
        sc->smallLeft = left;
        sc->smallPar = 0;
        sc->testWithhold = 0;
        sc->gbTag = base + xi;
        if (use_h) {
            cudaGraphSetConditional(hif, pending ? 1u : 0u);
            cudaGraphSetConditional(hw, left > 0 ? 1u : 0u);
        }
    }
}

// Launch of the small-system run (cooperative: every block resident); the
// caller has checked small_run_fits.
template <bool SIG1, bool WX, bool WY>
static cudaError_t launch_fsmall_t(cudaStream_t st, const DevSys &s, int rows) {
    const int ntiles = (s.N + kFastBlock - 1) / kFastBlock;
    const size_t smem = small_smem(rows, s.ncells);
    auto kern = k_fsmall<SIG1, WX, WY>;
    int resident = 0;
    cudaError_t e = kernel_setup((const void *)kern, kSmallThreads, smem, &resident);
    if (e) return e;
    DevSys a = s;
    int ra = rows, ua = 0;
    cudaGraphConditionalHandle h0 = 0, h1 = 0;
    void *args[] = {&a, &ra, &h0, &h1, &ua};
    return cudaLaunchCooperativeKernel((const void *)kern, dim3(ntiles), dim3(kSmallThreads), args, smem, st);
}

constexpr size_t kSmallMaxSmem = 200 * 1024;

bool small_run_fits(const DevSys &s) {
    if (!s.fast || !s.win16 || !s.smallRec || s.nBonded != 0 || s.wallOn || s.gravity > 0.0f || s.refWalls ||
        s.areaUnits > 0 || s.trace || s.N <= 0)
        return false;
    const int ntiles = (s.N + kFastBlock - 1) / kFastBlock;
    if (ntiles > kSmallMaxTiles) return false;
    const int rows = std::max(1, (s.nbrCap + 7) / 8);
    const size_t smem = small_smem(rows, s.ncells);
    if (smem > kSmallMaxSmem) return false;
    auto kern = s.sigmaOne ? (s.wrapx && s.wrapy ? k_fsmall<true, true, true> : nullptr)
                           : (s.wrapx && s.wrapy ? k_fsmall<false, true, true> : nullptr);
    if (!kern) return false;  // the small run is built for XY-periodic boxes
    int resident = 0;
    if (kernel_setup((const void *)kern, kSmallThreads, smem, &resident)) return false;
    return resident >= ntiles;
}

cudaError_t launch_small_run(cudaStream_t st, const DevSys &s) {
    const int rows = std::max(1, (s.nbrCap + 7) / 8);
    return s.sigmaOne ? launch_fsmall_t<true, true, true>(st, s, rows) : launch_fsmall_t<false, true, true>(st, s, rows);
}

// The small-system run as a graph node (cooperative), with the WHILE and IF
// handles it sets.
cudaError_t enqueue_small_run(Launch &L, const DevSys &s, cudaGraphConditionalHandle hw,
                              cudaGraphConditionalHandle hif) {
    const int rows = std::max(1, (s.nbrCap + 7) / 8);
    const int ntiles = (s.N + kFastBlock - 1) / kFastBlock;
    const size_t smem = small_smem(rows, s.ncells);
    cudaError_t e;
    int resident = 0;
    if (s.sigmaOne) {
        if ((e = kernel_setup((const void *)k_fsmall<true, true, true>, kSmallThreads, smem, &resident))) return e;
        e = L.kernel(k_fsmall<true, true, true>, dim3(ntiles), dim3(kSmallThreads), smem, s, rows, hw, hif, 1);
    } else {
        if ((e = kernel_setup((const void *)k_fsmall<false, true, true>, kSmallThreads, smem, &resident))) return e;
        e = L.kernel(k_fsmall<false, true, true>, dim3(ntiles), dim3(kSmallThreads), smem, s, rows, hw, hif, 1);
    }
    if (e) return e;
    return L.cooperative_last();
}

// The persistent kernel wherever every window can be one bulk copy (no
// bonded particles, or their cell-ordered mirror current) and sigma comes by
// type; one block per step block otherwise.
cudaError_t enqueue_step_fast(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h,
                              int use_h) {
    const bool mt = s.numTypes > 1, sg = !s.sigmaByType;
    const bool persist = !sg && (s.nBonded == 0 || s.cposOn);
    if (persist) {
        if (mt) return fstep_p_image<true, false>(L, s, mode, parity, h, use_h);
        return s.sigmaOne ? fstep_p_image<false, true>(L, s, mode, parity, h, use_h)
                          : fstep_p_image<false, false>(L, s, mode, parity, h, use_h);
    }
    if (mt) return sg ? fstep_image<true, true, false>(L, s, mode, parity, h, use_h)
                      : fstep_image<true, false, false>(L, s, mode, parity, h, use_h);
    if (sg) return fstep_image<false, true, false>(L, s, mode, parity, h, use_h);
    return s.sigmaOne ? fstep_image<false, false, true>(L, s, mode, parity, h, use_h)
                      : fstep_image<false, false, false>(L, s, mode, parity, h, use_h);
}

// =================================================== storage order <-> ids

__global__ void __launch_bounds__(kBlock) k_unperm2(const int *perm, const float2 *in, float2 *out, int N) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) out[__ldg(perm + i)] = in[i];
}

__global__ void __launch_bounds__(kBlock) k_unperm1(const int *perm, const float *in, float *out, int N) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) out[__ldg(perm + i)] = in[i];
}

__global__ void __launch_bounds__(kBlock) k_perm2(const int *perm, const float2 *in, float2 *out, int N) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) out[i] = in[__ldg(perm + i)];
}

// The constant arrays in storage order from the id-order originals (with
// ident: the storage order becomes the id order).
// The cell-ordered mirror brought up to the current positions.
__global__ void __launch_bounds__(kBlock) k_cpos_refresh(DevSys s, int parity) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.N) return;
    (parity ? s.cpos1 : s.cpos0)[s.cslot[i]] = (parity ? s.pos1 : s.pos0)[i];
}

cudaError_t enqueue_cpos_refresh(Launch &L, const DevSys &s, int parity) {
    if (!s.cslot || s.N == 0) return cudaSuccess;
    return L.kernel(k_cpos_refresh, dim3((s.N + kBlock - 1) / kBlock), dim3(kBlock), 0, s, parity);
}

__global__ void __launch_bounds__(kBlock) k_perm_consts(DevSys s, int ident) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.N) return;
    int id = i;
    if (ident)
        s.perm[i] = i;
    else
        id = s.perm[i];
    const_cast<float *>(s.mass)[i] = s.idMass[id];
    if (s.numTypes > 1) const_cast<int *>(s.typeId)[i] = s.idType[id];
    if (!s.sigmaByType) const_cast<float *>(s.sigma)[i] = s.idSigma[id];
    if (s.wallDelta) const_cast<float *>(s.wallDelta)[i] = s.idWallDelta[id];
    if (s.wallSig) const_cast<float *>(s.wallSig)[i] = s.idWallSig[id];
}

cudaError_t enqueue_unpermute2(Launch &L, const DevSys &s, const float2 *in, float2 *out) {
    return L.kernel(k_unperm2, dim3(force_blocks(s.N)), dim3(kBlock), 0, (const int *)s.perm, in, out, s.N);
}

cudaError_t enqueue_unpermute1(Launch &L, const DevSys &s, const float *in, float *out) {
    return L.kernel(k_unperm1, dim3(force_blocks(s.N)), dim3(kBlock), 0, (const int *)s.perm, in, out, s.N);
}

cudaError_t enqueue_permute2(Launch &L, const DevSys &s, const float2 *in, float2 *out) {
    return L.kernel(k_perm2, dim3(force_blocks(s.N)), dim3(kBlock), 0, (const int *)s.perm, in, out, s.N);
}

cudaError_t enqueue_perm_identity(Launch &L, const DevSys &s) {
    return L.kernel(k_perm_consts, dim3(force_blocks(s.N)), dim3(kBlock), 0, s, 1);
}

cudaError_t enqueue_perm_consts(Launch &L, const DevSys &s) {
    return L.kernel(k_perm_consts, dim3(force_blocks(s.N)), dim3(kBlock), 0, s, 0);
}

}  // namespace femmd
