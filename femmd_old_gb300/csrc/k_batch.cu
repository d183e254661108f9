// k_batch.cu -- many independent replicas advanced in one persistent launch.
//
// Each replica is a complete femmd2D system (its own box, cell grid, lists,
// bonds, triangles and run state), described by the same DevSys block as a
// single context.  One CTA owns a set of replicas (longest-processing-time
// assignment by the host) and runs the whole run(n) sequence of each -- the
// reference's Integrator::run (femmd2D/src/integrator.cpp:31-57): forced
// rebuild, first force pass and drift, n-1 steps with the half-skin rebuild
// rule, last step -- with block-level rebuilds and steps separated only by
// __syncthreads.  Replicas never exchange data, so there is no grid-wide
// synchronisation and no per-step launch: one kernel launch covers all
// replicas and all steps.
//
// The per-particle and per-triangle arithmetic is step_body.cuh /
// nn_body.cuh, the same code as the single-system kernels, and the list order
// is the same, so a replica's trajectory is bit-identical to running it alone.
// Energies are reduced per replica in FP32 inside the block.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include "femmd_internal.h"
#include "launch.h"
#include "device_common.cuh"
#include "nn_body.cuh"
#include "step_body.cuh"

namespace femmd {

namespace cg = cooperative_groups;

namespace {

// block-wide max of one value per thread (blockDim a multiple of 32, <= 1024)
__device__ __forceinline__ int block_max_int(int v, int *scr) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_max_int(v);
    __syncthreads();
    if (lane == 0) scr[warp] = v;
    __syncthreads();
    int t = 0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < nw ? scr[threadIdx.x] : 0;
        t = warp_max_int(t);
    }
    return t;
}

// One pass over the block for the step's four sums, the max and the any-bad
// flag (two barriers instead of ten).  scr holds 6 values per warp.  The
// results are valid in thread 0.
__device__ __forceinline__ void block_reduce_step(float &a, float &b, float &c, float &d, float &m, int &bad,
                                                  float *scr) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    a = warp_sum_f(a);
    b = warp_sum_f(b);
    c = warp_sum_f(c);
    d = warp_sum_f(d);
    m = warp_max(m);
    bad = __any_sync(0xffffffffu, bad);
    __syncthreads();  // scr may still be read by the previous reduction
    if (lane == 0) {
        float *w = scr + 6 * warp;
        w[0] = a;
        w[1] = b;
        w[2] = c;
        w[3] = d;
        w[4] = m;
        w[5] = bad ? 1.0f : 0.0f;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const bool in = lane < nw;
        const float *w = scr + 6 * lane;
        a = warp_sum_f(in ? w[0] : 0.0f);
        b = warp_sum_f(in ? w[1] : 0.0f);
        c = warp_sum_f(in ? w[2] : 0.0f);
        d = warp_sum_f(in ? w[3] : 0.0f);
        m = warp_max(in ? w[4] : 0.0f);
        bad = __any_sync(0xffffffffu, in && w[5] != 0.0f);
    }
}

// The threads that work on one replica: one CTA (Solo), or the two CTAs of
// a thread-block cluster (Pair).  Loops over particles, triangles and
// candidates are strided over the team; sync() is __syncthreads or the
// cluster barrier (release/acquire at cluster scope, so global writes made
// by either CTA before it are seen by both after it).  Every sync() is
// reached by every thread of the team the same number of times: no sync()
// sits under a condition that could differ between the two CTAs.
struct SoloTeam {
    static constexpr int size = 1;
    __device__ int rank() const { return 0; }
    __device__ void sync() const { __syncthreads(); }
    // combine one float/int partial per CTA in the leader (rank 0)
    __device__ float *slot(float *x, int) const { return x; }
};

struct PairTeam {
    static constexpr int size = 2;
    int r;
    __device__ int rank() const { return r; }
    __device__ void sync() const { cg::this_cluster().sync(); }
    // the leader's copy of a shared array, at this CTA's entries
    __device__ float *slot(float *x, int per) const {
        return cg::this_cluster().map_shared_rank(x, 0) + r * per;
    }
};

// NeighborList::update branch + binning + Verlet build for one replica
template <class Team>
__device__ __noinline__ void block_rebuild(const Team team, const DevSys &s, int parity, int *iscr, float *xch) {
    const float2 *pos = parity ? s.pos1 : s.pos0;
    const int lane = threadIdx.x & 31;
    const int t0 = team.rank() * blockDim.x + threadIdx.x, tstride = Team::size * blockDim.x;
    const bool lead = team.rank() == 0 && threadIdx.x == 0;
    if (lead && s.sc->rebuild) {
        s.sc->totalUpdates += 1;
        s.sc->dispHi = 0.0f;
    }
    // counting sort: warp-aggregated histogram (warp-uniform loop for the match)
    for (int base = t0 & ~31; base < s.N; base += tstride) {
        const int i = base + lane;
        const bool act = i < s.N;
        const unsigned active = __ballot_sync(0xffffffffu, act);
        if (act) {
            float2 p = pos[i];
            if (!(isfinite(p.x) && isfinite(p.y))) atomicOr(&s.sc->nonfinite, 1);
            if (outside_box(s, p)) atomicOr(&s.sc->outside, 1);
            int c = cell_col(p.x, p.y, s.ncx, s.ncy, s.Lx, s.Ly);
            s.cellOf[i] = c;
            unsigned peers = __match_any_sync(active, c);
            int leader = __ffs(peers) - 1;
            int b = 0;
            if (lane == leader) b = atomicAdd(&s.cellCount[c], __popc(peers));
            b = __shfl_sync(peers, b, leader);
            s.rank[i] = b + __popc(peers & ((1u << lane) - 1u));
        }
    }
    team.sync();
    // exclusive scan of the counts into cellStart, counts cleared (the
    // leading CTA alone; its barriers are its own)
    if (team.rank() == 0) {
        const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        int carry = 0;
        for (int cb = 0; cb < s.ncells; cb += blockDim.x) {
            const int c = cb + threadIdx.x;
            const int v = c < s.ncells ? s.cellCount[c] : 0;
            int x = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) iscr[warp] = x;
            __syncthreads();
            if (warp == 0) {
                int w = lane < nw ? iscr[lane] : 0, z = w;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    int y = __shfl_up_sync(0xffffffffu, z, o);
                    if (lane >= o) z += y;
                }
                iscr[lane] = z - w;
                if (lane == 31) iscr[32] = z;  // chunk total
            }
            __syncthreads();
            if (c < s.ncells) {
                s.cellStart[c] = carry + iscr[warp] + x - v;
                s.cellCount[c] = 0;
            }
            carry += iscr[32];
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            s.cellStart[s.ncells] = s.N;
            s.sc->nbrSum = 0ull;
            s.sc->maxCount = 0;
        }
    }
    team.sync();
    for (int i = t0; i < s.N; i += tstride) {
        int slot = s.cellStart[s.cellOf[i]] + s.rank[i];
        if (slot >= 0 && slot < s.N)
            s.unsorted[slot] = i;
        else
            atomicOr(&s.sc->overflow, 2);
    }
    team.sync();
    // crowded cells after a blow-up or inconsistent counts: skip the quadratic parts
    const bool skip = s.sc->nonfinite != 0 || (s.sc->overflow & 2);
    if (!skip)
        for (int i = t0; i < s.N; i += tstride) place_one<false>(s, pos, i, &s.sc->overflow);
    team.sync();
    const bool fast = fast_walk_ok(s);
    int kmax = 0;
    unsigned long long ksum = 0;
    if (!skip)
        for (int t = t0; t < s.N; t += tstride) {
            // the fast walk takes the particles in cell order (slot t of
            // cellSorted): neighbouring lanes walk nearly the same ranges
            int i, k;
            if (fast) {
                const float4 me = s.cellSorted[t];
                i = __float_as_int(me.z) & kIdMask;
                const int c = cell_col(me.x, me.y, s.ncx, s.ncy, s.Lx, s.Ly);  // the binning's cell
                ListOut o = list_out(s, i);
                k = build_fast_at<false>(s, i, c, make_float2(me.x, me.y), __float_as_int(me.w), o);
                o.finish(k, s.nbrCap);
            } else {
                i = t;
                ListOut o = list_out(s, i);
                k = build_general<false>(s, pos, i, o);
                o.finish(k, s.nbrCap);
            }
            s.nbrCount[i] = k;
            kmax = max(kmax, k);
            ksum += (unsigned long long)k;
        }
    if (ksum) atomicAdd(&s.sc->nbrSum, ksum);
    kmax = block_max_int(kmax, iscr);
    if (threadIdx.x == 0) *team.slot(xch, 1) = __int_as_float(kmax);
    team.sync();
    if (lead) {
        for (int q = 1; q < Team::size; q++) kmax = max(kmax, __float_as_int(xch[q]));
        s.sc->maxCount = kmax;
        if (kmax > s.nbrCap) s.sc->overflow |= 1;
        s.sc->builds += 1ull;
    }
    team.sync();
}

// one force evaluation + integration of a replica (k_tri_forces + k_step)
template <bool MT, bool SG, bool WX, bool WY, bool SIG1, class Team>
__device__ __noinline__ void block_step(const Team team, const DevSys &s, const PairEntry *tab, int mode, int parity,
                                        float *fscr, float *xch) {
    const float2 *pin = parity ? s.pos1 : s.pos0;
    float2 *pout = parity ? s.pos0 : s.pos1;
    const int t0 = team.rank() * blockDim.x + threadIdx.x, tstride = Team::size * blockDim.x;
    float etri = 0.0f;
    if (s.feaForces && s.ntri > 0) {
        for (int t = t0; t < s.ntri; t += tstride) etri += tri_force(s, pin, t);
        team.sync();  // every nodal force written before the gathers
    }
    float ue = 0.0f, we = 0.0f, ke = 0.0f, vvm = 0.0f;
    bool bad = false;
    for (int i = t0; i < s.N; i += tstride)
        particle_step<MT, SG, WX, WY, SIG1, false>(s, tab, i, mode, pin, pout, ue, we, ke, vvm, bad);
    int anybad = bad;
    block_reduce_step(etri, ue, we, ke, vvm, anybad, fscr);
    // the team's partials, added in rank order by the leader (one CTA: as is)
    if (threadIdx.x == 0) {
        float *x = team.slot(xch, 6);
        x[0] = etri;
        x[1] = ue;
        x[2] = we;
        x[3] = ke;
        x[4] = vvm;
        x[5] = anybad ? 1.0f : 0.0f;
    }
    team.sync();
    if (team.rank() == 0 && threadIdx.x == 0) {
        float te = xch[0], tu = xch[1], tw = xch[2], tk = xch[3], tm = xch[4];
        bool nb = xch[5] != 0.0f;
        for (int q = 1; q < Team::size; q++) {
            te += xch[6 * q];
            tu += xch[6 * q + 1];
            tw += xch[6 * q + 2];
            tk += xch[6 * q + 3];
            tm = fmaxf(tm, xch[6 * q + 4]);
            nb = nb || xch[6 * q + 5] != 0.0f;
        }
        DevScalars *sc = s.sc;
        if (nb) sc->nonfinite |= 1;
        const double U = (double)te + (double)tu, W = (double)tw, KE = (double)tk;
        sc->U = U;
        sc->W = W;
        int reb;
        if (mode == MODE_MID || mode == MODE_LAST) {
            sc->KE = KE;
            sc->vvMax = tm;
            float d = sc->dispHi + sqrtf(tm) * s.dt;  // md3dsystem.cpp:177
            reb = (double)d > s.halfSkin;              // nn.cpp:118
            int row = sc->obsRow;
            if (s.obs && row < s.obsCap) {
                double *o = s.obs + (size_t)row * kObsCols;
                o[0] = U;
                o[1] = W;
                o[2] = KE;
                o[3] = (double)tm;
                o[4] = (double)d;
                o[5] = (double)reb;
            }
            sc->obsRow = row + 1;
            sc->dispHi = d;
        } else {
            reb = (double)sc->dispHi > s.halfSkin;
        }
        sc->rebuild = reb;
        if (mode == MODE_FIRST || mode == MODE_MID) sc->stepNow += 1;
    }
    team.sync();
}

// The reference's Integrator::run (integrator.cpp:31-57) for replica r on a
// team: descriptor and pair table into shared memory, run start, forced
// rebuild, first force pass, steps with the half-skin rule, last step.
template <bool MT, bool SG, bool WX, bool WY, bool SIG1, class Team>
__device__ __forceinline__ void run_replica(const Team team, const DevSys *reps, int r, const int *parity0, int steps,
                                            DevSys &S, PairEntry *tab, float *fscr, int *iscr, float *xch) {
    {
        const int *src = (const int *)(reps + r);
        int *dst = (int *)&S;
        for (int w = threadIdx.x; w < (int)(sizeof(DevSys) / sizeof(int)); w += blockDim.x) dst[w] = src[w];
    }
    __syncthreads();
    const int nt = S.numTypes > 1 ? S.numTypes * S.numTypes : 1;
    for (int w = threadIdx.x; w < nt; w += blockDim.x) tab[w] = S.pair[w];
    if (team.rank() == 0 && threadIdx.x == 0) {
        // run start: NeighborList::update(1)
        DevScalars *c = S.sc;
        c->rebuild = 1;
        c->dispHi = 0.0f;
        c->totalUpdates = 0;
        c->obsRow = 0;
        c->stepNow = S.stepBase;
    }
    team.sync();
    int cur = parity0[r];
    block_rebuild(team, S, cur, iscr, xch);
    if (steps == 0) {
        block_step<MT, SG, WX, WY, SIG1>(team, S, tab, MODE_INIT, cur, fscr, xch);
    } else {
        block_step<MT, SG, WX, WY, SIG1>(team, S, tab, MODE_FIRST, cur, fscr, xch);
        cur ^= 1;
        for (int k = 1; k < steps; k++) {
            // the flag was written before the step's last sync(): the same
            // value in every CTA of the team
            if (S.sc->rebuild) block_rebuild(team, S, cur, iscr, xch);
            block_step<MT, SG, WX, WY, SIG1>(team, S, tab, MODE_MID, cur, fscr, xch);
            cur ^= 1;
        }
        if (S.sc->rebuild) block_rebuild(team, S, cur, iscr, xch);
        block_step<MT, SG, WX, WY, SIG1>(team, S, tab, MODE_LAST, cur, fscr, xch);
    }
    team.sync();
}

}  // namespace

// Replicas are handed out from a queue: 'order' lists them heaviest first,
// and each CTA takes the next one when it is free (greedy list scheduling,
// which also balances CTAs that share an SM).  queue[0] is the next index,
// queue[1] counts finished CTAs; the last CTA to finish resets the queue.
// MINB: resident CTAs per SM the register allocation must allow.
template <bool MT, bool SG, bool WX, bool WY, bool SIG1, int MINB>
__global__ void __launch_bounds__(1024, MINB) k_batch(const DevSys *__restrict__ reps, const int *__restrict__ order,
                                                      int nwork, int nbig, int *queue, const int *__restrict__ parity0,
                                                      int steps) {
    __shared__ DevSys S;
    __shared__ float fscr[6 * 32];
    __shared__ float xch[6 * 2];
    __shared__ int iscr[33];
    __shared__ int next;
    extern __shared__ PairEntry tab[];
    const SoloTeam team;
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(queue, 1);
        __syncthreads();
        const int q = next;
        __syncthreads();
        if (q >= nwork) break;
        run_replica<MT, SG, WX, WY, SIG1>(team, reps, order[q], parity0, steps, S, tab, fscr, iscr, xch);
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(queue + 1, 1) == (int)gridDim.x - 1) {
            queue[0] = 0;
            queue[1] = 0;
            queue[2] = 0;
        }
    }
}

// The same with the CTAs in pairs (thread-block clusters of two): first the
// order's nbig heaviest replicas, each run by a pair (particles, triangles
// and candidates split between the two CTAs; the leader's pick of the queue
// shared through its shared memory), then the rest one CTA each, from their
// own counter queue[2].  A replica much larger than the average work of a
// CTA then no longer sets the length of the whole launch.
template <bool MT, bool SG, bool WX, bool WY, bool SIG1>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(1024, 1)
    k_batch_pair(const DevSys *__restrict__ reps, const int *__restrict__ order, int nwork, int nbig, int *queue,
                 const int *__restrict__ parity0, int steps) {
    __shared__ DevSys S;
    __shared__ float fscr[6 * 32];
    __shared__ float xch[6 * 2];
    __shared__ int iscr[33];
    __shared__ int next;
    extern __shared__ PairEntry tab[];
    const PairTeam pair{(int)cg::this_cluster().block_rank()};
    for (;;) {
        if (pair.rank() == 0 && threadIdx.x == 0) next = atomicAdd(queue, 1);
        pair.sync();
        const int q = *cg::this_cluster().map_shared_rank(&next, 0);
        pair.sync();  // both have read the leader's pick before it changes
        if (q >= nbig) break;  // the same q in both CTAs
        run_replica<MT, SG, WX, WY, SIG1>(pair, reps, order[q], parity0, steps, S, tab, fscr, iscr, xch);
    }
    const SoloTeam solo;
    for (;;) {
        if (threadIdx.x == 0) next = nbig + atomicAdd(queue + 2, 1);
        __syncthreads();
        const int q = next;
        __syncthreads();
        if (q >= nwork) break;
        run_replica<MT, SG, WX, WY, SIG1>(solo, reps, order[q], parity0, steps, S, tab, fscr, iscr, xch);
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(queue + 1, 1) == (int)gridDim.x - 1) {
            queue[0] = 0;
            queue[1] = 0;
            queue[2] = 0;
        }
    }
}

namespace {

template <bool MT, bool SG, bool WX, bool WY, bool SIG1>
cudaError_t launch_batch(Launch &L, const BatchLaunch &b) {
    if (b.nbig > 0)
        return L.kernel(k_batch_pair<MT, SG, WX, WY, SIG1>, dim3(b.ctas), dim3(b.threads), b.smem, b.reps, b.order,
                        b.nwork, b.nbig, b.queue, b.parity, b.steps);
    if (b.minBlocks >= 2)
        return L.kernel(k_batch<MT, SG, WX, WY, SIG1, 2>, dim3(b.ctas), dim3(b.threads), b.smem, b.reps, b.order,
                        b.nwork, 0, b.queue, b.parity, b.steps);
    return L.kernel(k_batch<MT, SG, WX, WY, SIG1, 1>, dim3(b.ctas), dim3(b.threads), b.smem, b.reps, b.order,
                    b.nwork, 0, b.queue, b.parity, b.steps);
}

template <bool MT, bool SG, bool WX, bool WY>
cudaError_t pick_sig_b(Launch &L, const BatchLaunch &b) {
    if constexpr (!SG) {
        if (b.sigmaOne) return launch_batch<MT, SG, WX, WY, true>(L, b);
    }
    return launch_batch<MT, SG, WX, WY, false>(L, b);
}

template <bool MT, bool SG>
cudaError_t pick_image_b(Launch &L, const BatchLaunch &b) {
    if (b.wrapx && b.wrapy) return pick_sig_b<MT, SG, true, true>(L, b);
    if (b.wrapx) return pick_sig_b<MT, SG, true, false>(L, b);
    return pick_sig_b<MT, SG, false, false>(L, b);
}

}  // namespace

cudaError_t enqueue_batch(Launch &L, const BatchLaunch &b) {
    if (b.multiType) return b.sigmaByType ? pick_image_b<true, false>(L, b) : pick_image_b<true, true>(L, b);
    return b.sigmaByType ? pick_image_b<false, false>(L, b) : pick_image_b<false, true>(L, b);
}

}  // namespace femmd
