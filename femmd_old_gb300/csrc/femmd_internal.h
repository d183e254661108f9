// femmd_internal.h -- device data layout and kernel launch interface of the
// GB300 femmd2D timestep.  Shared by the kernel translation units and the
// host context (femmd_api.cu).
//
// HBM layout (structure of arrays, one context per system):
//   pos[2]  float2[N]    ping-pong positions (a step reads one, writes the other)
//   vel     float2[N]    half-step velocity between fused step kernels
//   acc     float2[N]    acceleration (written by the last step of a run)
//   mass    float[N], typeId int[N], sigma float[N] (only when sigma varies inside a type)
//   excl    int[N]       exclusion group (-1 = none)
//   cells   column-major cell index c = ix*ncy + iy (so the three cells of one stencil
//           column are adjacent), cellStart[ncells+1], sortedIds[N] (ascending id
//           inside a cell), cellSorted float4[N] = (x, y, id|type<<27, excl)
//   nbr     int4[cap/4][Ncap] Verlet lists (entry = id | type<<27), nbrCount[N]: entries
//           4g..4g+3 of particle i share the int4 at [g][i] (nbr_at)
//   bonds   per-particle incidence CSR (bStart, bEnt = {partner|sign<<31, r0 bits})
//   tris    triIdx int4[nt], triGeo float4[2nt] (neo-Hookean: Bm, vol0; Green: xm rows 1-2, area),
//           tStart/tEnt vertex->triangle incidence (t*4+slot), triF float2[3nt] per-step nodal forces
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace femmd {

constexpr int kIdBits = 27;
constexpr int kIdMask = (1 << kIdBits) - 1;
constexpr int kMaxTypes = 32;
constexpr int kBlock = 256;        // threads per block of the per-particle kernels
constexpr int kStepBlock = 128;    // threads per block of the step kernel
constexpr int kNnBlock = 256;      // threads per block of the list build
constexpr int kScanBlock = 1024;   // cells per block of the cell-start scan
constexpr int kObsCols = 6;        // per-step observable row: U, W, sum m v^2, max v^2, dispHi, rebuilt
constexpr int kTraceCols = 6;      // per-step trace row (ns): tri start/end, step start/end, rebuild start/end

// Per type-pair constants, all formed on the host with the reference's float
// operations (interactionsCuda.cu:43-55, 79-88) so that the kernel's per-pair
// arithmetic reproduces the reference bit for bit.
// The four values the pair loop reads first share one aligned 16 bytes.
struct __align__(16) PairEntry {
    float rcut2;  // (rc*rc)*sigma_ij*sigma_ij      (sigma by type)
    float c;      // 48*eps/(sigma_ij*sigma_ij)     (sigma by type)
    float eps4;   // 4*eps
    float us;     // uShift
    float sig2;   // sigma_ij*sigma_ij              (sigma by type)
    float rc;     // rc (units of sigma_ij)
    float eps48;  // 48*eps
    float pad;
};

// Energy sums are accumulated as 64-bit fixed point with kFixFrac fraction
// bits: every block adds its partial with one integer atomicAdd, which is
// exact and order-independent, so the totals are deterministic and no FP64
// work sits on the per-step path (GB300's FP64 pipe is narrow).
constexpr int kFixFrac = 24;

// Verlet list layout: entry k of particle i at nbr[nbr_at(k, i, Ncap)].
// Four consecutive entries of a particle share 16 bytes, and group g of every
// particle forms a row of Ncap int4, so the 32 lanes of a warp read a group
// of their particles with one coalesced 512-byte load and the list build
// stores one int4 per four entries.  The capacity is a multiple of 4.
__host__ __device__ __forceinline__ size_t nbr_at(int k, int i, int Ncap) {
    return ((size_t)(k >> 2) * Ncap + i) * 4 + (k & 3);
}
// The same storage as 16-bit entries (the fast mode's windowed blocks with
// win16): entry k of particle i at ((unsigned short *)nbr)[nbr16_at(k, i,
// Ncap)], eight entries of a particle to one 16-byte group.
__host__ __device__ __forceinline__ size_t nbr16_at(int k, int i, int Ncap) {
    return ((size_t)(k >> 3) * Ncap + i) * 8 + (k & 7);
}

struct DevScalars {
    double U, W, KE, Ufea;          // last force evaluation (FP64 from the fixed-point sums)
    float vvMax, dispHi;
    int rebuild, totalUpdates;
    unsigned int ticket, triTicket;
    int overflow, nonfinite, outside, maxCount;  // the first three are cleared together by the host
    int obsRow, stepNow;  // stepNow: index n of the positions x_n the next force evaluation sees
    unsigned long long nbrSum, builds;
    unsigned long long accU, accW, accK;  // fixed-point accumulators (two's complement)
    unsigned int vvMaxBits, pad1;         // max v^2 as float bits (v^2 >= 0)
    // the small-system run (k_fsmall): the tag base of its next launch's
    // exchanges, the steps one launch advanced, the steps left and the
    // position parity the next launch starts from (it ends on parity 0)
    unsigned int gbTag, pad2;
    int smallDone, smallLeft, smallPar;
    int testWithhold;  // the next small run's block 0 withholds its first exchange record (a test of the timeout)
};

enum StepMode { MODE_FORCES = 0, MODE_FIRST = 1, MODE_MID = 2, MODE_LAST = 3, MODE_INIT = 4 };

struct DevSys {
    int N, Ncap;
    int wrapx, wrapy;
    float Lx, Ly, dt, hdt;
    double halfSkin;
    int ncx, ncy, ncells;
    float nnRadiusSq;
    int imageExact;
    int numTypes, sigmaByType, sigmaOne;  // sigmaOne: every sigma_ij^2 of the table is exactly 1
    const PairEntry *pair;
    float2 *pos0, *pos1;
    float2 *vel, *acc, *forceOut;
    float *energyOut;
    const float *mass, *sigma;
    const int *typeId, *excl;
    int *cellOf, *rank, *cellCount, *cellStart, *blockSums, *unsorted, *sortedIds;
    float4 *cellSorted;
    int *nbr, *nbrCount;
    int nbrCap;
    int nBonded, bondForces, feaForces, feaLaw, bondKMode;
    const int *bStart;
    const int2 *bEnt;
    const int *tStart;
    const int *tEnt;
    int ntri;
    const int4 *triIdx;
    const float4 *triGeo;
    float2 *triF;
    float *triE;
    const float2 *refPos;
    float kBond, E, mu, lambda, C1, C2, C3;
    DevScalars *sc;
    double *obs;
    int obsCap;
    unsigned long long *trace;  // per-step device timestamps, or null
    // per-triangle (mu, lambda) when elastomers have their own material, else null
    const float2 *triLame;
    // moving harmonic walls (XPBC / NOPBC): bottom at y = 0, top at
    // y_w(n) = wallY0 - wallV * (n dt); particle i touches a wall closer than
    // wallDelta[i] = 2^(1/6) sigma_i and is pushed back with k_w * overlap
    int wallOn;
    float wallK, wallY0, wallV;
    const float *wallDelta;
    int stepBase;  // the context's step count when the run started
    // the reference's fixed walls, first in calcForces (interactions.cpp:83-93):
    // 1 = LJ walls on every side (NOPBC), 2 = harmonic top/bottom (XPBC); and
    // gravity f_y -= m g (interactions.cpp:111-126)
    int refWalls;
    float kWall, wallRc, gravity;
    const float *wallSig;  // sigma_i, with walls of either kind
    // area springs (calcAreaForcesCPU, interactions.cpp:696-750): after the
    // triangle forces the vertices are displaced in place, triangle by
    // triangle; walls and bonds (earlier in the reference's force order) read
    // the positions of [0, nPre) as they were before, kept in posPre
    float kArea;
    float2 *posPre;
    int nPre;
    int areaUnits;         // blocks of the area pass (0: area springs off)
    int areaSmem;          // bytes of shared memory per block
    const int4 *areaUnit;  // per block, 2 entries: {triangle list, triangles, vertices, lanes}, {A0 offset}
    const int *areaLane;   // per block and lane (32): first vertex of the lane's elastomer
    const int4 *areaIdx;   // per triangle of a mesh: its vertices inside the elastomer
    const float *areaA0;   // per block: A0 of triangle k for lane l at [k * lanes + l]
    // Fast force mode (femmd_set_force_mode): every rebuild stores the free
    // particles [nBonded, N) in cell order; perm[s] is the id of the particle
    // at storage slot s (slots below nBonded never move).  The per-particle
    // arrays above (state, mass, type, sigma, wall ranges, lists) are then in
    // storage order; the id-order originals of the constant ones are kept in
    // idMass..idWallSig.  imgD: a warp whose particles all lie at least imgD
    // inside every periodic edge has no pair that crosses the boundary.
    int fast;
    float imgD;
    int *perm;
    float2 *sPos, *sVel, *sAcc;  // rebuild scratch: the state in the new order
    int *sPerm;
    int *fBlockSums;             // free particles per block of cell slots
    const float *idMass, *idSigma, *idWallDelta, *idWallSig;
    const int *idType;
    // The step kernel's blocks of kFastBlock storage slots: a block of free
    // particles inside one cell column, or across two neighbouring ones,
    // stages the positions of its stencil window (up to kWinPieces cell-slot
    // ranges) in shared memory, and its lists hold window indices instead of
    // storage slots.  blockWin holds kWinInts ints per block (the kW*
    // offsets): piece p's cell slots start[p] .. start[p] + count[p] - 1 sit
    // at window entries off[p] ..; len: the entries the pieces span (len < 0:
    // the block reads global slots); groups: 16-byte list groups of the
    // block's longest list; col0, two: the block's first cell column and
    // whether it reaches into the next; row0[p], row1[p]: the cell rows piece
    // p covers (row1 < row0: none).  The window's last entry, kWinGhost, is
    // the ghost's.
    int *newCell;   // cell of the particle at each storage slot
    // With bonded particles (whose storage slots never move) the storage order
    // is not the cell order; cpos0/cpos1 mirror pos0/pos1 in cell-slot order
    // (written by the rebuild and by every drift; cslot: the cell slot of each
    // storage slot), so that every window is one bulk copy.  cposOn: the
    // mirror is current (off while area springs move vertices in place).
    float2 *cpos0, *cpos1;
    int *cslot;
    int cposOn;
    // win16: the entries of windowed step blocks are 16-bit window indices,
    // eight to a 16-byte group (nbr16_at); one particle kind, sigma by type,
    // no bonded particles.  Other blocks keep 32-bit entries (nbr_at).
    int win16;
    int *blockWin;
    // the small-system run's exchange records: three sets of kSmallMaxTiles
    // records {tag << 32 | max v^2 bits, U, W, K fixed point}
    unsigned long long *smallRec;
};

constexpr int kSmallMaxTiles = 128;  // step blocks of the largest system the small-system run takes

constexpr int kFastBlock = 128;  // storage slots per block of the fast step kernel
constexpr int kWinMax = 768;     // window entries per block (the ghost included)
constexpr int kWinGhost = kWinMax - 1;  // the window entry of the ghost slot
constexpr int kWinPieces = 8;    // cell-slot ranges of a window
constexpr int kWLen = 0, kWStart = 1, kWOff = kWStart + kWinPieces, kWCount = kWOff + kWinPieces,
              kWGroups = kWCount + kWinPieces, kWCol0 = kWGroups + 1, kWTwo = kWCol0 + 1, kWRow0 = kWTwo + 1,
              kWRow1 = kWRow0 + kWinPieces;
constexpr int kWinInts = kWRow1 + kWinPieces;  // ints of window data per block

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Kernel launch sink: direct stream launches, or nodes appended to a CUDA
// graph (optionally inside an IF body).  Implemented in femmd_api.cu.
struct Launch;

// ---- neighbour list (k_nn.cu)
// Cell binning + Verlet list on the positions of buffer 'parity'.  With
// check_flag the kernels return at once unless sc->rebuild is set.
cudaError_t enqueue_rebuild(Launch &L, const DevSys &s, int parity, int check_flag);
// Run start (NeighborList::update(1), nn.cpp:114-134): forced rebuild,
// dispHi = 0, totalUpdates = 1, per-step observable rows restart.
cudaError_t enqueue_run_start(Launch &L, const DevSys &s);

// The binning part of a rebuild (rebuild bookkeeping, counting, scan,
// scatter): cellOf, rank, cellStart and the unsorted slots.
cudaError_t enqueue_bin(Launch &L, const DevSys &s, int parity, int check);

// ---- fast force mode (k_fast.cu)
// Rebuild: binning, then the free particles stored in cell order and the
// Verlet lists built in the new storage order.
cudaError_t enqueue_rebuild_fast(Launch &L, const DevSys &s, int parity, int check);
// The step kernel of the fast mode (same modes and outputs as enqueue_step_after_tri).
cudaError_t enqueue_step_fast(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h,
                              int use_h);
// Storage order <-> particle id: out[perm[s]] = in[s] (float2 / float
// arrays), out[s] = in[perm[s]], perm = identity with the constants copied
// from the id-order originals, and the constants gathered through perm.
cudaError_t enqueue_unpermute2(Launch &L, const DevSys &s, const float2 *in, float2 *out);
cudaError_t enqueue_unpermute1(Launch &L, const DevSys &s, const float *in, float *out);
cudaError_t enqueue_permute2(Launch &L, const DevSys &s, const float2 *in, float2 *out);
cudaError_t enqueue_perm_identity(Launch &L, const DevSys &s);
cudaError_t enqueue_cpos_refresh(Launch &L, const DevSys &s, int parity);
// The small-system run (k_fsmall): whether a system qualifies (fast mode, one
// kind, no bonded particles, walls or gravity, XY-periodic, few step blocks,
// every block resident), and one cooperative launch of up to 'steps' middle
// steps, ending after a step that calls for a rebuild.
bool small_run_fits(const DevSys &s);
cudaError_t launch_small_run(cudaStream_t st, const DevSys &s);
cudaError_t enqueue_small_run(Launch &L, const DevSys &s, cudaGraphConditionalHandle hw,
                              cudaGraphConditionalHandle hif);
cudaError_t enqueue_perm_consts(Launch &L, const DevSys &s);

// ---- forces + integration (k_force.cu)
cudaError_t enqueue_step(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h, int use_h);
// enqueue_step in two parts: the triangle pass (reads positions only), then
// the area springs and the step kernel.
cudaError_t enqueue_tri(Launch &L, const DevSys &s, int parity);
cudaError_t enqueue_step_after_tri(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h,
                                   int use_h);
// leapFrogStep1 + applyPBC alone (integrator.cpp:100-127): buffer parity -> 1-parity
cudaError_t enqueue_drift(Launch &L, const DevSys &s, int parity);
// The same drift inside a run: the step counter advances by one (the drift
// makes x_{n+1}) instead of being set from stepBase.
cudaError_t enqueue_drift_in_run(Launch &L, const DevSys &s, int parity);
// Allow the area-spring kernel 'bytes' of dynamic shared memory.
cudaError_t area_smem_setup(int bytes);

// ---- adjoint (k_adjoint.cu)
// Seed at the final positions: xbar += dJ/dx of cWall * wall stress + cFea *
// FEA energy, direct parameter terms, and wOut = h vbar / m.
cudaError_t enqueue_adj_seed(Launch &L, const DevSys &s, const float2 *pos, float2 *xbar, const float2 *vbar,
                             float2 *wOut, float cWall, float cFea, float yw, double *sigAcc, double *gMu,
                             double *gLam);
// One reverse step at positions pos with weights w: xbar += (df/dx)^T w,
// parameter terms; with update, vbar += dt xbar and wOut = cNext vbar / m.
cudaError_t enqueue_adj_step(Launch &L, const DevSys &s, const float2 *pos, const float2 *w, float2 *triD,
                             double *gMu, double *gLam, float2 *xbar, float2 *vbar, float2 *wOut, float cNext,
                             int update, float yw, double *epsAcc, double *sigAcc);

// ---- observables (k_props.cu): cluster unfolding, centre of mass and
// velocity, feaVirial and cluster-virial terms, m v^2 per particle
// Properties::compute (properties.cpp:85-95) on the device: the values of
// Properties::evaluate at the end of each step, their window sums, and the
// last completed window's average and standard deviation (Prop,
// properties.h:5-13).  Order of the values: uKinetic, uPotential, uTotal,
// temperature, virial, feaVirial, pressure, clusterUKinetic, clusterVirial,
// molPressure.
cudaError_t enqueue_cluster_centroid(Launch &L, const DevSys &s, const float2 *pos, int ncl, const int2 *clRange,
                                     double2 *centroid);
constexpr int kNumProps = 10;
struct DevProps {
    double val[kNumProps], sum[kNumProps], sum2[kNumProps], avg[kNumProps], stdv[kNumProps];
    int count, windows, lastStep;
    unsigned ticket;
};
// After a step's LAST: reduce the term arrays of enqueue_props (fixed slices
// per block, added in block order by the last block), evaluate, accumulate,
// and close a window at steps past stepEqui that are multiples of stepAvg.
cudaError_t enqueue_props_accum(Launch &L, const DevSys &s, DevProps *P, double *partials, int blocks,
                                const double *clKin, int ncl, const double *feaVir, int ntri, const double *clVir,
                                int nvir, int stepAvg, int stepEqui);
cudaError_t enqueue_props(Launch &L, const DevSys &s, const float2 *pos, int ncl, const int2 *clRange,
                          const float *clMass, const int *clusterOf, double2 *unf, double2 *cmPos, double2 *cmVel,
                          double *clKin, double *feaVir, double *kin, double *clVir, int npart);
// (kin and clVir of particles [0, npart); the cluster virial is zero beyond
// the elastomers, which come first)

// ---- batched replicas (k_batch.cu): one persistent launch over many systems
struct BatchLaunch {
    const DevSys *reps;
    const int *order, *parity;
    int *queue;  // {next work index, finished CTAs, next single-CTA index}, zero before a launch
    int nwork, minBlocks;
    int nbig;    // the first nbig replicas of 'order' run on CTA pairs (0: none)
    int steps, ctas, threads;
    size_t smem;
    bool multiType, sigmaByType, sigmaOne, wrapx, wrapy, exact;
};
cudaError_t enqueue_batch(Launch &L, const BatchLaunch &b);

int force_blocks(int N);
int step_blocks(int N);
int tri_blocks(int ntri);
int scan_blocks(int ncells);

}  // namespace femmd
