// femmd_api.cu -- host context and C ABI (include/femmd.h) of the GB300
// femmd2D timestep.
//
// Setup calls mirror the reference's System.* surface
// (femmd2D/src/interface.cpp:229-600) and store their inputs in host arrays,
// computing derived data with the reference's float operations
// (Particles::addElastomer particles.cpp:295-385, Bonds::createBond
// bonds.cpp:14-29, NeighborList::init nn.cpp:200-227).  Compute happens only on
// the GPU: femmd_run enqueues the kernel sequence of Integrator::run
// (integrator.cpp:31-57) on the context stream --
//     run start (forced rebuild) -> first step -> (n-1) x [step -> IF rebuild] -> last step
// where each "[step -> IF rebuild]" unit is a node pair of a cached CUDA graph
// and the IF condition is set on the device by the step kernel's last block
// (the reference's dispHi > skin/2 test), so a run has no host round trip
// until it ends.  A neighbour-list capacity overflow found at the end rolls
// the run back to its start checkpoint, grows the list and repeats it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <climits>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <map>
#include <vector>

#include "femmd.h"
#include "femmd_internal.h"
#include "launch.h"

using namespace femmd;

namespace {

struct Cluster {
    int offset, nv, nt, tetOffset;
    float mass, rho;
};

template <typename T> struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t cnt) {
        if (cnt <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        if (cnt == 0) cnt = 1;
        cudaError_t e = cudaMalloc(&p, cnt * sizeof(T));
        if (e == cudaSuccess) n = cnt;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct GraphSet {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t x = nullptr;
    void release() {
        if (x) cudaGraphExecDestroy(x);
        if (g) cudaGraphDestroy(g);
        x = nullptr;
        g = nullptr;
    }
};

constexpr int kGraphUnits = 32;  // [step -> IF rebuild] units per cached graph
constexpr unsigned kPos = 1, kVel = 2, kAcc = 4, kForce = 8, kEnergy = 16, kAll = 31;

}  // namespace

// Trajectory frames (Integrator::doStep, integrator.cpp:20-26): positions and
// velocities copied device-to-host into pinned slots during a run and
// formatted by a writer thread.  Frames of a run are committed to the writer
// once the run (or the part of it before a slot had to be reused) is known
// to be free of list overflow, so a repeated run never writes a frame twice.
struct TrajFrame {
    int step, slot;
};

// What a frame is formatted with: the layout, the file, and the topology
// (copied from the context when it changes, so that the writer thread never
// reads the context).
struct FrameMeta {
    std::string path;
    int format = 0;
    std::vector<int> type, tri, bond;
    std::vector<float> mass, sigma;
    std::vector<int2> clusters;  // (offset, vertices)
    std::vector<float> clusterMass;
    float Lx = 0, Ly = 0, scale = 1;
};

struct Trajectory {
    bool on = false;
    FrameMeta meta;
    bool headerDone = false;  // the VTF layouts write their header with the first frame
    int every = 0;
    long long lastCommitted = LLONG_MIN;
    int N = 0;
    std::vector<float2 *> pos, vel;  // pinned slots
    std::vector<char> busy;
    std::vector<TrajFrame> pending;
    // writer
    std::thread th;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<TrajFrame> queue;
    bool stop = false;
    std::string error;
    long long written = 0;
};

struct femmd_ctx {
    int device = 0;
    std::string err;
    // MDSystem / Interactions state (host)
    bool inited = false;
    float Lx = 0, Ly = 0, dt = 0.005f, density = 0;
    int pbc = FEMMD_XYPBC, dev_flag = 1, numTypes = 1, steps = 0;
    std::vector<float> eps, rc, us;
    float rCutMax = 0;
    bool bondForces = false, feaForces = false;
    float kBond = 0, E = 0, nu = 0.3f, lambda = 0, mu = 0, C1 = 0, C2 = 0, C3 = 0, gravity = 0, kArea = 0;
    float kWall = 10.0f;  // Interactions::init (interactions.cpp:22)
    float scale = 1.0f;   // MDSystem::scale (set_scale): the cluster VTF radius is 0.5 scale + 0.5
    bool gravityForce = false, areaForces = false;
    int feaLaw = FEMMD_FEA_NEO_HOOKEAN, bondKMode = FEMMD_BONDK_KBOND, imageMode = FEMMD_IMAGE_EXACT;
    int bondMode = FEMMD_ELASTOMER_BONDS_ALL;
    float skin = 0.4f;
    float cellFactor = 1.0f;  // list cells of cellFactor * nnRadius (1: the reference's)
    // per-elastomer material (E, nu) where set; walls
    std::vector<float> elE, elNu;
    std::vector<char> elOwn;
    bool wallOn = false;
    float wallK = 0, wallY0 = 0, wallV = 0;
    // Particles
    std::vector<float2> pos, vel, acc, force, refPos;
    std::vector<float> mass, sigma, energy;
    std::vector<int> type, excl, cluster;
    int nexcl = 0;
    std::vector<Cluster> clusters;
    // Bonds and triangles
    std::vector<int> bond;  // 2 per bond
    std::vector<float> r0;
    std::vector<int> tri;   // 3 per triangle
    std::vector<float> xm, refVol;
    // NeighborList
    bool nnInit = false;
    float nnRadius = 0, nnRadiusSq = 0;
    int ncx = 0, ncy = 0, ncells = 0;
    // device
    cudaStream_t stream = nullptr;
    bool topoDirty = true, stateDirty = true, forcesValid = false, listBuilt = false;
    unsigned staleMask = 0;  // host copies older than the device: bits of kPos..kEnergy
    int cur = 0;
    int nbrCap = 0, Ncap = 0, nBonded = 0, sigmaByType = 1, sigmaOne = 0;
    DBuf<float2> dpos0, dpos1, dvel, dacc, dforce, dref, ckPos, ckVel, ckAcc, triF, triLame;
    DBuf<float> dmass, dsigma, denergy, triE, wallDelta, wallSig;
    bool ownMaterial = false, materialDirty = false;
    // area springs: kept positions and the per-mesh work list
    DBuf<float2> posPre;
    DBuf<int4> areaUnit, areaIdx;
    DBuf<int> areaLane;
    DBuf<float> areaA0;
    int areaUnits = 0, areaSmem = 0;
    std::string areaWhy;  // why the triangles cannot be scheduled ("" when they can)
    // observables: cluster ranges and masses, cluster of each particle, FP64 terms
    DBuf<int2> clRange;
    DBuf<float> clMass;
    DBuf<int> clusterOf;
    DBuf<double2> unf, cmPos, cmVel, centroid;
    DBuf<double> clKin, feaVir, kinTerm, clVir;
    // per-step property averaging (Properties::compute): on/off, window
    // length, equilibration steps, the device accumulator and its copy at
    // the start of a run (restored when the run is repeated)
    bool propAvg = false, propsUploaded = false, propsReset = false;
    int propAvgEvery = 1000, propEqui = 10000, propBlocks = 0;
    DBuf<DevProps> props, propsCk;
    DBuf<double> propPart;
    DBuf<int> dtype, dexcl, cellOf, rank, cellCount, cellStart, blockSums, unsorted, sortedIds, nbr, nbrCount, bStart, tStart,
        tEnt;
    DBuf<int2> bEnt;
    DBuf<int4> triIdx;
    DBuf<float4> triGeo, cellSorted;
    DBuf<PairEntry> pair;
    DBuf<double> obs;
    DBuf<unsigned long long> trace;
    bool tracing = false;
    DBuf<DevScalars> sc;
    DevScalars *hsc = nullptr;  // pinned mirror
    int obsCap = 0, obsRows = 0;
    GraphSet graphs[2][2];      // [parity][0: kGraphUnits units, 1: one unit]
    GraphSet smallGraph;        // the small-system run's WHILE graph (fast mode)
    bool smallGraphFailed = false;
    // the small run's exchange records and tag base are zero (set again after
    // a wait that gave up, which can leave records ahead of the tag base)
    bool smallClean = false;
    bool testExpire = false;  // femmd_test_expire_next_exchange
    // profiling
    bool profiling = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> forceEvents;
    std::vector<cudaEvent_t> eventPool;
    double profForceMs = 0, profRebuildMs = 0;
    long long profForceLaunches = 0, profRebuilds = 0, profKernels = 0;
    long long totalBuilds = 0;
    cudaEvent_t userEvents[64] = {};
    Trajectory traj;
    // adjoint: segment checkpoints of the last femmd_adjoint_forward and the
    // backward sweep's buffers
    struct {
        bool ready = false;
        int every = 0, endStep = 0, maxLen = 0;
        std::vector<int> segStart, segLen;
        std::vector<std::vector<char>> segReb;  // per segment: a rebuild followed MID unit u
        DBuf<float2> ckX, ckV, slots, finalX, finalV, finalA, xbar, vbar, w0, w1, triD;
        DBuf<double> gMu, gLam, epsAcc, sigAcc;
    } adj;
    double lastMeanNbr = 0;
    int lastMaxNbr = 0;
    // fast force mode: the storage order of the free particles (perm), the
    // rebuild's scratch, the id-order constants, the run-start copy of perm,
    // the step blocks' windows
    int forceMode = FEMMD_FORCE_REFERENCE;
    DBuf<int> perm, sPerm, fBlockSums, ckPerm, idType, newCell;
    DBuf<int> blockWin;
    DBuf<unsigned long long> smallRec;
    DBuf<float2> sPos, sVel, sAcc, cpos0, cpos1;
    DBuf<int> cslot;
    DBuf<float> idMass, idSigma, idWallDelta, idWallSig, xfer1;
    float imgD = 0;
};

// ------------------------------------------------------------------ errors

static femmd_status fail(femmd_ctx *c, femmd_status st, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return st;
}

#define CK(call)                                                                                       \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            return fail(ctx, FEMMD_CUDA_ERROR, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                                     \
    } while (0)

#define NEED(ctx)                                                   \
    do {                                                            \
        if (!(ctx)) return FEMMD_INVALID_ARG;                       \
        (ctx)->err.clear();                                         \
    } while (0)

// ------------------------------------------------------------- host physics

// Interactions::setElasticConstants (interactions.cpp:43-50)
static void lame(float E, float nu, float &mu, float &lambda) {
    lambda = E * nu / ((1.0f - 2.0f * nu) * (1.0f + nu));
    mu = E / (2.0f * (1.0f + nu));
}

static void set_elastic_constants(femmd_ctx *c) {
    lame(c->E, c->nu, c->mu, c->lambda);
    c->C1 = c->lambda + 2.0f * c->mu;
    c->C2 = c->lambda;
    c->C3 = c->mu;
}

// contact range of a wall in units of sigma: 2^(1/6) as the reference's
// wall routines form it (interactions.cpp:187), rounded to float
static float wall_range() { return (float)std::pow(2.0, 1.0 / 6.0); }

// pbcCalc (def.h:112)
static float wrap_coord(float r, float L) { return r - std::floor(r / L) * L; }

// invertMatrix (def.h:154-179)
static bool invert3(const float *m, float *out) {
    float inv[9], det;
    det = -m[2] * m[4] * m[6] + m[1] * m[5] * m[6] + m[2] * m[3] * m[7] - m[0] * m[5] * m[7] - m[1] * m[3] * m[8] +
          m[0] * m[4] * m[8];
    if (det == 0) return false;
    inv[0] = -m[5] * m[7] + m[4] * m[8];
    inv[1] = m[2] * m[7] - m[1] * m[8];
    inv[2] = -m[2] * m[4] + m[1] * m[5];
    inv[3] = m[5] * m[6] - m[3] * m[8];
    inv[4] = -m[2] * m[6] + m[0] * m[8];
    inv[5] = m[2] * m[3] - m[0] * m[5];
    inv[6] = -m[4] * m[6] + m[3] * m[7];
    inv[7] = m[1] * m[6] - m[0] * m[7];
    inv[8] = -m[1] * m[3] + m[0] * m[4];
    det = 1.0f / det;
    for (int i = 0; i < 9; i++) out[i] = inv[i] * det;
    return true;
}

static femmd_status download_state(femmd_ctx *ctx, unsigned what);

// Setup calls that change the system first bring device-newer state home.
#define HOSTSYNC(ctx)                                                 \
    do {                                                              \
        femmd_status hs_;                                             \
        if ((ctx)->staleMask && (hs_ = download_state((ctx), kAll))) return hs_; \
    } while (0)

static void mark_topology(femmd_ctx *c) {
    c->topoDirty = true;
    c->stateDirty = true;
    c->forcesValid = false;
    c->listBuilt = false;
}

static void release_graphs(femmd_ctx *c) {
    for (auto &p : c->graphs)
        for (auto &g : p) g.release();
    c->smallGraph.release();
}

static void release_device(femmd_ctx *c) {
    release_graphs(c);
    c->dpos0.release(); c->dpos1.release(); c->dvel.release(); c->dacc.release(); c->dforce.release();
    c->dref.release(); c->ckPos.release(); c->ckVel.release(); c->ckAcc.release(); c->triF.release();
    c->dmass.release(); c->dsigma.release(); c->denergy.release(); c->triE.release();
    c->dtype.release(); c->dexcl.release(); c->cellOf.release(); c->rank.release(); c->cellCount.release();
    c->cellStart.release(); c->blockSums.release(); c->sortedIds.release(); c->unsorted.release(); c->nbr.release();
    c->nbrCount.release(); c->bStart.release(); c->tStart.release(); c->tEnt.release(); c->bEnt.release();
    c->triIdx.release(); c->triGeo.release(); c->cellSorted.release(); c->pair.release();
    c->obs.release(); c->trace.release(); c->sc.release();
    c->triLame.release(); c->wallDelta.release(); c->wallSig.release();
    c->posPre.release(); c->areaUnit.release(); c->areaIdx.release(); c->areaLane.release(); c->areaA0.release();
    c->areaUnits = 0;
    c->clRange.release(); c->clMass.release(); c->clusterOf.release(); c->unf.release(); c->cmPos.release();
    c->cmVel.release(); c->clKin.release(); c->feaVir.release(); c->kinTerm.release(); c->clVir.release();
    c->props.release(); c->propsCk.release(); c->propPart.release(); c->centroid.release();
    c->propsUploaded = false;
    c->perm.release(); c->sPerm.release(); c->fBlockSums.release(); c->ckPerm.release(); c->idType.release();
    c->newCell.release(); c->blockWin.release(); c->smallRec.release(); c->sPos.release(); c->sVel.release(); c->sAcc.release();
    c->cpos0.release(); c->cpos1.release(); c->cslot.release();
    c->idMass.release(); c->idSigma.release(); c->idWallDelta.release(); c->idWallSig.release(); c->xfer1.release();
    auto &a = c->adj;
    a.ckX.release(); a.ckV.release(); a.slots.release(); a.finalX.release(); a.finalV.release(); a.finalA.release();
    a.xbar.release(); a.vbar.release(); a.w0.release(); a.w1.release(); a.triD.release();
    a.gMu.release(); a.gLam.release(); a.epsAcc.release(); a.sigAcc.release();
    a.ready = false;
    c->nbrCap = 0;
    c->obsCap = 0;
}

static void traj_stop(Trajectory &T);
static void traj_refresh_meta(femmd_ctx *ctx);

static void clear_system(femmd_ctx *c) {
    traj_stop(c->traj);  // MDSystem::init clears saveTrajectory (md3dsystem.cpp:65)
    c->traj.on = false;
    c->inited = false;
    c->Lx = c->Ly = 0;
    c->dt = 0.005f;
    c->density = 0;
    c->pbc = FEMMD_XYPBC;
    c->numTypes = 1;
    c->steps = 0;
    c->eps.clear(); c->rc.clear(); c->us.clear();
    c->rCutMax = 0;
    c->bondForces = c->feaForces = false;
    c->kBond = c->E = 0;
    c->nu = 0.3f;
    c->gravity = c->kArea = 0;
    c->gravityForce = false;
    c->kWall = 10.0f;
    c->skin = 0.4f;
    c->cellFactor = 1.0f;
    c->elE.clear(); c->elNu.clear(); c->elOwn.clear();
    c->wallOn = false;
    c->wallK = c->wallY0 = c->wallV = 0;
    c->pos.clear(); c->vel.clear(); c->acc.clear(); c->force.clear(); c->refPos.clear();
    c->mass.clear(); c->sigma.clear(); c->energy.clear(); c->type.clear(); c->excl.clear(); c->cluster.clear();
    c->nexcl = 0;
    c->clusters.clear();
    c->bond.clear(); c->r0.clear(); c->tri.clear(); c->xm.clear(); c->refVol.clear();
    c->nnInit = false;
    c->nnRadius = c->nnRadiusSq = 0;
    c->ncx = c->ncy = c->ncells = 0;
    c->totalBuilds = 0;
    set_elastic_constants(c);
    mark_topology(c);
}

static int add_particle_raw(femmd_ctx *c, float x, float y, float vx, float vy, float m, float sig, int typ) {
    int pid = (int)c->pos.size();
    c->pos.push_back(make_float2(x, y));
    c->vel.push_back(make_float2(vx, vy));
    c->acc.push_back(make_float2(0.f, 0.f));
    c->force.push_back(make_float2(0.f, 0.f));
    c->refPos.push_back(make_float2(0.f, 0.f));
    c->mass.push_back(m);
    c->sigma.push_back(sig);
    c->energy.push_back(0.f);
    c->type.push_back(typ);
    c->excl.push_back(-1);
    c->cluster.push_back(-1);
    c->density = (float)(int)c->pos.size() / (c->Lx * c->Ly);
    return pid;
}

static void create_bond_raw(femmd_ctx *c, int i, int j) {
    c->bond.push_back(i);
    c->bond.push_back(j);
    float dx = c->pos[i].x - c->pos[j].x;
    float dy = c->pos[i].y - c->pos[j].y;
    c->r0.push_back(std::sqrt(dx * dx + dy * dy));
}

// ------------------------------------------------------------- device upload

static DevSys make_sys(femmd_ctx *c) {
    DevSys s = {};
    s.N = (int)c->pos.size();
    s.Ncap = c->Ncap;
    s.wrapx = (c->pbc == FEMMD_XYPBC || c->pbc == FEMMD_XPBC);
    s.wrapy = (c->pbc == FEMMD_XYPBC);
    s.Lx = c->Lx;
    s.Ly = c->Ly;
    s.dt = c->dt;
    s.hdt = 0.5f * c->dt;
    s.halfSkin = 0.5 * (double)c->skin;
    s.ncx = c->ncx;
    s.ncy = c->ncy;
    s.ncells = c->ncells;
    s.nnRadiusSq = c->nnRadiusSq;
    s.imageExact = c->imageMode == FEMMD_IMAGE_EXACT;
    s.numTypes = c->numTypes;
    s.sigmaByType = c->sigmaByType;
    s.sigmaOne = c->sigmaOne;
    s.pair = c->pair.p;
    s.pos0 = c->dpos0.p;
    s.pos1 = c->dpos1.p;
    s.vel = c->dvel.p;
    s.acc = c->dacc.p;
    s.forceOut = c->dforce.p;
    s.energyOut = c->denergy.p;
    s.mass = c->dmass.p;
    s.sigma = c->dsigma.p;
    s.typeId = c->dtype.p;
    s.excl = c->dexcl.p;
    s.cellOf = c->cellOf.p;
    s.rank = c->rank.p;
    s.cellCount = c->cellCount.p;
    s.cellStart = c->cellStart.p;
    s.blockSums = c->blockSums.p;
    s.sortedIds = c->sortedIds.p;
    s.unsorted = c->unsorted.p;
    s.cellSorted = c->cellSorted.p;
    s.nbr = c->nbr.p;
    s.nbrCount = c->nbrCount.p;
    s.nbrCap = c->nbrCap;
    s.nBonded = c->nBonded;
    s.bondForces = c->bondForces && !c->r0.empty();
    s.feaForces = c->feaForces && !c->refVol.empty();
    s.feaLaw = c->feaLaw;
    s.bondKMode = c->bondKMode;
    s.bStart = c->bStart.p;
    s.bEnt = c->bEnt.p;
    s.tStart = c->tStart.p;
    s.tEnt = c->tEnt.p;
    s.ntri = (int)c->refVol.size();
    s.triIdx = c->triIdx.p;
    s.triGeo = c->triGeo.p;
    s.triF = c->triF.p;
    s.triE = c->triE.p;
    s.refPos = c->dref.p;
    s.kBond = c->kBond;
    s.E = c->E;
    s.mu = c->mu;
    s.lambda = c->lambda;
    s.C1 = c->C1;
    s.C2 = c->C2;
    s.C3 = c->C3;
    s.sc = c->sc.p;
    s.obs = c->obs.p;
    s.obsCap = c->obsCap;
    s.trace = c->tracing ? c->trace.p : nullptr;
    s.triLame = c->ownMaterial ? c->triLame.p : nullptr;
    s.wallOn = c->wallOn;
    s.wallK = c->wallK;
    s.wallY0 = c->wallY0;
    s.wallV = c->wallV;
    s.wallDelta = c->wallOn ? c->wallDelta.p : nullptr;
    s.stepBase = c->steps;
    s.refWalls = (!c->wallOn && c->pbc != FEMMD_XYPBC) ? (c->pbc == FEMMD_NOPBC ? 1 : 2) : 0;
    s.kWall = c->kWall;
    s.wallRc = wall_range();
    s.gravity = c->gravityForce ? c->gravity : 0.0f;
    s.wallSig = (c->wallOn || c->pbc != FEMMD_XYPBC) ? c->wallSig.p : nullptr;
    const bool area = c->areaForces && c->areaUnits > 0 && c->areaWhy.empty();
    s.kArea = c->kArea;
    s.areaUnits = area ? c->areaUnits : 0;
    s.areaSmem = c->areaSmem;
    s.areaUnit = c->areaUnit.p;
    s.areaLane = c->areaLane.p;
    s.areaIdx = c->areaIdx.p;
    s.areaA0 = c->areaA0.p;
    s.posPre = area ? c->posPre.p : nullptr;
    s.nPre = area ? c->nBonded : 0;
    s.fast = c->forceMode == FEMMD_FORCE_FAST;
    if (s.fast) {
        s.imgD = c->imgD;
        s.perm = c->perm.p;
        s.sPos = c->sPos.p;
        s.sVel = c->sVel.p;
        s.sAcc = c->sAcc.p;
        s.sPerm = c->sPerm.p;
        s.fBlockSums = c->fBlockSums.p;
        s.idMass = c->idMass.p;
        s.idType = c->idType.p;
        s.idSigma = c->idSigma.p;
        s.idWallDelta = s.wallDelta ? c->idWallDelta.p : nullptr;
        s.idWallSig = s.wallSig ? c->idWallSig.p : nullptr;
        s.newCell = c->newCell.p;
        s.blockWin = c->blockWin.p;
        s.smallRec = c->smallRec.p;
        s.win16 = (c->nBonded == 0 && s.numTypes == 1 && s.sigmaByType) ? 1 : 0;
        if (c->cslot.p) {
            s.cpos0 = c->cpos0.p;
            s.cpos1 = c->cpos1.p;
            s.cslot = c->cslot.p;
            s.cposOn = area ? 0 : 1;
        }
    }
    return s;
}

// Fast force mode: the device stores particles in its own order (perm[s] =
// id at slot s).  Host arrays are in id order; these convert on the way in
// and out through the rebuild's scratch arrays.
static bool fast_mode(const femmd_ctx *c) { return c->forceMode == FEMMD_FORCE_FAST; }

// Device array 'in' (storage order) to host 'out' (id order), N float2.
static cudaError_t fast_download2(femmd_ctx *c, const float2 *in, void *out) {
    const int N = (int)c->pos.size();
    DevSys s = make_sys(c);
    Launch L;
    L.stream = c->stream;
    cudaError_t e = enqueue_unpermute2(L, s, in, c->sPos.p);
    if (e) return e;
    return cudaMemcpyAsync(out, c->sPos.p, N * sizeof(float2), cudaMemcpyDeviceToHost, c->stream);
}

// Host 'in' (id order) to device array 'out' (storage order), N float2.
static cudaError_t fast_upload2(femmd_ctx *c, const void *in, float2 *out) {
    const int N = (int)c->pos.size();
    cudaError_t e = cudaMemcpyAsync(c->sPos.p, in, N * sizeof(float2), cudaMemcpyHostToDevice, c->stream);
    if (e) return e;
    DevSys s = make_sys(c);
    Launch L;
    L.stream = c->stream;
    return enqueue_permute2(L, s, c->sPos.p, out);
}

static femmd_status ensure_stream(femmd_ctx *ctx) {
    if (ctx->stream) return FEMMD_OK;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    CK(cudaMallocHost(&ctx->hsc, sizeof(DevScalars)));
    memset(ctx->hsc, 0, sizeof(DevScalars));
    return FEMMD_OK;
}

static femmd_status validate(femmd_ctx *ctx) {
    if (!ctx->inited) return fail(ctx, FEMMD_NOT_READY, "init(Lx, Ly) has not been called");
    if (!ctx->nnInit) return fail(ctx, FEMMD_NOT_READY, "init_neighbor_list() has not been called");
    int N = (int)ctx->pos.size();
    if (N > kIdMask) return fail(ctx, FEMMD_INVALID_ARG, "at most %d particles are supported", kIdMask);
    if (ctx->numTypes < 1 || ctx->numTypes > kMaxTypes)
        return fail(ctx, FEMMD_INVALID_ARG, "numTypes must be in [1, %d]", kMaxTypes);
    if ((int)ctx->eps.size() < ctx->numTypes * ctx->numTypes)
        return fail(ctx, FEMMD_INVALID_ARG, "pair table has %zu entries, numTypes^2 = %d needed", ctx->eps.size(),
                    ctx->numTypes * ctx->numTypes);
    for (int i = 0; i < N; i++) {
        if (ctx->type[i] < 0 || ctx->type[i] >= ctx->numTypes)
            return fail(ctx, FEMMD_INVALID_ARG, "particle %d has type %d outside [0, %d)", i, ctx->type[i],
                        ctx->numTypes);
        if (!(ctx->mass[i] != 0.0f)) return fail(ctx, FEMMD_INVALID_ARG, "particle %d has zero mass", i);
        if (!std::isfinite(ctx->pos[i].x) || !std::isfinite(ctx->pos[i].y) || !std::isfinite(ctx->vel[i].x) ||
            !std::isfinite(ctx->vel[i].y))
            return fail(ctx, FEMMD_INVALID_ARG, "particle %d has a non-finite position or velocity", i);
    }
    if (ctx->wallOn && ctx->pbc == FEMMD_XYPBC)
        return fail(ctx, FEMMD_INVALID_ARG, "walls need a box that is not periodic in y (PBC 0 or 1)");
    bool own = false;
    for (char o : ctx->elOwn) own = own || o;
    if (own && ctx->feaLaw != FEMMD_FEA_NEO_HOOKEAN)
        return fail(ctx, FEMMD_UNSUPPORTED, "per-elastomer materials are implemented for the neo-Hookean law");
    return FEMMD_OK;
}

// Per-triangle Lame constants (the elastomer's own (E, nu) through the same
// float operations as the global constants, or the global ones) and the
// per-particle wall contact ranges.
static femmd_status upload_material(femmd_ctx *ctx) {
    const int N = (int)ctx->pos.size(), nt = (int)ctx->refVol.size();
    cudaStream_t s = ctx->stream;
    ctx->ownMaterial = false;
    for (char o : ctx->elOwn) ctx->ownMaterial = ctx->ownMaterial || o;
    if (ctx->ownMaterial) {
        std::vector<float2> lm(std::max(nt, 1), make_float2(ctx->mu, ctx->lambda));
        for (size_t e = 0; e < ctx->clusters.size() && e < ctx->elOwn.size(); e++) {
            if (!ctx->elOwn[e]) continue;
            float mu, lambda;
            lame(ctx->elE[e], ctx->elNu[e], mu, lambda);
            const Cluster &cl = ctx->clusters[e];
            for (int t = cl.tetOffset; t < cl.tetOffset + cl.nt && t < nt; t++) lm[t] = make_float2(mu, lambda);
        }
        CK(ctx->triLame.ensure(lm.size()));
        CK(cudaMemcpyAsync(ctx->triLame.p, lm.data(), lm.size() * sizeof(float2), cudaMemcpyHostToDevice, s));
    }
    if ((ctx->wallOn || ctx->pbc != FEMMD_XYPBC) && N > 0) {
        std::vector<float> dl(N);
        const float range = wall_range();
        for (int i = 0; i < N; i++) dl[i] = range * ctx->sigma[i];
        CK(ctx->wallDelta.ensure(N));
        CK(ctx->wallSig.ensure(N));
        CK(cudaMemcpyAsync(ctx->wallDelta.p, dl.data(), N * sizeof(float), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->wallSig.p, ctx->sigma.data(), N * sizeof(float), cudaMemcpyHostToDevice, s));
        if (fast_mode(ctx)) {
            // id-order originals, then the storage-order copies through perm
            CK(ctx->idWallDelta.ensure(N));
            CK(ctx->idWallSig.ensure(N));
            CK(cudaMemcpyAsync(ctx->idWallDelta.p, dl.data(), N * sizeof(float), cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(ctx->idWallSig.p, ctx->sigma.data(), N * sizeof(float), cudaMemcpyHostToDevice, s));
            if (!ctx->topoDirty && !ctx->stateDirty) {
                DevSys ds = make_sys(ctx);
                ds.wallDelta = ctx->wallDelta.p;
                ds.wallSig = ctx->wallSig.p;
                ds.idWallDelta = ctx->idWallDelta.p;
                ds.idWallSig = ctx->idWallSig.p;
                Launch L;
                L.stream = s;
                CK(enqueue_perm_consts(L, ds));
            }
        }
    }
    CK(cudaStreamSynchronize(s));
    ctx->materialDirty = false;
    return FEMMD_OK;
}

// The area springs' work list (calcAreaForcesCPU, interactions.cpp:696-750).
// Each elastomer's triangles keep the reference's order and run serially in
// one lane.  Elastomers with the same mesh (vertex count and triangle list
// inside the elastomer) share blocks of up to 32 lanes, as many as the
// shared memory holds; A0 of every triangle is formed here from the
// reference positions by the reference's float operations, per elastomer
// (the rounding depends on where the elastomer was placed).
static femmd_status upload_area_schedule(femmd_ctx *ctx) {
    ctx->areaUnits = 0;
    ctx->areaSmem = 0;
    ctx->areaWhy.clear();
    const int nt = (int)ctx->refVol.size(), ncl = (int)ctx->clusters.size();
    if (nt == 0) return FEMMD_OK;
    std::vector<std::vector<int>> byCl(ncl);
    for (int t = 0; t < nt; t++) {
        const int *v = &ctx->tri[3 * (size_t)t];
        const int c = ctx->cluster[v[0]];
        bool ok = c >= 0 && c < ncl;
        for (int k = 0; ok && k < 3; k++)
            ok = ctx->cluster[v[k]] == c && v[k] >= ctx->clusters[c].offset &&
                 v[k] < ctx->clusters[c].offset + ctx->clusters[c].nv;
        if (!ok) {
            ctx->areaWhy = "a triangle's vertices lie in different elastomers";
            return FEMMD_OK;
        }
        byCl[c].push_back(t);
    }
    // meshes
    std::map<std::vector<int>, int> meshOf;
    std::vector<int4> idx;
    std::vector<int> meshBase, meshNt, meshNv;
    std::vector<std::vector<int>> members;
    for (int c = 0; c < ncl; c++) {
        if (byCl[c].empty()) continue;
        const int off = ctx->clusters[c].offset;
        std::vector<int> key(1, ctx->clusters[c].nv);
        for (int t : byCl[c])
            for (int k = 0; k < 3; k++) key.push_back(ctx->tri[3 * (size_t)t + k] - off);
        auto it = meshOf.find(key);
        int m;
        if (it == meshOf.end()) {
            m = (int)meshBase.size();
            meshOf.emplace(key, m);
            meshBase.push_back((int)idx.size());
            meshNt.push_back((int)byCl[c].size());
            meshNv.push_back(ctx->clusters[c].nv);
            members.emplace_back();
            for (size_t k = 1; k < key.size(); k += 3) idx.push_back(make_int4(key[k], key[k + 1], key[k + 2], 0));
        } else {
            m = it->second;
        }
        members[m].push_back(c);
    }
    const size_t limit = 200 * 1024;
    std::vector<int4> unit;
    std::vector<int> lane;
    std::vector<float> a0;
    size_t smem = 0;
    for (size_t m = 0; m < members.size(); m++) {
        const size_t mnt = meshNt[m], mnv = meshNv[m];
        auto bytes = [&](size_t nl) { return mnt * 16 + ((mnt * nl + 3) & ~(size_t)3) * 4 + mnv * (nl + 1) * 8; };
        size_t W = 32;
        while (W > 1 && bytes(W) > limit) W--;
        if (bytes(W) > limit) {
            ctx->areaWhy = "an elastomer's mesh does not fit one block's shared memory";
            return FEMMD_OK;
        }
        for (size_t j0 = 0; j0 < members[m].size(); j0 += W) {
            const int nl = (int)std::min(W, members[m].size() - j0);
            unit.push_back(make_int4(meshBase[m], (int)mnt, (int)mnv, nl));
            unit.push_back(make_int4((int)a0.size(), 0, 0, 0));
            const size_t a0b = a0.size();
            a0.resize(a0b + ((mnt * nl + 3) & ~(size_t)3));  // 16-byte ranges (copied in 16-byte pieces)
            for (int j = 0; j < 32; j++) lane.push_back(j < nl ? ctx->clusters[members[m][j0 + j]].offset : 0);
            for (int j = 0; j < nl; j++) {
                const int c = members[m][j0 + j];
                for (size_t k = 0; k < mnt; k++) {
                    const int *v = &ctx->tri[3 * (size_t)byCl[c][k]];
                    const float2 q0 = ctx->refPos[v[0]], q1 = ctx->refPos[v[1]], q2 = ctx->refPos[v[2]];
                    a0[a0b + k * nl + j] = 0.5f * ((q2.y - q0.y) * (q1.x - q0.x) - (q1.y - q0.y) * (q2.x - q0.x));
                }
            }
            smem = std::max(smem, bytes(nl));
        }
    }
    if (smem > 48 * 1024) CK(area_smem_setup((int)smem));
    cudaStream_t s = ctx->stream;
    CK(ctx->areaUnit.ensure(unit.size())); CK(ctx->areaIdx.ensure(idx.size()));
    CK(ctx->areaLane.ensure(lane.size())); CK(ctx->areaA0.ensure(std::max(a0.size(), (size_t)1)));
    CK(ctx->posPre.ensure(std::max(ctx->nBonded, 1)));
    CK(cudaMemcpyAsync(ctx->areaUnit.p, unit.data(), unit.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->areaIdx.p, idx.data(), idx.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->areaLane.p, lane.data(), lane.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->areaA0.p, a0.data(), a0.size() * sizeof(float), cudaMemcpyHostToDevice, s));
    ctx->areaUnits = (int)unit.size() / 2;
    ctx->areaSmem = (int)smem;
    return FEMMD_OK;
}

static femmd_status upload_topology(femmd_ctx *ctx) {
    femmd_status st;
    if ((st = ensure_stream(ctx))) return st;
    release_graphs(ctx);
    const int N = (int)ctx->pos.size();
    ctx->Ncap = std::max(32, (N + 31) / 32 * 32);
    // sigma as a function of type?
    {
        std::vector<float> st_sig(ctx->numTypes, 0.f);
        std::vector<char> seen(ctx->numTypes, 0);
        ctx->sigmaByType = 1;
        for (int i = 0; i < N; i++) {
            int t = ctx->type[i];
            if (!seen[t]) { seen[t] = 1; st_sig[t] = ctx->sigma[i]; }
            else if (st_sig[t] != ctx->sigma[i]) ctx->sigmaByType = 0;
        }
        std::vector<PairEntry> tab((size_t)ctx->numTypes * ctx->numTypes);
        for (int a = 0; a < ctx->numTypes; a++)
            for (int b = 0; b < ctx->numTypes; b++) {
                PairEntry &p = tab[a * ctx->numTypes + b];
                float e = ctx->eps[a * ctx->numTypes + b], r = ctx->rc[a * ctx->numTypes + b];
                float sij = (st_sig[a] + st_sig[b]) / 2.0f;  // pairForce: (sigma[i]+sigma[j])/2
                p.rcut2 = r * r * sij * sij;
                p.sig2 = sij * sij;
                p.c = 48.0f * e / (sij * sij);
                p.eps4 = 4.0f * e;
                p.us = ctx->us[a * ctx->numTypes + b];
                p.rc = r;
                p.eps48 = 48.0f * e;
                p.pad = 0.f;
            }
        // pairs of types that no particle has are never evaluated
        ctx->sigmaOne = ctx->sigmaByType;
        for (int a = 0; a < ctx->numTypes; a++)
            for (int b = 0; b < ctx->numTypes; b++)
                if (seen[a] && seen[b]) ctx->sigmaOne = ctx->sigmaOne && tab[a * ctx->numTypes + b].sig2 == 1.0f;
        CK(ctx->pair.ensure(tab.size()));
        CK(cudaMemcpyAsync(ctx->pair.p, tab.data(), tab.size() * sizeof(PairEntry), cudaMemcpyHostToDevice,
                           ctx->stream));
    }
    // positions hold one more slot: the ghost that pads the fast mode's lists
    CK(ctx->dpos0.ensure(N + 1)); CK(ctx->dpos1.ensure(N + 1)); CK(ctx->dvel.ensure(N)); CK(ctx->dacc.ensure(N));
    CK(ctx->dforce.ensure(N)); CK(ctx->denergy.ensure(N)); CK(ctx->dref.ensure(N));
    CK(ctx->ckPos.ensure(N)); CK(ctx->ckVel.ensure(N)); CK(ctx->ckAcc.ensure(N));
    CK(ctx->dmass.ensure(N)); CK(ctx->dtype.ensure(N)); CK(ctx->dexcl.ensure(N));
    CK(ctx->dsigma.ensure(ctx->sigmaByType ? 1 : N + 1));  // + the ghost slot
    CK(ctx->cellOf.ensure(N)); CK(ctx->rank.ensure(N)); CK(ctx->sortedIds.ensure(N)); CK(ctx->unsorted.ensure(N));
    CK(ctx->cellSorted.ensure(N)); CK(ctx->nbrCount.ensure(N));
    CK(ctx->cellCount.ensure(ctx->ncells));
    // cellStart: ncells + 1 words, padded: the fast list build copies
    // cell-start ranges rounded out to 16 bytes
    CK(ctx->cellStart.ensure(ctx->ncells + 8));
    CK(ctx->blockSums.ensure(scan_blocks(ctx->ncells)));
    CK(ctx->sc.ensure(1));
    cudaStream_t s = ctx->stream;
    if (N > 0) {
        CK(cudaMemcpyAsync(ctx->dmass.p, ctx->mass.data(), N * sizeof(float), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->dtype.p, ctx->type.data(), N * sizeof(int), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->dexcl.p, ctx->excl.data(), N * sizeof(int), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->dref.p, ctx->refPos.data(), N * sizeof(float2), cudaMemcpyHostToDevice, s));
        if (!ctx->sigmaByType) {
            static const float one = 1.0f;
            CK(cudaMemcpyAsync(ctx->dsigma.p, ctx->sigma.data(), N * sizeof(float), cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(ctx->dsigma.p + N, &one, sizeof(float), cudaMemcpyHostToDevice, s));
        }
    }
    CK(cudaMemsetAsync(ctx->cellCount.p, 0, sizeof(int) * std::max(ctx->ncells, 1), s));
    CK(cudaMemsetAsync(ctx->sc.p, 0, sizeof(DevScalars), s));
    // bonded incidences: bond order / triangle order per particle
    const int nb = (int)ctx->r0.size(), nt = (int)ctx->refVol.size();
    int nbd = 0;
    for (int v : ctx->bond) nbd = std::max(nbd, v + 1);
    for (int v : ctx->tri) nbd = std::max(nbd, v + 1);
    ctx->nBonded = nbd;
    {
        std::vector<int> bs(nbd + 1, 0), ts(nbd + 1, 0);
        for (int l = 0; l < nb; l++) { bs[ctx->bond[2 * l] + 1]++; bs[ctx->bond[2 * l + 1] + 1]++; }
        for (int v : ctx->tri) ts[v + 1]++;
        for (int v = 0; v < nbd; v++) { bs[v + 1] += bs[v]; ts[v + 1] += ts[v]; }
        std::vector<int2> be(std::max(bs[nbd], 1));
        std::vector<int> te(std::max(ts[nbd], 1));
        std::vector<int> fb2(bs.begin(), bs.end() - 1), ft(ts.begin(), ts.end() - 1);
        for (int l = 0; l < nb; l++) {
            int i = ctx->bond[2 * l], j = ctx->bond[2 * l + 1];
            int r0bits;
            memcpy(&r0bits, &ctx->r0[l], 4);
            be[fb2[i]++] = make_int2(j, r0bits);
            be[fb2[j]++] = make_int2((int)((unsigned)i | 0x80000000u), r0bits);
        }
        for (int t = 0; t < nt; t++)
            for (int k = 0; k < 3; k++) te[ft[ctx->tri[3 * t + k]]++] = t * 4 + k;
        CK(ctx->bStart.ensure(nbd + 1)); CK(ctx->tStart.ensure(nbd + 1));
        CK(ctx->bEnt.ensure(be.size())); CK(ctx->tEnt.ensure(te.size()));
        CK(cudaMemcpyAsync(ctx->bStart.p, bs.data(), bs.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->tStart.p, ts.data(), ts.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->bEnt.p, be.data(), be.size() * sizeof(int2), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->tEnt.p, te.data(), te.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        // triangle geometry from the reference positions
        std::vector<int4> ti(std::max(nt, 1));
        std::vector<float4> tg(2 * (size_t)std::max(nt, 1));
        for (int t = 0; t < nt; t++) {
            int p0 = ctx->tri[3 * t], p1 = ctx->tri[3 * t + 1], p2 = ctx->tri[3 * t + 2];
            ti[t] = make_int4(p0, p1, p2, 0);
            float X0 = ctx->refPos[p0].x, Y0 = ctx->refPos[p0].y, X1 = ctx->refPos[p1].x, Y1 = ctx->refPos[p1].y;
            float X2 = ctx->refPos[p2].x, Y2 = ctx->refPos[p2].y;
            if (ctx->feaLaw == FEMMD_FEA_NEO_HOOKEAN) {
                // calcFeaForcesCPU2 Dm, Bm, vol0 (interactions.cpp:589-602)
                float Dm00 = X0 - X2, Dm10 = Y0 - Y2, Dm01 = X1 - X2, Dm11 = Y1 - Y2;
                float detDm = Dm00 * Dm11 - Dm01 * Dm10;
                float vol0 = detDm / 2.0f;
                tg[2 * t] = make_float4(Dm11 / detDm, -Dm10 / detDm, -Dm01 / detDm, Dm00 / detDm);
                tg[2 * t + 1] = make_float4(vol0, 0.f, 0.f, 0.f);
            } else {
                // computeFeaForcesGPU xm and |area| (interactionsCuda.cu:364-383)
                float aa[9] = {1.0f, X0, Y0, 1.0f, X1, Y1, 1.0f, X2, Y2}, mm[9];
                if (!invert3(aa, mm)) memset(mm, 0, sizeof mm);
                float tv = std::fabs(0.5f * ((Y2 - Y0) * (X1 - X0) - (Y1 - Y0) * (X2 - X0)));
                tg[2 * t] = make_float4(mm[3], mm[4], mm[5], mm[6]);
                tg[2 * t + 1] = make_float4(mm[7], mm[8], tv, 0.f);
            }
        }
        CK(ctx->triIdx.ensure(ti.size())); CK(ctx->triGeo.ensure(tg.size()));
        CK(ctx->triF.ensure(3 * ti.size())); CK(ctx->triE.ensure(ti.size()));
        CK(cudaMemcpyAsync(ctx->triIdx.p, ti.data(), ti.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->triGeo.p, tg.data(), tg.size() * sizeof(float4), cudaMemcpyHostToDevice, s));
    }
    if (fast_mode(ctx) && N > 0) {
        CK(ctx->perm.ensure(N)); CK(ctx->sPerm.ensure(N)); CK(ctx->ckPerm.ensure(N)); CK(ctx->xfer1.ensure(N));
        CK(ctx->sPos.ensure(N)); CK(ctx->sVel.ensure(N)); CK(ctx->sAcc.ensure(N));
        CK(ctx->fBlockSums.ensure((N + 1023) / 1024));
        CK(ctx->newCell.ensure(N));
        CK(ctx->blockWin.ensure(kWinInts * (size_t)((N + kFastBlock - 1) / kFastBlock)));
        CK(ctx->smallRec.ensure(3 * 4 * (size_t)kSmallMaxTiles));
        ctx->smallClean = false;
        if (ctx->nBonded > 0) {
            // the cell-ordered position mirror (slot N: the ghost)
            CK(ctx->cpos0.ensure(N + 1)); CK(ctx->cpos1.ensure(N + 1)); CK(ctx->cslot.ensure(N));
            static const float2 far = make_float2(3.0e15f, 3.0e15f);
            CK(cudaMemcpyAsync(ctx->cpos0.p + N, &far, sizeof(float2), cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(ctx->cpos1.p + N, &far, sizeof(float2), cudaMemcpyHostToDevice, s));
        } else {
            ctx->cpos0.release(); ctx->cpos1.release(); ctx->cslot.release();
        }
        CK(ctx->idMass.ensure(N)); CK(ctx->idType.ensure(N)); CK(ctx->idSigma.ensure(ctx->sigmaByType ? 1 : N));
        CK(cudaMemcpyAsync(ctx->idMass.p, ctx->mass.data(), N * sizeof(float), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->idType.p, ctx->type.data(), N * sizeof(int), cudaMemcpyHostToDevice, s));
        if (!ctx->sigmaByType)
            CK(cudaMemcpyAsync(ctx->idSigma.p, ctx->sigma.data(), N * sizeof(float), cudaMemcpyHostToDevice, s));
        // the largest pair cutoff in length units: a particle farther than
        // that from every periodic edge has no interacting pair across it
        float rmax = ctx->nnRadius, smax = 0.0f;
        for (int i = 0; i < N; i++) smax = std::max(smax, ctx->sigma[i]);
        for (size_t q = 0; q < ctx->rc.size(); q++) rmax = std::max(rmax, ctx->rc[q] * smax);
        ctx->imgD = rmax + 1e-3f;
    }
    if ((st = upload_area_schedule(ctx))) return st;
    ctx->propsUploaded = false;
    if ((st = upload_material(ctx))) return st;
    ctx->topoDirty = false;
    ctx->listBuilt = false;
    CK(cudaStreamSynchronize(s));
    return FEMMD_OK;
}

static femmd_status upload_state(femmd_ctx *ctx) {
    const int N = (int)ctx->pos.size();
    cudaStream_t s = ctx->stream;
    if (N > 0) {
        CK(cudaMemcpyAsync(ctx->dpos0.p, ctx->pos.data(), N * sizeof(float2), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->dvel.p, ctx->vel.data(), N * sizeof(float2), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->dacc.p, ctx->acc.data(), N * sizeof(float2), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->dforce.p, ctx->force.data(), N * sizeof(float2), cudaMemcpyHostToDevice, s));
        // the ghost slot N, far outside the box (the fast mode's list
        // padding): its distance to any particle is beyond every cutoff, its
        // square finite
        static const float2 ghost = make_float2(3.0e15f, 3.0e15f);
        CK(cudaMemcpyAsync(ctx->dpos0.p + N, &ghost, sizeof(float2), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->dpos1.p + N, &ghost, sizeof(float2), cudaMemcpyHostToDevice, s));
        if (fast_mode(ctx)) {
            // the state arrives in id order: storage order = id order
            DevSys ds = make_sys(ctx);
            Launch L;
            L.stream = s;
            CK(enqueue_perm_identity(L, ds));
        }
    }
    ctx->cur = 0;
    ctx->stateDirty = false;
    ctx->listBuilt = false;
    ctx->staleMask = 0;
    CK(cudaStreamSynchronize(s));
    return FEMMD_OK;
}

// Bring the host copies named by 'what' up to date with the device.
static femmd_status download_state(femmd_ctx *ctx, unsigned what) {
    what &= ctx->staleMask;
    if (!what) return FEMMD_OK;
    const int N = (int)ctx->pos.size();
    cudaStream_t s = ctx->stream;
    if (N > 0 && fast_mode(ctx)) {
        if (what & kPos) CK(fast_download2(ctx, ctx->cur ? ctx->dpos1.p : ctx->dpos0.p, ctx->pos.data()));
        if (what & kVel) CK(fast_download2(ctx, ctx->dvel.p, ctx->vel.data()));
        if (what & kAcc) CK(fast_download2(ctx, ctx->dacc.p, ctx->acc.data()));
        if (what & kForce) CK(fast_download2(ctx, ctx->dforce.p, ctx->force.data()));
        if (what & kEnergy) {
            DevSys ds = make_sys(ctx);
            Launch L;
            L.stream = s;
            CK(enqueue_unpermute1(L, ds, ctx->denergy.p, ctx->xfer1.p));
            CK(cudaMemcpyAsync(ctx->energy.data(), ctx->xfer1.p, N * sizeof(float), cudaMemcpyDeviceToHost, s));
        }
        CK(cudaStreamSynchronize(s));
    } else if (N > 0) {
        if (what & kPos)
            CK(cudaMemcpyAsync(ctx->pos.data(), ctx->cur ? ctx->dpos1.p : ctx->dpos0.p, N * sizeof(float2),
                               cudaMemcpyDeviceToHost, s));
        if (what & kVel) CK(cudaMemcpyAsync(ctx->vel.data(), ctx->dvel.p, N * sizeof(float2), cudaMemcpyDeviceToHost, s));
        if (what & kAcc) CK(cudaMemcpyAsync(ctx->acc.data(), ctx->dacc.p, N * sizeof(float2), cudaMemcpyDeviceToHost, s));
        if (what & kForce)
            CK(cudaMemcpyAsync(ctx->force.data(), ctx->dforce.p, N * sizeof(float2), cudaMemcpyDeviceToHost, s));
        if (what & kEnergy)
            CK(cudaMemcpyAsync(ctx->energy.data(), ctx->denergy.p, N * sizeof(float), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    ctx->staleMask &= ~what;
    return FEMMD_OK;
}

static femmd_status read_scalars(femmd_ctx *ctx) {
    CK(cudaMemcpyAsync(ctx->hsc, ctx->sc.p, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return FEMMD_OK;
}

// Neighbour-list storage for capacity 'cap' per particle (rounded up to the
// list's groups of four).
static femmd_status alloc_list(femmd_ctx *ctx, int cap) {
    cap = (std::max(1, cap) + 3) / 4 * 4;
    // at least two groups of storage: the fast step kernel loads a
    // particle's first two groups before it knows the list's length
    CK(ctx->nbr.ensure((size_t)std::max(cap, 8) * ctx->Ncap));
    ctx->nbrCap = cap;
    release_graphs(ctx);
    return FEMMD_OK;
}

// Sizing pass: bin and count with capacity 0, then allocate max count * 1.25 + 8.
static femmd_status size_list(femmd_ctx *ctx, int min_cap) {
    DevSys s = make_sys(ctx);
    s.nbrCap = 0;
    Launch L;
    L.stream = ctx->stream;
    CK(cudaMemsetAsync(&ctx->sc.p->overflow, 0, 3 * sizeof(int), ctx->stream));
    CK(enqueue_rebuild(L, s, ctx->cur, 0));
    femmd_status st;
    if ((st = read_scalars(ctx))) return st;
    if (ctx->hsc->nonfinite) return fail(ctx, FEMMD_NONFINITE, "a position is NaN or infinite");
    int need = ctx->hsc->maxCount + ctx->hsc->maxCount / 4 + 8;
    CK(cudaMemsetAsync(&ctx->sc.p->overflow, 0, 3 * sizeof(int), ctx->stream));
    return alloc_list(ctx, std::max(need, min_cap));
}

static femmd_status props_buffers(femmd_ctx *ctx);

static femmd_status prepare(femmd_ctx *ctx) {
    femmd_status st;
    if (!ctx->nnInit) return fail(ctx, FEMMD_NOT_READY, "init_neighbor_list() has not been called");
    if ((ctx->topoDirty || ctx->materialDirty) && (st = validate(ctx))) return st;
    if (ctx->topoDirty) {
        if ((st = upload_topology(ctx))) return st;
        traj_refresh_meta(ctx);
    }
    if (ctx->stateDirty && (st = upload_state(ctx))) return st;
    if (ctx->materialDirty && (st = upload_material(ctx))) return st;
    if (ctx->nbrCap == 0 && (st = size_list(ctx, 0))) return st;
    if (ctx->areaForces && !ctx->areaWhy.empty())
        return fail(ctx, FEMMD_UNSUPPORTED, "area springs: %s", ctx->areaWhy.c_str());
    if (ctx->propAvg) {
        if (!ctx->propsUploaded) {
            if ((st = props_buffers(ctx))) return st;
            release_graphs(ctx);
        }
        if (!ctx->props.p || ctx->propsReset) {
            CK(ctx->props.ensure(1)); CK(ctx->propsCk.ensure(1));
            CK(cudaMemsetAsync(ctx->props.p, 0, sizeof(DevProps), ctx->stream));
            ctx->propsReset = false;
        }
    }
    return FEMMD_OK;
}

static femmd_status ensure_obs(femmd_ctx *ctx, int rows) {
    rows = std::min(rows, 1 << 20);
    if (rows <= ctx->obsCap) return FEMMD_OK;
    int cap = std::max(rows, 1024);
    CK(ctx->obs.ensure((size_t)cap * kObsCols));
    CK(ctx->trace.ensure((size_t)cap * kTraceCols));
    ctx->obsCap = cap;
    release_graphs(ctx);
    return FEMMD_OK;
}

// Cluster ranges, masses and the cluster of each particle, and the term
// arrays of the observables kernels.
static femmd_status props_buffers(femmd_ctx *ctx) {
    const int N = (int)ctx->pos.size(), nt = (int)ctx->refVol.size(), ncl = (int)ctx->clusters.size();
    cudaStream_t sm = ctx->stream;
    if (ncl > 0) {
        std::vector<int2> rg(ncl);
        std::vector<float> ms(ncl);
        for (int c = 0; c < ncl; c++) {
            rg[c] = make_int2(ctx->clusters[c].offset, ctx->clusters[c].nv);
            ms[c] = ctx->clusters[c].mass;
        }
        CK(ctx->clRange.ensure(ncl)); CK(ctx->clMass.ensure(ncl)); CK(ctx->clusterOf.ensure(N));
        CK(ctx->cmPos.ensure(ncl)); CK(ctx->cmVel.ensure(ncl)); CK(ctx->clKin.ensure(ncl));
        CK(ctx->feaVir.ensure(std::max(nt, 1)));
        CK(cudaMemcpyAsync(ctx->clRange.p, rg.data(), ncl * sizeof(int2), cudaMemcpyHostToDevice, sm));
        CK(cudaMemcpyAsync(ctx->clMass.p, ms.data(), ncl * sizeof(float), cudaMemcpyHostToDevice, sm));
        CK(cudaMemcpyAsync(ctx->clusterOf.p, ctx->cluster.data(), N * sizeof(int), cudaMemcpyHostToDevice, sm));
        CK(cudaMemsetAsync(ctx->feaVir.p, 0, sizeof(double) * std::max(nt, 1), sm));
    }
    CK(ctx->unf.ensure(std::max(N, 1))); CK(ctx->kinTerm.ensure(std::max(N, 1))); CK(ctx->clVir.ensure(std::max(N, 1)));
    // the accumulator's reduction: a fixed number of blocks per system size
    ctx->propBlocks = std::max(1, std::min(304, (N + 4095) / 4096));
    CK(ctx->propPart.ensure(3 * (size_t)ctx->propBlocks));
    CK(cudaStreamSynchronize(sm));  // the host vectors above are not pinned
    ctx->propsUploaded = true;
    return FEMMD_OK;
}

// The observables of a step that ended with LAST (positions of 'parity'),
// then their accumulation.
static cudaError_t enqueue_step_props(femmd_ctx *ctx, Launch &L, const DevSys &s, int parity) {
    const float2 *pc = parity ? s.pos1 : s.pos0;
    const int ncl = (int)ctx->clusters.size(), nt = (int)ctx->refVol.size();
    // the cluster virial lives on the elastomers' particles, the first ones
    const int ncp = ncl > 0 ? ctx->clusters.back().offset + ctx->clusters.back().nv : 0;
    cudaError_t e = enqueue_props(L, s, pc, ncl, ctx->clRange.p, ctx->clMass.p, ctx->clusterOf.p, ctx->unf.p,
                                  ctx->cmPos.p, ctx->cmVel.p, ctx->clKin.p, ctx->feaVir.p, ctx->kinTerm.p,
                                  ctx->clVir.p, ncp);
    if (e) return e;
    const bool tri = ncl > 0 && s.ntri > 0 && s.feaForces;
    return enqueue_props_accum(L, s, ctx->props.p, ctx->propPart.p, ctx->propBlocks, ncl > 0 ? ctx->clKin.p : nullptr,
                               ncl, tri ? ctx->feaVir.p : nullptr, nt, ctx->clVir.p, ncp, ctx->propAvgEvery,
                               ctx->propEqui);
}

// Graph of 'units' x [MID step on parity p -> IF(rebuild on 1-p)] starting at
// parity p (with property averaging: LAST, the properties, the drift).
static femmd_status build_graph(femmd_ctx *ctx, GraphSet &gs, int parity, int units) {
    gs.release();
    CK(cudaGraphCreate(&gs.g, 0));
    DevSys s = make_sys(ctx);
    Launch L;
    L.stream = ctx->stream;
    L.graph = gs.g;
    int p = parity;
    cudaGraphNode_t prevStep = nullptr, prevIf = nullptr;
    for (int u = 0; u < units; u++) {
        cudaGraphConditionalHandle h;
        CK(cudaGraphConditionalHandleCreate(&h, gs.g, 0, cudaGraphCondAssignDefault));
        if (ctx->propAvg) {
            // the step ends (LAST), its properties are accumulated, then the
            // next step's drift: the fused MID step's arithmetic, split
            CK(enqueue_step(L, s, MODE_LAST, p, h, 1));
            CK(enqueue_step_props(ctx, L, s, p));
            CK(enqueue_drift_in_run(L, s, p));
        } else {
            // The triangle pass needs only the drifted positions: it depends
            // on the previous step alone and runs beside that step's
            // conditional rebuild (which writes cells and lists, not
            // positions); the area springs and the step kernel wait for both.
            L.deps.clear();
            if (prevStep) L.deps.push_back(prevStep);
            CK(enqueue_tri(L, s, p));
            if (prevIf) L.deps.push_back(prevIf);
            CK(enqueue_step_after_tri(L, s, MODE_MID, p, h, 1));
            prevStep = L.deps.back();
        }
        Launch body;
        CK(L.begin_if(h, body));
        CK(enqueue_rebuild(body, s, 1 - p, 1));
        prevIf = L.deps.back();
        p = 1 - p;
    }
    CK(cudaGraphInstantiate(&gs.x, gs.g, 0));
    return FEMMD_OK;
}

// The run graph of a small fast-mode system: WHILE (steps left) { the
// cooperative small run; IF (rebuild) { the rebuild on parity 0 } }.
static femmd_status build_small_graph(femmd_ctx *ctx, const DevSys &s) {
    GraphSet &gs = ctx->smallGraph;
    gs.release();
    CK(cudaGraphCreate(&gs.g, 0));
    Launch L;
    L.stream = ctx->stream;
    L.graph = gs.g;
    cudaGraphConditionalHandle hw;
    CK(cudaGraphConditionalHandleCreate(&hw, gs.g, 1, cudaGraphCondAssignDefault));
    Launch body;
    CK(L.begin_while(hw, body));
    cudaGraphConditionalHandle hif;
    CK(cudaGraphConditionalHandleCreate(&hif, body.graph, 0, cudaGraphCondAssignDefault));
    CK(enqueue_small_run(body, s, hw, hif));
    Launch rb;
    CK(body.begin_if(hif, rb));
    CK(enqueue_rebuild(rb, s, 0, 1));
    CK(cudaGraphInstantiate(&gs.x, gs.g, 0));
    return FEMMD_OK;
}

// A run's middle steps of a small fast-mode system (small_run_fits): one
// graph launch whose WHILE loop runs the cooperative small run (each launch
// up to the step that calls for a rebuild) and the rebuild kernels between
// them, with no host round trip.  Without that graph (not instantiable here)
// the host loops over direct cooperative launches, waiting once per launch.
static femmd_status small_units(femmd_ctx *ctx, const DevSys &s, int units) {
    DevScalars *d = ctx->sc.p;
    // the small run starts from the current parity and ends on parity 0
    ctx->hsc->smallLeft = units;
    ctx->hsc->smallPar = ctx->cur;
    ctx->hsc->testWithhold = ctx->testExpire ? 1 : 0;
    ctx->testExpire = false;
    static_assert(offsetof(DevScalars, smallPar) == offsetof(DevScalars, smallLeft) + sizeof(int) &&
                      offsetof(DevScalars, testWithhold) == offsetof(DevScalars, smallLeft) + 2 * sizeof(int),
                  "small-run scalars");
    CK(cudaMemcpyAsync(&d->smallLeft, &ctx->hsc->smallLeft, 3 * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    ctx->cur = 0;
    if (!ctx->smallClean) {
        CK(cudaMemsetAsync(ctx->smallRec.p, 0, ctx->smallRec.n * sizeof(unsigned long long), ctx->stream));
        CK(cudaMemsetAsync(&d->gbTag, 0, sizeof(unsigned), ctx->stream));
        ctx->smallClean = true;
    }
    if (!ctx->smallGraphFailed && !ctx->smallGraph.x && build_small_graph(ctx, s) != FEMMD_OK) {
        ctx->smallGraph.release();
        ctx->smallGraphFailed = true;
        cudaGetLastError();
    }
    if (ctx->smallGraph.x) {
        CK(cudaGraphLaunch(ctx->smallGraph.x, ctx->stream));
        return FEMMD_OK;
    }
    Launch L;
    L.stream = ctx->stream;
    for (int left = units; left > 0;) {
        CK(launch_small_run(ctx->stream, s));
        femmd_status st;
        if ((st = read_scalars(ctx))) return st;
        const int k = ctx->hsc->smallDone;
        if (k <= 0 || ctx->hsc->smallLeft <= 0) {
            if (ctx->hsc->rebuild) CK(enqueue_rebuild(L, s, 0, 1));
            break;
        }
        left = ctx->hsc->smallLeft;
        if (ctx->hsc->rebuild) CK(enqueue_rebuild(L, s, 0, 1));
    }
    return FEMMD_OK;
}

static femmd_status launch_units(femmd_ctx *ctx, int units, bool use_graphs) {
    if (units <= 0) return FEMMD_OK;
    if (use_graphs && !ctx->propAvg) {
        const DevSys s = make_sys(ctx);
        if (small_run_fits(s)) return small_units(ctx, s, units);
    }
    if (!use_graphs) {
        DevSys s = make_sys(ctx);
        Launch L;
        L.stream = ctx->stream;
        if (ctx->profiling) {
            L.force_events = &ctx->forceEvents;
            L.event_pool = &ctx->eventPool;
        }
        for (int u = 0; u < units; u++) {
            if (ctx->propAvg) {
                CK(enqueue_step(L, s, MODE_LAST, ctx->cur, 0, 0));
                CK(enqueue_step_props(ctx, L, s, ctx->cur));
                CK(enqueue_drift_in_run(L, s, ctx->cur));
            } else {
                CK(enqueue_step(L, s, MODE_MID, ctx->cur, 0, 0));
            }
            CK(enqueue_rebuild(L, s, 1 - ctx->cur, 1));
            ctx->cur ^= 1;
        }
        ctx->profKernels += L.kernels;
        return FEMMD_OK;
    }
    femmd_status st;
    int big = units / kGraphUnits, rest = units % kGraphUnits;
    for (int b = 0; b < big; b++) {
        GraphSet &g = ctx->graphs[ctx->cur][0];
        if (!g.x && (st = build_graph(ctx, g, ctx->cur, kGraphUnits))) return st;
        CK(cudaGraphLaunch(g.x, ctx->stream));
        // kGraphUnits is even: parity unchanged
    }
    for (int r = 0; r < rest; r++) {
        GraphSet &g = ctx->graphs[ctx->cur][1];
        if (!g.x && (st = build_graph(ctx, g, ctx->cur, 1))) return st;
        CK(cudaGraphLaunch(g.x, ctx->stream));
        ctx->cur ^= 1;
    }
    return FEMMD_OK;
}

// ------------------------------------------------------------ trajectory

// FeaElements::unfoldPos (feaElements.cpp:86-150) on the host, float
// arithmetic as the reference, for one cluster of a frame.
static void unfold_cluster(const float2 *p, float *ux, float *uy, int off, int n, float Lx, float Ly) {
    float xmin = 100000, xmax = -100000, ymin = 100000, ymax = -100000;
    for (int k = 0; k < n; k++) {
        ux[k] = p[off + k].x;
        uy[k] = p[off + k].y;
        xmin = std::min(xmin, ux[k]);
        xmax = std::max(xmax, ux[k]);
        ymin = std::min(ymin, uy[k]);
        ymax = std::max(ymax, uy[k]);
    }
    if (xmax - xmin > Lx / 2) {
        float xc = 0;
        for (int k = 0; k < n; k++) {
            if (ux[k] > Lx / 2) ux[k] -= Lx;
            xc += ux[k];
        }
        if (xc / n < 0)
            for (int k = 0; k < n; k++) ux[k] += Lx;
    }
    if (ymax - ymin > Ly / 2) {
        float yc = 0;
        for (int k = 0; k < n; k++) {
            if (uy[k] > Ly / 2) uy[k] -= Ly;
            yc += uy[k];
        }
        if (yc / n < 0)
            for (int k = 0; k < n; k++) uy[k] += Ly;
    }
}

// Positions with every elastomer unfolded (FeaElements::unfoldPos,
// feaElements.cpp:86-150); the other particles keep their wrapped positions.
// (The reference reads unfoldedPos past the elastomers' vertices, which it
// never sizes for; here those particles are written where they are.)
static void unfolded_positions(const FrameMeta &M, int N, const float2 *p, std::vector<float> &ux,
                               std::vector<float> &uy) {
    ux.resize(N);
    uy.resize(N);
    for (int i = 0; i < N; i++) {
        ux[i] = p[i].x;
        uy[i] = p[i].y;
    }
    for (const int2 &c : M.clusters) unfold_cluster(p, ux.data() + c.x, uy.data() + c.x, c.x, c.y, M.Lx, M.Ly);
}

// The VTF type name of particle type t (md3dsystem.cpp:333: 'A' for type 0
// on; the reference's table ends at 'F', later letters continue it).
static char type_letter(int t) { return t >= 0 && t < 26 ? (char)('A' + t) : '?'; }

static FILE *open_out(const std::string &name, const char *mode, std::string &err) {
    FILE *f = fopen(name.c_str(), mode);
    if (!f) err = "cannot open " + name;
    return f;
}

// The per-frame file '<path><step, 9 digits><ext>' of saveVtk and saveVtkXML.
static std::string step_file(const FrameMeta &M, int step, const char *ext) {
    char num[32];
    snprintf(num, sizeof num, "%.9d", step);
    return M.path + num + ext;
}

// One frame in the reference's layouts (md3dsystem.cpp):
//   0 saveClusterXYZ's dump (:248-273; every particle), 1 saveXYZ (:232-246),
//   2 saveVtk (:275-328), 3 saveVTF (:330-353), 4 saveClusterVTF (:355-378),
//   5 saveVtkXML (:381-443), 6 saveVtkXMLBin (:451-522).
// Layouts 0, 1, 3 and 4 add to 'path' (started anew with 'truncate'; 'header'
// writes the VTF structure block first, as the reference does for s == 0);
// 2, 5 and 6 write one file per frame named by the step count.
static bool write_frame(const FrameMeta &M, int N, int step, const float2 *p, const float2 *v, bool truncate,
                        bool header, std::string &err) {
    const int nt = (int)M.tri.size() / 3;
    const int ncl = (int)M.clusters.size();
    if (M.format == 2) {
        if (M.clusters.empty()) return true;  // saveVtk writes nothing without elastomers
        FILE *f = open_out(step_file(M, step, ".vtk"), "w", err);
        if (!f) return false;
        std::vector<float> ux, uy;
        unfolded_positions(M, N, p, ux, uy);
        fprintf(f, "# vtk DataFile Version 3.1\nReally cool data\nASCII\nDATASET UNSTRUCTURED_GRID\n\n");
        fprintf(f, "POINTS %d FLOAT\n", N);
        for (int i = 0; i < N; i++) fprintf(f, "%f %f %f\n", ux[i], uy[i], 0.0f);
        fprintf(f, "\n");
        if (nt > 0) {
            fprintf(f, "CELLS %d %d\n", nt, 4 * nt);
            for (int t = 0; t < nt; t++) fprintf(f, "%d %d %d %d\n", 3, M.tri[3 * t], M.tri[3 * t + 1], M.tri[3 * t + 2]);
            fprintf(f, "\nCELL_TYPES %d\n", nt);
            for (int t = 0; t < nt; t++) fprintf(f, "%d ", 5);
            fprintf(f, "\n\n");
        }
        fprintf(f, "POINT_DATA %d\nSCALARS VelocitySquare FLOAT\nLOOKUP_TABLE default\n", N);
        for (int i = 0; i < N; i++) fprintf(f, "%f\n", v[i].x * v[i].x + v[i].y * v[i].y);
        fprintf(f, "\n\nVECTORS Velocity FLOAT\n");
        for (int i = 0; i < N; i++) fprintf(f, "%f %f %f\n", v[i].x, v[i].y, 0.0f);
        fclose(f);
        return true;
    }
    if (M.format == 5 || M.format == 6) {
        FILE *f = open_out(step_file(M, step, ".vtu"), M.format == 6 ? "wb" : "w", err);
        if (!f) return false;
        std::vector<float> ux, uy;
        unfolded_positions(M, N, p, ux, uy);
        if (M.format == 5) fprintf(f, "<?xml version=\"1.0\"?>\n");
        fprintf(f, "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n");
        fprintf(f, "\t<UnstructuredGrid>\n\t\t<Piece NumberOfPoints=\"%d\" NumberOfCells=\"%d\">\n", N, nt);
        if (M.format == 5) {
            fprintf(f, "\t\t\t<PointData Scalars=\"scalars\">\n");
            fprintf(f, "\t\t\t\t<DataArray type=\"Float32\" format=\"ascii\" Name=\"VelocitySquared\">\n");
            for (int i = 0; i < N; i++) fprintf(f, "%f ", v[i].x * v[i].x + v[i].y * v[i].y);
            fprintf(f, "\n\t\t\t\t</DataArray>\n\t\t\t</PointData>\n");
            fprintf(f, "\t\t\t<Points>\n");
            fprintf(f, "\t\t\t\t<DataArray type=\"Float32\" format=\"ascii\" NumberOfComponents=\"3\">\n");
            for (int i = 0; i < N; i++) fprintf(f, "%f %f %f ", ux[i], uy[i], 0.0f);
            fprintf(f, "\n\t\t\t\t</DataArray>\n\t\t\t</Points>\n");
            fprintf(f, "\t\t\t<Cells>\n");
            fprintf(f, "\t\t\t\t<DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n");
            for (int t = 0; t < nt; t++) fprintf(f, "%d %d %d ", M.tri[3 * t], M.tri[3 * t + 1], M.tri[3 * t + 2]);
            fprintf(f, "\n\t\t\t\t</DataArray>\n");
            fprintf(f, "\t\t\t\t<DataArray type=\"Int32\" format=\"ascii\" Name=\"offsets\">\n");
            for (int t = 0; t < nt; t++) fprintf(f, "%d ", 3 * (t + 1));
            fprintf(f, "\n\t\t\t\t</DataArray>\n");
            fprintf(f, "\t\t\t\t<DataArray type=\"Int32\" format=\"ascii\" Name=\"types\">\n");
            for (int t = 0; t < nt; t++) fprintf(f, "%d ", 5);
            fprintf(f, "\n\t\t\t\t</DataArray>\n\t\t\t</Cells>\n");
            fprintf(f, "\t\t</Piece>\n\t</UnstructuredGrid>\n</VTKFile>");
        } else {
            // appended raw arrays, each behind a 4-byte little-endian byte count;
            // the offsets count from the byte after '_'
            const uint32_t nVv = 4u * N, nPts = 12u * N, nCon = 12u * nt, nOff = 4u * nt, nTyp = (uint32_t)nt;
            const uint32_t oPts = nVv + 4, oCon = oPts + nPts + 4, oOff = oCon + nCon + 4, oTyp = oOff + nOff + 4;
            fprintf(f, "\t\t\t<PointData Scalars=\"scalars\">\n");
            fprintf(f, "\t\t\t\t<DataArray type=\"Float32\" format=\"appended\" Name=\"VelocitySquared\" offset=\"%d\"/>\n", 0);
            fprintf(f, "\t\t\t</PointData>\n\t\t\t<Points>\n");
            fprintf(f, "\t\t\t\t<DataArray type=\"Float32\" format=\"appended\" NumberOfComponents=\"3\" offset=\"%u\"/>\n",
                    oPts);
            fprintf(f, "\t\t\t</Points>\n\t\t\t<Cells>\n");
            fprintf(f, "\t\t\t\t<DataArray type=\"Int32\" Name=\"connectivity\" Format=\"appended\" offset=\"%u\"/>\n", oCon);
            fprintf(f, "\t\t\t\t<DataArray type=\"UInt32\" Name=\"offsets\" Format=\"appended\" offset=\"%u\"/>\n", oOff);
            fprintf(f, "\t\t\t\t<DataArray type=\"UInt8\" Name=\"types\" Format=\"appended\" offset=\"%u\"/>\n", oTyp);
            fprintf(f, "\t\t\t</Cells>\n\t\t</Piece>\n\t</UnstructuredGrid>\n");
            fprintf(f, "\t<AppendedData encoding=\"raw\">\n\t_");
            // the arrays are laid out in host memory and written with explicit
            // little-endian byte counts, so the file is the same on any host
            std::vector<unsigned char> raw;
            raw.reserve(20 + nVv + nPts + nCon + nOff + nTyp);
            auto put32 = [&](uint32_t w) {
                for (int b = 0; b < 4; b++) raw.push_back((unsigned char)(w >> (8 * b)));
            };
            auto putf = [&](float x) {
                uint32_t w;
                memcpy(&w, &x, 4);
                put32(w);
            };
            put32(nVv);
            for (int i = 0; i < N; i++) putf(v[i].x * v[i].x + v[i].y * v[i].y);
            put32(nPts);
            for (int i = 0; i < N; i++) {
                putf(ux[i]);
                putf(uy[i]);
                putf(0.0f);
            }
            put32(nCon);
            for (int t = 0; t < 3 * nt; t++) put32((uint32_t)M.tri[t]);
            put32(nOff);
            for (int t = 0; t < nt; t++) put32(3u * (t + 1));
            put32(nTyp);
            for (int t = 0; t < nt; t++) raw.push_back(5);
            fwrite(raw.data(), 1, raw.size(), f);
            fprintf(f, "\n\t</AppendedData>\n</VTKFile>");
        }
        const bool ok = !ferror(f);
        fclose(f);
        if (!ok) err = "write failed";
        return ok;
    }
    FILE *f = open_out(M.path, truncate ? "w" : "a", err);
    if (!f) return false;
    if (M.format == 1) {
        fprintf(f, "%d\n\n", N);
        for (int i = 0; i < N; i++) fprintf(f, "A\t%f\t%f\t%f\n", p[i].x, p[i].y, 0.0f);
    } else if (M.format == 3) {
        if (header) {
            // radius = sigma / 2 (Particles::addParticle, particles.cpp:218)
            for (int i = 0; i < N; i++)
                fprintf(f, "atom %d type %c radius %f\n", i, type_letter(M.type[i]), (double)M.sigma[i] / 2.0);
            for (size_t b = 0; 2 * b + 1 < M.bond.size(); b++) fprintf(f, "bond %d:%d\n", M.bond[2 * b], M.bond[2 * b + 1]);
            fprintf(f, "pbc %f %f %f\n", (double)M.Lx, (double)M.Ly, 1.0);
        }
        fprintf(f, "timestep\n");
        for (int i = 0; i < N; i++) fprintf(f, "%f %f %f\n", p[i].x, p[i].y, 0.0f);
    } else if (M.format == 4) {
        if (header) {
            // one atom per elastomer; the reference names atom i by the type
            // of particle i (md3dsystem.cpp:361), kept as it is
            for (int c = 0; c < ncl; c++)
                fprintf(f, "atom %d type %c radius %f\n", c, type_letter(c < N ? M.type[c] : 0),
                        0.5 * (double)M.scale + 0.5);
            fprintf(f, "pbc %f %f %f\n", (double)M.Lx, (double)M.Ly, 1.0);
        }
        fprintf(f, "timestep\n");
        // centre of mass of the unfolded elastomer, float sums in vertex
        // order (FeaElements::unfoldPos, feaElements.cpp:135-147)
        std::vector<float> ux, uy;
        unfolded_positions(M, N, p, ux, uy);
        for (int c = 0; c < ncl; c++) {
            const int off = M.clusters[c].x, nv = M.clusters[c].y;
            float xc = 0, yc = 0;
            for (int k = 0; k < nv; k++) {
                xc += M.mass[off + k] * ux[off + k];
                yc += M.mass[off + k] * uy[off + k];
            }
            fprintf(f, "%f %f %f\n", xc / M.clusterMass[c], yc / M.clusterMass[c], 0.0f);
        }
    } else {
        fprintf(f, "ITEM: TIMESTEP\n%d\nITEM: NUMBER OF ATOMS\n%d\n", step, N);
        fprintf(f, "ITEM: BOX BOUNDS pp pp pp\n%f %f\n%f %f\n%f %f\n", 0.0, (double)M.Lx, 0.0, (double)M.Ly, 0.0, 0.0);
        fprintf(f, "ITEM: ATOMS id type x y z vx vy vz\n");
        for (int i = 0; i < N; i++)
            fprintf(f, "%d %d %f %f %f %f %f %f\n", i, M.type[i], p[i].x, p[i].y, 0.0f, v[i].x, v[i].y, 0.0f);
    }
    const bool ok = !ferror(f);
    fclose(f);
    if (!ok) err = "write failed on " + M.path;
    return ok;
}

static void traj_writer(Trajectory *T) {
    for (;;) {
        TrajFrame fr;
        {
            std::unique_lock<std::mutex> lk(T->mu);
            T->cv.wait(lk, [&] { return T->stop || !T->queue.empty(); });
            if (T->queue.empty()) return;  // stop requested and drained
            fr = T->queue.front();
        }
        std::string err;
        const bool ok = write_frame(T->meta, T->N, fr.step, T->pos[fr.slot], T->vel[fr.slot], false, !T->headerDone, err);
        T->headerDone = true;
        {
            std::lock_guard<std::mutex> lk(T->mu);
            T->queue.pop_front();
            T->busy[fr.slot] = 0;
            if (!ok && T->error.empty()) T->error = err;
            T->written++;
        }
        T->cv.notify_all();
    }
}

// Wait until every committed frame is written.
static void traj_drain(Trajectory &T) {
    std::unique_lock<std::mutex> lk(T.mu);
    T.cv.wait(lk, [&] { return T.queue.empty(); });
}

static void traj_stop(Trajectory &T) {
    if (T.th.joinable()) {
        {
            std::lock_guard<std::mutex> lk(T.mu);
            T.stop = true;
        }
        T.cv.notify_all();
        T.th.join();
    }
    for (auto p : T.pos) cudaFreeHost(p);
    for (auto p : T.vel) cudaFreeHost(p);
    T.pos.clear();
    T.vel.clear();
    T.busy.clear();
    T.pending.clear();
    T.queue.clear();
    T.stop = false;
}

static void traj_commit(Trajectory &T) {
    if (T.pending.empty()) return;
    {
        std::lock_guard<std::mutex> lk(T.mu);
        for (const TrajFrame &f : T.pending) {
            T.queue.push_back(f);
            T.lastCommitted = std::max<long long>(T.lastCommitted, f.step);
        }
    }
    T.pending.clear();
    T.cv.notify_all();
}

static void traj_discard(Trajectory &T) {
    std::lock_guard<std::mutex> lk(T.mu);
    for (const TrajFrame &f : T.pending) T.busy[f.slot] = 0;
    T.pending.clear();
}

static femmd_status read_scalars(femmd_ctx *ctx);

// Capture the frame of step m from the current buffers.  When no pinned slot
// is free, the frames so far are committed if the run has not overflowed up
// to here (then 'aborted' stays false and the writer frees slots), else the
// run is abandoned for femmd_run to repeat.
static femmd_status traj_snapshot(femmd_ctx *ctx, int m, bool &aborted) {
    Trajectory &T = ctx->traj;
    const int N = (int)ctx->pos.size();
    constexpr int kSlots = 8;
    if (T.N != N) {
        traj_drain(T);
        for (auto p : T.pos) cudaFreeHost(p);
        for (auto p : T.vel) cudaFreeHost(p);
        T.pos.clear();
        T.vel.clear();
        T.busy.clear();
        T.N = N;
    }
    int slot = -1;
    {
        std::lock_guard<std::mutex> lk(T.mu);
        for (size_t k = 0; k < T.busy.size(); k++)
            if (!T.busy[k]) {
                slot = (int)k;
                break;
            }
    }
    if (slot < 0 && (int)T.busy.size() < kSlots) {
        float2 *p = nullptr, *v = nullptr;
        CK(cudaMallocHost(&p, std::max(N, 1) * sizeof(float2)));
        CK(cudaMallocHost(&v, std::max(N, 1) * sizeof(float2)));
        std::lock_guard<std::mutex> lk(T.mu);
        T.pos.push_back(p);
        T.vel.push_back(v);
        T.busy.push_back(0);
        slot = (int)T.busy.size() - 1;
    }
    if (slot < 0) {
        femmd_status st;
        if ((st = read_scalars(ctx))) return st;  // synchronises: the pending frames are in host memory
        if (ctx->hsc->overflow) {
            aborted = true;
            return FEMMD_OK;
        }
        traj_commit(T);
        std::unique_lock<std::mutex> lk(T.mu);
        T.cv.wait(lk, [&] {
            for (char b : T.busy)
                if (!b) return true;
            return false;
        });
        for (size_t k = 0; k < T.busy.size(); k++)
            if (!T.busy[k]) {
                slot = (int)k;
                break;
            }
    }
    {
        std::lock_guard<std::mutex> lk(T.mu);
        T.busy[slot] = 1;
    }
    const float2 *pc = ctx->cur ? ctx->dpos1.p : ctx->dpos0.p;
    if (fast_mode(ctx)) {
        CK(fast_download2(ctx, pc, T.pos[slot]));
        CK(fast_download2(ctx, ctx->dvel.p, T.vel[slot]));
    } else {
        CK(cudaMemcpyAsync(T.pos[slot], pc, N * sizeof(float2), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(T.vel[slot], ctx->dvel.p, N * sizeof(float2), cudaMemcpyDeviceToHost, ctx->stream));
    }
    T.pending.push_back({m, slot});
    return FEMMD_OK;
}

// The topology a frame is formatted with, from the context.
static void frame_meta(const femmd_ctx *ctx, FrameMeta &M) {
    M.type = ctx->type;
    M.tri = ctx->tri;
    M.bond = ctx->bond;
    M.mass = ctx->mass;
    M.sigma = ctx->sigma;
    M.clusters.clear();
    M.clusterMass.clear();
    for (const Cluster &c : ctx->clusters) {
        M.clusters.push_back(make_int2(c.offset, c.nv));
        M.clusterMass.push_back(c.mass);
    }
    M.Lx = ctx->Lx;
    M.Ly = ctx->Ly;
    M.scale = ctx->scale;
}

static void traj_refresh_meta(femmd_ctx *ctx) {
    Trajectory &T = ctx->traj;
    if (!T.on) return;
    traj_drain(T);
    frame_meta(ctx, T.meta);
}

static femmd_status run_once(femmd_ctx *ctx, int n, bool &aborted) {
    DevSys s = make_sys(ctx);
    Launch L;
    L.stream = ctx->stream;
    if (ctx->profiling) {
        L.force_events = &ctx->forceEvents;
        L.event_pool = &ctx->eventPool;
    }
    const bool graphs = !ctx->profiling;
    CK(enqueue_run_start(L, s));
    CK(enqueue_rebuild(L, s, ctx->cur, 1));
    if (n == 0) {
        CK(enqueue_step(L, s, MODE_INIT, ctx->cur, 0, 0));
        ctx->profKernels += L.kernels;
        return FEMMD_OK;
    }
    CK(enqueue_step(L, s, MODE_FIRST, ctx->cur, 0, 0));
    ctx->cur ^= 1;
    femmd_status st;
    // trajectory frames at the steps m in (s0, s0 + n] that are multiples of
    // 'every' (the reference's steps % trajectorySteps == 0).  Unit u of the
    // run computes the forces at x_{s0+u}; a frame inside the run replaces
    // its unit by LAST (completes v_m, keeps a_m), the copy, and the drift
    // (half kick with a_m, drift, wrap) followed by the rebuild check, which
    // is the unit's work bit for bit.
    const int s0 = ctx->steps;
    std::vector<int> frames;
    Trajectory &T = ctx->traj;
    if (T.on && T.every > 0)
        for (long long m = ((long long)s0 / T.every + 1) * T.every; m <= (long long)s0 + n; m += T.every)
            if (m > T.lastCommitted) frames.push_back((int)m);
    int u = 1;
    for (int m : frames) {
        const int upto = m - s0;
        if (upto >= n) break;
        if ((st = launch_units(ctx, upto - u, graphs))) return st;
        Launch D = L;
        D.kernels = 0;
        CK(enqueue_step(D, s, MODE_LAST, ctx->cur, 0, 0));
        if (ctx->propAvg) CK(enqueue_step_props(ctx, D, s, ctx->cur));
        if ((st = traj_snapshot(ctx, m, aborted))) return st;
        if (aborted) return FEMMD_OK;
        // the rest of the fused step: half kick with the stored a_m and drift
        // (a second force pass would repeat the area springs' displacement)
        CK(enqueue_drift_in_run(D, s, ctx->cur));
        ctx->cur ^= 1;
        CK(enqueue_rebuild(D, s, ctx->cur, 1));
        ctx->profKernels += D.kernels;
        u = upto + 1;
    }
    ctx->profKernels += L.kernels;
    if ((st = launch_units(ctx, n - u, graphs))) return st;
    Launch T2 = L;
    T2.kernels = 0;
    CK(enqueue_step(T2, s, MODE_LAST, ctx->cur, 0, 0));
    if (ctx->propAvg) CK(enqueue_step_props(ctx, T2, s, ctx->cur));
    ctx->profKernels += T2.kernels;
    if (!frames.empty() && frames.back() == s0 + n && (st = traj_snapshot(ctx, s0 + n, aborted))) return st;
    return FEMMD_OK;
}

static femmd_status collect_profile(femmd_ctx *ctx) {
    if (!ctx->profiling) return FEMMD_OK;
    CK(cudaStreamSynchronize(ctx->stream));
    for (auto &pr : ctx->forceEvents) {
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, pr.first, pr.second));
        ctx->profForceMs += ms;
        ctx->profForceLaunches++;
        ctx->eventPool.push_back(pr.first);
        ctx->eventPool.push_back(pr.second);
    }
    ctx->forceEvents.clear();
    return FEMMD_OK;
}

// ===================================================================== C ABI

extern "C" {

const char *femmd_version(void) { return "femmd-gb300 0.1 (sm_103a)"; }

femmd_status femmd_create(int device, femmd_ctx **out) {
    if (!out) return FEMMD_INVALID_ARG;
    femmd_ctx *c = new (std::nothrow) femmd_ctx();
    if (!c) return FEMMD_CUDA_ERROR;
    c->device = device;
    clear_system(c);
    *out = c;
    return FEMMD_OK;
}

void femmd_destroy(femmd_ctx *ctx) {
    if (!ctx) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    traj_stop(ctx->traj);
    release_device(ctx);
    for (auto &pr : ctx->forceEvents) { cudaEventDestroy(pr.first); cudaEventDestroy(pr.second); }
    for (auto e : ctx->eventPool) cudaEventDestroy(e);
    for (auto e : ctx->userEvents)
        if (e) cudaEventDestroy(e);
    if (ctx->hsc) cudaFreeHost(ctx->hsc);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char *femmd_last_error(const femmd_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

femmd_status femmd_init(femmd_ctx *ctx, double Lx, double Ly) {
    NEED(ctx);
    if (!(Lx > 0) || !(Ly > 0)) return fail(ctx, FEMMD_INVALID_ARG, "box lengths must be positive");
    clear_system(ctx);
    ctx->inited = true;
    ctx->Lx = (float)Lx;
    ctx->Ly = (float)Ly;
    // Interactions::init defaults: WCA, E = 0, nu = 0.3, kBond = 0
    ctx->eps = {1.0f};
    ctx->rc = {(float)std::pow(2.0, 1.0 / 6.0)};
    ctx->us = {1.0f};
    ctx->rCutMax = ctx->rc[0];
    return FEMMD_OK;
}

femmd_status femmd_reset(femmd_ctx *ctx) {
    NEED(ctx);
    clear_system(ctx);
    return FEMMD_OK;
}

femmd_status femmd_set_box(femmd_ctx *ctx, double Lx, double Ly) {
    NEED(ctx);
    HOSTSYNC(ctx);
    if (!(Lx > 0) || !(Ly > 0)) return fail(ctx, FEMMD_INVALID_ARG, "box lengths must be positive");
    ctx->Lx = (float)Lx;
    ctx->Ly = (float)Ly;
    mark_topology(ctx);
    return FEMMD_OK;
}

femmd_status femmd_get_box(const femmd_ctx *ctx, double *Lx, double *Ly) {
    if (!ctx || !Lx || !Ly) return FEMMD_INVALID_ARG;
    *Lx = ctx->Lx;
    *Ly = ctx->Ly;
    return FEMMD_OK;
}

femmd_status femmd_set_pbc(femmd_ctx *ctx, int pbc) {
    NEED(ctx);
    ctx->pbc = pbc == 0 ? FEMMD_NOPBC : pbc == 1 ? FEMMD_XPBC : FEMMD_XYPBC;
    ctx->materialDirty = true;  // the fixed walls need the per-particle sigma
    release_graphs(ctx);
    return FEMMD_OK;
}

femmd_status femmd_set_dev(femmd_ctx *ctx, int dev) {
    NEED(ctx);
    ctx->dev_flag = dev;
    return FEMMD_OK;
}

femmd_status femmd_set_dt(femmd_ctx *ctx, double dt) {
    NEED(ctx);
    ctx->dt = (float)dt;
    release_graphs(ctx);
    return FEMMD_OK;
}

femmd_status femmd_get_dt(const femmd_ctx *ctx, double *dt) {
    if (!ctx || !dt) return FEMMD_INVALID_ARG;
    *dt = ctx->dt;
    return FEMMD_OK;
}

femmd_status femmd_set_num_types(femmd_ctx *ctx, int n) {
    NEED(ctx);
    HOSTSYNC(ctx);
    if (n < 1 || n > kMaxTypes) return fail(ctx, FEMMD_INVALID_ARG, "numTypes must be in [1, %d]", kMaxTypes);
    ctx->numTypes = n;
    mark_topology(ctx);
    return FEMMD_OK;
}

femmd_status femmd_set_pair_potential(femmd_ctx *ctx, const double *eps, const double *rc, const double *us, int n2) {
    NEED(ctx);
    HOSTSYNC(ctx);
    int nt = ctx->numTypes;
    if (!eps || !rc || !us || n2 < nt * nt)
        return fail(ctx, FEMMD_INVALID_ARG, "pair tables need numTypes^2 = %d entries", nt * nt);
    ctx->eps.assign(nt * nt, 0.f);
    ctx->rc.assign(nt * nt, 0.f);
    ctx->us.assign(nt * nt, 0.f);
    ctx->rCutMax = 0;
    for (int i = 0; i < nt * nt; i++) {
        ctx->eps[i] = (float)eps[i];
        ctx->rc[i] = (float)rc[i];
        if (ctx->rc[i] > ctx->rCutMax) ctx->rCutMax = ctx->rc[i];
        ctx->us[i] = (float)us[i];
    }
    mark_topology(ctx);
    return FEMMD_OK;
}

femmd_status femmd_set_kbond(femmd_ctx *ctx, double k) {
    NEED(ctx);
    float kf = (float)k;
    if (kf > 0) { ctx->kBond = kf; ctx->bondForces = true; } else ctx->bondForces = false;
    release_graphs(ctx);
    return FEMMD_OK;
}

femmd_status femmd_set_youngs_modulus(femmd_ctx *ctx, double E) {
    NEED(ctx);
    float Ef = (float)E;
    if (Ef > 0) { ctx->E = Ef; ctx->feaForces = true; } else ctx->feaForces = false;
    set_elastic_constants(ctx);
    release_graphs(ctx);
    return FEMMD_OK;
}

femmd_status femmd_set_poisson_ratio(femmd_ctx *ctx, double nu) {
    NEED(ctx);
    ctx->nu = (float)nu;
    set_elastic_constants(ctx);
    release_graphs(ctx);
    return FEMMD_OK;
}

femmd_status femmd_set_elastomer_material(femmd_ctx *ctx, int elastomer, double E, double nu) {
    NEED(ctx);
    if (elastomer < 0 || elastomer >= (int)ctx->clusters.size())
        return fail(ctx, FEMMD_INVALID_ARG, "elastomer %d does not exist (%zu added)", elastomer, ctx->clusters.size());
    if (!(E > 0) || !(nu > -1.0 && nu < 0.5))
        return fail(ctx, FEMMD_INVALID_ARG, "need E > 0 and -1 < nu < 0.5 (got %g, %g)", E, nu);
    const size_t n = ctx->clusters.size();
    ctx->elE.resize(n, 0.0f);
    ctx->elNu.resize(n, 0.0f);
    ctx->elOwn.resize(n, 0);
    ctx->elE[elastomer] = (float)E;
    ctx->elNu[elastomer] = (float)nu;
    ctx->elOwn[elastomer] = 1;
    ctx->materialDirty = true;
    ctx->forcesValid = false;
    release_graphs(ctx);
    return FEMMD_OK;
}

femmd_status femmd_set_moving_wall(femmd_ctx *ctx, double k, double y0, double v) {
    NEED(ctx);
    if (!std::isfinite(k) || !std::isfinite(y0) || !std::isfinite(v))
        return fail(ctx, FEMMD_INVALID_ARG, "wall parameters must be finite");
    ctx->wallOn = k > 0;
    ctx->wallK = ctx->wallOn ? (float)k : 0.0f;
    ctx->wallY0 = (float)y0;
    ctx->wallV = (float)v;
    ctx->materialDirty = true;
    ctx->forcesValid = false;
    release_graphs(ctx);
    return FEMMD_OK;
}

// Force of the particles on the two walls at the current positions x_n
// (n = the context's step count): sum of k_w * overlap, float terms summed
// in double.
femmd_status femmd_get_wall_forces(femmd_ctx *ctx, double *top, double *bottom) {
    NEED(ctx);
    if (!top || !bottom) return fail(ctx, FEMMD_INVALID_ARG, "null output");
    *top = *bottom = 0.0;
    if (!ctx->wallOn) return FEMMD_OK;
    HOSTSYNC(ctx);
    femmd_status st;
    if ((st = download_state(ctx, kPos))) return st;
    const float range = wall_range();
    const float yw = ctx->wallY0 - ctx->wallV * ((float)ctx->steps * ctx->dt);
    double ft = 0.0, fb = 0.0;
    for (size_t i = 0; i < ctx->pos.size(); i++) {
        const float dl = range * ctx->sigma[i], y = ctx->pos[i].y;
        const float ht = (y + dl) - yw, hb = dl - y;
        if (ht > 0.0f) ft += (double)(ctx->wallK * ht);
        if (hb > 0.0f) fb += (double)(ctx->wallK * hb);
    }
    *top = ft;
    *bottom = fb;
    return FEMMD_OK;
}

// DukSystemSetGravity (interface.cpp:443-453): g > 0 sets and enables it,
// otherwise gravity is disabled (the stored value is kept)
femmd_status femmd_set_gravity(femmd_ctx *ctx, double g) {
    NEED(ctx);
    if (g > 0) {
        ctx->gravity = (float)g;
        ctx->gravityForce = true;
    } else {
        ctx->gravityForce = false;
    }
    ctx->forcesValid = false;
    release_graphs(ctx);
    return FEMMD_OK;
}

// DukSystemSetKArea (interface.cpp:466-476): k > 0 sets and enables the area
// springs, otherwise they are disabled (the stored value is kept)
femmd_status femmd_set_karea(femmd_ctx *ctx, double k) {
    NEED(ctx);
    const bool was = ctx->areaForces;
    if (k > 0) {
        ctx->kArea = (float)k;
        ctx->areaForces = true;
    } else {
        ctx->areaForces = false;
    }
    ctx->forcesValid = false;
    release_graphs(ctx);
    if (was && !ctx->areaForces && fast_mode(ctx) && ctx->cslot.p && ctx->listBuilt && !ctx->topoDirty &&
        !ctx->stateDirty) {
        // the mirror was not kept while the springs moved vertices: bring it
        // up to the current positions
        DevSys ds = make_sys(ctx);
        Launch L;
        L.stream = ctx->stream;
        CK(enqueue_cpos_refresh(L, ds, ctx->cur));
    }
    return FEMMD_OK;
}

femmd_status femmd_set_skin(femmd_ctx *ctx, double skin) {
    NEED(ctx);
    if (!(skin >= 0)) return fail(ctx, FEMMD_INVALID_ARG, "skin must be >= 0");
    ctx->skin = (float)skin;
    return FEMMD_OK;
}

// List cells of factor * (rc + skin) instead of the reference's (factor 1):
// fewer, larger cells.  Takes effect at the next femmd_init_neighbor_list.
// Any factor other than 1 changes the list order, so the pair sums round
// differently from the reference's.
femmd_status femmd_set_cell_factor(femmd_ctx *ctx, double factor) {
    NEED(ctx);
    if (!(factor >= 1.0) || !(factor <= 8.0)) return fail(ctx, FEMMD_INVALID_ARG, "cell factor must be in [1, 8]");
    ctx->cellFactor = (float)factor;
    return FEMMD_OK;
}

femmd_status femmd_set_neighbor_capacity(femmd_ctx *ctx, int cap) {
    NEED(ctx);
    if (cap < 0) return fail(ctx, FEMMD_INVALID_ARG, "capacity must be >= 0");
    femmd_status st;
    if (cap == 0) {
        ctx->nbrCap = 0;
        release_graphs(ctx);
        return FEMMD_OK;
    }
    if ((st = prepare(ctx))) return st;
    return alloc_list(ctx, cap);
}

femmd_status femmd_get_neighbor_capacity(const femmd_ctx *ctx, int *cap) {
    if (!ctx || !cap) return FEMMD_INVALID_ARG;
    *cap = ctx->nbrCap;
    return FEMMD_OK;
}

femmd_status femmd_set_fea_law(femmd_ctx *ctx, int law) {
    NEED(ctx);
    HOSTSYNC(ctx);
    if (law != FEMMD_FEA_NEO_HOOKEAN && law != FEMMD_FEA_GREEN_LINEAR)
        return fail(ctx, FEMMD_INVALID_ARG, "unknown FEA law %d", law);
    ctx->feaLaw = law;
    mark_topology(ctx);
    return FEMMD_OK;
}

femmd_status femmd_set_bond_k_mode(femmd_ctx *ctx, int mode) {
    NEED(ctx);
    if (mode != FEMMD_BONDK_KBOND && mode != FEMMD_BONDK_E_OVER_R0)
        return fail(ctx, FEMMD_INVALID_ARG, "unknown bond stiffness mode %d", mode);
    ctx->bondKMode = mode;
    release_graphs(ctx);
    return FEMMD_OK;
}

femmd_status femmd_set_image_mode(femmd_ctx *ctx, int mode) {
    NEED(ctx);
    if (mode != FEMMD_IMAGE_REFERENCE && mode != FEMMD_IMAGE_EXACT)
        return fail(ctx, FEMMD_INVALID_ARG, "unknown image mode %d", mode);
    ctx->imageMode = mode;
    release_graphs(ctx);
    return FEMMD_OK;
}

femmd_status femmd_set_force_mode(femmd_ctx *ctx, int mode) {
    NEED(ctx);
    if (mode != FEMMD_FORCE_REFERENCE && mode != FEMMD_FORCE_FAST)
        return fail(ctx, FEMMD_INVALID_ARG, "unknown force mode %d", mode);
    if (mode == ctx->forceMode) return FEMMD_OK;
    HOSTSYNC(ctx);  // the state comes home in id order, then goes up again in the new layout
    ctx->forceMode = mode;
    mark_topology(ctx);
    release_graphs(ctx);
    return FEMMD_OK;
}

femmd_status femmd_get_force_mode(const femmd_ctx *ctx, int *mode) {
    if (!ctx || !mode) return FEMMD_INVALID_ARG;
    *mode = ctx->forceMode;
    return FEMMD_OK;
}

femmd_status femmd_set_elastomer_bonds(femmd_ctx *ctx, int mode) {
    NEED(ctx);
    if (mode < 0 || mode > 2) return fail(ctx, FEMMD_INVALID_ARG, "unknown elastomer bond mode %d", mode);
    ctx->bondMode = mode;
    return FEMMD_OK;
}

femmd_status femmd_add_particle(femmd_ctx *ctx, double x, double y, double vx, double vy, double m, double sig,
                                int typ) {
    NEED(ctx);
    HOSTSYNC(ctx);
    if (!ctx->inited) return fail(ctx, FEMMD_NOT_READY, "init(Lx, Ly) has not been called");
    if ((int)ctx->pos.size() >= kIdMask) return fail(ctx, FEMMD_CAPACITY_OVERFLOW, "particle id space exhausted");
    add_particle_raw(ctx, (float)x, (float)y, (float)vx, (float)vy, (float)m, (float)sig, typ);
    mark_topology(ctx);
    return FEMMD_OK;
}

femmd_status femmd_add_particles(femmd_ctx *ctx, int n, const double *x, const double *y, const double *vx,
                                 const double *vy, const double *m, const double *sig, const int *typ) {
    NEED(ctx);
    HOSTSYNC(ctx);
    if (!ctx->inited) return fail(ctx, FEMMD_NOT_READY, "init(Lx, Ly) has not been called");
    if (n < 0 || (n > 0 && (!x || !y || !vx || !vy || !m || !sig || !typ)))
        return fail(ctx, FEMMD_INVALID_ARG, "bad particle arrays");
    if ((long long)ctx->pos.size() + n > kIdMask) return fail(ctx, FEMMD_CAPACITY_OVERFLOW, "too many particles");
    size_t want = ctx->pos.size() + (size_t)n;
    ctx->pos.reserve(want); ctx->vel.reserve(want); ctx->acc.reserve(want); ctx->force.reserve(want);
    ctx->refPos.reserve(want); ctx->mass.reserve(want); ctx->sigma.reserve(want); ctx->energy.reserve(want);
    ctx->type.reserve(want); ctx->excl.reserve(want); ctx->cluster.reserve(want);
    for (int k = 0; k < n; k++)
        add_particle_raw(ctx, (float)x[k], (float)y[k], (float)vx[k], (float)vy[k], (float)m[k], (float)sig[k], typ[k]);
    mark_topology(ctx);
    return FEMMD_OK;
}

femmd_status femmd_add_elastomer(femmd_ctx *ctx, const float *vert, int nv, const int *tet, int nt, double x,
                                 double y, int typ, int g, double sig, double M, int exclude) {
    NEED(ctx);
    HOSTSYNC(ctx);
    (void)g;
    if (!ctx->inited) return fail(ctx, FEMMD_NOT_READY, "init(Lx, Ly) has not been called");
    if (!vert || !tet || nv <= 0 || nt <= 0) return fail(ctx, FEMMD_INVALID_ARG, "empty mesh");
    for (int k = 0; k < 3 * nt; k++)
        if (tet[k] < 1 || tet[k] > nv)
            return fail(ctx, FEMMD_INVALID_ARG, "triangle index %d outside [1, %d] (indices are 1-based)", tet[k], nv);
    int offset = (int)ctx->pos.size();
    if (!ctx->clusters.empty() && (ctx->clusters[0].nv != nv || ctx->clusters[0].nt != nt))
        return fail(ctx, FEMMD_INVALID_ARG, "all elastomers must share one mesh (particles.cpp:301-325)");
    if (offset != (int)ctx->clusters.size() * nv)
        return fail(ctx, FEMMD_INVALID_ARG, "elastomers must be added before free particles (particles.cpp:301-325)");
    int exclusionGroupId = ctx->nexcl++;
    int ci = (int)ctx->clusters.size();
    Cluster cl = {offset, nv, nt, ci * nt, 0.f, 0.f};
    ctx->clusters.push_back(cl);
    float fx0 = (float)x, fy0 = (float)y;
    for (int i = 0; i < nv; i++) {
        float x1 = vert[2 * i] + fx0;
        float y1 = vert[2 * i + 1] + fy0;
        int pid = add_particle_raw(ctx, x1, y1, 0.f, 0.f, 0.f, (float)sig, typ);
        ctx->refPos[pid] = ctx->pos[pid];
        if (ctx->pbc == FEMMD_XYPBC) {
            ctx->pos[pid].x = wrap_coord(ctx->pos[pid].x, ctx->Lx);
            ctx->pos[pid].y = wrap_coord(ctx->pos[pid].y, ctx->Ly);
        } else if (ctx->pbc == FEMMD_XPBC) {
            ctx->pos[pid].x = wrap_coord(ctx->pos[pid].x, ctx->Lx);
        }
        if (exclude) ctx->excl[pid] = exclusionGroupId;
        ctx->cluster[pid] = ci;
    }
    float totVol = 0.f;
    int tetOffset = ci * nt;
    ctx->tri.resize(3 * (size_t)(tetOffset + nt));
    ctx->xm.resize(9 * (size_t)(tetOffset + nt));
    ctx->refVol.resize(tetOffset + nt);
    for (int i = 0; i < nt; i++) {
        int i0 = tet[3 * i] + offset - 1, i1 = tet[3 * i + 1] + offset - 1, i2 = tet[3 * i + 2] + offset - 1;
        int t = i + tetOffset;
        ctx->tri[3 * t] = i0;
        ctx->tri[3 * t + 1] = i1;
        ctx->tri[3 * t + 2] = i2;
        if (ctx->bondMode == FEMMD_ELASTOMER_BONDS_ALL) {
            create_bond_raw(ctx, i0, i1);
            create_bond_raw(ctx, i0, i2);
            create_bond_raw(ctx, i1, i2);
        }
        float aa[9], rx[3], ry[3];
        for (int j = 0; j < 3; j++) {
            int ip = ctx->tri[3 * t + j];
            aa[3 * j] = 1.0f;
            aa[3 * j + 1] = ctx->refPos[ip].x;
            aa[3 * j + 2] = ctx->refPos[ip].y;
            rx[j] = ctx->refPos[ip].x;
            ry[j] = ctx->refPos[ip].y;
        }
        if (!invert3(aa, &ctx->xm[9 * (size_t)t])) memset(&ctx->xm[9 * (size_t)t], 0, 9 * sizeof(float));
        float vol = (float)(0.5 * (double)((ry[2] - ry[0]) * (rx[1] - rx[0]) - (ry[1] - ry[0]) * (rx[2] - rx[0])));
        ctx->refVol[t] = vol;
        totVol += vol;
    }
    if (ctx->bondMode == FEMMD_ELASTOMER_BONDS_BOUNDARY) {
        // one bond per edge of exactly one triangle, triangle order, (0,1) (0,2) (1,2)
        std::vector<long long> keys(3 * (size_t)nt);
        for (int i = 0; i < nt; i++) {
            const int *q = &tet[3 * i];
            int e[3][2] = {{q[0], q[1]}, {q[0], q[2]}, {q[1], q[2]}};
            for (int k = 0; k < 3; k++)
                keys[3 * i + k] = (long long)std::min(e[k][0], e[k][1]) * 4294967296LL + std::max(e[k][0], e[k][1]);
        }
        std::vector<long long> sorted(keys);
        std::sort(sorted.begin(), sorted.end());
        for (int i = 0; i < nt; i++) {
            const int *q = &tet[3 * i];
            int e[3][2] = {{q[0], q[1]}, {q[0], q[2]}, {q[1], q[2]}};
            for (int k = 0; k < 3; k++) {
                auto rg = std::equal_range(sorted.begin(), sorted.end(), keys[3 * i + k]);
                if (rg.second - rg.first == 1) create_bond_raw(ctx, e[k][0] + offset - 1, e[k][1] + offset - 1);
            }
        }
    }
    Cluster &c = ctx->clusters[ci];
    c.mass = (float)M;
    c.rho = c.mass / totVol;
    for (int it = 0; it < nt; it++)
        for (int j = 0; j < 3; j++) {
            int ip = ctx->tri[3 * (size_t)(it + tetOffset) + j];
            // refVol indexed by the local triangle index, as particles.cpp:364
            float prod = c.rho * ctx->refVol[it];
            ctx->mass[ip] = (float)((double)ctx->mass[ip] + (double)prod / 3.0);
        }
    mark_topology(ctx);
    return FEMMD_OK;
}

femmd_status femmd_create_bond(femmd_ctx *ctx, int i, int j) {
    NEED(ctx);
    HOSTSYNC(ctx);
    int N = (int)ctx->pos.size();
    if (i < 0 || j < 0 || i >= N || j >= N || i == j)
        return fail(ctx, FEMMD_INVALID_ARG, "bond (%d, %d) needs two distinct particles in [0, %d)", i, j, N);
    create_bond_raw(ctx, i, j);
    mark_topology(ctx);
    return FEMMD_OK;
}

femmd_status femmd_set_velocities(femmd_ctx *ctx, double v0, uint64_t seed) {
    NEED(ctx);
    femmd_status st;
    if ((st = download_state(ctx, kAll))) return st;
    uint64_t z = seed;
    auto next = [&z]() {
        z += 0x9E3779B97F4A7C15ull;
        uint64_t r = z;
        r = (r ^ (r >> 30)) * 0xBF58476D1CE4E5B9ull;
        r = (r ^ (r >> 27)) * 0x94D049BB133111EBull;
        return r ^ (r >> 31);
    };
    const int N = (int)ctx->pos.size();
    const double twopi = 8.0 * std::atan(1.0);
    for (int p = 0; p < N; p++) {
        double s = (double)(next() >> 11) * (1.0 / 9007199254740992.0) * twopi;
        ctx->vel[p] = make_float2((float)(std::cos(s) * v0), (float)(std::sin(s) * v0));
    }
    // Particles::zeroCM (particles.cpp:246-261)
    float sx = 0, sy = 0, tm = 0;
    for (int p = 0; p < N; p++) { sx += ctx->vel[p].x * ctx->mass[p]; sy += ctx->vel[p].y * ctx->mass[p]; tm += ctx->mass[p]; }
    for (int p = 0; p < N; p++) { ctx->vel[p].x -= sx / tm; ctx->vel[p].y -= sy / tm; }
    ctx->stateDirty = true;
    return FEMMD_OK;
}

femmd_status femmd_allocate_cuda(femmd_ctx *ctx) {
    NEED(ctx);
    femmd_status st;
    if ((st = ensure_stream(ctx))) return st;
    if (ctx->nnInit) return prepare(ctx);
    return FEMMD_OK;
}

// NeighborList::init (nn.cpp:192-227): nnRadius = rCutMax + skin, cells of at least nnRadius
femmd_status femmd_init_neighbor_list(femmd_ctx *ctx) {
    NEED(ctx);
    HOSTSYNC(ctx);
    if (!ctx->inited) return fail(ctx, FEMMD_NOT_READY, "init(Lx, Ly) has not been called");
    float rc = 1.0f * ctx->rCutMax;
    ctx->nnRadius = rc + ctx->skin;
    ctx->nnRadiusSq = ctx->nnRadius * ctx->nnRadius;
    const float cell = ctx->nnRadius * ctx->cellFactor;
    int nx = (int)std::floor(ctx->Lx / cell), ny = (int)std::floor(ctx->Ly / cell);
    if (nx < 1 || ny < 1)
        return fail(ctx, FEMMD_INVALID_ARG, "box (%g, %g) is smaller than one list cell (%g)", ctx->Lx, ctx->Ly,
                    ctx->nnRadius);
    ctx->ncx = nx;
    ctx->ncy = ny;
    ctx->ncells = nx * ny;
    ctx->nnInit = true;
    mark_topology(ctx);
    ctx->nbrCap = 0;
    return FEMMD_OK;
}

femmd_status femmd_run(femmd_ctx *ctx, int steps) {
    NEED(ctx);
    if (steps < 0) return fail(ctx, FEMMD_INVALID_ARG, "steps must be >= 0");
    femmd_status st;
    if ((st = prepare(ctx))) return st;
    if ((int)ctx->pos.size() == 0) {
        ctx->steps += steps;
        return FEMMD_OK;
    }
    if ((st = ensure_obs(ctx, steps))) return st;
    const int N = (int)ctx->pos.size();
    for (int attempt = 0; attempt < 8; attempt++) {
        // start checkpoint (positions, velocities, accelerations)
        const float2 *pc = ctx->cur ? ctx->dpos1.p : ctx->dpos0.p;
        int cur0 = ctx->cur;
        CK(cudaMemcpyAsync(ctx->ckPos.p, pc, N * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->ckVel.p, ctx->dvel.p, N * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->ckAcc.p, ctx->dacc.p, N * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
        if (fast_mode(ctx))
            CK(cudaMemcpyAsync(ctx->ckPerm.p, ctx->perm.p, N * sizeof(int), cudaMemcpyDeviceToDevice, ctx->stream));
        if (ctx->propAvg)
            CK(cudaMemcpyAsync(ctx->propsCk.p, ctx->props.p, sizeof(DevProps), cudaMemcpyDeviceToDevice, ctx->stream));
        CK(cudaMemsetAsync(&ctx->sc.p->overflow, 0, 3 * sizeof(int), ctx->stream));  // overflow, nonfinite, outside
        if (ctx->tracing)
            CK(cudaMemsetAsync(ctx->trace.p, 0, (size_t)ctx->obsCap * kTraceCols * sizeof(unsigned long long),
                               ctx->stream));
        bool aborted = false;
        if ((st = run_once(ctx, steps, aborted))) return st;
        if ((st = collect_profile(ctx))) return st;
        if ((st = read_scalars(ctx))) return st;
        if (ctx->hsc->overflow & 2) return fail(ctx, FEMMD_CAPACITY_OVERFLOW, "inconsistent cell counts");
        if (ctx->hsc->overflow & 8) {
            ctx->smallClean = false;
            return fail(ctx, FEMMD_TIMEOUT,
                        "a bounded device wait expired (a copy to shared memory or a grid-wide exchange)");
        }
        if (!ctx->hsc->overflow && !aborted) {
            traj_commit(ctx->traj);
            ctx->steps += steps;
            ctx->staleMask |= kPos | kVel | kAcc | kForce;
            ctx->forcesValid = true;
            ctx->listBuilt = true;
            ctx->obsRows = std::min(ctx->hsc->obsRow, ctx->obsCap);
            ctx->totalBuilds = (long long)ctx->hsc->builds;
            if (ctx->hsc->nonfinite)
                return fail(ctx, FEMMD_NONFINITE, "a force became NaN or infinite during the run");
            return FEMMD_OK;
        }
        // roll back to the checkpoint, grow the list, repeat
        traj_discard(ctx->traj);
        ctx->cur = cur0;
        float2 *pd = ctx->cur ? ctx->dpos1.p : ctx->dpos0.p;
        CK(cudaMemcpyAsync(pd, ctx->ckPos.p, N * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->dvel.p, ctx->ckVel.p, N * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->dacc.p, ctx->ckAcc.p, N * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
        if (fast_mode(ctx)) {
            // the checkpoint's storage order and the constants in that order
            CK(cudaMemcpyAsync(ctx->perm.p, ctx->ckPerm.p, N * sizeof(int), cudaMemcpyDeviceToDevice, ctx->stream));
            DevSys ds = make_sys(ctx);
            Launch L;
            L.stream = ctx->stream;
            CK(enqueue_perm_consts(L, ds));
        }
        if (ctx->propAvg)
            CK(cudaMemcpyAsync(ctx->props.p, ctx->propsCk.p, sizeof(DevProps), cudaMemcpyDeviceToDevice, ctx->stream));
        int need = std::max(ctx->hsc->maxCount, ctx->nbrCap + ctx->nbrCap / 2);
        if ((st = alloc_list(ctx, need + need / 4 + 8))) return st;
    }
    return fail(ctx, FEMMD_CAPACITY_OVERFLOW, "neighbour list kept overflowing");
}

femmd_status femmd_do_step(femmd_ctx *ctx) {
    NEED(ctx);
    femmd_status st;
    if ((st = prepare(ctx))) return st;
    if (!ctx->listBuilt) return fail(ctx, FEMMD_NOT_READY, "do_step needs a previous run or build");
    if (ctx->pos.empty()) { ctx->steps++; return FEMMD_OK; }
    DevSys s = make_sys(ctx);
    Launch L;
    L.stream = ctx->stream;
    CK(cudaMemsetAsync(&ctx->sc.p->overflow, 0, 3 * sizeof(int), ctx->stream));
    CK(enqueue_drift(L, s, ctx->cur));
    ctx->cur ^= 1;
    CK(enqueue_rebuild(L, s, ctx->cur, 1));
    CK(enqueue_step(L, s, MODE_LAST, ctx->cur, 0, 0));
    if (ctx->propAvg) CK(enqueue_step_props(ctx, L, s, ctx->cur));
    if ((st = read_scalars(ctx))) return st;
    ctx->steps++;
    ctx->staleMask |= kPos | kVel | kAcc | kForce;
    if (ctx->hsc->overflow & 8)
        return fail(ctx, FEMMD_TIMEOUT, "a step block's copy to shared memory did not complete in time");
    if (ctx->hsc->overflow) return fail(ctx, FEMMD_CAPACITY_OVERFLOW, "neighbour list overflow in do_step; run() grows it");
    if (ctx->hsc->nonfinite) return fail(ctx, FEMMD_NONFINITE, "a force became NaN or infinite");
    return FEMMD_OK;
}

femmd_status femmd_build_neighbor_list(femmd_ctx *ctx) {
    NEED(ctx);
    femmd_status st;
    if ((st = prepare(ctx))) return st;
    if (ctx->pos.empty()) return FEMMD_OK;
    for (int attempt = 0; attempt < 4; attempt++) {
        DevSys s = make_sys(ctx);
        Launch L;
        L.stream = ctx->stream;
        CK(cudaMemsetAsync(&ctx->sc.p->overflow, 0, 3 * sizeof(int), ctx->stream));  // overflow, nonfinite, outside
        CK(enqueue_rebuild(L, s, ctx->cur, 0));
        if ((st = read_scalars(ctx))) return st;
        if (ctx->hsc->nonfinite) return fail(ctx, FEMMD_NONFINITE, "a position is NaN or infinite");
        if (ctx->hsc->overflow & 2) return fail(ctx, FEMMD_CAPACITY_OVERFLOW, "inconsistent cell counts");
        if (!ctx->hsc->overflow) {
            ctx->listBuilt = true;
            ctx->totalBuilds = (long long)ctx->hsc->builds;
            return FEMMD_OK;
        }
        int need = ctx->hsc->maxCount;
        if ((st = alloc_list(ctx, need + need / 4 + 8))) return st;
    }
    return fail(ctx, FEMMD_CAPACITY_OVERFLOW, "neighbour list kept overflowing");
}

femmd_status femmd_calc_forces(femmd_ctx *ctx) {
    NEED(ctx);
    femmd_status st;
    if ((st = prepare(ctx))) return st;
    if (ctx->pos.empty()) return FEMMD_OK;
    if (!ctx->listBuilt && (st = femmd_build_neighbor_list(ctx))) return st;
    DevSys s = make_sys(ctx);
    Launch L;
    L.stream = ctx->stream;
    CK(cudaMemsetAsync(&ctx->sc.p->nonfinite, 0, sizeof(int), ctx->stream));
    ctx->hsc->stepNow = ctx->steps;
    CK(cudaMemcpyAsync(&ctx->sc.p->stepNow, &ctx->hsc->stepNow, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(&ctx->sc.p->overflow, 0, sizeof(int), ctx->stream));
    CK(enqueue_step(L, s, MODE_FORCES, ctx->cur, 0, 0));
    if ((st = read_scalars(ctx))) return st;
    if (ctx->hsc->overflow & 8)
        return fail(ctx, FEMMD_TIMEOUT, "a step block's copy to shared memory did not complete in time");
    ctx->staleMask |= kForce | kEnergy;
    if (s.areaUnits > 0) ctx->staleMask |= kPos;  // the area springs moved the vertices
    ctx->forcesValid = true;
    if (ctx->hsc->nonfinite) return fail(ctx, FEMMD_NONFINITE, "a force became NaN or infinite");
    return FEMMD_OK;
}

femmd_status femmd_zero_stuff(femmd_ctx *ctx) {
    NEED(ctx);
    femmd_status st;
    if ((st = prepare(ctx))) return st;
    size_t N = ctx->pos.size();
    if (N) {
        CK(cudaMemsetAsync(ctx->dacc.p, 0, N * sizeof(float2), ctx->stream));
        CK(cudaMemsetAsync(ctx->dforce.p, 0, N * sizeof(float2), ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    ctx->staleMask |= kAcc | kForce;
    return FEMMD_OK;
}

femmd_status femmd_sync(femmd_ctx *ctx) {
    NEED(ctx);
    if (ctx->stream) CK(cudaStreamSynchronize(ctx->stream));
    return FEMMD_OK;
}

int femmd_get_num_particles(const femmd_ctx *ctx) { return ctx ? (int)ctx->pos.size() : 0; }
int femmd_get_num_bonds(const femmd_ctx *ctx) { return ctx ? (int)ctx->r0.size() : 0; }
int femmd_get_num_triangles(const femmd_ctx *ctx) { return ctx ? (int)ctx->refVol.size() : 0; }
int femmd_get_num_elastomers(const femmd_ctx *ctx) { return ctx ? (int)ctx->clusters.size() : 0; }
int femmd_get_steps(const femmd_ctx *ctx) { return ctx ? ctx->steps : 0; }

static femmd_status copy2(femmd_ctx *ctx, const std::vector<float2> &v, float *out) {
    if (!out) return fail(ctx, FEMMD_INVALID_ARG, "null output");
    if (!v.empty()) memcpy(out, v.data(), v.size() * sizeof(float2));
    return FEMMD_OK;
}

femmd_status femmd_get_positions(femmd_ctx *ctx, float *out) {
    NEED(ctx);
    femmd_status st;
    if ((st = download_state(ctx, kPos))) return st;
    return copy2(ctx, ctx->pos, out);
}
femmd_status femmd_get_velocities(femmd_ctx *ctx, float *out) {
    NEED(ctx);
    femmd_status st;
    if ((st = download_state(ctx, kVel))) return st;
    return copy2(ctx, ctx->vel, out);
}
femmd_status femmd_get_accelerations(femmd_ctx *ctx, float *out) {
    NEED(ctx);
    femmd_status st;
    if ((st = download_state(ctx, kAcc))) return st;
    return copy2(ctx, ctx->acc, out);
}
femmd_status femmd_get_forces(femmd_ctx *ctx, float *out) {
    NEED(ctx);
    femmd_status st;
    if ((st = download_state(ctx, kForce))) return st;
    return copy2(ctx, ctx->force, out);
}
femmd_status femmd_get_particle_energies(femmd_ctx *ctx, float *out) {
    NEED(ctx);
    femmd_status st;
    if ((st = download_state(ctx, kEnergy))) return st;
    if (!out) return fail(ctx, FEMMD_INVALID_ARG, "null output");
    if (!ctx->energy.empty()) memcpy(out, ctx->energy.data(), ctx->energy.size() * sizeof(float));
    return FEMMD_OK;
}
femmd_status femmd_get_masses(const femmd_ctx *ctx, float *out) {
    if (!ctx || !out) return FEMMD_INVALID_ARG;
    if (!ctx->mass.empty()) memcpy(out, ctx->mass.data(), ctx->mass.size() * sizeof(float));
    return FEMMD_OK;
}
femmd_status femmd_get_bonds(const femmd_ctx *ctx, int *pairs, float *rl) {
    if (!ctx) return FEMMD_INVALID_ARG;
    if (pairs && !ctx->bond.empty()) memcpy(pairs, ctx->bond.data(), ctx->bond.size() * sizeof(int));
    if (rl && !ctx->r0.empty()) memcpy(rl, ctx->r0.data(), ctx->r0.size() * sizeof(float));
    return FEMMD_OK;
}
femmd_status femmd_get_triangles(const femmd_ctx *ctx, int *tris, float *xm, float *area) {
    if (!ctx) return FEMMD_INVALID_ARG;
    if (tris && !ctx->tri.empty()) memcpy(tris, ctx->tri.data(), ctx->tri.size() * sizeof(int));
    if (xm && !ctx->xm.empty()) memcpy(xm, ctx->xm.data(), ctx->xm.size() * sizeof(float));
    if (area && !ctx->refVol.empty()) memcpy(area, ctx->refVol.data(), ctx->refVol.size() * sizeof(float));
    return FEMMD_OK;
}
femmd_status femmd_get_exclusion_groups(const femmd_ctx *ctx, int *out) {
    if (!ctx || !out) return FEMMD_INVALID_ARG;
    if (!ctx->excl.empty()) memcpy(out, ctx->excl.data(), ctx->excl.size() * sizeof(int));
    return FEMMD_OK;
}
femmd_status femmd_get_reference_positions(const femmd_ctx *ctx, float *out) {
    if (!ctx || !out) return FEMMD_INVALID_ARG;
    if (!ctx->refPos.empty()) memcpy(out, ctx->refPos.data(), ctx->refPos.size() * sizeof(float2));
    return FEMMD_OK;
}

femmd_status femmd_get_energies(femmd_ctx *ctx, double *out) {
    NEED(ctx);
    if (!out) return fail(ctx, FEMMD_INVALID_ARG, "null output");
    if (!ctx->sc.p) {
        for (int k = 0; k < 6; k++) out[k] = 0;
        return FEMMD_OK;
    }
    femmd_status st;
    if ((st = read_scalars(ctx))) return st;
    const DevScalars &h = *ctx->hsc;
    out[0] = h.U;
    out[1] = h.W;
    out[2] = h.KE;
    out[3] = h.vvMax;
    out[4] = h.dispHi;
    out[5] = h.totalUpdates;
    return FEMMD_OK;
}

femmd_status femmd_get_step_observables(femmd_ctx *ctx, double *out, int max_rows, int *rows) {
    NEED(ctx);
    if (!rows) return fail(ctx, FEMMD_INVALID_ARG, "null output");
    int n = std::min(ctx->obsRows, std::max(max_rows, 0));
    *rows = ctx->obsRows;
    if (n > 0 && out) {
        CK(cudaMemcpyAsync(out, ctx->obs.p, (size_t)n * kObsCols * sizeof(double), cudaMemcpyDeviceToHost,
                           ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return FEMMD_OK;
}

femmd_status femmd_get_grid(const femmd_ctx *ctx, int *ncx, int *ncy) {
    if (!ctx || !ncx || !ncy) return FEMMD_INVALID_ARG;
    *ncx = ctx->ncx;
    *ncy = ctx->ncy;
    return FEMMD_OK;
}

femmd_status femmd_get_cells(femmd_ctx *ctx, int *cell_start, int *cell_ids) {
    NEED(ctx);
    if (!ctx->listBuilt) return fail(ctx, FEMMD_NOT_READY, "no neighbour list has been built");
    const int N = (int)ctx->pos.size();
    // the device numbers cells column-major (ix*ncy + iy); the reference's
    // numbering is row-major (ix + iy*ncx)
    std::vector<int> start(ctx->ncells + 1), ids(N);
    CK(cudaMemcpyAsync(start.data(), ctx->cellStart.p, (ctx->ncells + 1) * sizeof(int), cudaMemcpyDeviceToHost,
                       ctx->stream));
    if (N) CK(cudaMemcpyAsync(ids.data(), ctx->sortedIds.p, N * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    std::vector<int> perm;
    if (fast_mode(ctx) && N) {
        perm.resize(N);
        CK(cudaMemcpyAsync(perm.data(), ctx->perm.p, N * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    if (!perm.empty()) {
        // storage slots to ids, ascending inside each cell as the reference's
        for (int &v : ids) v = perm[v];
        for (int c = 0; c < ctx->ncells; c++) std::sort(ids.begin() + start[c], ids.begin() + start[c + 1]);
    }
    int at = 0;
    for (int iy = 0; iy < ctx->ncy; iy++)
        for (int ix = 0; ix < ctx->ncx; ix++) {
            const int c = ix * ctx->ncy + iy;
            if (cell_start) cell_start[ix + iy * ctx->ncx] = at;
            for (int q = start[c]; q < start[c + 1]; q++) {
                if (cell_ids && at < N) cell_ids[at] = ids[q];
                at++;
            }
        }
    if (cell_start) cell_start[ctx->ncells] = at;
    return FEMMD_OK;
}

femmd_status femmd_get_neighbor_total(femmd_ctx *ctx, long long *total) {
    NEED(ctx);
    if (!total) return fail(ctx, FEMMD_INVALID_ARG, "null output");
    if (!ctx->listBuilt) return fail(ctx, FEMMD_NOT_READY, "no neighbour list has been built");
    femmd_status st;
    if ((st = read_scalars(ctx))) return st;
    *total = (long long)ctx->hsc->nbrSum;
    return FEMMD_OK;
}

femmd_status femmd_get_neighbors(femmd_ctx *ctx, int *nbr_start, int *nbr_list) {
    NEED(ctx);
    if (!ctx->listBuilt) return fail(ctx, FEMMD_NOT_READY, "no neighbour list has been built");
    const int N = (int)ctx->pos.size();
    std::vector<int> cnt(N);
    std::vector<int> raw((size_t)ctx->nbrCap * ctx->Ncap);
    std::vector<int> perm, slot, cellIds, bw;
    if (N) {
        CK(cudaMemcpyAsync(cnt.data(), ctx->nbrCount.p, N * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(raw.data(), ctx->nbr.p, raw.size() * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        if (fast_mode(ctx)) {
            perm.resize(N);
            cellIds.resize(N);
            bw.resize(kWinInts * (size_t)((N + kFastBlock - 1) / kFastBlock));
            CK(cudaMemcpyAsync(perm.data(), ctx->perm.p, N * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaMemcpyAsync(cellIds.data(), ctx->sortedIds.p, N * sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
            CK(cudaMemcpyAsync(bw.data(), ctx->blockWin.p, bw.size() * sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
        }
        CK(cudaStreamSynchronize(ctx->stream));
    }
    if (!perm.empty()) {
        // rows by particle id, entries as ids (the fast mode's list order
        // inside a row is not the reference's; the sets are)
        slot.resize(N);
        for (int q = 0; q < N; q++) slot[perm[q]] = q;
    }
    // fast mode: entry q of the particle at storage slot r, as a storage slot
    // (a windowed block's entry is an index into its window's cell slots)
    const bool win16 = fast_mode(ctx) && make_sys(ctx).win16;
    const unsigned short *raw16 = reinterpret_cast<const unsigned short *>(raw.data());
    auto fast_entry = [&](int r, int q) -> int {
        const int *b = &bw[kWinInts * (size_t)(r / kFastBlock)];
        if (b[kWLen] < 0) return raw[nbr_at(q, r, ctx->Ncap)] & kIdMask;  // (the high bits: the neighbour's type)
        const int w = win16 ? (int)raw16[nbr16_at(q, r, ctx->Ncap)] : raw[nbr_at(q, r, ctx->Ncap)] & kIdMask;
        for (int p = 0; p < kWinPieces; p++)
            if (w >= b[kWOff + p] && w < b[kWOff + p] + b[kWCount + p])
                return cellIds[b[kWStart + p] + (w - b[kWOff + p])];
        return -1;  // not an entry of the window: a mismatch the set comparison exposes
    };
    long long k = 0;
    for (int i = 0; i < N; i++) {
        if (nbr_start) nbr_start[i] = (int)k;
        const int r = perm.empty() ? i : slot[i];
        int c = std::min(cnt[r], ctx->nbrCap);
        for (int q = 0; q < c; q++) {
            if (nbr_list) {
                if (perm.empty()) {
                    nbr_list[k] = raw[nbr_at(q, r, ctx->Ncap)] & kIdMask;
                } else {
                    const int e = fast_entry(r, q);
                    nbr_list[k] = e >= 0 ? perm[e] : -1;
                }
            }
            k++;
        }
    }
    if (nbr_start) nbr_start[N] = (int)k;
    return FEMMD_OK;
}

femmd_status femmd_get_nn_stats(femmd_ctx *ctx, double *mean_neighbors, int *max_neighbors, long long *builds) {
    NEED(ctx);
    femmd_status st;
    if (!ctx->sc.p) return fail(ctx, FEMMD_NOT_READY, "nothing has run");
    if ((st = read_scalars(ctx))) return st;
    int N = (int)ctx->pos.size();
    if (mean_neighbors) *mean_neighbors = N ? (double)ctx->hsc->nbrSum / N : 0.0;
    if (max_neighbors) *max_neighbors = ctx->hsc->maxCount;
    if (builds) *builds = (long long)ctx->hsc->builds;
    return FEMMD_OK;
}

femmd_status femmd_info(const femmd_ctx *ctx, double *o) {
    if (!ctx || !o) return FEMMD_INVALID_ARG;
    o[0] = (double)ctx->pos.size();
    o[1] = (double)ctx->clusters.size();
    o[2] = (double)ctx->bond.size();  // bondList.size() as the reference reports (2 per bond)
    o[3] = (double)ctx->refVol.size();
    o[4] = ctx->dt;
    o[5] = ctx->kBond;
    o[6] = ctx->kArea;
    o[7] = ctx->E;
    o[8] = ctx->Lx;
    return FEMMD_OK;
}

femmd_status femmd_set_state(femmd_ctx *ctx, const float *p, const float *v) {
    NEED(ctx);
    femmd_status st;
    const size_t N = ctx->pos.size();
    if (!ctx->topoDirty && !ctx->stateDirty && ctx->stream && N) {
        // device copy current: copy the caller's arrays straight to the device;
        // the host copies become stale.  The next run starts with a forced rebuild.
        float2 *pd = ctx->cur ? ctx->dpos1.p : ctx->dpos0.p;
        if (fast_mode(ctx)) {
            if (p) CK(fast_upload2(ctx, p, pd));
            if (v) CK(fast_upload2(ctx, v, ctx->dvel.p));
        } else {
            if (p) CK(cudaMemcpyAsync(pd, p, N * sizeof(float2), cudaMemcpyHostToDevice, ctx->stream));
            if (v) CK(cudaMemcpyAsync(ctx->dvel.p, v, N * sizeof(float2), cudaMemcpyHostToDevice, ctx->stream));
        }
        CK(cudaStreamSynchronize(ctx->stream));
        ctx->listBuilt = false;
        if (p) ctx->staleMask |= kPos;
        if (v) ctx->staleMask |= kVel;
        return FEMMD_OK;
    }
    if ((st = download_state(ctx, kAll))) return st;
    if (p) memcpy(ctx->pos.data(), p, N * sizeof(float2));
    if (v) memcpy(ctx->vel.data(), v, N * sizeof(float2));
    ctx->stateDirty = true;
    return FEMMD_OK;
}

femmd_status femmd_get_state(femmd_ctx *ctx, float *p, float *v, float *a) {
    NEED(ctx);
    const size_t N = ctx->pos.size();
    if (!N) return FEMMD_OK;
    // device-current arrays go straight into the caller's buffers
    unsigned dev = ctx->staleMask;
    cudaStream_t s = ctx->stream;
    // device arrays in storage order pass through the unpermute (fast mode)
    auto d2h = [&](void *out, const float2 *in) -> cudaError_t {
        if (fast_mode(ctx)) return fast_download2(ctx, in, out);
        return cudaMemcpyAsync(out, in, N * sizeof(float2), cudaMemcpyDeviceToHost, s);
    };
    if (p) {
        if (dev & kPos)
            CK(d2h(p, ctx->cur ? ctx->dpos1.p : ctx->dpos0.p));
        else
            memcpy(p, ctx->pos.data(), N * sizeof(float2));
    }
    if (v) {
        if (dev & kVel) CK(d2h(v, ctx->dvel.p));
        else memcpy(v, ctx->vel.data(), N * sizeof(float2));
    }
    if (a) {
        if (dev & kAcc) CK(d2h(a, ctx->dacc.p));
        else memcpy(a, ctx->acc.data(), N * sizeof(float2));
    }
    if (dev && s) CK(cudaStreamSynchronize(s));
    return FEMMD_OK;
}

void *femmd_get_stream(femmd_ctx *ctx) {
    if (!ctx) return nullptr;
    if (ensure_stream(ctx) != FEMMD_OK) return nullptr;
    return (void *)ctx->stream;
}

femmd_status femmd_event_record(femmd_ctx *ctx, int slot) {
    NEED(ctx);
    if (slot < 0 || slot >= 64) return fail(ctx, FEMMD_INVALID_ARG, "event slot outside [0, 64)");
    femmd_status st;
    if ((st = ensure_stream(ctx))) return st;
    if (!ctx->userEvents[slot]) CK(cudaEventCreate(&ctx->userEvents[slot]));
    CK(cudaEventRecord(ctx->userEvents[slot], ctx->stream));
    return FEMMD_OK;
}

femmd_status femmd_event_elapsed(femmd_ctx *ctx, int a, int b, float *ms) {
    NEED(ctx);
    if (a < 0 || a >= 64 || b < 0 || b >= 64 || !ms || !ctx->userEvents[a] || !ctx->userEvents[b])
        return fail(ctx, FEMMD_INVALID_ARG, "unrecorded event slot");
    CK(cudaEventSynchronize(ctx->userEvents[b]));
    CK(cudaEventElapsedTime(ms, ctx->userEvents[a], ctx->userEvents[b]));
    return FEMMD_OK;
}

femmd_status femmd_set_trace(femmd_ctx *ctx, int on) {
    NEED(ctx);
    ctx->tracing = on != 0;
    release_graphs(ctx);
    return FEMMD_OK;
}

femmd_status femmd_get_trace(femmd_ctx *ctx, unsigned long long *out, int max_rows, int *rows) {
    NEED(ctx);
    if (!rows) return fail(ctx, FEMMD_INVALID_ARG, "null output");
    int n = std::min(ctx->obsRows, std::max(max_rows, 0));
    *rows = ctx->tracing ? ctx->obsRows : 0;
    if (ctx->tracing && n > 0 && out) {
        CK(cudaMemcpyAsync(out, ctx->trace.p, (size_t)n * kTraceCols * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return FEMMD_OK;
}

femmd_status femmd_set_profiling(femmd_ctx *ctx, int profile) {
    NEED(ctx);
    ctx->profiling = profile != 0;
    ctx->profForceMs = ctx->profRebuildMs = 0;
    ctx->profForceLaunches = ctx->profRebuilds = ctx->profKernels = 0;
    return FEMMD_OK;
}

femmd_status femmd_test_expire_next_exchange(femmd_ctx *ctx) {
    NEED(ctx);
    ctx->testExpire = true;
    return FEMMD_OK;
}

femmd_status femmd_get_profile(femmd_ctx *ctx, double *fms, long long *fl, double *rms, long long *rb,
                               long long *kl) {
    NEED(ctx);
    if (fms) *fms = ctx->profForceMs;
    if (fl) *fl = ctx->profForceLaunches;
    if (rms) *rms = ctx->profRebuildMs;
    if (rb) *rb = ctx->profRebuilds;
    if (kl) *kl = ctx->profKernels;
    return FEMMD_OK;
}


// ============================================================= trajectory

femmd_status femmd_set_trajectory(femmd_ctx *ctx, const char *path, int every, int format) {
    NEED(ctx);
    Trajectory &T = ctx->traj;
    traj_stop(T);
    T.on = false;
    if (!path || every <= 0) return FEMMD_OK;
    if (format < 0 || format > 6) return fail(ctx, FEMMD_INVALID_ARG, "format must be in 0..6 (femmd.h)");
    T.meta.path = path;
    T.meta.format = format;
    T.every = every;
    T.headerDone = false;
    T.error.clear();
    T.written = 0;
    T.N = 0;
    T.lastCommitted = (long long)ctx->steps;  // frames from the next step on
    if (format <= 1 || format == 3 || format == 4) {
        FILE *f = fopen(path, "w");  // a new trajectory starts a new file
        if (!f) return fail(ctx, FEMMD_INVALID_ARG, "cannot create %s", path);
        fclose(f);
    }
    T.on = true;
    traj_refresh_meta(ctx);
    T.th = std::thread(traj_writer, &T);
    return FEMMD_OK;
}

// save_vtk / save_vtf / save_cluster_vtf / save_cluster_xyz
// (interface.cpp:301-330) and the reference's other writers: the current
// state, now, in layout 'format' of femmd_set_trajectory.
femmd_status femmd_save_frame(femmd_ctx *ctx, const char *path, int format, int append) {
    NEED(ctx);
    if (!path) return fail(ctx, FEMMD_INVALID_ARG, "null path");
    if (format < 0 || format > 6) return fail(ctx, FEMMD_INVALID_ARG, "format must be in 0..6 (femmd.h)");
    femmd_status st;
    if ((st = download_state(ctx, kPos | kVel))) return st;
    FrameMeta M;
    frame_meta(ctx, M);
    M.path = path;
    M.format = format;
    std::string err;
    if (!write_frame(M, (int)ctx->pos.size(), ctx->steps, ctx->pos.data(), ctx->vel.data(), append == 0, append == 0,
                     err))
        return fail(ctx, FEMMD_INVALID_ARG, "%s", err.c_str());
    return FEMMD_OK;
}

// MDSystem::scale (DukSystemSetScale, interface.cpp:365-369).
femmd_status femmd_set_scale(femmd_ctx *ctx, double scale) {
    NEED(ctx);
    ctx->scale = (float)scale;  // real scale (md3dsystem.h:40)
    traj_refresh_meta(ctx);
    return FEMMD_OK;
}

femmd_status femmd_flush_trajectory(femmd_ctx *ctx, long long *frames_written) {
    NEED(ctx);
    Trajectory &T = ctx->traj;
    traj_drain(T);
    if (frames_written) {
        std::lock_guard<std::mutex> lk(T.mu);
        *frames_written = T.written;
    }
    if (!T.error.empty()) return fail(ctx, FEMMD_INVALID_ARG, "trajectory: %s", T.error.c_str());
    return FEMMD_OK;
}

// ============================================================== observables

// Properties::evaluate (properties.cpp:15-36) at the current state:
// out[0..9] = uKinetic, uPotential, uTotal, temperature, virial, feaVirial,
// pressure, clusterUKinetic, clusterVirial, molPressure.
femmd_status femmd_get_properties(femmd_ctx *ctx, double *out) {
    NEED(ctx);
    if (!out) return fail(ctx, FEMMD_INVALID_ARG, "null output");
    femmd_status st;
    if ((st = prepare(ctx))) return st;
    // the force pass of an evaluation must not move anything: with area
    // springs it displaces the vertices, so the positions are put back
    const bool area = ctx->areaForces && ctx->areaUnits > 0 && !ctx->pos.empty();
    const size_t np = ctx->pos.size();
    if (area) {
        CK(ctx->ckPos.ensure(np));
        CK(cudaMemcpyAsync(ctx->ckPos.p, ctx->cur ? ctx->dpos1.p : ctx->dpos0.p, np * sizeof(float2),
                           cudaMemcpyDeviceToDevice, ctx->stream));
    }
    if ((st = femmd_calc_forces(ctx))) return st;
    if (area)
        CK(cudaMemcpyAsync(ctx->cur ? ctx->dpos1.p : ctx->dpos0.p, ctx->ckPos.p, np * sizeof(float2),
                           cudaMemcpyDeviceToDevice, ctx->stream));
    const int N = (int)ctx->pos.size(), nt = (int)ctx->refVol.size(), ncl = (int)ctx->clusters.size();
    for (int k = 0; k < 10; k++) out[k] = 0.0;
    if (N == 0) return FEMMD_OK;
    cudaStream_t sm = ctx->stream;
    if ((st = props_buffers(ctx))) return st;
    DevSys s = make_sys(ctx);
    const float2 *pc = ctx->cur ? ctx->dpos1.p : ctx->dpos0.p;
    Launch L;
    L.stream = sm;
    CK(enqueue_props(L, s, pc, ncl, ctx->clRange.p, ctx->clMass.p, ctx->clusterOf.p, ctx->unf.p, ctx->cmPos.p,
                     ctx->cmVel.p, ctx->clKin.p, ctx->feaVir.p, ctx->kinTerm.p, ctx->clVir.p, N));
    std::vector<double> kin(N), cv(N), fv(std::max(nt, 1), 0.0), ck(std::max(ncl, 1), 0.0);
    CK(cudaMemcpyAsync(kin.data(), ctx->kinTerm.p, N * sizeof(double), cudaMemcpyDeviceToHost, sm));
    CK(cudaMemcpyAsync(cv.data(), ctx->clVir.p, N * sizeof(double), cudaMemcpyDeviceToHost, sm));
    if (ncl > 0) {
        CK(cudaMemcpyAsync(ck.data(), ctx->clKin.p, ncl * sizeof(double), cudaMemcpyDeviceToHost, sm));
        if (nt > 0) CK(cudaMemcpyAsync(fv.data(), ctx->feaVir.p, nt * sizeof(double), cudaMemcpyDeviceToHost, sm));
    }
    if ((st = read_scalars(ctx))) return st;
    double kinEneSum = 0, clusterVirial = 0, feaVirial = 0, clusterKin = 0;
    for (double v : kin) kinEneSum += v;
    for (double v : cv) clusterVirial += v;
    if (ncl > 0) {
        for (int t = 0; t < nt; t++) feaVirial += fv[t];
        for (int c = 0; c < ncl; c++) clusterKin += ck[c];
    }
    const double V = (double)ctx->Lx * (double)ctx->Ly;
    const double U = ctx->hsc->U, W = ctx->hsc->W;
    out[0] = 0.5 * kinEneSum / N;
    out[1] = U / N;
    out[2] = out[0] + out[1];
    out[3] = out[0];
    out[4] = W;
    out[5] = feaVirial;
    out[6] = 0.5 * kinEneSum / V + 0.5 * (W + feaVirial) / V;
    out[7] = ncl > 0 ? 0.5 * clusterKin / ncl : 0.0;
    out[8] = clusterVirial;
    out[9] = 0.5 * clusterKin / V - 0.5 * clusterVirial / V;
    return FEMMD_OK;
}

// FeaElements::calcClusterProps (feaElements.cpp:199-204) at the current
// state: unfoldPos's centre of mass and its velocity per cluster, and the
// periodic centroid of updateClustersCentroid; 2 doubles per cluster each
// (NULL to skip).
femmd_status femmd_get_clusters(femmd_ctx *ctx, double *cm, double *cm_vel, double *centroid) {
    NEED(ctx);
    femmd_status st;
    if ((st = prepare(ctx))) return st;
    const int N = (int)ctx->pos.size(), ncl = (int)ctx->clusters.size();
    if (N == 0 || ncl == 0) return FEMMD_OK;
    if ((st = props_buffers(ctx))) return st;
    CK(ctx->centroid.ensure(ncl));
    DevSys s = make_sys(ctx);
    const float2 *pc = ctx->cur ? ctx->dpos1.p : ctx->dpos0.p;
    Launch L;
    L.stream = ctx->stream;
    CK(enqueue_props(L, s, pc, ncl, ctx->clRange.p, ctx->clMass.p, ctx->clusterOf.p, ctx->unf.p, ctx->cmPos.p,
                     ctx->cmVel.p, ctx->clKin.p, ctx->feaVir.p, ctx->kinTerm.p, ctx->clVir.p, N));
    CK(enqueue_cluster_centroid(L, s, pc, ncl, ctx->clRange.p, ctx->centroid.p));
    if (cm) CK(cudaMemcpyAsync(cm, ctx->cmPos.p, ncl * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
    if (cm_vel) CK(cudaMemcpyAsync(cm_vel, ctx->cmVel.p, ncl * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
    if (centroid)
        CK(cudaMemcpyAsync(centroid, ctx->centroid.p, ncl * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return FEMMD_OK;
}

// Properties::compute (properties.cpp:85-95) at the end of every step of
// run() and do_step(): with on != 0 the properties of femmd_get_properties
// are evaluated after each step and accumulated; at steps past step_equi
// that are multiples of step_avg the window's average and standard deviation
// are kept and a new window starts (the reference's defaults: 1000, 10000).
// Switching on (again) starts from empty sums.
femmd_status femmd_set_property_averaging(femmd_ctx *ctx, int on, int step_avg, int step_equi) {
    NEED(ctx);
    if (on && (step_avg <= 0 || step_equi < 0))
        return fail(ctx, FEMMD_INVALID_ARG, "step_avg must be > 0 and step_equi >= 0");
    ctx->propAvg = on != 0;
    if (on) {
        ctx->propAvgEvery = step_avg;
        ctx->propEqui = step_equi;
        ctx->propsReset = true;
    }
    release_graphs(ctx);
    return FEMMD_OK;
}

femmd_status femmd_get_average_properties(femmd_ctx *ctx, double *avg, double *stdv, double *val, int *count,
                                          int *windows, int *last_step) {
    NEED(ctx);
    if (!ctx->props.p || ctx->propsReset) return fail(ctx, FEMMD_NOT_READY, "no step has been averaged");
    DevProps P;
    CK(cudaMemcpyAsync(&P, ctx->props.p, sizeof(DevProps), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < kNumProps; k++) {
        if (avg) avg[k] = P.avg[k];
        if (stdv) stdv[k] = P.stdv[k];
        if (val) val[k] = P.val[k];
    }
    if (count) *count = P.count;
    if (windows) *windows = P.windows;
    if (last_step) *last_step = P.lastStep;
    return FEMMD_OK;
}

// ================================================================== adjoint

static float wall_y_host(const femmd_ctx *ctx, int n) { return ctx->wallY0 - ctx->wallV * ((float)n * ctx->dt); }

static femmd_status adj_supported(femmd_ctx *ctx) {
    if (fast_mode(ctx))
        return fail(ctx, FEMMD_UNSUPPORTED, "the adjoint replays the reference-exact force mode; set it first");
    if (ctx->areaForces && !ctx->refVol.empty())
        return fail(ctx, FEMMD_UNSUPPORTED, "the adjoint does not implement the area springs");
    if (!ctx->wallOn && ctx->pbc != FEMMD_XYPBC)
        return fail(ctx, FEMMD_UNSUPPORTED, "the adjoint implements the moving walls, not the reference's fixed walls");
    if (ctx->feaForces && !ctx->refVol.empty() && ctx->feaLaw != FEMMD_FEA_NEO_HOOKEAN)
        return fail(ctx, FEMMD_UNSUPPORTED, "the adjoint implements the neo-Hookean triangle law");
    if (ctx->bondForces && !ctx->r0.empty() && ctx->bondKMode != FEMMD_BONDK_KBOND)
        return fail(ctx, FEMMD_UNSUPPORTED, "the adjoint implements bonds with the constant kBond");
    return FEMMD_OK;
}

femmd_status femmd_adjoint_forward(femmd_ctx *ctx, int steps, int every) {
    NEED(ctx);
    femmd_status st;
    if (steps < 1 || every < 1) return fail(ctx, FEMMD_INVALID_ARG, "steps and every must be >= 1");
    if ((st = prepare(ctx))) return st;
    if ((st = adj_supported(ctx))) return st;
    const int N = (int)ctx->pos.size();
    if (N == 0) return fail(ctx, FEMMD_NOT_READY, "no particles");
    auto &a = ctx->adj;
    a.ready = false;
    const int nseg = (steps + every - 1) / every;
    a.every = every;
    a.segStart.assign(nseg, 0);
    a.segLen.assign(nseg, 0);
    a.segReb.assign(nseg, std::vector<char>());
    CK(a.ckX.ensure((size_t)nseg * N));
    CK(a.ckV.ensure((size_t)nseg * N));
    for (int g = 0; g < nseg; g++) {
        const int len = std::min(every, steps - g * every);
        const float2 *pc = ctx->cur ? ctx->dpos1.p : ctx->dpos0.p;
        CK(cudaMemcpyAsync(a.ckX.p + (size_t)g * N, pc, N * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
        CK(cudaMemcpyAsync(a.ckV.p + (size_t)g * N, ctx->dvel.p, N * sizeof(float2), cudaMemcpyDeviceToDevice,
                           ctx->stream));
        a.segStart[g] = ctx->steps;
        a.segLen[g] = len;
        if ((st = femmd_run(ctx, len))) return st;
        // the run's MID unit u (forces at x_u) wrote observable row u-1, whose
        // last column says whether a rebuild followed it
        a.segReb[g].assign(len, 0);
        if (len > 1) {
            std::vector<double> o((size_t)(len - 1) * kObsCols);
            CK(cudaMemcpyAsync(o.data(), ctx->obs.p, o.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
            for (int u = 1; u < len; u++) a.segReb[g][u] = o[(size_t)(u - 1) * kObsCols + 5] != 0.0;
        }
    }
    a.maxLen = std::min(every, steps);
    a.endStep = ctx->steps;
    a.ready = true;
    return FEMMD_OK;
}

femmd_status femmd_adjoint_observable(femmd_ctx *ctx, double *wall_stress, double *fea_energy) {
    NEED(ctx);
    femmd_status st;
    if ((st = femmd_calc_forces(ctx))) return st;
    double ws = 0.0, fe = 0.0;
    if (ctx->wallOn) {
        double top, bottom;
        if ((st = femmd_get_wall_forces(ctx, &top, &bottom))) return st;
        ws = (top + bottom) / (2.0 * (double)ctx->Lx);
    }
    const int nt = (int)ctx->refVol.size();
    if (ctx->feaForces && nt > 0) {
        std::vector<float> e(nt);
        CK(cudaMemcpyAsync(e.data(), ctx->triE.p, nt * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        for (float v : e) fe += (double)v;
    }
    if (wall_stress) *wall_stress = ws;
    if (fea_energy) *fea_energy = fe;
    return FEMMD_OK;
}

// Recompute segment g from its checkpoint (the forward's kernels in the
// forward's order, launched directly) and record its positions in slots
// 0..K; returns the rebuild points (slot indices whose positions a list was
// built from).
static femmd_status adj_recompute(femmd_ctx *ctx, int g, std::vector<int> &rebuilt) {
    auto &a = ctx->adj;
    const int N = (int)ctx->pos.size(), K = a.segLen[g];
    cudaStream_t st = ctx->stream;
    CK(cudaMemcpyAsync(ctx->dpos0.p, a.ckX.p + (size_t)g * N, N * sizeof(float2), cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(ctx->dvel.p, a.ckV.p + (size_t)g * N, N * sizeof(float2), cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(a.slots.p, ctx->dpos0.p, N * sizeof(float2), cudaMemcpyDeviceToDevice, st));
    ctx->cur = 0;
    ctx->steps = a.segStart[g];
    DevSys s = make_sys(ctx);
    Launch L;
    L.stream = st;
    CK(cudaMemsetAsync(&ctx->sc.p->overflow, 0, 3 * sizeof(int), st));
    CK(enqueue_run_start(L, s));
    CK(enqueue_rebuild(L, s, 0, 1));
    CK(enqueue_step(L, s, MODE_FIRST, 0, 0, 0));
    int cur = 1;
    CK(cudaMemcpyAsync(a.slots.p + N, ctx->dpos1.p, N * sizeof(float2), cudaMemcpyDeviceToDevice, st));
    for (int u = 1; u < K; u++) {
        CK(enqueue_step(L, s, MODE_MID, cur, 0, 0));
        float2 *pout = cur ? ctx->dpos0.p : ctx->dpos1.p;
        CK(cudaMemcpyAsync(a.slots.p + (size_t)(u + 1) * N, pout, N * sizeof(float2), cudaMemcpyDeviceToDevice, st));
        // the rebuild kernels only where the forward rebuilt (elsewhere
        // their check would return at once); a disagreement is caught below
        if (a.segReb[g][u]) CK(enqueue_rebuild(L, s, 1 - cur, 1));
        cur ^= 1;
    }
    femmd_status e;
    if ((e = read_scalars(ctx))) return e;
    if (ctx->hsc->overflow || ctx->hsc->nonfinite)
        return fail(ctx, ctx->hsc->overflow ? FEMMD_CAPACITY_OVERFLOW : FEMMD_NONFINITE,
                    "the recomputed segment differs from the forward pass (overflow or non-finite force)");
    // MID step u (forces at slot u) writes observable row u-1; its rebuild
    // flag means a list was built from slot u+1
    rebuilt.assign(1, 0);
    const int rows = std::max(K - 1, 0);
    if (rows > 0) {
        std::vector<double> o((size_t)rows * kObsCols);
        CK(cudaMemcpyAsync(o.data(), ctx->obs.p, o.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int u = 1; u < K; u++) {
            const bool reb = o[(size_t)(u - 1) * kObsCols + 5] != 0.0;
            if (reb != (a.segReb[g][u] != 0))
                return fail(ctx, FEMMD_NOT_READY, "the recomputed segment's rebuilds differ from the forward pass");
            if (reb) rebuilt.push_back(u + 1);
        }
    }
    return FEMMD_OK;
}

femmd_status femmd_adjoint_backward(femmd_ctx *ctx, double c_wall, double c_fea, const float *xbar_final,
                                    const float *vbar_final, float *xbar_init, float *vbar_init, double *dJ_dE,
                                    double *dJ_dnu, double *dJ_dlog_eps, double *dJ_dlog_sigma) {
    NEED(ctx);
    auto &a = ctx->adj;
    if (!a.ready) return fail(ctx, FEMMD_NOT_READY, "femmd_adjoint_forward has not been run");
    if (ctx->steps != a.endStep || ctx->topoDirty || ctx->stateDirty || ctx->materialDirty)
        return fail(ctx, FEMMD_NOT_READY, "the system changed after femmd_adjoint_forward");
    femmd_status st;
    if ((st = adj_supported(ctx))) return st;
    const int N = (int)ctx->pos.size(), nt = (int)ctx->refVol.size();
    const int nseg = (int)a.segLen.size();
    cudaStream_t sm = ctx->stream;
    // keep the final state; the sweep overwrites the context's buffers
    CK(a.finalX.ensure(N)); CK(a.finalV.ensure(N)); CK(a.finalA.ensure(N));
    CK(a.slots.ensure((size_t)(a.maxLen + 1) * N));
    CK(a.xbar.ensure(N)); CK(a.vbar.ensure(N)); CK(a.w0.ensure(N)); CK(a.w1.ensure(N));
    CK(a.triD.ensure(3 * (size_t)std::max(nt, 1)));
    CK(a.gMu.ensure(std::max(nt, 1))); CK(a.gLam.ensure(std::max(nt, 1)));
    CK(a.epsAcc.ensure(N)); CK(a.sigAcc.ensure(N));
    if ((st = ensure_obs(ctx, a.maxLen))) return st;
    // FEA nodal forces and energies at x_N for the seed
    if ((st = femmd_calc_forces(ctx))) return st;
    const float2 *pN = ctx->cur ? ctx->dpos1.p : ctx->dpos0.p;
    CK(cudaMemcpyAsync(a.finalX.p, pN, N * sizeof(float2), cudaMemcpyDeviceToDevice, sm));
    CK(cudaMemcpyAsync(a.finalV.p, ctx->dvel.p, N * sizeof(float2), cudaMemcpyDeviceToDevice, sm));
    CK(cudaMemcpyAsync(a.finalA.p, ctx->dacc.p, N * sizeof(float2), cudaMemcpyDeviceToDevice, sm));
    CK(cudaMemsetAsync(a.gMu.p, 0, sizeof(double) * std::max(nt, 1), sm));
    CK(cudaMemsetAsync(a.gLam.p, 0, sizeof(double) * std::max(nt, 1), sm));
    CK(cudaMemsetAsync(a.epsAcc.p, 0, sizeof(double) * N, sm));
    CK(cudaMemsetAsync(a.sigAcc.p, 0, sizeof(double) * N, sm));
    if (xbar_final)
        CK(cudaMemcpyAsync(a.xbar.p, xbar_final, N * sizeof(float2), cudaMemcpyHostToDevice, sm));
    else
        CK(cudaMemsetAsync(a.xbar.p, 0, N * sizeof(float2), sm));
    if (vbar_final)
        CK(cudaMemcpyAsync(a.vbar.p, vbar_final, N * sizeof(float2), cudaMemcpyHostToDevice, sm));
    else
        CK(cudaMemsetAsync(a.vbar.p, 0, N * sizeof(float2), sm));
    float2 *wc = a.w0.p, *wn = a.w1.p;
    {
        DevSys s = make_sys(ctx);
        Launch L;
        L.stream = sm;
        CK(enqueue_adj_seed(L, s, a.finalX.p, a.xbar.p, a.vbar.p, wc, (float)c_wall, (float)c_fea,
                            wall_y_host(ctx, a.endStep), a.sigAcc.p, a.gMu.p, a.gLam.p));
    }
    const float dt = ctx->dt, h = 0.5f * ctx->dt;
    std::vector<int> rebuilt;
    for (int g = nseg - 1; g >= 0; g--) {
        if ((st = adj_recompute(ctx, g, rebuilt))) return st;
        const int K = a.segLen[g], s0 = a.segStart[g];
        DevSys s = make_sys(ctx);
        Launch L;
        L.stream = sm;
        int listFrom = -1;
        for (int k = K; k >= (g == 0 ? 0 : 1); k--) {
            int r = 0;
            for (int v : rebuilt)
                if (v <= k) r = std::max(r, v);
            const float2 *pk = a.slots.p + (size_t)k * N;
            if (r != listFrom) {
                DevSys sb = s;
                sb.pos0 = const_cast<float2 *>(a.slots.p + (size_t)r * N);
                CK(enqueue_rebuild(L, sb, 0, 0));
                listFrom = r;
            }
            const int n = s0 + k;
            const int update = k >= 1;
            const float cNext = (n - 1 == a.segStart[0]) ? h : dt;
            CK(enqueue_adj_step(L, s, pk, wc, a.triD.p, a.gMu.p, a.gLam.p, a.xbar.p, a.vbar.p, wn, cNext, update,
                                wall_y_host(ctx, n), a.epsAcc.p, a.sigAcc.p));
            if (update) std::swap(wc, wn);
        }
    }
    // outputs
    if (xbar_init) CK(cudaMemcpyAsync(xbar_init, a.xbar.p, N * sizeof(float2), cudaMemcpyDeviceToHost, sm));
    if (vbar_init) CK(cudaMemcpyAsync(vbar_init, a.vbar.p, N * sizeof(float2), cudaMemcpyDeviceToHost, sm));
    std::vector<double> gm(std::max(nt, 1)), gl(std::max(nt, 1)), ea(N), sa(N);
    CK(cudaMemcpyAsync(gm.data(), a.gMu.p, gm.size() * sizeof(double), cudaMemcpyDeviceToHost, sm));
    CK(cudaMemcpyAsync(gl.data(), a.gLam.p, gl.size() * sizeof(double), cudaMemcpyDeviceToHost, sm));
    CK(cudaMemcpyAsync(ea.data(), a.epsAcc.p, N * sizeof(double), cudaMemcpyDeviceToHost, sm));
    CK(cudaMemcpyAsync(sa.data(), a.sigAcc.p, N * sizeof(double), cudaMemcpyDeviceToHost, sm));
    // restore the final state
    CK(cudaMemcpyAsync(ctx->dpos0.p, a.finalX.p, N * sizeof(float2), cudaMemcpyDeviceToDevice, sm));
    CK(cudaMemcpyAsync(ctx->dvel.p, a.finalV.p, N * sizeof(float2), cudaMemcpyDeviceToDevice, sm));
    CK(cudaMemcpyAsync(ctx->dacc.p, a.finalA.p, N * sizeof(float2), cudaMemcpyDeviceToDevice, sm));
    CK(cudaStreamSynchronize(sm));
    ctx->cur = 0;
    ctx->steps = a.endStep;
    ctx->listBuilt = false;
    ctx->forcesValid = false;
    ctx->staleMask |= kPos | kVel | kAcc | kForce;
    if (dJ_dlog_eps) {
        double t = 0.0;
        for (double v : ea) t += v;
        *dJ_dlog_eps = t;
    }
    if (dJ_dlog_sigma) {
        double t = 0.0;
        for (double v : sa) t += v;
        *dJ_dlog_sigma = t;
    }
    // per elastomer: chain mu = E / (2 (1 + nu)), lambda = E nu / ((1 + nu)(1 - 2 nu))
    for (size_t e = 0; e < ctx->clusters.size(); e++) {
        const bool own = e < ctx->elOwn.size() && ctx->elOwn[e];
        const double E = own ? ctx->elE[e] : ctx->E, nu = own ? ctx->elNu[e] : ctx->nu;
        const double dmu_dE = 1.0 / (2.0 * (1.0 + nu)), dmu_dnu = -E / (2.0 * (1.0 + nu) * (1.0 + nu));
        const double D = (1.0 + nu) * (1.0 - 2.0 * nu);
        const double dla_dE = nu / D, dla_dnu = E * (1.0 + 2.0 * nu * nu) / (D * D);
        double sm_ = 0.0, sl = 0.0;
        const Cluster &cl = ctx->clusters[e];
        for (int t = cl.tetOffset; t < cl.tetOffset + cl.nt && t < nt; t++) {
            sm_ += gm[t];
            sl += gl[t];
        }
        if (dJ_dE) dJ_dE[e] = sm_ * dmu_dE + sl * dla_dE;
        if (dJ_dnu) dJ_dnu[e] = sm_ * dmu_dnu + sl * dla_dnu;
    }
    return FEMMD_OK;
}

}  // extern "C"

// ================================================================== batches
//
// A batch advances many contexts (replicas) in one persistent launch
// (k_batch.cu).  Each replica keeps its own device state; the batch only
// holds their descriptors and the CTA assignment.

struct femmd_batch {
    int device = 0;
    std::string err;
    cudaStream_t stream = nullptr;
    std::vector<femmd_ctx *> reps;
    int threads = 512, ctasPerSm = 2;
    DBuf<DevSys> dreps;
    DBuf<int> order, queue, parity;
    cudaEvent_t ev[64] = {};
    GraphSet graph;
    int graphSteps = -1, graphThreads = 0, graphCtas = 0;
    const void *graphReps = nullptr;
    bool splitLarge = true;  // femmd_batch_set_split
    int graphVariant = -1, graphNbig = -1;
    size_t graphSmem = 0;
    int ctas = 0;
};

static femmd_status bfail(femmd_batch *b, femmd_status st, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (b) b->err = buf;
    return st;
}

#define BCK(call)                                                                                     \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return bfail(b, FEMMD_CUDA_ERROR, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                         __LINE__);                                                                   \
    } while (0)

// Upload descriptors, parities and the longest-processing-time assignment.
static femmd_status batch_prepare(femmd_batch *b, int steps, BatchLaunch &bl, std::vector<DevSys> &sys) {
    const int R = (int)b->reps.size();
    for (femmd_ctx *c : b->reps) {
        femmd_status st;
        if (c->device != b->device) return bfail(b, FEMMD_INVALID_ARG, "replicas must share the batch's device");
        if ((st = ensure_stream(c)) || (st = prepare(c)) || (st = ensure_obs(c, steps)))
            return bfail(b, st, "replica: %s", c->err.c_str());
        if (fast_mode(c))
            return bfail(b, FEMMD_UNSUPPORTED, "the batched kernel runs the reference-exact force mode");
        if (c->areaForces && !c->refVol.empty())
            return bfail(b, FEMMD_UNSUPPORTED, "the batched kernel does not implement the area springs");
        if (c->traj.on)
            return bfail(b, FEMMD_UNSUPPORTED, "the batched kernel does not write trajectory frames");
        if (c->propAvg)
            return bfail(b, FEMMD_UNSUPPORTED, "the batched kernel does not average properties");
        // the replica's own uploads must land before the batch stream reads them
        BCK(cudaStreamSynchronize(c->stream));
    }
    sys.resize(R);
    std::vector<int> par(R);
    for (int r = 0; r < R; r++) {
        sys[r] = make_sys(b->reps[r]);
        par[r] = b->reps[r]->cur;
    }
    const DevSys &a = sys[0];
    for (int r = 1; r < R; r++) {
        const DevSys &x = sys[r];
        if ((x.numTypes > 1) != (a.numTypes > 1) || x.sigmaByType != a.sigmaByType || x.wrapx != a.wrapx ||
            x.wrapy != a.wrapy || x.numTypes != a.numTypes)
            return bfail(b, FEMMD_INVALID_ARG,
                         "replica %d differs from replica 0 in type count, sigma mode or periodicity", r);
    }
    // 1/dr2 by reciprocal or by division gives the same bits: the reciprocal
    // form is used only when every replica has unit sigma
    bool sigmaOne = true;
    for (int r = 0; r < R; r++) sigmaOne = sigmaOne && sys[r].sigmaOne;
    int sms = 0;
    BCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device));
    const int ctas = std::max(1, std::min(R, b->ctasPerSm * sms));
    // heaviest replica first: the kernel hands them out in this order to
    // whichever CTA is free (greedy list scheduling)
    std::vector<int> idx(R);
    std::vector<double> cost(R);
    for (int r = 0; r < R; r++) {
        idx[r] = r;
        cost[r] = (double)sys[r].N + (double)sys[r].ntri;
    }
    std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return cost[x] > cost[y]; });
    // heaviest first; empty replicas only count steps
    std::vector<int> ord;
    for (int r : idx)
        if (sys[r].N > 0) ord.push_back(r);
    BCK(b->dreps.ensure(R));
    BCK(b->order.ensure(std::max<size_t>(ord.size(), 1)));
    if (!b->queue.p) {
        BCK(b->queue.ensure(3));
        BCK(cudaMemsetAsync(b->queue.p, 0, 3 * sizeof(int), b->stream));
    }
    BCK(b->parity.ensure(R));
    BCK(cudaMemcpyAsync(b->dreps.p, sys.data(), R * sizeof(DevSys), cudaMemcpyHostToDevice, b->stream));
    if (!ord.empty())
        BCK(cudaMemcpyAsync(b->order.p, ord.data(), ord.size() * sizeof(int), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMemcpyAsync(b->parity.p, par.data(), R * sizeof(int), cudaMemcpyHostToDevice, b->stream));
    b->ctas = ctas;
    bl.reps = b->dreps.p;
    bl.order = b->order.p;
    bl.queue = b->queue.p;
    bl.nwork = (int)ord.size();
    // replicas heavier than a CTA's average share run on CTA pairs (a
    // thread-block cluster of two), so that none sets the launch's length
    // alone; pairs need an even grid
    bl.nbig = 0;
    if (b->splitLarge && ctas % 2 == 0 && ctas >= 2) {
        double total = 0.0;
        for (int r : ord) total += cost[r];
        const double share = total / ctas;
        while (bl.nbig < (int)ord.size() && cost[ord[bl.nbig]] > share) bl.nbig++;
    }
    bl.minBlocks = b->ctasPerSm >= 2 && b->threads > 512 ? 2 : 1;
    bl.parity = b->parity.p;
    bl.steps = steps;
    bl.ctas = ctas;
    bl.threads = b->threads;
    bl.smem = sizeof(PairEntry) * (size_t)(a.numTypes > 1 ? a.numTypes * a.numTypes : 1);
    bl.multiType = a.numTypes > 1;
    bl.sigmaByType = a.sigmaByType;
    bl.sigmaOne = sigmaOne;
    bl.wrapx = a.wrapx;
    bl.wrapy = a.wrapy;
    bl.exact = a.imageExact;
    return FEMMD_OK;
}

static femmd_status batch_launch(femmd_batch *b, const BatchLaunch &bl) {
    const int variant = bl.multiType | bl.sigmaByType << 1 | bl.sigmaOne << 2 | bl.wrapx << 3 | bl.wrapy << 4;
    const bool rebuild = !b->graph.x || b->graphSteps != bl.steps || b->graphThreads != bl.threads ||
                         b->graphCtas != bl.ctas || b->graphReps != (const void *)bl.reps ||
                         b->graphVariant != variant || b->graphSmem != bl.smem || b->graphNbig != bl.nbig;
    if (rebuild) {
        b->graph.release();
        BCK(cudaGraphCreate(&b->graph.g, 0));
        Launch L;
        L.stream = b->stream;
        L.graph = b->graph.g;
        BCK(enqueue_batch(L, bl));
        BCK(cudaGraphInstantiate(&b->graph.x, b->graph.g, 0));
        b->graphSteps = bl.steps;
        b->graphThreads = bl.threads;
        b->graphCtas = bl.ctas;
        b->graphReps = bl.reps;
        b->graphVariant = variant;
        b->graphSmem = bl.smem;
        b->graphNbig = bl.nbig;
    }
    BCK(cudaMemsetAsync(bl.queue, 0, 3 * sizeof(int), b->stream));
    BCK(cudaGraphLaunch(b->graph.x, b->stream));
    return FEMMD_OK;
}

static femmd_status batch_checkpoint(femmd_batch *b, bool restore) {
    for (femmd_ctx *c : b->reps) {
        const size_t n = c->pos.size() * sizeof(float2);
        if (!n) continue;
        float2 *pd = c->cur ? c->dpos1.p : c->dpos0.p;
        if (!restore) {
            BCK(cudaMemcpyAsync(c->ckPos.p, pd, n, cudaMemcpyDeviceToDevice, b->stream));
            BCK(cudaMemcpyAsync(c->ckVel.p, c->dvel.p, n, cudaMemcpyDeviceToDevice, b->stream));
            BCK(cudaMemcpyAsync(c->ckAcc.p, c->dacc.p, n, cudaMemcpyDeviceToDevice, b->stream));
            BCK(cudaMemsetAsync(&c->sc.p->overflow, 0, 3 * sizeof(int), b->stream));
        } else {
            BCK(cudaMemcpyAsync(pd, c->ckPos.p, n, cudaMemcpyDeviceToDevice, b->stream));
            BCK(cudaMemcpyAsync(c->dvel.p, c->ckVel.p, n, cudaMemcpyDeviceToDevice, b->stream));
            BCK(cudaMemcpyAsync(c->dacc.p, c->ckAcc.p, n, cudaMemcpyDeviceToDevice, b->stream));
        }
    }
    return FEMMD_OK;
}

static femmd_status batch_read(femmd_batch *b) {
    for (femmd_ctx *c : b->reps)
        if (!c->pos.empty())
            BCK(cudaMemcpyAsync(c->hsc, c->sc.p, sizeof(DevScalars), cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    return FEMMD_OK;
}

extern "C" {

femmd_status femmd_batch_create(int device, femmd_batch **out) {
    if (!out) return FEMMD_INVALID_ARG;
    femmd_batch *b = new (std::nothrow) femmd_batch();
    if (!b) return FEMMD_CUDA_ERROR;
    b->device = device;
    *out = b;
    return FEMMD_OK;
}

void femmd_batch_destroy(femmd_batch *b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    b->graph.release();
    b->dreps.release();
    b->order.release();
    b->queue.release();
    b->parity.release();
    for (auto e : b->ev)
        if (e) cudaEventDestroy(e);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

const char *femmd_batch_last_error(const femmd_batch *b) { return b ? b->err.c_str() : "null batch"; }

femmd_status femmd_batch_add(femmd_batch *b, femmd_ctx *ctx, int *index) {
    if (!b || !ctx) return FEMMD_INVALID_ARG;
    b->err.clear();
    for (femmd_ctx *c : b->reps)
        if (c == ctx) return bfail(b, FEMMD_INVALID_ARG, "context already in the batch");
    if (!ctx->nnInit) return bfail(b, FEMMD_NOT_READY, "add a replica after its init_neighbor_list()");
    b->reps.push_back(ctx);
    if (index) *index = (int)b->reps.size() - 1;
    return FEMMD_OK;
}

int femmd_batch_size(const femmd_batch *b) { return b ? (int)b->reps.size() : 0; }

femmd_status femmd_batch_set_launch(femmd_batch *b, int threads, int ctas_per_sm) {
    if (!b) return FEMMD_INVALID_ARG;
    if (threads < 32 || threads > 1024 || threads % 32 || ctas_per_sm < 1 || ctas_per_sm > 32)
        return bfail(b, FEMMD_INVALID_ARG, "threads must be a multiple of 32 in [32, 1024], CTAs per SM in [1, 32]");
    b->threads = threads;
    b->ctasPerSm = ctas_per_sm;
    return FEMMD_OK;
}

femmd_status femmd_batch_set_split(femmd_batch *b, int on) {
    if (!b) return FEMMD_INVALID_ARG;
    b->splitLarge = on != 0;
    return FEMMD_OK;
}

femmd_status femmd_batch_get_launch(const femmd_batch *b, int *threads, int *ctas_per_sm, int *ctas) {
    if (!b) return FEMMD_INVALID_ARG;
    if (threads) *threads = b->threads;
    if (ctas_per_sm) *ctas_per_sm = b->ctasPerSm;
    if (ctas) *ctas = b->ctas;
    return FEMMD_OK;
}

femmd_status femmd_batch_run(femmd_batch *b, int steps) {
    if (!b) return FEMMD_INVALID_ARG;
    b->err.clear();
    if (steps < 0) return bfail(b, FEMMD_INVALID_ARG, "steps must be >= 0");
    if (b->reps.empty()) return FEMMD_OK;
    if (!b->stream) {
        BCK(cudaSetDevice(b->device));
        BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    }
    femmd_status st;
    for (int attempt = 0; attempt < 8; attempt++) {
        BatchLaunch bl;
        std::vector<DevSys> sys;
        if ((st = batch_prepare(b, steps, bl, sys))) return st;
        if ((st = batch_checkpoint(b, false))) return st;
        if ((st = batch_launch(b, bl))) return st;
        if ((st = batch_read(b))) return st;
        bool over = false;
        for (femmd_ctx *c : b->reps) {
            if (c->pos.empty()) continue;
            if (c->hsc->overflow & 2) return bfail(b, FEMMD_CAPACITY_OVERFLOW, "inconsistent cell counts");
            over = over || c->hsc->overflow;
        }
        if (!over) {
            int bad = -1;
            for (size_t r = 0; r < b->reps.size(); r++) {
                femmd_ctx *c = b->reps[r];
                c->steps += steps;
                if (c->pos.empty()) continue;
                if (steps % 2) c->cur ^= 1;
                c->staleMask |= kPos | kVel | kAcc | kForce;
                c->forcesValid = true;
                c->listBuilt = true;
                c->obsRows = std::min(c->hsc->obsRow, c->obsCap);
                c->totalBuilds = (long long)c->hsc->builds;
                if (c->hsc->nonfinite && bad < 0) bad = (int)r;
            }
            if (bad >= 0) return bfail(b, FEMMD_NONFINITE, "replica %d: a force became NaN or infinite", bad);
            return FEMMD_OK;
        }
        // roll every replica back, grow the lists that overflowed, repeat
        if ((st = batch_checkpoint(b, true))) return st;
        BCK(cudaStreamSynchronize(b->stream));
        for (femmd_ctx *c : b->reps)
            if (!c->pos.empty() && c->hsc->overflow) {
                int need = std::max(c->hsc->maxCount, c->nbrCap + c->nbrCap / 2);
                if ((st = alloc_list(c, need + need / 4 + 8))) return bfail(b, st, "%s", c->err.c_str());
            }
    }
    return bfail(b, FEMMD_CAPACITY_OVERFLOW, "neighbour lists kept overflowing");
}

femmd_status femmd_batch_event_record(femmd_batch *b, int slot) {
    if (!b || slot < 0 || slot >= 64) return FEMMD_INVALID_ARG;
    if (!b->stream) {
        BCK(cudaSetDevice(b->device));
        BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    }
    if (!b->ev[slot]) BCK(cudaEventCreate(&b->ev[slot]));
    BCK(cudaEventRecord(b->ev[slot], b->stream));
    return FEMMD_OK;
}

femmd_status femmd_batch_event_elapsed(femmd_batch *b, int a, int c, float *ms) {
    if (!b || !ms || a < 0 || a >= 64 || c < 0 || c >= 64 || !b->ev[a] || !b->ev[c]) return FEMMD_INVALID_ARG;
    BCK(cudaEventSynchronize(b->ev[c]));
    BCK(cudaEventElapsedTime(ms, b->ev[a], b->ev[c]));
    return FEMMD_OK;
}

// Time each launch shape on the current states (restored after every trial)
// and keep the fastest.
femmd_status femmd_batch_autotune(femmd_batch *b, int trial_steps, int *threads_out, int *ctas_per_sm_out,
                                  double *best_ms) {
    if (!b) return FEMMD_INVALID_ARG;
    b->err.clear();
    if (b->reps.empty()) return bfail(b, FEMMD_NOT_READY, "empty batch");
    if (trial_steps < 1) trial_steps = 10;
    if (!b->stream) {
        BCK(cudaSetDevice(b->device));
        BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    }
    static const int cand[][2] = {{128, 8}, {256, 4}, {256, 8}, {512, 2}, {512, 4}, {1024, 1}, {1024, 2}};
    const int t0 = b->threads, c0 = b->ctasPerSm;
    {
        BatchLaunch bl;
        std::vector<DevSys> sys;
        femmd_status st;
        if ((st = batch_prepare(b, trial_steps, bl, sys))) return st;
    }
    if (femmd_status st = batch_read(b)) return st;
    std::vector<unsigned long long> builds0;
    for (femmd_ctx *c : b->reps) builds0.push_back(c->pos.empty() ? 0ull : c->hsc->builds);
    double best = 1e300;
    int bt = t0, bc = c0;
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0));
    BCK(cudaEventCreate(&e1));
    for (const auto &cd : cand) {
        b->threads = cd[0];
        b->ctasPerSm = cd[1];
        BatchLaunch bl;
        std::vector<DevSys> sys;
        femmd_status st;
        if ((st = batch_prepare(b, trial_steps, bl, sys))) return st;
        if ((st = batch_checkpoint(b, false))) return st;
        BCK(cudaMemsetAsync(bl.queue, 0, 2 * sizeof(int), b->stream));
        BCK(cudaEventRecord(e0, b->stream));
        cudaError_t le = cudaSuccess;
        {
            Launch L;
            L.stream = b->stream;
            le = enqueue_batch(L, bl);
        }
        BCK(cudaEventRecord(e1, b->stream));
        cudaError_t se = cudaStreamSynchronize(b->stream);
        if (le == cudaSuccess && se == cudaSuccess) {
            float ms = 0;
            BCK(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best) {
                best = ms;
                bt = cd[0];
                bc = cd[1];
            }
        } else {
            cudaGetLastError();  // a shape the device cannot run: skip it
        }
        if ((st = batch_checkpoint(b, true))) return st;
        for (size_t r = 0; r < b->reps.size(); r++)
            if (!b->reps[r]->pos.empty())
                BCK(cudaMemcpyAsync(&b->reps[r]->sc.p->builds, &builds0[r], sizeof(unsigned long long),
                                cudaMemcpyHostToDevice, b->stream));
        BCK(cudaStreamSynchronize(b->stream));
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->threads = bt;
    b->ctasPerSm = bc;
    if (threads_out) *threads_out = bt;
    if (ctas_per_sm_out) *ctas_per_sm_out = bc;
    if (best_ms) *best_ms = best;
    return FEMMD_OK;
}


// Rebuild cadence and cell size: time run(trial_steps) of the whole batch for
// every (skin, cell factor) pair on the current states (restored after each
// trial), then keep the fastest pair on every replica.  Opt-in: both change
// the lists' order and rebuild steps, so the trajectories no longer round as
// the reference's do.
femmd_status femmd_batch_autotune_lists(femmd_batch *b, int trial_steps, const double *skins, int nskins,
                                        const double *factors, int nfactors, double *best_skin,
                                        double *best_factor, double *best_ms) {
    if (!b || !skins || nskins < 1 || !factors || nfactors < 1) return FEMMD_INVALID_ARG;
    b->err.clear();
    if (b->reps.empty()) return bfail(b, FEMMD_NOT_READY, "empty batch");
    if (trial_steps < 1) trial_steps = 20;
    if (!b->stream) {
        BCK(cudaSetDevice(b->device));
        BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    }
    auto apply = [&](double skin, double f) -> femmd_status {
        for (femmd_ctx *c : b->reps) {
            femmd_status st;
            if ((st = femmd_set_skin(c, skin)) || (st = femmd_set_cell_factor(c, f)) ||
                (st = femmd_init_neighbor_list(c)))
                return bfail(b, st, "replica: %s", c->err.c_str());
        }
        return FEMMD_OK;
    };
    std::vector<float> skin0, fac0;
    for (femmd_ctx *c : b->reps) {
        skin0.push_back(c->skin);
        fac0.push_back(c->cellFactor);
    }
    double best = 1e300, bs = skin0[0], bf = fac0[0];
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0));
    BCK(cudaEventCreate(&e1));
    for (int i = 0; i < nskins; i++)
        for (int j = 0; j < nfactors; j++) {
            femmd_status st;
            if ((st = apply(skins[i], factors[j]))) return st;
            BatchLaunch bl;
            std::vector<DevSys> sys;
            if ((st = batch_prepare(b, trial_steps, bl, sys))) return st;
            if ((st = batch_checkpoint(b, false))) return st;
            BCK(cudaMemsetAsync(bl.queue, 0, 2 * sizeof(int), b->stream));
            BCK(cudaEventRecord(e0, b->stream));
            {
                Launch L;
                L.stream = b->stream;
                BCK(enqueue_batch(L, bl));
            }
            BCK(cudaEventRecord(e1, b->stream));
            BCK(cudaStreamSynchronize(b->stream));
            float ms = 0;
            BCK(cudaEventElapsedTime(&ms, e0, e1));
            if ((st = batch_read(b))) return st;
            bool over = false;
            for (femmd_ctx *c : b->reps) over = over || (!c->pos.empty() && c->hsc->overflow);
            if (!over && ms < best) {  // a trial whose lists overflowed is not a fair time
                best = ms;
                bs = skins[i];
                bf = factors[j];
            }
            if ((st = batch_checkpoint(b, true))) return st;
            BCK(cudaStreamSynchronize(b->stream));
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (femmd_status st = apply(bs, bf)) return st;
    if (best_skin) *best_skin = bs;
    if (best_factor) *best_factor = bf;
    if (best_ms) *best_ms = best;
    return FEMMD_OK;
}

}  // extern "C"
