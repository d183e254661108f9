// k_props.cu -- the observables of Properties::evaluate
// (femmd2D/src/properties.cpp:15-36) at the current state, with the cluster
// quantities of FeaElements::unfoldPos (feaElements.cpp:86-150) and the
// cluster virial of calcPairForcesNN (interactions.cpp:347-389).  Per-cluster,
// per-triangle and per-particle terms are formed in FP64 and written to
// arrays that the host sums in a fixed order.
#include <cuda_runtime.h>
#include "femmd_internal.h"
#include "launch.h"
#include "device_common.cuh"
#include "step_body.cuh"

namespace femmd {

namespace {

__device__ __forceinline__ double block_sum_d(double v, double *scr) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) scr[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) t = warp_sum(lane < nw ? scr[lane] : 0.0);
    __syncthreads();
    if (threadIdx.x == 0) scr[0] = t;
    __syncthreads();
    return scr[0];
}

// three block sums in one pass (a fixed tree); valid in thread 0
__device__ __forceinline__ void block_sum3_d(double *v, double *scr) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < 3; k++) v[k] = warp_sum(v[k]);
    __syncthreads();
    if (lane == 0)
        for (int k = 0; k < 3; k++) scr[3 * warp + k] = v[k];
    __syncthreads();
    if (threadIdx.x < 32)
        for (int k = 0; k < 3; k++) v[k] = warp_sum(lane < nw ? scr[3 * lane + k] : 0.0);
}

// sum over the warp, the same value in every lane (butterfly: a fixed order)
__device__ __forceinline__ double warp_sum_all(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace

// One warp per cluster (elastomer): unfold across the periodic boundary the
// reference's way (a cluster wider than half the box has its vertices beyond
// L/2 moved down by L, and all moved up by L again when their mean is
// negative), then the mass-weighted centre of mass and velocity and the
// cluster kinetic term M |v_cm|^2.  Warp reductions only: min/max exact,
// sums in FP64 in a fixed lane order.
constexpr int kClusterWarps = 4;

__global__ void __launch_bounds__(32 * kClusterWarps) k_props_cluster(DevSys s, const float2 *pos, int ncl,
                                                                      const int2 *clRange, const float *clMass,
                                                                      double2 *unf, double2 *cmPos, double2 *cmVel,
                                                                      double *clKin) {
    const int c = blockIdx.x * kClusterWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (c >= ncl) return;  // whole warps
    const int off = clRange[c].x, n = clRange[c].y;
    float xmin = 3.0e38f, ymin = 3.0e38f, xmax = -3.0e38f, ymax = -3.0e38f;
    for (int k = lane; k < n; k += 32) {
        const float2 p = pos[off + k];
        xmin = fminf(xmin, p.x);
        ymin = fminf(ymin, p.y);
        xmax = fmaxf(xmax, p.x);
        ymax = fmaxf(ymax, p.y);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        xmin = fminf(xmin, __shfl_xor_sync(0xffffffffu, xmin, o));
        ymin = fminf(ymin, __shfl_xor_sync(0xffffffffu, ymin, o));
        xmax = fmaxf(xmax, __shfl_xor_sync(0xffffffffu, xmax, o));
        ymax = fmaxf(ymax, __shfl_xor_sync(0xffffffffu, ymax, o));
    }
    const bool ux = xmax - xmin > s.Lx / 2.0f;  // whatever the periodicity, as the reference
    const bool uy = ymax - ymin > s.Ly / 2.0f;
    double sx = 0.0, sy = 0.0;
    if (ux || uy) {
        for (int k = lane; k < n; k += 32) {
            const float2 p = pos[off + k];
            double x = p.x, y = p.y;
            if (ux && p.x > s.Lx / 2.0f) x -= s.Lx;
            if (uy && p.y > s.Ly / 2.0f) y -= s.Ly;
            sx += x;
            sy += y;
        }
        sx = warp_sum_all(sx);
        sy = warp_sum_all(sy);
    }
    const bool upx = ux && sx / n < 0.0, upy = uy && sy / n < 0.0;
    double mx = 0.0, my = 0.0, mvx = 0.0, mvy = 0.0;
    for (int k = lane; k < n; k += 32) {
        const int i = off + k;
        const float2 p = pos[i], v = s.vel[i];
        double x = p.x, y = p.y;
        if (ux && p.x > s.Lx / 2.0f) x -= s.Lx;
        if (uy && p.y > s.Ly / 2.0f) y -= s.Ly;
        if (upx) x += s.Lx;
        if (upy) y += s.Ly;
        unf[i] = make_double2(x, y);
        const double m = s.mass[i];
        mx += m * x;
        my += m * y;
        mvx += m * v.x;
        mvy += m * v.y;
    }
    mx = warp_sum_all(mx);
    my = warp_sum_all(my);
    mvx = warp_sum_all(mvx);
    mvy = warp_sum_all(mvy);
    if (lane == 0) {
        const double M = clMass[c];
        cmPos[c] = make_double2(mx / M, my / M);
        const double vx = mvx / M, vy = mvy / M;
        cmVel[c] = make_double2(vx, vy);
        clKin[c] = M * (vx * vx + vy * vy);
    }
}

// FeaElements::updateClustersCentroid (feaElements.cpp:162-197): the
// centroid of a cluster in a periodic box from the mean of (cos, sin) of
// 2 pi x / L per axis, x_c = L (atan2(-<sin>, -<cos>) + pi) / (2 pi).  In
// FP64.  The reference averages the x sums again for y (feaElements.cpp:
// 192-193); here each axis uses its own sums.
__global__ void k_cluster_centroid(DevSys s, const float2 *pos, const int2 *clRange, double2 *centroid) {
    __shared__ double dscr[32];
    const int c = blockIdx.x;
    const int off = clRange[c].x, n = clRange[c].y;
    double cx = 0.0, sx = 0.0, cy = 0.0, sy = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const float2 p = pos[off + k];
        double sn, cs;
        sincospi(2.0 * (double)p.x / (double)s.Lx, &sn, &cs);
        cx += cs;
        sx += sn;
        sincospi(2.0 * (double)p.y / (double)s.Ly, &sn, &cs);
        cy += cs;
        sy += sn;
    }
    cx = block_sum_d(cx, dscr);
    sx = block_sum_d(sx, dscr);
    cy = block_sum_d(cy, dscr);
    sy = block_sum_d(sy, dscr);
    if (threadIdx.x == 0) {
        const double pi = 3.14159265358979323846;
        const double tx = atan2(-sx / n, -cx / n) + pi, ty = atan2(-sy / n, -cy / n) + pi;
        centroid[c] = make_double2((double)s.Lx * tx / (2.0 * pi), (double)s.Ly * ty / (2.0 * pi));
    }
}

cudaError_t enqueue_cluster_centroid(Launch &L, const DevSys &s, const float2 *pos, int ncl, const int2 *clRange,
                                     double2 *centroid) {
    if (ncl <= 0) return cudaSuccess;
    return L.kernel(k_cluster_centroid, dim3(ncl), dim3(128), 0, s, pos, clRange, centroid);
}

// feaVirial terms: per triangle sum over its vertices of f . unfolded position
// (interactions.cpp:681), with the nodal forces of the last force evaluation.
__global__ void __launch_bounds__(kBlock) k_props_tri(DevSys s, const double2 *unf, double *feaVir) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= s.ntri) return;
    const int4 q = __ldg(s.triIdx + t);
    const int v[3] = {q.x, q.y, q.z};
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float2 f = s.triF[3 * t + k];
        const double2 u = unf[v[k]];
        acc += (double)f.x * u.x + (double)f.y * u.y;
    }
    feaVir[t] = acc;
}

// Per particle of [0, n): m v^2 and the cluster virial 1/2 f_ij . (R_ci -
// R_cj) (nearest image) over its Verlet list, for pairs of two cluster
// particles.
template <bool WX, bool WY>
__global__ void __launch_bounds__(kStepBlock) k_props_particle(DevSys s, const float2 *pos, int n, const int *clusterOf,
                                                              const double2 *cmPos, double *kin, double *clVir) {
    extern __shared__ PairEntry tab[];
    const int nt2 = s.numTypes > 1 ? s.numTypes * s.numTypes : 1;
    for (int k = threadIdx.x; k < nt2; k += blockDim.x) tab[k] = s.pair[k];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 vi = s.vel[i];
    kin[i] = (double)s.mass[i] * ((double)vi.x * vi.x + (double)vi.y * vi.y);
    double cv = 0.0;
    const int ci = clusterOf ? clusterOf[i] : -1;
    if (ci >= 0) {
        const float2 pi = pos[i];
        const int cnt = min(s.nbrCount[i], s.nbrCap);
        const int ti = s.numTypes > 1 ? s.typeId[i] : 0;
        const float si = s.sigmaByType ? 0.0f : s.sigma[i];
        const double2 Ri = cmPos[ci];
        for (int k = 0; k < cnt; k++) {
            const int tag = s.nbr[nbr_at(k, i, s.Ncap)];
            const int j = tag & kIdMask;
            const int cj = clusterOf[j];
            if (cj < 0) continue;
            const float2 pj = pos[j];
            float dxr, dyr;
            bool wrapped = false;
            float dx = img<WX>(pi.x, pj.x, s.Lx, s.imageExact, dxr, wrapped);
            float dy = img<WY>(pi.y, pj.y, s.Ly, s.imageExact, dyr, wrapped);
            float dr2r = dxr * dxr + dyr * dyr;
            const PairEntry &pe = tab[s.numTypes > 1 ? ti * s.numTypes + ((unsigned)tag >> kIdBits) : 0];
            float rcut2, sig2, c;
            if (!s.sigmaByType) {
                float sij = (si + s.sigma[j]) / 2.0f;
                rcut2 = pe.rc * pe.rc * sij * sij;
                sig2 = sij * sij;
                c = pe.eps48 / sig2;
            } else {
                rcut2 = pe.rcut2;
                sig2 = pe.sig2;
                c = pe.c;
            }
            if (!(dr2r < rcut2)) continue;
            float dr2 = wrapped ? dx * dx + dy * dy : dr2r;
            float s2 = sig2 / dr2, s6 = s2 * s2 * s2;
            float fc = c * s6 * (s6 - 0.5f) * s2;
            const double2 Rj = cmPos[cj];
            double rx = Ri.x - Rj.x, ry = Ri.y - Rj.y;
            if (s.wrapx) {
                if (rx >= 0.5 * s.Lx) rx -= s.Lx;
                else if (rx < -0.5 * s.Lx) rx += s.Lx;
            }
            if (s.wrapy) {
                if (ry >= 0.5 * s.Ly) ry -= s.Ly;
                else if (ry < -0.5 * s.Ly) ry += s.Ly;
            }
            cv += 0.5 * ((double)(fc * dx) * rx + (double)(fc * dy) * ry);
        }
    }
    clVir[i] = cv;
}

// Properties::compute (properties.cpp:85-95) after a step: block b sums a
// fixed slice of the cluster-virial, feaVirial and cluster-kinetic terms;
// the grid's last block adds the slices in block order (the same result on
// every run), forms Properties::evaluate (properties.cpp:15-36) with the
// step's U, W and sum m v^2, then Properties::accumulate(1)
// (properties.cpp:56-70) and, at steps past stepEqui that are multiples of
// stepAvg, accumulate(2) and accumulate(0): the window's average and
// standard deviation, sqrt(max(sum2/n - avg^2, 0)) (properties.h:11), and a
// new window.
__global__ void __launch_bounds__(kBlock) k_props_accum(DevSys s, DevProps *P, double *part, const double *clKin,
                                                        int ncl, const double *feaVir, int ntri, const double *clVir,
                                                        int nvir, int stepAvg, int stepEqui) {
    __shared__ double dscr[3 * 32];
    __shared__ bool last;
    const int nb = gridDim.x, b = blockIdx.x;
    const int n3[3] = {nvir, feaVir ? ntri : 0, clKin ? ncl : 0};
    const double *arr[3] = {clVir, feaVir, clKin};
    double sums[3];
    for (int k = 0; k < 3; k++) {
        const int per = (n3[k] + nb - 1) / nb, lo = min(n3[k], b * per), hi = min(n3[k], lo + per);
        // four independent sums per thread (the loads overlap), then added
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
        const int st = blockDim.x;
        int i = lo + threadIdx.x;
        for (; i + 3 * st < hi; i += 4 * st) {
            a0 += arr[k][i];
            a1 += arr[k][i + st];
            a2 += arr[k][i + 2 * st];
            a3 += arr[k][i + 3 * st];
        }
        for (; i < hi; i += st) a0 += arr[k][i];
        sums[k] = (a0 + a1) + (a2 + a3);
    }
    block_sum3_d(sums, dscr);
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; k++) part[3 * b + k] = sums[k];
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(&P->ticket, 1u) == (unsigned)nb - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // the slices' sums: a fixed share per thread, then the block's fixed tree
    double pv[3] = {0.0, 0.0, 0.0};
    for (int q = threadIdx.x; q < nb; q += blockDim.x)
        for (int k = 0; k < 3; k++) pv[k] += part[3 * q + k];
    __syncthreads();  // dscr was used by this block's own slice sums
    block_sum3_d(pv, dscr);
    if (threadIdx.x != 0) return;
    const double cv = pv[0], fv = pv[1], ck = pv[2];
    const DevScalars *sc = s.sc;
    const double N = (double)s.N, V = (double)s.Lx * (double)s.Ly, KE = sc->KE, W = sc->W;
    double v[kNumProps];
    v[0] = 0.5 * KE / N;
    v[1] = sc->U / N;
    v[2] = v[0] + v[1];
    v[3] = v[0];
    v[4] = W;
    v[5] = fv;
    v[6] = 0.5 * KE / V + 0.5 * (W + fv) / V;
    v[7] = ncl > 0 ? 0.5 * ck / ncl : 0.0;
    v[8] = cv;
    v[9] = 0.5 * ck / V - 0.5 * cv / V;
    P->count += 1;
    for (int k = 0; k < kNumProps; k++) {
        P->val[k] = v[k];
        P->sum[k] += v[k];
        P->sum2[k] += v[k] * v[k];
    }
    const int step = sc->stepNow;
    if (step > stepEqui && stepAvg > 0 && step % stepAvg == 0) {
        const double n = (double)P->count;
        for (int k = 0; k < kNumProps; k++) {
            const double a = P->sum[k] / n;
            P->avg[k] = a;
            P->stdv[k] = sqrt(fmax(P->sum2[k] / n - a * a, 0.0));
            P->sum[k] = 0.0;
            P->sum2[k] = 0.0;
        }
        P->count = 0;
        P->windows += 1;
        P->lastStep = step;
    }
    P->ticket = 0;
}

cudaError_t enqueue_props_accum(Launch &L, const DevSys &s, DevProps *P, double *partials, int blocks,
                                const double *clKin, int ncl, const double *feaVir, int ntri, const double *clVir,
                                int nvir, int stepAvg, int stepEqui) {
    return L.kernel(k_props_accum, dim3(blocks), dim3(kBlock), 0, s, P, partials, clKin, ncl, feaVir, ntri, clVir,
                    nvir, stepAvg, stepEqui);
}

cudaError_t enqueue_props(Launch &L, const DevSys &s, const float2 *pos, int ncl, const int2 *clRange,
                          const float *clMass, const int *clusterOf, double2 *unf, double2 *cmPos, double2 *cmVel,
                          double *clKin, double *feaVir, double *kin, double *clVir, int npart) {
    cudaError_t e;
    if (ncl > 0) {
        if ((e = L.kernel(k_props_cluster, dim3((ncl + kClusterWarps - 1) / kClusterWarps), dim3(32 * kClusterWarps), 0,
                          s, pos, ncl, clRange, clMass, unf, cmPos, cmVel, clKin)))
            return e;
        if (s.ntri > 0 && s.feaForces) {
            if ((e = L.kernel(k_props_tri, dim3(tri_blocks(s.ntri)), dim3(kBlock), 0, s, (const double2 *)unf, feaVir)))
                return e;
        }
    }
    dim3 g(step_blocks(npart)), b(kStepBlock);
    size_t smt = sizeof(PairEntry) * (size_t)(s.numTypes > 1 ? s.numTypes * s.numTypes : 1);
    const int *co = ncl > 0 ? clusterOf : nullptr;
    if (s.wrapx && s.wrapy)
        return L.kernel(k_props_particle<true, true>, g, b, smt, s, pos, npart, co, (const double2 *)cmPos, kin, clVir);
    if (s.wrapx)
        return L.kernel(k_props_particle<true, false>, g, b, smt, s, pos, npart, co, (const double2 *)cmPos, kin, clVir);
    return L.kernel(k_props_particle<false, false>, g, b, smt, s, pos, npart, co, (const double2 *)cmPos, kin, clVir);
}

}  // namespace femmd
