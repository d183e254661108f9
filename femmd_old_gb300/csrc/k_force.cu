// k_force.cu -- forces and leapfrog integration of the femmd2D timestep.
//
// Reference path: Interactions::calcForces (femmd2D/src/interactions.cpp:83-109)
// = calcBondForcesCPU (:143-173), calcFeaForcesCPU2 (neo-Hookean, :532-689) or
// computeFeaForcesGPU (Green strain / linear C, interactionsCuda.cu:312-451),
// calcPairForcesNN with pairForce/ljforce (interactions.cpp:347-389,
// interactionsCuda.cu:43-100); and the leapfrog of Integrator::doStep
// (integrator.cpp:8-29, 100-135) with evalProps (md3dsystem.cpp:151-179).
//
// Per step:
//   k_tri_forces  thread per triangle: nodal forces of the triangle written to
//                 triF[3t+slot] (no atomics), energy reduced in FP64.
//   k_step        thread per particle: gathers bond incidences (bond order),
//                 triangle incidences (triangle order) and the Verlet list
//                 (list order) -- the order in which the reference's CPU path
//                 adds into force[i] -- then a = f/m and the leapfrog, fused:
//                 kick to v(t) and, unless it is the last step of a run, the
//                 next half kick and the drift into the other position buffer.
//                 FP32 per-particle sums, FP64 warp/block/grid reductions of
//                 U, W and sum m v^2 finished by the last block in fixed order
//                 (deterministic), which also updates dispHi and raises the
//                 rebuild flag / graph condition for the next step.
#include <cuda_runtime.h>
#include "femmd_internal.h"
#include "launch.h"
#include "device_common.cuh"

namespace femmd {

int force_blocks(int N) { return (N + kBlock - 1) / kBlock; }
int step_blocks(int N) { return (N + kStepBlock - 1) / kStepBlock; }
int tri_blocks(int ntri) { return (ntri + kBlock - 1) / kBlock; }

// ------------------------------------------------------------ triangles

// calcFeaForcesCPU2 (interactions.cpp:532-689) with Bm and vol0 precomputed
// from the reference positions by the same float operations.
__device__ __forceinline__ float tri_neo_hookean(const DevSys &s, const float2 *pos, int t, float2 &f0, float2 &f1,
                                                 float2 &f2) {
    int4 q = __ldg(s.triIdx + t);
    float2 r0 = pos[q.x], r1 = pos[q.y], r2 = pos[q.z];
    float4 bm = __ldg(s.triGeo + 2 * t);
    float vol0 = __ldg(s.triGeo + 2 * t + 1).x;
    const float L = s.Lx, Ly = s.Ly;
    float dx01 = r0.x - r1.x, dx02 = r0.x - r2.x, dy01 = r0.y - r1.y, dy02 = r0.y - r2.y;
    int k1x = (dx01 > L / 2.0f) - (dx01 < -L / 2.0f);
    int k2x = (dx02 > L / 2.0f) - (dx02 < -L / 2.0f);
    int k1y = (dy01 > Ly / 2.0f) - (dy01 < -Ly / 2.0f);
    int k2y = (dy02 > Ly / 2.0f) - (dy02 < -Ly / 2.0f);
    float Ds00, Ds10, Ds01, Ds11;
    if (s.imageExact) {
        Ds00 = diff_shift(r0.x, r2.x, -k2x, L);
        Ds10 = diff_shift(r0.y, r2.y, -k2y, Ly);
        Ds01 = diff_shift(r1.x, r2.x, k1x - k2x, L);
        Ds11 = diff_shift(r1.y, r2.y, k1y - k2y, Ly);
    } else {
        float r1x = r1.x, r2x = r2.x, r1y = r1.y, r2y = r2.y;
        if (k1x > 0) r1x += L;
        if (k1x < 0) r1x -= L;
        if (k2x > 0) r2x += L;
        if (k2x < 0) r2x -= L;
        if (k1y > 0) r1y += Ly;
        if (k1y < 0) r1y -= Ly;
        if (k2y > 0) r2y += Ly;
        if (k2y < 0) r2y -= Ly;
        Ds00 = r0.x - r2x;
        Ds10 = r0.y - r2y;
        Ds01 = r1x - r2x;
        Ds11 = r1y - r2y;
    }
    const float Bm00 = bm.x, Bm10 = bm.y, Bm01 = bm.z, Bm11 = bm.w;
    float F00 = Ds00 * Bm00 + Ds01 * Bm10;
    float F10 = Ds10 * Bm00 + Ds11 * Bm10;
    float F01 = Ds00 * Bm01 + Ds01 * Bm11;
    float F11 = Ds10 * Bm01 + Ds11 * Bm11;
    float detF = F00 * F11 - F01 * F10;
    float logJ = own_logf(detF);
    float llogJ = s.lambda * logJ;
    float iF00 = F11 / detF, iF10 = -F10 / detF, iF01 = -F01 / detF, iF11 = F00 / detF;
    const float mu = s.mu;
    float P00 = mu * (F00 - iF00) + llogJ * iF00;
    float P10 = mu * (F10 - iF01) + llogJ * iF01;
    float P01 = mu * (F01 - iF10) + llogJ * iF10;
    float P11 = mu * (F11 - iF11) + llogJ * iF11;
    float nv0 = -vol0;
    float H00 = nv0 * (P00 * Bm00 + P01 * Bm01);
    float H10 = nv0 * (P10 * Bm00 + P11 * Bm01);
    float H01 = nv0 * (P00 * Bm10 + P01 * Bm11);
    float H11 = nv0 * (P10 * Bm10 + P11 * Bm11);
    f0 = make_float2(H00, H10);
    f1 = make_float2(H01, H11);
    f2 = make_float2(-H00 - H01, -H10 - H11);
    // energy A0 [mu/2 (I1-2) - mu lnJ + lambda/2 ln^2 J], deviation form:
    // I1 - 2 - 2 lnJ summed from (F-I) entries to avoid first-order cancellation
    float d00 = F00 - 1.0f, d11 = F11 - 1.0f;
    float i1m2 = (2.0f * d00 + d00 * d00) + (2.0f * d11 + d11 * d11) + F01 * F01 + F10 * F10;
    float pe = 0.5f * mu * (i1m2 - 2.0f * logJ) + 0.5f * s.lambda * logJ * logJ;
    return pe * vol0;
}

// computeFeaForcesGPU (interactionsCuda.cu:312-451): Green strain, linear C,
// float arithmetic of the reference kernel; xm rows 1-2 and |area|
// precomputed from the reference positions.
__device__ __forceinline__ float tri_green(const DevSys &s, const float2 *pos, int t, float2 *f) {
    int4 q = __ldg(s.triIdx + t);
    int p[3] = {q.x, q.y, q.z};
    float rx[3], ry[3], X[3], Y[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float2 r = pos[p[i]];
        float2 R = __ldg(s.refPos + p[i]);
        rx[i] = r.x;
        ry[i] = r.y;
        X[i] = R.x;
        Y[i] = R.y;
    }
    const float L = s.Lx, Ly = s.Ly;
    float dx01 = rx[0] - rx[1];
    if (dx01 > L / 2.0f) rx[1] += L;
    if (dx01 < -L / 2.0f) rx[1] -= L;
    float dx02 = rx[0] - rx[2];
    if (dx02 > L / 2.0f) rx[2] += L;
    if (dx02 < -L / 2.0f) rx[2] -= L;
    float dy01 = ry[0] - ry[1];
    if (dy01 > Ly / 2.0f) ry[1] += Ly;
    if (dy01 < -Ly / 2.0f) ry[1] -= Ly;
    float dy02 = ry[0] - ry[2];
    if (dy02 > Ly / 2.0f) ry[2] += Ly;
    if (dy02 < -Ly / 2.0f) ry[2] -= Ly;
    float4 g0 = __ldg(s.triGeo + 2 * t), g1 = __ldg(s.triGeo + 2 * t + 1);
    float m1[3] = {g0.x, g0.y, g0.z};  // xm row 1
    float m2[3] = {g0.w, g1.x, g1.y};  // xm row 2
    float tetVol = g1.z;
    float a1 = 0.0f, a2 = 0.0f, b1 = 0.0f, b2 = 0.0f;
#pragma unroll
    for (int j = 0; j < 3; j++) {
        float ux = rx[j] - X[j], uy = ry[j] - Y[j];
        a1 = a1 + m1[j] * ux;
        b1 = b1 + m1[j] * uy;
        a2 = a2 + m2[j] * ux;
        b2 = b2 + m2[j] * uy;
    }
    float e00 = a1 + 0.5f * (a1 * a1 + b1 * b1);
    float e11 = b2 + 0.5f * (a2 * a2 + b2 * b2);
    float e01 = 0.5f * (a2 + b1 + a1 * a2 + b1 * b2);
    const float c1 = s.C1, c2 = s.C2, c3 = s.C3;
    float pesum = c1 * (e00 * e00 + e11 * e11) + 2.0f * c2 * (e00 * e11) + 4.0f * c3 * (e01 * e01);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float n1 = m1[i], n2 = m2[i];
        float fxs = -2.0f * c1 * e00 * n1 * (1.0f + a1) - 2.0f * c1 * e11 * n2 * a2 - 2.0f * c2 * e00 * n2 * a2 -
                    2.0f * c2 * e11 * n1 * (1.0f + a1) - 4.0f * c3 * e01 * n2 * (1.0f + a1) - 4.0f * c3 * e01 * n1 * a2;
        float fys = -2.0f * c1 * e00 * n1 * b1 - 2.0f * c1 * e11 * n2 * (1.0f + b2) - 2.0f * c2 * e00 * n2 * (1.0f + b2) -
                    2.0f * c2 * e11 * n1 * b1 - 4.0f * c3 * e01 * n1 * (1.0f + b2) - 4.0f * c3 * e01 * n2 * b1;
        f[i] = make_float2(fxs * tetVol, fys * tetVol);
    }
    return pesum * tetVol;
}

__global__ void __launch_bounds__(kBlock) k_tri_forces(DevSys s, int parity) {
    const float2 *pos = parity ? s.pos1 : s.pos0;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    float e = 0.0f;
    if (t < s.ntri) {
        float2 f[3];
        if (s.feaLaw == 0)
            e = tri_neo_hookean(s, pos, t, f[0], f[1], f[2]);
        else
            e = tri_green(s, pos, t, f);
        s.triF[3 * t + 0] = f[0];
        s.triF[3 * t + 1] = f[1];
        s.triF[3 * t + 2] = f[2];
        s.triE[t] = e;
    }
    // triangle energies go straight into the potential-energy accumulator
    __shared__ float red[kBlock / 32];
    e = warp_sum_f(e);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
    __syncthreads();
    if (threadIdx.x == 0) {
        float b = 0.0f;
        for (int w = 0; w < kBlock / 32; w++) b += red[w];
        bool bad = false;
        unsigned long long q = to_fixed(b, bad);
        if (bad) atomicOr(&s.sc->nonfinite, 2);
        else if (q) atomicAdd(&s.sc->accU, q);
    }
}

// ------------------------------------------------------------ particles

// minImage on one axis with the wrap known at compile time.  Sets *wrapped
// when the difference crossed the boundary (then the exact-image value can
// differ from the reference float value).
template <bool WRAP, bool EX>
__device__ __forceinline__ float img(float a, float b, float L, float &ref, bool &wrapped) {
    float d = a - b;
    ref = d;
    if (WRAP) {
        if (d >= 0.5f * L) {
            ref = d - L;
            wrapped = true;
            return EX ? ref + two_sum_err(a, -b, d) : ref;
        }
        if (d < -0.5f * L) {
            ref = d + L;
            wrapped = true;
            return EX ? ref + two_sum_err(a, -b, d) : ref;
        }
    }
    return d;
}

// One Lennard-Jones pair (pairForce/ljforce, interactionsCuda.cu:43-100) added
// into the running force in list order.  Energy and virial are accumulated
// doubled (u and fc*dr2 per ordered pair) and halved once per particle.
template <bool MT, bool SG, bool WX, bool WY, bool EX, bool SIG1>
__device__ __forceinline__ void lj_pair(const DevSys &s, const PairEntry *tab, const PairEntry &pe0, int ti, float si,
                                        float2 pi, int tag, float2 pj, float &fx, float &fy, float &u2, float &w2) {
    float dxr, dyr;
    bool wrapped = false;
    float dx = img<WX, EX>(pi.x, pj.x, s.Lx, dxr, wrapped);
    float dy = img<WY, EX>(pi.y, pj.y, s.Ly, dyr, wrapped);
    float dr2r = dxr * dxr + dyr * dyr;
    const PairEntry &pe = MT ? tab[ti * s.numTypes + ((unsigned)tag >> kIdBits)] : pe0;
    float rcut2, sig2, c;
    if (SG) {
        float sij = (si + __ldg(s.sigma + (tag & kIdMask))) / 2.0f;
        rcut2 = pe.rc * pe.rc * sij * sij;
        sig2 = sij * sij;
        c = pe.eps48 / sig2;
    } else {
        rcut2 = pe.rcut2;
        sig2 = pe.sig2;
        c = pe.c;
    }
    if (dr2r < rcut2) {
        float dr2 = (EX && wrapped) ? dx * dx + dy * dy : dr2r;
        // sigma^2/dr2; with sigma_ij = 1 the IEEE quotient 1/dr2 is the
        // correctly rounded reciprocal
        float dr2i = SIG1 ? __frcp_rn(dr2) : sig2 / dr2;
        float dr6i = dr2i * dr2i * dr2i;
        float fc = c * dr6i * (dr6i - 0.5f) * dr2i;
        fx += fc * dx;
        fy += fc * dy;
        u2 += pe.eps4 * dr6i * (dr6i - 1.0f) + pe.us;
        w2 += fc * dr2;
    }
}

template <bool MT, bool SG, bool WX, bool WY, bool EX, bool SIG1>
__global__ void __launch_bounds__(kStepBlock) k_step(DevSys s, int mode, int parity, cudaGraphConditionalHandle h,
                                                     int use_h) {
    const float2 *__restrict__ pin = parity ? s.pos1 : s.pos0;
    float2 *__restrict__ pout = parity ? s.pos0 : s.pos1;
    extern __shared__ PairEntry tab[];  // numTypes^2 entries (1 without types)
    __shared__ float red[3][kStepBlock / 32];
    __shared__ float redm[kStepBlock / 32];
    const int nt = s.numTypes;
    if (MT) {
        for (int q = threadIdx.x; q < nt * nt; q += blockDim.x) tab[q] = s.pair[q];
    } else if (threadIdx.x == 0) {
        tab[0] = s.pair[0];
    }
    __syncthreads();

    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float ue = 0.0f, we = 0.0f, ke = 0.0f, vvm = 0.0f, utri = 0.0f;
    bool bad = false;
    if (i < s.N) {
        const float2 pi = pin[i];
        const float Lx = s.Lx, Ly = s.Ly;
        float fx = 0.0f, fy = 0.0f;
        if (i < s.nBonded) {
            if (s.bondForces) {
                // calcBondForcesCPU: f on the bond's first particle, -f on the second
                const int qb = s.bStart[i], qe = s.bStart[i + 1];
                for (int q = qb; q < qe; q++) {
                    int2 en = __ldg(s.bEnt + q);
                    const bool second = en.x < 0;
                    const int j = en.x & 0x7fffffff;
                    const float r0 = __int_as_float(en.y);
                    const float2 pj = pin[j];
                    const float2 a = second ? pj : pi, b = second ? pi : pj;
                    float dxr, dyr;
                    bool wr = false;
                    float dx = img<WX, EX>(a.x, b.x, Lx, dxr, wr);
                    float dy = img<WY, EX>(a.y, b.y, Ly, dyr, wr);
                    float r = sqrtf(dx * dx + dy * dy);
                    float dl = r - r0;
                    float k = s.bondKMode ? s.E / r0 : s.kBond;
                    float kdr = -k * dl / r;
                    float f1 = kdr * dx, f2 = kdr * dy;
                    if (!second) {
                        fx += f1;
                        fy += f2;
                        ue += k * dl * dl;  // doubled like the pair terms
                    } else {
                        fx -= f1;
                        fy -= f2;
                    }
                }
            }
            if (s.feaForces) {
                const int qb = s.tStart[i], qe = s.tStart[i + 1];
                for (int q = qb; q < qe; q++) {
                    int en = __ldg(s.tEnt + q);
                    float2 f = s.triF[3 * (en >> 2) + (en & 3)];
                    fx += f.x;
                    fy += f.y;
                    if (mode == MODE_FORCES) utri += s.triE[en >> 2] / 3.0f;
                }
            }
        }
        // pairForce over the Verlet list, in list order (next entry prefetched)
        {
            const int cnt = min(s.nbrCount[i], s.nbrCap);
            const int *__restrict__ lst = s.nbr + i;
            const int stride = s.Ncap;
            const int ti = MT ? s.typeId[i] : 0;
            const float si = SG ? s.sigma[i] : 0.0f;
            const PairEntry pe0 = tab[0];
            int tag = cnt > 0 ? __ldg(lst) : 0;
            for (int k = 1; k <= cnt; k++) {
                lst += stride;
                const int tnext = k < cnt ? __ldg(lst) : 0;
                lj_pair<MT, SG, WX, WY, EX, SIG1>(s, tab, pe0, ti, si, pi, tag, pin[tag & kIdMask], fx, fy, ue, we);
                tag = tnext;
            }
        }
        ue *= 0.5f;
        we *= 0.5f;
        bad = !(isfinite(fx) && isfinite(fy));
        const float m = s.mass[i];
        const float ax = fx / m, ay = fy / m;
        const float dt = s.dt, hdt = s.hdt;
        if (mode == MODE_FORCES) {
            s.forceOut[i] = make_float2(fx, fy);
            s.energyOut[i] = ue + utri;
        } else if (mode == MODE_INIT) {
            s.acc[i] = make_float2(ax, ay);
            s.forceOut[i] = make_float2(fx, fy);
        } else {
            float2 v = s.vel[i];
            if (mode == MODE_MID || mode == MODE_LAST) {
                // leapFrogStep2 then evalProps
                v.x += hdt * ax;
                v.y += hdt * ay;
                float vv = v.x * v.x + v.y * v.y;
                vvm = vv;
                ke = m * vv;
            }
            if (mode == MODE_LAST) {
                s.vel[i] = v;
                s.acc[i] = make_float2(ax, ay);
                s.forceOut[i] = make_float2(fx, fy);
            } else {
                // next step's leapFrogStep1 + applyPBC
                v.x += hdt * ax;
                v.y += hdt * ay;
                float2 x = make_float2(pi.x + dt * v.x, pi.y + dt * v.y);
                if (WX) x.x = wrap_coord(x.x, Lx);
                if (WY) x.y = wrap_coord(x.y, Ly);
                pout[i] = x;
                s.vel[i] = v;
            }
        }
    }

    // ---- reductions: FP32 within the block, 64-bit fixed-point atomics across
    // blocks (exact, order-independent); the last block converts and finishes.
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float su = warp_sum_f(ue), sw = warp_sum_f(we), sk = warp_sum_f(ke);
    float mx = warp_max(vvm);
    unsigned anybad = __ballot_sync(0xffffffffu, bad);
    if (lane == 0) {
        red[0][warp] = su;
        red[1][warp] = sw;
        red[2][warp] = sk;
        redm[warp] = mx;
        if (anybad) atomicOr(&s.sc->nonfinite, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.0f, b = 0.0f, c = 0.0f, m = 0.0f;
        for (int w = 0; w < kStepBlock / 32; w++) {
            a += red[0][w];
            b += red[1][w];
            c += red[2][w];
            m = fmaxf(m, redm[w]);
        }
        bool ob = false;
        unsigned long long qa = to_fixed(a, ob), qb = to_fixed(b, ob), qc = to_fixed(c, ob);
        DevScalars *sc = s.sc;
        if (ob) atomicOr(&sc->nonfinite, 2);
        if (qa) atomicAdd(&sc->accU, qa);
        if (qb) atomicAdd(&sc->accW, qb);
        if (qc) atomicAdd(&sc->accK, qc);
        if (m > 0.0f) atomicMax(&sc->vvMaxBits, __float_as_uint(m));
        __threadfence();
        if (atomicAdd(&sc->ticket, 1u) == gridDim.x - 1) {
            __threadfence();
            // the grid's last block: every block's atomics are visible
            double U = from_fixed(atomicExch(&sc->accU, 0ull));
            double W = from_fixed(atomicExch(&sc->accW, 0ull));
            double KE = from_fixed(atomicExch(&sc->accK, 0ull));
            float vm2 = __uint_as_float(atomicExch(&sc->vvMaxBits, 0u));
            sc->U = U;
            sc->W = W;
            int reb;
            if (mode == MODE_MID || mode == MODE_LAST) {
                sc->KE = KE;
                sc->vvMax = vm2;
                float d = sc->dispHi + sqrtf(vm2) * s.dt;  // md3dsystem.cpp:177
                reb = (double)d > s.halfSkin;               // nn.cpp:118
                int row = sc->obsRow;
                if (s.obs && row < s.obsCap) {
                    double *o = s.obs + (size_t)row * kObsCols;
                    o[0] = U;
                    o[1] = W;
                    o[2] = KE;
                    o[3] = (double)vm2;
                    o[4] = (double)d;
                    o[5] = (double)reb;
                }
                sc->obsRow = row + 1;
                sc->dispHi = d;  // a rebuild (k_rebuild_begin) restarts it and counts the update
            } else {
                reb = (double)sc->dispHi > s.halfSkin;
            }
            sc->rebuild = reb;
            if (use_h) cudaGraphSetConditional(h, reb ? 1u : 0u);
            sc->ticket = 0;
        }
    }
}

// leapFrogStep1 + applyPBC on their own (c_doStep entry)
__global__ void __launch_bounds__(kBlock) k_drift(DevSys s, int parity) {
    const float2 *pin = parity ? s.pos1 : s.pos0;
    float2 *pout = parity ? s.pos0 : s.pos1;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.N) return;
    float2 v = s.vel[i], a = s.acc[i], p = pin[i];
    v.x += s.hdt * a.x;
    v.y += s.hdt * a.y;
    p.x += s.dt * v.x;
    p.y += s.dt * v.y;
    if (s.wrapx) p.x = wrap_coord(p.x, s.Lx);
    if (s.wrapy) p.y = wrap_coord(p.y, s.Ly);
    pout[i] = p;
    s.vel[i] = v;
}

template <bool MT, bool SG, bool WX, bool WY, bool EX, bool SIG1>
static cudaError_t launch_step(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h,
                               int use_h) {
    dim3 g(step_blocks(s.N)), b(kStepBlock);
    size_t smt = sizeof(PairEntry) * (size_t)(s.numTypes > 1 ? s.numTypes * s.numTypes : 1);
    return L.kernel(k_step<MT, SG, WX, WY, EX, SIG1>, g, b, smt, s, mode, parity, h, use_h);
}

template <bool MT, bool SG, bool WX, bool WY, bool EX>
static cudaError_t pick_sig(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h, int use_h) {
    if (!SG && s.sigmaOne) return launch_step<MT, SG, WX, WY, EX, true>(L, s, mode, parity, h, use_h);
    return launch_step<MT, SG, WX, WY, EX, false>(L, s, mode, parity, h, use_h);
}

template <bool MT, bool SG>
static cudaError_t pick_image(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h,
                              int use_h) {
    const bool ex = s.imageExact;
    if (s.wrapx && s.wrapy)
        return ex ? pick_sig<MT, SG, true, true, true>(L, s, mode, parity, h, use_h)
                  : pick_sig<MT, SG, true, true, false>(L, s, mode, parity, h, use_h);
    if (s.wrapx)
        return ex ? pick_sig<MT, SG, true, false, true>(L, s, mode, parity, h, use_h)
                  : pick_sig<MT, SG, true, false, false>(L, s, mode, parity, h, use_h);
    return pick_sig<MT, SG, false, false, false>(L, s, mode, parity, h, use_h);
}

cudaError_t enqueue_step(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h, int use_h) {
    cudaError_t e;
    if (s.feaForces && s.ntri > 0) {
        if ((e = L.kernel(k_tri_forces, dim3(tri_blocks(s.ntri)), dim3(kBlock), 0, s, parity))) return e;
    }
    cudaEvent_t e0 = L.mark();
    if (s.numTypes > 1)
        e = s.sigmaByType ? pick_image<true, false>(L, s, mode, parity, h, use_h)
                          : pick_image<true, true>(L, s, mode, parity, h, use_h);
    else
        e = s.sigmaByType ? pick_image<false, false>(L, s, mode, parity, h, use_h)
                          : pick_image<false, true>(L, s, mode, parity, h, use_h);
    cudaEvent_t e1 = L.mark();
    if (e0 && e1 && L.force_events) L.force_events->push_back({e0, e1});
    return e;
}

cudaError_t enqueue_drift(Launch &L, const DevSys &s, int parity) {
    return L.kernel(k_drift, dim3(force_blocks(s.N)), dim3(kBlock), 0, s, parity);
}

}  // namespace femmd
