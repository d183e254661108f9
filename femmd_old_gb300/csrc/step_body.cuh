// step_body.cuh -- per-triangle and per-particle work of the femmd2D timestep,
// shared by the plain kernels (k_force.cu) and the persistent batched kernel
// (k_batch.cu), so both execute the same arithmetic in the same order.
//
// Reference: calcFeaForcesCPU2 (femmd2D/src/interactions.cpp:532-689),
// computeFeaForcesGPU (interactionsCuda.cu:312-451), calcBondForcesCPU
// (interactions.cpp:143-173), pairForce/ljforce (interactionsCuda.cu:43-100),
// leapFrogStep1/2 + updateAcc + evalProps (integrator.cpp:100-135,
// md3dsystem.cpp:151-179).
#pragma once
#include <cuda_runtime.h>
#include "femmd_internal.h"
#include "device_common.cuh"

namespace femmd {

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
    float mu = s.mu, lambda = s.lambda;
    if (s.triLame) {
        const float2 ml = __ldg(s.triLame + t);
        mu = ml.x;
        lambda = ml.y;
    }
    float llogJ = lambda * logJ;
    float iF00 = F11 / detF, iF10 = -F10 / detF, iF01 = -F01 / detF, iF11 = F00 / detF;
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
    float pe = 0.5f * mu * (i1m2 - 2.0f * logJ) + 0.5f * lambda * logJ * logJ;
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

// Nodal forces of triangle t into triF, energy returned (law of s.feaLaw).
__device__ __forceinline__ float tri_force(const DevSys &s, const float2 *pos, int t) {
    float2 f[3];
    float e;
    if (s.feaLaw == 0)
        e = tri_neo_hookean(s, pos, t, f[0], f[1], f[2]);
    else
        e = tri_green(s, pos, t, f);
    s.triF[3 * t + 0] = f[0];
    s.triF[3 * t + 1] = f[1];
    s.triF[3 * t + 2] = f[2];
    s.triE[t] = e;
    return e;
}

// ------------------------------------------------------------ particles

// ljwallforce (femmd2D/src/interactionsCuda.cu:31-40), float operations as
// written there (its "zi6" is zi^9)
__device__ __forceinline__ float ljwallforce(float zi, float sigma, float &fz) {
    zi = sigma / zi;
    const float zi3 = zi * zi * zi;
    const float zi6 = zi3 * zi3 * zi3;
    const float u = 4.0f * zi6 * (zi6 - 1.0f) + 1.0f;
    const float fc = 48.0f * zi6 * (zi6 - 0.5f) / zi;
    fz = fabsf(fc);
    return u;
}

// The reference's fixed walls for particle i, added before every other
// force: calcWallForces (NOPBC, interactions.cpp:176-236) and
// calcTopBottomWallForces (XPBC, :238-286).
__device__ __forceinline__ void ref_walls(const DevSys &s, int i, float2 p, float &fx, float &fy, float &u) {
    const float s0 = s.wallSig[i];
    const float r = s0 * s.wallRc;
    float f;
    if (s.refWalls == 1) {
        if ((s.Ly - p.y) < r) {
            u += ljwallforce(s.Ly - p.y, s0, f);
            fy += -f;
        } else if (p.y < r) {
            u += ljwallforce(p.y, s0, f);
            fy += f;
        }
        if ((s.Lx - p.x) < r) {
            u += ljwallforce(s.Lx - p.x, s0, f);
            fx += -f;
        } else if (p.x < r) {
            u += ljwallforce(p.x, s0, f);
            fx += f;
        }
    } else {
        if ((s.Ly - p.y) < r) {
            const float yi = s.Ly - p.y;
            f = s.kWall * yi;
            u += (float)(0.5 * (double)s.kWall * (double)yi * (double)yi);
            fy += -f;
        } else if (p.y < r) {
            const float yi = p.y;
            f = s.kWall * yi;
            u += (float)(0.5 * (double)s.kWall * (double)yi * (double)yi);
            fy += f;
        }
    }
}

// top wall position when the positions are x_n: y0 - v (n dt), in float
__device__ __forceinline__ float wall_y(const DevSys &s, int n) { return s.wallY0 - s.wallV * ((float)n * s.dt); }

// minImage on one axis with the wrap known at compile time.  Sets *wrapped
// when the difference crossed the boundary (then the exact-image value can
// differ from the reference float value).
template <bool WRAP>
__device__ __forceinline__ float img(float a, float b, float L, bool ex, float &ref, bool &wrapped) {
    float d = a - b;
    ref = d;
    if (WRAP) {
        if (d >= 0.5f * L) {
            ref = d - L;
            wrapped = true;
            return ex ? ref + two_sum_err(a, -b, d) : ref;
        }
        if (d < -0.5f * L) {
            ref = d + L;
            wrapped = true;
            return ex ? ref + two_sum_err(a, -b, d) : ref;
        }
    }
    return d;
}

// One Lennard-Jones pair (pairForce/ljforce, interactionsCuda.cu:43-100) added
// into the running force in list order.  Energy and virial are accumulated
// doubled (u and fc*dr2 per ordered pair) and halved once per particle.
// The minimum image is the reference's float one (d - L / d + L); in exact
// image mode a pair inside the cutoff whose difference crossed the boundary
// takes the once-rounded value instead (ref + TwoSum error), a branch that
// only boundary pairs enter.
template <bool MT, bool SG, bool WX, bool WY, bool SIG1>
__device__ __forceinline__ void lj_pair(const DevSys &s, const PairEntry *tab, const PairEntry &pe0, int ti, float si,
                                        float2 pi, int tag, float2 pj, float &fx, float &fy, float &u2, float &w2) {
    float dx = pi.x - pj.x, dy = pi.y - pj.y;
    bool wrx = false, wry = false;
    // |d| >= L/2 is rare (boundary pairs): one compare on the common path
    if (WX && __builtin_expect(fabsf(dx) >= 0.5f * s.Lx, 0)) {
        const float h = 0.5f * s.Lx;
        if (dx >= h) {
            dx = dx - s.Lx;
            wrx = true;
        } else if (dx < -h) {
            dx = dx + s.Lx;
            wrx = true;
        }
    }
    if (WY && __builtin_expect(fabsf(dy) >= 0.5f * s.Ly, 0)) {
        const float h = 0.5f * s.Ly;
        if (dy >= h) {
            dy = dy - s.Ly;
            wry = true;
        } else if (dy < -h) {
            dy = dy + s.Ly;
            wry = true;
        }
    }
    float dr2 = dx * dx + dy * dy;
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
    if (dr2 < rcut2) {
        if (__builtin_expect((wrx || wry) && s.imageExact, 0)) {
            const float ex = pi.x - pj.x, ey = pi.y - pj.y;
            if (wrx) dx = dx + two_sum_err(pi.x, -pj.x, ex);
            if (wry) dy = dy + two_sum_err(pi.y, -pj.y, ey);
            dr2 = dx * dx + dy * dy;
        }
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

// The forces that come before the pair forces in the reference's CPU order
// for particle i at position pi: the fixed walls and gravity, then (bonded
// particles) the bond incidences in bond order and the triangles' nodal forces
// in triangle order.  ue collects the doubled bond energy, utri the triangle
// energy (MODE_FORCES only), uwall the wall energy.
template <bool WX, bool WY, bool RO>
__device__ __forceinline__ void bonded_forces(const DevSys &s, int i, int mode, const float2 *pin, float2 pi,
                                              float &fx, float &fy, float &ue, float &utri, float &uwall) {
    const float Lx = s.Lx, Ly = s.Ly;
    // walls and bonds come before the area springs in the reference's force
    // order: they see the positions from before that pass (posPre, for the
    // particles of [0, nPre); pin without area springs)
    if (s.refWalls) ref_walls(s, i, i < s.nPre ? s.posPre[i] : pi, fx, fy, uwall);
    if (s.gravity > 0.0f) fy -= s.mass[i] * s.gravity;
    if (i < s.nBonded) {
        if (s.bondForces) {
            // calcBondForcesCPU: f on the bond's first particle, -f on the second
            const float2 *pb = s.nPre > 0 ? s.posPre : pin;
            const float2 pw = s.nPre > 0 ? s.posPre[i] : pi;
            const int qb = s.bStart[i], qe = s.bStart[i + 1];
            for (int q = qb; q < qe; q++) {
                int2 en = __ldg(s.bEnt + q);
                const bool second = en.x < 0;
                const int j = en.x & 0x7fffffff;
                const float r0 = __int_as_float(en.y);
                const float2 pj = RO ? __ldg(pb + j) : pb[j];
                const float2 a = second ? pj : pw, b = second ? pw : pj;
                float dxr, dyr;
                bool wr = false;
                float dx = img<WX>(a.x, b.x, Lx, s.imageExact, dxr, wr);
                float dy = img<WY>(a.y, b.y, Ly, s.imageExact, dyr, wr);
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
}

// The rest of particle i's step once its force (fx, fy) is complete: halve
// the doubled energy and virial, add the wall energy and the moving walls,
// then the integration of the mode (kick, observables, next half kick and
// drift into pout) and the outputs of MODE_FORCES / MODE_INIT / MODE_LAST.
template <bool WX, bool WY>
__device__ __forceinline__ void finish_particle(const DevSys &s, int i, int mode, float2 pi, float2 *pout, float fx,
                                                float fy, float ue, float we, float utri, float uwall, float &ue_out,
                                                float &we_out, float &ke, float &vvm, bool &bad) {
    const float Lx = s.Lx, Ly = s.Ly;
    ue *= 0.5f;
    we *= 0.5f;
    ue += uwall;
    if (s.wallOn) {
        // harmonic walls after the pair forces: top wall at y_w(n), bottom at 0
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
            vvm = fmaxf(vvm, vv);
            ke += m * vv;
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
    ue_out += ue;
    we_out += we;
}

// One particle's step: bond, triangle and pair forces gathered in the order the
// reference's CPU path adds them into force[i], then the mode's integration.
// ue/we (doubled energy and virial), ke and vvm are accumulated by the caller.
// RO: the list and the neighbours' positions are read through the read-only
// path (written by an earlier kernel); the batched kernel rewrites both in the
// same launch and reads them with coherent loads (RO = false).
template <bool MT, bool SG, bool WX, bool WY, bool SIG1, bool RO = true, int PIPE = 0>
__device__ __forceinline__ void particle_step(const DevSys &s, const PairEntry *tab, int i, int mode,
                                              const float2 *pin, float2 *pout, float &ue_out,
                                              float &we_out, float &ke, float &vvm, bool &bad) {
    float ue = 0.0f, we = 0.0f, utri = 0.0f, uwall = 0.0f;
    const float2 pi = pin[i];
    float fx = 0.0f, fy = 0.0f;
    bonded_forces<WX, WY, RO>(s, i, mode, pin, pi, fx, fy, ue, utri, uwall);
    {
        // pairForce over the Verlet list, in list order.  The list comes in
        // 16-byte groups of four entries (nbr_at); the next group is in
        // flight while the current one is worked.  PIPE > 0: the four
        // neighbour positions of a group are gathered before its pair terms
        // are added in order; otherwise each is gathered at its turn (fewer
        // live registers, for the kernels whose occupancy needs them).
        const int cnt = min(s.nbrCount[i], s.nbrCap);
        const int4 *__restrict__ lst = reinterpret_cast<const int4 *>(s.nbr) + i;
        const size_t row = (size_t)s.Ncap;
        const int ti = MT ? s.typeId[i] : 0;
        const float si = SG ? s.sigma[i] : 0.0f;
        const PairEntry pe0 = tab[0];
        const int4 zero4 = make_int4(0, 0, 0, 0);
        int4 g = cnt > 0 ? (RO ? __ldg(lst) : *lst) : zero4;
        for (int base = 0; base < cnt; base += 4) {
            lst += row;
            const int4 gn = base + 4 < cnt ? (RO ? __ldg(lst) : *lst) : zero4;
            const int tags[4] = {g.x, g.y, g.z, g.w};
            if constexpr (PIPE == 2) {
                // two gathers in flight at a time
#pragma unroll
                for (int h = 0; h < 4; h += 2) {
                    float2 q[2];
#pragma unroll
                    for (int u = 0; u < 2; u++) {
                        const int j = tags[h + u] & kIdMask;
                        q[u] = base + h + u < cnt ? (RO ? __ldg(pin + j) : pin[j]) : make_float2(0.0f, 0.0f);
                    }
#pragma unroll
                    for (int u = 0; u < 2; u++)
                        if (base + h + u < cnt)
                            lj_pair<MT, SG, WX, WY, SIG1>(s, tab, pe0, ti, si, pi, tags[h + u], q[u], fx, fy, ue, we);
                }
            } else if constexpr (PIPE > 0) {
                float2 q[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int j = tags[u] & kIdMask;
                    q[u] = base + u < cnt ? (RO ? __ldg(pin + j) : pin[j]) : make_float2(0.0f, 0.0f);
                }
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (base + u < cnt)
                        lj_pair<MT, SG, WX, WY, SIG1>(s, tab, pe0, ti, si, pi, tags[u], q[u], fx, fy, ue, we);
            } else {
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    if (base + u < cnt) {
                        const int j = tags[u] & kIdMask;
                        lj_pair<MT, SG, WX, WY, SIG1>(s, tab, pe0, ti, si, pi, tags[u], RO ? __ldg(pin + j) : pin[j],
                                                      fx, fy, ue, we);
                    }
                }
            }
            g = gn;
        }
    }
    finish_particle<WX, WY>(s, i, mode, pi, pout, fx, fy, ue, we, utri, uwall, ue_out, we_out, ke, vvm, bad);
}

// End of a step kernel: the block's energy, virial, kinetic and max-speed
// sums in FP32, added across blocks as 64-bit fixed point with integer
// atomics (exact, order-independent); the grid's last block converts them,
// updates dispHi (md3dsystem.cpp:177), writes the observable row, sets the
// rebuild flag by the reference's test (nn.cpp:118) and the graph condition.
template <int BLOCK>
__device__ __forceinline__ void step_reduce(const DevSys &s, int mode, float ue, float we, float ke, float vvm,
                                            bool bad, cudaGraphConditionalHandle h, int use_h) {
    __shared__ float red[3][BLOCK / 32];
    __shared__ float redm[BLOCK / 32];
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
        for (int w = 0; w < BLOCK / 32; w++) {
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
            if (mode == MODE_FIRST || mode == MODE_MID) sc->stepNow += 1;  // the drift made x_{n+1}
            if (use_h) cudaGraphSetConditional(h, reb ? 1u : 0u);
            sc->ticket = 0;
            if (s.trace) {
                int row = sc->obsRow - ((mode == MODE_MID || mode == MODE_LAST) ? 1 : 0);
                if (row >= 0 && row < s.obsCap) s.trace[(size_t)row * kTraceCols + 3] = global_ns();
            }
        }
    }
}

}  // namespace femmd
