// k_adjoint.cu -- discrete adjoint of the femmd2D timestep.
//
// The forward step (Integrator::doStep, femmd2D/src/integrator.cpp:8-29) is
// kick-drift-kick leapfrog: v' = v_n + h a_n, x_{n+1} = x_n + dt v',
// a_{n+1} = f(x_{n+1}) / m, v_{n+1} = v' + h a_{n+1}  (h = dt/2).  Its exact
// reverse, with xbar = dJ/dx and vbar = dJ/dv carried backwards, is
//     w      = c vbar_{n+1} / m          (c = h at the last state, dt inside)
//     xbar  += (df/dx)^T w               at x_{n+1}
//     vbar  += dt xbar                   -> vbar_n
// and at the initial state one more xbar += (df/dx)^T w with c = h.  The
// forces are minus a gradient, so (df/dx)^T w is the directional derivative
// of the forces along the field w: for every interaction the same gather as
// the forward (bonds, triangles through the vertex incidence, the Verlet list
// in list order, walls), deterministic, no atomics on particle data.
//
// Parameter derivatives sum w . df/dtheta:
//   LJ eps (one scale on every eps_ab): f_LJ itself;
//   LJ sigma (one scale on every sigma_i, so sigma_ij and the wall contact
//     ranges scale with it): sigma_ij dfc/dsigma_ij = c s2 (12 s6^2 - 3 s6);
//   per-triangle mu and lambda: the neo-Hookean stress is linear in both,
//     P = mu (F - F^-T) + lambda ln J F^-T.
// They accumulate in FP64 per particle / per triangle (each owned by one
// thread, so the sums are deterministic) and are reduced on the host.
#include <cuda_runtime.h>
#include "femmd_internal.h"
#include "launch.h"
#include "device_common.cuh"
#include "step_body.cuh"

namespace femmd {

namespace {

// Edge matrix Ds of a triangle with the image shifts k (same operations as
// tri_neo_hookean in both image modes).
__device__ __forceinline__ void tri_edges(const DevSys &s, float2 r0, float2 r1, float2 r2, int k1x, int k2x, int k1y,
                                          int k2y, float &Ds00, float &Ds10, float &Ds01, float &Ds11) {
    const float L = s.Lx, Ly = s.Ly;
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
}

// Neo-Hookean triangle: nodal-force derivative along w, and w . df/dmu,
// w . df/dlambda.  Same image handling and float operations as
// tri_neo_hookean for the primal quantities.
__device__ __forceinline__ void tri_neo_hookean_jvp(const DevSys &s, const float2 *pos, const float2 *w, int t,
                                                    float2 &d0, float2 &d1, float &gmu, float &glam) {
    int4 q = __ldg(s.triIdx + t);
    float2 r0 = pos[q.x], r1 = pos[q.y], r2 = pos[q.z];
    float2 w0 = w[q.x], w1 = w[q.y], w2 = w[q.z];
    float4 bm = __ldg(s.triGeo + 2 * t);
    float vol0 = __ldg(s.triGeo + 2 * t + 1).x;
    const float L = s.Lx, Ly = s.Ly;
    float dx01 = r0.x - r1.x, dx02 = r0.x - r2.x, dy01 = r0.y - r1.y, dy02 = r0.y - r2.y;
    int k1x = (dx01 > L / 2.0f) - (dx01 < -L / 2.0f);
    int k2x = (dx02 > L / 2.0f) - (dx02 < -L / 2.0f);
    int k1y = (dy01 > Ly / 2.0f) - (dy01 < -Ly / 2.0f);
    int k2y = (dy02 > Ly / 2.0f) - (dy02 < -Ly / 2.0f);
    float Ds00, Ds10, Ds01, Ds11;
    tri_edges(s, r0, r1, r2, k1x, k2x, k1y, k2y, Ds00, Ds10, Ds01, Ds11);
    const float dDs00 = w0.x - w2.x, dDs10 = w0.y - w2.y, dDs01 = w1.x - w2.x, dDs11 = w1.y - w2.y;
    const float B00 = bm.x, B10 = bm.y, B01 = bm.z, B11 = bm.w;
    float F00 = Ds00 * B00 + Ds01 * B10, F10 = Ds10 * B00 + Ds11 * B10;
    float F01 = Ds00 * B01 + Ds01 * B11, F11 = Ds10 * B01 + Ds11 * B11;
    float dF00 = dDs00 * B00 + dDs01 * B10, dF10 = dDs10 * B00 + dDs11 * B10;
    float dF01 = dDs00 * B01 + dDs01 * B11, dF11 = dDs10 * B01 + dDs11 * B11;
    float det = F00 * F11 - F01 * F10;
    float ddet = (dF00 * F11 + F00 * dF11) - (dF01 * F10 + F01 * dF10);
    float logJ = own_logf(det);
    float dlogJ = ddet / det;
    float mu = s.mu, lambda = s.lambda;
    if (s.triLame) {
        const float2 ml = __ldg(s.triLame + t);
        mu = ml.x;
        lambda = ml.y;
    }
    float i00 = F11 / det, i10 = -F10 / det, i01 = -F01 / det, i11 = F00 / det;
    float di00 = (dF11 - i00 * ddet) / det, di10 = (-dF10 - i10 * ddet) / det;
    float di01 = (-dF01 - i01 * ddet) / det, di11 = (dF00 - i11 * ddet) / det;
    float ll = lambda * logJ, dll = lambda * dlogJ;
    // dP = mu (dF - dF^-T) + dll F^-T + ll dF^-T, F^-T entries (i00, i01; i10, i11)
    float dP00 = mu * (dF00 - di00) + dll * i00 + ll * di00;
    float dP10 = mu * (dF10 - di01) + dll * i01 + ll * di01;
    float dP01 = mu * (dF01 - di10) + dll * i10 + ll * di10;
    float dP11 = mu * (dF11 - di11) + dll * i11 + ll * di11;
    float nv0 = -vol0;
    d0 = make_float2(nv0 * (dP00 * B00 + dP01 * B01), nv0 * (dP10 * B00 + dP11 * B01));
    d1 = make_float2(nv0 * (dP00 * B10 + dP01 * B11), nv0 * (dP10 * B10 + dP11 * B11));
    // w . f_mu and w . f_lambda: the nodal forces of vertices 0 and 1 against
    // (w0 - w2) and (w1 - w2) (vertex 2 carries minus their sum)
    float Pm00 = F00 - i00, Pm10 = F10 - i01, Pm01 = F01 - i10, Pm11 = F11 - i11;
    float Hm00 = nv0 * (Pm00 * B00 + Pm01 * B01), Hm10 = nv0 * (Pm10 * B00 + Pm11 * B01);
    float Hm01 = nv0 * (Pm00 * B10 + Pm01 * B11), Hm11 = nv0 * (Pm10 * B10 + Pm11 * B11);
    float Pl00 = logJ * i00, Pl10 = logJ * i01, Pl01 = logJ * i10, Pl11 = logJ * i11;
    float Hl00 = nv0 * (Pl00 * B00 + Pl01 * B01), Hl10 = nv0 * (Pl10 * B00 + Pl11 * B01);
    float Hl01 = nv0 * (Pl00 * B10 + Pl01 * B11), Hl11 = nv0 * (Pl10 * B10 + Pl11 * B11);
    gmu = dDs00 * Hm00 + dDs10 * Hm10 + dDs01 * Hm01 + dDs11 * Hm11;
    glam = dDs00 * Hl00 + dDs10 * Hl10 + dDs01 * Hl01 + dDs11 * Hl11;
}

}  // namespace

// per triangle: nodal JVP into triD, parameter terms into gMu / gLam (FP64)
__global__ void __launch_bounds__(kBlock) k_adj_tri(DevSys s, const float2 *pos, const float2 *w, float2 *triD,
                                                     double *gMu, double *gLam) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= s.ntri) return;
    float2 d0, d1;
    float gm, gl;
    tri_neo_hookean_jvp(s, pos, w, t, d0, d1, gm, gl);
    triD[3 * t + 0] = d0;
    triD[3 * t + 1] = d1;
    triD[3 * t + 2] = make_float2(-d0.x - d1.x, -d0.y - d1.y);
    gMu[t] += (double)gm;
    gLam[t] += (double)gl;
}

// per particle: xbar += (df/dx)^T w at pos; then (update) vbar += dt xbar and
// the next weight wOut = cNext vbar / m.  epsAcc / sigAcc: w . df/d(log eps),
// w . df/d(log sigma), FP64 per particle.
template <bool WX, bool WY>
__global__ void __launch_bounds__(kStepBlock) k_adj_step(DevSys s, const float2 *pos, const float2 *w,
                                                          const float2 *triD, float2 *xbar, float2 *vbar,
                                                          float2 *wOut, float cNext, int update, float yw,
                                                          double *epsAcc, double *sigAcc) {
    extern __shared__ PairEntry tab[];
    const int nt2 = s.numTypes > 1 ? s.numTypes * s.numTypes : 1;
    for (int k = threadIdx.x; k < nt2; k += blockDim.x) tab[k] = s.pair[k];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.N) return;
    const float2 pi = pos[i], wi = w[i];
    const float Lx = s.Lx, Ly = s.Ly;
    float gx = 0.0f, gy = 0.0f;
    if (i < s.nBonded) {
        if (s.bondForces) {
            const int qb = s.bStart[i], qe = s.bStart[i + 1];
            for (int q = qb; q < qe; q++) {
                int2 en = __ldg(s.bEnt + q);
                const bool second = en.x < 0;
                const int j = en.x & 0x7fffffff;
                const float r0 = __int_as_float(en.y);
                const float2 pj = pos[j], wj = w[j];
                const float2 a = second ? pj : pi, b = second ? pi : pj;
                const float2 wa = second ? wj : wi, wb = second ? wi : wj;
                float dxr, dyr;
                bool wr = false;
                float dx = img<WX>(a.x, b.x, Lx, s.imageExact, dxr, wr);
                float dy = img<WY>(a.y, b.y, Ly, s.imageExact, dyr, wr);
                float r = sqrtf(dx * dx + dy * dy);
                float dl = r - r0;
                float k = s.bondKMode ? s.E / r0 : s.kBond;
                float kdr = -k * dl / r;
                float ddx = wa.x - wb.x, ddy = wa.y - wb.y;
                float dr = (dx * ddx + dy * ddy) / r;
                float dkdr = -k * r0 * dr / (r * r);
                float f1 = dkdr * dx + kdr * ddx, f2 = dkdr * dy + kdr * ddy;
                if (!second) {
                    gx += f1;
                    gy += f2;
                } else {
                    gx -= f1;
                    gy -= f2;
                }
            }
        }
        if (s.feaForces) {
            const int qb = s.tStart[i], qe = s.tStart[i + 1];
            for (int q = qb; q < qe; q++) {
                int en = __ldg(s.tEnt + q);
                float2 f = triD[3 * (en >> 2) + (en & 3)];
                gx += f.x;
                gy += f.y;
            }
        }
    }
    double ea = 0.0, sa = 0.0;
    {
        const int cnt = min(s.nbrCount[i], s.nbrCap);
        const int ti = s.numTypes > 1 ? s.typeId[i] : 0;
        const float si = s.sigmaByType ? 0.0f : s.sigma[i];
        float fex = 0.0f, fey = 0.0f, fsx = 0.0f, fsy = 0.0f;
        for (int k = 0; k < cnt; k++) {
            const int tag = s.nbr[nbr_at(k, i, s.Ncap)];
            const int j = tag & kIdMask;
            const float2 pj = pos[j];
            float dxr, dyr;
            bool wrapped = false;
            float dx = img<WX>(pi.x, pj.x, Lx, s.imageExact, dxr, wrapped);
            float dy = img<WY>(pi.y, pj.y, Ly, s.imageExact, dyr, wrapped);
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
            if (dr2r < rcut2) {
                float dr2 = wrapped ? dx * dx + dy * dy : dr2r;
                float s2 = sig2 / dr2;
                float s6 = s2 * s2 * s2;
                float fc = c * s6 * (s6 - 0.5f) * s2;
                float cs2 = c * s2;                                  // 48 eps / r^2
                float dfc = -(cs2 / dr2) * (7.0f * s6 * s6 - 2.0f * s6);  // d fc / d r^2
                const float2 wj = w[j];
                float ddx = wi.x - wj.x, ddy = wi.y - wj.y;
                float dot = dx * ddx + dy * ddy;
                gx += fc * ddx + 2.0f * dfc * dot * dx;
                gy += fc * ddy + 2.0f * dfc * dot * dy;
                fex += fc * dx;
                fey += fc * dy;
                float fs = cs2 * (12.0f * s6 * s6 - 3.0f * s6);
                fsx += fs * dx;
                fsy += fs * dy;
            }
        }
        ea = (double)wi.x * (double)fex + (double)wi.y * (double)fey;
        sa = (double)wi.x * (double)fsx + (double)wi.y * (double)fsy;
    }
    if (s.wallOn) {
        const float dl = s.wallDelta[i];
        const float ht = (pi.y + dl) - yw, hb = dl - pi.y;
        if (ht > 0.0f) {
            gy -= s.wallK * wi.y;
            sa += (double)wi.y * (double)(-s.wallK * dl);
        }
        if (hb > 0.0f) {
            gy -= s.wallK * wi.y;
            sa += (double)wi.y * (double)(s.wallK * dl);
        }
    }
    epsAcc[i] += ea;
    sigAcc[i] += sa;
    float2 xb = xbar[i];
    xb.x += gx;
    xb.y += gy;
    xbar[i] = xb;
    if (update) {
        float2 vb = vbar[i];
        vb.x += s.dt * xb.x;
        vb.y += s.dt * xb.y;
        vbar[i] = vb;
        const float m = s.mass[i];
        wOut[i] = make_float2(cNext * vb.x / m, cNext * vb.y / m);
    }
}

// Seed at the final positions x_N for J = cWall (F_top + F_bottom) / (2 Lx)
// + cFea U_fea (+ the caller's xbar, vbar seeds already in xbar / vbar):
// xbar += cFea * (-f_fea) + cWall * d(stress)/dx; the direct parameter terms
// go to gMu / gLam (triangle energies) and sigAcc (contact ranges).  Then
// w = h vbar / m.  triF holds the FEA nodal forces at x_N.
__global__ void __launch_bounds__(kBlock) k_adj_seed(DevSys s, const float2 *pos, float2 *xbar, const float2 *vbar,
                                                      float2 *wOut, float cWall, float cFea, float yw,
                                                      double *sigAcc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.N) return;
    float2 xb = xbar[i];
    if (cFea != 0.0f && s.feaForces && i < s.nBonded) {
        float fx = 0.0f, fy = 0.0f;
        const int qb = s.tStart[i], qe = s.tStart[i + 1];
        for (int q = qb; q < qe; q++) {
            int en = __ldg(s.tEnt + q);
            float2 f = s.triF[3 * (en >> 2) + (en & 3)];
            fx += f.x;
            fy += f.y;
        }
        xb.x -= cFea * fx;
        xb.y -= cFea * fy;
    }
    if (cWall != 0.0f && s.wallOn) {
        const float dl = s.wallDelta[i], y = pos[i].y;
        const float ht = (y + dl) - yw, hb = dl - y;
        const float a = cWall * s.wallK / (2.0f * s.Lx);
        double sa = 0.0;
        if (ht > 0.0f) {
            xb.y += a;
            sa += (double)a * (double)dl;
        }
        if (hb > 0.0f) {
            xb.y -= a;
            sa += (double)a * (double)dl;
        }
        sigAcc[i] += sa;
    }
    xbar[i] = xb;
    const float2 vb = vbar[i];
    const float m = s.mass[i];
    wOut[i] = make_float2(s.hdt * vb.x / m, s.hdt * vb.y / m);
}

// direct energy terms of the observable: cFea dU/dmu, dU/dlambda per triangle
__global__ void __launch_bounds__(kBlock) k_adj_seed_tri(DevSys s, const float2 *pos, float cFea, double *gMu,
                                                          double *gLam) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= s.ntri) return;
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
    tri_edges(s, r0, r1, r2, k1x, k2x, k1y, k2y, Ds00, Ds10, Ds01, Ds11);
    float F00 = Ds00 * bm.x + Ds01 * bm.y, F10 = Ds10 * bm.x + Ds11 * bm.y;
    float F01 = Ds00 * bm.z + Ds01 * bm.w, F11 = Ds10 * bm.z + Ds11 * bm.w;
    float logJ = own_logf(F00 * F11 - F01 * F10);
    float d00 = F00 - 1.0f, d11 = F11 - 1.0f;
    float i1m2 = (2.0f * d00 + d00 * d00) + (2.0f * d11 + d11 * d11) + F01 * F01 + F10 * F10;
    gMu[t] += (double)cFea * (double)vol0 * 0.5 * ((double)i1m2 - 2.0 * (double)logJ);
    gLam[t] += (double)cFea * (double)vol0 * 0.5 * (double)logJ * (double)logJ;
}

cudaError_t enqueue_adj_seed(Launch &L, const DevSys &s, const float2 *pos, float2 *xbar, const float2 *vbar,
                             float2 *wOut, float cWall, float cFea, float yw, double *sigAcc, double *gMu,
                             double *gLam) {
    cudaError_t e;
    if (s.feaForces && s.ntri > 0 && cFea != 0.0f) {
        if ((e = L.kernel(k_adj_seed_tri, dim3(tri_blocks(s.ntri)), dim3(kBlock), 0, s, pos, cFea, gMu, gLam)))
            return e;
    }
    return L.kernel(k_adj_seed, dim3(force_blocks(s.N)), dim3(kBlock), 0, s, pos, xbar, vbar, wOut, cWall, cFea, yw,
                    sigAcc);
}

cudaError_t enqueue_adj_step(Launch &L, const DevSys &s, const float2 *pos, const float2 *w, float2 *triD,
                             double *gMu, double *gLam, float2 *xbar, float2 *vbar, float2 *wOut, float cNext,
                             int update, float yw, double *epsAcc, double *sigAcc) {
    cudaError_t e;
    if (s.feaForces && s.ntri > 0) {
        if ((e = L.kernel(k_adj_tri, dim3(tri_blocks(s.ntri)), dim3(kBlock), 0, s, pos, w, triD, gMu, gLam)))
            return e;
    }
    dim3 g(step_blocks(s.N)), b(kStepBlock);
    size_t smt = sizeof(PairEntry) * (size_t)(s.numTypes > 1 ? s.numTypes * s.numTypes : 1);
    if (s.wrapx && s.wrapy)
        return L.kernel(k_adj_step<true, true>, g, b, smt, s, pos, w, (const float2 *)triD, xbar, vbar, wOut, cNext,
                        update, yw, epsAcc, sigAcc);
    if (s.wrapx)
        return L.kernel(k_adj_step<true, false>, g, b, smt, s, pos, w, (const float2 *)triD, xbar, vbar, wOut, cNext,
                        update, yw, epsAcc, sigAcc);
    return L.kernel(k_adj_step<false, false>, g, b, smt, s, pos, w, (const float2 *)triD, xbar, vbar, wOut, cNext,
                    update, yw, epsAcc, sigAcc);
}

}  // namespace femmd
