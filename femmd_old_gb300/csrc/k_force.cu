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
//                 triF[3t+slot] (no atomics); the block's energy in FP32, added
//                 across blocks as 64-bit fixed point.
//   k_area_keep,  with area springs only: the positions of the bonded range
//   k_area        kept for walls and bonds, then the vertices displaced in
//                 place triangle by triangle (one lane per elastomer).
//   k_step        thread per particle: gathers bond incidences (bond order),
//                 triangle incidences (triangle order) and the Verlet list
//                 (list order) -- the order in which the reference's CPU path
//                 adds into force[i] -- then a = f/m and the leapfrog, fused:
//                 kick to v(t) and, unless it is the last step of a run, the
//                 next half kick and the drift into the other position buffer.
//                 FP32 per-particle and per-block sums of U, W and sum m v^2,
//                 added across blocks as 64-bit fixed point with integer
//                 atomics (exact, order-independent, so deterministic); the
//                 last block converts them, updates dispHi and raises the
//                 rebuild flag / graph condition for the next step.
#include <cuda_runtime.h>
#include "femmd_internal.h"
#include "launch.h"
#include "device_common.cuh"
#include "step_body.cuh"

namespace femmd {

int force_blocks(int N) { return (N + kBlock - 1) / kBlock; }
int step_blocks(int N) { return (N + kStepBlock - 1) / kStepBlock; }
int tri_blocks(int ntri) { return (ntri + kBlock - 1) / kBlock; }

__global__ void __launch_bounds__(kBlock) k_tri_forces(DevSys s, int parity) {
    const float2 *pos = parity ? s.pos1 : s.pos0;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (s.trace && t == 0) {
        int row = s.sc->obsRow;
        if (row < s.obsCap) s.trace[(size_t)row * kTraceCols + 0] = global_ns();
    }
    float e = 0.0f;
    if (t < s.ntri) e = tri_force(s, pos, t);
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
        if (s.trace) {
            int row = s.sc->obsRow;
            if (row < s.obsCap) atomicMax(&s.trace[(size_t)row * kTraceCols + 1], global_ns());
        }
    }
}

// ------------------------------------------------------------ area springs
// calcAreaForcesCPU (interactions.cpp:696-750) moves positions, not forces,
// and triangle t reads the positions the earlier triangles left: within an
// elastomer the loop is serial (the hex-ring meshes chain every triangle to
// the one before).  Elastomers share no vertices, so each is one lane: a
// block of up to 32 lanes runs elastomers of the same mesh in lock step over
// the mesh's triangle list, with the vertices, the triangle list and each
// lane's reference areas A0 staged in shared memory.

constexpr int kAreaLanes = 32;

__global__ void __launch_bounds__(kBlock) k_area_keep(DevSys s, int parity) {
    const float2 *pin = parity ? s.pos1 : s.pos0;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < s.nPre) s.posPre[i] = pin[i];
}

// c = -kArea (A - A0) / A0 / 2 as the reference forms it: the exact product
// a b (a = -kArea/2, b = A - A0, 48 bits, exact in double) divided in double
// and rounded to float.  With a 48-bit dividend and a 24-bit divisor the
// double quotient never lands on or across a float rounding boundary that
// the exact quotient q does not, so the result is q rounded to float once.
// That is computed here without FP64 (slow on this part): y = ph / d from
// ph = RN(a b), the exact remainder r = ph - y d (one FMA), q - y =
// (r + pl) / d with pl = a b - ph (one FMA), and y moved by one unit when q
// lies clearly in a neighbour's rounding interval.  Ties within 2^-20 of an
// interval's half-width, and the corners of the float range, take the double
// division itself (out of line, so that it is not evaluated on the common
// path).  A zero product (the triangle kept its area) gives the signed zero
// y, as the double quotient does.
__device__ __noinline__ float area_coeff_f64(float a, float b, float d) {
    return __double2float_rn((double)a * (double)b / (double)d);
}

__device__ __forceinline__ float area_coeff(float a, float b, float d) {
    const float ph = __fmul_rn(a, b);
    const float pl = __fmaf_rn(a, b, -ph);
    const float y = __fdiv_rn(ph, d);
    const float r = __fmaf_rn(-y, d, ph);
    const unsigned ay = __float_as_uint(y) & 0x7fffffffu, aph = __float_as_uint(ph) & 0x7fffffffu,
                   ad = __float_as_uint(d) & 0x7fffffffu;
    // t = (|q| - |y|) |d|; |y| is kept while |t| < hb = ulp(y) |d| / 2
    const float t = __fadd_rn(r, pl) * (((__float_as_uint(d) ^ __float_as_uint(y)) & 0x80000000u) ? -1.0f : 1.0f);
    const float u = __uint_as_float((ay & 0x7f800000u) - (23u << 23));
    const float hb = 0.5f * u * fabsf(d), m = hb * 0x1p-20f, h3 = 3.0f * hb;
    const bool keep = fabsf(t) < hb - m;
    const bool up = t > hb + m && t < h3 - m;
    const bool down = t < -hb - m && t > -h3 + m;
    const bool dok = ad >= (31u << 23) && ad < (220u << 23);
    const bool fast = dok && aph >= (31u << 23) && aph < (220u << 23) && ay >= (31u << 23) && ay < (220u << 23) &&
                      (ay & 0x7fffffu) >= 2u && (keep || up || down);
    const float c = __uint_as_float(__float_as_uint(y) + (up ? 1u : 0u) - (down ? 1u : 0u));
    if (fast) return c;
    if (aph == 0u && dok) return y;
    return area_coeff_f64(a, b, d);
}

// Asynchronous global -> shared copies (cp.async): a lane issues all of its
// copies back to back and waits once, instead of one load latency per element.
__device__ __forceinline__ void copy_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src));
}
__device__ __forceinline__ void copy_async8(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src));
}
__device__ __forceinline__ void copy_async_wait() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// The newest value of vertex v after a triangle (t) stored n0, n1, n2 in that
// order; 'old' when the triangle did not touch v.
__device__ __forceinline__ float2 area_latest(int v, int4 t, float2 n0, float2 n1, float2 n2, float2 old) {
    return v == t.z ? n2 : v == t.y ? n1 : v == t.x ? n0 : old;
}

__global__ void __launch_bounds__(kAreaLanes) k_area(DevSys s, int parity) {
    extern __shared__ float4 smem4[];
    float2 *pos = parity ? s.pos1 : s.pos0;
    const int4 un = s.areaUnit[2 * blockIdx.x];  // triangle list, triangles, vertices, lanes
    const int a0base = s.areaUnit[2 * blockIdx.x + 1].x;
    const int nt = un.y, nv = un.z, nl = un.w, w = nl + 1;  // w: vertex stride (spreads the banks)
    const int lane = threadIdx.x;
    // shared memory: the mesh's triangle list, the lanes' A0 (padded to 16
    // bytes; the host pads each block's A0 range alike), the vertices
    int4 *idx = reinterpret_cast<int4 *>(smem4);
    float *a0 = reinterpret_cast<float *>(idx + nt);
    const int na = (nt * nl + 3) & ~3;
    float2 *sv = reinterpret_cast<float2 *>(a0 + na);
    for (int k = lane; k < nt; k += kAreaLanes) copy_async16(idx + k, s.areaIdx + un.x + k);
    for (int k = lane; k < na / 4; k += kAreaLanes) copy_async16(a0 + 4 * k, s.areaA0 + a0base + 4 * k);
    // coalesced over each elastomer's vertices, stored lane-minor
    for (int j = 0; j < nl; j++) {
        const int off = s.areaLane[blockIdx.x * kAreaLanes + j];
        for (int v = lane; v < nv; v += kAreaLanes) copy_async8(sv + v * w + j, pos + off + v);
    }
    copy_async_wait();
    __syncwarp();
    float e = 0.0f;  // a float sum, as the reference's potEnergy
    if (lane < nl && nt > 0) {
        // The lane's elastomer, triangle after triangle (calcAreaForcesCPU
        // order).  The next triangle's index, A0 and vertices are read before
        // this one stores; the vertices this one moved are passed on in
        // registers, so the chain from triangle to triangle is arithmetic only.
        float2 *mine = sv + lane;
        const float Lx = s.Lx, Ly = s.Ly, kA = s.kArea, ca = -0.5f * kA;
        const float hx = 0.5f * Lx, hy = 0.5f * Ly;
        int4 t = idx[0];
        float A0 = a0[lane];
        float2 v0 = mine[t.x * w], v1 = mine[t.y * w], v2 = mine[t.z * w];
        for (int k = 0; k < nt; k++) {
            const int kn = k + 1 < nt ? k + 1 : k;
            const int4 tn = idx[kn];
            const float A0n = a0[kn * nl + lane];
            float2 u0 = mine[tn.x * w], u1 = mine[tn.y * w], u2 = mine[tn.z * w];
            // r1 and r2 moved to r0's side by the half-box rule on both axes
            // (whatever the periodicity); the area A as float products halved
            // (the reference halves in double, which is exact)
            const float2 r0 = v0;
            float2 r1 = v1, r2 = v2;
            const float dx01 = r0.x - r1.x, dx02 = r0.x - r2.x;
            if (dx01 > hx) r1.x += Lx;
            if (dx01 < -hx) r1.x -= Lx;
            if (dx02 > hx) r2.x += Lx;
            if (dx02 < -hx) r2.x -= Lx;
            const float dy01 = r0.y - r1.y, dy02 = r0.y - r2.y;
            if (dy01 > hy) r1.y += Ly;
            if (dy01 < -hy) r1.y -= Ly;
            if (dy02 > hy) r2.y += Ly;
            if (dy02 < -hy) r2.y -= Ly;
            const float A = 0.5f * ((r2.y - r0.y) * (r1.x - r0.x) - (r1.y - r0.y) * (r2.x - r0.x));
            const float dA = A - A0;
            const float c = area_coeff(ca, dA, A0);
            const float f1x = c * (r2.y - r0.y), f1y = -c * (r2.x - r0.x);
            const float f2x = -c * (r1.y - r0.y), f2y = c * (r1.x - r0.x);
            const float f0x = -f1x - f2x, f0y = -f1y - f2y;
            // pos[p] += f[p] for p = 0, 1, 2 in turn (a repeated vertex sees
            // the earlier addition)
            const float2 n0 = make_float2(v0.x + f0x, v0.y + f0y);
            const float2 b1 = t.y == t.x ? n0 : v1;
            const float2 n1 = make_float2(b1.x + f1x, b1.y + f1y);
            const float2 b2 = t.z == t.y ? n1 : t.z == t.x ? n0 : v2;
            const float2 n2 = make_float2(b2.x + f2x, b2.y + f2y);
            mine[t.x * w] = n0;
            mine[t.y * w] = n1;
            mine[t.z * w] = n2;
            e += 0.5f * kA * dA * dA;
            v0 = area_latest(tn.x, t, n0, n1, n2, u0);
            v1 = area_latest(tn.y, t, n0, n1, n2, u1);
            v2 = area_latest(tn.z, t, n0, n1, n2, u2);
            t = tn;
            A0 = A0n;
        }
    }
    __syncwarp();
    for (int j = 0; j < nl; j++) {
        const int off = s.areaLane[blockIdx.x * kAreaLanes + j];
        for (int v = lane; v < nv; v += kAreaLanes) pos[off + v] = sv[v * w + j];
    }
    e = warp_sum_f(e);
    if (lane == 0) {
        bool bad = false;
        unsigned long long q = to_fixed(e, bad);
        if (bad) atomicOr(&s.sc->nonfinite, 2);
        else if (q) atomicAdd(&s.sc->accU, q);
    }
}

cudaError_t area_smem_setup(int bytes) {
    return cudaFuncSetAttribute(k_area, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

// Resident blocks per SM the register allocation must allow: 16 (64 warps,
// 32 registers) with several types, 12 (48 warps, 40 registers) for the
// pipelined one-type loop; both measured faster than the unconstrained
// allocation (44-54 registers) on the 1.5M-atom mixed system and a 1M-atom
// LJ fluid, the small spills notwithstanding.
template <bool MT, bool SG, bool WX, bool WY, bool SIG1>
__global__ void __launch_bounds__(kStepBlock, MT ? 16 : 12) k_step(DevSys s, int mode, int parity, cudaGraphConditionalHandle h,
                                                     int use_h) {
    const float2 *__restrict__ pin = parity ? s.pos1 : s.pos0;
    float2 *__restrict__ pout = parity ? s.pos0 : s.pos1;
    extern __shared__ PairEntry tab[];  // numTypes^2 entries (1 without types)
    const int nt = s.numTypes;
    if (MT) {
        for (int q = threadIdx.x; q < nt * nt; q += blockDim.x) tab[q] = s.pair[q];
    } else if (threadIdx.x == 0) {
        tab[0] = s.pair[0];
    }
    if (s.trace && blockIdx.x == 0 && threadIdx.x == 0) {
        int row = s.sc->obsRow;
        if (row < s.obsCap) s.trace[(size_t)row * kTraceCols + 2] = global_ns();
    }
    __syncthreads();

    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float ue = 0.0f, we = 0.0f, ke = 0.0f, vvm = 0.0f;
    bool bad = false;
    // one type: the four neighbour positions of a list group are gathered
    // together (measured faster on a 1M-atom LJ fluid); several types: two
    // at a time, which keeps registers low enough for the type-pair lookups
    // (115 us on the mixed system, against 118 us one at a time and 120 us
    // four at a time)
    if (i < s.N) particle_step<MT, SG, WX, WY, SIG1, true, MT ? 2 : 4>(s, tab, i, mode, pin, pout, ue, we, ke, vvm, bad);

    step_reduce<kStepBlock>(s, mode, ue, we, ke, vvm, bad, h, use_h);
}

// leapFrogStep1 + applyPBC on their own: the c_doStep entry (the step
// counter becomes stepBase + 1), or inside a run after a step that ended with
// LAST (the counter advances); the same float operations as the fused drift
// of k_step
__global__ void __launch_bounds__(kBlock) k_drift(DevSys s, int parity, int advance) {
    const float2 *pin = parity ? s.pos1 : s.pos0;
    float2 *pout = parity ? s.pos0 : s.pos1;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) s.sc->stepNow = advance ? s.sc->stepNow + 1 : s.stepBase + 1;
    if (i >= s.N) return;
    float2 v = s.vel[i], a = s.acc[i], p = pin[i];
    v.x += s.hdt * a.x;
    v.y += s.hdt * a.y;
    p.x += s.dt * v.x;
    p.y += s.dt * v.y;
    if (s.wrapx) p.x = wrap_coord(p.x, s.Lx);
    if (s.wrapy) p.y = wrap_coord(p.y, s.Ly);
    pout[i] = p;
    if (s.cposOn) (parity ? s.cpos0 : s.cpos1)[s.cslot[i]] = p;  // the fast mode's cell-ordered mirror
    s.vel[i] = v;
}

template <bool MT, bool SG, bool WX, bool WY, bool SIG1>
static cudaError_t launch_step(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h,
                               int use_h) {
    dim3 g(step_blocks(s.N)), b(kStepBlock);
    size_t smt = sizeof(PairEntry) * (size_t)(s.numTypes > 1 ? s.numTypes * s.numTypes : 1);
    return L.kernel(k_step<MT, SG, WX, WY, SIG1>, g, b, smt, s, mode, parity, h, use_h);
}

template <bool MT, bool SG, bool WX, bool WY>
static cudaError_t pick_sig(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h, int use_h) {
    if constexpr (!SG) {
        if (s.sigmaOne) return launch_step<MT, SG, WX, WY, true>(L, s, mode, parity, h, use_h);
    }
    return launch_step<MT, SG, WX, WY, false>(L, s, mode, parity, h, use_h);
}

template <bool MT, bool SG>
static cudaError_t pick_image(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h,
                              int use_h) {
    if (s.wrapx && s.wrapy) return pick_sig<MT, SG, true, true>(L, s, mode, parity, h, use_h);
    if (s.wrapx) return pick_sig<MT, SG, true, false>(L, s, mode, parity, h, use_h);
    return pick_sig<MT, SG, false, false>(L, s, mode, parity, h, use_h);
}

cudaError_t enqueue_tri(Launch &L, const DevSys &s, int parity) {
    if (s.feaForces && s.ntri > 0) return L.kernel(k_tri_forces, dim3(tri_blocks(s.ntri)), dim3(kBlock), 0, s, parity);
    return cudaSuccess;
}

cudaError_t enqueue_step(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h, int use_h) {
    cudaError_t e;
    if ((e = enqueue_tri(L, s, parity))) return e;
    return enqueue_step_after_tri(L, s, mode, parity, h, use_h);
}

cudaError_t enqueue_step_after_tri(Launch &L, const DevSys &s, int mode, int parity, cudaGraphConditionalHandle h,
                                   int use_h) {
    cudaError_t e;
    if (s.areaUnits > 0) {
        if ((e = L.kernel(k_area_keep, dim3(force_blocks(s.nPre)), dim3(kBlock), 0, s, parity))) return e;
        if ((e = L.kernel(k_area, dim3(s.areaUnits), dim3(kAreaLanes), (size_t)s.areaSmem, s, parity))) return e;
    }
    cudaEvent_t e0 = L.mark();
    if (s.fast)
        e = enqueue_step_fast(L, s, mode, parity, h, use_h);
    else if (s.numTypes > 1)
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
    return L.kernel(k_drift, dim3(force_blocks(s.N)), dim3(kBlock), 0, s, parity, 0);
}

cudaError_t enqueue_drift_in_run(Launch &L, const DevSys &s, int parity) {
    return L.kernel(k_drift, dim3(force_blocks(s.N)), dim3(kBlock), 0, s, parity, 1);
}

}  // namespace femmd
