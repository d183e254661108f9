// device_common.cuh -- device helpers shared by the kernels.  All arithmetic
// here is single-rounding IEEE (the library is compiled with -fmad=false, so
// nothing is contracted into FMA) and follows the reference's operation order
// where the reference defines one.
#pragma once
#include <cuda_runtime.h>
#include "femmd_internal.h"

namespace femmd {

// Knuth TwoSum error of s = a + b: a + b == s + err exactly.
__device__ __forceinline__ float two_sum_err(float a, float b, float s) {
    float bb = s - a;
    float t = s - bb;
    return (a - t) + (b - bb);
}

// minImage for one axis (femmd2D/src/def.h:91-93).  'ref' is the reference's
// float result; 'out' is the same difference rounded once from its exact
// value when 'exact' is set (a cross-boundary difference a - b - L otherwise
// carries the rounding of a - b, up to half an ulp of L).
__device__ __forceinline__ void image_axis(float a, float b, float L, bool wraps, bool exact, float &ref,
                                           float &out) {
    float d = a - b;
    ref = d;
    out = d;
    if (wraps) {
        if (d >= 0.5f * L) {
            float r = d - L;
            ref = r;
            out = exact ? r + two_sum_err(a, -b, d) : r;
        } else if (d < -0.5f * L) {
            float r = d + L;
            ref = r;
            out = exact ? r + two_sum_err(a, -b, d) : r;
        }
    }
}

// a - b + k L rounded once from the exact value (triangle unwrap, exact mode).
__device__ __forceinline__ float diff_shift(float a, float b, int k, float L) {
    float d = a - b;
    if (k == 0) return d;
    float e = two_sum_err(a, -b, d);
    float t = d + (float)k * L;
    return t + e;
}

// pbcCalc (femmd2D/src/def.h:112)
__device__ __forceinline__ float wrap_coord(float r, float L) { return r - floorf(r / L) * L; }

// cellId (femmd2D/src/nnCuda.cu:9-17): float multiply, IEEE divide, truncate;
// an index equal to the cell count is moved into the last cell.  Indices
// outside the grid (only reachable on a non-periodic axis, where the
// reference reads out of bounds) are clamped.
__device__ __forceinline__ void cell_xy(float x, float y, int ncx, int ncy, float Lx, float Ly, int &ix, int &iy) {
    ix = (int)(x * (float)ncx / Lx);
    if (ix == ncx) ix -= 1;
    iy = (int)(y * (float)ncy / Ly);
    if (iy == ncy) iy -= 1;
    ix = ix < 0 ? 0 : (ix >= ncx ? ncx - 1 : ix);
    iy = iy < 0 ? 0 : (iy >= ncy ? ncy - 1 : iy);
}

// the reference's row-major cell index ix + iy*ncx
__device__ __forceinline__ int cell_of(float x, float y, int ncx, int ncy, float Lx, float Ly) {
    int ix, iy;
    cell_xy(x, y, ncx, ncy, Lx, Ly, ix, iy);
    return ix + iy * ncx;
}

// the column-major index ix*ncy + iy used by the list build
__device__ __forceinline__ int cell_col(float x, float y, int ncx, int ncy, float Lx, float Ly) {
    int ix, iy;
    cell_xy(x, y, ncx, ncy, Lx, Ly, ix, iy);
    return ix * ncy + iy;
}

// Natural log by fdlibm-style reduction x = 2^k m, m in [sqrt(1/2), sqrt(2)),
// s = f/(2+f) with f = m-1, log(m) = f - s (f - R(s^2)), R from the Taylor
// series of 2 atanh(s); error within 2 ulp, and the same bits on host and device.
__device__ __forceinline__ float own_logf(float x) {
    if (!(x > 0.0f) || !(x < INFINITY)) return logf(x);
    unsigned u = __float_as_uint(x);
    int k = 0;
    if (u < 0x00800000u) {
        u = __float_as_uint(x * 16777216.0f);
        k = -24;
    }
    k += (int)((u >> 23) & 0xff) - 127;
    float m = __uint_as_float((u & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        k += 1;
    }
    float f = m - 1.0f;
    float s = f / (2.0f + f);
    float z = s * s;
    float R = z * (0.6666666666666666f + z * (0.4f + z * (0.2857142857142857f + z * 0.2222222222222222f)));
    float lm = f - s * (f - R);
    const float ln2_hi = 0.693145751953125f;
    const float ln2_lo = 1.428606765330187e-06f;
    float fk = (float)k;
    return (fk * ln2_lo + lm) + fk * ln2_hi;
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// float -> kFixFrac fixed point; sets *bad when out of range or not finite
__device__ __forceinline__ unsigned long long to_fixed(float x, bool &bad) {
    if (!(fabsf(x) < 549755813888.0f)) {  // 2^39
        bad = true;
        return 0ull;
    }
    return (unsigned long long)__float2ll_rn(x * (float)(1 << kFixFrac));
}
__device__ __forceinline__ double from_fixed(unsigned long long v) {
    return (double)(long long)v * (1.0 / (double)(1 << kFixFrac));
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_sum_int(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ int warp_max_int(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

}  // namespace femmd
