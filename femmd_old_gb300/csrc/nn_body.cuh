// nn_body.cuh -- per-cell and per-particle work of the neighbour-list rebuild,
// shared by the plain kernels (k_nn.cu) and the persistent batched kernel
// (k_batch.cu).  Reference: updateCellsCPU (femmd2D/src/nn.cpp:8-20) order
// inside a cell, buildNNCPUSerial (nn.cpp:22-62) with applyCellBC
// (nnCuda.cu:26-36).
#pragma once
#include <cuda_runtime.h>
#include "femmd_internal.h"
#include "device_common.cuh"

namespace femmd {

// Sort cell c's particle ids ascending, write its cellSorted entries and
// return the candidate count of its 3x3 stencil.
__device__ __forceinline__ int sort_cell(const DevSys &s, const float2 *pos, int c) {
    int cand = 0;
    int b = s.cellStart[c], e = s.cellStart[c + 1], n = e - b;
    int *ids = s.sortedIds + b;
    // Shell sort with gaps 3h+1 ending in insertion sort (a cell holds a
    // handful of particles; the gaps bound the work of crowded cells)
    int gap = 1;
    while (gap < n / 3) gap = 3 * gap + 1;
    for (; gap > 0; gap /= 3) {
        for (int k = gap; k < n; k++) {
            int v = ids[k];
            int m = k - gap;
            while (m >= 0 && ids[m] > v) {
                ids[m + gap] = ids[m];
                m -= gap;
            }
            ids[m + gap] = v;
        }
    }
    for (int k = 0; k < n; k++) {
        int id = ids[k];
        float2 p = pos[id];
        int tag = id | (s.numTypes > 1 ? (s.typeId[id] << kIdBits) : 0);
        s.cellSorted[b + k] = make_float4(p.x, p.y, __int_as_float(tag), __int_as_float(s.excl[id]));
    }
    // candidate count of the 3x3 stencil (capacity sizing)
    int cy = c / s.ncx, cx = c - cy * s.ncx;
    for (int dx = -1; dx <= 1; dx++)
        for (int dy = -1; dy <= 1; dy++) {
            int nx = cx + dx, ny = cy + dy;
            if (nx < 0) nx = s.ncx - 1; else if (nx == s.ncx) nx = 0;
            if (ny < 0) ny = s.ncy - 1; else if (ny == s.ncy) ny = 0;
            int nc = nx + ny * s.ncx;
            cand += s.cellStart[nc + 1] - s.cellStart[nc];
        }
    return cand;
}

// Verlet list of particle i in the reference's order; returns its length
// (entries beyond the capacity are counted, not written).  RO: the cell
// arrays are read through the read-only path (they were written by an
// earlier kernel); the batched kernel rewrites them in the same launch and
// reads them with coherent loads.
template <bool RO>
__device__ __forceinline__ int build_one(const DevSys &s, const float2 *pos, int i) {
    int k = 0;
    const int ncx = s.ncx, ncy = s.ncy, cap = s.nbrCap, Ncap = s.Ncap;
    const bool wx = s.wrapx, wy = s.wrapy;
    const float Lx = s.Lx, Ly = s.Ly, R2 = s.nnRadiusSq;
    int c = s.cellOf[i];
    int cy0 = c / ncx, cx0 = c - cy0 * ncx;
    float2 p = pos[i];
    int gi = s.excl[i];
    int *out = s.nbr + i;
    for (int dx = -1; dx <= 1; dx++) {
        int nx = cx0 + dx;
        if (nx < 0) nx = ncx - 1; else if (nx == ncx) nx = 0;
        for (int dy = -1; dy <= 1; dy++) {
            int ny = cy0 + dy;
            if (ny < 0) ny = ncy - 1; else if (ny == ncy) ny = 0;
            int nc = nx + ny * ncx;
            int qb = RO ? __ldg(s.cellStart + nc) : s.cellStart[nc];
            int qe = RO ? __ldg(s.cellStart + nc + 1) : s.cellStart[nc + 1];
            for (int q = qb; q < qe; q++) {
                float4 e = RO ? __ldg(s.cellSorted + q) : s.cellSorted[q];
                int tag = __float_as_int(e.z);
                int j = tag & kIdMask;
                int gj = __float_as_int(e.w);
                if (j != i && (gi == -1 || gj == -1 || gi != gj)) {
                    float dxr, dxo, dyr, dyo;
                    image_axis(p.x, e.x, Lx, wx, false, dxr, dxo);
                    image_axis(p.y, e.y, Ly, wy, false, dyr, dyo);
                    float dr2 = dxr * dxr + dyr * dyr;
                    if (dr2 <= R2) {
                        if (k < cap) out[(size_t)k * Ncap] = tag;
                        k++;
                    }
                }
            }
        }
    }
    s.nbrCount[i] = k;
    return k;
}

}  // namespace femmd
