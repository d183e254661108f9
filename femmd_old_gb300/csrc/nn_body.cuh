// nn_body.cuh -- per-particle work of the neighbour-list rebuild, shared by
// the plain kernels (k_nn.cu) and the persistent batched kernel (k_batch.cu).
//
// Reference: updateCellsCPU (femmd2D/src/nn.cpp:8-20) puts each cell's
// particles in ascending id order; buildNNCPUSerial (nn.cpp:22-62) walks the
// 3x3 stencil with dx outer, dy inner, cell indices wrapped as applyCellBC
// (nnCuda.cu:26-36), and keeps a pair when the minimum-image distance
// squared is within nnRadius^2 and the two are not in the same exclusion
// group.  The list order of every particle is that walk's order.
//
// Cells are numbered column-major (c = ix*ncy + iy): the dy = -1, 0, +1 cells
// of one stencil column are then adjacent in cellSorted, so a column is one
// contiguous range of candidates (two when it wraps in y), in the same order.
#pragma once
#include <cuda_runtime.h>
#include "femmd_internal.h"
#include "device_common.cuh"

namespace femmd {

// Place particle i at its ascending-id rank inside its cell: count the ids of
// the cell (scattered in arbitrary order by the counting sort) below i.
// Writes sortedIds and the cell-ordered float4 copy of the particle.
template <bool RO>
__device__ __forceinline__ void place_one(const DevSys &s, const float2 *pos, int i, int *bad) {
    const int c = s.cellOf[i];
    const int b = s.cellStart[c], e = s.cellStart[c + 1];
    int r = 0;
    for (int q = b; q < e; q++) r += (RO ? __ldg(s.unsorted + q) : s.unsorted[q]) < i;
    const int slot = b + r;
    if (slot >= e) {  // inconsistent cell contents: never write outside the cell
        atomicOr(bad, 2);
        return;
    }
    const float2 p = pos[i];
    const int tag = i | (s.numTypes > 1 ? (s.typeId[i] << kIdBits) : 0);
    s.sortedIds[slot] = i;
    s.cellSorted[slot] = make_float4(p.x, p.y, __int_as_float(tag), __int_as_float(s.excl[i]));
}

// Whether the fast walk below reproduces the reference's minimum image for
// every candidate: with at least 5 cells along a periodic axis and every
// position inside [0, L] there, a candidate from a neighbouring cell that did
// not wrap is closer than L/2 (no image), and one from a wrapped cell is at
// least L/2 away on the side the wrap says (exactly one shift of L).  Needs
// 3 distinct stencil cells per axis.
__device__ __forceinline__ bool fast_walk_ok(const DevSys &s) {
    return (s.wrapx ? s.ncx >= 5 : s.ncx >= 3) && (s.wrapy ? s.ncy >= 5 : s.ncy >= 3) && !s.sc->outside;
}

// One particle's list while it is written, in the packed layout of
// nbr_at: entries collect in 'buf' and leave as one 16-byte store per four
// (a quarter of the store requests of one word per entry).  Entries beyond
// the capacity (a multiple of 4) are counted by the caller, not written.
struct ListOut {
    int4 *p;     // the particle's current group of four
    int4 buf;    // the entries of the group so far, last in .w
    size_t row;  // int4 from one group of a particle to its next (Ncap)
    __device__ __forceinline__ void push(int tag, int k, int cap) {
        buf.x = buf.y;
        buf.y = buf.z;
        buf.z = buf.w;
        buf.w = tag;
        if ((k & 3) == 3 && k < cap) {
            *p = buf;
            p += row;
        }
    }
    // Store the last, partial group of a list of k entries (its unused
    // words are zero; readers stop at the count).  With k > cap (a multiple
    // of 4) every group that fits is already stored.
    __device__ __forceinline__ void finish(int k, int cap) {
        const int r = min(k, cap) & 3;
        if (r == 1)
            *p = make_int4(buf.w, 0, 0, 0);
        else if (r == 2)
            *p = make_int4(buf.z, buf.w, 0, 0);
        else if (r == 3)
            *p = make_int4(buf.y, buf.z, buf.w, 0);
    }
};

__device__ __forceinline__ ListOut list_out(const DevSys &s, int i) {
    ListOut o;
    o.p = reinterpret_cast<int4 *>(s.nbr) + i;
    o.buf = make_int4(0, 0, 0, 0);
    o.row = (size_t)s.Ncap;
    return o;
}

// A candidate is kept when within the list radius, not the particle itself
// (its tag is the particle's own: id and type), and not in the particle's
// exclusion group: gi == -1 || gj == -1 || gi != gj, which is gi == -1 ||
// gi != gj.
__device__ __forceinline__ bool walk_hit(float4 e, float sx, float sy, float2 p, int tagi, int gi, float R2) {
    const float dx = (p.x - e.x) - sx;
    const float dy = (p.y - e.y) - sy;
    const float dr2 = dx * dx + dy * dy;
    const int tag = __float_as_int(e.z);
    const int gj = __float_as_int(e.w);
    return dr2 <= R2 && tag != tagi && (gi == -1 || gi != gj);
}

// walk_hit specialised for a staged warp: EX, some lane of the warp is in an
// exclusion group (else only the self test remains); SX, the column is
// shifted by an image (else d - 0 is d itself, the same value).  Both are
// the same on every lane of a staged warp, so the warp runs one version.
template <bool EX, bool SX>
__device__ __forceinline__ bool walk_hit_t(float4 e, float sx, float2 p, int tagi, int gi, float R2) {
    const float dx = SX ? (p.x - e.x) - sx : p.x - e.x;
    const float dy = p.y - e.y;
    const float dr2 = dx * dx + dy * dy;
    const int tag = __float_as_int(e.z);
    return dr2 <= R2 && tag != tagi && (!EX || gi == -1 || gi != __float_as_int(e.w));
}

// The tag cellSorted holds for particle i (place_one).
__device__ __forceinline__ int own_tag(const DevSys &s, int i) {
    return i | (s.numTypes > 1 ? (s.typeId[i] << kIdBits) : 0);
}

// One contiguous candidate range with a known image shift (sx, sy): the
// reference's d - L / d + L is d - sx with sx = +L / -L, and d - 0 = d.
// Candidates are taken four at a time: the four loads are issued before any
// test, then the hits are appended in candidate order.
template <bool RO>
__device__ __forceinline__ void walk_range(const DevSys &s, int qb, int qe, float sx, float sy, float2 p, int tagi,
                                           int gi, float R2, int cap, ListOut &out, int &k) {
    int q = qb;
    for (; q + 4 <= qe; q += 4) {
        float4 e[4];
#pragma unroll
        for (int u = 0; u < 4; u++) e[u] = RO ? __ldg(s.cellSorted + q + u) : s.cellSorted[q + u];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (walk_hit(e[u], sx, sy, p, tagi, gi, R2)) {
                out.push(__float_as_int(e[u].z), k, cap);
                k++;
            }
        }
    }
    for (; q < qe; q++) {
        const float4 e = RO ? __ldg(s.cellSorted + q) : s.cellSorted[q];
        if (walk_hit(e, sx, sy, p, tagi, gi, R2)) {
            out.push(__float_as_int(e.z), k, cap);
            k++;
        }
    }
}

// Verlet list of particle i in the reference's order, written through out
// (the caller stores the last group with out.finish); returns its length
// (entries beyond the capacity are counted, not written).  RO: the cell
// arrays are read through the read-only path (written by an earlier
// kernel); the batched kernel rewrites them in the same launch (coherent
// loads).
template <bool RO>
__device__ __forceinline__ int build_fast_at(const DevSys &s, int i, int c, float2 p, int gi, ListOut &out) {
    const int ncx = s.ncx, ncy = s.ncy, cap = s.nbrCap;
    const float R2 = s.nnRadiusSq;
    const float Lx = s.wrapx ? s.Lx : 0.0f, Ly = s.wrapy ? s.Ly : 0.0f;
    const int ix = c / ncy, iy = c - ix * ncy;
    const int tagi = own_tag(s, i);
    int k = 0;
    const int *cs = s.cellStart;
#pragma unroll 1
    for (int dx = -1; dx <= 1; dx++) {
        int nx = ix + dx;
        float sx = 0.0f;
        if (nx < 0) {
            nx = ncx - 1;
            sx = -Lx;
        } else if (nx == ncx) {
            nx = 0;
            sx = Lx;
        }
        const int col = nx * ncy;
        if (iy > 0 && iy < ncy - 1) {
            const int qb = RO ? __ldg(cs + col + iy - 1) : cs[col + iy - 1];
            const int qe = RO ? __ldg(cs + col + iy + 2) : cs[col + iy + 2];
            walk_range<RO>(s, qb, qe, sx, 0.0f, p, tagi, gi, R2, cap, out, k);
        } else if (iy == 0) {
            // dy = -1 wraps to the top cell, then dy = 0, +1
            int qb = RO ? __ldg(cs + col + ncy - 1) : cs[col + ncy - 1];
            int qe = RO ? __ldg(cs + col + ncy) : cs[col + ncy];
            walk_range<RO>(s, qb, qe, sx, -Ly, p, tagi, gi, R2, cap, out, k);
            qb = RO ? __ldg(cs + col) : cs[col];
            qe = RO ? __ldg(cs + col + 2) : cs[col + 2];
            walk_range<RO>(s, qb, qe, sx, 0.0f, p, tagi, gi, R2, cap, out, k);
        } else {
            // dy = -1, 0, then dy = +1 wraps to the bottom cell
            int qb = RO ? __ldg(cs + col + ncy - 2) : cs[col + ncy - 2];
            int qe = RO ? __ldg(cs + col + ncy) : cs[col + ncy];
            walk_range<RO>(s, qb, qe, sx, 0.0f, p, tagi, gi, R2, cap, out, k);
            qb = RO ? __ldg(cs + col) : cs[col];
            qe = RO ? __ldg(cs + col + 1) : cs[col + 1];
            walk_range<RO>(s, qb, qe, sx, Ly, p, tagi, gi, R2, cap, out, k);
        }
    }
    return k;
}

// The walk of build_fast_at over candidates staged in shared memory: for
// stencil column d (dx = d - 1) the candidates of slots [wb[d], wb[d] +
// wl[d]) sit at cand[wo[d] + slot - wb[d]].  Same ranges, same order, same
// arithmetic as the walk over cellSorted (the rows of a staged warp never
// wrap in y: sy = 0).
template <bool EX, bool SX>
__device__ __forceinline__ void walk_staged(const float4 *cand, int lb, int le, float sx, float2 p, int tagi, int gi,
                                            float R2, int cap, ListOut &out, int &k) {
    int q = lb;
    for (; q + 4 <= le; q += 4) {
        float4 e[4];
#pragma unroll
        for (int u = 0; u < 4; u++) e[u] = cand[q + u];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (walk_hit_t<EX, SX>(e[u], sx, p, tagi, gi, R2)) {
                out.push(__float_as_int(e[u].z), k, cap);
                k++;
            }
        }
    }
    for (; q < le; q++) {
        const float4 e = cand[q];
        if (walk_hit_t<EX, SX>(e, sx, p, tagi, gi, R2)) {
            out.push(__float_as_int(e.z), k, cap);
            k++;
        }
    }
}

// The stencil of a particle whose cell row has no y-wrap (1 <= iy <= ncy -
// 2): per column d (dx = d - 1) the slot range [qb[d], qe[d]) of rows
// iy - 1 .. iy + 1 and the image shift sx[d].  Returns the columns.
__device__ __forceinline__ void stencil_columns(const DevSys &s, int ix, int iy, int *qb, int *qe, float *sx) {
    const int ncx = s.ncx, ncy = s.ncy;
    const float Lx = s.wrapx ? s.Lx : 0.0f;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        int nx = ix + d - 1;
        sx[d] = 0.0f;
        if (nx < 0) {
            nx = ncx - 1;
            sx[d] = -Lx;
        } else if (nx == ncx) {
            nx = 0;
            sx[d] = Lx;
        }
        const int col = nx * ncy;
        qb[d] = __ldg(s.cellStart + col + iy - 1);
        qe[d] = __ldg(s.cellStart + col + iy + 2);
    }
}

// build_fast_at over the three column windows staged in shared memory
// (column d's slots [wb[d], ...) at cand[wo[d] + slot - wb[d]]).
__device__ __forceinline__ int build_fast_staged(const DevSys &s, int i, float2 p, int gi, const float4 *cand,
                                                 const int *qb, const int *qe, const float *sx, const int *wb,
                                                 const int *wo, ListOut &out) {
    int k = 0;
    const int tagi = own_tag(s, i);
    const float R2 = s.nnRadiusSq;
    const int cap = s.nbrCap;
    // warp-uniform choices (the caller's staged warps are whole)
    const bool ex = __any_sync(0xffffffffu, gi != -1);
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const int lb = wo[d] + qb[d] - wb[d], le = wo[d] + qe[d] - wb[d];
        const bool shifted = sx[d] != 0.0f;  // the same on every lane: one cell column
        if (ex) {
            if (shifted)
                walk_staged<true, true>(cand, lb, le, sx[d], p, tagi, gi, R2, cap, out, k);
            else
                walk_staged<true, false>(cand, lb, le, sx[d], p, tagi, gi, R2, cap, out, k);
        } else {
            if (shifted)
                walk_staged<false, true>(cand, lb, le, sx[d], p, tagi, gi, R2, cap, out, k);
            else
                walk_staged<false, false>(cand, lb, le, sx[d], p, tagi, gi, R2, cap, out, k);
        }
    }
    return k;
}

template <bool RO>
__device__ __forceinline__ int build_fast(const DevSys &s, const float2 *pos, int i, ListOut &out) {
    return build_fast_at<RO>(s, i, s.cellOf[i], pos[i], s.excl[i], out);
}

// The general walk: any grid (1 or 2 cells along an axis visit the same cell
// more than once, as the reference does), any position, the minimum image
// decided per pair.
template <bool RO>
__device__ __forceinline__ int build_general(const DevSys &s, const float2 *pos, int i, ListOut &out) {
    int k = 0;
    const int ncx = s.ncx, ncy = s.ncy, cap = s.nbrCap;
    const bool wx = s.wrapx, wy = s.wrapy;
    const float Lx = s.Lx, Ly = s.Ly, R2 = s.nnRadiusSq;
    const int c = s.cellOf[i];
    const int ix = c / ncy, iy = c - ix * ncy;
    const float2 p = pos[i];
    const int gi = s.excl[i];
    for (int dx = -1; dx <= 1; dx++) {
        int nx = ix + dx;
        if (nx < 0) nx = ncx - 1; else if (nx == ncx) nx = 0;
        for (int dy = -1; dy <= 1; dy++) {
            int ny = iy + dy;
            if (ny < 0) ny = ncy - 1; else if (ny == ncy) ny = 0;
            const int nc = nx * ncy + ny;
            const int qb = RO ? __ldg(s.cellStart + nc) : s.cellStart[nc];
            const int qe = RO ? __ldg(s.cellStart + nc + 1) : s.cellStart[nc + 1];
            for (int q = qb; q < qe; q++) {
                const float4 e = RO ? __ldg(s.cellSorted + q) : s.cellSorted[q];
                const int tag = __float_as_int(e.z);
                const int j = tag & kIdMask;
                const int gj = __float_as_int(e.w);
                if (j != i && (gi == -1 || gj == -1 || gi != gj)) {
                    float dxr, dxo, dyr, dyo;
                    image_axis(p.x, e.x, Lx, wx, false, dxr, dxo);
                    image_axis(p.y, e.y, Ly, wy, false, dyr, dyo);
                    const float dr2 = dxr * dxr + dyr * dyr;
                    if (dr2 <= R2) {
                        out.push(tag, k, cap);
                        k++;
                    }
                }
            }
        }
    }
    return k;
}

// Position of particle i outside [0, L] on a periodic axis (only possible
// before the first step wraps it): the fast walk is then not used.
__device__ __forceinline__ bool outside_box(const DevSys &s, float2 p) {
    return (s.wrapx && !(p.x >= 0.0f && p.x <= s.Lx)) || (s.wrapy && !(p.y >= 0.0f && p.y <= s.Ly));
}

}  // namespace femmd
