// Device building blocks of the assembled 27-point block-stencil levels, shared by the
// per-colour kernels (k_coarse.cu) and the coarse-tail kernels (k_tail.cu).
#pragma once
#include <cuda_bf16.h>

#include "vfem_common.cuh"

namespace vfem {
namespace stencil {

// Stored stencil entries: the arithmetic type T itself, or bf16 for the FP32 levels of the mixed
// preconditioner (half the bytes a colour pass streams; the entries are rounded once, when the
// Galerkin operator is built, so the stored operator stays exactly symmetric).
template <typename T, typename TS>
__device__ __forceinline__ T sval(TS v) { return (T)v; }
template <>
__device__ __forceinline__ float sval<float, __nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <typename TS, typename T>
__device__ __forceinline__ TS sstore(T v) { return (TS)v; }
template <>
__device__ __forceinline__ __nv_bfloat16 sstore<__nv_bfloat16, float>(float v) { return __float2bfloat16_rn(v); }

// Node and element counts stay below 2^31 (checked when a grid is created), so index
// decodes use 32-bit unsigned division; a 64-bit division is a long software sequence.
__device__ __forceinline__ void decode(const int64_t n, const int nn1, const int nn2, int &i, int &j, int &k) {
    const uint32_t u = (uint32_t)n, t = u / (uint32_t)nn2;
    k = (int)(u - t * (uint32_t)nn2);
    const uint32_t q = t / (uint32_t)nn1;
    j = (int)(t - q * (uint32_t)nn1);
    i = (int)q;
}

// Assembled stencil rows are stored node-contiguous: the 27 blocks of node n occupy
// S[n * ROW + e], e = o*9 + 3r + c (o = (ox+1)*9 + (oy+1)*3 + (oz+1)), padded to ROW = 256
// entries (1 KB in FP32) so every row starts 16-byte aligned. One warp handles one row:
// lane l owns entries [8l, 8l+8) and a warp reduction sums the three row components, so a
// node costs one coalesced 1 KB read and a single memory round trip.
constexpr int ROW = 256;
constexpr int ROW_USED = 243;

__device__ __forceinline__ int64_t neighbour(const Geom &g, int64_t n, int i, int j, int k, int o) {
    // out-of-grid neighbours are clamped onto the node itself; their blocks are exactly zero
    // (no element contains both nodes), so they add nothing
    const int ox = o / 9 - 1, oy = (o / 3) % 3 - 1, oz = o % 3 - 1;
    const int64_t sx = (int64_t)g.nn[1] * g.nn[2], sy = g.nn[2];
    int64_t m = n;
    if ((ox < 0 && i > 0) || (ox > 0 && i + 1 < g.nn[0])) m += ox * sx;
    if ((oy < 0 && j > 0) || (oy > 0 && j + 1 < g.nn[1])) m += oy * sy;
    if ((oz < 0 && k > 0) || (oz > 0 && k + 1 < g.nn[2])) m += oz;
    return m;
}

template <typename T>
struct RowVec;
template <>
struct RowVec<float> {
    static __device__ __forceinline__ void load(const float *p, float *v) {
        const float4 a = reinterpret_cast<const float4 *>(p)[0];
        const float4 b = reinterpret_cast<const float4 *>(p)[1];
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    }
};
template <>
struct RowVec<double> {
    static __device__ __forceinline__ void load(const double *p, double *v) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double2 a = reinterpret_cast<const double2 *>(p)[q];
            v[2 * q] = a.x;
            v[2 * q + 1] = a.y;
        }
    }
};

template <typename T>
__device__ __forceinline__ T warp_reduce(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Lane-partial products of row n with u; v receives the lane's 8 row entries. The 8
// entries of a lane span at most two neighbour blocks (o_a and o_a + 1), so the lane forms
// two neighbour indices and walks its entries with a running (row, component) counter.
// After the call every lane holds the full sums (butterfly reduction).
template <typename T>
__device__ __forceinline__ void row_times_u(const Geom &g, const T *__restrict__ S, const T *__restrict__ u, int64_t n,
                                            int i, int j, int k, int lane, T *v, T &f0, T &f1, T &f2) {
    RowVec<T>::load(S + n * ROW + lane * 8, v);
    const int64_t ld = g.ld;
    const int e0 = lane * 8;
    const int oa = e0 / 9;
    const int64_t ma = neighbour(g, n, i, j, k, oa);
    const int64_t mb = oa < 26 ? neighbour(g, n, i, j, k, oa + 1) : ma;
    int rc = e0 - 9 * oa;  // position of the first entry inside its 3x3 block
    T p0 = T(0), p1 = T(0), p2 = T(0);
    bool second = false;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        if (e0 + q < ROW_USED) {
            const int r = rc / 3, c = rc - 3 * r;
            const T prod = v[q] * u[c * ld + (second ? mb : ma)];
            p0 += (r == 0) ? prod : T(0);
            p1 += (r == 1) ? prod : T(0);
            p2 += (r == 2) ? prod : T(0);
        }
        if (++rc == 9) {
            rc = 0;
            second = true;
        }
    }
    f0 = warp_reduce(p0);
    f1 = warp_reduce(p1);
    f2 = warp_reduce(p2);
}

template <typename T>
__device__ __forceinline__ void node_solve(uint8_t dm, T s0, T s1, T s2, const T *M, bool forward, T &u0, T &u1,
                                           T &u2) {
    if (dm) {
        T d[3] = {T(0), T(0), T(0)};
        const T bs[3] = {s0, s1, s2};
        if (forward) {
#pragma unroll
            for (int q = 0; q < 3; ++q)
                d[q] = (bs[q] - (M[3 * q] * d[0] + M[3 * q + 1] * d[1] + M[3 * q + 2] * d[2])) *
                       (T(!((dm >> q) & 1)) / M[4 * q]);
        } else {
#pragma unroll
            for (int q = 2; q >= 0; --q)
                d[q] = (bs[q] - (M[3 * q] * d[0] + M[3 * q + 1] * d[1] + M[3 * q + 2] * d[2])) *
                       (T(!((dm >> q) & 1)) / M[4 * q]);
        }
        u0 += d[0];
        u1 += d[1];
        u2 += d[2];
    } else {
        const T c00 = M[4] * M[8] - M[5] * M[7];
        const T c01 = M[5] * M[6] - M[3] * M[8];
        const T c02 = M[3] * M[7] - M[4] * M[6];
        const T det = M[0] * c00 + M[1] * c01 + M[2] * c02;
        const T id = T(1) / det;
        const T i00 = c00 * id, i01 = (M[2] * M[7] - M[1] * M[8]) * id, i02 = (M[1] * M[5] - M[2] * M[4]) * id;
        const T i10 = c01 * id, i11 = (M[0] * M[8] - M[2] * M[6]) * id, i12 = (M[2] * M[3] - M[0] * M[5]) * id;
        const T i20 = c02 * id, i21 = (M[1] * M[6] - M[0] * M[7]) * id, i22 = (M[0] * M[4] - M[1] * M[3]) * id;
        u0 += i00 * s0 + i01 * s1 + i02 * s2;
        u1 += i10 * s0 + i11 * s1 + i12 * s2;
        u2 += i20 * s0 + i21 * s1 + i22 * s2;
    }
}


// Block Gauss-Seidel update of node (i, j, k) by one warp (MultigridSolver.hh:323-378).
template <typename T>
__device__ __forceinline__ void gs_node_warp(const Geom &g, const T *__restrict__ S, T *u, const T *__restrict__ b,
                                             const uint8_t *__restrict__ dmask, int i, int j, int k, bool forward,
                                             int lane) {
    const int64_t n = g.node(i, j, k), ld = g.ld;
    const uint8_t dm = dmask[n];
    if (dm == 7) return;  // warp-uniform
    T v[8], f0, f1, f2;
    row_times_u<T>(g, S, u, n, i, j, k, lane, v, f0, f1, f2);
    // diagonal block entries 117..125 live in lanes 14 and 15
    T M[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) M[q] = __shfl_sync(0xffffffffu, v[(117 + q) % 8], (117 + q) / 8);
    if (lane == 0) {
        T u0 = u[n], u1 = u[ld + n], u2 = u[2 * ld + n];
        node_solve<T>(dm, b[n] - f0, b[ld + n] - f1, b[2 * ld + n] - f2, M, forward, u0, u1, u2);
        u[n] = u0;
        u[ld + n] = u1;
        u[2 * ld + n] = u2;
    }
}

// r = b - S u on nondetached rows, r = b elsewhere; Dirichlet components zeroed (one warp).
template <typename T>
__device__ __forceinline__ void residual_node_warp(const Geom &g, const T *__restrict__ S, const T *__restrict__ u,
                                                   const T *__restrict__ b, T *__restrict__ r,
                                                   const uint8_t *__restrict__ dmask, int64_t n, int i, int j, int k,
                                                   int lane) {
    const int64_t ld = g.ld;
    T f0 = T(0), f1 = T(0), f2 = T(0);
    if (j < g.nyv()) {
        T v[8];
        row_times_u<T>(g, S, u, n, i, j, k, lane, v, f0, f1, f2);
    }
    if (lane == 0) {
        const uint8_t dm = dmask[n];
        r[n] = (dm & 1) ? T(0) : b[n] - f0;
        r[ld + n] = (dm & 2) ? T(0) : b[ld + n] - f1;
        r[2 * ld + n] = (dm & 4) ? T(0) : b[2 * ld + n] - f2;
    }
}


// ---- plane layout (large levels): S[((o - 13)*9 + 3r + c) * ld + p], one thread per node ----
// p is the node's colour-ordered position: nodes grouped by colour (i&1, j&1, k&1), colours in
// ascending order 4cx+2cy+cz, each colour's nodes in lexicographic (i>>1, j>>1, k>>1) order.
// A Gauss-Seidel colour pass then streams a contiguous slice of every plane. The Galerkin
// operator is symmetric, so only the blocks of offsets o = 13..26 (the diagonal and the upper
// half) are stored: block (n, n + d_o) for o < 13 is the transpose of block (m, m + d_(26-o)) of
// the neighbour m = n + d_o, read at m's position. The neighbours of a warp's consecutive
// colour positions are consecutive positions of the neighbour colour, so those reads coalesce.
constexpr int HALF_OFFSETS = 14;
constexpr int PLANES = HALF_OFFSETS * 9;  // stored entries per node (STENCIL_PLANES)
__device__ __forceinline__ int half_count(int nn, int b) { return (nn + 1 - b) >> 1; }

__device__ __forceinline__ int64_t colour_pos(const Geom &g, int i, int j, int k) {
    const int cy = j & 1, cz = k & 1;
    return g.coff[4 * (i & 1) + 2 * cy + cz] + ((int64_t)(i >> 1) * g.hc1[cy] + (j >> 1)) * g.hc2[cz] + (k >> 1);
}

__device__ __forceinline__ void colour_node(const Geom &g, int64_t p, int &i, int &j, int &k) {
    const int64_t A = (int64_t)half_count(g.nn[0], 0) * g.nn[1] * g.nn[2];
    const int cx = p >= A;
    if (cx) p -= A;
    const int64_t B = (int64_t)half_count(g.nn[0], cx) * half_count(g.nn[1], 0) * g.nn[2];
    const int cy = p >= B;
    if (cy) p -= B;
    const int c1 = half_count(g.nn[1], cy);
    const int64_t C = (int64_t)half_count(g.nn[0], cx) * c1 * half_count(g.nn[2], 0);
    const int cz = p >= C;
    if (cz) p -= C;
    const int c2 = half_count(g.nn[2], cz);
    int ii, jj, kk;
    decode(p, c1, c2, ii, jj, kk);
    i = 2 * ii + cx;
    j = 2 * jj + cy;
    k = 2 * kk + cz;
}

// Split form for the plane layout: a block of SPLIT_SUB warps works on 32 nodes (lane =
// node). Row warps w = 1..SPLIT_ROWS sum the neighbour blocks o = w-1, w-1+7, w-1+14, w-1+21
// of their lane's node, issuing all of their loads before any arithmetic; warp 0 meanwhile
// loads the node's own data (right-hand side, iterate, diagonal block) and, after the
// barrier, combines the partial sums in a fixed order and finishes the node. Eight times as
// many threads as nodes keep enough loads in flight for a colour pass over a few tens of
// thousands of nodes.
constexpr int SPLIT_SUB = 8;
constexpr int SPLIT_ROWS = SPLIT_SUB - 1;
constexpr int SPLIT_NODES = 32;

template <typename T, typename TS = T>
__device__ __forceinline__ void stencil_row_part(const Geom &g, const TS *__restrict__ S, const T *__restrict__ u,
                                                 int64_t n, int64_t p, int i, int j, int k, int sub, T &f0, T &f1,
                                                 T &f2) {  // sub in [0, SPLIT_ROWS)
    const int64_t ld = g.ld;
    const int64_t sx = (int64_t)g.nn[1] * g.nn[2], sy = g.nn[2];
    T uu[4][3], ss[4][9];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const int o = sub + SPLIT_ROWS * t;
        if (o < 27) {
            const int ox = o / 9 - 1, oy = (o / 3) % 3 - 1, oz = o % 3 - 1;
            // a neighbour outside the grid has a zero block; read the node itself instead
            const bool in = (unsigned)(i + ox) < (unsigned)g.nn[0] && (unsigned)(j + oy) < (unsigned)g.nn[1] &&
                            (unsigned)(k + oz) < (unsigned)g.nn[2];
            const int64_t m = in ? n + ox * sx + oy * sy + oz : n;
#pragma unroll
            for (int c = 0; c < 3; ++c) uu[t][c] = u[c * ld + m];
            if (o >= 13) {
                const TS *blk = S + (int64_t)((o - 13) * 9) * ld + p;
#pragma unroll
                for (int e = 0; e < 9; ++e) ss[t][e] = sval<T>(blk[e * ld]);
            } else if (in) {
                // transpose of the neighbour's block towards this node (offset 26 - o)
                const TS *blk = S + (int64_t)((13 - o) * 9) * ld + colour_pos(g, i + ox, j + oy, k + oz);
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c) ss[t][3 * r + c] = sval<T>(blk[(3 * c + r) * ld]);
            } else {
#pragma unroll
                for (int e = 0; e < 9; ++e) ss[t][e] = T(0);
            }
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c) uu[t][c] = T(0);
#pragma unroll
            for (int e = 0; e < 9; ++e) ss[t][e] = T(0);
        }
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        f0 += ss[t][0] * uu[t][0] + ss[t][1] * uu[t][1] + ss[t][2] * uu[t][2];
        f1 += ss[t][3] * uu[t][0] + ss[t][4] * uu[t][1] + ss[t][5] * uu[t][2];
        f2 += ss[t][6] * uu[t][0] + ss[t][7] * uu[t][1] + ss[t][8] * uu[t][2];
    }
}

// Sum of the SPLIT_ROWS partials of lane `lane` (fixed order); part is [3][SPLIT_ROWS][32].
template <typename T>
__device__ __forceinline__ void split_sum(const T (*part)[SPLIT_ROWS][SPLIT_NODES], int lane, T &f0, T &f1, T &f2) {
    f0 = f1 = f2 = T(0);
#pragma unroll
    for (int w = 0; w < SPLIT_ROWS; ++w) {
        f0 += part[0][w][lane];
        f1 += part[1][w][lane];
        f2 += part[2][w][lane];
    }
}

// Full-weighting restriction onto coarse node (i, j, k) (MultigridSolver.hh:217-275); rows at or
// above the coarse nondetached height get zero.
template <typename T>
__device__ __forceinline__ void restrict_node(const Geom &gf, const Geom &gc, const T *__restrict__ fine,
                                              T *__restrict__ coarse, int i, int j, int k) {
    const int64_t cn = gc.node(i, j, k);
    T v0 = T(0), v1 = T(0), v2 = T(0);
    if (j < gc.nyv()) {
        const int fyv = gf.nyv();
        const int lo0 = max(2 * i - 1, 0), lo1 = max(2 * j - 1, 0), lo2 = max(2 * k - 1, 0);
        const int hi0 = min(2 * i + 2, gf.nn[0]), hi1 = min(2 * j + 2, fyv), hi2 = min(2 * k + 2, gf.nn[2]);
        const int64_t ld = gf.ld;
        for (int a = lo0; a < hi0; ++a) {
            const T wa = T(1) - T(abs(a - 2 * i)) * T(0.5);
            for (int bb = lo1; bb < hi1; ++bb) {
                const T wb = wa * (T(1) - T(abs(bb - 2 * j)) * T(0.5));
                for (int c = lo2; c < hi2; ++c) {
                    const T w = wb * (T(1) - T(abs(c - 2 * k)) * T(0.5));
                    const int64_t fn = gf.node(a, bb, c);
                    v0 += w * fine[fn];
                    v1 += w * fine[ld + fn];
                    v2 += w * fine[2 * ld + fn];
                }
            }
        }
    }
    coarse[cn] = v0;
    coarse[gc.ld + cn] = v1;
    coarse[2 * gc.ld + cn] = v2;
}

// Trilinear prolongation into fine node f (MultigridSolver.hh:163-212).
template <typename T, bool Accumulate>
__device__ __forceinline__ void interp_node(const Geom &gf, const Geom &gc, const T *__restrict__ coarse,
                                            T *__restrict__ fine, const int f[3]) {
    int ec[3], lf[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        ec[d] = min(f[d] / 2, gc.ne[d]);
        lf[d] = f[d] - 2 * ec[d];
    }
    const int64_t fn = gf.node(f[0], f[1], f[2]);
    const int64_t fld = gf.ld, cld = gc.ld;
    T a0 = Accumulate ? fine[fn] : T(0), a1 = Accumulate ? fine[fld + fn] : T(0),
      a2 = Accumulate ? fine[2 * fld + fn] : T(0);
#pragma unroll
    for (int cnl = 0; cnl < 8; ++cnl) {
        const int cb[3] = {(cnl >> 2) & 1, (cnl >> 1) & 1, cnl & 1};
        T coeff = T(1);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const T phi = (lf[d] == 1) ? T(0.5) : ((lf[d] == 0) ? (cb[d] ? T(0) : T(1)) : (cb[d] ? T(1) : T(0)));
            coeff *= phi;
        }
        if (coeff == T(0)) continue;
        const int64_t cidx = gc.node(ec[0] + cb[0], ec[1] + cb[1], ec[2] + cb[2]);
        a0 += coeff * coarse[cidx];
        a1 += coeff * coarse[cld + cidx];
        a2 += coeff * coarse[2 * cld + cidx];
    }
    fine[fn] = a0;
    fine[fld + fn] = a1;
    fine[2 * fld + fn] = a2;
}

}  // namespace stencil
}  // namespace vfem
