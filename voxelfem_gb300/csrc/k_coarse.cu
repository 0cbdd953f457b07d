// Coarse-level kernels: assembled 27-point block stencils (the reference's blockK,
// TensorProductSimulator.hh:885-930), full-weighting restriction and trilinear
// prolongation (MultigridSolver.hh:163-275) and Galerkin coarsening of element
// matrices (MultigridSolver.hh:712-819).
//
// Stencil layouts, block (n, n+o)(r, c) with o = (ox+1)*9 + (oy+1)*3 + (oz+1) (ascending
// neighbour index, the order of the reference's CSC columns):
//  * rows (small levels): S[n * 256 + o*9 + 3r + c], node-contiguous, padded to 256 entries;
//    one warp per node;
//  * planes (large levels): S[(o*9 + 3r + c) * NN + p], p the node's colour-ordered position
//    (stencil::colour_pos); one thread per node, and a colour pass reads contiguous slices.
// Element-matrix layout (levels >= 1): Ke[e*576 + 24*row + col].
#include <algorithm>
#include <type_traits>

#include "vfem_kernels.hpp"
#include "vfem_reduce.cuh"
#include "vfem_stencil.cuh"

namespace vfem {

namespace {

constexpr int BS = 256;
using stencil::decode;
using stencil::node_solve;
using stencil::ROW;
constexpr int WPB = BS / 32;  // warps (rows) per block

template <typename T, bool ZeroInit, bool Negate>
__global__ void __launch_bounds__(BS) stencil_apply_kernel(Geom g, const T *__restrict__ S, const T *__restrict__ u,
                                                           T *__restrict__ out) {
    VFEM_PDL_ENTRY();
    const int lane = threadIdx.x & 31;
    const int64_t n = blockIdx.x * (int64_t)WPB + (threadIdx.x >> 5);
    if (n >= g.NN) return;
    int i, j, k;
    decode(n, g.nn[1], g.nn[2], i, j, k);
    T v[8], f0, f1, f2;
    stencil::row_times_u<T>(g, S, u, n, i, j, k, lane, v, f0, f1, f2);
    if (lane == 0) {
        const int64_t ld = g.ld;
        const T s = Negate ? T(-1) : T(1);
        out[n] = (ZeroInit ? T(0) : out[n]) + s * f0;
        out[ld + n] = (ZeroInit ? T(0) : out[ld + n]) + s * f1;
        out[2 * ld + n] = (ZeroInit ? T(0) : out[2 * ld + n]) + s * f2;
    }
}

template <typename T>
__global__ void __launch_bounds__(BS) stencil_residual_kernel(Geom g, const T *__restrict__ S, const T *__restrict__ u,
                                                              const T *__restrict__ b, T *__restrict__ r,
                                                              const uint8_t *__restrict__ dmask) {
    VFEM_PDL_ENTRY();
    const int lane = threadIdx.x & 31;
    const int64_t n = blockIdx.x * (int64_t)WPB + (threadIdx.x >> 5);
    if (n >= g.NN) return;
    int i, j, k;
    decode(n, g.nn[1], g.nn[2], i, j, k);
    stencil::residual_node_warp<T>(g, S, u, b, r, dmask, n, i, j, k, lane);
}

// Block Gauss-Seidel colour pass from stencil rows (MultigridSolver.hh:323-334, 348-378),
// one warp per node of the colour.
template <typename T>
__global__ void __launch_bounds__(BS) gs_stencil_color_kernel(Geom g, const T *__restrict__ S, T *u,
                                                              const T *__restrict__ b,
                                                              const uint8_t *__restrict__ dmask, int cx, int cy,
                                                              int cz, int forward) {
    VFEM_PDL_ENTRY();
    // colour nodes over the full grid; detached rows (j >= nyv) are skipped
    const int n2 = (g.nn[2] - cz + 1) / 2, n1 = (g.nn[1] - cy + 1) / 2, n0 = (g.nn[0] - cx + 1) / 2;
    const int lane = threadIdx.x & 31;
    const int64_t t = blockIdx.x * (int64_t)WPB + (threadIdx.x >> 5);
    if (n1 <= 0 || t >= (int64_t)n0 * n1 * n2) return;
    int ii, jj, kk;
    decode(t, n1, n2, ii, jj, kk);
    if (cy + 2 * jj >= g.nyv()) return;
    stencil::gs_node_warp<T>(g, S, u, b, dmask, cx + 2 * ii, cy + 2 * jj, cz + 2 * kk, forward != 0, lane);
}

// Plane-layout kernels: blocks of SPLIT_SUB warps x 32 nodes (stencil::stencil_row_part).
// Apply / residual walk the colour-ordered positions p; a Gauss-Seidel colour pass walks the
// nodes of one colour, whose positions are contiguous. Warp 0 and the row warps take separate
// branches that meet at one named barrier (bar.sync counts arrivals from either site), so
// the registers warp 0 holds across the barrier do not add to the row warps' live set.
using stencil::SPLIT_NODES;
using stencil::SPLIT_ROWS;
using stencil::SPLIT_SUB;
constexpr int SPLIT_BS = SPLIT_SUB * SPLIT_NODES;

__device__ __forceinline__ void split_barrier() { asm volatile("bar.sync 1, %0;" ::"n"(SPLIT_BS) : "memory"); }

template <typename T, typename TS>
__device__ __forceinline__ void split_rows(const Geom &g, const TS *__restrict__ S, const T *__restrict__ u,
                                           int64_t n, int64_t p, int i, int j, int k, bool active, int sub, int lane,
                                           T (*part)[SPLIT_ROWS][SPLIT_NODES]) {
    T f0 = T(0), f1 = T(0), f2 = T(0);
    if (active) stencil::stencil_row_part<T, TS>(g, S, u, n, p, i, j, k, sub - 1, f0, f1, f2);
    part[0][sub - 1][lane] = f0;
    part[1][sub - 1][lane] = f1;
    part[2][sub - 1][lane] = f2;
    split_barrier();
}

template <typename T, typename TS, bool ZeroInit, bool Negate>
__global__ void __launch_bounds__(SPLIT_BS, sizeof(T) == 4 ? 4 : 2)
    stencil_apply_soa_kernel(Geom g, const TS *__restrict__ S, const T *__restrict__ u, T *__restrict__ out) {
    VFEM_PDL_ENTRY();
    __shared__ T part[3][SPLIT_ROWS][SPLIT_NODES];
    const int lane = threadIdx.x & 31, sub = threadIdx.x >> 5;
    const int64_t p = blockIdx.x * (int64_t)SPLIT_NODES + lane;
    const bool valid = p < g.NN;
    int i = 0, j = 0, k = 0;
    if (valid) stencil::colour_node(g, p, i, j, k);
    const int64_t n = g.node(i, j, k), ld = g.ld;
    if (sub > 0) {
        split_rows<T, TS>(g, S, u, n, p, i, j, k, valid, sub, lane, part);
        return;
    }
    T o[3] = {T(0), T(0), T(0)};
    if (valid && !ZeroInit) {
#pragma unroll
        for (int c = 0; c < 3; ++c) o[c] = out[c * ld + n];
    }
    split_barrier();
    if (!valid) return;
    T f0, f1, f2;
    stencil::split_sum<T>(part, lane, f0, f1, f2);
    if (Negate) { f0 = -f0; f1 = -f1; f2 = -f2; }
    out[n] = o[0] + f0;
    out[ld + n] = o[1] + f1;
    out[2 * ld + n] = o[2] + f2;
}

template <typename T, typename TS>
__global__ void __launch_bounds__(SPLIT_BS, sizeof(T) == 4 ? 4 : 2)
    stencil_residual_soa_kernel(Geom g, const TS *__restrict__ S, const T *__restrict__ u, const T *__restrict__ b,
                                T *__restrict__ r, const uint8_t *__restrict__ dmask) {
    VFEM_PDL_ENTRY();
    __shared__ T part[3][SPLIT_ROWS][SPLIT_NODES];
    const int lane = threadIdx.x & 31, sub = threadIdx.x >> 5;
    const int64_t p = blockIdx.x * (int64_t)SPLIT_NODES + lane;
    const bool valid = p < g.NN;
    int i = 0, j = 0, k = 0;
    if (valid) stencil::colour_node(g, p, i, j, k);
    const int64_t n = g.node(i, j, k), ld = g.ld;
    if (sub > 0) {
        split_rows<T, TS>(g, S, u, n, p, i, j, k, valid && j < g.nyv(), sub, lane, part);
        return;
    }
    T bb[3] = {T(0), T(0), T(0)};
    uint8_t dm = 7;
    if (valid) {
        dm = dmask[n];
#pragma unroll
        for (int c = 0; c < 3; ++c) bb[c] = b[c * ld + n];
    }
    split_barrier();
    if (!valid) return;
    T f0, f1, f2;
    stencil::split_sum<T>(part, lane, f0, f1, f2);
    r[n] = (dm & 1) ? T(0) : bb[0] - f0;
    r[ld + n] = (dm & 2) ? T(0) : bb[1] - f1;
    r[2 * ld + n] = (dm & 4) ? T(0) : bb[2] - f2;
}

template <typename T, typename TS>
__global__ void __launch_bounds__(SPLIT_BS, sizeof(T) == 4 ? 4 : 2)
    gs_stencil_color_soa_kernel(Geom g, const TS *__restrict__ S, T *u, const T *__restrict__ b,
                                const uint8_t *__restrict__ dmask, int cx, int cy, int cz, int forward) {
    VFEM_PDL_ENTRY();
    __shared__ T part[3][SPLIT_ROWS][SPLIT_NODES];
    // colour nodes over the full grid; detached rows (j >= nyv) are skipped
    const int n2 = (g.nn[2] - cz + 1) / 2, n1 = (g.nn[1] - cy + 1) / 2, n0 = (g.nn[0] - cx + 1) / 2;
    const int lane = threadIdx.x & 31, sub = threadIdx.x >> 5;
    const int64_t t = blockIdx.x * (int64_t)SPLIT_NODES + lane;
    bool valid = n1 > 0 && t < (int64_t)n0 * n1 * n2;
    int i = cx, j = cy, k = cz;
    if (valid) {
        int ii, jj, kk;
        decode(t, n1, n2, ii, jj, kk);
        i = cx + 2 * ii;
        j = cy + 2 * jj;
        k = cz + 2 * kk;
        valid = j < g.nyv();
    }
    const int64_t n = g.node(i, j, k), ld = g.ld;
    const int64_t p = stencil::colour_pos(g, i, j, k);
    if (sub > 0) {
        split_rows<T, TS>(g, S, u, n, p, i, j, k, valid, sub, lane, part);
        return;
    }
    T M[9], bb[3], uu[3];
    uint8_t dm = 7;
    if (valid) {
        dm = dmask[n];
#pragma unroll
        for (int e = 0; e < 9; ++e) M[e] = stencil::sval<T>(S[(int64_t)e * ld + p]);  // diagonal block (offset 13)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            bb[c] = b[c * ld + n];
            uu[c] = u[c * ld + n];
        }
    }
    split_barrier();
    if (!valid || dm == 7) return;
    T f0, f1, f2;
    stencil::split_sum<T>(part, lane, f0, f1, f2);
    stencil::node_solve<T>(dm, bb[0] - f0, bb[1] - f1, bb[2] - f2, M, forward != 0, uu[0], uu[1], uu[2]);
    u[n] = uu[0];
    u[ld + n] = uu[1];
    u[2 * ld + n] = uu[2];
}

// Line-pair colour passes on a plane-layout level: colours (cx, cy, 0) and (cx, cy, 1), adjacent
// in the reference's order, in one launch (z parity 0 then 1 forward, 1 then 0 backward). Among
// the nodes these two colours update, a node's stencil reaches only its own z-line, so each
// block owns linesPerBlock whole lines of the class and runs the first colour's nodes on them,
// a block barrier, then the second colour's; nodes go 32 at a time through the split form of
// gs_stencil_color_soa_kernel (same partial sums, same order, so the iterates are identical).
// Four launches per sweep instead of eight: the small levels' passes are launch-latency bound.
template <typename T, typename TS>
__global__ void __launch_bounds__(SPLIT_BS, sizeof(T) == 4 ? 4 : 2)
    gs_stencil_lines_soa_kernel(Geom g, const TS *__restrict__ S, T *u, const T *__restrict__ b,
                                const uint8_t *__restrict__ dmask, int cx, int cy, int linesPerBlock, int forward) {
    VFEM_PDL_ENTRY();
    __shared__ T part[3][SPLIT_ROWS][SPLIT_NODES];
    const int n1 = (g.nn[1] - cy + 1) / 2, n0 = (g.nn[0] - cx + 1) / 2;
    const int nlines = n0 * n1;
    const int l0 = (int)blockIdx.x * linesPerBlock;
    const int nl = max(0, min(linesPerBlock, nlines - l0));
    const int lane = threadIdx.x & 31, sub = threadIdx.x >> 5;
    const int nyv = g.nyv();
    const int64_t ld = g.ld;
#pragma unroll 1
    for (int s = 0; s < 2; ++s) {
        const int cz = forward ? s : 1 - s;
        const int nk = (g.nn[2] - cz + 1) / 2;
        const int cnt = nl * nk;
        for (int base = 0; base < cnt; base += SPLIT_NODES) {  // block-uniform trip count
            const int t = base + lane;
            bool valid = t < cnt;
            int i = cx, j = cy, k = cz;
            if (valid) {
                const int q = t / nk, kk = t - q * nk;
                const int line = l0 + q;
                const int ii = line / n1, jj = line - ii * n1;
                i = cx + 2 * ii;
                j = cy + 2 * jj;
                k = cz + 2 * kk;
                valid = j < nyv;
            }
            const int64_t n = g.node(i, j, k);
            const int64_t p = stencil::colour_pos(g, i, j, k);
            if (sub > 0) {
                T f0 = T(0), f1 = T(0), f2 = T(0);
                if (valid) stencil::stencil_row_part<T, TS>(g, S, u, n, p, i, j, k, sub - 1, f0, f1, f2);
                part[0][sub - 1][lane] = f0;
                part[1][sub - 1][lane] = f1;
                part[2][sub - 1][lane] = f2;
                split_barrier();  // partial sums ready
                split_barrier();  // warp 0 is done with them
            } else {
                T M[9], bb[3], uu[3];
                uint8_t dm = 7;
                if (valid) {
                    dm = dmask[n];
#pragma unroll
                    for (int e = 0; e < 9; ++e) M[e] = stencil::sval<T>(S[(int64_t)e * ld + p]);  // diagonal block (offset 13)
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        bb[c] = b[c * ld + n];
                        uu[c] = u[c * ld + n];
                    }
                }
                split_barrier();
                if (valid && dm != 7) {
                    T f0, f1, f2;
                    stencil::split_sum<T>(part, lane, f0, f1, f2);
                    stencil::node_solve<T>(dm, bb[0] - f0, bb[1] - f1, bb[2] - f2, M, forward != 0, uu[0], uu[1],
                                           uu[2]);
                    u[n] = uu[0];
                    u[ld + n] = uu[1];
                    u[2 * ld + n] = uu[2];
                }
                split_barrier();
            }
        }
        __syncthreads();  // the first colour's updates are visible before the second gathers
    }
}

// Full-weighting restriction (MultigridSolver.hh:217-275): coarse node gathers the
// 3^3 fine nodes [2I-1, 2I+1] clipped to the nondetached fine range, weights
// prod(1 - |d|/2); the first detached coarse layer is zeroed.
template <typename T>
__global__ void __launch_bounds__(BS) restrict_kernel(Geom gf, Geom gc, const T *__restrict__ fine,
                                                      T *__restrict__ coarse) {
    VFEM_PDL_ENTRY();
    const int cyv = gc.nyv();
    const int rows = cyv < gc.nn[1] ? cyv + 1 : cyv;
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= gc.NN) return;
    int i, j, k;
    decode(t, gc.nn[1], gc.nn[2], i, j, k);
    if (j >= rows) return;
    stencil::restrict_node<T>(gf, gc, fine, coarse, i, j, k);
}

// Trilinear prolongation (MultigridSolver.hh:163-212).
template <typename T, bool Accumulate>
__global__ void __launch_bounds__(BS) interp_kernel(Geom gf, Geom gc, const T *__restrict__ coarse,
                                                    T *__restrict__ fine) {
    VFEM_PDL_ENTRY();
    const int rows = Accumulate ? gf.nyv() : gf.nn[1];
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= gf.NN) return;
    int f[3];
    decode(t, gf.nn[1], gf.nn[2], f[0], f[1], f[2]);
    if (f[1] >= rows) return;
    stencil::interp_node<T, Accumulate>(gf, gc, coarse, fine, f);
}

template <typename T>
__global__ void zero_dirichlet_kernel(Geom g, T *__restrict__ u, const uint8_t *__restrict__ dmask) {
    VFEM_PDL_ENTRY();
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n >= g.NN) return;
    const uint8_t dm = dmask[n];
    if (!dm) return;
    if (dm & 1) u[n] = T(0);
    if (dm & 2) u[g.ld + n] = T(0);
    if (dm & 4) u[2 * g.ld + n] = T(0);
}

template <typename T>
__global__ void masked_zero_kernel(Geom g, T *__restrict__ u, int margin) {
    VFEM_PDL_ENTRY();
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= g.NN) return;
    int i, j, k;
    decode(t, g.nn[1], g.nn[2], i, j, k);
    if (j >= g.nyv() + margin) return;
    const int64_t n = g.node(i, j, k);
    u[n] = T(0);
    u[g.ld + n] = T(0);
    u[2 * g.ld + n] = T(0);
}

template <typename T>
__global__ void fill_kernel(T *__restrict__ p, T v, int64_t n) {
    VFEM_PDL_ENTRY();
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t < n) p[t] = v;
}

template <typename Tdst, typename Tsrc>
__global__ void cast_kernel(const Tsrc *__restrict__ s, Tdst *__restrict__ d, int64_t n) {
    VFEM_PDL_ENTRY();
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t < n) d[t] = (Tdst)s[t];
}

// Level-1 element matrices: Ke_c = sum_fi E_fi * Kc_fi (MultigridSolver.hh:724-738).
// One block per coarse element, thread t writes entry t.
template <typename T>
__global__ void __launch_bounds__(576) ke_level1_kernel(Geom g1, Geom g0, const T *__restrict__ Y0,
                                                        const T *__restrict__ Kc, T *__restrict__ Ke1) {
    __shared__ T sE[8];
    const int64_t e = blockIdx.x;
    const int t = threadIdx.x;
    const int ek = (int)(e % g1.ne[2]);
    const int64_t q = e / g1.ne[2];
    const int ej = (int)(q % g1.ne[1]), ei = (int)(q / g1.ne[1]);
    if (t < 8) sE[t] = Y0[g0.elem(2 * ei + ((t >> 2) & 1), 2 * ej + ((t >> 1) & 1), 2 * ek + (t & 1))];
    __syncthreads();
    T acc = T(0);
    if (ej < g1.maskedE()) {
#pragma unroll
        for (int fi = 0; fi < 8; ++fi) acc += sE[fi] * Kc[fi * 576 + t];
    }
    Ke1[e * 576 + t] = acc;
}

// Level-1 27-point stencil straight from the fine Young's moduli: block (n, n+o)(r, c) =
// sum over coarse elements e holding both nodes of sum_fi E_f(e, fi) Kc_fi[3ln+r][3lm+c]
// (the assembly of MultigridSolver.hh:724-738 without storing the element matrices).
// One block per node, thread q writes row entry q (coalesced 1 KB row).
template <typename T>
__global__ void __launch_bounds__(ROW) stencil_level1_kernel(Geom g1, Geom g0, const T *__restrict__ Y0,
                                                             const T *__restrict__ Kc, T *__restrict__ S) {
    __shared__ T sE[8][8];  // fine moduli of the 8 coarse elements around the node
    const int64_t n = blockIdx.x;
    const int q = threadIdx.x;
    int i, j, k;
    decode(n, g1.nn[1], g1.nn[2], i, j, k);
    if (q < 64) {
        const int slot = q >> 3, fi = q & 7;
        const int a = (slot >> 2) & 1, b = (slot >> 1) & 1, cc = slot & 1;
        const int ei = i - a, ej = j - b, ek = k - cc;
        T E = T(0);
        if (ei >= 0 && ej >= 0 && ek >= 0 && ei < g1.ne[0] && ej < g1.ne[1] && ek < g1.ne[2] && ej < g1.maskedE())
            E = Y0[g0.elem(2 * ei + ((fi >> 2) & 1), 2 * ej + ((fi >> 1) & 1), 2 * ek + (fi & 1))];
        sE[slot][fi] = E;
    }
    __syncthreads();
    T acc = T(0);
    if (q < stencil::ROW_USED) {
        const int o = q / 9, rc = q % 9, r = rc / 3, c = rc % 3;
        const int oo[3] = {o / 9 - 1, (o / 3) % 3 - 1, o % 3 - 1};
#pragma unroll
        for (int slot = 0; slot < 8; ++slot) {
            const int a = (slot >> 2) & 1, b = (slot >> 1) & 1, cc = slot & 1;
            const int ma = a + oo[0], mb = b + oo[1], mc = cc + oo[2];
            if (ma < 0 || ma > 1 || mb < 0 || mb > 1 || mc < 0 || mc > 1) continue;
            const int idx = (3 * (4 * a + 2 * b + cc) + r) * 24 + 3 * (4 * ma + 2 * mb + mc) + c;
#pragma unroll
            for (int fi = 0; fi < 8; ++fi) acc += sE[slot][fi] * Kc[fi * 576 + idx];
        }
    }
    S[n * ROW + q] = acc;
}

// Plane-layout variant: thread per (position p, neighbour offset o), o = 13 + blockIdx.y (the
// stored half), writing the nine entries of block (n, n+o). The Kc indices are warp-uniform (constant-cache
// broadcasts) and the eight fine moduli of each shared coarse element are loaded once for
// all nine entries.
template <typename T, typename TS>
__global__ void __launch_bounds__(BS) stencil_level1_soa_kernel(Geom g1, Geom g0, const T *__restrict__ Y0,
                                                                const T *__restrict__ Kc, TS *__restrict__ S, int rowLo,
                                                                int rowHi) {
    const int64_t p = blockIdx.x * (int64_t)BS + threadIdx.x;
    const int o = 13 + blockIdx.y;
    if (p >= g1.NN) return;
    int i, j, k;
    stencil::colour_node(g1, p, i, j, k);
    if (j < rowLo || j >= rowHi) return;  // outside the band being rebuilt
    const int oo[3] = {o / 9 - 1, (o / 3) % 3 - 1, o % 3 - 1};
    T acc[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) acc[e] = T(0);
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {
                const int ma = a + oo[0], mb = b + oo[1], mc = cc + oo[2];
                if (ma < 0 || ma > 1 || mb < 0 || mb > 1 || mc < 0 || mc > 1) continue;
                const int ei = i - a, ej = j - b, ek = k - cc;
                if (ei < 0 || ej < 0 || ek < 0 || ei >= g1.ne[0] || ej >= g1.ne[1] || ek >= g1.ne[2]) continue;
                if (ej >= g1.maskedE()) continue;
                T E[8];
#pragma unroll
                for (int fi = 0; fi < 8; ++fi)
                    E[fi] = Y0[g0.elem(2 * ei + ((fi >> 2) & 1), 2 * ej + ((fi >> 1) & 1), 2 * ek + (fi & 1))];
                const int ln = 4 * a + 2 * b + cc, lm = 4 * ma + 2 * mb + mc;
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const int idx = (3 * ln + r) * 24 + 3 * lm + c;
                        T v = acc[3 * r + c];
#pragma unroll
                        for (int fi = 0; fi < 8; ++fi) v += E[fi] * Kc[fi * 576 + idx];
                        acc[3 * r + c] = v;
                    }
            }
#pragma unroll
    for (int e = 0; e < 9; ++e) S[(int64_t)((o - 13) * 9 + e) * g1.ld + p] = stencil::sstore<TS>(acc[e]);
}

// Level-2 element matrices straight from the fine moduli: Ke_2(e) = sum over the 64 fine
// elements f inside e of E_f K2_f, K2_f = Phi_c^T Phi_fi^T K0 Phi_fi Phi_c for f in child c,
// position fi (the two coarsenings of MultigridSolver.hh:712-738 folded into one constant
// table). Children at or above the level-1 masked layer contribute nothing, as their level-1
// element matrices are zero. One block per EB2 elements, thread t owns entry t; each K2 entry
// is loaded once per block and applied to all EB2 elements.
constexpr int EB2 = 8;
template <typename T>
__global__ void __launch_bounds__(576) ke_level2_kernel(Geom g2, Geom g1, Geom g0, const T *__restrict__ Y0,
                                                        const T *__restrict__ K2, T *__restrict__ Ke2, int rowLo,
                                                        int rowHi) {
    __shared__ T sY[EB2][64];
    const int t = threadIdx.x;
    const int64_t e0 = (int64_t)blockIdx.x * EB2;
    // elements outside the row band [rowLo, rowHi) keep their matrices
    auto inBand = [&](int64_t e) {
        const int ej = (int)((e / g2.ne[2]) % g2.ne[1]);
        return e < g2.NE && ej >= rowLo && ej < rowHi;
    };
    bool any = false;
    for (int eb = 0; eb < EB2; ++eb) any = any || inBand(e0 + eb);
    if (!any) return;
    for (int q = t; q < EB2 * 64; q += 576) {
        const int eb = q >> 6, f = q & 63;
        const int64_t e = e0 + eb;
        T v = T(0);
        if (e < g2.NE) {
            const int ek = (int)(e % g2.ne[2]);
            const int64_t r = e / g2.ne[2];
            const int ej = (int)(r % g2.ne[1]), ei = (int)(r / g2.ne[1]);
            const int c = f >> 3, fi = f & 7;
            const int i1 = 2 * ei + ((c >> 2) & 1), j1 = 2 * ej + ((c >> 1) & 1), k1 = 2 * ek + (c & 1);
            if (ej < g2.maskedE() && j1 < g1.maskedE())
                v = Y0[g0.elem(2 * i1 + ((fi >> 2) & 1), 2 * j1 + ((fi >> 1) & 1), 2 * k1 + (fi & 1))];
        }
        sY[eb][f] = v;
    }
    __syncthreads();
    T acc[EB2];
#pragma unroll
    for (int eb = 0; eb < EB2; ++eb) acc[eb] = T(0);
#pragma unroll 4
    for (int f = 0; f < 64; ++f) {
        const T kv = K2[f * 576 + t];
#pragma unroll
        for (int eb = 0; eb < EB2; ++eb) acc[eb] += sY[eb][f] * kv;
    }
#pragma unroll
    for (int eb = 0; eb < EB2; ++eb)
        if (inBand(e0 + eb)) Ke2[(e0 + eb) * 576 + t] = acc[eb];
}

// Ke_c = sum_fi Phi_fi^T Ke_child(fi) Phi_fi (MultigridSolver.hh:712-722, 745-819).
// One block per coarse element, thread t owns entry t of the coarse matrix.
template <typename T>
__global__ void __launch_bounds__(576) ke_coarsen_kernel(Geom gc, Geom gf, const T *__restrict__ Kef,
                                                         const T *__restrict__ phis, T *__restrict__ Kec, int rowLo,
                                                         int rowHi) {
    __shared__ T sK[576];
    __shared__ T sT[576];
    __shared__ T sP[8 * 64];
    const int64_t e = blockIdx.x;
    const int t = threadIdx.x;
    const int ek = (int)(e % gc.ne[2]);
    const int64_t q = e / gc.ne[2];
    const int ej = (int)(q % gc.ne[1]), ei = (int)(q / gc.ne[1]);
    if (ej < rowLo || ej >= rowHi) return;  // outside the band being rebuilt (block-uniform)
    for (int qq = t; qq < 512; qq += 576) sP[qq] = phis[qq];
    const bool masked = ej >= gc.maskedE();
    T acc = T(0);
    const int row = t / 24, col = t % 24;
    for (int fi = 0; fi < 8; ++fi) {
        const int64_t ef = gf.elem(2 * ei + ((fi >> 2) & 1), 2 * ej + ((fi >> 1) & 1), 2 * ek + (fi & 1));
        __syncthreads();
        sK[t] = Kef[ef * 576 + t];
        __syncthreads();
        // T[row][3cn+d] = sum_fn K[row][3fn+d] phi[fn][cn]
        {
            const int cn = col / 3, d = col % 3;
            T v = T(0);
#pragma unroll
            for (int fn = 0; fn < 8; ++fn) v += sK[row * 24 + 3 * fn + d] * sP[fi * 64 + fn * 8 + cn];
            sT[t] = v;
        }
        __syncthreads();
        // Kc[3cm+d][col] += sum_fm phi[fm][cm] T[3fm+d][col]
        {
            const int cm = row / 3, d = row % 3;
            T v = T(0);
#pragma unroll
            for (int fm = 0; fm < 8; ++fm) v += sP[fi * 64 + fm * 8 + cm] * sT[(3 * fm + d) * 24 + col];
            acc += v;
        }
    }
    Kec[e * 576 + t] = masked ? T(0) : acc;
}

// Fine-level element matrices Ke = Y_e K0 (masked elements carry Y = 0).
template <typename T>
__global__ void __launch_bounds__(BS) ke_scaled_kernel(Geom g, const T *__restrict__ Y, const T *__restrict__ K0,
                                                       T *__restrict__ Ke) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= g.NE * 576) return;
    Ke[t] = Y[t / 576] * K0[t % 576];
}

// Assemble the 27-point block stencil from element matrices (TensorProductSimulator.hh:885-930).
// One block per node, thread q writes row entry q.
template <typename T>
__global__ void __launch_bounds__(ROW) stencil_from_ke_kernel(Geom g, const T *__restrict__ Ke, T *__restrict__ S) {
    const int64_t n = blockIdx.x;
    const int q = threadIdx.x;
    int i, j, k;
    decode(n, g.nn[1], g.nn[2], i, j, k);
    T acc = T(0);
    if (q < stencil::ROW_USED) {
        const int o = q / 9, rc = q % 9, r = rc / 3, c = rc % 3;
        const int oo[3] = {o / 9 - 1, (o / 3) % 3 - 1, o % 3 - 1};
        // incident elements (i-a, j-b, k-cc): node local index ln = 4a+2b+cc; neighbour local = ln + o
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int cc = 0; cc < 2; ++cc) {
                    const int ma = a + oo[0], mb = b + oo[1], mc = cc + oo[2];
                    if (ma < 0 || ma > 1 || mb < 0 || mb > 1 || mc < 0 || mc > 1) continue;
                    const int ei = i - a, ej = j - b, ek = k - cc;
                    if (ei < 0 || ej < 0 || ek < 0 || ei >= g.ne[0] || ej >= g.ne[1] || ek >= g.ne[2]) continue;
                    const int ln = 4 * a + 2 * b + cc, lm = 4 * ma + 2 * mb + mc;
                    acc += Ke[g.elem(ei, ej, ek) * 576 + (3 * ln + r) * 24 + 3 * lm + c];
                }
    }
    S[n * ROW + q] = acc;
}

template <typename T, typename TS>
__global__ void __launch_bounds__(BS) stencil_from_ke_soa_kernel(Geom g, const T *__restrict__ Ke,
                                                                 TS *__restrict__ S, int rowLo, int rowHi) {
    const int64_t p = blockIdx.x * (int64_t)BS + threadIdx.x;
    const int o = 13 + blockIdx.y;
    if (p >= g.NN) return;
    int i, j, k;
    stencil::colour_node(g, p, i, j, k);
    if (j < rowLo || j >= rowHi) return;  // outside the band being rebuilt
    const int oo[3] = {o / 9 - 1, (o / 3) % 3 - 1, o % 3 - 1};
    T acc[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) acc[e] = T(0);
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {
                const int ma = a + oo[0], mb = b + oo[1], mc = cc + oo[2];
                if (ma < 0 || ma > 1 || mb < 0 || mb > 1 || mc < 0 || mc > 1) continue;
                const int ei = i - a, ej = j - b, ek = k - cc;
                if (ei < 0 || ej < 0 || ek < 0 || ei >= g.ne[0] || ej >= g.ne[1] || ek >= g.ne[2]) continue;
                const int ln = 4 * a + 2 * b + cc, lm = 4 * ma + 2 * mb + mc;
                const T *ke = Ke + g.elem(ei, ej, ek) * 576;
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c) acc[3 * r + c] += ke[(3 * ln + r) * 24 + 3 * lm + c];
            }
#pragma unroll
    for (int e = 0; e < 9; ++e) S[(int64_t)((o - 13) * 9 + e) * g.ld + p] = stencil::sstore<TS>(acc[e]);
}

}  // namespace

// Node-contiguous rows keep the arithmetic type; only plane-layout stencils may be stored in bf16.
template <typename T, typename TS>
static void rowsNeedSameType(bool rows) {
    if (rows && !std::is_same<T, TS>::value) throw Error(ERR_ARG, "bf16 stencils need the plane layout");
}

template <typename T, typename TS>
void launch_stencil_apply(const Geom &g, const TS *S, const T *u, T *out, bool zeroInit, bool negate, bool rows,
                          cudaStream_t st) {
    rowsNeedSameType<T, TS>(rows);
    if (!rows) {
        const unsigned gs = gridFor(g.NN, SPLIT_NODES);
        if (zeroInit) {
            if (negate) launch_pdl(stencil_apply_soa_kernel<T, TS, true, true>, gs, SPLIT_BS, 0, st, g, S, u, out);
            else launch_pdl(stencil_apply_soa_kernel<T, TS, true, false>, gs, SPLIT_BS, 0, st, g, S, u, out);
        } else {
            if (negate) launch_pdl(stencil_apply_soa_kernel<T, TS, false, true>, gs, SPLIT_BS, 0, st, g, S, u, out);
            else launch_pdl(stencil_apply_soa_kernel<T, TS, false, false>, gs, SPLIT_BS, 0, st, g, S, u, out);
        }
        VFEM_LAUNCH_CHECK();
        return;
    }
    if constexpr (std::is_same<T, TS>::value) {
        const unsigned grid = gridFor(g.NN, WPB);
        if (zeroInit) {
            if (negate) launch_pdl(stencil_apply_kernel<T, true, true>, grid, BS, 0, st, g, S, u, out);
            else launch_pdl(stencil_apply_kernel<T, true, false>, grid, BS, 0, st, g, S, u, out);
        } else {
            if (negate) launch_pdl(stencil_apply_kernel<T, false, true>, grid, BS, 0, st, g, S, u, out);
            else launch_pdl(stencil_apply_kernel<T, false, false>, grid, BS, 0, st, g, S, u, out);
        }
        VFEM_LAUNCH_CHECK();
    }
}

template <typename T, typename TS>
void launch_stencil_residual(const Geom &g, const TS *S, const T *u, const T *b, T *r, const uint8_t *dmask, bool rows,
                             cudaStream_t st) {
    rowsNeedSameType<T, TS>(rows);
    if constexpr (std::is_same<T, TS>::value) {
        if (rows) {
            launch_pdl(stencil_residual_kernel<T>, gridFor(g.NN, WPB), BS, 0, st, g, S, u, b, r, dmask);
            VFEM_LAUNCH_CHECK();
            return;
        }
    }
    launch_pdl(stencil_residual_soa_kernel<T, TS>, gridFor(g.NN, SPLIT_NODES), SPLIT_BS, 0, st, g, S, u, b, r, dmask);
    VFEM_LAUNCH_CHECK();
}

template <typename T, typename TS>
void launch_gs_stencil_color(const Geom &g, const TS *S, T *u, const T *b, const uint8_t *dmask, int color,
                             bool forward, bool rows, cudaStream_t st) {
    rowsNeedSameType<T, TS>(rows);
    const int cx = (color >> 2) & 1, cy = (color >> 1) & 1, cz = color & 1;
    const int64_t n0 = (g.nn[0] - cx + 1) / 2, n1 = (g.nn[1] - cy + 1) / 2, n2 = (g.nn[2] - cz + 1) / 2;
    if (n1 <= 0) return;
    if constexpr (std::is_same<T, TS>::value) {
        if (rows) {
            launch_pdl(gs_stencil_color_kernel<T>, gridFor(n0 * n1 * n2, WPB), BS, 0, st, g, S, u, b, dmask, cx, cy,
                       cz, forward ? 1 : 0);
            VFEM_LAUNCH_CHECK();
            return;
        }
    }
    launch_pdl(gs_stencil_color_soa_kernel<T, TS>, gridFor(n0 * n1 * n2, SPLIT_NODES), SPLIT_BS, 0, st, g, S, u, b,
               dmask, cx, cy, cz, forward ? 1 : 0);
    VFEM_LAUNCH_CHECK();
}

template <typename T, typename TS>
void launch_gs_stencil_lines(const Geom &g, const TS *S, T *u, const T *b, const uint8_t *dmask, int cx, int cy,
                             bool forward, cudaStream_t st) {
    const int nlines = ((g.nn[0] - cx + 1) / 2) * ((g.nn[1] - cy + 1) / 2);
    if (nlines <= 0) return;
    // short lines share a 32-node round
    const int nk = (g.nn[2] + 1) / 2;
    const int per = std::max(1, SPLIT_NODES / nk);
    launch_pdl(gs_stencil_lines_soa_kernel<T, TS>, (unsigned)((nlines + per - 1) / per), SPLIT_BS, 0, st, g, S, u,
               b, dmask, cx, cy, per, forward ? 1 : 0);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_restrict(const Geom &gf, const Geom &gc, const T *fine, T *coarse, cudaStream_t st) {
    launch_pdl(restrict_kernel<T>, gridFor(gc.NN, BS), BS, 0, st, gf, gc, fine, coarse);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_interpolate(const Geom &gf, const Geom &gc, const T *coarse, T *fine, bool accumulate, cudaStream_t st) {
    const unsigned grid = gridFor(gf.NN, BS);
    if (accumulate) launch_pdl(interp_kernel<T, true>, grid, BS, 0, st, gf, gc, coarse, fine);
    else launch_pdl(interp_kernel<T, false>, grid, BS, 0, st, gf, gc, coarse, fine);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_zero_dirichlet(const Geom &g, T *u, const uint8_t *dmask, cudaStream_t st) {
    launch_pdl(zero_dirichlet_kernel<T>, gridFor(g.NN, BS), BS, 0, st, g, u, dmask);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_masked_zero(const Geom &g, T *u, int margin, cudaStream_t st) {
    launch_pdl(masked_zero_kernel<T>, gridFor(g.NN, BS), BS, 0, st, g, u, margin);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_fill(T *p, T v, int64_t n, cudaStream_t st) {
    if (n <= 0) return;
    launch_pdl(fill_kernel<T>, gridFor(n, BS), BS, 0, st, p, v, n);
    VFEM_LAUNCH_CHECK();
}

template <typename Tdst, typename Tsrc>
void launch_cast(const Tsrc *src, Tdst *dst, int64_t n, cudaStream_t st) {
    if (n <= 0) return;
    launch_pdl(cast_kernel<Tdst, Tsrc>, gridFor(n, BS), BS, 0, st, src, dst, n);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_ke_level1(const Geom &g1, const Geom &g0, const T *Y0, const T *Kc, T *Ke1, cudaStream_t st) {
    if (g1.NE > 2147483647LL) throw Error(ERR_ARG, "too many coarse elements");
    ke_level1_kernel<T><<<(unsigned)g1.NE, 576, 0, st>>>(g1, g0, Y0, Kc, Ke1);
    VFEM_LAUNCH_CHECK();
}

template <typename T, typename TS>
void launch_stencil_level1(const Geom &g1, const Geom &g0, const T *Y0, const T *Kc, TS *S, bool rows, cudaStream_t st,
                           int rowLo, int rowHi) {
    if (g1.NN > 2147483647LL) throw Error(ERR_ARG, "too many nodes");
    rowsNeedSameType<T, TS>(rows);
    if constexpr (std::is_same<T, TS>::value) {
        if (rows) {
            if (rowLo > 0 || rowHi < g1.nn[1]) throw Error(ERR_ARG, "band updates need plane-layout stencils");
            stencil_level1_kernel<T><<<(unsigned)g1.NN, ROW, 0, st>>>(g1, g0, Y0, Kc, S);
            VFEM_LAUNCH_CHECK();
            return;
        }
    }
    stencil_level1_soa_kernel<T, TS><<<dim3(gridFor(g1.NN, BS), stencil::HALF_OFFSETS), BS, 0, st>>>(g1, g0, Y0, Kc, S,
                                                                                                     rowLo, rowHi);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_ke_coarsen(const Geom &gc, const Geom &gf, const T *Kef, const T *phis, T *Kec, cudaStream_t st, int rowLo,
                       int rowHi) {
    if (gc.NE > 2147483647LL) throw Error(ERR_ARG, "too many coarse elements");
    ke_coarsen_kernel<T><<<(unsigned)gc.NE, 576, 0, st>>>(gc, gf, Kef, phis, Kec, rowLo, rowHi);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_ke_level2(const Geom &g2, const Geom &g1, const Geom &g0, const T *Y0, const T *K2, T *Ke2, cudaStream_t st,
                      int rowLo, int rowHi) {
    ke_level2_kernel<T><<<gridFor(g2.NE, EB2), 576, 0, st>>>(g2, g1, g0, Y0, K2, Ke2, rowLo, rowHi);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_ke_scaled(const Geom &g, const T *Y, const T *K0, T *Ke, cudaStream_t st) {
    ke_scaled_kernel<T><<<gridFor(g.NE * 576, BS), BS, 0, st>>>(g, Y, K0, Ke);
    VFEM_LAUNCH_CHECK();
}

template <typename T, typename TS>
void launch_stencil_from_ke(const Geom &g, const T *Ke, TS *S, bool rows, cudaStream_t st, int rowLo, int rowHi) {
    if (g.NN > 2147483647LL) throw Error(ERR_ARG, "too many nodes");
    rowsNeedSameType<T, TS>(rows);
    if constexpr (std::is_same<T, TS>::value) {
        if (rows) {
            if (rowLo > 0 || rowHi < g.nn[1]) throw Error(ERR_ARG, "band updates need plane-layout stencils");
            stencil_from_ke_kernel<T><<<(unsigned)g.NN, ROW, 0, st>>>(g, Ke, S);
            VFEM_LAUNCH_CHECK();
            return;
        }
    }
    stencil_from_ke_soa_kernel<T, TS><<<dim3(gridFor(g.NN, BS), stencil::HALF_OFFSETS), BS, 0, st>>>(g, Ke, S, rowLo,
                                                                                                     rowHi);
    VFEM_LAUNCH_CHECK();
}

#define VFEM_INST_STENCIL(T, TS)                                                                                      \
    template void launch_stencil_apply<T, TS>(const Geom &, const TS *, const T *, T *, bool, bool, bool, cudaStream_t); \
    template void launch_stencil_residual<T, TS>(const Geom &, const TS *, const T *, const T *, T *, const uint8_t *,   \
                                                 bool, cudaStream_t);                                                    \
    template void launch_gs_stencil_color<T, TS>(const Geom &, const TS *, T *, const T *, const uint8_t *, int, bool,   \
                                                 bool, cudaStream_t);                                                    \
    template void launch_gs_stencil_lines<T, TS>(const Geom &, const TS *, T *, const T *, const uint8_t *, int, int,    \
                                                 bool, cudaStream_t);                                                    \
    template void launch_stencil_level1<T, TS>(const Geom &, const Geom &, const T *, const T *, TS *, bool,             \
                                               cudaStream_t, int, int);                                                 \
    template void launch_stencil_from_ke<T, TS>(const Geom &, const T *, TS *, bool, cudaStream_t, int, int);
VFEM_INST_STENCIL(double, double)
VFEM_INST_STENCIL(float, float)
VFEM_INST_STENCIL(float, __nv_bfloat16)

#define VFEM_INST_COARSE(T)                                                                                           \
    template void launch_restrict<T>(const Geom &, const Geom &, const T *, T *, cudaStream_t);                       \
    template void launch_interpolate<T>(const Geom &, const Geom &, const T *, T *, bool, cudaStream_t);              \
    template void launch_zero_dirichlet<T>(const Geom &, T *, const uint8_t *, cudaStream_t);                         \
    template void launch_masked_zero<T>(const Geom &, T *, int, cudaStream_t);                                        \
    template void launch_fill<T>(T *, T, int64_t, cudaStream_t);                                                      \
    template void launch_ke_level1<T>(const Geom &, const Geom &, const T *, const T *, T *, cudaStream_t);           \
    template void launch_ke_coarsen<T>(const Geom &, const Geom &, const T *, const T *, T *, cudaStream_t, int, int); \
    template void launch_ke_level2<T>(const Geom &, const Geom &, const Geom &, const T *, const T *, T *,            \
                                      cudaStream_t, int, int);                                                        \
    template void launch_ke_scaled<T>(const Geom &, const T *, const T *, T *, cudaStream_t);
VFEM_INST_COARSE(double)
VFEM_INST_COARSE(float)
template void launch_cast<float, double>(const double *, float *, int64_t, cudaStream_t);
template void launch_cast<double, float>(const float *, double *, int64_t, cudaStream_t);

}  // namespace vfem
