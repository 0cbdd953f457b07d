// Fine-level (L0) kernels: matrix-free SIMP applyK, residual, coloured block
// Gauss-Seidel, Young's moduli, compliance sensitivity and element energy.
//
// Node-centric gather, one thread per node: the (up to) 8 incident elements are
// visited in the order of the reference's guarded stencil path
// (TPSStencils.hh:577-659): element (i-a, j-b, k-c) for a, b, c in {0,1}, in which
// the node has local index 4a+2b+c. K0 is a by-value kernel parameter (constant
// bank); its symmetry lets every thread scan a column K0[:, row].
#include "vfem_df.cuh"
#include "vfem_kernels.hpp"
#include "vfem_reduce.cuh"

#include <algorithm>
#include <cstdlib>
#include <type_traits>

namespace vfem {

namespace {

constexpr int BS = 256;

// 32-bit unsigned decode of a flat index into (i, j, k) for dimensions (., n1, n2): counts stay
// below 2^31 (checked when a grid is created); 64-bit division is a long software sequence.
__device__ __forceinline__ void decode3(int64_t n, int n1, int n2, int &i, int &j, int &k) {
    const uint32_t u = (uint32_t)n, t = u / (uint32_t)n2;
    k = (int)(u - t * (uint32_t)n2);
    const uint32_t q = t / (uint32_t)n1;
    j = (int)(t - q * (uint32_t)n1);
    i = (int)q;
}

__device__ __forceinline__ void decode_node(const Geom &g, int64_t n, int &i, int &j, int &k) {
    decode3(n, g.nn[1], g.nn[2], i, j, k);
}

// acc[r] (+/-)= E * sum_t K0[t][3*ln + r] * u_e[t] for element (ei,ej,ek).
template <typename T, int LN>
__device__ __forceinline__ void elem_rows(const Geom &g, const Mat24<T> &K, const T *__restrict__ u, int64_t base,
                                          T &c0, T &c1, T &c2) {
    const int64_t ld = g.ld;
    const int64_t sx = (int64_t)g.nn[1] * g.nn[2], sy = g.nn[2];
    c0 = c1 = c2 = T(0);
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const int64_t nm = base + ((m >> 2) & 1) * sx + ((m >> 1) & 1) * sy + (m & 1);
        const T u0 = u[nm], u1 = u[ld + nm], u2 = u[2 * ld + nm];
        c0 += K.a[(3 * m + 0) * 24 + 3 * LN + 0] * u0;
        c0 += K.a[(3 * m + 1) * 24 + 3 * LN + 0] * u1;
        c0 += K.a[(3 * m + 2) * 24 + 3 * LN + 0] * u2;
        c1 += K.a[(3 * m + 0) * 24 + 3 * LN + 1] * u0;
        c1 += K.a[(3 * m + 1) * 24 + 3 * LN + 1] * u1;
        c1 += K.a[(3 * m + 2) * 24 + 3 * LN + 1] * u2;
        c2 += K.a[(3 * m + 0) * 24 + 3 * LN + 2] * u0;
        c2 += K.a[(3 * m + 1) * 24 + 3 * LN + 2] * u1;
        c2 += K.a[(3 * m + 2) * 24 + 3 * LN + 2] * u2;
    }
}

// Element (i-A, j-B, k-Cc); an element outside the grid is clamped onto a valid one and
// weighted by E = 0, which keeps the gather branch-free (0 * finite adds nothing).
template <typename T, int A, int B, int Cc, bool Negate>
__device__ __forceinline__ void visit_elem(const Geom &g, const Mat24<T> &K, const T *__restrict__ Y,
                                           const T *__restrict__ u, int i, int j, int k, T &f0, T &f1, T &f2) {
    const int ei = i - A, ej = j - B, ek = k - Cc;
    const bool inb = ei >= 0 && ej >= 0 && ek >= 0 && ei < g.ne[0] && ej < g.ne[1] && ek < g.ne[2];
    const int ci = min(max(ei, 0), g.ne[0] - 1), cj = min(max(ej, 0), g.ne[1] - 1), ck = min(max(ek, 0), g.ne[2] - 1);
    const T E = inb ? Y[g.elem(ci, cj, ck)] : T(0);
    T c0, c1, c2;
    elem_rows<T, 4 * A + 2 * B + Cc>(g, K, u, g.node(ci, cj, ck), c0, c1, c2);
    if (Negate) { f0 -= E * c0; f1 -= E * c1; f2 -= E * c2; }
    else        { f0 += E * c0; f1 += E * c1; f2 += E * c2; }
}

template <typename T, bool Negate>
__device__ __forceinline__ void gather_ku(const Geom &g, const Mat24<T> &K, const T *__restrict__ Y,
                                          const T *__restrict__ u, int i, int j, int k, T &f0, T &f1, T &f2) {
    visit_elem<T, 0, 0, 0, Negate>(g, K, Y, u, i, j, k, f0, f1, f2);
    visit_elem<T, 0, 0, 1, Negate>(g, K, Y, u, i, j, k, f0, f1, f2);
    visit_elem<T, 0, 1, 0, Negate>(g, K, Y, u, i, j, k, f0, f1, f2);
    visit_elem<T, 0, 1, 1, Negate>(g, K, Y, u, i, j, k, f0, f1, f2);
    visit_elem<T, 1, 0, 0, Negate>(g, K, Y, u, i, j, k, f0, f1, f2);
    visit_elem<T, 1, 0, 1, Negate>(g, K, Y, u, i, j, k, f0, f1, f2);
    visit_elem<T, 1, 1, 0, Negate>(g, K, Y, u, i, j, k, f0, f1, f2);
    visit_elem<T, 1, 1, 1, Negate>(g, K, Y, u, i, j, k, f0, f1, f2);
}

// ---- K0 access inside unrolled loops ----
// The full table (a by-value kernel parameter; each entry is a constant-bank load) or, for
// cube elements, the 10 class values of k0_cube_class held in registers.
template <typename T, bool Cube>
struct K0View {
    static constexpr bool kCube = false;
    const Mat24<T> &K;
    __device__ explicit K0View(const Mat24<T> &K_) : K(K_) {}
    __device__ __forceinline__ T operator()(int row, int col) const { return K.a[row * 24 + col]; }
};
template <typename T>
struct K0View<T, true> {
    static constexpr bool kCube = true;
    T kv[10];
    __device__ explicit K0View(const Mat24<T> &K) {
#pragma unroll
        for (int c = 0; c < 10; ++c) kv[c] = K.cube[c];
    }
    __device__ __forceinline__ T operator()(int row, int col) const {
        const int c = k0_cube_class(row, col);
        return (c & 16) ? -kv[c & 15] : kv[c & 15];
    }
};

template <bool Cube>
struct K0DFView {
    const Mat24DF &K;
    __device__ explicit K0DFView(const Mat24DF &K_) : K(K_) {}
    __device__ __forceinline__ float hi(int row, int col) const { return K.hi[row * 24 + col]; }
    __device__ __forceinline__ float lo(int row, int col) const { return K.lo[row * 24 + col]; }
};
template <>
struct K0DFView<true> {
    float h[10], l[10];
    __device__ explicit K0DFView(const Mat24DF &K) {
#pragma unroll
        for (int c = 0; c < 10; ++c) {
            h[c] = K.cubeHi[c];
            l[c] = K.cubeLo[c];
        }
    }
    __device__ __forceinline__ float hi(int row, int col) const {
        const int c = k0_cube_class(row, col);
        return (c & 16) ? -h[c & 15] : h[c & 15];
    }
    __device__ __forceinline__ float lo(int row, int col) const {
        const int c = k0_cube_class(row, col);
        return (c & 16) ? -l[c & 15] : l[c & 15];
    }
};

// ---- neighbourhood form (FP32 levels of the mixed preconditioner) ----
// The 27 neighbours' displacements are loaded once into registers (81 loads instead of
// 8 elements x 8 nodes x 3 = 192), then every incident element's rows are formed from
// registers. The FP32 vectors carry a zeroed guard of Geom::nodeGuard() elements on either
// side and the FP32 moduli a ghost layer of zeros (Geom::padElem), so neither the loads nor
// the moduli need bounds checks: a neighbour outside the grid reads some finite value that
// only elements outside the grid use, and those carry E = 0.

// One x-plane (i + a - 1) of the 3x3x3 neighbourhood: P[3b + c][d] = u_d(i+a-1, j+b-1, k+c-1).
template <typename T>
__device__ __forceinline__ void load_plane(const Geom &g, const T *__restrict__ u, int64_t n, int a, T (&P)[9][3]) {
    const int64_t ld = g.ld;
    const int64_t sx = (int64_t)g.nn[1] * g.nn[2], sy = g.nn[2];
    const T *c0 = u + n + (a - 1) * sx;
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        const T *row = c0 + (b - 1) * sy;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const T *rd = row + d * ld;
#pragma unroll
            for (int c = 0; c < 3; ++c) P[3 * b + c][d] = rd[c - 1];
        }
    }
}

// E of element (i-A, j-B, k-C) at slot 4A+2B+C from the zero-padded moduli.
template <typename T>
__device__ __forceinline__ void load_elem_moduli(const Geom &g, const T *__restrict__ Yp, int i, int j, int k,
                                                 T (&E)[8]) {
    const int64_t px = (int64_t)(g.ne[1] + 2) * (g.ne[2] + 2), py = g.ne[2] + 2;
    const T *base = Yp + g.padElem(i, j, k);
#pragma unroll
    for (int s = 0; s < 8; ++s) E[s] = base[-(((s >> 2) & 1) * px) - ((s >> 1) & 1) * py - (s & 1)];
}

// rows 3LN..3LN+2 of K0 times the displacements of element (i-A, j-B, k-C), whose local
// node m sits at neighbour offset (ma - A, mb - B, mc - C): x-plane Plo (ma = 0) or Phi (ma = 1)
template <typename T, int A, int B, int C, typename KV>
__device__ __forceinline__ void elem_rows_planes(const KV &K, const T (&Plo)[9][3], const T (&Phi)[9][3], T &c0,
                                                 T &c1, T &c2) {
    constexpr int LN = 4 * A + 2 * B + C;
    c0 = c1 = c2 = T(0);
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const int ma = (m >> 2) & 1, mb = (m >> 1) & 1, mc = m & 1;
        const int q = (mb - B + 1) * 3 + (mc - C + 1);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const T v = ma ? Phi[q][d] : Plo[q][d];
            c0 += K(3 * m + d, 3 * LN + 0) * v;
            c1 += K(3 * m + d, 3 * LN + 1) * v;
            c2 += K(3 * m + d, 3 * LN + 2) * v;
        }
    }
}

template <typename T, int A, int B, int C, bool Negate, typename KV>
__device__ __forceinline__ void visit_planes(const KV &K, const T (&Plo)[9][3], const T (&Phi)[9][3],
                                             const T (&E)[8], T &f0, T &f1, T &f2) {
    T c0, c1, c2;
    elem_rows_planes<T, A, B, C>(K, Plo, Phi, c0, c1, c2);
    const T e = E[4 * A + 2 * B + C];
    if (Negate) { f0 -= e * c0; f1 -= e * c1; f2 -= e * c2; }
    else        { f0 += e * c0; f1 += e * c1; f2 += e * c2; }
}

// Elements behind the node in x (A = 1) use planes i-1 and i, those in front (A = 0) planes
// i and i+1, so at most two planes (54 values) are live at a time.
template <typename T, bool Negate, typename KV>
__device__ __forceinline__ void gather_ku_nbhd(const Geom &g, const KV &K, const T *__restrict__ Y,
                                               const T *__restrict__ u, int i, int j, int k, T &f0, T &f1, T &f2) {
    const int64_t n = g.node(i, j, k);
    T E[8], Pa[9][3], Pb[9][3];
    load_elem_moduli<T>(g, Y, i, j, k, E);
    load_plane<T>(g, u, n, 0, Pa);
    load_plane<T>(g, u, n, 1, Pb);
    visit_planes<T, 1, 0, 0, Negate>(K, Pa, Pb, E, f0, f1, f2);
    visit_planes<T, 1, 0, 1, Negate>(K, Pa, Pb, E, f0, f1, f2);
    visit_planes<T, 1, 1, 0, Negate>(K, Pa, Pb, E, f0, f1, f2);
    visit_planes<T, 1, 1, 1, Negate>(K, Pa, Pb, E, f0, f1, f2);
    load_plane<T>(g, u, n, 2, Pa);
    visit_planes<T, 0, 0, 0, Negate>(K, Pb, Pa, E, f0, f1, f2);
    visit_planes<T, 0, 0, 1, Negate>(K, Pb, Pa, E, f0, f1, f2);
    visit_planes<T, 0, 1, 0, Negate>(K, Pb, Pa, E, f0, f1, f2);
    visit_planes<T, 0, 1, 1, Negate>(K, Pb, Pa, E, f0, f1, f2);
}

// K u at a node: neighbourhood form in FP32, element-by-element loads in FP64 (where the
// 81 register neighbourhood would spill)
template <typename T, bool Negate, bool Cube>
__device__ __forceinline__ void gather_ku_any(const Geom &g, const Mat24<T> &K, const T *__restrict__ Y,
                                              const T *__restrict__ u, int i, int j, int k, T &f0, T &f1, T &f2) {
    if constexpr (sizeof(T) == 4) gather_ku_nbhd<T, Negate>(g, K0View<T, Cube>(K), Y, u, i, j, k, f0, f1, f2);
    else gather_ku<T, Negate>(g, K, Y, u, i, j, k, f0, f1, f2);
}

template <typename T, bool ZeroInit, bool Negate, bool WithDot, bool Cube>
__global__ void __launch_bounds__(BS, 2) applyk_fine_kernel(Geom g, const T *__restrict__ Y, const T *__restrict__ u,
                                                         T *__restrict__ out, const uint8_t *__restrict__ dmask,
                                                         int zeroDir, double *__restrict__ partials,
                                                         const Mat24<T> K) {
    VFEM_PDL_ENTRY();
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    double dot = 0.0;
    if (n < g.NN) {
        int i, j, k;
        decode_node(g, n, i, j, k);
        const int64_t ld = g.ld;
        if (j < g.nyv()) {
            T f0 = ZeroInit ? T(0) : out[n];
            T f1 = ZeroInit ? T(0) : out[ld + n];
            T f2 = ZeroInit ? T(0) : out[2 * ld + n];
            gather_ku_any<T, Negate, Cube>(g, K, Y, u, i, j, k, f0, f1, f2);
            if (zeroDir) {
                const uint8_t dm = dmask[n];
                if (dm & 1) f0 = T(0);
                if (dm & 2) f1 = T(0);
                if (dm & 4) f2 = T(0);
            }
            out[n] = f0;
            out[ld + n] = f1;
            out[2 * ld + n] = f2;
            if (WithDot) dot = (double)u[n] * f0 + (double)u[ld + n] * f1 + (double)u[2 * ld + n] * f2;
        } else if (ZeroInit) {
            out[n] = T(0);
            out[ld + n] = T(0);
            out[2 * ld + n] = T(0);
        }
    }
    if (WithDot) {
        const double s = block_sum<BS>(dot);
        if (threadIdx.x == 0) partials[blockIdx.x] = s;
    }
}

// r = b - K u (MultigridSolver.hh:527-541): b copied, stencil subtracted, Dirichlet zeroed.
// MB: resident blocks per SM the register budget is fitted to.
template <typename T, bool Cube, int MB = 2>
__global__ void __launch_bounds__(BS, MB) residual_fine_kernel(Geom g, const T *__restrict__ Y, const T *__restrict__ u,
                                                           const T *__restrict__ b, T *__restrict__ r,
                                                           const uint8_t *__restrict__ dmask, const Mat24<T> K) {
    VFEM_PDL_ENTRY();
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n >= g.NN) return;
    int i, j, k;
    decode_node(g, n, i, j, k);
    const int64_t ld = g.ld;
    T f0 = b[n], f1 = b[ld + n], f2 = b[2 * ld + n];
    if (j < g.nyv()) gather_ku_any<T, true, Cube>(g, K, Y, u, i, j, k, f0, f1, f2);
    const uint8_t dm = dmask[n];
    if (dm & 1) f0 = T(0);
    if (dm & 2) f1 = T(0);
    if (dm & 4) f2 = T(0);
    r[n] = f0;
    r[ld + n] = f1;
    r[2 * ld + n] = f2;
}

// Block Gauss-Seidel node update (MultigridSolver.hh:348-378).
template <typename T>
__device__ __forceinline__ void smooth_node_solve(uint8_t dm, T s0, T s1, T s2, const T *M, bool forward, T &u0, T &u1,
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
        // adjugate inverse of the 3x3 diagonal block
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

template <typename T, int A, int B, int Cc>
__device__ __forceinline__ void gs_visit(const Geom &g, const Mat24<T> &K, const T *__restrict__ Y, const T *u, int i,
                                         int j, int k, T &s0, T &s1, T &s2, T *M) {
    const int ei = i - A, ej = j - B, ek = k - Cc;
    const bool inb = ei >= 0 && ej >= 0 && ek >= 0 && ei < g.ne[0] && ej < g.ne[1] && ek < g.ne[2];
    const int ci = min(max(ei, 0), g.ne[0] - 1), cj = min(max(ej, 0), g.ne[1] - 1), ck = min(max(ek, 0), g.ne[2] - 1);
    constexpr int LN = 4 * A + 2 * B + Cc;
    const T E = inb ? Y[g.elem(ci, cj, ck)] : T(0);
    T c0, c1, c2;
    elem_rows<T, LN>(g, K, u, g.node(ci, cj, ck), c0, c1, c2);
    s0 -= E * c0;
    s1 -= E * c1;
    s2 -= E * c2;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) M[3 * r + c] += E * K.a[(3 * LN + r) * 24 + 3 * LN + c];
}

template <typename T, int A, int B, int C, typename KV>
__device__ __forceinline__ void gs_visit_planes(const KV &K, const T (&Plo)[9][3], const T (&Phi)[9][3],
                                                const T (&E)[8], T &s0, T &s1, T &s2, T *M) {
    constexpr int LN = 4 * A + 2 * B + C;
    const T e = E[LN];
    T c0, c1, c2;
    elem_rows_planes<T, A, B, C>(K, Plo, Phi, c0, c1, c2);
    s0 -= e * c0;
    s1 -= e * c1;
    s2 -= e * c2;
    if constexpr (!KV::kCube) {
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) M[3 * r + c] += e * K(3 * LN + r, 3 * LN + c);
    }
}

// Diagonal block of a node for cube elements: K0's node blocks have the diagonal entry of class
// 0 and the off-diagonal entries (d, r) of class 8 with sign xi[d] xi[r], the node's sides
// along axes d and r (k0_cube_class), so M = kv[0] sum(E) I + kv[8] (signed sums of E): 28
// additions instead of 72 FMAs.
template <typename T>
__device__ __forceinline__ void cube_diag_block(const K0View<T, true> &K, const T (&E)[8], T *M) {
    T sE = T(0), sxy = T(0), sxz = T(0), syz = T(0);
#pragma unroll
    for (int ln = 0; ln < 8; ++ln) {
        const int bx = (ln >> 2) & 1, by = (ln >> 1) & 1, bz = ln & 1;
        sE += E[ln];
        sxy += (bx == by) ? E[ln] : -E[ln];
        sxz += (bx == bz) ? E[ln] : -E[ln];
        syz += (by == bz) ? E[ln] : -E[ln];
    }
    const T d = K.kv[0], o = K.kv[8];
    M[0] = M[4] = M[8] = d * sE;
    M[1] = M[3] = o * sxy;
    M[2] = M[6] = o * sxz;
    M[5] = M[7] = o * syz;
}

// FP32 block Gauss-Seidel update of node (i, j, k) from its register neighbourhood (incident
// elements in elementsAdjacentNode order, TPSStencils.hh:47-73; node solve
// MultigridSolver.hh:348-378). Shared by the per-colour and the plane-pair sweeps, so both give
// bit-identical iterates.
template <typename KV>
__device__ __forceinline__ void gs_node_fp32(const Geom &g, const KV &Kv, const float *__restrict__ Y, float *u,
                                             const float *__restrict__ b, const uint8_t *__restrict__ dmask, int i,
                                             int j, int k, bool forward) {
    const int64_t n = g.node(i, j, k), ld = g.ld;
    const uint8_t dm = dmask[n];
    if (dm == 7) return;
    float s0 = b[n], s1 = b[ld + n], s2 = b[2 * ld + n];
    float M[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float E[8], Pa[9][3], Pb[9][3];
    load_elem_moduli<float>(g, Y, i, j, k, E);
    load_plane<float>(g, u, n, 0, Pa);
    load_plane<float>(g, u, n, 1, Pb);
    gs_visit_planes<float, 1, 1, 1>(Kv, Pa, Pb, E, s0, s1, s2, M);
    gs_visit_planes<float, 1, 0, 1>(Kv, Pa, Pb, E, s0, s1, s2, M);
    gs_visit_planes<float, 1, 1, 0>(Kv, Pa, Pb, E, s0, s1, s2, M);
    gs_visit_planes<float, 1, 0, 0>(Kv, Pa, Pb, E, s0, s1, s2, M);
    float u0 = Pb[4][0], u1 = Pb[4][1], u2 = Pb[4][2];
    load_plane<float>(g, u, n, 2, Pa);
    gs_visit_planes<float, 0, 1, 1>(Kv, Pb, Pa, E, s0, s1, s2, M);
    gs_visit_planes<float, 0, 0, 1>(Kv, Pb, Pa, E, s0, s1, s2, M);
    gs_visit_planes<float, 0, 1, 0>(Kv, Pb, Pa, E, s0, s1, s2, M);
    gs_visit_planes<float, 0, 0, 0>(Kv, Pb, Pa, E, s0, s1, s2, M);
    if constexpr (KV::kCube) cube_diag_block<float>(Kv, E, M);
    smooth_node_solve<float>(dm, s0, s1, s2, M, forward, u0, u1, u2);
    u[n] = u0;
    u[ld + n] = u1;
    u[2 * ld + n] = u2;
}

// One colour (x%2, y%2, z%2) = (cx, cy, cz) of multicoloured block Gauss-Seidel
// (MultigridSolver.hh:409-458); incident elements in elementsAdjacentNode order
// (TPSStencils.hh:47-73).
template <typename T, bool Cube>
__global__ void __launch_bounds__(BS, sizeof(T) == 4 ? 3 : 1) gs_fine_color_kernel(Geom g, const T *__restrict__ Y, T *u,
                                                           const T *__restrict__ b, const uint8_t *__restrict__ dmask,
                                                           int cx, int cy, int cz, int forward, const Mat24<T> K) {
    VFEM_PDL_ENTRY();
    // colour nodes over the full grid; detached rows (j >= nyv) are skipped
    const int n2 = (g.nn[2] - cz + 1) / 2, n1 = (g.nn[1] - cy + 1) / 2, n0 = (g.nn[0] - cx + 1) / 2;
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n1 <= 0 || t >= (int64_t)n0 * n1 * n2) return;
    int ii, jj, kk;
    decode3(t, n1, n2, ii, jj, kk);
    const int i = cx + 2 * ii, j = cy + 2 * jj, k = cz + 2 * kk;
    if (j >= g.nyv()) return;
    if constexpr (sizeof(T) == 4) {
        gs_node_fp32(g, K0View<T, Cube>(K), Y, u, b, dmask, i, j, k, forward != 0);
        return;
    }
    const int64_t n = g.node(i, j, k), ld = g.ld;
    const uint8_t dm = dmask[n];
    if (dm == 7) return;
    T s0 = b[n], s1 = b[ld + n], s2 = b[2 * ld + n];
    T M[9] = {T(0), T(0), T(0), T(0), T(0), T(0), T(0), T(0), T(0)};
    gs_visit<T, 1, 1, 1>(g, K, Y, u, i, j, k, s0, s1, s2, M);
    gs_visit<T, 0, 1, 1>(g, K, Y, u, i, j, k, s0, s1, s2, M);
    gs_visit<T, 1, 0, 1>(g, K, Y, u, i, j, k, s0, s1, s2, M);
    gs_visit<T, 0, 0, 1>(g, K, Y, u, i, j, k, s0, s1, s2, M);
    gs_visit<T, 1, 1, 0>(g, K, Y, u, i, j, k, s0, s1, s2, M);
    gs_visit<T, 0, 1, 0>(g, K, Y, u, i, j, k, s0, s1, s2, M);
    gs_visit<T, 1, 0, 0>(g, K, Y, u, i, j, k, s0, s1, s2, M);
    gs_visit<T, 0, 0, 0>(g, K, Y, u, i, j, k, s0, s1, s2, M);
    T u0 = u[n], u1 = u[ld + n], u2 = u[2 * ld + n];
    smooth_node_solve<T>(dm, s0, s1, s2, M, forward != 0, u0, u1, u2);
    u[n] = u0;
    u[ld + n] = u1;
    u[2 * ld + n] = u2;
}

// Barrier over the CTAs of one thread-block cluster with release / acquire semantics: the u
// updates of one sub-colour (global stores) are visible to every CTA of the cluster before any
// of them gathers the next sub-colour's neighbourhoods.
__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Plane-pair sweep: the four colours with x % 2 == cx in one launch. The stencil reaches only
// x +- 1, so while those colours run every x-plane of parity cx reads planes of the other parity
// (not updated in this launch) and its own: the planes are independent and the launch runs them
// all at once, one thread-block cluster per plane. Inside a plane the four colours (y % 2,
// z % 2) follow the reference's order (forward 0 -> 3, backward 3 -> 0) separated by cluster
// barriers; each CTA of the cluster owns a strip of rowsPerStrip y-rows. A sweep is two such
// launches (cx = 0 then 1 forward; 1 then 0 backward): the same node updates with the same
// operands as eight colour launches, so the iterates are identical, but u, E and b stream
// through DRAM about twice per sweep instead of once per colour.
template <bool Cube>
__global__ void __launch_bounds__(BS, 3) gs_fine_planes_kernel(Geom g, const float *__restrict__ Y, float *u,
                                                              const float *__restrict__ b,
                                                              const uint8_t *__restrict__ dmask, int cx,
                                                              int rowsPerStrip, int forward, const Mat24<float> K) {
    VFEM_PDL_ENTRY();
    const int i = cx + 2 * (int)blockIdx.y;
    const int j0 = (int)blockIdx.x * rowsPerStrip;
    const int j1 = min(j0 + rowsPerStrip, g.nyv());
    const K0View<float, Cube> Kv(K);
#pragma unroll 1
    for (int s = 0; s < 4; ++s) {
        const int sc = forward ? s : 3 - s;
        const int cy = sc >> 1, cz = sc & 1;
        const int jf = j0 + ((j0 & 1) != cy ? 1 : 0);
        const int nj = j1 > jf ? (j1 - jf + 1) / 2 : 0;
        const int nk = (g.nn[2] - cz + 1) / 2;
        const int cnt = nj * nk;
        for (int t = threadIdx.x; t < cnt; t += BS) {
            const int jj = (int)((uint32_t)t / (uint32_t)nk), kk = t - jj * nk;
            gs_node_fp32(g, Kv, Y, u, b, dmask, i, jf + 2 * jj, cz + 2 * kk, forward != 0);
        }
        if (s < 3) {
            if (gridDim.x > 1) cluster_barrier();
            else __syncthreads();
        }
    }
}

// Line-pair sweep: colours (cx, cy, 0) and (cx, cy, 1), adjacent in the reference's order, in
// one launch. Their nodes lie on the z-lines i % 2 == cx, j % 2 == cy, and among the nodes these
// two colours update a node reads only its own line's (k +- 1): the lines are independent. A CTA
// owns linesPerCta whole lines, updates the first colour's nodes on them, passes a block barrier,
// then updates the second colour's (z parity 0 then 1 forward, 1 then 0 backward). A sweep is
// four such launches; the node updates and their operands are those of the eight colour
// launches, so the iterates are identical.
template <bool Cube, int MB = 3>
__global__ void __launch_bounds__(BS, MB) gs_fine_lines_kernel(Geom g, const float *__restrict__ Y, float *u,
                                                             const float *__restrict__ b,
                                                             const uint8_t *__restrict__ dmask, int cx, int cy,
                                                             int linesPerCta, int forward, const Mat24<float> K) {
    VFEM_PDL_ENTRY();
    const int n1 = (g.nn[1] - cy + 1) / 2;  // lines of this class per x-plane
    const int nlines = ((g.nn[0] - cx + 1) / 2) * n1;
    const int l0 = (int)blockIdx.x * linesPerCta;
    const int nl = min(linesPerCta, nlines - l0);
    const int nyv = g.nyv();
    const K0View<float, Cube> Kv(K);
#pragma unroll 1
    for (int s = 0; s < 2; ++s) {
        const int cz = forward ? s : 1 - s;
        const int nk = (g.nn[2] - cz + 1) / 2;
        const int cnt = nl > 0 ? nl * nk : 0;
        for (int t = threadIdx.x; t < cnt; t += BS) {
            const int q = (int)((uint32_t)t / (uint32_t)nk), kk = t - q * nk;
            const int line = l0 + q;
            const int ii = (int)((uint32_t)line / (uint32_t)n1), jj = line - ii * n1;
            const int j = cy + 2 * jj;
            if (j < nyv) gs_node_fp32(g, Kv, Y, u, b, dmask, cx + 2 * ii, j, cz + 2 * kk, forward != 0);
        }
        if (s == 0) __syncthreads();
    }
}

// Staged line-pair sweep: the line-pair schedule with the CTA's neighbourhood in shared memory.
// A CTA owns linesPerCta consecutive lines (rows j = cy + 2 jj) of one x-plane i. It copies the
// u values of planes i-1..i+1, rows jbase..jbase+R-1 (R = 2 lines + 1, jbase the row below the
// first line) and z = -1..nz into shared memory, and the padded moduli of element planes
// i-1, i and element rows jbase..jbase+R-2, from the very addresses the other forms read. Each
// node then gathers its neighbourhood from shared memory; an update is written to shared and
// global memory (the second colour reads the first colour's updates from the tile). No other
// CTA reads this CTA's lines during the launch, so the tile stays exact; the arithmetic is the
// other forms', so are the iterates.
struct StagedTile {
    int R, NZ2, EZ2;  // rows, z extent with halo (nz + 2), padded element z extent (ne + 2)
    __device__ int uIdx(int c, int a, int r, int kk) const { return ((c * 3 + a) * R + r) * NZ2 + kk; }
    __device__ int eIdx(int a, int r, int kk) const { return (a * (R - 1) + r) * EZ2 + kk; }
};

template <typename KV>
__device__ __forceinline__ void gs_node_fp32_staged(const Geom &g, const KV &Kv, const StagedTile &T,
                                                    const float *sU0, float *sU, const float *sE, float *u,
                                                    const float *__restrict__ b, const uint8_t *__restrict__ dmask,
                                                    int i, int j, int k, int jbase, bool forward) {
    const int64_t n = g.node(i, j, k), ld = g.ld;
    const uint8_t dm = dmask[n];
    if (dm == 7) return;
    float s0 = b[n], s1 = b[ld + n], s2 = b[2 * ld + n];
    float M[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float E[8], Pa[9][3], Pb[9][3];
    const int r0 = j - jbase, kk0 = k + 1;  // the node's tile row and z index
    // E[4A + 2B + C]: element (i - A, j - B, k - C), element plane a = 1 - A, row r0 - B
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const int A = (s >> 2) & 1, B = (s >> 1) & 1, C = s & 1;
        E[s] = sE[T.eIdx(1 - A, r0 - B, k - C + 1)];
    }
    auto plane = [&](int a, float (&P)[9][3]) {
#pragma unroll
        for (int bb = 0; bb < 3; ++bb)
#pragma unroll
            for (int d = 0; d < 3; ++d)
#pragma unroll
                for (int c = 0; c < 3; ++c) P[3 * bb + c][d] = sU0[T.uIdx(d, a, r0 + bb - 1, kk0 + c - 1)];
    };
    plane(0, Pa);
    plane(1, Pb);
    gs_visit_planes<float, 1, 1, 1>(Kv, Pa, Pb, E, s0, s1, s2, M);
    gs_visit_planes<float, 1, 0, 1>(Kv, Pa, Pb, E, s0, s1, s2, M);
    gs_visit_planes<float, 1, 1, 0>(Kv, Pa, Pb, E, s0, s1, s2, M);
    gs_visit_planes<float, 1, 0, 0>(Kv, Pa, Pb, E, s0, s1, s2, M);
    float u0 = Pb[4][0], u1 = Pb[4][1], u2 = Pb[4][2];
    plane(2, Pa);
    gs_visit_planes<float, 0, 1, 1>(Kv, Pb, Pa, E, s0, s1, s2, M);
    gs_visit_planes<float, 0, 0, 1>(Kv, Pb, Pa, E, s0, s1, s2, M);
    gs_visit_planes<float, 0, 1, 0>(Kv, Pb, Pa, E, s0, s1, s2, M);
    gs_visit_planes<float, 0, 0, 0>(Kv, Pb, Pa, E, s0, s1, s2, M);
    if constexpr (KV::kCube) cube_diag_block<float>(Kv, E, M);
    smooth_node_solve<float>(dm, s0, s1, s2, M, forward, u0, u1, u2);
    sU[T.uIdx(0, 1, r0, kk0)] = u0;
    sU[T.uIdx(1, 1, r0, kk0)] = u1;
    sU[T.uIdx(2, 1, r0, kk0)] = u2;
    u[n] = u0;
    u[ld + n] = u1;
    u[2 * ld + n] = u2;
}

template <bool Cube>
__global__ void __launch_bounds__(BS, 3) gs_fine_staged_kernel(Geom g, const float *__restrict__ Y, float *u,
                                                              const float *__restrict__ b,
                                                              const uint8_t *__restrict__ dmask, int cx, int cy,
                                                              int linesPerCta, int forward, const Mat24<float> K) {
    VFEM_PDL_ENTRY();
    extern __shared__ float staged[];
    const int n1 = (g.nn[1] - cy + 1) / 2;
    const int i = cx + 2 * (int)blockIdx.y;
    const int jj0 = (int)blockIdx.x * linesPerCta;
    const int nl = min(linesPerCta, n1 - jj0);
    const int nyv = g.nyv();
    StagedTile T;
    T.R = 2 * linesPerCta + 1;
    T.NZ2 = g.nn[2] + 2;
    T.EZ2 = g.ne[2] + 2;
    const int jbase = cy + 2 * jj0 - 1;
    float *sU = staged;
    float *sE = staged + 9 * T.R * T.NZ2;
    // the tile: the addresses the unstaged forms gather from (guarded vector, padded moduli)
    const int64_t ld = g.ld;
    const int nU = 9 * T.R * T.NZ2;
    for (int q = threadIdx.x; q < nU; q += BS) {
        const int kk = q % T.NZ2, rest = q / T.NZ2;
        const int r = rest % T.R, ca = rest / T.R;
        const int a = ca % 3, c = ca / 3;
        // rows past nn[1] belong only to missing lines of the last CTA; row nn[1] itself (the one
        // past the last line) and planes / rows / z at -1 stay inside the vector's guard
        const int jr = jbase + r;
        sU[q] = jr <= g.nn[1] ? u[c * ld + g.node(i - 1 + a, jr, kk - 1)] : 0.f;
    }
    const int nE = 2 * (T.R - 1) * T.EZ2;
    for (int q = threadIdx.x; q < nE; q += BS) {
        const int kk = q % T.EZ2, rest = q / T.EZ2;
        const int r = rest % (T.R - 1), a = rest / (T.R - 1);
        const int je = min(jbase + r, g.ne[1]);  // rows past the grid read the zero ghost row
        sE[q] = Y[g.padElem(i - 1 + a, je, kk - 1)];
    }
    __syncthreads();
    const K0View<float, Cube> Kv(K);
#pragma unroll 1
    for (int s = 0; s < 2; ++s) {
        const int cz = forward ? s : 1 - s;
        const int nk = (g.nn[2] - cz + 1) / 2;
        const int cnt = nl > 0 ? nl * nk : 0;
        for (int t = threadIdx.x; t < cnt; t += BS) {
            const int q = (int)((uint32_t)t / (uint32_t)nk), kk = t - q * nk;
            const int j = cy + 2 * (jj0 + q);
            if (j < nyv)
                gs_node_fp32_staged(g, Kv, T, sU, sU, sE, u, b, dmask, i, j, cz + 2 * kk, jbase, forward != 0);
        }
        if (s == 0) __syncthreads();
    }
}

// ---------------- double-float FP64-accurate matvec ----------------
template <int LN, typename KV>
__device__ __forceinline__ void df_elem(const Geom &g, const KV &K, const float *__restrict__ uh_,
                                        const float *__restrict__ ul_, int64_t base, float *ch, float *cl) {
    const int64_t ld = g.ld;
    const int64_t sx = (int64_t)g.nn[1] * g.nn[2], sy = g.nn[2];
#pragma unroll
    for (int r = 0; r < 3; ++r) { ch[r] = 0.f; cl[r] = 0.f; }
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const int64_t nm = base + ((m >> 2) & 1) * sx + ((m >> 1) & 1) * sy + (m & 1);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float uh = uh_[c * ld + nm], ul = ul_[c * ld + nm];
#pragma unroll
            for (int r = 0; r < 3; ++r)
                df_fma_acc(K.hi(3 * m + c, 3 * LN + r), K.lo(3 * m + c, 3 * LN + r), uh, ul, ch[r], cl[r]);
        }
    }
}

template <int A, int B, int Cc, typename KV>
__device__ __forceinline__ void df_visit(const Geom &g, const KV &K, const float *__restrict__ Yh,
                                         const float *__restrict__ Yl, const float *__restrict__ uh,
                                         const float *__restrict__ ul, int i, int j, int k, float *fh, float *fl) {
    // zero-padded moduli: an element outside the grid reads E = 0; its node block is clamped
    // onto a valid element (keeps the loads predicated and the register count low)
    const int ei = i - A, ej = j - B, ek = k - Cc;
    const int64_t e = g.padElem(ei, ej, ek);
    const float eh = Yh[e], el = Yl[e];
    const int ci = min(max(ei, 0), g.ne[0] - 1), cj = min(max(ej, 0), g.ne[1] - 1), ck = min(max(ek, 0), g.ne[2] - 1);
    float ch[3], cl[3];
    df_elem<4 * A + 2 * B + Cc>(g, K, uh, ul, g.node(ci, cj, ck), ch, cl);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        // normalise the element sum, then accumulate E * contrib
        const float s = ch[r] + cl[r];
        const float sl = cl[r] - (s - ch[r]);
        df_fma_acc(eh, el, s, sl, fh[r], fl[r]);
    }
}

// out = K u with u given as its double-float split (uh + ul) and E as (Yh + Yl); out and the
// optional partial dot products u.out are FP64. No FP64 arithmetic in the inner loops.
// Yh, Yl are zero-padded element arrays (Geom::padElem) and uh, ul guarded vectors.
template <bool Cube>
__global__ void __launch_bounds__(BS) applyk_fine_df_kernel(Geom g, const float *__restrict__ Yh,
                                                            const float *__restrict__ Yl,
                                                            const float *__restrict__ uh,
                                                            const float *__restrict__ ul,
                                                            const double *__restrict__ u, double *__restrict__ out,
                                                            const uint8_t *__restrict__ dmask, int zeroDir,
                                                            double *__restrict__ partials, int withDot,
                                                            const double *__restrict__ rhs, const Mat24DF K) {
    VFEM_PDL_ENTRY();
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    double dot = 0.0;
    if (n < g.NN) {
        int i, j, k;
        decode_node(g, n, i, j, k);
        const int64_t ld = g.ld;
        double f[3] = {0.0, 0.0, 0.0};
        if (j < g.nyv()) {
            float fh[3] = {0.f, 0.f, 0.f}, fl[3] = {0.f, 0.f, 0.f};
            const K0DFView<Cube> Kv(K);
            df_visit<0, 0, 0>(g, Kv, Yh, Yl, uh, ul, i, j, k, fh, fl);
            df_visit<0, 0, 1>(g, Kv, Yh, Yl, uh, ul, i, j, k, fh, fl);
            df_visit<0, 1, 0>(g, Kv, Yh, Yl, uh, ul, i, j, k, fh, fl);
            df_visit<0, 1, 1>(g, Kv, Yh, Yl, uh, ul, i, j, k, fh, fl);
            df_visit<1, 0, 0>(g, Kv, Yh, Yl, uh, ul, i, j, k, fh, fl);
            df_visit<1, 0, 1>(g, Kv, Yh, Yl, uh, ul, i, j, k, fh, fl);
            df_visit<1, 1, 0>(g, Kv, Yh, Yl, uh, ul, i, j, k, fh, fl);
            df_visit<1, 1, 1>(g, Kv, Yh, Yl, uh, ul, i, j, k, fh, fl);
            const uint8_t dm = zeroDir ? dmask[n] : 0;
#pragma unroll
            for (int r = 0; r < 3; ++r) f[r] = ((dm >> r) & 1) ? 0.0 : (double)fh[r] + (double)fl[r];
            if (withDot) dot = u[n] * f[0] + u[ld + n] * f[1] + u[2 * ld + n] * f[2];
        }
        if (rhs) {
            // residual form: rhs - K u, zero on constrained components
            const uint8_t dm = dmask[n];
#pragma unroll
            for (int r = 0; r < 3; ++r) f[r] = ((dm >> r) & 1) ? 0.0 : rhs[r * ld + n] - f[r];
        }
        out[n] = f[0];
        out[ld + n] = f[1];
        out[2 * ld + n] = f[2];
    }
    if (withDot) {
        const double s = block_sum<BS>(dot);
        if (threadIdx.x == 0) partials[blockIdx.x] = s;
    }
}

// Zero-padded FP32 copies of the moduli: hi = fl(Y) and, if lo is given, lo = fl(Y - hi).
__global__ void pad_young_kernel(Geom g, const double *__restrict__ Y, float *__restrict__ hi,
                                 float *__restrict__ lo) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= g.padNE()) return;
    int pi, pj, pk;
    decode3(t, g.ne[1] + 2, g.ne[2] + 2, pi, pj, pk);
    const int i = pi - 1, j = pj - 1, k = pk - 1;
    const bool in = i >= 0 && j >= 0 && k >= 0 && i < g.ne[0] && j < g.ne[1] && k < g.ne[2];
    const double v = in ? Y[g.elem(i, j, k)] : 0.0;
    const float h = __double2float_rn(v);
    hi[t] = h;
    if (lo) lo[t] = __double2float_rn(v - (double)h);
}

__global__ void split_df_kernel(const double *__restrict__ src, float *__restrict__ hi, float *__restrict__ lo,
                                int64_t n) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= n) return;
    float h, l;
    df_split(src[t], h, l);
    hi[t] = h;
    lo[t] = l;
}

// ---------------- element-wise kernels ----------------
template <typename T>
__global__ void young_kernel(Geom g, const double *__restrict__ rho, T *__restrict__ Y, double E0, double Emin,
                             double gamma, double q, int law, int masking, int ipow) {
    const int64_t e = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (e >= g.NE) return;
    const int ej = (int)(((uint32_t)e / (uint32_t)g.ne[2]) % (uint32_t)g.ne[1]);
    double v;
    if (masking && ej >= g.maskedE()) {
        v = 0.0;
    } else {
        const double r = rho[e];
        if (law == 0) {
            // integer SIMP exponents (the usual 3) as repeated products: FP64 pow is a long
            // dependent sequence on this part; the product differs from it by an ulp or two
            double pw = r;
            if (ipow > 0)
                for (int t = 1; t < ipow; ++t) pw *= r;
            else
                pw = pow(r, gamma);
            v = Emin + pw * (E0 - Emin);
        }
        else v = Emin + r * (E0 - Emin) / (1 + q * (1 - r));
    }
    Y[e] = (T)v;
}

// TensorProductSimulator.hh:973-1005
// grad_e = wF * lam^T df/drho_e - wK * dE/drho_e * lam_e^T K0 u_e, df/drho_e the self-weight load
// of element e (g vol / 8 on each of its nodes). lam = u, wF = 1, wK = 1/2 is the compliance
// gradient (TensorProductSimulator.hh:973-1005); wF = wK = 1 is the adjoint-method gradient
// lam^T (df/drho - dK/drho u) of an objective whose adjoint state is lam.
__global__ void __launch_bounds__(BS) compliance_grad_kernel(Geom g, const double *__restrict__ rho,
                                                             const double *__restrict__ lam,
                                                             const double *__restrict__ u, double *__restrict__ grad,
                                                             double E0, double Emin, double gamma, double q, int law,
                                                             double gx, double gy, double gz, double vol, double wF,
                                                             double wK, const Mat24<double> K) {
    const int64_t e = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (e >= g.NE) return;
    int ei, ej, ek;
    decode3(e, g.ne[1], g.ne[2], ei, ej, ek);
    if (ej >= g.maskedE()) { grad[e] = 0.0; return; }
    const int64_t base = g.node(ei, ej, ek), ld = g.ld;
    const int64_t sx = (int64_t)g.nn[1] * g.nn[2], sy = g.nn[2];
    double ue[24], le[24];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const int64_t nm = base + ((m >> 2) & 1) * sx + ((m >> 1) & 1) * sy + (m & 1);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            ue[3 * m + c] = u[c * ld + nm];
            le[3 * m + c] = lam[c * ld + nm];
        }
    }
    double lKu = 0.0;
#pragma unroll
    for (int r = 0; r < 24; ++r) {
        double acc = 0.0;
#pragma unroll
        for (int c = 0; c < 24; ++c) acc += K.a[r * 24 + c] * ue[c];
        lKu += le[r] * acc;
    }
    const double rh = rho[e];
    double dE;
    if (law == 0) dE = gamma * pow(rh, gamma - 1.0) * (E0 - Emin);
    else dE = (1 + q) * (E0 - Emin) / ((1 + q * (1 - rh)) * (1 + q * (1 - rh)));
    double val = -wK * dE * lKu;
    if (gx != 0.0 || gy != 0.0 || gz != 0.0) {
#pragma unroll
        for (int l = 0; l < 8; ++l) val += wF * 0.125 * (gx * le[3 * l] + gy * le[3 * l + 1] + gz * le[3 * l + 2]) * vol;
    }
    grad[e] = val;
}

__global__ void __launch_bounds__(BS) element_energy_kernel(Geom g, const double *__restrict__ Y,
                                                            const double *__restrict__ u, double *__restrict__ out,
                                                            const Mat24<double> K) {
    const int64_t e = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (e >= g.NE) return;
    int ei, ej, ek;
    decode3(e, g.ne[1], g.ne[2], ei, ej, ek);
    const int64_t base = g.node(ei, ej, ek), ld = g.ld;
    const int64_t sx = (int64_t)g.nn[1] * g.nn[2], sy = g.nn[2];
    double ue[24];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const int64_t nm = base + ((m >> 2) & 1) * sx + ((m >> 1) & 1) * sy + (m & 1);
        ue[3 * m] = u[nm];
        ue[3 * m + 1] = u[ld + nm];
        ue[3 * m + 2] = u[2 * ld + nm];
    }
    double uKu = 0.0;
#pragma unroll
    for (int r = 0; r < 24; ++r) {
        double acc = 0.0;
#pragma unroll
        for (int c = 0; c < 24; ++c) acc += K.a[r * 24 + c] * ue[c];
        uKu += ue[r] * acc;
    }
    out[e] = 0.5 * Y[e] * uKu;
}

// Self-weight load (TensorProductSimulator.hh:1275-1286) gathered per node.
__global__ void gravity_load_kernel(Geom g, const double *__restrict__ rho, double *__restrict__ f, double gx,
                                    double gy, double gz, double vol) {
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n >= g.NN) return;
    int i, j, k;
    decode_node(g, n, i, j, k);
    double acc0 = 0, acc1 = 0, acc2 = 0;
    for (int a = 1; a >= 0; --a)
        for (int b = 1; b >= 0; --b)
            for (int c = 1; c >= 0; --c) {
                const int ei = i - a, ej = j - b, ek = k - c;
                if (ei < 0 || ej < 0 || ek < 0 || ei >= g.ne[0] || ej >= g.ne[1] || ek >= g.ne[2]) continue;
                if (ej >= g.maskedE()) continue;
                const double w = 0.125 * rho[g.elem(ei, ej, ek)] * vol;
                acc0 += gx * w;
                acc1 += gy * w;
                acc2 += gz * w;
            }
    f[n] += acc0;
    f[g.ld + n] += acc1;
    f[2 * g.ld + n] += acc2;
}

template <typename T>
__global__ void convert_kernel(const double *__restrict__ src, T *__restrict__ dst, int64_t n) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t < n) dst[t] = (T)src[t];
}

}  // namespace

template <typename T>
void launch_young_moduli(const Geom &g, const double *rho, T *Y, double E0, double Emin, double gamma, double q,
                         int law, bool masking, cudaStream_t st) {
    const int ipow = (gamma >= 1.0 && gamma <= 8.0 && gamma == (double)(int)gamma) ? (int)gamma : 0;
    young_kernel<T><<<gridFor(g.NE, BS), BS, 0, st>>>(g, rho, Y, E0, Emin, gamma, q, law, masking ? 1 : 0, ipow);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_convert(const void *src, bool srcDouble, T *dst, int64_t n, cudaStream_t st) {
    if (!srcDouble) throw Error(ERR_ARG, "launch_convert expects an FP64 source");
    convert_kernel<T><<<gridFor(n, BS), BS, 0, st>>>((const double *)src, dst, n);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_applyk_fine(const Geom &g, const T *Y, const T *u, T *out, const Mat24<T> &K0, bool zeroInit, bool negate,
                        const uint8_t *dmask, bool zeroDirichlet, double *partialDot, int partialBlocks,
                        cudaStream_t st) {
    const unsigned grid = gridFor(g.NN, BS);
    const int zd = zeroDirichlet ? 1 : 0;
    if (partialDot && (int)grid > partialBlocks) throw Error(ERR_ARG, "partial buffer too small");
    auto go = [&](auto cube) {
        constexpr bool C = decltype(cube)::value;
        if (partialDot)
            launch_pdl(applyk_fine_kernel<T, true, false, true, C>, grid, BS, 0, st, g, Y, u, out, dmask, zd, partialDot, K0);
        else if (zeroInit && negate)
            launch_pdl(applyk_fine_kernel<T, true, true, false, C>, grid, BS, 0, st, g, Y, u, out, dmask, zd, nullptr, K0);
        else if (zeroInit)
            launch_pdl(applyk_fine_kernel<T, true, false, false, C>, grid, BS, 0, st, g, Y, u, out, dmask, zd, nullptr, K0);
        else if (negate)
            launch_pdl(applyk_fine_kernel<T, false, true, false, C>, grid, BS, 0, st, g, Y, u, out, dmask, zd, nullptr, K0);
        else
            launch_pdl(applyk_fine_kernel<T, false, false, false, C>, grid, BS, 0, st, g, Y, u, out, dmask, zd, nullptr, K0);
    };
    if (sizeof(T) == 4 && K0.isCube) go(std::true_type{});
    else go(std::false_type{});
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_residual_fine(const Geom &g, const T *Y, const T *u, const T *b, T *r, const Mat24<T> &K0,
                          const uint8_t *dmask, cudaStream_t st) {
    // the cube-voxel FP32 residual fits 64 registers without spills: four resident blocks per SM
    // (measured 0.117 ms against 0.160 ms at two blocks, 12.8M DOF)
    const int occ = fineOccupancy() ? fineOccupancy() : 4;
    if (sizeof(T) == 4 && K0.isCube && occ == 4)
        launch_pdl(residual_fine_kernel<T, true, 4>, gridFor(g.NN, BS), BS, 0, st, g, Y, u, b, r, dmask, K0);
    else if (sizeof(T) == 4 && K0.isCube && occ == 3)
        launch_pdl(residual_fine_kernel<T, true, 3>, gridFor(g.NN, BS), BS, 0, st, g, Y, u, b, r, dmask, K0);
    else if (sizeof(T) == 4 && K0.isCube) launch_pdl(residual_fine_kernel<T, true>, gridFor(g.NN, BS), BS, 0, st, g, Y, u, b, r, dmask, K0);
    else launch_pdl(residual_fine_kernel<T, false>, gridFor(g.NN, BS), BS, 0, st, g, Y, u, b, r, dmask, K0);
    VFEM_LAUNCH_CHECK();
}

// Strips per x-plane (the cluster size) of the plane-pair sweep: about three resident CTAs per SM
// over the planes of one parity, at most 8 (the portable cluster size) and at least two rows per
// strip.
static int gsPlaneStrips(const Geom &g) {
    if (const char *e = std::getenv("VFEM_GS_PLANE_STRIPS")) {
        const int c = std::atoi(e);
        if (c >= 1 && c <= 8) return std::min(c, std::max(1, g.nn[1] / 2));
    }
    const int planes = (g.nn[0] + 1) / 2;
    int c = (3 * NUM_SMS) / planes;  // one wave of three CTAs per SM
    c = std::max(1, std::min(c, 8));
    while (c > 1 && (g.nn[1] + c - 1) / c < 2) --c;
    return c;
}

int fineOccupancy() {
    const char *e = std::getenv("VFEM_FINE_OCC");
    return e ? std::atoi(e) : 0;
}

int gsFineMode() {
    const char *e = std::getenv("VFEM_GS_MODE");
    if (!e) return GS_LINES;
    const std::string m(e);
    if (m == "colours") return GS_COLOURS;
    if (m == "planes") return GS_PLANES;
    if (m == "staged") return GS_STAGED;
    return GS_LINES;
}

// Lines per CTA of the staged sweep and its shared-memory bytes: about one 256-thread round of
// nodes per colour, within the 227 KB a CTA may use.
static int stagedLines(const Geom &g) { return std::max(1, BS / ((g.nn[2] + 1) / 2)); }
static size_t stagedBytes(const Geom &g, int lines) {
    const int R = 2 * lines + 1;
    return sizeof(float) * ((size_t)9 * R * (g.nn[2] + 2) + (size_t)2 * (R - 1) * (g.ne[2] + 2));
}

bool gsStagedFits(const Geom &g) { return stagedBytes(g, stagedLines(g)) <= 72 * 1024; }  // three CTAs per SM

void launch_gs_fine_staged(const Geom &g, const float *Y, float *u, const float *b, const uint8_t *dmask, int cx,
                           int cy, bool forward, const Mat24<float> &K0, cudaStream_t st) {
    const int planes = (g.nn[0] - cx + 1) / 2, n1 = (g.nn[1] - cy + 1) / 2;
    if (planes <= 0 || n1 <= 0) return;
    const int L = stagedLines(g);
    const size_t smem = stagedBytes(g, L);
    if (smem > 227 * 1024) throw Error(ERR_ARG, "staged sweep: tile too large for shared memory");
    static bool attrSet[2] = {false, false};
    auto kern = K0.isCube ? gs_fine_staged_kernel<true> : gs_fine_staged_kernel<false>;
    const int ki = K0.isCube ? 1 : 0;
    if (!attrSet[ki]) {
        VFEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
        attrSet[ki] = true;
    }
    const dim3 grid((unsigned)((n1 + L - 1) / L), (unsigned)planes);
    launch_pdl(kern, grid, BS, smem, st, g, Y, u, b, dmask, cx, cy, L, forward ? 1 : 0, K0);
    VFEM_LAUNCH_CHECK();
}

void launch_gs_fine_lines(const Geom &g, const float *Y, float *u, const float *b, const uint8_t *dmask, int cx,
                          int cy, bool forward, const Mat24<float> &K0, cudaStream_t st) {
    const int nlines = ((g.nn[0] - cx + 1) / 2) * ((g.nn[1] - cy + 1) / 2);
    if (nlines <= 0) return;
    // about one wave of three CTAs per SM, whole lines per CTA
    const int per = std::max(1, (nlines + 3 * NUM_SMS - 1) / (3 * NUM_SMS));
    const unsigned grid = (unsigned)((nlines + per - 1) / per);
    const int fw = forward ? 1 : 0;
    if (K0.isCube && fineOccupancy() == 4)
        launch_pdl(gs_fine_lines_kernel<true, 4>, grid, BS, 0, st, g, Y, u, b, dmask, cx, cy, per, fw, K0);
    else if (K0.isCube)
        launch_pdl(gs_fine_lines_kernel<true>, grid, BS, 0, st, g, Y, u, b, dmask, cx, cy, per, fw, K0);
    else
        launch_pdl(gs_fine_lines_kernel<false>, grid, BS, 0, st, g, Y, u, b, dmask, cx, cy, per, fw, K0);
    VFEM_LAUNCH_CHECK();
}

void launch_gs_fine_planes(const Geom &g, const float *Y, float *u, const float *b, const uint8_t *dmask, int cx,
                           bool forward, const Mat24<float> &K0, cudaStream_t st) {
    const int planes = (g.nn[0] - cx + 1) / 2;
    if (planes <= 0) return;
    const int strips = gsPlaneStrips(g);
    const int rows = (g.nn[1] + strips - 1) / strips;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(strips, planes, 1);
    cfg.blockDim = dim3(BS, 1, 1);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[2];
    int na = 0;
    attr[na].id = cudaLaunchAttributeClusterDimension;
    attr[na].val.clusterDim.x = strips;
    attr[na].val.clusterDim.y = 1;
    attr[na].val.clusterDim.z = 1;
    ++na;
    if (pdlEnabled()) {
        attr[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[na].val.programmaticStreamSerializationAllowed = 1;
        ++na;
    }
    cfg.attrs = attr;
    cfg.numAttrs = na;
    const int fw = forward ? 1 : 0;
    if (K0.isCube)
        cudaCheck(cudaLaunchKernelEx(&cfg, gs_fine_planes_kernel<true>, g, Y, u, b, dmask, cx, rows, fw, K0),
                  "kernel launch");
    else
        cudaCheck(cudaLaunchKernelEx(&cfg, gs_fine_planes_kernel<false>, g, Y, u, b, dmask, cx, rows, fw, K0),
                  "kernel launch");
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_gs_fine_color(const Geom &g, const T *Y, T *u, const T *b, const uint8_t *dmask, int color, bool forward,
                          const Mat24<T> &K0, cudaStream_t st) {
    const int cx = (color >> 2) & 1, cy = (color >> 1) & 1, cz = color & 1;
    const int64_t n0 = (g.nn[0] - cx + 1) / 2, n1 = (g.nn[1] - cy + 1) / 2, n2 = (g.nn[2] - cz + 1) / 2;
    if (n1 <= 0) return;
    if (sizeof(T) == 4 && K0.isCube)
        launch_pdl(gs_fine_color_kernel<T, true>, gridFor(n0 * n1 * n2, BS), BS, 0, st, g, Y, u, b, dmask, cx, cy, cz,
                                                                               forward ? 1 : 0, K0);
    else
        launch_pdl(gs_fine_color_kernel<T, false>, gridFor(n0 * n1 * n2, BS), BS, 0, st, g, Y, u, b, dmask, cx, cy, cz,
                                                                                forward ? 1 : 0, K0);
    VFEM_LAUNCH_CHECK();
}

void launch_applyk_fine_df(const Geom &g, const float *Yh, const float *Yl, const float *uh, const float *ul,
                           const double *u, double *out, const Mat24DF &K0, const uint8_t *dmask, bool zeroDirichlet,
                           double *partialDot, int partialBlocks, cudaStream_t st, const double *rhs) {
    const unsigned grid = gridFor(g.NN, BS);
    if (partialDot && (int)grid > partialBlocks) throw Error(ERR_ARG, "partial buffer too small");
    if (K0.isCube)
        launch_pdl(applyk_fine_df_kernel<true>, grid, BS, 0, st, g, Yh, Yl, uh, ul, u, out, dmask, zeroDirichlet ? 1 : 0,
                                                         partialDot, partialDot ? 1 : 0, rhs, K0);
    else
        launch_pdl(applyk_fine_df_kernel<false>, grid, BS, 0, st, g, Yh, Yl, uh, ul, u, out, dmask, zeroDirichlet ? 1 : 0,
                                                          partialDot, partialDot ? 1 : 0, rhs, K0);
    VFEM_LAUNCH_CHECK();
}

void launch_pad_young(const Geom &g, const double *Y, float *hi, float *lo, cudaStream_t st) {
    pad_young_kernel<<<gridFor(g.padNE(), BS), BS, 0, st>>>(g, Y, hi, lo);
    VFEM_LAUNCH_CHECK();
}

void launch_split_df(const double *src, float *hi, float *lo, int64_t n, cudaStream_t st) {
    split_df_kernel<<<gridFor(n, BS), BS, 0, st>>>(src, hi, lo, n);
    VFEM_LAUNCH_CHECK();
}

void launch_compliance_gradient(const Geom &g, const double *rho, const double *u, double *grad,
                                const Mat24<double> &K0, double E0, double Emin, double gamma, double q, int law,
                                const double *grav, double vol, cudaStream_t st) {
    launch_adjoint_sensitivity(g, rho, u, u, grad, K0, E0, Emin, gamma, q, law, grav, vol, 1.0, 0.5, st);
}

void launch_adjoint_sensitivity(const Geom &g, const double *rho, const double *lam, const double *u, double *grad,
                                const Mat24<double> &K0, double E0, double Emin, double gamma, double q, int law,
                                const double *grav, double vol, double wF, double wK, cudaStream_t st) {
    compliance_grad_kernel<<<gridFor(g.NE, BS), BS, 0, st>>>(g, rho, lam, u, grad, E0, Emin, gamma, q, law, grav[0],
                                                             grav[1], grav[2], vol, wF, wK, K0);
    VFEM_LAUNCH_CHECK();
}

void launch_element_energy(const Geom &g, const double *Y, const double *u, double *out, const Mat24<double> &K0,
                           cudaStream_t st) {
    element_energy_kernel<<<gridFor(g.NE, BS), BS, 0, st>>>(g, Y, u, out, K0);
    VFEM_LAUNCH_CHECK();
}

void launch_build_gravity_load(const Geom &g, const double *rho, double *f, const double *grav, double vol,
                               cudaStream_t st) {
    gravity_load_kernel<<<gridFor(g.NN, BS), BS, 0, st>>>(g, rho, f, grav[0], grav[1], grav[2], vol);
    VFEM_LAUNCH_CHECK();
}

#define VFEM_INST_FINE(T)                                                                                              \
    template void launch_young_moduli<T>(const Geom &, const double *, T *, double, double, double, double, int, bool, \
                                         cudaStream_t);                                                                \
    template void launch_convert<T>(const void *, bool, T *, int64_t, cudaStream_t);                                   \
    template void launch_applyk_fine<T>(const Geom &, const T *, const T *, T *, const Mat24<T> &, bool, bool,        \
                                        const uint8_t *, bool, double *, int, cudaStream_t);                           \
    template void launch_residual_fine<T>(const Geom &, const T *, const T *, const T *, T *, const Mat24<T> &,       \
                                          const uint8_t *, cudaStream_t);                                              \
    template void launch_gs_fine_color<T>(const Geom &, const T *, T *, const T *, const uint8_t *, int, bool,        \
                                          const Mat24<T> &, cudaStream_t);
VFEM_INST_FINE(double)
VFEM_INST_FINE(float)

}  // namespace vfem
