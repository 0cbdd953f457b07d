// Dense FP64 coarsest-level solve (blocked Cholesky + explicit inverse, replacing the
// reference's CHOLMOD factorisation, TensorProductSimulator.hh:1198-1230) and the
// PCG vector kernels with deterministic warp-shuffle reductions
// (MultigridSolver.hh:1047-1152, TensorProductSimulator.hh:414-459).
#include "vfem_kernels.hpp"

#include <algorithm>
#include <cstdlib>
#include "vfem_reduce.cuh"
#include "vfem_stencil.cuh"
#include "vfem_widen.h"

namespace vfem {

namespace {

constexpr int BS = 256;
constexpr int TB = DENSE_TILE;

// ---------------- dense assembly ----------------
template <typename T>
__global__ void dense_from_stencil_kernel(Geom g, const T *__restrict__ S, const int *__restrict__ red,
                                          double *__restrict__ A, int nfree, int rows) {
    // thread per (row dof of a node, stencil entry): row = 3n + r
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= g.NN * 243) return;
    const int64_t n = t / 243;
    const int q = (int)(t % 243);  // row entry of the node-contiguous stencil
    const int o = q / 9, r = (q % 9) / 3, c = q % 3;
    int i, j, k;
    stencil::decode(n, g.nn[1], g.nn[2], i, j, k);
    const int ni = i + o / 9 - 1, nj = j + (o / 3) % 3 - 1, nk = k + o % 3 - 1;
    if (ni < 0 || nj < 0 || nk < 0 || ni >= g.nn[0] || nj >= g.nn[1] || nk >= g.nn[2]) return;
    const int64_t m = g.node(ni, nj, nk);
    const int ra = red[3 * n + r], cb = red[3 * m + c];
    if (ra < 0 || cb < 0) return;
    T v;
    if (rows) v = S[n * 256 + q];
    else if (o >= 13) v = S[(int64_t)((o - 13) * 9 + 3 * r + c) * g.ld + stencil::colour_pos(g, i, j, k)];
    else v = S[(int64_t)((13 - o) * 9 + 3 * c + r) * g.ld + stencil::colour_pos(g, ni, nj, nk)];  // stored half
    A[(int64_t)ra * nfree + cb] = (double)v;
}

__global__ void symmetrize_kernel(double *A, int n) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= (int64_t)n * n) return;
    const int i = (int)(t / n), j = (int)(t % n);
    if (j >= i) return;
    const double v = 0.5 * (A[(int64_t)i * n + j] + A[(int64_t)j * n + i]);
    A[(int64_t)i * n + j] = v;
    A[(int64_t)j * n + i] = v;
}

// ---------------- blocked right-looking Cholesky (lower, in place, row-major) ----------------
// Step k: factor the diagonal tile and invert it (tile factor L_kk and its inverse), then
// the tiles below it are X = A_ik L_kk^{-T} and every trailing lower tile is updated with
// one TB x TB x TB product per block. Dependent FP64 operations cost tens of cycles and a
// division or square root hundreds on this part, so the only sequential chains are the
// TB pivot steps of each diagonal tile; panel solves and the triangular inverse become
// plain tile products against the inverted diagonal tiles.
// Tiles are read through L2 (ld.global.cg): in the persistent form other blocks rewrite them
// between the phases, and a stale line in this SM's L1 must not be used.
__device__ __forceinline__ void load_tile(const double *A, int n, int r0, int c0, double (*t)[TB + 1]) {
    const int ty = threadIdx.y, tx = threadIdx.x;
    t[ty][tx] = (r0 + ty < n && c0 + tx < n) ? __ldcg(A + (int64_t)(r0 + ty) * n + c0 + tx) : 0.0;
}

// 1/sqrt(d): single-precision seed refined by two Newton-Raphson steps,
// y <- y + y (1 - d y^2) / 2, each doubling the number of correct bits (24 -> 48 -> full).
// Pivots outside the single-precision normal range take the plain quotient.
__device__ __forceinline__ double rsqrt_newton(double d) {
    if (!(d > 1e-30 && d < 1e30)) return 1.0 / sqrt(d);
    double y = (double)rsqrtf((float)d);
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const double t = d * y;
        const double e = fma(-t, y, 1.0);
        y = fma(0.5 * y, e, y);
    }
    return y;
}

// 1/d: single-precision seed refined by two Newton-Raphson steps for the reciprocal,
// y <- y + y (1 - d y), each doubling the number of correct bits (24 -> 48 -> full).
// Pivots outside the single-precision normal range take the plain quotient.
__device__ __forceinline__ double recip_newton(double d) {
    if (!(d > 1e-30 && d < 1e30)) return 1.0 / d;
    double y = (double)__frcp_rn((float)d);
#pragma unroll
    for (int it = 0; it < 2; ++it) y = fma(y, fma(-d, y, 1.0), y);
    return y;
}

__device__ __forceinline__ void ldl_pivot(int j, double d, int nb, double *rd, double *dv, int *status) {
    if (!(d > 0.0)) {
        if (j < nb) atomicMax(status, 1);
        d = 1.0;
    }
    dv[j] = d;
    rd[j] = recip_newton(d);
}

// One block of TB x TB threads factors tile (k, k) in shared memory as U D U^T (U unit lower)
// and inverts U in the same sweep: W = U^{-1} follows from the elimination's row operations
// W_y -= U_yj W_j, which in step j touch the columns <= j of the rows below j while the
// rank-one update a_yx -= U_yj a_xj touches the columns > j, so one barrier per pivot serves
// both and a thread updates either an entry of the trailing triangle or one of W with the same
// two instructions. FP64 operations issue at about two per clock per SM here and a dependent
// one waits tens of cycles, so the only chain between steps is the next pivot's reciprocal,
// formed by its owner thread as soon as its last update lands. Written back: the Cholesky factor
// L = U D^{1/2} (lower tile of A) and L^{-1} = D^{-1/2} W (Dinv[k]).
__device__ __forceinline__ void chol_diag_body(double *A, double *Dinv, int n, int k, int *status) {
    __shared__ double sa[TB][TB + 1], sw[TB][TB + 1];
    __shared__ double rd[TB], dv[TB], rs[TB];
    const int ty = threadIdx.y, tx = threadIdx.x;
    const int kb = k * TB;
    const int nb = min(TB, n - kb);
    load_tile(A, n, kb, kb, sa);
    if (!(ty < nb && tx < nb)) sa[ty][tx] = (ty == tx) ? 1.0 : 0.0;
    sw[ty][tx] = (ty == tx) ? 1.0 : 0.0;
    __syncthreads();
    if (ty == 0 && tx == 0) ldl_pivot(0, sa[0][0], nb, rd, dv, status);
    __syncthreads();
    for (int j = 0; j < TB; ++j) {
        if (ty > j && tx <= ty) {
            const bool trailing = tx > j;
            const double m = sa[ty][j] * rd[j];  // U_yj; column j is final after step j - 1
            double *t = trailing ? &sa[ty][tx] : &sw[ty][tx];
            const double o = trailing ? sa[tx][j] : sw[j][tx];  // row j of W is final too
            const double v = fma(-m, o, *t);
            *t = v;
            if (tx == j + 1 && ty == j + 1) ldl_pivot(j + 1, v, nb, rd, dv, status);
        }
        __syncthreads();
    }
    if (ty == 0) rs[tx] = rsqrt_newton(dv[tx]);
    __syncthreads();
    if (ty < nb && tx < nb)
        A[(int64_t)(kb + ty) * n + kb + tx] = (tx < ty) ? sa[ty][tx] * rs[tx] : (tx == ty) ? dv[ty] * rs[ty] : 0.0;
    Dinv[(int64_t)k * TB * TB + ty * TB + tx] = (tx <= ty) ? sw[ty][tx] * rs[ty] : 0.0;
    __syncthreads();
}

__global__ void chol_diag_kernel(double *A, double *Dinv, int n, int k, int *status) {
    VFEM_PDL_ENTRY();
    chol_diag_body(A, Dinv, n, k, status);
}

// TB-term dot product of rows of two shared tiles, four independent chains
__device__ __forceinline__ double tile_dot(const double *a, int sa, const double *b, int sb) {
    double c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0;
#pragma unroll
    for (int q = 0; q < TB; q += 4) {
        c0 = fma(a[q * sa], b[q * sb], c0);
        c1 = fma(a[(q + 1) * sa], b[(q + 1) * sb], c1);
        c2 = fma(a[(q + 2) * sa], b[(q + 2) * sb], c2);
        c3 = fma(a[(q + 3) * sa], b[(q + 3) * sb], c3);
    }
    return (c0 + c1) + (c2 + c3);
}

// tiles (i, k), i > k: L_ik = A_ik L_kk^{-T}
__device__ __forceinline__ void chol_trsm_body(double *A, const double *Dinv, int n, int k, int tile) {
    __shared__ double sz[TB][TB + 1], sx[TB][TB + 1];
    const int ty = threadIdx.y, tx = threadIdx.x;
    const int kb = k * TB, r0 = kb + TB * (1 + tile);
    const int nb = min(TB, n - kb);
    sz[ty][tx] = __ldcg(Dinv + (int64_t)k * TB * TB + ty * TB + tx);
    load_tile(A, n, r0, kb, sx);
    __syncthreads();
    const double v = tile_dot(&sx[ty][0], 1, &sz[tx][0], 1);
    if (r0 + ty < n && tx < nb) A[(int64_t)(r0 + ty) * n + kb + tx] = v;
    __syncthreads();
}

__global__ void chol_trsm_kernel(double *A, const double *Dinv, int n, int k) {
    VFEM_PDL_ENTRY();
    chol_trsm_body(A, Dinv, n, k, blockIdx.x);
}

__device__ __forceinline__ void lower_tile_of(int idx, int &ii, int &jj) {
    ii = 0;
    while (idx > ii) { idx -= ii + 1; ++ii; }
    jj = idx;
}

// trailing tiles (i, j), k < j <= i: A_ij -= L_ik L_jk^T
__device__ __forceinline__ void chol_syrk_body(double *A, int n, int k, int tile) {
    __shared__ double sa[TB][TB + 1], sb[TB][TB + 1];
    int ii, jj;
    lower_tile_of(tile, ii, jj);
    const int i = k + 1 + ii, j = k + 1 + jj;
    const int ty = threadIdx.y, tx = threadIdx.x;
    const int kb = k * TB;
    load_tile(A, n, i * TB, kb, sa);
    load_tile(A, n, j * TB, kb, sb);
    __syncthreads();
    const double acc = tile_dot(&sa[ty][0], 1, &sb[tx][0], 1);
    const int gr = i * TB + ty, gc = j * TB + tx;
    if (gr < n && gc < n) A[(int64_t)gr * n + gc] = __ldcg(A + (int64_t)gr * n + gc) - acc;
    __syncthreads();
}

__global__ void chol_syrk_kernel(double *A, int n, int k) {
    VFEM_PDL_ENTRY();
    chol_syrk_body(A, n, k, blockIdx.x);
}

// Z = L^{-1}, right-looking over block rows. Step k: Z[k][c] = L_kk^{-1} Z[k][c] (c <= k),
// then Z[i][c] -= L[i][k] Z[k][c] for i > k.
__device__ __forceinline__ void trinv_diag_body(const double *Dinv, double *Z, int n, int k, int c) {
    __shared__ double sz[TB][TB + 1], sx[TB][TB + 1];
    const int ty = threadIdx.y, tx = threadIdx.x;
    const int r0 = k * TB, c0 = c * TB;
    sz[ty][tx] = __ldcg(Dinv + (int64_t)k * TB * TB + ty * TB + tx);
    load_tile(Z, n, r0, c0, sx);
    __syncthreads();
    const double v = tile_dot(&sz[ty][0], 1, &sx[0][tx], TB + 1);
    if (r0 + ty < n && c0 + tx < n) Z[(int64_t)(r0 + ty) * n + c0 + tx] = v;
    __syncthreads();
}

__global__ void trinv_diag_kernel(const double *Dinv, double *Z, int n, int k) {
    VFEM_PDL_ENTRY();
    trinv_diag_body(Dinv, Z, n, k, blockIdx.x);
}

__device__ __forceinline__ void trinv_update_body(const double *L, double *Z, int n, int k, int tile) {
    __shared__ double sa[TB][TB + 1], sb[TB][TB + 1];
    const int c = tile % (k + 1);
    const int i = k + 1 + tile / (k + 1);
    const int ty = threadIdx.y, tx = threadIdx.x;
    load_tile(L, n, i * TB, k * TB, sa);
    load_tile(Z, n, k * TB, c * TB, sb);
    __syncthreads();
    const double acc = tile_dot(&sa[ty][0], 1, &sb[0][tx], TB + 1);
    const int gr = i * TB + ty, gc = c * TB + tx;
    if (gr < n && gc < n) Z[(int64_t)gr * n + gc] = __ldcg(Z + (int64_t)gr * n + gc) - acc;
    __syncthreads();
}

__global__ void trinv_update_kernel(const double *L, double *Z, int n, int k) {
    VFEM_PDL_ENTRY();
    trinv_update_body(L, Z, n, k, blockIdx.x);
}

__global__ void identity_kernel(double *Z, int n) {
    VFEM_PDL_ENTRY();
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= (int64_t)n * n) return;
    Z[t] = (t / n == t % n) ? 1.0 : 0.0;
}

// Ainv = Z^T Z (lower tiles computed, mirrored). Z is lower triangular.
__device__ __forceinline__ void ztz_body(const double *Z, double *Ainv, int n, int nbt, int tile) {
    __shared__ double sa[TB][TB + 1], sb[TB][TB + 1];
    // map the tile index to lower tile (bi, bj), bj <= bi
    int idx = tile, bi = 0;
    while (idx > bi) { idx -= bi + 1; ++bi; }
    const int bj = idx;
    const int ty = threadIdx.y, tx = threadIdx.x;
    const int r0 = bi * TB, c0 = bj * TB;
    double acc = 0.0;
    for (int bk = bi; bk < nbt; ++bk) {
        const int k0 = bk * TB;
        sa[ty][tx] = (k0 + ty < n && r0 + tx < n) ? __ldcg(Z + (int64_t)(k0 + ty) * n + r0 + tx) : 0.0;
        sb[ty][tx] = (k0 + ty < n && c0 + tx < n) ? __ldcg(Z + (int64_t)(k0 + ty) * n + c0 + tx) : 0.0;
        __syncthreads();
#pragma unroll 8
        for (int q = 0; q < TB; ++q) acc += sa[q][ty] * sb[q][tx];
        __syncthreads();
    }
    const int gr = r0 + ty, gc = c0 + tx;
    if (gr < n && gc < n) {
        Ainv[(int64_t)gr * n + gc] = acc;
        Ainv[(int64_t)gc * n + gr] = acc;
    }
}

__global__ void ztz_kernel(const double *Z, double *Ainv, int n, int nbt) {
    VFEM_PDL_ENTRY();
    ztz_body(Z, Ainv, n, nbt, blockIdx.x);
}

__global__ void zero_upper_kernel(double *A, int n) {
    VFEM_PDL_ENTRY();
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= (int64_t)n * n) return;
    const int i = (int)(t / n), j = (int)(t % n);
    if (j > i) A[t] = 0.0;
}

// ---------------- the whole inverse in one cooperative launch ----------------
// Grid-wide barrier: a monotone arrival counter, barrier number e completes when it reaches
// e * gridDim.x. The wait is bounded: past the limit the block records a timeout (status 2) and
// leaves the kernel; the launch is cooperative, so every block is resident and the limit is
// only reached if something else went wrong.
__device__ __forceinline__ bool grid_barrier(unsigned *count, unsigned &epoch, int *status) {
    __shared__ int ok;
    ++epoch;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        __threadfence();
        atomicAdd(count, 1u);
        const unsigned target = epoch * gridDim.x;
        int good = 1;
        for (int it = 0;; ++it) {
            unsigned v;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(count) : "memory");
            if (v >= target) break;
            if (it > (1 << 22)) {
                atomicMax(status, 2);
                good = 0;
                break;
            }
            __nanosleep(32);
        }
        __threadfence();
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// The phases of dense_spd_inverse's launches, each block taking every gridDim.x-th tile of a
// phase and a grid-wide barrier where a launch boundary was: the same tile operations in the
// same order per tile, without ~5 nbt launch gaps on the chain of diagonal tiles.
__global__ void __launch_bounds__(TB *TB) dense_inverse_persistent_kernel(double *A, double *work, int n, int nbt,
                                                                          int *status, unsigned *count) {
    double *Z = work;
    double *Dinv = work + (size_t)n * n;
    const int G = gridDim.x, b = blockIdx.x;
    unsigned epoch = 0;
    for (int k = 0; k < nbt; ++k) {
        if (b == 0) chol_diag_body(A, Dinv, n, k, status);
        if (!grid_barrier(count, epoch, status)) return;
        const int m = nbt - k - 1;
        if (m > 0) {
            for (int t = b; t < m; t += G) chol_trsm_body(A, Dinv, n, k, t);
            if (!grid_barrier(count, epoch, status)) return;
            for (int t = b; t < m * (m + 1) / 2; t += G) chol_syrk_body(A, n, k, t);
            if (!grid_barrier(count, epoch, status)) return;
        }
    }
    const int tid = threadIdx.y * TB + threadIdx.x;
    for (int64_t t = (int64_t)b * TB * TB + tid; t < (int64_t)n * n; t += (int64_t)G * TB * TB) {
        const int i = (int)(t / n), j = (int)(t % n);
        if (j > i) A[t] = 0.0;
        Z[t] = (i == j) ? 1.0 : 0.0;
    }
    if (!grid_barrier(count, epoch, status)) return;
    for (int k = 0; k < nbt; ++k) {
        for (int c = b; c <= k; c += G) trinv_diag_body(Dinv, Z, n, k, c);
        if (!grid_barrier(count, epoch, status)) return;
        const int m = nbt - k - 1;
        if (m > 0) {
            for (int t = b; t < m * (k + 1); t += G) trinv_update_body(A, Z, n, k, t);
            if (!grid_barrier(count, epoch, status)) return;
        }
    }
    for (int t = b; t < nbt * (nbt + 1) / 2; t += G) {
        ztz_body(Z, A, n, nbt, t);
        __syncthreads();
    }
}

// ---------------- coarse solve ----------------
// nfree is read from device memory (it changes with the fabrication mask under captured graphs)
template <typename T>
__global__ void gather_free_kernel(const Geom g, const int *__restrict__ freeIdx, const int *__restrict__ nfreeDev,
                                   const T *__restrict__ b, double *__restrict__ out) {
    VFEM_PDL_ENTRY();
    const int nfree = *nfreeDev;
    const int t = blockIdx.x * BS + threadIdx.x;
    if (t >= nfree) return;
    const int d = freeIdx[t];
    out[t] = (double)b[(int64_t)(d % 3) * g.ld + d / 3];
}

template <typename T>
__global__ void symv_scatter_kernel(const Geom g, const double *__restrict__ Ainv, const int *__restrict__ freeIdx,
                                    const int *__restrict__ nfreeDev, const double *__restrict__ bf, T *__restrict__ x) {
    VFEM_PDL_ENTRY();
    const int nfree = *nfreeDev;
    const int row = blockIdx.x * (BS / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= nfree) return;
    double acc = 0.0;
    const double *a = Ainv + (int64_t)row * nfree;
    for (int c = lane; c < nfree; c += 32) acc += a[c] * bf[c];
    acc = warp_sum(acc);
    if (lane == 0) {
        const int d = freeIdx[row];
        x[(int64_t)(d % 3) * g.ld + d / 3] = (T)acc;
    }
}

// ---------------- reductions and CG vector kernels ----------------
// m-th node of the nondetached rows (rows < nn[1]) in node order; 32-bit division (counts < 2^31)
__device__ __forceinline__ int64_t masked_node(const Geom &g, int64_t m, int rows) {
    const uint32_t per = (uint32_t)rows * (uint32_t)g.nn[2];
    const uint32_t i = (uint32_t)m / per, rem = (uint32_t)m - i * per;
    return (int64_t)i * ((int64_t)g.nn[1] * g.nn[2]) + rem;
}

template <typename Ta, typename Tb>
__global__ void __launch_bounds__(BS) masked_dot_kernel(Geom g, const Ta *__restrict__ a, const Tb *__restrict__ b,
                                                        double *__restrict__ partials) {
    VFEM_PDL_ENTRY();
    const int rows = g.nyv();
    const int64_t M = (int64_t)g.nn[0] * rows * g.nn[2];
    double acc = 0.0;
    for (int64_t m = blockIdx.x * (int64_t)BS + threadIdx.x; m < M; m += (int64_t)gridDim.x * BS) {
        const int64_t n = masked_node(g, m, rows);
        acc += (double)a[n] * (double)b[n] + (double)a[g.ld + n] * (double)b[g.ld + n] +
               (double)a[2 * g.ld + n] * (double)b[2 * g.ld + n];
    }
    const double s = block_sum<BS>(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__device__ double sum_partials(const double *partials, int n) {
    double acc = 0.0;
    for (int q = threadIdx.x; q < n; q += BS) acc += partials[q];
    return block_sum<BS>(acc);
}

__global__ void finalize_kernel(const double *partials, int n, double *out) {
    VFEM_PDL_ENTRY();
    const double s = sum_partials(partials, n);
    if (threadIdx.x == 0) *out = s;
}

// sc: 0 rMr, 1 rMr_old, 2 beta, 3 alpha, 4 dAd, 5 rsq, 6 first
__global__ void cg_beta_kernel(const double *partials, int n, double *sc) {
    VFEM_PDL_ENTRY();
    const double s = sum_partials(partials, n);
    if (threadIdx.x == 0) {
        sc[1] = sc[0];
        sc[0] = s;
        sc[2] = (sc[6] != 0.0) ? 0.0 : s / sc[1];
        sc[6] = 0.0;
    }
}

__global__ void cg_alpha_kernel(const double *partials, int n, double *sc) {
    VFEM_PDL_ENTRY();
    const double s = sum_partials(partials, n);
    if (threadIdx.x == 0) {
        sc[4] = s;
        sc[3] = sc[0] / s;
    }
}

__global__ void cg_rsq_kernel(const double *partials, int n, double *sc, double *mirror) {
    VFEM_PDL_ENTRY();
    const double s = sum_partials(partials, n);
    if (threadIdx.x == 0) {
        sc[5] = s;
        if (mirror) *mirror = s;
    }
}

// FP32 -> FP64 widening on the integer units (vfem_widen.h): FP64 instructions, conversions
// included, issue at about two lanes per clock per SM here, and these vector kernels widen one
// float per degree of freedom. Equal to (double)f for every float.
__device__ __forceinline__ double widen(double v) { return v; }
__device__ __forceinline__ double widen(float f) {
    return __longlong_as_double((long long)vfem_widen_bits(__float_as_uint(f)));
}

// All loads are issued before the Dirichlet mask is applied (a load guarded by the mask would
// wait for it).
template <typename Ts>
__global__ void __launch_bounds__(BS) cg_precond_out_kernel(Geom g, const Ts *__restrict__ src, double *__restrict__ s,
                                                            const double *__restrict__ r,
                                                            const uint8_t *__restrict__ dmask,
                                                            double *__restrict__ partials) {
    VFEM_PDL_ENTRY();
    const int rows = g.nyv();
    double acc = 0.0;
    for (int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x; n < g.NN; n += (int64_t)gridDim.x * BS) {
        const uint8_t dm = dmask[n];
        const Ts a0 = src[n], a1 = src[g.ld + n], a2 = src[2 * g.ld + n];
        const double r0 = r[n], r1 = r[g.ld + n], r2 = r[2 * g.ld + n];
        const double s0 = (dm & 1) ? 0.0 : widen(a0);
        const double s1 = (dm & 2) ? 0.0 : widen(a1);
        const double s2 = (dm & 4) ? 0.0 : widen(a2);
        if (s) {
            s[n] = s0;
            s[g.ld + n] = s1;
            s[2 * g.ld + n] = s2;
        }
        const int j = (int)(((uint32_t)n / (uint32_t)g.nn[2]) % (uint32_t)g.nn[1]);
        if (j < rows) acc = fma(r2, s2, fma(r1, s1, fma(r0, s0, acc)));
    }
    const double t = block_sum<BS>(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

// Block maximum of the |v| bit patterns (see cg_direction_kernel) into amax[blockIdx.x].
__device__ __forceinline__ void block_absmax_store(unsigned long long m, double *amax) {
    __shared__ unsigned long long sh[BS / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long a = __shfl_xor_sync(0xffffffffu, m, o);
        m = a > m ? a : m;
    }
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long r = 0ull;
        for (int w = 0; w < BS / 32; ++w) r = sh[w] > r ? sh[w] : r;
        amax[blockIdx.x] = __longlong_as_double((long long)r);
    }
}

__device__ __forceinline__ void direction_store(double v, int64_t t, double *__restrict__ d, float *__restrict__ dh,
                                                float *__restrict__ dl, unsigned long long &m) {
    d[t] = v;
    if (dh) {
        const float h = __double2float_rn(v);
        dh[t] = h;
        dl[t] = __double2float_rn(v - (double)h);
    }
    const unsigned long long a = (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
    m = a > m ? a : m;
}

__global__ void cg_direction_kernel(Geom g, const double *__restrict__ s, double *__restrict__ d,
                                    const double *__restrict__ sc, float *__restrict__ dh, float *__restrict__ dl,
                                    double *__restrict__ amax) {
    VFEM_PDL_ENTRY();
    const double beta = sc[2];
    const int64_t N3 = 3 * g.ld;
    // |v| as the bit pattern with the sign cleared: for non-negative doubles the unsigned order
    // of the patterns is the numeric order, and NaN patterns exceed every number, so an integer
    // maximum (integer units; the FP64 units are the scarce ones here) propagates NaN
    unsigned long long m = 0ull;
    for (int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x; t < N3; t += (int64_t)gridDim.x * BS)
        direction_store(beta * d[t] + s[t], t, d, dh, dl, m);
    if (amax) block_absmax_store(m, amax);
}

// The same direction update with s formed on the fly from the preconditioner's iterate, as
// cg_precond_out_kernel forms it (Dirichlet components zeroed), so that s is never stored:
// the preconditioner step then only reduces r . s. Entries past NN in each component's
// stride are not touched (d stays zero there).
template <typename Ts>
__global__ void cg_direction_precond_kernel(Geom g, const Ts *__restrict__ src, const uint8_t *__restrict__ dmask,
                                            double *__restrict__ d, const double *__restrict__ sc,
                                            float *__restrict__ dh, float *__restrict__ dl,
                                            double *__restrict__ amax) {
    VFEM_PDL_ENTRY();
    const double beta = sc[2];
    unsigned long long m = 0ull;
    for (int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x; n < g.NN; n += (int64_t)gridDim.x * BS) {
        const uint8_t dm = dmask[n];
        Ts a[3];
        double dv[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            a[c] = src[c * g.ld + n];
            dv[c] = d[c * g.ld + n];
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double sv = ((dm >> c) & 1) ? 0.0 : widen(a[c]);
            direction_store(beta * dv[c] + sv, c * g.ld + n, d, dh, dl, m);
        }
    }
    if (amax) block_absmax_store(m, amax);
}

__global__ void __launch_bounds__(BS) cg_update_kernel(Geom g, double *__restrict__ x, double *__restrict__ r,
                                                       const double *__restrict__ d, const double *__restrict__ Ad,
                                                       const double *__restrict__ sc, double *__restrict__ partials,
                                                       float *__restrict__ b32, float *__restrict__ x32) {
    VFEM_PDL_ENTRY();
    const double alpha = sc[3];
    const int rows = g.nyv();
    const int64_t M = (int64_t)g.nn[0] * rows * g.nn[2];
    double acc = 0.0;
    for (int64_t m = blockIdx.x * (int64_t)BS + threadIdx.x; m < M; m += (int64_t)gridDim.x * BS) {
        const int64_t n = masked_node(g, m, rows);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int64_t q = c * g.ld + n;
            x[q] += alpha * d[q];
            const double rv = r[q] - alpha * Ad[q];
            r[q] = rv;
            acc += rv * rv;
            if (b32) {
                // the next FP32 V-cycle's right-hand side and zero initial iterate
                b32[q] = (float)rv;
                x32[q] = 0.f;
            }
        }
    }
    const double s = block_sum<BS>(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void copy_kernel(double *__restrict__ dst, const double *__restrict__ src, int64_t n) {
    VFEM_PDL_ENTRY();
    for (int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x; t < n; t += (int64_t)gridDim.x * BS) dst[t] = src[t];
}

template <typename T>
__global__ void enforce_dirichlet_kernel(Geom g, T *__restrict__ u, const uint8_t *__restrict__ dmask,
                                         const double *__restrict__ dval) {
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n >= g.NN) return;
    const uint8_t dm = dmask[n];
    if (!dm) return;
#pragma unroll
    for (int c = 0; c < 3; ++c)
        if ((dm >> c) & 1) u[c * g.ld + n] = dval ? (T)dval[c * g.ld + n] : T(0);
}

// The pivot reciprocals of the dense inverse applied elementwise (diagnostic).
__global__ void newton_helpers_kernel(const double *__restrict__ d, int64_t n, double *__restrict__ recip,
                                      double *__restrict__ rsqrt) {
    const int64_t i = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (i >= n) return;
    recip[i] = recip_newton(d[i]);
    rsqrt[i] = rsqrt_newton(d[i]);
}

}  // namespace

void launch_newton_helpers(const double *d, int64_t n, double *recip, double *rsqrt, cudaStream_t st) {
    if (n <= 0) return;
    newton_helpers_kernel<<<gridFor(n, BS), BS, 0, st>>>(d, n, recip, rsqrt);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_dense_from_stencil(const Geom &g, const T *S, const int *redIdx, double *A, int nfree, bool rows,
                               cudaStream_t st) {
    VFEM_CUDA(cudaMemsetAsync(A, 0, sizeof(double) * (size_t)nfree * nfree, st));
    dense_from_stencil_kernel<T><<<gridFor(g.NN * 243, BS), BS, 0, st>>>(g, S, redIdx, A, nfree, rows ? 1 : 0);
    VFEM_LAUNCH_CHECK();
}

void launch_symmetrize(double *A, int n, cudaStream_t st) {
    symmetrize_kernel<<<gridFor((int64_t)n * n, BS), BS, 0, st>>>(A, n);
    VFEM_LAUNCH_CHECK();
}

// VFEM_DENSE_PERSISTENT=1 selects the single cooperative launch. It is off by default: at 600
// free DOFs a whole rebuild took 2.06 ms with it against 1.99 ms with one launch per phase, whose
// programmatic dependent launches already overlap the launch gaps that ~190 grid barriers replace.
static bool densePersistent() {
    const char *e = std::getenv("VFEM_DENSE_PERSISTENT");
    return e && e[0] == '1';
}

void dense_spd_inverse(double *A, double *work, int n, int *status, cudaStream_t st,
                       const std::function<void(const std::string &)> &mark) {
    if (n <= 0) return;
    const dim3 tb(TB, TB);
    const int nbt = (n + TB - 1) / TB;
    double *Dinv = work + (size_t)n * n;
    if (!mark && densePersistent()) {
        // one cooperative launch: every block resident, at most one per SM, no more blocks than
        // the largest phase has tiles
        static int maxBlocks = 0;
        if (!maxBlocks) {
            int perSM = 0, dev = 0, sms = 0;
            VFEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, dense_inverse_persistent_kernel, TB * TB, 0));
            VFEM_CUDA(cudaGetDevice(&dev));
            VFEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            maxBlocks = std::max(1, std::min(perSM, 1) * sms);
        }
        const int G = std::max(1, std::min(maxBlocks, nbt * (nbt + 1) / 2));
        unsigned *count = reinterpret_cast<unsigned *>(Dinv + (size_t)TB * TB * nbt);
        VFEM_CUDA(cudaMemsetAsync(count, 0, sizeof(unsigned), st));
        void *args[] = {&A, &work, &n, (void *)&nbt, &status, &count};
        VFEM_CUDA(cudaLaunchCooperativeKernel((const void *)dense_inverse_persistent_kernel, dim3(G), tb, args, 0, st));
        return;
    }
    for (int k = 0; k < nbt; ++k) {
        launch_pdl(chol_diag_kernel, 1, tb, 0, st, A, Dinv, n, k, status);
        VFEM_LAUNCH_CHECK();
        if (mark) mark("coarsest:chol diag tiles");
        const int m = nbt - k - 1;
        if (m > 0) {
            launch_pdl(chol_trsm_kernel, m, tb, 0, st, A, (const double *)Dinv, n, k);
            VFEM_LAUNCH_CHECK();
            if (mark) mark("coarsest:chol panel solves");
            launch_pdl(chol_syrk_kernel, m * (m + 1) / 2, tb, 0, st, A, n, k);
            VFEM_LAUNCH_CHECK();
            if (mark) mark("coarsest:chol trailing updates");
        }
    }
    launch_pdl(zero_upper_kernel, gridFor((int64_t)n * n, BS), BS, 0, st, A, n);
    VFEM_LAUNCH_CHECK();
    launch_pdl(identity_kernel, gridFor((int64_t)n * n, BS), BS, 0, st, work, n);
    VFEM_LAUNCH_CHECK();
    if (mark) mark("coarsest:inverse init");
    for (int k = 0; k < nbt; ++k) {
        launch_pdl(trinv_diag_kernel, k + 1, tb, 0, st, (const double *)Dinv, work, n, k);
        VFEM_LAUNCH_CHECK();
        if (mark) mark("coarsest:trinv diag solves");
        const int m = nbt - k - 1;
        if (m > 0) {
            launch_pdl(trinv_update_kernel, m * (k + 1), tb, 0, st, (const double *)A, work, n, k);
            VFEM_LAUNCH_CHECK();
            if (mark) mark("coarsest:trinv updates");
        }
    }
    launch_pdl(ztz_kernel, nbt * (nbt + 1) / 2, tb, 0, st, (const double *)work, A, n, nbt);
    VFEM_LAUNCH_CHECK();
    if (mark) mark("coarsest:Z^T Z");
}

template <typename T>
void launch_coarse_solve(const Geom &g, const double *Ainv, const int *freeIdx, const int *nfreeDev, int nfreeCap,
                         const T *b, T *x, double *scratch, cudaStream_t st) {
    launch_fill<T>(x, T(0), 3 * g.ld, st);
    if (nfreeCap <= 0) return;
    launch_pdl(gather_free_kernel<T>, gridFor(nfreeCap, BS), BS, 0, st, g, freeIdx, nfreeDev, b, scratch);
    VFEM_LAUNCH_CHECK();
    launch_pdl(symv_scatter_kernel<T>, gridFor(nfreeCap, BS / 32), BS, 0, st, g, Ainv, freeIdx, nfreeDev, scratch, x);
    VFEM_LAUNCH_CHECK();
}

// Loop control of the device-resident PCG (a conditional WHILE node of a CUDA graph):
// sc[5] |r|^2, sc[7] |b|^2, sc[8] tol^2, sc[9] iterations done, sc[10] iteration limit,
// sc[11] iteration at which the residual became NaN (-1: the initial one). The loop continues
// while |r|^2 > tol^2 |b|^2 and the limit is not reached (MultigridSolver.hh:1068-1070).
__global__ void cg_loop_control_kernel(cudaGraphConditionalHandle h, double *sc, int initial) {
    const double rsq = sc[5];
    double it = sc[9];
    if (!initial) {
        it += 1.0;
        sc[9] = it;
    }
    unsigned cont = 1;
    if (isnan(rsq)) {
        if (sc[11] == 0.0) sc[11] = initial ? -1.0 : it;  // the first NaN is the one reported
        cont = 0;
    } else if (!(rsq > sc[8] * sc[7]) || it >= sc[10]) {
        cont = 0;
    }
    cudaGraphSetConditional(h, cont);
}

// The count and NaN record of cg_loop_control_kernel after an iteration run outside the loop
__global__ void cg_count_kernel(double *sc) {
    const double it = sc[9] + 1.0;
    sc[9] = it;
    if (isnan(sc[5]) && sc[11] == 0.0) sc[11] = it;
}

void launch_cg_count(double *sc, cudaStream_t st) {
    cg_count_kernel<<<1, 1, 0, st>>>(sc);
    VFEM_LAUNCH_CHECK();
}

void launch_cg_loop_control(cudaGraphConditionalHandle h, double *sc, bool initial, cudaStream_t st) {
    cg_loop_control_kernel<<<1, 1, 0, st>>>(h, sc, initial ? 1 : 0);
    VFEM_LAUNCH_CHECK();
}

// CG scalars before the first iteration; |r|^2 (sc[5]) and |b|^2 (sc[7]) are already in place
__global__ void cg_init_kernel(double *sc, double tol2, double maxIter) {
    sc[0] = 0.0;
    sc[6] = 1.0;
    sc[8] = tol2;
    sc[9] = 0.0;
    sc[10] = maxIter;
    sc[11] = 0.0;
}

void launch_cg_init(double *sc, double tol2, double maxIter, cudaStream_t st) {
    cg_init_kernel<<<1, 1, 0, st>>>(sc, tol2, maxIter);
    VFEM_LAUNCH_CHECK();
}

__global__ void axpy_kernel(int64_t n, double a, const double *__restrict__ xv, double *__restrict__ yv) {
    VFEM_PDL_ENTRY();
    for (int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x; t < n; t += (int64_t)gridDim.x * BS) yv[t] += a * xv[t];
}

void launch_axpy(int64_t n, double a, const double *x, double *y, cudaStream_t st) {
    if (n <= 0) return;
    launch_pdl(axpy_kernel, std::min<unsigned>(gridFor(n, BS), 4 * 152), BS, 0, st, n, a, x, y);
    VFEM_LAUNCH_CHECK();
}

__global__ void set_pair_kernel(int *p, int a, int b) {
    p[0] = a;
    p[1] = b;
}

void launch_set_pair(int *p, int a, int b, cudaStream_t st) {
    set_pair_kernel<<<1, 1, 0, st>>>(p, a, b);
    VFEM_LAUNCH_CHECK();
}

template <typename Ta, typename Tb>
void launch_masked_dot_partials(const Geom &g, const Ta *a, const Tb *b, double *partials, cudaStream_t st) {
    launch_pdl(masked_dot_kernel<Ta, Tb>, REDUCE_BLOCKS, BS, 0, st, g, a, b, partials);
    VFEM_LAUNCH_CHECK();
}

void launch_finalize(const double *partials, int n, double *out, cudaStream_t st) {
    launch_pdl(finalize_kernel, 1, BS, 0, st, partials, n, out);
    VFEM_LAUNCH_CHECK();
}
void launch_cg_beta(const double *partials, int n, double *sc, cudaStream_t st) {
    launch_pdl(cg_beta_kernel, 1, BS, 0, st, partials, n, sc);
    VFEM_LAUNCH_CHECK();
}
void launch_cg_alpha(const double *partials, int n, double *sc, cudaStream_t st) {
    launch_pdl(cg_alpha_kernel, 1, BS, 0, st, partials, n, sc);
    VFEM_LAUNCH_CHECK();
}
void launch_cg_rsq(const double *partials, int n, double *sc, double *mirror, cudaStream_t st) {
    launch_pdl(cg_rsq_kernel, 1, BS, 0, st, partials, n, sc, mirror);
    VFEM_LAUNCH_CHECK();
}

template <typename Ts>
void launch_cg_precond_out(const Geom &g, const Ts *src, double *s, const double *r, const uint8_t *dmask,
                           double *partials, cudaStream_t st) {
    launch_pdl(cg_precond_out_kernel<Ts>, REDUCE_BLOCKS, BS, 0, st, g, src, s, r, dmask, partials);
    VFEM_LAUNCH_CHECK();
}

void launch_cg_direction(const Geom &g, const double *s, double *d, const double *sc, float *dh, float *dl,
                         cudaStream_t st, double *amax) {
    launch_pdl(cg_direction_kernel, REDUCE_BLOCKS, BS, 0, st, g, s, d, sc, dh, dl, amax);
    VFEM_LAUNCH_CHECK();
}

template <typename Ts>
void launch_cg_direction_precond(const Geom &g, const Ts *src, const uint8_t *dmask, double *d, const double *sc,
                                 float *dh, float *dl, cudaStream_t st, double *amax) {
    launch_pdl(cg_direction_precond_kernel<Ts>, REDUCE_BLOCKS, BS, 0, st, g, src, dmask, d, sc, dh, dl, amax);
    VFEM_LAUNCH_CHECK();
}

void launch_cg_update(const Geom &g, double *x, double *r, const double *d, const double *Ad, const double *sc,
                      double *partials, cudaStream_t st, float *b32, float *x32) {
    launch_pdl(cg_update_kernel, REDUCE_BLOCKS, BS, 0, st, g, x, r, d, Ad, sc, partials, b32, x32);
    VFEM_LAUNCH_CHECK();
}

void launch_copy(double *dst, const double *src, int64_t n, cudaStream_t st) {
    launch_pdl(copy_kernel, REDUCE_BLOCKS, BS, 0, st, dst, src, n);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_enforce_dirichlet(const Geom &g, T *u, const uint8_t *dmask, const double *dval, cudaStream_t st) {
    enforce_dirichlet_kernel<T><<<gridFor(g.NN, BS), BS, 0, st>>>(g, u, dmask, dval);
    VFEM_LAUNCH_CHECK();
}

template void launch_dense_from_stencil<double>(const Geom &, const double *, const int *, double *, int, bool,
                                               cudaStream_t);
template void launch_dense_from_stencil<float>(const Geom &, const float *, const int *, double *, int, bool,
                                              cudaStream_t);
template void launch_coarse_solve<double>(const Geom &, const double *, const int *, const int *, int, const double *,
                                          double *, double *, cudaStream_t);
template void launch_coarse_solve<float>(const Geom &, const double *, const int *, const int *, int, const float *,
                                         float *, double *, cudaStream_t);
template void launch_masked_dot_partials<double, double>(const Geom &, const double *, const double *, double *,
                                                         cudaStream_t);
template void launch_masked_dot_partials<float, float>(const Geom &, const float *, const float *, double *,
                                                       cudaStream_t);
template void launch_cg_direction_precond<float>(const Geom &, const float *, const uint8_t *, double *,
                                                const double *, float *, float *, cudaStream_t, double *);
template void launch_cg_precond_out<double>(const Geom &, const double *, double *, const double *, const uint8_t *,
                                            double *, cudaStream_t);
template void launch_cg_precond_out<float>(const Geom &, const float *, double *, const double *, const uint8_t *,
                                           double *, cudaStream_t);
template void launch_enforce_dirichlet<double>(const Geom &, double *, const uint8_t *, const double *, cudaStream_t);
template void launch_enforce_dirichlet<float>(const Geom &, float *, const uint8_t *, const double *, cudaStream_t);

}  // namespace vfem
