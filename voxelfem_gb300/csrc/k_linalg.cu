// Dense FP64 coarsest-level solve (blocked Cholesky + explicit inverse, replacing the
// reference's CHOLMOD factorisation, TensorProductSimulator.hh:1198-1230) and the
// PCG vector kernels with deterministic warp-shuffle reductions
// (MultigridSolver.hh:1047-1152, TensorProductSimulator.hh:414-459).
#include "vfem_kernels.hpp"
#include "vfem_reduce.cuh"

namespace vfem {

namespace {

constexpr int BS = 256;
constexpr int TB = 32;  // dense tile size

// ---------------- dense assembly ----------------
template <typename T>
__global__ void dense_from_stencil_kernel(Geom g, const T *__restrict__ S, const int *__restrict__ red,
                                          double *__restrict__ A, int nfree) {
    // thread per (row dof of a node, stencil entry): row = 3n + r
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= g.NN * 243) return;
    const int64_t n = t / 243;
    const int q = (int)(t % 243);
    const int o = q / 9, r = (q % 9) / 3, c = q % 3;
    const int k = (int)(n % g.nn[2]);
    const int64_t tt = n / g.nn[2];
    const int j = (int)(tt % g.nn[1]), i = (int)(tt / g.nn[1]);
    const int ni = i + o / 9 - 1, nj = j + (o / 3) % 3 - 1, nk = k + o % 3 - 1;
    if (ni < 0 || nj < 0 || nk < 0 || ni >= g.nn[0] || nj >= g.nn[1] || nk >= g.nn[2]) return;
    const int64_t m = g.node(ni, nj, nk);
    const int ra = red[3 * n + r], cb = red[3 * m + c];
    if (ra < 0 || cb < 0) return;
    A[(int64_t)ra * nfree + cb] = (double)S[(int64_t)q * g.ld + n];
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
// Step k: factor the diagonal tile, solve the tiles below it, then update every trailing
// lower tile with one 32x32x32 product per block, so each step spreads over all SMs.
__device__ __forceinline__ void load_tile(const double *A, int n, int r0, int c0, double (*t)[TB + 1]) {
    const int ty = threadIdx.y, tx = threadIdx.x;
    t[ty][tx] = (r0 + ty < n && c0 + tx < n) ? A[(int64_t)(r0 + ty) * n + c0 + tx] : 0.0;
}

__global__ void chol_diag_kernel(double *A, int n, int k, int *status) {
    __shared__ double sl[TB][TB + 1];
    const int ty = threadIdx.y, tx = threadIdx.x;
    const int kb = k * TB;
    const int nb = min(TB, n - kb);
    load_tile(A, n, kb, kb, sl);
    if (!(ty < nb && tx < nb)) sl[ty][tx] = (ty == tx) ? 1.0 : 0.0;
    __syncthreads();
    for (int j = 0; j < nb; ++j) {
        if (ty == 0 && tx == 0) {
            const double d = sl[j][j];
            if (!(d > 0.0)) { atomicExch(status, 1); sl[j][j] = 1.0; }
            else sl[j][j] = sqrt(d);
        }
        __syncthreads();
        if (tx == 0 && ty > j && ty < nb) sl[ty][j] /= sl[j][j];
        __syncthreads();
        if (ty > j && tx > j && tx <= ty && ty < nb) sl[ty][tx] -= sl[ty][j] * sl[tx][j];
        __syncthreads();
    }
    if (ty < nb && tx < nb) A[(int64_t)(kb + ty) * n + kb + tx] = (tx <= ty) ? sl[ty][tx] : 0.0;
}

// tiles (i, k), i > k: X L_kk^T = A_ik
__global__ void chol_trsm_kernel(double *A, int n, int k) {
    __shared__ double sl[TB][TB + 1], sx[TB][TB + 1];
    const int ty = threadIdx.y, tx = threadIdx.x;
    const int kb = k * TB, r0 = kb + TB * (1 + blockIdx.x);
    const int nb = min(TB, n - kb);
    load_tile(A, n, kb, kb, sl);
    if (!(ty < nb && tx < nb)) sl[ty][tx] = (ty == tx) ? 1.0 : 0.0;
    load_tile(A, n, r0, kb, sx);
    __syncthreads();
    for (int j = 0; j < nb; ++j) {
        if (tx == j) {
            double v = sx[ty][j];
            for (int t = 0; t < j; ++t) v -= sx[ty][t] * sl[j][t];
            sx[ty][j] = v / sl[j][j];
        }
        __syncthreads();
    }
    if (r0 + ty < n && tx < nb) A[(int64_t)(r0 + ty) * n + kb + tx] = sx[ty][tx];
}

__device__ __forceinline__ void lower_tile_of(int idx, int &ii, int &jj) {
    ii = 0;
    while (idx > ii) { idx -= ii + 1; ++ii; }
    jj = idx;
}

// trailing tiles (i, j), k < j <= i: A_ij -= L_ik L_jk^T
__global__ void chol_syrk_kernel(double *A, int n, int k) {
    __shared__ double sa[TB][TB + 1], sb[TB][TB + 1];
    int ii, jj;
    lower_tile_of(blockIdx.x, ii, jj);
    const int i = k + 1 + ii, j = k + 1 + jj;
    const int ty = threadIdx.y, tx = threadIdx.x;
    const int kb = k * TB;
    load_tile(A, n, i * TB, kb, sa);
    load_tile(A, n, j * TB, kb, sb);
    __syncthreads();
    double acc = 0.0;
#pragma unroll 8
    for (int q = 0; q < TB; ++q) acc += sa[ty][q] * sb[tx][q];
    const int gr = i * TB + ty, gc = j * TB + tx;
    if (gr < n && gc < n) A[(int64_t)gr * n + gc] -= acc;
}

// Z = L^{-1}, right-looking over block columns of L. Step k: Z[k][c] = L_kk^{-1} Z[k][c] (c <= k),
// then Z[i][c] -= L[i][k] Z[k][c] for i > k.
__global__ void trinv_diag_kernel(const double *L, double *Z, int n, int k) {
    __shared__ double sl[TB][TB + 1], sx[TB][TB + 1];
    const int c = blockIdx.x;
    const int ty = threadIdx.y, tx = threadIdx.x;
    const int r0 = k * TB, c0 = c * TB;
    const int nb = min(TB, n - r0);
    load_tile(L, n, r0, r0, sl);
    if (!(ty < nb && tx < nb)) sl[ty][tx] = (ty == tx) ? 1.0 : 0.0;
    load_tile(Z, n, r0, c0, sx);
    __syncthreads();
    for (int r = 0; r < TB; ++r) {
        if (ty == r) {
            double v = sx[r][tx];
            for (int t = 0; t < r; ++t) v -= sl[r][t] * sx[t][tx];
            sx[r][tx] = v / sl[r][r];
        }
        __syncthreads();
    }
    if (r0 + ty < n && c0 + tx < n) Z[(int64_t)(r0 + ty) * n + c0 + tx] = sx[ty][tx];
}

__global__ void trinv_update_kernel(const double *L, double *Z, int n, int k) {
    __shared__ double sa[TB][TB + 1], sb[TB][TB + 1];
    const int c = blockIdx.x % (k + 1);
    const int i = k + 1 + blockIdx.x / (k + 1);
    const int ty = threadIdx.y, tx = threadIdx.x;
    load_tile(L, n, i * TB, k * TB, sa);
    load_tile(Z, n, k * TB, c * TB, sb);
    __syncthreads();
    double acc = 0.0;
#pragma unroll 8
    for (int q = 0; q < TB; ++q) acc += sa[ty][q] * sb[q][tx];
    const int gr = i * TB + ty, gc = c * TB + tx;
    if (gr < n && gc < n) Z[(int64_t)gr * n + gc] -= acc;
}

__global__ void identity_kernel(double *Z, int n) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= (int64_t)n * n) return;
    Z[t] = (t / n == t % n) ? 1.0 : 0.0;
}

// Ainv = Z^T Z (lower tiles computed, mirrored). Z is lower triangular.
__global__ void ztz_kernel(const double *Z, double *Ainv, int n, int nbt) {
    __shared__ double sa[TB][TB + 1], sb[TB][TB + 1];
    // map blockIdx.x to lower tile (bi, bj), bj <= bi
    int idx = blockIdx.x, bi = 0;
    while (idx > bi) { idx -= bi + 1; ++bi; }
    const int bj = idx;
    const int ty = threadIdx.y, tx = threadIdx.x;
    const int r0 = bi * TB, c0 = bj * TB;
    double acc = 0.0;
    for (int bk = bi; bk < nbt; ++bk) {
        const int k0 = bk * TB;
        sa[ty][tx] = (k0 + ty < n && r0 + tx < n) ? Z[(int64_t)(k0 + ty) * n + r0 + tx] : 0.0;
        sb[ty][tx] = (k0 + ty < n && c0 + tx < n) ? Z[(int64_t)(k0 + ty) * n + c0 + tx] : 0.0;
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

__global__ void zero_upper_kernel(double *A, int n) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= (int64_t)n * n) return;
    const int i = (int)(t / n), j = (int)(t % n);
    if (j > i) A[t] = 0.0;
}

// ---------------- coarse solve ----------------
template <typename T>
__global__ void gather_free_kernel(const Geom g, const int *__restrict__ freeIdx, int nfree, const T *__restrict__ b,
                                   double *__restrict__ out) {
    const int t = blockIdx.x * BS + threadIdx.x;
    if (t >= nfree) return;
    const int d = freeIdx[t];
    out[t] = (double)b[(int64_t)(d % 3) * g.ld + d / 3];
}

template <typename T>
__global__ void symv_scatter_kernel(const Geom g, const double *__restrict__ Ainv, const int *__restrict__ freeIdx,
                                    int nfree, const double *__restrict__ bf, T *__restrict__ x) {
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
__device__ __forceinline__ int64_t masked_node(const Geom &g, int64_t m, int rows) {
    const int64_t per = (int64_t)rows * g.nn[2];
    const int64_t i = m / per, rem = m % per;
    return i * ((int64_t)g.nn[1] * g.nn[2]) + rem;
}

template <typename Ta, typename Tb>
__global__ void __launch_bounds__(BS) masked_dot_kernel(Geom g, const Ta *__restrict__ a, const Tb *__restrict__ b,
                                                        double *__restrict__ partials) {
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
    const double s = sum_partials(partials, n);
    if (threadIdx.x == 0) *out = s;
}

// sc: 0 rMr, 1 rMr_old, 2 beta, 3 alpha, 4 dAd, 5 rsq, 6 first
__global__ void cg_beta_kernel(const double *partials, int n, double *sc) {
    const double s = sum_partials(partials, n);
    if (threadIdx.x == 0) {
        sc[1] = sc[0];
        sc[0] = s;
        sc[2] = (sc[6] != 0.0) ? 0.0 : s / sc[1];
        sc[6] = 0.0;
    }
}

__global__ void cg_alpha_kernel(const double *partials, int n, double *sc) {
    const double s = sum_partials(partials, n);
    if (threadIdx.x == 0) {
        sc[4] = s;
        sc[3] = sc[0] / s;
    }
}

__global__ void cg_rsq_kernel(const double *partials, int n, double *sc, double *mirror) {
    const double s = sum_partials(partials, n);
    if (threadIdx.x == 0) {
        sc[5] = s;
        if (mirror) *mirror = s;
    }
}

template <typename Ts>
__global__ void __launch_bounds__(BS) cg_precond_out_kernel(Geom g, const Ts *__restrict__ src, double *__restrict__ s,
                                                            const double *__restrict__ r,
                                                            const uint8_t *__restrict__ dmask,
                                                            double *__restrict__ partials) {
    const int rows = g.nyv();
    double acc = 0.0;
    for (int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x; n < g.NN; n += (int64_t)gridDim.x * BS) {
        const uint8_t dm = dmask[n];
        const double s0 = (dm & 1) ? 0.0 : (double)src[n];
        const double s1 = (dm & 2) ? 0.0 : (double)src[g.ld + n];
        const double s2 = (dm & 4) ? 0.0 : (double)src[2 * g.ld + n];
        s[n] = s0;
        s[g.ld + n] = s1;
        s[2 * g.ld + n] = s2;
        const int j = (int)((n / g.nn[2]) % g.nn[1]);
        if (j < rows) acc += r[n] * s0 + r[g.ld + n] * s1 + r[2 * g.ld + n] * s2;
    }
    const double t = block_sum<BS>(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

__global__ void cg_direction_kernel(Geom g, const double *__restrict__ s, double *__restrict__ d,
                                    const double *__restrict__ sc, float *__restrict__ dh, float *__restrict__ dl) {
    const double beta = sc[2];
    const int64_t N3 = 3 * g.ld;
    for (int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x; t < N3; t += (int64_t)gridDim.x * BS) {
        const double v = beta * d[t] + s[t];
        d[t] = v;
        if (dh) {
            const float h = __double2float_rn(v);
            dh[t] = h;
            dl[t] = __double2float_rn(v - (double)h);
        }
    }
}

__global__ void __launch_bounds__(BS) cg_update_kernel(Geom g, double *__restrict__ x, double *__restrict__ r,
                                                       const double *__restrict__ d, const double *__restrict__ Ad,
                                                       const double *__restrict__ sc, double *__restrict__ partials) {
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
        }
    }
    const double s = block_sum<BS>(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void copy_kernel(double *__restrict__ dst, const double *__restrict__ src, int64_t n) {
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

}  // namespace

template <typename T>
void launch_dense_from_stencil(const Geom &g, const T *S, const int *redIdx, double *A, int nfree, cudaStream_t st) {
    VFEM_CUDA(cudaMemsetAsync(A, 0, sizeof(double) * (size_t)nfree * nfree, st));
    dense_from_stencil_kernel<T><<<gridFor(g.NN * 243, BS), BS, 0, st>>>(g, S, redIdx, A, nfree);
    VFEM_LAUNCH_CHECK();
}

void launch_symmetrize(double *A, int n, cudaStream_t st) {
    symmetrize_kernel<<<gridFor((int64_t)n * n, BS), BS, 0, st>>>(A, n);
    VFEM_LAUNCH_CHECK();
}

void dense_spd_inverse(double *A, double *work, int n, int *status, cudaStream_t st) {
    if (n <= 0) return;
    const dim3 tb(TB, TB);
    const int nbt = (n + TB - 1) / TB;
    for (int k = 0; k < nbt; ++k) {
        chol_diag_kernel<<<1, tb, 0, st>>>(A, n, k, status);
        VFEM_LAUNCH_CHECK();
        const int m = nbt - k - 1;
        if (m > 0) {
            chol_trsm_kernel<<<m, tb, 0, st>>>(A, n, k);
            VFEM_LAUNCH_CHECK();
            chol_syrk_kernel<<<m * (m + 1) / 2, tb, 0, st>>>(A, n, k);
            VFEM_LAUNCH_CHECK();
        }
    }
    zero_upper_kernel<<<gridFor((int64_t)n * n, BS), BS, 0, st>>>(A, n);
    VFEM_LAUNCH_CHECK();
    identity_kernel<<<gridFor((int64_t)n * n, BS), BS, 0, st>>>(work, n);
    VFEM_LAUNCH_CHECK();
    for (int k = 0; k < nbt; ++k) {
        trinv_diag_kernel<<<k + 1, tb, 0, st>>>(A, work, n, k);
        VFEM_LAUNCH_CHECK();
        const int m = nbt - k - 1;
        if (m > 0) {
            trinv_update_kernel<<<m * (k + 1), tb, 0, st>>>(A, work, n, k);
            VFEM_LAUNCH_CHECK();
        }
    }
    ztz_kernel<<<nbt * (nbt + 1) / 2, tb, 0, st>>>(work, A, n, nbt);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_coarse_solve(const Geom &g, const double *Ainv, const int *freeIdx, int nfree, const T *b, T *x,
                         double *scratch, cudaStream_t st) {
    launch_fill<T>(x, T(0), 3 * g.ld, st);
    if (nfree <= 0) return;
    gather_free_kernel<T><<<gridFor(nfree, BS), BS, 0, st>>>(g, freeIdx, nfree, b, scratch);
    VFEM_LAUNCH_CHECK();
    symv_scatter_kernel<T><<<gridFor(nfree, BS / 32), BS, 0, st>>>(g, Ainv, freeIdx, nfree, scratch, x);
    VFEM_LAUNCH_CHECK();
}

template <typename Ta, typename Tb>
void launch_masked_dot_partials(const Geom &g, const Ta *a, const Tb *b, double *partials, cudaStream_t st) {
    masked_dot_kernel<Ta, Tb><<<REDUCE_BLOCKS, BS, 0, st>>>(g, a, b, partials);
    VFEM_LAUNCH_CHECK();
}

void launch_finalize(const double *partials, int n, double *out, cudaStream_t st) {
    finalize_kernel<<<1, BS, 0, st>>>(partials, n, out);
    VFEM_LAUNCH_CHECK();
}
void launch_cg_beta(const double *partials, int n, double *sc, cudaStream_t st) {
    cg_beta_kernel<<<1, BS, 0, st>>>(partials, n, sc);
    VFEM_LAUNCH_CHECK();
}
void launch_cg_alpha(const double *partials, int n, double *sc, cudaStream_t st) {
    cg_alpha_kernel<<<1, BS, 0, st>>>(partials, n, sc);
    VFEM_LAUNCH_CHECK();
}
void launch_cg_rsq(const double *partials, int n, double *sc, double *mirror, cudaStream_t st) {
    cg_rsq_kernel<<<1, BS, 0, st>>>(partials, n, sc, mirror);
    VFEM_LAUNCH_CHECK();
}

template <typename Ts>
void launch_cg_precond_out(const Geom &g, const Ts *src, double *s, const double *r, const uint8_t *dmask,
                           double *partials, cudaStream_t st) {
    cg_precond_out_kernel<Ts><<<REDUCE_BLOCKS, BS, 0, st>>>(g, src, s, r, dmask, partials);
    VFEM_LAUNCH_CHECK();
}

void launch_cg_direction(const Geom &g, const double *s, double *d, const double *sc, float *dh, float *dl,
                         cudaStream_t st) {
    cg_direction_kernel<<<REDUCE_BLOCKS, BS, 0, st>>>(g, s, d, sc, dh, dl);
    VFEM_LAUNCH_CHECK();
}

void launch_cg_update(const Geom &g, double *x, double *r, const double *d, const double *Ad, const double *sc,
                      double *partials, cudaStream_t st) {
    cg_update_kernel<<<REDUCE_BLOCKS, BS, 0, st>>>(g, x, r, d, Ad, sc, partials);
    VFEM_LAUNCH_CHECK();
}

void launch_copy(double *dst, const double *src, int64_t n, cudaStream_t st) {
    copy_kernel<<<REDUCE_BLOCKS, BS, 0, st>>>(dst, src, n);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_enforce_dirichlet(const Geom &g, T *u, const uint8_t *dmask, const double *dval, cudaStream_t st) {
    enforce_dirichlet_kernel<T><<<gridFor(g.NN, BS), BS, 0, st>>>(g, u, dmask, dval);
    VFEM_LAUNCH_CHECK();
}

template void launch_dense_from_stencil<double>(const Geom &, const double *, const int *, double *, int, cudaStream_t);
template void launch_dense_from_stencil<float>(const Geom &, const float *, const int *, double *, int, cudaStream_t);
template void launch_coarse_solve<double>(const Geom &, const double *, const int *, int, const double *, double *,
                                          double *, cudaStream_t);
template void launch_coarse_solve<float>(const Geom &, const double *, const int *, int, const float *, float *,
                                         double *, cudaStream_t);
template void launch_masked_dot_partials<double, double>(const Geom &, const double *, const double *, double *,
                                                         cudaStream_t);
template void launch_masked_dot_partials<float, float>(const Geom &, const float *, const float *, double *,
                                                       cudaStream_t);
template void launch_cg_precond_out<double>(const Geom &, const double *, double *, const double *, const uint8_t *,
                                            double *, cudaStream_t);
template void launch_cg_precond_out<float>(const Geom &, const float *, double *, const double *, const uint8_t *,
                                           double *, cudaStream_t);
template void launch_enforce_dirichlet<double>(const Geom &, double *, const uint8_t *, const double *, cudaStream_t);
template void launch_enforce_dirichlet<float>(const Geom &, float *, const uint8_t *, const double *, cudaStream_t);

}  // namespace vfem
