// Kernels of the bilinear-quadrilateral (2D) path: matrix-free fine operator, coloured block
// Gauss-Seidel, Galerkin coarse element matrices and 9-point block stencils, grid transfers,
// the dense coarsest solve's gather/scatter, the CG vector kernels and the sensitivities.
// Every kernel is FP64 (the 2D problems of the reference are small; FP64 keeps them exact).
#include <algorithm>

#include "vfem_2d.hpp"
#include "vfem_df.cuh"
#include "vfem_kernels.hpp"
#include "vfem_reduce.cuh"

namespace vfem {
namespace {

constexpr int BS = 256;

// 3 x 3 patch of node displacements around (i, j); out-of-grid nodes read as zero.
template <typename T>
struct Patch {
    T u[3][3][2];
};

template <typename T>
__device__ __forceinline__ void load_patch(const Geom2 &g, const T *__restrict__ u, int i, int j, Patch<T> &p) {
#pragma unroll
    for (int di = 0; di < 3; ++di)
#pragma unroll
        for (int dj = 0; dj < 3; ++dj) {
            const int ii = i - 1 + di, jj = j - 1 + dj;
            const bool in = ii >= 0 && jj >= 0 && ii < g.nn[0] && jj < g.nn[1];
            const int64_t m = in ? g.node(ii, jj) : 0;
            p.u[di][dj][0] = in ? u[m] : T(0);
            p.u[di][dj][1] = in ? u[g.NN + m] : T(0);
        }
}

// (K u)_n and the diagonal block of K at node (i, j) from the four incident elements
// (TPSStencils.hh:189-390; m_smoothNode's Finest stencil, MultigridSolver.hh:277-292).
template <bool DIAG, typename T>
__device__ __forceinline__ void fine_row(const Geom2 &g, const T *__restrict__ Y, const Mat8T<T> &K0,
                                         const Patch<T> &p, int i, int j, T f[2], T M[4]) {
    f[0] = f[1] = T(0);
    if (DIAG) M[0] = M[1] = M[2] = M[3] = T(0);
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            const int ei = i - a, ej = j - b;
            if (ei < 0 || ej < 0 || ei >= g.ne[0] || ej >= g.ne[1]) continue;
            const T E = Y[g.elem(ei, ej)];
            const int ln = 2 * a + b;
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const int row = 2 * ln + c;
                T acc = T(0);
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    const int pi = 1 - a + (m >> 1), pj = 1 - b + (m & 1);
                    acc += K0.a[(2 * m) * 8 + row] * p.u[pi][pj][0] + K0.a[(2 * m + 1) * 8 + row] * p.u[pi][pj][1];
                }
                f[c] += E * acc;
                if (DIAG) {
                    M[2 * c] += E * K0.a[row * 8 + 2 * ln];
                    M[2 * c + 1] += E * K0.a[row * 8 + 2 * ln + 1];
                }
            }
        }
}

// m_smoothNode (MultigridSolver.hh:348-378): block solve, pointwise on partially fixed nodes.
template <typename T>
__device__ __forceinline__ void node_solve(uint8_t dm, const T bms[2], const T M[4], bool forward, T du[2]) {
    if (dm) {
        T ud[2] = {T(0), T(0)};
        if (forward) {
            ud[0] = (bms[0] - (M[0] * ud[0] + M[1] * ud[1])) * ((T)!(dm & 1) / M[0]);
            ud[1] = (bms[1] - (M[2] * ud[0] + M[3] * ud[1])) * ((T)!(dm >> 1 & 1) / M[3]);
        } else {
            ud[1] = (bms[1] - (M[2] * ud[0] + M[3] * ud[1])) * ((T)!(dm >> 1 & 1) / M[3]);
            ud[0] = (bms[0] - (M[0] * ud[0] + M[1] * ud[1])) * ((T)!(dm & 1) / M[0]);
        }
        du[0] = ud[0];
        du[1] = ud[1];
    } else {
        const T det = M[0] * M[3] - M[1] * M[2];
        const T id = T(1) / det;
        du[0] = (M[3] * bms[0] - M[1] * bms[1]) * id;
        du[1] = (M[0] * bms[1] - M[2] * bms[0]) * id;
    }
}

// Shared epilogue of the operator kernels (mode 0 apply, mode 1 residual).
template <typename T>
__device__ __forceinline__ double finish_row(const Geom2 &g, int64_t n, int j, int nyv, int mode, const T f[2],
                                             const T *__restrict__ b, const uint8_t *__restrict__ dmask, int zeroDir,
                                             const double *__restrict__ dotv, T *__restrict__ out) {
    const uint8_t dm = dmask ? dmask[n] : 0;
    T v[2];
    if (mode == 0) {
        const bool live = j < nyv;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            v[c] = live ? f[c] : T(0);
            if (zeroDir && (dm >> c & 1)) v[c] = T(0);
            out[c * g.NN + n] = v[c];
        }
        if (dotv && live) return dotv[n] * (double)v[0] + dotv[g.NN + n] * (double)v[1];
        return 0.0;
    }
    const int h = min(nyv + MARGIN, g.nn[1]);
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        if (j < h) v[c] = b[c * g.NN + n] - (j < nyv ? f[c] : T(0));
        else v[c] = out[c * g.NN + n];
        if (dm >> c & 1) v[c] = T(0);
        out[c * g.NN + n] = v[c];
    }
    return 0.0;
}

template <typename T>
__global__ void __launch_bounds__(BS) applyk2_fine_kernel(Geom2 g, const T *__restrict__ Y, Mat8T<T> K0,
                                                          const T *__restrict__ u, T *__restrict__ out, int mode,
                                                          const T *__restrict__ b, const uint8_t *__restrict__ dmask,
                                                          int zeroDir, const double *__restrict__ dotv,
                                                          double *__restrict__ partials) {
    VFEM_PDL_ENTRY();
    const int nyv = g.nyv();
    double dacc = 0.0;
    for (int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x; n < g.NN; n += (int64_t)gridDim.x * BS) {
        const int i = (int)(n / g.nn[1]), j = (int)(n - (int64_t)i * g.nn[1]);
        T f[2] = {T(0), T(0)}, M[4];
        if (j < nyv) {
            Patch<T> p;
            load_patch(g, u, i, j, p);
            fine_row<false>(g, Y, K0, p, i, j, f, M);
        }
        dacc += finish_row(g, n, j, nyv, mode, f, b, dmask, zeroDir, dotv, out);
    }
    if (partials) {
        const double s = block_sum<BS>(dacc);
        if (threadIdx.x == 0) partials[blockIdx.x] = s;
    }
}

// The fine operator in double-float on the FP32 pipe: FP64-class accuracy (about 2^-44 per
// operation) without FP64 arithmetic. u and Y arrive pre-split into hi/lo floats (the split's
// FP64 subtraction stays out of the per-node loop), K0 as hi/lo float tables; only the epilogue
// (result, residual form, dot partial) is FP64. Modes as applyk2_fine_kernel.
__global__ void __launch_bounds__(BS) applyk2_df_kernel(Geom2 g, const float *__restrict__ Yh,
                                                        const float *__restrict__ Yl, Mat8T<float> Kh,
                                                        Mat8T<float> Kl, const float *__restrict__ uh,
                                                        const float *__restrict__ ul, double *__restrict__ out,
                                                        int mode, const double *__restrict__ b,
                                                        const uint8_t *__restrict__ dmask, int zeroDir,
                                                        const double *__restrict__ dotv,
                                                        double *__restrict__ partials) {
    VFEM_PDL_ENTRY();
    const int nyv = g.nyv();
    double dacc = 0.0;
    for (int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x; n < g.NN; n += (int64_t)gridDim.x * BS) {
        const int i = (int)(n / g.nn[1]), j = (int)(n - (int64_t)i * g.nn[1]);
        double f[2] = {0.0, 0.0};
        if (j < nyv) {
            Patch<float> ph, pl;
            load_patch(g, uh, i, j, ph);
            load_patch(g, ul, i, j, pl);
            float fh[2] = {0.f, 0.f}, fl[2] = {0.f, 0.f};
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int bb = 0; bb < 2; ++bb) {
                    const int ei = i - a, ej = j - bb;
                    if (ei < 0 || ej < 0 || ei >= g.ne[0] || ej >= g.ne[1]) continue;
                    const int64_t e = g.elem(ei, ej);
                    const float eh = Yh[e], el = Yl[e];
                    const int ln = 2 * a + bb;
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        const int row = 2 * ln + c;
                        float ah = 0.f, al = 0.f;
#pragma unroll
                        for (int m = 0; m < 4; ++m) {
                            const int pi = 1 - a + (m >> 1), pj = 1 - bb + (m & 1);
#pragma unroll
                            for (int d = 0; d < 2; ++d) {
                                const int k = (2 * m + d) * 8 + row;
                                df_fma_acc(Kh.a[k], Kl.a[k], ph.u[pi][pj][d], pl.u[pi][pj][d], ah, al);
                            }
                        }
                        df_fma_acc(eh, el, ah, al, fh[c], fl[c]);
                    }
                }
            f[0] = (double)fh[0] + (double)fl[0];
            f[1] = (double)fh[1] + (double)fl[1];
        }
        dacc += finish_row(g, n, j, nyv, mode, f, b, dmask, zeroDir, dotv, out);
    }
    if (partials) {
        const double s = block_sum<BS>(dacc);
        if (threadIdx.x == 0) partials[blockIdx.x] = s;
    }
}

__device__ __forceinline__ bool color_node(const Geom2 &g, int color, int nyv, int64_t t, int &i, int &j) {
    const int o0 = color >> 1 & 1, o1 = color & 1;
    const int cj = (nyv - o1 + 1) >> 1;
    if (cj <= 0) return false;
    const int ci = (g.nn[0] - o0 + 1) >> 1;
    if (t >= (int64_t)ci * cj) return false;
    const int ii = (int)(t / cj), jj = (int)(t - (int64_t)ii * cj);
    i = 2 * ii + o0;
    j = 2 * jj + o1;
    return true;
}

// visitNodesMulticolored with 4 colours (MultigridSolver.hh:409-458) on the fine level
template <typename T>
__global__ void __launch_bounds__(BS) gs2_fine_kernel(Geom2 g, const T *__restrict__ Y, Mat8T<T> K0,
                                                      T *__restrict__ u, const T *__restrict__ b,
                                                      const uint8_t *__restrict__ dmask, int color, int forward) {
    VFEM_PDL_ENTRY();
    int i, j;
    if (!color_node(g, color, g.nyv(), blockIdx.x * (int64_t)BS + threadIdx.x, i, j)) return;
    const int64_t n = g.node(i, j);
    const uint8_t dm = dmask[n];
    if (dm == 3) return;
    Patch<T> p;
    load_patch(g, u, i, j, p);
    T f[2], M[4];
    fine_row<true>(g, Y, K0, p, i, j, f, M);
    const T bms[2] = {b[n] - f[0], b[g.NN + n] - f[1]};
    T du[2];
    node_solve(dm, bms, M, forward != 0, du);
    u[n] = p.u[1][1][0] + du[0];
    u[g.NN + n] = p.u[1][1][1] + du[1];
}

// Ke[E] = sum_f Y0[f] Kc[pos(f)] over the S x S fine elements of coarse element E
// (MultigridSolver.hh:724-819 unrolled down to the fine level); one thread per (E, row).
__global__ void __launch_bounds__(BS) ke2_coarse_kernel(Geom2 gc, int fineNe1, int S, const double *__restrict__ Y0,
                                                        const double *__restrict__ Kc, double *__restrict__ Ke) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    const int64_t e = t >> 3;
    const int r = (int)(t & 7);
    if (e >= gc.NE) return;
    const int ci = (int)(e / gc.ne[1]), cj = (int)(e - (int64_t)ci * gc.ne[1]);
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (cj < gc.maskedE()) {
        for (int pi = 0; pi < S; ++pi) {
            const double *yrow = Y0 + (int64_t)(ci * S + pi) * fineNe1 + (int64_t)cj * S;
            for (int pj = 0; pj < S; ++pj) {
                const double E = yrow[pj];
                const double *k = Kc + ((int64_t)(pi * S + pj) * 64 + r * 8);
#pragma unroll
                for (int c = 0; c < 8; ++c) acc[c] += E * k[c];
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) Ke[e * 64 + r * 8 + c] = acc[c];
}

// blockK as a 9-point stencil (MultigridSolver.hh:846-905 assembly)
__global__ void __launch_bounds__(BS) stencil2_from_ke_kernel(Geom2 g, const double *__restrict__ Ke,
                                                              double *__restrict__ S) {
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n >= g.NN) return;
    const int i = (int)(n / g.nn[1]), j = (int)(n - (int64_t)i * g.nn[1]);
    double acc[36];
#pragma unroll
    for (int k = 0; k < 36; ++k) acc[k] = 0.0;
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            const int ei = i - a, ej = j - b;
            if (ei < 0 || ej < 0 || ei >= g.ne[0] || ej >= g.ne[1]) continue;
            const double *K = Ke + g.elem(ei, ej) * 64;
            const int ln = 2 * a + b;
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const int o = ((m >> 1) - a + 1) * 3 + ((m & 1) - b + 1);
#pragma unroll
                for (int r = 0; r < 2; ++r)
#pragma unroll
                    for (int c = 0; c < 2; ++c) acc[o * 4 + 2 * r + c] += K[(2 * ln + r) * 8 + 2 * m + c];
            }
        }
#pragma unroll
    for (int k = 0; k < 36; ++k) S[(int64_t)k * g.NN + n] = acc[k];
}

template <bool DIAG, typename T>
__device__ __forceinline__ void stencil_row(const Geom2 &g, const T *__restrict__ S, const Patch<T> &p, int64_t n,
                                            T f[2], T M[4]) {
    f[0] = f[1] = T(0);
#pragma unroll
    for (int o = 0; o < 9; ++o) {
        const int di = o / 3, dj = o % 3;
        const T s00 = S[(int64_t)(o * 4 + 0) * g.NN + n], s01 = S[(int64_t)(o * 4 + 1) * g.NN + n];
        const T s10 = S[(int64_t)(o * 4 + 2) * g.NN + n], s11 = S[(int64_t)(o * 4 + 3) * g.NN + n];
        f[0] += s00 * p.u[di][dj][0] + s01 * p.u[di][dj][1];
        f[1] += s10 * p.u[di][dj][0] + s11 * p.u[di][dj][1];
        if (DIAG && o == 4) {
            M[0] = s00; M[1] = s01; M[2] = s10; M[3] = s11;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(BS) stencil2_apply_kernel(Geom2 g, const T *__restrict__ S, const T *__restrict__ u,
                                                            T *__restrict__ out, int mode, const T *__restrict__ b,
                                                            const uint8_t *__restrict__ dmask) {
    VFEM_PDL_ENTRY();
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n >= g.NN) return;
    const int nyv = g.nyv();
    const int i = (int)(n / g.nn[1]), j = (int)(n - (int64_t)i * g.nn[1]);
    T f[2] = {T(0), T(0)}, M[4];
    if (j < nyv) {
        Patch<T> p;
        load_patch(g, u, i, j, p);
        stencil_row<false>(g, S, p, n, f, M);
    }
    finish_row(g, n, j, nyv, mode, f, b, dmask, 0, nullptr, out);
}

template <typename T>
__global__ void __launch_bounds__(BS) gs2_stencil_kernel(Geom2 g, const T *__restrict__ S, T *__restrict__ u,
                                                         const T *__restrict__ b, const uint8_t *__restrict__ dmask,
                                                         int color, int forward) {
    VFEM_PDL_ENTRY();
    int i, j;
    if (!color_node(g, color, g.nyv(), blockIdx.x * (int64_t)BS + threadIdx.x, i, j)) return;
    const int64_t n = g.node(i, j);
    const uint8_t dm = dmask[n];
    if (dm == 3) return;
    Patch<T> p;
    load_patch(g, u, i, j, p);
    T f[2], M[4];
    stencil_row<true>(g, S, p, n, f, M);
    const T bms[2] = {b[n] - f[0], b[g.NN + n] - f[1]};
    T du[2];
    node_solve(dm, bms, M, forward != 0, du);
    u[n] = p.u[1][1][0] + du[0];
    u[g.NN + n] = p.u[1][1][1] + du[1];
}

// MultigridSolver.hh:217-275 (full weighting over the nondetached fine rows)
template <typename T>
__global__ void __launch_bounds__(BS) restrict2_kernel(Geom2 gf, Geom2 gc, const T *__restrict__ fine,
                                                       T *__restrict__ coarse) {
    VFEM_PDL_ENTRY();
    const int64_t cn = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (cn >= gc.NN) return;
    const int i = (int)(cn / gc.nn[1]), j = (int)(cn - (int64_t)i * gc.nn[1]);
    const int cyv = gc.nyv(), fyv = gf.nyv();
    if (j > cyv || (j == cyv && cyv == gc.nn[1])) return;
    T v0 = T(0), v1 = T(0);
    if (j < cyv) {
        const int alo = max(2 * i - 1, 0), ahi = min(2 * i + 2, gf.nn[0]);
        const int blo = max(2 * j - 1, 0), bhi = min(2 * j + 2, fyv);
        for (int a = alo; a < ahi; ++a)
            for (int b = blo; b < bhi; ++b) {
                const T w = (T(1) - abs(a - 2 * i) * T(0.5)) * (T(1) - abs(b - 2 * j) * T(0.5));
                const int64_t fn = gf.node(a, b);
                v0 += w * fine[fn];
                v1 += w * fine[gf.NN + fn];
            }
    }
    coarse[cn] = v0;
    coarse[gc.NN + cn] = v1;
}

// MultigridSolver.hh:163-212
template <typename T>
__global__ void __launch_bounds__(BS) interp2_kernel(Geom2 gf, Geom2 gc, const T *__restrict__ coarse,
                                                     T *__restrict__ fine, int accumulate) {
    VFEM_PDL_ENTRY();
    const int64_t fn = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (fn >= gf.NN) return;
    const int i = (int)(fn / gf.nn[1]), j = (int)(fn - (int64_t)i * gf.nn[1]);
    const int fyv = accumulate ? gf.nyv() : gf.nn[1];
    if (j >= fyv) return;
    const int f[2] = {i, j};
    int ec[2], lf[2];
#pragma unroll
    for (int d = 0; d < 2; ++d) {
        ec[d] = min(f[d] / 2, gc.ne[d]);
        lf[d] = f[d] - 2 * ec[d];
    }
    T acc0 = accumulate ? fine[fn] : T(0), acc1 = accumulate ? fine[gf.NN + fn] : T(0);
#pragma unroll
    for (int cn = 0; cn < 4; ++cn) {
        const int cb[2] = {cn >> 1, cn & 1};
        T coeff = T(1);
#pragma unroll
        for (int d = 0; d < 2; ++d)
            coeff *= (lf[d] == 1) ? T(0.5) : ((lf[d] == 0) ? (cb[d] ? T(0) : T(1)) : (cb[d] ? T(1) : T(0)));
        if (coeff == T(0)) continue;
        const int64_t c = gc.node(ec[0] + cb[0], ec[1] + cb[1]);
        acc0 += coeff * coarse[c];
        acc1 += coeff * coarse[gc.NN + c];
    }
    fine[fn] = acc0;
    fine[gf.NN + fn] = acc1;
}

template <typename T>
__global__ void zero_dirichlet2_kernel(Geom2 g, T *__restrict__ u, const uint8_t *__restrict__ dmask) {
    VFEM_PDL_ENTRY();
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n >= g.NN) return;
    const uint8_t dm = dmask[n];
    if (dm & 1) u[n] = T(0);
    if (dm & 2) u[g.NN + n] = T(0);
}

template <typename T>
__global__ void enforce_dirichlet2_kernel(Geom2 g, T *__restrict__ u, const uint8_t *__restrict__ dmask,
                                          const double *__restrict__ dval) {
    VFEM_PDL_ENTRY();
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n >= g.NN) return;
    const uint8_t dm = dmask[n];
    if (dm & 1) u[n] = dval ? (T)dval[n] : T(0);
    if (dm & 2) u[g.NN + n] = dval ? (T)dval[g.NN + n] : T(0);
}

template <typename T>
__global__ void masked_zero2_kernel(Geom2 g, T *__restrict__ u, int margin) {
    VFEM_PDL_ENTRY();
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n >= g.NN) return;
    const int j = (int)(n % g.nn[1]);
    if (j >= min(g.nyv() + margin, g.nn[1])) return;
    u[n] = T(0);
    u[g.NN + n] = T(0);
}

__global__ void dense2_from_stencil_kernel(Geom2 g, const double *__restrict__ S, const int *__restrict__ red,
                                           double *__restrict__ A, int nfree) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= g.NN * 9) return;
    const int64_t n = t / 9;
    const int o = (int)(t - n * 9);
    const int i = (int)(n / g.nn[1]), j = (int)(n - (int64_t)i * g.nn[1]);
    const int mi = i + o / 3 - 1, mj = j + o % 3 - 1;
    if (mi < 0 || mj < 0 || mi >= g.nn[0] || mj >= g.nn[1]) return;
    const int64_t m = g.node(mi, mj);
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int rr = red[2 * n + r];
        if (rr < 0) continue;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const int cc = red[2 * m + c];
            if (cc < 0) continue;
            A[(int64_t)rr * nfree + cc] = S[(int64_t)(o * 4 + 2 * r + c) * g.NN + n];
        }
    }
}

template <typename T>
__global__ void gather_free2_kernel(Geom2 g, const int *__restrict__ freeIdx, const int *__restrict__ nfreeDev,
                                    const T *__restrict__ b, double *__restrict__ out) {
    VFEM_PDL_ENTRY();
    const int nfree = *nfreeDev;
    const int t = blockIdx.x * BS + threadIdx.x;
    if (t >= nfree) return;
    const int d = freeIdx[t];
    out[t] = (double)b[(int64_t)(d & 1) * g.NN + (d >> 1)];
}

template <typename T>
__global__ void symv_scatter2_kernel(Geom2 g, const double *__restrict__ Ainv, const int *__restrict__ freeIdx,
                                     const int *__restrict__ nfreeDev, const double *__restrict__ bf,
                                     T *__restrict__ x) {
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
        x[(int64_t)(d & 1) * g.NN + (d >> 1)] = (T)acc;
    }
}

template <typename T>
__global__ void fill2_kernel(T *__restrict__ p, int64_t n) {
    VFEM_PDL_ENTRY();
    for (int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x; t < n; t += (int64_t)gridDim.x * BS) p[t] = T(0);
}

// ---------------- CG vector kernels (MultigridSolver.hh:1047-1152) ----------------
__global__ void __launch_bounds__(BS) dot2_kernel(Geom2 g, const double *__restrict__ a, const double *__restrict__ b,
                                                  double *__restrict__ partials) {
    VFEM_PDL_ENTRY();
    const int nyv = g.nyv();
    double acc = 0.0;
    for (int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x; n < g.NN; n += (int64_t)gridDim.x * BS) {
        if ((int)(n % g.nn[1]) >= nyv) continue;
        acc += a[n] * b[n] + a[g.NN + n] * b[g.NN + n];
    }
    const double s = block_sum<BS>(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

template <typename Ts>
__global__ void __launch_bounds__(BS) precond_out2_kernel(Geom2 g, const Ts *__restrict__ src,
                                                          double *__restrict__ s, const double *__restrict__ r,
                                                          const uint8_t *__restrict__ dmask,
                                                          double *__restrict__ partials) {
    VFEM_PDL_ENTRY();
    const int nyv = g.nyv();
    double acc = 0.0;
    for (int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x; n < g.NN; n += (int64_t)gridDim.x * BS) {
        const uint8_t dm = dmask[n];
        const double s0 = (dm & 1) ? 0.0 : (double)src[n], s1 = (dm & 2) ? 0.0 : (double)src[g.NN + n];
        s[n] = s0;
        s[g.NN + n] = s1;
        if ((int)(n % g.nn[1]) < nyv) acc += r[n] * s0 + r[g.NN + n] * s1;
    }
    const double t = block_sum<BS>(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

// d = beta d + s; when dh is given also the double-float split of the new d (dh + dl)
__global__ void direction2_kernel(Geom2 g, const double *__restrict__ s, double *__restrict__ d,
                                  const double *__restrict__ sc, float *__restrict__ dh, float *__restrict__ dl) {
    VFEM_PDL_ENTRY();
    const double beta = sc[2];
    for (int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x; t < 2 * g.NN; t += (int64_t)gridDim.x * BS) {
        const double v = beta * d[t] + s[t];
        d[t] = v;
        if (dh) df_split(v, dh[t], dl[t]);
    }
}

__global__ void __launch_bounds__(BS) cg_update2_kernel(Geom2 g, double *__restrict__ x, double *__restrict__ r,
                                                        const double *__restrict__ d, const double *__restrict__ Ad,
                                                        const double *__restrict__ sc, double *__restrict__ partials) {
    VFEM_PDL_ENTRY();
    const double alpha = sc[3];
    const int nyv = g.nyv();
    double acc = 0.0;
    for (int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x; n < g.NN; n += (int64_t)gridDim.x * BS) {
        if ((int)(n % g.nn[1]) >= nyv) continue;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const int64_t k = c * g.NN + n;
            x[k] += alpha * d[k];
            const double rv = r[k] - alpha * Ad[k];
            r[k] = rv;
            acc += rv * rv;
        }
    }
    const double s = block_sum<BS>(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// ---------------- sensitivities and loads ----------------
__device__ __forceinline__ void elem_disp(const Geom2 &g, const double *__restrict__ u, int i, int j, double ue[8]) {
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        const int64_t nm = g.node(i + (m >> 1), j + (m & 1));
        ue[2 * m] = u[nm];
        ue[2 * m + 1] = u[g.NN + nm];
    }
}

__global__ void young2_kernel(Geom2 g, const double *__restrict__ rho, double *__restrict__ Y, double E0,
                              double Emin, double gamma, double q, int law, int maskedE) {
    const int64_t e = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (e >= g.NE) return;
    const int j = (int)(e % g.ne[1]);
    const double r = rho[e];
    double y = law == 0 ? Emin + pow(r, gamma) * (E0 - Emin) : Emin + r * (E0 - Emin) / (1 + q * (1 - r));
    Y[e] = j >= maskedE ? 0.0 : y;
}

// TensorProductSimulator.hh:973-1055
__global__ void adjoint2_kernel(Geom2 g, const double *__restrict__ rho, const double *__restrict__ lam,
                                const double *__restrict__ u, double *__restrict__ out, Mat8 K0, double E0,
                                double Emin, double gamma, double q, int law, double gx, double gy, double vol,
                                double wF, double wK) {
    const int64_t e = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (e >= g.NE) return;
    const int i = (int)(e / g.ne[1]), j = (int)(e - (int64_t)i * g.ne[1]);
    if (j >= g.maskedE()) {
        out[e] = 0.0;
        return;
    }
    double le[8], ue[8];
    elem_disp(g, lam, i, j, le);
    elem_disp(g, u, i, j, ue);
    double lKu = 0.0;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        double acc = 0.0;
#pragma unroll
        for (int c = 0; c < 8; ++c) acc += K0.a[r * 8 + c] * ue[c];
        lKu += le[r] * acc;
    }
    const double x = rho[e];
    const double dY = law == 0 ? gamma * pow(x, gamma - 1.0) * (E0 - Emin)
                               : (1 + q) * (E0 - Emin) / ((1 + q * (1 - x)) * (1 + q * (1 - x)));
    double val = -wK * dY * lKu;
    if (gx != 0.0 || gy != 0.0) {
        double sg = 0.0;
#pragma unroll
        for (int l = 0; l < 4; ++l) sg += gx * le[2 * l] + gy * le[2 * l + 1];
        val += wF * 0.25 * vol * sg;
    }
    out[e] = val;
}

__global__ void energy2_kernel(Geom2 g, const double *__restrict__ Y, const double *__restrict__ u,
                               double *__restrict__ out, Mat8 K0) {
    const int64_t e = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (e >= g.NE) return;
    const int i = (int)(e / g.ne[1]), j = (int)(e - (int64_t)i * g.ne[1]);
    double ue[8];
    elem_disp(g, u, i, j, ue);
    double uKu = 0.0;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        double acc = 0.0;
#pragma unroll
        for (int c = 0; c < 8; ++c) acc += K0.a[r * 8 + c] * ue[c];
        uKu += ue[r] * acc;
    }
    out[e] = 0.5 * Y[e] * uKu;
}

// TensorProductSimulator.hh:1269-1288 (the integrated bilinear shape function is 1/4)
__global__ void gravity2_kernel(Geom2 g, const double *__restrict__ rho, double *__restrict__ f, double gx,
                                double gy, double vol) {
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n >= g.NN) return;
    const int i = (int)(n / g.nn[1]), j = (int)(n - (int64_t)i * g.nn[1]);
    double s = 0.0;
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            const int ei = i - a, ej = j - b;
            if (ei < 0 || ej < 0 || ei >= g.ne[0] || ej >= g.ne[1] || ej >= g.maskedE()) continue;
            s += 0.25 * rho[g.elem(ei, ej)] * vol;
        }
    f[n] += gx * s;
    f[g.NN + n] += gy * s;
}

// x = sum_i c_i u_i on the nondetached rows, 0 on the detached ones (the layer-by-layer
// initial guesses, LayerByLayer.hh:55-209); c from device memory (cDev) or by value
__global__ void __launch_bounds__(BS) subspace_combine2_kernel(Geom2 g, LblVectors U, int s, const double *cDev,
                                                               LblCoeffs cv, double *__restrict__ x) {
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n >= g.NN) return;
    const bool live = (int)(n % g.nn[1]) < g.nyv();
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        double v = 0.0;
        if (live) {
#pragma unroll
            for (int i = 0; i < LBL_MAX_HISTORY; ++i)
                if (i < s) v += (cDev ? cDev[i] : cv.c[i]) * U.u[i][c * g.NN + n];
        }
        x[c * g.NN + n] = v;
    }
}

unsigned colorBlocks(const Geom2 &g) {
    const int64_t per = (int64_t)((g.nn[0] + 1) / 2) * ((g.nn[1] + 1) / 2);
    return gridFor(per, BS);
}

}  // namespace

void launch2_young(const Geom2 &g, const double *rho, double *Y, double E0, double Emin, double gamma, double q,
                   int law, bool masking, cudaStream_t st) {
    young2_kernel<<<gridFor(g.NE, BS), BS, 0, st>>>(g, rho, Y, E0, Emin, gamma, q, law,
                                                    masking ? g.firstMaskedE : (int)LAYER_MASK_NONE);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch2_applyk_fine(const Geom2 &g, const T *Y, const Mat8T<T> &K0, const T *u, T *out, int mode, const T *b,
                         const uint8_t *dmask, bool zeroDir, const double *dotv, double *partials, cudaStream_t st) {
    const unsigned grid = partials ? (unsigned)REDUCE_BLOCKS : gridFor(g.NN, BS);
    launch_pdl(applyk2_fine_kernel<T>, grid, BS, 0, st, g, Y, K0, u, out, mode, b, dmask, zeroDir ? 1 : 0, dotv,
               partials);
    VFEM_LAUNCH_CHECK();
}

void launch2_applyk_df(const Geom2 &g, const float *Yh, const float *Yl, const Mat8T<float> &Kh,
                       const Mat8T<float> &Kl, const float *uh, const float *ul, double *out, int mode,
                       const double *b, const uint8_t *dmask, bool zeroDir, const double *dotv, double *partials,
                       cudaStream_t st) {
    const unsigned grid = partials ? (unsigned)REDUCE_BLOCKS : gridFor(g.NN, BS);
    launch_pdl(applyk2_df_kernel, grid, BS, 0, st, g, Yh, Yl, Kh, Kl, uh, ul, out, mode, b, dmask, zeroDir ? 1 : 0,
               dotv, partials);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch2_gs_fine(const Geom2 &g, const T *Y, const Mat8T<T> &K0, T *u, const T *b, const uint8_t *dmask, int color,
                     bool forward, cudaStream_t st) {
    launch_pdl(gs2_fine_kernel<T>, colorBlocks(g), BS, 0, st, g, Y, K0, u, b, dmask, color, forward ? 1 : 0);
    VFEM_LAUNCH_CHECK();
}

void launch2_ke_coarse(const Geom2 &gc, const Geom2 &g0, int level, const double *Y0, const double *Kc, double *Ke,
                       cudaStream_t st) {
    ke2_coarse_kernel<<<gridFor(gc.NE * 8, BS), BS, 0, st>>>(gc, g0.ne[1], 1 << level, Y0, Kc, Ke);
    VFEM_LAUNCH_CHECK();
}

void launch2_stencil_from_ke(const Geom2 &g, const double *Ke, double *S, cudaStream_t st) {
    stencil2_from_ke_kernel<<<gridFor(g.NN, BS), BS, 0, st>>>(g, Ke, S);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch2_stencil_apply(const Geom2 &g, const T *S, const T *u, T *out, int mode, const T *b, const uint8_t *dmask,
                           cudaStream_t st) {
    launch_pdl(stencil2_apply_kernel<T>, gridFor(g.NN, BS), BS, 0, st, g, S, u, out, mode, b, dmask);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch2_gs_stencil(const Geom2 &g, const T *S, T *u, const T *b, const uint8_t *dmask, int color, bool forward,
                        cudaStream_t st) {
    launch_pdl(gs2_stencil_kernel<T>, colorBlocks(g), BS, 0, st, g, S, u, b, dmask, color, forward ? 1 : 0);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch2_restrict(const Geom2 &gf, const Geom2 &gc, const T *fine, T *coarse, cudaStream_t st) {
    launch_pdl(restrict2_kernel<T>, gridFor(gc.NN, BS), BS, 0, st, gf, gc, fine, coarse);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch2_interpolate(const Geom2 &gf, const Geom2 &gc, const T *coarse, T *fine, bool accumulate, cudaStream_t st) {
    launch_pdl(interp2_kernel<T>, gridFor(gf.NN, BS), BS, 0, st, gf, gc, coarse, fine, accumulate ? 1 : 0);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch2_zero_dirichlet(const Geom2 &g, T *u, const uint8_t *dmask, cudaStream_t st) {
    launch_pdl(zero_dirichlet2_kernel<T>, gridFor(g.NN, BS), BS, 0, st, g, u, dmask);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch2_enforce_dirichlet(const Geom2 &g, T *u, const uint8_t *dmask, const double *dval, cudaStream_t st) {
    launch_pdl(enforce_dirichlet2_kernel<T>, gridFor(g.NN, BS), BS, 0, st, g, u, dmask, dval);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch2_masked_zero(const Geom2 &g, T *u, int margin, cudaStream_t st) {
    launch_pdl(masked_zero2_kernel<T>, gridFor(g.NN, BS), BS, 0, st, g, u, margin);
    VFEM_LAUNCH_CHECK();
}

void launch2_dense_from_stencil(const Geom2 &g, const double *S, const int *red, double *A, int nfree,
                                cudaStream_t st) {
    launch_fill<double>(A, 0.0, (int64_t)nfree * nfree, st);
    dense2_from_stencil_kernel<<<gridFor(g.NN * 9, BS), BS, 0, st>>>(g, S, red, A, nfree);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch2_coarse_solve(const Geom2 &g, const double *Ainv, const int *freeIdx, const int *nfreeDev, int nfreeCap,
                          const T *b, T *x, double *scratch, cudaStream_t st) {
    launch_pdl(fill2_kernel<T>, std::min<unsigned>(gridFor(2 * g.NN, BS), 4 * NUM_SMS), BS, 0, st, x, 2 * g.NN);
    VFEM_LAUNCH_CHECK();
    if (nfreeCap <= 0) return;
    launch_pdl(gather_free2_kernel<T>, gridFor(nfreeCap, BS), BS, 0, st, g, freeIdx, nfreeDev, b, scratch);
    VFEM_LAUNCH_CHECK();
    launch_pdl(symv_scatter2_kernel<T>, gridFor(nfreeCap, BS / 32), BS, 0, st, g, Ainv, freeIdx, nfreeDev,
               (const double *)scratch, x);
    VFEM_LAUNCH_CHECK();
}

void launch2_dot_partials(const Geom2 &g, const double *a, const double *b, double *partials, cudaStream_t st) {
    launch_pdl(dot2_kernel, REDUCE_BLOCKS, BS, 0, st, g, a, b, partials);
    VFEM_LAUNCH_CHECK();
}

template <typename Ts>
void launch2_precond_out(const Geom2 &g, const Ts *src, double *s, const double *r, const uint8_t *dmask,
                         double *partials, cudaStream_t st) {
    launch_pdl(precond_out2_kernel<Ts>, REDUCE_BLOCKS, BS, 0, st, g, src, s, r, dmask, partials);
    VFEM_LAUNCH_CHECK();
}

void launch2_direction(const Geom2 &g, const double *s, double *d, const double *sc, cudaStream_t st, float *dh,
                       float *dl) {
    launch_pdl(direction2_kernel, std::min<unsigned>(gridFor(2 * g.NN, BS), 4 * NUM_SMS), BS, 0, st, g, s, d, sc, dh,
               dl);
    VFEM_LAUNCH_CHECK();
}

void launch2_cg_update(const Geom2 &g, double *x, double *r, const double *d, const double *Ad, const double *sc,
                       double *partials, cudaStream_t st) {
    launch_pdl(cg_update2_kernel, REDUCE_BLOCKS, BS, 0, st, g, x, r, d, Ad, sc, partials);
    VFEM_LAUNCH_CHECK();
}

void launch2_adjoint(const Geom2 &g, const double *rho, const double *lam, const double *u, double *out,
                     const Mat8 &K0, double E0, double Emin, double gamma, double q, int law, const double grav[2],
                     double vol, double wF, double wK, cudaStream_t st) {
    adjoint2_kernel<<<gridFor(g.NE, BS), BS, 0, st>>>(g, rho, lam, u, out, K0, E0, Emin, gamma, q, law, grav[0],
                                                      grav[1], vol, wF, wK);
    VFEM_LAUNCH_CHECK();
}

void launch2_element_energy(const Geom2 &g, const double *Y, const double *u, double *out, const Mat8 &K0,
                            cudaStream_t st) {
    energy2_kernel<<<gridFor(g.NE, BS), BS, 0, st>>>(g, Y, u, out, K0);
    VFEM_LAUNCH_CHECK();
}

void launch2_gravity_load(const Geom2 &g, const double *rho, double *f, const double grav[2], double vol,
                          cudaStream_t st) {
    gravity2_kernel<<<gridFor(g.NN, BS), BS, 0, st>>>(g, rho, f, grav[0], grav[1], vol);
    VFEM_LAUNCH_CHECK();
}

void launch2_subspace_combine(const Geom2 &g, const LblVectors &U, int s, const double *cDev, const LblCoeffs &cv,
                              double *x, cudaStream_t st) {
    if (s < 0 || s > LBL_MAX_HISTORY) throw Error(ERR_ARG, "history size out of range");
    subspace_combine2_kernel<<<gridFor(g.NN, BS), BS, 0, st>>>(g, U, s, cDev, cv, x);
    VFEM_LAUNCH_CHECK();
}


#define VFEM_2D_INSTANTIATE(T)                                                                                         \
    template void launch2_applyk_fine<T>(const Geom2 &, const T *, const Mat8T<T> &, const T *, T *, int, const T *,   \
                                         const uint8_t *, bool, const double *, double *, cudaStream_t);               \
    template void launch2_gs_fine<T>(const Geom2 &, const T *, const Mat8T<T> &, T *, const T *, const uint8_t *, int, \
                                     bool, cudaStream_t);                                                              \
    template void launch2_stencil_apply<T>(const Geom2 &, const T *, const T *, T *, int, const T *, const uint8_t *,  \
                                           cudaStream_t);                                                              \
    template void launch2_gs_stencil<T>(const Geom2 &, const T *, T *, const T *, const uint8_t *, int, bool,          \
                                        cudaStream_t);                                                                 \
    template void launch2_restrict<T>(const Geom2 &, const Geom2 &, const T *, T *, cudaStream_t);                     \
    template void launch2_interpolate<T>(const Geom2 &, const Geom2 &, const T *, T *, bool, cudaStream_t);            \
    template void launch2_zero_dirichlet<T>(const Geom2 &, T *, const uint8_t *, cudaStream_t);                        \
    template void launch2_enforce_dirichlet<T>(const Geom2 &, T *, const uint8_t *, const double *, cudaStream_t);     \
    template void launch2_masked_zero<T>(const Geom2 &, T *, int, cudaStream_t);                                       \
    template void launch2_coarse_solve<T>(const Geom2 &, const double *, const int *, const int *, int, const T *, T *, \
                                          double *, cudaStream_t);                                                     \
    template void launch2_precond_out<T>(const Geom2 &, const T *, double *, const double *, const uint8_t *, double *, \
                                         cudaStream_t);
VFEM_2D_INSTANTIATE(float)
VFEM_2D_INSTANTIATE(double)

}  // namespace vfem
