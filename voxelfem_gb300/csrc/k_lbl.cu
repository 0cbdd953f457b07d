// Initial guesses of the warm-started layer-by-layer evaluation (LayerByLayer.hh:55-209):
// a combination of the solutions of the previous (taller) builds. The subspace guess
// (InitGenSubspace) is the Galerkin projection of the new problem onto the span of the last s
// solutions u_i: A c = b with A_ij = u_i . K u_j and b_i = u_i . f (both for the NEW mask), solved
// in the least-squares sense with singular values below s * eps * sigma_max dropped
// (Eigen::JacobiSVD::solve semantics), g = sum_i c_i u_i on the nondetached nodes. The reference
// updates A and b by recurrences over the removed layers; this file forms them directly from
// s matvecs and dot products, which the GPU does in a fraction of a millisecond.
#include "vfem_kernels.hpp"
#include "vfem_reduce.cuh"

namespace vfem {

namespace {

constexpr int BS = 256;

// Symmetric eigendecomposition (cyclic Jacobi) and minimum-norm least-squares solve of an
// s x s system; one thread.
__device__ void sym_pinv_solve(double A[LBL_MAX_HISTORY][LBL_MAX_HISTORY], const double *b, int s, double *c) {
    double V[LBL_MAX_HISTORY][LBL_MAX_HISTORY];
    for (int i = 0; i < s; ++i)
        for (int j = 0; j < s; ++j) V[i][j] = i == j ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < s; ++i) {
            diag += A[i][i] * A[i][i];
            for (int j = i + 1; j < s; ++j) off += A[i][j] * A[i][j];
        }
        if (off <= 1e-32 * diag || off == 0.0) break;
        for (int p = 0; p < s; ++p)
            for (int q = p + 1; q < s; ++q) {
                if (A[p][q] == 0.0) continue;
                const double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
                for (int k = 0; k < s; ++k) {  // columns p, q
                    const double akp = A[k][p], akq = A[k][q];
                    A[k][p] = cs * akp - sn * akq;
                    A[k][q] = sn * akp + cs * akq;
                }
                for (int k = 0; k < s; ++k) {  // rows p, q
                    const double apk = A[p][k], aqk = A[q][k];
                    A[p][k] = cs * apk - sn * aqk;
                    A[q][k] = sn * apk + cs * aqk;
                }
                for (int k = 0; k < s; ++k) {
                    const double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = cs * vkp - sn * vkq;
                    V[k][q] = sn * vkp + cs * vkq;
                }
            }
    }
    double smax = 0.0;
    for (int i = 0; i < s; ++i) smax = fmax(smax, fabs(A[i][i]));
    const double thr = (double)(s > 1 ? s : 1) * 2.220446049250313e-16 * smax;
    for (int i = 0; i < s; ++i) c[i] = 0.0;
    for (int k = 0; k < s; ++k) {
        const double lam = A[k][k];
        if (!(fabs(lam) > thr)) continue;
        double vb = 0.0;
        for (int i = 0; i < s; ++i) vb += V[i][k] * b[i];
        for (int i = 0; i < s; ++i) c[i] += V[i][k] * vb / lam;
    }
}

// partials: for p = 0 .. s(s+1)/2 - 1 the pairs (i <= j) of u_i . K u_j, then s entries u_i . f;
// each nb doubles. Writes c[0..s).
__global__ void subspace_solve_kernel(const double *__restrict__ partials, int nb, int s, double *__restrict__ c) {
    __shared__ double vals[LBL_MAX_HISTORY * (LBL_MAX_HISTORY + 3) / 2];
    const int np = s * (s + 1) / 2 + s;
    for (int p = 0; p < np; ++p) {
        double acc = 0.0;
        for (int q = threadIdx.x; q < nb; q += BS) acc += partials[(int64_t)p * nb + q];
        acc = block_sum<BS>(acc);
        if (threadIdx.x == 0) vals[p] = acc;
    }
    if (threadIdx.x == 0) {
        double A[LBL_MAX_HISTORY][LBL_MAX_HISTORY], b[LBL_MAX_HISTORY];
        int p = 0;
        for (int i = 0; i < s; ++i)
            for (int j = i; j < s; ++j) {
                A[i][j] = A[j][i] = vals[p];
                ++p;
            }
        for (int i = 0; i < s; ++i) b[i] = vals[p + i];
        sym_pinv_solve(A, b, s, c);
    }
}

// x = sum_i c_i u_i on the nondetached nodes, 0 on the detached ones; c from device memory
// (cDev) or by value.
__global__ void __launch_bounds__(BS) subspace_combine_kernel(Geom g, LblVectors U, int s, const double *cDev,
                                                              LblCoeffs cv, double *__restrict__ x) {
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n >= g.NN) return;
    const int j = (int)(((uint32_t)n / (uint32_t)g.nn[2]) % (uint32_t)g.nn[1]);
    const bool live = j < g.nyv();
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        double v = 0.0;
        if (live) {
#pragma unroll
            for (int i = 0; i < LBL_MAX_HISTORY; ++i)
                if (i < s) v += (cDev ? cDev[i] : cv.c[i]) * U.u[i][c * g.ld + n];
        }
        x[c * g.ld + n] = v;
    }
}

}  // namespace

void launch_subspace_solve(const double *partials, int nb, int s, double *c, cudaStream_t st) {
    if (s < 1 || s > LBL_MAX_HISTORY) throw Error(ERR_ARG, "history size out of range");
    subspace_solve_kernel<<<1, BS, 0, st>>>(partials, nb, s, c);
    VFEM_LAUNCH_CHECK();
}

void launch_subspace_combine(const Geom &g, const LblVectors &U, int s, const double *cDev, const LblCoeffs &cv,
                             double *x, cudaStream_t st) {
    if (s < 0 || s > LBL_MAX_HISTORY) throw Error(ERR_ARG, "history size out of range");
    subspace_combine_kernel<<<gridFor(g.NN, BS), BS, 0, st>>>(g, U, s, cDev, cv, x);
    VFEM_LAUNCH_CHECK();
}

}  // namespace vfem
