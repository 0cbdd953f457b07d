// Device kernels of the Method of Moving Asymptotes (MethodOfMovingAsymptotes.hh): the
// n-length parts of an outer step (asymptotes, move limits, the approximation's p and q) and of
// the primal-dual interior-point subproblem (Newton direction, step, residuals). Each kernel is
// one grid-stride pass that also leaves per-block partial sums / maxima / minima of the
// quantities the host needs (K rows of `nb` partials); rows_reduce_kernel folds them. The m
// constraint rows (m <= MMA_MAX_M) are loop-unrolled; the (m+1)-sized linear algebra runs on
// the host.
#include "vfem_kernels.hpp"

namespace vfem {

namespace {

constexpr int BS = 256;
constexpr double RAA0 = 1e-5, ALBEFA = 0.1, MOVE = 0.5, ASYINIT = 0.5;

template <typename F>
__device__ __forceinline__ void block_rows(double (&v)[MMA_MAX_ROWS], int K, double *partials, int nb, F combine,
                                           double identity) {
    __shared__ double sh[BS / 32][MMA_MAX_ROWS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < MMA_MAX_ROWS; ++k) {
        double a = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a = combine(a, __shfl_xor_sync(0xffffffffu, a, o));
        if (lane == 0) sh[w][k] = a;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double a = identity;
        for (int q = 0; q < BS / 32; ++q) a = combine(a, sh[q][threadIdx.x]);
        partials[(int64_t)threadIdx.x * nb + blockIdx.x] = a;
    }
    __syncthreads();
}

struct Sum {
    __device__ double operator()(double a, double b) const { return a + b; }
};
struct Max {
    __device__ double operator()(double a, double b) const { return fmax(a, b); }
};

// Asymptotes (:73-95) and move limits (:96-99). mode 0: l, u at x -/+ asyinit (xmax - xmin);
// mode 1: the gamma rule from the last three iterates.
__global__ void mma_bounds_kernel(int64_t n, int mode, const double *__restrict__ x0, const double *__restrict__ x1,
                                  const double *__restrict__ x2, const double *__restrict__ xmin,
                                  const double *__restrict__ xmax, double *__restrict__ l, double *__restrict__ u,
                                  double *__restrict__ alpha, double *__restrict__ beta) {
    for (int64_t j = blockIdx.x * (int64_t)BS + threadIdx.x; j < n; j += (int64_t)gridDim.x * BS) {
        const double x = x0[j], xd = xmax[j] - xmin[j];
        double lj, uj;
        if (mode == 0) {
            lj = x - ASYINIT * xd;
            uj = x + ASYINIT * xd;
        } else {
            const double a = x1[j];
            const double gam = (x - a) * (a - x2[j]) > 0 ? 1.2 : 0.7;
            lj = fmax(fmin(x - gam * (a - l[j]), x - 0.01 * xd), x - 10 * xd);
            uj = fmin(fmax(x + gam * (u[j] - a), x + 0.01 * xd), x + 10 * xd);
        }
        l[j] = lj;
        u[j] = uj;
        alpha[j] = fmax(fmax(xmin[j], lj + ALBEFA * (x - lj)), x - MOVE * xd);
        beta[j] = fmin(fmin(xmax[j], uj - ALBEFA * (uj - x)), x + MOVE * xd);
    }
}

// p, q of the approximation around x (:127-134); rho_i / (xmax - xmin) per row when gcmma, raa0 /
// (xmax - xmin) otherwise. Partials: rows 0..m of sum_j p_ij / (u_j - x_j) + q_ij / (x_j - l_j).
__global__ void mma_pq_kernel(int64_t n, int m1, const double *__restrict__ x, const double *__restrict__ u,
                              const double *__restrict__ l, const double *__restrict__ xmin,
                              const double *__restrict__ xmax, const double *__restrict__ df, int gcmma, MmaRows rho,
                              double *__restrict__ p, double *__restrict__ q, double *__restrict__ partials) {
    double acc[MMA_MAX_ROWS];
#pragma unroll
    for (int k = 0; k < MMA_MAX_ROWS; ++k) acc[k] = 0.0;
    for (int64_t j = blockIdx.x * (int64_t)BS + threadIdx.x; j < n; j += (int64_t)gridDim.x * BS) {
        const double ux = u[j] - x[j], xl = x[j] - l[j], xd = xmax[j] - xmin[j];
        const double ux2 = ux * ux, xl2 = xl * xl;
#pragma unroll
        for (int i = 0; i < MMA_MAX_ROWS; ++i) {
            if (i >= m1) break;
            const double g = df[(int64_t)i * n + j];
            const double gp = fmax(g, 0.0), gm = fmax(-g, 0.0);
            const double ro = (gcmma ? rho.v[i] : RAA0) / xd;
            const double pi = ux2 * (1.001 * gp + 0.001 * gm + ro);
            const double qi = xl2 * (0.001 * gp + 1.001 * gm + ro);
            p[(int64_t)i * n + j] = pi;
            q[(int64_t)i * n + j] = qi;
            acc[i] += pi / ux + qi / xl;
        }
    }
    block_rows(acc, m1, partials, gridDim.x, Sum(), 0.0);
}

// Rows 0..m of sum_j |df_ij| (xmax_j - xmin_j) (GCMMA's first rho, :137-144).
__global__ void mma_absdf_kernel(int64_t n, int m1, const double *__restrict__ df, const double *__restrict__ xmin,
                                 const double *__restrict__ xmax, double *__restrict__ partials) {
    double acc[MMA_MAX_ROWS];
#pragma unroll
    for (int k = 0; k < MMA_MAX_ROWS; ++k) acc[k] = 0.0;
    for (int64_t j = blockIdx.x * (int64_t)BS + threadIdx.x; j < n; j += (int64_t)gridDim.x * BS) {
        const double xd = xmax[j] - xmin[j];
#pragma unroll
        for (int i = 0; i < MMA_MAX_ROWS; ++i) {
            if (i >= m1) break;
            acc[i] += fabs(df[(int64_t)i * n + j]) * xd;
        }
    }
    block_rows(acc, m1, partials, gridDim.x, Sum(), 0.0);
}

// At x: rows 0..m of g_i(x) = sum_j p_ij / (u_j - x_j) + q_ij / (x_j - l_j), then row m + 1 of
// sum_j (u - l)(x - xk)^2 / ((u - x)(x - l)(xmax - xmin)) (GCMMA, :146-149).
__global__ void mma_eval_kernel(int64_t n, int m1, const double *__restrict__ x, const double *__restrict__ xk,
                                const double *__restrict__ u, const double *__restrict__ l,
                                const double *__restrict__ xmin, const double *__restrict__ xmax,
                                const double *__restrict__ p, const double *__restrict__ q,
                                double *__restrict__ partials) {
    double acc[MMA_MAX_ROWS];
#pragma unroll
    for (int k = 0; k < MMA_MAX_ROWS; ++k) acc[k] = 0.0;
    for (int64_t j = blockIdx.x * (int64_t)BS + threadIdx.x; j < n; j += (int64_t)gridDim.x * BS) {
        const double ux = u[j] - x[j], xl = x[j] - l[j];
#pragma unroll
        for (int i = 0; i < MMA_MAX_ROWS; ++i) {
            if (i >= m1) break;
            acc[i] += p[(int64_t)i * n + j] / ux + q[(int64_t)i * n + j] / xl;
        }
        const double dxk = x[j] - xk[j];
        const double t = (u[j] - l[j]) * dxk * dxk / (ux * xl * (xmax[j] - xmin[j]));
#pragma unroll
        for (int i = 0; i < MMA_MAX_ROWS; ++i)
            if (i == m1) acc[i] += t;
    }
    block_rows(acc, m1 + 1, partials, gridDim.x, Sum(), 0.0);
}

// psi-derivative pieces at the subproblem point: plam, qlam, dpsi/dx (:262-267)
__device__ __forceinline__ void psi(int64_t n, int m, int64_t j, double ux, double xl, const double *p,
                                    const double *q, const MmaRows &lam, double &plam, double &qlam, double &dpsi) {
    plam = p[j];
    qlam = q[j];
#pragma unroll
    for (int i = 1; i < MMA_MAX_ROWS; ++i) {
        if (i > m) break;
        plam += lam.v[i - 1] * p[(int64_t)i * n + j];
        qlam += lam.v[i - 1] * q[(int64_t)i * n + j];
    }
    dpsi = plam / (ux * ux) - qlam / (xl * xl);
}

// init_vars (:243-268): x, xi, eta; partials rows 0..m-1 of g_i (constraint rows 1..m).
__global__ void mma_sub_init_kernel(int64_t n, int m, const double *__restrict__ alpha,
                                    const double *__restrict__ beta, const double *__restrict__ u,
                                    const double *__restrict__ l, const double *__restrict__ p,
                                    const double *__restrict__ q, double *__restrict__ x, double *__restrict__ xi,
                                    double *__restrict__ eta, double *__restrict__ partials) {
    double acc[MMA_MAX_ROWS];
#pragma unroll
    for (int k = 0; k < MMA_MAX_ROWS; ++k) acc[k] = 0.0;
    for (int64_t j = blockIdx.x * (int64_t)BS + threadIdx.x; j < n; j += (int64_t)gridDim.x * BS) {
        const double xj = 0.5 * (alpha[j] + beta[j]);
        x[j] = xj;
        xi[j] = fmax(1.0 / (xj - alpha[j]), 1.0);
        eta[j] = fmax(1.0 / (beta[j] - xj), 1.0);
        const double ux = u[j] - xj, xl = xj - l[j];
#pragma unroll
        for (int i = 1; i < MMA_MAX_ROWS; ++i) {
            if (i > m) break;
            acc[i - 1] += p[(int64_t)i * n + j] / ux + q[(int64_t)i * n + j] / xl;
        }
    }
    block_rows(acc, m, partials, gridDim.x, Sum(), 0.0);
}

// solve_for_newton_direction, n-length part (:271-281, :299-305): dx, Dx, G; partials rows:
// M entries (i <= k, m(m+1)/2), then m rows of G_i . (dx / Dx), then the three residual sums of
// squares (eq_a, eq_e, eq_f) at eps and the current point.
__global__ void mma_sub_dir1_kernel(int64_t n, int m, double eps, MmaRows lam, const double *__restrict__ x,
                                    const double *__restrict__ xi, const double *__restrict__ eta,
                                    const double *__restrict__ alpha, const double *__restrict__ beta,
                                    const double *__restrict__ u, const double *__restrict__ l,
                                    const double *__restrict__ p, const double *__restrict__ q, double *__restrict__ dxv,
                                    double *__restrict__ Dxv, double *__restrict__ G, double *__restrict__ partials) {
    double acc[MMA_MAX_ROWS];
#pragma unroll
    for (int k = 0; k < MMA_MAX_ROWS; ++k) acc[k] = 0.0;
    const int nM = m * (m + 1) / 2;
    for (int64_t j = blockIdx.x * (int64_t)BS + threadIdx.x; j < n; j += (int64_t)gridDim.x * BS) {
        const double xj = x[j], xa = xj - alpha[j], bx = beta[j] - xj;
        const double ux = u[j] - xj, xl = xj - l[j];
        double plam, qlam, dpsi;
        psi(n, m, j, ux, xl, p, q, lam, plam, qlam, dpsi);
        const double dx = dpsi - eps / xa + eps / bx;
        const double Dx = 2 * plam / (ux * (ux * ux)) + 2 * qlam / (xl * (xl * xl)) + xi[j] / xa + eta[j] / bx;
        dxv[j] = dx;
        Dxv[j] = Dx;
        double g[MMA_MAX_M];
#pragma unroll
        for (int i = 0; i < MMA_MAX_M; ++i) {
            if (i >= m) break;
            g[i] = p[(int64_t)(i + 1) * n + j] / (ux * ux) - q[(int64_t)(i + 1) * n + j] / (xl * xl);
            G[(int64_t)i * n + j] = g[i];
        }
        int t = 0;
#pragma unroll
        for (int i = 0; i < MMA_MAX_M; ++i) {
            if (i >= m) break;
#pragma unroll
            for (int k = i; k < MMA_MAX_M; ++k) {
                if (k >= m) break;
                acc[t] += g[i] * (g[k] / Dx);
                ++t;
            }
        }
#pragma unroll
        for (int i = 0; i < MMA_MAX_M; ++i) {
            if (i >= m) break;
            acc[nM + i] += g[i] * (dx / Dx);
        }
        const double ea = dpsi - xi[j] + eta[j], ee = xi[j] * xa - eps, ef = eta[j] * bx - eps;
        acc[nM + m] += ea * ea;
        acc[nM + m + 1] += ee * ee;
        acc[nM + m + 2] += ef * ef;
    }
    block_rows(acc, nM + m + 3, partials, gridDim.x, Sum(), 0.0);
}

// Newton direction from the dual solution (:306-310) and the n-length part of the step bound
// (:378-390): partial row 0 = min over j of dx/(x - alpha), dx/(x - beta), dxi/xi, deta/eta
// (stored negated, so the block reduction is a maximum).
__global__ void mma_sub_dir2_kernel(int64_t n, int m, double eps, MmaRows dlam, const double *__restrict__ x,
                                    const double *__restrict__ xi, const double *__restrict__ eta,
                                    const double *__restrict__ alpha, const double *__restrict__ beta,
                                    const double *__restrict__ dxv, const double *__restrict__ Dxv,
                                    const double *__restrict__ G, double *__restrict__ ddx, double *__restrict__ dxi,
                                    double *__restrict__ deta, double *__restrict__ partials) {
    double acc[MMA_MAX_ROWS];
#pragma unroll
    for (int k = 0; k < MMA_MAX_ROWS; ++k) acc[k] = -INFINITY;
    for (int64_t j = blockIdx.x * (int64_t)BS + threadIdx.x; j < n; j += (int64_t)gridDim.x * BS) {
        double gl = 0.0;
#pragma unroll
        for (int i = 0; i < MMA_MAX_M; ++i) {
            if (i >= m) break;
            gl += G[(int64_t)i * n + j] * dlam.v[i];
        }
        const double xj = x[j], xa = xj - alpha[j], xb = xj - beta[j];
        const double d = -(dxv[j] + gl) / Dxv[j];
        const double dxij = -xi[j] + eps / xa - xi[j] * d / xa;
        const double detaj = -eta[j] + eps / (beta[j] - xj) + eta[j] * d / (beta[j] - xj);
        ddx[j] = d;
        dxi[j] = dxij;
        deta[j] = detaj;
        const double mn = fmin(fmin(d / xa, d / xb), fmin(dxij / xi[j], detaj / eta[j]));
        acc[0] = fmax(acc[0], -mn);
    }
    block_rows(acc, 1, partials, gridDim.x, Max(), -INFINITY);
}

// newton_step(step) followed by squared_residual / KKT_inf_norm's n-length parts at the new point
// (:392-420, :224-238). Partials rows: 0..m-1 g_i, then sums of squares of eq_a, eq_e, eq_f,
// then their maxima of |.|.
__global__ void mma_sub_move_kernel(int64_t n, int m, double step, double eps, MmaRows lam, double *__restrict__ x,
                                    double *__restrict__ xi, double *__restrict__ eta,
                                    const double *__restrict__ ddx, const double *__restrict__ dxi,
                                    const double *__restrict__ deta, const double *__restrict__ alpha,
                                    const double *__restrict__ beta, const double *__restrict__ u,
                                    const double *__restrict__ l, const double *__restrict__ p,
                                    const double *__restrict__ q, double *__restrict__ partials) {
    double sums[MMA_MAX_ROWS], maxs[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int k = 0; k < MMA_MAX_ROWS; ++k) sums[k] = 0.0;
    for (int64_t j = blockIdx.x * (int64_t)BS + threadIdx.x; j < n; j += (int64_t)gridDim.x * BS) {
        const double xj = x[j] + step * ddx[j];
        const double xij = xi[j] + step * dxi[j];
        const double etaj = eta[j] + step * deta[j];
        x[j] = xj;
        xi[j] = xij;
        eta[j] = etaj;
        const double ux = u[j] - xj, xl = xj - l[j];
        double plam, qlam, dpsi;
        psi(n, m, j, ux, xl, p, q, lam, plam, qlam, dpsi);
#pragma unroll
        for (int i = 1; i < MMA_MAX_ROWS; ++i) {
            if (i > m) break;
            sums[i - 1] += p[(int64_t)i * n + j] / ux + q[(int64_t)i * n + j] / xl;
        }
        const double ea = dpsi - xij + etaj, ee = xij * (xj - alpha[j]) - eps, ef = etaj * (beta[j] - xj) - eps;
        sums[m] += ea * ea;
        sums[m + 1] += ee * ee;
        sums[m + 2] += ef * ef;
        maxs[0] = fmax(maxs[0], fabs(ea));
        maxs[1] = fmax(maxs[1], fabs(ee));
        maxs[2] = fmax(maxs[2], fabs(ef));
    }
    block_rows(sums, m + 3, partials, gridDim.x, Sum(), 0.0);
    double mx[MMA_MAX_ROWS];
#pragma unroll
    for (int k = 0; k < MMA_MAX_ROWS; ++k) mx[k] = k < 3 ? maxs[k] : 0.0;
    block_rows(mx, 3, partials + (int64_t)(m + 3) * gridDim.x, gridDim.x, Max(), 0.0);
}

// Fold K rows of nb partials: rows [0, nsum) summed, the rest maximised.
__global__ void mma_rows_reduce_kernel(const double *__restrict__ partials, int K, int nsum, int nb,
                                       double *__restrict__ out) {
    __shared__ double sh[BS / 32];
    for (int k = 0; k < K; ++k) {
        const bool isSum = k < nsum;
        double a = isSum ? 0.0 : -INFINITY;
        for (int t = threadIdx.x; t < nb; t += BS) {
            const double v = partials[(int64_t)k * nb + t];
            a = isSum ? a + v : fmax(a, v);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double b = __shfl_xor_sync(0xffffffffu, a, o);
            a = isSum ? a + b : fmax(a, b);
        }
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = a;
        __syncthreads();
        if (threadIdx.x == 0) {
            double r = sh[0];
            for (int w = 1; w < BS / 32; ++w) r = isSum ? r + sh[w] : fmax(r, sh[w]);
            out[k] = r;
        }
        __syncthreads();
    }
}

unsigned blocksFor(int64_t n) {
    int64_t b = (n + BS - 1) / BS;
    if (b > REDUCE_BLOCKS) b = REDUCE_BLOCKS;
    if (b < 1) b = 1;
    return (unsigned)b;
}

}  // namespace

unsigned mma_blocks(int64_t n) { return blocksFor(n); }

void launch_mma_bounds(int64_t n, int mode, const double *x0, const double *x1, const double *x2, const double *xmin,
                       const double *xmax, double *l, double *u, double *alpha, double *beta, cudaStream_t st) {
    mma_bounds_kernel<<<blocksFor(n), BS, 0, st>>>(n, mode, x0, x1, x2, xmin, xmax, l, u, alpha, beta);
    VFEM_LAUNCH_CHECK();
}
void launch_mma_pq(int64_t n, int m1, const double *x, const double *u, const double *l, const double *xmin,
                   const double *xmax, const double *df, bool gcmma, const MmaRows &rho, double *p, double *q,
                   double *partials, cudaStream_t st) {
    mma_pq_kernel<<<blocksFor(n), BS, 0, st>>>(n, m1, x, u, l, xmin, xmax, df, gcmma ? 1 : 0, rho, p, q, partials);
    VFEM_LAUNCH_CHECK();
}
void launch_mma_absdf(int64_t n, int m1, const double *df, const double *xmin, const double *xmax, double *partials,
                      cudaStream_t st) {
    mma_absdf_kernel<<<blocksFor(n), BS, 0, st>>>(n, m1, df, xmin, xmax, partials);
    VFEM_LAUNCH_CHECK();
}
void launch_mma_eval(int64_t n, int m1, const double *x, const double *xk, const double *u, const double *l,
                     const double *xmin, const double *xmax, const double *p, const double *q, double *partials,
                     cudaStream_t st) {
    mma_eval_kernel<<<blocksFor(n), BS, 0, st>>>(n, m1, x, xk, u, l, xmin, xmax, p, q, partials);
    VFEM_LAUNCH_CHECK();
}
void launch_mma_sub_init(int64_t n, int m, const double *alpha, const double *beta, const double *u, const double *l,
                         const double *p, const double *q, double *x, double *xi, double *eta, double *partials,
                         cudaStream_t st) {
    mma_sub_init_kernel<<<blocksFor(n), BS, 0, st>>>(n, m, alpha, beta, u, l, p, q, x, xi, eta, partials);
    VFEM_LAUNCH_CHECK();
}
void launch_mma_sub_dir1(int64_t n, int m, double eps, const MmaRows &lam, const double *x, const double *xi,
                         const double *eta, const double *alpha, const double *beta, const double *u, const double *l,
                         const double *p, const double *q, double *dx, double *Dx, double *G, double *partials,
                         cudaStream_t st) {
    mma_sub_dir1_kernel<<<blocksFor(n), BS, 0, st>>>(n, m, eps, lam, x, xi, eta, alpha, beta, u, l, p, q, dx, Dx, G,
                                                     partials);
    VFEM_LAUNCH_CHECK();
}
void launch_mma_sub_dir2(int64_t n, int m, double eps, const MmaRows &dlam, const double *x, const double *xi,
                         const double *eta, const double *alpha, const double *beta, const double *dx,
                         const double *Dx, const double *G, double *ddx, double *dxi, double *deta, double *partials,
                         cudaStream_t st) {
    mma_sub_dir2_kernel<<<blocksFor(n), BS, 0, st>>>(n, m, eps, dlam, x, xi, eta, alpha, beta, dx, Dx, G, ddx, dxi,
                                                     deta, partials);
    VFEM_LAUNCH_CHECK();
}
void launch_mma_sub_move(int64_t n, int m, double step, double eps, const MmaRows &lam, double *x, double *xi,
                         double *eta, const double *ddx, const double *dxi, const double *deta, const double *alpha,
                         const double *beta, const double *u, const double *l, const double *p, const double *q,
                         double *partials, cudaStream_t st) {
    mma_sub_move_kernel<<<blocksFor(n), BS, 0, st>>>(n, m, step, eps, lam, x, xi, eta, ddx, dxi, deta, alpha, beta, u,
                                                     l, p, q, partials);
    VFEM_LAUNCH_CHECK();
}
void launch_mma_rows_reduce(const double *partials, int K, int nsum, int nb, double *out, cudaStream_t st) {
    mma_rows_reduce_kernel<<<1, BS, 0, st>>>(partials, K, nsum, nb, out);
    VFEM_LAUNCH_CHECK();
}

}  // namespace vfem
