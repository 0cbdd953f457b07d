// Method of Moving Asymptotes (MethodOfMovingAsymptotes.hh, Svanberg's MMA / GCMMA) with the
// n-length vectors on the device (k_mma.cu) and the (m+1)-sized linear algebra on the host. The
// objective and constraint values and gradients come from caller callbacks, which receive the
// iterate in host memory; their gradient is uploaded once per evaluation.
#include "vfem_mma.hpp"

#include <algorithm>
#include <cmath>
#include <limits>

namespace vfem {

MMAOpt::MMAOpt(int64_t n_, int m_, const double *xmin_, const double *xmax_, MmaFn f_, MmaGrad df_, void *user_)
    : n(n_), m(m_), f(f_), df(df_), user(user_) {
    if (n < 1) throw Error(ERR_ARG, "numVars must be positive");
    if (m < 1 || m > MMA_MAX_M) throw Error(ERR_ARG, "the device optimiser takes 1.." + std::to_string(MMA_MAX_M) + " constraints");
    VFEM_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    nb = (int)mma_blocks(n);
    xmin.alloc(n);
    xmax.alloc(n);
    VFEM_CUDA(cudaMemcpy(xmin.p, xmin_, n * sizeof(double), cudaMemcpyDefault));
    VFEM_CUDA(cudaMemcpy(xmax.p, xmax_, n * sizeof(double), cudaMemcpyDefault));
    for (auto &h : hist) h.alloc(n);
    for (DevBuf<double> *b : {&l, &u, &alpha, &beta, &xs, &xi, &eta, &dx, &Dx, &ddx, &dxi, &deta}) b->alloc(n);
    p.alloc((int64_t)(m + 1) * n);
    q.alloc((int64_t)(m + 1) * n);
    dfd.alloc((int64_t)(m + 1) * n);
    G.alloc((int64_t)m * n);
    partials.alloc((int64_t)MMA_MAX_ROWS * nb);
    red.alloc(MMA_MAX_ROWS);
    xHost.resize(n);
    dfHost.resize((size_t)(m + 1) * n);
    a.assign(m, 0.0);
    c.assign(m, 1000.0);
    d.assign(m, 1.0);
}

MMAOpt::~MMAOpt() {
    if (st) cudaStreamDestroy(st);
}

// Fold K rows of partials (the first nsum summed, the rest maximised) into host values.
std::vector<double> MMAOpt::fold(int K, int nsum) {
    launch_mma_rows_reduce(partials.p, K, nsum, nb, red.p, st);
    std::vector<double> out(K);
    VFEM_CUDA(cudaMemcpyAsync(out.data(), red.p, K * sizeof(double), cudaMemcpyDeviceToHost, st));
    VFEM_CUDA(cudaStreamSynchronize(st));
    return out;
}

void MMAOpt::setInitialVar(const double *x0) {
    push();
    VFEM_CUDA(cudaMemcpyAsync(hist[order[0]].p, x0, n * sizeof(double), cudaMemcpyDefault, st));
    VFEM_CUDA(cudaStreamSynchronize(st));
}

// FixedSizeDeque<AXd>::addToHistory: a new front slot, the oldest dropped beyond three
void MMAOpt::push() {
    const int slot = hs < 3 ? hs : order[2];
    for (int i = 2; i > 0; --i) order[i] = order[i - 1];
    order[0] = slot;
    hs = std::min(hs + 1, 3);
}

void MMAOpt::evalF(const double *xd, double *fout) {
    VFEM_CUDA(cudaMemcpyAsync(xHost.data(), xd, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    VFEM_CUDA(cudaStreamSynchronize(st));
    if (f(user, xHost.data(), n, fout)) throw Error(ERR_ARG, "objective callback failed");
}

void MMAOpt::evalDF(const double *xd) {
    VFEM_CUDA(cudaMemcpyAsync(xHost.data(), xd, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    VFEM_CUDA(cudaStreamSynchronize(st));
    if (df(user, xHost.data(), n, dfHost.data())) throw Error(ERR_ARG, "gradient callback failed");
    VFEM_CUDA(cudaMemcpyAsync(dfd.p, dfHost.data(), dfHost.size() * sizeof(double), cudaMemcpyHostToDevice, st));
}

void MMAOpt::getOptimalVar(double *out) {
    if (hs == 0) throw Error(ERR_STATE, "Must specify an initial value");
    VFEM_CUDA(cudaMemcpyAsync(out, hist[order[0]].p, n * sizeof(double), cudaMemcpyDefault, st));
    VFEM_CUDA(cudaStreamSynchronize(st));
}

// MMA::step (MethodOfMovingAsymptotes.hh:73-134)
void MMAOpt::step() {
    if (hs == 0) throw Error(ERR_STATE, "Must specify an initial value");
    ++outerIter;
    const double *x = hist[order[0]].p;
    const int mode = outerIter <= 2 ? 0 : 1;
    if (mode == 1 && hs < 3) throw Error(ERR_STATE, "MMA history too short");
    launch_mma_bounds(n, mode, x, mode ? hist[order[1]].p : x, mode ? hist[order[2]].p : x, xmin.p, xmax.p, l.p, u.p,
                      alpha.p, beta.p, st);
    fcur.assign(m + 1, 0.0);
    evalF(x, fcur.data());
    evalDF(x);
    MmaRows rho{};
    if (gcmma) {
        innerIter = 0;
        std::vector<double> diff(m + 1, 0.0);
        while (true) {
            // next_rho (:137-156)
            if (innerIter == 0) {
                launch_mma_absdf(n, m + 1, dfd.p, xmin.p, xmax.p, partials.p, st);
                const std::vector<double> s = fold(m + 1, m + 1);
                for (int i = 0; i <= m; ++i) rho.v[i] = std::max(0.1 / (double)n * s[i], 1e-6);
            } else {
                launch_mma_eval(n, m + 1, xs.p, x, u.p, l.p, xmin.p, xmax.p, p.p, q.p, partials.p, st);
                const double dd = fold(m + 2, m + 2)[m + 1];
                for (int i = 0; i <= m; ++i) {
                    const double delta = diff[i] / dd;
                    if (!(delta < 0)) rho.v[i] = std::min(1.1 * (rho.v[i] + delta), 10 * rho.v[i]);
                }
            }
            launch_mma_pq(n, m + 1, x, u.p, l.p, xmin.p, xmax.p, dfd.p, true, rho, p.p, q.p, partials.p, st);
            const std::vector<double> g0 = fold(m + 1, m + 1);
            r.assign(m + 1, 0.0);
            for (int i = 0; i <= m; ++i) r[i] = fcur[i] - g0[i];
            subsolve();
            ++innerIter;
            // isFeasible (:184-187): f(x_inner) against the approximation at x_inner
            std::vector<double> fi(m + 1);
            evalF(xs.p, fi.data());
            launch_mma_eval(n, m + 1, xs.p, x, u.p, l.p, xmin.p, xmax.p, p.p, q.p, partials.p, st);
            const std::vector<double> gi = fold(m + 2, m + 2);
            double mx = -std::numeric_limits<double>::infinity();
            for (int i = 0; i <= m; ++i) {
                diff[i] = fi[i] - (gi[i] + r[i]);
                mx = std::max(mx, diff[i]);
            }
            if (mx < 0 || innerIter >= maxInner) break;
        }
        innerIter = 0;
    } else {
        launch_mma_pq(n, m + 1, x, u.p, l.p, xmin.p, xmax.p, dfd.p, false, rho, p.p, q.p, partials.p, st);
        const std::vector<double> g0 = fold(m + 1, m + 1);
        r.assign(m + 1, 0.0);
        for (int i = 0; i <= m; ++i) r[i] = fcur[i] - g0[i];
        subsolve();
    }
    // x_history.addToHistory(subproblem solution)
    push();
    VFEM_CUDA(cudaMemcpyAsync(hist[order[0]].p, xs.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    VFEM_CUDA(cudaStreamSynchronize(st));
}

// Gaussian elimination with partial pivoting on the (m+1) x (m+1) dual system
static std::vector<double> dense_solve(std::vector<double> M, std::vector<double> b, int N) {
    for (int k = 0; k < N; ++k) {
        int piv = k;
        for (int i = k + 1; i < N; ++i)
            if (std::fabs(M[i * N + k]) > std::fabs(M[piv * N + k])) piv = i;
        if (piv != k) {
            for (int j = 0; j < N; ++j) std::swap(M[k * N + j], M[piv * N + j]);
            std::swap(b[k], b[piv]);
        }
        for (int i = k + 1; i < N; ++i) {
            const double f = M[i * N + k] / M[k * N + k];
            for (int j = k; j < N; ++j) M[i * N + j] -= f * M[k * N + j];
            b[i] -= f * b[k];
        }
    }
    std::vector<double> x(N);
    for (int i = N - 1; i >= 0; --i) {
        double s = b[i];
        for (int j = i + 1; j < N; ++j) s -= M[i * N + j] * x[j];
        x[i] = s / M[i * N + i];
    }
    return x;
}

// Subproblem::subsolve (:206-224): primal-dual interior point, eps = 1, 0.1, ..., 1e-7, at most
// ten Newton steps per eps with halving line search on the squared KKT residual.
void MMAOpt::subsolve() {
    const int M1 = m + 1, nM = m * (m + 1) / 2;
    std::vector<double> y(m, 1.0), lam(m, 1.0), s(m, 1.0), mu(m);
    double z = 1.0, zeta = 1.0;
    for (int i = 0; i < m; ++i) mu[i] = std::max(c[i] / 2, 1.0);
    launch_mma_sub_init(n, m, alpha.p, beta.p, u.p, l.p, p.p, q.p, xs.p, xi.p, eta.p, partials.p, st);
    std::vector<double> g = fold(m, m);
    const std::vector<double> rr(r.begin() + 1, r.end());
    auto rows = [&](const std::vector<double> &v) {
        MmaRows R{};
        for (int i = 0; i < (int)v.size(); ++i) R.v[i] = v[i];
        return R;
    };
    // host parts of the squared residual and of the KKT infinity norm (eq_b, eq_c, eq_d, eq_g,
    // eq_h, eq_i; :453-461)
    auto hostRes = [&](double eps, double &sq, double &mx) {
        sq = 0.0;
        mx = 0.0;
        double ec = a0 - zeta;
        for (int i = 0; i < m; ++i) ec -= lam[i] * a[i];
        auto add = [&](double v) {
            sq += v * v;
            mx = std::max(mx, std::fabs(v));
        };
        for (int i = 0; i < m; ++i) add(c[i] + d[i] * y[i] - lam[i] - mu[i]);
        add(ec);
        for (int i = 0; i < m; ++i) add(g[i] - a[i] * z - y[i] + s[i] + rr[i]);
        for (int i = 0; i < m; ++i) add(mu[i] * y[i] - eps);
        add(zeta * z - eps);
        for (int i = 0; i < m; ++i) add(lam[i] * s[i] - eps);
    };
    double eps = 1.0;
    while (eps > 1e-7) {
        double resOld = 0.0;
        for (int it = 0; it < 10; ++it) {
            // solve_for_newton_direction (:271-320)
            launch_mma_sub_dir1(n, m, eps, rows(lam), xs.p, xi.p, eta.p, alpha.p, beta.p, u.p, l.p, p.p, q.p, dx.p,
                                Dx.p, G.p, partials.p, st);
            const std::vector<double> d1 = fold(nM + m + 3, nM + m + 3);
            std::vector<double> Dy(m), dy(m);
            for (int i = 0; i < m; ++i) {
                Dy[i] = d[i] + mu[i] / y[i];
                dy[i] = c[i] + d[i] * y[i] - lam[i] - eps / y[i];
            }
            std::vector<double> Mx((size_t)M1 * M1, 0.0), rhs(M1, 0.0);
            int t = 0;
            for (int i = 0; i < m; ++i)
                for (int k = i; k < m; ++k, ++t) Mx[i * M1 + k] = Mx[k * M1 + i] = d1[t];
            for (int i = 0; i < m; ++i) {
                Mx[i * M1 + i] += s[i] / lam[i] + 1.0 / Dy[i];
                Mx[i * M1 + m] = Mx[m * M1 + i] = a[i];
            }
            Mx[m * M1 + m] = -zeta / z;
            double la = 0.0;
            for (int i = 0; i < m; ++i) {
                rhs[i] = g[i] - a[i] * z - y[i] + rr[i] + eps / lam[i] + dy[i] / Dy[i] - d1[nM + i];
                la += lam[i] * a[i];
            }
            rhs[m] = a0 - la - eps / z;
            const std::vector<double> sol = dense_solve(Mx, rhs, M1);
            std::vector<double> dlam(sol.begin(), sol.begin() + m);
            const double dz = sol[m];
            std::vector<double> dyv(m), dmu(m), ds(m);
            for (int i = 0; i < m; ++i) {
                dyv[i] = dlam[i] / Dy[i] - dy[i] / Dy[i];
                dmu[i] = (eps - mu[i] * dyv[i]) / y[i] - mu[i];
                ds[i] = (eps - s[i] * dlam[i]) / lam[i] - s[i];
            }
            const double dzeta = (eps - zeta * dz) / z - zeta;
            if (it == 0) {
                double hs_, hm_;
                hostRes(eps, hs_, hm_);
                resOld = d1[nM + m] + d1[nM + m + 1] + d1[nM + m + 2] + hs_;
            }
            launch_mma_sub_dir2(n, m, eps, rows(dlam), xs.p, xi.p, eta.p, alpha.p, beta.p, dx.p, Dx.p, G.p, ddx.p,
                                dxi.p, deta.p, partials.p, st);
            double mc = -fold(1, 0)[0];
            for (int i = 0; i < m; ++i)
                mc = std::min({mc, dyv[i] / y[i], ds[i] / s[i], dmu[i] / mu[i], dlam[i] / lam[i]});
            mc = std::min({mc, dz / z, dzeta / zeta});
            double stp = 1.0 / std::max(-1.01 * mc, 1.0);
            // newton_step_backtrack (:365-376)
            double kktDev = 0.0;
            auto move = [&](double sgnStep) {
                for (int i = 0; i < m; ++i) {
                    y[i] += sgnStep * dyv[i];
                    lam[i] += sgnStep * dlam[i];
                    mu[i] += sgnStep * dmu[i];
                    s[i] += sgnStep * ds[i];
                }
                z += sgnStep * dz;
                zeta += sgnStep * dzeta;
                launch_mma_sub_move(n, m, sgnStep, eps, rows(lam), xs.p, xi.p, eta.p, ddx.p, dxi.p, deta.p, alpha.p,
                                    beta.p, u.p, l.p, p.p, q.p, partials.p, st);
                const std::vector<double> mv = fold(m + 6, m + 3);
                for (int i = 0; i < m; ++i) g[i] = mv[i];
                double hs_, hm_;
                hostRes(eps, hs_, hm_);
                kktDev = std::max({mv[m + 3], mv[m + 4], mv[m + 5], hm_});
                return mv[m] + mv[m + 1] + mv[m + 2] + hs_;
            };
            double res = move(stp);
            while (res > resOld) {
                stp /= 2;
                res = move(-stp);
            }
            resOld = res;
            if (kktDev <= 0.9 * eps) break;
        }
        eps *= 0.1;
    }
}

}  // namespace vfem
