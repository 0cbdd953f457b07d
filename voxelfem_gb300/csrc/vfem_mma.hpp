// Method of Moving Asymptotes on the device (MethodOfMovingAsymptotes.hh); see vfem_mma.cpp.
#pragma once
#include <cstdint>
#include <vector>

#include "vfem_common.cuh"
#include "vfem_kernels.hpp"

namespace vfem {

// f: objective and constraints at x (m + 1 values); df: their gradients ((m + 1) x n, row-major).
// x is host memory. A nonzero return aborts the step.
using MmaFn = int (*)(void *user, const double *x, int64_t n, double *f_out);
using MmaGrad = int (*)(void *user, const double *x, int64_t n, double *df_out);

class MMAOpt {
public:
    MMAOpt(int64_t n, int m, const double *xmin, const double *xmax, MmaFn f, MmaGrad df, void *user);
    ~MMAOpt();
    MMAOpt(const MMAOpt &) = delete;
    MMAOpt &operator=(const MMAOpt &) = delete;
    void setInitialVar(const double *x0);
    void step();
    void getOptimalVar(double *out);
    bool gcmma = false;
    int maxInner = 1000;  // bound on GCMMA's inner loop (the reference loops until feasible)

private:
    int64_t n;
    int m, nb = 1;
    MmaFn f;
    MmaGrad df;
    void *user;
    cudaStream_t st = nullptr;
    int outerIter = 0, innerIter = 0;
    DevBuf<double> hist[3];
    int order[3] = {0, 1, 2}, hs = 0;  // history slots, newest first
    DevBuf<double> xmin, xmax, l, u, alpha, beta, p, q, dfd, G;
    DevBuf<double> xs, xi, eta, dx, Dx, ddx, dxi, deta;  // subproblem
    DevBuf<double> partials, red;
    std::vector<double> xHost, dfHost, fcur, r, a, c, d;
    const double a0 = 1.0;
    void push();
    std::vector<double> fold(int K, int nsum);
    void evalF(const double *xd, double *fout);
    void evalDF(const double *xd);
    void subsolve();
};

}  // namespace vfem
