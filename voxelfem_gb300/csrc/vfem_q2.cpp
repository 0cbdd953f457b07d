// Triquadratic voxel grid (TensorProductSimulator<Real, 2, 2, 2>, TPSStencils.hh:135-186): the
// element stiffness, SIMP moduli, zero-displacement supports, the matrix-free applyK and the
// 27-colour block Gauss-Seidel sweep of the reference's generic (Q2) multigrid smoother
// (MultigridSolver.hh:277-321, 409-442), in FP64 or FP32, and timing hooks.
#include "vfem_engine.hpp"

#include <cstring>
#include <type_traits>

#include "vfem_element.hpp"

namespace vfem {

GridQ2::GridQ2(const int ne_[3], const double bmin_[3], const double bmax_[3]) {
    for (int d = 0; d < 3; ++d) {
        if (ne_[d] <= 0) throw Error(ERR_ARG, "elementsPerDimension must be positive");
        if (!(bmax_[d] > bmin_[d])) throw Error(ERR_ARG, "invalid domain bounding box");
        ne[d] = ne_[d];
        nn[d] = 2 * ne_[d] + 1;
        bmin[d] = bmin_[d];
        bmax[d] = bmax_[d];
        h[d] = (bmax[d] - bmin[d]) / ne[d];
    }
    NN = (int64_t)nn[0] * nn[1] * nn[2];
    NE = (int64_t)ne[0] * ne[1] * ne[2];
    if (3 * NN >= (int64_t(1) << 31)) throw Error(ERR_ARG, "grid too large");
    VFEM_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    egeom = makeGeom(ne);
    rho.alloc(NE);
    Y.alloc(NE);
    Yf.alloc(NE);
    Yhi.alloc(NE);
    Ylo.alloc(NE);
    VFEM_CUDA(cudaMemsetAsync(rho.p, 0, NE * sizeof(double), stream));
    dmask_h.assign(NN, 0);
    dmask.alloc(NN);
    K0.assign(6561, 0.0);
    K0f.assign(6561, 0.f);
    K0lo.assign(6561, 0.f);
    K0d.alloc(6561);
    uploadMask();
    setETensor(1.0, 0.0);
    updateYoungModuli();
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

GridQ2::~GridQ2() {
    mg1.reset();
    q1.reset();
    if (cgHost) cudaFreeHost(cgHost);
    if (stream) cudaStreamDestroy(stream);
}

void GridQ2::setETensor(double E, double nu_) {
    if (!(nu_ < 0.5) || !(nu_ > -1.0)) throw Error(ERR_ARG, "Poisson ratio must lie in (-1, 0.5)");
    Eyoung = E;
    nu = nu_;
    element_stiffness_q2(E, nu, h, K0.data());
    for (int t = 0; t < 6561; ++t) {
        K0f[t] = (float)K0[t];
        K0lo[t] = (float)(K0[t] - (double)K0f[t]);
    }
    VFEM_CUDA(cudaMemcpy(K0d.p, K0.data(), 6561 * sizeof(double), cudaMemcpyHostToDevice));
}

void GridQ2::setParams(double E0_, double Emin_, double gamma_, double q_, int law_) {
    E0 = E0_;
    Emin = Emin_;
    gamma = gamma_;
    q = q_;
    law = law_;
    updateYoungModuli();
}

void GridQ2::updateYoungModuli() {
    launch_young_moduli<double>(egeom, rho.p, Y.p, E0, Emin, gamma, q, law, false, stream);
    launch_cast<float, double>(Y.p, Yf.p, NE, stream);
    launch_split_df(Y.p, Yhi.p, Ylo.p, NE, stream);
}

// out = K u in double-float arithmetic (FP64-class result, no FP64 arithmetic in the sums)
void GridQ2::applyDF(const double *u, double *out, bool zeroDirichlet, cudaStream_t st) {
    uhi.alloc(3 * NN);
    ulo.alloc(3 * NN);
    launch_split_df(u, uhi.p, ulo.p, 3 * NN, st);
    q2_upload_k0f(K0f.data(), st);  // constant memory is shared by every Q2 grid
    q2_upload_k0lo(K0lo.data(), st);
    launch_applyk_q2_df(ne, Yhi.p, Ylo.p, uhi.p, ulo.p, out, dmask.p, zeroDirichlet, st);
}

void GridQ2::setDensities(const double *r) {
    VFEM_CUDA(cudaMemcpyAsync(rho.p, r, NE * sizeof(double), cudaMemcpyDefault, stream));
    updateYoungModuli();
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

void GridQ2::uploadMask() {
    VFEM_CUDA(cudaMemcpyAsync(dmask.p, dmask_h.data(), NN, cudaMemcpyHostToDevice, stream));
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

// Zero-displacement supports on the nodes inside the box [mn, mx] (node (I, J, K) at
// bmin + (I, J, K) h / 2), components in cmask.
void GridQ2::addDirichlet(const double mn[3], const double mx[3], unsigned cmask) {
    for (int I = 0; I < nn[0]; ++I) {
        const double px = bmin[0] + 0.5 * I * h[0];
        if (px < mn[0] || px > mx[0]) continue;
        for (int J = 0; J < nn[1]; ++J) {
            const double py = bmin[1] + 0.5 * J * h[1];
            if (py < mn[1] || py > mx[1]) continue;
            for (int K = 0; K < nn[2]; ++K) {
                const double pz = bmin[2] + 0.5 * K * h[2];
                if (pz < mn[2] || pz > mx[2]) continue;
                dmask_h[((int64_t)I * nn[1] + J) * nn[2] + K] |= (uint8_t)(cmask & 7u);
            }
        }
    }
    uploadMask();
    boxes.push_back(Box{{mn[0], mn[1], mn[2]}, {mx[0], mx[1], mx[2]}, cmask & 7u});
    mg1.reset();
    q1.reset();
    q1Coarsenings = -1;
}

static void allocWork(LevelData<double> &D, int64_t n3) { D.x.alloc(n3); D.b.alloc(n3); D.r.alloc(n3); }
static void allocWork(LevelData<float> &D, int64_t n3) { D.x.alloc(n3); D.b.alloc(n3); D.r.alloc(n3); }

template <>
LevelData<double> &GridQ2::work<double>() {
    allocWork(w64, 3 * NN);
    return w64;
}
template <>
LevelData<float> &GridQ2::work<float>() {
    allocWork(w32, 3 * NN);
    return w32;
}

template <typename T>
static void toT(const double *src, T *dst, int64_t n, cudaStream_t st) {
    if (std::is_same<T, double>::value) VFEM_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    else launch_cast<float, double>(src, (float *)dst, n, st);
}
template <typename T>
static void fromT(const T *src, double *dst, int64_t n, cudaStream_t st) {
    if (std::is_same<T, double>::value) VFEM_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    else launch_cast<double, float>((const float *)src, dst, n, st);
}

template <typename T>
const T *GridQ2::kernelK0() {
    if (std::is_same<T, float>::value) {
        q2_upload_k0f(K0f.data(), stream);  // constant memory is shared by every Q2 grid
        return nullptr;
    }
    return (const T *)K0d.p;
}

template <typename T>
void GridQ2::applyKT(const double *u, double *out, bool zeroDirichlet) {
    auto &D = work<T>();
    const int64_t n3 = 3 * NN;
    toT<T>(u, D.x.p, n3, stream);
    const T *Yt = std::is_same<T, double>::value ? (const T *)Y.p : (const T *)Yf.p;
    launch_applyk_q2<T>(ne, kernelK0<T>(), Yt, D.x.p, D.r.p, dmask.p, zeroDirichlet, stream);
    fromT<T>(D.r.p, out, n3, stream);
}

template <typename T>
void GridQ2::smoothT(double *u, const double *b, bool forward) {
    auto &D = work<T>();
    const int64_t n3 = 3 * NN;
    toT<T>(u, D.x.p, n3, stream);
    toT<T>(b, D.b.p, n3, stream);
    const T *Yt = std::is_same<T, double>::value ? (const T *)Y.p : (const T *)Yf.p;
    launch_gs_q2_sweep<T>(ne, kernelK0<T>(), Yt, D.x.p, D.b.p, dmask.p, forward, stream);
    fromT<T>(D.x.p, u, n3, stream);
}

void GridQ2::applyK(const double *u, double *out, int precision, bool zeroDirichlet) {
    View vu, vo;
    viewIn(vu, u, 3 * NN * sizeof(double), stream);
    viewOut(vo, out, 3 * NN * sizeof(double));
    if (precision == PREC_FP64) applyKT<double>((const double *)vu.d, (double *)vo.d, zeroDirichlet);
    else if (precision == 2) applyDF((const double *)vu.d, (double *)vo.d, zeroDirichlet, stream);
    else applyKT<float>((const double *)vu.d, (double *)vo.d, zeroDirichlet);
    finishOut(vo, stream);
}

void GridQ2::smooth(double *u, const double *b, bool forward, int precision) {
    View vu, vb;
    viewInOut(vu, u, 3 * NN * sizeof(double), stream);
    viewIn(vb, b, 3 * NN * sizeof(double), stream);
    if (precision == PREC_FP64) smoothT<double>((double *)vu.d, (const double *)vb.d, forward);
    else smoothT<float>((double *)vu.d, (const double *)vb.d, forward);
    finishOut(vu, stream);
}

double GridQ2::timeSmooth(int precision, int reps, double *bytes) {
    if (reps <= 0) throw Error(ERR_ARG, "reps must be positive");
    auto run = [&](auto tag) {
        using T = decltype(tag);
        auto &D = work<T>();
        const T *Yt = std::is_same<T, double>::value ? (const T *)Y.p : (const T *)Yf.p;
        launch_fill<T>(D.x.p, T(0.5), 3 * NN, stream);
        launch_fill<T>(D.b.p, T(1), 3 * NN, stream);
        const T *K = kernelK0<T>();
        launch_gs_q2_sweep<T>(ne, K, Yt, D.x.p, D.b.p, dmask.p, true, stream);
        cudaEvent_t e0, e1;
        VFEM_CUDA(cudaEventCreate(&e0));
        VFEM_CUDA(cudaEventCreate(&e1));
        VFEM_CUDA(cudaEventRecord(e0, stream));
        for (int r = 0; r < reps; ++r) launch_gs_q2_sweep<T>(ne, K, Yt, D.x.p, D.b.p, dmask.p, true, stream);
        VFEM_CUDA(cudaEventRecord(e1, stream));
        VFEM_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        VFEM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        *bytes = (double)sizeof(T) * (9.0 * NN + NE);
        return (double)ms / reps;
    };
    return precision == PREC_FP64 ? run(double()) : run(float());
}

// Average device time of one applyK launch on resident data, with its algorithmic bytes
// s * (6 NN + NE) (read u, write K u, read E).
double GridQ2::timeApplyK(int precision, int reps, double *bytes) {
    if (reps <= 0) throw Error(ERR_ARG, "reps must be positive");
    if (precision == 2) {
        auto &D = work<double>();
        launch_fill<double>(D.x.p, 0.5, 3 * NN, stream);
        applyDF(D.x.p, D.r.p, false, stream);
        cudaEvent_t e0, e1;
        VFEM_CUDA(cudaEventCreate(&e0));
        VFEM_CUDA(cudaEventCreate(&e1));
        VFEM_CUDA(cudaEventRecord(e0, stream));
        for (int r = 0; r < reps; ++r) launch_applyk_q2_df(ne, Yhi.p, Ylo.p, uhi.p, ulo.p, D.r.p, dmask.p, false, stream);
        VFEM_CUDA(cudaEventRecord(e1, stream));
        VFEM_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        VFEM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        *bytes = 8.0 * (6.0 * NN + NE);
        return (double)ms / reps;
    }
    auto run = [&](auto tag) {
        using T = decltype(tag);
        auto &D = work<T>();
        const T *Yt = std::is_same<T, double>::value ? (const T *)Y.p : (const T *)Yf.p;
        launch_fill<T>(D.x.p, T(0.5), 3 * NN, stream);
        const T *K = kernelK0<T>();
        launch_applyk_q2<T>(ne, K, Yt, D.x.p, D.r.p, dmask.p, false, stream);
        cudaEvent_t e0, e1;
        VFEM_CUDA(cudaEventCreate(&e0));
        VFEM_CUDA(cudaEventCreate(&e1));
        VFEM_CUDA(cudaEventRecord(e0, stream));
        for (int r = 0; r < reps; ++r) launch_applyk_q2<T>(ne, K, Yt, D.x.p, D.r.p, dmask.p, false, stream);
        VFEM_CUDA(cudaEventRecord(e1, stream));
        VFEM_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        VFEM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        *bytes = (double)sizeof(T) * (6.0 * NN + NE);
        return (double)ms / reps;
    };
    return precision == PREC_FP64 ? run(double()) : run(float());
}

// The trilinear grid on the same mesh carries the same material, densities and supports; its
// FP32 multigrid hierarchy is the coarse correction of the Q2 preconditioner.
void GridQ2::prepareQ1(int coarsenings) {
    if (!q1 || q1Coarsenings != coarsenings) {
        mg1.reset();
        q1 = std::make_unique<Grid>(ne, bmin, bmax);
        const double zero[3] = {0.0, 0.0, 0.0};
        for (const Box &b : boxes) q1->addDirichlet(zero, b.mn, b.mx, b.cmask);
        mg1 = std::make_unique<MG>(q1.get(), coarsenings);
        mg1->setPrecision(PREC_MIXED);
        mg1->symmetricGS = true;
        q1Coarsenings = coarsenings;
    }
    if (q1->Eyoung != Eyoung || q1->nu != nu) q1->setETensor(Eyoung, nu);
    q1->E0 = E0;
    q1->Emin = Emin;
    q1->gamma = gamma;
    q1->q = q;
    q1->law = law;
    VFEM_CUDA(cudaStreamSynchronize(stream));
    VFEM_CUDA(cudaMemcpy(q1->rho.p, rho.p, NE * sizeof(double), cudaMemcpyDeviceToDevice));
    q1->updateYoungModuli();
    VFEM_CUDA(cudaStreamSynchronize(q1->stream));
    mg1->ensureStiffness();
}

// z = M r: Q2 forward sweeps from zero, the residual restricted to the trilinear mesh, one V-cycle
// there, the prolongated correction, Q2 backward sweeps (a symmetric preconditioner). The result
// stays in the FP32 work vector w32.x. Runs on the trilinear grid's stream (the Q2 stream is
// idle whenever this is called).
void GridQ2::precondition(const double *r, int64_t sweeps) {
    cudaStream_t st = q1->stream;
    auto &W = work<float>();
    const int64_t n3 = 3 * NN;
    launch_cast<float, double>(r, W.b.p, n3, st);
    launch_fill<float>(W.x.p, 0.f, n3, st);
    q2_upload_k0f(K0f.data(), st);
    for (int64_t s = 0; s < sweeps; ++s) launch_gs_q2_sweep<float>(ne, nullptr, Yf.p, W.x.p, W.b.p, dmask.p, true, st);
    launch_applyk_q2<float>(ne, nullptr, Yf.p, W.x.p, W.r.p, dmask.p, true, st);
    launch_q2_residual_combine<float>(NN, W.b.p, W.r.p, W.r.p, dmask.p, st);
    auto &F = mg1->lv[0].d32;
    launch_restrict_q2_q1<float>(ne, W.r.p, F.b.p, st);
    mg1->vcycleOnFineRhs(sweeps);
    launch_interp_q1_q2<float>(ne, F.x.p, W.x.p, true, st);
    for (int64_t s = 0; s < sweeps; ++s) launch_gs_q2_sweep<float>(ne, nullptr, Yf.p, W.x.p, W.b.p, dmask.p, false, st);
}

// MultigridSolver.hh:1047-1152 recurrences (masked dot products over all nodes, deferred first
// direction) with the Q2 operator and the preconditioner above.
PcgStats GridQ2::pcg(double *x, const double *b, int64_t maxIter, double tol, int coarsenings, int64_t sweeps) {
    if (coarsenings < 1) throw Error(ERR_ARG, "the Q2 preconditioner needs at least one coarsening of the trilinear mesh");
    VFEM_CUDA(cudaStreamSynchronize(stream));
    prepareQ1(coarsenings);
    cudaStream_t st = q1->stream;
    const int64_t n3 = 3 * NN;
    cgX.alloc(n3);
    cgR.alloc(n3);
    cgS.alloc(n3);
    cgD.alloc(n3);
    cgAd.alloc(n3);
    cgPart.alloc(REDUCE_BLOCKS + 1);
    cgSc.alloc(16);
    if (!cgHost) VFEM_CUDA(cudaMallocHost(&cgHost, 16 * sizeof(double)));
    const int n2[3] = {2 * ne[0], 2 * ne[1], 2 * ne[2]};
    const Geom gq = makeGeom(n2);  // the Q2 nodes as the nodes of a trilinear grid: reductions and updates
    View vx, vb;
    viewInOut(vx, x, n3 * sizeof(double), st);
    viewIn(vb, b, n3 * sizeof(double), st);
    VFEM_CUDA(cudaMemcpyAsync(cgX.p, vx.d, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
    launch_zero_dirichlet<double>(gq, cgX.p, dmask.p, st);
    const double *B = (const double *)vb.d;
    launch_masked_dot_partials<double, double>(gq, B, B, cgPart.p, st);
    launch_finalize(cgPart.p, REDUCE_BLOCKS, cgSc.p + 7, st);
    if (outerDF) applyDF(cgX.p, cgAd.p, true, st);
    else launch_applyk_q2<double>(ne, K0d.p, Y.p, cgX.p, cgAd.p, dmask.p, true, st);
    launch_q2_residual_combine<double>(NN, B, cgAd.p, cgR.p, dmask.p, st);
    launch_masked_dot_partials<double, double>(gq, cgR.p, cgR.p, cgPart.p, st);
    launch_finalize(cgPart.p, REDUCE_BLOCKS, cgSc.p + 5, st);
    launch_cg_init(cgSc.p, tol * tol, (double)maxIter, st);
    launch_fill<double>(cgD.p, 0.0, n3, st);
    VFEM_CUDA(cudaMemcpyAsync(cgHost, cgSc.p, 16 * sizeof(double), cudaMemcpyDeviceToHost, st));
    VFEM_CUDA(cudaStreamSynchronize(st));
    PcgStats stats;
    stats.bnorm2 = cgHost[7];
    double rsq = cgHost[5];
    if (std::isnan(rsq)) throw Error(ERR_NAN, "NaN encountered");
    int64_t it = 0;
    while (it < maxIter && rsq > tol * tol * stats.bnorm2) {
        precondition(cgR.p, sweeps);
        launch_cg_precond_out<float>(gq, work<float>().x.p, cgS.p, cgR.p, dmask.p, cgPart.p, st);
        launch_cg_beta(cgPart.p, REDUCE_BLOCKS, cgSc.p, st);
        launch_cg_direction(gq, cgS.p, cgD.p, cgSc.p, nullptr, nullptr, st);
        if (outerDF) applyDF(cgD.p, cgAd.p, true, st);
        else launch_applyk_q2<double>(ne, K0d.p, Y.p, cgD.p, cgAd.p, dmask.p, true, st);
        launch_masked_dot_partials<double, double>(gq, cgD.p, cgAd.p, cgPart.p, st);
        launch_cg_alpha(cgPart.p, REDUCE_BLOCKS, cgSc.p, st);
        launch_cg_update(gq, cgX.p, cgR.p, cgD.p, cgAd.p, cgSc.p, cgPart.p, st);
        launch_cg_rsq(cgPart.p, REDUCE_BLOCKS, cgSc.p, nullptr, st);
        VFEM_CUDA(cudaMemcpyAsync(cgHost, cgSc.p, 16 * sizeof(double), cudaMemcpyDeviceToHost, st));
        VFEM_CUDA(cudaStreamSynchronize(st));
        rsq = cgHost[5];
        ++it;
        if (std::isnan(rsq)) throw Error(ERR_NAN, "NaN encountered at iteration" + std::to_string(it));
    }
    VFEM_CUDA(cudaMemcpyAsync(vx.d, cgX.p, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
    finishOut(vx, st);
    VFEM_CUDA(cudaStreamSynchronize(st));
    stats.iterations = it;
    stats.rsq = rsq;
    stats.relres = stats.bnorm2 > 0 ? std::sqrt(rsq / stats.bnorm2) : std::sqrt(rsq);
    return stats;
}

void q2Restrict(const int neFine[3], const double *fine, double *coarse) {
    for (int d = 0; d < 3; ++d)
        if (neFine[d] % 2) throw Error(ERR_ARG, "Grid size must be divisible by 2 for a coarsening");
    const int64_t nf = (int64_t)(2 * neFine[0] + 1) * (2 * neFine[1] + 1) * (2 * neFine[2] + 1);
    const int64_t nc = (int64_t)(neFine[0] + 1) * (neFine[1] + 1) * (neFine[2] + 1);
    View vf, vc;
    viewIn(vf, fine, 3 * nf * sizeof(double), 0);
    viewOut(vc, coarse, 3 * nc * sizeof(double));
    launch_restrict_q2<double>(neFine, (const double *)vf.d, (double *)vc.d, 0);
    finishOut(vc, 0);
    VFEM_CUDA(cudaDeviceSynchronize());
}

void q2Interpolate(const int neFine[3], const double *coarse, double *fine, bool accumulate) {
    for (int d = 0; d < 3; ++d)
        if (neFine[d] % 2) throw Error(ERR_ARG, "Grid size must be divisible by 2 for a coarsening");
    const int64_t nf = (int64_t)(2 * neFine[0] + 1) * (2 * neFine[1] + 1) * (2 * neFine[2] + 1);
    const int64_t nc = (int64_t)(neFine[0] + 1) * (neFine[1] + 1) * (neFine[2] + 1);
    View vc, vf;
    viewIn(vc, coarse, 3 * nc * sizeof(double), 0);
    viewInOut(vf, fine, 3 * nf * sizeof(double), 0);
    launch_interp_q2<double>(neFine, (const double *)vc.d, (double *)vf.d, accumulate, 0);
    finishOut(vf, 0);
    VFEM_CUDA(cudaDeviceSynchronize());
}

}  // namespace vfem
