// Triquadratic voxel grid (TensorProductSimulator<Real, 2, 2, 2>, TPSStencils.hh:135-186): the
// element stiffness, SIMP moduli, zero-displacement supports, the matrix-free applyK and the
// 27-colour block Gauss-Seidel sweep of the reference's generic (Q2) multigrid smoother
// (MultigridSolver.hh:277-321, 409-442), in FP64 or FP32, and timing hooks.
#include "vfem_engine.hpp"

#include <cstring>
#include <type_traits>

#include "vfem_element.hpp"

namespace vfem {

// 1-D coarse Q2 shape function lc (0, 1, 2 on the reference nodes 0, 1/2, 1) at x
static double q2Lagrange(int lc, double x) {
    return lc == 0 ? 2 * (x - 0.5) * (x - 1.0) : (lc == 1 ? -4 * x * (x - 1.0) : 2 * x * (x - 0.5));
}

// phi_f(i, j): coarse shape function j at local node i of child f = 4 fx + 2 fy + fz, which lies
// at coarse reference coordinates ((2 fx + a) / 4, ...) for i = 9 a + 3 b + c
// (getCompressedElementInterpolationOperator, MultigridSolver.hh:664-687)
static double q2ChildPhi(int f, int i, int j) {
    const int fd[3] = {f >> 2 & 1, f >> 1 & 1, f & 1};
    const int ia[3] = {i / 9, (i / 3) % 3, i % 3}, ja[3] = {j / 9, (j / 3) % 3, j % 3};
    double v = 1.0;
    for (int d = 0; d < 3; ++d) v *= q2Lagrange(ja[d], 0.25 * (2 * fd[d] + ia[d]));
    return v;
}

// Kc[f] = I_f^T K0 I_f for the 8 children (coarsenedFineK0s, MultigridSolver.hh:106-119, 712-722)
void q2CoarsenedK0(const double *K0, std::vector<double> &Kc) {
    Kc.assign(8 * 6561, 0.0);
    std::vector<double> T(6561);
    for (int f = 0; f < 8; ++f) {
        double phi[27 * 27];
        for (int i = 0; i < 27; ++i)
            for (int j = 0; j < 27; ++j) phi[27 * i + j] = q2ChildPhi(f, i, j);
        for (int r = 0; r < 81; ++r)
            for (int j = 0; j < 27; ++j)
                for (int d = 0; d < 3; ++d) {
                    double acc = 0.0;
                    for (int i = 0; i < 27; ++i) acc += K0[81 * r + 3 * i + d] * phi[27 * i + j];
                    T[81 * r + 3 * j + d] = acc;
                }
        double *out = Kc.data() + 6561 * f;
        for (int j = 0; j < 27; ++j)
            for (int c = 0; c < 3; ++c)
                for (int q = 0; q < 81; ++q) {
                    double acc = 0.0;
                    for (int i = 0; i < 27; ++i) acc += phi[27 * i + j] * T[81 * (3 * i + c) + q];
                    out[81 * (3 * j + c) + q] = acc;
                }
    }
}

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
    q2CoarsenedK0(K0.data(), Kc);
    ++version;
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
    ++version;
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
    ++version;
    qCoarsenings = -1;  // the coarsened supports and the coarsest free DOFs change
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

// ---- the triquadratic multigrid hierarchy (MultigridSolver<double, 2, 2, 2>) ----

void GridQ2::setHierarchy(int kind) {
    if (kind != Q2_HIER_Q2 && kind != Q2_HIER_P) throw Error(ERR_ARG, "unknown triquadratic hierarchy");
    hierarchy = kind;
}

void GridQ2::setPrecision(int precision) {
    if (precision != PREC_FP64 && precision != PREC_MIXED) throw Error(ERR_ARG, "precision must be fp64 or mixed");
    vprecision = precision;
    outerDF = precision == PREC_MIXED;
}

// Levels, coarsened supports and the coarsest free DOFs for `coarsenings` coarsenings, then the
// element matrices and the coarsest inverse in `precision` whenever the moduli, K0 or the
// supports changed (MultigridSolver.hh:35-121, 846-905).
void GridQ2::prepareHierarchy(int coarsenings, int precision) {
    if (coarsenings < 1) throw Error(ERR_ARG, "the triquadratic hierarchy needs at least one coarsening");
    if (qCoarsenings != coarsenings) {
        for (int d = 0; d < 3; ++d)
            if (ne[d] % (1 << coarsenings))
                throw Error(ERR_ARG, "Grid size currently must be divisible by 2^numCoarseningLevels (nonuniform coarsening not yet implemented)");
        qCoarsenings = -1;
        qlv.clear();
        qlv.resize(coarsenings);
        const std::vector<uint8_t> *fm = &dmask_h;
        const int *fne = ne;
        for (int l = 1; l <= coarsenings; ++l) {
            Q2Level &C = qlv[l - 1];
            for (int d = 0; d < 3; ++d) C.ne[d] = fne[d] / 2;
            const int cn[3] = {2 * C.ne[0] + 1, 2 * C.ne[1] + 1, 2 * C.ne[2] + 1};
            const int fn[3] = {2 * fne[0] + 1, 2 * fne[1] + 1, 2 * fne[2] + 1};
            C.NN = (int64_t)cn[0] * cn[1] * cn[2];
            C.NE = (int64_t)C.ne[0] * C.ne[1] * C.ne[2];
            // a constrained fine node marks the coarse nodes of the vertex, edge or face of its
            // coarse element on which it lies, every node along an axis where it is interior
            // (MultigridSolver.hh:57-104)
            C.dmask_h.assign(C.NN, 0);
            for (int I = 0; I < fn[0]; ++I)
                for (int J = 0; J < fn[1]; ++J)
                    for (int K = 0; K < fn[2]; ++K) {
                        const uint8_t m = (*fm)[((int64_t)I * fn[1] + J) * fn[2] + K];
                        if (!m) continue;
                        const int P[3] = {I, J, K};
                        int ec[3], pb[3];
                        for (int d = 0; d < 3; ++d) {
                            ec[d] = std::min(P[d] / 4, C.ne[d] - 1);
                            const int t = P[d] - 4 * ec[d];
                            pb[d] = t == 0 ? 0 : (t == 4 ? 2 : -1);
                        }
                        for (int ln = 0; ln < 27; ++ln) {
                            const int la[3] = {ln / 9, (ln / 3) % 3, ln % 3};
                            if ((pb[0] >= 0 && pb[0] != la[0]) || (pb[1] >= 0 && pb[1] != la[1]) ||
                                (pb[2] >= 0 && pb[2] != la[2]))
                                continue;
                            C.dmask_h[((int64_t)(2 * ec[0] + la[0]) * cn[1] + 2 * ec[1] + la[1]) * cn[2] + 2 * ec[2] + la[2]] |= m;
                        }
                    }
            C.dmask.alloc(C.NN);
            VFEM_CUDA(cudaMemcpyAsync(C.dmask.p, C.dmask_h.data(), C.NN, cudaMemcpyHostToDevice, stream));
            fm = &C.dmask_h;
            fne = C.ne;
        }
        // free DOFs (3 n + c) of the coarsest level, solved directly
        const Q2Level &C = qlv.back();
        std::vector<int> red(3 * C.NN, -1), fr;
        for (int64_t n = 0; n < C.NN; ++n)
            for (int c = 0; c < 3; ++c)
                if (!((C.dmask_h[n] >> c) & 1)) {
                    red[3 * n + c] = (int)fr.size();
                    fr.push_back((int)(3 * n + c));
                }
        if (fr.size() > 30000) throw Error(ERR_ARG, "coarsest level too large for the dense direct solve; use more coarsening levels");
        qNfree = (int)fr.size();
        const int cap = std::max(qNfree, 1);
        qFreeIdx.alloc(cap);
        qRedIdx.alloc(red.size());
        qNfreeDev.alloc(1);
        qStatus.alloc(1);
        qAinv.alloc((size_t)cap * cap);
        qWork.alloc(dense_inverse_work_size(cap));
        qScratch.alloc(cap);
        if (qNfree) VFEM_CUDA(cudaMemcpyAsync(qFreeIdx.p, fr.data(), fr.size() * sizeof(int), cudaMemcpyHostToDevice, stream));
        VFEM_CUDA(cudaMemcpyAsync(qRedIdx.p, red.data(), red.size() * sizeof(int), cudaMemcpyHostToDevice, stream));
        VFEM_CUDA(cudaMemcpyAsync(qNfreeDev.p, &qNfree, sizeof(int), cudaMemcpyHostToDevice, stream));
        VFEM_CUDA(cudaStreamSynchronize(stream));
        qCoarsenings = coarsenings;
        qVersion = 0;
    }
    if (qVersion != version || qPrecision != precision) {
        if (precision == PREC_FP64) buildHierarchyT<double>();
        else buildHierarchyT<float>();
        qVersion = version;
        qPrecision = precision;
    }
}

template <typename T>
static DevBuf<T> &keBuf(Q2Level &C);
template <>
DevBuf<double> &keBuf<double>(Q2Level &C) { return C.Ke64; }
template <>
DevBuf<float> &keBuf<float>(Q2Level &C) { return C.Ke32; }

// Level 1 from the coarsened full-density matrices and the fine moduli, each level below from
// the one above (MultigridSolver.hh:745-819), then the reduced coarsest operator and its FP64
// inverse. The element matrices of the other precision are released.
template <typename T>
void GridQ2::buildHierarchyT() {
    cudaStream_t st = stream;
    DevBuf<T> *kcp;
    if constexpr (std::is_same<T, double>::value) kcp = &Kc64;
    else kcp = &Kc32;
    DevBuf<T> &KcT = *kcp;
    KcT.alloc(8 * 6561);
    std::vector<T> kc(Kc.begin(), Kc.end());
    VFEM_CUDA(cudaMemcpyAsync(KcT.p, kc.data(), kc.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    const T *Yt = std::is_same<T, double>::value ? (const T *)Y.p : (const T *)Yf.p;
    for (int l = 1; l <= qCoarsenings; ++l) {
        Q2Level &C = qlv[l - 1];
        if constexpr (std::is_same<T, double>::value) C.Ke32 = DevBuf<float>();
        else C.Ke64 = DevBuf<double>();
        DevBuf<T> &Ke = keBuf<T>(C);
        // one zero matrix after the last element: the level kernels' out-of-grid incidences read it
        Ke.alloc((C.NE + 1) * 6561);
        VFEM_CUDA(cudaMemsetAsync(Ke.p + C.NE * 6561, 0, 6561 * sizeof(T), st));
        if (l == 1) launch_q2mg_level1<T>(C.ne, KcT.p, Yt, Ke.p, st);
        else launch_q2mg_galerkin<T>(C.ne, keBuf<T>(qlv[l - 2]).p, Ke.p, st);
    }
    Q2Level &C = qlv.back();
    if (qNfree > 0) {
        launch_q2mg_dense<T>(C.ne, keBuf<T>(C).p, qFreeIdx.p, qRedIdx.p, qNfree, qAinv.p, st);
        launch_symmetrize(qAinv.p, qNfree, st);
        VFEM_CUDA(cudaMemsetAsync(qStatus.p, 0, sizeof(int), st));
        dense_spd_inverse(qAinv.p, qWork.p, qNfree, qStatus.p, st);
        int status = 0;
        VFEM_CUDA(cudaMemcpyAsync(&status, qStatus.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        VFEM_CUDA(cudaStreamSynchronize(st));
        if (status) {
            qVersion = 0;
            check_dense_status(status);
        }
    }
    VFEM_CUDA(cudaStreamSynchronize(st));
}

template <typename T>
LevelData<T> &GridQ2::qwork(int l) {
    if (l == 0) return work<T>();
    Q2Level &C = qlv[l - 1];
    LevelData<T> *D;
    if constexpr (std::is_same<T, double>::value) D = &C.w64;
    else D = &C.w32;
    allocWork(*D, 3 * C.NN);
    return *D;
}

template <typename T>
const T *GridQ2::qKe(int l) {
    return keBuf<T>(qlv[l - 1]).p;
}

// Level 0 runs the matrix-free fine kernels (for FP32 with K0 in constant memory, uploaded by
// the caller), the levels below the element-matrix kernels.
template <typename T>
void GridQ2::qSmoothT(int l, T *u, const T *b, bool forward) {
    if (l == 0) {
        const T *Yt = std::is_same<T, double>::value ? (const T *)Y.p : (const T *)Yf.p;
        const T *K = std::is_same<T, double>::value ? (const T *)K0d.p : nullptr;
        launch_gs_q2_sweep<T>(ne, K, Yt, u, b, dmask.p, forward, stream);
    } else {
        launch_q2mg_gs_sweep<T>(qlv[l - 1].ne, qKe<T>(l), u, b, qlv[l - 1].dmask.p, forward, stream);
    }
}

template <typename T>
void GridQ2::qResidualT(int l, const T *u, const T *b, T *r) {
    if (l == 0) {
        const T *Yt = std::is_same<T, double>::value ? (const T *)Y.p : (const T *)Yf.p;
        const T *K = std::is_same<T, double>::value ? (const T *)K0d.p : nullptr;
        launch_applyk_q2<T>(ne, K, Yt, u, r, dmask.p, false, stream);
        launch_q2_residual_combine<T>(NN, b, r, r, dmask.p, stream);
    } else {
        launch_q2mg_apply<T>(qlv[l - 1].ne, qKe<T>(l), u, b, r, qlv[l - 1].dmask.p, true, stream);
    }
}

template <typename T>
void GridQ2::qCoarseSolveT(const T *b, T *x) {
    const int *nl = qlv.back().ne;
    const int n2[3] = {2 * nl[0], 2 * nl[1], 2 * nl[2]};
    launch_coarse_solve<T>(makeGeom(n2), qAinv.p, qFreeIdx.p, qNfreeDev.p, qNfree, b, x, qScratch.p, stream);
}

// MultigridSolver.hh:617-658 on a residual system (zero Dirichlet values)
template <typename T>
void GridQ2::vcycleQ2T(int l, int64_t sweeps) {
    LevelData<T> &D = qwork<T>(l);
    if (l == qCoarsenings) {
        qCoarseSolveT<T>(D.b.p, D.x.p);
        return;
    }
    const int *nl = levelNe(l);
    const int n2[3] = {2 * nl[0], 2 * nl[1], 2 * nl[2]};
    launch_zero_dirichlet<T>(makeGeom(n2), D.x.p, levelMask(l), stream);
    for (int64_t s = 0; s < sweeps; ++s) qSmoothT<T>(l, D.x.p, D.b.p, true);
    qResidualT<T>(l, D.x.p, D.b.p, D.r.p);
    LevelData<T> &Cd = qwork<T>(l + 1);
    launch_restrict_q2<T>(nl, D.r.p, Cd.b.p, stream);
    launch_fill<T>(Cd.x.p, T(0), 3 * levelNN(l + 1), stream);
    vcycleQ2T<T>(l + 1, sweeps);
    launch_interp_q2<T>(nl, Cd.x.p, D.x.p, true, stream);
    for (int64_t s = 0; s < sweeps; ++s) qSmoothT<T>(l, D.x.p, D.b.p, !symmetricGS);
}

// qwork<T>(0).x = one V-cycle from zero on the right-hand side r (device FP64)
template <typename T>
void GridQ2::preconditionQ2T(const double *r, int64_t sweeps) {
    LevelData<T> &D = qwork<T>(0);
    toT<T>(r, D.b.p, 3 * NN, stream);
    launch_fill<T>(D.x.p, T(0), 3 * NN, stream);
    if (std::is_same<T, float>::value) q2_upload_k0f(K0f.data(), stream);  // constant memory is shared by every Q2 grid
    vcycleQ2T<T>(0, sweeps);
}

int64_t GridQ2::mgLevelNodes(int coarsenings, int l) {
    prepareHierarchy(coarsenings, vprecision);
    if (l < 0 || l > coarsenings) throw Error(ERR_ARG, "level out of range");
    return levelNN(l);
}

void GridQ2::mgLevelDirichlet(int coarsenings, int l, uint8_t *out) {
    const int64_t n = mgLevelNodes(coarsenings, l);
    const std::vector<uint8_t> &m = l == 0 ? dmask_h : qlv[l - 1].dmask_h;
    std::memcpy(out, m.data(), n);
}

void GridQ2::mgLevelKe(int coarsenings, int l, int precision, double *out) {
    prepareHierarchy(coarsenings, precision);
    if (l < 1 || l > coarsenings) throw Error(ERR_ARG, "element matrices exist on levels 1..coarsenings");
    const int64_t n = qlv[l - 1].NE * 6561;
    View vo;
    viewOut(vo, out, n * sizeof(double));
    if (precision == PREC_FP64) VFEM_CUDA(cudaMemcpyAsync(vo.d, qKe<double>(l), n * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    else fromT<float>(qKe<float>(l), (double *)vo.d, n, stream);
    finishOut(vo, stream);
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

void GridQ2::mgSmooth(int coarsenings, int l, double *u, const double *b, bool forward, int precision) {
    const int64_t n3 = 3 * mgLevelNodes(coarsenings, l);
    prepareHierarchy(coarsenings, precision);
    View vu, vb;
    viewInOut(vu, u, n3 * sizeof(double), stream);
    viewIn(vb, b, n3 * sizeof(double), stream);
    auto run = [&](auto tag) {
        using T = decltype(tag);
        LevelData<T> &D = qwork<T>(l);
        toT<T>((const double *)vu.d, D.x.p, n3, stream);
        toT<T>((const double *)vb.d, D.b.p, n3, stream);
        if (std::is_same<T, float>::value) q2_upload_k0f(K0f.data(), stream);
        qSmoothT<T>(l, D.x.p, D.b.p, forward);
        fromT<T>(D.x.p, (double *)vu.d, n3, stream);
    };
    if (precision == PREC_FP64) run(double());
    else run(float());
    finishOut(vu, stream);
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

void GridQ2::mgResidual(int coarsenings, int l, const double *u, const double *b, double *r, int precision) {
    const int64_t n3 = 3 * mgLevelNodes(coarsenings, l);
    prepareHierarchy(coarsenings, precision);
    View vu, vb, vr;
    viewIn(vu, u, n3 * sizeof(double), stream);
    viewIn(vb, b, n3 * sizeof(double), stream);
    viewOut(vr, r, n3 * sizeof(double));
    auto run = [&](auto tag) {
        using T = decltype(tag);
        LevelData<T> &D = qwork<T>(l);
        toT<T>((const double *)vu.d, D.x.p, n3, stream);
        toT<T>((const double *)vb.d, D.b.p, n3, stream);
        if (std::is_same<T, float>::value) q2_upload_k0f(K0f.data(), stream);
        qResidualT<T>(l, D.x.p, D.b.p, D.r.p);
        fromT<T>(D.r.p, (double *)vr.d, n3, stream);
    };
    if (precision == PREC_FP64) run(double());
    else run(float());
    finishOut(vr, stream);
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

void GridQ2::mgCoarseSolve(int coarsenings, const double *b, double *x, int precision) {
    const int64_t n3 = 3 * mgLevelNodes(coarsenings, coarsenings);
    prepareHierarchy(coarsenings, precision);
    View vb, vx;
    viewIn(vb, b, n3 * sizeof(double), stream);
    viewOut(vx, x, n3 * sizeof(double));
    auto run = [&](auto tag) {
        using T = decltype(tag);
        LevelData<T> &D = qwork<T>(coarsenings);
        toT<T>((const double *)vb.d, D.b.p, n3, stream);
        qCoarseSolveT<T>(D.b.p, D.x.p);
        fromT<T>(D.x.p, (double *)vx.d, n3, stream);
    };
    if (precision == PREC_FP64) run(double());
    else run(float());
    finishOut(vx, stream);
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

void GridQ2::mgVcycle(int coarsenings, const double *b, double *x, int64_t sweeps, int precision) {
    prepareHierarchy(coarsenings, precision);
    const int64_t n3 = 3 * NN;
    View vb, vx;
    viewIn(vb, b, n3 * sizeof(double), stream);
    viewOut(vx, x, n3 * sizeof(double));
    if (precision == PREC_FP64) {
        preconditionQ2T<double>((const double *)vb.d, sweeps);
        fromT<double>(qwork<double>(0).x.p, (double *)vx.d, n3, stream);
    } else {
        preconditionQ2T<float>((const double *)vb.d, sweeps);
        fromT<float>(qwork<float>(0).x.p, (double *)vx.d, n3, stream);
    }
    finishOut(vx, stream);
    VFEM_CUDA(cudaStreamSynchronize(stream));
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
// direction) with the Q2 operator and one V-cycle of the chosen hierarchy as the preconditioner.
PcgStats GridQ2::pcg(double *x, const double *b, int64_t maxIter, double tol, int coarsenings, int64_t sweeps) {
    if (coarsenings < 1) throw Error(ERR_ARG, "the Q2 preconditioner needs at least one coarsening");
    VFEM_CUDA(cudaStreamSynchronize(stream));
    const bool pmg = hierarchy == Q2_HIER_P;
    if (pmg) {
        if (vprecision != PREC_MIXED) throw Error(ERR_ARG, "the p-multigrid preconditioner runs in mixed precision only");
        prepareQ1(coarsenings);
    } else {
        prepareHierarchy(coarsenings, vprecision);
    }
    cudaStream_t st = pmg ? q1->stream : stream;
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
        if (pmg) {
            precondition(cgR.p, sweeps);
            launch_cg_precond_out<float>(gq, work<float>().x.p, cgS.p, cgR.p, dmask.p, cgPart.p, st);
        } else if (vprecision == PREC_FP64) {
            preconditionQ2T<double>(cgR.p, sweeps);
            launch_cg_precond_out<double>(gq, work<double>().x.p, cgS.p, cgR.p, dmask.p, cgPart.p, st);
        } else {
            preconditionQ2T<float>(cgR.p, sweeps);
            launch_cg_precond_out<float>(gq, work<float>().x.p, cgS.p, cgR.p, dmask.p, cgPart.p, st);
        }
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
