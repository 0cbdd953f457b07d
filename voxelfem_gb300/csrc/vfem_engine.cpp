// Host engine: grid state, multigrid hierarchy, MG-preconditioned CG and the
// topology-optimisation problem. See vfem_engine.hpp.
#include "vfem_engine.hpp"

#include <cstdlib>

#include <algorithm>
#include <cstring>

#include "vfem_element.hpp"

namespace vfem {

uint64_t &launchCounter() {
    static uint64_t counter = 0;
    return counter;
}

bool pdlEnabled() {
    static const bool on = [] {
        const char *env = std::getenv("VFEM_PDL");
        return !(env && env[0] == '0');
    }();
    return on;
}

// ---------------------------------------------------------------------------
// caller-memory views
// ---------------------------------------------------------------------------
bool isDevicePtr(const void *p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

void viewIn(View &v, const void *p, size_t bytes, cudaStream_t st) {
    if (!p && bytes) throw Error(ERR_ARG, "null input pointer");
    v.user = const_cast<void *>(p);
    v.bytes = bytes;
    if (isDevicePtr(p)) {
        v.d = const_cast<void *>(p);
        v.staged = false;
    } else {
        v.tmp.alloc(bytes);
        v.d = v.tmp.p;
        v.staged = true;
        if (bytes) VFEM_CUDA(cudaMemcpyAsync(v.d, p, bytes, cudaMemcpyHostToDevice, st));
    }
}

void viewOut(View &v, void *p, size_t bytes) {
    if (!p && bytes) throw Error(ERR_ARG, "null output pointer");
    v.user = p;
    v.bytes = bytes;
    if (isDevicePtr(p)) {
        v.d = p;
        v.staged = false;
    } else {
        v.tmp.alloc(bytes);
        v.d = v.tmp.p;
        v.staged = true;
    }
}

void viewInOut(View &v, void *p, size_t bytes, cudaStream_t st) {
    viewIn(v, p, bytes, st);
}

void finishOut(View &v, cudaStream_t st) {
    if (v.staged && v.bytes) VFEM_CUDA(cudaMemcpyAsync(v.user, v.d, v.bytes, cudaMemcpyDeviceToHost, st));
    VFEM_CUDA(cudaStreamSynchronize(st));
}

// ---------------------------------------------------------------------------
// Grid (TensorProductSimulator<double, 1, 1, 1>)
// ---------------------------------------------------------------------------
Grid::Grid(const int ne[3], const double bmin_[3], const double bmax_[3]) {
    for (int d = 0; d < 3; ++d) {
        if (ne[d] <= 0) throw Error(ERR_ARG, "elementsPerDimension must be positive");
        if (!(bmax_[d] > bmin_[d])) throw Error(ERR_ARG, "invalid domain bounding box");
        bmin[d] = bmin_[d];
        bmax[d] = bmax_[d];
        h[d] = (bmax[d] - bmin[d]) / ne[d];
    }
    g = makeGeom(ne);
    // device index decodes are 32-bit
    if (3 * g.NN >= (int64_t(1) << 31) || g.NE >= (int64_t(1) << 31)) throw Error(ERR_ARG, "grid too large");
    VFEM_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    rho.alloc(g.NE);
    Y.alloc(g.NE);
    VFEM_CUDA(cudaMemsetAsync(rho.p, 0, rho.bytes(), stream));  // NDVector zero-initialises densities
    dmask_h.assign(g.NN, 0);
    dval_h.assign(3 * g.NN, 0.0);
    force_h.assign(3 * g.NN, 0.0);
    dmask.alloc(g.NN);
    dval.alloc(3 * g.NN);
    dynMask.alloc(2);
    g.dyn = dynMask.p;
    uploadMask();
    uploadBC();
    setETensor(1.0, 0.0);
    updateYoungModuli();
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

Grid::~Grid() {
    if (stream) cudaStreamDestroy(stream);
}

void Grid::setETensor(double E, double nu_) {
    if (!(nu_ < 0.5) || !(nu_ > -1.0)) throw Error(ERR_ARG, "Poisson ratio must lie in (-1, 0.5)");
    Eyoung = E;
    nu = nu_;
    element_stiffness(E, nu, h, K0.a);
    ++k0Version;
    for (int t = 0; t < 576; ++t) {
        K0f.a[t] = (float)K0.a[t];
        K0df.hi[t] = (float)K0.a[t];
        K0df.lo[t] = (float)(K0.a[t] - (double)K0df.hi[t]);
    }
    tcTiles.assign(2048, 0);
    tcOk = tc_fit_k0(K0.a, &tcScale, tcTiles.data());
    if (tcOk) {
        tcB.alloc(2048);
        VFEM_CUDA(cudaMemcpy(tcB.p, tcTiles.data(), 2048 * sizeof(uint16_t), cudaMemcpyHostToDevice));
    }
    if (!tcStatus.p) {
        tcStatus.alloc(1);
        VFEM_CUDA(cudaMemset(tcStatus.p, 0, sizeof(int)));
    }
    double kv[10];
    const bool cube = k0_cube_values(K0.a, kv);
    K0.isCube = K0f.isCube = K0df.isCube = cube ? 1 : 0;
    for (int c = 0; c < 10; ++c) {
        K0.cube[c] = cube ? kv[c] : 0.0;
        K0f.cube[c] = (float)K0.cube[c];
        K0df.cubeHi[c] = (float)K0.cube[c];
        K0df.cubeLo[c] = (float)(K0.cube[c] - (double)K0df.cubeHi[c]);
    }
    ++densVersion;  // stiffness depends on K0
    ++materialVersion;
}

void Grid::setParams(double E0_, double Emin_, double gamma_, double q_, int law_) {
    E0 = E0_;
    Emin = Emin_;
    gamma = gamma_;
    q = q_;
    law = law_;
    updateYoungModuli();
}

void Grid::updateYoungModuli(bool maskOnly) {
    const bool masking = maskH < bmax[BUILD_DIR];
    launch_young_moduli<double>(g, rho.p, Y.p, E0, Emin, gamma, q, law, masking, stream);
    YfValid = false;
    YfpValid = false;
    YdfValid = false;
    ++densVersion;
    if (!maskOnly) ++materialVersion;
}

void Grid::youngDF(const float **hi, const float **lo) {
    if (!YdfValid) {
        Yhi.alloc(g.padNE());
        Ylo.alloc(g.padNE());
        launch_pad_young(g, Y.p, Yhi.p, Ylo.p, stream);
        YdfValid = true;
    }
    *hi = Yhi.p;
    *lo = Ylo.p;
}

const float *Grid::youngFPad() {
    if (!YfpValid) {
        Yfp.alloc(g.padNE());
        launch_pad_young(g, Y.p, Yfp.p, nullptr, stream);
        YfpValid = true;
    }
    return Yfp.p;
}

const float *Grid::youngF() {
    if (!YfValid) {
        Yf.alloc(g.NE);
        // the FP32 moduli are the rounded FP64 ones
        launch_cast<float, double>(Y.p, Yf.p, g.NE, stream);
        YfValid = true;
    }
    return Yf.p;
}

void Grid::setDensities(const double *r, bool checkRange) {
    if (checkRange) {
        std::vector<double> hostCopy(g.NE);
        if (isDevicePtr(r)) VFEM_CUDA(cudaMemcpy(hostCopy.data(), r, g.NE * sizeof(double), cudaMemcpyDeviceToHost));
        else std::memcpy(hostCopy.data(), r, g.NE * sizeof(double));
        for (double v : hostCopy)
            if (v > 1.0 || v < 0.0) throw Error(ERR_ARG, "Density value has to be in between 0 and 1");
    }
    VFEM_CUDA(cudaMemcpyAsync(rho.p, r, g.NE * sizeof(double), cudaMemcpyDefault, stream));
    updateYoungModuli();
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

void Grid::setUniformDensities(double v) {
    if (v > 1.0 || v < 0.0) throw Error(ERR_ARG, "Density value has to be in between 0 and 1");
    std::vector<double> hv(g.NE, v);
    VFEM_CUDA(cudaMemcpyAsync(rho.p, hv.data(), g.NE * sizeof(double), cudaMemcpyHostToDevice, stream));
    updateYoungModuli();
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

void Grid::getDensities(double *out) {
    VFEM_CUDA(cudaMemcpyAsync(out, rho.p, g.NE * sizeof(double), cudaMemcpyDefault, stream));
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

void Grid::getYoungModuli(double *out) {
    VFEM_CUDA(cudaMemcpyAsync(out, Y.p, g.NE * sizeof(double), cudaMemcpyDefault, stream));
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

void Grid::uploadBC() {
    VFEM_CUDA(cudaMemcpyAsync(dmask.p, dmask_h.data(), g.NN, cudaMemcpyHostToDevice, stream));
    VFEM_CUDA(cudaMemcpyAsync(dval.p, dval_h.data(), 3 * g.NN * sizeof(double), cudaMemcpyHostToDevice, stream));
    VFEM_CUDA(cudaStreamSynchronize(stream));
    dvalNonzero = std::any_of(dval_h.begin(), dval_h.end(), [](double v) { return v != 0.0; });
    ++bcVersion;
}

// TensorProductSimulator.hh:241-252 with BCBuilder::setDirichlet (:73-88).
void Grid::addDirichlet(const double u[3], const double mn[3], const double mx[3], unsigned cmask) {
    std::vector<uint8_t> m = dmask_h;
    std::vector<double> v = dval_h;
    const int64_t NN = g.NN;
    for (int i = 0; i < g.nn[0]; ++i) {
        const double px = bmin[0] + i * h[0];
        if (px < mn[0] || px > mx[0]) continue;
        for (int j = 0; j < g.nn[1]; ++j) {
            const double py = bmin[1] + j * h[1];
            if (py < mn[1] || py > mx[1]) continue;
            for (int k = 0; k < g.nn[2]; ++k) {
                const double pz = bmin[2] + k * h[2];
                if (pz < mn[2] || pz > mx[2]) continue;
                const int64_t n = g.node(i, j, k);
                for (int c = 0; c < 3; ++c) {
                    if (!((cmask >> c) & 1)) continue;
                    if (!((m[n] >> c) & 1)) {
                        m[n] |= (uint8_t)(1u << c);
                        v[c * NN + n] = u[c];
                    } else if (std::abs(v[c * NN + n] - u[c]) > 1e-10) {
                        throw Error(ERR_ARG, "Conflicting dirichlet displacements.");
                    }
                }
            }
        }
    }
    dmask_h.swap(m);
    dval_h.swap(v);
    uploadBC();
}

// TensorProductSimulator.hh:2042-2053
void Grid::applySymmetry(const int axes[3], const int maxFace[3]) {
    for (int64_t n = 0; n < g.NN; ++n) {
        const int k = (int)(n % g.nn[2]);
        const int j = (int)((n / g.nn[2]) % g.nn[1]);
        const int i = (int)(n / ((int64_t)g.nn[1] * g.nn[2]));
        const int idx[3] = {i, j, k};
        for (int d = 0; d < 3; ++d) {
            if (!axes[d]) continue;
            const double p = bmin[d] + idx[d] * h[d];
            if (std::abs(p - (maxFace[d] ? bmax[d] : bmin[d])) < 1e-10) {
                dmask_h[n] |= (uint8_t)(1u << d);
                dval_h[d * g.NN + n] = 0.0;
            }
        }
    }
    uploadBC();
}

void Grid::setForces(const double *f) {
    forceDevValid = false;
    if (isDevicePtr(f)) VFEM_CUDA(cudaMemcpy(force_h.data(), f, 3 * g.NN * sizeof(double), cudaMemcpyDeviceToHost));
    else std::memcpy(force_h.data(), f, 3 * g.NN * sizeof(double));
}

void Grid::getDirichletMask(uint8_t *out) const {
    if (isDevicePtr(out)) VFEM_CUDA(cudaMemcpy(out, dmask_h.data(), g.NN, cudaMemcpyHostToDevice));
    else std::memcpy(out, dmask_h.data(), g.NN);
}

void Grid::setGravity(const double gv[3]) {
    for (int c = 0; c < 3; ++c) grav[c] = gv[c];
}

// TensorProductSimulator.hh:290-303
void Grid::setMaskHeight(double hgt, bool update) {
    if (hgt < 0 || hgt > bmax[BUILD_DIR])
        throw Error(ERR_ARG, "Fabrication height has to be in between 0 and the domain height");
    maskH = hgt;
    const double fl = std::ceil(hgt / h[BUILD_DIR] - 1e-10);
    g.firstMaskedE = (int)fl;
    g.firstDetN = g.firstMaskedE + 1;
    uploadMask();
    ++maskVersion;
    if (update) updateYoungModuli(true);
}

void Grid::uploadMask() { launch_set_pair(dynMask.p, g.firstMaskedE, g.firstDetN, stream); }

void Grid::setMaskLayer(int64_t l) { setMaskHeight(h[BUILD_DIR] * (double)l, true); }

void Grid::applyK(const double *u, double *out) {
    View vu, vo;
    viewIn(vu, u, 3 * g.NN * sizeof(double), stream);
    viewOut(vo, out, 3 * g.NN * sizeof(double));
    launch_applyk_fine<double>(g, Y.p, (const double *)vu.d, (double *)vo.d, K0, true, false, dmask.p, false,
                               nullptr, 0, stream);
    finishOut(vo, stream);
}

void Grid::buildLoadDev(double *f) {
    VFEM_CUDA(cudaMemcpyAsync(f, force_h.data(), 3 * g.NN * sizeof(double), cudaMemcpyHostToDevice, stream));
    if (grav[0] * grav[0] + grav[1] * grav[1] + grav[2] * grav[2] != 0)
        launch_build_gravity_load(g, rho.p, f, grav, vol(), stream);
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

void Grid::buildLoadAsync(double *f) {
    if (!forceDevValid) {
        forceDev.alloc(3 * g.NN);
        VFEM_CUDA(cudaMemcpy(forceDev.p, force_h.data(), 3 * g.NN * sizeof(double), cudaMemcpyHostToDevice));
        forceDevValid = true;
    }
    VFEM_CUDA(cudaMemcpyAsync(f, forceDev.p, 3 * g.NN * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    if (grav[0] * grav[0] + grav[1] * grav[1] + grav[2] * grav[2] != 0)
        launch_build_gravity_load(g, rho.p, f, grav, vol(), stream);
}

std::unique_ptr<Grid> Grid::clone() const {
    auto c = std::make_unique<Grid>(g.ne, bmin, bmax);
    c->setETensor(Eyoung, nu);
    c->E0 = E0;
    c->Emin = Emin;
    c->gamma = gamma;
    c->q = q;
    c->law = law;
    VFEM_CUDA(cudaStreamSynchronize(stream));
    VFEM_CUDA(cudaMemcpy(c->rho.p, rho.p, g.NE * sizeof(double), cudaMemcpyDeviceToDevice));
    c->dmask_h = dmask_h;
    c->dval_h = dval_h;
    c->force_h = force_h;
    c->uploadBC();
    for (int d = 0; d < 3; ++d) c->grav[d] = grav[d];
    if (maskH < std::numeric_limits<double>::infinity()) c->setMaskHeight(maskH, false);
    c->updateYoungModuli();
    VFEM_CUDA(cudaStreamSynchronize(c->stream));
    return c;
}

void Grid::buildLoad(double *out) {
    View vo;
    viewOut(vo, out, 3 * g.NN * sizeof(double));
    buildLoadDev((double *)vo.d);
    finishOut(vo, stream);
}

void Grid::complianceGradient(const double *u, double *out) {
    View vu, vo;
    viewIn(vu, u, 3 * g.NN * sizeof(double), stream);
    viewOut(vo, out, g.NE * sizeof(double));
    launch_compliance_gradient(g, rho.p, (const double *)vu.d, (double *)vo.d, K0, E0, Emin, gamma, q, law, grav,
                               vol(), stream);
    finishOut(vo, stream);
}

void Grid::adjointSensitivity(const double *lam, const double *u, double wF, double wK, double *out) {
    View vl, vu, vo;
    viewIn(vl, lam, 3 * g.NN * sizeof(double), stream);
    viewIn(vu, u, 3 * g.NN * sizeof(double), stream);
    viewOut(vo, out, g.NE * sizeof(double));
    launch_adjoint_sensitivity(g, rho.p, (const double *)vl.d, (const double *)vu.d, (double *)vo.d, K0, E0, Emin,
                               gamma, q, law, grav, vol(), wF, wK, stream);
    finishOut(vo, stream);
}

void Grid::elementEnergy(const double *u, double *out) {
    View vu, vo;
    viewIn(vu, u, 3 * g.NN * sizeof(double), stream);
    viewOut(vo, out, g.NE * sizeof(double));
    launch_element_energy(g, Y.p, (const double *)vu.d, (double *)vo.d, K0, stream);
    finishOut(vo, stream);
}

// ---------------------------------------------------------------------------
// MG (MultigridSolver<double, 1, 1, 1>)
// ---------------------------------------------------------------------------
MG::MG(Grid *fine_, int coarsenings) : fine(fine_) {
    if (coarsenings < 0) throw Error(ERR_ARG, "numCoarseningLevels must be >= 0");
    // Stencil layout switch-over (node count up to which a level keeps node-contiguous rows);
    // VFEM_STENCIL_ROWS_MAX_NODES overrides it (planes measured faster at every level of the
    // 256x128x128 hierarchy, so the default is 0).
    if (const char *env = std::getenv("VFEM_STENCIL_ROWS_MAX_NODES")) rowsMaxNodes = std::atoll(env);
    lv.resize(coarsenings + 1);
    lv[0].g = fine->g;
    for (int d = 0; d < 3; ++d) lv[0].h[d] = fine->h[d];
    int ne[3] = {fine->g.ne[0], fine->g.ne[1], fine->g.ne[2]};
    for (int l = 1; l <= coarsenings; ++l) {
        for (int d = 0; d < 3; ++d) {
            if (ne[d] % 2 == 1)
                throw Error(ERR_ARG,
                            "Grid size currently must be divisible by 2^numCoarseningLevels (nonuniform coarsening "
                            "not yet implemented)");
            ne[d] /= 2;
        }
        lv[l].g = makeGeom(ne);
        for (int d = 0; d < 3; ++d) lv[l].h[d] = (fine->bmax[d] - fine->bmin[d]) / ne[d];
    }
    lv[0].dmask_h = fine->dmask_h;
    coarsenDirichlet();
    for (int l = 1; l < L(); ++l) {
        lv[l].dmask.alloc(lv[l].g.NN);
        VFEM_CUDA(cudaMemcpy(lv[l].dmask.p, lv[l].dmask_h.data(), lv[l].g.NN, cudaMemcpyHostToDevice));
        lv[l].dyn.alloc(2);
        lv[l].g.dyn = lv[l].dyn.p;
    }
    // propagate an existing fabrication mask (MultigridSolver.hh:1022-1028)
    if (fine->maskH < std::numeric_limits<double>::infinity()) {
        for (int l = 1; l < L(); ++l) {
            const double fl = std::ceil(fine->maskH / lv[l].h[BUILD_DIR] - 1e-10);
            lv[l].g.firstMaskedE = (int)fl;
            lv[l].g.firstDetN = lv[l].g.firstMaskedE + 1;
        }
    }
    for (int l = 1; l < L(); ++l) launch_set_pair(lv[l].dyn.p, lv[l].g.firstMaskedE, lv[l].g.firstDetN, fine->stream);
    nfreeDev.alloc(1);
    const int64_t NN = fine->g.NN;
    rbuf.alloc(3 * NN);
    s.alloc(3 * NN);
    dvec.alloc(3 * NN);
    Ad.alloc(3 * NN);
    dhi.alloc(3 * NN, fine->g.nodeGuard());  // read by the unchecked double-float gather
    dlo.alloc(3 * NN, fine->g.nodeGuard());
    partialCount = std::max<int>(REDUCE_BLOCKS, (int)gridFor(NN, 256));
    partials.alloc(partialCount);
    sc.alloc(16);
    VFEM_CUDA(cudaMallocHost(&hostSc, 17 * sizeof(double)));  // [16]: coarse SPD flag
    std::memset(hostSc, 0, 17 * sizeof(double));
    setupCoarsestIndex();
    if (const char *env = std::getenv("VFEM_OVERLAP_STIFFNESS")) overlapStiffness = env[0] != '0';
    if (const char *env = std::getenv("VFEM_PEEL_FIRST")) peelFirst = env[0] != '0';
    if (const char *env = std::getenv("VFEM_BAND_UPDATE")) bandUpdates = env[0] != '0';
    if (const char *env = std::getenv("VFEM_STENCIL_BF16")) bf16Stencils = env[0] != '0';
    if (const char *env = std::getenv("VFEM_STENCIL_LINES_MAX_NODES")) stencilLinesMaxNodes = std::atoll(env);
    if (const char *env = std::getenv("VFEM_TAIL_MAX_NODES")) tailMaxNodes = std::atoll(env);
    if (const char *env = std::getenv("VFEM_REBUILD_STREAMS")) twoStreamRebuild = env[0] != '1';
    VFEM_CUDA(cudaStreamCreateWithFlags(&stiffStream, cudaStreamNonBlocking));
    VFEM_CUDA(cudaStreamCreateWithFlags(&stiffStream2, cudaStreamNonBlocking));
    VFEM_CUDA(cudaEventCreateWithFlags(&evStiffFork, cudaEventDisableTiming));
    VFEM_CUDA(cudaEventCreateWithFlags(&evLevelsReady, cudaEventDisableTiming));
    VFEM_CUDA(cudaEventCreateWithFlags(&evCoarseReady, cudaEventDisableTiming));
}

MG::~MG() {
    clearGraphs();
    if (stiffStream) cudaStreamSynchronize(stiffStream);
    if (evStiffFork) cudaEventDestroy(evStiffFork);
    if (evLevelsReady) cudaEventDestroy(evLevelsReady);
    if (evCoarseReady) cudaEventDestroy(evCoarseReady);
    if (stiffStream) cudaStreamDestroy(stiffStream);
    if (stiffStream2) {
        cudaStreamSynchronize(stiffStream2);
        cudaStreamDestroy(stiffStream2);
    }
    for (cudaEvent_t e : evKe) cudaEventDestroy(e);
    if (hostSc) cudaFreeHost(hostSc);
    if (copyDone) cudaEventDestroy(copyDone);
    if (copyStream) cudaStreamDestroy(copyStream);
}

void MG::clearGraphs() {
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
    graphKernels.clear();
    for (auto &kv : loopGraphs) cudaGraphExecDestroy(kv.second);
    loopGraphs.clear();
    loopKernels.clear();
    for (auto &kv : peelGraphs)
        for (auto &e : kv.second.part)
            if (e) cudaGraphExecDestroy(e);
    peelGraphs.clear();
    graphX = nullptr;
}

void MG::vcycleOnFineRhs(int64_t sweeps) {
    if (precision != PREC_MIXED) throw Error(ERR_STATE, "the fine-rhs V-cycle runs in mixed precision");
    auto &D = lv[0].d32;
    launch_fill<float>(D.x.p, 0.f, 3 * lv[0].g.NN, fine->stream);
    vcycleT<float>(0, sweeps, true, true);
}

// Dirichlet coarsening (MultigridSolver.hh:58-103): a fine constrained node on a coarse
// element's vertex/edge/face constrains every coarse node of that vertex/edge/face.
void MG::coarsenDirichlet() {
    for (int l = 1; l < L(); ++l) {
        const Level &F = lv[l - 1];
        Level &Cl = lv[l];
        Cl.dmask_h.assign(Cl.g.NN, 0);
        for (int64_t fn = 0; fn < F.g.NN; ++fn) {
            const uint8_t fm = F.dmask_h[fn];
            if (!fm) continue;
            const int fidx[3] = {(int)(fn / ((int64_t)F.g.nn[1] * F.g.nn[2])), (int)((fn / F.g.nn[2]) % F.g.nn[1]),
                                 (int)(fn % F.g.nn[2])};
            int e[3], pob[3];
            for (int d = 0; d < 3; ++d) {
                const double p = fine->bmin[d] + fidx[d] * F.h[d];
                const double fi = (p - fine->bmin[d]) / Cl.h[d];
                int ed;
                if (std::abs(fi - Cl.g.ne[d]) < 1e-10) ed = Cl.g.ne[d] - 1;
                else ed = (int)fi;
                if (ed >= Cl.g.ne[d]) throw Error(ERR_ARG, "Point out of bounds");
                e[d] = ed;
                const double cref = (p - (fine->bmin[d] + ed * Cl.h[d])) / Cl.h[d];
                pob[d] = std::abs(cref) < 1e-9 ? 0 : (std::abs(cref - 1.0) < 1e-9 ? 1 : -1);
            }
            for (int ln = 0; ln < 8; ++ln) {
                const int lb[3] = {(ln >> 2) & 1, (ln >> 1) & 1, ln & 1};
                bool ok = true;
                for (int d = 0; d < 3; ++d)
                    if (pob[d] != -1 && pob[d] != lb[d]) ok = false;
                if (!ok) continue;
                Cl.dmask_h[Cl.g.node(e[0] + lb[0], e[1] + lb[1], e[2] + lb[2])] |= fm;
            }
        }
    }
}

// Fixed coarsest DOFs: Dirichlet components plus every component of a detached node
// (TensorProductSimulator.hh:1181-1195).
void MG::setupCoarsestIndex() {
    const Level &C = lv.back();
    const std::vector<uint8_t> &dm = (L() == 1) ? fine->dmask_h : C.dmask_h;
    std::vector<int> red(3 * C.g.NN, -1), fr;
    const int nyv = C.g.nyv();
    for (int64_t n = 0; n < C.g.NN; ++n) {
        const int j = (int)((n / C.g.nn[2]) % C.g.nn[1]);
        for (int c = 0; c < 3; ++c) {
            if ((dm[n] >> c) & 1) continue;
            if (j >= nyv) continue;
            red[3 * n + c] = (int)fr.size();
            fr.push_back((int)(3 * n + c));
        }
    }
    if (L() == 1 && fine->dvalNonzero) throw Error(ERR_ARG, "Nonzero Dirichlet constraints currently unsupported");
    if (fr.size() > 30000) throw Error(ERR_ARG, "coarsest level too large for the dense direct solve; use more coarsening levels");
    const int nf = (int)fr.size();
    if (nf > nfreeCap || !freeIdx.p) {
        clearGraphs();  // buffers baked into graphs move
        nfreeCap = std::max(nf, 1);
        freeIdx.alloc(nfreeCap);
        Ainv.alloc((size_t)nfreeCap * nfreeCap);
        work.alloc(dense_inverse_work_size(nfreeCap));
        cscratch.alloc(nfreeCap);
        status.alloc(1);
    }
    nfree = nf;
    redIdx.alloc(red.size());
    cudaStream_t st = fine->stream;
    VFEM_CUDA(cudaMemcpyAsync(redIdx.p, red.data(), red.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    if (nf) VFEM_CUDA(cudaMemcpyAsync(freeIdx.p, fr.data(), fr.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    // pageable-memory copies return once staged, so red / fr may go out of scope
    launch_set_pair(nfreeDev.p, nf, 0, st);
    stiffnessValid = false;
}

void MG::setBf16Stencils(bool on) {
    if (on != bf16Stencils) {
        bf16Stencils = on;
        stiffnessValid = false;
        levelsValid = false;
        clearGraphs();
    }
}

void MG::setSweepForm(int form) {
    if (form != GS_LINES && form != GS_COLOURS && form != GS_PLANES && form != GS_STAGED)
        throw Error(ERR_ARG, "unknown sweep form");
    if (form != sweepForm) {
        sweepForm = form;
        clearGraphs();  // captured V-cycles hold the launches of the previous form
    }
}

void MG::setPrecision(int p) {
    if (p != PREC_FP64 && p != PREC_MIXED) throw Error(ERR_ARG, "unknown precision");
    if (p != precision) {
        precision = p;
        stiffnessValid = false;
        levelsValid = false;
        clearGraphs();
    }
}

void MG::setMaskLayer(int64_t layer) {
    fine->setMaskLayer(layer);
    lv[0].g = fine->g;
    for (int l = 1; l < L(); ++l) {
        const double fl = std::ceil(fine->maskH / lv[l].h[BUILD_DIR] - 1e-10);
        lv[l].g.firstMaskedE = (int)fl;
        lv[l].g.firstDetN = lv[l].g.firstMaskedE + 1;
        launch_set_pair(lv[l].dyn.p, lv[l].g.firstMaskedE, lv[l].g.firstDetN, fine->stream);
    }
    // captured graphs read the mask, the free-DOF count and the free-DOF list from device
    // memory, so they stay valid; only a larger coarsest system reallocates
    setupCoarsestIndex();
}

void MG::allocLevels() {
    for (int l = 0; l < L(); ++l) {
        const int64_t n3 = 3 * lv[l].g.NN;
        if (precision == PREC_FP64) {
            auto &D = lv[l].d64;
            D.x.alloc(n3); D.b.alloc(n3); D.r.alloc(n3);
        } else {
            auto &D = lv[l].d32;
            // the fine FP32 iterate is read by the unchecked neighbourhood gathers
            D.x.alloc(n3, l == 0 ? lv[0].g.nodeGuard() : 0); D.b.alloc(n3); D.r.alloc(n3);
        }
    }
}

static void syncFineGeom(MG &mg) {
    // the fine level shares the grid's (possibly masked) geometry
    mg.lv[0].g = mg.fine->g;
    // captured graphs hold K0 (kernel parameters) and the matvec kind chosen for it
    if (mg.graphK0Version != mg.fine->k0Version) {
        mg.clearGraphs();
        mg.graphK0Version = mg.fine->k0Version;
    }
}

template <typename T>
struct Tr;
template <>
struct Tr<double> {
    static const double *Y(Grid &g) { return g.Y.p; }
    static const double *Yfine(Grid &g) { return g.Y.p; }
    static const Mat24<double> &K0(Grid &g) { return g.K0; }
    static DevBuf<double> &Kc(MG &m) { return m.Kc64; }
    static DevBuf<double> &K2(MG &m) { return m.K2_64; }
    static DevBuf<double> &phis(MG &m) { return m.phis64; }
};
template <>
struct Tr<float> {
    static const float *Y(Grid &g) { return g.youngF(); }
    static const float *Yfine(Grid &g) { return g.youngFPad(); }
    static const Mat24<float> &K0(Grid &g) { return g.K0f; }
    static DevBuf<float> &Kc(MG &m) { return m.Kc32; }
    static DevBuf<float> &K2(MG &m) { return m.K2_32; }
    static DevBuf<float> &phis(MG &m) { return m.phis32; }
};

template <typename T>
static void uploadConst(DevBuf<T> &dst, const double *src, size_t n) {
    std::vector<T> tmp(src, src + n);
    dst.alloc(n);
    VFEM_CUDA(cudaMemcpy(dst.p, tmp.data(), n * sizeof(T), cudaMemcpyHostToDevice));
}

// MultigridSolver.hh:846-905: element matrices level by level, assembled stencils for the
// smoothing levels, and the dense inverse of the reduced coarsest operator.
template <typename T>
void MG::updateStiffnessT(bool overlap, int bandLo, int bandHi) {
    syncFineGeom(*this);
    allocLevels();
    cudaStream_t st = fine->stream;
    double phis[8][64];
    interpolation_phis(phis);
    // coarsening tables depend only on K0: rebuilt when the element stiffness changes
    const uint64_t constKey = fine->k0Version * 2 + (std::is_same<T, double>::value ? 1 : 0);
    if (constVersion[std::is_same<T, double>::value ? 1 : 0] != constKey) {
        std::vector<double> Kc(8 * 576, 0.0);
        for (int fi = 0; fi < 8; ++fi) coarsen_element(phis[fi], fine->K0.a, &Kc[fi * 576]);
        uploadConst(Tr<T>::Kc(*this), Kc.data(), Kc.size());
        uploadConst(Tr<T>::phis(*this), &phis[0][0], 512);
        if (L() > 2) {
            // K2[8c + fi] = Phi_c^T Kc[fi] Phi_c: the fine element at position fi of level-1 child c
            std::vector<double> K2(64 * 576, 0.0);
            for (int c = 0; c < 8; ++c)
                for (int fi = 0; fi < 8; ++fi) coarsen_element(phis[c], &Kc[fi * 576], &K2[(8 * c + fi) * 576]);
            uploadConst(Tr<T>::K2(*this), K2.data(), K2.size());
        }
        constVersion[std::is_same<T, double>::value ? 1 : 0] = constKey;
    }
    const T *Y0 = Tr<T>::Y(*fine);  // may enqueue the FP32 conversion on the solver stream
    // gs: the stream the rebuild runs on (the side stream forks after everything it reads)
    cudaStream_t gs = st;
    if (overlap && !stiffMarks && L() > 1 && stiffStream) {
        VFEM_CUDA(cudaEventRecord(evStiffFork, st));
        VFEM_CUDA(cudaStreamWaitEvent(stiffStream, evStiffFork, 0));
        gs = stiffStream;
    }
    auto mark = [&](const std::string &name) {
        if (!stiffMarks) return;
        cudaEvent_t e;
        VFEM_CUDA(cudaEventCreate(&e));
        VFEM_CUDA(cudaEventRecord(e, st));
        stiffMarks->emplace_back(name, e);
    };
    mark("start");
    if (L() == 1) {
        // direct solve on the fine grid: Ke = Y K0 (TensorProductSimulator.hh:1198-1230)
        auto &D = lv[0].data<T>();
        D.Ke.alloc((size_t)lv[0].g.NE * 576);
        lv[0].rows = lv[0].g.NN <= rowsMaxNodes;
        D.S.alloc((size_t)(lv[0].rows ? 256 : STENCIL_PLANES) * lv[0].g.NN);
        std::vector<double> k0(fine->K0.a, fine->K0.a + 576);
        DevBuf<T> K0d;
        uploadConst(K0d, k0.data(), 576);
        launch_ke_scaled<T>(lv[0].g, Y0, K0d.p, D.Ke.p, st);
        launch_stencil_from_ke<T>(lv[0].g, D.Ke.p, D.S.p, lv[0].rows, st);
        VFEM_CUDA(cudaStreamSynchronize(st));
    } else if (gs != st && L() > 2 && twoStreamRebuild) {
        // Two side streams. gs: the element-matrix chain of levels 2.., the coarsest level's
        // stencil, its dense operator and inverse (the critical path of the rebuild); gs2: the
        // stencils of the smoothing levels, each after its level's element matrices. gs joins gs2
        // before evCoarseReady, so that event still stands for the whole rebuild.
        const bool band = bandLo >= 0;
        VFEM_CUDA(cudaStreamWaitEvent(stiffStream2, evStiffFork, 0));
        cudaStream_t gs2 = stiffStream2;
        if ((int)evKe.size() < L()) {
            for (int l = (int)evKe.size(); l < L(); ++l) {
                cudaEvent_t e;
                VFEM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
                evKe.push_back(e);
            }
        }
        for (int l = 1; l < L() && (!band || bandLo < bandHi); ++l) {
            auto &D = lv[l].data<T>();
            lv[l].rows = lv[l].g.NN <= rowsMaxNodes;
            const bool half = std::is_same<T, float>::value && halfStencil(l);
            if (half) D.Sh.alloc((size_t)STENCIL_PLANES * lv[l].g.NN);
            else D.S.alloc((size_t)(lv[l].rows ? 256 : STENCIL_PLANES) * lv[l].g.NN);
            const int eLo = band ? (bandLo >> l) : 0;
            const int eHi = band ? ((bandHi - 1) >> l) + 1 : lv[l].g.ne[1];
            const int nLo = eLo, nHi = band ? eHi + 1 : lv[l].g.nn[1];
            if (l == 1) {
                if (half)
                    launch_stencil_level1<T>(lv[1].g, lv[0].g, Y0, Tr<T>::Kc(*this).p, D.Sh.p, lv[1].rows, gs2, nLo,
                                             nHi);
                else
                    launch_stencil_level1<T>(lv[1].g, lv[0].g, Y0, Tr<T>::Kc(*this).p, D.S.p, lv[1].rows, gs2, nLo,
                                             nHi);
                continue;
            }
            D.Ke.alloc((size_t)lv[l].g.NE * 576);
            if (l == 2)
                launch_ke_level2<T>(lv[2].g, lv[1].g, lv[0].g, Y0, Tr<T>::K2(*this).p, D.Ke.p, gs, eLo, eHi);
            else
                launch_ke_coarsen<T>(lv[l].g, lv[l - 1].g, lv[l - 1].data<T>().Ke.p, Tr<T>::phis(*this).p, D.Ke.p, gs,
                                     eLo, eHi);
            // the coarsest level's stencil feeds the dense operator (gs); the others smooth (gs2)
            cudaStream_t ss = (l == L() - 1) ? gs : gs2;
            if (ss == gs2) {
                VFEM_CUDA(cudaEventRecord(evKe[l], gs));
                VFEM_CUDA(cudaStreamWaitEvent(gs2, evKe[l], 0));
            }
            if (half) launch_stencil_from_ke<T>(lv[l].g, D.Ke.p, D.Sh.p, lv[l].rows, ss, nLo, nHi);
            else launch_stencil_from_ke<T>(lv[l].g, D.Ke.p, D.S.p, lv[l].rows, ss, nLo, nHi);
        }
        VFEM_CUDA(cudaEventRecord(evLevelsReady, gs2));
    } else {
        const bool band = bandLo >= 0;
        for (int l = 1; l < L() && (!band || bandLo < bandHi); ++l) {
            auto &D = lv[l].data<T>();
            lv[l].rows = lv[l].g.NN <= rowsMaxNodes;
            const bool half = std::is_same<T, float>::value && halfStencil(l);
            if (half) D.Sh.alloc((size_t)STENCIL_PLANES * lv[l].g.NN);
            else D.S.alloc((size_t)(lv[l].rows ? 256 : STENCIL_PLANES) * lv[l].g.NN);
            // level-l element rows whose matrices change, and the node rows whose stencils do
            const int eLo = band ? (bandLo >> l) : 0;
            const int eHi = band ? ((bandHi - 1) >> l) + 1 : lv[l].g.ne[1];
            const int nLo = eLo, nHi = band ? eHi + 1 : lv[l].g.nn[1];
            if (l == 1) {
                // the level-1 stencil comes straight from the fine moduli; no level-1 element
                // matrices are stored
                if (half)
                    launch_stencil_level1<T>(lv[1].g, lv[0].g, Y0, Tr<T>::Kc(*this).p, D.Sh.p, lv[1].rows, gs, nLo,
                                             nHi);
                else
                    launch_stencil_level1<T>(lv[1].g, lv[0].g, Y0, Tr<T>::Kc(*this).p, D.S.p, lv[1].rows, gs, nLo,
                                             nHi);
                mark("galerkin:L1 stencil");
            } else {
                D.Ke.alloc((size_t)lv[l].g.NE * 576);
                if (l == 2)
                    launch_ke_level2<T>(lv[2].g, lv[1].g, lv[0].g, Y0, Tr<T>::K2(*this).p, D.Ke.p, gs, eLo, eHi);
                else
                    launch_ke_coarsen<T>(lv[l].g, lv[l - 1].g, lv[l - 1].data<T>().Ke.p, Tr<T>::phis(*this).p, D.Ke.p,
                                         gs, eLo, eHi);
                mark("galerkin:L" + std::to_string(l) + " element matrices");
                if (half) launch_stencil_from_ke<T>(lv[l].g, D.Ke.p, D.Sh.p, lv[l].rows, gs, nLo, nHi);
                else launch_stencil_from_ke<T>(lv[l].g, D.Ke.p, D.S.p, lv[l].rows, gs, nLo, nHi);
                mark("galerkin:L" + std::to_string(l) + " stencil");
            }
        }
        VFEM_CUDA(cudaEventRecord(evLevelsReady, gs));
    }
    if (L() == 1) VFEM_CUDA(cudaEventRecord(evLevelsReady, gs));
    // dense reduced coarsest operator, FP64 inverse
    const Level &C = lv.back();
    if (nfree > 0) {
        launch_dense_from_stencil<T>(C.g, lv.back().data<T>().S.p, redIdx.p, Ainv.p, nfree, lv.back().rows, gs);
        launch_symmetrize(Ainv.p, nfree, gs);
        VFEM_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), gs));
        mark("coarsest:dense assembly");
        if (stiffMarks) dense_spd_inverse(Ainv.p, work.p, nfree, status.p, gs, mark);
        else dense_spd_inverse(Ainv.p, work.p, nfree, status.p, gs);
        // the positive-definiteness flag is read back once the stream reaches it
        VFEM_CUDA(cudaMemcpyAsync(&hostSc[16], status.p, sizeof(int), cudaMemcpyDeviceToHost, gs));
        spdCheckPending = true;
    }
    if (gs != st) VFEM_CUDA(cudaStreamWaitEvent(gs, evLevelsReady, 0));  // the stencils' stream
    VFEM_CUDA(cudaEventRecord(evCoarseReady, gs));
    stiffnessValid = true;
    stiffnessPrecision = precision;
    stiffnessDensVersion = fine->densVersion;
    stiffnessMaskVersion = fine->maskVersion;
    stiffnessMaterialVersion = fine->materialVersion;
    stiffnessMaskE = fine->g.firstMaskedE;
    levelsValid = true;
    if (bandLo >= 0) ++bandRebuilds;
    else ++fullRebuilds;
}

void MG::updateStiffness(bool overlap, int bandLo, int bandHi) {
    // a rebuild still in flight on the side stream finishes before this one starts
    VFEM_CUDA(cudaStreamWaitEvent(fine->stream, evCoarseReady, 0));
    if (precision == PREC_FP64) updateStiffnessT<double>(overlap, bandLo, bandHi);
    else updateStiffnessT<float>(overlap, bandLo, bandHi);
    if (!overlap) VFEM_CUDA(cudaStreamWaitEvent(fine->stream, evCoarseReady, 0));
    rebuildInFlight = overlap;
}

void MG::ensureStiffness(bool deferCheck, bool overlap) {
    syncFineGeom(*this);
    if (!stiffnessValid || stiffnessPrecision != precision || stiffnessDensVersion != fine->densVersion ||
        stiffnessMaskVersion != fine->maskVersion) {
        // only the fabrication mask moved since the last build: rebuild the band of level
        // operators between the old and the new masked element row
        bool band = bandUpdates && levelsValid && stiffnessPrecision == precision &&
                    stiffnessMaterialVersion == fine->materialVersion && stiffnessMaskE >= 0 && L() > 1;
        for (int l = 1; band && l < L(); ++l) band = lv[l].g.NN > rowsMaxNodes;  // plane-layout stencils only
        if (band) {
            const int ne1 = fine->g.ne[BUILD_DIR];
            const int a = std::min(stiffnessMaskE, ne1), b = std::min(fine->g.firstMaskedE, ne1);
            updateStiffness(overlap, std::min(a, b), std::max(a, b));
        } else {
            updateStiffness(overlap);
        }
    }
    if (!overlap) {
        VFEM_CUDA(cudaStreamWaitEvent(fine->stream, evCoarseReady, 0));
        rebuildInFlight = false;
    }
    if (!deferCheck) checkStiffness();
}

// Raise the coarsest factorisation's positive-definiteness failure, if one is pending.
void MG::checkStiffness() {
    if (!spdCheckPending) return;
    VFEM_CUDA(cudaStreamWaitEvent(fine->stream, evCoarseReady, 0));
    rebuildInFlight = false;
    VFEM_CUDA(cudaStreamSynchronize(fine->stream));
    spdCheckPending = false;
    int hs = 0;
    std::memcpy(&hs, &hostSc[16], sizeof(int));
    if (hs) {
        stiffnessValid = false;
        levelsValid = false;
        check_dense_status(hs);
    }
}

template <typename T>
void MG::smoothT(int l, bool forward) {
    cudaStream_t st = fine->stream;
    auto &D = lv[l].data<T>();
    const uint8_t *dm = (l == 0) ? fine->dmask.p : lv[l].dmask.p;
    if constexpr (std::is_same<T, float>::value) {
        const int mode = l == 0 ? (sweepForm >= 0 ? sweepForm : gsFineMode()) : GS_COLOURS;
        if (mode == GS_PLANES) {
            // two launches: the x-even colours then the x-odd ones (reversed backward)
            for (int h = 0; h < 2; ++h)
                launch_gs_fine_planes(lv[0].g, Tr<T>::Yfine(*fine), D.x.p, D.b.p, dm, forward ? h : 1 - h, forward,
                                      Tr<T>::K0(*fine), st);
            return;
        }
        if (mode == GS_LINES || mode == GS_STAGED) {
            // four launches: colour pairs (0, 1), (2, 3), (4, 5), (6, 7), reversed backward
            const bool staged = mode == GS_STAGED && gsStagedFits(lv[0].g);
            for (int h = 0; h < 4; ++h) {
                const int c = forward ? h : 3 - h;
                if (staged)
                    launch_gs_fine_staged(lv[0].g, Tr<T>::Yfine(*fine), D.x.p, D.b.p, dm, (c >> 1) & 1, c & 1,
                                          forward, Tr<T>::K0(*fine), st);
                else
                    launch_gs_fine_lines(lv[0].g, Tr<T>::Yfine(*fine), D.x.p, D.b.p, dm, (c >> 1) & 1, c & 1,
                                         forward, Tr<T>::K0(*fine), st);
            }
            return;
        }
    }
    if (l > 0 && !lv[l].rows && lv[l].g.NN <= stencilLinesMaxNodes) {
        // small plane-layout levels: colour pairs on whole z-lines, four launches per sweep
        for (int h = 0; h < 4; ++h) {
            const int c = forward ? h : 3 - h;
            withStencil<T>(l, [&](auto S) {
                launch_gs_stencil_lines<T>(lv[l].g, S, D.x.p, D.b.p, dm, (c >> 1) & 1, c & 1, forward, st);
            });
        }
        return;
    }
    for (int c = 0; c < 8; ++c) {
        const int color = forward ? c : 7 - c;
        if (l == 0) launch_gs_fine_color<T>(lv[0].g, Tr<T>::Yfine(*fine), D.x.p, D.b.p, dm, color, forward, Tr<T>::K0(*fine), st);
        else
            withStencil<T>(l, [&](auto S) {
                launch_gs_stencil_color<T>(lv[l].g, S, D.x.p, D.b.p, dm, color, forward, lv[l].rows, st);
            });
    }
}

template <typename T>
void MG::residualT(int l) {
    cudaStream_t st = fine->stream;
    auto &D = lv[l].data<T>();
    if (l == 0) launch_residual_fine<T>(lv[0].g, Tr<T>::Yfine(*fine), D.x.p, D.b.p, D.r.p, Tr<T>::K0(*fine), fine->dmask.p, st);
    else
        withStencil<T>(l, [&](auto S) {
            launch_stencil_residual<T>(lv[l].g, S, D.x.p, D.b.p, D.r.p, lv[l].dmask.p, lv[l].rows, st);
        });
}

int MG::tailStart() const {
    int t = L() - 1;  // the coarsest level always ends the tail
    // the tail kernels read FP32 node-contiguous rows: plane-layout and bf16 levels stay outside
    while (t - 1 >= 1 && lv[t - 1].g.NN <= tailMaxNodes && lv[t - 1].rows && !halfStencil(t - 1)) --t;
    return (t < L() - 1) ? t : L();
}

// MultigridSolver.hh:617-658
template <typename T>
void MG::vcycleT(int l, int64_t sweeps, bool residualSystem, bool xZero) {
    cudaStream_t st = fine->stream;
    auto &D = lv[l].data<T>();
    if (std::is_same<T, float>::value && residualSystem && l >= 1 && l == tailStart()) {
        // small levels: one CTA runs the down leg, the dense solve runs on the whole GPU,
        // one CTA runs the up leg
        TailParams<T> P;
        P.nlev = L() - l;
        if (P.nlev > MAX_TAIL_LEVELS) throw Error(ERR_ARG, "too many tail levels");
        P.sweeps = (int)sweeps;
        P.symmetric = symmetricGS ? 1 : 0;
        for (int t = 0; t < P.nlev; ++t) {
            auto &Q = lv[l + t].data<T>();
            P.lv[t] = TailLevel<T>{lv[l + t].g, Q.S.p, Q.x.p, Q.b.p, Q.r.p, lv[l + t].dmask.p};
        }
        launch_tail_down<T>(P, st);
        auto &Dc = lv.back().data<T>();
        launch_coarse_solve<T>(lv.back().g, Ainv.p, freeIdx.p, nfreeDev.p, nfreeCap, Dc.b.p, Dc.x.p, cscratch.p, st);
        launch_tail_up<T>(P, st);
        return;
    }
    if (l == L() - 1) {
        launch_coarse_solve<T>(lv[l].g, Ainv.p, freeIdx.p, nfreeDev.p, nfreeCap, D.b.p, D.x.p, cscratch.p, st);
        return;
    }
    const uint8_t *dm = (l == 0) ? fine->dmask.p : lv[l].dmask.p;
    // enforceDirichletConditions (MultigridSolver.hh:628): a no-op on an iterate that is zero on
    // every row the level reads (the fresh preconditioner iterate, a just masked-zeroed coarse one)
    if (!xZero) {
        if (residualSystem || l > 0 || !fine->dvalNonzero) launch_zero_dirichlet<T>(lv[l].g, D.x.p, dm, st);
        else launch_enforce_dirichlet<T>(lv[l].g, D.x.p, dm, fine->dval.p, st);
    }
    for (int64_t i = 0; i < sweeps; ++i) smoothT<T>(l, true);
    residualT<T>(l);
    auto &Dc = lv[l + 1].data<T>();
    launch_restrict<T>(lv[l].g, lv[l + 1].g, D.r.p, Dc.b.p, st);
    launch_masked_zero<T>(lv[l + 1].g, Dc.x.p, MARGIN, st);
    vcycleT<T>(l + 1, sweeps, true, true);
    launch_interpolate<T>(lv[l].g, lv[l + 1].g, Dc.x.p, D.x.p, true, st);
    for (int64_t i = 0; i < sweeps; ++i) smoothT<T>(l, !symmetricGS);
}

template <typename T>
void MG::vcyclePartT(int part, int64_t sweeps) {
    cudaStream_t st = fine->stream;
    const int ts = tailStart();
    const bool tail = std::is_same<T, float>::value && ts < L();  // the tail takes over at level ts >= 1
    const int bottom = tail ? ts : L() - 1;
    TailParams<T> P;
    if (tail) {
        P.nlev = L() - ts;
        if (P.nlev > MAX_TAIL_LEVELS) throw Error(ERR_ARG, "too many tail levels");
        P.sweeps = (int)sweeps;
        P.symmetric = symmetricGS ? 1 : 0;
        for (int t = 0; t < P.nlev; ++t) {
            auto &Q = lv[ts + t].data<T>();
            P.lv[t] = TailLevel<T>{lv[ts + t].g, Q.S.p, Q.x.p, Q.b.p, Q.r.p, lv[ts + t].dmask.p};
        }
    }
    auto down = [&](int l) {
        // the first iteration's iterates are zero on every row read: no Dirichlet zeroing (vcycleT)
        auto &D = lv[l].data<T>();
        for (int64_t i = 0; i < sweeps; ++i) smoothT<T>(l, true);
        residualT<T>(l);
        auto &Dc = lv[l + 1].data<T>();
        launch_restrict<T>(lv[l].g, lv[l + 1].g, D.r.p, Dc.b.p, st);
        launch_masked_zero<T>(lv[l + 1].g, Dc.x.p, MARGIN, st);
    };
    if (part == 0) {
        down(0);
        return;
    }
    if (part == 1) {
        for (int l = 1; l < bottom; ++l) down(l);
        if (tail) launch_tail_down<T>(P, st);
        return;
    }
    auto &Dc = lv.back().data<T>();
    launch_coarse_solve<T>(lv.back().g, Ainv.p, freeIdx.p, nfreeDev.p, nfreeCap, Dc.b.p, Dc.x.p, cscratch.p, st);
    if (tail) launch_tail_up<T>(P, st);
    for (int l = bottom - 1; l >= 0; --l) {
        auto &D = lv[l].data<T>();
        auto &Dn = lv[l + 1].data<T>();
        launch_interpolate<T>(lv[l].g, lv[l + 1].g, Dn.x.p, D.x.p, true, st);
        for (int64_t i = 0; i < sweeps; ++i) smoothT<T>(l, !symmetricGS);
    }
}

// MultigridSolver.hh:587-609
template <typename T>
void MG::fmgT(int l, int64_t sweeps, bool residualSystem) {
    cudaStream_t st = fine->stream;
    auto &D = lv[l].data<T>();
    if (l == L() - 1) {
        launch_coarse_solve<T>(lv[l].g, Ainv.p, freeIdx.p, nfreeDev.p, nfreeCap, D.b.p, D.x.p, cscratch.p, st);
        return;
    }
    auto &Dc = lv[l + 1].data<T>();
    launch_restrict<T>(lv[l].g, lv[l + 1].g, D.b.p, Dc.b.p, st);
    fmgT<T>(l + 1, sweeps, residualSystem);
    launch_interpolate<T>(lv[l].g, lv[l + 1].g, Dc.x.p, D.x.p, false, st);
    vcycleT<T>(l, sweeps, residualSystem);
}

// Preconditioner s = M^{-1} r (MultigridSolver.hh:547-580): zero initial guess,
// residual system, mgIter V-cycles (or FMG + mgIter-1 V-cycles).
template <typename T>
void MG::preconditionT(const double *r, int64_t mgIter, int64_t sweeps, bool fmg, bool prepared) {
    cudaStream_t st = fine->stream;
    if (sweeps == 0) return;  // applyPreconditionerInv returns without touching the MG iterate
    auto &D = lv[0].data<T>();
    const int64_t n3 = 3 * lv[0].g.NN;
    if (!prepared) {
        launch_fill<T>(D.x.p, T(0), n3, st);
        if (mgIter == 0) return;
        if (std::is_same<T, double>::value) launch_copy((double *)D.b.p, r, n3, st);
        else launch_cast<float, double>(r, (float *)D.b.p, n3, st);
    }
    if (fmg) {
        fmgT<T>(0, sweeps, true);
        for (int64_t i = 1; i < mgIter; ++i) vcycleT<T>(0, sweeps, true);
    } else {
        for (int64_t i = 0; i < mgIter; ++i) vcycleT<T>(0, sweeps, true, i == 0);
    }
}

void MG::prepareFusedInit(int64_t mgIter, int64_t sweeps) {
    fusedInitOn = precision == PREC_MIXED && mgIter > 0 && sweeps > 0;
    if (!fusedInitOn) return;
    allocLevels();
    auto &D = lv[0].d32;
    const int64_t n3 = 3 * lv[0].g.NN;
    launch_fill<float>(D.x.p, 0.f, n3, fine->stream);
    launch_cast<float, double>(rbuf.p, D.b.p, n3, fine->stream);
}

// One PCG iteration (MultigridSolver.hh:1108-1144), enqueued without host synchronisation.
void MG::cgIteration(double *x, int64_t mgIter, int64_t sweeps, bool fmg, bool hostMirror) {
    cudaStream_t st = fine->stream;
    const Geom &g = lv[0].g;
    if (mgIter > 0) {
        if (precision == PREC_FP64) {
            preconditionT<double>(rbuf.p, mgIter, sweeps, fmg);
            launch_cg_precond_out<double>(g, lv[0].d64.x.p, s.p, rbuf.p, fine->dmask.p, partials.p, st);
        } else {
            // the previous cg_update (or the solve's start) left b32 = (float) r and x32 = 0
            preconditionT<float>(rbuf.p, mgIter, sweeps, fmg, fusedInit());
            // s is not stored: the direction update forms it again from the FP32 iterate
            launch_cg_precond_out<float>(g, lv[0].d32.x.p, (double *)nullptr, rbuf.p, fine->dmask.p, partials.p, st);
        }
    } else {
        launch_cg_precond_out<double>(g, rbuf.p, s.p, rbuf.p, fine->dmask.p, partials.p, st);
    }
    cgIterationRest(x, mgIter, hostMirror);
}

void MG::cgIterationRest(double *x, int64_t mgIter, bool hostMirror) {
    cudaStream_t st = fine->stream;
    const Geom &g = lv[0].g;
    launch_cg_beta(partials.p, REDUCE_BLOCKS, sc.p, st);
    outerDirection(mgIter > 0 && precision != PREC_FP64 ? lv[0].d32.x.p : nullptr);
    const int nb = outerMatvecApply(dvec.p, Ad.p, partials.p, nullptr, true);
    launch_cg_alpha(partials.p, nb, sc.p, st);
    if (fusedInit())
        launch_cg_update(g, x, rbuf.p, dvec.p, Ad.p, sc.p, partials.p, st, lv[0].d32.b.p, lv[0].d32.x.p);
    else
        launch_cg_update(g, x, rbuf.p, dvec.p, Ad.p, sc.p, partials.p, st);
    launch_cg_rsq(partials.p, REDUCE_BLOCKS, sc.p, nullptr, st);
    if (hostMirror) VFEM_CUDA(cudaMemcpyAsync(hostSc, sc.p, 16 * sizeof(double), cudaMemcpyDeviceToHost, st));
}

int MG::outerKind() const {
    if (precision != PREC_MIXED || outerMatvec == MATVEC_FP64) return 0;
    if (outerMatvec == MATVEC_DF && fine->tcOk) return 2;
    return 1;
}

void MG::outerDirection(const float *precondIterate) {
    const int kind = outerKind();
    if (kind == 2) umax.alloc(REDUCE_BLOCKS);
    float *dh = kind == 1 ? dhi.p : nullptr, *dl = kind == 1 ? dlo.p : nullptr;
    double *am = kind == 2 ? umax.p : nullptr;
    if (precondIterate)
        launch_cg_direction_precond<float>(lv[0].g, precondIterate, fine->dmask.p, dvec.p, sc.p, dh, dl, fine->stream,
                                           am);
    else
        launch_cg_direction(lv[0].g, s.p, dvec.p, sc.p, dh, dl, fine->stream, am);
}

int MG::outerMatvecApply(const double *u, double *out, double *partialsOut, const double *rhs, bool uReady) {
    const Geom &g = lv[0].g;
    cudaStream_t st = fine->stream;
    const int kind = outerKind();
    if (kind == 2) {
        const float *yh, *yl;
        fine->youngDF(&yh, &yl);
        umax.alloc(REDUCE_BLOCKS);
        if (!uReady) launch_absmax_partials(u, 3 * g.ld, umax.p, st);
        return launch_applyk_fine_tc(g, yh, yl, u, umax.p, out, fine->tcB.p, fine->tcScale, fine->dmask.p, true,
                                     partialsOut, partialCount, fine->tcStatus.p, st, rhs);
    }
    if (kind == 1) {
        const float *yh, *yl;
        fine->youngDF(&yh, &yl);
        if (!uReady) launch_split_df(u, dhi.p, dlo.p, 3 * g.ld, st);
        launch_applyk_fine_df(g, yh, yl, dhi.p, dlo.p, u, out, fine->K0df, fine->dmask.p, true, partialsOut,
                              partialCount, st, rhs);
        return (int)gridFor(g.NN, 256);
    }
    if (rhs) {
        launch_residual_fine<double>(g, fine->Y.p, u, rhs, out, fine->K0, fine->dmask.p, st);
        return 0;
    }
    launch_applyk_fine<double>(g, fine->Y.p, u, out, fine->K0, true, false, fine->dmask.p, true, partialsOut,
                               partialCount, st);
    return (int)gridFor(g.NN, 256);
}

void MG::outerApply(const double *u, double *out, const double *rhs) {
    syncFineGeom(*this);
    cudaStream_t st = fine->stream;
    const size_t bytes = 3 * fine->g.NN * sizeof(double);
    View vu, vo, vr;
    viewIn(vu, u, bytes, st);
    if (rhs) viewIn(vr, rhs, bytes, st);
    viewOut(vo, out, bytes);
    outerMatvecApply((const double *)vu.d, (double *)vo.d, nullptr, rhs ? (const double *)vr.d : nullptr, false);
    finishOut(vo, st);
    VFEM_CUDA(cudaStreamSynchronize(st));
    checkTensorStatus();
}

void MG::checkTensorStatus() {
    if (outerKind() != 2) return;
    int v = 0;
    VFEM_CUDA(cudaMemcpyAsync(&v, fine->tcStatus.p, sizeof(int), cudaMemcpyDeviceToHost, fine->stream));
    VFEM_CUDA(cudaStreamSynchronize(fine->stream));
    if (v) {
        VFEM_CUDA(cudaMemsetAsync(fine->tcStatus.p, 0, sizeof(int), fine->stream));
        throw Error(ERR_CUDA, "tensor-core matvec: a wait for the tensor core timed out");
    }
}

static uint64_t countKernelNodes(cudaGraph_t graph) {
    size_t n = 0;
    VFEM_CUDA(cudaGraphGetNodes(graph, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    VFEM_CUDA(cudaGraphGetNodes(graph, nodes.data(), &n));
    uint64_t k = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType ty;
        VFEM_CUDA(cudaGraphNodeGetType(nd, &ty));
        if (ty == cudaGraphNodeTypeKernel) ++k;
    }
    return k;
}

// [loop control (initial)] -> WHILE( [one PCG iteration] -> [loop control] )
cudaGraphExec_t MG::loopGraph(const GraphKey &key, double *x, int64_t mgIter, int64_t sweeps, bool fmg) {
    if (graphX != x) clearGraphs();
    auto it = loopGraphs.find(key);
    if (it != loopGraphs.end()) return it->second;
    cudaStream_t st = fine->stream;
    cudaGraph_t top;
    VFEM_CUDA(cudaGraphCreate(&top, 0));
    cudaGraphExec_t exec = nullptr;
    try {
        cudaGraphConditionalHandle h;
        VFEM_CUDA(cudaGraphConditionalHandleCreate(&h, top, 0, cudaGraphCondAssignDefault));
        VFEM_CUDA(cudaStreamBeginCaptureToGraph(st, top, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        launch_cg_loop_control(h, sc.p, true, st);
        VFEM_CUDA(cudaStreamEndCapture(st, &top));
        cudaGraphNode_t init;
        size_t n = 1;
        VFEM_CUDA(cudaGraphGetNodes(top, &init, &n));
        cudaGraphNodeParams p = {};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = h;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        cudaGraphNode_t loop;
        VFEM_CUDA(cudaGraphAddNode(&loop, top, &init, nullptr, 1, &p));
        cudaGraph_t body = p.conditional.phGraph_out[0];
        VFEM_CUDA(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        try {
            cgIteration(x, mgIter, sweeps, fmg, false);
            launch_cg_loop_control(h, sc.p, false, st);
        } catch (...) {
            cudaStreamEndCapture(st, &body);
            throw;
        }
        VFEM_CUDA(cudaStreamEndCapture(st, &body));
        const uint64_t k = countKernelNodes(body);
        VFEM_CUDA(cudaGraphInstantiate(&exec, top, 0));
        launchCounter() -= k + 1;  // the captures launched nothing
        loopKernels[key] = k;
    } catch (...) {
        cudaGraphDestroy(top);
        throw;
    }
    cudaGraphDestroy(top);
    graphX = x;
    return loopGraphs.emplace(key, exec).first->second;
}

// [set IF from the loop's initial condition] -> IF( part `part` of the first iteration )
const MG::PeelGraphs &MG::peelGraph(const GraphKey &key, double *x, int64_t sweeps) {
    auto it = peelGraphs.find(key);
    if (it != peelGraphs.end()) return it->second;
    cudaStream_t st = fine->stream;
    PeelGraphs pg;
    try {
        for (int part = 0; part < 3; ++part) {
            cudaGraph_t top;
            VFEM_CUDA(cudaGraphCreate(&top, 0));
            try {
                cudaGraphConditionalHandle h;
                VFEM_CUDA(cudaGraphConditionalHandleCreate(&h, top, 0, cudaGraphCondAssignDefault));
                VFEM_CUDA(cudaStreamBeginCaptureToGraph(st, top, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
                launch_cg_loop_control(h, sc.p, true, st);
                VFEM_CUDA(cudaStreamEndCapture(st, &top));
                cudaGraphNode_t init;
                size_t n = 1;
                VFEM_CUDA(cudaGraphGetNodes(top, &init, &n));
                cudaGraphNodeParams p = {};
                p.type = cudaGraphNodeTypeConditional;
                p.conditional.handle = h;
                p.conditional.type = cudaGraphCondTypeIf;
                p.conditional.size = 1;
                cudaGraphNode_t node;
                VFEM_CUDA(cudaGraphAddNode(&node, top, &init, nullptr, 1, &p));
                cudaGraph_t body = p.conditional.phGraph_out[0];
                VFEM_CUDA(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
                try {
                    if (part == 0 && !fusedInit()) {
                        const int64_t n3 = 3 * lv[0].g.NN;
                        launch_fill<float>(lv[0].d32.x.p, 0.f, n3, st);
                        launch_cast<float, double>(rbuf.p, lv[0].d32.b.p, n3, st);
                    }
                    vcyclePartT<float>(part, sweeps);
                    if (part == 2) {
                        launch_cg_precond_out<float>(lv[0].g, lv[0].d32.x.p, (double *)nullptr, rbuf.p,
                                                     fine->dmask.p, partials.p, st);
                        cgIterationRest(x, 1, false);
                        launch_cg_count(sc.p, st);
                    }
                } catch (...) {
                    cudaStreamEndCapture(st, &body);
                    throw;
                }
                VFEM_CUDA(cudaStreamEndCapture(st, &body));
                pg.kernels += countKernelNodes(body) + 1;
                VFEM_CUDA(cudaGraphInstantiate(&pg.part[part], top, 0));
            } catch (...) {
                cudaGraphDestroy(top);
                throw;
            }
            cudaGraphDestroy(top);
        }
    } catch (...) {
        for (auto &e : pg.part)
            if (e) cudaGraphExecDestroy(e);
        throw;
    }
    launchCounter() -= pg.kernels;  // the captures launched nothing
    return peelGraphs.emplace(key, pg).first->second;
}

static double readScalar(double *dev, cudaStream_t st) {
    double v = 0;
    VFEM_CUDA(cudaMemcpyAsync(&v, dev, sizeof(double), cudaMemcpyDeviceToHost, st));
    VFEM_CUDA(cudaStreamSynchronize(st));
    return v;
}

void MG::pcgStart(double *x, const double *b, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps, bool fmg,
                  bool dirichletSatisfied) {
    syncFineGeom(*this);
    if (L() == 1) throw Error(ERR_ARG, "the asynchronous solve needs at least one coarsening level");
    if (pending) throw Error(ERR_STATE, "a solve is already in flight on this solver");
    cudaStream_t st = fine->stream;
    const Geom &g = lv[0].g;
    if (precision == PREC_MIXED) {
        fine->youngF();
        fine->youngFPad();
        const float *yh, *yl;
        if (outerMatvec != MATVEC_FP64) fine->youngDF(&yh, &yl);
        if (outerKind() == 2) umax.alloc(REDUCE_BLOCKS);
    }
    allocLevels();
    // the hierarchy rebuild (if the densities or the mask changed) forks onto the side stream
    // here and the solve's start below runs meanwhile (positive definiteness is checked in
    // pcgFinish)
    if (mgIter > 0) ensureStiffness(true, overlapStiffness);
    const bool rebuilding = rebuildInFlight;  // forked here or by the caller (MG::pcg)
    if (!dirichletSatisfied) launch_enforce_dirichlet<double>(g, x, fine->dmask.p, fine->dval.p, st);
    launch_masked_dot_partials<double, double>(g, b, b, partials.p, st);
    launch_finalize(partials.p, REDUCE_BLOCKS, sc.p + 7, st);
    // initial residual through the outer operator, like every later product
    outerMatvecApply(x, rbuf.p, nullptr, b, false);
    launch_masked_dot_partials<double, double>(g, rbuf.p, rbuf.p, partials.p, st);
    launch_finalize(partials.p, REDUCE_BLOCKS, sc.p + 5, st);
    launch_cg_init(sc.p, tol * tol, (double)maxIter, st);
    prepareFusedInit(mgIter, sweeps);
    launch_fill<double>(dvec.p, 0.0, 3 * g.NN, st);
    pendingKey = GraphKey{mgIter, sweeps, fmg ? 1 : 0, symmetricGS ? 1 : 0, precision, outerMatvec};
    cudaGraphExec_t exec = loopGraph(pendingKey, x, mgIter, sweeps, fmg);
    pendingPeeled = peelFirst && rebuilding && precision == PREC_MIXED && mgIter == 1 && !fmg && sweeps > 0;
    if (pendingPeeled) {
        // the first iteration joins the rebuild where it needs it
        const PeelGraphs &pg = peelGraph(pendingKey, x, sweeps);
        VFEM_CUDA(cudaGraphLaunch(pg.part[0], st));
        VFEM_CUDA(cudaStreamWaitEvent(st, evLevelsReady, 0));
        VFEM_CUDA(cudaGraphLaunch(pg.part[1], st));
        VFEM_CUDA(cudaStreamWaitEvent(st, evCoarseReady, 0));
        VFEM_CUDA(cudaGraphLaunch(pg.part[2], st));
    } else {
        VFEM_CUDA(cudaStreamWaitEvent(st, evCoarseReady, 0));  // join the side-stream rebuild
    }
    rebuildInFlight = false;
    VFEM_CUDA(cudaGraphLaunch(exec, st));
    pending = true;
}

PcgStats MG::pcgFinish() {
    if (!pending) throw Error(ERR_STATE, "no solve in flight");
    pending = false;
    cudaStream_t st = fine->stream;
    VFEM_CUDA(cudaMemcpyAsync(hostSc, sc.p, 16 * sizeof(double), cudaMemcpyDeviceToHost, st));
    checkStiffness();  // synchronises the stream
    VFEM_CUDA(cudaStreamSynchronize(st));
    checkTensorStatus();
    PcgStats stats;
    stats.iterations = (int64_t)hostSc[9];
    stats.rsq = hostSc[5];
    stats.bnorm2 = hostSc[7];
    if (pendingPeeled && stats.iterations > 0)
        launchCounter() += 3 + peelGraphs[pendingKey].kernels + 1 + (loopKernels[pendingKey] + 1) * (uint64_t)(stats.iterations - 1);
    else
        launchCounter() += (pendingPeeled ? 3 : 0) + 1 + (loopKernels[pendingKey] + 1) * (uint64_t)stats.iterations;
    if (hostSc[11] < 0.0) throw Error(ERR_NAN, "NaN encountered");
    if (hostSc[11] > 0.0) throw Error(ERR_NAN, "NaN encountered at iteration" + std::to_string((int64_t)hostSc[11]));
    stats.relres = stats.bnorm2 > 0 ? std::sqrt(stats.rsq / stats.bnorm2) : std::sqrt(stats.rsq);
    return stats;
}

// MultigridSolver.hh:1047-1152
PcgStats MG::pcgDevice(double *x, const double *b, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps,
                       bool fmg, bool dirichletSatisfied, PcgCallback cb, void *user) {
    syncFineGeom(*this);
    if (useGraphs && deviceLoop && !cb && L() > 1) {
        // one graph launch runs every iteration (conditional WHILE node)
        pcgStart(x, b, maxIter, tol, mgIter, sweeps, fmg, dirichletSatisfied);
        return pcgFinish();
    }
    cudaStream_t st = fine->stream;
    const Geom &g = lv[0].g;
    PcgStats stats;
    if (!dirichletSatisfied) launch_enforce_dirichlet<double>(g, x, fine->dmask.p, fine->dval.p, st);
    launch_masked_dot_partials<double, double>(g, b, b, partials.p, st);
    launch_finalize(partials.p, REDUCE_BLOCKS, sc.p + 7, st);
    const double bnorm2 = readScalar(sc.p + 7, st);
    if (L() > 1) {
        // initial residual through the outer operator, like every later product
        outerMatvecApply(x, rbuf.p, nullptr, b, false);
    } else {
        launch_residual_fine<double>(g, fine->Y.p, x, b, rbuf.p, fine->K0, fine->dmask.p, st);
    }
    launch_masked_dot_partials<double, double>(g, rbuf.p, rbuf.p, partials.p, st);
    launch_finalize(partials.p, REDUCE_BLOCKS, sc.p + 5, st);
    double rsq = readScalar(sc.p + 5, st);
    if (std::isnan(rsq)) throw Error(ERR_NAN, "NaN encountered");
    stats.bnorm2 = bnorm2;

    if (L() == 1) {
        // direct solve branch (MultigridSolver.hh:1056-1064)
        if (!(rsq < tol * tol * bnorm2)) {
            ensureStiffness();
            if (precision == PREC_FP64) launch_coarse_solve<double>(g, Ainv.p, freeIdx.p, nfreeDev.p, nfreeCap, b, x, cscratch.p, st);
            else throw Error(ERR_ARG, "numCoarseningLevels == 0 requires FP64 precision");
            launch_residual_fine<double>(g, fine->Y.p, x, b, rbuf.p, fine->K0, fine->dmask.p, st);
            launch_masked_dot_partials<double, double>(g, rbuf.p, rbuf.p, partials.p, st);
            launch_finalize(partials.p, REDUCE_BLOCKS, sc.p + 5, st);
            rsq = readScalar(sc.p + 5, st);
            stats.iterations = 1;
            if (cb) cb(user, 1, std::sqrt(rsq), x, rbuf.p);
        }
        stats.rsq = rsq;
        stats.relres = bnorm2 > 0 ? std::sqrt(rsq / bnorm2) : std::sqrt(rsq);
        return stats;
    }

    // CG scalars: first-iteration flag set, r.Minv.r = 0
    double init[16] = {0};
    init[5] = rsq;
    init[6] = 1.0;
    init[7] = bnorm2;
    VFEM_CUDA(cudaMemcpyAsync(sc.p, init, sizeof(init), cudaMemcpyHostToDevice, st));
    launch_fill<double>(dvec.p, 0.0, 3 * g.NN, st);
    VFEM_CUDA(cudaStreamSynchronize(st));

    // everything the iteration reads must exist before a graph is captured (no allocation while capturing)
    if (precision == PREC_MIXED) {
        fine->youngF();
        fine->youngFPad();
        const float *yh, *yl;
        if (outerMatvec != MATVEC_FP64) fine->youngDF(&yh, &yl);
        if (outerKind() == 2) umax.alloc(REDUCE_BLOCKS);
        allocLevels();
    }
    prepareFusedInit(mgIter, sweeps);
    const GraphKey key{mgIter, sweeps, fmg ? 1 : 0, symmetricGS ? 1 : 0, precision, outerMatvec};
    bool updated = false;
    int64_t i = 0;
    while ((i++ < maxIter) && (rsq > tol * tol * bnorm2)) {
        if (mgIter > 0 && !updated) {
            ensureStiffness();
            updated = true;
        }
        if (useGraphs) {
            if (graphX != x) clearGraphs();
            auto it = graphs.find(key);
            if (it == graphs.end()) {
                cudaGraph_t graph;
                VFEM_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                try {
                    cgIteration(x, mgIter, sweeps, fmg);
                } catch (...) {
                    cudaStreamEndCapture(st, &graph);
                    throw;
                }
                VFEM_CUDA(cudaStreamEndCapture(st, &graph));
                cudaGraphExec_t exec;
                VFEM_CUDA(cudaGraphInstantiate(&exec, graph, 0));
                size_t nNodes = 0;
                VFEM_CUDA(cudaGraphGetNodes(graph, nullptr, &nNodes));
                std::vector<cudaGraphNode_t> nodes(nNodes);
                VFEM_CUDA(cudaGraphGetNodes(graph, nodes.data(), &nNodes));
                uint64_t kernels = 0;
                for (auto nd : nodes) {
                    cudaGraphNodeType ty;
                    VFEM_CUDA(cudaGraphNodeGetType(nd, &ty));
                    if (ty == cudaGraphNodeTypeKernel) ++kernels;
                }
                cudaGraphDestroy(graph);
                it = graphs.emplace(key, exec).first;
                graphKernels[key] = kernels;
                launchCounter() -= kernels;  // the capture itself launched nothing
                graphX = x;
            }
            VFEM_CUDA(cudaGraphLaunch(it->second, st));
            launchCounter() += graphKernels[key];
        } else {
            cgIteration(x, mgIter, sweeps, fmg);
        }
        VFEM_CUDA(cudaStreamSynchronize(st));
        rsq = hostSc[5];
        if (std::isnan(rsq)) throw Error(ERR_NAN, "NaN encountered at iteration" + std::to_string(i));
        if (cb) {
            if (cb(user, i, std::sqrt(rsq), x, rbuf.p)) break;
        }
    }
    checkTensorStatus();
    stats.iterations = i - 1;
    stats.rsq = rsq;
    stats.relres = bnorm2 > 0 ? std::sqrt(rsq / bnorm2) : std::sqrt(rsq);
    return stats;
}

PcgStats MG::pcg(double *x, const double *b, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps, bool fmg,
                 bool dirichletSatisfied, PcgCallback cb, void *user) {
    cudaStream_t st = fine->stream;
    const int64_t n3 = 3 * fine->g.NN;
    const size_t bytes = n3 * sizeof(double);
    // iterate in an internal buffer so that captured graphs stay valid across calls
    xbuf.alloc(n3);
    const bool bHost = !isDevicePtr(b);
    if (bHost) bbuf.alloc(n3);
    const double *bd = bHost ? bbuf.p : b;
    syncFineGeom(*this);
    if (mgIter > 0 && L() > 1) {
        // the uploads run on a side stream while the Galerkin rebuild (which needs only the
        // densities) runs on the solver stream; the solve waits for both
        if (!copyStream) {
            VFEM_CUDA(cudaStreamCreateWithFlags(&copyStream, cudaStreamNonBlocking));
            VFEM_CUDA(cudaEventCreateWithFlags(&copyDone, cudaEventDisableTiming));
        }
        VFEM_CUDA(cudaMemcpyAsync(xbuf.p, x, bytes, cudaMemcpyDefault, copyStream));
        if (bHost) VFEM_CUDA(cudaMemcpyAsync(bbuf.p, b, bytes, cudaMemcpyHostToDevice, copyStream));
        VFEM_CUDA(cudaEventRecord(copyDone, copyStream));
        // the device-resident solve leaves the rebuild on the side stream (joined before its
        // graph launch); every other path joins it here
        const bool overlap = overlapStiffness && useGraphs && deviceLoop && !cb;
        ensureStiffness(true, overlap);
        VFEM_CUDA(cudaStreamWaitEvent(st, copyDone, 0));
    } else {
        VFEM_CUDA(cudaMemcpyAsync(xbuf.p, x, bytes, cudaMemcpyDefault, st));
        if (bHost) VFEM_CUDA(cudaMemcpyAsync(bbuf.p, b, bytes, cudaMemcpyHostToDevice, st));
    }
    PcgStats stats = pcgDevice(xbuf.p, bd, maxIter, tol, mgIter, sweeps, fmg, dirichletSatisfied, cb, user);
    VFEM_CUDA(cudaMemcpyAsync(x, xbuf.p, bytes, cudaMemcpyDefault, st));
    VFEM_CUDA(cudaStreamSynchronize(st));
    return stats;
}


// ---------------------------------------------------------------------------
// Per-level operations on caller FP64 vectors (MultigridSolver python bindings,
// VoxelFEM.cc:155-195). In mixed precision the level kernels run in FP32.
// ---------------------------------------------------------------------------
enum LevelOpKind { OP_APPLYK = 0, OP_RESIDUAL = 1, OP_SMOOTH = 2, OP_RESTRICT = 3, OP_INTERP = 4, OP_COARSE = 5,
                   OP_ZERODIR = 6 };

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
void MG::applyKLevelT(int l, const T *u, T *out, bool zeroInit, bool negate) {
    cudaStream_t st = fine->stream;
    if (l == 0)
        launch_applyk_fine<T>(lv[0].g, Tr<T>::Yfine(*fine), u, out, Tr<T>::K0(*fine), zeroInit, negate, fine->dmask.p, false,
                              nullptr, 0, st);
    else
        withStencil<T>(l, [&](auto S) {
            launch_stencil_apply<T>(lv[l].g, S, u, out, zeroInit, negate, lv[l].rows, st);
        });
}

template <typename T>
void MG::levelOp(int l, int op, const double *a, const double *b, double *out, bool flag) {
    cudaStream_t st = fine->stream;
    if (l < 0 || l >= L()) throw Error(ERR_ARG, "level out of range");
    if (op == OP_RESTRICT || op == OP_INTERP) {
        if (l + 1 >= L()) throw Error(ERR_ARG, "no coarser level");
    }
    if (l > 0 || op == OP_COARSE || L() == 1) ensureStiffness();
    syncFineGeom(*this);
    allocLevels();
    auto &D = lv[l].data<T>();
    const int64_t n3 = 3 * lv[l].g.NN;
    const uint8_t *dm = (l == 0) ? fine->dmask.p : lv[l].dmask.p;
    switch (op) {
    case OP_APPLYK: {
        toT<T>(a, D.x.p, n3, st);
        applyKLevelT<T>(l, D.x.p, D.r.p, true, false);
        fromT<T>(D.r.p, out, n3, st);
        break;
    }
    case OP_RESIDUAL: {
        toT<T>(a, D.x.p, n3, st);
        toT<T>(b, D.b.p, n3, st);
        residualT<T>(l);
        fromT<T>(D.r.p, out, n3, st);
        break;
    }
    case OP_SMOOTH: {
        toT<T>(a, D.x.p, n3, st);
        toT<T>(b, D.b.p, n3, st);
        smoothT<T>(l, flag);
        fromT<T>(D.x.p, out, n3, st);
        break;
    }
    case OP_RESTRICT: {
        auto &Dc = lv[l + 1].data<T>();
        toT<T>(a, D.r.p, n3, st);
        launch_restrict<T>(lv[l].g, lv[l + 1].g, D.r.p, Dc.b.p, st);
        fromT<T>(Dc.b.p, out, 3 * lv[l + 1].g.NN, st);
        break;
    }
    case OP_INTERP: {
        auto &Dc = lv[l + 1].data<T>();
        toT<T>(a, Dc.x.p, 3 * lv[l + 1].g.NN, st);
        toT<T>(b, D.x.p, n3, st);
        launch_interpolate<T>(lv[l].g, lv[l + 1].g, Dc.x.p, D.x.p, flag, st);
        fromT<T>(D.x.p, out, n3, st);
        break;
    }
    case OP_COARSE: {
        auto &Dc = lv.back().data<T>();
        const int64_t nc = 3 * lv.back().g.NN;
        toT<T>(a, Dc.b.p, nc, st);
        launch_coarse_solve<T>(lv.back().g, Ainv.p, freeIdx.p, nfreeDev.p, nfreeCap, Dc.b.p, Dc.x.p, cscratch.p, st);
        fromT<T>(Dc.x.p, out, nc, st);
        break;
    }
    case OP_ZERODIR: {
        toT<T>(a, D.x.p, n3, st);
        launch_zero_dirichlet<T>(lv[l].g, D.x.p, dm, st);
        fromT<T>(D.x.p, out, n3, st);
        break;
    }
    }
}

static int64_t levelNN(const MG &m, int l) {
    if (l < 0 || l >= m.L()) throw Error(ERR_ARG, "level out of range");
    return m.lv[l].g.NN;
}

#define VFEM_LEVEL_CALL(l, op, A, nA, B, nB, OUT, nOUT, flag)                                                    \
    do {                                                                                                         \
        cudaStream_t st_ = fine->stream;                                                                         \
        View va_, vb_, vo_;                                                                                      \
        viewIn(va_, A, (nA) * sizeof(double), st_);                                                              \
        if (B) viewIn(vb_, B, (nB) * sizeof(double), st_);                                                       \
        viewOut(vo_, OUT, (nOUT) * sizeof(double));                                                              \
        if (precision == PREC_FP64)                                                                              \
            levelOp<double>(l, op, (const double *)va_.d, (const double *)vb_.d, (double *)vo_.d, flag);         \
        else levelOp<float>(l, op, (const double *)va_.d, (const double *)vb_.d, (double *)vo_.d, flag);         \
        finishOut(vo_, st_);                                                                                     \
    } while (0)

void MG::applyK(int l, const double *u, double *out) {
    const int64_t n = 3 * levelNN(*this, l);
    VFEM_LEVEL_CALL(l, OP_APPLYK, u, n, (const double *)nullptr, 0, out, n, false);
}
void MG::residual(int l, const double *u, const double *b, double *r) {
    const int64_t n = 3 * levelNN(*this, l);
    VFEM_LEVEL_CALL(l, OP_RESIDUAL, u, n, b, n, r, n, false);
}
void MG::smooth(int l, double *u, const double *b, bool forward) {
    const int64_t n = 3 * levelNN(*this, l);
    if (l == L() - 1 && L() > 1) throw Error(ERR_ARG, "the coarsest level is solved directly, not smoothed");
    VFEM_LEVEL_CALL(l, OP_SMOOTH, u, n, b, n, u, n, forward);
}
void MG::restrictTo(int l, const double *f, double *c) {
    const int64_t n = 3 * levelNN(*this, l);
    const int64_t nc = 3 * levelNN(*this, l + 1);
    VFEM_LEVEL_CALL(l, OP_RESTRICT, f, n, (const double *)nullptr, 0, c, nc, false);
}
void MG::interpolate(int l, const double *c, double *f, bool accumulate) {
    const int64_t n = 3 * levelNN(*this, l);
    const int64_t nc = 3 * levelNN(*this, l + 1);
    VFEM_LEVEL_CALL(l, OP_INTERP, c, nc, f, n, f, n, accumulate);
}
void MG::coarseSolve(const double *b, double *x) {
    const int64_t n = 3 * levelNN(*this, L() - 1);
    VFEM_LEVEL_CALL(L() - 1, OP_COARSE, b, n, (const double *)nullptr, 0, x, n, false);
}
void MG::zeroDirichlet(int l, double *u) {
    const int64_t n = 3 * levelNN(*this, l);
    VFEM_LEVEL_CALL(l, OP_ZERODIR, u, n, (const double *)nullptr, 0, u, n, false);
}

// MultigridSolver.hh:547-573 (stiffness matrices rebuilt unless unchanged)
void MG::solve(const double *u0, const double *f, int64_t steps, int64_t sweeps, bool zeroDirichletFlag, bool fmg,
               double *out) {
    cudaStream_t st = fine->stream;
    const int64_t n3 = 3 * fine->g.NN;
    View vu, vf, vo;
    viewIn(vu, u0, n3 * sizeof(double), st);
    viewIn(vf, f, n3 * sizeof(double), st);
    viewOut(vo, out, n3 * sizeof(double));
    ensureStiffness();
    syncFineGeom(*this);
    allocLevels();
    auto run = [&](auto tag) {
        using T = decltype(tag);
        auto &D = lv[0].data<T>();
        toT<T>((const double *)vu.d, D.x.p, n3, st);
        if (steps > 0) {
            toT<T>((const double *)vf.d, D.b.p, n3, st);
            if (fmg) {
                fmgT<T>(0, sweeps, zeroDirichletFlag);
                for (int64_t i = 1; i < steps; ++i) vcycleT<T>(0, sweeps, zeroDirichletFlag);
            } else {
                for (int64_t i = 0; i < steps; ++i) vcycleT<T>(0, sweeps, zeroDirichletFlag);
            }
        }
        fromT<T>(D.x.p, (double *)vo.d, n3, st);
    };
    if (precision == PREC_FP64) run(double());
    else run(float());
    finishOut(vo, st);
}

// ---------------------------------------------------------------------------
// Problem: MG compliance objective + filter chain + total volume constraint
// ---------------------------------------------------------------------------
namespace {
struct Backend3D : ProblemBackend {
    MG *mg;
    Grid *grid;
    explicit Backend3D(MG *m) : mg(m), grid(m->fine) {}
    int64_t numElems() const override { return grid->g.NE; }
    int64_t numDofs() const override { return 3 * grid->g.NN; }
    void filterDims(int dims[3], int &ndim) const override {
        for (int d = 0; d < 3; ++d) dims[d] = grid->g.ne[d];
        ndim = 3;
    }
    cudaStream_t stream() const override { return grid->stream; }
    void buildLoad(double *f) override { grid->buildLoadDev(f); }
    void setPhysical(const double *rho) override {
        VFEM_CUDA(cudaMemcpyAsync(grid->rho.p, rho, grid->g.NE * sizeof(double), cudaMemcpyDeviceToDevice,
                                  grid->stream));
        grid->updateYoungModuli();
    }
    PcgStats solve(double *u, const double *f, int64_t cgIter, double tol, int64_t mgIter, int64_t sweeps,
                   bool fmg) override {
        VFEM_CUDA(cudaStreamSynchronize(grid->stream));
        return mg->pcgDevice(u, f, cgIter, tol, mgIter, sweeps, fmg, false, nullptr, nullptr);
    }
    double dotAll(const double *a, const double *b, double *partials) override {
        cudaStream_t st = grid->stream;
        Geom gall = grid->g;
        gall.firstDetN = (int)LAYER_MASK_NONE;  // every node, whatever the fabrication mask
        gall.dyn = nullptr;
        launch_masked_dot_partials<double, double>(gall, a, b, partials, st);
        launch_finalize(partials, REDUCE_BLOCKS, partials + REDUCE_BLOCKS, st);
        double v = 0;
        VFEM_CUDA(cudaMemcpyAsync(&v, partials + REDUCE_BLOCKS, sizeof(double), cudaMemcpyDeviceToHost, st));
        VFEM_CUDA(cudaStreamSynchronize(st));
        return v;
    }
    void complianceGradient(const double *u, double *out) override {
        launch_compliance_gradient(grid->g, grid->rho.p, u, out, grid->K0, grid->E0, grid->Emin, grid->gamma, grid->q,
                                   grid->law, grid->grav, grid->vol(), grid->stream);
    }
};
}  // namespace

std::unique_ptr<ProblemBackend> makeBackend(MG *mg) { return std::unique_ptr<ProblemBackend>(new Backend3D(mg)); }

Problem::Problem(MG *mg_, const std::vector<FilterSpec> &filters_, double volfrac_)
    : Problem(makeBackend(mg_), filters_, volfrac_) {}

Problem::Problem(std::unique_ptr<ProblemBackend> be_, const std::vector<FilterSpec> &filters_, double volfrac_)
    : be(std::move(be_)), filters(filters_), volfrac(volfrac_) {
    for (const auto &f : filters) {
        if (f.kind == 0 && f.radius < 0) throw Error(ERR_ARG, "negative filter radius");
        if (f.kind == 1 && !(f.beta > 0)) throw Error(ERR_ARG, "Beta parameter has to be positive");
        if (f.kind != 0 && f.kind != 1) throw Error(ERR_ARG, "unknown filter kind");
    }
    const int64_t ne = be->numElems(), nd = be->numDofs();
    vars.resize(filters.size() + 1);
    for (auto &v : vars) v.alloc(ne);
    f.alloc(nd);
    u.alloc(nd);
    gradBuf.alloc(ne);
    scratch.alloc(ne);
    scratch2.alloc(ne);
    stepped.alloc(ne);
    x0.alloc(ne);
    dJ.alloc(ne);
    dc.alloc(ne);
    partials.alloc(REDUCE_BLOCKS + 8);
    // the load is fixed when the objective is built (TopologyOptimizationObjective.hh:34-37)
    be->buildLoad(f.p);
    launch_fill<double>(u.p, 0.0, nd, be->stream());
    VFEM_CUDA(cudaStreamSynchronize(be->stream()));
}

void Problem::applyFilter(const FilterSpec &fs, const double *in, double *out) {
    int dims[3], nd;
    be->filterDims(dims, nd);
    if (fs.kind == 0) launch_smoothing_filter(dims, fs.radius, fs.type, in, out, be->stream(), nd);
    else launch_projection(be->numElems(), fs.beta, in, out, be->stream());
}

void Problem::filterApply(const double *x, double *out) {
    cudaStream_t st = be->stream();
    const int64_t ne = be->numElems();
    if (filters.empty()) {
        VFEM_CUDA(cudaMemcpyAsync(out, x, ne * sizeof(double), cudaMemcpyDeviceToDevice, st));
        return;
    }
    const double *src = x;
    for (size_t i = 0; i < filters.size(); ++i) {
        double *dst = (i + 1 == filters.size()) ? out : ((i % 2 == 0) ? scratch.p : scratch2.p);
        applyFilter(filters[i], src, dst);
        src = dst;
    }
}

// FilterChain::backprop (TopologyOptimizationFilter.hh:162-175); g is overwritten.
void Problem::backprop(double *g) {
    cudaStream_t st = be->stream();
    const int64_t ne = be->numElems();
    int dims[3], nd;
    be->filterDims(dims, nd);
    for (size_t i = filters.size(); i-- > 0;) {
        if (filters[i].kind == 0) launch_smoothing_filter(dims, filters[i].radius, filters[i].type, g, scratch.p, st, nd);
        else launch_projection_backprop(ne, filters[i].beta, g, vars[i].p, scratch.p, st);
        VFEM_CUDA(cudaMemcpyAsync(g, scratch.p, ne * sizeof(double), cudaMemcpyDeviceToDevice, st));
    }
}

double Problem::meanDev(const double *x) {
    cudaStream_t st = be->stream();
    launch_sum_partials(x, be->numElems(), partials.p, st);
    launch_finalize(partials.p, REDUCE_BLOCKS, partials.p + REDUCE_BLOCKS, st);
    double v = 0;
    VFEM_CUDA(cudaMemcpyAsync(&v, partials.p + REDUCE_BLOCKS, sizeof(double), cudaMemcpyDeviceToHost, st));
    VFEM_CUDA(cudaStreamSynchronize(st));
    return v / (double)be->numElems();
}

// TopologyOptimizationProblem.hh:41-50 and MultigridComplianceObjective::updateCache
void Problem::setVars(const double *x, bool /*device*/) {
    cudaStream_t st = be->stream();
    const int64_t ne = be->numElems();
    VFEM_CUDA(cudaMemcpyAsync(vars[0].p, x, ne * sizeof(double), cudaMemcpyDefault, st));
    for (size_t i = 0; i < filters.size(); ++i) applyFilter(filters[i], vars[i].p, vars[i + 1].p);
    be->setPhysical(vars.back().p);
    if (zeroInit) launch_fill<double>(u.p, 0.0, be->numDofs(), st);
    lastStats = be->solve(u.p, f.p, cgIter, tol, mgIter, mgSweeps, fmg);
    varsSet = true;
}

double Problem::objective() {
    if (!varsSet) throw Error(ERR_STATE, "Must call setVars first!");
    // 0.5 f.u over all nodes (TopologyOptimizationObjective.hh:41-43)
    return 0.5 * be->dotAll(f.p, u.p, partials.p);
}

void Problem::gradientDev(double *out) {
    be->complianceGradient(u.p, out);
    backprop(out);
}

void Problem::gradient(double *out, bool /*device*/) {
    if (!varsSet) throw Error(ERR_STATE, "Must call setVars first!");
    gradientDev(gradBuf.p);
    VFEM_CUDA(cudaMemcpyAsync(out, gradBuf.p, be->numElems() * sizeof(double), cudaMemcpyDefault, be->stream()));
    VFEM_CUDA(cudaStreamSynchronize(be->stream()));
}

double Problem::constraint() {
    if (!varsSet) throw Error(ERR_STATE, "Must call setVars first!");
    return 1.0 - meanDev(vars.back().p) / volfrac;
}

void Problem::jacobianDev(double *out) {
    launch_fill<double>(out, -1.0 / (volfrac * (double)be->numElems()), be->numElems(), be->stream());
    backprop(out);
}

void Problem::jacobian(double *out, bool /*device*/) {
    if (!varsSet) throw Error(ERR_STATE, "Must call setVars first!");
    jacobianDev(gradBuf.p);
    VFEM_CUDA(cudaMemcpyAsync(out, gradBuf.p, be->numElems() * sizeof(double), cudaMemcpyDefault, be->stream()));
    VFEM_CUDA(cudaStreamSynchronize(be->stream()));
}

// TopologyOptimizationProblem::evaluateOCConstraintAtVars (TopologyOptimizationProblem.hh:58-66)
double Problem::constraintAtVars(const double *x) {
    filterApply(x, gradBuf.p);
    return 1.0 - meanDev(gradBuf.p) / volfrac;
}

// OptimalityCriterion.hh:51-138
int64_t Problem::ocStep(double m, double p, double ctol, const double *objectiveGradient) {
    if (!varsSet) throw Error(ERR_STATE, "Must call setVars first!");
    cudaStream_t st = be->stream();
    const int64_t ne = be->numElems();
    if (objectiveGradient)
        VFEM_CUDA(cudaMemcpyAsync(dJ.p, objectiveGradient, ne * sizeof(double), cudaMemcpyDefault, st));
    else
        gradientDev(dJ.p);
    jacobianDev(dc.p);
    VFEM_CUDA(cudaMemcpyAsync(x0.p, vars[0].p, ne * sizeof(double), cudaMemcpyDeviceToDevice, st));
    int64_t probes = 0;
    auto ceval = [&](double lambda) {
        ++probes;
        launch_oc_update(ne, x0.p, dJ.p, dc.p, lambda, m, p, stepped.p, st);
        return constraintAtVars(stepped.p);
    };
    const double dilation = 32;
    const int64_t guard = 100;
    double lmid = 0.5 * (lambda_min + lambda_max);
    lambda_max = dilation * lambda_max + (1 - dilation) * lmid;
    lambda_min = std::max(dilation * lambda_min + (1 - dilation) * lmid, 0.01);
    int64_t nit = 0;
    for (; nit < guard; ++nit) {
        if (ceval(lambda_min) < 0) break;
        lambda_max = lambda_min;
        lambda_min /= 2;
    }
    if (nit == guard) throw Error(ERR_STATE, "Bracketing constraint(lambda_min) < 0 failed (100 times).");
    if (nit == 0)
        for (; nit < guard; ++nit) {
            if (ceval(lambda_max) > 0) break;
            lambda_min = lambda_max;
            lambda_max *= 2;
        }
    if (nit == guard) throw Error(ERR_STATE, "Bracketing constraint(lambda_max) > 0 failed (100 times).");
    double viol;
    for (int64_t bis = 0;; ++bis) {
        lmid = 0.5 * (lambda_min + lambda_max);
        viol = ceval(lmid);
        if (std::abs(viol) <= ctol) break;
        if (bis > 2000) throw Error(ERR_STATE, "OC bisection did not reach the constraint tolerance");
        if (viol < 0) lambda_min = lmid;
        if (viol > 0) lambda_max = lmid;
    }
    // stepped holds the accepted update; setVars overwrites scratch buffers, so copy first
    VFEM_CUDA(cudaMemcpyAsync(x0.p, stepped.p, ne * sizeof(double), cudaMemcpyDeviceToDevice, st));
    setVars(x0.p, true);
    return probes;
}

void Problem::getU(double *out, bool /*device*/) {
    VFEM_CUDA(cudaMemcpyAsync(out, u.p, be->numDofs() * sizeof(double), cudaMemcpyDefault, be->stream()));
    VFEM_CUDA(cudaStreamSynchronize(be->stream()));
}

void Problem::getPhysical(double *out, bool /*device*/) {
    VFEM_CUDA(cudaMemcpyAsync(out, vars.back().p, be->numElems() * sizeof(double), cudaMemcpyDefault, be->stream()));
    VFEM_CUDA(cudaStreamSynchronize(be->stream()));
}


// ---------------------------------------------------------------------------
// Benchmark hook: time one hot kernel on the solver stream with CUDA events.
//   0 fine applyK FP64      1 fine applyK FP32     2 fine applyK double-float
//   3 fine GS sweep FP32    4 fine GS sweep FP64   5 fine residual FP32
//   6 level-1 GS sweep FP32 7 level-1 residual FP32
// ---------------------------------------------------------------------------
double MG::kernelBytes(int which) const {
    const double nn = (double)lv[0].g.NN, ne = (double)lv[0].g.NE;
    switch (which) {
    case 0: return 8.0 * (6 * nn + ne);
    case 1: return 4.0 * (6 * nn + ne);
    case 2: case 10: return 8.0 * (6 * nn + ne);
    case 3: return 4.0 * (9 * nn + ne);
    case 4: return 8.0 * (9 * nn + ne);
    case 5: return 4.0 * (9 * nn + ne);
    case 6: case 7: case 8: case 9: {
        // one pass over the level's stencil plus x, b, r (or x read and written)
        const Level &lvl = lv[which >= 8 ? 2 : 1];
        const double n1 = (double)lvl.g.NN;
        return 4.0 * (9 * n1 + (lvl.rows ? 256 : STENCIL_PLANES) * n1);
    }
    }
    return 0;
}

double MG::timeKernel(int which, int reps) {
    if (reps <= 0) throw Error(ERR_ARG, "reps must be positive");
    if ((which == 6 || which == 7) && L() < 3) throw Error(ERR_ARG, "level-1 kernels need at least two coarsenings");
    if ((which == 8 || which == 9) && L() < 4) throw Error(ERR_ARG, "level-2 kernels need at least three coarsenings");
    syncFineGeom(*this);
    cudaStream_t st = fine->stream;
    const Geom &g = lv[0].g;
    const int64_t n3 = 3 * g.NN;
    auto &F = lv[0].d32;
    auto &D = lv[0].d64;
    const bool need32 = which == 1 || which == 3 || which == 5 || (which >= 6 && which <= 9);
    if (need32) {
        if (which >= 6) {
            if (precision != PREC_MIXED) throw Error(ERR_ARG, "level-1 FP32 kernels need mixed precision");
            ensureStiffness();
        }
        for (int l = 0; l < (which >= 8 ? 3 : which >= 6 ? 2 : 1); ++l) {
            auto &Q = lv[l].d32;
            const int64_t m3 = 3 * lv[l].g.NN;
            Q.x.alloc(m3, l == 0 ? lv[0].g.nodeGuard() : 0); Q.b.alloc(m3); Q.r.alloc(m3);
            launch_fill<float>(Q.x.p, 0.5f, m3, st);
            launch_fill<float>(Q.b.p, 1.0f, m3, st);
        }
    } else {
        D.x.alloc(n3); D.b.alloc(n3); D.r.alloc(n3);
        launch_fill<double>(D.x.p, 0.5, n3, st);
        launch_fill<double>(D.b.p, 1.0, n3, st);
        if (which == 2) launch_split_df(D.x.p, dhi.p, dlo.p, n3, st);
        if (which == 10) {
            if (!fine->tcOk) throw Error(ERR_ARG, "K0 has no scaled small-integer form for the tensor-core matvec");
            umax.alloc(REDUCE_BLOCKS);
            launch_absmax_partials(D.x.p, n3, umax.p, st);
        }
    }
    auto run = [&]() {
        switch (which) {
        case 0: launch_applyk_fine<double>(g, fine->Y.p, D.x.p, D.r.p, fine->K0, true, false, fine->dmask.p, false, nullptr, 0, st); break;
        case 1: launch_applyk_fine<float>(g, fine->youngFPad(), F.x.p, F.r.p, fine->K0f, true, false, fine->dmask.p, false, nullptr, 0, st); break;
        case 2: {
            const float *yh, *yl;
            fine->youngDF(&yh, &yl);
            launch_applyk_fine_df(g, yh, yl, dhi.p, dlo.p, D.x.p, D.r.p, fine->K0df, fine->dmask.p, true, nullptr, 0, st);
            break;
        }
        case 10: {
            const float *yh, *yl;
            fine->youngDF(&yh, &yl);
            launch_applyk_fine_tc(g, yh, yl, D.x.p, umax.p, D.r.p, fine->tcB.p, fine->tcScale, fine->dmask.p, true,
                                  nullptr, 0, fine->tcStatus.p, st);
            break;
        }
        case 3: smoothT<float>(0, true); break;
        case 4: smoothT<double>(0, true); break;
        case 5: residualT<float>(0); break;
        case 6: smoothT<float>(1, true); break;
        case 7: residualT<float>(1); break;
        case 8: smoothT<float>(2, true); break;
        case 9: residualT<float>(2); break;
        default: throw Error(ERR_ARG, "unknown kernel id");
        }
    };
    run();  // warm-up
    cudaEvent_t e0, e1;
    VFEM_CUDA(cudaEventCreate(&e0));
    VFEM_CUDA(cudaEventCreate(&e1));
    VFEM_CUDA(cudaEventRecord(e0, st));
    for (int r = 0; r < reps; ++r) run();
    VFEM_CUDA(cudaEventRecord(e1, st));
    VFEM_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    VFEM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms / reps;
}


// ---------------------------------------------------------------------------
// Phase breakdown (benchmark hook)
// ---------------------------------------------------------------------------
std::vector<std::pair<std::string, double>> MG::profile(int64_t mgIter, int64_t sweeps, int reps) {
    if (L() < 2) throw Error(ERR_ARG, "profile needs at least one coarsening level");
    syncFineGeom(*this);
    cudaStream_t st = fine->stream;
    const Geom &g = lv[0].g;
    std::vector<std::pair<std::string, double>> out;
    std::map<std::string, double> acc;
    std::vector<std::string> order;
    cudaEvent_t ev[2];
    VFEM_CUDA(cudaEventCreate(&ev[0]));
    VFEM_CUDA(cudaEventCreate(&ev[1]));
    auto timed = [&](const std::string &name, auto &&fn) {
        VFEM_CUDA(cudaEventRecord(ev[0], st));
        fn();
        VFEM_CUDA(cudaEventRecord(ev[1], st));
        VFEM_CUDA(cudaEventSynchronize(ev[1]));
        float ms = 0;
        VFEM_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        if (!acc.count(name)) order.push_back(name);
        acc[name] += ms;
    };
    // hierarchy rebuild, with the step marks of updateStiffnessT
    for (int r = 0; r < reps; ++r) {
        std::vector<std::pair<std::string, cudaEvent_t>> marks;
        stiffMarks = &marks;
        try {
            timed("galerkin+coarse_inverse", [&] { updateStiffness(); });
        } catch (...) {
            stiffMarks = nullptr;
            throw;
        }
        stiffMarks = nullptr;
        for (size_t q = 1; q < marks.size(); ++q) {
            float ms = 0;
            VFEM_CUDA(cudaEventElapsedTime(&ms, marks[q - 1].second, marks[q].second));
            if (!acc.count(marks[q].first)) order.push_back(marks[q].first);
            acc[marks[q].first] += ms;
        }
        for (auto &m : marks) cudaEventDestroy(m.second);
    }
    if (precision == PREC_MIXED) {
        fine->youngF();
        fine->youngFPad();
        const float *yh, *yl;
        fine->youngDF(&yh, &yl);
    }
    allocLevels();
    launch_fill<double>(rbuf.p, 1e-3, 3 * g.NN, st);
    launch_fill<double>(dvec.p, 0.0, 3 * g.NN, st);
    xbuf.alloc(3 * g.NN);
    launch_fill<double>(xbuf.p, 0.0, 3 * g.NN, st);
    auto body = [&](auto tag) {
        using T = decltype(tag);
        auto &D0 = lv[0].data<T>();
        const int64_t n3 = 3 * g.NN;
        timed("precond:init", [&] {
            launch_fill<T>(D0.x.p, T(0), n3, st);
            if (std::is_same<T, double>::value) launch_copy((double *)D0.b.p, rbuf.p, n3, st);
            else launch_cast<float, double>(rbuf.p, (float *)D0.b.p, n3, st);
        });
        const int ts = std::is_same<T, float>::value ? std::min(tailStart(), L() - 1) : L() - 1;
        for (int l = 0; l < ts; ++l) {
            auto &D = lv[l].data<T>();
            auto &Dc = lv[l + 1].data<T>();
            const uint8_t *dm = (l == 0) ? fine->dmask.p : lv[l].dmask.p;
            const std::string tagl = "L" + std::to_string(l) + ":";
            timed(tagl + "presmooth", [&] {
                launch_zero_dirichlet<T>(lv[l].g, D.x.p, dm, st);
                for (int64_t i = 0; i < sweeps; ++i) smoothT<T>(l, true);
            });
            timed(tagl + "residual", [&] { residualT<T>(l); });
            timed(tagl + "restrict", [&] {
                launch_restrict<T>(lv[l].g, lv[l + 1].g, D.r.p, Dc.b.p, st);
                launch_masked_zero<T>(lv[l + 1].g, Dc.x.p, MARGIN, st);
            });
        }
        if (ts < L() - 1) {
            timed("tail:L" + std::to_string(ts) + "..coarsest (down, dense solve, up)",
                  [&] { vcycleT<T>(ts, sweeps, true); });
        } else {
            auto &Dc = lv.back().data<T>();
            timed("coarsest:solve", [&] {
                launch_coarse_solve<T>(lv.back().g, Ainv.p, freeIdx.p, nfreeDev.p, nfreeCap, Dc.b.p, Dc.x.p, cscratch.p, st);
            });
        }
        for (int l = ts - 1; l >= 0; --l) {
            auto &D = lv[l].data<T>();
            auto &Dc = lv[l + 1].data<T>();
            const std::string tagl = "L" + std::to_string(l) + ":";
            timed(tagl + "interp", [&] { launch_interpolate<T>(lv[l].g, lv[l + 1].g, Dc.x.p, D.x.p, true, st); });
            timed(tagl + "postsmooth", [&] {
                for (int64_t i = 0; i < sweeps; ++i) smoothT<T>(l, !symmetricGS);
            });
        }
        timed("cg:precond_out+beta", [&] {
            launch_cg_precond_out<T>(g, D0.x.p, std::is_same<T, float>::value ? nullptr : s.p, rbuf.p,
                                     fine->dmask.p, partials.p, st);
            launch_cg_beta(partials.p, REDUCE_BLOCKS, sc.p, st);
        });
    };
    VFEM_CUDA(cudaMemsetAsync(sc.p, 0, 16 * sizeof(double), st));
    for (int r = 0; r < reps; ++r) {
        if (precision == PREC_FP64) body(double());
        else body(float());
        timed("cg:direction", [&] { outerDirection(precision == PREC_FP64 ? nullptr : lv[0].d32.x.p); });
        timed("cg:matvec+alpha", [&] {
            const int nb = outerMatvecApply(dvec.p, Ad.p, partials.p, nullptr, true);
            launch_cg_alpha(partials.p, nb, sc.p, st);
        });
        timed("cg:update+rsq", [&] {
            launch_cg_update(g, xbuf.p, rbuf.p, dvec.p, Ad.p, sc.p, partials.p, st);
            launch_cg_rsq(partials.p, REDUCE_BLOCKS, sc.p, nullptr, st);
        });
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    for (const auto &name : order) out.emplace_back(name, acc[name] / reps);
    return out;
}

}  // namespace vfem
