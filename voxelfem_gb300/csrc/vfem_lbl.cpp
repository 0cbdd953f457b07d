// Layer-by-layer evaluation (LayerByLayerEvaluator::run, LayerByLayer.hh:223-296): one
// elasticity solve per partial build height l (elements in layers >= l masked, nodes above
// detached), accumulating the compliance f.u over the nondetached nodes and the compliance
// gradient. The solves run on `slots` persistent solver instances (grid copy + multigrid
// hierarchy + buffers), each driving a device-resident PCG loop (one CUDA graph launch per
// solve, convergence decided on the device, graph valid for every mask height) on its own
// stream; the host refills a slot once its solve has finished. With zero initial guesses the
// heights are independent and spread over the slots. With the warm-start generators
// (LayerByLayer.hh:55-209; the initial guess combines the chain's previous solutions, formed on
// the device) each slot solves a contiguous chain of heights in order; one slot reproduces the
// reference's sequential algorithm.
#include <algorithm>
#include <chrono>
#include <thread>

#include "vfem_engine.hpp"

namespace vfem {

LBL::Slot::~Slot() {
    if (done) cudaEventDestroy(done);
}

LBL::LBL(Grid *src_, int coarsenings_, int64_t slots, int precision_)
    : src(src_), coarsenings(coarsenings_), precision(precision_) {
    if (coarsenings < 1) throw Error(ERR_ARG, "layer-by-layer solves need at least one coarsening level");
    if (precision != PREC_FP64 && precision != PREC_MIXED) throw Error(ERR_ARG, "unknown precision");
    if (slots < 1) throw Error(ERR_ARG, "slots must be positive");
    const int64_t NN = src->g.NN, NE = src->g.NE;
    for (int64_t s = 0; s < slots; ++s) {
        auto sl = std::make_unique<Slot>();
        sl->grid = src->clone();
        sl->mg = std::make_unique<MG>(sl->grid.get(), coarsenings);
        sl->mg->setPrecision(precision);
        // concurrent slots already fill the GPU while one slot's hierarchy is rebuilt: splitting
        // the first iteration around the rebuild then only costs (128 heights at 128^3, 4 slots:
        // 2.00 s split, 1.89 s not)
        if (slots > 1) sl->mg->peelFirst = false;
        sl->x.alloc(3 * NN);
        sl->f.alloc(3 * NN);
        sl->gtmp.alloc(NE);
        sl->gacc.alloc(NE);
        sl->cpl.alloc(1);
        VFEM_CUDA(cudaEventCreateWithFlags(&sl->done, cudaEventDisableTiming));
        S.push_back(std::move(sl));
    }
    VFEM_CUDA(cudaMallocHost(&cplHost, slots * sizeof(double)));
}

LBL::~LBL() {
    for (auto &sl : S) cudaStreamSynchronize(sl->grid->stream);
    if (cplHost) cudaFreeHost(cplHost);
}

// Bring every slot's grid to the source's current densities, material, loads and supports.
void LBL::syncSource() {
    VFEM_CUDA(cudaStreamSynchronize(src->stream));
    for (auto &sl : S) {
        Grid &g = *sl->grid;
        if (g.Eyoung != src->Eyoung || g.nu != src->nu) g.setETensor(src->Eyoung, src->nu);
        g.E0 = src->E0;
        g.Emin = src->Emin;
        g.gamma = src->gamma;
        g.q = src->q;
        g.law = src->law;
        for (int d = 0; d < 3; ++d) g.grav[d] = src->grav[d];
        if (g.force_h != src->force_h) {
            g.force_h = src->force_h;
            g.forceDevValid = false;
        }
        if (g.dmask_h != src->dmask_h || g.dval_h != src->dval_h) {
            throw Error(ERR_STATE, "supports changed after the layer-by-layer evaluator was created");
        }
        VFEM_CUDA(cudaMemcpyAsync(g.rho.p, src->rho.p, src->g.NE * sizeof(double), cudaMemcpyDeviceToDevice, g.stream));
        g.updateYoungModuli();
        ++g.densVersion;
    }
}

void LBL::setSweepForm(int form) {
    for (auto &sl : S) sl->mg->setSweepForm(form);
}

void LBL::setInit(int kind, int history) {
    if (kind < LBL_INIT_ZERO || kind > LBL_INIT_SUBSPACE) throw Error(ERR_ARG, "Unrecognized init method");
    if (kind == LBL_INIT_SUBSPACE && (history < 1 || history > LBL_MAX_HISTORY))
        throw Error(ERR_ARG, "subspace size must lie in 1.." + std::to_string(LBL_MAX_HISTORY));
    initKind = kind;
    historySize = kind == LBL_INIT_CONSTANT ? 1 : kind == LBL_INIT_FD ? 2 : kind == LBL_INIT_SUBSPACE ? history : 0;
}

// The slot's initial guess for `layer` into sl.x (mask and load of the layer already set).
void LBL::guess(Slot &sl, int64_t layer, int ny, bool zeroInit) {
    Grid &g = *sl.grid;
    MG &mg = *sl.mg;
    cudaStream_t st = g.stream;
    const int64_t n3 = 3 * g.g.NN;
    if (!zeroInit && layer == ny && haveFull) {
        VFEM_CUDA(cudaMemcpyAsync(sl.x.p, uFull.p, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
        return;
    }
    const int hs = sl.hs;
    LblVectors U{};
    for (int i = 0; i < hs; ++i) U.u[i] = sl.hist[sl.order[i]].p;
    LblCoeffs cv{};
    if (initKind == LBL_INIT_ZERO || hs == 0) {
        launch_fill<double>(sl.x.p, 0.0, n3, st);
    } else if (initKind == LBL_INIT_CONSTANT || (initKind == LBL_INIT_FD && hs == 1)) {
        cv.c[0] = 1.0;  // InitGenFD with one solution: copy it
        launch_subspace_combine(g.g, U, 1, nullptr, cv, sl.x.p, st);
    } else if (initKind == LBL_INIT_FD) {
        cv.c[0] = 2.0;  // g = 2 u(0) - u(1)
        cv.c[1] = -1.0;
        launch_subspace_combine(g.g, U, 2, nullptr, cv, sl.x.p, st);
    } else {
        // InitGenSubspace: A_ij = u_i . K u_j, b_i = u_i . f over the nondetached nodes
        const int np = hs * (hs + 1) / 2 + hs;
        sl.subPart.alloc((int64_t)np * REDUCE_BLOCKS);
        sl.subC.alloc(LBL_MAX_HISTORY);
        for (int j = 0; j < hs; ++j) {
            sl.Ku[j].alloc(n3);
            mg.outerMatvecApply(U.u[j], sl.Ku[j].p, nullptr, nullptr, false);
        }
        int p = 0;
        for (int i = 0; i < hs; ++i)
            for (int j = i; j < hs; ++j, ++p)
                launch_masked_dot_partials<double, double>(g.g, U.u[i], sl.Ku[j].p, sl.subPart.p + (int64_t)p * REDUCE_BLOCKS,
                                                           st);
        for (int i = 0; i < hs; ++i, ++p)
            launch_masked_dot_partials<double, double>(g.g, U.u[i], sl.f.p, sl.subPart.p + (int64_t)p * REDUCE_BLOCKS, st);
        launch_subspace_solve(sl.subPart.p, REDUCE_BLOCKS, hs, sl.subC.p, st);
        launch_subspace_combine(g.g, U, hs, sl.subC.p, cv, sl.x.p, st);
    }
}

// finalizeLayer's history update: the newest solution first, the oldest dropped
void LBL::pushHistory(Slot &sl) {
    if (historySize == 0) return;
    const int64_t n3 = 3 * sl.grid->g.NN;
    int slot;
    if (sl.hs < historySize) {
        slot = sl.hs;
        for (int i = sl.hs; i > 0; --i) sl.order[i] = sl.order[i - 1];
        ++sl.hs;
    } else {
        slot = sl.order[sl.hs - 1];
        for (int i = sl.hs - 1; i > 0; --i) sl.order[i] = sl.order[i - 1];
    }
    sl.order[0] = slot;
    sl.hist[slot].alloc(n3);
    VFEM_CUDA(cudaMemcpyAsync(sl.hist[slot].p, sl.x.p, n3 * sizeof(double), cudaMemcpyDeviceToDevice, sl.grid->stream));
}

void LBL::run(const int64_t *layers, int64_t count, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps,
              bool fmg, bool zeroInit, double *compliance, int64_t *iterations, double *gradSum) {
    if (count <= 0) return;
    const int ny = src->g.ne[BUILD_DIR];
    for (int64_t t = 0; t < count; ++t)
        if (layers[t] < 1 || layers[t] > ny) throw Error(ERR_ARG, "layer height out of range");
    syncSource();
    const int64_t ns = std::min<int64_t>((int64_t)S.size(), count);
    const int64_t NN = src->g.NN, NE = src->g.NE;
    const bool warm = initKind != LBL_INIT_ZERO;
    for (int64_t s = 0; s < (int64_t)S.size(); ++s) {
        Slot &sl = *S[s];
        sl.queue.clear();
        sl.qpos = 0;
        sl.hs = 0;
        sl.idx = -1;
    }
    if (warm) {
        // contiguous chains, the first ones one height longer when count % ns != 0
        int64_t t = 0;
        for (int64_t s = 0; s < ns; ++s) {
            const int64_t len = count / ns + (s < count % ns ? 1 : 0);
            for (int64_t k = 0; k < len; ++k) S[s]->queue.push_back(t++);
        }
    }
    for (int64_t s = 0; s < ns; ++s)
        VFEM_CUDA(cudaMemsetAsync(S[s]->gacc.p, 0, NE * sizeof(double), S[s]->grid->stream));
    if (!zeroInit && !uFull.p) uFull.alloc(3 * NN);

    auto start = [&](int64_t s, int64_t idx) {
        Slot &sl = *S[s];
        Grid &g = *sl.grid;
        MG &mg = *sl.mg;
        cudaStream_t st = g.stream;
        mg.setMaskLayer(layers[idx]);
        g.buildLoadAsync(sl.f.p);
        guess(sl, layers[idx], ny, zeroInit);
        // the guess satisfies the (zero) supports already
        mg.pcgStart(sl.x.p, sl.f.p, maxIter, tol, mgIter, sweeps, fmg, true);
        // compliance over the nondetached nodes (maskedNodalDotProduct)
        launch_masked_dot_partials<double, double>(g.g, sl.f.p, sl.x.p, mg.partials.p, st);
        launch_finalize(mg.partials.p, REDUCE_BLOCKS, sl.cpl.p, st);
        VFEM_CUDA(cudaMemcpyAsync(cplHost + s, sl.cpl.p, sizeof(double), cudaMemcpyDeviceToHost, st));
        // accumulateComplianceGradient (masked elements contribute zero)
        launch_compliance_gradient(g.g, g.rho.p, sl.x.p, sl.gtmp.p, g.K0, g.E0, g.Emin, g.gamma, g.q, g.law, g.grav,
                                   g.vol(), st);
        launch_axpy(NE, 1.0, sl.gtmp.p, sl.gacc.p, st);
        if (layers[idx] == ny) {
            if (!uFull.p) uFull.alloc(3 * NN);
            VFEM_CUDA(cudaMemcpyAsync(uFull.p, sl.x.p, 3 * NN * sizeof(double), cudaMemcpyDeviceToDevice, st));
        }
        if (warm && sl.qpos < sl.queue.size()) pushHistory(sl);  // another height follows in this chain
        VFEM_CUDA(cudaEventRecord(sl.done, st));
        sl.idx = idx;
    };
    auto nextOf = [&](int64_t s, int64_t &next) -> int64_t {
        Slot &sl = *S[s];
        if (warm) return sl.qpos < sl.queue.size() ? sl.queue[sl.qpos++] : -1;
        return next < count ? next++ : -1;
    };

    int64_t next = 0, remaining = count;
    for (int64_t s = 0; s < ns; ++s) {
        const int64_t idx = nextOf(s, next);
        if (idx >= 0) start(s, idx);
    }
    while (remaining > 0) {
        bool progressed = false;
        for (int64_t s = 0; s < ns; ++s) {
            Slot &sl = *S[s];
            if (sl.idx < 0) continue;
            const cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaErrorNotReady) continue;
            VFEM_CUDA(q);
            const PcgStats st = sl.mg->pcgFinish();
            compliance[sl.idx] = cplHost[s];
            if (iterations) iterations[sl.idx] = st.iterations;
            sl.idx = -1;
            --remaining;
            progressed = true;
            const int64_t idx = nextOf(s, next);
            if (idx >= 0) start(s, idx);
        }
        if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    haveFull = haveFull || std::find(layers, layers + count, (int64_t)ny) != layers + count;
    if (gradSum) {
        Slot &s0 = *S[0];
        cudaStream_t st = s0.grid->stream;
        for (int64_t s = 1; s < ns; ++s) {
            VFEM_CUDA(cudaStreamSynchronize(S[s]->grid->stream));
            launch_axpy(NE, 1.0, S[s]->gacc.p, s0.gacc.p, st);
        }
        VFEM_CUDA(cudaMemcpyAsync(gradSum, s0.gacc.p, NE * sizeof(double), cudaMemcpyDefault, st));
    }
    for (auto &sl : S) VFEM_CUDA(cudaStreamSynchronize(sl->grid->stream));
}

}  // namespace vfem
