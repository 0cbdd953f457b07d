// Layer-by-layer evaluation (LayerByLayerEvaluator::run, LayerByLayer.hh:223-296): one
// elasticity solve per partial build height l (elements in layers >= l masked, nodes above
// detached), accumulating the compliance f.u over the nondetached nodes and the compliance
// gradient. Every height starts from a zero initial guess, so the solves are independent:
// they are spread over `slots` solver instances (grid copy + multigrid hierarchy + buffers),
// each driving a device-resident PCG loop (one CUDA graph launch per solve, convergence
// decided on the device) on its own stream. Slots run concurrently; the host only refills a
// slot once its solve has finished. slots = 1 is the same work issued one height at a time.
#include <chrono>
#include <thread>

#include "vfem_engine.hpp"

namespace vfem {

namespace {

struct Slot {
    std::unique_ptr<Grid> grid;
    std::unique_ptr<MG> mg;
    DevBuf<double> x, f, gtmp, gacc, cpl;
    cudaEvent_t done = nullptr;
    int64_t idx = -1;
    ~Slot() {
        if (done) cudaEventDestroy(done);
    }
};

struct PinnedDoubles {
    double *p = nullptr;
    explicit PinnedDoubles(size_t n) { VFEM_CUDA(cudaMallocHost(&p, n * sizeof(double))); }
    ~PinnedDoubles() {
        if (p) cudaFreeHost(p);
    }
};

}  // namespace

void lblRun(Grid &src, int coarsenings, const int64_t *layers, int64_t count, int64_t slots, int precision,
            int outerMatvec, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps, bool fmg,
            double *compliance, int64_t *iterations, double *gradSum) {
    if (count <= 0) return;
    const int ny = src.g.ne[BUILD_DIR];
    for (int64_t t = 0; t < count; ++t)
        if (layers[t] < 1 || layers[t] > ny) throw Error(ERR_ARG, "layer height out of range");
    const int64_t ns = std::max<int64_t>(1, std::min<int64_t>(slots, count));
    const int64_t NN = src.g.NN, NE = src.g.NE;
    std::vector<std::unique_ptr<Slot>> S;
    for (int64_t s = 0; s < ns; ++s) {
        auto sl = std::make_unique<Slot>();
        sl->grid = src.clone();
        sl->mg = std::make_unique<MG>(sl->grid.get(), coarsenings);
        sl->mg->setPrecision(precision);
        sl->mg->outerMatvec = outerMatvec;
        sl->x.alloc(3 * NN);
        sl->f.alloc(3 * NN);
        sl->gtmp.alloc(NE);
        sl->gacc.alloc(NE);
        sl->cpl.alloc(1);
        VFEM_CUDA(cudaMemsetAsync(sl->gacc.p, 0, NE * sizeof(double), sl->grid->stream));
        VFEM_CUDA(cudaEventCreateWithFlags(&sl->done, cudaEventDisableTiming));
        S.push_back(std::move(sl));
    }
    PinnedDoubles cplHost(ns);

    auto start = [&](int64_t s, int64_t idx) {
        Slot &sl = *S[s];
        Grid &g = *sl.grid;
        MG &mg = *sl.mg;
        cudaStream_t st = g.stream;
        mg.setMaskLayer(layers[idx]);
        g.buildLoadAsync(sl.f.p);
        launch_fill<double>(sl.x.p, 0.0, 3 * NN, st);
        mg.pcgStart(sl.x.p, sl.f.p, maxIter, tol, mgIter, sweeps, fmg, true);
        // compliance over the nondetached nodes (maskedNodalDotProduct)
        launch_masked_dot_partials<double, double>(g.g, sl.f.p, sl.x.p, mg.partials.p, st);
        launch_finalize(mg.partials.p, REDUCE_BLOCKS, sl.cpl.p, st);
        VFEM_CUDA(cudaMemcpyAsync(cplHost.p + s, sl.cpl.p, sizeof(double), cudaMemcpyDeviceToHost, st));
        // accumulateComplianceGradient (masked elements contribute zero)
        launch_compliance_gradient(g.g, g.rho.p, sl.x.p, sl.gtmp.p, g.K0, g.E0, g.Emin, g.gamma, g.q, g.law, g.grav,
                                   g.vol(), st);
        launch_axpy(NE, 1.0, sl.gtmp.p, sl.gacc.p, st);
        VFEM_CUDA(cudaEventRecord(sl.done, st));
        sl.idx = idx;
    };

    int64_t next = 0, remaining = count;
    for (int64_t s = 0; s < ns && next < count; ++s) start(s, next++);
    while (remaining > 0) {
        bool progressed = false;
        for (int64_t s = 0; s < ns; ++s) {
            Slot &sl = *S[s];
            if (sl.idx < 0) continue;
            const cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaErrorNotReady) continue;
            VFEM_CUDA(q);
            const PcgStats st = sl.mg->pcgFinish();
            compliance[sl.idx] = cplHost.p[s];
            if (iterations) iterations[sl.idx] = st.iterations;
            sl.idx = -1;
            --remaining;
            progressed = true;
            if (next < count) start(s, next++);
        }
        if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    if (gradSum) {
        Slot &s0 = *S[0];
        cudaStream_t st = s0.grid->stream;
        for (int64_t s = 1; s < ns; ++s) {
            VFEM_CUDA(cudaStreamSynchronize(S[s]->grid->stream));
            launch_axpy(NE, 1.0, S[s]->gacc.p, s0.gacc.p, st);
        }
        VFEM_CUDA(cudaMemcpyAsync(gradSum, s0.gacc.p, NE * sizeof(double), cudaMemcpyDefault, st));
        VFEM_CUDA(cudaStreamSynchronize(st));
    }
    for (auto &sl : S) VFEM_CUDA(cudaStreamSynchronize(sl->grid->stream));
}

}  // namespace vfem
