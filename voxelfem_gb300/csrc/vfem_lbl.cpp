// Layer-by-layer evaluation (LayerByLayerEvaluator::run, LayerByLayer.hh:223-296): one
// elasticity solve per partial build height l (elements in layers >= l masked, nodes above
// detached), accumulating the compliance f.u over the nondetached nodes and the compliance
// gradient. Every height starts from a zero initial guess, so the solves are independent:
// they are spread over `slots` persistent solver instances (grid copy + multigrid hierarchy +
// buffers), each driving a device-resident PCG loop (one CUDA graph launch per solve,
// convergence decided on the device, graph valid for every mask height) on its own stream.
// Slots run concurrently; the host refills a slot once its solve has finished. One slot is the
// same work issued one height at a time.
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

void LBL::run(const int64_t *layers, int64_t count, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps,
              bool fmg, double *compliance, int64_t *iterations, double *gradSum) {
    if (count <= 0) return;
    const int ny = src->g.ne[BUILD_DIR];
    for (int64_t t = 0; t < count; ++t)
        if (layers[t] < 1 || layers[t] > ny) throw Error(ERR_ARG, "layer height out of range");
    syncSource();
    const int64_t ns = std::min<int64_t>((int64_t)S.size(), count);
    const int64_t NN = src->g.NN, NE = src->g.NE;
    for (int64_t s = 0; s < ns; ++s)
        VFEM_CUDA(cudaMemsetAsync(S[s]->gacc.p, 0, NE * sizeof(double), S[s]->grid->stream));

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
        VFEM_CUDA(cudaMemcpyAsync(cplHost + s, sl.cpl.p, sizeof(double), cudaMemcpyDeviceToHost, st));
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
            compliance[sl.idx] = cplHost[s];
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
    }
    for (auto &sl : S) VFEM_CUDA(cudaStreamSynchronize(sl->grid->stream));
}

}  // namespace vfem
