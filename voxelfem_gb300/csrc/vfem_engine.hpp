// Host engine of the GB300 VoxelFEM solve path: the voxel grid (TensorProductSimulator),
// the geometric multigrid hierarchy with its MG-preconditioned CG (MultigridSolver) and
// the topology-optimisation problem with the OC optimiser. All state lives on the device;
// this layer only sequences kernels on one CUDA stream and captures CUDA graphs.
#pragma once
#include <cmath>
#include <limits>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "vfem_common.cuh"
#include "vfem_kernels.hpp"

namespace vfem {

enum Precision { PREC_FP64 = 0, PREC_MIXED = 1 };
// Outer CG matvec of the mixed solve. MATVEC_DF: FP64-class accuracy without FP64 arithmetic,
// on the tensor cores (integer-slice operands) when K0 is a scaled small-integer matrix, else in
// double-float on the FP32 units; MATVEC_DF_SIMT forces the double-float kernel.
enum OuterMatvec { MATVEC_FP64 = 0, MATVEC_DF = 1, MATVEC_DF_SIMT = 2 };

bool isDevicePtr(const void *p);

// Device-accessible view of caller memory; host memory is staged through a device buffer.
struct View {
    void *user = nullptr;
    void *d = nullptr;
    size_t bytes = 0;
    bool staged = false;
    DevBuf<char> tmp;
};
void viewIn(View &v, const void *p, size_t bytes, cudaStream_t st);
void viewOut(View &v, void *p, size_t bytes);
void viewInOut(View &v, void *p, size_t bytes, cudaStream_t st);
void finishOut(View &v, cudaStream_t st);

class Grid {
public:
    Grid(const int ne[3], const double bmin[3], const double bmax[3]);
    ~Grid();
    Grid(const Grid &) = delete;
    Grid &operator=(const Grid &) = delete;

    Geom g;
    double bmin[3], bmax[3], h[3];
    double Eyoung = 1.0, nu = 0.0;  // ETensor(1, 0) default (TensorProductSimulator.hh:2114)
    Mat24<double> K0;
    Mat24<float> K0f;
    Mat24DF K0df;
    // K0 = tcScale * C with C a small-integer matrix: bf16 B tiles of the tensor-core matvec
    bool tcOk = false;
    double tcScale = 0.0;
    std::vector<uint16_t> tcTiles;
    DevBuf<uint16_t> tcB;
    DevBuf<int> tcStatus;  // nonzero: a tensor-core wait timed out
    double E0 = 1.0, Emin = 1e-4, gamma = 3.0, q = 3.0;  // TensorProductSimulator.hh:2137-2141
    int law = 0;                                          // 0 SIMP, 1 RAMP
    double maskH = std::numeric_limits<double>::infinity();
    double grav[3] = {0, 0, 0};

    DevBuf<double> rho, Y;
    DevBuf<float> Yf, Yfp, Yhi, Ylo;  // FP32 moduli; zero-padded FP32; zero-padded double-float pair
    bool YfValid = false, YfpValid = false, YdfValid = false;
    std::vector<uint8_t> dmask_h;
    std::vector<double> dval_h;   // SoA, stride NN
    std::vector<double> force_h;  // dense nodal forces, SoA
    DevBuf<int> dynMask;  // device {firstMaskedE, firstDetN} (Geom::dyn)
    void uploadMask();
    DevBuf<uint8_t> dmask;
    DevBuf<double> dval;
    bool dvalNonzero = false;
    uint64_t densVersion = 1, bcVersion = 1, maskVersion = 1, k0Version = 1;
    // bumped by every change of the moduli except a fabrication-mask change (densities, material,
    // interpolation parameters, K0): a mask-only change allows a band-partial Galerkin update
    uint64_t materialVersion = 1;
    cudaStream_t stream = nullptr;

    void setETensor(double E, double nu);
    void setParams(double E0_, double Emin_, double gamma_, double q_, int law_);
    void setDensities(const double *rho, bool checkRange);
    void setUniformDensities(double v);
    void getDensities(double *out);
    void getYoungModuli(double *out);
    void updateYoungModuli(bool maskOnly = false);
    const float *youngFPad();  // zero-padded FP32 moduli (Geom::padElem layout)
    const float *youngF();
    void youngDF(const float **hi, const float **lo);  // double-float split of Y
    void addDirichlet(const double u[3], const double mn[3], const double mx[3], unsigned cmask);
    void applySymmetry(const int axes[3], const int maxFace[3]);
    void setForces(const double *f);
    void getDirichletMask(uint8_t *out) const;
    void setGravity(const double gv[3]);
    void setMaskLayer(int64_t l);
    void setMaskHeight(double hgt, bool update);
    void applyK(const double *u, double *out);
    void buildLoad(double *out);
    void complianceGradient(const double *u, double *out);
    void adjointSensitivity(const double *lam, const double *u, double wF, double wK, double *out);
    void elementEnergy(const double *u, double *out);
    double vol() const { return h[0] * h[1] * h[2]; }

    // device-side helpers
    void buildLoadDev(double *f_dev);
    void buildLoadAsync(double *f_dev);  // stream-ordered, no host synchronisation
    void uploadBC();
    DevBuf<double> forceDev;  // device copy of force_h (refreshed by setForces)
    bool forceDevValid = false;
    // a new grid with the same geometry, material, densities, boundary conditions, loads and mask
    std::unique_ptr<Grid> clone() const;
};

template <typename T>
struct LevelData {
    DevBuf<T> x, b, r, S, Ke;
    DevBuf<__nv_bfloat16> Sh;  // the stencil in bf16 (FP32 smoothing levels with bf16 stencils)
};

struct Level {
    Geom g;
    double h[3];
    bool rows = true;  // stencil layout: node-contiguous rows (small levels) or planes (large)
    std::vector<uint8_t> dmask_h;
    DevBuf<uint8_t> dmask;
    DevBuf<int> dyn;  // device {firstMaskedE, firstDetN} (Geom::dyn)
    LevelData<double> d64;
    LevelData<float> d32;
    template <typename T>
    LevelData<T> &data();
};
template <>
inline LevelData<double> &Level::data<double>() { return d64; }
template <>
inline LevelData<float> &Level::data<float>() { return d32; }

struct PcgStats {
    int64_t iterations = 0;
    double relres = 0;
    double rsq = 0, bnorm2 = 0;
    int status = 0;
};

using PcgCallback = int (*)(void *user, int64_t it, double rnorm, const double *x_dev, const double *r_dev);

class MG {
public:
    MG(Grid *fine, int coarsenings);
    ~MG();
    MG(const MG &) = delete;
    MG &operator=(const MG &) = delete;

    Grid *fine;
    std::vector<Level> lv;
    int precision = PREC_FP64;
    int outerMatvec = MATVEC_DF;
    bool symmetricGS = true;
    bool useGraphs = true;
    // Levels from tailStart to the coarsest run in the single-CTA tail kernels (FP32 V-cycle only;
    // L() when no level is small enough).
    int tailStart() const;
    int64_t tailMaxNodes = 0;
    int64_t rowsMaxNodes = 0;  // levels up to this size store node-contiguous stencil rows (default: none)
    // plane-layout levels up to this size sweep colour pairs on whole z-lines (four launches per
    // sweep instead of eight; VFEM_STENCIL_LINES_MAX_NODES sets it). Off by default: on the
    // 70,785-node level 2 of the 256x128x128 hierarchy a line-pair sweep took 0.049 ms against
    // 0.037 ms for eight colour launches (17-node lines fill half of each 32-node round, and the
    // rounds of a block run one after another).
    int64_t stencilLinesMaxNodes = 0;
    // When set, the stiffness update records a CUDA event after each of its steps (profiling).
    std::vector<std::pair<std::string, cudaEvent_t>> *stiffMarks = nullptr;

    int L() const { return (int)lv.size(); }
    void setPrecision(int p);
    void setMaskLayer(int64_t l);
    // overlap: build on stiffStream (see below) instead of the solver stream. bandLo < bandHi: a
    // band-partial update after a fabrication-mask change (MultigridSolver.hh:907-1017): only the
    // level operators that the fine element rows [bandLo, bandHi) reach are rebuilt (the coarsest
    // inverse is always refactored, as the reference refactors its CHOLMOD factor).
    void updateStiffness(bool overlap = false, int bandLo = -1, int bandHi = -1);
    // band-partial updates are on unless VFEM_BAND_UPDATE=0
    bool bandUpdates = true;
    // form of the FP32 fine Gauss-Seidel sweep (GS_LINES, GS_COLOURS or GS_PLANES; VFEM_GS_MODE
    // gives the default); every form gives identical iterates
    int sweepForm = -1;
    void setSweepForm(int form);
    // Mixed precision: the assembled stencils of the smoothing levels (1 .. L-2, plane layout)
    // stored in bf16, rounded once when built (the operator stays symmetric), read and applied
    // in FP32; the coarsest level stays FP32 for its dense inverse. VFEM_STENCIL_BF16 sets it.
    bool bf16Stencils = false;
    void setBf16Stencils(bool on);
    bool halfStencil(int l) const {
        return precision == PREC_MIXED && bf16Stencils && l >= 1 && l < L() - 1 && !lv[l].rows;
    }
    // fn(S) with the level's stencil pointer in its stored type
    template <typename T, typename F>
    void withStencil(int l, F &&fn) {
        auto &D = lv[l].data<T>();
        if constexpr (std::is_same<T, float>::value) {
            if (halfStencil(l)) {
                fn((const __nv_bfloat16 *)D.Sh.p);
                return;
            }
        }
        fn((const T *)D.S.p);
    }
    int stiffnessMaskE = -1;              // fine masked element row the operators were built for
    // the level operators (levels >= 1) are current for stiffnessMaskE; stiffnessValid also
    // covers the coarsest dense inverse, which a change of the free coarsest DOFs invalidates
    bool levelsValid = false;
    uint64_t stiffnessMaterialVersion = 0;
    int64_t fullRebuilds = 0, bandRebuilds = 0;  // counters (diagnostic)
    // The asynchronous solve rebuilds the hierarchy on side streams: the solve's start (the
    // initial residual through the outer matvec, its norms, the first preconditioner input) and
    // the split first iteration (PeelGraphs) run on the solver stream while the smoothing levels'
    // stencils (evLevelsReady) and the coarsest dense inverse (evCoarseReady, which also covers the
    // stencils) are built; the loop graph follows evCoarseReady. (No wait can sit inside the
    // device-side WHILE loop, whose body admits no event nodes.) VFEM_OVERLAP_STIFFNESS=0 keeps the
    // rebuild on the solver stream.
    cudaStream_t stiffStream = nullptr;
    cudaStream_t stiffStream2 = nullptr;  // the smoothing levels' stencils beside the chain
    std::vector<cudaEvent_t> evKe;        // level l's element matrices written (stiffStream)
    bool twoStreamRebuild = true;         // VFEM_REBUILD_STREAMS=1: the whole rebuild on stiffStream
    cudaEvent_t evStiffFork = nullptr, evLevelsReady = nullptr, evCoarseReady = nullptr;
    bool overlapStiffness = true;
    bool rebuildInFlight = false;  // a side-stream rebuild forked and not yet joined by the solver stream

    // per-level operations on caller FP64 vectors (level sizes)
    void applyK(int l, const double *u, double *out);
    void residual(int l, const double *u, const double *b, double *r);
    void smooth(int l, double *u, const double *b, bool forward);
    void restrictTo(int l, const double *fine, double *coarse);
    void interpolate(int l, const double *coarse, double *fine, bool accumulate);
    void coarseSolve(const double *b, double *x);
    void zeroDirichlet(int l, double *u);
    void solve(const double *u0, const double *f, int64_t steps, int64_t sweeps, bool zeroDirichletFlag, bool fmg,
               double *out);
    PcgStats pcg(double *x, const double *b, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps, bool fmg,
                 bool dirichletSatisfied, PcgCallback cb, void *user);
    // PCG on device-resident FP64 buffers (no staging); used by pcg() and by the problem layer.
    // Asynchronous device-resident PCG (at least one coarsening): pcgStart enqueues the whole
    // solve on the grid's stream (host synchronisation only inside a stiffness update);
    // pcgFinish waits for it and returns the statistics.
    void pcgStart(double *x, const double *b, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps, bool fmg,
                  bool dirichletSatisfied);
    PcgStats pcgFinish();
    bool pending = false;
    PcgStats pcgDevice(double *x, const double *b, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps,
                       bool fmg, bool dirichletSatisfied, PcgCallback cb, void *user);
    double lastTrueRelres = -1;
    // Average device time (ms) of one launch of a hot kernel, timed with CUDA events on the
    // solver stream (benchmark hook).
    double timeKernel(int which, int reps);
    // Sum of algorithmic bytes for the kernels of timeKernel().
    double kernelBytes(int which) const;
    // Warm-cache breakdown of one PCG iteration and of the hierarchy rebuild: (phase, ms) pairs,
    // averaged over reps, each phase bracketed by CUDA events on the solver stream.
    std::vector<std::pair<std::string, double>> profile(int64_t mgIter, int64_t sweeps, int reps);

    // coarsest level
    int nfree = 0, nfreeCap = 0;  // free coarsest DOFs now / allocated for
    DevBuf<int> nfreeDev;          // device copy of nfree (read by the coarse solve)
    DevBuf<int> freeIdx, redIdx;
    DevBuf<double> Ainv, work, cscratch;
    DevBuf<int> status;
    bool stiffnessValid = false;
    int stiffnessPrecision = -1;
    uint64_t stiffnessDensVersion = 0, stiffnessMaskVersion = 0, stiffnessBcVersion = 0;

    // CG workspace
    DevBuf<double> rbuf, s, dvec, Ad, partials, sc, xbuf, bbuf;
    // side stream of the host-buffer solve: its uploads overlap the Galerkin rebuild
    cudaStream_t copyStream = nullptr;
    cudaEvent_t copyDone = nullptr;
    DevBuf<float> dhi, dlo;  // double-float split of the search direction
    DevBuf<double> umax;     // partial maxima of |operand| of the tensor-core matvec
    // kind of the mixed outer matvec in use: 0 FP64, 1 double-float (FP32 units), 2 tensor cores
    int outerKind() const;
    // d = beta d + s with the side outputs the outer matvec needs
    // d = beta d + s; with the FP32 V-cycle iterate given, s is formed from it on the fly
    void outerDirection(const float *precondIterate = nullptr);
    // out = K u (rhs: rhs - K u) with the outer matvec; uReady: u's side data (split or maxima)
    // are current. Returns the number of partial dots written when partialsOut is given.
    int outerMatvecApply(const double *u, double *out, double *partialsOut, const double *rhs, bool uReady);
    void checkTensorStatus();
    // out = K u (rhs: rhs - K u) through the mixed solve's outer matvec on caller vectors
    void outerApply(const double *u, double *out, const double *rhs);
    uint64_t graphK0Version = 0;
    double *hostSc = nullptr;  // pinned mirror of sc
    int partialCount = 0;

    // Galerkin constants
    DevBuf<double> Kc64, K2_64, phis64;
    DevBuf<float> Kc32, K2_32, phis32;

    // CUDA graphs of one preconditioned CG iteration, keyed by solver options
    struct GraphKey {
        int64_t mgIter, sweeps;
        int fmg, sym, prec, matvec;
        bool operator<(const GraphKey &o) const {
            return std::tie(mgIter, sweeps, fmg, sym, prec, matvec) <
                   std::tie(o.mgIter, o.sweeps, o.fmg, o.sym, o.prec, o.matvec);
        }
    };
    GraphKey pendingKey{};  // graph of the solve in flight
    std::map<GraphKey, cudaGraphExec_t> graphs;
    std::map<GraphKey, uint64_t> graphKernels;  // kernel nodes per captured graph
    // device-resident PCG: a graph whose conditional WHILE node repeats one iteration until
    // convergence, so a solve is one graph launch with no host round trip per iteration
    std::map<GraphKey, cudaGraphExec_t> loopGraphs;
    std::map<GraphKey, uint64_t> loopKernels;  // kernel nodes per loop body
    bool deviceLoop = true;
    cudaGraphExec_t loopGraph(const GraphKey &key, double *x, int64_t mgIter, int64_t sweeps, bool fmg);
    const double *graphX = nullptr;  // buffers baked into captured graphs
    void clearGraphs();
    // The first iteration of a mixed solve whose hierarchy is being rebuilt on the side stream
    // runs as three graphs split where the rebuild's events are joined: level 0's down leg (needs
    // nothing rebuilt), the down legs below it (after evLevelsReady), and the coarsest solve, the
    // up legs and the rest of the iteration (after evCoarseReady); the device-resident loop
    // follows. Each graph runs its part under an IF node that holds the loop's own condition, so
    // the iterates and the iteration count are those of the single loop graph.
    // VFEM_PEEL_FIRST=0 keeps the single graph.
    struct PeelGraphs {
        cudaGraphExec_t part[3] = {nullptr, nullptr, nullptr};
        uint64_t kernels = 0;  // kernel nodes of the three IF bodies
    };
    std::map<GraphKey, PeelGraphs> peelGraphs;
    bool peelFirst = true;
    bool pendingPeeled = false;
    const PeelGraphs &peelGraph(const GraphKey &key, double *x, int64_t sweeps);

private:
    void allocLevels();
    void coarsenDirichlet();
    void setupCoarsestIndex();
    template <typename T>
    void updateStiffnessT(bool overlap, int bandLo, int bandHi);
    template <typename T>
    void smoothT(int l, bool forward);
    template <typename T>
    void residualT(int l);
    // xZero: the level's iterate is known to be zero on every row the level reads
    template <typename T>
    void vcycleT(int l, int64_t sweeps, bool residualSystem, bool xZero = false);
    template <typename T>
    void fmgT(int l, int64_t sweeps, bool residualSystem);
    template <typename T>
    void preconditionT(const double *r, int64_t mgIter, int64_t sweeps, bool fmg, bool prepared = false);
    // mixed solves: cg_update writes the FP32 V-cycle's b and zero x (set up once per solve by
    // prepareFusedInit after the initial residual)
    bool fusedInitOn = false;
    bool fusedInit() const { return fusedInitOn; }
    void prepareFusedInit(int64_t mgIter, int64_t sweeps);
    template <typename T>
    void applyKLevelT(int l, const T *u, T *out, bool zeroInit, bool negate);
    void cgIteration(double *x, int64_t mgIter, int64_t sweeps, bool fmg, bool hostMirror = true);
    // the iteration after its preconditioner: direction, matvec, step, residual norm
    void cgIterationRest(double *x, int64_t mgIter, bool hostMirror);
    // vcycleT<T>(0, sweeps, true) in three parts with the same launches in the same order:
    // 0 = level 0's down leg, 1 = the down legs below it, 2 = the coarsest solve and the up legs
    template <typename T>
    void vcyclePartT(int part, int64_t sweeps);

public:
    // One FP32 V-cycle on the fine level's right-hand side lv[0].d32.b (zero initial guess),
    // result in lv[0].d32.x (mixed precision; stiffness must be current).
    void vcycleOnFineRhs(int64_t sweeps);
    // overlap = false joins any side-stream rebuild still in flight before returning
    void ensureStiffness(bool deferCheck = false, bool overlap = false);
    void checkStiffness();
    bool spdCheckPending = false;
    uint64_t constVersion[2] = {0, 0};  // K0 version of the uploaded coarsening tables (FP32, FP64)
    template <typename T>
    void levelOp(int l, int op, const double *a, const double *b, double *out, bool flag);
};

// Topology optimisation problem: MG compliance objective, a filter chain and one total-volume
// constraint (TopologyOptimizationProblem.hh, TopologyOptimizationObjective.hh:71-105,
// TopologyOptimizationConstraint.hh:24-40) with the OC step (OptimalityCriterion.hh:51-138).
struct FilterSpec {
    int kind;  // 0 smoothing, 1 projection
    int radius;
    int type;  // smoothing: 0 Const, 1 Linear
    double beta;
};

// What the problem needs from a simulator and its multigrid solver (3D: Grid + MG, 2D: Grid2 + MG2).
struct ProblemBackend {
    virtual ~ProblemBackend() = default;
    virtual int64_t numElems() const = 0;
    virtual int64_t numDofs() const = 0;  // length of u and f
    virtual void filterDims(int dims[3], int &ndim) const = 0;
    virtual cudaStream_t stream() const = 0;
    virtual void buildLoad(double *f) = 0;             // device
    virtual void setPhysical(const double *rho) = 0;  // device densities -> simulator, moduli updated
    virtual PcgStats solve(double *u, const double *f, int64_t cgIter, double tol, int64_t mgIter, int64_t sweeps,
                           bool fmg) = 0;
    virtual double dotAll(const double *a, const double *b, double *partials) = 0;  // over every node
    virtual void complianceGradient(const double *u, double *out) = 0;              // device, per element
};
std::unique_ptr<ProblemBackend> makeBackend(MG *mg);

class Problem {
public:
    Problem(MG *mg, const std::vector<FilterSpec> &filters, double volfrac);
    Problem(std::unique_ptr<ProblemBackend> be, const std::vector<FilterSpec> &filters, double volfrac);
    std::unique_ptr<ProblemBackend> be;
    std::vector<FilterSpec> filters;
    double volfrac;
    int64_t cgIter = 100;
    double tol = 1e-5;
    int64_t mgIter = 1, mgSweeps = 2;
    bool fmg = true, zeroInit = false;
    bool varsSet = false;
    PcgStats lastStats;
    double lambda_min = 1, lambda_max = 2;
    std::vector<DevBuf<double>> vars;  // chain intermediates [0] design ... [nf] physical
    DevBuf<double> f, u, gradBuf, scratch, scratch2, partials, stepped, x0, dJ, dc;

    void setVars(const double *x, bool device);
    double objective();
    void gradient(double *out, bool device);
    double constraint();
    void jacobian(double *out, bool device);
    // objectiveGradient (host or device, numVars doubles): use it instead of evaluating the
    // objective gradient (a gradient computed elsewhere, e.g. by an autograd backward)
    int64_t ocStep(double m, double p, double ctol, const double *objectiveGradient = nullptr);
    void getU(double *out, bool device);
    void getPhysical(double *out, bool device);
    void filterApply(const double *x_dev, double *out_dev);
    void backprop(double *g_dev);

private:
    void applyFilter(const FilterSpec &fs, const double *in, double *out);
    double meanDev(const double *x);
    double constraintAtVars(const double *x_dev);
    void gradientDev(double *out);
    void jacobianDev(double *out);
};

// A level below the fine one of the triquadratic multigrid hierarchy: a Q2 mesh with half the
// elements per axis of the level above, its coarsened supports, one 81 x 81 element matrix per
// element (element-major) and its work vectors.
struct Q2Level {
    int ne[3];
    int64_t NN, NE;
    std::vector<uint8_t> dmask_h;
    DevBuf<uint8_t> dmask;
    DevBuf<double> Ke64;
    DevBuf<float> Ke32;
    LevelData<double> w64;
    LevelData<float> w32;
};

// Preconditioner of the triquadratic PCG: the reference's hierarchy of halved Q2 meshes
// (MultigridSolver<double, 2, 2, 2>), or a p-multigrid step onto the trilinear mesh.
enum Q2Hierarchy { Q2_HIER_Q2 = 0, Q2_HIER_P = 1 };

// Triquadratic voxel grid (vfem_q2.cpp): K0, moduli, supports, applyK, the 27-colour block
// Gauss-Seidel sweep and the PCG with its multigrid preconditioner.
class GridQ2 {
public:
    GridQ2(const int ne[3], const double bmin[3], const double bmax[3]);
    ~GridQ2();
    GridQ2(const GridQ2 &) = delete;
    GridQ2 &operator=(const GridQ2 &) = delete;
    int ne[3], nn[3];
    int64_t NN, NE;
    double bmin[3], bmax[3], h[3];
    double Eyoung = 1.0, nu = 0.0, E0 = 1.0, Emin = 1e-4, gamma = 3.0, q = 3.0;
    int law = 0;
    Geom egeom;  // element grid (for the moduli kernel)
    std::vector<double> K0;
    std::vector<float> K0f, K0lo;  // fl(K0) and K0 - fl(K0)
    DevBuf<double> K0d, rho, Y;
    DevBuf<float> Yf, Yhi, Ylo;   // FP32 moduli; double-float split of Y
    DevBuf<float> uhi, ulo;       // double-float split of the outer matvec's operand
    bool outerDF = true;          // PCG matvec in double-float (else FP64)
    std::vector<uint8_t> dmask_h;
    DevBuf<uint8_t> dmask;
    LevelData<double> w64;
    LevelData<float> w32;
    cudaStream_t stream = nullptr;

    void setETensor(double E, double nu);
    void setParams(double E0_, double Emin_, double gamma_, double q_, int law_);
    void setDensities(const double *rho);
    void addDirichlet(const double mn[3], const double mx[3], unsigned cmask);
    // precision: PREC_FP64, PREC_MIXED (FP32) or 2 (double-float, FP64-class on the FP32 units)
    void applyK(const double *u, double *out, int precision, bool zeroDirichlet);
    void smooth(double *u, const double *b, bool forward, int precision);
    double timeApplyK(int precision, int reps, double *bytes);
    // one forward block Gauss-Seidel sweep (27 colour passes) on resident data; bytes s (9 nn + ne)
    double timeSmooth(int precision, int reps, double *bytes);
    // PCG on K u = b (zero-displacement supports) with an FP64 outer iteration and a p-multigrid
    // preconditioner: Q2 block Gauss-Seidel smoothing around one FP32 V-cycle of the trilinear
    // problem on the same mesh (`coarsenings` coarsenings); x in/out.
    PcgStats pcg(double *x, const double *b, int64_t maxIter, double tol, int coarsenings, int64_t sweeps);
    int hierarchy = Q2_HIER_Q2;   // preconditioner of pcg (Q2Hierarchy)
    int vprecision = PREC_MIXED;  // V-cycle precision of the Q2 hierarchy
    bool symmetricGS = true;      // backward post-smoothing sweeps
    void setHierarchy(int kind);
    // PREC_FP64: FP64 V-cycle and outer matvec (the reference's method); PREC_MIXED: FP32 V-cycle
    // and double-float outer matvec
    void setPrecision(int precision);
    // The Q2 hierarchy with `coarsenings` coarsenings, built on demand in `precision`; level 0 is
    // this grid. Vectors are host or device (numNodes(l), 3) fields.
    int64_t mgLevelNodes(int coarsenings, int l);
    void mgLevelDirichlet(int coarsenings, int l, uint8_t *out);
    void mgLevelKe(int coarsenings, int l, int precision, double *out);
    void mgSmooth(int coarsenings, int l, double *u, const double *b, bool forward, int precision);
    void mgResidual(int coarsenings, int l, const double *u, const double *b, double *r, int precision);
    void mgCoarseSolve(int coarsenings, const double *b, double *x, int precision);
    // x = one V-cycle from zero on K x = b (the preconditioner of pcg)
    void mgVcycle(int coarsenings, const double *b, double *x, int64_t sweeps, int precision);

private:
    uint64_t version = 1;                // bumped when the moduli, K0 or the supports change
    std::vector<double> Kc;              // 8 x 6561 coarsened full-density element matrices
    std::vector<Q2Level> qlv;            // levels 1..L of the Q2 hierarchy
    int qCoarsenings = -1, qPrecision = -1;
    uint64_t qVersion = 0;
    int qNfree = 0;
    DevBuf<double> Kc64;
    DevBuf<float> Kc32;
    DevBuf<int> qFreeIdx, qRedIdx, qNfreeDev, qStatus;
    DevBuf<double> qAinv, qWork, qScratch;
    void prepareHierarchy(int coarsenings, int precision);
    template <typename T>
    void buildHierarchyT();
    template <typename T>
    LevelData<T> &qwork(int l);
    template <typename T>
    const T *qKe(int l);
    template <typename T>
    void qSmoothT(int l, T *u, const T *b, bool forward);
    template <typename T>
    void qResidualT(int l, const T *u, const T *b, T *r);
    template <typename T>
    void qCoarseSolveT(const T *b, T *x);
    template <typename T>
    void vcycleQ2T(int l, int64_t sweeps);
    template <typename T>
    void preconditionQ2T(const double *r, int64_t sweeps);
    const int *levelNe(int l) const { return l == 0 ? ne : qlv[l - 1].ne; }
    const uint8_t *levelMask(int l) const { return l == 0 ? dmask.p : qlv[l - 1].dmask.p; }
    int64_t levelNN(int l) const { return l == 0 ? NN : qlv[l - 1].NN; }
    struct Box {
        double mn[3], mx[3];
        unsigned cmask;
    };
    std::vector<Box> boxes;              // supports, replayed on the trilinear grid
    std::unique_ptr<Grid> q1;            // trilinear grid on the same mesh
    std::unique_ptr<MG> mg1;
    int q1Coarsenings = -1;
    DevBuf<double> cgX, cgR, cgS, cgD, cgAd, cgPart, cgSc;
    double *cgHost = nullptr;
    void prepareQ1(int coarsenings);
    void applyDF(const double *u, double *out, bool zeroDirichlet, cudaStream_t st);
    void precondition(const double *r, int64_t sweeps);
    void updateYoungModuli();
    void uploadMask();
    template <typename T>
    LevelData<T> &work();
    template <typename T>
    const T *kernelK0();
    template <typename T>
    void applyKT(const double *u, double *out, bool zeroDirichlet);
    template <typename T>
    void smoothT(double *u, const double *b, bool forward);
};
// Q2 restriction / prolongation between a grid with neFine elements per axis and its 2x coarsening.
void q2Restrict(const int neFine[3], const double *fine, double *coarse);
// Kc[f] = I_f^T K0 I_f, f = 4 fx + 2 fy + fz: the 8 coarsened full-density Q2 element matrices
void q2CoarsenedK0(const double *K0, std::vector<double> &Kc);
void q2Interpolate(const int neFine[3], const double *coarse, double *fine, bool accumulate);

// Layer-by-layer solves of partial-build heights (layers[t] element layers built) over
// persistent concurrent solver instances cloned from `src` (vfem_lbl.cpp).
// Initial guesses of the layer-by-layer solves (LayerByLayer.hh:55-209 generators)
enum LblInit { LBL_INIT_ZERO = 0, LBL_INIT_CONSTANT = 1, LBL_INIT_FD = 2, LBL_INIT_SUBSPACE = 3 };

class LBL {
public:
    LBL(Grid *src, int coarsenings, int64_t slots, int precision);
    ~LBL();
    LBL(const LBL &) = delete;
    LBL &operator=(const LBL &) = delete;
    // kind LblInit; history: the subspace size N of "N=<N>" (LBL_INIT_SUBSPACE)
    void setInit(int kind, int history);
    // fine-sweep form of every slot's solver (MG::setSweepForm)
    void setSweepForm(int form);
    // Heights layers[0..count) in the given order (the reference runs them from the full design
    // down). Zero guesses: every height is independent and the heights are spread over the
    // slots. Warm starts: the heights are cut into min(slots, count) contiguous chains, each
    // solved in order on its slot with the generator's history of that chain (one slot: the
    // reference's sequential algorithm). zeroInit false: the full-design height starts from
    // the previous run's full-design solution.
    void run(const int64_t *layers, int64_t count, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps,
             bool fmg, bool zeroInit, double *compliance, int64_t *iterations, double *gradSum);
    Grid *src;
    int coarsenings, precision;
    int initKind = LBL_INIT_SUBSPACE, historySize = 3;

private:
    struct Slot {
        std::unique_ptr<Grid> grid;
        std::unique_ptr<MG> mg;
        DevBuf<double> x, f, gtmp, gacc, cpl;
        DevBuf<double> hist[LBL_MAX_HISTORY], Ku[LBL_MAX_HISTORY], subPart, subC;
        int order[LBL_MAX_HISTORY] = {0};  // hist buffer of the i-th most recent solution
        int hs = 0;                        // history size
        std::vector<int64_t> queue;        // indices into layers, in solve order
        size_t qpos = 0;
        cudaEvent_t done = nullptr;
        int64_t idx = -1;
        ~Slot();
    };
    std::vector<std::unique_ptr<Slot>> S;
    double *cplHost = nullptr;
    DevBuf<double> uFull;  // full-design solution of the last run
    bool haveFull = false;
    void syncSource();
    void guess(Slot &sl, int64_t layer, int ny, bool zeroInit);
    void pushHistory(Slot &sl);
};

}  // namespace vfem
