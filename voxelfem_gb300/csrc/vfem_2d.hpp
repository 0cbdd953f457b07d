// Bilinear quadrilateral voxels (TensorProductSimulator<double, 1, 1>): geometry, kernel
// launchers (k_2d.cu) and the host engine (vfem_2d.cpp). Nodal vector fields are SoA with two
// components, component c of node n at [c * NN + n] (the reference's column-major VField);
// node (i, j) -> i * (ny + 1) + j, element (i, j) -> i * ny + j, element local node l = 2a + b
// for the corner (i + a, j + b), element DOF 2 l + c.
#pragma once
#include <limits>
#include <map>
#include <vector>

#include "vfem_common.cuh"
#include "vfem_engine.hpp"

namespace vfem {

struct Geom2 {
    int ne[2], nn[2];
    int64_t NE, NN;
    int firstMaskedE = (int)LAYER_MASK_NONE;  // first masked element row along y
    int firstDetN = (int)LAYER_MASK_NONE;     // first detached node row along y
    // Device copy {firstMaskedE, firstDetN}: kernels read the mask from it, so captured graphs
    // stay valid when the fabrication height changes.
    const int *dyn = nullptr;
    __host__ __device__ int detN() const {
#if defined(__CUDA_ARCH__)
        if (dyn) return dyn[1];
#endif
        return firstDetN;
    }
    __host__ __device__ int maskedE() const {
#if defined(__CUDA_ARCH__)
        if (dyn) return dyn[0];
#endif
        return firstMaskedE;
    }
    __host__ __device__ int nyv() const { const int d = detN(); return d < nn[1] ? d : nn[1]; }
    __host__ __device__ int64_t node(int i, int j) const { return (int64_t)i * nn[1] + j; }
    __host__ __device__ int64_t elem(int i, int j) const { return (int64_t)i * ne[1] + j; }
};

inline Geom2 makeGeom2(const int ne[2]) {
    Geom2 g;
    for (int d = 0; d < 2; ++d) { g.ne[d] = ne[d]; g.nn[d] = ne[d] + 1; }
    g.NE = (int64_t)ne[0] * ne[1];
    g.NN = (int64_t)g.nn[0] * g.nn[1];
    return g;
}

// 8 x 8 element matrix passed by value (kernel parameters live in the constant bank).
template <typename T>
struct Mat8T {
    T a[64];
};
using Mat8 = Mat8T<double>;

// ---------------- kernels (k_2d.cu) ----------------
void launch2_young(const Geom2 &g, const double *rho, double *Y, double E0, double Emin, double gamma, double q,
                   int law, bool masking, cudaStream_t st);
// The V-cycle kernels exist for T = float (mixed precision) and T = double.
// Fine-level matrix-free operator. mode 0: out = K u on the nondetached rows, 0 on detached
// rows; Dirichlet components zeroed when zeroDir; partials (when given) of dotv . out over the
// nondetached rows. mode 1: residual, out = b - K u on rows < nyv + MARGIN (rows above keep
// their values) and Dirichlet components zeroed everywhere (MultigridSolver.hh:527-541).
template <typename T>
void launch2_applyk_fine(const Geom2 &g, const T *Y, const Mat8T<T> &K0, const T *u, T *out, int mode, const T *b,
                         const uint8_t *dmask, bool zeroDir, const double *dotv, double *partials, cudaStream_t st);
// The same operator in double-float arithmetic on the FP32 pipe: Y = Yh + Yl, K0 = Kh + Kl,
// u = uh + ul (pre-split), FP64 result.
void launch2_applyk_df(const Geom2 &g, const float *Yh, const float *Yl, const Mat8T<float> &Kh,
                       const Mat8T<float> &Kl, const float *uh, const float *ul, double *out, int mode,
                       const double *b, const uint8_t *dmask, bool zeroDir, const double *dotv, double *partials,
                       cudaStream_t st);
template <typename T>
void launch2_gs_fine(const Geom2 &g, const T *Y, const Mat8T<T> &K0, T *u, const T *b, const uint8_t *dmask, int color,
                     bool forward, cudaStream_t st);
// Element matrices of coarse level l: Ke[E] = sum over the 4^l fine elements f of E of
// Y0[f] Kc[pos(f)] (Kc: 4^l x 64, the fine K0 carried up through the interpolation);
// zero for masked coarse elements.
void launch2_ke_coarse(const Geom2 &gc, const Geom2 &g0, int level, const double *Y0, const double *Kc, double *Ke,
                       cudaStream_t st);
// 9-point block stencils S[(o * 4 + 2 r + c) * NN + n], o = 3 (di + 1) + (dj + 1), from Ke.
void launch2_stencil_from_ke(const Geom2 &g, const double *Ke, double *S, cudaStream_t st);
// Stencil operator, modes as launch2_applyk_fine (detached rows of a stencil are zero).
template <typename T>
void launch2_stencil_apply(const Geom2 &g, const T *S, const T *u, T *out, int mode, const T *b, const uint8_t *dmask,
                           cudaStream_t st);
template <typename T>
void launch2_gs_stencil(const Geom2 &g, const T *S, T *u, const T *b, const uint8_t *dmask, int color, bool forward,
                        cudaStream_t st);
template <typename T>
void launch2_restrict(const Geom2 &gf, const Geom2 &gc, const T *fine, T *coarse, cudaStream_t st);
template <typename T>
void launch2_interpolate(const Geom2 &gf, const Geom2 &gc, const T *coarse, T *fine, bool accumulate, cudaStream_t st);
template <typename T>
void launch2_zero_dirichlet(const Geom2 &g, T *u, const uint8_t *dmask, cudaStream_t st);
template <typename T>
void launch2_enforce_dirichlet(const Geom2 &g, T *u, const uint8_t *dmask, const double *dval, cudaStream_t st);
template <typename T>
void launch2_masked_zero(const Geom2 &g, T *u, int margin, cudaStream_t st);
void launch2_dense_from_stencil(const Geom2 &g, const double *S, const int *red, double *A, int nfree, cudaStream_t st);
// x = A^{-1} b on the free DOFs (nfreeDev[0] of them, at most nfreeCap), zero elsewhere
template <typename T>
void launch2_coarse_solve(const Geom2 &g, const double *Ainv, const int *freeIdx, const int *nfreeDev, int nfreeCap,
                          const T *b, T *x, double *scratch, cudaStream_t st);
void launch2_dot_partials(const Geom2 &g, const double *a, const double *b, double *partials, cudaStream_t st);
// s = src (FP64 or FP32) with Dirichlet components zeroed; partials of r . s (nondetached rows)
template <typename Ts>
void launch2_precond_out(const Geom2 &g, const Ts *src, double *s, const double *r, const uint8_t *dmask,
                         double *partials, cudaStream_t st);
// d = beta d + s (beta = sc[2]); with dh, dl also the double-float split of d
void launch2_direction(const Geom2 &g, const double *s, double *d, const double *sc, cudaStream_t st,
                       float *dh = nullptr, float *dl = nullptr);
void launch2_cg_update(const Geom2 &g, double *x, double *r, const double *d, const double *Ad, const double *sc,
                       double *partials, cudaStream_t st);
// Sensitivity lam^T (wF df/drho - wK dK/drho u) per element (compliance: lam = u, wF = 1, wK = 1/2).
void launch2_adjoint(const Geom2 &g, const double *rho, const double *lam, const double *u, double *out,
                     const Mat8 &K0, double E0, double Emin, double gamma, double q, int law, const double grav[2],
                     double vol, double wF, double wK, cudaStream_t st);
void launch2_element_energy(const Geom2 &g, const double *Y, const double *u, double *out, const Mat8 &K0,
                            cudaStream_t st);
void launch2_gravity_load(const Geom2 &g, const double *rho, double *f, const double grav[2], double vol,
                          cudaStream_t st);

void launch2_subspace_combine(const Geom2 &g, const LblVectors &U, int s, const double *cDev, const LblCoeffs &cv,
                              double *x, cudaStream_t st);

// ---------------- host engine (vfem_2d.cpp) ----------------
class Grid2 {
public:
    Grid2(const int ne[2], const double bmin[2], const double bmax[2]);
    ~Grid2();
    Grid2(const Grid2 &) = delete;
    Grid2 &operator=(const Grid2 &) = delete;
    Geom2 g;
    double bmin[2], bmax[2], h[2];
    double Eyoung = 1.0, nu = 0.0;  // ETensor(1, 0) default (TensorProductSimulator.hh:2114)
    double E0 = 1.0, Emin = 1e-4, gamma = 3.0, q = 3.0;
    int law = 0;
    double grav[2] = {0, 0};
    double maskH = std::numeric_limits<double>::infinity();
    Mat8 K0;
    cudaStream_t stream = nullptr;
    DevBuf<double> rho, Y, dval, force;
    DevBuf<uint8_t> dmask;
    std::vector<uint8_t> hmask;
    std::vector<double> hval, hforce;
    bool dvalNonzero = false;
    // bumped on every change of the moduli or K0 / of K0 / of the boundary conditions
    uint64_t version = 0, k0Version = 0, bcVersion = 0;

    double vol() const { return h[0] * h[1]; }
    void setETensor(double E, double nu_);
    void setParams(double E0_, double Emin_, double gamma_, double q_, int law_);
    void setDensities(const double *rho_, bool checkRange);
    void setUniformDensities(double v);
    void updateYoungModuli();
    void addDirichlet(const double u[2], const double mn[2], const double mx[2], unsigned cmask);
    void applySymmetry(const int axes[2], const int maxFace[2]);
    void setForces(const double *f);
    void setGravity(const double gv[2]);
    void setMaskLayer(int64_t l);
    void setMaskHeight(double hgt, bool update);
    void uploadBC();
    void applyK(const double *u, double *out);
    void buildLoadDev(double *f);
    void adjoint(const double *lam, const double *u, double wF, double wK, double *out);
    void elementEnergy(const double *u, double *out);
    // same dimensions, material, loads and supports (densities are copied by the caller)
    std::unique_ptr<Grid2> clone() const;
};

class MG2 {
public:
    MG2(Grid2 *fine, int coarsenings);
    ~MG2();
    MG2(const MG2 &) = delete;
    MG2 &operator=(const MG2 &) = delete;
    struct Level {
        Geom2 g;
        double h[2];
        std::vector<uint8_t> hmask;
        DevBuf<uint8_t> dmask;  // levels >= 1 (level 0 uses the simulator's)
        DevBuf<int> dyn;
        DevBuf<double> x, b, r, Ke, S, Kc;
        DevBuf<float> x32, b32, r32, S32;  // mixed precision: the FP32 V-cycle's vectors and stencils
        double maskH = std::numeric_limits<double>::infinity();
    };
    Grid2 *fine;
    std::vector<Level> lv;
    bool symmetricGS = true, useGraphs = true;
    int precision = PREC_FP64;  // PREC_MIXED: FP32 V-cycle as the preconditioner of FP64 CG
    // CG matvec of the mixed solve: MATVEC_DF (default: double-float on the FP32 pipe) or MATVEC_FP64
    int outerMatvec = MATVEC_DF;
    void setOuterMatvec(int kind);
    int L() const { return (int)lv.size(); }
    int64_t levelNN(int l) const;
    void setPrecision(int p);
    const uint8_t *levelMask(int l) const;

    void setMaskLayer(int64_t l);
    void updateStiffness();
    void applyK(int l, const double *u, double *out);
    void residual(int l, const double *u, const double *b, double *r);
    void smooth(int l, double *u, const double *b, bool forward);
    void restrictTo(int l, const double *fine, double *coarse);
    void interpolate(int l, const double *coarse, double *fine, bool accumulate);
    void coarseSolve(const double *b, double *x);
    void zeroDirichlet(int l, double *u);
    void solve(const double *u, const double *f, int64_t steps, int64_t sweeps, bool zeroDirichlet, bool fmg,
               double *xout);
    // x, b host or device arrays of 2 NN doubles
    PcgStats pcg(double *x, const double *b, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps, bool fmg,
                 bool dirichletSatisfied, PcgCallback cb, void *user);
    // x, b device arrays
    PcgStats pcgDev(double *x, const double *b, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps, bool fmg,
                    bool dirichletSatisfied, PcgCallback cb, void *user);
    // Asynchronous device-resident solve: pcgStart enqueues it on the simulator's stream (no host
    // synchronisation once the stiffness is built), pcgFinish waits and returns the statistics.
    void pcgStart(double *x, const double *b, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps, bool fmg,
                  bool dirichletSatisfied);
    PcgStats pcgFinish();
    double timeKernel(int which, int reps);
    void syncFine();

private:
    template <typename T>
    struct LB {
        T *x, *b, *r;
        const T *S;
    };
    template <typename T>
    LB<T> lb(int l);
    template <typename T>
    const T *fineY() const;
    template <typename T>
    const Mat8T<T> &fineK0() const;
    template <typename T>
    void levelOperatorT(int l, const T *u, T *out, int mode, const T *b);
    template <typename T>
    void smoothLevelT(int l, T *u, const T *b, bool forward);
    template <typename T>
    void coarseSolveDevT(const T *b, T *x);
    template <typename T>
    void vcycleT(int l, int64_t sweeps, bool residualSystem);
    template <typename T>
    void fmgDownT(int l, int64_t sweeps, bool residualSystem);
    template <typename T>
    void runCyclesT(int64_t steps, int64_t sweeps, bool residualSystem, bool fmg);
    void refreshSingle();
    // CG matvec (and the initial residual when b is given): FP64, or double-float in mixed mode.
    // uSplit: u is the CG direction, whose split the direction kernel already wrote into dh, dl.
    void outerOperator(const double *u, double *out, int mode, const double *b, bool zeroDir, const double *dotv,
                       double *partials, bool uSplit);
    bool dfOuter() const { return precision == PREC_MIXED && outerMatvec == MATVEC_DF; }
    void refreshDF();  // the split moduli and K0 (outside captured regions)
    DevBuf<float> Y32, Yh, Yl, dh, dl;
    Mat8T<float> K0f, K0lo;
    uint64_t dfVersion = ~0ull;

    void ensureStiffness();
    void levelOperator(int l, const double *u, double *out, int mode, const double *b);
    void smoothLevel(int l, double *u, const double *b, bool forward);
    void coarseSolveDev(const double *b, double *x);
    void runCycles(int64_t steps, int64_t sweeps, bool residualSystem, bool fmg);
    void cgIteration(double *x, int64_t mgIter, int64_t sweeps, bool fmg);
    cudaGraphExec_t loopGraph(double *x, int64_t mgIter, int64_t sweeps, bool fmg);
    void clearGraphs();

    uint64_t builtVersion = ~0ull, k0Version = ~0ull, bcVersion = ~0ull;
    int builtMaskE = -1;
    bool stiffValid = false;
    // coarsest dense inverse; the free-DOF count lives on the device too, so captured graphs
    // stay valid when the fabrication mask changes it
    DevBuf<double> Ainv, work, cscratch, rbuf, dvec, Ad, sbuf, partials, sc;
    DevBuf<int> freeIdx, redIdx, status, nfreeDev;
    int nfree = 0, nfreeCap = 0;
    double *hostSc = nullptr;
    bool pending = false;
    struct Key {
        int64_t mgIter, sweeps;
        int fmg, sym;
        double *x;
        bool operator<(const Key &o) const {
            if (mgIter != o.mgIter) return mgIter < o.mgIter;
            if (sweeps != o.sweeps) return sweeps < o.sweeps;
            if (fmg != o.fmg) return fmg < o.fmg;
            if (sym != o.sym) return sym < o.sym;
            return x < o.x;
        }
    };
    std::map<Key, cudaGraphExec_t> graphs;
    std::map<Key, uint64_t> graphKernels;
    Key pendingKey{};
};

// Layer-by-layer evaluation over 2D simulators (LayerByLayerEvaluator::run, LayerByLayer.hh:223-296),
// organised like the 3D evaluator: `slots` persistent solver copies on their own streams, zero
// initial guesses spread over them, warm starts (constant / fd / subspace) as chains of heights.
class LBL2 {
public:
    LBL2(Grid2 *src, int coarsenings, int64_t slots, int precision);
    ~LBL2();
    LBL2(const LBL2 &) = delete;
    LBL2 &operator=(const LBL2 &) = delete;
    void setInit(int kind, int history);
    void run(const int64_t *layers, int64_t count, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps,
             bool fmg, bool zeroInit, double *compliance, int64_t *iterations, double *gradSum);

private:
    struct Slot {
        std::unique_ptr<Grid2> grid;
        std::unique_ptr<MG2> mg;
        DevBuf<double> x, f, gtmp, gacc, cpl, part, subPart, subC;
        DevBuf<double> hist[LBL_MAX_HISTORY], Ku[LBL_MAX_HISTORY];
        int order[LBL_MAX_HISTORY] = {0};
        int hs = 0;
        std::vector<int64_t> queue;
        size_t qpos = 0;
        int64_t idx = -1;
        cudaEvent_t done = nullptr;
        ~Slot();
    };
    Grid2 *src;
    int coarsenings;
    int initKind = LBL_INIT_SUBSPACE, historySize = 3;
    std::vector<std::unique_ptr<Slot>> S;
    double *cplHost = nullptr;
    DevBuf<double> uFull;
    bool haveFull = false;
    void syncSource();
    void guess(Slot &sl, int64_t layer, int ny, bool zeroInit);
    void pushHistory(Slot &sl);
};

// Problem backend of the 2D simulator (compliance objective, filters and OC over a Grid2 + MG2).
std::unique_ptr<ProblemBackend> makeBackend2D(MG2 *mg);

}  // namespace vfem
