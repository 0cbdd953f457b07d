// Launchers for the VoxelFEM GB300 kernels (sm_103a). All nodal vectors are SoA with
// component stride Geom::ld; element fields are flat row-major (x slowest, z fastest).
#pragma once
#include <cuda_bf16.h>

#include <functional>
#include <string>

#include "vfem_common.cuh"

namespace vfem {

// Dense 24x24 element matrix passed by value: kernel parameters live in the constant
// bank, so warp-uniform indexing is a broadcast.
template <typename T>
struct Mat24 {
    T a[576];
    // Equal element sizes (isotropic material): a[row * 24 + col] = +-cube[class], with
    // k0_cube_class(row, col) = class | 16 * negative. Kernels then hold the 10 values in
    // registers instead of reading 576 constants.
    T cube[10];
    int isCube = 0;
};

// Double-float copy of K0 for the FP64-accurate FP32 matvec.
struct Mat24DF {
    float hi[576];
    float lo[576];
    float cubeHi[10], cubeLo[10];
    int isCube = 0;
};

// Entry (3m+d, 3n+r) of the stiffness matrix of a cube element (nodes l = 4x+2y+z, isotropic
// material) depends only on which axes separate nodes m and n: for d == r on whether axis d
// does and on how many of the other two do (6 classes); for d != r on whether axes d and r
// both or neither separate them and on whether the third axis does (4 classes), with sign
// xi_m[d] xi_n[r] (xi = +-1 the node's side along the axis). Returns class | 16 * negative.
__host__ __device__ constexpr int k0_cube_class(int row, int col) {
    const int m = row / 3, d = row % 3, n = col / 3, r = col % 3;
    const int dd = ((m >> (2 - d)) ^ (n >> (2 - d))) & 1;
    if (d == r) {
        int others = 0;
        for (int a = 0; a < 3; ++a)
            if (a != d) others += ((m >> (2 - a)) ^ (n >> (2 - a))) & 1;
        return 3 * dd + others;
    }
    const int t = 3 - d - r;
    const int dr = ((m >> (2 - r)) ^ (n >> (2 - r))) & 1;
    const int dt = ((m >> (2 - t)) ^ (n >> (2 - t))) & 1;
    const int xm = 2 * ((m >> (2 - d)) & 1) - 1, xn = 2 * ((n >> (2 - r)) & 1) - 1;
    return (6 + 2 * (dd == dr ? 1 : 0) + dt) | (xm * xn < 0 ? 16 : 0);
}

// kv[c] from K (24 x 24, row-major) if every entry matches the cube pattern to round-off.
bool k0_cube_values(const double *K, double kv[10]);

// Stored entries per node of a plane-layout stencil: the diagonal and upper-half blocks
// (offsets 13..26) of the symmetric Galerkin operator.
constexpr int STENCIL_PLANES = 14 * 9;

// ---------------- fine level (k_fine.cu) ----------------
template <typename T>
void launch_young_moduli(const Geom &g, const double *rho, T *Y, double E0, double Emin, double gamma, double q,
                         int law, bool masking, cudaStream_t st);
template <typename T>
void launch_convert(const void *src, bool srcDouble, T *dst, int64_t n, cudaStream_t st);

// Fine-level gathers. T = double: Y is the plain moduli array. T = float: Y is the zero-padded
// FP32 copy (launch_pad_young) and u a vector with a zeroed guard of Geom::nodeGuard() elements
// on either side (DevBuf::alloc(n, guard)).
// out = +-K u (+ out if !zeroInit). zeroDirichlet zeroes constrained components of out.
// partialDot (optional, FP64 path only) receives per-block partials of sum(u . out) over nondetached rows.
template <typename T>
void launch_applyk_fine(const Geom &g, const T *Y, const T *u, T *out, const Mat24<T> &K0, bool zeroInit,
                        bool negate, const uint8_t *dmask, bool zeroDirichlet, double *partialDot,
                        int partialBlocks, cudaStream_t st);
// r = b - K u on nondetached rows, r = b elsewhere; constrained components zeroed.
template <typename T>
void launch_residual_fine(const Geom &g, const T *Y, const T *u, const T *b, T *r, const Mat24<T> &K0,
                          const uint8_t *dmask, cudaStream_t st);
// One colour pass of block Gauss-Seidel on the fine level.
// One FP32 fine sweep's four colours with x % 2 == cx (all x-planes of that parity at once, one
// thread-block cluster per plane); identical iterates to the four colour launches.
void launch_gs_fine_planes(const Geom &g, const float *Y, float *u, const float *b, const uint8_t *dmask, int cx,
                           bool forward, const Mat24<float> &K0, cudaStream_t st);
// The FP32 fine sweep's colours (x%2, y%2) = (cx, cy) with z parity 0 then 1 (1 then 0
// backward): all z-lines of that class at once, whole lines per CTA; identical iterates to the
// two colour launches.
void launch_gs_fine_lines(const Geom &g, const float *Y, float *u, const float *b, const uint8_t *dmask, int cx,
                          int cy, bool forward, const Mat24<float> &K0, cudaStream_t st);
// Form of the FP32 fine sweep: four line-pair launches (default), two plane-pair launches or
// eight colour launches (VFEM_GS_MODE = lines / planes / colours).
enum { GS_COLOURS = 0, GS_LINES = 1, GS_PLANES = 2, GS_STAGED = 3 };
// The line-pair sweep with each CTA's neighbourhood staged in shared memory; gsStagedFits says
// whether the tile of this grid fits (long z lines do not).
void launch_gs_fine_staged(const Geom &g, const float *Y, float *u, const float *b, const uint8_t *dmask, int cx,
                           int cy, bool forward, const Mat24<float> &K0, cudaStream_t st);
bool gsStagedFits(const Geom &g);
int gsFineMode();
// Resident blocks per SM the FP32 cube-voxel fine kernels are fitted to (VFEM_FINE_OCC = 2, 3 or
// 4; 0: the defaults, four for the residual and three for the Gauss-Seidel sweep, whose 80-register
// form is faster than its 64-register one)
int fineOccupancy();
template <typename T>
void launch_gs_fine_color(const Geom &g, const T *Y, T *u, const T *b, const uint8_t *dmask, int color, bool forward,
                          const Mat24<T> &K0, cudaStream_t st);
// FP64-accurate matvec in double-float arithmetic: out = K u with u = uh + ul and Y = Yh + Yl
// given as float pairs; out (and the partial dots u.out) in FP64.
// With rhs given, out = rhs - K u with constrained components zeroed (residual form).
void launch_applyk_fine_df(const Geom &g, const float *Yh, const float *Yl, const float *uh, const float *ul,
                           const double *u, double *out, const Mat24DF &K0, const uint8_t *dmask, bool zeroDirichlet,
                           double *partialDot, int partialBlocks, cudaStream_t st, const double *rhs = nullptr);
// Zero-padded (Geom::padElem) FP32 moduli: hi = fl(Y), and lo = fl(Y - hi) when lo is given.
void launch_pad_young(const Geom &g, const double *Y, float *hi, float *lo, cudaStream_t st);
// hi = fl(v), lo = fl(v - hi)
void launch_split_df(const double *src, float *hi, float *lo, int64_t n, cudaStream_t st);

void launch_compliance_gradient(const Geom &g, const double *rho, const double *u, double *grad, const Mat24<double> &K0,
                                double E0, double Emin, double gamma, double q, int law, const double *grav,
                                double vol, cudaStream_t st);
// grad_e = wF lam^T df/drho_e - wK dE/drho_e lam_e^T K0 u_e (self-weight load term only with gravity).
void launch_adjoint_sensitivity(const Geom &g, const double *rho, const double *lam, const double *u, double *grad,
                                const Mat24<double> &K0, double E0, double Emin, double gamma, double q, int law,
                                const double *grav, double vol, double wF, double wK, cudaStream_t st);
void launch_element_energy(const Geom &g, const double *Y, const double *u, double *out, const Mat24<double> &K0,
                           cudaStream_t st);
void launch_build_gravity_load(const Geom &g, const double *rho, double *f, const double *grav, double vol,
                               cudaStream_t st);

// ---------------- coarse levels (k_coarse.cu) ----------------
// Stencil kernels take the level's layout: rows (node-contiguous, 256 entries per node, one
// warp per node) or planes (243 planes of NN, one thread per node).
// Stencil kernels: T the arithmetic type, TS the stored entries' type (T, or bf16 for the
// plane-layout FP32 levels of the mixed preconditioner).
template <typename T, typename TS>
void launch_stencil_apply(const Geom &g, const TS *S, const T *u, T *out, bool zeroInit, bool negate, bool rows,
                          cudaStream_t st);
template <typename T, typename TS>
void launch_stencil_residual(const Geom &g, const TS *S, const T *u, const T *b, T *r, const uint8_t *dmask, bool rows,
                             cudaStream_t st);
template <typename T, typename TS>
void launch_gs_stencil_color(const Geom &g, const TS *S, T *u, const T *b, const uint8_t *dmask, int color,
                             bool forward, bool rows, cudaStream_t st);
// Colours (cx, cy, 0) and (cx, cy, 1) of a plane-layout level in one launch (whole z-lines per
// block); identical iterates to the two colour launches.
template <typename T, typename TS>
void launch_gs_stencil_lines(const Geom &g, const TS *S, T *u, const T *b, const uint8_t *dmask, int cx, int cy,
                             bool forward, cudaStream_t st);
template <typename T>
void launch_restrict(const Geom &gf, const Geom &gc, const T *fine, T *coarse, cudaStream_t st);
template <typename T>
void launch_interpolate(const Geom &gf, const Geom &gc, const T *coarse, T *fine, bool accumulate, cudaStream_t st);
template <typename T>
void launch_zero_dirichlet(const Geom &g, T *u, const uint8_t *dmask, cudaStream_t st);
template <typename T>
void launch_masked_zero(const Geom &g, T *u, int margin, cudaStream_t st);
template <typename T>
void launch_fill(T *p, T v, int64_t n, cudaStream_t st);
// Galerkin coarsening. Element matrices are stored element-major: Ke[e * 576 + 24*row + col].
template <typename T>
void launch_ke_level1(const Geom &g1, const Geom &g0, const T *Y0, const T *Kc /*8*576*/, T *Ke1, cudaStream_t st);
// Level-1 stencil assembled directly from the fine Young's moduli (no element matrices).
// rowLo, rowHi: only the (level-1 node / level-l element / level-l node) rows in [rowLo, rowHi)
// are rebuilt (band-partial update); the defaults rebuild everything
template <typename T, typename TS>
void launch_stencil_level1(const Geom &g1, const Geom &g0, const T *Y0, const T *Kc, TS *S, bool rows, cudaStream_t st,
                           int rowLo = 0, int rowHi = 2147483647);
// Level-2 element matrices from the fine moduli and the 64 folded constant matrices K2.
template <typename T>
void launch_ke_level2(const Geom &g2, const Geom &g1, const Geom &g0, const T *Y0, const T *K2, T *Ke2, cudaStream_t st,
                      int rowLo = 0, int rowHi = 2147483647);
template <typename T>
void launch_ke_coarsen(const Geom &gc, const Geom &gf, const T *Kef, const T *phis /*8*64*/, T *Kec, cudaStream_t st,
                       int rowLo = 0, int rowHi = 2147483647);
template <typename T>
void launch_ke_scaled(const Geom &g, const T *Y, const T *K0, T *Ke, cudaStream_t st);
template <typename T, typename TS>
void launch_stencil_from_ke(const Geom &g, const T *Ke, TS *S, bool rows, cudaStream_t st, int rowLo = 0,
                            int rowHi = 2147483647);
template <typename Tdst, typename Tsrc>
void launch_cast(const Tsrc *src, Tdst *dst, int64_t n, cudaStream_t st);

// ---------------- single-CTA coarse tail of the V-cycle (k_tail.cu) ----------------
constexpr int MAX_TAIL_LEVELS = 8;
template <typename T>
struct TailLevel {
    Geom g;
    const T *S;
    T *x, *b, *r;
    const uint8_t *dmask;
};
template <typename T>
struct TailParams {
    int nlev;  // tail levels including the coarsest (solved between the two launches)
    int sweeps;
    int symmetric;
    TailLevel<T> lv[MAX_TAIL_LEVELS];
};
template <typename T>
void launch_tail_down(const TailParams<T> &P, cudaStream_t st);
template <typename T>
void launch_tail_up(const TailParams<T> &P, cudaStream_t st);

// ---------------- dense coarsest solve + vector ops (k_linalg.cu) ----------------
template <typename T>
void launch_dense_from_stencil(const Geom &g, const T *S, const int *redIdx, double *A, int nfree, bool rows,
                               cudaStream_t st);
void launch_symmetrize(double *A, int n, cudaStream_t st);
// In place: A (n x n, row-major) -> A^{-1} via blocked Cholesky; status[0] set nonzero if not SPD.
// work holds dense_inverse_work_size(n) doubles.
// mark(name), when given, is called after each phase has been enqueued (profiling).
// Tile edge of the blocked factorisation: the sequential chain is one diagonal tile per step,
// so small tiles shorten it; the FP64 work of the whole inverse does not depend on the tile.
constexpr int DENSE_TILE = 16;
inline size_t dense_inverse_work_size(int n) {
    // Z, the inverted diagonal tiles, and one word for the persistent form's grid barrier
    return (size_t)n * n + (size_t)DENSE_TILE * DENSE_TILE * ((n + DENSE_TILE - 1) / DENSE_TILE) + 1;
}
// The dense inverse's status word: 1 = not positive definite, 2 = a grid-wide barrier of the
// single-launch form timed out.
inline void check_dense_status(int s) {
    if (s == 2) throw Error(ERR_CUDA, "coarsest inverse: a grid-wide barrier timed out");
    if (s) throw Error(ERR_NOT_SPD, "Coarsest stiffness matrix is not positive definite");
}
// 1/d and 1/sqrt(d) through the dense inverse's pivot helpers (single-precision seed and two
// Newton-Raphson steps), elementwise; a diagnostic of their accuracy.
void launch_newton_helpers(const double *d, int64_t n, double *recip, double *rsqrt, cudaStream_t st);
void dense_spd_inverse(double *A, double *work, int n, int *status, cudaStream_t st,
                       const std::function<void(const std::string &)> &mark = nullptr);
// x = A^{-1} b on the free DOFs (nfreeDev[0] of them, at most nfreeCap), zero elsewhere.
template <typename T>
void launch_coarse_solve(const Geom &g, const double *Ainv, const int *freeIdx, const int *nfreeDev, int nfreeCap,
                         const T *b, T *x, double *scratch, cudaStream_t st);
// Sets the WHILE condition of a device-resident PCG loop from the CG scalars (initial: before
// the first iteration, else after one; counts iterations, flags a NaN residual).
void launch_cg_loop_control(cudaGraphConditionalHandle h, double *sc, bool initial, cudaStream_t st);
// the iteration count and NaN record of one iteration run outside the loop
void launch_cg_count(double *sc, cudaStream_t st);
// sc[0] = 0, first-iteration flag, tolerance, iteration counter and limit, NaN flag
void launch_cg_init(double *sc, double tol2, double maxIter, cudaStream_t st);
// y += a x
void launch_axpy(int64_t n, double a, const double *x, double *y, cudaStream_t st);
// p[0] = a, p[1] = b, ordered on the stream
void launch_set_pair(int *p, int a, int b, cudaStream_t st);

// Deterministic masked reductions: fixed grid of REDUCE_BLOCKS partials, then one block.
constexpr int REDUCE_BLOCKS = 4 * NUM_SMS;
template <typename Ta, typename Tb>
void launch_masked_dot_partials(const Geom &g, const Ta *a, const Tb *b, double *partials, cudaStream_t st);
// scalars layout for the CG loop (double[16]):
//   0 rMr, 1 rMr_old, 2 beta, 3 alpha, 4 dAd, 5 rsq, 6 first, 7 bnorm2
void launch_finalize(const double *partials, int n, double *out, cudaStream_t st);
void launch_cg_beta(const double *partials, int n, double *sc, cudaStream_t st);
void launch_cg_alpha(const double *partials, int n, double *sc, cudaStream_t st);
void launch_cg_rsq(const double *partials, int n, double *sc, double *hostMirror, cudaStream_t st);
// s <- (s with Dirichlet comps zeroed) where s comes from src (FP64 or FP32); partials of r.s (masked).
// With s == nullptr only the partials are formed (launch_cg_direction_precond forms s itself).
template <typename Ts>
void launch_cg_precond_out(const Geom &g, const Ts *src, double *s, const double *r, const uint8_t *dmask,
                           double *partials, cudaStream_t st);
// d = beta d + s; when dh is given also writes the double-float split of d into (dh, dl), when
// amax is given the REDUCE_BLOCKS partial maxima of |d| (NaN propagates).
void launch_cg_direction(const Geom &g, const double *s, double *d, const double *sc, float *dh, float *dl,
                         cudaStream_t st, double *amax = nullptr);
// launch_cg_direction with s formed from the preconditioner iterate src as launch_cg_precond_out
// forms it (instantiated for FP32 iterates).
template <typename Ts>
void launch_cg_direction_precond(const Geom &g, const Ts *src, const uint8_t *dmask, double *d, const double *sc,
                                 float *dh, float *dl, cudaStream_t st, double *amax = nullptr);

// ---------------- warm starts of the layer-by-layer evaluation (k_lbl.cu) ----------------
constexpr int LBL_MAX_HISTORY = 8;
struct LblVectors {
    const double *u[LBL_MAX_HISTORY];
};
struct LblCoeffs {
    double c[LBL_MAX_HISTORY];
};
// c = pinv(A) b from the dot partials (pairs i <= j of u_i . K u_j, then u_i . f; nb each)
void launch_subspace_solve(const double *partials, int nb, int s, double *c, cudaStream_t st);
// x = sum_i c_i u_i on nondetached nodes (c from cDev if given, else cv), zero elsewhere
void launch_subspace_combine(const Geom &g, const LblVectors &U, int s, const double *cDev, const LblCoeffs &cv,
                             double *x, cudaStream_t st);

// ---------------- further density filters (k_filters.cu) ----------------
// dims: the input grid (Upsample: coarse nodes; VertexToCell: vertices; Langelaar: cells). ndim 2:
// a 2D grid given as (dims[0], dims[1], 1) (the reference's N = 2 instantiations).
void launch_upsample(const int dims[3], int factor, const double *in, double *out, cudaStream_t st, int ndim = 3);
void launch_upsample_backprop(const int dims[3], int factor, const double *g, double *out, cudaStream_t st);
void launch_vertex_to_cell(const int vdims[3], const double *in, double *out, cudaStream_t st, int ndim = 3);
void launch_vertex_to_cell_backprop(const int vdims[3], const double *g, double *out, cudaStream_t st, int ndim = 3);
// out: the previous output on entry (the own-voxel term of the supporting region); smax: cached
void launch_langelaar(const int dims[3], const double *in, double *out, double *smax, cudaStream_t st, int ndim = 3);
void launch_langelaar_backprop(const int dims[3], const double *g, const double *vars, const double *filt,
                               const double *smax, double *lam, double *out, cudaStream_t st, int ndim = 3);

// ---------------- Method of Moving Asymptotes (k_mma.cu) ----------------
// Row-major (m+1) x n arrays for df, p, q and m x n for G; partials are K rows of
// mma_blocks(n) entries.
constexpr int MMA_MAX_M = 3;      // constraints handled on the device
constexpr int MMA_MAX_ROWS = 12;  // partial rows of one kernel (>= m(m+1)/2 + m + 3)
struct MmaRows {
    double v[MMA_MAX_ROWS];
};
unsigned mma_blocks(int64_t n);
void launch_mma_bounds(int64_t n, int mode, const double *x0, const double *x1, const double *x2, const double *xmin,
                       const double *xmax, double *l, double *u, double *alpha, double *beta, cudaStream_t st);
void launch_mma_pq(int64_t n, int m1, const double *x, const double *u, const double *l, const double *xmin,
                   const double *xmax, const double *df, bool gcmma, const MmaRows &rho, double *p, double *q,
                   double *partials, cudaStream_t st);
void launch_mma_absdf(int64_t n, int m1, const double *df, const double *xmin, const double *xmax, double *partials,
                      cudaStream_t st);
void launch_mma_eval(int64_t n, int m1, const double *x, const double *xk, const double *u, const double *l,
                     const double *xmin, const double *xmax, const double *p, const double *q, double *partials,
                     cudaStream_t st);
void launch_mma_sub_init(int64_t n, int m, const double *alpha, const double *beta, const double *u, const double *l,
                         const double *p, const double *q, double *x, double *xi, double *eta, double *partials,
                         cudaStream_t st);
void launch_mma_sub_dir1(int64_t n, int m, double eps, const MmaRows &lam, const double *x, const double *xi,
                         const double *eta, const double *alpha, const double *beta, const double *u, const double *l,
                         const double *p, const double *q, double *dx, double *Dx, double *G, double *partials,
                         cudaStream_t st);
void launch_mma_sub_dir2(int64_t n, int m, double eps, const MmaRows &dlam, const double *x, const double *xi,
                         const double *eta, const double *alpha, const double *beta, const double *dx,
                         const double *Dx, const double *G, double *ddx, double *dxi, double *deta, double *partials,
                         cudaStream_t st);
void launch_mma_sub_move(int64_t n, int m, double step, double eps, const MmaRows &lam, double *x, double *xi,
                         double *eta, const double *ddx, const double *dxi, const double *deta, const double *alpha,
                         const double *beta, const double *u, const double *l, const double *p, const double *q,
                         double *partials, cudaStream_t st);
void launch_mma_rows_reduce(const double *partials, int K, int nsum, int nb, double *out, cudaStream_t st);

// ---------------- tensor-core outer matvec (k_tc.cu) ----------------
// K0 = scale * C with C an integer matrix whose row sums keep the bf16 MMA accumulators exact;
// fills the B tiles (2048 bf16). False when K0 has no such form.
bool tc_fit_k0(const double K0[576], double *scale, uint16_t bTiles[2048]);
int tc_matvec_blocks(const Geom &g, int maxBlocks);
// REDUCE_BLOCKS partial maxima of |u[0..n)| (NaN propagates)
void launch_absmax_partials(const double *u, int64_t n, double *partials, cudaStream_t st);
// out = K u (or rhs - K u) to FP64-class accuracy on the tensor cores; umax holds the partial
// maxima of |u|. Constrained components of out zeroed (zeroDirichlet), detached rows zero.
// Returns the number of partial dots u . out written (one per CTA) when partialDot is given.
// A bounded wait that expires sets *status.
int launch_applyk_fine_tc(const Geom &g, const float *Yh, const float *Yl, const double *u, const double *umax,
                          double *out, const uint16_t *bTiles, double scale, const uint8_t *dmask, bool zeroDirichlet,
                          double *partialDot, int partialBlocks, int *status, cudaStream_t st,
                          const double *rhs = nullptr);
// b32, x32 (optional): also write (float) r and 0 on the nondetached rows (the next FP32
// V-cycle's right-hand side and initial iterate)
void launch_cg_update(const Geom &g, double *x, double *r, const double *d, const double *Ad, const double *sc,
                      double *partials, cudaStream_t st,
                      float *b32 = nullptr, float *x32 = nullptr);
void launch_copy(double *dst, const double *src, int64_t n, cudaStream_t st);
template <typename T>
void launch_enforce_dirichlet(const Geom &g, T *u, const uint8_t *dmask, const double *dval, cudaStream_t st);

// ---------------- topology optimisation (k_topopt.cu) ----------------
// ndim 2: a (dims[0], dims[1]) grid with dims[2] == 1 and a 2D neighbourhood
// (SmoothingFilter::ApplyImpl<2>, TopologyOptimizationFilter.hh:329-397).
void launch_smoothing_filter(const int dims[3], int radius, int type, const double *in, double *out, cudaStream_t st,
                             int ndim = 3);
// Allocation-free density filter: taps in a file-scope device array (radius <= noalloc_filter_max_radius()).
void launch_smoothing_filter_noalloc(const int dims[3], int radius, int type, const double *in, double *out,
                                     cudaStream_t st);
int noalloc_filter_max_radius();
void launch_projection(int64_t n, double beta, const double *in, double *out, cudaStream_t st);
void launch_projection_backprop(int64_t n, double beta, const double *in, const double *vars, double *out,
                                cudaStream_t st);
void launch_oc_update(int64_t n, const double *x0, const double *dJ, const double *dc, double lambda, double m,
                      double p, double *out, cudaStream_t st);
void launch_sum_partials(const double *x, int64_t n, double *partials, cudaStream_t st);

// ---------------- triquadratic voxels (k_q2.cu) ----------------
// K0 is 81 x 81 (device pointer, FP64 kernels); the FP32 kernels read the copy uploaded with
// q2_upload_k0f. ne = elements per axis; vectors are (3, (2ne+1)^3) SoA.
void q2_upload_k0f(const float *K0f, cudaStream_t st);
void q2_upload_k0lo(const float *K0lo, cudaStream_t st);  // K0 - fl(K0), for the double-float matvec
// out = K u in double-float arithmetic (u = uh + ul, Y = Yh + Yl; unpadded arrays), FP64 out
void launch_applyk_q2_df(const int ne[3], const float *Yh, const float *Yl, const float *uh, const float *ul,
                         double *out, const uint8_t *dmask, bool zeroDirichlet, cudaStream_t st);
template <typename T>
void launch_applyk_q2(const int ne[3], const T *K0, const T *Y, const T *u, T *out, const uint8_t *dmask,
                      bool zeroDirichlet, cudaStream_t st);
// one block Gauss-Seidel sweep over the 27 colours (forward 0..26, backward 26..0)
template <typename T>
void launch_gs_q2_sweep(const int ne[3], const T *K0, const T *Y, T *u, const T *b, const uint8_t *dmask, bool forward,
                        cudaStream_t st);
template <typename T>
void launch_restrict_q2(const int neFine[3], const T *fine, T *coarse, cudaStream_t st);
template <typename T>
void launch_interp_q2(const int neFine[3], const T *coarse, T *fine, bool accumulate, cudaStream_t st);
// Q1 (even-indexed nodes) <-> Q2 on the same mesh: trilinear prolongation and its transpose
template <typename T>
void launch_interp_q1_q2(const int ne[3], const T *q1, T *q2, bool accumulate, cudaStream_t st);
template <typename T>
void launch_restrict_q2_q1(const int ne[3], const T *q2, T *q1, cudaStream_t st);
// r = b - Ku on the free components
template <typename T>
void launch_q2_residual_combine(int64_t NN, const T *b, const T *Ku, T *r, const uint8_t *dmask, cudaStream_t st);

// Triquadratic multigrid hierarchy: element matrices Ke (element-major, 6561 per element) on the
// levels below the fine one.
// level 1 (neCoarse elements per axis): Ke[e] = sum_f Y[child_f(e)] Kc[f], Kc 8 x 6561
template <typename T>
void launch_q2mg_level1(const int neCoarse[3], const T *Kc, const T *Y, T *Ke, cudaStream_t st);
// level l >= 2: KeCoarse[e] = sum_f I_f^T KeFine[child_f(e)] I_f
template <typename T>
void launch_q2mg_galerkin(const int neCoarse[3], const T *KeFine, T *KeCoarse, cudaStream_t st);
// one block Gauss-Seidel sweep over the 27 colours with the element matrices
template <typename T>
void launch_q2mg_gs_sweep(const int ne[3], const T *Ke, T *u, const T *b, const uint8_t *dmask, bool forward,
                          cudaStream_t st);
// out = K u, or out = b - K u when b is given; constrained components zeroed when zeroDirichlet
template <typename T>
void launch_q2mg_apply(const int ne[3], const T *Ke, const T *u, const T *b, T *out, const uint8_t *dmask,
                       bool zeroDirichlet, cudaStream_t st);
// A (nfree x nfree, zeroed here) = the operator on the free DOFs freeIdx (3 n + c; redIdx inverse)
template <typename T>
void launch_q2mg_dense(const int ne[3], const T *Ke, const int *freeIdx, const int *redIdx, int nfree, double *A,
                       cudaStream_t st);

}  // namespace vfem
