/*
 * vfem.h -- C ABI of the GB300 VoxelFEM solve-and-sensitivity library (libvfem.so).
 *
 * Drop-in boundary for VoxelFEM's pybind11 module `pyVoxelFEM`
 * (python_bindings/VoxelFEM.cc) on the hot path: TensorProductSimulator<double,1,1,1>,
 * MultigridSolver<double,1,1,1>, the compliance objective / filter chain / volume
 * constraint of TopologyOptimizationProblem and the OC optimiser.
 *
 * Conventions
 *   - Every function returns an int status (VFEM_OK on success). On failure the
 *     thread-local message of vfem_last_error() holds the text the reference would
 *     throw (std::runtime_error / std::logic_error in the reference).
 *   - Nodal vector fields are (numNodes, 3) arrays in column-major order: component c
 *     of node n at [c * numNodes + n] (the reference's Eigen ColMajor VField,
 *     TensorProductSimulator.hh:180). Element fields are flat row-major grid order.
 *   - Node (i, j, k) has index (i * ny1 + j) * nz1 + k (NDVector.hh:249-265).
 *   - Array arguments may be host or device pointers (detected per call); host arrays
 *     are staged and the call returns after the result is back in host memory.
 *   - Handles are not thread safe; one handle is used by one thread at a time.
 */
#ifndef VFEM_H
#define VFEM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VFEM_OK 0
#define VFEM_ERR_ARG 1      /* invalid argument or size (std::runtime_error in the reference) */
#define VFEM_ERR_CUDA 2     /* CUDA runtime failure */
#define VFEM_ERR_NAN 3      /* "NaN encountered" (std::logic_error, MultigridSolver.hh:1082-1084) */
#define VFEM_ERR_STATE 4    /* e.g. "Must call setVars first!" */
#define VFEM_ERR_NOT_SPD 5  /* coarsest operator not positive definite (CHOLMOD failure) */

#define VFEM_PREC_FP64 0    /* the method as the reference runs it, FP64 throughout */
#define VFEM_PREC_MIXED 1   /* FP32 V-cycle inside FP64 outer CG */

#define VFEM_MATVEC_FP64 0  /* outer CG matvec in native FP64 */
#define VFEM_MATVEC_DF 1    /* outer CG matvec with FP64-class accuracy without FP64 arithmetic: tensor cores
                               when K0 is a scaled small-integer matrix (cube voxels, rational nu), else
                               double-float on the FP32 units */
#define VFEM_MATVEC_DF_SIMT 2 /* outer CG matvec in double-float on the FP32 units only */

typedef struct vfem_grid vfem_grid; /* TensorProductSimulator<double, 1, 1, 1> */
typedef struct vfem_mg vfem_mg;     /* MultigridSolver<double, 1, 1, 1> */
typedef struct vfem_problem vfem_problem; /* TopologyOptimizationProblem + MultigridComplianceObjective */

typedef struct vfem_pcg_stats {
    int64_t iterations;  /* CG iterations executed */
    double relres;       /* final ||r|| / ||b|| over non-detached nodes */
    double rsq;          /* final ||r||^2 */
    double bnorm2;       /* ||b||^2 */
} vfem_pcg_stats;

/* Per-iteration callback (it_callback / residual_cb, MultigridSolver.hh:1147-1150):
 * receives the iteration, ||r|| and device pointers to x and r (valid during the call).
 * A nonzero return stops the iteration. */
typedef int (*vfem_pcg_callback)(void *user, int64_t it, double rnorm, const double *x_dev, const double *r_dev);

const char *vfem_last_error(void);
int vfem_version(void);
int vfem_device_synchronize(void);

/* ---------------- TensorProductSimulator (TensorProductSimulator.hh) ---------------- */
/* factory TensorProductSimulator([1,1,1], bbox, dims) (VoxelFEM.cc:423-430; ctor TensorProductSimulator.hh:209-279) */
int vfem_grid_create(const int64_t elems[3], const double bbox_min[3], const double bbox_max[3], vfem_grid **out);
int vfem_grid_destroy(vfem_grid *g);
/* numNodes / numElements / NbElementsPerDimension (VoxelFEM.cc:77-78, 113-115) */
int vfem_grid_dims(const vfem_grid *g, int64_t elems[3], int64_t *num_nodes, int64_t *num_elements);
/* ETensor setter = readMaterial of an isotropic material (TensorProductSimulator.hh:333-347) */
int vfem_grid_set_etensor(vfem_grid *g, double young, double poisson);
int vfem_grid_get_etensor(const vfem_grid *g, double *young, double *poisson);
/* fullDensityElementStiffnessMatrix (TensorProductSimulator.hh:658), 24x24 row-major */
int vfem_grid_get_k0(const vfem_grid *g, double *out576);
/* Diagnostic (no reference counterpart): *cube = 1 when K0 has the equal-edge (cube) structure the
 * fine-level FP32 and double-float kernels exploit (10 distinct entries up to sign), else 0. */
int vfem_grid_k0_is_cube(const vfem_grid *g, int *cube);
/* E_0, E_min, gamma, q, interpolationLaw properties (VoxelFEM.cc:116-121, TensorProductSimulator.hh:160-164) */
int vfem_grid_set_material_params(vfem_grid *g, double E0, double Emin, double gamma, double q, int law);
int vfem_grid_get_material_params(const vfem_grid *g, double *E0, double *Emin, double *gamma, double *q, int *law);
/* setDensities / getDensities / setUniformDensities (TensorProductSimulator.hh:296-371) */
int vfem_grid_set_densities(vfem_grid *g, const double *rho);
int vfem_grid_get_densities(vfem_grid *g, double *rho_out);
int vfem_grid_set_uniform_densities(vfem_grid *g, double value);
/* getYoungModulusScaleFactor (TensorProductSimulator.hh:550) */
int vfem_grid_get_young_moduli(vfem_grid *g, double *out);
/* addDirichletCondition(u, minCorner, maxCorner, componentMask) (TensorProductSimulator.hh:241-252);
 * component_mask bit c constrains component c ("xyz" = 7) */
int vfem_grid_add_dirichlet(vfem_grid *g, const double u[3], const double min_corner[3], const double max_corner[3],
                            uint32_t component_mask);
/* applySymmetryConditions (TensorProductSimulator.hh:2042-2053) */
int vfem_grid_apply_symmetry(vfem_grid *g, const int axes[3], const int max_face[3]);
/* nodal force boundary conditions (BCBuilder::setForce, TensorProductSimulator.hh:95): dense (nn, 3) field */
int vfem_grid_set_nodal_forces(vfem_grid *g, const double *forces);
/* getDirichletMask (TensorProductSimulator.hh:256-263): per node, bit c set if component c is constrained */
int vfem_grid_get_dirichlet_mask(const vfem_grid *g, uint8_t *mask_out);
/* gravity property (TensorProductSimulator.hh:216-217) */
int vfem_grid_set_gravity(vfem_grid *g, const double gravity[3]);
int vfem_grid_get_gravity(const vfem_grid *g, double gravity[3]);
/* setFabricationMaskHeightByLayer / getFabricationMaskHeight (TensorProductSimulator.hh:326-331) */
int vfem_grid_set_mask_layer(vfem_grid *g, int64_t layer);
int vfem_grid_get_mask_height(const vfem_grid *g, double *height);
/* applyK(u) (TensorProductSimulator.hh:1411-1438, TPSStencils.hh:431-728) */
int vfem_grid_apply_k(vfem_grid *g, const double *u, double *out);
/* buildLoadVector (TensorProductSimulator.hh:1269-1288) */
int vfem_grid_build_load(vfem_grid *g, double *out);
/* complianceGradient(u) (TensorProductSimulator.hh:973-1005) */
int vfem_grid_compliance_gradient(vfem_grid *g, const double *u, double *grad_out);
/* Layer-by-layer evaluation (LayerByLayerEvaluator, LayerByLayer.hh:223-296). vfem_lbl_create
 * clones g into `slots` persistent solver instances (numCoarseningLevels = coarsenings;
 * precision 0 = FP64, 1 = mixed FP32 V-cycle with FP64-class outer matvec) that run
 * concurrently, each on its own stream; the initial guesses follow vfem_lbl_set_init. vfem_lbl_run takes
 * g's current densities, material and loads (its supports must be unchanged) and, for each
 * t < count, solves the grid masked to layers[t] element layers (1..ny): compliance_out[t] = f.u
 * over the nondetached nodes, iterations_out[t] (may be NULL) the PCG iterations,
 * gradient_sum_out (ne, may be NULL, host or device) the sum of the compliance gradients.
 * g itself is not modified; it must outlive the evaluator. */
typedef struct vfem_lbl vfem_lbl;
int vfem_lbl_create(vfem_grid *g, int64_t coarsenings, int64_t slots, int precision, vfem_lbl **out);
int vfem_lbl_destroy(vfem_lbl *e);
/* Initial guesses (LayerByLayerEvaluator::selectInitMethod, LayerByLayer.hh:253-259): kind 0 "zero",
 * 1 "constant", 2 "fd", 3 "N=<history>" (subspace of the last `history` solutions, 1..8; the
 * default, N=3). With a warm-start kind the heights are solved as min(slots, count) contiguous
 * chains, each in order on one slot (one slot: the reference's sequential algorithm); with
 * "zero" the heights are independent and spread over the slots. */
int vfem_lbl_set_init(vfem_lbl *e, int kind, int history);
/* Form of every slot's FP32 fine sweep, as vfem_mg_set_sweep_form (no reference counterpart). */
int vfem_lbl_set_sweep_form(vfem_lbl *e, int form);
/* zero_init 0: the full-design height starts from the previous run's full-design solution */
int vfem_lbl_run(vfem_lbl *e, const int64_t *layers, int64_t count, int64_t max_iter, double tol,
                 int64_t mg_iterations, int64_t mg_smoothing_iterations, int full_multigrid, int zero_init,
                 double *compliance_out, int64_t *iterations_out, double *gradient_sum_out);

/* Adjoint-method sensitivity (no reference counterpart; generalises complianceGradient,
 * TensorProductSimulator.hh:973-1005): grad_e = load_weight * lambda^T df/drho_e
 * - stiffness_weight * dE/drho_e * lambda_e^T K0 u_e, df/drho_e the self-weight load of element e.
 * lambda = u, weights (1, 1/2) reproduce complianceGradient; (1, 1) is the backward of a solve whose
 * adjoint state is lambda. */
int vfem_grid_adjoint_sensitivity(vfem_grid *g, const double *lambda, const double *u, double load_weight,
                                  double stiffness_weight, double *grad_out);
/* elementEnergyDensity(u) (TensorProductSimulator.hh:638-654) */
int vfem_grid_element_energy(vfem_grid *g, const double *u, double *out);

/* ---------------- MultigridSolver (MultigridSolver.hh) ---------------- */
/* tps.multigridSolver(numCoarseningLevels) (VoxelFEM.cc:93, MultigridSolver.hh:35-121) */
int vfem_mg_create(vfem_grid *g, int num_coarsening_levels, vfem_mg **out);
int vfem_mg_destroy(vfem_mg *mg);
int vfem_mg_num_levels(const vfem_mg *mg, int *levels);
/* getSimulator(l).NbElementsPerDimension (VoxelFEM.cc:156) */
int vfem_mg_level_dims(const vfem_mg *mg, int level, int64_t elems[3]);
/* coarsened Dirichlet mask of level l (MultigridSolver.hh:58-103) */
int vfem_mg_level_dirichlet_mask(const vfem_mg *mg, int level, uint8_t *mask_out);
/* precision of the V-cycle (VFEM_PREC_*) and kind of outer matvec (VFEM_MATVEC_*); no reference counterpart */
int vfem_mg_set_precision(vfem_mg *mg, int precision, int outer_matvec);
/* outer matvec the mixed solve uses now: 0 FP64, 1 double-float (FP32 units), 2 tensor cores;
 * no reference counterpart */
int vfem_mg_outer_matvec_kind(const vfem_mg *mg, int *kind);
/* out = K u with constrained components zeroed (rhs given: rhs - K u), through the outer matvec
 * of the current precision setting (diagnostic; no reference counterpart) */
int vfem_mg_outer_apply(vfem_mg *mg, const double *u, const double *rhs, double *out);
/* Diagnostic (no reference counterpart, no GPU needed): whether K0 (24 x 24, row-major) is a
 * scale times a small-integer matrix that keeps the tensor-core matvec exact, and its bf16 B
 * tiles. */
int vfem_tc_fit_k0(const double *k0_576, double *scale, uint16_t *tiles_2048, int *ok);
/* Diagnostic (no reference counterpart): 1/d and 1/sqrt(d) for n doubles through the pivot
 * helpers of the coarsest dense inverse (single-precision seed plus two Newton-Raphson steps;
 * the plain quotient outside (1e-30, 1e30)). Host or device arrays. */
int vfem_debug_pivot_reciprocals(const double *d, int64_t n, double *recip_out, double *rsqrt_out);
/* Form of the FP32 fine Gauss-Seidel sweep of the mixed V-cycle (no reference counterpart; every
 * form runs the reference's colour order and gives identical iterates): VFEM_SWEEP_LINES (default:
 * four launches, colour pairs on whole z-lines), VFEM_SWEEP_COLOURS (eight colour launches) or
 * VFEM_SWEEP_PLANES (two launches, one thread-block cluster per x-plane). */
#define VFEM_SWEEP_COLOURS 0
#define VFEM_SWEEP_LINES 1
#define VFEM_SWEEP_PLANES 2
#define VFEM_SWEEP_STAGED 3 /* VFEM_SWEEP_LINES with each CTA's neighbourhood staged in shared memory */
int vfem_mg_set_sweep_form(vfem_mg *mg, int form);
/* Mixed precision (no reference counterpart): store the assembled stencils of the smoothing
 * levels 1 .. L-2 in bf16 (on != 0) instead of FP32; they are read and applied in FP32 and the
 * coarsest level stays FP32. The outer FP64 CG keeps the solution's accuracy. */
int vfem_mg_set_stencil_bf16(vfem_mg *mg, int on);
/* Diagnostic (no reference counterpart): how many hierarchy rebuilds this solver ran in full and
 * how many as band-partial updates after a fabrication-mask change (the reference's
 * m_partialStiffnessMatrixUpdate, MultigridSolver.hh:907-1017). */
int vfem_mg_stiffness_rebuilds(const vfem_mg *mg, int64_t *full, int64_t *band);
/* CUDA-graph capture of the CG iteration (default on); no reference counterpart */
int vfem_mg_set_use_graphs(vfem_mg *mg, int use);
/* Execution option (no reference counterpart): with graphs on, a solve without a callback runs as
 * one graph whose conditional WHILE node repeats the iteration on the device (default, 1); 0
 * launches one graph per iteration from a host loop. Results are identical. */
int vfem_mg_set_device_loop(vfem_mg *mg, int on);
/* setSymmetricGaussSeidel (MultigridSolver.hh:123-125) */
int vfem_mg_set_symmetric_gs(vfem_mg *mg, int symmetric);
/* setFabricationMaskHeightByLayer (MultigridSolver.hh:1022-1028) */
int vfem_mg_set_mask_layer(vfem_mg *mg, int64_t layer);
/* updateStiffnessMatrices (MultigridSolver.hh:846-905) */
int vfem_mg_update_stiffness(vfem_mg *mg);
/* applyK(l, u) (MultigridSolver.hh:471-504) */
int vfem_mg_apply_k(vfem_mg *mg, int level, const double *u, double *out);
/* computeResidual(l, u, b) (MultigridSolver.hh:527-541) */
int vfem_mg_residual(vfem_mg *mg, int level, const double *u, const double *b, double *r_out);
/* one multicoloured Gauss-Seidel sweep smoothingMulticoloredGS(l, u, b, forward) (MultigridSolver.hh:452-458) */
int vfem_mg_smooth(vfem_mg *mg, int level, double *u_inout, const double *b, int forward);
/* restriction(l -> l+1) (MultigridSolver.hh:217-275) */
int vfem_mg_restrict(vfem_mg *mg, int level, const double *fine, double *coarse_out);
/* accum_interpolation / interpolation (l+1 -> l) (MultigridSolver.hh:179-212) */
int vfem_mg_interpolate(vfem_mg *mg, int level, const double *coarse, double *fine_inout, int accumulate);
/* coarsest direct solve (TensorProductSimulator::solve, TensorProductSimulator.hh:1198-1230) */
int vfem_mg_coarse_solve(vfem_mg *mg, const double *b, double *x_out);
/* zeroOutDirichletComponents(l, u) (MultigridSolver.hh:508-511) */
int vfem_mg_zero_dirichlet(vfem_mg *mg, int level, double *u_inout);
/* solve(u, f, numSteps, numSmoothingSteps, stiffnessUpdated, zeroDirichlet, fullMultigrid) (MultigridSolver.hh:547-573) */
int vfem_mg_solve(vfem_mg *mg, const double *u, const double *f, int64_t num_steps, int64_t num_smoothing_steps,
                  int zero_dirichlet, int full_multigrid, double *x_out);
/* preconditionedConjugateGradient(u, b, maxIter, tol, it_callback, mgIterations, mgSmoothingIterations,
 * fullMultigrid, dirichletAlreadySatisfied) (MultigridSolver.hh:1047-1152, VoxelFEM.cc:174-191); x in/out */
int vfem_mg_pcg(vfem_mg *mg, double *x_inout, const double *b, int64_t max_iter, double tol, int64_t mg_iterations,
                int64_t mg_smoothing_iterations, int full_multigrid, int dirichlet_already_satisfied,
                vfem_pcg_callback cb, void *user, vfem_pcg_stats *stats);

/* Benchmark hooks (no reference counterpart): the CUDA stream the solver launches on, the
 * average device time of one launch of a hot kernel (ids in vfem_mg_time_kernel's comment
 * in vfem_engine.cpp: 0 fine applyK FP64, 1 fine applyK FP32, 2 fine applyK double-float,
 * 3/4 fine GS sweep FP32/FP64, 5 fine residual FP32, 6/7 level-1 GS sweep / residual FP32,
 * 8/9 level-2 GS sweep / residual FP32, 10 fine applyK on the tensor cores) with its algorithmic bytes, and a counter of the library's
 * kernel launches (graph replays included). */
int vfem_mg_get_stream(const vfem_mg *mg, void **stream);
int vfem_mg_time_kernel(vfem_mg *mg, int kernel, int reps, double *ms, double *bytes);
int vfem_kernel_launch_count(uint64_t *count);
/* Warm-cache phase breakdown of one PCG iteration (per level and per CG kernel) and of the
 * hierarchy rebuild, averaged over reps: up to max_entries '\n'-separated names in names_out
 * (capacity names_cap bytes) and times in ms_out; the count is returned in num_entries. */
int vfem_mg_profile(vfem_mg *mg, int64_t mg_iterations, int64_t mg_smoothing_iterations, int reps, char *names_out,
                    int64_t names_cap, double *ms_out, int max_entries, int *num_entries);

/* ---------------- filters (TopologyOptimizationFilter.hh) ---------------- */
/* SmoothingFilter::apply (= backprop) (TopologyOptimizationFilter.hh:285-400); type 0 Const, 1 Linear */
int vfem_smoothing_filter(const int64_t dims[3], int radius, int type, const double *in, double *out);
/* Allocation-free variant of vfem_smoothing_filter; it has no counterpart in the reference.
 * For callers that cannot call cudaMalloc: code under a fixed device-memory budget or inside a
 * host application that owns every device allocation (a plug-in may use only the buffers it is
 * handed), and loops that cannot afford the device synchronisation of cudaMalloc/cudaFree (the
 * tens of filter applications of every OC bisection). It allocates nothing: the tap table lives
 * in a fixed device array inside libvfem.so (about 44 KB), held by every GPU that loads the
 * library until exit, which bounds the radius to 6 (larger radii are rejected with
 * VFEM_ERR_ARG). The filter is the 3D one: its result equals vfem_smoothing_filter on the same
 * dims (a grid one voxel thick is filtered in 3D, its z offsets reflected onto the one layer;
 * 2D callers use vfem_smoothing_filter2). in_dev and out_dev must be device pointers; the work is
 * enqueued on `stream` (a cudaStream_t, 0 for the default stream) and the call returns without
 * waiting. The first call on a device, with that device current, looks up the array's device
 * address; make that first call before any stream capture on the device. Every call rebuilds the
 * tap table in the shared array, so calls that overlap on the GPU (e.g. on two streams) race on
 * it. */
int vfem_smoothing_filter_noalloc(const int64_t dims[3], int radius, int type, const double *in_dev, double *out_dev,
                                  void *stream);
/* ProjectionFilter::apply / backprop (TopologyOptimizationFilter.hh:199-225) */
int vfem_projection_apply(int64_t n, double beta, const double *in, double *out);
int vfem_projection_backprop(int64_t n, double beta, const double *in, const double *vars, double *out);

/* ---------------- topology optimisation problem ---------------- */
/* TopologyOptimizationProblem(sim, MultigridComplianceObjective(mg), [TotalVolumeConstraint(volfrac)], filters)
 * (VoxelFEM.cc:221-277, TopologyOptimizationProblem.hh:17-155); filter i is a smoothing filter
 * (kinds[i] = 0: radii[i], types[i]) or a projection (kinds[i] = 1: betas[i]). */
int vfem_problem_create(vfem_mg *mg, int num_filters, const int *kinds, const int *radii, const int *types,
                        const double *betas, double volume_fraction, vfem_problem **out);
int vfem_problem_destroy(vfem_problem *p);
/* MultigridComplianceObjective fields cgIter, tol, mgIterations, mgSmoothingIterations, fullMultigrid, zeroInit
 * (TopologyOptimizationObjective.hh:98-104) */
int vfem_problem_set_solver(vfem_problem *p, int64_t cg_iter, double tol, int64_t mg_iterations,
                            int64_t mg_smoothing_iterations, int full_multigrid, int zero_init);
/* setVars (TopologyOptimizationProblem.hh:41-50) */
int vfem_problem_set_vars(vfem_problem *p, const double *x);
int vfem_problem_get_vars(vfem_problem *p, double *x_out);
/* evaluateObjective (= compliance 1/2 f.u) / evaluateObjectiveGradient (TopologyOptimizationProblem.hh:69-84) */
int vfem_problem_objective(vfem_problem *p, double *value);
int vfem_problem_gradient(vfem_problem *p, double *grad_out);
/* evaluateConstraints / evaluateConstraintsJacobian (TopologyOptimizationProblem.hh:90-121) */
int vfem_problem_constraint(vfem_problem *p, double *value);
int vfem_problem_jacobian(vfem_problem *p, double *jac_out);
/* ComplianceObjective::u() and FilterChain::physicalVars() */
int vfem_problem_get_u(vfem_problem *p, double *u_out);
int vfem_problem_get_physical(vfem_problem *p, double *x_out);
int vfem_problem_last_solve(vfem_problem *p, vfem_pcg_stats *stats);
/* OCOptimizer::step(m, p, ctol) (OptimalityCriterion.hh:51-138); probes = constraint evaluations */
int vfem_problem_oc_step(vfem_problem *p, double m, double pexp, double ctol, int64_t *probes);
/* The same OC step with the objective gradient (numVars doubles, host or device) supplied by the
 * caller instead of evaluateObjectiveGradient, e.g. from a torch.autograd backward pass through
 * the same problem; no reference counterpart (the reference's step always evaluates it). */
int vfem_problem_oc_step_with_gradient(vfem_problem *p, double m, double pexp, double ctol,
                                       const double *objective_gradient, int64_t *probes);

/* ---- triquadratic voxels (TensorProductSimulator<double, 2, 2, 2>, TPSStencils.hh:135-186) ----
 * Nodes (2 nx + 1)(2 ny + 1)(2 nz + 1), index (I ny' + J) nz' + K; nodal fields (nn, 3)
 * column-major as for trilinear grids. precision 0 = FP64, 1 = FP32. */
typedef struct vfem_q2 vfem_q2;
int vfem_q2_create(const int64_t elems[3], const double bbox_min[3], const double bbox_max[3], vfem_q2 **out);
int vfem_q2_destroy(vfem_q2 *g);
int vfem_q2_dims(const vfem_q2 *g, int64_t *num_nodes, int64_t *num_elements);
/* setETensor (isotropic E, nu) and E_0, E_min, gamma, q, interpolationLaw, as for vfem_grid_* */
int vfem_q2_set_etensor(vfem_q2 *g, double young, double poisson);
int vfem_q2_set_material_params(vfem_q2 *g, double E0, double Emin, double gamma, double q, int law);
int vfem_q2_set_densities(vfem_q2 *g, const double *rho);
/* fullDensityElementStiffnessMatrix: 81 x 81 row-major, DOF 3l + c, l = 9a + 3b + c, 3^3 Gauss points */
int vfem_q2_get_k0(const vfem_q2 *g, double *out6561);
/* zero-displacement supports on the nodes inside [min, max], components in cmask (bit c = component c) */
int vfem_q2_add_dirichlet(vfem_q2 *g, const double min_corner[3], const double max_corner[3], int cmask);
int vfem_q2_get_dirichlet_mask(const vfem_q2 *g, uint8_t *mask_out);
/* applyK (TPSStencils.hh:135-186); precision VFEM_PREC_FP64, VFEM_PREC_MIXED (FP32 arithmetic) or
 * 2 (double-float: FP64-class on the FP32 units); zero_dirichlet zeroes the constrained
 * components of the result */
int vfem_q2_apply_k(vfem_q2 *g, const double *u, double *out, int precision, int zero_dirichlet);
/* one 27-colour block Gauss-Seidel sweep on K u = b (MultigridSolver.hh:277-321, 409-442); u in/out */
int vfem_q2_smooth(vfem_q2 *g, double *u_inout, const double *b, int forward, int precision);
/* Q2 restriction (P^T) and prolongation (P) between a grid of elems_fine elements per axis and its
 * 2x coarsening (MultigridSolver.hh:137-275) */
int vfem_q2_restrict(const int64_t elems_fine[3], const double *fine, double *coarse);
int vfem_q2_interpolate(const int64_t elems_fine[3], const double *coarse, double *fine, int accumulate);
/* Benchmark hook (no reference counterpart): average device time of one applyK on resident data and
 * its algorithmic bytes s (6 nn + ne). */
int vfem_q2_time_apply_k(vfem_q2 *g, int precision, int reps, double *ms, double *bytes);
/* Benchmark hook (no reference counterpart): one forward Gauss-Seidel sweep (27 colours) on
 * resident data, with its algorithmic bytes s (9 nn + ne). */
int vfem_q2_time_smooth(vfem_q2 *g, int precision, int reps, double *ms, double *bytes);
/* preconditionedConjugateGradient on a triquadratic grid (MultigridSolver.hh:1047-1152 recurrences,
 * FP64 outer iteration, one V-cycle from zero per iteration with mg_smoothing_iterations sweeps
 * before and after). x in/out. The preconditioner's hierarchy (vfem_q2_set_hierarchy):
 *   VFEM_Q2_HIERARCHY_Q2 (default): the reference's MultigridSolver<double, 2, 2, 2>, replacing
 *     MultigridSolver(fineSimulator, numCoarseningLevels) of a degree-2 simulator
 *     (MultigridSolver.hh:35-121): `coarsenings` halvings of the Q2 mesh; level 1 applies the fine
 *     moduli to the 8 coarsened full-density element matrices, the levels below hold Galerkin
 *     element matrices, the coarsest is solved directly (FP64 dense inverse in place of CHOLMOD);
 *   VFEM_Q2_HIERARCHY_P: Q2 block Gauss-Seidel around one FP32 V-cycle of the trilinear problem on
 *     the same mesh with `coarsenings` coarsenings (a p-multigrid step; mixed precision only).
 * vfem_q2_set_precision: VFEM_PREC_FP64 (the reference's method: FP64 V-cycle and CG matvec) or
 * VFEM_PREC_MIXED (default: FP32 V-cycle, double-float CG matvec). */
#define VFEM_Q2_HIERARCHY_Q2 0
#define VFEM_Q2_HIERARCHY_P 1
int vfem_q2_set_hierarchy(vfem_q2 *g, int hierarchy);
int vfem_q2_set_precision(vfem_q2 *g, int precision);
/* outer matvec of vfem_q2_pcg: VFEM_MATVEC_FP64 or VFEM_MATVEC_DF; no reference counterpart */
int vfem_q2_set_outer_matvec(vfem_q2 *g, int outer_matvec);
int vfem_q2_pcg(vfem_q2 *g, int64_t coarsenings, double *x_inout, const double *b, int64_t max_iter, double tol,
                int64_t mg_smoothing_iterations, vfem_pcg_stats *stats);
/* Levels of the Q2 hierarchy with `coarsenings` coarsenings (level 0 = this grid), built on
 * demand in `precision`; vectors (numNodes(level), 3) column-major, host or device.
 * num_nodes: MultigridSolver::getSimulator(l).numNodes(); dirichlet: the coarsened support bits
 * (MultigridSolver.hh:57-104); ke: the level's element matrices (levels 1..coarsenings,
 * numElements x 81 x 81, row-major; m_getCoarsenedStiffnessMatrix, MultigridSolver.hh:745-819);
 * smooth: smoothingMulticoloredGS(l, u, b, forward) (MultigridSolver.hh:452-458); residual:
 * computeResidual(l, u, b, r) (MultigridSolver.hh:527-541); coarse_solve: the coarsest
 * direct solve; vcycle: applyPreconditionerInv(b) with one V-cycle (MultigridSolver.hh:576-580). */
int vfem_q2_mg_num_nodes(vfem_q2 *g, int64_t coarsenings, int level, int64_t *num_nodes);
int vfem_q2_mg_level_dirichlet(vfem_q2 *g, int64_t coarsenings, int level, uint8_t *mask_out);
int vfem_q2_mg_level_ke(vfem_q2 *g, int64_t coarsenings, int level, int precision, double *out);
int vfem_q2_mg_smooth(vfem_q2 *g, int64_t coarsenings, int level, double *u_inout, const double *b, int forward,
                      int precision);
int vfem_q2_mg_residual(vfem_q2 *g, int64_t coarsenings, int level, const double *u, const double *b, double *r,
                        int precision);
int vfem_q2_mg_coarse_solve(vfem_q2 *g, int64_t coarsenings, const double *b, double *x, int precision);
int vfem_q2_mg_vcycle(vfem_q2 *g, int64_t coarsenings, const double *b, double *x, int64_t mg_smoothing_iterations,
                      int precision);

/* ---------------- Method of Moving Asymptotes (MethodOfMovingAsymptotes.hh; pyOptimizer.MMA,
 * python_bindings/Optimizer.cc:16-22) ----------------
 * MMA(numVars, numConstr, xmin, xmax, f, df_dx): the n-length work on the GPU, the (m+1)-sized
 * dual system on the host. f writes the objective and the m constraint values at x (host
 * memory); df_dx writes their gradients as an (m+1) x n row-major array. Nonzero returns abort
 * the step. Device optimiser: 1 <= m <= 3. */
typedef int (*vfem_mma_f)(void *user, const double *x, int64_t n, double *f_out);
typedef int (*vfem_mma_df)(void *user, const double *x, int64_t n, double *df_out);
typedef struct vfem_mma vfem_mma;
int vfem_mma_create(int64_t num_vars, int num_constraints, const double *xmin, const double *xmax, vfem_mma_f f,
                    vfem_mma_df df_dx, void *user, vfem_mma **out);
int vfem_mma_destroy(vfem_mma *o);
int vfem_mma_set_initial_var(vfem_mma *o, const double *x0);  /* MMA::setInitialVar */
int vfem_mma_enable_gcmma(vfem_mma *o, int enable);           /* MMA::enableGCMMA */
int vfem_mma_step(vfem_mma *o);                               /* MMA::step */
/* MMA::getOptimalVar (not bound by the reference module; the current iterate) */
int vfem_mma_get_optimal_var(vfem_mma *o, double *x_out);

/* ---------------- further filters (TopologyOptimizationFilter.hh:402-709) ----------------
 * UpsampleFilter(factor): in_dims coarse nodes -> (in_dims - 1) * factor + 1 fine nodes,
 * trilinear; VertexToCellFilter: vertex_dims -> vertex_dims - 1 cells, corner mean;
 * LangelaarFilter: the overhang filter along y, stateful like the reference's (its output buffer
 * enters the next application through the own-voxel term of the supporting region; backprop
 * uses the smax and filtered values of the last application). Arrays host or device. */
int vfem_upsample_filter(const int64_t in_dims[3], int64_t factor, const double *in, double *out);
int vfem_upsample_filter_backprop(const int64_t in_dims[3], int64_t factor, const double *g, double *out);
int vfem_vertex_to_cell_filter(const int64_t vertex_dims[3], const double *in, double *out);
int vfem_vertex_to_cell_filter_backprop(const int64_t vertex_dims[3], const double *g, double *out);
typedef struct vfem_langelaar vfem_langelaar;
int vfem_langelaar_create(const int64_t dims[3], vfem_langelaar **out);
int vfem_langelaar_destroy(vfem_langelaar *h);
int vfem_langelaar_apply(vfem_langelaar *h, const double *in, double *out);
int vfem_langelaar_backprop(vfem_langelaar *h, const double *g, const double *vars, double *out);
/* The same filters on 2D grids (the reference's N = 2 instantiations; the Langelaar region is the
 * voxel below and its x neighbours). The 2D Langelaar handle takes vfem_langelaar_apply/_backprop/_destroy. */
int vfem_upsample_filter2(const int64_t in_dims[2], int64_t factor, const double *in, double *out);
int vfem_upsample_filter2_backprop(const int64_t in_dims[2], int64_t factor, const double *g, double *out);
int vfem_vertex_to_cell_filter2(const int64_t vertex_dims[2], const double *in, double *out);
int vfem_vertex_to_cell_filter2_backprop(const int64_t vertex_dims[2], const double *g, double *out);
int vfem_langelaar2_create(const int64_t dims[2], vfem_langelaar **out);

/* ---------------- 2D: TensorProductSimulator<double, 1, 1> / MultigridSolver<double, 1, 1> ----------------
 * The bilinear-quadrilateral instantiation the module registers beside the 3D one
 * (VoxelFEM.cc:413-414, factory TensorProductSimulator([1, 1], bbox, dims)). Nodal fields are
 * (numNodes, 2) column-major, node (i, j) -> i * ny1 + j; the isotropic elasticity tensor is the
 * plane-stress one of MeshFEM's ElasticityTensor<Real, 2>::setIsotropic. Each entry point
 * mirrors the 3D one of the same name (same reference line, same error behaviour). */
typedef struct vfem_grid2 vfem_grid2; /* TensorProductSimulator<double, 1, 1> */
typedef struct vfem_mg2 vfem_mg2;     /* MultigridSolver<double, 1, 1> */
int vfem_grid2_create(const int64_t elems[2], const double bbox_min[2], const double bbox_max[2], vfem_grid2 **out);
int vfem_grid2_destroy(vfem_grid2 *g);
int vfem_grid2_dims(const vfem_grid2 *g, int64_t elems[2], int64_t *num_nodes, int64_t *num_elements);
int vfem_grid2_set_etensor(vfem_grid2 *g, double young, double poisson);
int vfem_grid2_get_etensor(const vfem_grid2 *g, double *young, double *poisson);
/* fullDensityElementStiffnessMatrix, 8x8 row-major, DOF 2 l + c with local node l = 2 dx + dy */
int vfem_grid2_get_k0(const vfem_grid2 *g, double *out64);
int vfem_grid2_set_material_params(vfem_grid2 *g, double E0, double Emin, double gamma, double q, int law);
int vfem_grid2_get_material_params(const vfem_grid2 *g, double *E0, double *Emin, double *gamma, double *q, int *law);
int vfem_grid2_set_densities(vfem_grid2 *g, const double *rho);
int vfem_grid2_get_densities(vfem_grid2 *g, double *rho_out);
int vfem_grid2_set_uniform_densities(vfem_grid2 *g, double value);
int vfem_grid2_get_young_moduli(vfem_grid2 *g, double *out);
/* component_mask bit c constrains component c ("xy" = 3) */
int vfem_grid2_add_dirichlet(vfem_grid2 *g, const double u[2], const double min_corner[2], const double max_corner[2],
                             uint32_t component_mask);
int vfem_grid2_apply_symmetry(vfem_grid2 *g, const int axes[2], const int max_face[2]);
int vfem_grid2_set_nodal_forces(vfem_grid2 *g, const double *forces);
int vfem_grid2_get_dirichlet_mask(const vfem_grid2 *g, uint8_t *mask_out);
/* Dirichlet values as an (nn, 2) field (getDirichletVarsAndValues, VoxelFEM.cc:93) */
int vfem_grid2_get_dirichlet_values(const vfem_grid2 *g, double *values_out);
int vfem_grid2_set_gravity(vfem_grid2 *g, const double gravity[2]);
int vfem_grid2_get_gravity(const vfem_grid2 *g, double gravity[2]);
int vfem_grid2_set_mask_layer(vfem_grid2 *g, int64_t layer);
int vfem_grid2_get_mask_height(const vfem_grid2 *g, double *height);
int vfem_grid2_apply_k(vfem_grid2 *g, const double *u, double *out);
int vfem_grid2_build_load(vfem_grid2 *g, double *out);
int vfem_grid2_compliance_gradient(vfem_grid2 *g, const double *u, double *grad_out);
int vfem_grid2_adjoint_sensitivity(vfem_grid2 *g, const double *lambda, const double *u, double load_weight,
                                   double stiffness_weight, double *out);
int vfem_grid2_element_energy(vfem_grid2 *g, const double *u, double *out);
int vfem_mg2_create(vfem_grid2 *g, int num_coarsening_levels, vfem_mg2 **out);
int vfem_mg2_destroy(vfem_mg2 *mg);
int vfem_mg2_num_levels(const vfem_mg2 *mg, int *levels);
int vfem_mg2_level_dims(const vfem_mg2 *mg, int level, int64_t elems[2]);
int vfem_mg2_level_dirichlet_mask(const vfem_mg2 *mg, int level, uint8_t *mask_out);
/* precision: VFEM_PREC_FP64 (the reference's method) or VFEM_PREC_MIXED (the PCG preconditioner's
 * V-cycle in FP32 inside FP64 CG; no reference counterpart). The per-level entry points and
 * vfem_mg2_solve stay FP64. */
int vfem_mg2_set_precision(vfem_mg2 *mg, int precision);
/* CG matvec of the mixed solve: VFEM_MATVEC_DF (default, double-float on the FP32 units) or VFEM_MATVEC_FP64 */
int vfem_mg2_set_outer_matvec(vfem_mg2 *mg, int kind);
int vfem_mg2_set_use_graphs(vfem_mg2 *mg, int use);
int vfem_mg2_set_symmetric_gs(vfem_mg2 *mg, int symmetric);
int vfem_mg2_set_mask_layer(vfem_mg2 *mg, int64_t layer);
int vfem_mg2_update_stiffness(vfem_mg2 *mg);
int vfem_mg2_apply_k(vfem_mg2 *mg, int level, const double *u, double *out);
int vfem_mg2_residual(vfem_mg2 *mg, int level, const double *u, const double *b, double *r_out);
int vfem_mg2_smooth(vfem_mg2 *mg, int level, double *u_inout, const double *b, int forward);
int vfem_mg2_restrict(vfem_mg2 *mg, int level, const double *fine, double *coarse_out);
int vfem_mg2_interpolate(vfem_mg2 *mg, int level, const double *coarse, double *fine_inout, int accumulate);
int vfem_mg2_coarse_solve(vfem_mg2 *mg, const double *b, double *x_out);
int vfem_mg2_zero_dirichlet(vfem_mg2 *mg, int level, double *u_inout);
int vfem_mg2_solve(vfem_mg2 *mg, const double *u, const double *f, int64_t num_steps, int64_t num_smoothing_steps,
                   int zero_dirichlet, int full_multigrid, double *x_out);
int vfem_mg2_pcg(vfem_mg2 *mg, double *x_inout, const double *b, int64_t max_iter, double tol, int64_t mg_iterations,
                 int64_t mg_smoothing_iterations, int full_multigrid, int dirichlet_already_satisfied,
                 vfem_pcg_callback cb, void *user, vfem_pcg_stats *stats);
/* Benchmark hook (no reference counterpart): average device time of one launch on resident data.
 * kernel 0: fine applyK (FP64), 1: fine 4-colour Gauss-Seidel sweep, 2: one V-cycle (1 and 2 in the
 * solver's precision), 3: one PCG iteration, 4: fine applyK in double-float. */
int vfem_mg2_time_kernel(vfem_mg2 *mg, int kernel, int reps, double *ms);
/* TopologyOptimizationProblem + MultigridComplianceObjective over the 2D solver; the handle takes
 * every vfem_problem_* call (filters as in vfem_problem_create, smoothing over the 2D neighbourhood). */
/* Layer-by-layer evaluation over a 2D simulator: as vfem_lbl_create / _set_init / _run. */
typedef struct vfem_lbl2 vfem_lbl2;
int vfem_lbl2_create(vfem_grid2 *g, int64_t coarsenings, int64_t slots, int precision, vfem_lbl2 **out);
int vfem_lbl2_destroy(vfem_lbl2 *e);
int vfem_lbl2_set_init(vfem_lbl2 *e, int kind, int history);
int vfem_lbl2_run(vfem_lbl2 *e, const int64_t *layers, int64_t count, int64_t max_iter, double tol,
                  int64_t mg_iterations, int64_t mg_smoothing_iterations, int full_multigrid, int zero_init,
                  double *compliance_out, int64_t *iterations_out, double *gradient_sum_out);
/* SmoothingFilter::apply on a 2D (dims[0], dims[1]) grid (ApplyImpl<2>, TopologyOptimizationFilter.hh:329-397) */
int vfem_smoothing_filter2(const int64_t dims[2], int radius, int type, const double *in, double *out);
int vfem_problem2_create(vfem_mg2 *mg, int num_filters, const int *kinds, const int *radii, const int *types,
                         const double *betas, double volume_fraction, vfem_problem **out);

#ifdef __cplusplus
}
#endif
#endif /* VFEM_H */
