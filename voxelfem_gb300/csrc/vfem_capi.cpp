// extern "C" boundary over the host engine; see include/vfem.h.
#include "../../include/vfem.h"

#include <cstring>
#include <string>

#include "vfem_2d.hpp"
#include "vfem_engine.hpp"
#include "vfem_mma.hpp"

using namespace vfem;

struct vfem_grid {
    Grid g;
    vfem_grid(const int ne[3], const double mn[3], const double mx[3]) : g(ne, mn, mx) {}
};
struct vfem_mg {
    MG m;
    vfem_mg(Grid *g, int l) : m(g, l) {}
};
struct vfem_problem {
    Problem p;
    vfem_problem(MG *m, const std::vector<FilterSpec> &f, double v) : p(m, f, v) {}
    vfem_problem(std::unique_ptr<ProblemBackend> b, const std::vector<FilterSpec> &f, double v)
        : p(std::move(b), f, v) {}
};
struct vfem_grid2 {
    Grid2 g;
    vfem_grid2(const int ne[2], const double mn[2], const double mx[2]) : g(ne, mn, mx) {}
};
struct vfem_mg2 {
    MG2 m;
    vfem_mg2(Grid2 *g, int l) : m(g, l) {}
};
struct vfem_lbl2 {
    LBL2 e;
    vfem_lbl2(Grid2 *g, int c, int64_t s, int p) : e(g, c, s, p) {}
};

namespace {
thread_local std::string g_last_error;

template <class F>
int guarded(F &&f) {
    try {
        f();
        return VFEM_OK;
    } catch (const vfem::Error &e) {
        g_last_error = e.what();
        return e.code;
    } catch (const std::exception &e) {
        g_last_error = e.what();
        return VFEM_ERR_ARG;
    } catch (...) {
        g_last_error = "unknown error";
        return VFEM_ERR_ARG;
    }
}

void need(const void *p, const char *what) {
    if (!p) throw Error(ERR_ARG, std::string("null ") + what);
}
}  // namespace

extern "C" {

const char *vfem_last_error(void) { return g_last_error.c_str(); }
int vfem_version(void) { return 1; }
int vfem_device_synchronize(void) {
    return guarded([&] { VFEM_CUDA(cudaDeviceSynchronize()); });
}

int vfem_grid_create(const int64_t elems[3], const double bbox_min[3], const double bbox_max[3], vfem_grid **out) {
    return guarded([&] {
        need(elems, "elems"); need(bbox_min, "bbox"); need(bbox_max, "bbox"); need(out, "out");
        int ne[3];
        for (int d = 0; d < 3; ++d) {
            if (elems[d] <= 0 || elems[d] > (1 << 20)) throw Error(ERR_ARG, "invalid elementsPerDimension");
            ne[d] = (int)elems[d];
        }
        *out = new vfem_grid(ne, bbox_min, bbox_max);
    });
}
int vfem_grid_destroy(vfem_grid *g) {
    return guarded([&] { delete g; });
}
int vfem_grid_dims(const vfem_grid *g, int64_t elems[3], int64_t *num_nodes, int64_t *num_elements) {
    return guarded([&] {
        need(g, "grid");
        for (int d = 0; d < 3; ++d) elems[d] = g->g.g.ne[d];
        if (num_nodes) *num_nodes = g->g.g.NN;
        if (num_elements) *num_elements = g->g.g.NE;
    });
}
int vfem_grid_set_etensor(vfem_grid *g, double young, double poisson) {
    return guarded([&] { need(g, "grid"); g->g.setETensor(young, poisson); });
}
int vfem_grid_get_etensor(const vfem_grid *g, double *young, double *poisson) {
    return guarded([&] { need(g, "grid"); *young = g->g.Eyoung; *poisson = g->g.nu; });
}
int vfem_grid_get_k0(const vfem_grid *g, double *out576) {
    return guarded([&] { need(g, "grid"); need(out576, "out"); std::memcpy(out576, g->g.K0.a, 576 * sizeof(double)); });
}
int vfem_grid_k0_is_cube(const vfem_grid *g, int *cube) {
    return guarded([&] { need(g, "grid"); need(cube, "out"); *cube = g->g.K0.isCube; });
}
int vfem_grid_set_material_params(vfem_grid *g, double E0, double Emin, double gamma, double q, int law) {
    return guarded([&] {
        need(g, "grid");
        if (law != 0 && law != 1) throw Error(ERR_ARG, "unknown interpolation law");
        g->g.setParams(E0, Emin, gamma, q, law);
        VFEM_CUDA(cudaStreamSynchronize(g->g.stream));
    });
}
int vfem_grid_get_material_params(const vfem_grid *g, double *E0, double *Emin, double *gamma, double *q, int *law) {
    return guarded([&] {
        need(g, "grid");
        *E0 = g->g.E0; *Emin = g->g.Emin; *gamma = g->g.gamma; *q = g->g.q; *law = g->g.law;
    });
}
int vfem_grid_set_densities(vfem_grid *g, const double *rho) {
    return guarded([&] { need(g, "grid"); need(rho, "rho"); g->g.setDensities(rho, false); });
}
int vfem_grid_get_densities(vfem_grid *g, double *rho_out) {
    return guarded([&] { need(g, "grid"); need(rho_out, "out"); g->g.getDensities(rho_out); });
}
int vfem_grid_set_uniform_densities(vfem_grid *g, double value) {
    return guarded([&] { need(g, "grid"); g->g.setUniformDensities(value); });
}
int vfem_grid_get_young_moduli(vfem_grid *g, double *out) {
    return guarded([&] { need(g, "grid"); need(out, "out"); g->g.getYoungModuli(out); });
}
int vfem_grid_add_dirichlet(vfem_grid *g, const double u[3], const double min_corner[3], const double max_corner[3],
                            uint32_t component_mask) {
    return guarded([&] {
        need(g, "grid"); need(u, "u"); need(min_corner, "minCorner"); need(max_corner, "maxCorner");
        if (component_mask > 7) throw Error(ERR_ARG, "invalid component mask");
        g->g.addDirichlet(u, min_corner, max_corner, component_mask);
    });
}
int vfem_grid_apply_symmetry(vfem_grid *g, const int axes[3], const int max_face[3]) {
    return guarded([&] { need(g, "grid"); need(axes, "axes"); need(max_face, "maxFace"); g->g.applySymmetry(axes, max_face); });
}
int vfem_grid_set_nodal_forces(vfem_grid *g, const double *forces) {
    return guarded([&] { need(g, "grid"); need(forces, "forces"); g->g.setForces(forces); });
}
int vfem_grid_get_dirichlet_mask(const vfem_grid *g, uint8_t *mask_out) {
    return guarded([&] { need(g, "grid"); need(mask_out, "out"); g->g.getDirichletMask(mask_out); });
}
int vfem_grid_set_gravity(vfem_grid *g, const double gravity[3]) {
    return guarded([&] { need(g, "grid"); need(gravity, "gravity"); g->g.setGravity(gravity); });
}
int vfem_grid_get_gravity(const vfem_grid *g, double gravity[3]) {
    return guarded([&] { need(g, "grid"); for (int c = 0; c < 3; ++c) gravity[c] = g->g.grav[c]; });
}
int vfem_grid_set_mask_layer(vfem_grid *g, int64_t layer) {
    return guarded([&] {
        need(g, "grid");
        g->g.setMaskLayer(layer);
        VFEM_CUDA(cudaStreamSynchronize(g->g.stream));
    });
}
int vfem_grid_get_mask_height(const vfem_grid *g, double *height) {
    return guarded([&] { need(g, "grid"); *height = g->g.maskH; });
}
int vfem_grid_apply_k(vfem_grid *g, const double *u, double *out) {
    return guarded([&] { need(g, "grid"); g->g.applyK(u, out); });
}
int vfem_grid_build_load(vfem_grid *g, double *out) {
    return guarded([&] { need(g, "grid"); g->g.buildLoad(out); });
}
struct vfem_lbl {
    vfem::LBL e;
    vfem_lbl(vfem::Grid *g, int c, int64_t s, int p) : e(g, c, s, p) {}
};
int vfem_lbl_create(vfem_grid *g, int64_t coarsenings, int64_t slots, int precision, vfem_lbl **out) {
    return guarded([&] {
        need(g, "grid");
        need(out, "out");
        *out = new vfem_lbl(&g->g, (int)coarsenings, slots, precision);
    });
}
int vfem_lbl_destroy(vfem_lbl *e) {
    return guarded([&] { delete e; });
}
int vfem_lbl_set_sweep_form(vfem_lbl *e, int form) {
    return guarded([&] {
        need(e, "evaluator");
        e->e.setSweepForm(form);
    });
}
int vfem_lbl_set_init(vfem_lbl *e, int kind, int history) {
    return guarded([&] {
        need(e, "evaluator");
        e->e.setInit(kind, history);
    });
}
int vfem_lbl_run(vfem_lbl *e, const int64_t *layers, int64_t count, int64_t max_iter, double tol,
                 int64_t mg_iterations, int64_t mg_smoothing_iterations, int full_multigrid, int zero_init,
                 double *compliance_out, int64_t *iterations_out, double *gradient_sum_out) {
    return guarded([&] {
        need(e, "evaluator");
        need(layers, "layers");
        need(compliance_out, "compliance_out");
        e->e.run(layers, count, max_iter, tol, mg_iterations, mg_smoothing_iterations, full_multigrid != 0,
                 zero_init != 0, compliance_out, iterations_out, gradient_sum_out);
    });
}
int vfem_grid_adjoint_sensitivity(vfem_grid *g, const double *lambda, const double *u, double load_weight,
                                  double stiffness_weight, double *grad_out) {
    return guarded([&] {
        need(g, "grid");
        need(lambda, "lambda");
        need(u, "u");
        need(grad_out, "grad_out");
        g->g.adjointSensitivity(lambda, u, load_weight, stiffness_weight, grad_out);
    });
}
int vfem_grid_compliance_gradient(vfem_grid *g, const double *u, double *grad_out) {
    return guarded([&] { need(g, "grid"); g->g.complianceGradient(u, grad_out); });
}
int vfem_grid_element_energy(vfem_grid *g, const double *u, double *out) {
    return guarded([&] { need(g, "grid"); g->g.elementEnergy(u, out); });
}

int vfem_mg_create(vfem_grid *g, int num_coarsening_levels, vfem_mg **out) {
    return guarded([&] { need(g, "grid"); need(out, "out"); *out = new vfem_mg(&g->g, num_coarsening_levels); });
}
int vfem_mg_destroy(vfem_mg *mg) {
    return guarded([&] { delete mg; });
}
int vfem_mg_num_levels(const vfem_mg *mg, int *levels) {
    return guarded([&] { need(mg, "mg"); *levels = mg->m.L(); });
}
int vfem_mg_level_dims(const vfem_mg *mg, int level, int64_t elems[3]) {
    return guarded([&] {
        need(mg, "mg");
        if (level < 0 || level >= mg->m.L()) throw Error(ERR_ARG, "level out of range");
        for (int d = 0; d < 3; ++d) elems[d] = mg->m.lv[level].g.ne[d];
    });
}
int vfem_mg_level_dirichlet_mask(const vfem_mg *mg, int level, uint8_t *mask_out) {
    return guarded([&] {
        need(mg, "mg");
        if (level < 0 || level >= mg->m.L()) throw Error(ERR_ARG, "level out of range");
        const std::vector<uint8_t> &m = level == 0 ? mg->m.fine->dmask_h : mg->m.lv[level].dmask_h;
        std::memcpy(mask_out, m.data(), m.size());
    });
}
int vfem_mg_set_precision(vfem_mg *mg, int precision, int outer_matvec) {
    return guarded([&] {
        need(mg, "mg");
        if (outer_matvec != MATVEC_FP64 && outer_matvec != MATVEC_DF && outer_matvec != MATVEC_DF_SIMT)
            throw Error(ERR_ARG, "unknown matvec kind");
        mg->m.setPrecision(precision);
        if (mg->m.outerMatvec != outer_matvec) mg->m.clearGraphs();
        mg->m.outerMatvec = outer_matvec;
    });
}
int vfem_mg_outer_apply(vfem_mg *mg, const double *u, const double *rhs, double *out) {
    return guarded([&] {
        need(mg, "mg");
        need(u, "u");
        need(out, "out");
        mg->m.outerApply(u, out, rhs);
    });
}
int vfem_mg_outer_matvec_kind(const vfem_mg *mg, int *kind) {
    return guarded([&] {
        need(mg, "mg");
        need(kind, "kind");
        *kind = mg->m.outerKind();
    });
}
int vfem_tc_fit_k0(const double *k0_576, double *scale, uint16_t *tiles_2048, int *ok) {
    return guarded([&] {
        need(k0_576, "K0");
        need(scale, "scale");
        need(tiles_2048, "tiles");
        need(ok, "ok");
        *ok = tc_fit_k0(k0_576, scale, tiles_2048) ? 1 : 0;
    });
}
int vfem_debug_pivot_reciprocals(const double *d, int64_t n, double *recip_out, double *rsqrt_out) {
    return guarded([&] {
        need(d, "d");
        need(recip_out, "recip");
        need(rsqrt_out, "rsqrt");
        if (n < 0) throw Error(ERR_ARG, "Invalid input size");
        if (n == 0) return;
        cudaStream_t st = nullptr;
        View vi, vr, vs;
        viewIn(vi, d, n * sizeof(double), st);
        viewOut(vr, recip_out, n * sizeof(double));
        viewOut(vs, rsqrt_out, n * sizeof(double));
        launch_newton_helpers((const double *)vi.d, n, (double *)vr.d, (double *)vs.d, st);
        finishOut(vr, st);
        finishOut(vs, st);
    });
}
int vfem_mg_set_stencil_bf16(vfem_mg *mg, int on) {
    return guarded([&] {
        need(mg, "mg");
        mg->m.setBf16Stencils(on != 0);
    });
}
int vfem_mg_set_sweep_form(vfem_mg *mg, int form) {
    return guarded([&] {
        need(mg, "mg");
        mg->m.setSweepForm(form);
    });
}
int vfem_mg_stiffness_rebuilds(const vfem_mg *mg, int64_t *full, int64_t *band) {
    return guarded([&] {
        need(mg, "mg");
        need(full, "full");
        need(band, "band");
        *full = mg->m.fullRebuilds;
        *band = mg->m.bandRebuilds;
    });
}
int vfem_mg_set_device_loop(vfem_mg *mg, int on) {
    return guarded([&] {
        need(mg, "mg");
        mg->m.deviceLoop = on != 0;
    });
}
int vfem_mg_set_use_graphs(vfem_mg *mg, int use) {
    return guarded([&] { need(mg, "mg"); mg->m.useGraphs = use != 0; mg->m.clearGraphs(); });
}
int vfem_mg_set_symmetric_gs(vfem_mg *mg, int symmetric) {
    return guarded([&] { need(mg, "mg"); mg->m.symmetricGS = symmetric != 0; });
}
int vfem_mg_set_mask_layer(vfem_mg *mg, int64_t layer) {
    return guarded([&] {
        need(mg, "mg");
        mg->m.setMaskLayer(layer);
        VFEM_CUDA(cudaStreamSynchronize(mg->m.fine->stream));
    });
}
int vfem_mg_update_stiffness(vfem_mg *mg) {
    return guarded([&] { need(mg, "mg"); mg->m.updateStiffness(); });
}
int vfem_mg_apply_k(vfem_mg *mg, int level, const double *u, double *out) {
    return guarded([&] { need(mg, "mg"); mg->m.applyK(level, u, out); });
}
int vfem_mg_residual(vfem_mg *mg, int level, const double *u, const double *b, double *r_out) {
    return guarded([&] { need(mg, "mg"); mg->m.residual(level, u, b, r_out); });
}
int vfem_mg_smooth(vfem_mg *mg, int level, double *u_inout, const double *b, int forward) {
    return guarded([&] { need(mg, "mg"); mg->m.smooth(level, u_inout, b, forward != 0); });
}
int vfem_mg_restrict(vfem_mg *mg, int level, const double *fine, double *coarse_out) {
    return guarded([&] { need(mg, "mg"); mg->m.restrictTo(level, fine, coarse_out); });
}
int vfem_mg_interpolate(vfem_mg *mg, int level, const double *coarse, double *fine_inout, int accumulate) {
    return guarded([&] { need(mg, "mg"); mg->m.interpolate(level, coarse, fine_inout, accumulate != 0); });
}
int vfem_mg_coarse_solve(vfem_mg *mg, const double *b, double *x_out) {
    return guarded([&] { need(mg, "mg"); mg->m.coarseSolve(b, x_out); });
}
int vfem_mg_zero_dirichlet(vfem_mg *mg, int level, double *u_inout) {
    return guarded([&] { need(mg, "mg"); mg->m.zeroDirichlet(level, u_inout); });
}
int vfem_mg_solve(vfem_mg *mg, const double *u, const double *f, int64_t num_steps, int64_t num_smoothing_steps,
                  int zero_dirichlet, int full_multigrid, double *x_out) {
    return guarded([&] {
        need(mg, "mg");
        mg->m.solve(u, f, num_steps, num_smoothing_steps, zero_dirichlet != 0, full_multigrid != 0, x_out);
    });
}
int vfem_mg_pcg(vfem_mg *mg, double *x_inout, const double *b, int64_t max_iter, double tol, int64_t mg_iterations,
                int64_t mg_smoothing_iterations, int full_multigrid, int dirichlet_already_satisfied,
                vfem_pcg_callback cb, void *user, vfem_pcg_stats *stats) {
    return guarded([&] {
        need(mg, "mg"); need(x_inout, "x"); need(b, "b");
        if (max_iter < 0 || mg_iterations < 0 || mg_smoothing_iterations < 0) throw Error(ERR_ARG, "negative count");
        PcgStats s = mg->m.pcg(x_inout, b, max_iter, tol, mg_iterations, mg_smoothing_iterations, full_multigrid != 0,
                               dirichlet_already_satisfied != 0, cb, user);
        if (stats) {
            stats->iterations = s.iterations;
            stats->relres = s.relres;
            stats->rsq = s.rsq;
            stats->bnorm2 = s.bnorm2;
        }
    });
}

int vfem_mg_get_stream(const vfem_mg *mg, void **stream) {
    return guarded([&] { need(mg, "mg"); *stream = (void *)mg->m.fine->stream; });
}
int vfem_mg_time_kernel(vfem_mg *mg, int kernel, int reps, double *ms, double *bytes) {
    return guarded([&] {
        need(mg, "mg");
        const double t = mg->m.timeKernel(kernel, reps);
        if (ms) *ms = t;
        if (bytes) *bytes = mg->m.kernelBytes(kernel);
    });
}
int vfem_mg_profile(vfem_mg *mg, int64_t mg_iterations, int64_t mg_smoothing_iterations, int reps, char *names_out,
                    int64_t names_cap, double *ms_out, int max_entries, int *num_entries) {
    return guarded([&] {
        need(mg, "mg"); need(names_out, "names"); need(ms_out, "ms"); need(num_entries, "count");
        auto prof = mg->m.profile(mg_iterations, mg_smoothing_iterations, reps);
        std::string names;
        int n = 0;
        for (const auto &kv : prof) {
            if (n >= max_entries) break;
            names += kv.first + "\n";
            ms_out[n++] = kv.second;
        }
        if ((int64_t)names.size() + 1 > names_cap) throw Error(ERR_ARG, "name buffer too small");
        std::memcpy(names_out, names.c_str(), names.size() + 1);
        *num_entries = n;
    });
}
int vfem_kernel_launch_count(uint64_t *count) {
    return guarded([&] { *count = launchCounter(); });
}

int vfem_lbl2_create(vfem_grid2 *g, int64_t coarsenings, int64_t slots, int precision, vfem_lbl2 **out) {
    return guarded([&] {
        need(g, "grid"); need(out, "out");
        *out = new vfem_lbl2(&g->g, (int)coarsenings, slots, precision);
    });
}
int vfem_lbl2_destroy(vfem_lbl2 *e) {
    return guarded([&] { delete e; });
}
int vfem_lbl2_set_init(vfem_lbl2 *e, int kind, int history) {
    return guarded([&] { need(e, "evaluator"); e->e.setInit(kind, history); });
}
int vfem_lbl2_run(vfem_lbl2 *e, const int64_t *layers, int64_t count, int64_t max_iter, double tol,
                  int64_t mg_iterations, int64_t mg_smoothing_iterations, int full_multigrid, int zero_init,
                  double *compliance_out, int64_t *iterations_out, double *gradient_sum_out) {
    return guarded([&] {
        need(e, "evaluator"); need(layers, "layers"); need(compliance_out, "compliance_out");
        e->e.run(layers, count, max_iter, tol, mg_iterations, mg_smoothing_iterations, full_multigrid != 0,
                 zero_init != 0, compliance_out, iterations_out, gradient_sum_out);
    });
}
int vfem_smoothing_filter2(const int64_t dims[2], int radius, int type, const double *in, double *out) {
    return guarded([&] {
        need(dims, "dims");
        int d[3] = {0, 0, 1};
        for (int i = 0; i < 2; ++i) {
            if (dims[i] <= 0) throw Error(ERR_ARG, "invalid dims");
            d[i] = (int)dims[i];
        }
        if (type != 0 && type != 1) throw Error(ERR_ARG, "Unexpected smoothing kernel type");
        const int64_t n = (int64_t)d[0] * d[1];
        cudaStream_t st = nullptr;
        View vi, vo;
        viewIn(vi, in, n * sizeof(double), st);
        viewOut(vo, out, n * sizeof(double));
        launch_smoothing_filter(d, radius, type, (const double *)vi.d, (double *)vo.d, st, 2);
        finishOut(vo, st);
    });
}
int vfem_smoothing_filter(const int64_t dims[3], int radius, int type, const double *in, double *out) {
    return guarded([&] {
        need(dims, "dims");
        int d[3];
        for (int i = 0; i < 3; ++i) {
            if (dims[i] <= 0) throw Error(ERR_ARG, "invalid dims");
            d[i] = (int)dims[i];
        }
        if (type != 0 && type != 1) throw Error(ERR_ARG, "Unexpected smoothing kernel type");
        const int64_t n = (int64_t)d[0] * d[1] * d[2];
        cudaStream_t st = nullptr;
        View vi, vo;
        viewIn(vi, in, n * sizeof(double), st);
        viewOut(vo, out, n * sizeof(double));
        launch_smoothing_filter(d, radius, type, (const double *)vi.d, (double *)vo.d, st);
        finishOut(vo, st);
    });
}
int vfem_smoothing_filter_noalloc(const int64_t dims[3], int radius, int type, const double *in_dev,
                                  double *out_dev, void *stream) {
    return guarded([&] {
        need(dims, "dims"); need(in_dev, "in"); need(out_dev, "out");
        int d[3];
        for (int i = 0; i < 3; ++i) {
            if (dims[i] <= 0 || dims[i] > (1 << 20)) throw Error(ERR_ARG, "invalid dims");
            d[i] = (int)dims[i];
        }
        if (type != 0 && type != 1) throw Error(ERR_ARG, "Unexpected smoothing kernel type");
        if (!isDevicePtr(in_dev) || !isDevicePtr(out_dev))
            throw Error(ERR_ARG, "the allocation-free filter takes device pointers only (host arrays would need staging)");
        launch_smoothing_filter_noalloc(d, radius, type, in_dev, out_dev, (cudaStream_t)stream);
    });
}
int vfem_projection_apply(int64_t n, double beta, const double *in, double *out) {
    return guarded([&] {
        if (!(beta > 0)) throw Error(ERR_ARG, "Beta parameter has to be positive");
        View vi, vo;
        viewIn(vi, in, n * sizeof(double), nullptr);
        viewOut(vo, out, n * sizeof(double));
        launch_projection(n, beta, (const double *)vi.d, (double *)vo.d, nullptr);
        finishOut(vo, nullptr);
    });
}
int vfem_projection_backprop(int64_t n, double beta, const double *in, const double *vars, double *out) {
    return guarded([&] {
        if (!(beta > 0)) throw Error(ERR_ARG, "Beta parameter has to be positive");
        View vi, vv, vo;
        viewIn(vi, in, n * sizeof(double), nullptr);
        viewIn(vv, vars, n * sizeof(double), nullptr);
        viewOut(vo, out, n * sizeof(double));
        launch_projection_backprop(n, beta, (const double *)vi.d, (const double *)vv.d, (double *)vo.d, nullptr);
        finishOut(vo, nullptr);
    });
}

int vfem_problem_create(vfem_mg *mg, int num_filters, const int *kinds, const int *radii, const int *types,
                        const double *betas, double volume_fraction, vfem_problem **out) {
    return guarded([&] {
        need(mg, "mg"); need(out, "out");
        std::vector<FilterSpec> f;
        for (int i = 0; i < num_filters; ++i) f.push_back({kinds[i], radii[i], types[i], betas[i]});
        *out = new vfem_problem(&mg->m, f, volume_fraction);
    });
}
int vfem_problem_destroy(vfem_problem *p) {
    return guarded([&] { delete p; });
}
int vfem_problem_set_solver(vfem_problem *p, int64_t cg_iter, double tol, int64_t mg_iterations,
                            int64_t mg_smoothing_iterations, int full_multigrid, int zero_init) {
    return guarded([&] {
        need(p, "problem");
        p->p.cgIter = cg_iter; p->p.tol = tol; p->p.mgIter = mg_iterations; p->p.mgSweeps = mg_smoothing_iterations;
        p->p.fmg = full_multigrid != 0; p->p.zeroInit = zero_init != 0;
    });
}
int vfem_problem_set_vars(vfem_problem *p, const double *x) {
    return guarded([&] { need(p, "problem"); need(x, "x"); p->p.setVars(x, isDevicePtr(x)); });
}
int vfem_problem_get_vars(vfem_problem *p, double *x_out) {
    return guarded([&] {
        need(p, "problem");
        VFEM_CUDA(cudaMemcpy(x_out, p->p.vars[0].p, p->p.be->numElems() * sizeof(double), cudaMemcpyDefault));
    });
}
int vfem_problem_objective(vfem_problem *p, double *value) {
    return guarded([&] { need(p, "problem"); *value = p->p.objective(); });
}
int vfem_problem_gradient(vfem_problem *p, double *grad_out) {
    return guarded([&] { need(p, "problem"); p->p.gradient(grad_out, isDevicePtr(grad_out)); });
}
int vfem_problem_constraint(vfem_problem *p, double *value) {
    return guarded([&] { need(p, "problem"); *value = p->p.constraint(); });
}
int vfem_problem_jacobian(vfem_problem *p, double *jac_out) {
    return guarded([&] { need(p, "problem"); p->p.jacobian(jac_out, isDevicePtr(jac_out)); });
}
int vfem_problem_get_u(vfem_problem *p, double *u_out) {
    return guarded([&] { need(p, "problem"); p->p.getU(u_out, isDevicePtr(u_out)); });
}
int vfem_problem_get_physical(vfem_problem *p, double *x_out) {
    return guarded([&] { need(p, "problem"); p->p.getPhysical(x_out, isDevicePtr(x_out)); });
}
int vfem_problem_last_solve(vfem_problem *p, vfem_pcg_stats *stats) {
    return guarded([&] {
        need(p, "problem");
        stats->iterations = p->p.lastStats.iterations;
        stats->relres = p->p.lastStats.relres;
        stats->rsq = p->p.lastStats.rsq;
        stats->bnorm2 = p->p.lastStats.bnorm2;
    });
}
int vfem_problem_oc_step(vfem_problem *p, double m, double pexp, double ctol, int64_t *probes) {
    return guarded([&] {
        need(p, "problem");
        const int64_t n = p->p.ocStep(m, pexp, ctol);
        if (probes) *probes = n;
    });
}
int vfem_problem_oc_step_with_gradient(vfem_problem *p, double m, double pexp, double ctol,
                                       const double *objective_gradient, int64_t *probes) {
    return guarded([&] {
        need(p, "problem");
        need(objective_gradient, "objective gradient");
        const int64_t n = p->p.ocStep(m, pexp, ctol, objective_gradient);
        if (probes) *probes = n;
    });
}

// ---- triquadratic voxels ----
struct vfem_q2 {
    GridQ2 g;
    vfem_q2(const int ne[3], const double mn[3], const double mx[3]) : g(ne, mn, mx) {}
};
int vfem_q2_create(const int64_t elems[3], const double bbox_min[3], const double bbox_max[3], vfem_q2 **out) {
    return guarded([&] {
        need(elems, "elems");
        need(out, "out");
        int ne[3];
        for (int d = 0; d < 3; ++d) {
            if (elems[d] <= 0 || elems[d] > (1 << 20)) throw Error(ERR_ARG, "elementsPerDimension out of range");
            ne[d] = (int)elems[d];
        }
        *out = new vfem_q2(ne, bbox_min, bbox_max);
    });
}
int vfem_q2_destroy(vfem_q2 *g) {
    return guarded([&] { delete g; });
}
int vfem_q2_dims(const vfem_q2 *g, int64_t *num_nodes, int64_t *num_elements) {
    return guarded([&] {
        need(g, "grid");
        if (num_nodes) *num_nodes = g->g.NN;
        if (num_elements) *num_elements = g->g.NE;
    });
}
int vfem_q2_set_etensor(vfem_q2 *g, double young, double poisson) {
    return guarded([&] { need(g, "grid"); g->g.setETensor(young, poisson); });
}
int vfem_q2_set_material_params(vfem_q2 *g, double E0, double Emin, double gamma, double q, int law) {
    return guarded([&] {
        need(g, "grid");
        if (law != 0 && law != 1) throw Error(ERR_ARG, "unknown interpolation law");
        g->g.setParams(E0, Emin, gamma, q, law);
    });
}
int vfem_q2_set_densities(vfem_q2 *g, const double *rho) {
    return guarded([&] { need(g, "grid"); need(rho, "rho"); g->g.setDensities(rho); });
}
int vfem_q2_get_k0(const vfem_q2 *g, double *out6561) {
    return guarded([&] { need(g, "grid"); need(out6561, "out"); std::memcpy(out6561, g->g.K0.data(), 6561 * sizeof(double)); });
}
int vfem_q2_add_dirichlet(vfem_q2 *g, const double min_corner[3], const double max_corner[3], int cmask) {
    return guarded([&] {
        need(g, "grid");
        need(min_corner, "min_corner");
        need(max_corner, "max_corner");
        g->g.addDirichlet(min_corner, max_corner, (unsigned)cmask);
    });
}
int vfem_q2_get_dirichlet_mask(const vfem_q2 *g, uint8_t *mask_out) {
    return guarded([&] {
        need(g, "grid");
        need(mask_out, "out");
        if (isDevicePtr(mask_out)) VFEM_CUDA(cudaMemcpy(mask_out, g->g.dmask_h.data(), g->g.NN, cudaMemcpyHostToDevice));
        else std::memcpy(mask_out, g->g.dmask_h.data(), g->g.NN);
    });
}
int vfem_q2_apply_k(vfem_q2 *g, const double *u, double *out, int precision, int zero_dirichlet) {
    return guarded([&] {
        need(g, "grid");
        need(u, "u");
        need(out, "out");
        g->g.applyK(u, out, precision, zero_dirichlet != 0);
    });
}
int vfem_q2_smooth(vfem_q2 *g, double *u_inout, const double *b, int forward, int precision) {
    return guarded([&] {
        need(g, "grid");
        need(u_inout, "u");
        need(b, "b");
        g->g.smooth(u_inout, b, forward != 0, precision);
    });
}
int vfem_q2_restrict(const int64_t elems_fine[3], const double *fine, double *coarse) {
    return guarded([&] {
        need(elems_fine, "elems");
        need(fine, "fine");
        need(coarse, "coarse");
        const int ne[3] = {(int)elems_fine[0], (int)elems_fine[1], (int)elems_fine[2]};
        q2Restrict(ne, fine, coarse);
    });
}
int vfem_q2_interpolate(const int64_t elems_fine[3], const double *coarse, double *fine, int accumulate) {
    return guarded([&] {
        need(elems_fine, "elems");
        need(fine, "fine");
        need(coarse, "coarse");
        const int ne[3] = {(int)elems_fine[0], (int)elems_fine[1], (int)elems_fine[2]};
        q2Interpolate(ne, coarse, fine, accumulate != 0);
    });
}
int vfem_q2_set_outer_matvec(vfem_q2 *g, int outer_matvec) {
    return guarded([&] {
        need(g, "grid");
        if (outer_matvec != MATVEC_FP64 && outer_matvec != MATVEC_DF) throw Error(ERR_ARG, "unknown matvec kind");
        g->g.outerDF = outer_matvec == MATVEC_DF;
    });
}
int vfem_q2_pcg(vfem_q2 *g, int64_t coarsenings, double *x_inout, const double *b, int64_t max_iter, double tol,
                int64_t mg_smoothing_iterations, vfem_pcg_stats *stats) {
    return guarded([&] {
        need(g, "grid");
        need(x_inout, "x");
        need(b, "b");
        const PcgStats s = g->g.pcg(x_inout, b, max_iter, tol, (int)coarsenings, mg_smoothing_iterations);
        if (stats) {
            stats->iterations = s.iterations;
            stats->relres = s.relres;
            stats->rsq = s.rsq;
            stats->bnorm2 = s.bnorm2;
        }
    });
}
int vfem_q2_set_hierarchy(vfem_q2 *g, int hierarchy) {
    return guarded([&] {
        need(g, "grid");
        g->g.setHierarchy(hierarchy);
    });
}
int vfem_q2_set_precision(vfem_q2 *g, int precision) {
    return guarded([&] {
        need(g, "grid");
        g->g.setPrecision(precision);
    });
}
static void q2Level(vfem_q2 *g, int64_t coarsenings, int level) {
    need(g, "grid");
    if (coarsenings < 1 || coarsenings > 30) throw Error(ERR_ARG, "the triquadratic hierarchy needs at least one coarsening");
    if (level < 0 || level > coarsenings) throw Error(ERR_ARG, "level out of range");
}
static void q2Precision(int precision) {
    if (precision != PREC_FP64 && precision != PREC_MIXED) throw Error(ERR_ARG, "precision must be fp64 or mixed");
}
int vfem_q2_mg_num_nodes(vfem_q2 *g, int64_t coarsenings, int level, int64_t *num_nodes) {
    return guarded([&] {
        q2Level(g, coarsenings, level);
        need(num_nodes, "num_nodes");
        *num_nodes = g->g.mgLevelNodes((int)coarsenings, level);
    });
}
int vfem_q2_mg_level_dirichlet(vfem_q2 *g, int64_t coarsenings, int level, uint8_t *mask_out) {
    return guarded([&] {
        q2Level(g, coarsenings, level);
        need(mask_out, "mask_out");
        g->g.mgLevelDirichlet((int)coarsenings, level, mask_out);
    });
}
int vfem_q2_mg_level_ke(vfem_q2 *g, int64_t coarsenings, int level, int precision, double *out) {
    return guarded([&] {
        q2Level(g, coarsenings, level);
        q2Precision(precision);
        need(out, "out");
        g->g.mgLevelKe((int)coarsenings, level, precision, out);
    });
}
int vfem_q2_mg_smooth(vfem_q2 *g, int64_t coarsenings, int level, double *u_inout, const double *b, int forward,
                      int precision) {
    return guarded([&] {
        q2Level(g, coarsenings, level);
        q2Precision(precision);
        need(u_inout, "u");
        need(b, "b");
        g->g.mgSmooth((int)coarsenings, level, u_inout, b, forward != 0, precision);
    });
}
int vfem_q2_mg_residual(vfem_q2 *g, int64_t coarsenings, int level, const double *u, const double *b, double *r,
                        int precision) {
    return guarded([&] {
        q2Level(g, coarsenings, level);
        q2Precision(precision);
        need(u, "u");
        need(b, "b");
        need(r, "r");
        g->g.mgResidual((int)coarsenings, level, u, b, r, precision);
    });
}
int vfem_q2_mg_coarse_solve(vfem_q2 *g, int64_t coarsenings, const double *b, double *x, int precision) {
    return guarded([&] {
        q2Level(g, coarsenings, 0);
        q2Precision(precision);
        need(b, "b");
        need(x, "x");
        g->g.mgCoarseSolve((int)coarsenings, b, x, precision);
    });
}
int vfem_q2_mg_vcycle(vfem_q2 *g, int64_t coarsenings, const double *b, double *x, int64_t mg_smoothing_iterations,
                      int precision) {
    return guarded([&] {
        q2Level(g, coarsenings, 0);
        q2Precision(precision);
        need(b, "b");
        need(x, "x");
        if (mg_smoothing_iterations < 0) throw Error(ERR_ARG, "mgSmoothingIterations must be non-negative");
        g->g.mgVcycle((int)coarsenings, b, x, mg_smoothing_iterations, precision);
    });
}
int vfem_q2_time_smooth(vfem_q2 *g, int precision, int reps, double *ms, double *bytes) {
    return guarded([&] {
        need(g, "grid");
        need(ms, "ms");
        need(bytes, "bytes");
        *ms = g->g.timeSmooth(precision, reps, bytes);
    });
}
int vfem_q2_time_apply_k(vfem_q2 *g, int precision, int reps, double *ms, double *bytes) {
    return guarded([&] {
        need(g, "grid");
        need(ms, "ms");
        need(bytes, "bytes");
        *ms = g->g.timeApplyK(precision, reps, bytes);
    });
}


// ---- 2D: TensorProductSimulator<double, 1, 1> / MultigridSolver<double, 1, 1> ----
int vfem_grid2_create(const int64_t elems[2], const double bbox_min[2], const double bbox_max[2], vfem_grid2 **out) {
    return guarded([&] {
        need(elems, "elems"); need(bbox_min, "bbox"); need(bbox_max, "bbox"); need(out, "out");
        int ne[2];
        for (int d = 0; d < 2; ++d) {
            if (elems[d] <= 0 || elems[d] > (1 << 24)) throw Error(ERR_ARG, "invalid elementsPerDimension");
            ne[d] = (int)elems[d];
        }
        if ((int64_t)(ne[0] + 1) * (ne[1] + 1) > ((int64_t)1 << 31)) throw Error(ERR_ARG, "grid too large");
        *out = new vfem_grid2(ne, bbox_min, bbox_max);
    });
}
int vfem_grid2_destroy(vfem_grid2 *g) {
    return guarded([&] { delete g; });
}
int vfem_grid2_dims(const vfem_grid2 *g, int64_t elems[2], int64_t *num_nodes, int64_t *num_elements) {
    return guarded([&] {
        need(g, "grid");
        if (elems) for (int d = 0; d < 2; ++d) elems[d] = g->g.g.ne[d];
        if (num_nodes) *num_nodes = g->g.g.NN;
        if (num_elements) *num_elements = g->g.g.NE;
    });
}
int vfem_grid2_set_etensor(vfem_grid2 *g, double young, double poisson) {
    return guarded([&] {
        need(g, "grid");
        g->g.setETensor(young, poisson);
    });
}
int vfem_grid2_get_etensor(const vfem_grid2 *g, double *young, double *poisson) {
    return guarded([&] {
        need(g, "grid");
        *young = g->g.Eyoung;
        *poisson = g->g.nu;
    });
}
int vfem_grid2_get_k0(const vfem_grid2 *g, double *out64) {
    return guarded([&] {
        need(g, "grid"); need(out64, "out");
        std::memcpy(out64, g->g.K0.a, 64 * sizeof(double));
    });
}
int vfem_grid2_set_material_params(vfem_grid2 *g, double E0, double Emin, double gamma, double q, int law) {
    return guarded([&] { need(g, "grid"); g->g.setParams(E0, Emin, gamma, q, law); });
}
int vfem_grid2_get_material_params(const vfem_grid2 *g, double *E0, double *Emin, double *gamma, double *q, int *law) {
    return guarded([&] {
        need(g, "grid");
        *E0 = g->g.E0; *Emin = g->g.Emin; *gamma = g->g.gamma; *q = g->g.q; *law = g->g.law;
    });
}
int vfem_grid2_set_densities(vfem_grid2 *g, const double *rho) {
    return guarded([&] { need(g, "grid"); need(rho, "rho"); g->g.setDensities(rho, true); });
}
int vfem_grid2_get_densities(vfem_grid2 *g, double *rho_out) {
    return guarded([&] {
        need(g, "grid"); need(rho_out, "out");
        VFEM_CUDA(cudaMemcpy(rho_out, g->g.rho.p, g->g.g.NE * sizeof(double), cudaMemcpyDefault));
    });
}
int vfem_grid2_set_uniform_densities(vfem_grid2 *g, double value) {
    return guarded([&] { need(g, "grid"); g->g.setUniformDensities(value); });
}
int vfem_grid2_get_young_moduli(vfem_grid2 *g, double *out) {
    return guarded([&] {
        need(g, "grid"); need(out, "out");
        VFEM_CUDA(cudaMemcpy(out, g->g.Y.p, g->g.g.NE * sizeof(double), cudaMemcpyDefault));
    });
}
int vfem_grid2_add_dirichlet(vfem_grid2 *g, const double u[2], const double min_corner[2], const double max_corner[2],
                             uint32_t component_mask) {
    return guarded([&] {
        need(g, "grid"); need(u, "u"); need(min_corner, "minCorner"); need(max_corner, "maxCorner");
        g->g.addDirichlet(u, min_corner, max_corner, component_mask);
    });
}
int vfem_grid2_apply_symmetry(vfem_grid2 *g, const int axes[2], const int max_face[2]) {
    return guarded([&] { need(g, "grid"); need(axes, "axes"); need(max_face, "max_face"); g->g.applySymmetry(axes, max_face); });
}
int vfem_grid2_set_nodal_forces(vfem_grid2 *g, const double *forces) {
    return guarded([&] { need(g, "grid"); need(forces, "forces"); g->g.setForces(forces); });
}
int vfem_grid2_get_dirichlet_mask(const vfem_grid2 *g, uint8_t *mask_out) {
    return guarded([&] {
        need(g, "grid"); need(mask_out, "out");
        VFEM_CUDA(cudaMemcpy(mask_out, g->g.hmask.data(), g->g.g.NN, cudaMemcpyDefault));
    });
}
int vfem_grid2_get_dirichlet_values(const vfem_grid2 *g, double *values_out) {
    return guarded([&] {
        need(g, "grid"); need(values_out, "out");
        VFEM_CUDA(cudaMemcpy(values_out, g->g.hval.data(), 2 * g->g.g.NN * sizeof(double), cudaMemcpyDefault));
    });
}
int vfem_grid2_set_gravity(vfem_grid2 *g, const double gravity[2]) {
    return guarded([&] { need(g, "grid"); need(gravity, "gravity"); g->g.setGravity(gravity); });
}
int vfem_grid2_get_gravity(const vfem_grid2 *g, double gravity[2]) {
    return guarded([&] {
        need(g, "grid"); need(gravity, "gravity");
        gravity[0] = g->g.grav[0];
        gravity[1] = g->g.grav[1];
    });
}
int vfem_grid2_set_mask_layer(vfem_grid2 *g, int64_t layer) {
    return guarded([&] { need(g, "grid"); g->g.setMaskLayer(layer); });
}
int vfem_grid2_get_mask_height(const vfem_grid2 *g, double *height) {
    return guarded([&] { need(g, "grid"); need(height, "height"); *height = g->g.maskH; });
}
int vfem_grid2_apply_k(vfem_grid2 *g, const double *u, double *out) {
    return guarded([&] { need(g, "grid"); g->g.applyK(u, out); });
}
int vfem_grid2_build_load(vfem_grid2 *g, double *out) {
    return guarded([&] {
        need(g, "grid");
        View vo;
        viewOut(vo, out, 2 * g->g.g.NN * sizeof(double));
        g->g.buildLoadDev((double *)vo.d);
        finishOut(vo, g->g.stream);
    });
}
int vfem_grid2_compliance_gradient(vfem_grid2 *g, const double *u, double *grad_out) {
    return guarded([&] { need(g, "grid"); g->g.adjoint(u, u, 1.0, 0.5, grad_out); });
}
int vfem_grid2_adjoint_sensitivity(vfem_grid2 *g, const double *lambda, const double *u, double load_weight,
                                   double stiffness_weight, double *out) {
    return guarded([&] { need(g, "grid"); g->g.adjoint(lambda, u, load_weight, stiffness_weight, out); });
}
int vfem_grid2_element_energy(vfem_grid2 *g, const double *u, double *out) {
    return guarded([&] { need(g, "grid"); g->g.elementEnergy(u, out); });
}
int vfem_mg2_create(vfem_grid2 *g, int num_coarsening_levels, vfem_mg2 **out) {
    return guarded([&] {
        need(g, "grid"); need(out, "out");
        *out = new vfem_mg2(&g->g, num_coarsening_levels);
    });
}
int vfem_mg2_destroy(vfem_mg2 *mg) {
    return guarded([&] { delete mg; });
}
int vfem_mg2_num_levels(const vfem_mg2 *mg, int *levels) {
    return guarded([&] { need(mg, "mg"); *levels = mg->m.L(); });
}
int vfem_mg2_level_dims(const vfem_mg2 *mg, int level, int64_t elems[2]) {
    return guarded([&] {
        need(mg, "mg");
        if (level < 0 || level >= mg->m.L()) throw Error(ERR_ARG, "level out of range");
        elems[0] = mg->m.lv[level].g.ne[0];
        elems[1] = mg->m.lv[level].g.ne[1];
    });
}
int vfem_mg2_level_dirichlet_mask(const vfem_mg2 *mg, int level, uint8_t *mask_out) {
    return guarded([&] {
        need(mg, "mg"); need(mask_out, "out");
        if (level < 0 || level >= mg->m.L()) throw Error(ERR_ARG, "level out of range");
        const std::vector<uint8_t> &m = level == 0 ? mg->m.fine->hmask : mg->m.lv[level].hmask;
        VFEM_CUDA(cudaMemcpy(mask_out, m.data(), m.size(), cudaMemcpyDefault));
    });
}
int vfem_mg2_set_precision(vfem_mg2 *mg, int precision) {
    return guarded([&] { need(mg, "mg"); mg->m.setPrecision(precision); });
}
int vfem_mg2_set_outer_matvec(vfem_mg2 *mg, int kind) {
    return guarded([&] { need(mg, "mg"); mg->m.setOuterMatvec(kind); });
}
int vfem_mg2_set_use_graphs(vfem_mg2 *mg, int use) {
    return guarded([&] { need(mg, "mg"); mg->m.useGraphs = use != 0; });
}
int vfem_mg2_set_symmetric_gs(vfem_mg2 *mg, int symmetric) {
    return guarded([&] { need(mg, "mg"); mg->m.symmetricGS = symmetric != 0; });
}
int vfem_mg2_set_mask_layer(vfem_mg2 *mg, int64_t layer) {
    return guarded([&] { need(mg, "mg"); mg->m.setMaskLayer(layer); });
}
int vfem_mg2_update_stiffness(vfem_mg2 *mg) {
    return guarded([&] { need(mg, "mg"); mg->m.updateStiffness(); });
}
int vfem_mg2_apply_k(vfem_mg2 *mg, int level, const double *u, double *out) {
    return guarded([&] { need(mg, "mg"); mg->m.applyK(level, u, out); });
}
int vfem_mg2_residual(vfem_mg2 *mg, int level, const double *u, const double *b, double *r_out) {
    return guarded([&] { need(mg, "mg"); mg->m.residual(level, u, b, r_out); });
}
int vfem_mg2_smooth(vfem_mg2 *mg, int level, double *u_inout, const double *b, int forward) {
    return guarded([&] { need(mg, "mg"); mg->m.smooth(level, u_inout, b, forward != 0); });
}
int vfem_mg2_restrict(vfem_mg2 *mg, int level, const double *fine, double *coarse_out) {
    return guarded([&] { need(mg, "mg"); mg->m.restrictTo(level, fine, coarse_out); });
}
int vfem_mg2_interpolate(vfem_mg2 *mg, int level, const double *coarse, double *fine_inout, int accumulate) {
    return guarded([&] { need(mg, "mg"); mg->m.interpolate(level, coarse, fine_inout, accumulate != 0); });
}
int vfem_mg2_coarse_solve(vfem_mg2 *mg, const double *b, double *x_out) {
    return guarded([&] { need(mg, "mg"); mg->m.coarseSolve(b, x_out); });
}
int vfem_mg2_zero_dirichlet(vfem_mg2 *mg, int level, double *u_inout) {
    return guarded([&] { need(mg, "mg"); mg->m.zeroDirichlet(level, u_inout); });
}
int vfem_mg2_solve(vfem_mg2 *mg, const double *u, const double *f, int64_t num_steps, int64_t num_smoothing_steps,
                   int zero_dirichlet, int full_multigrid, double *x_out) {
    return guarded([&] {
        need(mg, "mg");
        if (num_steps < 0 || num_smoothing_steps < 0) throw Error(ERR_ARG, "negative count");
        mg->m.solve(u, f, num_steps, num_smoothing_steps, zero_dirichlet != 0, full_multigrid != 0, x_out);
    });
}
int vfem_mg2_pcg(vfem_mg2 *mg, double *x_inout, const double *b, int64_t max_iter, double tol, int64_t mg_iterations,
                 int64_t mg_smoothing_iterations, int full_multigrid, int dirichlet_already_satisfied,
                 vfem_pcg_callback cb, void *user, vfem_pcg_stats *stats) {
    return guarded([&] {
        need(mg, "mg"); need(x_inout, "x"); need(b, "b");
        if (max_iter < 0 || mg_iterations < 0 || mg_smoothing_iterations < 0) throw Error(ERR_ARG, "negative count");
        PcgStats s = mg->m.pcg(x_inout, b, max_iter, tol, mg_iterations, mg_smoothing_iterations, full_multigrid != 0,
                               dirichlet_already_satisfied != 0, cb, user);
        if (stats) {
            stats->iterations = s.iterations;
            stats->relres = s.relres;
            stats->rsq = s.rsq;
            stats->bnorm2 = s.bnorm2;
        }
    });
}
int vfem_mg2_time_kernel(vfem_mg2 *mg, int kernel, int reps, double *ms) {
    return guarded([&] {
        need(mg, "mg"); need(ms, "ms");
        if (reps <= 0) throw Error(ERR_ARG, "reps must be positive");
        *ms = mg->m.timeKernel(kernel, reps);
    });
}
int vfem_problem2_create(vfem_mg2 *mg, int num_filters, const int *kinds, const int *radii, const int *types,
                         const double *betas, double volume_fraction, vfem_problem **out) {
    return guarded([&] {
        need(mg, "mg"); need(out, "out");
        std::vector<FilterSpec> f;
        for (int i = 0; i < num_filters; ++i) f.push_back({kinds[i], radii[i], types[i], betas[i]});
        *out = new vfem_problem(makeBackend2D(&mg->m), f, volume_fraction);
    });
}

}  // extern "C"

// ---------------- Method of Moving Asymptotes ----------------
struct vfem_mma {
    vfem::MMAOpt o;
    vfem_mma(int64_t n, int m, const double *xmin, const double *xmax, vfem_mma_f f, vfem_mma_df df, void *user)
        : o(n, m, xmin, xmax, f, df, user) {}
};
int vfem_mma_create(int64_t num_vars, int num_constraints, const double *xmin, const double *xmax, vfem_mma_f f,
                    vfem_mma_df df_dx, void *user, vfem_mma **out) {
    return guarded([&] {
        need(xmin, "xmin");
        need(xmax, "xmax");
        if (!f || !df_dx) throw vfem::Error(vfem::ERR_ARG, "f and df_dx callbacks are required");
        need(out, "out");
        *out = new vfem_mma(num_vars, num_constraints, xmin, xmax, f, df_dx, user);
    });
}
int vfem_mma_destroy(vfem_mma *o) {
    return guarded([&] { delete o; });
}
int vfem_mma_set_initial_var(vfem_mma *o, const double *x0) {
    return guarded([&] {
        need(o, "optimizer");
        need(x0, "x0");
        o->o.setInitialVar(x0);
    });
}
int vfem_mma_enable_gcmma(vfem_mma *o, int enable) {
    return guarded([&] {
        need(o, "optimizer");
        o->o.gcmma = enable != 0;
    });
}
int vfem_mma_step(vfem_mma *o) {
    return guarded([&] {
        need(o, "optimizer");
        o->o.step();
    });
}
int vfem_mma_get_optimal_var(vfem_mma *o, double *x_out) {
    return guarded([&] {
        need(o, "optimizer");
        need(x_out, "x");
        o->o.getOptimalVar(x_out);
    });
}

// ---------------- Upsample / VertexToCell / Langelaar filters ----------------
namespace {
void dims3(const int64_t d[3], int out[3], int minimum, const char *msg) {
    for (int a = 0; a < 3; ++a) {
        if (d[a] < minimum || d[a] > (int64_t)1 << 30) throw vfem::Error(vfem::ERR_ARG, msg);
        out[a] = (int)d[a];
    }
}
// run a filter kernel on caller arrays (host or device) of nin and nout doubles
template <typename F>
void filter_call(const double *in, int64_t nin, double *out, int64_t nout, F launch) {
    vfem::View vi, vo;
    vfem::viewIn(vi, in, nin * sizeof(double), 0);
    vfem::viewOut(vo, out, nout * sizeof(double));
    launch((const double *)vi.d, (double *)vo.d);
    vfem::finishOut(vo, 0);
    VFEM_CUDA(cudaDeviceSynchronize());
}
int64_t prod3(const int d[3]) { return (int64_t)d[0] * d[1] * d[2]; }
}  // namespace

int vfem_upsample_filter(const int64_t in_dims[3], int64_t factor, const double *in, double *out) {
    return guarded([&] {
        need(in, "in");
        need(out, "out");
        int d[3];
        dims3(in_dims, d, 2, "Interpolation can only be applied to a 2^d grid or larger");
        if (factor < 1) throw vfem::Error(vfem::ERR_ARG, "factor must be positive");
        const int F = (int)factor;
        const int o[3] = {(d[0] - 1) * F + 1, (d[1] - 1) * F + 1, (d[2] - 1) * F + 1};
        filter_call(in, prod3(d), out, prod3(o), [&](const double *a, double *b) { vfem::launch_upsample(d, F, a, b, 0); });
    });
}
int vfem_upsample_filter_backprop(const int64_t in_dims[3], int64_t factor, const double *g, double *out) {
    return guarded([&] {
        need(g, "g");
        need(out, "out");
        int d[3];
        dims3(in_dims, d, 2, "Interpolation can only be applied to a 2^d grid or larger");
        if (factor < 1) throw vfem::Error(vfem::ERR_ARG, "factor must be positive");
        const int F = (int)factor;
        const int o[3] = {(d[0] - 1) * F + 1, (d[1] - 1) * F + 1, (d[2] - 1) * F + 1};
        filter_call(g, prod3(o), out, prod3(d), [&](const double *a, double *b) { vfem::launch_upsample_backprop(d, F, a, b, 0); });
    });
}
int vfem_vertex_to_cell_filter(const int64_t vertex_dims[3], const double *in, double *out) {
    return guarded([&] {
        need(in, "in");
        need(out, "out");
        int d[3];
        dims3(vertex_dims, d, 2, "Input grid must be 2^d or larger.");
        const int e[3] = {d[0] - 1, d[1] - 1, d[2] - 1};
        filter_call(in, prod3(d), out, prod3(e), [&](const double *a, double *b) { vfem::launch_vertex_to_cell(d, a, b, 0); });
    });
}
int vfem_vertex_to_cell_filter_backprop(const int64_t vertex_dims[3], const double *g, double *out) {
    return guarded([&] {
        need(g, "g");
        need(out, "out");
        int d[3];
        dims3(vertex_dims, d, 2, "Input grid must be 2^d or larger.");
        const int e[3] = {d[0] - 1, d[1] - 1, d[2] - 1};
        filter_call(g, prod3(e), out, prod3(d), [&](const double *a, double *b) { vfem::launch_vertex_to_cell_backprop(d, a, b, 0); });
    });
}

struct vfem_langelaar {
    int d[3];
    int ndim = 3;
    int64_t n;
    vfem::DevBuf<double> out, smax, filt, lam, vars, g;
};
int vfem_langelaar_create(const int64_t dims[3], vfem_langelaar **h) {
    return guarded([&] {
        need(h, "handle");
        auto f = std::make_unique<vfem_langelaar>();
        dims3(dims, f->d, 1, "invalid grid dimensions");
        f->n = prod3(f->d);
        for (auto *b : {&f->out, &f->smax, &f->filt, &f->lam, &f->vars, &f->g}) b->alloc(f->n);
        VFEM_CUDA(cudaMemset(f->out.p, 0, f->n * sizeof(double)));
        VFEM_CUDA(cudaMemset(f->smax.p, 0, f->n * sizeof(double)));
        VFEM_CUDA(cudaMemset(f->filt.p, 0, f->n * sizeof(double)));
        *h = f.release();
    });
}
// ---- 2D variants (the N = 2 instantiations of the same filters) ----
namespace {
void dims2(const int64_t *d, int out[3], int64_t minimum, const char *msg) {
    if (!d) throw vfem::Error(vfem::ERR_ARG, "null dims");
    for (int a = 0; a < 2; ++a) {
        if (d[a] < minimum || d[a] > (int64_t)1 << 30) throw vfem::Error(vfem::ERR_ARG, msg);
        out[a] = (int)d[a];
    }
    out[2] = 1;
}
}  // namespace
int vfem_upsample_filter2(const int64_t in_dims[2], int64_t factor, const double *in, double *out) {
    return guarded([&] {
        need(in, "in");
        need(out, "out");
        int d[3];
        dims2(in_dims, d, 2, "Interpolation can only be applied to a 2^d grid or larger");
        if (factor < 1) throw vfem::Error(vfem::ERR_ARG, "factor must be positive");
        const int F = (int)factor;
        const int o[3] = {(d[0] - 1) * F + 1, (d[1] - 1) * F + 1, 1};
        filter_call(in, prod3(d), out, prod3(o), [&](const double *a, double *b) { vfem::launch_upsample(d, F, a, b, 0, 2); });
    });
}
int vfem_upsample_filter2_backprop(const int64_t in_dims[2], int64_t factor, const double *g, double *out) {
    return guarded([&] {
        need(g, "g");
        need(out, "out");
        int d[3];
        dims2(in_dims, d, 2, "Interpolation can only be applied to a 2^d grid or larger");
        if (factor < 1) throw vfem::Error(vfem::ERR_ARG, "factor must be positive");
        const int F = (int)factor;
        const int o[3] = {(d[0] - 1) * F + 1, (d[1] - 1) * F + 1, 1};
        filter_call(g, prod3(o), out, prod3(d), [&](const double *a, double *b) { vfem::launch_upsample_backprop(d, F, a, b, 0); });
    });
}
int vfem_vertex_to_cell_filter2(const int64_t vertex_dims[2], const double *in, double *out) {
    return guarded([&] {
        need(in, "in");
        need(out, "out");
        int d[3];
        dims2(vertex_dims, d, 2, "Input grid must be 2^d or larger.");
        const int e[3] = {d[0] - 1, d[1] - 1, 1};
        filter_call(in, prod3(d), out, prod3(e), [&](const double *a, double *b) { vfem::launch_vertex_to_cell(d, a, b, 0, 2); });
    });
}
int vfem_vertex_to_cell_filter2_backprop(const int64_t vertex_dims[2], const double *g, double *out) {
    return guarded([&] {
        need(g, "g");
        need(out, "out");
        int d[3];
        dims2(vertex_dims, d, 2, "Input grid must be 2^d or larger.");
        const int e[3] = {d[0] - 1, d[1] - 1, 1};
        filter_call(g, prod3(e), out, prod3(d),
                    [&](const double *a, double *b) { vfem::launch_vertex_to_cell_backprop(d, a, b, 0, 2); });
    });
}
int vfem_langelaar2_create(const int64_t dims[2], vfem_langelaar **h) {
    return guarded([&] {
        need(h, "handle");
        auto f = std::make_unique<vfem_langelaar>();
        dims2(dims, f->d, 1, "invalid grid dimensions");
        f->ndim = 2;
        f->n = prod3(f->d);
        for (auto *b : {&f->out, &f->smax, &f->filt, &f->lam, &f->vars, &f->g}) b->alloc(f->n);
        VFEM_CUDA(cudaMemset(f->out.p, 0, f->n * sizeof(double)));
        VFEM_CUDA(cudaMemset(f->smax.p, 0, f->n * sizeof(double)));
        VFEM_CUDA(cudaMemset(f->filt.p, 0, f->n * sizeof(double)));
        *h = f.release();
    });
}
int vfem_langelaar_destroy(vfem_langelaar *h) {
    return guarded([&] { delete h; });
}
int vfem_langelaar_apply(vfem_langelaar *h, const double *in, double *out) {
    return guarded([&] {
        need(h, "handle");
        need(in, "in");
        need(out, "out");
        VFEM_CUDA(cudaMemcpy(h->vars.p, in, h->n * sizeof(double), cudaMemcpyDefault));
        vfem::launch_langelaar(h->d, h->vars.p, h->out.p, h->smax.p, 0, h->ndim);
        VFEM_CUDA(cudaMemcpy(h->filt.p, h->out.p, h->n * sizeof(double), cudaMemcpyDeviceToDevice));
        VFEM_CUDA(cudaMemcpy(out, h->out.p, h->n * sizeof(double), cudaMemcpyDefault));
    });
}
int vfem_langelaar_backprop(vfem_langelaar *h, const double *g, const double *vars, double *out) {
    return guarded([&] {
        need(h, "handle");
        need(g, "g");
        need(vars, "vars");
        need(out, "out");
        VFEM_CUDA(cudaMemcpy(h->g.p, g, h->n * sizeof(double), cudaMemcpyDefault));
        VFEM_CUDA(cudaMemcpy(h->vars.p, vars, h->n * sizeof(double), cudaMemcpyDefault));
        vfem::DevBuf<double> res(h->n);
        vfem::launch_langelaar_backprop(h->d, h->g.p, h->vars.p, h->filt.p, h->smax.p, h->lam.p, res.p, 0, h->ndim);
        VFEM_CUDA(cudaMemcpy(out, res.p, h->n * sizeof(double), cudaMemcpyDefault));
    });
}
