// Host engine of the bilinear-quadrilateral path (TensorProductSimulator<double, 1, 1> and
// MultigridSolver<double, 1, 1>): element mathematics, boundary conditions and the fabrication
// mask on the host; moduli, operators, the multigrid hierarchy and the PCG loop on the device.
#include "vfem_2d.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>

#include "vfem_kernels.hpp"

namespace vfem {

// ---------------------------------------------------------------------------
// Element mathematics
// ---------------------------------------------------------------------------
// K0_ij = vol sum_q w_q eps_i : C : eps_j with two Gauss points per axis
// (TensorProductSimulator.hh:67-80); C is MeshFEM's 2D isotropic tensor
// (ElasticityTensor<Real, 2>::setIsotropic: lambda = E nu / ((1 + nu)(1 - nu)), plane stress).
static void element_stiffness_2d(double E, double nu, const double h[2], double K0[64]) {
    const double lam = E * nu / ((1 + nu) * (1 - nu));
    const double mu = E / (2 * (1 + nu));
    const double q[2] = {0.5 - 0.5 / std::sqrt(3.0), 0.5 + 0.5 / std::sqrt(3.0)};
    double acc[64] = {0};
    for (int qp = 0; qp < 4; ++qp) {
        const double x[2] = {q[(qp >> 1) & 1], q[qp & 1]};
        double G[4][2];
        for (int l = 0; l < 4; ++l) {
            const int bit[2] = {(l >> 1) & 1, l & 1};
            double val[2], der[2];
            for (int d = 0; d < 2; ++d) {
                val[d] = bit[d] ? x[d] : 1.0 - x[d];
                der[d] = (bit[d] ? 1.0 : -1.0) / h[d];
            }
            G[l][0] = der[0] * val[1];
            G[l][1] = val[0] * der[1];
        }
        for (int a = 0; a < 4; ++a)
            for (int c = 0; c < 2; ++c)
                for (int b = 0; b < 4; ++b)
                    for (int d = 0; d < 2; ++d) {
                        const double dot = G[a][0] * G[b][0] + G[a][1] * G[b][1];
                        const double ee = 0.5 * ((c == d ? dot : 0.0) + G[a][d] * G[b][c]);
                        acc[(2 * a + c) * 8 + 2 * b + d] += 0.25 * (lam * G[a][c] * G[b][d] + 2 * mu * ee);
                    }
    }
    const double vol = h[0] * h[1];
    for (int i = 0; i < 8; ++i)
        for (int j = i; j < 8; ++j) {
            K0[i * 8 + j] = acc[i * 8 + j] * vol;
            K0[j * 8 + i] = K0[i * 8 + j];
        }
}

// I_c = phi_c (x) Id_2: coarse element DOFs -> DOFs of child c = 2 fx + fy
// (MultigridSolver.hh:664-687)
static void child_interp_2d(int c, double I[64]) {
    const int fx = c >> 1, fy = c & 1;
    std::fill(I, I + 64, 0.0);
    for (int fn = 0; fn < 4; ++fn) {
        const double p[2] = {0.5 * (fn >> 1) + 0.5 * fx, 0.5 * (fn & 1) + 0.5 * fy};
        for (int cn = 0; cn < 4; ++cn) {
            const double v = ((cn >> 1) ? p[0] : 1 - p[0]) * ((cn & 1) ? p[1] : 1 - p[1]);
            for (int d = 0; d < 2; ++d) I[(2 * fn + d) * 8 + 2 * cn + d] = v;
        }
    }
}

static void matmul8(const double *A, const double *B, double *C) {
    for (int i = 0; i < 8; ++i)
        for (int j = 0; j < 8; ++j) {
            double acc = 0;
            for (int k = 0; k < 8; ++k) acc += A[i * 8 + k] * B[k * 8 + j];
            C[i * 8 + j] = acc;
        }
}

// The fine K0 seen from a level-l element: for the fine element at (pi, pj) inside it,
// P = I_{c0} I_{c1} ... I_{c_{l-1}} (c_k its ancestor's child index at level k) and
// table[pos] = P^T K0 P, symmetrised (MultigridSolver.hh:712-819 composed down to level 0).
static std::vector<double> coarsened_table_2d(const double K0[64], int level) {
    const int S = 1 << level;
    std::vector<double> out((size_t)S * S * 64);
    double Ic[4][64];
    for (int c = 0; c < 4; ++c) child_interp_2d(c, Ic[c]);
    for (int pi = 0; pi < S; ++pi)
        for (int pj = 0; pj < S; ++pj) {
            double P[64], T[64];
            for (int t = 0; t < 64; ++t) P[t] = (t / 8 == t % 8) ? 1.0 : 0.0;
            for (int k = 0; k < level; ++k) {
                const int c = 2 * ((pi >> k) & 1) + ((pj >> k) & 1);
                matmul8(P, Ic[c], T);
                std::memcpy(P, T, sizeof(P));
            }
            double KP[64], R[64];
            matmul8(K0, P, KP);
            for (int i = 0; i < 8; ++i)
                for (int j = 0; j < 8; ++j) {
                    double acc = 0;
                    for (int k = 0; k < 8; ++k) acc += P[k * 8 + i] * KP[k * 8 + j];
                    R[i * 8 + j] = acc;
                }
            double *dst = &out[((size_t)pi * S + pj) * 64];
            for (int i = 0; i < 8; ++i)
                for (int j = 0; j < 8; ++j) dst[i * 8 + j] = 0.5 * (R[i * 8 + j] + R[j * 8 + i]);
        }
    return out;
}

// ---------------------------------------------------------------------------
// Grid2
// ---------------------------------------------------------------------------
Grid2::Grid2(const int ne[2], const double mn[2], const double mx[2]) {
    for (int d = 0; d < 2; ++d) {
        if (ne[d] <= 0) throw Error(ERR_ARG, "invalid elementsPerDimension");
        if (!(mx[d] > mn[d])) throw Error(ERR_ARG, "empty domain");
        bmin[d] = mn[d];
        bmax[d] = mx[d];
        h[d] = (mx[d] - mn[d]) / ne[d];
    }
    g = makeGeom2(ne);
    element_stiffness_2d(Eyoung, nu, h, K0.a);
    VFEM_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    rho.alloc(g.NE);
    Y.alloc(g.NE);
    dval.alloc(2 * g.NN);
    force.alloc(2 * g.NN);
    dmask.alloc(g.NN);
    hmask.assign(g.NN, 0);
    hval.assign(2 * g.NN, 0.0);
    hforce.assign(2 * g.NN, 0.0);
    VFEM_CUDA(cudaMemsetAsync(rho.p, 0, g.NE * sizeof(double), stream));  // NDVector zero-initialised
    uploadBC();
    updateYoungModuli();
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

Grid2::~Grid2() {
    if (stream) cudaStreamDestroy(stream);
}

void Grid2::setETensor(double E, double nu_) {
    Eyoung = E;
    nu = nu_;
    element_stiffness_2d(Eyoung, nu, h, K0.a);
    ++version;
    ++k0Version;
}

void Grid2::setParams(double E0_, double Emin_, double gamma_, double q_, int law_) {
    if (law_ != 0 && law_ != 1) throw Error(ERR_ARG, "unknown interpolation law");
    E0 = E0_; Emin = Emin_; gamma = gamma_; q = q_; law = law_;
    updateYoungModuli();
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

void Grid2::setDensities(const double *r, bool checkRange) {
    if (checkRange) {
        std::vector<double> hostCopy(g.NE);
        VFEM_CUDA(cudaMemcpy(hostCopy.data(), r, g.NE * sizeof(double), cudaMemcpyDefault));
        for (double v : hostCopy)
            if (v > 1.0 || v < 0.0) throw Error(ERR_ARG, "Density value has to be in between 0 and 1");
    }
    VFEM_CUDA(cudaMemcpyAsync(rho.p, r, g.NE * sizeof(double), cudaMemcpyDefault, stream));
    updateYoungModuli();
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

void Grid2::setUniformDensities(double v) {
    if (v > 1.0 || v < 0.0) throw Error(ERR_ARG, "Density value has to be in between 0 and 1");
    std::vector<double> hv(g.NE, v);
    setDensities(hv.data(), false);
}

// TensorProductSimulator.hh:2088-2102
void Grid2::updateYoungModuli() {
    launch2_young(g, rho.p, Y.p, E0, Emin, gamma, q, law, maskH < bmax[BUILD_DIR], stream);
    ++version;
}

// TensorProductSimulator.hh:241-252 with BCBuilder::setDirichlet :73-88
void Grid2::addDirichlet(const double u[2], const double mn[2], const double mx[2], unsigned cmask) {
    std::vector<uint8_t> m = hmask;
    std::vector<double> v = hval;
    for (int i = 0; i < g.nn[0]; ++i) {
        const double px = bmin[0] + i * h[0];
        if (px < mn[0] || px > mx[0]) continue;
        for (int j = 0; j < g.nn[1]; ++j) {
            const double py = bmin[1] + j * h[1];
            if (py < mn[1] || py > mx[1]) continue;
            const int64_t n = g.node(i, j);
            for (int c = 0; c < 2; ++c) {
                if (!((cmask >> c) & 1)) continue;
                if (!((m[n] >> c) & 1)) {
                    m[n] |= (uint8_t)(1u << c);
                    v[c * g.NN + n] = u[c];
                } else if (std::abs(v[c * g.NN + n] - u[c]) > 1e-10) {
                    throw Error(ERR_ARG, "Conflicting dirichlet displacements.");
                }
            }
        }
    }
    hmask.swap(m);
    hval.swap(v);
    uploadBC();
}

// TensorProductSimulator.hh:2042-2053
void Grid2::applySymmetry(const int axes[2], const int maxFace[2]) {
    for (int64_t n = 0; n < g.NN; ++n) {
        const int idx[2] = {(int)(n / g.nn[1]), (int)(n % g.nn[1])};
        for (int d = 0; d < 2; ++d) {
            if (!axes[d]) continue;
            const double p = bmin[d] + idx[d] * h[d];
            if (std::abs(p - (maxFace[d] ? bmax[d] : bmin[d])) < 1e-10) {
                hmask[n] |= (uint8_t)(1u << d);
                hval[d * g.NN + n] = 0.0;
            }
        }
    }
    uploadBC();
}

void Grid2::setForces(const double *f) {
    VFEM_CUDA(cudaMemcpy(hforce.data(), f, 2 * g.NN * sizeof(double), cudaMemcpyDefault));
    uploadBC();
}

void Grid2::setGravity(const double gv[2]) {
    grav[0] = gv[0];
    grav[1] = gv[1];
}

void Grid2::uploadBC() {
    dvalNonzero = false;
    for (double v : hval)
        if (v != 0.0) dvalNonzero = true;
    VFEM_CUDA(cudaMemcpyAsync(dmask.p, hmask.data(), g.NN, cudaMemcpyHostToDevice, stream));
    VFEM_CUDA(cudaMemcpyAsync(dval.p, hval.data(), 2 * g.NN * sizeof(double), cudaMemcpyHostToDevice, stream));
    VFEM_CUDA(cudaMemcpyAsync(force.p, hforce.data(), 2 * g.NN * sizeof(double), cudaMemcpyHostToDevice, stream));
    VFEM_CUDA(cudaStreamSynchronize(stream));
    ++bcVersion;
}

// TensorProductSimulator.hh:290-303, 327-331
void Grid2::setMaskHeight(double hgt, bool update) {
    if (hgt < 0 || hgt > bmax[BUILD_DIR])
        throw Error(ERR_ARG, "Fabrication height (" + std::to_string(hgt) + ") has to be in between 0 and " +
                                 std::to_string(bmax[BUILD_DIR]));
    maskH = hgt;
    const double fe = std::ceil(hgt / h[BUILD_DIR] - 1e-10);
    g.firstMaskedE = (int)fe;
    g.firstDetN = g.firstMaskedE + 1;
    if (update) updateYoungModuli();
    VFEM_CUDA(cudaStreamSynchronize(stream));
}

void Grid2::setMaskLayer(int64_t l) {
    if (l < 0) throw Error(ERR_ARG, "negative layer count");
    setMaskHeight(h[BUILD_DIR] * (double)l, true);
}

void Grid2::applyK(const double *u, double *out) {
    View vu, vo;
    viewIn(vu, u, 2 * g.NN * sizeof(double), stream);
    viewOut(vo, out, 2 * g.NN * sizeof(double));
    launch2_applyk_fine<double>(g, Y.p, K0, (const double *)vu.d, (double *)vo.d, 0, nullptr, nullptr, false, nullptr,
                        nullptr, stream);
    finishOut(vo, stream);
}

// TensorProductSimulator.hh:1269-1288
void Grid2::buildLoadDev(double *f) {
    VFEM_CUDA(cudaMemcpyAsync(f, force.p, 2 * g.NN * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    if (grav[0] != 0.0 || grav[1] != 0.0) launch2_gravity_load(g, rho.p, f, grav, vol(), stream);
}

void Grid2::adjoint(const double *lam, const double *u, double wF, double wK, double *out) {
    View vl, vu, vo;
    viewIn(vl, lam, 2 * g.NN * sizeof(double), stream);
    viewIn(vu, u, 2 * g.NN * sizeof(double), stream);
    viewOut(vo, out, g.NE * sizeof(double));
    launch2_adjoint(g, rho.p, (const double *)vl.d, (const double *)vu.d, (double *)vo.d, K0, E0, Emin, gamma, q, law,
                    grav, vol(), wF, wK, stream);
    finishOut(vo, stream);
}

void Grid2::elementEnergy(const double *u, double *out) {
    View vu, vo;
    viewIn(vu, u, 2 * g.NN * sizeof(double), stream);
    viewOut(vo, out, g.NE * sizeof(double));
    launch2_element_energy(g, Y.p, (const double *)vu.d, (double *)vo.d, K0, stream);
    finishOut(vo, stream);
}

std::unique_ptr<Grid2> Grid2::clone() const {
    std::unique_ptr<Grid2> c(new Grid2(g.ne, bmin, bmax));
    if (c->Eyoung != Eyoung || c->nu != nu) c->setETensor(Eyoung, nu);
    c->E0 = E0; c->Emin = Emin; c->gamma = gamma; c->q = q; c->law = law;
    c->grav[0] = grav[0];
    c->grav[1] = grav[1];
    c->hmask = hmask;
    c->hval = hval;
    c->hforce = hforce;
    c->uploadBC();
    return c;
}

// ---------------------------------------------------------------------------
// MG2
// ---------------------------------------------------------------------------
static int maskedRow(double hgt, double hy) { return (int)std::ceil(hgt / hy - 1e-10); }

MG2::MG2(Grid2 *f, int coarsenings) : fine(f) {
    if (coarsenings < 0) throw Error(ERR_ARG, "negative number of coarsening levels");
    int ne[2] = {f->g.ne[0], f->g.ne[1]};
    lv.resize(coarsenings + 1);
    lv[0].g = f->g;
    lv[0].h[0] = f->h[0];
    lv[0].h[1] = f->h[1];
    lv[0].hmask = f->hmask;
    for (int l = 1; l <= coarsenings; ++l) {
        for (int d = 0; d < 2; ++d) {
            if (ne[d] % 2 == 1) throw Error(ERR_ARG, "Grid size currently must be divisible by 2^numCoarseningLevels");
            ne[d] /= 2;
        }
        Level &c = lv[l];
        const Level &p = lv[l - 1];
        c.g = makeGeom2(ne);
        for (int d = 0; d < 2; ++d) c.h[d] = (f->bmax[d] - f->bmin[d]) / ne[d];
        c.hmask.assign(c.g.NN, 0);
        // Dirichlet coarsening (MultigridSolver.hh:58-103)
        for (int64_t fn = 0; fn < p.g.NN; ++fn) {
            const uint8_t fm = p.hmask[fn];
            if (!fm) continue;
            const int fidx[2] = {(int)(fn / p.g.nn[1]), (int)(fn % p.g.nn[1])};
            int e[2], pob[2];
            for (int d = 0; d < 2; ++d) {
                const double pos = f->bmin[d] + fidx[d] * p.h[d];
                const double fd = (pos - f->bmin[d]) / c.h[d];
                const int ed = std::abs(fd - c.g.ne[d]) < 1e-10 ? c.g.ne[d] - 1 : (int)fd;
                e[d] = ed;
                const double cref = (pos - (f->bmin[d] + ed * c.h[d])) / c.h[d];
                pob[d] = std::abs(cref) < 1e-9 ? 0 : (std::abs(cref - 1.0) < 1e-9 ? 1 : -1);
            }
            for (int ln = 0; ln < 4; ++ln) {
                const int lb[2] = {ln >> 1, ln & 1};
                bool ok = true;
                for (int d = 0; d < 2; ++d)
                    if (pob[d] != -1 && pob[d] != lb[d]) ok = false;
                if (!ok) continue;
                c.hmask[c.g.node(e[0] + lb[0], e[1] + lb[1])] |= fm;
            }
        }
    }
    const int64_t L = (int64_t)lv.size();
    for (int l = 0; l < L; ++l) {
        Level &v = lv[l];
        v.dyn.alloc(2);
        v.x.alloc(2 * v.g.NN);
        v.b.alloc(2 * v.g.NN);
        v.r.alloc(2 * v.g.NN);
        VFEM_CUDA(cudaMemset(v.x.p, 0, 2 * v.g.NN * sizeof(double)));
        VFEM_CUDA(cudaMemset(v.b.p, 0, 2 * v.g.NN * sizeof(double)));
        VFEM_CUDA(cudaMemset(v.r.p, 0, 2 * v.g.NN * sizeof(double)));
        if (l > 0 || L == 1) {
            v.Ke.alloc(v.g.NE * 64);
            v.S.alloc(36 * v.g.NN);
        }
        if (l > 0) {
            v.dmask.alloc(v.g.NN);
            VFEM_CUDA(cudaMemcpy(v.dmask.p, v.hmask.data(), v.g.NN, cudaMemcpyHostToDevice));
        }
    }
    const int64_t n2 = 2 * lv[0].g.NN;
    rbuf.alloc(n2);
    dvec.alloc(n2);
    Ad.alloc(n2);
    sbuf.alloc(n2);
    VFEM_CUDA(cudaMemset(rbuf.p, 0, n2 * sizeof(double)));
    partials.alloc(REDUCE_BLOCKS + 8);
    sc.alloc(16);
    status.alloc(1);
    VFEM_CUDA(cudaMallocHost(&hostSc, 16 * sizeof(double)));
    syncFine();
}

MG2::~MG2() {
    clearGraphs();
    if (hostSc) cudaFreeHost(hostSc);
}

void MG2::clearGraphs() {
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
    graphKernels.clear();
}

// Pick up changes of the simulator (moduli, material, mask height) since the last call.
void MG2::syncFine() {
    Grid2 &f = *fine;
    if (f.maskH != lv[0].maskH || builtMaskE < 0) {
        for (int l = 0; l < L(); ++l) {
            Level &v = lv[l];
            v.maskH = f.maskH;
            if (f.maskH < f.bmax[BUILD_DIR]) {
                v.g.firstMaskedE = maskedRow(f.maskH, v.h[BUILD_DIR]);
                v.g.firstDetN = v.g.firstMaskedE + 1;
            } else {
                v.g.firstMaskedE = (int)LAYER_MASK_NONE;
                v.g.firstDetN = (int)LAYER_MASK_NONE;
            }
            launch_set_pair(v.dyn.p, v.g.firstMaskedE, v.g.firstDetN, f.stream);
            v.g.dyn = v.dyn.p;
        }
        builtMaskE = lv[0].g.firstMaskedE;
        stiffValid = false;
    }
    if (f.bcVersion != bcVersion) {
        bcVersion = f.bcVersion;
        clearGraphs();
    }
    if (f.k0Version != k0Version) {
        k0Version = f.k0Version;
        clearGraphs();  // K0 is a kernel parameter of the captured launches
        for (int l = 1; l < L(); ++l) {
            std::vector<double> t = coarsened_table_2d(f.K0.a, l);
            lv[l].Kc.alloc(t.size());
            VFEM_CUDA(cudaMemcpyAsync(lv[l].Kc.p, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice, f.stream));
        }
        if (L() == 1) {
            lv[0].Kc.alloc(64);
            VFEM_CUDA(cudaMemcpyAsync(lv[0].Kc.p, f.K0.a, 64 * sizeof(double), cudaMemcpyHostToDevice, f.stream));
        }
        VFEM_CUDA(cudaStreamSynchronize(f.stream));
        stiffValid = false;
    }
}

const uint8_t *MG2::levelMask(int l) const { return l == 0 ? fine->dmask.p : lv[l].dmask.p; }

void MG2::setMaskLayer(int64_t l) {
    fine->setMaskLayer(l);
    syncFine();
}

// MultigridSolver.hh:846-905 and the coarsest factorisation (TensorProductSimulator.hh:1181-1230)
void MG2::ensureStiffness() {
    syncFine();
    if (stiffValid && builtVersion == fine->version) return;
    cudaStream_t st = fine->stream;
    const int first = L() == 1 ? 0 : 1;
    for (int l = first; l < L(); ++l) {
        launch2_ke_coarse(lv[l].g, lv[0].g, l, fine->Y.p, lv[l].Kc.p, lv[l].Ke.p, st);
        launch2_stencil_from_ke(lv[l].g, lv[l].Ke.p, lv[l].S.p, st);
    }
    // reduced dense operator of the coarsest level: Dirichlet components and detached rows fixed
    Level &C = lv.back();
    const std::vector<uint8_t> &cm = (L() == 1) ? fine->hmask : C.hmask;
    std::vector<int> red(2 * C.g.NN, -1), fr;
    for (int64_t n = 0; n < C.g.NN; ++n) {
        const int j = (int)(n % C.g.nn[1]);
        for (int c = 0; c < 2; ++c) {
            if ((cm[n] >> c & 1) || j >= C.g.firstDetN) continue;
            red[2 * n + c] = (int)fr.size();
            fr.push_back((int)(2 * n + c));
        }
    }
    nfree = (int)fr.size();
    if (nfree > nfreeCap) {
        // buffers sized for the unmasked coarsest level; captured graphs hold their addresses
        if (nfree > 30000)
            throw Error(ERR_ARG, "coarsest level too large for the dense direct solve; use more coarsening levels");
        clearGraphs();
        nfreeCap = nfree;
        Ainv.alloc((size_t)nfreeCap * nfreeCap);
        work.alloc(dense_inverse_work_size(nfreeCap));
        cscratch.alloc(nfreeCap);
        freeIdx.alloc(nfreeCap);
        redIdx.alloc(2 * C.g.NN);
        nfreeDev.alloc(1);
    }
    VFEM_CUDA(cudaMemcpyAsync(redIdx.p, red.data(), red.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    if (nfree) VFEM_CUDA(cudaMemcpyAsync(freeIdx.p, fr.data(), fr.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    if (nfreeCap) launch_set_pair(nfreeDev.p, nfree, 0, st);
    if (nfree) {
        launch2_dense_from_stencil(C.g, C.S.p, redIdx.p, Ainv.p, nfree, st);
        launch_symmetrize(Ainv.p, nfree, st);
        VFEM_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), st));
        dense_spd_inverse(Ainv.p, work.p, nfree, status.p, st);
        int bad = 0;
        VFEM_CUDA(cudaMemcpyAsync(&bad, status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        VFEM_CUDA(cudaStreamSynchronize(st));
        if (bad == 2) check_dense_status(bad);
        if (bad) throw Error(ERR_NOT_SPD, "Coarsest matrix not positive definite");
    }
    if (precision == PREC_MIXED) refreshSingle();
    VFEM_CUDA(cudaStreamSynchronize(st));
    builtVersion = fine->version;
    stiffValid = true;
}

void MG2::updateStiffness() {
    stiffValid = false;
    ensureStiffness();
}

template <>
MG2::LB<double> MG2::lb<double>(int l) {
    return {lv[l].x.p, lv[l].b.p, lv[l].r.p, lv[l].S.p};
}
template <>
MG2::LB<float> MG2::lb<float>(int l) {
    return {lv[l].x32.p, lv[l].b32.p, lv[l].r32.p, lv[l].S32.p};
}
template <>
const double *MG2::fineY<double>() const {
    return fine->Y.p;
}
template <>
const float *MG2::fineY<float>() const {
    return Y32.p;
}
template <>
const Mat8T<double> &MG2::fineK0<double>() const {
    return fine->K0;
}
template <>
const Mat8T<float> &MG2::fineK0<float>() const {
    return K0f;
}

// operator of level l (fine: matrix-free; coarser: stencils); mode 0 apply, 1 residual
template <typename T>
void MG2::levelOperatorT(int l, const T *u, T *out, int mode, const T *b) {
    cudaStream_t st = fine->stream;
    if (l == 0)
        launch2_applyk_fine<T>(lv[0].g, fineY<T>(), fineK0<T>(), u, out, mode, b, fine->dmask.p, false, nullptr, nullptr,
                               st);
    else launch2_stencil_apply<T>(lv[l].g, lb<T>(l).S, u, out, mode, b, lv[l].dmask.p, st);
}

template <typename T>
void MG2::smoothLevelT(int l, T *u, const T *b, bool forward) {
    cudaStream_t st = fine->stream;
    for (int ci = 0; ci < 4; ++ci) {
        const int color = forward ? ci : 3 - ci;
        if (l == 0) launch2_gs_fine<T>(lv[0].g, fineY<T>(), fineK0<T>(), u, b, fine->dmask.p, color, forward, st);
        else launch2_gs_stencil<T>(lv[l].g, lb<T>(l).S, u, b, lv[l].dmask.p, color, forward, st);
    }
}

template <typename T>
void MG2::coarseSolveDevT(const T *b, T *x) {
    const Level &C = lv.back();
    launch2_coarse_solve<T>(C.g, Ainv.p, freeIdx.p, nfreeDev.p, nfreeCap, b, x, cscratch.p, fine->stream);
}

// MultigridSolver.hh:617-658
template <typename T>
void MG2::vcycleT(int l, int64_t sweeps, bool residualSystem) {
    cudaStream_t st = fine->stream;
    const LB<T> v = lb<T>(l);
    if (l == L() - 1) {
        coarseSolveDevT<T>(v.b, v.x);
        return;
    }
    const Geom2 &g = lv[l].g;
    if (residualSystem || l > 0 || !fine->dvalNonzero) launch2_zero_dirichlet<T>(g, v.x, levelMask(l), st);
    else launch2_enforce_dirichlet<T>(g, v.x, levelMask(l), fine->dval.p, st);
    for (int64_t t = 0; t < sweeps; ++t) smoothLevelT<T>(l, v.x, v.b, true);
    levelOperatorT<T>(l, v.x, v.r, 1, v.b);
    const LB<T> c = lb<T>(l + 1);
    launch2_restrict<T>(g, lv[l + 1].g, v.r, c.b, st);
    launch2_masked_zero<T>(lv[l + 1].g, c.x, MARGIN, st);
    vcycleT<T>(l + 1, sweeps, true);
    launch2_interpolate<T>(g, lv[l + 1].g, c.x, v.x, true, st);
    for (int64_t t = 0; t < sweeps; ++t) smoothLevelT<T>(l, v.x, v.b, !symmetricGS);
}

// MultigridSolver.hh:587-609
template <typename T>
void MG2::fmgDownT(int l, int64_t sweeps, bool residualSystem) {
    cudaStream_t st = fine->stream;
    const LB<T> v = lb<T>(l);
    if (l == L() - 1) {
        coarseSolveDevT<T>(v.b, v.x);
        return;
    }
    const LB<T> c = lb<T>(l + 1);
    launch2_restrict<T>(lv[l].g, lv[l + 1].g, v.b, c.b, st);
    fmgDownT<T>(l + 1, sweeps, residualSystem);
    launch2_interpolate<T>(lv[l].g, lv[l + 1].g, c.x, v.x, false, st);
    vcycleT<T>(l, sweeps, residualSystem);
}

template <typename T>
void MG2::runCyclesT(int64_t steps, int64_t sweeps, bool residualSystem, bool fmg) {
    if (fmg) {
        fmgDownT<T>(0, sweeps, residualSystem);
        for (int64_t i = 1; i < steps; ++i) vcycleT<T>(0, sweeps, residualSystem);
    } else {
        for (int64_t i = 0; i < steps; ++i) vcycleT<T>(0, sweeps, residualSystem);
    }
}

void MG2::levelOperator(int l, const double *u, double *out, int mode, const double *b) {
    levelOperatorT<double>(l, u, out, mode, b);
}
void MG2::smoothLevel(int l, double *u, const double *b, bool forward) { smoothLevelT<double>(l, u, b, forward); }
void MG2::coarseSolveDev(const double *b, double *x) { coarseSolveDevT<double>(b, x); }
void MG2::runCycles(int64_t steps, int64_t sweeps, bool residualSystem, bool fmg) {
    runCyclesT<double>(steps, sweeps, residualSystem, fmg);
}

void MG2::refreshDF() {
    if (!dfOuter() || dfVersion == fine->version) return;
    const int64_t ne = lv[0].g.NE, n2 = 2 * lv[0].g.NN;
    Yh.alloc(ne);
    Yl.alloc(ne);
    dh.alloc(n2);
    dl.alloc(n2);
    launch_split_df(fine->Y.p, Yh.p, Yl.p, ne, fine->stream);
    for (int t = 0; t < 64; ++t) {
        K0f.a[t] = (float)fine->K0.a[t];
        K0lo.a[t] = (float)(fine->K0.a[t] - (double)K0f.a[t]);
    }
    dfVersion = fine->version;
}

void MG2::outerOperator(const double *u, double *out, int mode, const double *b, bool zeroDir, const double *dotv,
                        double *partials, bool uSplit) {
    const Geom2 &g = lv[0].g;
    if (dfOuter()) {
        if (!uSplit) launch_split_df(u, dh.p, dl.p, 2 * g.NN, fine->stream);
        launch2_applyk_df(g, Yh.p, Yl.p, K0f, K0lo, dh.p, dl.p, out, mode, b, fine->dmask.p, zeroDir, dotv, partials,
                          fine->stream);
    } else {
        launch2_applyk_fine<double>(g, fine->Y.p, fine->K0, u, out, mode, b, fine->dmask.p, zeroDir, dotv, partials,
                                    fine->stream);
    }
}

void MG2::setOuterMatvec(int kind) {
    if (kind != MATVEC_FP64 && kind != MATVEC_DF) throw Error(ERR_ARG, "unknown outer matvec");
    if (kind == outerMatvec) return;
    outerMatvec = kind;
    clearGraphs();
}

void MG2::setPrecision(int p) {
    if (p != PREC_FP64 && p != PREC_MIXED) throw Error(ERR_ARG, "unknown precision");
    if (p == precision) return;
    precision = p;
    clearGraphs();
    if (p == PREC_MIXED) {
        for (int l = 0; l < L(); ++l) {
            Level &v = lv[l];
            const int64_t n2 = 2 * v.g.NN;
            v.x32.alloc(n2);
            v.b32.alloc(n2);
            v.r32.alloc(n2);
            VFEM_CUDA(cudaMemset(v.x32.p, 0, n2 * sizeof(float)));
            VFEM_CUDA(cudaMemset(v.b32.p, 0, n2 * sizeof(float)));
            VFEM_CUDA(cudaMemset(v.r32.p, 0, n2 * sizeof(float)));
            if (l > 0) v.S32.alloc(36 * v.g.NN);
        }
        Y32.alloc(lv[0].g.NE);
    }
    stiffValid = false;
}

// the FP32 copies of the fine moduli, K0 and the coarse stencils (mixed precision)
void MG2::refreshSingle() {
    cudaStream_t st = fine->stream;
    launch_cast<float, double>(fine->Y.p, Y32.p, lv[0].g.NE, st);
    for (int t = 0; t < 64; ++t) {
        K0f.a[t] = (float)fine->K0.a[t];
        K0lo.a[t] = (float)(fine->K0.a[t] - (double)K0f.a[t]);
    }
    for (int l = 1; l < L(); ++l) launch_cast<float, double>(lv[l].S.p, lv[l].S32.p, 36 * lv[l].g.NN, st);
}

// MultigridSolver.hh:547-573
void MG2::solve(const double *u, const double *f, int64_t steps, int64_t sweeps, bool zeroDirichlet, bool fmg,
                double *xout) {
    ensureStiffness();
    cudaStream_t st = fine->stream;
    const size_t bytes = 2 * lv[0].g.NN * sizeof(double);
    View vu, vf, vo;
    viewIn(vu, u, bytes, st);
    viewIn(vf, f, bytes, st);
    viewOut(vo, xout, bytes);
    VFEM_CUDA(cudaMemcpyAsync(lv[0].x.p, vu.d, bytes, cudaMemcpyDeviceToDevice, st));
    if (steps > 0) {
        VFEM_CUDA(cudaMemcpyAsync(lv[0].b.p, vf.d, bytes, cudaMemcpyDeviceToDevice, st));
        if (L() == 1) coarseSolveDev(lv[0].b.p, lv[0].x.p);
        else runCycles(steps, sweeps, zeroDirichlet, fmg);
    }
    VFEM_CUDA(cudaMemcpyAsync(vo.d, lv[0].x.p, bytes, cudaMemcpyDeviceToDevice, st));
    finishOut(vo, st);
}

// one PCG iteration on the device (MultigridSolver.hh:1071-1147); scalars in sc
void MG2::cgIteration(double *x, int64_t mgIter, int64_t sweeps, bool fmg) {
    cudaStream_t st = fine->stream;
    const Geom2 &g = lv[0].g;
    if (mgIter > 0 && precision == PREC_MIXED) {
        // FP32 V-cycle on the FP64 residual (its rounding is the only precision change)
        if (sweeps != 0) {
            launch_fill<float>(lv[0].x32.p, 0.f, 2 * g.NN, st);
            launch_cast<float, double>(rbuf.p, lv[0].b32.p, 2 * g.NN, st);
            runCyclesT<float>(mgIter, sweeps, true, fmg);
        }
        launch2_precond_out<float>(g, lv[0].x32.p, sbuf.p, rbuf.p, fine->dmask.p, partials.p, st);
    } else {
        const double *src = rbuf.p;
        if (mgIter > 0) {
            if (sweeps != 0) {
                launch_fill<double>(lv[0].x.p, 0.0, 2 * g.NN, st);  // zero initial guess
                VFEM_CUDA(cudaMemcpyAsync(lv[0].b.p, rbuf.p, 2 * g.NN * sizeof(double), cudaMemcpyDeviceToDevice, st));
                runCycles(mgIter, sweeps, true, fmg);
            }
            src = lv[0].x.p;
        }
        launch2_precond_out<double>(g, src, sbuf.p, rbuf.p, fine->dmask.p, partials.p, st);
    }
    launch_cg_beta(partials.p, REDUCE_BLOCKS, sc.p, st);
    if (dfOuter()) launch2_direction(g, sbuf.p, dvec.p, sc.p, st, dh.p, dl.p);
    else launch2_direction(g, sbuf.p, dvec.p, sc.p, st);
    outerOperator(dvec.p, Ad.p, 0, nullptr, true, dvec.p, partials.p, dfOuter());
    launch_cg_alpha(partials.p, REDUCE_BLOCKS, sc.p, st);
    launch2_cg_update(g, x, rbuf.p, dvec.p, Ad.p, sc.p, partials.p, st);
    launch_cg_rsq(partials.p, REDUCE_BLOCKS, sc.p, nullptr, st);
}

static uint64_t countKernels(cudaGraph_t gr) {
    size_t n = 0;
    VFEM_CUDA(cudaGraphGetNodes(gr, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    VFEM_CUDA(cudaGraphGetNodes(gr, nodes.data(), &n));
    uint64_t k = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType ty;
        VFEM_CUDA(cudaGraphNodeGetType(nd, &ty));
        if (ty == cudaGraphNodeTypeKernel) ++k;
    }
    return k;
}

// [loop control (initial)] -> WHILE( [one PCG iteration] -> [loop control] )
cudaGraphExec_t MG2::loopGraph(double *x, int64_t mgIter, int64_t sweeps, bool fmg) {
    const Key key{mgIter, sweeps, fmg ? 1 : 0, (symmetricGS ? 1 : 0) | (precision << 1) | (outerMatvec << 2), x};
    auto it = graphs.find(key);
    if (it != graphs.end()) return it->second;
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
            cgIteration(x, mgIter, sweeps, fmg);
            launch_cg_loop_control(h, sc.p, false, st);
        } catch (...) {
            cudaStreamEndCapture(st, &body);
            throw;
        }
        VFEM_CUDA(cudaStreamEndCapture(st, &body));
        const uint64_t k = countKernels(body);
        VFEM_CUDA(cudaGraphInstantiate(&exec, top, 0));
        launchCounter() -= k + 1;  // the captures launched nothing
        graphKernels[key] = k;
    } catch (...) {
        cudaGraphDestroy(top);
        throw;
    }
    cudaGraphDestroy(top);
    return graphs.emplace(key, exec).first->second;
}

static double readDev(const double *dev, cudaStream_t st) {
    double v = 0;
    VFEM_CUDA(cudaMemcpyAsync(&v, dev, sizeof(double), cudaMemcpyDeviceToHost, st));
    VFEM_CUDA(cudaStreamSynchronize(st));
    return v;
}

// MultigridSolver.hh:1047-1152; x and b are device vectors of 2 NN doubles
PcgStats MG2::pcgDev(double *x, const double *b, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps, bool fmg,
                     bool dirichletSatisfied, PcgCallback cb, void *user) {
    if (L() > 1 && useGraphs && !cb) {
        // one graph launch runs every iteration (conditional WHILE node)
        pcgStart(x, b, maxIter, tol, mgIter, sweeps, fmg, dirichletSatisfied);
        return pcgFinish();
    }
    syncFine();
    cudaStream_t st = fine->stream;
    const Geom2 &g = lv[0].g;
    PcgStats stats;
    if (!dirichletSatisfied) launch2_enforce_dirichlet<double>(g, x, fine->dmask.p, fine->dval.p, st);
    launch2_dot_partials(g, b, b, partials.p, st);
    launch_finalize(partials.p, REDUCE_BLOCKS, sc.p + 7, st);
    refreshDF();
    outerOperator(x, rbuf.p, 1, b, true, nullptr, nullptr, false);
    launch2_dot_partials(g, rbuf.p, rbuf.p, partials.p, st);
    launch_finalize(partials.p, REDUCE_BLOCKS, sc.p + 5, st);
    launch_cg_init(sc.p, tol * tol, (double)maxIter, st);
    launch_fill<double>(dvec.p, 0.0, 2 * g.NN, st);
    const double bnorm2 = readDev(sc.p + 7, st);
    double rsq = readDev(sc.p + 5, st);
    stats.bnorm2 = bnorm2;
    if (std::isnan(rsq)) throw Error(ERR_NAN, "NaN encountered");
    if (mgIter > 0 || L() == 1) ensureStiffness();

    if (L() == 1) {
        // direct solve branch (MultigridSolver.hh:1056-1064)
        if (!(rsq < tol * tol * bnorm2)) {
            coarseSolveDev(b, x);
            launch2_applyk_fine<double>(g, fine->Y.p, fine->K0, x, rbuf.p, 1, b, fine->dmask.p, true, nullptr, nullptr, st);
            launch2_dot_partials(g, rbuf.p, rbuf.p, partials.p, st);
            launch_finalize(partials.p, REDUCE_BLOCKS, sc.p + 5, st);
            rsq = readDev(sc.p + 5, st);
            stats.iterations = 1;
            if (cb) cb(user, 1, std::sqrt(rsq), x, rbuf.p);
        }
        stats.rsq = rsq;
    } else {
        int64_t i = 0;
        while (i < maxIter && rsq > tol * tol * bnorm2) {
            ++i;
            cgIteration(x, mgIter, sweeps, fmg);
            rsq = readDev(sc.p + 5, st);
            if (std::isnan(rsq)) throw Error(ERR_NAN, "NaN encountered at iteration" + std::to_string(i));
            if (cb && cb(user, i, std::sqrt(rsq), x, rbuf.p)) break;
        }
        stats.iterations = i;
        stats.rsq = rsq;
    }
    stats.relres = bnorm2 > 0 ? std::sqrt(stats.rsq / bnorm2) : std::sqrt(stats.rsq);
    return stats;
}

void MG2::pcgStart(double *x, const double *b, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps, bool fmg,
                   bool dirichletSatisfied) {
    if (L() == 1) throw Error(ERR_ARG, "the asynchronous solve needs at least one coarsening level");
    if (pending) throw Error(ERR_STATE, "a solve is already in flight on this solver");
    if (mgIter > 0) ensureStiffness();
    else syncFine();
    cudaStream_t st = fine->stream;
    const Geom2 &g = lv[0].g;
    if (!dirichletSatisfied) launch2_enforce_dirichlet<double>(g, x, fine->dmask.p, fine->dval.p, st);
    launch2_dot_partials(g, b, b, partials.p, st);
    launch_finalize(partials.p, REDUCE_BLOCKS, sc.p + 7, st);
    refreshDF();
    outerOperator(x, rbuf.p, 1, b, true, nullptr, nullptr, false);  // initial residual through the CG matvec
    launch2_dot_partials(g, rbuf.p, rbuf.p, partials.p, st);
    launch_finalize(partials.p, REDUCE_BLOCKS, sc.p + 5, st);
    launch_cg_init(sc.p, tol * tol, (double)maxIter, st);
    launch_fill<double>(dvec.p, 0.0, 2 * g.NN, st);
    pendingKey = Key{mgIter, sweeps, fmg ? 1 : 0, (symmetricGS ? 1 : 0) | (precision << 1) | (outerMatvec << 2), x};
    VFEM_CUDA(cudaGraphLaunch(loopGraph(x, mgIter, sweeps, fmg), st));
    VFEM_CUDA(cudaMemcpyAsync(hostSc, sc.p, 16 * sizeof(double), cudaMemcpyDeviceToHost, st));
    pending = true;
}

PcgStats MG2::pcgFinish() {
    if (!pending) throw Error(ERR_STATE, "no solve in flight");
    pending = false;
    VFEM_CUDA(cudaStreamSynchronize(fine->stream));
    PcgStats stats;
    stats.iterations = (int64_t)hostSc[9];
    stats.rsq = hostSc[5];
    stats.bnorm2 = hostSc[7];
    launchCounter() += 1 + (graphKernels[pendingKey] + 1) * (uint64_t)stats.iterations;
    if (hostSc[11] < 0.0) throw Error(ERR_NAN, "NaN encountered");
    if (hostSc[11] > 0.0) throw Error(ERR_NAN, "NaN encountered at iteration" + std::to_string((int64_t)hostSc[11]));
    stats.relres = stats.bnorm2 > 0 ? std::sqrt(stats.rsq / stats.bnorm2) : std::sqrt(stats.rsq);
    return stats;
}

PcgStats MG2::pcg(double *x, const double *b, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps, bool fmg,
                  bool dirichletSatisfied, PcgCallback cb, void *user) {
    cudaStream_t st = fine->stream;
    const size_t bytes = 2 * lv[0].g.NN * sizeof(double);
    View vx, vb;
    viewIn(vx, x, bytes, st);
    viewIn(vb, b, bytes, st);
    PcgStats s = pcgDev((double *)vx.d, (const double *)vb.d, maxIter, tol, mgIter, sweeps, fmg, dirichletSatisfied,
                        cb, user);
    if (vx.staged) VFEM_CUDA(cudaMemcpyAsync(x, vx.d, bytes, cudaMemcpyDeviceToHost, st));
    VFEM_CUDA(cudaStreamSynchronize(st));
    return s;
}

// ---- per-level entry points (MultigridSolver python bindings) ----
int64_t MG2::levelNN(int l) const {
    if (l < 0 || l >= L()) throw Error(ERR_ARG, "level out of range");
    return lv[l].g.NN;
}

void MG2::applyK(int l, const double *u, double *out) {
    const size_t bytes = 2 * levelNN(l) * sizeof(double);
    if (l > 0) ensureStiffness();
    else syncFine();
    View vu, vo;
    viewIn(vu, u, bytes, fine->stream);
    viewOut(vo, out, bytes);
    levelOperator(l, (const double *)vu.d, (double *)vo.d, 0, nullptr);
    finishOut(vo, fine->stream);
}

void MG2::residual(int l, const double *u, const double *b, double *r) {
    const size_t bytes = 2 * levelNN(l) * sizeof(double);
    if (l > 0) ensureStiffness();
    else syncFine();
    View vu, vb, vo;
    viewIn(vu, u, bytes, fine->stream);
    viewIn(vb, b, bytes, fine->stream);
    viewOut(vo, r, bytes);
    VFEM_CUDA(cudaMemsetAsync(vo.d, 0, bytes, fine->stream));
    levelOperator(l, (const double *)vu.d, (double *)vo.d, 1, (const double *)vb.d);
    finishOut(vo, fine->stream);
}

void MG2::smooth(int l, double *u, const double *b, bool forward) {
    const size_t bytes = 2 * levelNN(l) * sizeof(double);
    if (l > 0) ensureStiffness();
    else syncFine();
    View vu, vb;
    viewIn(vu, u, bytes, fine->stream);
    viewIn(vb, b, bytes, fine->stream);
    smoothLevel(l, (double *)vu.d, (const double *)vb.d, forward);
    if (vu.staged) VFEM_CUDA(cudaMemcpyAsync(u, vu.d, bytes, cudaMemcpyDeviceToHost, fine->stream));
    VFEM_CUDA(cudaStreamSynchronize(fine->stream));
}

void MG2::restrictTo(int l, const double *fv, double *cv) {
    if (l < 0 || l + 1 >= L()) throw Error(ERR_ARG, "level out of range");
    syncFine();
    View vf, vc;
    viewIn(vf, fv, 2 * lv[l].g.NN * sizeof(double), fine->stream);
    viewOut(vc, cv, 2 * lv[l + 1].g.NN * sizeof(double));
    VFEM_CUDA(cudaMemsetAsync(vc.d, 0, 2 * lv[l + 1].g.NN * sizeof(double), fine->stream));
    launch2_restrict(lv[l].g, lv[l + 1].g, (const double *)vf.d, (double *)vc.d, fine->stream);
    finishOut(vc, fine->stream);
}

void MG2::interpolate(int l, const double *cv, double *fv, bool accumulate) {
    if (l < 0 || l + 1 >= L()) throw Error(ERR_ARG, "level out of range");
    syncFine();
    const size_t fb = 2 * lv[l].g.NN * sizeof(double);
    View vc, vf;
    viewIn(vc, cv, 2 * lv[l + 1].g.NN * sizeof(double), fine->stream);
    viewIn(vf, fv, fb, fine->stream);
    launch2_interpolate(lv[l].g, lv[l + 1].g, (const double *)vc.d, (double *)vf.d, accumulate, fine->stream);
    if (vf.staged) VFEM_CUDA(cudaMemcpyAsync(fv, vf.d, fb, cudaMemcpyDeviceToHost, fine->stream));
    VFEM_CUDA(cudaStreamSynchronize(fine->stream));
}

void MG2::coarseSolve(const double *b, double *x) {
    ensureStiffness();
    const size_t bytes = 2 * lv.back().g.NN * sizeof(double);
    View vb, vx;
    viewIn(vb, b, bytes, fine->stream);
    viewOut(vx, x, bytes);
    coarseSolveDev((const double *)vb.d, (double *)vx.d);
    finishOut(vx, fine->stream);
}

void MG2::zeroDirichlet(int l, double *u) {
    const size_t bytes = 2 * levelNN(l) * sizeof(double);
    View vu;
    viewIn(vu, u, bytes, fine->stream);
    launch2_zero_dirichlet(lv[l].g, (double *)vu.d, levelMask(l), fine->stream);
    if (vu.staged) VFEM_CUDA(cudaMemcpyAsync(u, vu.d, bytes, cudaMemcpyDeviceToHost, fine->stream));
    VFEM_CUDA(cudaStreamSynchronize(fine->stream));
}

// Benchmark hook: average device time of one launch of a hot kernel on resident data.
// which: 0 fine applyK (FP64), 1 fine 4-colour GS sweep, 2 one V-cycle, 3 one PCG iteration, 4 fine
// applyK in double-float (sweeps and cycles in the solver's precision).
double MG2::timeKernel(int which, int reps) {
    ensureStiffness();
    cudaStream_t st = fine->stream;
    const Geom2 &g = lv[0].g;
    DevBuf<double> xt(2 * g.NN);
    VFEM_CUDA(cudaMemsetAsync(xt.p, 0, 2 * g.NN * sizeof(double), st));
    const int savedOuter = outerMatvec, savedPrec = precision;
    if (which == 4) {  // the double-float operator on a split copy of the fine iterate
        precision = PREC_MIXED;
        outerMatvec = MATVEC_DF;
        dfVersion = ~0ull;
        refreshDF();
        launch_split_df(lv[0].x.p, dh.p, dl.p, 2 * g.NN, st);
        precision = savedPrec;
        outerMatvec = savedOuter;
        dfVersion = ~0ull;
    }
    launch_cg_init(sc.p, 0.0, 1.0, st);
    auto body = [&]() {
        switch (which) {
        case 0:
            launch2_applyk_fine<double>(g, fine->Y.p, fine->K0, lv[0].x.p, lv[0].r.p, 0, nullptr, nullptr, false, nullptr,
                                nullptr, st);
            break;
        case 1:
            if (precision == PREC_MIXED) smoothLevelT<float>(0, lv[0].x32.p, lv[0].b32.p, true);
            else smoothLevel(0, lv[0].x.p, lv[0].b.p, true);
            break;
        case 2:
            if (precision == PREC_MIXED) runCyclesT<float>(1, 1, true, false);
            else runCycles(1, 1, true, false);
            break;
        case 4:
            launch2_applyk_df(g, Yh.p, Yl.p, K0f, K0lo, dh.p, dl.p, lv[0].r.p, 0, nullptr, nullptr, false, nullptr,
                              nullptr, st);
            break;
        default: cgIteration(xt.p, 1, 1, false); break;
        }
    };
    cudaGraph_t gr;
    cudaGraphExec_t ex;
    VFEM_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    body();
    VFEM_CUDA(cudaStreamEndCapture(st, &gr));
    const uint64_t k = countKernels(gr);
    launchCounter() -= k;
    VFEM_CUDA(cudaGraphInstantiate(&ex, gr, 0));
    cudaEvent_t e0, e1;
    VFEM_CUDA(cudaEventCreate(&e0));
    VFEM_CUDA(cudaEventCreate(&e1));
    for (int w = 0; w < 3; ++w) VFEM_CUDA(cudaGraphLaunch(ex, st));
    VFEM_CUDA(cudaEventRecord(e0, st));
    for (int r = 0; r < reps; ++r) VFEM_CUDA(cudaGraphLaunch(ex, st));
    VFEM_CUDA(cudaEventRecord(e1, st));
    VFEM_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    VFEM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    launchCounter() += k * (uint64_t)(reps + 3);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGraphExecDestroy(ex);
    cudaGraphDestroy(gr);
    return ms / reps;
}

// ---------------------------------------------------------------------------
// LBL2: layer-by-layer evaluation (LayerByLayerEvaluator::run, LayerByLayer.hh:223-296)
// ---------------------------------------------------------------------------
LBL2::Slot::~Slot() {
    if (done) cudaEventDestroy(done);
}

LBL2::LBL2(Grid2 *src_, int coarsenings_, int64_t slots, int precision) : src(src_), coarsenings(coarsenings_) {
    if (coarsenings < 1) throw Error(ERR_ARG, "layer-by-layer solves need at least one coarsening level");
    if (slots < 1) throw Error(ERR_ARG, "slots must be positive");
    const int64_t NN = src->g.NN, NE = src->g.NE;
    for (int64_t s = 0; s < slots; ++s) {
        std::unique_ptr<Slot> sl(new Slot());
        sl->grid = src->clone();
        sl->mg.reset(new MG2(sl->grid.get(), coarsenings));
        sl->mg->setPrecision(precision);
        sl->x.alloc(2 * NN);
        sl->f.alloc(2 * NN);
        sl->gtmp.alloc(NE);
        sl->gacc.alloc(NE);
        sl->cpl.alloc(1);
        sl->part.alloc(REDUCE_BLOCKS + 8);
        VFEM_CUDA(cudaEventCreateWithFlags(&sl->done, cudaEventDisableTiming));
        S.push_back(std::move(sl));
    }
    VFEM_CUDA(cudaMallocHost(&cplHost, slots * sizeof(double)));
}

LBL2::~LBL2() {
    for (auto &sl : S) cudaStreamSynchronize(sl->grid->stream);
    if (cplHost) cudaFreeHost(cplHost);
}

// Bring every slot's simulator to the source's densities, material and loads.
void LBL2::syncSource() {
    VFEM_CUDA(cudaStreamSynchronize(src->stream));
    for (auto &sl : S) {
        Grid2 &g = *sl->grid;
        if (g.Eyoung != src->Eyoung || g.nu != src->nu) g.setETensor(src->Eyoung, src->nu);
        g.E0 = src->E0; g.Emin = src->Emin; g.gamma = src->gamma; g.q = src->q; g.law = src->law;
        g.grav[0] = src->grav[0];
        g.grav[1] = src->grav[1];
        if (g.hmask != src->hmask || g.hval != src->hval)
            throw Error(ERR_STATE, "supports changed after the layer-by-layer evaluator was created");
        if (g.hforce != src->hforce) {
            g.hforce = src->hforce;
            g.uploadBC();
        }
        VFEM_CUDA(cudaMemcpyAsync(g.rho.p, src->rho.p, src->g.NE * sizeof(double), cudaMemcpyDeviceToDevice, g.stream));
        g.updateYoungModuli();
    }
}

void LBL2::setInit(int kind, int history) {
    if (kind < LBL_INIT_ZERO || kind > LBL_INIT_SUBSPACE) throw Error(ERR_ARG, "Unrecognized init method");
    if (kind == LBL_INIT_SUBSPACE && (history < 1 || history > LBL_MAX_HISTORY))
        throw Error(ERR_ARG, "subspace size must lie in 1.." + std::to_string(LBL_MAX_HISTORY));
    initKind = kind;
    historySize = kind == LBL_INIT_CONSTANT ? 1 : kind == LBL_INIT_FD ? 2 : kind == LBL_INIT_SUBSPACE ? history : 0;
}

// The slot's initial guess for `layer` into sl.x (mask and load of the layer already set),
// LayerByLayer.hh:55-209.
void LBL2::guess(Slot &sl, int64_t layer, int ny, bool zeroInit) {
    Grid2 &g = *sl.grid;
    MG2 &mg = *sl.mg;
    cudaStream_t st = g.stream;
    const int64_t n2 = 2 * g.g.NN;
    const Geom2 &gl = mg.lv[0].g;  // level 0 with the device mask
    if (!zeroInit && layer == ny && haveFull) {
        VFEM_CUDA(cudaMemcpyAsync(sl.x.p, uFull.p, n2 * sizeof(double), cudaMemcpyDeviceToDevice, st));
        return;
    }
    const int hs = sl.hs;
    LblVectors U{};
    for (int i = 0; i < hs; ++i) U.u[i] = sl.hist[sl.order[i]].p;
    LblCoeffs cv{};
    if (initKind == LBL_INIT_ZERO || hs == 0) {
        launch_fill<double>(sl.x.p, 0.0, n2, st);
    } else if (initKind == LBL_INIT_CONSTANT || (initKind == LBL_INIT_FD && hs == 1)) {
        cv.c[0] = 1.0;
        launch2_subspace_combine(gl, U, 1, nullptr, cv, sl.x.p, st);
    } else if (initKind == LBL_INIT_FD) {
        cv.c[0] = 2.0;  // 2 u(0) - u(1)
        cv.c[1] = -1.0;
        launch2_subspace_combine(gl, U, 2, nullptr, cv, sl.x.p, st);
    } else {
        // InitGenSubspace: A_ij = u_i . K u_j, b_i = u_i . f over the nondetached nodes
        const int np = hs * (hs + 1) / 2 + hs;
        sl.subPart.alloc((int64_t)np * REDUCE_BLOCKS);
        sl.subC.alloc(LBL_MAX_HISTORY);
        for (int j = 0; j < hs; ++j) {
            sl.Ku[j].alloc(n2);
            launch2_applyk_fine<double>(gl, g.Y.p, g.K0, U.u[j], sl.Ku[j].p, 0, nullptr, g.dmask.p, true, nullptr, nullptr, st);
        }
        int p = 0;
        for (int i = 0; i < hs; ++i)
            for (int j = i; j < hs; ++j, ++p)
                launch2_dot_partials(gl, U.u[i], sl.Ku[j].p, sl.subPart.p + (int64_t)p * REDUCE_BLOCKS, st);
        for (int i = 0; i < hs; ++i, ++p)
            launch2_dot_partials(gl, U.u[i], sl.f.p, sl.subPart.p + (int64_t)p * REDUCE_BLOCKS, st);
        launch_subspace_solve(sl.subPart.p, REDUCE_BLOCKS, hs, sl.subC.p, st);
        launch2_subspace_combine(gl, U, hs, sl.subC.p, cv, sl.x.p, st);
    }
}

void LBL2::pushHistory(Slot &sl) {
    if (historySize == 0) return;
    const int64_t n2 = 2 * sl.grid->g.NN;
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
    sl.hist[slot].alloc(n2);
    VFEM_CUDA(cudaMemcpyAsync(sl.hist[slot].p, sl.x.p, n2 * sizeof(double), cudaMemcpyDeviceToDevice, sl.grid->stream));
}

void LBL2::run(const int64_t *layers, int64_t count, int64_t maxIter, double tol, int64_t mgIter, int64_t sweeps,
               bool fmg, bool zeroInit, double *compliance, int64_t *iterations, double *gradSum) {
    if (count <= 0) return;
    const int ny = src->g.ne[BUILD_DIR];
    for (int64_t t = 0; t < count; ++t)
        if (layers[t] < 1 || layers[t] > ny) throw Error(ERR_ARG, "layer height out of range");
    syncSource();
    const int64_t ns = std::min<int64_t>((int64_t)S.size(), count);
    const int64_t NN = src->g.NN, NE = src->g.NE;
    const bool warm = initKind != LBL_INIT_ZERO;
    for (auto &slp : S) {
        slp->queue.clear();
        slp->qpos = 0;
        slp->hs = 0;
        slp->idx = -1;
    }
    if (warm) {
        int64_t t = 0;
        for (int64_t s = 0; s < ns; ++s) {
            const int64_t len = count / ns + (s < count % ns ? 1 : 0);
            for (int64_t k = 0; k < len; ++k) S[s]->queue.push_back(t++);
        }
    }
    for (int64_t s = 0; s < ns; ++s)
        VFEM_CUDA(cudaMemsetAsync(S[s]->gacc.p, 0, NE * sizeof(double), S[s]->grid->stream));
    if (!uFull.p) uFull.alloc(2 * NN);

    auto start = [&](int64_t s, int64_t idx) {
        Slot &sl = *S[s];
        Grid2 &g = *sl.grid;
        MG2 &mg = *sl.mg;
        cudaStream_t st = g.stream;
        mg.setMaskLayer(layers[idx]);
        g.buildLoadDev(sl.f.p);
        guess(sl, layers[idx], ny, zeroInit);
        mg.pcgStart(sl.x.p, sl.f.p, maxIter, tol, mgIter, sweeps, fmg, true);
        // compliance f.u over the nondetached nodes
        launch2_dot_partials(mg.lv[0].g, sl.f.p, sl.x.p, sl.part.p, st);
        launch_finalize(sl.part.p, REDUCE_BLOCKS, sl.cpl.p, st);
        VFEM_CUDA(cudaMemcpyAsync(cplHost + s, sl.cpl.p, sizeof(double), cudaMemcpyDeviceToHost, st));
        launch2_adjoint(g.g, g.rho.p, sl.x.p, sl.x.p, sl.gtmp.p, g.K0, g.E0, g.Emin, g.gamma, g.q, g.law, g.grav, g.vol(),
                        1.0, 0.5, st);
        launch_axpy(NE, 1.0, sl.gtmp.p, sl.gacc.p, st);
        if (layers[idx] == ny)
            VFEM_CUDA(cudaMemcpyAsync(uFull.p, sl.x.p, 2 * NN * sizeof(double), cudaMemcpyDeviceToDevice, st));
        if (warm && sl.qpos < sl.queue.size()) pushHistory(sl);
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

// ---------------------------------------------------------------------------
// Problem backend
// ---------------------------------------------------------------------------
namespace {
struct Backend2D : ProblemBackend {
    MG2 *mg;
    Grid2 *grid;
    explicit Backend2D(MG2 *m) : mg(m), grid(m->fine) {}
    int64_t numElems() const override { return grid->g.NE; }
    int64_t numDofs() const override { return 2 * grid->g.NN; }
    void filterDims(int dims[3], int &ndim) const override {
        dims[0] = grid->g.ne[0];
        dims[1] = grid->g.ne[1];
        dims[2] = 1;
        ndim = 2;
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
        return mg->pcgDev(u, f, cgIter, tol, mgIter, sweeps, fmg, false, nullptr, nullptr);
    }
    double dotAll(const double *a, const double *b, double *partials) override {
        cudaStream_t st = grid->stream;
        Geom2 gall = grid->g;
        gall.firstDetN = (int)LAYER_MASK_NONE;
        gall.dyn = nullptr;
        launch2_dot_partials(gall, a, b, partials, st);
        launch_finalize(partials, REDUCE_BLOCKS, partials + REDUCE_BLOCKS, st);
        double v = 0;
        VFEM_CUDA(cudaMemcpyAsync(&v, partials + REDUCE_BLOCKS, sizeof(double), cudaMemcpyDeviceToHost, st));
        VFEM_CUDA(cudaStreamSynchronize(st));
        return v;
    }
    void complianceGradient(const double *u, double *out) override {
        launch2_adjoint(grid->g, grid->rho.p, u, u, out, grid->K0, grid->E0, grid->Emin, grid->gamma, grid->q,
                        grid->law, grid->grav, grid->vol(), 1.0, 0.5, grid->stream);
    }
};
}  // namespace

std::unique_ptr<ProblemBackend> makeBackend2D(MG2 *mg) { return std::unique_ptr<ProblemBackend>(new Backend2D(mg)); }

}  // namespace vfem
