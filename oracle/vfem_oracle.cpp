// vfem_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A plain CPU (C++17 + OpenMP) restatement of VoxelFEM's solve-and-sensitivity
// path for trilinear (Q1) hexahedral voxels. It is the parity checker for the
// CUDA library and the timed CPU baseline; it is never linked into, loaded by,
// or called from the product path.
//
// PARITY UNPINNED: the reference cannot be compiled (its MeshFEM submodule,
// Eigen, TBB and CHOLMOD are absent) and ships no tests, golden vectors or
// fixtures. This file follows the reference source line by line instead; each
// function cites the reference file:line it restates. Independent checks of
// this restatement (exact symbolic K0, Galerkin identity, symmetry, FD
// gradients) live in tests/.
//
// Layout conventions (identical to the reference):
//   * node (i,j,k) -> (i*ny1 + j)*nz1 + k, last index fastest
//     (NDVector.hh:249-265, TensorProductSimulator.hh:209-279);
//   * element local node l = 4*dx + 2*dy + dz; element DOF = 3*l + c;
//   * nodal vector fields are SoA: component c of node n at [c*nn + n]
//     (Eigen ColMajor VField, TensorProductSimulator.hh:180).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int BUILD_DIR = 1;  // TensorProductSimulator.hh:1851
constexpr long LAYER_MASK_NONE = std::numeric_limits<int>::max();
constexpr int MARGIN = 4;     // VOXELFEM_SIMD_WIDTH margin, MultigridSolver.hh:532

thread_local std::string g_err;

using Mat24 = std::array<double, 576>;

struct Sim {
    long ne[3], nn[3];
    size_t NE, NN;
    double bmin[3], bmax[3], h[3];
    double K0[576];
    double K0diag[8][9];
    double E_young = 1.0, nu = 0.0;  // ETensor(1, 0) default, TensorProductSimulator.hh:2114
    double E0 = 1, Emin = 1e-4, gamma = 3, q = 3;  // :2137-2141
    int law = 0;                                     // 0 = SIMP, 1 = RAMP
    std::vector<double> rho, Y;
    std::vector<uint8_t> dmask;
    std::vector<double> dval;
    std::vector<double> force;  // dense nodal forces, SoA
    double grav[3] = {0, 0, 0};
    double maskH = std::numeric_limits<double>::infinity();
    long firstMaskedE = LAYER_MASK_NONE, firstDetN = LAYER_MASK_NONE;
    std::vector<Mat24> Kcache;  // per-element Ke (coarse levels)

    size_t node(long i, long j, long k) const { return ((size_t)i * nn[1] + j) * nn[2] + k; }
    size_t elem(long i, long j, long k) const { return ((size_t)i * ne[1] + j) * ne[2] + k; }
    void nodeIdx(size_t n, long &i, long &j, long &k) const {
        k = n % nn[2]; n /= nn[2]; j = n % nn[1]; i = n / nn[1];
    }
    void elemIdx(size_t e, long &i, long &j, long &k) const {
        k = e % ne[2]; e /= ne[2]; j = e % ne[1]; i = e / ne[1];
    }
    double nodePos(long idx, int d) const { return bmin[d] + idx * h[d]; }
    long nondetNodes() const { return std::min<long>(firstDetN, nn[1]); }
    long nonmaskedElems() const { return std::min<long>(firstMaskedE, ne[1]); }
    bool elemMasked(long ej) const { return ej >= firstMaskedE; }
    bool nodeDetached(long nj) const { return nj >= firstDetN; }
    double vol() const { return h[0] * h[1] * h[2]; }
};

// ---------------------------------------------------------------------------
// Element stiffness (TensorProductSimulator.hh:67-80, 2078-2086;
// TensorProductPolynomialInterpolant.hh:129-232; TensorProductQuadrature.hh:134-143).
// K0_ij = vol * sum_q w_q eps(phi_i) : C : eps(phi_j) with 2-point Gauss per axis;
// eps(phi_{n,c}) = sym(e_c (x) grad N_n); isotropic C from (E, nu).
// ---------------------------------------------------------------------------
void computeK0(Sim &s) {
    const double lam = s.E_young * s.nu / ((1 + s.nu) * (1 - 2 * s.nu));
    const double mu = s.E_young / (2 * (1 + s.nu));
    const double gp[2] = {0.21132486540518711775, 0.78867513459481288225};
    double K[576];
    std::fill(K, K + 576, 0.0);
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 2; ++c) {
                const double xi[3] = {gp[a], gp[b], gp[c]};
                double grad[8][3];
                for (int l = 0; l < 8; ++l) {
                    int bits[3] = {(l >> 2) & 1, (l >> 1) & 1, l & 1};
                    for (int d = 0; d < 3; ++d) {
                        double v = 1.0;
                        for (int e = 0; e < 3; ++e) {
                            if (e == d) v *= (bits[e] ? 1.0 : -1.0) / s.h[e];
                            else v *= bits[e] ? xi[e] : (1.0 - xi[e]);
                        }
                        grad[l][d] = v;
                    }
                }
                // strain of each vector basis function
                double eps[24][3][3];
                for (int l = 0; l < 8; ++l)
                    for (int cc = 0; cc < 3; ++cc) {
                        double (&E)[3][3] = eps[3 * l + cc];
                        for (int i = 0; i < 3; ++i)
                            for (int j = 0; j < 3; ++j) E[i][j] = 0;
                        for (int i = 0; i < 3; ++i) { E[cc][i] = 0.5 * grad[l][i]; E[i][cc] = 0.5 * grad[l][i]; }
                        E[cc][cc] = grad[l][cc];
                    }
                for (int i = 0; i < 24; ++i)
                    for (int j = i; j < 24; ++j) {
                        double tri = eps[i][0][0] + eps[i][1][1] + eps[i][2][2];
                        double trj = eps[j][0][0] + eps[j][1][1] + eps[j][2][2];
                        double dd = 0;
                        for (int p = 0; p < 3; ++p)
                            for (int r = 0; r < 3; ++r) dd += eps[i][p][r] * eps[j][p][r];
                        K[i * 24 + j] += 0.125 * (lam * tri * trj + 2 * mu * dd);
                    }
            }
    const double v = s.vol();
    for (int i = 0; i < 24; ++i)
        for (int j = i; j < 24; ++j) {
            s.K0[i * 24 + j] = K[i * 24 + j] * v;
            s.K0[j * 24 + i] = s.K0[i * 24 + j];
        }
    for (int l = 0; l < 8; ++l)
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) s.K0diag[l][3 * r + c] = s.K0[(3 * l + r) * 24 + 3 * l + c];
}

void initSim(Sim &s, const long ne[3], const double bmin[3], const double bmax[3]) {
    for (int d = 0; d < 3; ++d) {
        s.ne[d] = ne[d];
        s.nn[d] = ne[d] + 1;
        s.bmin[d] = bmin[d];
        s.bmax[d] = bmax[d];
        s.h[d] = (bmax[d] - bmin[d]) / ne[d];
    }
    s.NE = (size_t)ne[0] * ne[1] * ne[2];
    s.NN = (size_t)s.nn[0] * s.nn[1] * s.nn[2];
    s.rho.assign(s.NE, 0.0);  // NDVector zero-initialised
    s.Y.assign(s.NE, 0.0);
    s.dmask.assign(s.NN, 0);
    s.dval.assign(3 * s.NN, 0.0);
    s.force.assign(3 * s.NN, 0.0);
    computeK0(s);
}

// TensorProductSimulator.hh:2055-2060
double unmaskedY(const Sim &s, size_t e) {
    if (s.law == 0) return s.Emin + std::pow(s.rho[e], s.gamma) * (s.E0 - s.Emin);
    return s.Emin + s.rho[e] * (s.E0 - s.Emin) / (1 + s.q * (1 - s.rho[e]));
}

// TensorProductSimulator.hh:2088-2102
void updateY(Sim &s) {
    const bool masking = s.maskH < s.bmax[BUILD_DIR];
#pragma omp parallel for schedule(static)
    for (long e = 0; e < (long)s.NE; ++e) {
        long i, j, k;
        s.elemIdx(e, i, j, k);
        s.Y[e] = (masking && s.elemMasked(j)) ? 0.0 : unmaskedY(s, e);
    }
}

// TensorProductSimulator.hh:290-303
void setMaskHeight(Sim &s, double hgt, bool update) {
    if (hgt < 0 || hgt > s.bmax[BUILD_DIR]) throw std::runtime_error("Fabrication height out of range");
    s.maskH = hgt;
    s.firstMaskedE = (long)std::ceil(hgt / s.h[BUILD_DIR] - 1e-10);
    s.firstDetN = s.firstMaskedE + 1;
    if (update) updateY(s);
}

// TensorProductSimulator.hh:241-252 with BCBuilder::setDirichlet :73-88
void addDirichlet(Sim &s, const double u[3], const double mn[3], const double mx[3], uint8_t cmask) {
    for (size_t n = 0; n < s.NN; ++n) {
        long idx[3];
        s.nodeIdx(n, idx[0], idx[1], idx[2]);
        bool inside = true;
        for (int d = 0; d < 3; ++d) {
            double p = s.nodePos(idx[d], d);
            if (p < mn[d] || p > mx[d]) inside = false;
        }
        if (!inside) continue;
        for (int c = 0; c < 3; ++c) {
            if (!(cmask >> c & 1)) continue;
            if (!(s.dmask[n] >> c & 1)) {
                s.dmask[n] |= (uint8_t)(1 << c);
                s.dval[c * s.NN + n] = u[c];
            } else if (std::abs(s.dval[c * s.NN + n] - u[c]) > 1e-10) {
                throw std::runtime_error("Conflicting dirichlet displacements.");
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Matrix-free Q1 applyK (TPSStencils.hh:431-728): node-centric gather over the
// (up to) 8 incident elements; detached rows skipped and, for ZeroInit, zeroed.
// ---------------------------------------------------------------------------
template <bool ZeroInit, bool Negate>
void applyK_fine(const Sim &s, const double *u, double *res) {
    const long nyv = s.nondetNodes();
    const size_t NN = s.NN;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < s.nn[0]; ++i)
        for (long j = 0; j < nyv; ++j)
            for (long k = 0; k < s.nn[2]; ++k) {
                const size_t n = s.node(i, j, k);
                double f[3];
                for (int c = 0; c < 3; ++c) f[c] = ZeroInit ? 0.0 : res[c * NN + n];
                // element order of the guarded path: (0,0,0),(0,0,-1),(0,-1,0),(0,-1,-1),(-1,0,0),...
                for (int a = 0; a < 2; ++a)
                    for (int b = 0; b < 2; ++b)
                        for (int cc = 0; cc < 2; ++cc) {
                            const long ei = i - a, ej = j - b, ek = k - cc;
                            if (ei < 0 || ej < 0 || ek < 0 || ei >= s.ne[0] || ej >= s.ne[1] || ek >= s.ne[2]) continue;
                            const double E = s.Y[s.elem(ei, ej, ek)];
                            const int ln = 4 * a + 2 * b + cc;
                            double ue[24];
                            for (int m = 0; m < 8; ++m) {
                                size_t nm = s.node(ei + (m >> 2 & 1), ej + (m >> 1 & 1), ek + (m & 1));
                                for (int c = 0; c < 3; ++c) ue[3 * m + c] = u[c * NN + nm];
                            }
                            for (int c = 0; c < 3; ++c) {
                                const int row = 3 * ln + c;
                                double contrib = 0;
                                for (int jj = 0; jj < 24; ++jj) contrib += s.K0[jj * 24 + row] * ue[jj];
                                if (Negate) f[c] -= E * contrib;
                                else f[c] += E * contrib;
                            }
                        }
                for (int c = 0; c < 3; ++c) res[c * NN + n] = f[c];
            }
    if (ZeroInit && nyv < s.nn[1]) {
#pragma omp parallel for schedule(static)
        for (long i = 0; i < s.nn[0]; ++i)
            for (long j = nyv; j < s.nn[1]; ++j)
                for (long k = 0; k < s.nn[2]; ++k)
                    for (int c = 0; c < 3; ++c) res[c * NN + s.node(i, j, k)] = 0.0;
    }
}

// Cached-Ke element-loop applyK (TensorProductSimulator.hh:1418-1434).
template <bool ZeroInit, bool Negate>
void applyK_cached(const Sim &s, const double *u, double *res) {
    const size_t NN = s.NN;
    if (ZeroInit) std::fill(res, res + 3 * NN, 0.0);
    for (int col = 0; col < 8; ++col) {
        const long o[3] = {col >> 2 & 1, col >> 1 & 1, col & 1};
#pragma omp parallel for schedule(static)
        for (long i = o[0]; i < s.ne[0]; i += 2)
            for (long j = o[1]; j < s.ne[1]; j += 2)
                for (long k = o[2]; k < s.ne[2]; k += 2) {
                    const Mat24 &Ke = s.Kcache[s.elem(i, j, k)];
                    size_t nodes[8];
                    double ue[24], y[24];
                    for (int m = 0; m < 8; ++m) {
                        nodes[m] = s.node(i + (m >> 2 & 1), j + (m >> 1 & 1), k + (m & 1));
                        for (int c = 0; c < 3; ++c) ue[3 * m + c] = u[c * NN + nodes[m]];
                    }
                    for (int r = 0; r < 24; ++r) {
                        double acc = 0;
                        for (int c = 0; c < 24; ++c) acc += Ke[r * 24 + c] * ue[c];
                        y[r] = acc;
                    }
                    for (int m = 0; m < 8; ++m)
                        for (int c = 0; c < 3; ++c) res[c * NN + nodes[m]] += Negate ? -y[3 * m + c] : y[3 * m + c];
                }
    }
}

// TensorProductSimulator.hh:1269-1288 (integrated Q1 shape function = 1/8)
void buildLoad(const Sim &s, double *f) {
    std::copy(s.force.begin(), s.force.end(), f);
    if (s.grav[0] * s.grav[0] + s.grav[1] * s.grav[1] + s.grav[2] * s.grav[2] != 0) {
        for (size_t e = 0; e < s.NE; ++e) {
            long i, j, k;
            s.elemIdx(e, i, j, k);
            if (s.elemMasked(j)) continue;
            for (int l = 0; l < 8; ++l) {
                size_t n = s.node(i + (l >> 2 & 1), j + (l >> 1 & 1), k + (l & 1));
                for (int c = 0; c < 3; ++c) f[c * s.NN + n] += s.grav[c] * (0.125 * s.rho[e] * s.vol());
            }
        }
    }
}

// TensorProductSimulator.hh:973-1005
void complianceGradient(const Sim &s, const double *u, double *g) {
    const bool sw = s.grav[0] * s.grav[0] + s.grav[1] * s.grav[1] + s.grav[2] * s.grav[2] != 0;
#pragma omp parallel for schedule(static)
    for (long e = 0; e < (long)s.NE; ++e) {
        long i, j, k;
        s.elemIdx(e, i, j, k);
        if (s.elemMasked(j)) { g[e] = 0; continue; }
        double ue[24];
        for (int m = 0; m < 8; ++m) {
            size_t nm = s.node(i + (m >> 2 & 1), j + (m >> 1 & 1), k + (m & 1));
            for (int c = 0; c < 3; ++c) ue[3 * m + c] = u[c * s.NN + nm];
        }
        double uKu = 0;
        for (int r = 0; r < 24; ++r) {
            double acc = 0;
            for (int c = 0; c < 24; ++c) acc += s.K0[r * 24 + c] * ue[c];
            uKu += ue[r] * acc;
        }
        double val;
        if (s.law == 0) val = -0.5 * s.gamma * std::pow(s.rho[e], s.gamma - 1.0) * (s.E0 - s.Emin) * uKu;
        else val = -0.5 * (1 + s.q) * (s.E0 - s.Emin) / std::pow(1 + s.q * (1 - s.rho[e]), 2) * uKu;
        if (sw)
            for (int l = 0; l < 8; ++l)
                val += 0.125 * (s.grav[0] * ue[3 * l] + s.grav[1] * ue[3 * l + 1] + s.grav[2] * ue[3 * l + 2]) * s.vol();
        g[e] = val;
    }
}

// TensorProductSimulator.hh:638-654
void elementEnergy(const Sim &s, const double *u, double *out) {
#pragma omp parallel for schedule(static)
    for (long e = 0; e < (long)s.NE; ++e) {
        long i, j, k;
        s.elemIdx(e, i, j, k);
        double ue[24];
        for (int m = 0; m < 8; ++m) {
            size_t nm = s.node(i + (m >> 2 & 1), j + (m >> 1 & 1), k + (m & 1));
            for (int c = 0; c < 3; ++c) ue[3 * m + c] = u[c * s.NN + nm];
        }
        double uKu = 0;
        for (int r = 0; r < 24; ++r) {
            double acc = 0;
            for (int c = 0; c < 24; ++c) acc += s.K0[r * 24 + c] * ue[c];
            uKu += ue[r] * acc;
        }
        out[e] = 0.5 * s.Y[e] * uKu;
    }
}

// ---------------------------------------------------------------------------
// Dense Cholesky on the reduced coarsest system (replaces CHOLMOD,
// TensorProductSimulator.hh:1181-1230).
// ---------------------------------------------------------------------------
struct DenseChol {
    long n = 0;
    std::vector<double> L;
    std::vector<long> freeIdx;  // reduced -> full DOF (node-major 3*n+c)
    void factor(std::vector<double> &A, long nfree) {
        n = nfree;
        L.swap(A);
        for (long j = 0; j < n; ++j) {
            double d = L[j * n + j];
            for (long k = 0; k < j; ++k) d -= L[j * n + k] * L[j * n + k];
            if (!(d > 0)) throw std::runtime_error("Coarsest matrix not positive definite");
            d = std::sqrt(d);
            L[j * n + j] = d;
#pragma omp parallel for schedule(static) if (n > 256)
            for (long i = j + 1; i < n; ++i) {
                double v = L[i * n + j];
                for (long k = 0; k < j; ++k) v -= L[i * n + k] * L[j * n + k];
                L[i * n + j] = v / d;
            }
        }
    }
    void solve(std::vector<double> &b) const {
        for (long i = 0; i < n; ++i) {
            double v = b[i];
            for (long k = 0; k < i; ++k) v -= L[i * n + k] * b[k];
            b[i] = v / L[i * n + i];
        }
        for (long i = n - 1; i >= 0; --i) {
            double v = b[i];
            for (long k = i + 1; k < n; ++k) v -= L[k * n + i] * b[k];
            b[i] = v / L[i * n + i];
        }
    }
};

// ---------------------------------------------------------------------------
// Multigrid solver (MultigridSolver.hh)
// ---------------------------------------------------------------------------
struct MG {
    Sim *fine;
    std::vector<std::unique_ptr<Sim>> owned;
    std::vector<Sim *> sims;
    std::vector<std::vector<double>> x, b, r;
    std::vector<double> Ad, dvec;
    std::array<Mat24, 8> Kc;    // coarsenedFineK0s
    std::array<std::array<double, 64>, 8> phis;  // phis[fi][fine_n*8 + coarse_n]
    // blockK as 27-block stencils for levels 2..L-2: [n][27][9]
    std::vector<std::vector<double>> blockK;
    DenseChol chol;
    bool cholValid = false;
    bool symmetricGS = true;
    long cachedLayer = LAYER_MASK_NONE;
    bool stiffnessValid = false;

    int L() const { return (int)sims.size(); }
    Sim &sim(int l) { return *sims[l]; }
};

// MultigridSolver.hh:664-687
void buildPhis(MG &mg) {
    for (int fine_n = 0; fine_n < 8; ++fine_n) {
        double half[3] = {0.5 * (fine_n >> 2 & 1), 0.5 * (fine_n >> 1 & 1), 0.5 * (fine_n & 1)};
        int fi = 0;
        for (int fx = 0; fx < 2; ++fx)
            for (int fy = 0; fy < 2; ++fy)
                for (int fz = 0; fz < 2; ++fz) {
                    double p[3] = {half[0] + 0.5 * fx, half[1] + 0.5 * fy, half[2] + 0.5 * fz};
                    for (int cn = 0; cn < 8; ++cn) {
                        double v = 1;
                        for (int d = 0; d < 3; ++d) {
                            int bit = cn >> (2 - d) & 1;
                            v *= bit ? p[d] : (1 - p[d]);
                        }
                        mg.phis[fi][fine_n * 8 + cn] = v;
                    }
                    ++fi;
                }
    }
}

// MultigridSolver.hh:712-722: Ke_c += I^T Ke_f I with I = phi (x) Id_3
void accumulateCoarsened(const double *phi, const double *Kf, double *Kc) {
    double T[576];  // Kf * I
    for (int r = 0; r < 24; ++r)
        for (int cn = 0; cn < 8; ++cn)
            for (int d = 0; d < 3; ++d) {
                double acc = 0;
                for (int fn = 0; fn < 8; ++fn) acc += Kf[r * 24 + 3 * fn + d] * phi[fn * 8 + cn];
                T[r * 24 + 3 * cn + d] = acc;
            }
    for (int cm = 0; cm < 8; ++cm)
        for (int d = 0; d < 3; ++d)
            for (int c = 0; c < 24; ++c) {
                double acc = 0;
                for (int fm = 0; fm < 8; ++fm) acc += phi[fm * 8 + cm] * T[(3 * fm + d) * 24 + c];
                Kc[(3 * cm + d) * 24 + c] += acc;
            }
}

// MultigridSolver.hh:35-121
MG *createMG(Sim *fine, int numCoarsening) {
    auto *mg = new MG();
    mg->fine = fine;
    mg->sims.push_back(fine);
    long ne[3] = {fine->ne[0], fine->ne[1], fine->ne[2]};
    for (int l = 1; l <= numCoarsening; ++l) {
        for (int d = 0; d < 3; ++d) {
            if (ne[d] % 2 == 1) {
                delete mg;
                throw std::runtime_error("Grid size currently must be divisible by 2^numCoarseningLevels");
            }
            ne[d] /= 2;
        }
        auto s = std::make_unique<Sim>();
        initSim(*s, ne, fine->bmin, fine->bmax);
        s->E_young = fine->E_young;
        s->nu = fine->nu;
        computeK0(*s);
        Sim &finer = *mg->sims.back();
        Sim &coarser = *s;
        // Dirichlet coarsening (:58-103)
        for (size_t fn = 0; fn < finer.NN; ++fn) {
            if (!finer.dmask[fn]) continue;
            long fidx[3];
            finer.nodeIdx(fn, fidx[0], fidx[1], fidx[2]);
            long e[3];
            int pob[3];
            for (int d = 0; d < 3; ++d) {
                double p = finer.nodePos(fidx[d], d);
                double rel = p - coarser.bmin[d];
                double fidxd = rel / coarser.h[d];
                long ed;
                if (std::abs(fidxd - coarser.ne[d]) < 1e-10) ed = coarser.ne[d] - 1;
                else ed = (long)fidxd;
                e[d] = ed;
                double cref = (p - coarser.nodePos(ed, d)) / coarser.h[d];
                pob[d] = std::abs(cref) < 1e-9 ? 0 : (std::abs(cref - 1.0) < 1e-9 ? 1 : -1);
            }
            for (int ln = 0; ln < 8; ++ln) {
                int lb[3] = {ln >> 2 & 1, ln >> 1 & 1, ln & 1};
                bool ok = true;
                for (int d = 0; d < 3; ++d)
                    if (pob[d] != -1 && pob[d] != lb[d]) ok = false;
                if (!ok) continue;
                size_t cn = coarser.node(e[0] + lb[0], e[1] + lb[1], e[2] + lb[2]);
                uint8_t cm = finer.dmask[fn];
                for (int c = 0; c < 3; ++c)
                    if (cm >> c & 1) {
                        if (!(coarser.dmask[cn] >> c & 1)) {
                            coarser.dmask[cn] |= (uint8_t)(1 << c);
                            coarser.dval[c * coarser.NN + cn] = 0.0;
                        }
                    }
            }
        }
        mg->owned.push_back(std::move(s));
        mg->sims.push_back(mg->owned.back().get());
    }
    for (int l = 0; l < mg->L(); ++l) {
        size_t n3 = 3 * mg->sim(l).NN;
        mg->x.emplace_back(n3, 0.0);
        mg->b.emplace_back(n3, 0.0);
        mg->r.emplace_back(n3, 0.0);
    }
    mg->blockK.resize(mg->L());
    buildPhis(*mg);
    for (int fi = 0; fi < 8; ++fi) {
        std::fill(mg->Kc[fi].begin(), mg->Kc[fi].end(), 0.0);
        accumulateCoarsened(mg->phis[fi].data(), fine->K0, mg->Kc[fi].data());
    }
    return mg;
}

// Level-1 element matrix (MultigridSolver.hh:724-738)
void firstLevelKe(MG &mg, long ci, long cj, long ck, double *out) {
    Sim &f = mg.sim(0);
    int fi = 0;
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 2; ++c) {
                double E = f.Y[f.elem(2 * ci + a, 2 * cj + b, 2 * ck + c)];
                for (int t = 0; t < 576; ++t) out[t] = (fi == 0) ? E * mg.Kc[fi][t] : out[t] + E * mg.Kc[fi][t];
                ++fi;
            }
}

// Recursive coarsening (MultigridSolver.hh:745-819)
void coarsenedKe(MG &mg, int l, long ci, long cj, long ck, double *out) {
    Sim &coarser = mg.sim(l);
    if (coarser.elemMasked(cj)) { std::fill(out, out + 576, 0.0); return; }
    if (l == 1) { firstLevelKe(mg, ci, cj, ck, out); return; }
    std::fill(out, out + 576, 0.0);
    double child[576];
    int fi = 0;
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 2; ++c) {
                coarsenedKe(mg, l - 1, 2 * ci + a, 2 * cj + b, 2 * ck + c, child);
                accumulateCoarsened(mg.phis[fi].data(), child, out);
                ++fi;
            }
}

// MultigridSolver.hh:846-905 (full recomputation) with blockK held as a 27-block stencil
void updateStiffness(MG &mg) {
    const int L = mg.L();
    for (int l = 1; l < L; ++l) {
        Sim &s = mg.sim(l);
        const bool useBlockK = l < L - 1;
        if (l == 1 && useBlockK) continue;
        std::vector<Mat24> Ke(s.NE);
#pragma omp parallel for schedule(dynamic, 16)
        for (long e = 0; e < (long)s.NE; ++e) {
            long i, j, k;
            s.elemIdx(e, i, j, k);
            coarsenedKe(mg, l, i, j, k, Ke[e].data());
        }
        if (useBlockK) {
            std::vector<double> &B = mg.blockK[l];
            B.assign(s.NN * 243, 0.0);
#pragma omp parallel for schedule(static)
            for (long n = 0; n < (long)s.NN; ++n) {
                long i, j, k;
                s.nodeIdx(n, i, j, k);
                double *row = &B[n * 243];
                for (int a = 0; a < 2; ++a)
                    for (int b = 0; b < 2; ++b)
                        for (int c = 0; c < 2; ++c) {
                            long ei = i - a, ej = j - b, ek = k - c;
                            if (ei < 0 || ej < 0 || ek < 0 || ei >= s.ne[0] || ej >= s.ne[1] || ek >= s.ne[2]) continue;
                            const Mat24 &K = Ke[s.elem(ei, ej, ek)];
                            int ln = 4 * a + 2 * b + c;
                            for (int m = 0; m < 8; ++m) {
                                int mb[3] = {m >> 2 & 1, m >> 1 & 1, m & 1};
                                int o = (mb[0] - a + 1) * 9 + (mb[1] - b + 1) * 3 + (mb[2] - c + 1);
                                for (int r = 0; r < 3; ++r)
                                    for (int cc = 0; cc < 3; ++cc) row[o * 9 + 3 * r + cc] += K[(3 * ln + r) * 24 + 3 * m + cc];
                            }
                        }
            }
        } else {
            s.Kcache = std::move(Ke);
        }
    }
    mg.cholValid = false;
    mg.stiffnessValid = true;
}

// Coarsest direct solve (TensorProductSimulator.hh:1181-1230)
void coarseSolve(MG &mg, const double *bvec, double *xout) {
    Sim &s = mg.sim(mg.L() - 1);
    const size_t NN = s.NN;
    std::vector<char> fixed(3 * NN, 0);
    for (size_t n = 0; n < NN; ++n) {
        long i, j, k;
        s.nodeIdx(n, i, j, k);
        for (int c = 0; c < 3; ++c) {
            if (s.dmask[n] >> c & 1) {
                if (s.dval[c * NN + n] != 0) throw std::runtime_error("Nonzero Dirichlet constraints currently unsupported");
                fixed[3 * n + c] = 1;
            }
            if (s.nodeDetached(j)) fixed[3 * n + c] = 1;
        }
    }
    if (!mg.cholValid) {
        std::vector<long> red(3 * NN, -1);
        mg.chol.freeIdx.clear();
        for (size_t d = 0; d < 3 * NN; ++d)
            if (!fixed[d]) { red[d] = (long)mg.chol.freeIdx.size(); mg.chol.freeIdx.push_back((long)d); }
        const long nf = (long)mg.chol.freeIdx.size();
        std::vector<double> A((size_t)nf * nf, 0.0);
        for (size_t e = 0; e < s.NE; ++e) {
            long i, j, k;
            s.elemIdx(e, i, j, k);
            const Mat24 &K = s.Kcache[e];
            for (int a = 0; a < 8; ++a) {
                size_t na = s.node(i + (a >> 2 & 1), j + (a >> 1 & 1), k + (a & 1));
                for (int b = 0; b < 8; ++b) {
                    size_t nb = s.node(i + (b >> 2 & 1), j + (b >> 1 & 1), k + (b & 1));
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c) {
                            long ra = red[3 * na + r], cb = red[3 * nb + c];
                            if (ra < 0 || cb < 0) continue;
                            A[(size_t)ra * nf + cb] += K[(3 * a + r) * 24 + 3 * b + c];
                        }
                }
            }
        }
        mg.chol.factor(A, nf);
        mg.cholValid = true;
    }
    std::vector<double> rhs(mg.chol.n);
    for (long t = 0; t < mg.chol.n; ++t) {
        long d = mg.chol.freeIdx[t];
        rhs[t] = bvec[(d % 3) * NN + d / 3];
    }
    mg.chol.solve(rhs);
    std::fill(xout, xout + 3 * NN, 0.0);
    for (long t = 0; t < mg.chol.n; ++t) {
        long d = mg.chol.freeIdx[t];
        xout[(d % 3) * NN + d / 3] = rhs[t];
    }
}

// Per-level applyK (MultigridSolver.hh:471-504)
template <bool ZeroInit, bool Negate>
void applyK_level(MG &mg, int l, const double *u, double *res) {
    Sim &s = mg.sim(l);
    const size_t NN = s.NN;
    if (l == 0) return applyK_fine<ZeroInit, Negate>(s, u, res);
    if (l == 1) {
        const long nyv = std::min<long>(s.nondetNodes() + 0, s.nn[1]);
        if (ZeroInit) {
            for (long i = 0; i < s.nn[0]; ++i)
                for (long j = 0; j < nyv; ++j)
                    for (long k = 0; k < s.nn[2]; ++k)
                        for (int c = 0; c < 3; ++c) res[c * NN + s.node(i, j, k)] = 0.0;
        }
        const long nev = s.nonmaskedElems();
        for (int col = 0; col < 8; ++col) {
            const long o[3] = {col >> 2 & 1, col >> 1 & 1, col & 1};
            if (o[1] >= nev) continue;
#pragma omp parallel for schedule(static)
            for (long i = o[0]; i < s.ne[0]; i += 2)
                for (long j = o[1]; j < nev; j += 2)
                    for (long k = o[2]; k < s.ne[2]; k += 2) {
                        size_t nodes[8];
                        double ue[24], y[24], Ke[576];
                        for (int m = 0; m < 8; ++m) {
                            nodes[m] = s.node(i + (m >> 2 & 1), j + (m >> 1 & 1), k + (m & 1));
                            for (int c = 0; c < 3; ++c) ue[3 * m + c] = u[c * NN + nodes[m]];
                        }
                        // Ke_u_local = sum_f E_f (Kc_f u_local)
                        Sim &f = mg.sim(0);
                        int fi = 0;
                        for (int t = 0; t < 24; ++t) y[t] = 0;
                        for (int a = 0; a < 2; ++a)
                            for (int b = 0; b < 2; ++b)
                                for (int c = 0; c < 2; ++c) {
                                    double E = f.Y[f.elem(2 * i + a, 2 * j + b, 2 * k + c)];
                                    for (int rr = 0; rr < 24; ++rr) {
                                        double acc = 0;
                                        for (int cc = 0; cc < 24; ++cc) acc += mg.Kc[fi][rr * 24 + cc] * ue[cc];
                                        y[rr] += E * acc;
                                    }
                                    ++fi;
                                }
                        (void)Ke;
                        for (int m = 0; m < 8; ++m)
                            for (int c = 0; c < 3; ++c) res[c * NN + nodes[m]] += Negate ? -y[3 * m + c] : y[3 * m + c];
                    }
        }
        return;
    }
    if (!mg.stiffnessValid) updateStiffness(mg);
    if (l < mg.L() - 1) {
        // blockK SpMV over all rows (CSCMatrix::applyTransposeParallel)
        const std::vector<double> &B = mg.blockK[l];
#pragma omp parallel for schedule(static)
        for (long n = 0; n < (long)NN; ++n) {
            long i, j, k;
            s.nodeIdx(n, i, j, k);
            double f[3];
            for (int c = 0; c < 3; ++c) f[c] = ZeroInit ? 0.0 : res[c * NN + n];
            for (int o = 0; o < 27; ++o) {
                long ni = i + o / 9 - 1, nj = j + (o / 3) % 3 - 1, nk = k + o % 3 - 1;
                if (ni < 0 || nj < 0 || nk < 0 || ni >= s.nn[0] || nj >= s.nn[1] || nk >= s.nn[2]) continue;
                size_t m = s.node(ni, nj, nk);
                const double *blk = &B[n * 243 + o * 9];
                for (int r = 0; r < 3; ++r) {
                    double v = blk[3 * r] * u[m] + blk[3 * r + 1] * u[NN + m] + blk[3 * r + 2] * u[2 * NN + m];
                    f[r] += Negate ? -v : v;
                }
            }
            for (int c = 0; c < 3; ++c) res[c * NN + n] = f[c];
        }
        return;
    }
    applyK_cached<ZeroInit, Negate>(s, u, res);
}

void zeroDirichlet(const Sim &s, double *u) {
    for (size_t n = 0; n < s.NN; ++n)
        if (s.dmask[n])
            for (int c = 0; c < 3; ++c)
                if (s.dmask[n] >> c & 1) u[c * s.NN + n] = 0.0;
}

void enforceDirichlet(const Sim &s, double *u, bool zero) {
    for (size_t n = 0; n < s.NN; ++n)
        if (s.dmask[n])
            for (int c = 0; c < 3; ++c)
                if (s.dmask[n] >> c & 1) u[c * s.NN + n] = zero ? 0.0 : s.dval[c * s.NN + n];
}

// MultigridSolver.hh:527-541
void computeResidual(MG &mg, int l, const double *u, const double *bb, double *res) {
    Sim &s = mg.sim(l);
    const size_t NN = s.NN;
    const long h = std::min<long>(std::min<long>(s.firstDetN, s.nn[1]) + MARGIN, s.nn[1]);
    for (long i = 0; i < s.nn[0]; ++i)
        for (long j = 0; j < h; ++j)
            for (long k = 0; k < s.nn[2]; ++k)
                for (int c = 0; c < 3; ++c) {
                    size_t n = s.node(i, j, k);
                    res[c * NN + n] = bb[c * NN + n];
                }
    applyK_level<false, true>(mg, l, u, res);
    zeroDirichlet(s, res);
}

// 3x3 inverse via the adjugate
void inv3(const double *M, double *Mi) {
    double c00 = M[4] * M[8] - M[5] * M[7];
    double c01 = M[5] * M[6] - M[3] * M[8];
    double c02 = M[3] * M[7] - M[4] * M[6];
    double det = M[0] * c00 + M[1] * c01 + M[2] * c02;
    double id = 1.0 / det;
    Mi[0] = c00 * id;
    Mi[1] = (M[2] * M[7] - M[1] * M[8]) * id;
    Mi[2] = (M[1] * M[5] - M[2] * M[4]) * id;
    Mi[3] = c01 * id;
    Mi[4] = (M[0] * M[8] - M[2] * M[6]) * id;
    Mi[5] = (M[2] * M[3] - M[0] * M[5]) * id;
    Mi[6] = c02 * id;
    Mi[7] = (M[1] * M[6] - M[0] * M[7]) * id;
    Mi[8] = (M[0] * M[4] - M[1] * M[3]) * id;
}

// m_smoothNode (MultigridSolver.hh:348-378): block GS, pointwise GS on partial Dirichlet nodes
inline void smoothNodeSolve(uint8_t dm, const double *bms, const double *M, double *un, bool forward) {
    if (dm) {
        double ud[3] = {0, 0, 0};
        if (forward) {
            for (int i = 0; i < 3; ++i)
                ud[i] = (bms[i] - (M[3 * i] * ud[0] + M[3 * i + 1] * ud[1] + M[3 * i + 2] * ud[2])) *
                        ((double)!(dm >> i & 1) / M[4 * i]);
        } else {
            for (int i = 2; i >= 0; --i)
                ud[i] = (bms[i] - (M[3 * i] * ud[0] + M[3 * i + 1] * ud[1] + M[3 * i + 2] * ud[2])) *
                        ((double)!(dm >> i & 1) / M[4 * i]);
        }
        for (int c = 0; c < 3; ++c) un[c] += ud[c];
    } else {
        double Mi[9];
        inv3(M, Mi);
        for (int r = 0; r < 3; ++r) un[r] += Mi[3 * r] * bms[0] + Mi[3 * r + 1] * bms[1] + Mi[3 * r + 2] * bms[2];
    }
}

// smoothingMulticoloredGS + visitNodesMulticolored (MultigridSolver.hh:409-458) with the
// Finest (:277-292), SecondFinest (:294-321) and BlockK (:323-334) node stencils.
void smoothGS(MG &mg, int l, double *u, const double *bb, bool forward) {
    Sim &s = mg.sim(l);
    const size_t NN = s.NN;
    const long nyv = s.nondetNodes();
    Sim &f0 = mg.sim(0);
    for (int ci = 0; ci < 8; ++ci) {
        const int col = forward ? ci : 7 - ci;
        const long o[3] = {col >> 2 & 1, col >> 1 & 1, col & 1};
#pragma omp parallel for schedule(static)
        for (long i = o[0]; i < s.nn[0]; i += 2)
            for (long j = o[1]; j < nyv; j += 2)
                for (long k = o[2]; k < s.nn[2]; k += 2) {
                    const size_t n = s.node(i, j, k);
                    const uint8_t dm = s.dmask[n];
                    if (dm == 7) continue;
                    double bms[3] = {bb[n], bb[NN + n], bb[2 * NN + n]};
                    double M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                    if (l >= 2) {
                        const double *row = &mg.blockK[l][n * 243];
                        for (int oo = 0; oo < 27; ++oo) {
                            long ni = i + oo / 9 - 1, nj = j + (oo / 3) % 3 - 1, nk = k + oo % 3 - 1;
                            if (ni < 0 || nj < 0 || nk < 0 || ni >= s.nn[0] || nj >= s.nn[1] || nk >= s.nn[2]) continue;
                            size_t m = s.node(ni, nj, nk);
                            const double *blk = row + oo * 9;
                            for (int r = 0; r < 3; ++r)
                                bms[r] -= blk[3 * r] * u[m] + blk[3 * r + 1] * u[NN + m] + blk[3 * r + 2] * u[2 * NN + m];
                            if (oo == 13)
                                for (int t = 0; t < 9; ++t) M[t] = blk[t];
                        }
                    } else {
                        // incident element order of elementsAdjacentNode (TPSStencils.hh:47-73)
                        for (int inc = 0; inc < 8; ++inc) {
                            const int a = !(inc & 1), b = !(inc & 2), c = !(inc & 4);
                            const long ei = i - a, ej = j - b, ek = k - c;
                            if (ei < 0 || ej < 0 || ek < 0 || ei >= s.ne[0] || ej >= s.ne[1] || ek >= s.ne[2]) continue;
                            const int ln = 4 * a + 2 * b + c;
                            double ue[24];
                            for (int m = 0; m < 8; ++m) {
                                size_t nm = s.node(ei + (m >> 2 & 1), ej + (m >> 1 & 1), ek + (m & 1));
                                for (int cc = 0; cc < 3; ++cc) ue[3 * m + cc] = u[cc * NN + nm];
                            }
                            if (l == 0) {
                                const double E = s.Y[s.elem(ei, ej, ek)];
                                for (int r = 0; r < 3; ++r) {
                                    double acc = 0;
                                    for (int t = 0; t < 24; ++t) acc += s.K0[t * 24 + 3 * ln + r] * ue[t];
                                    bms[r] -= E * acc;
                                }
                                for (int t = 0; t < 9; ++t) M[t] += E * s.K0diag[ln][t];
                            } else {
                                double cols[24 * 3];
                                int fi = 0;
                                for (int fa = 0; fa < 2; ++fa)
                                    for (int fb = 0; fb < 2; ++fb)
                                        for (int fc = 0; fc < 2; ++fc) {
                                            double E = f0.Y[f0.elem(2 * ei + fa, 2 * ej + fb, 2 * ek + fc)];
                                            for (int t = 0; t < 24; ++t)
                                                for (int r = 0; r < 3; ++r) {
                                                    double v = E * mg.Kc[fi][t * 24 + 3 * ln + r];
                                                    cols[t * 3 + r] = (fi == 0) ? v : cols[t * 3 + r] + v;
                                                }
                                            ++fi;
                                        }
                                for (int r = 0; r < 3; ++r) {
                                    double acc = 0;
                                    for (int t = 0; t < 24; ++t) acc += cols[t * 3 + r] * ue[t];
                                    bms[r] -= acc;
                                }
                                for (int r = 0; r < 3; ++r)
                                    for (int cc = 0; cc < 3; ++cc) M[3 * r + cc] += cols[(3 * ln + r) * 3 + cc];
                            }
                        }
                    }
                    double un[3] = {u[n], u[NN + n], u[2 * NN + n]};
                    smoothNodeSolve(dm, bms, M, un, forward);
                    u[n] = un[0]; u[NN + n] = un[1]; u[2 * NN + n] = un[2];
                }
    }
}

// MultigridSolver.hh:217-275
void restriction(MG &mg, int l, const double *vals, double *res) {
    Sim &fs = mg.sim(l), &cs = mg.sim(l + 1);
    const long cyv = cs.nondetNodes(), fyv = fs.nondetNodes();
    const size_t FN = fs.NN, CN = cs.NN;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < cs.nn[0]; ++i)
        for (long j = 0; j < cyv; ++j)
            for (long k = 0; k < cs.nn[2]; ++k) {
                double v[3] = {0, 0, 0};
                long lo[3] = {std::max(2 * i - 1, 0L), std::max(2 * j - 1, 0L), std::max(2 * k - 1, 0L)};
                long hi[3] = {std::min(2 * i + 2, fs.nn[0]), std::min(2 * j + 2, fyv), std::min(2 * k + 2, fs.nn[2])};
                for (long a = lo[0]; a < hi[0]; ++a)
                    for (long b = lo[1]; b < hi[1]; ++b)
                        for (long c = lo[2]; c < hi[2]; ++c) {
                            double w = (1 - std::abs(a - 2 * i) * 0.5) * (1 - std::abs(b - 2 * j) * 0.5) *
                                       (1 - std::abs(c - 2 * k) * 0.5);
                            size_t fn = fs.node(a, b, c);
                            for (int d = 0; d < 3; ++d) v[d] += w * vals[d * FN + fn];
                        }
                size_t cn = cs.node(i, j, k);
                for (int d = 0; d < 3; ++d) res[d * CN + cn] = v[d];
            }
    if (cyv != cs.nn[1]) {
        for (long i = 0; i < cs.nn[0]; ++i)
            for (long k = 0; k < cs.nn[2]; ++k)
                for (int d = 0; d < 3; ++d) res[d * CN + cs.node(i, cyv, k)] = 0.0;
    }
}

// MultigridSolver.hh:163-212 (accumulate=true: accum_interpolation; else interpolation)
void interpolate(MG &mg, int l, const double *cvals, double *out, bool accumulate) {
    Sim &fs = mg.sim(l), &cs = mg.sim(l + 1);
    const size_t FN = fs.NN, CN = cs.NN;
    const long fyv = accumulate ? fs.nondetNodes() : fs.nn[1];
#pragma omp parallel for schedule(static)
    for (long i = 0; i < fs.nn[0]; ++i)
        for (long j = 0; j < fyv; ++j)
            for (long k = 0; k < fs.nn[2]; ++k) {
                long f[3] = {i, j, k}, ec[3], lf[3];
                for (int d = 0; d < 3; ++d) {
                    ec[d] = std::min(f[d] / 2, cs.ne[d]);
                    lf[d] = f[d] - 2 * ec[d];
                }
                double acc[3] = {0, 0, 0};
                size_t fn = fs.node(i, j, k);
                if (accumulate)
                    for (int d = 0; d < 3; ++d) acc[d] = out[d * FN + fn];
                for (int cn = 0; cn < 8; ++cn) {
                    int cb[3] = {cn >> 2 & 1, cn >> 1 & 1, cn & 1};
                    double coeff = 1;
                    for (int d = 0; d < 3; ++d) {
                        double phi = (lf[d] == 1) ? 0.5 : ((lf[d] == 0) ? (cb[d] ? 0.0 : 1.0) : (cb[d] ? 1.0 : 0.0));
                        coeff *= phi;
                    }
                    if (coeff == 0) continue;
                    size_t cidx = cs.node(ec[0] + cb[0], ec[1] + cb[1], ec[2] + cb[2]);
                    for (int d = 0; d < 3; ++d) acc[d] += coeff * cvals[d * CN + cidx];
                }
                for (int d = 0; d < 3; ++d) out[d * FN + fn] = acc[d];
            }
}

void maskedSetZero(const Sim &s, double *u, int margin) {
    const long h = std::min<long>(std::min<long>(s.firstDetN, s.nn[1]) + margin, s.nn[1]);
    for (long i = 0; i < s.nn[0]; ++i)
        for (long j = 0; j < h; ++j)
            for (long k = 0; k < s.nn[2]; ++k)
                for (int c = 0; c < 3; ++c) u[c * s.NN + s.node(i, j, k)] = 0.0;
}

// MultigridSolver.hh:617-658
void vcycle(MG &mg, int l, long sweeps, bool residualSystem) {
    const int coarsest = mg.L() - 1;
    if (l == coarsest) { coarseSolve(mg, mg.b[l].data(), mg.x[l].data()); return; }
    Sim &s = mg.sim(l);
    enforceDirichlet(s, mg.x[l].data(), residualSystem);
    for (long t = 0; t < sweeps; ++t) smoothGS(mg, l, mg.x[l].data(), mg.b[l].data(), true);
    computeResidual(mg, l, mg.x[l].data(), mg.b[l].data(), mg.r[l].data());
    restriction(mg, l, mg.r[l].data(), mg.b[l + 1].data());
    maskedSetZero(mg.sim(l + 1), mg.x[l + 1].data(), MARGIN);
    vcycle(mg, l + 1, sweeps, true);
    interpolate(mg, l, mg.x[l + 1].data(), mg.x[l].data(), true);
    for (long t = 0; t < sweeps; ++t) smoothGS(mg, l, mg.x[l].data(), mg.b[l].data(), !mg.symmetricGS);
}

// MultigridSolver.hh:587-609
void fullMultigrid(MG &mg, int l, long sweeps, bool residualSystem) {
    const int coarsest = mg.L() - 1;
    if (l == coarsest) { coarseSolve(mg, mg.b[l].data(), mg.x[l].data()); return; }
    restriction(mg, l, mg.b[l].data(), mg.b[l + 1].data());
    fullMultigrid(mg, l + 1, sweeps, residualSystem);
    interpolate(mg, l, mg.x[l + 1].data(), mg.x[l].data(), false);
    vcycle(mg, l, sweeps, residualSystem);
}

// MultigridSolver.hh:547-573
void mgSolve(MG &mg, const double *u0, const double *f, long steps, long sweeps, bool zeroDirichlet, bool fmg) {
    const size_t n3 = 3 * mg.sim(0).NN;
    std::copy(u0, u0 + n3, mg.x[0].begin());
    if (steps == 0) return;
    if (f != mg.b[0].data()) std::copy(f, f + n3, mg.b[0].begin());
    if (fmg) {
        fullMultigrid(mg, 0, sweeps, zeroDirichlet);
        for (long i = 1; i < steps; ++i) vcycle(mg, 0, sweeps, zeroDirichlet);
    } else {
        for (long i = 0; i < steps; ++i) vcycle(mg, 0, sweeps, zeroDirichlet);
    }
}

double maskedDot(const Sim &s, const double *a, const double *b) {
    const long h = s.nondetNodes();
    const size_t blk = (size_t)h * s.nn[2];
    std::vector<double> part(s.nn[0], 0.0);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < s.nn[0]; ++i) {
        double acc = 0;
        const size_t st = s.node(i, 0, 0);
        for (int c = 0; c < 3; ++c)
            for (size_t t = 0; t < blk; ++t) acc += a[c * s.NN + st + t] * b[c * s.NN + st + t];
        part[i] = acc;
    }
    double tot = 0;
    for (double p : part) tot += p;
    return tot;
}

template <class F>
void maskedVisit(const Sim &s, int margin, F &&f) {
    const long h = std::min<long>(std::min<long>(s.firstDetN, s.nn[1]) + margin, s.nn[1]);
    const size_t blk = (size_t)h * s.nn[2];
#pragma omp parallel for schedule(static)
    for (long i = 0; i < s.nn[0]; ++i) f(s.node(i, 0, 0), blk);
}

// MultigridSolver.hh:1047-1152
int pcg(MG &mg, double *x, const double *bvec, long maxIter, double tol, long mgIter, long sweeps, bool fmg,
        bool dirichletSatisfied, long *itersOut, double *relresOut, void (*cb)(long, double)) {
    Sim &fs = mg.sim(0);
    const size_t NN = fs.NN, n3 = 3 * NN;
    if (mg.L() == 1) throw std::runtime_error("numCoarseningLevels == 0 is not supported by the oracle");
    std::vector<double> &r = mg.b[0];
    std::vector<double> &s = mg.x[0];
    mg.Ad.resize(n3);
    mg.dvec.resize(n3);
    if (!dirichletSatisfied) enforceDirichlet(fs, x, false);
    const double bnorm2 = maskedDot(fs, bvec, bvec);
    computeResidual(mg, 0, x, bvec, r.data());
    double rsq = maskedDot(fs, r.data(), r.data());
    if (std::isnan(rsq)) throw std::logic_error("NaN encountered");
    double rMr = 0;
    bool updated = false;
    long i = 0;
    double *d = nullptr;
    while ((i++ < maxIter) && (rsq > tol * tol * bnorm2)) {
        if (mgIter > 0) {
            if (!updated) { updateStiffness(mg); updated = true; }
            if (d == s.data()) {
                d = mg.dvec.data();
                maskedVisit(fs, MARGIN, [&](size_t st, size_t blk) {
                    for (int c = 0; c < 3; ++c) std::copy(s.begin() + c * NN + st, s.begin() + c * NN + st + blk, d + c * NN + st);
                });
            }
            if (sweeps != 0) {
                std::vector<double> zero(n3, 0.0);
                mgSolve(mg, zero.data(), r.data(), mgIter, sweeps, true, fmg);
            }
        } else {
            std::copy(r.begin(), r.end(), s.begin());
        }
        zeroDirichlet(fs, s.data());
        const double old = rMr;
        rMr = maskedDot(fs, r.data(), s.data());
        if (d) {
            const double beta = rMr / old;
#pragma omp parallel for schedule(static)
            for (long t = 0; t < (long)n3; ++t) d[t] = beta * d[t] + s[t];
        } else {
            d = s.data();
        }
        applyK_level<true, false>(mg, 0, d, mg.Ad.data());
        zeroDirichlet(fs, mg.Ad.data());
        const double alpha = rMr / maskedDot(fs, d, mg.Ad.data());
        maskedVisit(fs, 0, [&](size_t st, size_t blk) {
            for (int c = 0; c < 3; ++c)
                for (size_t t = 0; t < blk; ++t) x[c * NN + st + t] += alpha * d[c * NN + st + t];
        });
        maskedVisit(fs, 0, [&](size_t st, size_t blk) {
            for (int c = 0; c < 3; ++c)
                for (size_t t = 0; t < blk; ++t) r[c * NN + st + t] -= alpha * mg.Ad[c * NN + st + t];
        });
        rsq = maskedDot(fs, r.data(), r.data());
        if (std::isnan(rsq)) throw std::logic_error("NaN encountered at iteration" + std::to_string(i));
        if (cb) cb(i, std::sqrt(rsq));
    }
    if (itersOut) *itersOut = std::min(i, maxIter + 1) - 1;
    if (relresOut) *relresOut = bnorm2 > 0 ? std::sqrt(rsq / bnorm2) : std::sqrt(rsq);
    return 0;
}

// ---------------------------------------------------------------------------
// Filters (TopologyOptimizationFilter.hh:189-245, 285-400) and the volume
// constraint (TopologyOptimizationConstraint.hh:24-40).
// ---------------------------------------------------------------------------
inline long reflectIndex(long i, long s) {
    while (i < 0 || i >= s) {
        if (i >= s) i = 2 * s - i - 1;
        if (i < 0) i = -i - 1;
    }
    return i;
}

void smoothingFilter(const long dims[3], int radius, int type, const double *in, double *out) {
    const double rp1 = 1.0 + radius;
    std::vector<std::array<long, 3>> offs;
    std::vector<double> ws;
    double W = 0;
    for (long a = -radius; a <= radius; ++a)
        for (long b = -radius; b <= radius; ++b)
            for (long c = -radius; c <= radius; ++c) {
                double w = type == 1 ? rp1 - std::sqrt((double)(a * a + b * b + c * c)) : 1.0;
                if (w <= 0) continue;
                offs.push_back({a, b, c});
                ws.push_back(w);
                W += w;
            }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < dims[0]; ++i)
        for (long j = 0; j < dims[1]; ++j)
            for (long k = 0; k < dims[2]; ++k) {
                double acc = 0;
                for (size_t t = 0; t < offs.size(); ++t) {
                    long ni = reflectIndex(i + offs[t][0], dims[0]);
                    long nj = reflectIndex(j + offs[t][1], dims[1]);
                    long nk = reflectIndex(k + offs[t][2], dims[2]);
                    acc += ws[t] * in[(ni * dims[1] + nj) * dims[2] + nk];
                }
                out[(i * dims[1] + j) * dims[2] + k] = acc / W;
            }
}

void projectionApply(long n, double beta, const double *in, double *out) {
    const double th = std::tanh(0.5 * beta);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) out[i] = (th + std::tanh(beta * (in[i] - 0.5))) / (2 * th);
}

void projectionBackprop(long n, double beta, const double *in, const double *vars, double *out) {
    const double scale = 1.0 / (2 * std::tanh(0.5 * beta) / beta);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
        const double t = std::tanh(beta * (vars[i] - 0.5));
        out[i] = in[i] * (1.0 - t * t) * scale;
    }
}

// ---------------------------------------------------------------------------
// Topology optimisation problem with MG compliance objective, a filter chain
// and one total-volume constraint (TopologyOptimizationProblem.hh:41-121,
// TopologyOptimizationObjective.hh:71-105), and the OC step
// (OptimalityCriterion.hh:51-138).
// ---------------------------------------------------------------------------
struct FilterSpec { int kind; int radius; int type; double beta; };  // kind 0 smoothing, 1 projection

struct TOP {
    MG *mg;
    std::vector<FilterSpec> filters;
    double volfrac;
    std::vector<std::vector<double>> vars;  // chain intermediates
    std::vector<double> f, u;
    long cgIter = 100;
    double tol = 1e-5;
    long mgIter = 1, mgSweeps = 2;
    bool fmg = true, zeroInit = false;
    bool varsSet = false;
    long lastIters = 0;
    double lambda_min = 1, lambda_max = 2;
};

void applyFilter(const TOP &t, const FilterSpec &fs, const double *in, double *out) {
    const Sim &s = *t.mg->sims[0];
    if (fs.kind == 0) smoothingFilter(s.ne, fs.radius, fs.type, in, out);
    else projectionApply((long)s.NE, fs.beta, in, out);
}

void backpropFilter(const TOP &t, const FilterSpec &fs, const double *in, const double *vars, double *out) {
    const Sim &s = *t.mg->sims[0];
    if (fs.kind == 0) smoothingFilter(s.ne, fs.radius, fs.type, in, out);
    else projectionBackprop((long)s.NE, fs.beta, in, vars, out);
}

void topSetVars(TOP &t, const double *x) {
    Sim &s = *t.mg->sims[0];
    const size_t ne = s.NE;
    t.vars.assign(t.filters.size() + 1, std::vector<double>(ne));
    std::copy(x, x + ne, t.vars[0].begin());
    for (size_t i = 0; i < t.filters.size(); ++i) applyFilter(t, t.filters[i], t.vars[i].data(), t.vars[i + 1].data());
    // MultigridComplianceObjective::updateCache
    for (size_t e = 0; e < ne; ++e) {
        double v = t.vars.back()[e];
        if (v > 1.0 || v < 0) throw std::runtime_error("Density value out of range");
    }
    s.rho = t.vars.back();
    updateY(s);
    if (t.zeroInit) std::fill(t.u.begin(), t.u.end(), 0.0);
    double rel;
    pcg(*t.mg, t.u.data(), t.f.data(), t.cgIter, t.tol, t.mgIter, t.mgSweeps, t.fmg, false, &t.lastIters, &rel, nullptr);
    t.varsSet = true;
}

void topBackprop(const TOP &t, std::vector<double> &g) {
    std::vector<double> scratch(g.size());
    for (size_t i = t.filters.size(); i-- > 0;) {
        backpropFilter(t, t.filters[i], g.data(), t.vars[i].data(), scratch.data());
        g.swap(scratch);
    }
}

double topObjective(const TOP &t) {
    const Sim &s = *t.mg->sims[0];
    double acc = 0;
    for (size_t i = 0; i < 3 * s.NN; ++i) acc += t.f[i] * t.u[i];
    return 0.5 * acc;
}

void topGradient(TOP &t, double *out) {
    const Sim &s = *t.mg->sims[0];
    std::vector<double> g(s.NE);
    complianceGradient(s, t.u.data(), g.data());
    topBackprop(t, g);
    std::copy(g.begin(), g.end(), out);
}

double topConstraint(const TOP &t) {
    const std::vector<double> &x = t.vars.back();
    double m = 0;
    for (double v : x) m += v;
    m /= (double)x.size();
    return 1.0 - m / t.volfrac;
}

void topJacobian(TOP &t, double *out) {
    const Sim &s = *t.mg->sims[0];
    std::vector<double> g(s.NE, -1.0 / (t.volfrac * (double)s.NE));
    topBackprop(t, g);
    std::copy(g.begin(), g.end(), out);
}

double topConstraintAtVars(const TOP &t, std::vector<double> &x) {
    std::vector<double> scratch(x.size());
    for (const auto &fs : t.filters) {
        applyFilter(t, fs, x.data(), scratch.data());
        x.swap(scratch);
    }
    double m = 0;
    for (double v : x) m += v;
    m /= (double)x.size();
    return 1.0 - m / t.volfrac;
}

int ocStep(TOP &t, double m, double p, double ctol, long *probes) {
    const Sim &s = *t.mg->sims[0];
    const size_t n = s.NE;
    std::vector<double> dJ(n), dc(n);
    topGradient(t, dJ.data());
    topJacobian(t, dc.data());
    const std::vector<double> x0 = t.vars[0];
    std::vector<double> stepped(n), tmp;
    long nprobe = 0;
    auto ceval = [&](double lambda) {
        ++nprobe;
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)n; ++i) {
            double res = x0[i] * std::pow(dJ[i] / (dc[i] * lambda), p);
            res = std::min(std::max(std::min(std::max(res, x0[i] - m), x0[i] + m), 0.0), 1.0);
            if (!std::isfinite(res)) res = x0[i];
            stepped[i] = res;
        }
        tmp = stepped;
        return topConstraintAtVars(t, tmp);
    };
    const double dilation = 32;
    const long guard = 100;
    double lmid = 0.5 * (t.lambda_min + t.lambda_max);
    t.lambda_max = dilation * t.lambda_max + (1 - dilation) * lmid;
    t.lambda_min = std::max(dilation * t.lambda_min + (1 - dilation) * lmid, 0.01);
    long nit = 0;
    for (; nit < guard; ++nit) {
        if (ceval(t.lambda_min) < 0) break;
        t.lambda_max = t.lambda_min;
        t.lambda_min /= 2;
    }
    if (nit == guard) throw std::runtime_error("Bracketing constraint(lambda_min) < 0 failed");
    if (nit == 0)
        for (; nit < guard; ++nit) {
            if (ceval(t.lambda_max) > 0) break;
            t.lambda_min = t.lambda_max;
            t.lambda_max *= 2;
        }
    if (nit == guard) throw std::runtime_error("Bracketing constraint(lambda_max) > 0 failed");
    double viol;
    do {
        lmid = 0.5 * (t.lambda_min + t.lambda_max);
        viol = ceval(lmid);
        if (std::abs(viol) <= ctol) break;
        ++nit;
        if (viol < 0) t.lambda_min = lmid;
        if (viol > 0) t.lambda_max = lmid;
    } while (true);
    if (probes) *probes = nprobe;
    topSetVars(t, stepped.data());
    return 0;
}

template <class F>
int guarded(F &&f) {
    try {
        f();
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return 1;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// C interface used by the tests and by the benchmark's CPU baseline leg.
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// Triquadratic voxels (TensorProductSimulator<double, 2, 2, 2>).
// K0: TensorProductSimulator.hh:54-80 with TensorProductQuadrature<(2 * 2)...> (3 Gauss points
// per axis); local node l = 9a + 3b + c (NDArrayIndexer flattening, last index fastest).
// applyK: element loop (TPSStencils.hh:135-186 gathers per node; summing element products is
// the same operator). Smoother: visitNodesMulticolored with 27 colours (MultigridSolver.hh:
// 409-442) and the Finest node stencil (:277-292). Transfers: phis / interpolation /
// restriction (MultigridSolver.hh:137-275) as tensor products of 1-D Q2 interpolation matrices.
// ---------------------------------------------------------------------------
struct Q2Grid {
    long ne[3], nn[3];
    size_t NN, NE;
    size_t node(long I, long J, long K) const { return ((size_t)I * nn[1] + J) * nn[2] + K; }
    size_t elem(long i, long j, long k) const { return ((size_t)i * ne[1] + j) * ne[2] + k; }
};

Q2Grid q2grid(const long ne[3]) {
    Q2Grid g;
    for (int d = 0; d < 3; ++d) {
        g.ne[d] = ne[d];
        g.nn[d] = 2 * ne[d] + 1;
    }
    g.NN = (size_t)g.nn[0] * g.nn[1] * g.nn[2];
    g.NE = (size_t)ne[0] * ne[1] * ne[2];
    return g;
}

// Lagrange basis on the equispaced nodes {0, 1/2, 1}: value and derivative of basis a at x
double lag2(int a, double x) {
    const double xs[3] = {0.0, 0.5, 1.0};
    double v = 1.0;
    for (int m = 0; m < 3; ++m)
        if (m != a) v *= (x - xs[m]) / (xs[a] - xs[m]);
    return v;
}
double lag2d(int a, double x) {
    const double xs[3] = {0.0, 0.5, 1.0};
    double acc = 0.0;
    for (int m = 0; m < 3; ++m) {
        if (m == a) continue;
        double t = 1.0 / (xs[a] - xs[m]);
        for (int p = 0; p < 3; ++p)
            if (p != a && p != m) t *= (x - xs[p]) / (xs[a] - xs[p]);
        acc += t;
    }
    return acc;
}

// Gauss-Legendre points and weights on [0, 1] (n = 3 or 4)
void gauss01(int n, double *x, double *w) {
    if (n == 3) {
        const double r = std::sqrt(0.6);
        const double xm[3] = {-r, 0.0, r}, wm[3] = {5.0 / 9, 8.0 / 9, 5.0 / 9};
        for (int i = 0; i < 3; ++i) { x[i] = 0.5 * (xm[i] + 1); w[i] = 0.5 * wm[i]; }
    } else if (n == 4) {
        const double a = std::sqrt(3.0 / 7 - 2.0 / 7 * std::sqrt(6.0 / 5)), b = std::sqrt(3.0 / 7 + 2.0 / 7 * std::sqrt(6.0 / 5));
        const double wa = (18 + std::sqrt(30.0)) / 36, wb = (18 - std::sqrt(30.0)) / 36;
        const double xm[4] = {-b, -a, a, b}, wm[4] = {wb, wa, wa, wb};
        for (int i = 0; i < 4; ++i) { x[i] = 0.5 * (xm[i] + 1); w[i] = 0.5 * wm[i]; }
    } else {
        throw std::runtime_error("unsupported quadrature order");
    }
}

void q2K0(double E, double nu, const double h[3], int npts, double *K) {
    const double lam = E * nu / ((1 + nu) * (1 - 2 * nu)), mu = E / (2 * (1 + nu));
    double gx[4], gw[4];
    gauss01(npts, gx, gw);
    std::fill(K, K + 6561, 0.0);
    for (int qa = 0; qa < npts; ++qa)
        for (int qb = 0; qb < npts; ++qb)
            for (int qc = 0; qc < npts; ++qc) {
                const double p[3] = {gx[qa], gx[qb], gx[qc]};
                const double w = gw[qa] * gw[qb] * gw[qc] * h[0] * h[1] * h[2];
                double G[27][3];
                for (int l = 0; l < 27; ++l) {
                    const int id[3] = {l / 9, (l / 3) % 3, l % 3};
                    for (int d = 0; d < 3; ++d) {
                        double g = 1.0;
                        for (int e = 0; e < 3; ++e) g *= (e == d) ? lag2d(id[e], p[e]) / h[e] : lag2(id[e], p[e]);
                        G[l][d] = g;
                    }
                }
                // eps(phi_{l,c}) = sym(e_c (x) grad N_l); sigma = lam tr(eps) I + 2 mu eps
                for (int i = 0; i < 81; ++i) {
                    const int li = i / 3, ci = i % 3;
                    for (int j = 0; j < 81; ++j) {
                        const int lj = j / 3, cj = j % 3;
                        double epsIepsJ = 0.5 * G[li][cj] * G[lj][ci];
                        if (ci == cj) epsIepsJ += 0.5 * (G[li][0] * G[lj][0] + G[li][1] * G[lj][1] + G[li][2] * G[lj][2]);
                        K[i * 81 + j] += w * (lam * G[li][ci] * G[lj][cj] + 2 * mu * epsIepsJ);
                    }
                }
            }
}

void q2ApplyK(const Q2Grid &g, const double *K, const double *Y, const double *u, double *out) {
    std::fill(out, out + 3 * g.NN, 0.0);
    // element layers of one x parity share no node: each parity's layers run in parallel
    for (int parity = 0; parity < 2; ++parity)
#pragma omp parallel for schedule(dynamic, 1)
    for (long i = parity; i < g.ne[0]; i += 2)
        for (long j = 0; j < g.ne[1]; ++j)
            for (long k = 0; k < g.ne[2]; ++k) {
                size_t nodes[27];
                double ue[81], fe[81];
                for (int l = 0; l < 27; ++l) {
                    nodes[l] = g.node(2 * i + l / 9, 2 * j + (l / 3) % 3, 2 * k + l % 3);
                    for (int c = 0; c < 3; ++c) ue[3 * l + c] = u[c * g.NN + nodes[l]];
                }
                const double E = Y[g.elem(i, j, k)];
                for (int r = 0; r < 81; ++r) {
                    double acc = 0.0;
                    for (int t = 0; t < 81; ++t) acc += K[r * 81 + t] * ue[t];
                    fe[r] = E * acc;
                }
                for (int l = 0; l < 27; ++l)
                    for (int c = 0; c < 3; ++c) out[c * g.NN + nodes[l]] += fe[3 * l + c];
            }
}

void q2Smooth(const Q2Grid &g, const double *K, const double *Y, const uint8_t *dmask, double *u, const double *b,
              bool forward) {
    for (int ci = 0; ci < 27; ++ci) {
        const int col = forward ? ci : 26 - ci;
        const long lo[3] = {col / 9, (col / 3) % 3, col % 3};
        long inc[3];
        for (int d = 0; d < 3; ++d) inc[d] = (lo[d] == 1) ? 2 : 4;
        for (long I = lo[0]; I < g.nn[0]; I += inc[0])
            for (long J = lo[1]; J < g.nn[1]; J += inc[1])
                for (long Kk = lo[2]; Kk < g.nn[2]; Kk += inc[2]) {
                    const size_t n = g.node(I, J, Kk);
                    const uint8_t dm = dmask[n];
                    if (dm == 7) continue;
                    double bms[3] = {b[n], b[g.NN + n], b[2 * g.NN + n]};
                    double M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                    // incident elements: per axis, corner nodes (even) lie in elements I/2 - 1 and I/2
                    const long P[3] = {I, J, Kk};
                    long el[3][2], ll[3][2];
                    int cnt[3];
                    for (int d = 0; d < 3; ++d) {
                        cnt[d] = 0;
                        if (P[d] % 2) { el[d][0] = (P[d] - 1) / 2; ll[d][0] = 1; cnt[d] = 1; }
                        else {
                            if (P[d] / 2 - 1 >= 0) { el[d][cnt[d]] = P[d] / 2 - 1; ll[d][cnt[d]] = 2; ++cnt[d]; }
                            if (P[d] / 2 < g.ne[d]) { el[d][cnt[d]] = P[d] / 2; ll[d][cnt[d]] = 0; ++cnt[d]; }
                        }
                    }
                    for (int a = 0; a < cnt[0]; ++a)
                        for (int bb = 0; bb < cnt[1]; ++bb)
                            for (int c = 0; c < cnt[2]; ++c) {
                                const long ei = el[0][a], ej = el[1][bb], ek = el[2][c];
                                const int ln = 9 * ll[0][a] + 3 * ll[1][bb] + ll[2][c];
                                const double E = Y[g.elem(ei, ej, ek)];
                                for (int r = 0; r < 3; ++r) {
                                    double acc = 0.0;
                                    for (int m = 0; m < 27; ++m) {
                                        const size_t nm = g.node(2 * ei + m / 9, 2 * ej + (m / 3) % 3, 2 * ek + m % 3);
                                        for (int cc = 0; cc < 3; ++cc) acc += K[(3 * ln + r) * 81 + 3 * m + cc] * u[cc * g.NN + nm];
                                    }
                                    bms[r] -= E * acc;
                                    for (int cc = 0; cc < 3; ++cc) M[3 * r + cc] += E * K[(3 * ln + r) * 81 + 3 * ln + cc];
                                }
                            }
                    double un[3] = {u[n], u[g.NN + n], u[2 * g.NN + n]};
                    smoothNodeSolve(dm, bms, M, un, forward);
                    for (int c = 0; c < 3; ++c) u[c * g.NN + n] = un[c];
                }
    }
}

// 1-D Q2 prolongation (fine nodes 0..4 nec) x (coarse nodes 0..2 nec), dense
std::vector<double> q2P1d(long nec) {
    const long nf = 4 * nec + 1, nc = 2 * nec + 1;
    std::vector<double> P((size_t)nf * nc, 0.0);
    for (long f = 0; f < nf; ++f) {
        const long e = std::min(f / 4, nec - 1);
        const double x = (f - 4.0 * e) / 4.0;
        for (int a = 0; a < 3; ++a) P[(size_t)f * nc + 2 * e + a] = lag2(a, x);
    }
    return P;
}

void q2Interp(const long neF[3], const double *coarse, double *fine, bool accumulate) {
    const long nec[3] = {neF[0] / 2, neF[1] / 2, neF[2] / 2};
    std::vector<double> P[3] = {q2P1d(nec[0]), q2P1d(nec[1]), q2P1d(nec[2])};
    const long nf[3] = {2 * neF[0] + 1, 2 * neF[1] + 1, 2 * neF[2] + 1}, nc[3] = {2 * nec[0] + 1, 2 * nec[1] + 1, 2 * nec[2] + 1};
    const size_t NF = (size_t)nf[0] * nf[1] * nf[2], NC = (size_t)nc[0] * nc[1] * nc[2];
    for (long I = 0; I < nf[0]; ++I)
        for (long J = 0; J < nf[1]; ++J)
            for (long K = 0; K < nf[2]; ++K) {
                double acc[3] = {0, 0, 0};
                for (long a = 0; a < nc[0]; ++a) {
                    const double wa = P[0][(size_t)I * nc[0] + a];
                    if (wa == 0.0) continue;
                    for (long b = 0; b < nc[1]; ++b) {
                        const double wb = P[1][(size_t)J * nc[1] + b];
                        if (wb == 0.0) continue;
                        for (long c = 0; c < nc[2]; ++c) {
                            const double wc = P[2][(size_t)K * nc[2] + c];
                            if (wc == 0.0) continue;
                            const size_t cn = ((size_t)a * nc[1] + b) * nc[2] + c;
                            for (int r = 0; r < 3; ++r) acc[r] += wa * wb * wc * coarse[r * NC + cn];
                        }
                    }
                }
                const size_t fn = ((size_t)I * nf[1] + J) * nf[2] + K;
                for (int r = 0; r < 3; ++r) fine[r * NF + fn] = (accumulate ? fine[r * NF + fn] : 0.0) + acc[r];
            }
}

void q2Restrict(const long neF[3], const double *fine, double *coarse) {
    const long nec[3] = {neF[0] / 2, neF[1] / 2, neF[2] / 2};
    std::vector<double> P[3] = {q2P1d(nec[0]), q2P1d(nec[1]), q2P1d(nec[2])};
    const long nf[3] = {2 * neF[0] + 1, 2 * neF[1] + 1, 2 * neF[2] + 1}, nc[3] = {2 * nec[0] + 1, 2 * nec[1] + 1, 2 * nec[2] + 1};
    const size_t NF = (size_t)nf[0] * nf[1] * nf[2], NC = (size_t)nc[0] * nc[1] * nc[2];
    std::fill(coarse, coarse + 3 * NC, 0.0);
    for (long I = 0; I < nf[0]; ++I)
        for (long J = 0; J < nf[1]; ++J)
            for (long K = 0; K < nf[2]; ++K) {
                const size_t fn = ((size_t)I * nf[1] + J) * nf[2] + K;
                for (long a = 0; a < nc[0]; ++a) {
                    const double wa = P[0][(size_t)I * nc[0] + a];
                    if (wa == 0.0) continue;
                    for (long b = 0; b < nc[1]; ++b) {
                        const double wb = P[1][(size_t)J * nc[1] + b];
                        if (wb == 0.0) continue;
                        for (long c = 0; c < nc[2]; ++c) {
                            const double wc = P[2][(size_t)K * nc[2] + c];
                            if (wc == 0.0) continue;
                            const size_t cn = ((size_t)a * nc[1] + b) * nc[2] + c;
                            for (int r = 0; r < 3; ++r) coarse[r * NC + cn] += wa * wb * wc * fine[r * NF + fn];
                        }
                    }
                }
            }
}

// ---------------------------------------------------------------------------
// Triquadratic multigrid hierarchy (MultigridSolver<double, 2, 2, 2>): every level is a Q2 mesh
// with half the elements of the one above (MultigridSolver.hh:35-121). Level 1 applies the
// fine moduli to the 8 coarsened full-density element matrices (:294-321, :471-500, :724-738);
// levels 2 and below hold Galerkin element matrices I_f^T K_f I_f summed over the 8 children
// (:745-819), which the reference assembles into blockK (here they stay per element: the same
// operator); the coarsest level is solved directly on its free DOFs (TensorProductSimulator.hh:
// 1181-1230, dense Cholesky in place of CHOLMOD).
// ---------------------------------------------------------------------------

// phis[f](fine_n, coarse_n) (MultigridSolver.hh:664-687): coarse shape function coarse_n at
// fine node fine_n of child f = 4 fx + 2 fy + fz, whose local node (a, b, c) lies at coarse
// reference coordinates ((2 fx + a) / 4, (2 fy + b) / 4, (2 fz + c) / 4).
double q2Phi(int f, int fn, int cn) {
    const int fd[3] = {f >> 2 & 1, f >> 1 & 1, f & 1};
    const int fa[3] = {fn / 9, (fn / 3) % 3, fn % 3}, ca[3] = {cn / 9, (cn / 3) % 3, cn % 3};
    double v = 1.0;
    for (int d = 0; d < 3; ++d) v *= lag2(ca[d], (2.0 * fd[d] + fa[d]) / 4.0);
    return v;
}

// Kc += I_f^T Kf I_f with I_f[3i + c, 3j + d] = phi_f(i, j) delta_cd (MultigridSolver.hh:712-722)
void q2AccumulateCoarsened(int f, const double *Kf, double *Kc) {
    double phi[27 * 27];
    for (int i = 0; i < 27; ++i)
        for (int j = 0; j < 27; ++j) phi[i * 27 + j] = q2Phi(f, i, j);
    std::vector<double> T(6561);
    for (int r = 0; r < 81; ++r)
        for (int j = 0; j < 27; ++j)
            for (int d = 0; d < 3; ++d) {
                double acc = 0.0;
                for (int i = 0; i < 27; ++i) acc += Kf[r * 81 + 3 * i + d] * phi[i * 27 + j];
                T[r * 81 + 3 * j + d] = acc;
            }
    for (int j = 0; j < 27; ++j)
        for (int c = 0; c < 3; ++c)
            for (int q = 0; q < 81; ++q) {
                double acc = 0.0;
                for (int i = 0; i < 27; ++i) acc += phi[i * 27 + j] * T[(3 * i + c) * 81 + q];
                Kc[(3 * j + c) * 81 + q] += acc;
            }
}

struct Q2MG {
    std::vector<Q2Grid> g;                   // levels 0..L
    std::vector<std::vector<uint8_t>> dm;    // Dirichlet component bits per level
    std::vector<double> K0, Y;               // fine element matrix, fine moduli
    std::vector<double> Kc;                  // 8 x 6561 coarsened full-density matrices
    std::vector<std::vector<double>> Ke;     // level l >= 1: NE_l x 6561
    std::vector<std::vector<double>> x, b, r;
    DenseChol chol;
    bool symmetricGS = true;
    int L() const { return (int)g.size() - 1; }
};

// Dirichlet coarsening (MultigridSolver.hh:57-104): a constrained fine node marks every coarse
// node of the vertex, edge or face of its coarse element on which it lies (all nodes along an
// axis where it is interior), with the fine node's components.
void q2CoarsenDirichlet(const Q2Grid &F, const std::vector<uint8_t> &dmF, const Q2Grid &C, std::vector<uint8_t> &dmC) {
    dmC.assign(C.NN, 0);
    for (long I = 0; I < F.nn[0]; ++I)
        for (long J = 0; J < F.nn[1]; ++J)
            for (long K = 0; K < F.nn[2]; ++K) {
                const uint8_t m = dmF[F.node(I, J, K)];
                if (!m) continue;
                const long P[3] = {I, J, K};
                long ec[3], pb[3];
                for (int d = 0; d < 3; ++d) {
                    ec[d] = std::min(P[d] / 4, C.ne[d] - 1);
                    const long t = P[d] - 4 * ec[d];
                    pb[d] = t == 0 ? 0 : (t == 4 ? 2 : -1);
                }
                for (int ln = 0; ln < 27; ++ln) {
                    const long la[3] = {ln / 9, (ln / 3) % 3, ln % 3};
                    bool on = true;
                    for (int d = 0; d < 3; ++d)
                        if (pb[d] != -1 && pb[d] != la[d]) on = false;
                    if (on) dmC[C.node(2 * ec[0] + la[0], 2 * ec[1] + la[1], 2 * ec[2] + la[2])] |= m;
                }
            }
}

long q2Child(const Q2Grid &F, long ci, long cj, long ck, int f) {
    return (long)F.elem(2 * ci + (f >> 2 & 1), 2 * cj + (f >> 1 & 1), 2 * ck + (f & 1));
}

// Element matrices of every level below the fine one (MultigridSolver.hh:745-819, 846-905)
void q2BuildLevels(Q2MG &m) {
    m.Kc.assign(8 * 6561, 0.0);
    for (int f = 0; f < 8; ++f) q2AccumulateCoarsened(f, m.K0.data(), m.Kc.data() + (size_t)f * 6561);
    m.Ke.assign(m.g.size(), {});
    for (int l = 1; l <= m.L(); ++l) {
        const Q2Grid &C = m.g[l], &F = m.g[l - 1];
        std::vector<double> &K = m.Ke[l];
        K.assign(C.NE * 6561, 0.0);
#pragma omp parallel for schedule(dynamic, 1)
        for (long e = 0; e < (long)C.NE; ++e) {
            const long ci = e / (C.ne[1] * C.ne[2]), cj = (e / C.ne[2]) % C.ne[1], ck = e % C.ne[2];
            double *out = K.data() + (size_t)e * 6561;
            for (int f = 0; f < 8; ++f) {
                const long ef = q2Child(F, ci, cj, ck, f);
                if (l == 1) {
                    const double E = m.Y[ef];
                    const double *Kc = m.Kc.data() + (size_t)f * 6561;
                    for (int q = 0; q < 6561; ++q) out[q] = (f == 0) ? E * Kc[q] : out[q] + E * Kc[q];
                } else {
                    q2AccumulateCoarsened(f, m.Ke[l - 1].data() + (size_t)ef * 6561, out);
                }
            }
        }
    }
    // coarsest: reduced dense system on the free DOFs (node-major 3 n + c)
    const Q2Grid &C = m.g[m.L()];
    std::vector<long> red(3 * C.NN, -1);
    m.chol.freeIdx.clear();
    for (size_t n = 0; n < C.NN; ++n)
        for (int c = 0; c < 3; ++c)
            if (!(m.dm[m.L()][n] >> c & 1)) { red[3 * n + c] = (long)m.chol.freeIdx.size(); m.chol.freeIdx.push_back((long)(3 * n + c)); }
    const long nf = (long)m.chol.freeIdx.size();
    std::vector<double> A((size_t)nf * nf, 0.0);
    for (long e = 0; e < (long)C.NE; ++e) {
        const long ci = e / (C.ne[1] * C.ne[2]), cj = (e / C.ne[2]) % C.ne[1], ck = e % C.ne[2];
        const double *K = m.Ke[m.L()].data() + (size_t)e * 6561;
        for (int a = 0; a < 27; ++a) {
            const size_t na = C.node(2 * ci + a / 9, 2 * cj + (a / 3) % 3, 2 * ck + a % 3);
            for (int bb = 0; bb < 27; ++bb) {
                const size_t nb = C.node(2 * ci + bb / 9, 2 * cj + (bb / 3) % 3, 2 * ck + bb % 3);
                for (int r = 0; r < 3; ++r)
                    for (int c = 0; c < 3; ++c) {
                        const long ra = red[3 * na + r], cb = red[3 * nb + c];
                        if (ra < 0 || cb < 0) continue;
                        A[(size_t)ra * nf + cb] += K[(3 * a + r) * 81 + 3 * bb + c];
                    }
            }
        }
    }
    m.chol.factor(A, nf);
}

Q2MG *q2mgCreate(const long ne[3], const double *K0, const double *Y, const uint8_t *dmask, int coarsenings) {
    if (coarsenings < 1) throw std::runtime_error("the triquadratic hierarchy needs at least one coarsening");
    auto m = std::make_unique<Q2MG>();
    long n[3] = {ne[0], ne[1], ne[2]};
    for (int l = 0; l <= coarsenings; ++l) {
        if (l > 0)
            for (int d = 0; d < 3; ++d) {
                if (n[d] % 2) throw std::runtime_error("Grid size currently must be divisible by 2^numCoarseningLevels");
                n[d] /= 2;
            }
        m->g.push_back(q2grid(n));
    }
    m->K0.assign(K0, K0 + 6561);
    m->Y.assign(Y, Y + m->g[0].NE);
    m->dm.resize(m->g.size());
    m->dm[0].assign(dmask, dmask + m->g[0].NN);
    for (int l = 1; l <= coarsenings; ++l) q2CoarsenDirichlet(m->g[l - 1], m->dm[l - 1], m->g[l], m->dm[l]);
    q2BuildLevels(*m);
    for (const Q2Grid &g : m->g) {
        m->x.emplace_back(3 * g.NN, 0.0);
        m->b.emplace_back(3 * g.NN, 0.0);
        m->r.emplace_back(3 * g.NN, 0.0);
    }
    return m.release();
}

// out = K_l u with the level's element matrices (element loop, cached-Ke applyK)
void q2ElemApply(const Q2Grid &g, const double *Ke, const double *u, double *out) {
    std::fill(out, out + 3 * g.NN, 0.0);
    for (int parity = 0; parity < 2; ++parity)
#pragma omp parallel for schedule(dynamic, 1)
        for (long i = parity; i < g.ne[0]; i += 2)
            for (long j = 0; j < g.ne[1]; ++j)
                for (long k = 0; k < g.ne[2]; ++k) {
                    size_t nodes[27];
                    double ue[81];
                    for (int l = 0; l < 27; ++l) {
                        nodes[l] = g.node(2 * i + l / 9, 2 * j + (l / 3) % 3, 2 * k + l % 3);
                        for (int c = 0; c < 3; ++c) ue[3 * l + c] = u[c * g.NN + nodes[l]];
                    }
                    const double *K = Ke + (size_t)g.elem(i, j, k) * 6561;
                    for (int rr = 0; rr < 81; ++rr) {
                        double acc = 0.0;
                        for (int t = 0; t < 81; ++t) acc += K[rr * 81 + t] * ue[t];
                        out[(rr % 3) * g.NN + nodes[rr / 3]] += acc;
                    }
                }
}

// 27-colour block Gauss-Seidel with the level's element matrices (NodeSmoothStencilSecondFinest
// and NodeSmoothStencilBlockK, MultigridSolver.hh:294-334, 409-442)
void q2ElemSmooth(const Q2Grid &g, const double *Ke, const uint8_t *dmask, double *u, const double *b, bool forward) {
    for (int ci = 0; ci < 27; ++ci) {
        const int col = forward ? ci : 26 - ci;
        const long lo[3] = {col / 9, (col / 3) % 3, col % 3};
        long inc[3];
        for (int d = 0; d < 3; ++d) inc[d] = (lo[d] == 1) ? 2 : 4;
#pragma omp parallel for schedule(dynamic, 1)
        for (long I = lo[0]; I < g.nn[0]; I += inc[0])
            for (long J = lo[1]; J < g.nn[1]; J += inc[1])
                for (long Kk = lo[2]; Kk < g.nn[2]; Kk += inc[2]) {
                    const size_t n = g.node(I, J, Kk);
                    const uint8_t dmn = dmask[n];
                    if (dmn == 7) continue;
                    double bms[3] = {b[n], b[g.NN + n], b[2 * g.NN + n]};
                    double M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                    const long P[3] = {I, J, Kk};
                    long el[3][2], ll[3][2];
                    int cnt[3];
                    for (int d = 0; d < 3; ++d) {
                        cnt[d] = 0;
                        if (P[d] % 2) { el[d][0] = (P[d] - 1) / 2; ll[d][0] = 1; cnt[d] = 1; }
                        else {
                            if (P[d] / 2 - 1 >= 0) { el[d][cnt[d]] = P[d] / 2 - 1; ll[d][cnt[d]] = 2; ++cnt[d]; }
                            if (P[d] / 2 < g.ne[d]) { el[d][cnt[d]] = P[d] / 2; ll[d][cnt[d]] = 0; ++cnt[d]; }
                        }
                    }
                    for (int a = 0; a < cnt[0]; ++a)
                        for (int bb = 0; bb < cnt[1]; ++bb)
                            for (int c = 0; c < cnt[2]; ++c) {
                                const long ei = el[0][a], ej = el[1][bb], ek = el[2][c];
                                const int ln = 9 * ll[0][a] + 3 * ll[1][bb] + ll[2][c];
                                const double *K = Ke + (size_t)g.elem(ei, ej, ek) * 6561;
                                for (int rr = 0; rr < 3; ++rr) {
                                    double acc = 0.0;
                                    for (int mm = 0; mm < 27; ++mm) {
                                        const size_t nm = g.node(2 * ei + mm / 9, 2 * ej + (mm / 3) % 3, 2 * ek + mm % 3);
                                        for (int cc = 0; cc < 3; ++cc) acc += K[(3 * ln + rr) * 81 + 3 * mm + cc] * u[cc * g.NN + nm];
                                    }
                                    bms[rr] -= acc;
                                    for (int cc = 0; cc < 3; ++cc) M[3 * rr + cc] += K[(3 * ln + rr) * 81 + 3 * ln + cc];
                                }
                            }
                    double un[3] = {u[n], u[g.NN + n], u[2 * g.NN + n]};
                    smoothNodeSolve(dmn, bms, M, un, forward);
                    for (int c = 0; c < 3; ++c) u[c * g.NN + n] = un[c];
                }
    }
}

void q2mgZeroDirichlet(const Q2Grid &g, const std::vector<uint8_t> &dm, double *u) {
    for (size_t n = 0; n < g.NN; ++n)
        for (int c = 0; c < 3; ++c)
            if (dm[n] >> c & 1) u[c * g.NN + n] = 0.0;
}

void q2mgSmooth(Q2MG &m, int l, double *u, const double *b, bool forward) {
    if (l == 0) q2Smooth(m.g[0], m.K0.data(), m.Y.data(), m.dm[0].data(), u, b, forward);
    else q2ElemSmooth(m.g[l], m.Ke[l].data(), m.dm[l].data(), u, b, forward);
}

// computeResidual (MultigridSolver.hh:527-541): r = b - K_l u, zero on constrained components
void q2mgResidual(Q2MG &m, int l, const double *u, const double *b, double *r) {
    const Q2Grid &g = m.g[l];
    std::vector<double> Ku(3 * g.NN);
    if (l == 0) q2ApplyK(g, m.K0.data(), m.Y.data(), u, Ku.data());
    else q2ElemApply(g, m.Ke[l].data(), u, Ku.data());
    for (size_t t = 0; t < 3 * g.NN; ++t) r[t] = b[t] - Ku[t];
    q2mgZeroDirichlet(g, m.dm[l], r);
}

void q2mgCoarseSolve(Q2MG &m, const double *bvec, double *xout) {
    const size_t NN = m.g[m.L()].NN;
    std::vector<double> rhs(m.chol.n);
    for (long t = 0; t < m.chol.n; ++t) {
        const long d = m.chol.freeIdx[t];
        rhs[t] = bvec[(d % 3) * NN + d / 3];
    }
    m.chol.solve(rhs);
    std::fill(xout, xout + 3 * NN, 0.0);
    for (long t = 0; t < m.chol.n; ++t) {
        const long d = m.chol.freeIdx[t];
        xout[(d % 3) * NN + d / 3] = rhs[t];
    }
}

// MultigridSolver.hh:617-658 (residual system: zero Dirichlet values)
void q2mgVcycle(Q2MG &m, int l, long sweeps) {
    if (l == m.L()) { q2mgCoarseSolve(m, m.b[l].data(), m.x[l].data()); return; }
    q2mgZeroDirichlet(m.g[l], m.dm[l], m.x[l].data());
    for (long t = 0; t < sweeps; ++t) q2mgSmooth(m, l, m.x[l].data(), m.b[l].data(), true);
    q2mgResidual(m, l, m.x[l].data(), m.b[l].data(), m.r[l].data());
    const long neF[3] = {m.g[l].ne[0], m.g[l].ne[1], m.g[l].ne[2]};
    q2Restrict(neF, m.r[l].data(), m.b[l + 1].data());
    std::fill(m.x[l + 1].begin(), m.x[l + 1].end(), 0.0);
    q2mgVcycle(m, l + 1, sweeps);
    q2Interp(neF, m.x[l + 1].data(), m.x[l].data(), true);
    for (long t = 0; t < sweeps; ++t) q2mgSmooth(m, l, m.x[l].data(), m.b[l].data(), !m.symmetricGS);
}

double q2Dot(size_t n, const double *a, const double *b) {
    double acc = 0.0;
    for (size_t t = 0; t < n; ++t) acc += a[t] * b[t];
    return acc;
}

// MultigridSolver.hh:1047-1152 with one V-cycle from zero as the preconditioner
void q2mgPcg(Q2MG &m, double *x, const double *bvec, long maxIter, double tol, long sweeps, long *itersOut,
             double *relresOut) {
    const Q2Grid &g = m.g[0];
    const size_t n3 = 3 * g.NN;
    std::vector<double> r(n3), s, d, Ad(n3);
    q2mgZeroDirichlet(g, m.dm[0], x);
    const double bnorm2 = q2Dot(n3, bvec, bvec);
    q2mgResidual(m, 0, x, bvec, r.data());
    double rsq = q2Dot(n3, r.data(), r.data()), rMr = 0.0;
    long i = 0;
    while ((i++ < maxIter) && (rsq > tol * tol * bnorm2)) {
        std::copy(r.begin(), r.end(), m.b[0].begin());
        std::fill(m.x[0].begin(), m.x[0].end(), 0.0);
        q2mgVcycle(m, 0, sweeps);
        s = m.x[0];
        q2mgZeroDirichlet(g, m.dm[0], s.data());
        const double old = rMr;
        rMr = q2Dot(n3, r.data(), s.data());
        if (d.empty()) d = s;
        else
            for (size_t t = 0; t < n3; ++t) d[t] = rMr / old * d[t] + s[t];
        q2ApplyK(g, m.K0.data(), m.Y.data(), d.data(), Ad.data());
        q2mgZeroDirichlet(g, m.dm[0], Ad.data());
        const double alpha = rMr / q2Dot(n3, d.data(), Ad.data());
        for (size_t t = 0; t < n3; ++t) x[t] += alpha * d[t];
        for (size_t t = 0; t < n3; ++t) r[t] -= alpha * Ad[t];
        rsq = q2Dot(n3, r.data(), r.data());
        if (std::isnan(rsq)) throw std::logic_error("NaN encountered at iteration" + std::to_string(i));
    }
    if (itersOut) *itersOut = std::min(i, maxIter + 1) - 1;
    if (relresOut) *relresOut = bnorm2 > 0 ? std::sqrt(rsq / bnorm2) : std::sqrt(rsq);
}

extern "C" {

const char *ovf_last_error() { return g_err.c_str(); }
int ovf_num_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void ovf_set_num_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n);
#else
    (void)n;
#endif
}

void *ovf_sim_create(const long ne[3], const double bmin[3], const double bmax[3]) {
    auto *s = new Sim();
    initSim(*s, ne, bmin, bmax);
    updateY(*s);
    return s;
}
void ovf_sim_destroy(void *s) { delete (Sim *)s; }
void ovf_sim_set_material(void *sp, double E, double nu) {
    Sim &s = *(Sim *)sp;
    s.E_young = E;
    s.nu = nu;
    computeK0(s);
}
void ovf_sim_set_params(void *sp, double E0, double Emin, double gamma, double q, int law) {
    Sim &s = *(Sim *)sp;
    s.E0 = E0; s.Emin = Emin; s.gamma = gamma; s.q = q; s.law = law;
    updateY(s);
}
int ovf_sim_set_densities(void *sp, const double *rho) {
    Sim &s = *(Sim *)sp;
    return guarded([&] {
        for (size_t e = 0; e < s.NE; ++e) s.rho[e] = rho[e];
        updateY(s);
    });
}
void ovf_sim_get_Y(void *sp, double *out) { Sim &s = *(Sim *)sp; std::copy(s.Y.begin(), s.Y.end(), out); }
void ovf_sim_get_K0(void *sp, double *out) { Sim &s = *(Sim *)sp; std::copy(s.K0, s.K0 + 576, out); }
int ovf_sim_add_dirichlet(void *sp, const double u[3], const double mn[3], const double mx[3], int cmask) {
    Sim &s = *(Sim *)sp;
    return guarded([&] { addDirichlet(s, u, mn, mx, (uint8_t)cmask); });
}
void ovf_sim_set_forces(void *sp, const double *f) { Sim &s = *(Sim *)sp; std::copy(f, f + 3 * s.NN, s.force.begin()); }
void ovf_sim_set_gravity(void *sp, const double g[3]) { Sim &s = *(Sim *)sp; for (int c = 0; c < 3; ++c) s.grav[c] = g[c]; }
void ovf_sim_get_dirichlet_mask(void *sp, uint8_t *out) { Sim &s = *(Sim *)sp; std::copy(s.dmask.begin(), s.dmask.end(), out); }
int ovf_sim_set_mask_layer(void *sp, long l) {
    Sim &s = *(Sim *)sp;
    return guarded([&] { setMaskHeight(s, s.h[BUILD_DIR] * l, true); });
}
void ovf_sim_apply_k(void *sp, const double *u, double *out) { applyK_fine<true, false>(*(Sim *)sp, u, out); }
void ovf_sim_build_load(void *sp, double *f) { buildLoad(*(Sim *)sp, f); }
void ovf_sim_compliance_gradient(void *sp, const double *u, double *g) { complianceGradient(*(Sim *)sp, u, g); }
void ovf_sim_element_energy(void *sp, const double *u, double *e) { elementEnergy(*(Sim *)sp, u, e); }

void *ovf_mg_create(void *sp, int levels) {
    MG *mg = nullptr;
    if (guarded([&] { mg = createMG((Sim *)sp, levels); })) return nullptr;
    return mg;
}
void ovf_mg_destroy(void *m) { delete (MG *)m; }
void ovf_mg_set_symmetric(void *m, int sym) { ((MG *)m)->symmetricGS = sym != 0; }
int ovf_mg_num_levels(void *m) { return ((MG *)m)->L(); }
void ovf_mg_level_dims(void *m, int l, long *ne_out) {
    Sim &s = ((MG *)m)->sim(l);
    for (int d = 0; d < 3; ++d) ne_out[d] = s.ne[d];
}
// Propagates the fine mask height to every level (MultigridSolver.hh:1022-1028)
int ovf_mg_set_mask_layer(void *m, long l) {
    MG &mg = *(MG *)m;
    return guarded([&] {
        Sim &f = mg.sim(0);
        setMaskHeight(f, f.h[BUILD_DIR] * l, true);
        for (int k = 1; k < mg.L(); ++k) setMaskHeight(mg.sim(k), f.maskH, false);
        mg.stiffnessValid = false;
    });
}
void ovf_mg_level_dirichlet_mask(void *m, int l, uint8_t *out) {
    Sim &s = ((MG *)m)->sim(l);
    std::copy(s.dmask.begin(), s.dmask.end(), out);
}
int ovf_mg_update_stiffness(void *m) { return guarded([&] { updateStiffness(*(MG *)m); }); }
int ovf_mg_apply_k(void *m, int l, const double *u, double *out) {
    return guarded([&] { applyK_level<true, false>(*(MG *)m, l, u, out); });
}
int ovf_mg_residual(void *m, int l, const double *u, const double *b, double *r) {
    return guarded([&] { computeResidual(*(MG *)m, l, u, b, r); });
}
int ovf_mg_smooth(void *m, int l, double *u, const double *b, int forward) {
    return guarded([&] {
        MG &mg = *(MG *)m;
        if (!mg.stiffnessValid && l >= 2) updateStiffness(mg);
        smoothGS(mg, l, u, b, forward != 0);
    });
}
int ovf_mg_restrict(void *m, int l, const double *fine, double *coarse) {
    return guarded([&] { restriction(*(MG *)m, l, fine, coarse); });
}
int ovf_mg_interpolate(void *m, int l, const double *coarse, double *fine, int accumulate) {
    return guarded([&] { interpolate(*(MG *)m, l, coarse, fine, accumulate != 0); });
}
int ovf_mg_coarse_solve(void *m, const double *b, double *x) {
    return guarded([&] {
        MG &mg = *(MG *)m;
        if (!mg.stiffnessValid) updateStiffness(mg);
        coarseSolve(mg, b, x);
    });
}
int ovf_mg_solve(void *m, const double *u, const double *f, long steps, long sweeps, int zeroDirichlet, int fmg, double *out) {
    return guarded([&] {
        MG &mg = *(MG *)m;
        updateStiffness(mg);
        mgSolve(mg, u, f, steps, sweeps, zeroDirichlet != 0, fmg != 0);
        std::copy(mg.x[0].begin(), mg.x[0].end(), out);
    });
}
int ovf_mg_pcg(void *m, double *x, const double *b, long maxIter, double tol, long mgIter, long sweeps, int fmg,
               int dirichletSatisfied, long *iters, double *relres, void (*cb)(long, double)) {
    return guarded([&] {
        pcg(*(MG *)m, x, b, maxIter, tol, mgIter, sweeps, fmg != 0, dirichletSatisfied != 0, iters, relres, cb);
    });
}

void ovf_smoothing_filter(const long dims[3], int radius, int type, const double *in, double *out) {
    smoothingFilter(dims, radius, type, in, out);
}
void ovf_projection_apply(long n, double beta, const double *in, double *out) { projectionApply(n, beta, in, out); }
void ovf_projection_backprop(long n, double beta, const double *in, const double *vars, double *out) {
    projectionBackprop(n, beta, in, vars, out);
}

// filters: array of (kind, radius, type, beta)
void *ovf_top_create(void *m, int nfilters, const int *kinds, const int *radii, const int *types, const double *betas,
                     double volfrac) {
    MG &mg = *(MG *)m;
    auto *t = new TOP();
    t->mg = &mg;
    for (int i = 0; i < nfilters; ++i) t->filters.push_back({kinds[i], radii[i], types[i], betas[i]});
    t->volfrac = volfrac;
    Sim &s = mg.sim(0);
    t->f.assign(3 * s.NN, 0.0);
    buildLoad(s, t->f.data());
    t->u.assign(3 * s.NN, 0.0);
    return t;
}
void ovf_top_destroy(void *t) { delete (TOP *)t; }
void ovf_top_set_solver(void *tp, long cgIter, double tol, long mgIter, long sweeps, int fmg, int zeroInit) {
    TOP &t = *(TOP *)tp;
    t.cgIter = cgIter; t.tol = tol; t.mgIter = mgIter; t.mgSweeps = sweeps; t.fmg = fmg != 0; t.zeroInit = zeroInit != 0;
}
int ovf_top_set_vars(void *t, const double *x) { return guarded([&] { topSetVars(*(TOP *)t, x); }); }
double ovf_top_objective(void *t) { return topObjective(*(TOP *)t); }
int ovf_top_gradient(void *t, double *out) { return guarded([&] { topGradient(*(TOP *)t, out); }); }
double ovf_top_constraint(void *t) { return topConstraint(*(TOP *)t); }
int ovf_top_jacobian(void *t, double *out) { return guarded([&] { topJacobian(*(TOP *)t, out); }); }
void ovf_top_get_u(void *tp, double *out) { TOP &t = *(TOP *)tp; std::copy(t.u.begin(), t.u.end(), out); }
void ovf_top_get_design(void *tp, double *out) { TOP &t = *(TOP *)tp; std::copy(t.vars.front().begin(), t.vars.front().end(), out); }
void ovf_top_get_physical(void *tp, double *out) { TOP &t = *(TOP *)tp; std::copy(t.vars.back().begin(), t.vars.back().end(), out); }
long ovf_top_last_iters(void *tp) { return ((TOP *)tp)->lastIters; }
int ovf_top_oc_step(void *t, double m, double p, double ctol, long *probes) {
    return guarded([&] { ocStep(*(TOP *)t, m, p, ctol, probes); });
}


// ---- triquadratic voxels ----
void ovf_q2_k0(double E, double nu, const double h[3], int npts, double *out) { q2K0(E, nu, h, npts, out); }
void ovf_q2_apply_k(const long ne[3], const double *K, const double *Y, const double *u, double *out) {
    q2ApplyK(q2grid(ne), K, Y, u, out);
}
void ovf_q2_smooth(const long ne[3], const double *K, const double *Y, const uint8_t *dmask, double *u,
                   const double *b, int forward) {
    q2Smooth(q2grid(ne), K, Y, dmask, u, b, forward != 0);
}
void ovf_q2_interp(const long neF[3], const double *coarse, double *fine, int accumulate) {
    q2Interp(neF, coarse, fine, accumulate != 0);
}
void ovf_q2_restrict(const long neF[3], const double *fine, double *coarse) { q2Restrict(neF, fine, coarse); }
// ---- triquadratic multigrid hierarchy ----
void *ovf_q2mg_create(const long ne[3], const double *K0, const double *Y, const uint8_t *dmask, int coarsenings) {
    Q2MG *m = nullptr;
    guarded([&] { m = q2mgCreate(ne, K0, Y, dmask, coarsenings); });
    return m;
}
void ovf_q2mg_destroy(void *m) { delete (Q2MG *)m; }
void ovf_q2mg_level_dims(void *mp, int l, long *ne) {
    const Q2Grid &g = ((Q2MG *)mp)->g.at(l);
    for (int d = 0; d < 3; ++d) ne[d] = g.ne[d];
}
void ovf_q2mg_level_dirichlet(void *mp, int l, uint8_t *out) {
    const auto &v = ((Q2MG *)mp)->dm.at(l);
    std::copy(v.begin(), v.end(), out);
}
void ovf_q2mg_level_ke(void *mp, int l, double *out) {
    const auto &v = ((Q2MG *)mp)->Ke.at(l);
    std::copy(v.begin(), v.end(), out);
}
void ovf_q2mg_coarsened_k0(void *mp, double *out) {
    const auto &v = ((Q2MG *)mp)->Kc;
    std::copy(v.begin(), v.end(), out);
}
int ovf_q2mg_smooth(void *mp, int l, double *u, const double *b, int forward) {
    return guarded([&] { q2mgSmooth(*(Q2MG *)mp, l, u, b, forward != 0); });
}
int ovf_q2mg_residual(void *mp, int l, const double *u, const double *b, double *r) {
    return guarded([&] { q2mgResidual(*(Q2MG *)mp, l, u, b, r); });
}
int ovf_q2mg_coarse_solve(void *mp, const double *b, double *x) {
    return guarded([&] { q2mgCoarseSolve(*(Q2MG *)mp, b, x); });
}
int ovf_q2mg_vcycle(void *mp, const double *b, double *x, long sweeps) {
    return guarded([&] {
        Q2MG &m = *(Q2MG *)mp;
        std::copy(b, b + m.b[0].size(), m.b[0].begin());
        std::fill(m.x[0].begin(), m.x[0].end(), 0.0);
        q2mgVcycle(m, 0, sweeps);
        std::copy(m.x[0].begin(), m.x[0].end(), x);
    });
}
int ovf_q2mg_pcg(void *mp, double *x, const double *b, long maxIter, double tol, long sweeps, long *iters,
                 double *relres) {
    return guarded([&] { q2mgPcg(*(Q2MG *)mp, x, b, maxIter, tol, sweeps, iters, relres); });
}
}  // extern "C"
