// Host-side element mathematics for trilinear (Q1) hexahedra, evaluated once per
// material / stretching change and uploaded to the device.
//
//  * full-density element stiffness K0 (TensorProductSimulator.hh:67-80, 2078-2086):
//    K0_ij = vol * sum_q w_q eps_i(q) : C : eps_j(q), two Gauss points per axis
//    (TensorProductQuadrature.hh:134-143); eps(phi_{n,c}) = sym(e_c (x) grad N_n)
//    (TensorProductPolynomialInterpolant.hh:197-232); C isotropic from (E, nu);
//  * the compressed element interpolation operator phi_fi (MultigridSolver.hh:664-687);
//  * the coarsened fine stiffness Kc_fi = I_fi^T K0 I_fi (MultigridSolver.hh:712-722).
#include "vfem_element.hpp"

#include <algorithm>
#include <cmath>
#include <vector>

#include "vfem_kernels.hpp"

namespace vfem {

void element_stiffness(double E, double nu, const double h[3], double K0[576]) {
    const double lam = E * nu / ((1 + nu) * (1 - 2 * nu));
    const double mu = E / (2 * (1 + nu));
    const double q[2] = {0.5 - 0.5 / std::sqrt(3.0), 0.5 + 0.5 / std::sqrt(3.0)};
    double acc[576] = {0};
    for (int qp = 0; qp < 8; ++qp) {
        const double x[3] = {q[(qp >> 2) & 1], q[(qp >> 1) & 1], q[qp & 1]};
        // gradients of the 8 trilinear shape functions (physical coordinates)
        double G[8][3];
        for (int l = 0; l < 8; ++l) {
            const int bit[3] = {(l >> 2) & 1, (l >> 1) & 1, l & 1};
            double val[3], der[3];
            for (int d = 0; d < 3; ++d) {
                val[d] = bit[d] ? x[d] : 1.0 - x[d];
                der[d] = (bit[d] ? 1.0 : -1.0) / h[d];
            }
            G[l][0] = der[0] * val[1] * val[2];
            G[l][1] = val[0] * der[1] * val[2];
            G[l][2] = val[0] * val[1] * der[2];
        }
        // eps_i : C : eps_j = lam tr(eps_i) tr(eps_j) + 2 mu eps_i : eps_j, with
        // eps(phi_{a,c}) = sym(e_c (x) G_a): tr = G_a[c],
        // eps(a,c):eps(b,d) = 0.5 (delta_cd G_a.G_b + G_a[d] G_b[c]).
        for (int a = 0; a < 8; ++a)
            for (int c = 0; c < 3; ++c)
                for (int b = 0; b < 8; ++b)
                    for (int d = 0; d < 3; ++d) {
                        const double dot = G[a][0] * G[b][0] + G[a][1] * G[b][1] + G[a][2] * G[b][2];
                        const double ee = 0.5 * ((c == d ? dot : 0.0) + G[a][d] * G[b][c]);
                        acc[(3 * a + c) * 24 + 3 * b + d] += 0.125 * (lam * G[a][c] * G[b][d] + 2 * mu * ee);
                    }
    }
    const double vol = h[0] * h[1] * h[2];
    for (int i = 0; i < 24; ++i)
        for (int j = i; j < 24; ++j) {
            K0[i * 24 + j] = acc[i * 24 + j] * vol;
            K0[j * 24 + i] = K0[i * 24 + j];
        }
}

void interpolation_phis(double phis[8][64]) {
    // phis[fi][fine_n * 8 + coarse_n]: coarse shape function coarse_n at fine node fine_n
    // of child element fi (fi = 4 fx + 2 fy + fz, nodes l = 4 dx + 2 dy + dz).
    for (int fi = 0; fi < 8; ++fi)
        for (int fn = 0; fn < 8; ++fn)
            for (int cn = 0; cn < 8; ++cn) {
                double v = 1.0;
                for (int d = 0; d < 3; ++d) {
                    const int sh = 2 - d;
                    const double p = 0.5 * (((fi >> sh) & 1) + ((fn >> sh) & 1));
                    v *= ((cn >> sh) & 1) ? p : 1.0 - p;
                }
                phis[fi][fn * 8 + cn] = v;
            }
}

void coarsen_element(const double phi[64], const double Kf[576], double Kc[576]) {
    double T[576];
    for (int r = 0; r < 24; ++r)
        for (int cn = 0; cn < 8; ++cn)
            for (int d = 0; d < 3; ++d) {
                double s = 0;
                for (int fn = 0; fn < 8; ++fn) s += Kf[r * 24 + 3 * fn + d] * phi[fn * 8 + cn];
                T[r * 24 + 3 * cn + d] = s;
            }
    for (int cm = 0; cm < 8; ++cm)
        for (int d = 0; d < 3; ++d)
            for (int c = 0; c < 24; ++c) {
                double s = 0;
                for (int fm = 0; fm < 8; ++fm) s += phi[fm * 8 + cm] * T[(3 * fm + d) * 24 + c];
                Kc[(3 * cm + d) * 24 + c] += s;
            }
}

// Equispaced quadratic Lagrange basis on [0, 1] (nodes 0, 1/2, 1) and its derivative.
static void q2_basis1d(double x, double v[3], double dv[3]) {
    v[0] = 2 * (x - 0.5) * (x - 1.0);
    v[1] = -4 * x * (x - 1.0);
    v[2] = 2 * x * (x - 0.5);
    dv[0] = 4 * x - 3;
    dv[1] = -8 * x + 4;
    dv[2] = 4 * x - 1;
}

void element_stiffness_q2(double E, double nu, const double h[3], double K0[6561]) {
    const double lam = E * nu / ((1 + nu) * (1 - 2 * nu));
    const double mu = E / (2 * (1 + nu));
    const double r = 0.5 * std::sqrt(0.6);
    const double qp[3] = {0.5 - r, 0.5, 0.5 + r}, qw[3] = {5.0 / 18, 8.0 / 18, 5.0 / 18};
    std::vector<double> acc(6561, 0.0);
    for (int qa = 0; qa < 3; ++qa)
        for (int qb = 0; qb < 3; ++qb)
            for (int qc = 0; qc < 3; ++qc) {
                const double w = qw[qa] * qw[qb] * qw[qc];
                double v[3][3], dv[3][3];
                q2_basis1d(qp[qa], v[0], dv[0]);
                q2_basis1d(qp[qb], v[1], dv[1]);
                q2_basis1d(qp[qc], v[2], dv[2]);
                double G[27][3];
                for (int l = 0; l < 27; ++l) {
                    const int a = l / 9, b = (l / 3) % 3, c = l % 3;
                    G[l][0] = dv[0][a] * v[1][b] * v[2][c] / h[0];
                    G[l][1] = v[0][a] * dv[1][b] * v[2][c] / h[1];
                    G[l][2] = v[0][a] * v[1][b] * dv[2][c] / h[2];
                }
                for (int a = 0; a < 27; ++a)
                    for (int c = 0; c < 3; ++c)
                        for (int b = 0; b < 27; ++b)
                            for (int d = 0; d < 3; ++d) {
                                const double dot = G[a][0] * G[b][0] + G[a][1] * G[b][1] + G[a][2] * G[b][2];
                                const double ee = 0.5 * ((c == d ? dot : 0.0) + G[a][d] * G[b][c]);
                                acc[(3 * a + c) * 81 + 3 * b + d] += w * (lam * G[a][c] * G[b][d] + 2 * mu * ee);
                            }
            }
    const double vol = h[0] * h[1] * h[2];
    for (int i = 0; i < 81; ++i)
        for (int j = i; j < 81; ++j) {
            K0[i * 81 + j] = acc[i * 81 + j] * vol;
            K0[j * 81 + i] = K0[i * 81 + j];
        }
}

bool k0_cube_values(const double *K, double kv[10]) {
    double amax = 0.0;
    for (int t = 0; t < 576; ++t) amax = std::max(amax, std::fabs(K[t]));
    bool set[10] = {false};
    for (int row = 0; row < 24; ++row)
        for (int col = 0; col < 24; ++col) {
            const int c = k0_cube_class(row, col);
            const double v = (c & 16) ? -K[row * 24 + col] : K[row * 24 + col];
            const int k = c & 15;
            if (!set[k]) {
                kv[k] = v;
                set[k] = true;
            } else if (std::fabs(kv[k] - v) > 1e-13 * amax) {
                return false;
            }
        }
    return true;
}

}  // namespace vfem
