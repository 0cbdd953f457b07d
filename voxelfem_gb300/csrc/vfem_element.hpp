// Host-side Q1 element mathematics (see vfem_element.cpp).
#pragma once

namespace vfem {

// Full-density element stiffness for an isotropic material (E, nu) on an h[0] x h[1] x h[2] voxel.
// DOF ordering 3 * l + c with local node l = 4 dx + 2 dy + dz.
void element_stiffness(double E, double nu, const double h[3], double K0[576]);
// Triquadratic (27-node) element: 81 x 81, DOF 3l + r, local node l = 9a + 3b + c,
// 3-point Gauss per axis (exact for the degree-4 integrand).
void element_stiffness_q2(double E, double nu, const double h[3], double K0[6561]);

// Compressed element interpolation operators, phis[fi][fine_n * 8 + coarse_n].
void interpolation_phis(double phis[8][64]);

// Kc += (phi (x) Id_3)^T Kf (phi (x) Id_3).
void coarsen_element(const double phi[64], const double Kf[576], double Kc[576]);

}  // namespace vfem
