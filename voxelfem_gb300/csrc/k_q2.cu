// Triquadratic (Q2) voxel kernels (TPSStencils.hh:135-186, MultigridSolver.hh:277-321,
// 409-442): matrix-free SIMP applyK, the 27-colour block Gauss-Seidel sweep and the Q2
// restriction / prolongation between a grid and its 2x coarsening.
//
// Nodes: (2 nx + 1)(2 ny + 1)(2 nz + 1), index (I * NY + J) * NZ + K. Element (i, j, k) owns
// nodes (2i + a, 2j + b, 2k + c), local index l = 9a + 3b + c; K0 is 81 x 81 with DOF 3l + r.
// A node's parity (I&1, J&1, K&1) fixes where it sits in its incident elements: an even
// coordinate is a corner (local 0 of element I/2, local 2 of element I/2 - 1), an odd one is
// the middle (local 1 of element (I-1)/2). The kernels run one node parity (applyK) or one
// colour (smoother) per launch, so every warp reads the same K0 rows: K0 lives in constant
// memory (FP32, 26 KB) or in global memory (FP64, 52 KB) and its reads are broadcasts.
#include "vfem_df.cuh"
#include "vfem_kernels.hpp"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>

namespace vfem {

__constant__ float c_K0q2f[81 * 81];
__constant__ float c_K0q2lo[81 * 81];  // K0 - c_K0q2f (double-float matvec)

namespace {

constexpr int BS = 256;

struct Q2Dims {
    int ne[3], nn[3];
    int64_t NN, NE;
};

__device__ __forceinline__ int64_t q2node(const Q2Dims &d, int I, int J, int K) {
    return ((int64_t)I * d.nn[1] + J) * d.nn[2] + K;
}

template <typename T>
struct Q2K;
template <>
struct Q2K<float> {
    static __device__ __forceinline__ float at(const float *, int r, int c) { return c_K0q2f[r * 81 + c]; }
};
template <>
struct Q2K<double> {
    static __device__ __forceinline__ double at(const double *K, int r, int c) { return __ldg(K + r * 81 + c); }
};

// Incident elements of a node along one axis: count, element index and local coordinate.
__device__ __forceinline__ int axis_elems(int I, int ne, int *ei, int *la) {
    if (I & 1) {
        ei[0] = (I - 1) >> 1;
        la[0] = 1;
        return 1;
    }
    int n = 0;
    if ((I >> 1) < ne) { ei[n] = I >> 1; la[n] = 0; ++n; }
    if ((I >> 1) - 1 >= 0) { ei[n] = (I >> 1) - 1; la[n] = 2; ++n; }
    return n;
}

// s -= E_e K0[3ln + r, :] u_e over the node's incident elements (and M += E_e K0 diagonal block)
template <typename T, bool WithM>
__device__ __forceinline__ void q2_gather(const Q2Dims &d, const T *Kg, const T *__restrict__ Y,
                                          const T *__restrict__ u, int I, int J, int K, T &s0, T &s1, T &s2, T *M) {
    int ex[2], ey[2], ez[2], ax[2], ay[2], az[2];
    const int nx = axis_elems(I, d.ne[0], ex, ax), ny = axis_elems(J, d.ne[1], ey, ay), nz = axis_elems(K, d.ne[2], ez, az);
    const int64_t ld = d.NN;
    for (int p = 0; p < nx; ++p)
        for (int q = 0; q < ny; ++q)
            for (int w = 0; w < nz; ++w) {
                const int ei = ex[p], ej = ey[q], ek = ez[w];
                const int ln = 9 * ax[p] + 3 * ay[q] + az[w];
                const T E = Y[((int64_t)ei * d.ne[1] + ej) * d.ne[2] + ek];
                T c0 = T(0), c1 = T(0), c2 = T(0);
#pragma unroll 3
                for (int m = 0; m < 27; ++m) {
                    const int64_t nm = q2node(d, 2 * ei + m / 9, 2 * ej + (m / 3) % 3, 2 * ek + m % 3);
                    const T u0 = u[nm], u1 = u[ld + nm], u2 = u[2 * ld + nm];
                    // symmetric K0: column 3ln + r read as row (3m + c)
                    c0 += Q2K<T>::at(Kg, 3 * m, 3 * ln) * u0 + Q2K<T>::at(Kg, 3 * m + 1, 3 * ln) * u1 +
                          Q2K<T>::at(Kg, 3 * m + 2, 3 * ln) * u2;
                    c1 += Q2K<T>::at(Kg, 3 * m, 3 * ln + 1) * u0 + Q2K<T>::at(Kg, 3 * m + 1, 3 * ln + 1) * u1 +
                          Q2K<T>::at(Kg, 3 * m + 2, 3 * ln + 1) * u2;
                    c2 += Q2K<T>::at(Kg, 3 * m, 3 * ln + 2) * u0 + Q2K<T>::at(Kg, 3 * m + 1, 3 * ln + 2) * u1 +
                          Q2K<T>::at(Kg, 3 * m + 2, 3 * ln + 2) * u2;
                }
                s0 -= E * c0;
                s1 -= E * c1;
                s2 -= E * c2;
                if (WithM) {
#pragma unroll
                    for (int r = 0; r < 3; ++r)
#pragma unroll
                        for (int c = 0; c < 3; ++c) M[3 * r + c] += E * Q2K<T>::at(Kg, 3 * ln + r, 3 * ln + c);
                }
            }
}

// FP32 form with the node parity (PX, PY, PZ) as template parameters: every incident-element
// slot has a compile-time local index, so each K0 entry is a constant-bank operand of its FFMA
// (no load instruction). Even axes have two slots (local 0 of element I/2, local 2 of element
// I/2 - 1, either may fall outside the grid), odd axes one (local 1 of element (I-1)/2).
template <int P>
__device__ __forceinline__ bool q2_slot(int I, int ne, int s, int &e) {
    if (P) {
        e = (I - 1) >> 1;
        return true;
    }
    e = s == 0 ? (I >> 1) : (I >> 1) - 1;
    return e >= 0 && e < ne;
}

template <int P, int S>
struct Q2Local {
    static constexpr int value = P ? 1 : (S == 0 ? 0 : 2);
};

template <int PX, int PY, int PZ, bool WithM>
__device__ __forceinline__ void q2_gather_f32(const Q2Dims &d, const float *__restrict__ Y, const float *__restrict__ u,
                                              int I, int J, int K, float &s0, float &s1, float &s2, float *M);

template <int PX, int PY, int PZ, bool WithM, int SA, int SB, int SC>
__device__ __forceinline__ void q2_slot_f32(const Q2Dims &d, const float *__restrict__ Y, const float *__restrict__ u,
                                            int I, int J, int K, float &s0, float &s1, float &s2, float *M) {
    int ei, ej, ek;
    if (!q2_slot<PX>(I, d.ne[0], SA, ei) || !q2_slot<PY>(J, d.ne[1], SB, ej) || !q2_slot<PZ>(K, d.ne[2], SC, ek)) return;
    constexpr int LN = 9 * Q2Local<PX, SA>::value + 3 * Q2Local<PY, SB>::value + Q2Local<PZ, SC>::value;
    const float E = Y[((int64_t)ei * d.ne[1] + ej) * d.ne[2] + ek];
    const int64_t ld = d.NN;
    const int64_t base = q2node(d, 2 * ei, 2 * ej, 2 * ek);
    const int64_t sx = (int64_t)d.nn[1] * d.nn[2], sy = d.nn[2];
    float c0 = 0.f, c1 = 0.f, c2 = 0.f;
#pragma unroll
    for (int m = 0; m < 27; ++m) {
        const int64_t nm = base + (m / 9) * sx + ((m / 3) % 3) * sy + (m % 3);
        const float u0 = u[nm], u1 = u[ld + nm], u2 = u[2 * ld + nm];
        c0 += c_K0q2f[(3 * m) * 81 + 3 * LN] * u0 + c_K0q2f[(3 * m + 1) * 81 + 3 * LN] * u1 +
              c_K0q2f[(3 * m + 2) * 81 + 3 * LN] * u2;
        c1 += c_K0q2f[(3 * m) * 81 + 3 * LN + 1] * u0 + c_K0q2f[(3 * m + 1) * 81 + 3 * LN + 1] * u1 +
              c_K0q2f[(3 * m + 2) * 81 + 3 * LN + 1] * u2;
        c2 += c_K0q2f[(3 * m) * 81 + 3 * LN + 2] * u0 + c_K0q2f[(3 * m + 1) * 81 + 3 * LN + 2] * u1 +
              c_K0q2f[(3 * m + 2) * 81 + 3 * LN + 2] * u2;
    }
    s0 -= E * c0;
    s1 -= E * c1;
    s2 -= E * c2;
    if (WithM) {
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) M[3 * r + c] += E * c_K0q2f[(3 * LN + r) * 81 + 3 * LN + c];
    }
}

template <int PX, int PY, int PZ, bool WithM>
__device__ __forceinline__ void q2_gather_f32(const Q2Dims &d, const float *__restrict__ Y, const float *__restrict__ u,
                                              int I, int J, int K, float &s0, float &s1, float &s2, float *M) {
    q2_slot_f32<PX, PY, PZ, WithM, 0, 0, 0>(d, Y, u, I, J, K, s0, s1, s2, M);
    if (!PZ) q2_slot_f32<PX, PY, PZ, WithM, 0, 0, 1>(d, Y, u, I, J, K, s0, s1, s2, M);
    if (!PY) {
        q2_slot_f32<PX, PY, PZ, WithM, 0, 1, 0>(d, Y, u, I, J, K, s0, s1, s2, M);
        if (!PZ) q2_slot_f32<PX, PY, PZ, WithM, 0, 1, 1>(d, Y, u, I, J, K, s0, s1, s2, M);
    }
    if (!PX) {
        q2_slot_f32<PX, PY, PZ, WithM, 1, 0, 0>(d, Y, u, I, J, K, s0, s1, s2, M);
        if (!PZ) q2_slot_f32<PX, PY, PZ, WithM, 1, 0, 1>(d, Y, u, I, J, K, s0, s1, s2, M);
        if (!PY) {
            q2_slot_f32<PX, PY, PZ, WithM, 1, 1, 0>(d, Y, u, I, J, K, s0, s1, s2, M);
            if (!PZ) q2_slot_f32<PX, PY, PZ, WithM, 1, 1, 1>(d, Y, u, I, J, K, s0, s1, s2, M);
        }
    }
}

// Double-float form of q2_slot_f32: K0 = c_K0q2f + c_K0q2lo, u = uh + ul, E = Yh + Yl;
// (fh, fl) += E_e K0[3 LN + r, :] u_e.
template <int PX, int PY, int PZ, int SA, int SB, int SC>
__device__ __forceinline__ void q2_slot_df(const Q2Dims &d, const float *__restrict__ Yh, const float *__restrict__ Yl,
                                           const float *__restrict__ uh, const float *__restrict__ ul, int I, int J,
                                           int K, float *fh, float *fl) {
    int ei, ej, ek;
    if (!q2_slot<PX>(I, d.ne[0], SA, ei) || !q2_slot<PY>(J, d.ne[1], SB, ej) || !q2_slot<PZ>(K, d.ne[2], SC, ek)) return;
    constexpr int LN = 9 * Q2Local<PX, SA>::value + 3 * Q2Local<PY, SB>::value + Q2Local<PZ, SC>::value;
    const int64_t e = ((int64_t)ei * d.ne[1] + ej) * d.ne[2] + ek;
    const float eh = Yh[e], el = Yl[e];
    const int64_t ld = d.NN;
    const int64_t base = q2node(d, 2 * ei, 2 * ej, 2 * ek);
    const int64_t sx = (int64_t)d.nn[1] * d.nn[2], sy = d.nn[2];
    float ch[3] = {0.f, 0.f, 0.f}, cl[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int m = 0; m < 27; ++m) {
        const int64_t nm = base + (m / 9) * sx + ((m / 3) % 3) * sy + (m % 3);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float vh = uh[c * ld + nm], vl = ul[c * ld + nm];
#pragma unroll
            for (int r = 0; r < 3; ++r)
                df_fma_acc(c_K0q2f[(3 * m + c) * 81 + 3 * LN + r], c_K0q2lo[(3 * m + c) * 81 + 3 * LN + r], vh, vl,
                           ch[r], cl[r]);
        }
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const float s = ch[r] + cl[r];
        const float sl = cl[r] - (s - ch[r]);
        df_fma_acc(eh, el, s, sl, fh[r], fl[r]);
    }
}

// out = K u to FP64-class accuracy on the FP32 units, at the nodes of parity class (PX, PY, PZ);
// constrained components zeroed when asked; optional partial dots u . out per block.
template <int PX, int PY, int PZ>
__global__ void __launch_bounds__(BS) applyk_q2_df_kernel(Q2Dims d, const float *__restrict__ Yh,
                                                          const float *__restrict__ Yl, const float *__restrict__ uh,
                                                          const float *__restrict__ ul, double *__restrict__ out,
                                                          const uint8_t *__restrict__ dmask, int zeroDir) {
    const int n0 = (d.nn[0] - PX + 1) / 2, n1 = (d.nn[1] - PY + 1) / 2, n2 = (d.nn[2] - PZ + 1) / 2;
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= (int64_t)n0 * n1 * n2) return;
    const uint32_t tt = (uint32_t)t, q = tt / (uint32_t)n2;
    const int K = 2 * (int)(tt - q * (uint32_t)n2) + PZ;
    const int J = 2 * (int)(q % (uint32_t)n1) + PY, I = 2 * (int)(q / (uint32_t)n1) + PX;
    float fh[3] = {0.f, 0.f, 0.f}, fl[3] = {0.f, 0.f, 0.f};
    q2_slot_df<PX, PY, PZ, 0, 0, 0>(d, Yh, Yl, uh, ul, I, J, K, fh, fl);
    if (!PZ) q2_slot_df<PX, PY, PZ, 0, 0, 1>(d, Yh, Yl, uh, ul, I, J, K, fh, fl);
    if (!PY) {
        q2_slot_df<PX, PY, PZ, 0, 1, 0>(d, Yh, Yl, uh, ul, I, J, K, fh, fl);
        if (!PZ) q2_slot_df<PX, PY, PZ, 0, 1, 1>(d, Yh, Yl, uh, ul, I, J, K, fh, fl);
    }
    if (!PX) {
        q2_slot_df<PX, PY, PZ, 1, 0, 0>(d, Yh, Yl, uh, ul, I, J, K, fh, fl);
        if (!PZ) q2_slot_df<PX, PY, PZ, 1, 0, 1>(d, Yh, Yl, uh, ul, I, J, K, fh, fl);
        if (!PY) {
            q2_slot_df<PX, PY, PZ, 1, 1, 0>(d, Yh, Yl, uh, ul, I, J, K, fh, fl);
            if (!PZ) q2_slot_df<PX, PY, PZ, 1, 1, 1>(d, Yh, Yl, uh, ul, I, J, K, fh, fl);
        }
    }
    const int64_t n = q2node(d, I, J, K), ld = d.NN;
    const uint8_t dm = zeroDir ? dmask[n] : 0;
#pragma unroll
    for (int r = 0; r < 3; ++r) out[r * ld + n] = ((dm >> r) & 1) ? 0.0 : (double)fh[r] + (double)fl[r];
}

template <int PX, int PY, int PZ>
__global__ void __launch_bounds__(BS) applyk_q2_f32_kernel(Q2Dims d, const float *__restrict__ Y,
                                                           const float *__restrict__ u, float *__restrict__ out,
                                                           const uint8_t *__restrict__ dmask, int zeroDir) {
    const int n0 = (d.nn[0] - PX + 1) / 2, n1 = (d.nn[1] - PY + 1) / 2, n2 = (d.nn[2] - PZ + 1) / 2;
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= (int64_t)n0 * n1 * n2) return;
    const uint32_t tt = (uint32_t)t, q = tt / (uint32_t)n2;
    const int K = 2 * (int)(tt - q * (uint32_t)n2) + PZ;
    const int J = 2 * (int)(q % (uint32_t)n1) + PY, I = 2 * (int)(q / (uint32_t)n1) + PX;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
    q2_gather_f32<PX, PY, PZ, false>(d, Y, u, I, J, K, s0, s1, s2, nullptr);
    const int64_t n = q2node(d, I, J, K), ld = d.NN;
    const uint8_t dm = zeroDir ? dmask[n] : 0;
    out[n] = (dm & 1) ? 0.f : -s0;
    out[ld + n] = (dm & 2) ? 0.f : -s1;
    out[2 * ld + n] = (dm & 4) ? 0.f : -s2;
}

// out = K u at the nodes of one parity class (px, py, pz); constrained components zeroed when asked
template <typename T>
__global__ void __launch_bounds__(BS) applyk_q2_kernel(Q2Dims d, const T *Kg, const T *__restrict__ Y,
                                                       const T *__restrict__ u, T *__restrict__ out,
                                                       const uint8_t *__restrict__ dmask, int zeroDir) {
    const int par = blockIdx.y;
    const int px = (par >> 2) & 1, py = (par >> 1) & 1, pz = par & 1;
    const int n0 = (d.nn[0] - px + 1) / 2, n1 = (d.nn[1] - py + 1) / 2, n2 = (d.nn[2] - pz + 1) / 2;
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= (int64_t)n0 * n1 * n2) return;
    const uint32_t tt = (uint32_t)t, q = tt / (uint32_t)n2;
    const int K = 2 * (int)(tt - q * (uint32_t)n2) + pz;
    const int J = 2 * (int)(q % (uint32_t)n1) + py, I = 2 * (int)(q / (uint32_t)n1) + px;
    T s0 = T(0), s1 = T(0), s2 = T(0);
    q2_gather<T, false>(d, Kg, Y, u, I, J, K, s0, s1, s2, nullptr);
    const int64_t n = q2node(d, I, J, K), ld = d.NN;
    const uint8_t dm = zeroDir ? dmask[n] : 0;
    out[n] = (dm & 1) ? T(0) : -s0;
    out[ld + n] = (dm & 2) ? T(0) : -s1;
    out[2 * ld + n] = (dm & 4) ? T(0) : -s2;
}

template <typename T>
__device__ __forceinline__ void q2_node_update(uint8_t dm, T s0, T s1, T s2, const T *M, bool forward, T &u0, T &u1,
                                               T &u2) {
    if (dm) {
        // pointwise Gauss-Seidel on the free components (MultigridSolver.hh:352-366)
        T dd[3] = {T(0), T(0), T(0)};
        const T bs[3] = {s0, s1, s2};
        if (forward) {
#pragma unroll
            for (int r = 0; r < 3; ++r)
                dd[r] = (bs[r] - (M[3 * r] * dd[0] + M[3 * r + 1] * dd[1] + M[3 * r + 2] * dd[2])) *
                        (T(!((dm >> r) & 1)) / M[4 * r]);
        } else {
#pragma unroll
            for (int r = 2; r >= 0; --r)
                dd[r] = (bs[r] - (M[3 * r] * dd[0] + M[3 * r + 1] * dd[1] + M[3 * r + 2] * dd[2])) *
                        (T(!((dm >> r) & 1)) / M[4 * r]);
        }
        u0 += dd[0];
        u1 += dd[1];
        u2 += dd[2];
    } else {
        const T c00 = M[4] * M[8] - M[5] * M[7], c01 = M[5] * M[6] - M[3] * M[8], c02 = M[3] * M[7] - M[4] * M[6];
        const T id = T(1) / (M[0] * c00 + M[1] * c01 + M[2] * c02);
        u0 += (c00 * s0 + (M[2] * M[7] - M[1] * M[8]) * s1 + (M[1] * M[5] - M[2] * M[4]) * s2) * id;
        u1 += (c01 * s0 + (M[0] * M[8] - M[2] * M[6]) * s1 + (M[2] * M[3] - M[0] * M[5]) * s2) * id;
        u2 += (c02 * s0 + (M[1] * M[6] - M[0] * M[7]) * s1 + (M[0] * M[4] - M[1] * M[3]) * s2) * id;
    }
}

template <int PX, int PY, int PZ>
__global__ void __launch_bounds__(BS) gs_q2_f32_kernel(Q2Dims d, const float *__restrict__ Y, float *u,
                                                       const float *__restrict__ b, const uint8_t *__restrict__ dmask,
                                                       int ca, int cb, int cc, int forward) {
    const int ia = ca == 1 ? 2 : 4, ib = cb == 1 ? 2 : 4, ic = cc == 1 ? 2 : 4;
    const int n0 = (d.nn[0] - 1 - ca) / ia + 1, n1 = (d.nn[1] - 1 - cb) / ib + 1, n2 = (d.nn[2] - 1 - cc) / ic + 1;
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (ca >= d.nn[0] || cb >= d.nn[1] || cc >= d.nn[2] || t >= (int64_t)n0 * n1 * n2) return;
    const uint32_t tt = (uint32_t)t, q = tt / (uint32_t)n2;
    const int K = cc + ic * (int)(tt - q * (uint32_t)n2);
    const int J = cb + ib * (int)(q % (uint32_t)n1), I = ca + ia * (int)(q / (uint32_t)n1);
    const int64_t n = q2node(d, I, J, K), ld = d.NN;
    const uint8_t dm = dmask[n];
    if (dm == 7) return;
    float s0 = b[n], s1 = b[ld + n], s2 = b[2 * ld + n];
    float M[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    q2_gather_f32<PX, PY, PZ, true>(d, Y, u, I, J, K, s0, s1, s2, M);
    float u0 = u[n], u1 = u[ld + n], u2 = u[2 * ld + n];
    q2_node_update<float>(dm, s0, s1, s2, M, forward != 0, u0, u1, u2);
    u[n] = u0;
    u[ld + n] = u1;
    u[2 * ld + n] = u2;
}

// Node update of gs_q2_f32_kernel for node (I, J, K) of parity (PX, PY, PZ)
template <int PX, int PY, int PZ>
__device__ __forceinline__ void gs_q2_node_f32(const Q2Dims &d, const float *__restrict__ Y, float *u,
                                               const float *__restrict__ b, const uint8_t *__restrict__ dmask, int I,
                                               int J, int K, int forward) {
    const int64_t n = q2node(d, I, J, K), ld = d.NN;
    const uint8_t dm = dmask[n];
    if (dm == 7) return;
    float s0 = b[n], s1 = b[ld + n], s2 = b[2 * ld + n];
    float M[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    q2_gather_f32<PX, PY, PZ, true>(d, Y, u, I, J, K, s0, s1, s2, M);
    float u0 = u[n], u1 = u[ld + n], u2 = u[2 * ld + n];
    q2_node_update<float>(dm, s0, s1, s2, M, forward != 0, u0, u1, u2);
    u[n] = u0;
    u[ld + n] = u1;
    u[2 * ld + n] = u2;
}

// The three colours (a, b, 0..2) of the FP32 sweep in one launch (2..0 backward): they are
// consecutive in the reference's order, and a node of the class (a, b) couples to the nodes of
// its own class only along its own z-line (the next line of the class is one or two elements
// away on either side), so each block owns linesPerBlock whole lines and runs the three colours
// on them with a block barrier between. The same node updates in the same order as the three
// colour launches, with u read from DRAM once per class instead of once per colour.
template <int PX, int PY>
__global__ void __launch_bounds__(BS, 4) gs_q2_lines_f32_kernel(Q2Dims d, const float *__restrict__ Y, float *u,
                                                             const float *__restrict__ b,
                                                             const uint8_t *__restrict__ dmask, int ca, int cb,
                                                             int linesPerBlock, int forward) {
    const int ia = ca == 1 ? 2 : 4, ib = cb == 1 ? 2 : 4;
    const int n0 = (d.nn[0] - 1 - ca) / ia + 1, n1 = (d.nn[1] - 1 - cb) / ib + 1;
    const int nlines = n0 * n1;
    const int l0 = (int)blockIdx.x * linesPerBlock;
    const int nl = max(0, min(linesPerBlock, nlines - l0));
#pragma unroll 1
    for (int s = 0; s < 3; ++s) {
        const int cc = forward ? s : 2 - s;
        if (cc < d.nn[2]) {
            const int ic = cc == 1 ? 2 : 4;
            const int nk = (d.nn[2] - 1 - cc) / ic + 1;
            const int cnt = nl * nk;
            for (int t = threadIdx.x; t < cnt; t += BS) {
                const int q = t / nk, kk = t - q * nk;
                const int line = l0 + q;
                const int ii = line / n1, jj = line - ii * n1;
                const int I = ca + ia * ii, J = cb + ib * jj, K = cc + ic * kk;
                if (cc == 1) gs_q2_node_f32<PX, PY, 1>(d, Y, u, b, dmask, I, J, K, forward);
                else gs_q2_node_f32<PX, PY, 0>(d, Y, u, b, dmask, I, J, K, forward);
            }
        }
        __syncthreads();
    }
}

// One colour (a, b, c) of the 27-colour block Gauss-Seidel sweep: nodes a + inc_a * s along x
// (inc 4 for corner-type a in {0, 2}, 2 for the middle a = 1), likewise in y and z.
template <typename T>
__global__ void __launch_bounds__(BS) gs_q2_color_kernel(Q2Dims d, const T *Kg, const T *__restrict__ Y, T *u,
                                                         const T *__restrict__ b, const uint8_t *__restrict__ dmask,
                                                         int ca, int cb, int cc, int forward) {
    const int ia = ca == 1 ? 2 : 4, ib = cb == 1 ? 2 : 4, ic = cc == 1 ? 2 : 4;
    const int n0 = (d.nn[0] - 1 - ca) / ia + 1, n1 = (d.nn[1] - 1 - cb) / ib + 1, n2 = (d.nn[2] - 1 - cc) / ic + 1;
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (ca >= d.nn[0] || cb >= d.nn[1] || cc >= d.nn[2] || t >= (int64_t)n0 * n1 * n2) return;
    const uint32_t tt = (uint32_t)t, q = tt / (uint32_t)n2;
    const int K = cc + ic * (int)(tt - q * (uint32_t)n2);
    const int J = cb + ib * (int)(q % (uint32_t)n1), I = ca + ia * (int)(q / (uint32_t)n1);
    const int64_t n = q2node(d, I, J, K), ld = d.NN;
    const uint8_t dm = dmask[n];
    if (dm == 7) return;
    T s0 = b[n], s1 = b[ld + n], s2 = b[2 * ld + n];
    T M[9] = {T(0), T(0), T(0), T(0), T(0), T(0), T(0), T(0), T(0)};
    q2_gather<T, true>(d, Kg, Y, u, I, J, K, s0, s1, s2, M);
    T u0 = u[n], u1 = u[ld + n], u2 = u[2 * ld + n];
    if (dm) {
        // pointwise Gauss-Seidel on the free components (MultigridSolver.hh:352-366)
        T dd[3] = {T(0), T(0), T(0)};
        const T bs[3] = {s0, s1, s2};
        if (forward) {
#pragma unroll
            for (int r = 0; r < 3; ++r)
                dd[r] = (bs[r] - (M[3 * r] * dd[0] + M[3 * r + 1] * dd[1] + M[3 * r + 2] * dd[2])) *
                        (T(!((dm >> r) & 1)) / M[4 * r]);
        } else {
#pragma unroll
            for (int r = 2; r >= 0; --r)
                dd[r] = (bs[r] - (M[3 * r] * dd[0] + M[3 * r + 1] * dd[1] + M[3 * r + 2] * dd[2])) *
                        (T(!((dm >> r) & 1)) / M[4 * r]);
        }
        u0 += dd[0];
        u1 += dd[1];
        u2 += dd[2];
    } else {
        const T c00 = M[4] * M[8] - M[5] * M[7], c01 = M[5] * M[6] - M[3] * M[8], c02 = M[3] * M[7] - M[4] * M[6];
        const T id = T(1) / (M[0] * c00 + M[1] * c01 + M[2] * c02);
        u0 += (c00 * s0 + (M[2] * M[7] - M[1] * M[8]) * s1 + (M[1] * M[5] - M[2] * M[4]) * s2) * id;
        u1 += (c01 * s0 + (M[0] * M[8] - M[2] * M[6]) * s1 + (M[2] * M[3] - M[0] * M[5]) * s2) * id;
        u2 += (c02 * s0 + (M[1] * M[6] - M[0] * M[7]) * s1 + (M[0] * M[4] - M[1] * M[3]) * s2) * id;
    }
    u[n] = u0;
    u[ld + n] = u1;
    u[2 * ld + n] = u2;
}

// Weights of the coarse Q2 shape functions lc = 0, 1, 2 at the fine node with local position
// t = f - 4e in 0..4 of its coarse element e (reference coordinate t / 4): N0 = 2 (x - 1/2)(x - 1),
// N1 = -4 x (x - 1), N2 = 2 x (x - 1/2). All are dyadic, exact in FP32.
__device__ __forceinline__ double q2_axis_weight(int t, int lc) {
    switch (3 * t + lc) {
    case 0: return 1.0;
    case 3: return 0.375;
    case 4: return 0.75;
    case 5: return -0.125;
    case 7: return 1.0;
    case 9: return -0.125;
    case 10: return 0.75;
    case 11: return 0.375;
    case 14: return 1.0;
    default: return 0.0;
    }
}

// Coarse nodes (base + lc) and weights of fine node f along one axis: one node for an even local
// position (coinciding nodes), three for an odd one.
template <typename T>
__device__ __forceinline__ int q2_axis(int f, int nec, int &base, int *lc, T *w) {
    int e = f >> 2;
    if (e >= nec) e = nec - 1;
    base = 2 * e;
    const int t = f - 4 * e;
    if (!(t & 1)) {
        lc[0] = t >> 1;
        w[0] = T(1);
        return 1;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        lc[c] = c;
        w[c] = (T)q2_axis_weight(t, c);
    }
    return 3;
}

// fine (=|+=) P coarse: the coarse Q2 interpolant evaluated at the fine nodes (MultigridSolver.hh:137-212),
// summed in the vectors' precision
template <typename T>
__global__ void __launch_bounds__(BS) interp_q2_kernel(Q2Dims df, Q2Dims dc, const T *__restrict__ coarse,
                                                       T *__restrict__ fine, int accumulate) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= df.NN) return;
    const uint32_t tt = (uint32_t)t, q = tt / (uint32_t)df.nn[2];
    const int F[3] = {(int)(q / (uint32_t)df.nn[1]), (int)(q % (uint32_t)df.nn[1]), (int)(tt - q * (uint32_t)df.nn[2])};
    int base[3], lc[3][3], cnt[3];
    T w[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) cnt[a] = q2_axis<T>(F[a], dc.ne[a], base[a], lc[a], w[a]);
    T acc[3] = {T(0), T(0), T(0)};
    for (int a = 0; a < cnt[0]; ++a)
        for (int b = 0; b < cnt[1]; ++b) {
            const T wab = w[0][a] * w[1][b];
            for (int c = 0; c < cnt[2]; ++c) {
                const T wt = wab * w[2][c];
                const int64_t cn = q2node(dc, base[0] + lc[0][a], base[1] + lc[1][b], base[2] + lc[2][c]);
#pragma unroll
                for (int r = 0; r < 3; ++r) acc[r] += wt * coarse[r * dc.NN + cn];
            }
        }
    const int64_t n = q2node(df, F[0], F[1], F[2]);
#pragma unroll
    for (int r = 0; r < 3; ++r) fine[r * df.NN + n] = (accumulate ? fine[r * df.NN + n] : T(0)) + acc[r];
}

// coarse = P^T fine: coarse node C gathers the fine nodes [2C - 3, 2C + 3] (per axis) whose
// interpolation stencil contains it, with the same weights (MultigridSolver.hh:217-275)
template <typename T>
__global__ void __launch_bounds__(BS) restrict_q2_kernel(Q2Dims df, Q2Dims dc, const T *__restrict__ fine,
                                                         T *__restrict__ coarse) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= dc.NN) return;
    const uint32_t tt = (uint32_t)t, q = tt / (uint32_t)dc.nn[2];
    const int C[3] = {(int)(q / (uint32_t)dc.nn[1]), (int)(q % (uint32_t)dc.nn[1]), (int)(tt - q * (uint32_t)dc.nn[2])};
    int fo[3][7], cnt[3];
    T wt[3][7];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        cnt[a] = 0;
#pragma unroll
        for (int s = 0; s < 7; ++s) {
            const int f = 2 * C[a] - 3 + s;
            if (f < 0 || f >= df.nn[a]) continue;
            int e = f >> 2;
            if (e >= dc.ne[a]) e = dc.ne[a] - 1;
            const int lc = C[a] - 2 * e;
            if (lc < 0 || lc > 2) continue;
            const double wv = q2_axis_weight(f - 4 * e, lc);
            if (wv == 0.0) continue;
            fo[a][cnt[a]] = f;
            wt[a][cnt[a]] = (T)wv;
            ++cnt[a];
        }
    }
    T acc[3] = {T(0), T(0), T(0)};
    for (int s = 0; s < cnt[0]; ++s)
        for (int v = 0; v < cnt[1]; ++v) {
            const T wsv = wt[0][s] * wt[1][v];
            for (int z = 0; z < cnt[2]; ++z) {
                const T w = wsv * wt[2][z];
                const int64_t fn = q2node(df, fo[0][s], fo[1][v], fo[2][z]);
#pragma unroll
                for (int r = 0; r < 3; ++r) acc[r] += w * fine[r * df.NN + fn];
            }
        }
    const int64_t cn = q2node(dc, C[0], C[1], C[2]);
#pragma unroll
    for (int r = 0; r < 3; ++r) coarse[r * dc.NN + cn] = acc[r];
}

// ---- Q2 <-> Q1 on the same mesh (the p-multigrid step of the Q2 preconditioner) ----
// Q1 nodes are the even-indexed Q2 nodes; the trilinear interpolant at a Q2 node is the
// tensor product of weight 1 (even index 2i -> i) and 1/2, 1/2 (odd index 2i+1 -> i, i+1).
template <typename T>
__global__ void __launch_bounds__(BS) interp_q1_q2_kernel(Q2Dims d, const T *__restrict__ q1, T *__restrict__ q2,
                                                          int accumulate) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= d.NN) return;
    const uint32_t tt = (uint32_t)t, q = tt / (uint32_t)d.nn[2];
    const int F[3] = {(int)(q / (uint32_t)d.nn[1]), (int)(q % (uint32_t)d.nn[1]), (int)(tt - q * (uint32_t)d.nn[2])};
    const int n1[3] = {d.ne[0] + 1, d.ne[1] + 1, d.ne[2] + 1};
    const int64_t N1 = (int64_t)n1[0] * n1[1] * n1[2];
    int lo[3], cnt[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lo[a] = F[a] >> 1;
        cnt[a] = (F[a] & 1) ? 2 : 1;
    }
    T acc[3] = {T(0), T(0), T(0)};
    const T w = T(1) / T(cnt[0] * cnt[1] * cnt[2]);
    for (int a = 0; a < cnt[0]; ++a)
        for (int b = 0; b < cnt[1]; ++b)
            for (int c = 0; c < cnt[2]; ++c) {
                const int64_t m = ((int64_t)(lo[0] + a) * n1[1] + lo[1] + b) * n1[2] + lo[2] + c;
#pragma unroll
                for (int r = 0; r < 3; ++r) acc[r] += q1[r * N1 + m];
            }
    const int64_t n = q2node(d, F[0], F[1], F[2]);
#pragma unroll
    for (int r = 0; r < 3; ++r) q2[r * d.NN + n] = (accumulate ? q2[r * d.NN + n] : T(0)) + w * acc[r];
}

template <typename T>
__global__ void __launch_bounds__(BS) restrict_q2_q1_kernel(Q2Dims d, const T *__restrict__ q2, T *__restrict__ q1) {
    const int n1[3] = {d.ne[0] + 1, d.ne[1] + 1, d.ne[2] + 1};
    const int64_t N1 = (int64_t)n1[0] * n1[1] * n1[2];
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= N1) return;
    const uint32_t tt = (uint32_t)t, q = tt / (uint32_t)n1[2];
    const int C[3] = {(int)(q / (uint32_t)n1[1]), (int)(q % (uint32_t)n1[1]), (int)(tt - q * (uint32_t)n1[2])};
    T acc[3] = {T(0), T(0), T(0)};
    for (int a = -1; a <= 1; ++a) {
        const int I = 2 * C[0] + a;
        if (I < 0 || I >= d.nn[0]) continue;
        const T wa = a ? T(0.5) : T(1);
        for (int b = -1; b <= 1; ++b) {
            const int J = 2 * C[1] + b;
            if (J < 0 || J >= d.nn[1]) continue;
            const T wb = b ? T(0.5) : T(1);
            for (int c = -1; c <= 1; ++c) {
                const int K = 2 * C[2] + c;
                if (K < 0 || K >= d.nn[2]) continue;
                const T w = wa * wb * (c ? T(0.5) : T(1));
                const int64_t n = q2node(d, I, J, K);
#pragma unroll
                for (int r = 0; r < 3; ++r) acc[r] += w * q2[r * d.NN + n];
            }
        }
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) q1[r * N1 + t] = acc[r];
}

// r = b - Ku on the free components (Ku already masked to zero on constrained ones)
template <typename T>
__global__ void __launch_bounds__(BS) q2_residual_combine_kernel(int64_t NN, const T *__restrict__ b,
                                                                 const T *__restrict__ Ku, T *__restrict__ r,
                                                                 const uint8_t *__restrict__ dmask) {
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n >= NN) return;
    const uint8_t dm = dmask[n];
#pragma unroll
    for (int c = 0; c < 3; ++c) r[c * NN + n] = ((dm >> c) & 1) ? T(0) : b[c * NN + n] - Ku[c * NN + n];
}

// ---- the triquadratic multigrid hierarchy (MultigridSolver<double, 2, 2, 2>) ----
// Levels below the fine one hold one 81 x 81 element matrix per element, element-major
// (Ke[e * 6561 + 81 r + c]), as the operator that the reference applies through its level-1
// stencil (the 8 coarsened full-density matrices weighted by the fine moduli) and its blockK.

// Level 1: Ke[e] = sum_f Y[child_f(e)] Kc_f over the 8 children f = 4 fx + 2 fy + fz
// (MultigridSolver.hh:724-738)
template <typename T>
__global__ void __launch_bounds__(BS) q2mg_level1_kernel(Q2Dims dc, Q2Dims df, const T *__restrict__ Kc,
                                                         const T *__restrict__ Y, T *__restrict__ Ke) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= dc.NE * 6561) return;
    const int64_t e = t / 6561;
    const int q = (int)(t - e * 6561);
    const int ck = (int)(e % dc.ne[2]), cj = (int)((e / dc.ne[2]) % dc.ne[1]), ci = (int)(e / ((int64_t)dc.ne[1] * dc.ne[2]));
    T acc = T(0);
#pragma unroll
    for (int f = 0; f < 8; ++f) {
        const int64_t ef = ((int64_t)(2 * ci + (f >> 2 & 1)) * df.ne[1] + 2 * cj + (f >> 1 & 1)) * df.ne[2] + 2 * ck + (f & 1);
        const T v = __ldg(Y + ef) * __ldg(Kc + f * 6561 + q);
        acc = f == 0 ? v : acc + v;
    }
    Ke[t] = acc;
}

// Level l >= 2: Ke_c[e] = sum_f I_f^T Ke_f[child_f(e)] I_f (MultigridSolver.hh:712-722, 745-819).
// I_f[3i + c, 3j + d] = phi_f(i, j) delta_cd; phi_f(i, j) is a product of 1-D weights with at
// most 2 nonzeros per coarse node and axis, so a coarse node j draws on at most 8 fine nodes i.
// One CTA per coarse element; the child's matrix and the right product I_f stage in shared
// memory, the left product accumulates in registers (26 entries per thread).
constexpr int GAL_THREADS = 256;
constexpr int GAL_PER_THREAD = (6561 + GAL_THREADS - 1) / GAL_THREADS;

template <typename T>
__global__ void __launch_bounds__(GAL_THREADS) q2mg_galerkin_kernel(Q2Dims dc, Q2Dims df, const T *__restrict__ Kf,
                                                                    T *__restrict__ Kc) {
    extern __shared__ __align__(16) unsigned char gal_smem[];
    T *S = reinterpret_cast<T *>(gal_smem);
    T *Tm = S + 6561;
    T *nzw = Tm + 6561;                                     // [27][8] weights
    int *nzi = reinterpret_cast<int *>(nzw + 27 * 8);       // [27][8] fine local nodes
    int *nzc = nzi + 27 * 8;                                // [27] counts
    const int64_t e = blockIdx.x;
    const int ck = (int)(e % dc.ne[2]), cj = (int)((e / dc.ne[2]) % dc.ne[1]), ci = (int)(e / ((int64_t)dc.ne[1] * dc.ne[2]));
    T acc[GAL_PER_THREAD];
#pragma unroll
    for (int s = 0; s < GAL_PER_THREAD; ++s) acc[s] = T(0);
    for (int f = 0; f < 8; ++f) {
        const int fd[3] = {f >> 2 & 1, f >> 1 & 1, f & 1};
        const int64_t ef = ((int64_t)(2 * ci + fd[0]) * df.ne[1] + 2 * cj + fd[1]) * df.ne[2] + 2 * ck + fd[2];
        const T *src = Kf + ef * 6561;
        for (int q = threadIdx.x; q < 6561; q += GAL_THREADS) S[q] = src[q];
        if (threadIdx.x < 27) {
            // nonzeros of column j of phi_f, fine local node i ascending
            const int j = threadIdx.x, ja[3] = {j / 9, (j / 3) % 3, j % 3};
            int n = 0;
            for (int a = 0; a < 3; ++a) {
                const double wa = q2_axis_weight(2 * fd[0] + a, ja[0]);
                if (wa == 0.0) continue;
                for (int b = 0; b < 3; ++b) {
                    const double wb = q2_axis_weight(2 * fd[1] + b, ja[1]);
                    if (wb == 0.0) continue;
                    for (int c = 0; c < 3; ++c) {
                        const double wc = q2_axis_weight(2 * fd[2] + c, ja[2]);
                        if (wc == 0.0) continue;
                        nzw[8 * j + n] = (T)(wa * wb * wc);
                        nzi[8 * j + n] = 9 * a + 3 * b + c;
                        ++n;
                    }
                }
            }
            nzc[j] = n;
        }
        __syncthreads();
        // Tm[r][3 j + d] = sum_i S[r][3 i + d] phi_f(i, j)
        for (int q = threadIdx.x; q < 6561; q += GAL_THREADS) {
            const int r = q / 81, cc = q - 81 * r, j = cc / 3, d = cc - 3 * j;
            T v = T(0);
            for (int t = 0; t < nzc[j]; ++t) v += S[81 * r + 3 * nzi[8 * j + t] + d] * nzw[8 * j + t];
            Tm[q] = v;
        }
        __syncthreads();
        // acc[3 j + c][q] += sum_i phi_f(i, j) Tm[3 i + c][q]
#pragma unroll
        for (int s = 0; s < GAL_PER_THREAD; ++s) {
            const int q = threadIdx.x + GAL_THREADS * s;
            if (q < 6561) {
                const int R = q / 81, Q = q - 81 * R, j = R / 3, c = R - 3 * j;
                T v = T(0);
                for (int t = 0; t < nzc[j]; ++t) v += nzw[8 * j + t] * Tm[81 * (3 * nzi[8 * j + t] + c) + Q];
                acc[s] += v;
            }
        }
        __syncthreads();
    }
    T *dst = Kc + e * 6561;
#pragma unroll
    for (int s = 0; s < GAL_PER_THREAD; ++s) {
        const int q = threadIdx.x + GAL_THREADS * s;
        if (q < 6561) dst[q] = acc[s];
    }
}

// Incident elements of node I along one axis in ascending element order (local coordinate 2 in
// element I/2 - 1, then 0 in element I/2; 1 in element (I-1)/2 for an odd I)
__device__ __forceinline__ int axis_elems_asc(int I, int ne, int *ei, int *la) {
    if (I & 1) {
        ei[0] = (I - 1) >> 1;
        la[0] = 1;
        return 1;
    }
    int n = 0;
    if ((I >> 1) - 1 >= 0) { ei[n] = (I >> 1) - 1; la[n] = 2; ++n; }
    if ((I >> 1) < ne) { ei[n] = I >> 1; la[n] = 0; ++n; }
    return n;
}

// Offsets of an element's 81 nodal values (column 3 m + comp, m = 9 a + 3 b + c) from its
// first node's x-component, for the level's node layout; filled by the first 81 threads.
__device__ __forceinline__ void q2mg_column_offsets(const Q2Dims &d, int *off) {
    const int t = threadIdx.x;
    if (t < 81) {
        const int m = t / 3, comp = t - 3 * m;
        off[t] = (int)(comp * d.NN + ((int64_t)(m / 9) * d.nn[1] + (m / 3) % 3) * d.nn[2] + m % 3);
    }
}

// Incident element slot s (0..N-1) of node I along one axis: N = 1 for an odd I (local 1 of
// element (I-1)/2), N = 2 for an even I (local 2 of element I/2 - 1, then local 0 of element
// I/2). Returns false when the slot's element lies outside the grid.
template <int N>
__device__ __forceinline__ bool axis_slot(int I, int ne, int s, int &e, int &l) {
    if (N == 1) {
        e = (I - 1) >> 1;
        l = 1;
        return true;
    }
    e = (I >> 1) - 1 + s;
    l = s ? 0 : 2;
    return e >= 0 && e < ne;
}

// One warp per node: s_r = sum over the incident elements of row 3 ln + r of Ke times the
// element's nodal values. The number of incident elements per axis (NX, NY, NZ: 1 for an odd
// coordinate, 2 for an even one) is fixed per launch; a slot outside the grid reads the zero
// element matrix stored after the last element (index NE), so every launch runs the same fully
// unrolled loop and the loads of successive elements overlap. Lane t takes columns t, t + 32,
// t + 64 of the 3 rows (each nodal value loaded once for its 3 products); lanes 0..8 also sum the
// 3 x 3 diagonal block M (lane 3 r + c). The sums end reduced over the warp in every lane.
template <typename T, int NX, int NY, int NZ>
__device__ __forceinline__ void q2mg_node_rows(const Q2Dims &d, const T *__restrict__ Ke, const T *u,
                                               const int *off, int I, int J, int K, int lane, T &a0, T &a1, T &a2,
                                               T &mv) {
    const int o0 = off[lane], o1 = off[lane + 32], o2 = lane < 17 ? off[lane + 64] : 0;
#pragma unroll
    for (int sa = 0; sa < NX; ++sa)
#pragma unroll
        for (int sb = 0; sb < NY; ++sb)
#pragma unroll
            for (int sc = 0; sc < NZ; ++sc) {
                int eX, eY, eZ, lX, lY, lZ;
                const bool in = axis_slot<NX>(I, d.ne[0], sa, eX, lX) & axis_slot<NY>(J, d.ne[1], sb, eY, lY) &
                                axis_slot<NZ>(K, d.ne[2], sc, eZ, lZ);
                const int ln = 9 * lX + 3 * lY + lZ;
                const int64_t e = in ? ((int64_t)eX * d.ne[1] + eY) * d.ne[2] + eZ : d.NE;
                const T *Kr = Ke + e * 6561 + 243 * ln;
                const T *ub = u + (in ? q2node(d, 2 * eX, 2 * eY, 2 * eZ) : 0);
                T v = ub[o0];
                a0 += __ldg(Kr + lane) * v;
                a1 += __ldg(Kr + 81 + lane) * v;
                a2 += __ldg(Kr + 162 + lane) * v;
                v = ub[o1];
                a0 += __ldg(Kr + 32 + lane) * v;
                a1 += __ldg(Kr + 113 + lane) * v;
                a2 += __ldg(Kr + 194 + lane) * v;
                if (lane < 17) {
                    v = ub[o2];
                    a0 += __ldg(Kr + 64 + lane) * v;
                    a1 += __ldg(Kr + 145 + lane) * v;
                    a2 += __ldg(Kr + 226 + lane) * v;
                }
                if (lane < 9) mv += __ldg(Kr + 81 * (lane / 3) + 3 * ln + lane % 3);
            }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
}

// One colour (a, b, c) of the 27-colour block Gauss-Seidel sweep on a level with element
// matrices (NodeSmoothStencilSecondFinest / NodeSmoothStencilBlockK, MultigridSolver.hh:294-378);
// NX = 1 for the middle colour a = 1, else 2 (likewise NY, NZ)
template <typename T, int NX, int NY, int NZ>
__global__ void __launch_bounds__(BS) q2mg_gs_kernel(Q2Dims d, const T *__restrict__ Ke, T *u,
                                                     const T *__restrict__ b, const uint8_t *__restrict__ dmask,
                                                     int ca, int cb, int cc, int forward) {
    __shared__ int off[81];
    q2mg_column_offsets(d, off);
    __syncthreads();
    const int ia = ca == 1 ? 2 : 4, ib = cb == 1 ? 2 : 4, ic = cc == 1 ? 2 : 4;
    const int n0 = (d.nn[0] - 1 - ca) / ia + 1, n1 = (d.nn[1] - 1 - cb) / ib + 1, n2 = (d.nn[2] - 1 - cc) / ic + 1;
    const int64_t w = (blockIdx.x * (int64_t)BS + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= (int64_t)n0 * n1 * n2) return;  // uniform over the warp
    const int64_t q = w / n2;
    const int K = cc + ic * (int)(w - q * n2);
    const int J = cb + ib * (int)(q % n1), I = ca + ia * (int)(q / n1);
    const int64_t n = q2node(d, I, J, K), ld = d.NN;
    const uint8_t dm = dmask[n];
    if (dm == 7) return;
    T a0 = T(0), a1 = T(0), a2 = T(0), mv = T(0);
    q2mg_node_rows<T, NX, NY, NZ>(d, Ke, u, off, I, J, K, lane, a0, a1, a2, mv);
    T M[9];
#pragma unroll
    for (int t = 0; t < 9; ++t) M[t] = __shfl_sync(0xffffffffu, mv, t);
    if (lane == 0) {
        T u0 = u[n], u1 = u[ld + n], u2 = u[2 * ld + n];
        q2_node_update<T>(dm, b[n] - a0, b[ld + n] - a1, b[2 * ld + n] - a2, M, forward != 0, u0, u1, u2);
        u[n] = u0;
        u[ld + n] = u1;
        u[2 * ld + n] = u2;
    }
}

// out = K u (Residual: out = b - K u) at the nodes of one parity class (PX, PY, PZ: odd
// coordinates), zero on the constrained components when zeroDirichlet (computeResidual,
// MultigridSolver.hh:527-541); one warp per node
template <typename T, bool Residual, int PX, int PY, int PZ>
__global__ void __launch_bounds__(BS) q2mg_apply_kernel(Q2Dims d, const T *__restrict__ Ke, const T *__restrict__ u,
                                                        const T *__restrict__ b, T *__restrict__ out,
                                                        const uint8_t *__restrict__ dmask, int zeroDirichlet) {
    __shared__ int off[81];
    q2mg_column_offsets(d, off);
    __syncthreads();
    const int n0 = (d.nn[0] - PX + 1) / 2, n1 = (d.nn[1] - PY + 1) / 2, n2 = (d.nn[2] - PZ + 1) / 2;
    const int64_t w = (blockIdx.x * (int64_t)BS + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= (int64_t)n0 * n1 * n2) return;
    const int64_t q = w / n2;
    const int K = 2 * (int)(w - q * n2) + PZ, J = 2 * (int)(q % n1) + PY, I = 2 * (int)(q / n1) + PX;
    T a0 = T(0), a1 = T(0), a2 = T(0), mv = T(0);
    q2mg_node_rows<T, 2 - PX, 2 - PY, 2 - PZ>(d, Ke, u, off, I, J, K, lane, a0, a1, a2, mv);
    if (lane == 0) {
        const int64_t n = q2node(d, I, J, K);
        const uint8_t dm = zeroDirichlet ? dmask[n] : 0;
        const T v[3] = {a0, a1, a2};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const T r = Residual ? b[c * d.NN + n] - v[c] : v[c];
            out[c * d.NN + n] = ((dm >> c) & 1) ? T(0) : r;
        }
    }
}

// Dense reduced coarsest operator: one thread per free row (DOF 3 n + c), summing its element
// rows over the incident elements in ascending order (TensorProductSimulator.hh:1198-1230)
template <typename T>
__global__ void __launch_bounds__(BS) q2mg_dense_kernel(Q2Dims d, const T *__restrict__ Ke, const int *__restrict__ freeIdx,
                                                        const int *__restrict__ redIdx, int nfree, double *A) {
    const int i = blockIdx.x * BS + threadIdx.x;
    if (i >= nfree) return;
    const int dof = freeIdx[i], n = dof / 3, c = dof - 3 * n;
    const int K = n % d.nn[2], J = (n / d.nn[2]) % d.nn[1], I = n / (d.nn[2] * d.nn[1]);
    int ex[2], lx[2], ey[2], ly[2], ez[2], lz[2];
    const int cx = axis_elems_asc(I, d.ne[0], ex, lx), cy = axis_elems_asc(J, d.ne[1], ey, ly),
              cz = axis_elems_asc(K, d.ne[2], ez, lz);
    double *row = A + (int64_t)i * nfree;
    for (int a = 0; a < cx; ++a)
        for (int b = 0; b < cy; ++b)
            for (int z = 0; z < cz; ++z) {
                const int64_t e = ((int64_t)ex[a] * d.ne[1] + ey[b]) * d.ne[2] + ez[z];
                const int ln = 9 * lx[a] + 3 * ly[b] + lz[z];
                const T *Kr = Ke + e * 6561 + 81 * (3 * ln + c);
                for (int m = 0; m < 27; ++m) {
                    const int64_t nm = q2node(d, 2 * ex[a] + m / 9, 2 * ey[b] + (m / 3) % 3, 2 * ez[z] + m % 3);
                    for (int dd = 0; dd < 3; ++dd) {
                        const int col = redIdx[3 * nm + dd];
                        if (col >= 0) row[col] += (double)Kr[3 * m + dd];
                    }
                }
            }
}

Q2Dims dims_of(const int ne[3]) {
    Q2Dims d;
    for (int a = 0; a < 3; ++a) {
        d.ne[a] = ne[a];
        d.nn[a] = 2 * ne[a] + 1;
    }
    d.NN = (int64_t)d.nn[0] * d.nn[1] * d.nn[2];
    d.NE = (int64_t)ne[0] * ne[1] * ne[2];
    return d;
}

}  // namespace

void q2_upload_k0f(const float *K0f, cudaStream_t st) {
    VFEM_CUDA(cudaMemcpyToSymbolAsync(c_K0q2f, K0f, sizeof(float) * 81 * 81, 0, cudaMemcpyHostToDevice, st));
}

void q2_upload_k0lo(const float *K0lo, cudaStream_t st) {
    VFEM_CUDA(cudaMemcpyToSymbolAsync(c_K0q2lo, K0lo, sizeof(float) * 81 * 81, 0, cudaMemcpyHostToDevice, st));
}

void launch_applyk_q2_df(const int ne[3], const float *Yh, const float *Yl, const float *uh, const float *ul,
                         double *out, const uint8_t *dmask, bool zeroDirichlet, cudaStream_t st) {
    const Q2Dims d = dims_of(ne);
    const int64_t per = (int64_t)(ne[0] + 1) * (ne[1] + 1) * (ne[2] + 1);
    const unsigned gs = gridFor(per, BS);
    const int zd = zeroDirichlet ? 1 : 0;
    applyk_q2_df_kernel<0, 0, 0><<<gs, BS, 0, st>>>(d, Yh, Yl, uh, ul, out, dmask, zd);
    applyk_q2_df_kernel<0, 0, 1><<<gs, BS, 0, st>>>(d, Yh, Yl, uh, ul, out, dmask, zd);
    applyk_q2_df_kernel<0, 1, 0><<<gs, BS, 0, st>>>(d, Yh, Yl, uh, ul, out, dmask, zd);
    applyk_q2_df_kernel<0, 1, 1><<<gs, BS, 0, st>>>(d, Yh, Yl, uh, ul, out, dmask, zd);
    applyk_q2_df_kernel<1, 0, 0><<<gs, BS, 0, st>>>(d, Yh, Yl, uh, ul, out, dmask, zd);
    applyk_q2_df_kernel<1, 0, 1><<<gs, BS, 0, st>>>(d, Yh, Yl, uh, ul, out, dmask, zd);
    applyk_q2_df_kernel<1, 1, 0><<<gs, BS, 0, st>>>(d, Yh, Yl, uh, ul, out, dmask, zd);
    applyk_q2_df_kernel<1, 1, 1><<<gs, BS, 0, st>>>(d, Yh, Yl, uh, ul, out, dmask, zd);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_applyk_q2(const int ne[3], const T *K0, const T *Y, const T *u, T *out, const uint8_t *dmask,
                      bool zeroDirichlet, cudaStream_t st) {
    const Q2Dims d = dims_of(ne);
    const int64_t per = (int64_t)(ne[0] + 1) * (ne[1] + 1) * (ne[2] + 1);  // largest parity class
    if constexpr (std::is_same<T, float>::value) {
        const unsigned gs = gridFor(per, BS);
        const int zd = zeroDirichlet ? 1 : 0;
        applyk_q2_f32_kernel<0, 0, 0><<<gs, BS, 0, st>>>(d, Y, u, out, dmask, zd);
        applyk_q2_f32_kernel<0, 0, 1><<<gs, BS, 0, st>>>(d, Y, u, out, dmask, zd);
        applyk_q2_f32_kernel<0, 1, 0><<<gs, BS, 0, st>>>(d, Y, u, out, dmask, zd);
        applyk_q2_f32_kernel<0, 1, 1><<<gs, BS, 0, st>>>(d, Y, u, out, dmask, zd);
        applyk_q2_f32_kernel<1, 0, 0><<<gs, BS, 0, st>>>(d, Y, u, out, dmask, zd);
        applyk_q2_f32_kernel<1, 0, 1><<<gs, BS, 0, st>>>(d, Y, u, out, dmask, zd);
        applyk_q2_f32_kernel<1, 1, 0><<<gs, BS, 0, st>>>(d, Y, u, out, dmask, zd);
        applyk_q2_f32_kernel<1, 1, 1><<<gs, BS, 0, st>>>(d, Y, u, out, dmask, zd);
    } else {
        applyk_q2_kernel<T><<<dim3(gridFor(per, BS), 8), BS, 0, st>>>(d, K0, Y, u, out, dmask, zeroDirichlet ? 1 : 0);
    }
    VFEM_LAUNCH_CHECK();
}

// Form of the FP32 triquadratic sweep: one launch per (a, b) class with its three colours on
// whole z-lines (default), or one launch per colour (VFEM_Q2_GS_FORM=colours).
static bool q2GsLines() {
    const char *e = std::getenv("VFEM_Q2_GS_FORM");
    return !(e && std::strcmp(e, "colours") == 0);
}

template <int PX, int PY>
static void gs_q2_lines(const Q2Dims &d, const float *Y, float *u, const float *b, const uint8_t *dmask, int ca,
                        int cb, bool forward, cudaStream_t st) {
    const int ia = ca == 1 ? 2 : 4, ib = cb == 1 ? 2 : 4;
    const int nlines = ((d.nn[0] - 1 - ca) / ia + 1) * ((d.nn[1] - 1 - cb) / ib + 1);
    // lines per block (VFEM_Q2_LINES_PER_BLOCK): on the 128^3 grid a sweep took 3.46 ms with 2,
    // 3.89 ms with 4, 4.24 ms with 3, 5.49 ms with 1, against 4.27 ms for the 27 colour launches
    int lpb = 2;
    if (const char *e = std::getenv("VFEM_Q2_LINES_PER_BLOCK")) lpb = std::max(1, std::atoi(e));
    const unsigned blocks = (unsigned)((nlines + lpb - 1) / lpb);
    gs_q2_lines_f32_kernel<PX, PY><<<blocks, BS, 0, st>>>(d, Y, u, b, dmask, ca, cb, lpb, forward ? 1 : 0);
}

template <typename T>
void launch_gs_q2_sweep(const int ne[3], const T *K0, const T *Y, T *u, const T *b, const uint8_t *dmask, bool forward,
                        cudaStream_t st) {
    const Q2Dims d = dims_of(ne);
    if constexpr (std::is_same<T, float>::value) {
        if (q2GsLines()) {
            for (int s = 0; s < 9; ++s) {
                const int cls = forward ? s : 8 - s;
                const int ca = cls / 3, cb = cls % 3;
                if (ca >= d.nn[0] || cb >= d.nn[1]) continue;
                switch (2 * (ca == 1) + (cb == 1)) {
                case 0: gs_q2_lines<0, 0>(d, Y, u, b, dmask, ca, cb, forward, st); break;
                case 1: gs_q2_lines<0, 1>(d, Y, u, b, dmask, ca, cb, forward, st); break;
                case 2: gs_q2_lines<1, 0>(d, Y, u, b, dmask, ca, cb, forward, st); break;
                default: gs_q2_lines<1, 1>(d, Y, u, b, dmask, ca, cb, forward, st); break;
                }
                VFEM_LAUNCH_CHECK();
            }
            return;
        }
    }
    for (int s = 0; s < 27; ++s) {
        const int col = forward ? s : 26 - s;
        const int ca = col / 9, cb = (col / 3) % 3, cc = col % 3;
        const int ia = ca == 1 ? 2 : 4, ib = cb == 1 ? 2 : 4, ic = cc == 1 ? 2 : 4;
        if (ca >= d.nn[0] || cb >= d.nn[1] || cc >= d.nn[2]) continue;
        const int64_t cnt = (int64_t)((d.nn[0] - 1 - ca) / ia + 1) * ((d.nn[1] - 1 - cb) / ib + 1) *
                            ((d.nn[2] - 1 - cc) / ic + 1);
        const unsigned gs = gridFor(cnt, BS);
        const int fw = forward ? 1 : 0;
        if constexpr (std::is_same<T, float>::value) {
            const int px = ca == 1, py = cb == 1, pz = cc == 1;
            switch (4 * px + 2 * py + pz) {
            case 0: gs_q2_f32_kernel<0, 0, 0><<<gs, BS, 0, st>>>(d, Y, u, b, dmask, ca, cb, cc, fw); break;
            case 1: gs_q2_f32_kernel<0, 0, 1><<<gs, BS, 0, st>>>(d, Y, u, b, dmask, ca, cb, cc, fw); break;
            case 2: gs_q2_f32_kernel<0, 1, 0><<<gs, BS, 0, st>>>(d, Y, u, b, dmask, ca, cb, cc, fw); break;
            case 3: gs_q2_f32_kernel<0, 1, 1><<<gs, BS, 0, st>>>(d, Y, u, b, dmask, ca, cb, cc, fw); break;
            case 4: gs_q2_f32_kernel<1, 0, 0><<<gs, BS, 0, st>>>(d, Y, u, b, dmask, ca, cb, cc, fw); break;
            case 5: gs_q2_f32_kernel<1, 0, 1><<<gs, BS, 0, st>>>(d, Y, u, b, dmask, ca, cb, cc, fw); break;
            case 6: gs_q2_f32_kernel<1, 1, 0><<<gs, BS, 0, st>>>(d, Y, u, b, dmask, ca, cb, cc, fw); break;
            default: gs_q2_f32_kernel<1, 1, 1><<<gs, BS, 0, st>>>(d, Y, u, b, dmask, ca, cb, cc, fw); break;
            }
        } else {
            gs_q2_color_kernel<T><<<gs, BS, 0, st>>>(d, K0, Y, u, b, dmask, ca, cb, cc, fw);
        }
        VFEM_LAUNCH_CHECK();
    }
}

template <typename T>
void launch_restrict_q2(const int neFine[3], const T *fine, T *coarse, cudaStream_t st) {
    const int nec[3] = {neFine[0] / 2, neFine[1] / 2, neFine[2] / 2};
    const Q2Dims df = dims_of(neFine), dc = dims_of(nec);
    restrict_q2_kernel<T><<<gridFor(dc.NN, BS), BS, 0, st>>>(df, dc, fine, coarse);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_interp_q2(const int neFine[3], const T *coarse, T *fine, bool accumulate, cudaStream_t st) {
    const int nec[3] = {neFine[0] / 2, neFine[1] / 2, neFine[2] / 2};
    const Q2Dims df = dims_of(neFine), dc = dims_of(nec);
    interp_q2_kernel<T><<<gridFor(df.NN, BS), BS, 0, st>>>(df, dc, coarse, fine, accumulate ? 1 : 0);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_interp_q1_q2(const int ne[3], const T *q1, T *q2, bool accumulate, cudaStream_t st) {
    const Q2Dims d = dims_of(ne);
    interp_q1_q2_kernel<T><<<gridFor(d.NN, BS), BS, 0, st>>>(d, q1, q2, accumulate ? 1 : 0);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_restrict_q2_q1(const int ne[3], const T *q2, T *q1, cudaStream_t st) {
    const Q2Dims d = dims_of(ne);
    restrict_q2_q1_kernel<T><<<gridFor((int64_t)(ne[0] + 1) * (ne[1] + 1) * (ne[2] + 1), BS), BS, 0, st>>>(d, q2, q1);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_q2_residual_combine(int64_t NN, const T *b, const T *Ku, T *r, const uint8_t *dmask, cudaStream_t st) {
    q2_residual_combine_kernel<T><<<gridFor(NN, BS), BS, 0, st>>>(NN, b, Ku, r, dmask);
    VFEM_LAUNCH_CHECK();
}

// ---- triquadratic multigrid hierarchy ----
template <typename T>
void launch_q2mg_level1(const int neCoarse[3], const T *Kc, const T *Y, T *Ke, cudaStream_t st) {
    const int nef[3] = {2 * neCoarse[0], 2 * neCoarse[1], 2 * neCoarse[2]};
    const Q2Dims dc = dims_of(neCoarse), df = dims_of(nef);
    q2mg_level1_kernel<T><<<gridFor(dc.NE * 6561, BS), BS, 0, st>>>(dc, df, Kc, Y, Ke);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_q2mg_galerkin(const int neCoarse[3], const T *KeFine, T *KeCoarse, cudaStream_t st) {
    const int nef[3] = {2 * neCoarse[0], 2 * neCoarse[1], 2 * neCoarse[2]};
    const Q2Dims dc = dims_of(neCoarse), df = dims_of(nef);
    const size_t smem = sizeof(T) * (2 * 6561 + 27 * 8) + sizeof(int) * (27 * 8 + 27);
    // set on every call (once per hierarchy build): the attribute belongs to the current device
    VFEM_CUDA(cudaFuncSetAttribute(q2mg_galerkin_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (dc.NE > 0) q2mg_galerkin_kernel<T><<<(unsigned)dc.NE, GAL_THREADS, smem, st>>>(dc, df, KeFine, KeCoarse);
    VFEM_LAUNCH_CHECK();
}

template <typename T, int NX, int NY, int NZ>
static void gs_colour(const Q2Dims &d, unsigned gs, const T *Ke, T *u, const T *b, const uint8_t *dmask, int ca,
                      int cb, int cc, int fw, cudaStream_t st) {
    q2mg_gs_kernel<T, NX, NY, NZ><<<gs, BS, 0, st>>>(d, Ke, u, b, dmask, ca, cb, cc, fw);
}

template <typename T>
void launch_q2mg_gs_sweep(const int ne[3], const T *Ke, T *u, const T *b, const uint8_t *dmask, bool forward,
                          cudaStream_t st) {
    const Q2Dims d = dims_of(ne);
    for (int s = 0; s < 27; ++s) {
        const int col = forward ? s : 26 - s;
        const int ca = col / 9, cb = (col / 3) % 3, cc = col % 3;
        const int ia = ca == 1 ? 2 : 4, ib = cb == 1 ? 2 : 4, ic = cc == 1 ? 2 : 4;
        if (ca >= d.nn[0] || cb >= d.nn[1] || cc >= d.nn[2]) continue;
        const int64_t cnt = (int64_t)((d.nn[0] - 1 - ca) / ia + 1) * ((d.nn[1] - 1 - cb) / ib + 1) *
                            ((d.nn[2] - 1 - cc) / ic + 1);
        const unsigned gs = gridFor(32 * cnt, BS);
        const int fw = forward ? 1 : 0;
        switch (4 * (ca == 1) + 2 * (cb == 1) + (cc == 1)) {
        case 0: gs_colour<T, 2, 2, 2>(d, gs, Ke, u, b, dmask, ca, cb, cc, fw, st); break;
        case 1: gs_colour<T, 2, 2, 1>(d, gs, Ke, u, b, dmask, ca, cb, cc, fw, st); break;
        case 2: gs_colour<T, 2, 1, 2>(d, gs, Ke, u, b, dmask, ca, cb, cc, fw, st); break;
        case 3: gs_colour<T, 2, 1, 1>(d, gs, Ke, u, b, dmask, ca, cb, cc, fw, st); break;
        case 4: gs_colour<T, 1, 2, 2>(d, gs, Ke, u, b, dmask, ca, cb, cc, fw, st); break;
        case 5: gs_colour<T, 1, 2, 1>(d, gs, Ke, u, b, dmask, ca, cb, cc, fw, st); break;
        case 6: gs_colour<T, 1, 1, 2>(d, gs, Ke, u, b, dmask, ca, cb, cc, fw, st); break;
        default: gs_colour<T, 1, 1, 1>(d, gs, Ke, u, b, dmask, ca, cb, cc, fw, st); break;
        }
        VFEM_LAUNCH_CHECK();
    }
}

template <typename T, bool R, int PX, int PY, int PZ>
static void apply_class(const Q2Dims &d, const T *Ke, const T *u, const T *b, T *out, const uint8_t *dmask, int zd,
                        cudaStream_t st) {
    const int64_t cnt = (int64_t)((d.nn[0] - PX + 1) / 2) * ((d.nn[1] - PY + 1) / 2) * ((d.nn[2] - PZ + 1) / 2);
    q2mg_apply_kernel<T, R, PX, PY, PZ><<<gridFor(32 * cnt, BS), BS, 0, st>>>(d, Ke, u, b, out, dmask, zd);
}

template <typename T, bool R>
static void apply_classes(const Q2Dims &d, const T *Ke, const T *u, const T *b, T *out, const uint8_t *dmask, int zd,
                          cudaStream_t st) {
    apply_class<T, R, 0, 0, 0>(d, Ke, u, b, out, dmask, zd, st);
    apply_class<T, R, 0, 0, 1>(d, Ke, u, b, out, dmask, zd, st);
    apply_class<T, R, 0, 1, 0>(d, Ke, u, b, out, dmask, zd, st);
    apply_class<T, R, 0, 1, 1>(d, Ke, u, b, out, dmask, zd, st);
    apply_class<T, R, 1, 0, 0>(d, Ke, u, b, out, dmask, zd, st);
    apply_class<T, R, 1, 0, 1>(d, Ke, u, b, out, dmask, zd, st);
    apply_class<T, R, 1, 1, 0>(d, Ke, u, b, out, dmask, zd, st);
    apply_class<T, R, 1, 1, 1>(d, Ke, u, b, out, dmask, zd, st);
}

template <typename T>
void launch_q2mg_apply(const int ne[3], const T *Ke, const T *u, const T *b, T *out, const uint8_t *dmask,
                       bool zeroDirichlet, cudaStream_t st) {
    const Q2Dims d = dims_of(ne);
    if (b) apply_classes<T, true>(d, Ke, u, b, out, dmask, zeroDirichlet ? 1 : 0, st);
    else apply_classes<T, false>(d, Ke, u, nullptr, out, dmask, zeroDirichlet ? 1 : 0, st);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_q2mg_dense(const int ne[3], const T *Ke, const int *freeIdx, const int *redIdx, int nfree, double *A,
                       cudaStream_t st) {
    const Q2Dims d = dims_of(ne);
    VFEM_CUDA(cudaMemsetAsync(A, 0, sizeof(double) * (size_t)nfree * nfree, st));
    if (nfree > 0) q2mg_dense_kernel<T><<<gridFor(nfree, BS), BS, 0, st>>>(d, Ke, freeIdx, redIdx, nfree, A);
    VFEM_LAUNCH_CHECK();
}

#define VFEM_INST_Q2(T)                                                                                               \
    template void launch_applyk_q2<T>(const int[3], const T *, const T *, const T *, T *, const uint8_t *, bool,      \
                                      cudaStream_t);                                                                  \
    template void launch_gs_q2_sweep<T>(const int[3], const T *, const T *, T *, const T *, const uint8_t *, bool,    \
                                        cudaStream_t);                                                                \
    template void launch_restrict_q2<T>(const int[3], const T *, T *, cudaStream_t);                                  \
    template void launch_interp_q2<T>(const int[3], const T *, T *, bool, cudaStream_t);                              \
    template void launch_interp_q1_q2<T>(const int[3], const T *, T *, bool, cudaStream_t);                           \
    template void launch_restrict_q2_q1<T>(const int[3], const T *, T *, cudaStream_t);                               \
    template void launch_q2_residual_combine<T>(int64_t, const T *, const T *, T *, const uint8_t *, cudaStream_t); \
    template void launch_q2mg_level1<T>(const int[3], const T *, const T *, T *, cudaStream_t);                       \
    template void launch_q2mg_galerkin<T>(const int[3], const T *, T *, cudaStream_t);                                \
    template void launch_q2mg_gs_sweep<T>(const int[3], const T *, T *, const T *, const uint8_t *, bool,             \
                                          cudaStream_t);                                                              \
    template void launch_q2mg_apply<T>(const int[3], const T *, const T *, const T *, T *, const uint8_t *, bool,     \
                                       cudaStream_t);                                                                 \
    template void launch_q2mg_dense<T>(const int[3], const T *, const int *, const int *, int, double *, cudaStream_t);
VFEM_INST_Q2(double)
VFEM_INST_Q2(float)

}  // namespace vfem
