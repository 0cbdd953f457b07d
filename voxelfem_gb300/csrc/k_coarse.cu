// Coarse-level kernels: assembled 27-point block stencils (the reference's blockK,
// TensorProductSimulator.hh:885-930), full-weighting restriction and trilinear
// prolongation (MultigridSolver.hh:163-275) and Galerkin coarsening of element
// matrices (MultigridSolver.hh:712-819).
//
// Stencil layout: S[(o*9 + 3r + c) * ld + n] is block (n, n+o)(r, c) with
// o = (ox+1)*9 + (oy+1)*3 + (oz+1); rows are visited in ascending neighbour
// index, the order of the reference's CSC columns.
// Element-matrix layout (levels >= 1): Ke[e*576 + 24*row + col].
#include "vfem_kernels.hpp"
#include "vfem_reduce.cuh"

namespace vfem {

namespace {

constexpr int BS = 256;

__device__ __forceinline__ void decode(const int64_t n, const int nn1, const int nn2, int &i, int &j, int &k) {
    k = (int)(n % nn2);
    const int64_t t = n / nn2;
    j = (int)(t % nn1);
    i = (int)(t / nn1);
}

// Branch-free row gather: neighbours outside the grid are clamped to a valid node; their
// stencil blocks are exactly zero (no element contains both nodes), so they add nothing and
// every load of the row can be in flight at once.
template <typename T, bool Negate>
__device__ __forceinline__ void stencil_row(const Geom &g, const T *__restrict__ S, const T *__restrict__ u, int64_t n,
                                            int i, int j, int k, T &f0, T &f1, T &f2) {
    const int64_t ld = g.ld;
    const int64_t sx = (int64_t)g.nn[1] * g.nn[2], sy = g.nn[2];
    const int64_t dx[3] = {i > 0 ? -sx : 0, 0, i + 1 < g.nn[0] ? sx : 0};
    const int64_t dy[3] = {j > 0 ? -sy : 0, 0, j + 1 < g.nn[1] ? sy : 0};
    const int64_t dz[3] = {k > 0 ? -1 : 0, 0, k + 1 < g.nn[2] ? 1 : 0};
#pragma unroll
    for (int o = 0; o < 27; ++o) {
        const int64_t m = n + dx[o / 9] + dy[(o / 3) % 3] + dz[o % 3];
        const T u0 = u[m], u1 = u[ld + m], u2 = u[2 * ld + m];
        const T *blk = S + (int64_t)(o * 9) * ld + n;
        const T v0 = blk[0] * u0 + blk[ld] * u1 + blk[2 * ld] * u2;
        const T v1 = blk[3 * ld] * u0 + blk[4 * ld] * u1 + blk[5 * ld] * u2;
        const T v2 = blk[6 * ld] * u0 + blk[7 * ld] * u1 + blk[8 * ld] * u2;
        if (Negate) { f0 -= v0; f1 -= v1; f2 -= v2; }
        else        { f0 += v0; f1 += v1; f2 += v2; }
    }
}

template <typename T, bool ZeroInit, bool Negate>
__global__ void __launch_bounds__(BS) stencil_apply_kernel(Geom g, const T *__restrict__ S, const T *__restrict__ u,
                                                           T *__restrict__ out) {
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n >= g.NN) return;
    int i, j, k;
    decode(n, g.nn[1], g.nn[2], i, j, k);
    const int64_t ld = g.ld;
    T f0 = ZeroInit ? T(0) : out[n], f1 = ZeroInit ? T(0) : out[ld + n], f2 = ZeroInit ? T(0) : out[2 * ld + n];
    stencil_row<T, Negate>(g, S, u, n, i, j, k, f0, f1, f2);
    out[n] = f0;
    out[ld + n] = f1;
    out[2 * ld + n] = f2;
}

template <typename T>
__global__ void __launch_bounds__(BS) stencil_residual_kernel(Geom g, const T *__restrict__ S, const T *__restrict__ u,
                                                              const T *__restrict__ b, T *__restrict__ r,
                                                              const uint8_t *__restrict__ dmask) {
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n >= g.NN) return;
    int i, j, k;
    decode(n, g.nn[1], g.nn[2], i, j, k);
    const int64_t ld = g.ld;
    T f0 = b[n], f1 = b[ld + n], f2 = b[2 * ld + n];
    if (j < g.nyv()) stencil_row<T, true>(g, S, u, n, i, j, k, f0, f1, f2);
    const uint8_t dm = dmask[n];
    if (dm & 1) f0 = T(0);
    if (dm & 2) f1 = T(0);
    if (dm & 4) f2 = T(0);
    r[n] = f0;
    r[ld + n] = f1;
    r[2 * ld + n] = f2;
}

template <typename T>
__device__ __forceinline__ void node_solve(uint8_t dm, T s0, T s1, T s2, const T *M, bool forward, T &u0, T &u1,
                                           T &u2) {
    if (dm) {
        T d[3] = {T(0), T(0), T(0)};
        const T bs[3] = {s0, s1, s2};
        if (forward) {
#pragma unroll
            for (int q = 0; q < 3; ++q)
                d[q] = (bs[q] - (M[3 * q] * d[0] + M[3 * q + 1] * d[1] + M[3 * q + 2] * d[2])) *
                       (T(!((dm >> q) & 1)) / M[4 * q]);
        } else {
#pragma unroll
            for (int q = 2; q >= 0; --q)
                d[q] = (bs[q] - (M[3 * q] * d[0] + M[3 * q + 1] * d[1] + M[3 * q + 2] * d[2])) *
                       (T(!((dm >> q) & 1)) / M[4 * q]);
        }
        u0 += d[0];
        u1 += d[1];
        u2 += d[2];
    } else {
        const T c00 = M[4] * M[8] - M[5] * M[7];
        const T c01 = M[5] * M[6] - M[3] * M[8];
        const T c02 = M[3] * M[7] - M[4] * M[6];
        const T det = M[0] * c00 + M[1] * c01 + M[2] * c02;
        const T id = T(1) / det;
        const T i00 = c00 * id, i01 = (M[2] * M[7] - M[1] * M[8]) * id, i02 = (M[1] * M[5] - M[2] * M[4]) * id;
        const T i10 = c01 * id, i11 = (M[0] * M[8] - M[2] * M[6]) * id, i12 = (M[2] * M[3] - M[0] * M[5]) * id;
        const T i20 = c02 * id, i21 = (M[1] * M[6] - M[0] * M[7]) * id, i22 = (M[0] * M[4] - M[1] * M[3]) * id;
        u0 += i00 * s0 + i01 * s1 + i02 * s2;
        u1 += i10 * s0 + i11 * s1 + i12 * s2;
        u2 += i20 * s0 + i21 * s1 + i22 * s2;
    }
}

// Block Gauss-Seidel colour pass from stencil rows (MultigridSolver.hh:323-334, 348-378).
template <typename T>
__global__ void __launch_bounds__(BS) gs_stencil_color_kernel(Geom g, const T *__restrict__ S, T *u,
                                                              const T *__restrict__ b,
                                                              const uint8_t *__restrict__ dmask, int cx, int cy,
                                                              int cz, int forward) {
    const int n2 = (g.nn[2] - cz + 1) / 2, n1 = (g.nyv() - cy + 1) / 2, n0 = (g.nn[0] - cx + 1) / 2;
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n1 <= 0 || t >= (int64_t)n0 * n1 * n2) return;
    const int kk = (int)(t % n2);
    const int64_t q = t / n2;
    const int jj = (int)(q % n1), ii = (int)(q / n1);
    const int i = cx + 2 * ii, j = cy + 2 * jj, k = cz + 2 * kk;
    const int64_t n = g.node(i, j, k), ld = g.ld;
    const uint8_t dm = dmask[n];
    if (dm == 7) return;
    T s0 = b[n], s1 = b[ld + n], s2 = b[2 * ld + n];
    stencil_row<T, true>(g, S, u, n, i, j, k, s0, s1, s2);
    T M[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) M[e] = S[(int64_t)(13 * 9 + e) * ld + n];
    T u0 = u[n], u1 = u[ld + n], u2 = u[2 * ld + n];
    node_solve<T>(dm, s0, s1, s2, M, forward != 0, u0, u1, u2);
    u[n] = u0;
    u[ld + n] = u1;
    u[2 * ld + n] = u2;
}

// Full-weighting restriction (MultigridSolver.hh:217-275): coarse node gathers the
// 3^3 fine nodes [2I-1, 2I+1] clipped to the nondetached fine range, weights
// prod(1 - |d|/2); the first detached coarse layer is zeroed.
template <typename T>
__global__ void __launch_bounds__(BS) restrict_kernel(Geom gf, Geom gc, const T *__restrict__ fine,
                                                      T *__restrict__ coarse) {
    const int cyv = gc.nyv();
    const int rows = cyv < gc.nn[1] ? cyv + 1 : cyv;
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= (int64_t)gc.nn[0] * rows * gc.nn[2]) return;
    int i, j, k;
    decode(t, rows, gc.nn[2], i, j, k);
    const int64_t cn = gc.node(i, j, k);
    T v0 = T(0), v1 = T(0), v2 = T(0);
    if (j < cyv) {
        const int fyv = gf.nyv();
        const int lo0 = max(2 * i - 1, 0), lo1 = max(2 * j - 1, 0), lo2 = max(2 * k - 1, 0);
        const int hi0 = min(2 * i + 2, gf.nn[0]), hi1 = min(2 * j + 2, fyv), hi2 = min(2 * k + 2, gf.nn[2]);
        const int64_t ld = gf.ld;
        for (int a = lo0; a < hi0; ++a) {
            const T wa = T(1) - T(abs(a - 2 * i)) * T(0.5);
            for (int bb = lo1; bb < hi1; ++bb) {
                const T wb = wa * (T(1) - T(abs(bb - 2 * j)) * T(0.5));
                for (int c = lo2; c < hi2; ++c) {
                    const T w = wb * (T(1) - T(abs(c - 2 * k)) * T(0.5));
                    const int64_t fn = gf.node(a, bb, c);
                    v0 += w * fine[fn];
                    v1 += w * fine[ld + fn];
                    v2 += w * fine[2 * ld + fn];
                }
            }
        }
    }
    coarse[cn] = v0;
    coarse[gc.ld + cn] = v1;
    coarse[2 * gc.ld + cn] = v2;
}

// Trilinear prolongation (MultigridSolver.hh:163-212).
template <typename T, bool Accumulate>
__global__ void __launch_bounds__(BS) interp_kernel(Geom gf, Geom gc, const T *__restrict__ coarse,
                                                    T *__restrict__ fine) {
    const int rows = Accumulate ? gf.nyv() : gf.nn[1];
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= (int64_t)gf.nn[0] * rows * gf.nn[2]) return;
    int f[3];
    decode(t, rows, gf.nn[2], f[0], f[1], f[2]);
    int ec[3], lf[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        ec[d] = min(f[d] / 2, gc.ne[d]);
        lf[d] = f[d] - 2 * ec[d];
    }
    const int64_t fn = gf.node(f[0], f[1], f[2]);
    const int64_t fld = gf.ld, cld = gc.ld;
    T a0 = Accumulate ? fine[fn] : T(0), a1 = Accumulate ? fine[fld + fn] : T(0),
      a2 = Accumulate ? fine[2 * fld + fn] : T(0);
#pragma unroll
    for (int cnl = 0; cnl < 8; ++cnl) {
        const int cb[3] = {(cnl >> 2) & 1, (cnl >> 1) & 1, cnl & 1};
        T coeff = T(1);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const T phi = (lf[d] == 1) ? T(0.5) : ((lf[d] == 0) ? (cb[d] ? T(0) : T(1)) : (cb[d] ? T(1) : T(0)));
            coeff *= phi;
        }
        if (coeff == T(0)) continue;
        const int64_t cidx = gc.node(ec[0] + cb[0], ec[1] + cb[1], ec[2] + cb[2]);
        a0 += coeff * coarse[cidx];
        a1 += coeff * coarse[cld + cidx];
        a2 += coeff * coarse[2 * cld + cidx];
    }
    fine[fn] = a0;
    fine[fld + fn] = a1;
    fine[2 * fld + fn] = a2;
}

template <typename T>
__global__ void zero_dirichlet_kernel(Geom g, T *__restrict__ u, const uint8_t *__restrict__ dmask) {
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (n >= g.NN) return;
    const uint8_t dm = dmask[n];
    if (!dm) return;
    if (dm & 1) u[n] = T(0);
    if (dm & 2) u[g.ld + n] = T(0);
    if (dm & 4) u[2 * g.ld + n] = T(0);
}

template <typename T>
__global__ void masked_zero_kernel(Geom g, T *__restrict__ u, int rows) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= (int64_t)g.nn[0] * rows * g.nn[2]) return;
    int i, j, k;
    decode(t, rows, g.nn[2], i, j, k);
    const int64_t n = g.node(i, j, k);
    u[n] = T(0);
    u[g.ld + n] = T(0);
    u[2 * g.ld + n] = T(0);
}

template <typename T>
__global__ void fill_kernel(T *__restrict__ p, T v, int64_t n) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t < n) p[t] = v;
}

template <typename Tdst, typename Tsrc>
__global__ void cast_kernel(const Tsrc *__restrict__ s, Tdst *__restrict__ d, int64_t n) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t < n) d[t] = (Tdst)s[t];
}

// Level-1 element matrices: Ke_c = sum_fi E_fi * Kc_fi (MultigridSolver.hh:724-738).
// One block per coarse element, thread t writes entry t.
template <typename T>
__global__ void __launch_bounds__(576) ke_level1_kernel(Geom g1, Geom g0, const T *__restrict__ Y0,
                                                        const T *__restrict__ Kc, T *__restrict__ Ke1) {
    __shared__ T sE[8];
    const int64_t e = blockIdx.x;
    const int t = threadIdx.x;
    const int ek = (int)(e % g1.ne[2]);
    const int64_t q = e / g1.ne[2];
    const int ej = (int)(q % g1.ne[1]), ei = (int)(q / g1.ne[1]);
    if (t < 8) sE[t] = Y0[g0.elem(2 * ei + ((t >> 2) & 1), 2 * ej + ((t >> 1) & 1), 2 * ek + (t & 1))];
    __syncthreads();
    T acc = T(0);
    if (ej < g1.firstMaskedE) {
#pragma unroll
        for (int fi = 0; fi < 8; ++fi) acc += sE[fi] * Kc[fi * 576 + t];
    }
    Ke1[e * 576 + t] = acc;
}

// Level-1 27-point stencil straight from the fine Young's moduli: block (n, n+o)(r, c) =
// sum over coarse elements e holding both nodes of sum_fi E_f(e, fi) Kc_fi[3ln+r][3lm+c]
// (the assembly of MultigridSolver.hh:724-738 without storing the element matrices).
// Thread per (node n, entry q), q = blockIdx.y: the Kc index is warp-uniform.
template <typename T>
__global__ void __launch_bounds__(BS) stencil_level1_kernel(Geom g1, Geom g0, const T *__restrict__ Y0,
                                                            const T *__restrict__ Kc, T *__restrict__ S) {
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    const int q = blockIdx.y;
    if (n >= g1.NN) return;
    int i, j, k;
    decode(n, g1.nn[1], g1.nn[2], i, j, k);
    const int o = q / 9, rc = q % 9, r = rc / 3, c = rc % 3;
    const int oo[3] = {o / 9 - 1, (o / 3) % 3 - 1, o % 3 - 1};
    T acc = T(0);
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {
                const int ma = a + oo[0], mb = b + oo[1], mc = cc + oo[2];
                if (ma < 0 || ma > 1 || mb < 0 || mb > 1 || mc < 0 || mc > 1) continue;
                const int ei = i - a, ej = j - b, ek = k - cc;
                if (ei < 0 || ej < 0 || ek < 0 || ei >= g1.ne[0] || ej >= g1.ne[1] || ek >= g1.ne[2]) continue;
                if (ej >= g1.firstMaskedE) continue;
                const int idx = (3 * (4 * a + 2 * b + cc) + r) * 24 + 3 * (4 * ma + 2 * mb + mc) + c;
#pragma unroll
                for (int fi = 0; fi < 8; ++fi) {
                    const T E = Y0[g0.elem(2 * ei + ((fi >> 2) & 1), 2 * ej + ((fi >> 1) & 1), 2 * ek + (fi & 1))];
                    acc += E * Kc[fi * 576 + idx];
                }
            }
    S[(int64_t)q * g1.ld + n] = acc;
}

// Ke_c = sum_fi Phi_fi^T Ke_child(fi) Phi_fi (MultigridSolver.hh:712-722, 745-819).
// One block per coarse element, thread t owns entry t of the coarse matrix.
template <typename T>
__global__ void __launch_bounds__(576) ke_coarsen_kernel(Geom gc, Geom gf, const T *__restrict__ Kef,
                                                         const T *__restrict__ phis, T *__restrict__ Kec) {
    __shared__ T sK[576];
    __shared__ T sT[576];
    __shared__ T sP[8 * 64];
    const int64_t e = blockIdx.x;
    const int t = threadIdx.x;
    for (int q = t; q < 512; q += 576) sP[q] = phis[q];
    const int ek = (int)(e % gc.ne[2]);
    const int64_t q = e / gc.ne[2];
    const int ej = (int)(q % gc.ne[1]), ei = (int)(q / gc.ne[1]);
    const bool masked = ej >= gc.firstMaskedE;
    T acc = T(0);
    const int row = t / 24, col = t % 24;
    for (int fi = 0; fi < 8; ++fi) {
        const int64_t ef = gf.elem(2 * ei + ((fi >> 2) & 1), 2 * ej + ((fi >> 1) & 1), 2 * ek + (fi & 1));
        __syncthreads();
        sK[t] = Kef[ef * 576 + t];
        __syncthreads();
        // T[row][3cn+d] = sum_fn K[row][3fn+d] phi[fn][cn]
        {
            const int cn = col / 3, d = col % 3;
            T v = T(0);
#pragma unroll
            for (int fn = 0; fn < 8; ++fn) v += sK[row * 24 + 3 * fn + d] * sP[fi * 64 + fn * 8 + cn];
            sT[t] = v;
        }
        __syncthreads();
        // Kc[3cm+d][col] += sum_fm phi[fm][cm] T[3fm+d][col]
        {
            const int cm = row / 3, d = row % 3;
            T v = T(0);
#pragma unroll
            for (int fm = 0; fm < 8; ++fm) v += sP[fi * 64 + fm * 8 + cm] * sT[(3 * fm + d) * 24 + col];
            acc += v;
        }
    }
    Kec[e * 576 + t] = masked ? T(0) : acc;
}

// Fine-level element matrices Ke = Y_e K0 (masked elements carry Y = 0).
template <typename T>
__global__ void __launch_bounds__(BS) ke_scaled_kernel(Geom g, const T *__restrict__ Y, const T *__restrict__ K0,
                                                       T *__restrict__ Ke) {
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= g.NE * 576) return;
    Ke[t] = Y[t / 576] * K0[t % 576];
}

// Assemble the 27-point block stencil from element matrices (TensorProductSimulator.hh:885-930).
// Thread per (node n, stencil entry q); q = blockIdx.y.
template <typename T>
__global__ void __launch_bounds__(BS) stencil_from_ke_kernel(Geom g, const T *__restrict__ Ke, T *__restrict__ S) {
    const int64_t n = blockIdx.x * (int64_t)BS + threadIdx.x;
    const int q = blockIdx.y;
    if (n >= g.NN) return;
    int i, j, k;
    decode(n, g.nn[1], g.nn[2], i, j, k);
    const int o = q / 9, rc = q % 9, r = rc / 3, c = rc % 3;
    const int oo[3] = {o / 9 - 1, (o / 3) % 3 - 1, o % 3 - 1};
    T acc = T(0);
    // incident elements (i-a, j-b, k-cc): node local index ln = 4a+2b+cc; neighbour local = ln + o
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {
                const int ma = a + oo[0], mb = b + oo[1], mc = cc + oo[2];
                if (ma < 0 || ma > 1 || mb < 0 || mb > 1 || mc < 0 || mc > 1) continue;
                const int ei = i - a, ej = j - b, ek = k - cc;
                if (ei < 0 || ej < 0 || ek < 0 || ei >= g.ne[0] || ej >= g.ne[1] || ek >= g.ne[2]) continue;
                const int ln = 4 * a + 2 * b + cc, lm = 4 * ma + 2 * mb + mc;
                acc += Ke[g.elem(ei, ej, ek) * 576 + (3 * ln + r) * 24 + 3 * lm + c];
            }
    S[(int64_t)q * g.ld + n] = acc;
}

}  // namespace

template <typename T>
void launch_stencil_apply(const Geom &g, const T *S, const T *u, T *out, bool zeroInit, bool negate, cudaStream_t st) {
    const unsigned grid = gridFor(g.NN, BS);
    if (zeroInit) {
        if (negate) stencil_apply_kernel<T, true, true><<<grid, BS, 0, st>>>(g, S, u, out);
        else stencil_apply_kernel<T, true, false><<<grid, BS, 0, st>>>(g, S, u, out);
    } else {
        if (negate) stencil_apply_kernel<T, false, true><<<grid, BS, 0, st>>>(g, S, u, out);
        else stencil_apply_kernel<T, false, false><<<grid, BS, 0, st>>>(g, S, u, out);
    }
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_stencil_residual(const Geom &g, const T *S, const T *u, const T *b, T *r, const uint8_t *dmask,
                             cudaStream_t st) {
    stencil_residual_kernel<T><<<gridFor(g.NN, BS), BS, 0, st>>>(g, S, u, b, r, dmask);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_gs_stencil_color(const Geom &g, const T *S, T *u, const T *b, const uint8_t *dmask, int color, bool forward,
                             cudaStream_t st) {
    const int cx = (color >> 2) & 1, cy = (color >> 1) & 1, cz = color & 1;
    const int64_t n0 = (g.nn[0] - cx + 1) / 2, n1 = (g.nyv() - cy + 1) / 2, n2 = (g.nn[2] - cz + 1) / 2;
    if (n1 <= 0) return;
    gs_stencil_color_kernel<T><<<gridFor(n0 * n1 * n2, BS), BS, 0, st>>>(g, S, u, b, dmask, cx, cy, cz,
                                                                          forward ? 1 : 0);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_restrict(const Geom &gf, const Geom &gc, const T *fine, T *coarse, cudaStream_t st) {
    const int cyv = gc.nyv();
    const int rows = cyv < gc.nn[1] ? cyv + 1 : cyv;
    restrict_kernel<T><<<gridFor((int64_t)gc.nn[0] * rows * gc.nn[2], BS), BS, 0, st>>>(gf, gc, fine, coarse);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_interpolate(const Geom &gf, const Geom &gc, const T *coarse, T *fine, bool accumulate, cudaStream_t st) {
    const int rows = accumulate ? gf.nyv() : gf.nn[1];
    const unsigned grid = gridFor((int64_t)gf.nn[0] * rows * gf.nn[2], BS);
    if (accumulate) interp_kernel<T, true><<<grid, BS, 0, st>>>(gf, gc, coarse, fine);
    else interp_kernel<T, false><<<grid, BS, 0, st>>>(gf, gc, coarse, fine);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_zero_dirichlet(const Geom &g, T *u, const uint8_t *dmask, cudaStream_t st) {
    zero_dirichlet_kernel<T><<<gridFor(g.NN, BS), BS, 0, st>>>(g, u, dmask);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_masked_zero(const Geom &g, T *u, int margin, cudaStream_t st) {
    int rows = g.nyv() + margin;
    if (rows > g.nn[1]) rows = g.nn[1];
    masked_zero_kernel<T><<<gridFor((int64_t)g.nn[0] * rows * g.nn[2], BS), BS, 0, st>>>(g, u, rows);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_fill(T *p, T v, int64_t n, cudaStream_t st) {
    if (n <= 0) return;
    fill_kernel<T><<<gridFor(n, BS), BS, 0, st>>>(p, v, n);
    VFEM_LAUNCH_CHECK();
}

template <typename Tdst, typename Tsrc>
void launch_cast(const Tsrc *src, Tdst *dst, int64_t n, cudaStream_t st) {
    if (n <= 0) return;
    cast_kernel<Tdst, Tsrc><<<gridFor(n, BS), BS, 0, st>>>(src, dst, n);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_ke_level1(const Geom &g1, const Geom &g0, const T *Y0, const T *Kc, T *Ke1, cudaStream_t st) {
    if (g1.NE > 2147483647LL) throw Error(ERR_ARG, "too many coarse elements");
    ke_level1_kernel<T><<<(unsigned)g1.NE, 576, 0, st>>>(g1, g0, Y0, Kc, Ke1);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_stencil_level1(const Geom &g1, const Geom &g0, const T *Y0, const T *Kc, T *S, cudaStream_t st) {
    dim3 grid(gridFor(g1.NN, BS), 243);
    stencil_level1_kernel<T><<<grid, BS, 0, st>>>(g1, g0, Y0, Kc, S);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_ke_coarsen(const Geom &gc, const Geom &gf, const T *Kef, const T *phis, T *Kec, cudaStream_t st) {
    if (gc.NE > 2147483647LL) throw Error(ERR_ARG, "too many coarse elements");
    ke_coarsen_kernel<T><<<(unsigned)gc.NE, 576, 0, st>>>(gc, gf, Kef, phis, Kec);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_ke_scaled(const Geom &g, const T *Y, const T *K0, T *Ke, cudaStream_t st) {
    ke_scaled_kernel<T><<<gridFor(g.NE * 576, BS), BS, 0, st>>>(g, Y, K0, Ke);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_stencil_from_ke(const Geom &g, const T *Ke, T *S, cudaStream_t st) {
    dim3 grid(gridFor(g.NN, BS), 243);
    stencil_from_ke_kernel<T><<<grid, BS, 0, st>>>(g, Ke, S);
    VFEM_LAUNCH_CHECK();
}

#define VFEM_INST_COARSE(T)                                                                                           \
    template void launch_stencil_apply<T>(const Geom &, const T *, const T *, T *, bool, bool, cudaStream_t);         \
    template void launch_stencil_residual<T>(const Geom &, const T *, const T *, const T *, T *, const uint8_t *,     \
                                             cudaStream_t);                                                           \
    template void launch_gs_stencil_color<T>(const Geom &, const T *, T *, const T *, const uint8_t *, int, bool,     \
                                             cudaStream_t);                                                           \
    template void launch_restrict<T>(const Geom &, const Geom &, const T *, T *, cudaStream_t);                       \
    template void launch_interpolate<T>(const Geom &, const Geom &, const T *, T *, bool, cudaStream_t);              \
    template void launch_zero_dirichlet<T>(const Geom &, T *, const uint8_t *, cudaStream_t);                         \
    template void launch_masked_zero<T>(const Geom &, T *, int, cudaStream_t);                                        \
    template void launch_fill<T>(T *, T, int64_t, cudaStream_t);                                                      \
    template void launch_ke_level1<T>(const Geom &, const Geom &, const T *, const T *, T *, cudaStream_t);           \
    template void launch_stencil_level1<T>(const Geom &, const Geom &, const T *, const T *, T *, cudaStream_t);      \
    template void launch_ke_coarsen<T>(const Geom &, const Geom &, const T *, const T *, T *, cudaStream_t);          \
    template void launch_stencil_from_ke<T>(const Geom &, const T *, T *, cudaStream_t);                              \
    template void launch_ke_scaled<T>(const Geom &, const T *, const T *, T *, cudaStream_t);
VFEM_INST_COARSE(double)
VFEM_INST_COARSE(float)
template void launch_cast<float, double>(const double *, float *, int64_t, cudaStream_t);
template void launch_cast<double, float>(const float *, double *, int64_t, cudaStream_t);

}  // namespace vfem
