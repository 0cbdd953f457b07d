// Density filters beyond smoothing and projection (TopologyOptimizationFilter.hh:402-709):
// UpsampleFilter (trilinear, degree 1), VertexToCellFilter and LangelaarFilter (the
// additive-manufacturing overhang filter, build direction y). Grids are row-major (x slowest,
// z fastest).
#include "vfem_kernels.hpp"

#include <cmath>

namespace vfem {

namespace {

constexpr int BS = 256;

__device__ __forceinline__ int64_t flat3(int i, int j, int k, int d1, int d2) {
    return ((int64_t)i * d1 + j) * d2 + k;
}

// UpsampleFilter::ApplyImpl (:445-470): fine node n lies in the coarse cell with min corner
// c = min(n / F, in - 2) at local coordinate t = (n - F c) / F; the trilinear interpolant of the
// cell's 8 coarse values is sampled there. Nodes shared by cells get weights exactly 0 or 1, so
// every cell gives them the same value.
__global__ void upsample_kernel(int a0, int a1, int a2, int F, int flat, const double *__restrict__ in,
                                double *__restrict__ out) {
    const int f1 = (a1 - 1) * F + 1, f2 = (a2 - 1) * F + 1;
    const int64_t nf = (int64_t)((a0 - 1) * F + 1) * f1 * f2;
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= nf) return;
    const int n2 = (int)(t % f2), n1 = (int)((t / f2) % f1), n0 = (int)(t / ((int64_t)f1 * f2));
    const int n[3] = {n0, n1, n2}, a[3] = {a0, a1, a2};
    int c[3];
    double x[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        c[d] = (flat && d == 2) ? 0 : min(n[d] / F, a[d] - 2);
        x[d] = (double)(n[d] - F * c[d]) / (double)F;
    }
    double v = 0.0;
#pragma unroll
    for (int corner = 0; corner < 8; ++corner) {
        const int b0 = (corner >> 2) & 1, b1 = (corner >> 1) & 1, b2 = corner & 1;
        if (flat && b2) continue;  // 2D grid: no z axis
        const double w = (b0 ? x[0] : 1.0 - x[0]) * (b1 ? x[1] : 1.0 - x[1]) * (b2 ? x[2] : 1.0 - x[2]);
        v += w * in[flat3(c[0] + b0, c[1] + b1, c[2] + b2, a1, a2)];
    }
    out[t] = v;
}

// UpsampleFilter::BackpropImpl (:474-505): coarse node c collects phi(|n - F c| / F) d_dout(n)
// over the fine nodes of its incident cells, phi the degree-1 basis 1 - s per axis.
__global__ void upsample_backprop_kernel(int a0, int a1, int a2, int F, const double *__restrict__ g,
                                         double *__restrict__ out) {
    const int64_t nc = (int64_t)a0 * a1 * a2;
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= nc) return;
    const int f1 = (a1 - 1) * F + 1, f2 = (a2 - 1) * F + 1;
    const int c2 = (int)(t % a2), c1 = (int)((t / a2) % a1), c0 = (int)(t / ((int64_t)a1 * a2));
    const int c[3] = {c0, c1, c2}, a[3] = {a0, a1, a2};
    int lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        lo[d] = F * c[d] - (c[d] > 0 ? F - 1 : 0);
        hi[d] = F * c[d] + 1 + (c[d] < a[d] - 1 ? F - 1 : 0);
    }
    double acc = 0.0;
    for (int i = lo[0]; i < hi[0]; ++i) {
        const double wi = 1.0 - (double)abs(i - F * c0) / F;
        for (int j = lo[1]; j < hi[1]; ++j) {
            const double wj = 1.0 - (double)abs(j - F * c1) / F;
            for (int k = lo[2]; k < hi[2]; ++k) {
                const double wk = 1.0 - (double)abs(k - F * c2) / F;
                acc += wi * wj * wk * g[flat3(i, j, k, f1, f2)];
            }
        }
    }
    out[t] = acc;
}

// VertexToCellFilter (:536-575): cell value = mean of its 8 corner values; backprop gives each
// vertex 1/8 of the gradients of the cells containing it.
// flat: a 2D grid (v2 == 1, no z axis): cell = mean of its 4 corners.
__global__ void vertex_to_cell_kernel(int v0, int v1, int v2, int flat, const double *__restrict__ in,
                                      double *__restrict__ out) {
    const int e1 = v1 - 1, e2 = flat ? 1 : v2 - 1;
    const int64_t ne = (int64_t)(v0 - 1) * e1 * e2;
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= ne) return;
    const int k = (int)(t % e2), j = (int)((t / e2) % e1), i = (int)(t / ((int64_t)e1 * e2));
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        if (flat && (c & 1)) continue;
        s += in[flat3(i + ((c >> 2) & 1), j + ((c >> 1) & 1), k + (c & 1), v1, v2)];
    }
    out[t] = s * (flat ? 0.25 : 0.125);
}

__global__ void vertex_to_cell_backprop_kernel(int v0, int v1, int v2, int flat, const double *__restrict__ g,
                                               double *__restrict__ out) {
    const int64_t nv = (int64_t)v0 * v1 * v2;
    const int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (t >= nv) return;
    const int e0 = v0 - 1, e1 = v1 - 1, e2 = flat ? 1 : v2 - 1;
    const int k = (int)(t % v2), j = (int)((t / v2) % v1), i = (int)(t / ((int64_t)v1 * v2));
    double s = 0.0;
    for (int a = i - 1; a <= i; ++a)
        for (int b = j - 1; b <= j; ++b)
            for (int c = flat ? k : k - 1; c <= k; ++c)
                if (a >= 0 && b >= 0 && c >= 0 && a < e0 && b < e1 && c < e2) s += g[flat3(a, b, c, e1, e2)];
    out[t] = s * (flat ? 0.25 : 0.125);
}

// ---- LangelaarFilter (:577-709), build direction y ----
// The supporting region of voxel (i, j, k), j >= 1, follows NDVector::visitSupportingRegion
// (NDVector.hh:211-229) as written: the voxel below (i, j-1, k), then for d = 0 the voxels
// (i-1, j-1, k) and (i+1, j-1, k), and for d = 1 (the build axis itself) (i, j-2, k) and
// (i, j, k) -- the voxel itself, whose output value at that point is the one left by the
// previous application. z neighbours are not in the region, so every z plane is independent:
// one CTA per plane walks the layers with a barrier between them. On a 2D grid (flat: N = 2,
// d2 == 1) the loop over d stops after d = 0: the region is the voxel below and its x neighbours.
constexpr double LP = 40.0, LQ = 40.0 - 1.58, LEPS = 1e-4;

__device__ __forceinline__ double lsmin(double a, double b) {
    return 0.5 * (a + b - sqrt((a - b) * (a - b) + LEPS) + sqrt(LEPS));
}
__device__ __forceinline__ double dsmin1(double a, double b) {
    return 0.5 * (1 - (a - b) / sqrt((a - b) * (a - b) + LEPS));
}
__device__ __forceinline__ double dsmin2(double a, double b) {
    return 0.5 * (1 + (a - b) / sqrt((a - b) * (a - b) + LEPS));
}

// sum over the supporting region of f^P (with the indices of the region's members)
__device__ __forceinline__ double support_sum(const double *f, int i, int j, int k, int d0, int d1, int d2, int flat) {
    double s = pow(f[flat3(i, j - 1, k, d1, d2)], LP);
    if (i - 1 >= 0) s += pow(f[flat3(i - 1, j - 1, k, d1, d2)], LP);
    if (i + 1 < d0) s += pow(f[flat3(i + 1, j - 1, k, d1, d2)], LP);
    if (flat) return s;
    if (j - 2 >= 0) s += pow(f[flat3(i, j - 2, k, d1, d2)], LP);
    s += pow(f[flat3(i, j, k, d1, d2)], LP);
    return s;
}

// out holds the previous application's output on entry (its own-voxel term); smax and the
// filtered field are kept for the backprop.
__global__ void langelaar_apply_kernel(int d0, int d1, int d2, int flat, const double *__restrict__ in, double *out,
                                       double *__restrict__ smaxOut) {
    const int k = blockIdx.x;
    for (int i = threadIdx.x; i < d0; i += blockDim.x) out[flat3(i, 0, k, d1, d2)] = in[flat3(i, 0, k, d1, d2)];
    __syncthreads();
    for (int j = 1; j < d1; ++j) {
        for (int i = threadIdx.x; i < d0; i += blockDim.x) {
            const double sm = pow(support_sum(out, i, j, k, d0, d1, d2, flat), 1.0 / LQ);
            const int64_t e = flat3(i, j, k, d1, d2);
            smaxOut[e] = sm;
            out[e] = lsmin(in[e], sm);
        }
        __syncthreads();
    }
}

// computeLagrangeMultipliers (:620-640) and backprop (:598-606). vars: the filter's input,
// filt / smax: cached from the last apply. lam: scratch (the multipliers).
__global__ void langelaar_backprop_kernel(int d0, int d1, int d2, int flat, const double *__restrict__ g,
                                          const double *__restrict__ vars, const double *__restrict__ filt,
                                          const double *__restrict__ smax, double *lam, double *__restrict__ out) {
    const int k = blockIdx.x;
    for (int i = threadIdx.x; i < d0; i += blockDim.x) lam[flat3(i, d1 - 1, k, d1, d2)] = g[flat3(i, d1 - 1, k, d1, d2)];
    __syncthreads();
    // d(i', L+1, k) / d(member): sminDerivative = dsmin_dx2(vars, smax) * P f_m^(P-1) / Q * S^(1/Q - 1)
    for (int L = d1 - 2; L >= 0; --L) {
        const int up = L + 1;
        // gather into layer L from the voxels of layer L+1 whose regions contain it (pre-update values)
        for (int i = threadIdx.x; i < d0; i += blockDim.x) {
            double acc = g[flat3(i, L, k, d1, d2)];
            for (int ip = i - 1; ip <= i + 1; ++ip) {
                if (ip < 0 || ip >= d0) continue;
                const int64_t e = flat3(ip, up, k, d1, d2);
                const double S = support_sum(filt, ip, up, k, d0, d1, d2, flat);
                const double fm = filt[flat3(i, L, k, d1, d2)];
                const double der = dsmin2(vars[e], smax[e]) * (LP * pow(fm, LP - 1) / LQ * pow(S, 1.0 / LQ - 1));
                acc += lam[e] * der;
            }
            lam[flat3(i, L, k, d1, d2)] = acc;
        }
        __syncthreads();
        // the own-voxel term of layer L+1 (the last member visited, :631-637); not a member in 2D
        for (int i = threadIdx.x; i < d0 && !flat; i += blockDim.x) {
            const int64_t e = flat3(i, up, k, d1, d2);
            const double S = support_sum(filt, i, up, k, d0, d1, d2, flat);
            const double der = dsmin2(vars[e], smax[e]) * (LP * pow(filt[e], LP - 1) / LQ * pow(S, 1.0 / LQ - 1));
            lam[e] += lam[e] * der;
        }
        __syncthreads();
    }
    for (int j = 0; j < d1; ++j)
        for (int i = threadIdx.x; i < d0; i += blockDim.x) {
            const int64_t e = flat3(i, j, k, d1, d2);
            out[e] = j == 0 ? lam[e] : lam[e] * dsmin1(vars[e], smax[e]);
        }
}

}  // namespace

void launch_upsample(const int dims[3], int factor, const double *in, double *out, cudaStream_t st, int ndim) {
    const int64_t nf = (int64_t)((dims[0] - 1) * factor + 1) * ((dims[1] - 1) * factor + 1) * ((dims[2] - 1) * factor + 1);
    upsample_kernel<<<gridFor(nf, BS), BS, 0, st>>>(dims[0], dims[1], dims[2], factor, ndim == 2 ? 1 : 0, in, out);
    VFEM_LAUNCH_CHECK();
}
void launch_upsample_backprop(const int dims[3], int factor, const double *g, double *out, cudaStream_t st) {
    upsample_backprop_kernel<<<gridFor((int64_t)dims[0] * dims[1] * dims[2], BS), BS, 0, st>>>(dims[0], dims[1],
                                                                                              dims[2], factor, g, out);
    VFEM_LAUNCH_CHECK();
}
void launch_vertex_to_cell(const int vdims[3], const double *in, double *out, cudaStream_t st, int ndim) {
    const int flat = ndim == 2 ? 1 : 0;
    vertex_to_cell_kernel<<<gridFor((int64_t)(vdims[0] - 1) * (vdims[1] - 1) * (flat ? 1 : vdims[2] - 1), BS), BS, 0,
                            st>>>(vdims[0], vdims[1], vdims[2], flat, in, out);
    VFEM_LAUNCH_CHECK();
}
void launch_vertex_to_cell_backprop(const int vdims[3], const double *g, double *out, cudaStream_t st, int ndim) {
    vertex_to_cell_backprop_kernel<<<gridFor((int64_t)vdims[0] * vdims[1] * vdims[2], BS), BS, 0, st>>>(
        vdims[0], vdims[1], vdims[2], ndim == 2 ? 1 : 0, g, out);
    VFEM_LAUNCH_CHECK();
}
void launch_langelaar(const int dims[3], const double *in, double *out, double *smax, cudaStream_t st, int ndim) {
    const int threads = dims[0] >= 256 ? 256 : ((dims[0] + 31) / 32) * 32;
    langelaar_apply_kernel<<<dims[2], threads, 0, st>>>(dims[0], dims[1], dims[2], ndim == 2 ? 1 : 0, in, out, smax);
    VFEM_LAUNCH_CHECK();
}
void launch_langelaar_backprop(const int dims[3], const double *g, const double *vars, const double *filt,
                               const double *smax, double *lam, double *out, cudaStream_t st, int ndim) {
    const int threads = dims[0] >= 256 ? 256 : ((dims[0] + 31) / 32) * 32;
    langelaar_backprop_kernel<<<dims[2], threads, 0, st>>>(dims[0], dims[1], dims[2], ndim == 2 ? 1 : 0, g, vars, filt,
                                                           smax, lam, out);
    VFEM_LAUNCH_CHECK();
}

}  // namespace vfem
