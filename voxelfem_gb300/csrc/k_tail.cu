// Single-CTA coarse tail of the V-cycle (FP32 levels of the mixed-precision
// preconditioner). Below a few thousand nodes a level's kernels are latency-bound:
// a 27-point colour pass over ~1,000 nodes lasts a few microseconds, and the
// reference V-cycle (MultigridSolver.hh:617-658) issues ~35 of them per level.
// tail_down runs, for every tail level except the coarsest, the zeroing of the
// Dirichlet components, the pre-smoothing sweeps (8 colours each), the residual and
// the restriction; tail_up runs the prolongation and the post-smoothing sweeps.
// Consecutive steps are separated by __syncthreads(); the coarsest level's dense
// solve runs between the two launches on the whole GPU.
#include "vfem_kernels.hpp"
#include "vfem_stencil.cuh"

namespace vfem {

namespace {

constexpr int TB = 512;

template <typename T>
__device__ void zero_dirichlet_all(const TailLevel<T> &L) {
    for (int64_t n = threadIdx.x; n < L.g.NN; n += TB) {
        const uint8_t dm = L.dmask[n];
        if (!dm) continue;
        if (dm & 1) L.x[n] = T(0);
        if (dm & 2) L.x[L.g.ld + n] = T(0);
        if (dm & 4) L.x[2 * L.g.ld + n] = T(0);
    }
}

template <typename T>
__device__ void sweep(const TailLevel<T> &L, bool forward) {
    const Geom &g = L.g;
    for (int c = 0; c < 8; ++c) {
        const int color = forward ? c : 7 - c;
        const int cx = (color >> 2) & 1, cy = (color >> 1) & 1, cz = color & 1;
        const int n2 = (g.nn[2] - cz + 1) / 2, n1 = (g.nyv() - cy + 1) / 2, n0 = (g.nn[0] - cx + 1) / 2;
        const int cnt = n1 > 0 ? n0 * n1 * n2 : 0;
        for (int t = threadIdx.x >> 5; t < cnt; t += TB / 32) {
            const int kk = t % n2, q = t / n2;
            const int jj = q % n1, ii = q / n1;
            stencil::gs_node_warp<T>(g, L.S, L.x, L.b, L.dmask, cx + 2 * ii, cy + 2 * jj, cz + 2 * kk, forward,
                                     threadIdx.x & 31);
        }
        __syncthreads();
    }
}

template <typename T>
__global__ void __launch_bounds__(TB) tail_down_kernel(TailParams<T> P) {
    for (int t = 0; t + 1 < P.nlev; ++t) {
        const TailLevel<T> &L = P.lv[t];
        const TailLevel<T> &Cl = P.lv[t + 1];
        zero_dirichlet_all<T>(L);
        __syncthreads();
        for (int s = 0; s < P.sweeps; ++s) sweep<T>(L, true);
        for (int64_t n = threadIdx.x >> 5; n < L.g.NN; n += TB / 32) {
            int i, j, k;
            stencil::decode(n, L.g.nn[1], L.g.nn[2], i, j, k);
            stencil::residual_node_warp<T>(L.g, L.S, L.x, L.b, L.r, L.dmask, n, i, j, k, threadIdx.x & 31);
        }
        __syncthreads();
        {
            const int cyv = Cl.g.nyv();
            const int rows = cyv < Cl.g.nn[1] ? cyv + 1 : cyv;
            const int64_t cnt = (int64_t)Cl.g.nn[0] * rows * Cl.g.nn[2];
            for (int64_t q = threadIdx.x; q < cnt; q += TB) {
                int i, j, k;
                stencil::decode(q, rows, Cl.g.nn[2], i, j, k);
                stencil::restrict_node<T>(L.g, Cl.g, L.r, Cl.b, i, j, k);
            }
            // zero the coarse iterate on the nondetached rows plus the margin
            int zr = Cl.g.nyv() + MARGIN;
            if (zr > Cl.g.nn[1]) zr = Cl.g.nn[1];
            const int64_t zc = (int64_t)Cl.g.nn[0] * zr * Cl.g.nn[2];
            for (int64_t q = threadIdx.x; q < zc; q += TB) {
                int i, j, k;
                stencil::decode(q, zr, Cl.g.nn[2], i, j, k);
                const int64_t n = Cl.g.node(i, j, k);
                Cl.x[n] = T(0);
                Cl.x[Cl.g.ld + n] = T(0);
                Cl.x[2 * Cl.g.ld + n] = T(0);
            }
        }
        __syncthreads();
    }
}

template <typename T>
__global__ void __launch_bounds__(TB) tail_up_kernel(TailParams<T> P) {
    for (int t = P.nlev - 2; t >= 0; --t) {
        const TailLevel<T> &L = P.lv[t];
        const TailLevel<T> &Cl = P.lv[t + 1];
        const int rows = L.g.nyv();
        const int64_t cnt = (int64_t)L.g.nn[0] * rows * L.g.nn[2];
        for (int64_t q = threadIdx.x; q < cnt; q += TB) {
            int f[3];
            stencil::decode(q, rows, L.g.nn[2], f[0], f[1], f[2]);
            stencil::interp_node<T, true>(L.g, Cl.g, Cl.x, L.x, f);
        }
        __syncthreads();
        for (int s = 0; s < P.sweeps; ++s) sweep<T>(L, !P.symmetric);
    }
}

}  // namespace

template <typename T>
void launch_tail_down(const TailParams<T> &P, cudaStream_t st) {
    tail_down_kernel<T><<<1, TB, 0, st>>>(P);
    VFEM_LAUNCH_CHECK();
}

template <typename T>
void launch_tail_up(const TailParams<T> &P, cudaStream_t st) {
    tail_up_kernel<T><<<1, TB, 0, st>>>(P);
    VFEM_LAUNCH_CHECK();
}

template void launch_tail_down<float>(const TailParams<float> &, cudaStream_t);
template void launch_tail_up<float>(const TailParams<float> &, cudaStream_t);
template void launch_tail_down<double>(const TailParams<double> &, cudaStream_t);
template void launch_tail_up<double>(const TailParams<double> &, cudaStream_t);

}  // namespace vfem
