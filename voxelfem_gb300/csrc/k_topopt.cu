// Topology-optimisation element kernels: the reflecting linear/constant density
// filter (TopologyOptimizationFilter.hh:285-400), the tanh Heaviside projection and
// its derivative (:189-245) and the optimality-criteria update
// (OptimalityCriterion.hh:64-83).
#include <mutex>
#include <vector>

#include "vfem_kernels.hpp"
#include "vfem_reduce.cuh"

namespace vfem {

namespace {

constexpr int BS = 256;

__device__ __forceinline__ int reflect_index(int i, int s) {
    // reflect across the min/max faces: -2,-1,0,1,2 -> 1,0,0,1,2 (repeated for narrow grids)
    for (int guard = 0; guard < 64 && (i < 0 || i >= s); ++guard) {
        if (i >= s) i = 2 * s - i - 1;
        if (i < 0) i = -i - 1;
    }
    return i;
}

__global__ void __launch_bounds__(BS) smoothing_filter_kernel(int d0, int d1, int d2, const double *__restrict__ in,
                                                              double *__restrict__ out, const int *__restrict__ offs,
                                                              const double *__restrict__ w, int ntaps, double W) {
    const int64_t e = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (e >= (int64_t)d0 * d1 * d2) return;
    const int k = (int)(e % d2);
    const int64_t t = e / d2;
    const int j = (int)(t % d1), i = (int)(t / d1);
    double acc = 0.0;
    for (int q = 0; q < ntaps; ++q) {
        const int ni = reflect_index(i + offs[3 * q], d0);
        const int nj = reflect_index(j + offs[3 * q + 1], d1);
        const int nk = reflect_index(k + offs[3 * q + 2], d2);
        acc += w[q] * in[((int64_t)ni * d1 + nj) * d2 + nk];
    }
    out[e] = acc / W;
}

__global__ void projection_kernel(int64_t n, double beta, double th, const double *__restrict__ in,
                                  double *__restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (i < n) out[i] = (th + tanh(beta * (in[i] - 0.5))) / (2 * th);
}

__global__ void projection_backprop_kernel(int64_t n, double beta, double scale, const double *__restrict__ in,
                                           const double *__restrict__ vars, double *__restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (i < n) {
        const double t = tanh(beta * (vars[i] - 0.5));
        out[i] = in[i] * (1.0 - t * t) * scale;
    }
}

__global__ void oc_update_kernel(int64_t n, const double *__restrict__ x0, const double *__restrict__ dJ,
                                 const double *__restrict__ dc, double lambda, double m, double p,
                                 double *__restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (i >= n) return;
    const double x = x0[i];
    const double raw = x * pow(dJ[i] / (dc[i] * lambda), p);
    double r = fmin(fmax(fmin(fmax(raw, x - m), x + m), 0.0), 1.0);
    // fmin/fmax would drop a NaN; the reference keeps x0 for a non-finite update
    // (an infinite update is clamped to x0 + m, which is finite).
    if (isnan(raw)) r = x;
    out[i] = r;
}

__global__ void __launch_bounds__(BS) sum_kernel(const double *__restrict__ x, int64_t n, double *__restrict__ partials) {
    double acc = 0.0;
    for (int64_t t = blockIdx.x * (int64_t)BS + threadIdx.x; t < n; t += (int64_t)gridDim.x * BS) acc += x[t];
    const double s = block_sum<BS>(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the density filter.
//
// For callers that cannot call cudaMalloc: code running under a fixed device-memory budget
// or inside a host application that owns every device allocation (a plug-in that may only
// use the buffers it is handed), and loops that cannot afford the implicit device
// synchronisation of cudaMalloc/cudaFree (e.g. the tens of filter applications of every OC
// bisection). The tap table lives in the file-scope array below, which every GPU that loads
// this library holds until the process exits. Its size bounds the filter radius to
// NOALLOC_MAX_RADIUS. Every call rewrites the table on the caller's stream, so calls that
// overlap on the GPU (different streams) race on it.
//
// Layout: [0] total weight W, [1] number of positive taps, then NOALLOC_MAX_TAPS weights,
// then the taps' offsets as 3 ints each. The taps keep the reference's lexicographic order
// over [-r, r]^3 with the non-positive weights left out, as the allocating path's table does.
// ---------------------------------------------------------------------------
constexpr int NOALLOC_MAX_RADIUS = 6;
constexpr int NOALLOC_MAX_TAPS = (2 * NOALLOC_MAX_RADIUS + 1) * (2 * NOALLOC_MAX_RADIUS + 1) *
                                 (2 * NOALLOC_MAX_RADIUS + 1);
constexpr int NOALLOC_HEADER = 2;
constexpr int NOALLOC_SCRATCH_DOUBLES = NOALLOC_HEADER + NOALLOC_MAX_TAPS + (3 * NOALLOC_MAX_TAPS + 1) / 2;
static __device__ __align__(256) double g_filter_scratch[NOALLOC_SCRATCH_DOUBLES];

constexpr int TAPS_BS = 1024;

// One thread per candidate offset computes its weight; an ordered block-wide prefix count
// places the positive ones in lexicographic order. W is then summed by one warp in a fixed
// order (each lane a contiguous run of taps, then the 32 partial sums in lane order), so the
// result is deterministic and within a few units in the last place of the allocating path's
// sequential sum (a single FP64 chain of up to 2197 dependent adds would be ~70 us here).
__global__ void __launch_bounds__(TAPS_BS) noalloc_taps_kernel(int radius, int type, double *scratch) {
    __shared__ int warpCount[TAPS_BS / 32];
    __shared__ int runBase;
    const int side = 2 * radius + 1, ncand = side * side * side;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double *wts = scratch + NOALLOC_HEADER;
    int *offs = reinterpret_cast<int *>(wts + NOALLOC_MAX_TAPS);
    const double rp1 = 1.0 + radius;
    if (threadIdx.x == 0) runBase = 0;
    __syncthreads();
    for (int base = 0; base < ncand; base += TAPS_BS) {
        const int q = base + (int)threadIdx.x;
        int a = 0, b = 0, c = 0;
        double w = 0.0;
        if (q < ncand) {
            a = q / (side * side) - radius;
            b = (q / side) % side - radius;
            c = q % side - radius;
            w = type == 1 ? rp1 - sqrt((double)(a * a + b * b + c * c)) : 1.0;
        }
        const bool keep = q < ncand && w > 0;
        const unsigned ball = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) warpCount[warp] = __popc(ball);
        __syncthreads();
        int before = runBase;
        for (int v = 0; v < warp; ++v) before += warpCount[v];
        before += __popc(ball & ((1u << lane) - 1u));
        if (keep) {
            wts[before] = w;
            offs[3 * before] = a;
            offs[3 * before + 1] = b;
            offs[3 * before + 2] = c;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int tot = 0;
            for (int v = 0; v < TAPS_BS / 32; ++v) tot += warpCount[v];
            runBase += tot;
        }
        __syncthreads();
    }
    if (warp == 0) {
        const int ntaps = runBase;
        const int per = (ntaps + 31) / 32;
        double part = 0.0;
        for (int t = lane * per; t < min(ntaps, (lane + 1) * per); ++t) part += wts[t];
        double W = 0.0;
        for (int v = 0; v < 32; ++v) W += __shfl_sync(0xffffffffu, part, v);
        if (lane == 0) {
            scratch[0] = W;
            scratch[1] = (double)ntaps;
        }
    }
}

__global__ void __launch_bounds__(BS) smoothing_filter_noalloc_kernel(int d0, int d1, int d2,
                                                                      const double *__restrict__ in,
                                                                      double *__restrict__ out,
                                                                      const double *__restrict__ scratch) {
    const int64_t e = blockIdx.x * (int64_t)BS + threadIdx.x;
    if (e >= (int64_t)d0 * d1 * d2) return;
    const int k = (int)(e % d2);
    const int64_t t = e / d2;
    const int j = (int)(t % d1), i = (int)(t / d1);
    const double *wts = scratch + NOALLOC_HEADER;
    const int *offs = reinterpret_cast<const int *>(wts + NOALLOC_MAX_TAPS);
    const int ntaps = __double2int_rn(scratch[1]);
    double acc = 0.0;
    for (int q = 0; q < ntaps; ++q) {
        const int ni = reflect_index(i + offs[3 * q], d0);
        const int nj = reflect_index(j + offs[3 * q + 1], d1);
        const int nk = reflect_index(k + offs[3 * q + 2], d2);
        acc += wts[q] * in[((int64_t)ni * d1 + nj) * d2 + nk];
    }
    out[e] = acc / scratch[0];
}

struct TapCache {
    int radius = -1, type = -1, ndim = -1;
    DevBuf<int> offs;
    DevBuf<double> w;
    int ntaps = 0;
    double W = 0;
};

thread_local TapCache g_taps;

}  // namespace

void launch_smoothing_filter(const int dims[3], int radius, int type, const double *in, double *out, cudaStream_t st,
                             int ndim) {
    if (radius < 0) throw Error(ERR_ARG, "negative filter radius");
    if (ndim != 2 && ndim != 3) throw Error(ERR_ARG, "smoothing filter: unsupported dimension");
    if (ndim == 2 && dims[2] != 1) throw Error(ERR_ARG, "smoothing filter: a 2D grid has dims[2] == 1");
    if (g_taps.radius != radius || g_taps.type != type || g_taps.ndim != ndim) {
        const int rz = ndim == 2 ? 0 : radius;
        std::vector<int> offs;
        std::vector<double> ws;
        const double rp1 = 1.0 + radius;
        double W = 0;
        for (int a = -radius; a <= radius; ++a)
            for (int b = -radius; b <= radius; ++b)
                for (int c = -rz; c <= rz; ++c) {
                    const double w = type == 1 ? rp1 - std::sqrt((double)(a * a + b * b + c * c)) : 1.0;
                    if (w <= 0) continue;
                    offs.push_back(a);
                    offs.push_back(b);
                    offs.push_back(c);
                    ws.push_back(w);
                    W += w;
                }
        g_taps.offs.alloc(offs.size());
        g_taps.w.alloc(ws.size());
        VFEM_CUDA(cudaMemcpy(g_taps.offs.p, offs.data(), offs.size() * sizeof(int), cudaMemcpyHostToDevice));
        VFEM_CUDA(cudaMemcpy(g_taps.w.p, ws.data(), ws.size() * sizeof(double), cudaMemcpyHostToDevice));
        g_taps.ntaps = (int)ws.size();
        g_taps.W = W;
        g_taps.radius = radius;
        g_taps.type = type;
        g_taps.ndim = ndim;
    }
    const int64_t n = (int64_t)dims[0] * dims[1] * dims[2];
    smoothing_filter_kernel<<<gridFor(n, BS), BS, 0, st>>>(dims[0], dims[1], dims[2], in, out, g_taps.offs.p,
                                                           g_taps.w.p, g_taps.ntaps, g_taps.W);
    VFEM_LAUNCH_CHECK();
}

void launch_projection(int64_t n, double beta, const double *in, double *out, cudaStream_t st) {
    projection_kernel<<<gridFor(n, BS), BS, 0, st>>>(n, beta, std::tanh(0.5 * beta), in, out);
    VFEM_LAUNCH_CHECK();
}

void launch_projection_backprop(int64_t n, double beta, const double *in, const double *vars, double *out,
                                cudaStream_t st) {
    const double scale = 1.0 / (2 * std::tanh(0.5 * beta) / beta);
    projection_backprop_kernel<<<gridFor(n, BS), BS, 0, st>>>(n, beta, scale, in, vars, out);
    VFEM_LAUNCH_CHECK();
}

void launch_oc_update(int64_t n, const double *x0, const double *dJ, const double *dc, double lambda, double m,
                      double p, double *out, cudaStream_t st) {
    oc_update_kernel<<<gridFor(n, BS), BS, 0, st>>>(n, x0, dJ, dc, lambda, m, p, out);
    VFEM_LAUNCH_CHECK();
}

void launch_sum_partials(const double *x, int64_t n, double *partials, cudaStream_t st) {
    sum_kernel<<<REDUCE_BLOCKS, BS, 0, st>>>(x, n, partials);
    VFEM_LAUNCH_CHECK();
}


// Device address of the filter scratch array, looked up once per device (with that device
// current) by the first call on it.
static double *noalloc_scratch_address() {
    static std::mutex mu;
    static double *addr[64] = {nullptr};
    int dev = 0;
    VFEM_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) throw Error(ERR_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        VFEM_CUDA(cudaGetSymbolAddress(&p, g_filter_scratch));
        addr[dev] = (double *)p;
    }
    return addr[dev];
}

int noalloc_filter_max_radius() { return NOALLOC_MAX_RADIUS; }

void launch_smoothing_filter_noalloc(const int dims[3], int radius, int type, const double *in, double *out,
                                     cudaStream_t st) {
    if (radius < 0 || radius > NOALLOC_MAX_RADIUS)
        throw Error(ERR_ARG, "filter radius " + std::to_string(radius) + " exceeds the maximum " +
                                 std::to_string(NOALLOC_MAX_RADIUS) + " of the allocation-free filter");
    double *scratch = noalloc_scratch_address();
    noalloc_taps_kernel<<<1, TAPS_BS, 0, st>>>(radius, type, scratch);
    VFEM_LAUNCH_CHECK();
    const int64_t n = (int64_t)dims[0] * dims[1] * dims[2];
    smoothing_filter_noalloc_kernel<<<gridFor(n, BS), BS, 0, st>>>(dims[0], dims[1], dims[2], in, out, scratch);
    VFEM_LAUNCH_CHECK();
}

}  // namespace vfem
