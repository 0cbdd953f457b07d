// Common device/host helpers for the VoxelFEM GB300 kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

namespace vfem {

// Error carrying a status code back through the C ABI.
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

enum Status { OK = 0, ERR_ARG = 1, ERR_CUDA = 2, ERR_NAN = 3, ERR_STATE = 4, ERR_NOT_SPD = 5 };

inline void cudaCheck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw Error(ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define VFEM_CUDA(x) ::vfem::cudaCheck((x), #x)
// Every kernel launch goes through this check, which also counts it (graph replays are
// counted from the captured node count).
uint64_t &launchCounter();
#define VFEM_LAUNCH_CHECK()                                              \
    do {                                                                 \
        ::vfem::cudaCheck(cudaGetLastError(), "kernel launch");          \
        ++::vfem::launchCounter();                                       \
    } while (0)

// Programmatic dependent launch. Kernels of the solve's inner loops start with
// VFEM_PDL_ENTRY(): they wait for the previous kernel of the stream to complete (and its memory
// to be visible), then allow the next kernel to be scheduled, so its launch overlaps this
// kernel's execution. Launched without the attribute, the entry is a no-op.
#if defined(__CUDA_ARCH__)
#define VFEM_PDL_ENTRY()                                                    \
    do {                                                                    \
        asm volatile("griddepcontrol.wait;" ::: "memory");                  \
        asm volatile("griddepcontrol.launch_dependents;" ::: "memory");     \
    } while (0)
#else
#define VFEM_PDL_ENTRY() \
    do {                 \
    } while (0)
#endif

// Process-wide switch of programmatic dependent launch (on unless VFEM_PDL=0).
bool pdlEnabled();

// kernel<<<grid, block, smem, st>>>(args...) with programmatic stream serialisation; the kernel
// must begin with VFEM_PDL_ENTRY().
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdlEnabled() ? 1 : 0;
    cudaCheck(cudaLaunchKernelEx(&cfg, kernel, args...), "kernel launch");
}

constexpr int BUILD_DIR = 1;         // layers are stacked along y (TensorProductSimulator.hh:1851)
constexpr int64_t LAYER_MASK_NONE = 2147483647;
constexpr int MARGIN = 4;            // detached-node margin copied with b (MultigridSolver.hh:532)
constexpr int NUM_SMS = 152;

// Geometry of one level of the voxel hierarchy (Q1 hexahedra).
struct Geom {
    int ne[3];       // elements per axis
    int nn[3];       // nodes per axis = ne + 1
    int64_t NE, NN;  // element / node counts
    int64_t ld;      // leading dimension of a nodal SoA vector (component stride), padded
    int firstMaskedE;  // first masked element layer along y (or LAYER_MASK_NONE)
    int firstDetN;     // first detached node layer along y
    // Device copy {firstMaskedE, firstDetN} of the level's mask. When set, kernels read the
    // mask from it, launch over the full grid and skip the detached rows, so a captured CUDA
    // graph stays valid when the fabrication mask height changes.
    const int *dyn = nullptr;
    // Colour-ordered node positions (plane-layout stencils): colour c = 4(i&1) + 2(j&1) + (k&1)
    // starts at coff[c]; hc1[b], hc2[b] = nodes with j&1 == b, k&1 == b along y, z.
    int64_t coff[8];
    int hc1[2], hc2[2];
    __host__ __device__ int detN() const {
#if defined(__CUDA_ARCH__)
        if (dyn) return dyn[1];
#endif
        return firstDetN;
    }
    __host__ __device__ int maskedE() const {
#if defined(__CUDA_ARCH__)
        if (dyn) return dyn[0];
#endif
        return firstMaskedE;
    }
    __host__ __device__ int nyv() const { const int d = detN(); return d < nn[1] ? d : nn[1]; }  // nondetached node rows
    __host__ __device__ int nev() const { const int m = maskedE(); return m < ne[1] ? m : ne[1]; }
    __host__ __device__ int64_t node(int i, int j, int k) const { return ((int64_t)i * nn[1] + j) * nn[2] + k; }
    __host__ __device__ int64_t elem(int i, int j, int k) const { return ((int64_t)i * ne[1] + j) * ne[2] + k; }
    // Zero-padded element arrays carry one ghost layer on every side: element (i, j, k),
    // -1 <= i <= ne[0], sits at padElem(i, j, k); padNE() elements in all.
    __host__ __device__ int64_t padElem(int i, int j, int k) const {
        return ((int64_t)(i + 1) * (ne[1] + 2) + (j + 1)) * (ne[2] + 2) + (k + 1);
    }
    __host__ __device__ int64_t padNE() const { return (int64_t)(ne[0] + 2) * (ne[1] + 2) * (ne[2] + 2); }
    // Guard (in elements) that a nodal gather reaching one node past the grid in every
    // direction needs before and after a 3 x NN vector.
    __host__ __device__ int64_t nodeGuard() const { return (int64_t)nn[1] * nn[2] + nn[2] + 1; }
};

inline int64_t padTo(int64_t n, int64_t a) { return (n + a - 1) / a * a; }

inline Geom makeGeom(const int ne[3]) {
    Geom g;
    for (int d = 0; d < 3; ++d) { g.ne[d] = ne[d]; g.nn[d] = ne[d] + 1; }
    g.NE = (int64_t)ne[0] * ne[1] * ne[2];
    g.NN = (int64_t)g.nn[0] * g.nn[1] * g.nn[2];
    g.ld = g.NN;  // SoA component stride: exactly the (nn, 3) column-major VField layout
    g.firstMaskedE = (int)LAYER_MASK_NONE;
    g.firstDetN = (int)LAYER_MASK_NONE;
    auto half = [](int n, int b) { return (n + 1 - b) >> 1; };
    for (int b = 0; b < 2; ++b) {
        g.hc1[b] = half(g.nn[1], b);
        g.hc2[b] = half(g.nn[2], b);
    }
    for (int c = 0; c < 8; ++c) {
        const int cx = (c >> 2) & 1, cy = (c >> 1) & 1, cz = c & 1;
        g.coff[c] = (cx ? (int64_t)half(g.nn[0], 0) * g.nn[1] * g.nn[2] : 0) +
                    (int64_t)half(g.nn[0], cx) * ((cy ? (int64_t)half(g.nn[1], 0) * g.nn[2] : 0) +
                                                  (int64_t)half(g.nn[1], cy) * (cz ? half(g.nn[2], 0) : 0));
    }
    return g;
}

inline unsigned gridFor(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 2147483647LL) g = 2147483647LL;
    return (unsigned)g;
}

// Owning device buffer.
template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    size_t guard = 0;  // zeroed elements before p[0] and after p[n - 1]
    DevBuf() = default;
    explicit DevBuf(size_t count) { alloc(count); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n), guard(o.guard) { o.p = nullptr; o.n = 0; o.guard = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept {
        if (this != &o) {
            release();
            p = o.p; n = o.n; guard = o.guard;
            o.p = nullptr; o.n = 0; o.guard = 0;
        }
        return *this;
    }
    ~DevBuf() { release(); }
    // count elements addressed from p, plus `guard` zeroed elements on either side (gathers that
    // read past the ends of the array without bounds checks stay inside the allocation)
    void alloc(size_t count, size_t guard_ = 0) {
        if (count == n && guard_ == guard && p) return;
        release();
        if (count) {
            T *base = nullptr;
            VFEM_CUDA(cudaMalloc(&base, (count + 2 * guard_) * sizeof(T)));
            if (guard_) {
                VFEM_CUDA(cudaMemset(base, 0, guard_ * sizeof(T)));
                VFEM_CUDA(cudaMemset(base + guard_ + count, 0, guard_ * sizeof(T)));
            }
            p = base + guard_;
            guard = guard_;
        }
        n = count;
    }
    void release() {
        if (p) cudaFree(p - guard);
        p = nullptr;
        n = 0;
        guard = 0;
    }
    size_t bytes() const { return n * sizeof(T); }
};

}  // namespace vfem
