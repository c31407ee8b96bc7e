// Shared helpers of the GB300 SARAS hot-path library: error reporting,
// padded device array layout and FP64 arithmetic with explicit rounding.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <utility>

#include "../../include/saras_gb300.h"

namespace saras {

// Records a message for saras_last_error() on the calling thread.
void set_error(const char *fmt, ...);
saras_status cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define SARAS_CUDA(call)                                                          \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) return ::saras::cuda_fail(e_, #call, __FILE__, __LINE__); \
    } while (0)

#define SARAS_TRY(call)                               \
    do {                                              \
        saras_status s_ = (call);                     \
        if (s_ != SARAS_OK) return s_;                \
    } while (0)

// Padded level array: core (0..n-1 per axis) plus one ghost layer.  Element
// (i,j,k) sits at (i+1)*s0 + (j+1)*s1 + (k+KOFF): each k-row starts its core
// on a 32-byte boundary (KOFF = 4 elements) so rows load with aligned
// vector accesses; the ghost k=-1 sits at KOFF-1.
constexpr int KOFF = 4;

struct Lay {
    int n0, n1, n2;  // core extents (n1 == 1 for the planar case)
    int64_t s0, s1;  // element strides of i and j (k stride 1)
    int64_t size;    // elements including alignment padding

    __host__ __device__ __forceinline__ int64_t at(int i, int j, int k) const {
        return (int64_t)(i + 1) * s0 + (int64_t)(j + 1) * s1 + (int64_t)(k + KOFF);
    }
};

// Row-split position of cell (i, j, k) (the MIXED form's finest level, see
// Level::rs): each row holds its red cells ((i + j + k) even), then its
// black cells, each in k order.
__host__ __device__ __forceinline__ int64_t rs_at(const Lay &L, int i, int j, int k) {
    return L.at(i, j, 0) + (k >> 1) + (int64_t)(((i + j + k) & 1) * (L.n2 >> 1));
}

inline Lay make_lay(int n0, int n1, int n2) {
    Lay l;
    l.n0 = n0;
    l.n1 = n1;
    l.n2 = n2;
    l.s1 = ((int64_t)n2 + KOFF + 1 + 3) / 4 * 4;
    l.s0 = l.s1 * (n1 + 2);
    l.size = l.s0 * (n0 + 2);
    return l;
}

// Exact coarsest solve of the MIXED form by fast diagonalisation: per axis
// the eigenvectors V (row i, column mode), V^-1 (row mode) and eigenvalues
// of the level's 1-D operator (coarse_fd.cpp).  ok = 0: red-black sweeps.
constexpr int FD_MAX_CELLS = 4096;
constexpr int FD_MAX_N = 64;
constexpr double FD_TOL_MAX = 1e-9;  // coarsest tolerances at or below this take the exact solve
constexpr int FD_MIN_CELLS = 512;    // ... on coarsest levels of at least this many cells
struct FDiag {
    const double *v[3], *vi[3], *lam[3];
    double lam_tol;  // |eigenvalue sum| at or below this is the null mode
    int ok;
};
inline int64_t fd_elems(const Lay &L) {
    const int n[3] = {L.n0, L.n1, L.n2};
    int64_t e = 0;
    for (int d = 0; d < 3; d++) e += 2 * (int64_t)n[d] * n[d] + n[d];
    return e;
}
inline bool fd_fits(const Lay &L) {
    const int64_t cells = (int64_t)L.n0 * L.n1 * L.n2;
    return cells >= FD_MIN_CELLS && cells <= FD_MAX_CELLS && L.n0 <= FD_MAX_N && L.n1 <= FD_MAX_N &&
           L.n2 <= FD_MAX_N;
}

// FP64 with explicit rounding: these never contract into fused
// multiply-adds, which keeps the exact kernels' results bit-identical to the
// reference's separately rounded operations.
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }

inline unsigned cdiv(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

// Programmatic dependent launch: the V-cycle kernels are launched with
// programmatic stream serialisation, so the next kernel's blocks are
// scheduled while this one drains.  Every such kernel first lets its
// dependants launch and then waits until the kernel before it has finished
// and its writes are visible; launched without the attribute both are no-ops.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                       Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Visits the core cells of a level for grid-wide reductions: each warp takes
// whole k-rows (32-bit index arithmetic only) and its lanes stride along k,
// so loads stay coalesced.
template <class LY, class Fn>
__device__ __forceinline__ void for_core_rows(const LY &L, Fn &&fn) {
    const int lane = threadIdx.x & 31;
    const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    const int rows = L.n0 * L.n1;
    for (int r = warp; r < rows; r += nwarps) {
        const int i = r / L.n1, j = r - i * L.n1;
        for (int k = lane; k < L.n2; k += 32) fn(i, j, k);
    }
}

}  // namespace saras
