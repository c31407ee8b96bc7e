// Multigrid solve with a fixed, file-scope device scratch: the entry point
// saras_mg_solve_static allocates no device memory.  It serves callers that
// cannot allocate at solve time: cudaMalloc and cudaFree synchronise the
// whole device (stalling the caller's other streams), a caching allocator
// that has reserved the free HBM leaves nothing for a second allocator, and
// a time step must not fail half-way for want of memory.  The scratch is a
// static __device__ array of SARAS_STATIC_SCRATCH_BYTES; grids whose
// hierarchy does not fit are rejected before any device work.

#include "mg_fast.cuh"

namespace saras {
saras_status mg_solve_in_scratch(const saras_grid_desc *gd, const saras_mg_params *prm, cudaStream_t stream,
                                 char *scratch, size_t scratch_bytes, double *lhs, const double *rhs,
                                 const int64_t st[3], double *res_hist, int32_t hist_cap, int32_t *n_cycles);
}

namespace {

constexpr size_t kScratchBytes = SARAS_STATIC_SCRATCH_BYTES;
static __device__ __align__(256) double g_scratch[kScratchBytes / sizeof(double)];

}  // namespace

extern "C" saras_status saras_mg_solve_static(const saras_grid_desc *grid, const saras_mg_params *prm,
                                              void *stream, double *lhs, const double *rhs,
                                              const int64_t strides[3], double *res_hist, int32_t hist_cap,
                                              int32_t *n_cycles) {
    if (!grid || !prm || !lhs || !rhs || !strides) {
        saras::set_error("null argument");
        return SARAS_BAD_ARG;
    }
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        saras::set_error("no CUDA device");
        return SARAS_NO_DEVICE;
    }
    // the array's device address on the current device, looked up on every
    // call (a cudaDeviceReset loads the module again at another address;
    // the lookup costs microseconds against a solve)
    void *base = nullptr;
    e = cudaGetSymbolAddress(&base, g_scratch);
    if (e != cudaSuccess) return saras::cuda_fail(e, "cudaGetSymbolAddress", __FILE__, __LINE__);
    return saras::mg_solve_in_scratch(grid, prm, (cudaStream_t)stream, static_cast<char *>(base), kScratchBytes,
                                      lhs, rhs, strides, res_hist, hist_cap, n_cycles);
}
