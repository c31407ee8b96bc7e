// Entry points of the C ABI that need no device: error reporting, grid
// metrics, level counts, the Neumann null vector and the RBC coefficients.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "grid_host.h"

namespace saras {

static thread_local char g_err[512] = {0};

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

saras_status cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
    set_error("%s failed at %s:%d: %s", what, file, line, cudaGetErrorString(e));
    cudaGetLastError();
    if (e == cudaErrorMemoryAllocation) return SARAS_OOM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return SARAS_NO_DEVICE;
    return SARAS_CUDA_ERR;
}

}  // namespace saras

extern "C" {

const char *saras_status_string(saras_status s) {
    switch (s) {
    case SARAS_OK: return "OK";
    case SARAS_NOT_CONVERGED: return "NOT_CONVERGED";
    case SARAS_BAD_ARG: return "BAD_ARG";
    case SARAS_OOM: return "OOM";
    case SARAS_BUDGET: return "BUDGET";
    case SARAS_TIMEOUT: return "TIMEOUT";
    case SARAS_CUDA_ERR: return "CUDA_ERR";
    case SARAS_NO_DEVICE: return "NO_DEVICE";
    case SARAS_DIVERGED: return "DIVERGED";
    case SARAS_NAN: return "NAN";
    }
    return "UNKNOWN";
}

const char *saras_last_error(void) { return saras::g_err; }

saras_status saras_grid_metrics(const saras_grid_desc *grid, int32_t levels, int32_t level, int32_t axis, double *x,
                                double *xixx, double *xix2, int32_t *n_out) {
    if (!grid) return SARAS_BAD_ARG;
    saras::HostGrid g;
    saras_status s = g.build(*grid, levels);
    if (s != SARAS_OK) return s;
    if (level < 0 || level >= g.levels || axis < 0 || axis > 2 || !g.active(axis)) return SARAS_BAD_ARG;
    const saras::AxisLevel &a = g.lv[(size_t)level][(size_t)axis];
    for (int i = 0; i < a.n + 2; i++) {
        if (x) x[i] = a.x[(size_t)i];
        if (xixx) xixx[i] = a.xixx[(size_t)i];
        if (xix2) xix2[i] = a.xix2[(size_t)i];
    }
    if (n_out) *n_out = a.n;
    return SARAS_OK;
}

int32_t saras_reference_levels(const saras_grid_desc *grid) {
    if (!grid) return -1;
    saras::HostGrid g;
    if (g.build(*grid, 0) != SARAS_OK) return -1;
    return g.levels;
}

saras_status saras_neumann_null_vector(const saras_grid_desc *grid, int32_t axis, double *w) {
    if (!grid || !w) return SARAS_BAD_ARG;
    saras::HostGrid g;
    saras_status s = g.build(*grid, 0);
    if (s != SARAS_OK) return s;
    if (axis < 0 || axis > 2 || !g.active(axis)) return SARAS_BAD_ARG;
    saras::neumann_null_vector(g, axis, w);
    return SARAS_OK;
}

saras_status saras_rbc_coefficients(int32_t rbc_type, double ra, double pr, double *nu, double *kappa, double *fb) {
    // timestep::timestep (lib/timestep/timestep.cc:74-99) and
    // buoyantForce::buoyantForce (lib/force/buoyantForce.cc:45-57)
    double n, k, f;
    switch (rbc_type) {
    case 1: n = pr; k = 1.0; f = ra * pr; break;
    case 2: n = std::sqrt(pr / ra); k = 1.0 / std::sqrt(pr * ra); f = 1.0; break;
    case 3: n = 1.0; k = 1.0 / pr; f = ra; break;
    case 4: n = std::sqrt(pr / ra); k = 1.0 / std::sqrt(pr * ra); f = pr; break;
    default:
        saras::set_error("invalid RBC type %d", rbc_type);
        return SARAS_BAD_ARG;
    }
    if (nu) *nu = n;
    if (kappa) *kappa = k;
    if (fb) *fb = f;
    return SARAS_OK;
}

}  // extern "C"
