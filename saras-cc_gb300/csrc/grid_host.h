// Host-side grid geometry of the GB300 solver: cell centres and tanh
// stretching metrics of every multigrid level, computed once in FP64 on the
// host and uploaded; the GPU never evaluates tanh.
//
// Follows grid::grid, createUniformGrid, mgGridMetrics, createTanHypGrid and
// setVCDepth (lib/grid/grid.cc:61-742) for a single rank, and the per-level
// copies poisson::copyDerivs makes (lib/poisson/poisson.cc:501-622).
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/saras_gb300.h"

namespace saras {

// One coordinate direction at one multigrid level; arrays hold indices
// -1..n (n + 2 values, offset by one).
struct AxisLevel {
    int n = 0;
    std::vector<double> xi, x, xi_x, xixx, xix2;
    double at(const std::vector<double> &a, int i) const { return a[(size_t)(i + 1)]; }
};

struct HostGrid {
    int dims = 3;
    int N[3] = {1, 1, 1};
    double L[3] = {1, 1, 1};
    int mesh[3] = {0, 0, 0};
    double beta[3] = {1, 1, 1};
    bool per[3] = {false, false, false};
    int pad = 1;
    double dxi[3] = {1, 1, 1};
    int levels = 0;                          // vcdGlo + 1
    std::vector<std::vector<AxisLevel>> lv;  // lv[level][axis]
    // Finest-level field metrics with the field pad: indices -pad..N+pad-1.
    std::vector<double> fx[3], fxi_x[3], fxixx[3], fxix2[3];

    bool active(int d) const { return dims == 3 || d != 1; }
    // Builds the geometry; `levels_override` > 0 replaces setVCDepth.
    saras_status build(const saras_grid_desc &g, int levels_override);
    // setVCDepth's global depth (vcdGlo) for the descriptor already stored.
    int reference_depth() const;
};

// Left null vector of the 1-D all-Neumann finest-level operator.
void neumann_null_vector(const HostGrid &g, int axis, double *w);

// Eigen-decomposition A = V diag(lam) V^-1 of the 1-D operator
// cm u(i-1) + cp u(i+1) - 2 a2 u(i) of one axis with its ghost rule folded
// in (periodic, or the mirrored sign sg_lo / sg_hi: +1 Neumann, -1
// Dirichlet); V and Vi are n x n row major.  False when the operator is not
// similar to a symmetric one through a diagonal scaling (coarse_fd.cpp).
bool coarse_axis_eigen(int n, const double *cm, const double *cp, const double *a2, bool per, int sg_lo, int sg_hi,
                       double *V, double *Vi, double *lam);

}  // namespace saras
