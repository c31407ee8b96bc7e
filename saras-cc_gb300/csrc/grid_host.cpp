// Host grid geometry (see grid_host.h).  The arithmetic of every metric is
// written in the reference's operation order so the tables are bit-identical
// to what lib/grid/grid.cc produces with the same libm.
#include "grid_host.h"

#include <algorithm>
#include <cmath>

namespace saras {

namespace {

// Cell centre and metrics of the tanh map at transformed coordinate xi
// (grid.cc:443-463 for the finest level, grid.cc:628-648 for coarse levels).
void stretch(int type, double beta, double len, double xi, double &x, double &fx, double &fxx,
             double &fx2) {
    const double thb = std::tanh(beta);
    const double btl = beta * len;
    if (type == SARAS_MESH_DOUBLE_TANH) {
        x = len * (1.0 - std::tanh(beta * (1.0 - 2.0 * xi)) / thb) / 2.0;
        const double ndx = x / len;
        fx = thb / (btl * (1.0 - std::pow((1.0 - 2.0 * ndx) * thb, 2)));
        fxx = -4.0 * std::pow(thb, 3) * (1.0 - 2.0 * ndx) /
              (len * btl * std::pow(1.0 - std::pow(thb * (1.0 - 2.0 * ndx), 2), 2));
    } else {
        x = len * (1.0 - std::tanh(beta * (1.0 - xi)) / thb);
        const double ndx = x / len;
        fx = thb / (btl * (1.0 - std::pow((1.0 - ndx) * thb, 2)));
        fxx = -2.0 * std::pow(thb, 3) * (1.0 - ndx) /
              (len * btl * std::pow(1.0 - std::pow(thb * (1.0 - ndx), 2), 2));
    }
    fx2 = std::pow(fx, 2.0);
}

}  // namespace

int HostGrid::reference_depth() const {
    // grid::setVCDepth (grid.cc:688-716): deepest halving that divides every
    // active extent, one less if that would leave a single cell, one less
    // again when no axis is periodic.
    int depth = 0;
    for (;;) {
        const int div = int(std::pow(2, depth));
        bool rem = false;
        for (int d = 0; d < 3; d++)
            if (active(d) && N[d] % div) rem = true;
        if (rem) break;
        depth++;
    }
    depth--;
    const int div = int(std::pow(2, depth));
    int smallest = 1 << 30;
    for (int d = 0; d < 3; d++)
        if (active(d)) smallest = std::min(smallest, N[d] / div);
    if (smallest == 1) depth--;
    bool periodic = false;
    for (int d = 0; d < 3; d++)
        if (active(d) && per[d]) periodic = true;
    if (!periodic) depth--;
    return depth;
}

saras_status HostGrid::build(const saras_grid_desc &g, int levels_override) {
    if (g.dims != 2 && g.dims != 3) return SARAS_BAD_ARG;
    if (g.pad != 1 && g.pad != 2) return SARAS_BAD_ARG;
    dims = g.dims;
    pad = g.pad;
    for (int d = 0; d < 3; d++) {
        N[d] = g.n[d];
        L[d] = g.len[d];
        mesh[d] = g.mesh_type[d];
        beta[d] = g.beta[d];
        per[d] = g.periodic[d] != 0;
    }
    if (dims == 2) {
        N[1] = 1;
        mesh[1] = SARAS_MESH_UNIFORM;
    }
    for (int d = 0; d < 3; d++) {
        if (!active(d)) continue;
        if (N[d] < 2 || N[d] > (1 << 20) || !(L[d] > 0.0) || mesh[d] < 0 || mesh[d] > 2)
            return SARAS_BAD_ARG;
        if (mesh[d] != SARAS_MESH_UNIFORM && !(beta[d] > 0.0)) return SARAS_BAD_ARG;
    }
    for (int d = 0; d < 3; d++) dxi[d] = 1.0 / double(N[d]);
    if (dims == 2) dxi[1] = 1.0;

    int depth = reference_depth();
    if (levels_override > 0) {
        const int f = 1 << (levels_override - 1);
        for (int d = 0; d < 3; d++)
            if (active(d) && (N[d] % f != 0 || N[d] / f < 2)) return SARAS_BAD_ARG;
        depth = levels_override - 1;
    }
    if (depth < 0) return SARAS_BAD_ARG;
    levels = depth + 1;

    lv.assign((size_t)levels, std::vector<AxisLevel>(3));
    for (int d = 0; d < 3; d++) {
        // Transformed coordinate of the finest level including the field pad
        // (grid::createXiEtaZeta, grid.cc:318-340) and the uniform map
        // (grid::createUniformGrid, grid.cc:358-391).
        const int p = (dims == 2 && d == 1) ? 1 : pad;
        const int m = N[d] + 2 * p;
        std::vector<double> xi((size_t)m), x((size_t)m), f1((size_t)m), f2((size_t)m), f3((size_t)m);
        for (int i = -p; i < N[d] + p; i++) {
            xi[(size_t)(i + p)] = double(2 * i + 1) * dxi[d] / 2;
            x[(size_t)(i + p)] = L[d] * xi[(size_t)(i + p)];
            f1[(size_t)(i + p)] = 1.0 / L[d];
            f2[(size_t)(i + p)] = 0.0;
            f3[(size_t)(i + p)] = std::pow(f1[(size_t)(i + p)], 2.0);
        }
        // Multigrid levels with the uniform defaults (grid::mgGridMetrics()).
        for (int l = 0; l < levels; l++) {
            AxisLevel &a = lv[(size_t)l][(size_t)d];
            a.n = (dims == 2 && d == 1) ? 1 : int(N[d] / std::pow(2, l));
            const size_t cnt = (size_t)(a.n + 2);
            a.xi.assign(cnt, 0.0);
            a.x.assign(cnt, 0.0);
            a.xi_x.assign(cnt, 1.0 / L[d]);
            a.xixx.assign(cnt, 0.0);
            a.xix2.assign(cnt, std::pow(1.0 / L[d], 2.0));
            if (!active(d)) continue;
            if (l == 0) {
                for (int i = -1; i <= a.n; i++) {
                    a.xi[(size_t)(i + 1)] = xi[(size_t)(i + p)];
                    a.x[(size_t)(i + 1)] = x[(size_t)(i + p)];
                }
            } else {
                const AxisLevel &f = lv[(size_t)(l - 1)][(size_t)d];
                for (int i = 0; i < a.n; i++) {
                    a.xi[(size_t)(i + 1)] = (f.xi[(size_t)(2 * i + 1)] + f.xi[(size_t)(2 * i + 2)]) / 2.0;
                    a.x[(size_t)(i + 1)] = L[d] * a.xi[(size_t)(i + 1)];
                }
                a.xi[0] = -a.xi[1];
                a.x[0] = -a.x[1];
                a.xi[(size_t)(a.n + 1)] = 1.0 + a.xi[1];
                a.x[(size_t)(a.n + 1)] = L[d] + a.x[1];
            }
        }
        // Tanh stretching (grid::createTanHypGrid and mgGridMetrics(dim)).
        if (active(d) && mesh[d] != SARAS_MESH_UNIFORM) {
            for (int i = 0; i < N[d]; i++) {
                const size_t q = (size_t)(i + p);
                stretch(mesh[d], beta[d], L[d], xi[q], x[q], f1[q], f2[q], f3[q]);
            }
            for (int s = 0; s < p; s++) {  // left pad images of the right end
                const size_t q = (size_t)s, src = (size_t)(N[d] - p + s + p);
                x[q] = x[src] - L[d];
                f1[q] = f1[src];
                f2[q] = f2[src];
                f3[q] = f3[src];
            }
            for (int s = 0; s < p; s++) {  // right pad images of the left end
                const size_t q = (size_t)(N[d] + s + p), src = (size_t)(s + p);
                x[q] = L[d] + x[src];
                f1[q] = f1[src];
                f2[q] = f2[src];
                f3[q] = f3[src];
            }
            AxisLevel &a0 = lv[0][(size_t)d];
            for (int i = -1; i <= a0.n; i++) {
                const size_t q = (size_t)(i + p), o = (size_t)(i + 1);
                a0.x[o] = x[q];
                a0.xi_x[o] = f1[q];
                a0.xixx[o] = f2[q];
                a0.xix2[o] = f3[q];
            }
            for (int l = 1; l < levels; l++) {
                AxisLevel &a = lv[(size_t)l][(size_t)d];
                const int n = a.n;
                for (int i = 0; i < n; i++) {
                    const size_t o = (size_t)(i + 1);
                    stretch(mesh[d], beta[d], L[d], a.xi[o], a.x[o], a.xi_x[o], a.xixx[o], a.xix2[o]);
                }
                a.x[0] = -a.x[1];
                a.xi_x[0] = a.xi_x[(size_t)n];
                a.xixx[0] = a.xixx[(size_t)n];
                a.xix2[0] = a.xix2[(size_t)n];
                a.x[(size_t)(n + 1)] = L[d] + a.x[1];
                a.xi_x[(size_t)(n + 1)] = a.xi_x[1];
                a.xixx[(size_t)(n + 1)] = a.xixx[1];
                a.xix2[(size_t)(n + 1)] = a.xix2[1];
            }
        }
        fx[d] = x;
        fxi_x[d] = f1;
        fxixx[d] = f2;
        fxix2[d] = f3;
    }
    return SARAS_OK;
}

// Left null vector of the 1-D finest-level operator with Neumann ghosts on
// both ends: row i reads a_i u_{i-1} + b_i u_i + c_i u_{i+1} with
// a = xix2*ihx2 - xixx*i2hx, c = xix2*ihx2 + xixx*i2hx, b = -(a + c) and the
// ghost folded into the diagonal.  w solves w^T A = 0 by forward recurrence.
void neumann_null_vector(const HostGrid &g, int axis, double *w) {
    const AxisLevel &a = g.lv[0][(size_t)axis];
    const int n = a.n;
    const double h = g.dxi[axis];
    const double ih2 = 1.0 / (h * h), i2h = 0.5 / h;
    std::vector<double> lo((size_t)n), up((size_t)n);
    for (int i = 0; i < n; i++) {
        const double c2 = a.xix2[(size_t)(i + 1)] * ih2, c1 = a.xixx[(size_t)(i + 1)] * i2h;
        lo[(size_t)i] = c2 - c1;  // coefficient of u_{i-1}
        up[(size_t)i] = c2 + c1;  // coefficient of u_{i+1}
    }
    // Column j of A: up[j-1] w_{j-1} + diag_j w_j + lo[j+1] w_{j+1} = 0 with
    // diag_0 = -up[0], diag_j = -(lo[j] + up[j]), diag_{n-1} = -lo[n-1].
    // Equivalent flux form: w_{j+1} lo[j+1] = w_j up[j].
    w[0] = 1.0;
    for (int j = 0; j + 1 < n; j++) w[j + 1] = w[j] * up[(size_t)j] / lo[(size_t)(j + 1)];
    double m = 0.0;
    for (int j = 0; j < n; j++) m = std::max(m, std::fabs(w[j]));
    for (int j = 0; j < n; j++) w[j] /= m;
}

}  // namespace saras
