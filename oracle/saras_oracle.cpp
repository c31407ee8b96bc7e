/*
 * saras_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the checker, never the product).
 *
 * CPU restatement of SARAS-CC's data-parallel hot path with single-MPI-rank
 * semantics: the grid metrics (lib/grid/grid.cc), the cell-centred multigrid
 * Poisson solve (lib/poisson/poisson.cc, poisson_d3.cc, poisson_d2.cc) and the
 * low-storage RK3 time step with its CN Jacobi sweeps and FD stencils
 * (lib/timestep/lsRK3_d3.cc, predictors.cc, timestep.cc; lib/field/ (derivative, vfield, sfield, plainsf, plainvf, field);
 * lib/boundary/dirichlet.cc, neumann.cc; lib/force/buoyantForce.cc).
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it.
 *
 * Every floating-point expression keeps the reference's operation order and
 * association; the file is compiled with -ffp-contract=off so that no
 * multiply-add is fused.  OpenMP threads split the outer loops exactly where
 * the reference's own "#pragma omp parallel for" does; all results except the
 * L1/L2 residual sums are independent of the thread count, and those sums are
 * taken in a fixed order here.
 *
 * Parity status: the reference cannot be compiled in this environment (it
 * requires MPI, Blitz++, yaml-cpp and HDF5) and stores no golden vectors.
 * This restatement is pinned against the reference's own known answer -- the
 * TEST_POISSON manufactured solution of tests/mgTest (p = r^2/6 in 3D,
 * r^2/4 in 2D) -- against the analytic tanh-grid formulas and against the
 * level counts of setVCDepth.  Exact solutions of the equations pin it to
 * discretisation order: manufactured Poisson solutions on stretched meshes,
 * the Taylor-Green vortex of lib/initial/taylorGreen.cc, and sine modes
 * decaying between no-slip, moving and heat-flux walls.  The Blitz++
 * stencil operators central12n, central22n, central14n and central24n
 * (lib/field/derivative.cc:104-318) come from a third-party library that is
 * absent here (version unpinned); they are restated from their published
 * definitions, (F[+1]-F[-1])*0.5, (F[-1]-2F)+F[+1] and the fourth-order
 * pair over /12, and parity at that boundary is unpinned: their formulas are
 * held by polynomial exactness, their rounding order is this restatement's.
 */
#include "../include/saras_gb300.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

/* Padded 3-D array indexed from -pad, row-major (i, j, k), k fastest: the
 * layout of a reindexed blitz::Array<real,3>. */
struct Arr3 {
    int n[3] = {0, 0, 0};
    int p[3] = {0, 0, 0};
    int64_t s0 = 0, s1 = 0;
    std::vector<double> v;

    void init(int nx, int ny, int nz, int px, int py, int pz) {
        n[0] = nx; n[1] = ny; n[2] = nz;
        p[0] = px; p[1] = py; p[2] = pz;
        s1 = nz + 2 * pz;
        s0 = s1 * (ny + 2 * py);
        v.assign((size_t)(s0 * (nx + 2 * px)), 0.0);
    }
    inline double &operator()(int i, int j, int k) {
        return v[(size_t)((i + p[0]) * s0 + (j + p[1]) * s1 + (k + p[2]))];
    }
    inline double operator()(int i, int j, int k) const {
        return v[(size_t)((i + p[0]) * s0 + (j + p[1]) * s1 + (k + p[2]))];
    }
    int lo(int d) const { return -p[d]; }
    int hi(int d) const { return n[d] + p[d] - 1; }
    void fill(double x) { std::fill(v.begin(), v.end(), x); }
};

/* 1-D array indexed from `base` (a reindexed blitz::Array<real,1>). */
struct Vec1 {
    int base = 0;
    std::vector<double> v;
    void init(int lo, int hi) { base = lo; v.assign((size_t)(hi - lo + 1), 0.0); }
    inline double &operator[](int i) { return v[(size_t)(i - base)]; }
    inline double operator[](int i) const { return v[(size_t)(i - base)]; }
};

int g_threads = 1;

/* ------------------------------------------------------------------ grid -- */

/* Single-rank restatement of class grid (lib/grid/grid.cc:61-742). */
struct Grid {
    int dims = 3;
    int N[3];
    double L[3];
    int mt[3];
    double beta[3];
    bool per[3];
    int pad[3];
    double dxi[3];
    int vcdGlo = 0;
    Vec1 xiG[3], xG[3];            /* global xi and physical x, -pad..N+pad-1 */
    Vec1 xi_x[3], xixx[3], xix2[3];/* local metrics (global on one rank) */
    std::vector<Vec1> gm;          /* globalMetrics: 15 arrays per level */

    bool active(int d) const { return dims == 3 || d != 1; }

    /* grid::setVCDepth (grid.cc:678-742); the local depth equals the global
     * one on a single rank. */
    int vc_depth() const {
        std::vector<int> ms;
        for (int d = 0; d < 3; d++)
            if (active(d)) ms.push_back(N[d]);
        int v = 0;
        while (true) {
            int dv = int(std::pow(2, v));
            bool rem = false;
            for (int s : ms) rem = rem || (s % dv) > 0;
            if (rem) break;
            v += 1;
        }
        v -= 1;
        int dv = int(std::pow(2, v));
        int mn = 1 << 30;
        for (int s : ms) mn = std::min(mn, s / dv);
        if (mn == 1) v -= 1;
        bool anyPer = false;
        for (int d = 0; d < 3; d++)
            if (active(d)) anyPer = anyPer || per[d];
        if (!anyPer) v -= 1;
        return v;
    }

    /* grid::mgGridMetrics() (grid.cc:521-596): uniform defaults, coarse xi
     * from the mean of the two children. */
    void mg_metrics_uniform() {
        gm.assign(15 * (vcdGlo + 1), Vec1());
        for (int lev = 0; lev <= vcdGlo; lev++) {
            int mgN[3];
            for (int d = 0; d < 3; d++) mgN[d] = int(N[d] / std::pow(2, lev));
            int ls = 15 * lev;
            for (int d = 0; d < 3; d++)
                for (int q = 0; q < 5; q++) gm[ls + 5 * d + q].init(-1, mgN[d]);
            for (int d = 0; d < 3; d++) {
                if (!active(d)) continue;
                int sls = ls + 5 * d;
                if (lev == 0) {
                    for (int i = -1; i <= mgN[d]; i++) {
                        gm[sls][i] = xiG[d][i];
                        gm[sls + 1][i] = xG[d][i];
                    }
                } else {
                    int cLen = mgN[d];
                    Vec1 &tr = gm[sls], &ph = gm[sls + 1];
                    for (int i = 0; i < cLen; i++) {
                        tr[i] = (gm[sls - 15][2 * i] + gm[sls - 15][2 * i + 1]) / 2.0;
                        ph[i] = L[d] * tr[i];
                    }
                    tr[-1] = -tr[0];
                    ph[-1] = -ph[0];
                    tr[cLen] = 1.0 + tr[0];
                    ph[cLen] = L[d] + ph[0];
                }
                for (int i = -1; i <= mgN[d]; i++) {
                    gm[sls + 2][i] = 1.0 / L[d];
                    gm[sls + 3][i] = 0.0;
                    gm[sls + 4][i] = std::pow(gm[sls + 2][i], 2.0);
                }
            }
        }
    }

    /* Stretching function and its metrics: the bodies of the loops in
     * grid::createTanHypGrid (grid.cc:442-464) and mgGridMetrics(dim)
     * (grid.cc:627-649). */
    void tanh_point(int d, double xi, double &x, double &fx, double &fxx, double &fx2) const {
        double thb = std::tanh(beta[d]);
        double btl = beta[d] * L[d];
        if (mt[d] - 1) {
            x = L[d] * (1.0 - std::tanh(beta[d] * (1.0 - 2.0 * xi)) / thb) / 2.0;
            double ndx = x / L[d];
            fx = thb / (btl * (1.0 - std::pow((1.0 - 2.0 * ndx) * thb, 2)));
            fxx = -4.0 * std::pow(thb, 3) * (1.0 - 2.0 * ndx) /
                  (L[d] * btl * std::pow(1.0 - std::pow(thb * (1.0 - 2.0 * ndx), 2), 2));
            fx2 = std::pow(fx, 2.0);
        } else {
            x = L[d] * (1.0 - std::tanh(beta[d] * (1.0 - xi)) / thb);
            double ndx = x / L[d];
            fx = thb / (btl * (1.0 - std::pow((1.0 - ndx) * thb, 2)));
            fxx = -2.0 * std::pow(thb, 3) * (1.0 - ndx) /
                  (L[d] * btl * std::pow(1.0 - std::pow(thb * (1.0 - ndx), 2), 2));
            fx2 = std::pow(fx, 2.0);
        }
    }

    /* grid::createTanHypGrid (grid.cc:411-508) and mgGridMetrics(dim)
     * (grid.cc:603-666). */
    void tanh_axis(int d) {
        int p = pad[d];
        Vec1 fx, fxx, fx2;
        fx.init(-p, N[d] + p - 1);
        fxx.init(-p, N[d] + p - 1);
        fx2.init(-p, N[d] + p - 1);
        for (int i = 0; i < N[d]; i++) tanh_point(d, xiG[d][i], xG[d][i], fx[i], fxx[i], fx2[i]);
        for (int m = 0; m < p; m++) {
            int idx = -p + m, src = N[d] - p + m;
            xG[d][idx] = xG[d][src] - L[d];
            fx[idx] = fx[src];
            fxx[idx] = fxx[src];
            fx2[idx] = fx2[src];
        }
        for (int m = 0; m < p; m++) {
            int idx = N[d] + m, src = m;
            xG[d][idx] = L[d] + xG[d][src];
            fx[idx] = fx[src];
            fxx[idx] = fxx[src];
            fx2[idx] = fx2[src];
        }
        for (int i = -1; i <= N[d]; i++) {
            gm[5 * d + 0][i] = xiG[d][i];
            gm[5 * d + 1][i] = xG[d][i];
            gm[5 * d + 2][i] = fx[i];
            gm[5 * d + 3][i] = fxx[i];
            gm[5 * d + 4][i] = fx2[i];
        }
        xi_x[d] = fx;
        xixx[d] = fxx;
        xix2[d] = fx2;
        for (int lev = 1; lev <= vcdGlo; lev++) {
            int ls = 5 * d + 15 * lev;
            int nl = int(gm[ls].v.size()) - 2;
            Vec1 ph, f1, f2, f3;
            ph.init(-1, nl);
            f1.init(-1, nl);
            f2.init(-1, nl);
            f3.init(-1, nl);
            for (int i = 0; i < nl; i++) tanh_point(d, gm[ls][i], ph[i], f1[i], f2[i], f3[i]);
            ph[-1] = -ph[0];
            f1[-1] = f1[nl - 1];
            f2[-1] = f2[nl - 1];
            f3[-1] = f3[nl - 1];
            ph[nl] = L[d] + ph[0];
            f1[nl] = f1[0];
            f2[nl] = f2[0];
            f3[nl] = f3[0];
            gm[ls + 1] = ph;
            gm[ls + 2] = f1;
            gm[ls + 3] = f2;
            gm[ls + 4] = f3;
        }
    }

    /* grid::grid (grid.cc:61-159) for one rank.  levels > 0 overrides the
     * V-cycle depth (vcdGlo = levels - 1). */
    int build(const saras_grid_desc &g, int levels) {
        dims = g.dims;
        if (dims != 2 && dims != 3) return SARAS_BAD_ARG;
        for (int d = 0; d < 3; d++) {
            N[d] = g.n[d];
            L[d] = g.len[d];
            mt[d] = g.mesh_type[d];
            beta[d] = g.beta[d];
            per[d] = g.periodic[d] != 0;
            pad[d] = g.pad;
        }
        if (g.pad != 1 && g.pad != 2) return SARAS_BAD_ARG;
        if (dims == 2) {
            N[1] = 1;
            pad[1] = 1;
            mt[1] = 0;
        }
        for (int d = 0; d < 3; d++) {
            if (N[d] < 1 || !(L[d] > 0.0) || mt[d] < 0 || mt[d] > 2) return SARAS_BAD_ARG;
            if (active(d) && N[d] < 2) return SARAS_BAD_ARG;
        }
        for (int d = 0; d < 3; d++) dxi[d] = 1.0 / double(N[d]);
        if (dims == 2) dxi[1] = 1.0;
        for (int d = 0; d < 3; d++) {
            xiG[d].init(-pad[d], N[d] + pad[d] - 1);
            xG[d].init(-pad[d], N[d] + pad[d] - 1);
            xi_x[d].init(-pad[d], N[d] + pad[d] - 1);
            xixx[d].init(-pad[d], N[d] + pad[d] - 1);
            xix2[d].init(-pad[d], N[d] + pad[d] - 1);
            for (int i = -pad[d]; i < N[d] + pad[d]; i++) xiG[d][i] = double(2 * i + 1) * dxi[d] / 2;
        }
        /* grid::createUniformGrid (grid.cc:358-391) */
        for (int d = 0; d < 3; d++) {
            if (!active(d)) continue;
            for (int i = -pad[d]; i < N[d] + pad[d]; i++) {
                xG[d][i] = L[d] * xiG[d][i];
                xi_x[d][i] = 1.0 / L[d];
                xixx[d][i] = 0.0;
                xix2[d][i] = std::pow(xi_x[d][i], 2.0);
            }
        }
        vcdGlo = vc_depth();
        if (levels > 0) {
            int f = 1 << (levels - 1);
            for (int d = 0; d < 3; d++)
                if (active(d) && (N[d] % f != 0 || N[d] / f < 2)) return SARAS_BAD_ARG;
            vcdGlo = levels - 1;
        }
        if (vcdGlo < 0) return SARAS_BAD_ARG;
        mg_metrics_uniform();
        for (int d = 0; d < 3; d++)
            if (active(d) && mt[d] > 0) tanh_axis(d);
        return SARAS_OK;
    }
};

/* ------------------------------------------------------------- multigrid -- */

/* Single-rank restatement of class poisson / multigrid_d3 / multigrid_d2
 * (lib/poisson/poisson.cc, poisson_d3.cc, poisson_d2.cc). */
struct Multigrid {
    const Grid &g;
    saras_mg_params prm;
    bool d3;
    int nl = 0;
    std::vector<Arr3> lhs, rhs, tmp, smd;
    std::vector<std::array<int, 3>> nn;
    std::vector<Vec1> X[3], C1[3], C2[3]; /* x(n), xixx(n), xix2(n): -1..N_n */
    std::vector<double> ihx2[3], i2hx[3];
    int maxCount = 0;
    int vLevel = 0;
    bool zeroBC = false;
    Arr3 wallX, wallY, wallZ; /* TEST_POISSON wall values (level 0) */

    explicit Multigrid(const Grid &gr) : g(gr) {}

    /* poisson::poisson (poisson.cc:66-92): setStagBounds, setCoefficients,
     * copyDerivs, initializeArrays; multigrid_d*::initDirichlet. */
    void setup(const saras_mg_params &p) {
        prm = p;
        d3 = g.dims == 3;
        nl = g.vcdGlo + 1;
        lhs.resize(nl); rhs.resize(nl); tmp.resize(nl); smd.resize(nl);
        nn.resize(nl);
        for (int d = 0; d < 3; d++) {
            X[d].resize(nl); C1[d].resize(nl); C2[d].resize(nl);
            ihx2[d].assign(nl, 0.0); i2hx[d].assign(nl, 0.0);
        }
        for (int l = 0; l < nl; l++) {
            for (int d = 0; d < 3; d++) nn[l][d] = g.N[d] / int(std::pow(2, l));
            if (!d3) nn[l][1] = 1;
            lhs[l].init(nn[l][0], nn[l][1], nn[l][2], 1, 1, 1);
            rhs[l].init(nn[l][0], nn[l][1], nn[l][2], 1, 1, 1);
            tmp[l].init(nn[l][0], nn[l][1], nn[l][2], 1, 1, 1);
            smd[l].init(nn[l][0], nn[l][1], nn[l][2], 1, 1, 1);
            for (int d = 0; d < 3; d++) {
                if (!g.active(d)) continue;
                int hInc = (1 << l);
                double h = hInc * g.dxi[d];
                double h2 = std::pow(h, 2);
                i2hx[d][l] = 0.5 / h;
                ihx2[d][l] = 1.0 / h2;
                X[d][l].init(-1, nn[l][d]);
                C1[d][l].init(-1, nn[l][d]);
                C2[d][l].init(-1, nn[l][d]);
                for (int i = -1; i <= nn[l][d]; i++) {
                    X[d][l][i] = g.gm[15 * l + 5 * d + 1][i];
                    C1[d][l][i] = g.gm[15 * l + 5 * d + 3][i];
                    C2[d][l][i] = g.gm[15 * l + 5 * d + 4][i];
                }
            }
        }
        int cg[3];
        for (int d = 0; d < 3; d++) cg[d] = g.N[d] / int(std::pow(2, g.vcdGlo));
        if (d3)
            maxCount = int(2.5 * cg[0] * cg[1] * cg[2]);
        else
            maxCount = int(2.5 * cg[0] * cg[2]);
        /* initDirichlet (poisson_d3.cc:824-873, poisson_d2.cc) */
        int n0 = nn[0][0], n1 = nn[0][1], n2 = nn[0][2];
        wallX.init(1, n1, n2, 0, 1, 1);
        wallY.init(n0, 1, n2, 1, 0, 1);
        wallZ.init(n0, n1, 1, 1, 1, 0);
        if (d3) {
            double xd = g.L[0] / 2.0, yd = g.L[1] / 2.0, zd = g.L[2] / 2.0;
            for (int j = 0; j < n1; j++)
                for (int k = 0; k < n2; k++) {
                    double y = g.xG[1][j] - 0.5, z = g.xG[2][k] - 0.5;
                    wallX(0, j, k) = (xd * xd + y * y + z * z) / 6.0;
                }
            for (int i = 0; i < n0; i++)
                for (int k = 0; k < n2; k++) {
                    double x = g.xG[0][i] - 0.5, z = g.xG[2][k] - 0.5;
                    wallY(i, 0, k) = (x * x + yd * yd + z * z) / 6.0;
                }
            for (int i = 0; i < n0; i++)
                for (int j = 0; j < n1; j++) {
                    double x = g.xG[0][i] - 0.5, y = g.xG[1][j] - 0.5;
                    wallZ(i, j, 0) = (x * x + y * y + zd * zd) / 6.0;
                }
        } else {
            double xd = g.L[0] / 2.0, zd = g.L[2] / 2.0;
            for (int k = 0; k < n2; k++) {
                double z = g.xG[2][k] - 0.5;
                wallX(0, 0, k) = (xd * xd + z * z) / 4.0;
            }
            for (int i = 0; i < n0; i++) {
                double x = g.xG[0][i] - 0.5;
                wallZ(i, 0, 0) = (x * x + zd * zd) / 4.0;
            }
        }
    }

    /* One face of imposeBC: ghost value from the interior value `u` of the
     * face kind (poisson_d3.cc:880-950, poisson_d2.cc imposeBC). */
    inline double ghost(int kind, double u, double wall) const {
        if (kind == SARAS_BC_NEUMANN) return u;
        if (kind == SARAS_BC_DIRICHLET) return -u;
        return zeroBC ? -u : 2.0 * wall - u;
    }

    /* multigrid_d*::updateFace with a single rank: periodic axes copy full
     * planes, x then y then z (poisson_d3.cc:955-993; mpidata self-sends). */
    void update_face(Arr3 &a) {
        int n0 = a.n[0], n1 = a.n[1], n2 = a.n[2];
        if (g.per[0]) {
            for (int j = a.lo(1); j <= a.hi(1); j++) {
                if (!d3 && j != 0) continue;
                for (int k = -1; k <= n2; k++) {
                    a(n0, j, k) = a(0, j, k);
                    a(-1, j, k) = a(n0 - 1, j, k);
                }
            }
        }
        if (d3 && g.per[1]) {
            for (int i = -1; i <= n0; i++)
                for (int k = -1; k <= n2; k++) {
                    a(i, n1, k) = a(i, 0, k);
                    a(i, -1, k) = a(i, n1 - 1, k);
                }
        }
        if (g.per[2]) {
            for (int i = -1; i <= n0; i++)
                for (int j = a.lo(1); j <= a.hi(1); j++) {
                    if (!d3 && j != 0) continue;
                    a(i, j, n2) = a(i, j, 0);
                    a(i, j, -1) = a(i, j, n2 - 1);
                }
        }
    }

    /* multigrid_d*::imposeBC (poisson_d3.cc:876-952, poisson_d2.cc). */
    void impose_bc() {
        Arr3 &a = lhs[vLevel];
        update_face(a);
        int n0 = a.n[0], n1 = a.n[1], n2 = a.n[2];
        bool lvl0 = vLevel == 0;
        if (!g.per[0]) {
            int k0 = prm.bc_kind[0], k1 = prm.bc_kind[1];
            for (int j = -1; j <= n1; j++) {
                if (!d3 && j != 0) continue;
                for (int k = -1; k <= n2; k++) {
                    double w = lvl0 ? wallX(0, j, k) : 0.0;
                    a(-1, j, k) = ghost(k0, a(0, j, k), w);
                    a(n0, j, k) = ghost(k1, a(n0 - 1, j, k), w);
                }
            }
        }
        if (d3 && !g.per[1]) {
            int k0 = prm.bc_kind[2], k1 = prm.bc_kind[3];
            for (int i = -1; i <= n0; i++)
                for (int k = -1; k <= n2; k++) {
                    double w = lvl0 ? wallY(i, 0, k) : 0.0;
                    a(i, -1, k) = ghost(k0, a(i, 0, k), w);
                    a(i, n1, k) = ghost(k1, a(i, n1 - 1, k), w);
                }
        }
        if (!g.per[2]) {
            int k0 = prm.bc_kind[4], k1 = prm.bc_kind[5];
            for (int i = -1; i <= n0; i++)
                for (int j = -1; j <= n1; j++) {
                    if (!d3 && j != 0) continue;
                    double w = lvl0 ? wallZ(i, j, 0) : 0.0;
                    a(i, j, -1) = ghost(k0, a(i, j, 0), w);
                    a(i, j, n2) = ghost(k1, a(i, j, n2 - 1), w);
                }
        }
    }

    /* SOR-RBGS update of one cell (poisson_d3.cc:109-116; poisson_d2.cc). */
    inline double rbgs_value(int l, const Arr3 &u, const Arr3 &f, int i, int j, int k) const {
        const double w = prm.sor_param;
        const double cx2 = C2[0][l][i], cx1 = C1[0][l][i];
        const double cz2 = C2[2][l][k], cz1 = C1[2][l][k];
        const double hx2 = ihx2[0][l], hx1 = i2hx[0][l], hz2 = ihz2_(l), hz1 = i2hx[2][l];
        if (d3) {
            const double cy2 = C2[1][l][j], cy1 = C1[1][l][j];
            const double hy2 = ihx2[1][l], hy1 = i2hx[1][l];
            return (1.0 - w) * u(i, j, k) +
                   (cx2 * hx2 * (u(i + 1, j, k) + u(i - 1, j, k)) +
                    cx1 * hx1 * (u(i + 1, j, k) - u(i - 1, j, k)) +
                    cy2 * hy2 * (u(i, j + 1, k) + u(i, j - 1, k)) +
                    cy1 * hy1 * (u(i, j + 1, k) - u(i, j - 1, k)) +
                    cz2 * hz2 * (u(i, j, k + 1) + u(i, j, k - 1)) +
                    cz1 * hz1 * (u(i, j, k + 1) - u(i, j, k - 1)) -
                    f(i, j, k)) * w / (2.0 * (hx2 * cx2 + hy2 * cy2 + hz2 * cz2));
        }
        return (1.0 - w) * u(i, 0, k) +
               (cx2 * hx2 * (u(i + 1, 0, k) + u(i - 1, 0, k)) +
                cx1 * hx1 * (u(i + 1, 0, k) - u(i - 1, 0, k)) +
                cz2 * hz2 * (u(i, 0, k + 1) + u(i, 0, k - 1)) +
                cz1 * hz1 * (u(i, 0, k + 1) - u(i, 0, k - 1)) -
                f(i, 0, k)) * w / (2.0 * (hx2 * cx2 + hz2 * cz2));
    }
    inline double ihz2_(int l) const { return ihx2[2][l]; }

    /* f - A u at one cell (poisson_d3.cc:81-87; poisson_d2.cc:79-84). */
    inline double residual_value(int l, const Arr3 &u, const Arr3 &f, int i, int j, int k) const {
        const double cx2 = C2[0][l][i], cx1 = C1[0][l][i];
        const double cz2 = C2[2][l][k], cz1 = C1[2][l][k];
        const double hx2 = ihx2[0][l], hx1 = i2hx[0][l], hz2 = ihx2[2][l], hz1 = i2hx[2][l];
        if (d3) {
            const double cy2 = C2[1][l][j], cy1 = C1[1][l][j];
            const double hy2 = ihx2[1][l], hy1 = i2hx[1][l];
            return f(i, j, k) -
                   (cx2 * hx2 * (u(i + 1, j, k) - 2.0 * u(i, j, k) + u(i - 1, j, k)) +
                    cx1 * hx1 * (u(i + 1, j, k) - u(i - 1, j, k)) +
                    cy2 * hy2 * (u(i, j + 1, k) - 2.0 * u(i, j, k) + u(i, j - 1, k)) +
                    cy1 * hy1 * (u(i, j + 1, k) - u(i, j - 1, k)) +
                    cz2 * hz2 * (u(i, j, k + 1) - 2.0 * u(i, j, k) + u(i, j, k - 1)) +
                    cz1 * hz1 * (u(i, j, k + 1) - u(i, j, k - 1)));
        }
        return f(i, 0, k) -
               (cx2 * hx2 * (u(i + 1, 0, k) - 2.0 * u(i, 0, k) + u(i - 1, 0, k)) +
                cx1 * hx1 * (u(i + 1, 0, k) - u(i - 1, 0, k)) +
                cz2 * hz2 * (u(i, 0, k + 1) - 2.0 * u(i, 0, k) + u(i, 0, k - 1)) +
                cz1 * hz1 * (u(i, 0, k + 1) - u(i, 0, k - 1)));
    }

    /* One colour of RBGS as the reference's parity loops: red cells are the
     * parities (0,0,0),(1,1,0),(1,0,1),(0,1,1), black (1,0,0),(0,1,0),
     * (0,0,1),(1,1,1) (poisson_d3.cc:104-242); 2D (0,0),(1,1) / (1,0),(0,1). */
    void colour_sweep(int colour) {
        int l = vLevel;
        Arr3 &u = lhs[l];
        const Arr3 &f = rhs[l];
        const int n0 = nn[l][0], n1 = nn[l][1], n2 = nn[l][2];
        static const int red3[4][3] = {{0, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}};
        static const int blk3[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 1}};
        static const int red2[2][2] = {{0, 0}, {1, 1}};
        static const int blk2[2][2] = {{1, 0}, {0, 1}};
        if (d3) {
            const int (*cf)[3] = colour == 0 ? red3 : blk3;
            for (int c = 0; c < 4; c++) {
                const int pi = cf[c][0], pj = cf[c][1], pk = cf[c][2];
#pragma omp parallel for num_threads(g_threads) schedule(static)
                for (int i = pi; i < n0; i += 2)
                    for (int j = pj; j < n1; j += 2)
                        for (int k = pk; k < n2; k += 2) u(i, j, k) = rbgs_value(l, u, f, i, j, k);
            }
        } else {
            const int (*cf)[2] = colour == 0 ? red2 : blk2;
            for (int c = 0; c < 2; c++) {
                const int pi = cf[c][0], pk = cf[c][1];
#pragma omp parallel for num_threads(g_threads) schedule(static)
                for (int i = pi; i < n0; i += 2)
                    for (int k = pk; k < n2; k += 2) u(i, 0, k) = rbgs_value(l, u, f, i, 0, k);
            }
        }
    }

    /* multigrid_d*::smooth (poisson_d3.cc:96-246). */
    void smooth(int count) {
        tmp[vLevel].fill(0.0);
        for (int n = 0; n < count; n++) {
            impose_bc();
            colour_sweep(0);
            update_face(lhs[vLevel]);
            colour_sweep(1);
        }
        impose_bc();
    }

    /* max |f - A u| over the core (poisson_d3.cc:398-415). */
    double max_residual(int l, double init) {
        const Arr3 &u = lhs[l], &f = rhs[l];
        const int n0 = nn[l][0], n1 = nn[l][1], n2 = nn[l][2];
        double m = init;
#pragma omp parallel for num_threads(g_threads) reduction(max : m) schedule(static)
        for (int i = 0; i < n0; i++)
            for (int j = 0; j < n1; j++)
                for (int k = 0; k < n2; k++) {
                    double t = std::fabs(residual_value(l, u, f, i, j, k));
                    if (t > m) m = t;
                }
        return m;
    }

    /* multigrid_d*::solve (poisson_d3.cc:249-432): RBGS to an absolute
     * tolerance, at most maxCount + 1 sweeps. */
    int coarsest_solve() {
        int iterCount = 0;
        int sweeps = 0;
        while (true) {
            impose_bc();
            colour_sweep(0);
            update_face(lhs[vLevel]);
            colour_sweep(1);
            sweeps++;
            double gmax = max_residual(vLevel, -1.0e-10);
            if (gmax < prm.mg_tolerance) break;
            iterCount += 1;
            if (iterCount > maxCount) {
                if (prm.print_residual)
                    std::printf("WARNING: Iterations for solution at coarsest level not converging.\n");
                break;
            }
        }
        impose_bc();
        return sweeps;
    }

    /* multigrid_d*::computeResidual (poisson_d3.cc:71-93). */
    void compute_residual() {
        int l = vLevel;
        Arr3 &t = tmp[l];
        t.fill(0.0);
        const Arr3 &u = lhs[l], &f = rhs[l];
        const int n0 = nn[l][0], n1 = nn[l][1], n2 = nn[l][2];
#pragma omp parallel for num_threads(g_threads) schedule(static)
        for (int i = 0; i < n0; i++)
            for (int j = 0; j < n1; j++)
                for (int k = 0; k < n2; k++) t(i, j, k) = residual_value(l, u, f, i, j, k);
    }

    /* multigrid_d3::coarsen regular branch (poisson_d3.cc:483-511);
     * multigrid_d2::coarsen (poisson_d2.cc: mean of four). */
    void coarsen() {
        int pl = vLevel;
        vLevel += 1;
        int l = vLevel;
        const Arr3 &t = tmp[pl];
        Arr3 &r = rhs[l];
        const int n0 = nn[l][0], n1 = nn[l][1], n2 = nn[l][2];
        if (d3) {
            const Vec1 &xc = X[0][l], &yc = X[1][l], &zc = X[2][l];
            const Vec1 &xf = X[0][pl], &yf = X[1][pl], &zf = X[2][pl];
#pragma omp parallel for num_threads(g_threads) schedule(static)
            for (int i = 0; i < n0; i++) {
                int i2 = i * 2;
                for (int j = 0; j < n1; j++) {
                    int j2 = j * 2;
                    for (int k = 0; k < n2; k++) {
                        int k2 = k * 2;
                        double v000 = (xc[i] - xf[i2]) * (yc[j] - yf[j2]) * (zc[k] - zf[k2]);
                        double v100 = (xf[i2 + 1] - xc[i]) * (yc[j] - yf[j2]) * (zc[k] - zf[k2]);
                        double v010 = (xc[i] - xf[i2]) * (yf[j2 + 1] - yc[j]) * (zc[k] - zf[k2]);
                        double v001 = (xc[i] - xf[i2]) * (yc[j] - yf[j2]) * (zf[k2 + 1] - zc[k]);
                        double v011 = (xc[i] - xf[i2]) * (yf[j2 + 1] - yc[j]) * (zf[k2 + 1] - zc[k]);
                        double v101 = (xf[i2 + 1] - xc[i]) * (yc[j] - yf[j2]) * (zf[k2 + 1] - zc[k]);
                        double v110 = (xf[i2 + 1] - xc[i]) * (yf[j2 + 1] - yc[j]) * (zc[k] - zf[k2]);
                        double v111 = (xf[i2 + 1] - xc[i]) * (yf[j2 + 1] - yc[j]) * (zf[k2 + 1] - zc[k]);
                        double vT = (xf[i2 + 1] - xf[i2]) * (yf[j2 + 1] - yf[j2]) * (zf[k2 + 1] - zf[k2]);
                        r(i, j, k) = (v111 * t(i2 + 1, j2 + 1, k2 + 1) + v000 * t(i2, j2, k2) +
                                      v110 * t(i2 + 1, j2 + 1, k2) + v001 * t(i2, j2, k2 + 1) +
                                      v101 * t(i2 + 1, j2, k2 + 1) + v010 * t(i2, j2 + 1, k2) +
                                      v011 * t(i2, j2 + 1, k2 + 1) + v100 * t(i2 + 1, j2, k2)) / vT;
                    }
                }
            }
        } else {
#pragma omp parallel for num_threads(g_threads) schedule(static)
            for (int i = 0; i < n0; i++) {
                int i2 = i * 2;
                for (int k = 0; k < n2; k++) {
                    int k2 = k * 2;
                    r(i, 0, k) = (t(i2 + 1, 0, k2 + 1) + t(i2, 0, k2) + t(i2 + 1, 0, k2) + t(i2, 0, k2 + 1)) / 4;
                }
            }
        }
    }

    /* multigrid_d*::prolong regular branch (poisson_d3.cc:516-560). */
    void prolong() {
        int pl = vLevel;
        vLevel -= 1;
        int l = vLevel;
        Arr3 &f = lhs[l];
        const Arr3 &c = lhs[pl];
        f.fill(0.0);
        const int n0 = nn[l][0], n1 = nn[l][1], n2 = nn[l][2];
#pragma omp parallel for num_threads(g_threads) schedule(static)
        for (int i = 0; i < n0; i++)
            for (int j = 0; j < n1; j++)
                for (int k = 0; k < n2; k++) f(i, j, k) = c(i / 2, j / 2, k / 2);
    }

    /* poisson::vCycle (poisson.cc:203-279). */
    void v_cycle(int *coarse_sweeps) {
        vLevel = 0;
        zeroBC = false;
        smooth(prm.pre_smooth);
        zeroBC = true;
        for (int i = 0; i < g.vcdGlo; i++) {
            compute_residual();
            smd[vLevel].v = lhs[vLevel].v;
            coarsen();
            lhs[vLevel].fill(0.0);
            if (vLevel == g.vcdGlo && prm.solve_flag) {
                int s = coarsest_solve();
                if (coarse_sweeps) *coarse_sweeps += s;
            } else {
                smooth(prm.pre_smooth);
            }
        }
        for (int i = 0; i < g.vcdGlo; i++) {
            prolong();
            std::vector<double> &a = lhs[vLevel].v;
            const std::vector<double> &b = smd[vLevel].v;
            for (size_t q = 0; q < a.size(); q++) a[q] += b[q];
            zeroBC = vLevel != 0;
            smooth(prm.post_smooth);
        }
    }

    /* multigrid_d*::computeError (poisson_d3.cc:563-663). */
    double compute_error(int normOrder) {
        const Arr3 &u = lhs[0], &f = rhs[0];
        const int n0 = nn[0][0], n1 = nn[0][1], n2 = nn[0][2];
        int pointCount = d3 ? g.N[0] * g.N[1] * g.N[2] : g.N[0] * g.N[2];
        double num = 0.0, den = 0.0;
        if (normOrder == 0) {
            num = max_residual(0, 0.0);
            for (int i = 0; i < n0; i++)
                for (int j = 0; j < n1; j++)
                    for (int k = 0; k < n2; k++) den = std::max(den, std::fabs(f(i, j, k)));
            return den ? num / den : num;
        }
        std::vector<double> pn((size_t)n0, 0.0), pd((size_t)n0, 0.0);
#pragma omp parallel for num_threads(g_threads) schedule(static)
        for (int i = 0; i < n0; i++) {
            double a = 0.0, b = 0.0;
            for (int j = 0; j < n1; j++)
                for (int k = 0; k < n2; k++) {
                    double t = residual_value(0, u, f, i, j, k);
                    if (normOrder == 1) {
                        a += std::fabs(t);
                        b += std::fabs(f(i, j, k));
                    } else {
                        a += t * t;
                        b += std::pow(f(i, j, k), 2);
                    }
                }
            pn[(size_t)i] = a;
            pd[(size_t)i] = b;
        }
        for (int i = 0; i < n0; i++) {
            num += pn[(size_t)i];
            den += pd[(size_t)i];
        }
        if (normOrder == 1) return den ? num / den : num / pointCount;
        return den ? std::sqrt(num / pointCount) / std::sqrt(den / pointCount)
                   : std::sqrt(num / pointCount);
    }

    /* poisson::mgSolve (poisson.cc:109-189).  `out`/`in` address element
     * (0,0,0) of caller arrays with the given strides. */
    int mg_solve(double *out, const double *in, const int64_t *st, double *hist, int cap, int *ncyc,
                 int *coarse_sweeps) {
        vLevel = 0;
        for (int l = 0; l < nl; l++) {
            lhs[l].fill(0.0);
            rhs[l].fill(0.0);
            smd[l].fill(0.0);
        }
        const int n0 = nn[0][0], n1 = nn[0][1], n2 = nn[0][2];
        for (int i = 0; i < n0; i++)
            for (int j = 0; j < n1; j++)
                for (int k = 0; k < n2; k++) {
                    int64_t o = i * st[0] + j * st[1] + k * st[2];
                    rhs[0](i, j, k) = in[o];
                    lhs[0](i, j, k) = out[o];
                }
        int cyc = 0;
        double r = 0.0;
        for (int c = 0; c < prm.vc_count; c++) {
            v_cycle(coarse_sweeps);
            r = compute_error(prm.res_type);
            cyc++;
            if (hist && c < cap) hist[c] = r;
            if (prm.print_residual) std::printf("\nResidual after V Cycle %d is %.3e\n", c, r);
            if (!prm.test_poisson && r < prm.vc_tolerance) break;
        }
        for (int i = -1; i <= n0; i++)
            for (int j = -1; j <= n1; j++)
                for (int k = -1; k <= n2; k++) {
                    int64_t o = i * st[0] + j * st[1] + k * st[2];
                    out[o] = lhs[0](i, j, k);
                }
        if (ncyc) *ncyc = cyc;
        if (prm.test_poisson) return SARAS_OK;
        return r < prm.vc_tolerance ? SARAS_OK : SARAS_NOT_CONVERGED;
    }
};

/* ------------------------------------------------------------------- RK3 -- */

/* Single-rank restatement of lsRK3_d3/lsRK3_d2::timeAdvance and the field
 * operations it calls. */
struct Rk3 {
    Grid g;
    saras_rk3_params prm;
    bool d3 = true;
    int pad = 1;
    Arr3 Vx, Vy, Vz, P, T, Pp, mgRHS;
    Arr3 nseX, nseY, nseZ, tmpRHS, tvX, tvY, tvZ, tSF, pgX, pgY, pgZ, iterTemp;
    Multigrid *mg = nullptr;
    double dih[3], dih2[3];  /* derivative: ihx = 1/dXi, ihx2 = pow(ihx, 2) */
    double tih2[3], ti2h[3]; /* timestep: ihx2 = 1/pow(dXi,2), i2hx = 0.5/dXi */
    double mi2d[3];          /* vfield/sfield: i2dx = 1/(2 dXi) (vfield.cc:133-135) */
    int ds = 1;              /* Differentiation Scheme: 1 (pad 1) or 2 (pad 2) */
    double ua = 0, ub = 0, uc = 0, ud = 0; /* upwind stencil weights (vfield.cc:114-130) */
    double hwall[6];
    int maxIterations = 0;

    ~Rk3() { delete mg; }

    void alloc(Arr3 &a) { a.init(g.N[0], g.N[1], g.N[2], g.pad[0], g.pad[1], g.pad[2]); }

    int setup(const saras_grid_desc &gd, const saras_rk3_params &p) {
        int s = g.build(gd, p.mg.levels);
        if (s) return s;
        if (gd.pad != 1 && gd.pad != 2) return SARAS_BAD_ARG;
        if (p.nl_scheme < 1 || p.nl_scheme > 3) return SARAS_BAD_ARG;
        if (p.integration < 0 || p.integration > 2) return SARAS_BAD_ARG;
        prm = p;
        d3 = g.dims == 3;
        /* grid::grid (grid.cc:69-77): the pad width follows dScheme */
        ds = gd.pad;
        /* vfield::vfield / sfield::sfield (vfield.cc:107-130, sfield.cc:89-
         * 111): firstOrder upwinding for dScheme 1, omega = "Central Bias" */
        const double omega = p.up_param;
        if (ds == 1) {
            ua = 2.0 - omega;
            ub = 2.0 * (1.0 - omega);
            uc = -omega;
        } else {
            ua = 1.0 - omega;
            ub = 4.0 - 3.0 * omega;
            uc = 3.0 * (1.0 - omega);
            ud = -omega;
        }
        Arr3 *all[] = {&Vx, &Vy, &Vz, &P, &T, &Pp, &mgRHS, &nseX, &nseY, &nseZ, &tmpRHS,
                       &tvX, &tvY, &tvZ, &tSF, &pgX, &pgY, &pgZ, &iterTemp};
        for (Arr3 *a : all) alloc(*a);
        mg = new Multigrid(g);
        mg->setup(p.mg);
        for (int d = 0; d < 3; d++) {
            dih[d] = 1.0 / g.dxi[d];
            dih2[d] = std::pow(dih[d], 2.0);
            double h2 = std::pow(g.dxi[d], 2.0);
            ti2h[d] = 0.5 / g.dxi[d];
            tih2[d] = 1.0 / h2;
            mi2d[d] = 1.0 / (2.0 * g.dxi[d]);
        }
        /* neumann::neumann (lib/boundary/neumann.cc:50-66) */
        hwall[0] = 2 * g.xG[0][0];
        hwall[1] = 2 * (g.xG[0][g.N[0] - 1] - g.L[0]);
        hwall[2] = 2 * g.xG[1][0];
        hwall[3] = 2 * (g.xG[1][g.N[1] - 1] - g.L[1]);
        hwall[4] = 2 * g.xG[2][0];
        hwall[5] = 2 * (g.xG[2][g.N[2] - 1] - g.L[2]);
        maxIterations = p.max_iterations > 0
                            ? p.max_iterations
                            : int(std::pow(std::log(g.N[0] * g.N[1] * g.N[2]), 3));
        return SARAS_OK;
    }

    /* True on the first and last core cell of axis d: every rank of a
     * single-rank run is first and last on every axis (derivative.cc:80-
     * 86), periodic or not, so the dScheme-2 boundary forms apply there. */
    inline bool edge(int d, int idx) const { return idx == 0 || idx == g.N[d] - 1; }

    /* calcDerivative1_{x,y,z} (derivative.cc:104-204).  dScheme 1:
     * central12n = (F+ - F-) * 0.5.  dScheme 2: central14n in the interior
     * and 0.5 * (F+ - F-) on the first and last core cell.  Blitz++ (not
     * vendored) defines central14n; it is taken here as the unique 5-point
     * fourth-order central first difference in index units,
     * (8 (F+1 - F-1) - (F+2 - F-2)) / 12 -- the operation order is this
     * build's, shared with the GPU. */
    inline double d1(const Arr3 &F, int d, int i, int j, int k) const {
        int o[3] = {0, 0, 0};
        o[d] = 1;
        int idx = d == 0 ? i : (d == 1 ? j : k);
        const double fp = F(i + o[0], j + o[1], k + o[2]), fm = F(i - o[0], j - o[1], k - o[2]);
        double c;
        if (ds == 1) {
            c = (fp - fm) * 0.5;
        } else if (edge(d, idx)) {
            c = 0.5 * (fp - fm);
        } else {
            const double fp2 = F(i + 2 * o[0], j + 2 * o[1], k + 2 * o[2]);
            const double fm2 = F(i - 2 * o[0], j - 2 * o[1], k - 2 * o[2]);
            c = (8.0 * (fp - fm) - (fp2 - fm2)) / 12.0;
        }
        return g.xi_x[d][idx] * (c * dih[d]);
    }
    /* One direction of Morinishi's skew-symmetric convection term,
     * second-order branch (dScheme 1): vfield::morinishiNLin
     * (vfield.cc:271-474) and sfield::morinishiNLin (sfield.cc:200-323).
     * adv = Va * xi * (F+ - F-) * i2d, div = xi * (Va+ F+ - Va- F-) * i2d
     * (the Blitz products tempXX = V.Vx*Vx etc. at the neighbours); the
     * caller subtracts (adv + div)/2. */
    inline double mterm(const Arr3 &F, const Arr3 &Va, int d, int i, int j, int k) const {
        int o[3] = {0, 0, 0};
        o[d] = 1;
        int idx = d == 0 ? i : (d == 1 ? j : k);
        const int ip = i + o[0], jp = j + o[1], kp = k + o[2];
        const int im = i - o[0], jm = j - o[1], km = k - o[2];
        const double x = g.xi_x[d][idx];
        /* fourth-order branch (dScheme 2) away from the first and last
         * point.  The reference tests the last z point against the y extent
         * (core.ubound(1), vfield.cc:337,427; sfield.cc:239,290), so along z
         * the second-order form is taken at k == 0 and k == Ny - 1 (0 for a
         * planar run) and k = Nz - 1 uses the fourth-order form, which reads
         * the second ghost layer. */
        const int last = (d == 2 ? g.N[1] : g.N[d]) - 1;
        if (ds == 2 && idx != 0 && idx != last) {
            const int ip2 = i + 2 * o[0], jp2 = j + 2 * o[1], kp2 = k + 2 * o[2];
            const int im2 = i - 2 * o[0], jm2 = j - 2 * o[1], km2 = k - 2 * o[2];
            const double adv = Va(i, j, k) * x *
                               (-F(ip2, jp2, kp2) + 8.0 * F(ip, jp, kp) - 8.0 * F(im, jm, km) + F(im2, jm2, km2)) *
                               mi2d[d] / 6.0;
            const double div = x *
                               (-(Va(ip2, jp2, kp2) * F(ip2, jp2, kp2)) + 8.0 * (Va(ip, jp, kp) * F(ip, jp, kp)) -
                                8.0 * (Va(im, jm, km) * F(im, jm, km)) + Va(im2, jm2, km2) * F(im2, jm2, km2)) *
                               mi2d[d] / 6.0;
            return (adv + div) / 2;
        }
        const double adv = Va(i, j, k) * x * (F(ip, jp, kp) - F(im, jm, km)) * mi2d[d];
        const double div = x * (Va(ip, jp, kp) * F(ip, jp, kp) - Va(im, jm, km) * F(im, jm, km)) * mi2d[d];
        return (adv + div) / 2;
    }
    /* One direction of the hybrid upwind convection term, vfield::upwindNLin
     * (vfield.cc:475-690) and sfield::upwindNLin (sfield.cc:324-495): the
     * cell Peclet number |u| dh / diffCoeff (dh = x(i+1) - x(i)) picks the
     * central form below "Peclet Limit", else the stencil biased against
     * the local velocity.  dScheme 1 takes first-order upwinding with
     * second-order central differences; dScheme 2 second-order upwinding
     * with fourth-order central differences, and second-order central
     * differences on the first and last core cell.  The caller subtracts
     * the returned value. */
    inline double uterm(const Arr3 &F, const Arr3 &Va, double dcoef, int d, int i, int j, int k) const {
        int o[3] = {0, 0, 0};
        o[d] = 1;
        int idx = d == 0 ? i : (d == 1 ? j : k);
        const double u = Va(i, j, k);
        const double x = g.xi_x[d][idx];
        const double f0 = F(i, j, k);
        const double fp = F(i + o[0], j + o[1], k + o[2]), fm = F(i - o[0], j - o[1], k - o[2]);
        if (ds == 1) {
            const double dh = g.xG[d][idx + 1] - g.xG[d][idx];
            const double pe = std::fabs(u) * dh / dcoef;
            if (pe < prm.pe_limit) return u * x * (fp - fm) * mi2d[d];
            if (u > 0) return u * x * (-ua * fm + ub * f0 - uc * fp) * mi2d[d];
            return u * x * (ua * fp - ub * f0 + uc * fm) * mi2d[d];
        }
        if (edge(d, idx)) return u * x * (fp - fm) * mi2d[d];
        const double fp2 = F(i + 2 * o[0], j + 2 * o[1], k + 2 * o[2]);
        const double fm2 = F(i - 2 * o[0], j - 2 * o[1], k - 2 * o[2]);
        const double dh = g.xG[d][idx + 1] - g.xG[d][idx];
        const double pe = std::fabs(u) * dh / dcoef;
        if (pe < prm.pe_limit) return u * x * (-fp2 + 8.0 * fp - 8.0 * fm + fm2) * mi2d[d] / 6.0;
        if (u > 0) return u * x * (ua * fm2 - ub * fm + uc * f0 - ud * fp) * mi2d[d];
        return u * x * (-ua * fp2 + ub * fp - uc * f0 + ud * fm) * mi2d[d];
    }
    /* calcDerivative2{xx,yy,zz} (derivative.cc:206-318).  dScheme 1:
     * central12n and central22n = (F- - 2F) + F+.  dScheme 2: central14n
     * as in d1 and central24n taken as (16 (F+1 + F-1) - 30 F - (F+2 + F-2))
     * / 12 in the interior; 0.5 (F+ - F-) and (F+ - 2F) + F- (the
     * reference's own boundary forms, derivative.cc:214-223) on the first
     * and last core cell. */
    inline double d2(const Arr3 &F, int d, int i, int j, int k) const {
        int o[3] = {0, 0, 0};
        o[d] = 1;
        int idx = d == 0 ? i : (d == 1 ? j : k);
        const double f0 = F(i, j, k);
        double fp = F(i + o[0], j + o[1], k + o[2]), fm = F(i - o[0], j - o[1], k - o[2]);
        double c1, c2;
        if (ds == 1) {
            c1 = (fp - fm) * 0.5;
            c2 = fm - 2.0 * f0 + fp;
        } else if (edge(d, idx)) {
            c1 = 0.5 * (fp - fm);
            c2 = fp - 2.0 * f0 + fm;
        } else {
            const double fp2 = F(i + 2 * o[0], j + 2 * o[1], k + 2 * o[2]);
            const double fm2 = F(i - 2 * o[0], j - 2 * o[1], k - 2 * o[2]);
            c1 = (8.0 * (fp - fm) - (fp2 - fm2)) / 12.0;
            c2 = (16.0 * (fp + fm) - 30.0 * f0 - (fp2 + fm2)) / 12.0;
        }
        return g.xixx[d][idx] * (c1 * dih[d]) + g.xix2[d][idx] * (c2 * dih2[d]);
    }

    template <class Fn> void core_loop(Fn fn) {
        const int n0 = g.N[0], n1 = g.N[1], n2 = g.N[2];
#pragma omp parallel for num_threads(g_threads) schedule(static)
        for (int i = 0; i < n0; i++)
            for (int j = 0; j < n1; j++)
                for (int k = 0; k < n2; k++) fn(i, j, k);
    }
    template <class Fn> void full_loop(Arr3 &a, Fn fn) {
        const size_t n = a.v.size();
#pragma omp parallel for num_threads(g_threads) schedule(static)
        for (size_t q = 0; q < n; q++) fn(q);
    }

    /* field::syncFaces on one rank: periodic pad slabs, x then y then z
     * (lib/parallel/mpidata.cc:371-383). */
    void sync_faces(Arr3 &a) {
        const int n0 = a.n[0], n1 = a.n[1], n2 = a.n[2];
        if (g.per[0])
            for (int m = 0; m < a.p[0]; m++)
                for (int j = a.lo(1); j <= a.hi(1); j++)
                    for (int k = a.lo(2); k <= a.hi(2); k++) {
                        a(n0 + m, j, k) = a(m, j, k);
                        a(-a.p[0] + m, j, k) = a(n0 - a.p[0] + m, j, k);
                    }
        if (d3 && g.per[1])
            for (int m = 0; m < a.p[1]; m++)
                for (int i = a.lo(0); i <= a.hi(0); i++)
                    for (int k = a.lo(2); k <= a.hi(2); k++) {
                        a(i, n1 + m, k) = a(i, m, k);
                        a(i, -a.p[1] + m, k) = a(i, n1 - a.p[1] + m, k);
                    }
        if (g.per[2])
            for (int m = 0; m < a.p[2]; m++)
                for (int i = a.lo(0); i <= a.hi(0); i++)
                    for (int j = a.lo(1); j <= a.hi(1); j++) {
                        a(i, j, n2 + m) = a(i, j, m);
                        a(i, j, -a.p[2] + m) = a(i, j, n2 - a.p[2] + m);
                    }
    }

    /* sfield::imposeBCs / vfield::imposeV*BC (sfield.cc:520-547,
     * vfield.cc:751-857) with dirichlet/neumann writers
     * (lib/boundary/dirichlet.cc:72-76, neumann.cc:87-93). */
    void impose_bcs(Arr3 &a, const saras_field_bc &bc) {
        sync_faces(a);
        const int nd[3] = {a.n[0], a.n[1], a.n[2]};
        for (int d = 0; d < 3; d++) {
            if (!g.active(d) || g.per[d]) continue;
            for (int side = 0; side < 2; side++) {
                int face = 2 * d + side;
                int gi = side == 0 ? -1 : nd[d];
                int si = side == 0 ? 0 : nd[d] - 1;
                double val = bc.value[face];
                double kh = val * hwall[face];
                int a0 = (d + 1) % 3, a1 = (d + 2) % 3;
                for (int p0 = a.lo(a0); p0 <= a.hi(a0); p0++)
                    for (int p1 = a.lo(a1); p1 <= a.hi(a1); p1++) {
                        int gidx[3], sidx[3];
                        gidx[d] = gi; sidx[d] = si;
                        gidx[a0] = p0; sidx[a0] = p0;
                        gidx[a1] = p1; sidx[a1] = p1;
                        double s = a(sidx[0], sidx[1], sidx[2]);
                        a(gidx[0], gidx[1], gidx[2]) =
                            bc.type[face] == SARAS_FBC_DIRICHLET ? 2.0 * val - s : s - kh;
                    }
            }
        }
    }

    /* timestep::solveVx/Vy/Vz/T (lib/timestep/predictors.cc:59-423). */
    int cn_solve(Arr3 &F, const Arr3 &R, double coef, double beta, const saras_field_bc &bc, int *iters) {
        const double dt = prm.dt;
        const double hx2 = tih2[0], hx1 = ti2h[0], hy2 = tih2[1], hy1 = ti2h[1], hz2 = tih2[2],
                     hz1 = ti2h[2];
        int iterCount = 0;
        while (true) {
            core_loop([&](int i, int j, int k) {
                const double cx2 = g.xix2[0][i], cx1 = g.xixx[0][i];
                const double cz2 = g.xix2[2][k], cz1 = g.xixx[2][k];
                if (d3) {
                    const double cy2 = g.xix2[1][j], cy1 = g.xixx[1][j];
                    iterTemp(i, j, k) =
                        ((hx2 * cx2 * (F(i + 1, j, k) + F(i - 1, j, k)) +
                          hx1 * cx1 * (F(i + 1, j, k) - F(i - 1, j, k)) +
                          hy2 * cy2 * (F(i, j + 1, k) + F(i, j - 1, k)) +
                          hy1 * cy1 * (F(i, j + 1, k) - F(i, j - 1, k)) +
                          hz2 * cz2 * (F(i, j, k + 1) + F(i, j, k - 1)) +
                          hz1 * cz1 * (F(i, j, k + 1) - F(i, j, k - 1))) *
                             dt * coef * beta + R(i, j, k)) /
                        (1.0 + 2.0 * dt * coef * beta * (hx2 * cx2 + hy2 * cy2 + hz2 * cz2));
                } else {
                    iterTemp(i, j, k) =
                        ((hx2 * cx2 * (F(i + 1, j, k) + F(i - 1, j, k)) +
                          hx1 * cx1 * (F(i + 1, j, k) - F(i - 1, j, k)) +
                          hz2 * cz2 * (F(i, j, k + 1) + F(i, j, k - 1)) +
                          hz1 * cz1 * (F(i, j, k + 1) - F(i, j, k - 1))) *
                             dt * coef * beta + R(i, j, k)) /
                        (1.0 + 2.0 * dt * coef * beta * (hx2 * cx2 + hz2 * cz2));
                }
            });
            /* F = iterTemp copies the whole padded array; the sweep never
             * writes iterTemp's pads (timestep.cc:117-118 allocates it
             * without a fill), taken here as zero -- what a fresh
             * allocation reads.  The boundary conditions then rewrite the
             * first ghost layer; on wall axes the second stays zero. */
            full_loop(F, [&](size_t q) { F.v[q] = iterTemp.v[q]; });
            impose_bcs(F, bc);
            double m = 0.0;
            const int n0 = g.N[0], n1 = g.N[1], n2 = g.N[2];
#pragma omp parallel for num_threads(g_threads) reduction(max : m) schedule(static)
            for (int i = 0; i < n0; i++)
                for (int j = 0; j < n1; j++)
                    for (int k = 0; k < n2; k++) {
                        const double cx2 = g.xix2[0][i], cx1 = g.xixx[0][i];
                        const double cz2 = g.xix2[2][k], cz1 = g.xixx[2][k];
                        double v;
                        if (d3) {
                            const double cy2 = g.xix2[1][j], cy1 = g.xixx[1][j];
                            v = F(i, j, k) - beta * dt * coef * (
                                    cx2 * (F(i + 1, j, k) - 2.0 * F(i, j, k) + F(i - 1, j, k)) * hx2 +
                                    cx1 * (F(i + 1, j, k) - F(i - 1, j, k)) * hx1 +
                                    cy2 * (F(i, j + 1, k) - 2.0 * F(i, j, k) + F(i, j - 1, k)) * hy2 +
                                    cy1 * (F(i, j + 1, k) - F(i, j - 1, k)) * hy1 +
                                    cz2 * (F(i, j, k + 1) - 2.0 * F(i, j, k) + F(i, j, k - 1)) * hz2 +
                                    cz1 * (F(i, j, k + 1) - F(i, j, k - 1)) * hz1);
                        } else {
                            v = F(i, j, k) - beta * dt * coef * (
                                    cx2 * (F(i + 1, j, k) - 2.0 * F(i, j, k) + F(i - 1, j, k)) * hx2 +
                                    cx1 * (F(i + 1, j, k) - F(i - 1, j, k)) * hx1 +
                                    cz2 * (F(i, j, k + 1) - 2.0 * F(i, j, k) + F(i, j, k - 1)) * hz2 +
                                    cz1 * (F(i, j, k + 1) - F(i, j, k - 1)) * hz1);
                        }
                        double t = std::fabs(v - R(i, j, k));
                        if (t > m) m = t;
                    }
            if (iters) *iters += 1;
            if (m < prm.cn_tolerance) return SARAS_OK;
            iterCount += 1;
            if (iterCount > maxIterations) return SARAS_DIVERGED;
        }
    }

    /* H += the diffusion term of F over the core, x then y then z
     * (vfield::computeDiff, vfield.cc:150-203; sfield::computeDiff,
     * sfield.cc:133-158). */
    void diff_into(const Arr3 &F, Arr3 &H) {
        core_loop([&](int i, int j, int k) {
            H(i, j, k) += d2(F, 0, i, j, k);
            if (d3) H(i, j, k) += d2(F, 1, i, j, k);
            H(i, j, k) += d2(F, 2, i, j, k);
        });
    }
    /* H -= the convection of F by V over the core, direction by direction
     * (computeNLin, vfield.cc:205-269, sfield.cc:160-198): nlScheme 1 the
     * standard form u dF/dx, 2 hybrid upwinding with diffusion coefficient
     * dcoef, 3 Morinishi.  A planar run has no y direction; the reference's
     * upwind loops still visit it with Vy = 0, which subtracts a zero. */
    void nlin_into(const Arr3 &F, Arr3 &H, double dcoef) {
        const int nl = prm.nl_scheme;
        core_loop([&](int i, int j, int k) {
            for (int d = 0; d < 3; d++) {
                if (!d3 && d == 1) continue;
                const Arr3 &Va = d == 0 ? Vx : (d == 1 ? Vy : Vz);
                double t;
                if (nl == 3)
                    t = mterm(F, Va, d, i, j, k);
                else if (nl == 2)
                    t = uterm(F, Va, dcoef, d, i, j, k);
                else
                    t = Va(i, j, k) * d1(F, d, i, j, k);
                H(i, j, k) -= t;
            }
        });
    }
    /* mgRHS = div V * scale, mgSolve into Pp, Pp.syncFaces(), P += Pp,
     * V -= fac * grad Pp, boundary conditions of V, P and T (lsRK3_d3.cc:
     * 270-304, eulerCN_d3.cc:240-268). */
    void project(double scale, double fac, int *mgc) {
        Arr3 *vel[3] = {&Vx, &Vy, &Vz};
        Arr3 *pg[3] = {&pgX, &pgY, &pgZ};
        const saras_field_bc *vbc[3] = {&prm.bc_vx, &prm.bc_vy, &prm.bc_vz};
        mgRHS.fill(0.0);
        core_loop([&](int i, int j, int k) {
            mgRHS(i, j, k) += d1(Vx, 0, i, j, k);
            if (d3) mgRHS(i, j, k) += d1(Vy, 1, i, j, k);
            mgRHS(i, j, k) += d1(Vz, 2, i, j, k);
        });
        full_loop(mgRHS, [&](size_t q) { mgRHS.v[q] *= scale; });
        int64_t st[3] = {Pp.s0, Pp.s1, 1};
        double *pp0 = &Pp(0, 0, 0);
        const double *rh0 = &mgRHS(0, 0, 0);
        int nc = 0;
        int ms = mg->mg_solve(pp0, rh0, st, nullptr, 0, &nc, nullptr);
        if (mgc) *mgc += nc;
        (void)ms;
        sync_faces(Pp);
        full_loop(P, [&](size_t q) { P.v[q] += Pp.v[q]; });
        core_loop([&](int i, int j, int k) {
            pgX(i, j, k) = d1(Pp, 0, i, j, k);
            if (d3) pgY(i, j, k) = d1(Pp, 1, i, j, k);
            pgZ(i, j, k) = d1(Pp, 2, i, j, k);
        });
        for (int c = 0; c < 3; c++) {
            Arr3 &F = *vel[c];
            full_loop(*pg[c], [&](size_t q) {
                pg[c]->v[q] *= fac;
                F.v[q] -= pg[c]->v[q];
            });
        }
        for (int c = 0; c < 3; c++) {
            if (!d3 && c == 1) continue;
            impose_bcs(*vel[c], *vbc[c]);
        }
        impose_bcs(P, prm.bc_p);
        if (prm.with_scalar) impose_bcs(T, prm.bc_t);
    }

    /* eulerCN_d3::timeAdvance(V, P[, T]) (lib/timestep/eulerCN_d3.cc:
     * 88-176, 178-268); eulerCN_d2 skips Vy.  Crank-Nicolson weights
     * alpha = beta = 1/2 (eulerCN_d3.cc:62-63). */
    int euler_advance(int *mgc, int *cni) {
        const double alphCN2 = 1.0 / 2.0, betaCN2 = 1.0 / 2.0;
        const bool sc = prm.with_scalar != 0;
        const double nu = prm.nu, kappa = prm.kappa, dt = prm.dt;
        Arr3 *vel[3] = {&Vx, &Vy, &Vz};
        Arr3 *nse[3] = {&nseX, &nseY, &nseZ};
        Arr3 *pg[3] = {&pgX, &pgY, &pgZ};
        const saras_field_bc *vbc[3] = {&prm.bc_vx, &prm.bc_vy, &prm.bc_vz};
        for (int c = 0; c < 3; c++) nse[c]->fill(0.0);
        tmpRHS.fill(0.0);
        for (int c = 0; c < 3; c++) {
            if (!d3 && c == 1) continue;
            diff_into(*vel[c], *nse[c]);
        }
        {
            const double f = nu * alphCN2;
            for (int c = 0; c < 3; c++) full_loop(*nse[c], [&](size_t q) { nse[c]->v[q] *= f; });
        }
        if (sc) {
            diff_into(T, tmpRHS);
            const double f = kappa * alphCN2;
            full_loop(tmpRHS, [&](size_t q) { tmpRHS.v[q] *= f; });
        }
        for (int c = 0; c < 3; c++) {
            if (!d3 && c == 1) continue;
            nlin_into(*vel[c], *nse[c], nu);
        }
        if (sc) nlin_into(T, tmpRHS, kappa);
        /* buoyantForce::addForcing (buoyantForce.cc:64-69); the zero forcing
         * of a run without temperature adds nothing */
        if (sc)
            for (int c = 0; c < 3; c++) {
                const double gt = prm.g_terms[c];
                full_loop(*nse[c], [&](size_t q) { nse[c]->v[q] -= gt * T.v[q]; });
            }
        for (int c = 0; c < 3; c++) pg[c]->fill(0.0);
        core_loop([&](int i, int j, int k) {
            pgX(i, j, k) = d1(P, 0, i, j, k);
            if (d3) pgY(i, j, k) = d1(P, 1, i, j, k);
            pgZ(i, j, k) = d1(P, 2, i, j, k);
        });
        for (int c = 0; c < 3; c++) {
            Arr3 &F = *vel[c];
            full_loop(*nse[c], [&](size_t q) {
                nse[c]->v[q] -= pg[c]->v[q];
                nse[c]->v[q] *= dt;
                nse[c]->v[q] += F.v[q];
            });
            sync_faces(*nse[c]);
        }
        if (sc) {
            full_loop(tmpRHS, [&](size_t q) {
                tmpRHS.v[q] *= dt;
                tmpRHS.v[q] += T.v[q];
            });
            sync_faces(tmpRHS);
        }
        for (int c = 0; c < 3; c++) {
            if (!d3 && c == 1) continue;
            int s = cn_solve(*vel[c], *nse[c], nu, betaCN2, *vbc[c], cni);
            if (s) return s;
        }
        if (sc) {
            int s = cn_solve(T, tmpRHS, kappa, betaCN2, prm.bc_t, cni);
            if (s) return s;
        }
        project(1.0 / dt, dt, mgc);
        return SARAS_OK;
    }

    /* vfield::computeTStp (vfield.cc:691-719): the maximum over the core of
     * |u|/avgDx + |v|/avgDy + |w|/avgDz, avgD = L/N; the caller divides the
     * Courant number by it. */
    double cfl_max() const {
        const double ax = g.L[0] / g.N[0], ay = g.L[1] / g.N[1], az = g.L[2] / g.N[2];
        double m = 0.0;
        for (int i = 0; i < g.N[0]; i++)
            for (int j = 0; j < g.N[1]; j++)
                for (int k = 0; k < g.N[2]; k++) {
                    double v = std::fabs(Vx(i, j, k)) / ax;
                    if (d3) v = v + std::fabs(Vy(i, j, k)) / ay;
                    v = v + std::fabs(Vz(i, j, k)) / az;
                    if (v > m) m = v;
                }
        return m;
    }

    /* tseries::writeTSData(T) (tseries.cc:291-488) and writeTSData()
     * (tseries.cc:209-289) on one rank: the sums run sequentially in the
     * reference's loop order.  Returns SARAS_DIVERGED on the divergence
     * abort (tseries.cc:216-222). */
    int tseries(const saras_run_params &rp, double time, double dt, saras_tseries_row &row, double &oldDiv) {
        const int n0 = g.N[0], n1 = g.N[1], n2 = g.N[2];
        const bool sc = prm.with_scalar != 0;
        double divVal = 0.0;
        for (int i = 0; i < n0; i++)
            for (int j = 0; j < n1; j++)
                for (int k = 0; k < n2; k++) {
                    double dv = 0.0;
                    dv += d1(Vx, 0, i, j, k);
                    if (d3) dv += d1(Vy, 1, i, j, k);
                    dv += d1(Vz, 2, i, j, k);
                    if (std::fabs(dv) > divVal) divVal = std::fabs(dv);
                }
        const double divSlope = divVal - oldDiv;
        const bool abort = divVal > 1e3 && divSlope > 0;
        oldDiv = divVal;
        const double totalVol = d3 ? g.L[0] * g.L[1] * g.L[2] : g.L[0] * g.L[2];
        auto dvx = [&](int i) { return g.dxi[0] / g.xi_x[0][i]; };
        auto dvy = [&](int j) { return g.dxi[1] / g.xi_x[1][j]; };
        auto dvz = [&](int k) { return g.dxi[2] / g.xi_x[2][k]; };
        row = saras_tseries_row{};
        row.time = time;
        row.dt = dt;
        row.divergence = divVal;
        if (!sc) {
            double ke = 0.0;
            for (int i = 0; i < n0; i++)
                for (int j = 0; j < n1; j++)
                    for (int k = 0; k < n2; k++) {
                        if (d3)
                            ke += (std::pow(Vx(i, j, k), 2.0) + std::pow(Vy(i, j, k), 2.0) +
                                   std::pow(Vz(i, j, k), 2.0)) * 0.5 * dvx(i) * dvy(j) * dvz(k);
                        else
                            ke += (std::pow(Vx(i, j, k), 2.0) + std::pow(Vz(i, j, k), 2.0)) * 0.5 * dvx(i) * dvz(k);
                    }
            ke /= totalVol;
            row.ke = ke;
            row.urms = std::sqrt(2.0 * ke);
            return abort ? SARAS_DIVERGED : SARAS_OK;
        }
        /* tseries::tseries (tseries.cc:105-150): on one rank both walls are
         * ours; wallDn is set by the bottom wall, then by the top wall */
        const bool zG = !(rp.g_axis[2] == 0);
        double csArea, wallDn;
        bool tWall;
        if (zG) {
            csArea = d3 ? g.L[0] * g.L[1] : g.L[0];
            csArea *= rp.prob_type == 9 ? 1 : 2;
            tWall = rp.prob_type < 9;
            wallDn = g.xG[2][0];
            if (tWall) wallDn = g.L[2] - g.xG[2][n2 - 1];
        } else {
            csArea = d3 ? g.L[1] * g.L[2] : g.L[2];
            tWall = true;
            wallDn = g.xG[0][0];
            wallDn = g.L[0] - g.xG[0][n0 - 1];
        }
        double localDt = 0.0;
        if (zG) {
            for (int i = 0; i < n0; i++)
                for (int j = 0; j < n1; j++) {
                    const double dArea = d3 ? dvx(i) * dvy(j) : dvx(i);
                    localDt += (1.0 - std::fabs(T(i, j, 0))) / wallDn * dArea;
                }
            if (tWall)
                for (int i = 0; i < n0; i++)
                    for (int j = 0; j < n1; j++) {
                        const double dArea = d3 ? dvx(i) * dvy(j) : dvx(i);
                        localDt += std::fabs(T(i, j, n2 - 1)) / wallDn * dArea;
                    }
        } else {
            for (int j = 0; j < n1; j++)
                for (int k = 0; k < n2; k++) {
                    const double dArea = d3 ? dvy(j) * dvz(k) : dvz(k);
                    localDt += (1.0 - std::fabs(T(0, j, k))) / wallDn * dArea;
                }
            for (int j = 0; j < n1; j++)
                for (int k = 0; k < n2; k++) {
                    const double dArea = d3 ? dvy(j) * dvz(k) : dvz(k);
                    localDt += std::fabs(T(n0 - 1, j, k)) / wallDn * dArea;
                }
        }
        double ke = 0.0, te = 0.0, uzt = 0.0;
        for (int i = 0; i < n0; i++)
            for (int j = 0; j < n1; j++)
                for (int k = 0; k < n2; k++) {
                    const double dVol = d3 ? dvx(i) * dvy(j) * dvz(k) : dvx(i) * dvz(k);
                    const double t = T(i, j, k);
                    const double theta = zG ? t + g.xG[2][k] - 1.0 : t + g.xG[0][i] - 1.0;
                    if (d3)
                        ke += (std::pow(Vx(i, j, k), 2.0) + std::pow(Vy(i, j, k), 2.0) +
                               std::pow(Vz(i, j, k), 2.0)) * 0.5 * dVol;
                    else
                        ke += (std::pow(Vx(i, j, k), 2.0) + std::pow(Vz(i, j, k), 2.0)) * 0.5 * dVol;
                    te += std::pow(theta, 2.0) * 0.5 * dVol;
                    uzt += (zG ? Vz(i, j, k) : Vx(i, j, k)) * t * dVol;
                }
        ke /= totalVol;
        te /= totalVol;
        row.nu_vol = 1.0 + (uzt / totalVol) / prm.kappa;
        row.nu_wall = localDt / csArea;
        row.re = std::sqrt(2.0 * ke) / prm.nu;
        row.ke = ke;
        row.te = te;
        row.urms = std::sqrt(2.0 * ke);
        return abort ? SARAS_DIVERGED : SARAS_OK;
    }

    /* scalar_d3::solvePDE / hydro_d3::solvePDE time loop (scalar_d3.cc:
     * 184-262) without probes and file output. */
    int run(const saras_run_params &rp, double &time, saras_tseries_row *rows, int cap, int *nrows, int *nsteps,
            int *mgc, int *cni) {
        const double tStp = prm.dt;
        double dt = prm.dt;
        double oldDiv = 1.0e10;
        int nr = 0, steps = 0, s = 0;
        saras_tseries_row row;
        s = tseries(rp, time, dt, row, oldDiv);
        if (nr < cap) rows[nr] = row;
        nr++;
        while (!s) {
            s = prm.integration == 1 ? euler_advance(mgc, cni) : time_advance(mgc, cni);
            if (s) break;
            if (rp.use_cfl) {
                dt = rp.courant / cfl_max();
                if (dt > tStp) dt = tStp;
                prm.dt = dt;
            }
            steps += 1;
            time += dt;
            if (steps % rp.io_count == 0) {
                s = tseries(rp, time, dt, row, oldDiv);
                if (nr < cap) rows[nr] = row;
                nr++;
                if (s) break;
            }
            if (std::fabs(rp.t_max - time) < 0.5 * dt) break;
            if (rp.max_steps > 0 && steps >= rp.max_steps) break;
        }
        if (nrows) *nrows = nr;
        if (nsteps) *nsteps = steps;
        return s;
    }

    /* lsRK3_d3::timeAdvance(V, P[, T]) (lib/timestep/lsRK3_d3.cc:94-177,
     * 190-305); lsRK3_d2 skips Vy. */
    int time_advance(int *mgc, int *cni) {
        static const double alph[3] = {4.0 / 15.0, 1.0 / 15.0, 1.0 / 6.0};
        static const double bet[3] = {4.0 / 15.0, 1.0 / 15.0, 1.0 / 6.0};
        static const double gam[3] = {8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};
        static const double zet[3] = {0.0, -17.0 / 60.0, -5.0 / 12.0};
        const bool sc = prm.with_scalar != 0;
        const double nu = prm.nu, kappa = prm.kappa, dt = prm.dt;
        Arr3 *vel[3] = {&Vx, &Vy, &Vz};
        Arr3 *nse[3] = {&nseX, &nseY, &nseZ};
        Arr3 *tv[3] = {&tvX, &tvY, &tvZ};
        Arr3 *pg[3] = {&pgX, &pgY, &pgZ};
        const saras_field_bc *vbc[3] = {&prm.bc_vx, &prm.bc_vy, &prm.bc_vz};
        for (int rk = 0; rk < 3; rk++) {
            for (int c = 0; c < 3; c++) nse[c]->fill(0.0);
            tmpRHS.fill(0.0);
            if (rk > 0) {
                for (int c = 0; c < 3; c++) {
                    double z = zet[rk];
                    full_loop(*nse[c], [&](size_t q) { nse[c]->v[q] += z * tv[c]->v[q]; });
                }
                if (sc) full_loop(tmpRHS, [&](size_t q) { tmpRHS.v[q] += zet[rk] * tSF.v[q]; });
            }
            /* diffusion */
            for (int c = 0; c < 3; c++) tv[c]->fill(0.0);
            tSF.fill(0.0);
            for (int c = 0; c < 3; c++) {
                if (!d3 && c == 1) continue;
                diff_into(*vel[c], *tv[c]);
            }
            if (sc) diff_into(T, tSF);
            {
                double an = alph[rk] * nu, ak = alph[rk] * kappa;
                for (int c = 0; c < 3; c++)
                    full_loop(*nse[c], [&](size_t q) { nse[c]->v[q] += an * tv[c]->v[q]; });
                if (sc) full_loop(tmpRHS, [&](size_t q) { tmpRHS.v[q] += ak * tSF.v[q]; });
            }
            /* forcing and pressure gradient */
            for (int c = 0; c < 3; c++) tv[c]->fill(0.0);
            tSF.fill(0.0);
            if (sc) {
                for (int c = 0; c < 3; c++) {
                    double gt = prm.g_terms[c];
                    full_loop(*tv[c], [&](size_t q) { tv[c]->v[q] -= gt * T.v[q]; });
                }
            }
            for (int c = 0; c < 3; c++) pg[c]->fill(0.0);
            core_loop([&](int i, int j, int k) {
                pgX(i, j, k) = d1(P, 0, i, j, k);
                if (d3) pgY(i, j, k) = d1(P, 1, i, j, k);
                pgZ(i, j, k) = d1(P, 2, i, j, k);
            });
            for (int c = 0; c < 3; c++)
                full_loop(*tv[c], [&](size_t q) { tv[c]->v[q] -= pg[c]->v[q]; });
            {
                double ab = alph[rk] + bet[rk];
                for (int c = 0; c < 3; c++)
                    full_loop(*nse[c], [&](size_t q) { nse[c]->v[q] += ab * tv[c]->v[q]; });
                if (sc) full_loop(tmpRHS, [&](size_t q) { tmpRHS.v[q] += ab * tSF.v[q]; });
            }
            /* non-linear terms */
            for (int c = 0; c < 3; c++) tv[c]->fill(0.0);
            tSF.fill(0.0);
            for (int c = 0; c < 3; c++) {
                if (!d3 && c == 1) continue;
                nlin_into(*vel[c], *tv[c], nu);
            }
            if (sc) nlin_into(T, tSF, kappa);
            {
                double gm = gam[rk];
                for (int c = 0; c < 3; c++)
                    full_loop(*nse[c], [&](size_t q) { nse[c]->v[q] += gm * tv[c]->v[q]; });
                if (sc) full_loop(tmpRHS, [&](size_t q) { tmpRHS.v[q] += gm * tSF.v[q]; });
            }
            for (int c = 0; c < 3; c++) {
                Arr3 &F = *vel[c];
                full_loop(*nse[c], [&](size_t q) {
                    nse[c]->v[q] *= dt;
                    nse[c]->v[q] += F.v[q];
                });
                sync_faces(*nse[c]);
            }
            if (sc) {
                full_loop(tmpRHS, [&](size_t q) {
                    tmpRHS.v[q] *= dt;
                    tmpRHS.v[q] += T.v[q];
                });
                sync_faces(tmpRHS);
            }
            /* CN Jacobi predictors */
            for (int c = 0; c < 3; c++) {
                if (!d3 && c == 1) continue;
                int s = cn_solve(*vel[c], *nse[c], nu, bet[rk], *vbc[c], cni);
                if (s) return s;
            }
            if (sc) {
                int s = cn_solve(T, tmpRHS, kappa, bet[rk], prm.bc_t, cni);
                if (s) return s;
            }
            /* pressure correction */
            project(1.0 / ((alph[rk] + bet[rk]) * dt), (alph[rk] + bet[rk]) * dt, mgc);
        }
        return SARAS_OK;
    }
};

void copy_in(Arr3 &a, const double *src, const int64_t *st) {
    if (!src) return;
    for (int i = a.lo(0); i <= a.hi(0); i++)
        for (int j = a.lo(1); j <= a.hi(1); j++)
            for (int k = a.lo(2); k <= a.hi(2); k++) a(i, j, k) = src[i * st[0] + j * st[1] + k * st[2]];
}
void copy_out(const Arr3 &a, double *dst, const int64_t *st) {
    if (!dst) return;
    for (int i = a.lo(0); i <= a.hi(0); i++)
        for (int j = a.lo(1); j <= a.hi(1); j++)
            for (int k = a.lo(2); k <= a.hi(2); k++) dst[i * st[0] + j * st[1] + k * st[2]] = a(i, j, k);
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

} // namespace

extern "C" {

void oracle_set_threads(int n) { g_threads = n > 0 ? n : 1; }

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int oracle_num_levels(const saras_grid_desc *gd, int levels) {
    Grid g;
    if (g.build(*gd, levels)) return -1;
    return g.vcdGlo + 1;
}

/* Per-level metric arrays as poisson::copyDerivs holds them (-1..n_l). */
int oracle_grid_metrics(const saras_grid_desc *gd, int levels, int level, int axis, double *x,
                        double *xixx, double *xix2, int *n_out) {
    Grid g;
    int s = g.build(*gd, levels);
    if (s) return s;
    if (level < 0 || level > g.vcdGlo || axis < 0 || axis > 2 || !g.active(axis)) return SARAS_BAD_ARG;
    const Vec1 &X = g.gm[15 * level + 5 * axis + 1];
    const Vec1 &A = g.gm[15 * level + 5 * axis + 3];
    const Vec1 &B = g.gm[15 * level + 5 * axis + 4];
    int n = int(X.v.size()) - 2;
    for (int i = -1; i <= n; i++) {
        if (x) x[i + 1] = X[i];
        if (xixx) xixx[i + 1] = A[i];
        if (xix2) xix2[i + 1] = B[i];
    }
    if (n_out) *n_out = n;
    return SARAS_OK;
}

/* Finest-level local metrics with the field pad (grid.cc:138-140, 491-503):
 * xi_x, xixx, xix2, x over -pad..n+pad-1. */
int oracle_field_metrics(const saras_grid_desc *gd, int axis, double *x, double *xi_x, double *xixx,
                         double *xix2) {
    Grid g;
    int s = g.build(*gd, 0);
    if (s) return s;
    int p = g.pad[axis];
    for (int i = -p; i < g.N[axis] + p; i++) {
        if (x) x[i + p] = g.xG[axis][i];
        if (xi_x) xi_x[i + p] = g.xi_x[axis][i];
        if (xixx) xixx[i + p] = g.xixx[axis][i];
        if (xix2) xix2[i + p] = g.xix2[axis][i];
    }
    return SARAS_OK;
}

/* poisson::mgSolve on caller arrays addressed at element (0,0,0). */
int oracle_mg_solve(const saras_grid_desc *gd, const saras_mg_params *prm, double *lhs, const double *rhs,
                    const int64_t *strides, double *res_hist, int hist_cap, int *n_cycles,
                    int *coarse_sweeps, double *seconds) {
    Grid g;
    int s = g.build(*gd, prm->levels);
    if (s) return s;
    if (prm->vc_count < 1 || prm->pre_smooth < 0 || prm->post_smooth < 0) return SARAS_BAD_ARG;
    Multigrid mg(g);
    mg.setup(*prm);
    if (coarse_sweeps) *coarse_sweeps = 0;
    double t0 = now_s();
    s = mg.mg_solve(lhs, rhs, strides, res_hist, hist_cap, n_cycles, coarse_sweeps);
    if (seconds) *seconds = now_s() - t0;
    return s;
}

/* One field operator of the time step on a padded field, over the core
 * (test hook for the stencils): op 1 calcDerivative1 along `axis`, op 2
 * calcDerivative2 along `axis`, op 3 the convection term of F by the
 * velocity (vx, vy, vz) as computeNLin adds it to a zero H, with diffusion
 * coefficient `dcoef` for the upwind Peclet number.  out receives the core
 * (its pads are left alone). */
int oracle_field_op(const saras_grid_desc *gd, const saras_rk3_params *prm, int op, int axis, double dcoef,
                    const double *f, const double *vx, const double *vy, const double *vz, double *out,
                    const int64_t *strides) {
    Rk3 r;
    int s = r.setup(*gd, *prm);
    if (s) return s;
    if (op < 1 || op > 3 || axis < 0 || axis > 2 || !r.g.active(axis)) return SARAS_BAD_ARG;
    copy_in(r.T, f, strides);
    copy_in(r.Vx, vx, strides);
    if (gd->dims == 3) copy_in(r.Vy, vy, strides);
    copy_in(r.Vz, vz, strides);
    r.tSF.fill(0.0);
    if (op == 3)
        r.nlin_into(r.T, r.tSF, dcoef);
    else
        r.core_loop([&](int i, int j, int k) {
            r.tSF(i, j, k) = op == 1 ? r.d1(r.T, axis, i, j, k) : r.d2(r.T, axis, i, j, k);
        });
    for (int i = 0; i < r.g.N[0]; i++)
        for (int j = 0; j < r.g.N[1]; j++)
            for (int k = 0; k < r.g.N[2]; k++) out[i * strides[0] + j * strides[1] + k * strides[2]] = r.tSF(i, j, k);
    return SARAS_OK;
}

/* The time loop (Rk3::run) on caller fields, which are updated. */
int oracle_rk3_loop(const saras_grid_desc *gd, const saras_rk3_params *prm, const saras_run_params *rp, double *vx,
                    double *vy, double *vz, double *p, double *t, double *pp, const int64_t *strides, double *time,
                    saras_tseries_row *rows, int cap, int *n_rows, int *n_steps, double *dt_out) {
    Rk3 r;
    int s = r.setup(*gd, *prm);
    if (s) return s;
    if (rp->io_count < 1) return SARAS_BAD_ARG;
    copy_in(r.Vx, vx, strides);
    if (gd->dims == 3) copy_in(r.Vy, vy, strides);
    copy_in(r.Vz, vz, strides);
    copy_in(r.P, p, strides);
    if (prm->with_scalar) copy_in(r.T, t, strides);
    copy_in(r.Pp, pp, strides);
    s = r.run(*rp, *time, rows, cap, n_rows, n_steps, nullptr, nullptr);
    if (dt_out) *dt_out = r.prm.dt;
    copy_out(r.Vx, vx, strides);
    if (gd->dims == 3) copy_out(r.Vy, vy, strides);
    copy_out(r.Vz, vz, strides);
    copy_out(r.P, p, strides);
    if (prm->with_scalar) copy_out(r.T, t, strides);
    copy_out(r.Pp, pp, strides);
    return s;
}

/* One time-series row and the CFL maximum of caller fields. */
int oracle_tseries(const saras_grid_desc *gd, const saras_rk3_params *prm, const saras_run_params *rp,
                   const double *vx, const double *vy, const double *vz, const double *t, const int64_t *strides,
                   double time, saras_tseries_row *row, double *cfl_max) {
    Rk3 r;
    int s = r.setup(*gd, *prm);
    if (s) return s;
    copy_in(r.Vx, vx, strides);
    if (gd->dims == 3) copy_in(r.Vy, vy, strides);
    copy_in(r.Vz, vz, strides);
    if (prm->with_scalar) copy_in(r.T, t, strides);
    double oldDiv = 1.0e10;
    s = r.tseries(*rp, time, prm->dt, *row, oldDiv);
    if (cfl_max) *cfl_max = r.cfl_max();
    return s;
}

/* `nsteps` calls of lsRK3 (integration 0 or 2) or eulerCN (integration 1)
 * timeAdvance on full padded fields (pad 1 or 2). */
int oracle_rk3_run(const saras_grid_desc *gd, const saras_rk3_params *prm, double *vx, double *vy,
                   double *vz, double *p, double *t, double *pp, const int64_t *strides, int nsteps,
                   int *mg_cycles, int *cn_iters, double *seconds) {
    Rk3 r;
    int s = r.setup(*gd, *prm);
    if (s) return s;
    copy_in(r.Vx, vx, strides);
    if (gd->dims == 3) copy_in(r.Vy, vy, strides);
    copy_in(r.Vz, vz, strides);
    copy_in(r.P, p, strides);
    if (prm->with_scalar) copy_in(r.T, t, strides);
    copy_in(r.Pp, pp, strides);
    if (mg_cycles) *mg_cycles = 0;
    if (cn_iters) *cn_iters = 0;
    double t0 = now_s();
    for (int n = 0; n < nsteps && !s; n++)
        s = prm->integration == 1 ? r.euler_advance(mg_cycles, cn_iters) : r.time_advance(mg_cycles, cn_iters);
    if (seconds) *seconds = now_s() - t0;
    copy_out(r.Vx, vx, strides);
    if (gd->dims == 3) copy_out(r.Vy, vy, strides);
    copy_out(r.Vz, vz, strides);
    copy_out(r.P, p, strides);
    if (prm->with_scalar) copy_out(r.T, t, strides);
    copy_out(r.Pp, pp, strides);
    return s;
}

} // extern "C"
