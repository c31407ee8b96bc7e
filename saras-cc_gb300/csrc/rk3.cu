// Time step of SARAS on GB300 -- the low-storage RK3 (lsRK3) and the
// Euler/Crank-Nicolson (eulerCN) integrators: the sub-step stencils around
// the pressure-Poisson solve, one fused kernel per stage of the reference's
// sequence of full-array Blitz operations.
//
// Reference: lsRK3_d3::timeAdvance(V,P,T) and (V,P) (lib/timestep/
// lsRK3_d3.cc:94-177, 190-305; lsRK3_d2.cc), eulerCN_d3::timeAdvance
// (lib/timestep/eulerCN_d3.cc:88-268; eulerCN_d2.cc), timestep::solveVx/Vy/
// Vz/T (lib/timestep/predictors.cc:59-423), vfield/sfield::computeDiff,
// computeNLin (nlScheme 1 standard, 2 hybrid upwind, 3 Morinishi),
// divergence, gradient (lib/field/vfield.cc, sfield.cc, plainsf.cc),
// derivative::calcDerivative1_* / 2** with dScheme 1 and 2
// (lib/field/derivative.cc:104-318), field BC writers (lib/boundary/
// dirichlet.cc, neumann.cc) and buoyantForce::addForcing
// (lib/force/buoyantForce.cc:64-69).
//
// Every per-cell value is formed in the reference's operation order with
// separately rounded FP64 operations, so one step is bit-identical to the
// single-rank reference arithmetic (given the same multigrid form).  The
// Blitz stencils are taken as central12n = (F[+1]-F[-1])*0.5, central22n =
// (F[-1]-2F)+F[+1], central14n = (8(F[+1]-F[-1]) - (F[+2]-F[-2]))/12 and
// central24n = (16(F[+1]+F[-1]) - 30F - (F[+2]+F[-2]))/12.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <math_constants.h>

#include "mg_fast.cuh"

namespace saras {
saras_status mg_solve_resident(saras_mg *h, int32_t *n_cycles);
}

using namespace saras;

namespace {

constexpr int BX = 128;
constexpr int RK_TABLES = 11;  // per-axis metric tables of a handle (RkTab)

// Field layout: core plus `p` ghost layers on x and z and `py` on y (1 for
// the planar case, grid.cc:91-95).  Element (i,j,k) sits at (i+p)*s0 +
// (j+py)*s1 + (k+KOFF): k-rows start their core on a 32-byte boundary and
// the ghosts k = -p.. -1 sit just below.  With p = 1 this is the multigrid
// level layout (Lay).
struct FLay {
    int n0, n1, n2;
    int p, py;
    int64_t s0, s1;
    int64_t size;

    __host__ __device__ __forceinline__ int64_t at(int i, int j, int k) const {
        return (int64_t)(i + p) * s0 + (int64_t)(j + py) * s1 + (int64_t)(k + KOFF);
    }
    __host__ __device__ __forceinline__ int ext(int a) const { return a == 0 ? n0 : (a == 1 ? n1 : n2); }
    __host__ __device__ __forceinline__ int pad(int a) const { return a == 1 ? py : p; }
};

FLay make_flay(int n0, int n1, int n2, int p, int py) {
    FLay l;
    l.n0 = n0;
    l.n1 = n1;
    l.n2 = n2;
    l.p = p;
    l.py = py;
    l.s1 = ((int64_t)n2 + KOFF + p + 3) / 4 * 4;
    l.s0 = l.s1 * (n1 + 2 * py);
    l.size = l.s0 * (n0 + 2 * p);
    return l;
}

// Per-axis finest-level metric tables over core indices and scalars.
struct RkTab {
    const double *xi_x[3], *xixx[3], *xix2[3];
    const double *a2[3], *a1[3];  // ihx2*xix2, i2hx*xixx (timestep coefficients)
    const double *dh[3];          // x(i+1) - x(i): the upwind Peclet length
    const double *dv[3];          // dXi / xi_x: cell extent (tseries volumes and areas)
    const double *xc[3];          // cell-centre coordinate x(i)
    // the FAST stencil form's folded coefficients
    const double *k1[3];   // xi_x / (2 dXi): first derivative, second order
    const double *k2a[3];  // xixx / (2 dXi): the first-derivative part of the second derivative
    const double *k2b[3];  // xix2 / dXi^2: its second-difference part
};
struct RkScal {
    double ih[3], ih2d[3];  // derivative: 1/dXi, pow(1/dXi, 2)
    double ih2t[3], i2ht[3]; // timestep: 1/pow(dXi,2), 0.5/dXi
    double i2d[3];           // vfield/sfield: 1/(2 dXi) (vfield.cc:133-135)
    double pe_limit;         // "Peclet Limit"
    double ua, ub, uc, ud;   // upwind stencil weights (vfield.cc:114-130)
    double dc_v, dc_t;       // diffusion coefficients of V and T (Peclet number)
};

// Field boundary rules: periodic flags, per face Dirichlet (2v) or Neumann
// (v * hWall) constants.
struct FBC {
    int per[3];
    int type[6];
    double two_v[6];
    double kh[6];
};

struct Stage {
    int rk;
    int euler;  // eulerCN right-hand side instead of the RK3 sub-stage
    int nls;    // non-linear scheme 1, 2 or 3
    double zeta, anu, akap, ab, gam, dt;
    double g[3];
};

template <class LY>
__device__ __forceinline__ int64_t axis_stride(const LY &L, int a) {
    return a == 0 ? L.s0 : (a == 1 ? L.s1 : 1);
}
template <class LY>
__device__ __forceinline__ int axis_ext(const LY &L, int a) {
    return a == 0 ? L.n0 : (a == 1 ? L.n1 : L.n2);
}

// calcDerivative1 (derivative.cc:104-204): xi_x * (c * ihx), c = central12n
// for dScheme 1; for dScheme 2 central14n, or 0.5*(F+ - F-) on the first and
// last core cell of the axis (on one rank every axis has both).
template <int DS, class LY>
__device__ __forceinline__ double d1(const double *F, const LY &L, const RkTab &T, const RkScal &S, int a,
                                     int idx, int64_t c) {
    const int64_t st = axis_stride(L, a);
    const double fp = F[c + st], fm = F[c - st];
    double cc;
    if (DS == 1) {
        cc = rmul(rsub(fp, fm), 0.5);
    } else if (idx == 0 || idx == axis_ext(L, a) - 1) {
        cc = rmul(0.5, rsub(fp, fm));
    } else {
        cc = rdiv(rsub(rmul(8.0, rsub(fp, fm)), rsub(F[c + 2 * st], F[c - 2 * st])), 12.0);
    }
    return rmul(T.xi_x[a][idx], rmul(cc, S.ih[a]));
}

// calcDerivative2 (derivative.cc:206-318): xixx*(c1*ihx) + xix2*(c2*ihx2);
// dScheme 2 takes the reference's F+ - 2F + F- on the first and last cell.
template <int DS>
__device__ __forceinline__ double d2(const double *F, const FLay &L, const RkTab &T, const RkScal &S, int a,
                                     int idx, int64_t c) {
    const int64_t st = axis_stride(L, a);
    const double fp = F[c + st], fm = F[c - st], f0 = F[c];
    double c1, c2;
    if (DS == 1) {
        c1 = rmul(rsub(fp, fm), 0.5);
        c2 = radd(rsub(fm, rmul(2.0, f0)), fp);
    } else if (idx == 0 || idx == L.ext(a) - 1) {
        c1 = rmul(0.5, rsub(fp, fm));
        c2 = radd(rsub(fp, rmul(2.0, f0)), fm);
    } else {
        const double fp2 = F[c + 2 * st], fm2 = F[c - 2 * st];
        c1 = rdiv(rsub(rmul(8.0, rsub(fp, fm)), rsub(fp2, fm2)), 12.0);
        c2 = rdiv(rsub(rsub(rmul(16.0, radd(fp, fm)), rmul(30.0, f0)), radd(fp2, fm2)), 12.0);
    }
    return radd(rmul(T.xixx[a][idx], rmul(c1, S.ih[a])), rmul(T.xix2[a][idx], rmul(c2, S.ih2d[a])));
}

// One direction of Morinishi's skew-symmetric convection term
// (vfield.cc:271-474, sfield.cc:200-323): (adv + div)/2 with
// adv = Va*xi*dF*i2d and div = xi*d(Va F)*i2d, the products standing for the
// Blitz temporaries tempXX = V.Vx*Vx etc.  dF is F+ - F- (dScheme 1, and
// dScheme 2 at the first and last point) or (-F+2 + 8F+1 - 8F-1 + F-2)/6.
// The reference tests the last z point against the y extent (core.ubound(1),
// vfield.cc:337,427), which is kept: along z the second-order form is taken
// at k = 0 and k = n1 - 1.
template <int DS>
__device__ __forceinline__ double mterm(const double *F, const double *Va, const FLay &L, const RkTab &T,
                                        const RkScal &S, int a, int idx, int64_t c) {
    const int64_t st = axis_stride(L, a);
    const double x = T.xi_x[a][idx];
    const int last = (a == 2 ? L.n1 : L.ext(a)) - 1;
    if (DS == 2 && idx != 0 && idx != last) {
        const double f2 = F[c + 2 * st], f1 = F[c + st], g1 = F[c - st], g2 = F[c - 2 * st];
        const double sf = radd(rsub(radd(-f2, rmul(8.0, f1)), rmul(8.0, g1)), g2);
        const double sv = radd(rsub(radd(-rmul(Va[c + 2 * st], f2), rmul(8.0, rmul(Va[c + st], f1))),
                                    rmul(8.0, rmul(Va[c - st], g1))),
                               rmul(Va[c - 2 * st], g2));
        const double adv = rdiv(rmul(rmul(rmul(Va[c], x), sf), S.i2d[a]), 6.0);
        const double div = rdiv(rmul(rmul(x, sv), S.i2d[a]), 6.0);
        return rdiv(radd(adv, div), 2.0);
    }
    const double adv = rmul(rmul(rmul(Va[c], x), rsub(F[c + st], F[c - st])), S.i2d[a]);
    const double div = rmul(rmul(x, rsub(rmul(Va[c + st], F[c + st]), rmul(Va[c - st], F[c - st]))), S.i2d[a]);
    return rdiv(radd(adv, div), 2.0);
}

// One direction of the hybrid upwind convection term (vfield.cc:475-690,
// sfield.cc:324-495): below the "Peclet Limit" (Pe = |u| dh / diffCoeff)
// central differences, above it the stencil biased against the local
// velocity; dScheme 1 first-order upwinding with second-order central
// differences, dScheme 2 second-order upwinding with fourth-order central
// differences and second-order central differences on the end cells.
template <int DS>
__device__ __forceinline__ double uterm(const double *F, const double *Va, const FLay &L, const RkTab &T,
                                        const RkScal &S, double dcoef, int a, int idx, int64_t c) {
    const int64_t st = axis_stride(L, a);
    const double u = Va[c];
    const double ux = rmul(u, T.xi_x[a][idx]);
    const double f0 = F[c], fp = F[c + st], fm = F[c - st];
    if (DS == 2 && (idx == 0 || idx == L.ext(a) - 1)) return rmul(rmul(ux, rsub(fp, fm)), S.i2d[a]);
    const double pe = rdiv(rmul(fabs(u), T.dh[a][idx]), dcoef);
    if (DS == 1) {
        if (pe < S.pe_limit) return rmul(rmul(ux, rsub(fp, fm)), S.i2d[a]);
        if (u > 0) return rmul(rmul(ux, rsub(radd(rmul(-S.ua, fm), rmul(S.ub, f0)), rmul(S.uc, fp))), S.i2d[a]);
        return rmul(rmul(ux, radd(rsub(rmul(S.ua, fp), rmul(S.ub, f0)), rmul(S.uc, fm))), S.i2d[a]);
    }
    const double fp2 = F[c + 2 * st], fm2 = F[c - 2 * st];
    if (pe < S.pe_limit)
        return rdiv(rmul(rmul(ux, radd(rsub(radd(-fp2, rmul(8.0, fp)), rmul(8.0, fm)), fm2)), S.i2d[a]), 6.0);
    if (u > 0)
        return rmul(rmul(ux, rsub(radd(rsub(rmul(S.ua, fm2), rmul(S.ub, fm)), rmul(S.uc, f0)), rmul(S.ud, fp))),
                    S.i2d[a]);
    return rmul(rmul(ux, radd(rsub(radd(rmul(-S.ua, fp2), rmul(S.ub, fp)), rmul(S.uc, f0)), rmul(S.ud, fm))),
                S.i2d[a]);
}

// The convection contribution of one direction for the selected scheme; the
// caller subtracts it.  nlScheme 1 is u dF/dx (vfield.cc:205-245).
template <int DS>
__device__ __forceinline__ double nterm(int nls, const double *F, const double *Va, const FLay &L,
                                        const RkTab &T, const RkScal &S, double dcoef, int a, int idx,
                                        int64_t c) {
    if (nls == 3) return mterm<DS>(F, Va, L, T, S, a, idx, c);
    if (nls == 2) return uterm<DS>(F, Va, L, T, S, dcoef, a, idx, c);
    return rmul(Va[c], d1<DS>(F, L, T, S, a, idx, c));
}

struct Fields {
    const double *V[3];
    const double *P, *T;
    double *nse[3], *nl[3];
    double *tmpR, *nlT;
};

// Right-hand side of one field at one cell.  RK3 sub-stage (lsRK3_d3.cc:
// 199-268): zeta*NL_prev + alpha*nu*Diff + (alpha+beta)*(F - grad P) +
// gamma*NL, times dt, plus the field; NL is kept for the next stage.
// eulerCN (eulerCN_d3.cc:178-241): Diff*(nu/2) - NL - F - grad P, times dt,
// plus the field.  comp 0..2 are the velocity components, 3 the scalar.
template <bool D3, bool SC, int DS>
__device__ __forceinline__ void rhs_cell(const Fields &f, const FLay &L, const RkTab &T, const RkScal &S,
                                         const Stage &sg, int comp, int i, int j, int k, int64_t c,
                                         double &rhs_out, double &nl_out) {
    const int id[3] = {i, j, k};
    const bool vel = comp < 3;
    const double *F = vel ? f.V[comp] : f.T;
    const double dcoef = vel ? S.dc_v : S.dc_t;
    double dif = radd(0.0, d2<DS>(F, L, T, S, 0, i, c));
    if (D3) dif = radd(dif, d2<DS>(F, L, T, S, 1, j, c));
    dif = radd(dif, d2<DS>(F, L, T, S, 2, k, c));
    if (sg.euler) {
        double h = rmul(dif, vel ? sg.anu : sg.akap);
        h = rsub(h, nterm<DS>(sg.nls, F, f.V[0], L, T, S, dcoef, 0, i, c));
        if (D3) h = rsub(h, nterm<DS>(sg.nls, F, f.V[1], L, T, S, dcoef, 1, j, c));
        h = rsub(h, nterm<DS>(sg.nls, F, f.V[2], L, T, S, dcoef, 2, k, c));
        if (vel) {
            if (SC) h = rsub(h, rmul(sg.g[comp], f.T[c]));
            h = rsub(h, d1<DS>(f.P, L, T, S, comp, id[comp], c));
        }
        h = rmul(h, sg.dt);
        rhs_out = radd(h, F[c]);
        nl_out = 0.0;
        return;
    }
    double r = 0.0;
    if (sg.rk > 0) r = radd(r, rmul(sg.zeta, vel ? f.nl[comp][c] : f.nlT[c]));
    r = radd(r, rmul(vel ? sg.anu : sg.akap, dif));
    double t = 0.0;
    if (vel) {
        if (SC) t = rsub(t, rmul(sg.g[comp], f.T[c]));
        t = rsub(t, d1<DS>(f.P, L, T, S, comp, id[comp], c));
    }
    r = radd(r, rmul(sg.ab, t));  // for T: the zero forcing, multAdd still runs
    double n = rsub(0.0, nterm<DS>(sg.nls, F, f.V[0], L, T, S, dcoef, 0, i, c));
    if (D3) n = rsub(n, nterm<DS>(sg.nls, F, f.V[1], L, T, S, dcoef, 1, j, c));
    n = rsub(n, nterm<DS>(sg.nls, F, f.V[2], L, T, S, dcoef, 2, k, c));
    r = radd(r, rmul(sg.gam, n));
    r = rmul(r, sg.dt);
    rhs_out = radd(r, F[c]);
    nl_out = n;
}

// ---- the FAST stencil form ----
// The same right-hand sides and Crank-Nicolson sweeps with the reference's
// operation order relaxed, for runs that do not need bit parity: the
// metric products folded into per-index tables (k1, k2a, k2b), the compiler
// free to contract a product into the add that follows (FMA), divisions by
// the stencils' constants taken as products with their reciprocals, and the
// Peclet test |u| dh / D < limit taken as |u| dh < limit D.  Values agree
// with the separately rounded form to rounding; they are not bit-identical
// to it.

// calcDerivative1: (F+ - F-) xi_x / (2 dXi); dScheme 2 interior
// (8 (F+ - F-) - (F+2 - F-2)) xi_x / (12 dXi).
template <int DS, class LY>
__device__ __forceinline__ double f_d1(const double *F, const LY &L, const RkTab &T, int a, int idx, int64_t c) {
    const int64_t st = axis_stride(L, a);
    const double df = F[c + st] - F[c - st];
    const double k = T.k1[a][idx];
    if (DS == 1 || idx == 0 || idx == axis_ext(L, a) - 1) return df * k;
    return (8.0 * df - (F[c + 2 * st] - F[c - 2 * st])) * (k * (1.0 / 6.0));
}

// calcDerivative2: xixx d/dXi + xix2 d2/dXi2 with the same stencils as d2.
template <int DS>
__device__ __forceinline__ double f_d2(const double *F, const FLay &L, const RkTab &T, int a, int idx, int64_t c) {
    const int64_t st = axis_stride(L, a);
    const double fp = F[c + st], fm = F[c - st], f0 = F[c];
    const double ka = T.k2a[a][idx], kb = T.k2b[a][idx];
    if (DS == 1 || idx == 0 || idx == L.ext(a) - 1) return (fp - fm) * ka + ((fp + fm) - 2.0 * f0) * kb;
    const double fp2 = F[c + 2 * st], fm2 = F[c - 2 * st];
    const double c1 = 8.0 * (fp - fm) - (fp2 - fm2);
    const double c2 = 16.0 * (fp + fm) - 30.0 * f0 - (fp2 + fm2);
    return c1 * (ka * (1.0 / 6.0)) + c2 * (kb * (1.0 / 12.0));
}

// Morinishi's term (mterm): (Va xi dF + xi d(Va F)) / (4 dXi), or with the
// fourth-order differences / (24 dXi).
template <int DS>
__device__ __forceinline__ double f_mterm(const double *F, const double *Va, const FLay &L, const RkTab &T,
                                          const RkScal &S, int a, int idx, int64_t c) {
    const int64_t st = axis_stride(L, a);
    const double x = T.xi_x[a][idx];
    const int last = (a == 2 ? L.n1 : L.ext(a)) - 1;
    if (DS == 2 && idx != 0 && idx != last) {
        const double f2 = F[c + 2 * st], f1 = F[c + st], g1 = F[c - st], g2 = F[c - 2 * st];
        const double sf = ((8.0 * f1 - f2) - 8.0 * g1) + g2;
        const double sv = ((8.0 * (Va[c + st] * f1) - Va[c + 2 * st] * f2) - 8.0 * (Va[c - st] * g1)) +
                          Va[c - 2 * st] * g2;
        return (Va[c] * sf + sv) * (x * S.i2d[a] * (1.0 / 12.0));
    }
    const double fp = F[c + st], fm = F[c - st];
    return (Va[c] * (fp - fm) + (Va[c + st] * fp - Va[c - st] * fm)) * (x * S.i2d[a] * 0.5);
}

// The hybrid upwind term (uterm).
template <int DS>
__device__ __forceinline__ double f_uterm(const double *F, const double *Va, const FLay &L, const RkTab &T,
                                          const RkScal &S, double dcoef, int a, int idx, int64_t c) {
    const int64_t st = axis_stride(L, a);
    const double u = Va[c];
    const double uk = u * T.xi_x[a][idx] * S.i2d[a];
    const double f0 = F[c], fp = F[c + st], fm = F[c - st];
    if (DS == 2 && (idx == 0 || idx == L.ext(a) - 1)) return uk * (fp - fm);
    const bool central = fabs(u) * T.dh[a][idx] < S.pe_limit * dcoef;
    if (DS == 1) {
        if (central) return uk * (fp - fm);
        if (u > 0) return uk * ((S.ub * f0 - S.ua * fm) - S.uc * fp);
        return uk * ((S.ua * fp - S.ub * f0) + S.uc * fm);
    }
    const double fp2 = F[c + 2 * st], fm2 = F[c - 2 * st];
    if (central) return uk * (((8.0 * fp - fp2) - 8.0 * fm) + fm2) * (1.0 / 6.0);
    if (u > 0) return uk * (((S.ua * fm2 - S.ub * fm) + S.uc * f0) - S.ud * fp);
    return uk * (((S.ub * fp - S.ua * fp2) - S.uc * f0) + S.ud * fm);
}

template <int DS>
__device__ __forceinline__ double f_nterm(int nls, const double *F, const double *Va, const FLay &L,
                                          const RkTab &T, const RkScal &S, double dcoef, int a, int idx,
                                          int64_t c) {
    if (nls == 3) return f_mterm<DS>(F, Va, L, T, S, a, idx, c);
    if (nls == 2) return f_uterm<DS>(F, Va, L, T, S, dcoef, a, idx, c);
    return Va[c] * f_d1<DS>(F, L, T, a, idx, c);
}

// rhs_cell's sums in the FAST form.
template <bool D3, bool SC, int DS>
__device__ __forceinline__ void f_rhs_cell(const Fields &f, const FLay &L, const RkTab &T, const RkScal &S,
                                           const Stage &sg, int comp, int i, int j, int k, int64_t c,
                                           double &rhs_out, double &nl_out) {
    const int id[3] = {i, j, k};
    const bool vel = comp < 3;
    const double *F = vel ? f.V[comp] : f.T;
    const double dcoef = vel ? S.dc_v : S.dc_t;
    double dif = f_d2<DS>(F, L, T, 0, i, c) + f_d2<DS>(F, L, T, 2, k, c);
    if (D3) dif += f_d2<DS>(F, L, T, 1, j, c);
    double n = f_nterm<DS>(sg.nls, F, f.V[0], L, T, S, dcoef, 0, i, c) +
               f_nterm<DS>(sg.nls, F, f.V[2], L, T, S, dcoef, 2, k, c);
    if (D3) n += f_nterm<DS>(sg.nls, F, f.V[1], L, T, S, dcoef, 1, j, c);
    double t = 0.0;  // forcing minus the pressure gradient
    if (vel) {
        t = -f_d1<DS>(f.P, L, T, comp, id[comp], c);
        if (SC) t -= sg.g[comp] * f.T[c];
    }
    const double a = vel ? sg.anu : sg.akap;
    if (sg.euler) {
        rhs_out = (a * dif - n + t) * sg.dt + F[c];
        nl_out = 0.0;
        return;
    }
    double r = a * dif + sg.ab * t - sg.gam * n;
    if (sg.rk > 0) r += sg.zeta * (vel ? f.nl[comp][c] : f.nlT[c]);
    rhs_out = r * sg.dt + F[c];
    nl_out = -n;
}

template <bool D3, bool SC, int DS, bool FAST>
__global__ void k_rhs(Fields f, FLay L, RkTab T, RkScal S, Stage sg) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = D3 ? (int)blockIdx.y : 0;
    const int i = blockIdx.z;
    if (k >= L.n2) return;
    const int64_t c = L.at(i, j, k);
    for (int comp = 0; comp < (SC ? 4 : 3); comp++) {
        if (!D3 && comp == 1) continue;
        double r, n;
        if (FAST)
            f_rhs_cell<D3, SC, DS>(f, L, T, S, sg, comp, i, j, k, c, r, n);
        else
            rhs_cell<D3, SC, DS>(f, L, T, S, sg, comp, i, j, k, c, r, n);
        if (comp < 3) {
            f.nse[comp][c] = r;
            if (!sg.euler) f.nl[comp][c] = n;
        } else {
            f.tmpR[c] = r;
            if (!sg.euler) f.nlT[c] = n;
        }
    }
}

// One Jacobi sweep of (1 - beta*dt*coef*L) u = rhs (predictors.cc:65-91).
// bdc = beta*dt*coef (the FAST form's folded factor).
template <bool D3, bool FAST>
__global__ void k_cn_jacobi(const double *__restrict__ F, const double *__restrict__ R, double *__restrict__ out,
                            FLay L, RkTab T, double dt, double coef, double beta, double den_fac, double bdc) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = D3 ? (int)blockIdx.y : 0;
    const int i = blockIdx.z;
    if (k >= L.n2) return;
    const int64_t c = L.at(i, j, k);
    const double xp = F[c + L.s0], xm = F[c - L.s0], zp = F[c + 1], zm = F[c - 1];
    if (FAST) {
        double s = T.a2[0][i] * (xp + xm) + T.a1[0][i] * (xp - xm);
        s += T.a2[2][k] * (zp + zm) + T.a1[2][k] * (zp - zm);
        double d3 = T.a2[0][i] + T.a2[2][k];
        if (D3) {
            const double yp = F[c + L.s1], ym = F[c - L.s1];
            s += T.a2[1][j] * (yp + ym) + T.a1[1][j] * (yp - ym);
            d3 += T.a2[1][j];
        }
        out[c] = (s * bdc + R[c]) / (den_fac * d3 + 1.0);
        return;
    }
    double s = radd(rmul(T.a2[0][i], radd(xp, xm)), rmul(T.a1[0][i], rsub(xp, xm)));
    double d3 = T.a2[0][i];
    if (D3) {
        const double yp = F[c + L.s1], ym = F[c - L.s1];
        s = radd(s, rmul(T.a2[1][j], radd(yp, ym)));
        s = radd(s, rmul(T.a1[1][j], rsub(yp, ym)));
        d3 = radd(d3, T.a2[1][j]);
    }
    s = radd(s, rmul(T.a2[2][k], radd(zp, zm)));
    s = radd(s, rmul(T.a1[2][k], rsub(zp, zm)));
    d3 = radd(d3, T.a2[2][k]);
    const double num = radd(rmul(rmul(rmul(s, dt), coef), beta), R[c]);
    out[c] = rdiv(num, radd(1.0, rmul(den_fac, d3)));
}

__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) {
        const double w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// max |u - beta*dt*coef*L u - rhs| over the core (predictors.cc:96-131),
// per-block partials.
template <bool D3, bool FAST>
__global__ void k_cn_resid(const double *__restrict__ F, const double *__restrict__ R, FLay L, RkTab T, RkScal S,
                           double bdc, double *__restrict__ part) {
    double m = 0.0;
    for_core_rows(L, [&](int i, int j, int k) {
        const int64_t c = L.at(i, j, k);
        const double u = F[c], u2 = rmul(2.0, u);
        const double xp = F[c + L.s0], xm = F[c - L.s0], zp = F[c + 1], zm = F[c - 1];
        if (FAST) {
            // the a2 / a1 tables are xix2 / dXi^2 and xixx / (2 dXi)
            double s = T.a2[0][i] * ((xp + xm) - u2) + T.a1[0][i] * (xp - xm);
            s += T.a2[2][k] * ((zp + zm) - u2) + T.a1[2][k] * (zp - zm);
            if (D3) {
                const double yp = F[c + L.s1], ym = F[c - L.s1];
                s += T.a2[1][j] * ((yp + ym) - u2) + T.a1[1][j] * (yp - ym);
            }
            const double t = fabs((u - bdc * s) - R[c]);
            if (t > m) m = t;
            if (!isfinite(t)) m = CUDART_INF;
            return;
        }
        double s = radd(rmul(rmul(T.xix2[0][i], radd(rsub(xp, u2), xm)), S.ih2t[0]),
                        rmul(rmul(T.xixx[0][i], rsub(xp, xm)), S.i2ht[0]));
        if (D3) {
            const double yp = F[c + L.s1], ym = F[c - L.s1];
            s = radd(s, rmul(rmul(T.xix2[1][j], radd(rsub(yp, u2), ym)), S.ih2t[1]));
            s = radd(s, rmul(rmul(T.xixx[1][j], rsub(yp, ym)), S.i2ht[1]));
        }
        s = radd(s, rmul(rmul(T.xix2[2][k], radd(rsub(zp, u2), zm)), S.ih2t[2]));
        s = radd(s, rmul(rmul(T.xixx[2][k], rsub(zp, zm)), S.i2ht[2]));
        const double v = rsub(u, rmul(bdc, s));
        const double t = fabs(rsub(v, R[c]));
        if (t > m) m = t;
        if (!isfinite(t)) m = CUDART_INF;
    });
    __shared__ double sh[32];
    m = warp_max(m);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        v = warp_max(v);
        if (threadIdx.x == 0) part[blockIdx.x] = v;
    }
}

__global__ void k_max_final(const double *__restrict__ part, int nb, double *__restrict__ out) {
    double m = 0.0;
    for (int b = threadIdx.x; b < nb; b += 32) {
        const double v = part[b];
        if (v > m) m = v;
    }
    m = warp_max(m);
    if (threadIdx.x == 0) out[0] = m;
}

// Time-series and CFL reductions of the current fields (tseries::
// writeTSData, tseries.cc:209-488; vfield::computeTStp, vfield.cc:691-719).
// Per cell in the reference's operation order; the sums then run per thread,
// per warp and per block in a fixed order (partials of NTS values per block).
struct TsPar {
    int zg;             // gravity along z: Nusselt through the z walls
    int twall;          // the top (far) wall counts
    double wall_dn;     // wallDn
    double avg[3];      // L/N, the CFL spacings
};
enum { TS_KE = 0, TS_TE, TS_UZT, TS_DTW, TS_DIV, TS_CFL, NTS };

__device__ __forceinline__ double block_sum(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x < 32) {
        r = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    return r;
}
__device__ __forceinline__ double block_max(double v, double *sh) {
    v = warp_max(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x < 32) {
        r = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        r = warp_max(r);
    }
    return r;
}

template <bool D3, bool SC, int DS>
__global__ void k_tseries(const double *__restrict__ vx, const double *__restrict__ vy,
                          const double *__restrict__ vz, const double *__restrict__ tf, FLay L, RkTab T, RkScal S,
                          TsPar tp, double *__restrict__ part) {
    double acc[NTS] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for_core_rows(L, [&](int i, int j, int k) {
        const int64_t c = L.at(i, j, k);
        const double u = vx[c], w = vz[c], v = D3 ? vy[c] : 0.0;
        const double dvx = T.dv[0][i], dvz = T.dv[2][k], dvy = D3 ? T.dv[1][j] : 1.0;
        const double s2 = D3 ? radd(radd(rmul(u, u), rmul(v, v)), rmul(w, w)) : radd(rmul(u, u), rmul(w, w));
        if (SC) {
            const double dvol = D3 ? rmul(rmul(dvx, dvy), dvz) : rmul(dvx, dvz);
            const double t = tf[c];
            const double theta = rsub(radd(t, tp.zg ? T.xc[2][k] : T.xc[0][i]), 1.0);
            acc[TS_KE] += rmul(rmul(s2, 0.5), dvol);
            acc[TS_TE] += rmul(rmul(rmul(theta, theta), 0.5), dvol);
            acc[TS_UZT] += rmul(rmul(tp.zg ? w : u, t), dvol);
            if (tp.zg) {
                const double da = D3 ? rmul(dvx, dvy) : dvx;
                if (k == 0) acc[TS_DTW] += rmul(rdiv(rsub(1.0, fabs(t)), tp.wall_dn), da);
                if (tp.twall && k == L.n2 - 1) acc[TS_DTW] += rmul(rdiv(fabs(t), tp.wall_dn), da);
            } else {
                const double da = D3 ? rmul(dvy, dvz) : dvz;
                if (i == 0) acc[TS_DTW] += rmul(rdiv(rsub(1.0, fabs(t)), tp.wall_dn), da);
                if (tp.twall && i == L.n0 - 1) acc[TS_DTW] += rmul(rdiv(fabs(t), tp.wall_dn), da);
            }
        } else {
            acc[TS_KE] += D3 ? rmul(rmul(rmul(rmul(s2, 0.5), dvx), dvy), dvz) : rmul(rmul(rmul(s2, 0.5), dvx), dvz);
        }
        double d = radd(0.0, d1<DS>(vx, L, T, S, 0, i, c));
        if (D3) d = radd(d, d1<DS>(vy, L, T, S, 1, j, c));
        d = radd(d, d1<DS>(vz, L, T, S, 2, k, c));
        acc[TS_DIV] = fmax(acc[TS_DIV], fabs(d));
        double cf = rdiv(fabs(u), tp.avg[0]);
        if (D3) cf = radd(cf, rdiv(fabs(v), tp.avg[1]));
        cf = radd(cf, rdiv(fabs(w), tp.avg[2]));
        acc[TS_CFL] = fmax(acc[TS_CFL], cf);
    });
    __shared__ double sh[32];
    for (int q = 0; q < NTS; q++) {
        const double r = q >= TS_DIV ? block_max(acc[q], sh) : block_sum(acc[q], sh);
        if (threadIdx.x == 0) part[(int64_t)blockIdx.x * NTS + q] = r;
    }
}

// Sums (maxima) of the per-block partials, one block, fixed order.
__global__ void k_tseries_final(const double *__restrict__ part, int nb, double *__restrict__ out) {
    __shared__ double sh[32];
    for (int q = 0; q < NTS; q++) {
        double a = 0.0;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            const double v = part[(int64_t)b * NTS + q];
            a = q >= TS_DIV ? fmax(a, v) : a + v;
        }
        const double r = q >= TS_DIV ? block_max(a, sh) : block_sum(a, sh);
        if (threadIdx.x == 0) out[q] = r;
    }
}

enum { FBC_PERIODIC = 0, FBC_WALL = 1, FBC_ZERO_OUTER = 2 };

// Ghost planes of a field along `axis`, over the full padded extents of the
// other two axes: the periodic copy of all ghost layers (field::syncFaces on
// one rank, mpidata.cc:371-397), the wall writers of the first ghost layer
// (dirichlet.cc:72-76, neumann.cc:87-93), or zeros in the second ghost layer
// of a wall axis.
__global__ void k_fbc(double *u, FLay L, FBC B, int axis, int mode) {
    const int o0 = axis == 0 ? 1 : 0, o1 = axis == 2 ? 1 : 2;
    const int b = (int)(blockIdx.x * blockDim.x + threadIdx.x) - L.pad(o1);
    const int a = (int)blockIdx.y - L.pad(o0);
    if (b >= L.ext(o1) + L.pad(o1)) return;
    const int n = L.ext(axis);
    int q[3];
    q[o0] = a;
    q[o1] = b;
    auto at = [&](int x) {
        q[axis] = x;
        return L.at(q[0], q[1], q[2]);
    };
    if (mode == FBC_PERIODIC) {
        const int p = L.pad(axis);
        for (int m = 0; m < p; m++) {
            u[at(n + m)] = u[at(m)];
            u[at(-p + m)] = u[at(n - p + m)];
        }
        return;
    }
    if (mode == FBC_ZERO_OUTER) {
        u[at(-2)] = 0.0;
        u[at(n + 1)] = 0.0;
        return;
    }
    const int f0 = 2 * axis, f1 = 2 * axis + 1;
    const double lo = u[at(0)], hi = u[at(n - 1)];
    u[at(-1)] = B.type[f0] == SARAS_FBC_DIRICHLET ? rsub(B.two_v[f0], lo) : rsub(lo, B.kh[f0]);
    u[at(n)] = B.type[f1] == SARAS_FBC_DIRICHLET ? rsub(B.two_v[f1], hi) : rsub(hi, B.kh[f1]);
}

// divergence of V into the multigrid RHS (level layout), scaled
// (lsRK3_d3.cc:272-276, eulerCN_d3.cc:243-244).
template <bool D3, int DS>
__global__ void k_divergence(const double *__restrict__ vx, const double *__restrict__ vy,
                             const double *__restrict__ vz, double *__restrict__ out, FLay L, Lay LM, RkTab T,
                             RkScal S, double scale) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = D3 ? (int)blockIdx.y : 0;
    const int i = blockIdx.z;
    if (k >= L.n2) return;
    const int64_t c = L.at(i, j, k);
    double d = radd(0.0, d1<DS>(vx, L, T, S, 0, i, c));
    if (D3) d = radd(d, d1<DS>(vy, L, T, S, 1, j, c));
    d = radd(d, d1<DS>(vz, L, T, S, 2, k, c));
    out[LM.at(i, j, k)] = rmul(d, scale);
}

// P += Pp; V -= fac * grad Pp (lsRK3_d3.cc:281-294, eulerCN_d3.cc:253-260).
// Pp is the multigrid level-0 iterate (one ghost layer: the fourth-order
// stencil reaches two cells only away from the end cells).
template <bool D3, int DS>
__global__ void k_correct(double *__restrict__ vx, double *__restrict__ vy, double *__restrict__ vz,
                          double *__restrict__ p, const double *__restrict__ pp, FLay L, Lay LM, RkTab T,
                          RkScal S, double fac) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = D3 ? (int)blockIdx.y : 0;
    const int i = blockIdx.z;
    if (k >= L.n2) return;
    const int64_t c = L.at(i, j, k), cm = LM.at(i, j, k);
    p[c] = radd(p[c], pp[cm]);
    vx[c] = rsub(vx[c], rmul(d1<DS>(pp, LM, T, S, 0, i, cm), fac));
    if (D3) vy[c] = rsub(vy[c], rmul(d1<DS>(pp, LM, T, S, 1, j, cm), fac));
    vz[c] = rsub(vz[c], rmul(d1<DS>(pp, LM, T, S, 2, k, cm), fac));
}

// Dense padded host box <-> device layout over the box -q..n+q-1 per axis
// (q = the box's ghost layers, at most the layout's).
template <class LY>
__global__ void k_box_in(const double *__restrict__ src, int64_t s0, int64_t s1, double *__restrict__ dst, LY L,
                         int qx, int qy) {
    const int k = (int)(blockIdx.x * blockDim.x + threadIdx.x) - qx;
    const int j = (int)blockIdx.y - qy, i = (int)blockIdx.z - qx;
    if (k >= L.n2 + qx) return;
    dst[L.at(i, j, k)] = src[(int64_t)i * s0 + (int64_t)j * s1 + k];
}
template <class LY>
__global__ void k_box_out(const double *__restrict__ src, LY L, double *__restrict__ dst, int64_t s0, int64_t s1,
                          int qx, int qy) {
    const int k = (int)(blockIdx.x * blockDim.x + threadIdx.x) - qx;
    const int j = (int)blockIdx.y - qy, i = (int)blockIdx.z - qx;
    if (k >= L.n2 + qx) return;
    dst[(int64_t)i * s0 + (int64_t)j * s1 + k] = src[L.at(i, j, k)];
}

}  // namespace

struct saras_rk3 {
    HostGrid grid;
    saras_rk3_params prm{};
    bool d3 = true;
    bool sc = true;
    int ds = 1;  // Differentiation Scheme (the grid's pad)
    cudaStream_t stream = nullptr;
    saras_mg *mg = nullptr;
    FLay L{};
    double *V[3] = {nullptr, nullptr, nullptr}, *Vb[3] = {nullptr, nullptr, nullptr};
    double *P = nullptr, *T = nullptr, *Tb = nullptr;
    double *nse[3] = {nullptr, nullptr, nullptr}, *nl[3] = {nullptr, nullptr, nullptr};
    double *tmpR = nullptr, *nlT = nullptr;
    double *tab = nullptr;
    RkTab tabs{};
    RkScal scal{};
    FBC bc[5]{};
    double *part = nullptr, *red = nullptr, *red_host = nullptr;
    int nblocks = 0;
    double *stage = nullptr;
    int64_t bst[3] = {0, 0, 0};
    int64_t box_elems = 0;
    int max_iterations = 0;
    int64_t launches = 0;
    int64_t dev_bytes = 0;
    int nfields = 0;  // the first allocations are the fields (cleared on retarget)
    std::vector<double *> allocs;
};

namespace {

inline int bxfor(int n) { return std::min(BX, (n + 31) / 32 * 32); }

saras_status rk_alloc(saras_rk3 *h, double **p, int64_t n) {
    cudaError_t e = cudaMalloc((void **)p, (size_t)std::max<int64_t>(n, 1) * sizeof(double));
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("cudaMalloc failed in the time integrator: %s", cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? SARAS_OOM : SARAS_CUDA_ERR;
    }
    h->allocs.push_back(*p);
    h->dev_bytes += std::max<int64_t>(n, 1) * (int64_t)sizeof(double);
    return SARAS_OK;
}

FBC make_fbc(const saras_rk3 *h, const saras_field_bc &b) {
    FBC f{};
    const HostGrid &g = h->grid;
    // neumann::neumann (lib/boundary/neumann.cc:50-66): hWall from the cell
    // centres next to the wall
    double hw[6];
    for (int d = 0; d < 3; d++) {
        const std::vector<double> &x = g.fx[d];
        const int p = (g.dims == 2 && d == 1) ? 1 : g.pad;
        hw[2 * d] = 2 * x[(size_t)p];
        hw[2 * d + 1] = 2 * (x[(size_t)(g.N[d] - 1 + p)] - g.L[d]);
    }
    for (int d = 0; d < 3; d++) f.per[d] = g.per[d] ? 1 : 0;
    for (int q = 0; q < 6; q++) {
        f.type[q] = b.type[q];
        f.two_v[q] = 2.0 * b.value[q];
        f.kh[q] = b.value[q] * hw[q];
    }
    return f;
}

void fbc_pass(saras_rk3 *h, cudaStream_t s, double *u, const FBC &B, int axis, int mode) {
    const FLay &L = h->L;
    const int o0 = axis == 0 ? 1 : 0, o1 = axis == 2 ? 1 : 2;
    const int acnt = L.ext(o0) + 2 * L.pad(o0), bcnt = L.ext(o1) + 2 * L.pad(o1);
    const int bx = bxfor(bcnt);
    k_fbc<<<dim3(cdiv(bcnt, bx), (unsigned)acnt), bx, 0, s>>>(u, L, B, axis, mode);
    h->launches++;
}

// field::syncFaces then the wall writers, x, y, z (sfield.cc:520-547).  After
// a Crank-Nicolson sweep (`after_sweep`) the field was assigned from the
// sweep's iterTemp, whose pads the reference never writes (timestep.cc:
// 117-118) and which read as zero; the first ghost layer and every periodic
// ghost are rewritten below, so only the second ghost layer of the wall
// axes keeps that zero.
void impose(saras_rk3 *h, cudaStream_t s, double *u, const FBC &B, bool after_sweep = false) {
    if (after_sweep && h->L.p > 1)
        for (int axis = 0; axis < 3; axis++)
            if (h->grid.active(axis) && !B.per[axis]) fbc_pass(h, s, u, B, axis, FBC_ZERO_OUTER);
    for (int pass = 0; pass < 2; pass++) {
        for (int axis = 0; axis < 3; axis++) {
            if (!h->d3 && axis == 1) continue;
            if ((pass == 0) != (bool)B.per[axis]) continue;
            fbc_pass(h, s, u, B, axis, pass == 0 ? FBC_PERIODIC : FBC_WALL);
        }
    }
}

dim3 cgrid(const FLay &L, bool d3, int bx) {
    return dim3(cdiv(L.n2, bx), d3 ? (unsigned)L.n1 : 1u, (unsigned)L.n0);
}

saras_status cn_solve(saras_rk3 *h, cudaStream_t s, int comp, const double *rhs, double coef, double beta,
                      int *iters) {
    const FLay &L = h->L;
    const int bx = bxfor(L.n2);
    const double dt = h->prm.dt;
    const double den_fac = 2.0 * dt * coef * beta;  // 2.0 * dt * nu * beta, left to right
    const double bdc = beta * dt * coef;            // beta * dt * nu, left to right
    double **cur = comp < 3 ? &h->V[comp] : &h->T;
    double **alt = comp < 3 ? &h->Vb[comp] : &h->Tb;
    const FBC &B = h->bc[comp < 3 ? comp : 4];
    int iterCount = 0;
    for (;;) {
        using JK = void (*)(const double *, const double *, double *, FLay, RkTab, double, double, double, double,
                            double);
        using RK = void (*)(const double *, const double *, FLay, RkTab, RkScal, double, double *);
        static const JK jk[2][2] = {{k_cn_jacobi<false, false>, k_cn_jacobi<false, true>},
                                    {k_cn_jacobi<true, false>, k_cn_jacobi<true, true>}};
        static const RK rk[2][2] = {{k_cn_resid<false, false>, k_cn_resid<false, true>},
                                    {k_cn_resid<true, false>, k_cn_resid<true, true>}};
        const int d3 = h->d3 ? 1 : 0, fast = h->prm.stencil_form == SARAS_STENCIL_FAST ? 1 : 0;
        jk[d3][fast]<<<cgrid(L, h->d3, bx), bx, 0, s>>>(*cur, rhs, *alt, L, h->tabs, dt, coef, beta, den_fac, bdc);
        h->launches++;
        std::swap(*cur, *alt);
        impose(h, s, *cur, B, true);
        rk[d3][fast]<<<h->nblocks, 256, 0, s>>>(*cur, rhs, L, h->tabs, h->scal, bdc, h->part);
        k_max_final<<<1, 32, 0, s>>>(h->part, h->nblocks, h->red);
        h->launches += 2;
        SARAS_CUDA(cudaMemcpyAsync(h->red_host, h->red, sizeof(double), cudaMemcpyDeviceToHost, s));
        SARAS_CUDA(cudaStreamSynchronize(s));
        if (iters) *iters += 1;
        const double m = h->red_host[0];
        if (!std::isfinite(m)) {
            set_error("non-finite residual in the Crank-Nicolson sweeps");
            return SARAS_NAN;
        }
        if (m < h->prm.cn_tolerance) return SARAS_OK;
        iterCount += 1;
        if (iterCount > h->max_iterations) {
            set_error("Jacobi iterations for component %d not converging", comp);
            return SARAS_DIVERGED;
        }
    }
}

using RhsKernel = void (*)(Fields, FLay, RkTab, RkScal, Stage);

template <bool FAST>
RhsKernel rhs_kernel_of(bool d3, bool sc, int ds) {
    // (dimension, scalar, differentiation scheme) -> kernel
    static const RhsKernel ks[2][2][2] = {
        {{k_rhs<false, false, 1, FAST>, k_rhs<false, false, 2, FAST>},
         {k_rhs<false, true, 1, FAST>, k_rhs<false, true, 2, FAST>}},
        {{k_rhs<true, false, 1, FAST>, k_rhs<true, false, 2, FAST>},
         {k_rhs<true, true, 1, FAST>, k_rhs<true, true, 2, FAST>}}};
    return ks[d3 ? 1 : 0][sc ? 1 : 0][ds == 2 ? 1 : 0];
}

RhsKernel rhs_kernel(bool d3, bool sc, int ds, bool fast) {
    return fast ? rhs_kernel_of<true>(d3, sc, ds) : rhs_kernel_of<false>(d3, sc, ds);
}

void launch_rhs(saras_rk3 *h, const Stage &sg) {
    Fields f;
    for (int d = 0; d < 3; d++) {
        f.V[d] = h->V[d];
        f.nse[d] = h->nse[d];
        f.nl[d] = h->nl[d];
    }
    f.P = h->P;
    f.T = h->T;
    f.tmpR = h->tmpR;
    f.nlT = h->nlT;
    const int bx = bxfor(h->L.n2);
    const RhsKernel k = rhs_kernel(h->d3, h->sc, h->ds, h->prm.stencil_form == SARAS_STENCIL_FAST);
    k<<<cgrid(h->L, h->d3, bx), bx, 0, h->stream>>>(f, h->L, h->tabs, h->scal, sg);
    h->launches++;
}

Stage base_stage(const saras_rk3 *h) {
    Stage sg{};
    sg.nls = h->prm.nl_scheme;
    sg.dt = h->prm.dt;
    for (int d = 0; d < 3; d++) sg.g[d] = h->prm.g_terms[d];
    return sg;
}

// lsRK3 weights (lsRK3_d3.cc:63-66) and the Crank-Nicolson weights of
// eulerCN (alpha = beta = 1/2, eulerCN_d3.cc:62-63).
const double RK_ALPH[3] = {4.0 / 15.0, 1.0 / 15.0, 1.0 / 6.0};
const double RK_BET[3] = {4.0 / 15.0, 1.0 / 15.0, 1.0 / 6.0};
const double RK_GAM[3] = {8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};
const double RK_ZET[3] = {0.0, -17.0 / 60.0, -5.0 / 12.0};
const double CN_ALPH = 1.0 / 2.0, CN_BET = 1.0 / 2.0;

// First half of a sub-stage, up to the pressure solve: the right-hand
// sides, the predictor sweeps and the divergence into the multigrid RHS
// (lsRK3_d3.cc:199-276, eulerCN_d3.cc:178-244).
saras_status stage_begin(saras_rk3 *h, int rk, int *cni) {
    cudaStream_t s = h->stream;
    const FLay &L = h->L;
    const int bx = bxfor(L.n2);
    const double nu = h->prm.nu, kappa = h->prm.kappa, dt = h->prm.dt;
    const bool euler = h->prm.integration == 1;
    Stage sg = base_stage(h);
    double beta, scale;
    if (euler) {
        sg.euler = 1;
        sg.anu = nu * CN_ALPH;
        sg.akap = kappa * CN_ALPH;
        beta = CN_BET;
        scale = 1.0 / dt;
    } else {
        sg.rk = rk;
        sg.zeta = RK_ZET[rk];
        sg.anu = RK_ALPH[rk] * nu;
        sg.akap = RK_ALPH[rk] * kappa;
        sg.ab = RK_ALPH[rk] + RK_BET[rk];
        sg.gam = RK_GAM[rk];
        beta = RK_BET[rk];
        scale = 1.0 / ((RK_ALPH[rk] + RK_BET[rk]) * dt);
    }
    launch_rhs(h, sg);
    for (int comp = 0; comp < 3; comp++) {
        if (!h->d3 && comp == 1) continue;
        SARAS_TRY(cn_solve(h, s, comp, h->nse[comp], nu, beta, cni));
    }
    if (h->sc) SARAS_TRY(cn_solve(h, s, 3, h->tmpR, kappa, beta, cni));
    Level &m0 = h->mg->lv[0];
    using DK = void (*)(const double *, const double *, const double *, double *, FLay, Lay, RkTab, RkScal, double);
    static const DK dks[2][2] = {{k_divergence<false, 1>, k_divergence<false, 2>},
                                 {k_divergence<true, 1>, k_divergence<true, 2>}};
    dks[h->d3 ? 1 : 0][h->ds == 2 ? 1 : 0]<<<cgrid(L, h->d3, bx), bx, 0, s>>>(h->V[0], h->V[1], h->V[2], m0.rhs, L,
                                                                          m0.lay, h->tabs, h->scal, scale);
    h->launches++;
    SARAS_CUDA(cudaGetLastError());
    return SARAS_OK;
}

// Second half, after the pressure solve left Pp in the multigrid level-0
// iterate: P += Pp, V -= fac grad Pp and the boundary conditions of V, P
// and T (lsRK3_d3.cc:278-304, eulerCN_d3.cc:246-268).
saras_status stage_end(saras_rk3 *h, int rk) {
    cudaStream_t s = h->stream;
    const FLay &L = h->L;
    const int bx = bxfor(L.n2);
    const double dt = h->prm.dt;
    const double fac = h->prm.integration == 1 ? dt : (RK_ALPH[rk] + RK_BET[rk]) * dt;
    Level &m0 = h->mg->lv[0];
    using CK = void (*)(double *, double *, double *, double *, const double *, FLay, Lay, RkTab, RkScal, double);
    static const CK cks[2][2] = {{k_correct<false, 1>, k_correct<false, 2>}, {k_correct<true, 1>, k_correct<true, 2>}};
    cks[h->d3 ? 1 : 0][h->ds == 2 ? 1 : 0]<<<cgrid(L, h->d3, bx), bx, 0, s>>>(h->V[0], h->V[1], h->V[2], h->P,
                                                                          m0.lhs, L, m0.lay, h->tabs, h->scal, fac);
    h->launches++;
    for (int comp = 0; comp < 3; comp++) {
        if (!h->d3 && comp == 1) continue;
        impose(h, s, h->V[comp], h->bc[comp]);
    }
    impose(h, s, h->P, h->bc[3]);
    if (h->sc) impose(h, s, h->T, h->bc[4]);
    SARAS_CUDA(cudaGetLastError());
    return SARAS_OK;
}

// lsRK3_d3::timeAdvance (lsRK3_d3.cc:190-305): three sub-stages; eulerCN_d3::
// timeAdvance (eulerCN_d3.cc:88-268): one.
saras_status time_advance(saras_rk3 *h, int *mgc, int *cni) {
    const int stages = h->prm.integration == 1 ? 1 : 3;
    for (int rk = 0; rk < stages; rk++) {
        SARAS_TRY(stage_begin(h, rk, cni));
        int nc = 0;
        saras_status st = mg_solve_resident(h->mg, &nc);
        if (mgc) *mgc += nc;
        h->launches += h->mg->last_launches;
        if (st != SARAS_OK && st != SARAS_NOT_CONVERGED) return st;  // mgSolve itself never fails
        SARAS_TRY(stage_end(h, rk));
    }
    return SARAS_OK;
}

// The NTS reductions of the current fields into h->red_host.
saras_status ts_reduce(saras_rk3 *h, const saras_run_params *rp) {
    const HostGrid &g = h->grid;
    const FLay &L = h->L;
    TsPar tp{};
    tp.zg = !(rp->g_axis[2] == 0);
    // tseries::tseries (tseries.cc:105-150): on one rank both walls are ours;
    // wallDn is set by the bottom wall and then by the top wall
    if (tp.zg) {
        const int p2 = g.pad;
        tp.twall = rp->prob_type < 9;
        tp.wall_dn = g.fx[2][(size_t)p2];
        if (tp.twall) tp.wall_dn = g.L[2] - g.fx[2][(size_t)(p2 + g.N[2] - 1)];
    } else {
        const int p0 = g.pad;
        tp.twall = 1;
        tp.wall_dn = g.L[0] - g.fx[0][(size_t)(p0 + g.N[0] - 1)];
    }
    for (int d = 0; d < 3; d++) tp.avg[d] = g.L[d] / g.N[d];
    using TK = void (*)(const double *, const double *, const double *, const double *, FLay, RkTab, RkScal, TsPar,
                        double *);
    static const TK ks[2][2][2] = {
        {{k_tseries<false, false, 1>, k_tseries<false, false, 2>}, {k_tseries<false, true, 1>, k_tseries<false, true, 2>}},
        {{k_tseries<true, false, 1>, k_tseries<true, false, 2>}, {k_tseries<true, true, 1>, k_tseries<true, true, 2>}}};
    cudaStream_t s = h->stream;
    ks[h->d3 ? 1 : 0][h->sc ? 1 : 0][h->ds == 2 ? 1 : 0]<<<h->nblocks, 256, 0, s>>>(
        h->V[0], h->V[1], h->V[2], h->T, L, h->tabs, h->scal, tp, h->part);
    k_tseries_final<<<1, 256, 0, s>>>(h->part, h->nblocks, h->red);
    h->launches += 2;
    SARAS_CUDA(cudaMemcpyAsync(h->red_host, h->red, NTS * sizeof(double), cudaMemcpyDeviceToHost, s));
    SARAS_CUDA(cudaStreamSynchronize(s));
    return SARAS_OK;
}

// tseries::writeTSData(T) / writeTSData() from the reductions (tseries.cc:
// 216-222, 246, 445-450): the totals per volume, Nusselt numbers,
// Reynolds number and the divergence abort test.
saras_status ts_row(saras_rk3 *h, const saras_run_params *rp, double time, double dt, saras_tseries_row *row,
                    double *old_div) {
    SARAS_TRY(ts_reduce(h, rp));
    const HostGrid &g = h->grid;
    const double *r = h->red_host;
    const double divVal = r[TS_DIV];
    const bool abort = divVal > 1e3 && divVal - *old_div > 0;
    *old_div = divVal;
    const double totalVol = h->d3 ? g.L[0] * g.L[1] * g.L[2] : g.L[0] * g.L[2];
    *row = saras_tseries_row{};
    row->time = time;
    row->dt = dt;
    row->divergence = divVal;
    const double ke = r[TS_KE] / totalVol;
    row->ke = ke;
    row->urms = std::sqrt(2.0 * ke);
    if (h->sc) {
        const bool zg = !(rp->g_axis[2] == 0);
        double csArea;
        if (zg) {
            csArea = h->d3 ? g.L[0] * g.L[1] : g.L[0];
            csArea *= rp->prob_type == 9 ? 1 : 2;
        } else {
            csArea = h->d3 ? g.L[1] * g.L[2] : g.L[2];
        }
        row->te = r[TS_TE] / totalVol;
        row->nu_vol = 1.0 + (r[TS_UZT] / totalVol) / h->prm.kappa;
        row->nu_wall = r[TS_DTW] / csArea;
        row->re = std::sqrt(2.0 * ke) / h->prm.nu;
    }
    if (abort) {
        set_error("divergence exceeds permissible limits (%g)", divVal);
        return SARAS_DIVERGED;
    }
    return SARAS_OK;
}

saras_status step_once(saras_rk3 *h, int *mgc, int *cni) { return time_advance(h, mgc, cni); }

// scalar_d3::solvePDE / hydro_d3::solvePDE (scalar_d3.cc:184-262)
saras_status rk3_run(saras_rk3 *h, const saras_run_params *rp, double *time, saras_tseries_row *rows, int cap,
                     int *n_rows, int *n_steps) {
    const double tStp = h->prm.dt;
    double dt = h->prm.dt;
    double old_div = 1.0e10;
    int nr = 0, steps = 0;
    saras_tseries_row row;
    saras_status st = ts_row(h, rp, *time, dt, &row, &old_div);
    if (nr < cap && rows) rows[nr] = row;
    nr++;
    while (st == SARAS_OK) {
        st = step_once(h, nullptr, nullptr);
        if (st != SARAS_OK) break;
        if (rp->use_cfl) {
            st = ts_reduce(h, rp);
            if (st != SARAS_OK) break;
            dt = rp->courant / h->red_host[TS_CFL];
            if (dt > tStp) dt = tStp;
            h->prm.dt = dt;
        }
        steps += 1;
        *time += dt;
        if (steps % rp->io_count == 0) {
            st = ts_row(h, rp, *time, dt, &row, &old_div);
            if (nr < cap && rows) rows[nr] = row;
            nr++;
            if (st != SARAS_OK) break;
        }
        if (std::fabs(rp->t_max - *time) < 0.5 * dt) break;
        if (rp->max_steps > 0 && steps >= rp->max_steps) break;
    }
    if (n_rows) *n_rows = nr;
    if (n_steps) *n_steps = steps;
    return st;
}

saras_status check_params(const saras_grid_desc *gd, const saras_rk3_params *p) {
    if (gd->pad != 1 && gd->pad != 2) {
        set_error("the time step takes Differentiation Scheme 1 (pad 1) or 2 (pad 2)");
        return SARAS_BAD_ARG;
    }
    if (p->nl_scheme < 1 || p->nl_scheme > 3 || p->integration < 0 || p->integration > 2 || !(p->dt > 0.0) ||
        !(p->nu >= 0.0) || !(p->kappa >= 0.0) || p->max_iterations < 0 ||
        (p->stencil_form != SARAS_STENCIL_EXACT && p->stencil_form != SARAS_STENCIL_FAST)) {
        set_error("invalid time-step parameters");
        return SARAS_BAD_ARG;
    }
    return SARAS_OK;
}

// Everything of a handle that follows the grid's stretching and the
// parameters: metric tables (h->tab already allocated), derivative and
// upwind constants, boundary constants, the CN iteration cap.
saras_status rk3_configure(saras_rk3 *h, const saras_grid_desc *gd, const saras_rk3_params *p) {
    h->prm = *p;
    SARAS_TRY(h->grid.build(*gd, p->mg.levels));
    h->d3 = h->grid.dims == 3;
    h->sc = p->with_scalar != 0;
    h->ds = gd->pad;
    const HostGrid &g = h->grid;
    // metric tables: xi_x, xixx, xix2, a2, a1, dh, dv, xc per axis over the
    // core, and the FAST form's k1, k2a, k2b
    constexpr int NT = RK_TABLES;
    const int n[3] = {h->L.n0, h->L.n1, h->L.n2};
    const int64_t tot = NT * (int64_t)(n[0] + n[1] + n[2]);
    std::vector<double> host((size_t)tot, 0.0);
    int64_t off = 0;
    for (int d = 0; d < 3; d++) {
        const int p0 = (g.dims == 2 && d == 1) ? 1 : g.pad;
        double ih = 1.0 / g.dxi[d];
        h->scal.ih[d] = ih;
        h->scal.ih2d[d] = std::pow(ih, 2.0);
        const double hx2 = std::pow(g.dxi[d], 2.0);
        h->scal.i2ht[d] = 0.5 / g.dxi[d];
        h->scal.i2d[d] = 1.0 / (2.0 * g.dxi[d]);
        h->scal.ih2t[d] = 1.0 / hx2;
        double *dst[NT];
        for (int q = 0; q < NT; q++) dst[q] = h->tab + off + (int64_t)q * n[d];
        h->tabs.xi_x[d] = dst[0];
        h->tabs.xixx[d] = dst[1];
        h->tabs.xix2[d] = dst[2];
        h->tabs.a2[d] = dst[3];
        h->tabs.a1[d] = dst[4];
        h->tabs.dh[d] = dst[5];
        h->tabs.dv[d] = dst[6];
        h->tabs.xc[d] = dst[7];
        h->tabs.k1[d] = dst[8];
        h->tabs.k2a[d] = dst[9];
        h->tabs.k2b[d] = dst[10];
        for (int i = 0; i < n[d]; i++) {
            const size_t q = (size_t)(i + p0);
            const double v[NT] = {g.fxi_x[d][q],
                                  g.fxixx[d][q],
                                  g.fxix2[d][q],
                                  h->scal.ih2t[d] * g.fxix2[d][q],
                                  h->scal.i2ht[d] * g.fxixx[d][q],
                                  g.fx[d][q + 1] - g.fx[d][q],
                                  g.dxi[d] / g.fxi_x[d][q],
                                  g.fx[d][q],
                                  g.fxi_x[d][q] * (0.5 * ih),
                                  g.fxixx[d][q] * (0.5 * ih),
                                  g.fxix2[d][q] * h->scal.ih2d[d]};
            for (int qq = 0; qq < NT; qq++) host[(size_t)(off + (int64_t)qq * n[d] + i)] = v[qq];
        }
        off += NT * (int64_t)n[d];
    }
    // pageable source: staged before the call returns, ordered on the stream
    SARAS_CUDA(cudaMemcpyAsync(h->tab, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    // vfield::vfield / sfield::sfield (vfield.cc:107-130): first-order
    // upwinding for dScheme 1, omega = "Central Bias"
    const double omega = p->up_param;
    h->scal.ud = 0.0;
    if (h->ds == 1) {
        h->scal.ua = 2.0 - omega;
        h->scal.ub = 2.0 * (1.0 - omega);
        h->scal.uc = -omega;
    } else {
        h->scal.ua = 1.0 - omega;
        h->scal.ub = 4.0 - 3.0 * omega;
        h->scal.uc = 3.0 * (1.0 - omega);
        h->scal.ud = -omega;
    }
    h->scal.pe_limit = p->pe_limit;
    h->scal.dc_v = p->nu;
    h->scal.dc_t = p->kappa;
    h->bc[0] = make_fbc(h, p->bc_vx);
    h->bc[1] = make_fbc(h, p->bc_vy);
    h->bc[2] = make_fbc(h, p->bc_vz);
    h->bc[3] = make_fbc(h, p->bc_p);
    h->bc[4] = make_fbc(h, p->bc_t);
    // timestep::timestep (timestep.cc:115): int(pow(log(Nx*Ny*Nz), 3))
    h->max_iterations = p->max_iterations > 0 ? p->max_iterations
                                              : int(std::pow(std::log(g.N[0] * g.N[1] * g.N[2]), 3));
    return SARAS_OK;
}

saras_status rk3_create(const saras_grid_desc *gd, const saras_rk3_params *p, void *stream, saras_rk3 *h) {
    SARAS_TRY(check_params(gd, p));
    HostGrid g;
    SARAS_TRY(g.build(*gd, p->mg.levels));
    const bool d3 = g.dims == 3;
    h->stream = (cudaStream_t)stream;
    SARAS_TRY(saras_mg_create(gd, &p->mg, stream, &h->mg));
    h->L = make_flay(g.N[0], d3 ? g.N[1] : 1, g.N[2], g.pad, d3 ? g.pad : 1);
    const int64_t sz = h->L.size;
    for (int d = 0; d < 3; d++) {
        SARAS_TRY(rk_alloc(h, &h->V[d], sz));
        SARAS_TRY(rk_alloc(h, &h->Vb[d], sz));
        SARAS_TRY(rk_alloc(h, &h->nse[d], sz));
        SARAS_TRY(rk_alloc(h, &h->nl[d], sz));
    }
    SARAS_TRY(rk_alloc(h, &h->P, sz));
    SARAS_TRY(rk_alloc(h, &h->T, sz));
    SARAS_TRY(rk_alloc(h, &h->Tb, sz));
    SARAS_TRY(rk_alloc(h, &h->tmpR, sz));
    SARAS_TRY(rk_alloc(h, &h->nlT, sz));
    h->nfields = (int)h->allocs.size();
    for (double *q : h->allocs) SARAS_CUDA(cudaMemsetAsync(q, 0, (size_t)sz * sizeof(double), h->stream));
    const int n[3] = {h->L.n0, h->L.n1, h->L.n2};
    SARAS_TRY(rk_alloc(h, &h->tab, RK_TABLES * (int64_t)(n[0] + n[1] + n[2])));
    SARAS_TRY(rk3_configure(h, gd, p));
    const int64_t cells = (int64_t)n[0] * n[1] * n[2];
    h->nblocks = (int)std::max<int64_t>(1, std::min<int64_t>(1216, (cells + 255) / 256));
    SARAS_TRY(rk_alloc(h, &h->part, (int64_t)h->nblocks * NTS));
    SARAS_TRY(rk_alloc(h, &h->red, NTS));
    SARAS_CUDA(cudaMallocHost((void **)&h->red_host, NTS * sizeof(double)));
    // dense host box of a field: core plus pad (1 on y for the planar case)
    const int px = h->L.p, py = h->L.py;
    h->bst[2] = 1;
    h->bst[1] = n[2] + 2 * px;
    h->bst[0] = h->bst[1] * (n[1] + 2 * py);
    h->box_elems = h->bst[0] * (n[0] + 2 * px);
    SARAS_TRY(rk_alloc(h, &h->stage, h->box_elems));
    SARAS_CUDA(cudaStreamSynchronize(h->stream));
    return SARAS_OK;
}

void rk3_free(saras_rk3 *h) {
    for (double *p : h->allocs) cudaFree(p);
    if (h->red_host) cudaFreeHost(h->red_host);
    if (h->mg) saras_mg_destroy(h->mg);
}

// Host box <-> device field.  Fields in the time-step layout move over their
// whole padded box; the pressure correction lives in the multigrid level
// layout (one ghost layer), so only its core and first ghost layer move and
// the host's outer layer is left as it was.
saras_status box_transfer(saras_rk3 *h, double *field, bool level_layout, const double *src_host,
                          double *dst_host, const int64_t st[3]) {
    for (int d = 0; d < 3; d++)
        if (st[d] != h->bst[d]) {
            set_error("time-step fields must be C-contiguous padded arrays");
            return SARAS_BAD_ARG;
        }
    cudaStream_t s = h->stream;
    const FLay &L = h->L;
    const int64_t origin = L.p * h->bst[0] + L.py * h->bst[1] + L.p;
    const size_t bytes = (size_t)h->box_elems * sizeof(double);
    const int qx = level_layout ? 1 : L.p, qy = level_layout ? 1 : L.py;
    const int bx = bxfor(L.n2 + 2 * qx);
    const dim3 g(cdiv(L.n2 + 2 * qx, bx), (unsigned)(L.n1 + 2 * qy), (unsigned)(L.n0 + 2 * qx));
    const Lay &LM = h->mg->lv[0].lay;
    if (src_host) {
        SARAS_CUDA(cudaMemcpyAsync(h->stage, src_host - origin, bytes, cudaMemcpyHostToDevice, s));
        if (level_layout)
            k_box_in<<<g, bx, 0, s>>>(h->stage + origin, h->bst[0], h->bst[1], field, LM, qx, qy);
        else
            k_box_in<<<g, bx, 0, s>>>(h->stage + origin, h->bst[0], h->bst[1], field, L, qx, qy);
    } else {
        if (level_layout && L.p > 1) {
            // keep the host's second ghost layer: stage the host box first
            SARAS_CUDA(cudaMemcpyAsync(h->stage, dst_host - origin, bytes, cudaMemcpyHostToDevice, s));
        }
        if (level_layout)
            k_box_out<<<g, bx, 0, s>>>(field, LM, h->stage + origin, h->bst[0], h->bst[1], qx, qy);
        else
            k_box_out<<<g, bx, 0, s>>>(field, L, h->stage + origin, h->bst[0], h->bst[1], qx, qy);
        SARAS_CUDA(cudaMemcpyAsync(dst_host - origin, h->stage, bytes, cudaMemcpyDeviceToHost, s));
    }
    SARAS_CUDA(cudaStreamSynchronize(s));
    return SARAS_OK;
}

}  // namespace

namespace saras {

int rk3_stages(const saras_rk3 *h) { return h->prm.integration == 1 ? 1 : 3; }
saras_status rk3_stage_begin(saras_rk3 *h, int stage) { return stage_begin(h, stage, nullptr); }
saras_status rk3_stage_end(saras_rk3 *h, int stage) { return stage_end(h, stage); }
saras_mg *rk3_multigrid(saras_rk3 *h) { return h->mg; }
int64_t rk3_device_bytes(const saras_rk3 *h) { return h->dev_bytes; }

saras_status rk3_retarget(saras_rk3 *h, const saras_grid_desc *gd, const saras_rk3_params *p) {
    SARAS_TRY(check_params(gd, p));
    const HostGrid &o = h->grid;
    bool same = gd->dims == o.dims && gd->pad == o.pad && p->mg.levels == h->prm.mg.levels;
    for (int d = 0; d < 3; d++) same = same && gd->n[d] == o.N[d] && (gd->periodic[d] != 0) == o.per[d];
    if (!same) {
        set_error("a time-step handle is re-pointed only at a grid of its own shape");
        return SARAS_BAD_ARG;
    }
    SARAS_TRY(mg_retarget(h->mg, gd));
    h->mg->prm.vc_count = p->mg.vc_count;
    h->mg->prm.vc_tolerance = p->mg.vc_tolerance;
    SARAS_TRY(rk3_configure(h, gd, p));
    for (int q = 0; q < h->nfields; q++)
        SARAS_CUDA(cudaMemsetAsync(h->allocs[(size_t)q], 0, (size_t)h->L.size * sizeof(double), h->stream));
    return SARAS_OK;
}

int64_t rk3_estimate_bytes(const saras_grid_desc *gd, const saras_rk3_params *prm) {
    const bool d3 = gd->dims == 3;
    const FLay L = make_flay(gd->n[0], d3 ? gd->n[1] : 1, gd->n[2], gd->pad, d3 ? gd->pad : 1);
    const int64_t box = (int64_t)(gd->n[0] + 2 * L.p) * ((d3 ? gd->n[1] : 1) + 2 * L.py) * (gd->n[2] + 2 * L.p);
    const int64_t tabs = 8 * (int64_t)(gd->n[0] + gd->n[1] + gd->n[2]) + 1216 * NTS + NTS;
    return (17 * L.size + box + tabs) * (int64_t)sizeof(double) + mg_estimate_bytes(gd, &prm->mg);
}

}  // namespace saras

extern "C" {

saras_status saras_rk3_create(const saras_grid_desc *grid, const saras_rk3_params *prm, void *stream,
                              saras_rk3 **out) {
    if (!grid || !prm || !out) {
        set_error("null argument");
        return SARAS_BAD_ARG;
    }
    *out = nullptr;
    saras_rk3 *h = new saras_rk3();
    saras_status s = rk3_create(grid, prm, stream, h);
    if (s != SARAS_OK) {
        rk3_free(h);
        delete h;
        return s;
    }
    *out = h;
    return SARAS_OK;
}

saras_status saras_rk3_upload(saras_rk3 *h, const double *vx, const double *vy, const double *vz, const double *p,
                              const double *t, const double *pp, const int64_t strides[3]) {
    if (!h || !strides) return SARAS_BAD_ARG;
    const double *src[6] = {vx, vy, vz, p, t, pp};
    double *dst[6] = {h->V[0], h->V[1], h->V[2], h->P, h->T, h->mg->lv[0].lhs};
    for (int q = 0; q < 6; q++) {
        if (!src[q] || (q == 1 && !h->d3) || (q == 4 && !h->sc)) continue;
        SARAS_TRY(box_transfer(h, dst[q], q == 5, src[q], nullptr, strides));
    }
    return SARAS_OK;
}

saras_status saras_rk3_download(saras_rk3 *h, double *vx, double *vy, double *vz, double *p, double *t, double *pp,
                                const int64_t strides[3]) {
    if (!h || !strides) return SARAS_BAD_ARG;
    double *dst[6] = {vx, vy, vz, p, t, pp};
    double *src[6] = {h->V[0], h->V[1], h->V[2], h->P, h->T, h->mg->lv[0].lhs};
    for (int q = 0; q < 6; q++) {
        if (!dst[q] || (q == 1 && !h->d3) || (q == 4 && !h->sc)) continue;
        SARAS_TRY(box_transfer(h, src[q], q == 5, nullptr, dst[q], strides));
    }
    return SARAS_OK;
}

saras_status saras_rk3_step(saras_rk3 *h, int32_t nsteps, int32_t *mg_cycles, int32_t *cn_iters) {
    if (!h || nsteps < 0) return SARAS_BAD_ARG;
    int mgc = 0, cni = 0;
    h->launches = 0;
    saras_status st = SARAS_OK;
    for (int n = 0; n < nsteps && st == SARAS_OK; n++)
        st = time_advance(h, &mgc, &cni);
    if (mg_cycles) *mg_cycles = mgc;
    if (cn_iters) *cn_iters = cni;
    return st;
}

saras_status saras_rk3_destroy(saras_rk3 *h) {
    if (!h) return SARAS_OK;
    cudaStreamSynchronize(h->stream);
    rk3_free(h);
    delete h;
    return SARAS_OK;
}

int64_t saras_rk3_last_launches(const saras_rk3 *h) { return h ? h->launches : -1; }

saras_status saras_rk3_tseries(saras_rk3 *h, const saras_run_params *rp, double time, saras_tseries_row *row) {
    if (!h || !rp || !row) return SARAS_BAD_ARG;
    double old_div = 1.0e10;
    h->launches = 0;
    return ts_row(h, rp, time, h->prm.dt, row, &old_div);
}

saras_status saras_rk3_cfl_dt(saras_rk3 *h, double courant, double *dt) {
    if (!h || !dt) return SARAS_BAD_ARG;
    saras_run_params rp{};
    rp.g_axis[2] = -1.0;
    h->launches = 0;
    SARAS_TRY(ts_reduce(h, &rp));
    *dt = courant / h->red_host[TS_CFL];
    return SARAS_OK;
}

saras_status saras_rk3_run(saras_rk3 *h, const saras_run_params *rp, double *time, saras_tseries_row *rows,
                           int32_t row_cap, int32_t *n_rows, int32_t *n_steps) {
    if (!h || !rp || !time || row_cap < 0 || rp->io_count < 1 || (rp->use_cfl && !(rp->courant > 0.0))) {
        set_error("invalid time-loop parameters");
        return SARAS_BAD_ARG;
    }
    h->launches = 0;
    int nr = 0, ns = 0;
    saras_status st = rk3_run(h, rp, time, rows, row_cap, &nr, &ns);
    if (n_rows) *n_rows = nr;
    if (n_steps) *n_steps = ns;
    return st;
}

}  // extern "C"
