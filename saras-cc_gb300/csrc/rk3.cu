// Low-storage RK3 time step of SARAS on GB300: the sub-step stencils around
// the pressure-Poisson solve, one fused kernel per stage of the reference's
// sequence of full-array Blitz operations.
//
// Reference: lsRK3_d3::timeAdvance(V,P,T) and (V,P) (lib/timestep/
// lsRK3_d3.cc:94-177, 190-305; lsRK3_d2.cc), timestep::solveVx/Vy/Vz/T
// (lib/timestep/predictors.cc:59-423), vfield/sfield::computeDiff,
// computeNLin (nlScheme 1 and 3, Morinishi's second-order branch),
// divergence, gradient (lib/field/vfield.cc,
// sfield.cc, plainsf.cc), derivative::calcDerivative1_* / 2** with
// dScheme 1 (lib/field/derivative.cc:104-318), field BC writers
// (lib/boundary/dirichlet.cc, neumann.cc) and buoyantForce::addForcing
// (lib/force/buoyantForce.cc:64-69).
//
// Every per-cell value is formed in the reference's operation order with
// separately rounded FP64 operations, so one step is bit-identical to the
// single-rank reference arithmetic (given the same multigrid form).  The
// Blitz stencils are taken as central12n = (F[+1]-F[-1])*0.5 and
// central22n = (F[-1]-2F)+F[+1].
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <math_constants.h>

#include "mg_handle.cuh"

namespace saras {
saras_status mg_solve_resident(saras_mg *h, int32_t *n_cycles);
}

using namespace saras;

namespace {

constexpr int BX = 128;

// Per-axis finest-level metric tables over core indices and scalars.
struct RkTab {
    const double *xi_x[3], *xixx[3], *xix2[3];
    const double *a2[3], *a1[3];  // ihx2*xix2, i2hx*xixx (timestep coefficients)
};
struct RkScal {
    double ih[3], ih2d[3];  // derivative: 1/dXi, pow(1/dXi, 2)
    double ih2t[3], i2ht[3]; // timestep: 1/pow(dXi,2), 0.5/dXi
    double i2d[3];           // vfield/sfield: 1/(2 dXi) (vfield.cc:133-135)
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
    double zeta, anu, akap, ab, gam, dt;
    double g[3];
};

__device__ __forceinline__ int64_t axis_stride(const Lay &L, int a) { return a == 0 ? L.s0 : (a == 1 ? L.s1 : 1); }

// calcDerivative1 (derivative.cc:104-204): xi_x * ((F+ - F-) * 0.5 * ihx)
__device__ __forceinline__ double d1(const double *F, const Lay &L, const RkTab &T, const RkScal &S, int a,
                                     int idx, int64_t c) {
    const int64_t st = axis_stride(L, a);
    const double c12 = rmul(rsub(F[c + st], F[c - st]), 0.5);
    return rmul(T.xi_x[a][idx], rmul(c12, S.ih[a]));
}

// calcDerivative2 (derivative.cc:206-318): xixx*(c12*ihx) + xix2*(c22*ihx2)
__device__ __forceinline__ double d2(const double *F, const Lay &L, const RkTab &T, const RkScal &S, int a,
                                     int idx, int64_t c) {
    const int64_t st = axis_stride(L, a);
    const double fp = F[c + st], fm = F[c - st];
    const double c12 = rmul(rsub(fp, fm), 0.5);
    const double c22 = radd(rsub(fm, rmul(2.0, F[c])), fp);
    return radd(rmul(T.xixx[a][idx], rmul(c12, S.ih[a])), rmul(T.xix2[a][idx], rmul(c22, S.ih2d[a])));
}

// One direction of Morinishi's skew-symmetric convection term, second-order
// branch (dScheme 1; vfield.cc:271-474, sfield.cc:200-323):
// (adv + div)/2 with adv = Va*xi*(F+ - F-)*i2d and div = xi*(Va+ F+ - Va- F-)*i2d,
// the products standing for the Blitz temporaries tempXX = V.Vx*Vx etc.
__device__ __forceinline__ double mterm(const double *F, const double *Va, const Lay &L, const RkTab &T,
                                        const RkScal &S, int a, int idx, int64_t c) {
    const int64_t st = axis_stride(L, a);
    const double x = T.xi_x[a][idx];
    const double adv = rmul(rmul(rmul(Va[c], x), rsub(F[c + st], F[c - st])), S.i2d[a]);
    const double div = rmul(rmul(x, rsub(rmul(Va[c + st], F[c + st]), rmul(Va[c - st], F[c - st]))), S.i2d[a]);
    return rdiv(radd(adv, div), 2.0);
}

struct Fields {
    const double *V[3];
    const double *P, *T;
    double *nse[3], *nl[3];
    double *tmpR, *nlT;
};

// Right-hand sides of one RK3 sub-stage for every velocity component and T
// (lsRK3_d3.cc:199-252): zeta*NL_prev + alpha*nu*Diff + (alpha+beta)*(F - grad P)
// + gamma*NL, times dt, plus the field.  NL is kept for the next stage.
template <bool D3, bool SC, int NLS>
__global__ void k_rk3_rhs(Fields f, Lay L, RkTab T, RkScal S, Stage sg) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = D3 ? (int)blockIdx.y : 0;
    const int i = blockIdx.z;
    if (k >= L.n2) return;
    const int64_t c = L.at(i, j, k);
    const int id[3] = {i, j, k};
    for (int comp = 0; comp < 3; comp++) {
        if (!D3 && comp == 1) continue;
        const double *F = f.V[comp];
        double r = 0.0;
        if (sg.rk > 0) r = radd(r, rmul(sg.zeta, f.nl[comp][c]));
        double dif = radd(0.0, d2(F, L, T, S, 0, i, c));
        if (D3) dif = radd(dif, d2(F, L, T, S, 1, j, c));
        dif = radd(dif, d2(F, L, T, S, 2, k, c));
        r = radd(r, rmul(sg.anu, dif));
        double t = 0.0;
        if (SC) t = rsub(t, rmul(sg.g[comp], f.T[c]));
        t = rsub(t, d1(f.P, L, T, S, comp, id[comp], c));
        r = radd(r, rmul(sg.ab, t));
        double n;
        if (NLS == 3) {
            n = rsub(0.0, mterm(F, f.V[0], L, T, S, 0, i, c));
            if (D3) n = rsub(n, mterm(F, f.V[1], L, T, S, 1, j, c));
            n = rsub(n, mterm(F, f.V[2], L, T, S, 2, k, c));
        } else {
            n = rsub(0.0, rmul(f.V[0][c], d1(F, L, T, S, 0, i, c)));
            if (D3) n = rsub(n, rmul(f.V[1][c], d1(F, L, T, S, 1, j, c)));
            n = rsub(n, rmul(f.V[2][c], d1(F, L, T, S, 2, k, c)));
        }
        r = radd(r, rmul(sg.gam, n));
        r = rmul(r, sg.dt);
        r = radd(r, F[c]);
        f.nse[comp][c] = r;
        f.nl[comp][c] = n;
    }
    if (SC) {
        const double *F = f.T;
        double r = 0.0;
        if (sg.rk > 0) r = radd(r, rmul(sg.zeta, f.nlT[c]));
        double dif = radd(0.0, d2(F, L, T, S, 0, i, c));
        if (D3) dif = radd(dif, d2(F, L, T, S, 1, j, c));
        dif = radd(dif, d2(F, L, T, S, 2, k, c));
        r = radd(r, rmul(sg.akap, dif));
        r = radd(r, rmul(sg.ab, 0.0));  // zeroForcing adds nothing, multAdd still runs
        double n;
        if (NLS == 3) {
            n = rsub(0.0, mterm(F, f.V[0], L, T, S, 0, i, c));
            if (D3) n = rsub(n, mterm(F, f.V[1], L, T, S, 1, j, c));
            n = rsub(n, mterm(F, f.V[2], L, T, S, 2, k, c));
        } else {
            n = rsub(0.0, rmul(f.V[0][c], d1(F, L, T, S, 0, i, c)));
            if (D3) n = rsub(n, rmul(f.V[1][c], d1(F, L, T, S, 1, j, c)));
            n = rsub(n, rmul(f.V[2][c], d1(F, L, T, S, 2, k, c)));
        }
        r = radd(r, rmul(sg.gam, n));
        r = rmul(r, sg.dt);
        r = radd(r, F[c]);
        f.tmpR[c] = r;
        f.nlT[c] = n;
    }
}

// One Jacobi sweep of (1 - beta*dt*coef*L) u = rhs (predictors.cc:65-91).
template <bool D3>
__global__ void k_cn_jacobi(const double *__restrict__ F, const double *__restrict__ R, double *__restrict__ out,
                            Lay L, RkTab T, double dt, double coef, double beta, double den_fac) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = D3 ? (int)blockIdx.y : 0;
    const int i = blockIdx.z;
    if (k >= L.n2) return;
    const int64_t c = L.at(i, j, k);
    const double xp = F[c + L.s0], xm = F[c - L.s0], zp = F[c + 1], zm = F[c - 1];
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
template <bool D3>
__global__ void k_cn_resid(const double *__restrict__ F, const double *__restrict__ R, Lay L, RkTab T, RkScal S,
                           double bdc, double *__restrict__ part) {
    double m = 0.0;
    for_core_rows(L, [&](int i, int j, int k) {
        const int64_t c = L.at(i, j, k);
        const double u = F[c], u2 = rmul(2.0, u);
        const double xp = F[c + L.s0], xm = F[c - L.s0], zp = F[c + 1], zm = F[c - 1];
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

// Ghost planes of a field (field::syncFaces then the wall BC writers).
__global__ void k_fbc(double *u, Lay L, FBC B, int axis, int wall_pass, int a_lo, int b_lo, int b_cnt) {
    const int b = b_lo + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int a = a_lo + (int)blockIdx.y;
    if (b >= b_lo + b_cnt) return;
    const int n[3] = {L.n0, L.n1, L.n2};
    int lo[3], hi[3], in0[3], in1[3];
    const int o0 = axis == 0 ? 1 : 0, o1 = axis == 2 ? 1 : 2;
    lo[axis] = -1;
    hi[axis] = n[axis];
    in0[axis] = 0;
    in1[axis] = n[axis] - 1;
    lo[o0] = hi[o0] = in0[o0] = in1[o0] = a;
    lo[o1] = hi[o1] = in0[o1] = in1[o1] = b;
    const int64_t glo = L.at(lo[0], lo[1], lo[2]), ghi = L.at(hi[0], hi[1], hi[2]);
    const int64_t ilo = L.at(in0[0], in0[1], in0[2]), ihi = L.at(in1[0], in1[1], in1[2]);
    if (!wall_pass) {
        u[ghi] = u[ilo];
        u[glo] = u[ihi];
        return;
    }
    const int f0 = 2 * axis, f1 = 2 * axis + 1;
    u[glo] = B.type[f0] == SARAS_FBC_DIRICHLET ? rsub(B.two_v[f0], u[ilo]) : rsub(u[ilo], B.kh[f0]);
    u[ghi] = B.type[f1] == SARAS_FBC_DIRICHLET ? rsub(B.two_v[f1], u[ihi]) : rsub(u[ihi], B.kh[f1]);
}

// divergence of V into the multigrid RHS, scaled (lsRK3_d3.cc:272-276).
template <bool D3>
__global__ void k_divergence(const double *__restrict__ vx, const double *__restrict__ vy,
                             const double *__restrict__ vz, double *__restrict__ out, Lay L, RkTab T, RkScal S,
                             double scale) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = D3 ? (int)blockIdx.y : 0;
    const int i = blockIdx.z;
    if (k >= L.n2) return;
    const int64_t c = L.at(i, j, k);
    double d = radd(0.0, d1(vx, L, T, S, 0, i, c));
    if (D3) d = radd(d, d1(vy, L, T, S, 1, j, c));
    d = radd(d, d1(vz, L, T, S, 2, k, c));
    out[c] = rmul(d, scale);
}

// P += Pp; V -= (alpha+beta) dt grad Pp (lsRK3_d3.cc:281-294).
template <bool D3>
__global__ void k_correct(double *__restrict__ vx, double *__restrict__ vy, double *__restrict__ vz,
                          double *__restrict__ p, const double *__restrict__ pp, Lay L, RkTab T, RkScal S,
                          double fac) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = D3 ? (int)blockIdx.y : 0;
    const int i = blockIdx.z;
    if (k >= L.n2) return;
    const int64_t c = L.at(i, j, k);
    p[c] = radd(p[c], pp[c]);
    vx[c] = rsub(vx[c], rmul(d1(pp, L, T, S, 0, i, c), fac));
    if (D3) vy[c] = rsub(vy[c], rmul(d1(pp, L, T, S, 1, j, c), fac));
    vz[c] = rsub(vz[c], rmul(d1(pp, L, T, S, 2, k, c), fac));
}

// Dense padded box <-> level layout (full box including the ghost layer).
__global__ void k_box_in(const double *__restrict__ src, int64_t s0, int64_t s1, double *__restrict__ dst, Lay L,
                         int jlo, int jhi) {
    const int k = (int)(blockIdx.x * blockDim.x + threadIdx.x) - 1;
    const int j = jlo + (int)blockIdx.y, i = (int)blockIdx.z - 1;
    if (k > L.n2 || j > jhi) return;
    dst[L.at(i, j, k)] = src[(int64_t)i * s0 + (int64_t)j * s1 + k];
}
__global__ void k_box_out(const double *__restrict__ src, Lay L, double *__restrict__ dst, int64_t s0, int64_t s1,
                          int jlo, int jhi) {
    const int k = (int)(blockIdx.x * blockDim.x + threadIdx.x) - 1;
    const int j = jlo + (int)blockIdx.y, i = (int)blockIdx.z - 1;
    if (k > L.n2 || j > jhi) return;
    dst[(int64_t)i * s0 + (int64_t)j * s1 + k] = src[L.at(i, j, k)];
}

}  // namespace

struct saras_rk3 {
    HostGrid grid;
    saras_rk3_params prm{};
    bool d3 = true;
    bool sc = true;
    cudaStream_t stream = nullptr;
    saras_mg *mg = nullptr;
    Lay L{};
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
    std::vector<double *> allocs;
};

namespace {

inline int bxfor(int n) { return std::min(BX, (n + 31) / 32 * 32); }

saras_status rk_alloc(saras_rk3 *h, double **p, int64_t n) {
    cudaError_t e = cudaMalloc((void **)p, (size_t)std::max<int64_t>(n, 1) * sizeof(double));
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("cudaMalloc failed in the RK3 integrator: %s", cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? SARAS_OOM : SARAS_CUDA_ERR;
    }
    h->allocs.push_back(*p);
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

// field::syncFaces then the wall writers, x, y, z (sfield.cc:520-547).
void impose(saras_rk3 *h, cudaStream_t s, double *u, const FBC &B) {
    const Lay &L = h->L;
    for (int pass = 0; pass < 2; pass++) {
        for (int axis = 0; axis < 3; axis++) {
            if (!h->d3 && axis == 1) continue;
            if ((pass == 0) != (bool)B.per[axis]) continue;
            const int n[3] = {L.n0, L.n1, L.n2};
            const int o0 = axis == 0 ? 1 : 0, o1 = axis == 2 ? 1 : 2;
            const int acnt = n[o0] + 2, bcnt = n[o1] + 2;
            const int bx = bxfor(bcnt);
            k_fbc<<<dim3(cdiv(bcnt, bx), (unsigned)acnt), bx, 0, s>>>(u, L, B, axis, pass, -1, -1, bcnt);
            h->launches++;
        }
    }
}

dim3 cgrid(const Lay &L, bool d3, int bx) { return dim3(cdiv(L.n2, bx), d3 ? (unsigned)L.n1 : 1u, (unsigned)L.n0); }

saras_status cn_solve(saras_rk3 *h, cudaStream_t s, int comp, const double *rhs, double coef, double beta,
                      int *iters) {
    const Lay &L = h->L;
    const int bx = bxfor(L.n2);
    const double dt = h->prm.dt;
    const double den_fac = 2.0 * dt * coef * beta;  // 2.0 * dt * nu * beta, left to right
    const double bdc = beta * dt * coef;            // beta * dt * nu, left to right
    double **cur = comp < 3 ? &h->V[comp] : &h->T;
    double **alt = comp < 3 ? &h->Vb[comp] : &h->Tb;
    const FBC &B = h->bc[comp < 3 ? comp : 4];
    int iterCount = 0;
    for (;;) {
        if (h->d3)
            k_cn_jacobi<true><<<cgrid(L, true, bx), bx, 0, s>>>(*cur, rhs, *alt, L, h->tabs, dt, coef, beta, den_fac);
        else
            k_cn_jacobi<false><<<cgrid(L, false, bx), bx, 0, s>>>(*cur, rhs, *alt, L, h->tabs, dt, coef, beta,
                                                                   den_fac);
        h->launches++;
        std::swap(*cur, *alt);
        impose(h, s, *cur, B);
        if (h->d3)
            k_cn_resid<true><<<h->nblocks, 256, 0, s>>>(*cur, rhs, L, h->tabs, h->scal, bdc, h->part);
        else
            k_cn_resid<false><<<h->nblocks, 256, 0, s>>>(*cur, rhs, L, h->tabs, h->scal, bdc, h->part);
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

// lsRK3_d3::timeAdvance (lsRK3_d3.cc:190-305)
saras_status time_advance(saras_rk3 *h, int *mgc, int *cni) {
    static const double alph[3] = {4.0 / 15.0, 1.0 / 15.0, 1.0 / 6.0};
    static const double bet[3] = {4.0 / 15.0, 1.0 / 15.0, 1.0 / 6.0};
    static const double gam[3] = {8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};
    static const double zet[3] = {0.0, -17.0 / 60.0, -5.0 / 12.0};
    cudaStream_t s = h->stream;
    const Lay &L = h->L;
    const int bx = bxfor(L.n2);
    const double nu = h->prm.nu, kappa = h->prm.kappa, dt = h->prm.dt;
    Level &m0 = h->mg->lv[0];
    for (int rk = 0; rk < 3; rk++) {
        Stage sg;
        sg.rk = rk;
        sg.zeta = zet[rk];
        sg.anu = alph[rk] * nu;
        sg.akap = alph[rk] * kappa;
        sg.ab = alph[rk] + bet[rk];
        sg.gam = gam[rk];
        sg.dt = dt;
        for (int d = 0; d < 3; d++) sg.g[d] = h->prm.g_terms[d];
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
        const dim3 g = cgrid(L, h->d3, bx);
        {
            // (dimension, scalar, non-linear scheme) -> kernel
            using K = void (*)(Fields, Lay, RkTab, RkScal, Stage);
            const K ks[2][2][2] = {{{k_rk3_rhs<false, false, 1>, k_rk3_rhs<false, false, 3>},
                                    {k_rk3_rhs<false, true, 1>, k_rk3_rhs<false, true, 3>}},
                                   {{k_rk3_rhs<true, false, 1>, k_rk3_rhs<true, false, 3>},
                                    {k_rk3_rhs<true, true, 1>, k_rk3_rhs<true, true, 3>}}};
            ks[h->d3 ? 1 : 0][h->sc ? 1 : 0][h->prm.nl_scheme == 3 ? 1 : 0]<<<g, bx, 0, s>>>(f, L, h->tabs, h->scal,
                                                                                          sg);
        }
        h->launches++;
        for (int comp = 0; comp < 3; comp++) {
            if (!h->d3 && comp == 1) continue;
            SARAS_TRY(cn_solve(h, s, comp, h->nse[comp], nu, bet[rk], cni));
        }
        if (h->sc) SARAS_TRY(cn_solve(h, s, 3, h->tmpR, kappa, bet[rk], cni));
        const double scale = 1.0 / ((alph[rk] + bet[rk]) * dt);
        if (h->d3)
            k_divergence<true><<<g, bx, 0, s>>>(h->V[0], h->V[1], h->V[2], m0.rhs, L, h->tabs, h->scal, scale);
        else
            k_divergence<false><<<g, bx, 0, s>>>(h->V[0], h->V[1], h->V[2], m0.rhs, L, h->tabs, h->scal, scale);
        h->launches++;
        int nc = 0;
        saras_status st = mg_solve_resident(h->mg, &nc);
        if (mgc) *mgc += nc;
        h->launches += h->mg->last_launches;
        if (st != SARAS_OK && st != SARAS_NOT_CONVERGED) return st;  // mgSolve itself never fails
        const double fac = (alph[rk] + bet[rk]) * dt;
        if (h->d3)
            k_correct<true><<<g, bx, 0, s>>>(h->V[0], h->V[1], h->V[2], h->P, m0.lhs, L, h->tabs, h->scal, fac);
        else
            k_correct<false><<<g, bx, 0, s>>>(h->V[0], h->V[1], h->V[2], h->P, m0.lhs, L, h->tabs, h->scal, fac);
        h->launches++;
        for (int comp = 0; comp < 3; comp++) {
            if (!h->d3 && comp == 1) continue;
            impose(h, s, h->V[comp], h->bc[comp]);
        }
        impose(h, s, h->P, h->bc[3]);
        if (h->sc) impose(h, s, h->T, h->bc[4]);
    }
    SARAS_CUDA(cudaGetLastError());
    return SARAS_OK;
}

saras_status rk3_create(const saras_grid_desc *gd, const saras_rk3_params *p, void *stream, saras_rk3 *h) {
    if (gd->pad != 1) {
        set_error("the RK3 stencils use Differentiation Scheme 1 (pad 1)");
        return SARAS_BAD_ARG;
    }
    if ((p->nl_scheme != 1 && p->nl_scheme != 3) || !(p->dt > 0.0) || !(p->nu >= 0.0) || !(p->kappa >= 0.0) || p->max_iterations < 0) {
        set_error("invalid RK3 parameters");
        return SARAS_BAD_ARG;
    }
    h->prm = *p;
    SARAS_TRY(h->grid.build(*gd, p->mg.levels));
    h->d3 = h->grid.dims == 3;
    h->sc = p->with_scalar != 0;
    h->stream = (cudaStream_t)stream;
    SARAS_TRY(saras_mg_create(gd, &p->mg, stream, &h->mg));
    const HostGrid &g = h->grid;
    h->L = make_lay(g.N[0], h->d3 ? g.N[1] : 1, g.N[2]);
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
    for (double *q : h->allocs) SARAS_CUDA(cudaMemset(q, 0, (size_t)sz * sizeof(double)));
    // metric tables: xi_x, xixx, xix2, a2, a1 per axis over the core
    const int n[3] = {h->L.n0, h->L.n1, h->L.n2};
    const int64_t tot = 5 * (int64_t)(n[0] + n[1] + n[2]);
    std::vector<double> host((size_t)tot, 0.0);
    SARAS_TRY(rk_alloc(h, &h->tab, tot));
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
        double *dst[5];
        for (int q = 0; q < 5; q++) dst[q] = h->tab + off + (int64_t)q * n[d];
        h->tabs.xi_x[d] = dst[0];
        h->tabs.xixx[d] = dst[1];
        h->tabs.xix2[d] = dst[2];
        h->tabs.a2[d] = dst[3];
        h->tabs.a1[d] = dst[4];
        for (int i = 0; i < n[d]; i++) {
            const size_t q = (size_t)(i + p0);
            const double v[5] = {g.fxi_x[d][q], g.fxixx[d][q], g.fxix2[d][q], h->scal.ih2t[d] * g.fxix2[d][q],
                                 h->scal.i2ht[d] * g.fxixx[d][q]};
            for (int qq = 0; qq < 5; qq++) host[(size_t)(off + (int64_t)qq * n[d] + i)] = v[qq];
        }
        off += 5 * (int64_t)n[d];
    }
    SARAS_CUDA(cudaMemcpy(h->tab, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice));
    h->bc[0] = make_fbc(h, p->bc_vx);
    h->bc[1] = make_fbc(h, p->bc_vy);
    h->bc[2] = make_fbc(h, p->bc_vz);
    h->bc[3] = make_fbc(h, p->bc_p);
    h->bc[4] = make_fbc(h, p->bc_t);
    const int64_t cells = (int64_t)n[0] * n[1] * n[2];
    h->nblocks = (int)std::max<int64_t>(1, std::min<int64_t>(1216, (cells + 255) / 256));
    SARAS_TRY(rk_alloc(h, &h->part, h->nblocks));
    SARAS_TRY(rk_alloc(h, &h->red, 4));
    SARAS_CUDA(cudaMallocHost((void **)&h->red_host, 4 * sizeof(double)));
    // timestep::timestep (timestep.cc:115): int(pow(log(Nx*Ny*Nz), 3))
    h->max_iterations = p->max_iterations > 0 ? p->max_iterations
                                              : int(std::pow(std::log(g.N[0] * g.N[1] * g.N[2]), 3));
    const int py = h->d3 ? 1 : 1;
    h->bst[2] = 1;
    h->bst[1] = n[2] + 2;
    h->bst[0] = h->bst[1] * (n[1] + 2 * py);
    h->box_elems = h->bst[0] * (n[0] + 2);
    SARAS_TRY(rk_alloc(h, &h->stage, h->box_elems));
    SARAS_CUDA(cudaDeviceSynchronize());
    return SARAS_OK;
}

void rk3_free(saras_rk3 *h) {
    for (double *p : h->allocs) cudaFree(p);
    if (h->red_host) cudaFreeHost(h->red_host);
    if (h->mg) saras_mg_destroy(h->mg);
}

saras_status box_transfer(saras_rk3 *h, double *field, const double *src_host, double *dst_host,
                          const int64_t st[3]) {
    for (int d = 0; d < 3; d++)
        if (st[d] != h->bst[d]) {
            set_error("RK3 fields must be C-contiguous padded arrays");
            return SARAS_BAD_ARG;
        }
    cudaStream_t s = h->stream;
    const Lay &L = h->L;
    const int64_t origin = h->bst[0] + h->bst[1] + 1;
    const size_t bytes = (size_t)h->box_elems * sizeof(double);
    const int bx = bxfor(L.n2 + 2);
    const dim3 g(cdiv(L.n2 + 2, bx), (unsigned)L.n1 + 2, (unsigned)L.n0 + 2);
    if (src_host) {
        SARAS_CUDA(cudaMemcpyAsync(h->stage, src_host - origin, bytes, cudaMemcpyHostToDevice, s));
        k_box_in<<<g, bx, 0, s>>>(h->stage + origin, h->bst[0], h->bst[1], field, L, -1, L.n1);
    } else {
        k_box_out<<<g, bx, 0, s>>>(field, L, h->stage + origin, h->bst[0], h->bst[1], -1, L.n1);
        SARAS_CUDA(cudaMemcpyAsync(dst_host - origin, h->stage, bytes, cudaMemcpyDeviceToHost, s));
    }
    SARAS_CUDA(cudaStreamSynchronize(s));
    return SARAS_OK;
}

}  // namespace

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
        SARAS_TRY(box_transfer(h, dst[q], src[q], nullptr, strides));
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
        SARAS_TRY(box_transfer(h, src[q], nullptr, dst[q], strides));
    }
    return SARAS_OK;
}

saras_status saras_rk3_step(saras_rk3 *h, int32_t nsteps, int32_t *mg_cycles, int32_t *cn_iters) {
    if (!h || nsteps < 0) return SARAS_BAD_ARG;
    int mgc = 0, cni = 0;
    h->launches = 0;
    saras_status st = SARAS_OK;
    for (int n = 0; n < nsteps && st == SARAS_OK; n++) st = time_advance(h, &mgc, &cni);
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

}  // extern "C"
