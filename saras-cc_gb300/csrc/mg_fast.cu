// FP64 and MIXED forms of the SARAS multigrid solve on GB300.
//
// FP64 form: the reference V-cycle (poisson.cc:203-279) with the stencil
// coefficients folded per axis (c- = xix2*ihx2 - xixx*i2hx, c+ = ... +,
// stored once per level), omega/D stored per cell, ghost cells folded into
// the stencil (Neumann: ghost = own value, Dirichlet: minus it, periodic:
// the wrapped neighbour), residual and restriction fused into one pass and
// the saved copy smd replaced by an in-place correction.  Results agree with
// the FP64_EXACT form to rounding.
//
// MIXED form: FP32 V-cycle (smoothing, restriction, prolongation) on the
// error equation A e = r inside an FP64 defect-correction loop; the finest
// residual r = f - A u, the update u += e, the coarsest solve and the
// null-space projection (compensated sums) are FP64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <math_constants.h>

#include "mg_fast.cuh"
#include "mg_stencil.cuh"

using namespace saras;

namespace {

constexpr int BX = 128;

// ------------------------------------------------------------ kernels ----

// FP64 colour sweep with omega/D stored per cell.
template <bool D3, bool W1>
__global__ void k_rbgs64(double *u, const double *__restrict__ f, const double *__restrict__ wd, Lay L,
                         Tab3<double> t, Bnd b, int colour, double omc) {
    pdl_enter();
    const int kk = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = D3 ? (int)blockIdx.y : 0;
    const int i = blockIdx.z;
    const int k = 2 * kk + ((i + j + colour) & 1);
    if (k >= L.n2) return;
    const int64_t c = L.at(i, j, k);
    const double uc = u[c];
    const double s = offdiag<double, D3>(u, L, t, b, i, j, k, c, uc) - f[c];
    u[c] = W1 ? s * wd[c] : fmat(s, wd[c], omc * uc);
}

// FP32 colour sweep; the diagonal is rebuilt from the 1-D tables.
template <bool D3>
__global__ void k_rbgs32(float *e, const float *__restrict__ r, Lay L, Tab3<float> t, Bnd b, int colour, float w,
                         float omc) {
    pdl_enter();
    const int kk = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = D3 ? (int)blockIdx.y : 0;
    const int i = blockIdx.z;
    const int k = 2 * kk + ((i + j + colour) & 1);
    if (k >= L.n2) return;
    const int64_t c = L.at(i, j, k);
    const float uc = e[c];
    const float s = offdiag<float, D3>(e, L, t, b, i, j, k, c, uc) - r[c];
    e[c] = fmat(omc, uc, sweep_div(w * s, diag<float, D3>(t, i, j, k)));
}

// Colour sweep with eight consecutive cells per thread along k: the rows a
// strip needs (own, j+-1, i+-1, f and omega/D) are loaded as aligned 16-byte
// vectors, so many loads are in flight per thread, and only the four cells of
// the sweep's colour are stored.  Used when n_z is a multiple of 8; the core
// of every row starts on a 32-byte boundary (Lay).
template <class T, bool D3, bool WD, bool W1 = false>
__global__ void k_rbgs_v8(T *u, const T *__restrict__ f, const T *__restrict__ wd, Lay L, Tab3<T> t, Bnd b,
                          int colour, T w, T omc) {
    pdl_enter();
    const int k0 = 8 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = D3 ? (int)(blockIdx.y * blockDim.y + threadIdx.y) : 0;
    const int i = blockIdx.z;
    if (k0 >= L.n2 || j >= L.n1) return;
    rbgs_strip8<T, D3, WD, W1>(u, f, wd, L, t, b, colour, w, omc, i, j, k0);
}

// The FP64 form's colour sweep (omega/D stored per cell) on 4-cell strips:
// strip_update's WD arithmetic cell for cell, with half of k_rbgs_v8's
// registers per thread (8-cell FP64 strips take 128), so that twice the
// warps hide the loads' latency.
template <bool D3, bool W1>
__global__ void __launch_bounds__(128, 8) k_rbgs_v4wd(double *u, const double *__restrict__ f,
                                                   const double *__restrict__ wd, Lay L, Tab3<double> t, Bnd b,
                                                   int colour, double omc) {
    pdl_enter();
    const int k0 = 4 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = D3 ? (int)(blockIdx.y * blockDim.y + threadIdx.y) : 0;
    const int i = blockIdx.z;
    if (k0 >= L.n2 || j >= L.n1) return;
    const int64_t c0 = L.at(i, j, k0);
    double cur[4], xm[4], xp[4], ym[4], yp[4], fr[4], wv[4];
    auto ldu = [](const double *q, double (&o)[4]) {
        const double2 a = *reinterpret_cast<const double2 *>(q);
        const double2 c = *reinterpret_cast<const double2 *>(q + 2);
        o[0] = a.x; o[1] = a.y; o[2] = c.x; o[3] = c.y;
    };
    auto mirror = [](const double (&c)[4], int sg, double (&o)[4]) {
#pragma unroll
        for (int q = 0; q < 4; q++) o[q] = sg > 0 ? c[q] : -c[q];
    };
    ldu(u + c0, cur);
    if (i > 0) ldu(u + c0 - L.s0, xm);
    else if (b.per[0]) ldu(u + c0 + (int64_t)(L.n0 - 1) * L.s0, xm);
    else mirror(cur, b.sg_lo[0], xm);
    if (i < L.n0 - 1) ldu(u + c0 + L.s0, xp);
    else if (b.per[0]) ldu(u + c0 - (int64_t)(L.n0 - 1) * L.s0, xp);
    else mirror(cur, b.sg_hi[0], xp);
    if (D3) {
        if (j > 0) ldu(u + c0 - L.s1, ym);
        else if (b.per[1]) ldu(u + c0 + (int64_t)(L.n1 - 1) * L.s1, ym);
        else mirror(cur, b.sg_lo[1], ym);
        if (j < L.n1 - 1) ldu(u + c0 + L.s1, yp);
        else if (b.per[1]) ldu(u + c0 - (int64_t)(L.n1 - 1) * L.s1, yp);
        else mirror(cur, b.sg_hi[1], yp);
    }
    ld4(f + c0, fr);
    ld4(wd + c0, wv);
    const double left = k0 > 0 ? u[c0 - 1] : (b.per[2] ? u[c0 + L.n2 - 1] : (b.sg_lo[2] > 0 ? cur[0] : -cur[0]));
    const double right =
        k0 + 4 < L.n2 ? u[c0 + 4] : (b.per[2] ? u[c0 + 4 - L.n2] : (b.sg_hi[2] > 0 ? cur[3] : -cur[3]));
    const double cmx = t.cm[0][i], cpx = t.cp[0][i];
    double cmy = 0.0, cpy = 0.0;
    if (D3) {
        cmy = t.cm[1][j];
        cpy = t.cp[1][j];
    }
    const int t0 = (colour + i + j + k0) & 1;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        if ((q & 1) != t0) continue;
        const int k = k0 + q;
        const double zm = q > 0 ? cur[q - 1] : left;
        const double zp = q < 3 ? cur[q + 1] : right;
        double sm = fmat(cmx, xm[q], -fr[q]);
        sm = fmat(cpx, xp[q], sm);
        if (D3) {
            sm = fmat(cmy, ym[q], sm);
            sm = fmat(cpy, yp[q], sm);
        }
        sm = fmat(t.cm[2][k], zm, sm);
        sm = fmat(t.cp[2][k], zp, sm);
        u[c0 + q] = W1 ? sm * wv[q] : fmat(sm, wv[q], omc * cur[q]);
    }
}

// Fused residual and restriction: one thread per coarse cell forms the
// residuals of its 2x2x2 children and their weighted sum (the coarsen
// weights v_abc / vTot of poisson_d3.cc:494-508, factorised per axis).
template <class T, class TO, bool D3>
__global__ void k_resid_restrict(const T *__restrict__ u, const T *__restrict__ f, Lay Lf, Tab3<T> t, Bnd b,
                                 WTab<T> w, TO *__restrict__ rc, Lay Lc, const T *__restrict__ dd,
                                 TO *__restrict__ ezero) {
    pdl_enter();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = D3 ? (int)blockIdx.y : 0;
    const int i = blockIdx.z;
    if (k >= Lc.n2) return;
    const int i2 = 2 * i, j2 = 2 * j, k2 = 2 * k;
    T out;
    if (D3) {
        T sy[2];
        for (int a = 0; a < 2; a++) {
            T sz[2];
            for (int bb = 0; bb < 2; bb++) {
                const T r0 = resid<T, true>(u, f, Lf, t, b, i2 + a, j2 + bb, k2, dd);
                const T r1 = resid<T, true>(u, f, Lf, t, b, i2 + a, j2 + bb, k2 + 1, dd);
                sz[bb] = fmat(w.w1[2][k], r1, w.w0[2][k] * r0);
            }
            sy[a] = fmat(w.w1[1][j], sz[1], w.w0[1][j] * sz[0]);
        }
        out = fmat(w.w1[0][i], sy[1], w.w0[0][i] * sy[0]);
    } else {
        const T r00 = resid<T, false>(u, f, Lf, t, b, i2, 0, k2, dd);
        const T r01 = resid<T, false>(u, f, Lf, t, b, i2, 0, k2 + 1, dd);
        const T r10 = resid<T, false>(u, f, Lf, t, b, i2 + 1, 0, k2, dd);
        const T r11 = resid<T, false>(u, f, Lf, t, b, i2 + 1, 0, k2 + 1, dd);
        out = ((r00 + r01) + (r10 + r11)) * T(0.25);
    }
    rc[Lc.at(i, j, k)] = (TO)out;
    if (ezero) ezero[Lc.at(i, j, k)] = TO(0);  // the coarse level's error starts from zero
}

// Fused residual and restriction, four coarse cells along k per thread (fine
// n_z a multiple of 8), the same arithmetic as k_resid_restrict.
template <class T, bool D3>
__global__ void __launch_bounds__(128, 4) k_resid_restrict8(const T *__restrict__ u, const T *__restrict__ f, Lay Lf, Tab3<T> t, Bnd b,
                                  WTab<T> w, T *__restrict__ rc, Lay Lc, const T *__restrict__ dd,
                                  T *__restrict__ ezero) {
    pdl_enter();
    const int kc0 = 4 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = D3 ? (int)(blockIdx.y * blockDim.y + threadIdx.y) : 0;
    const int i = blockIdx.z;
    if (kc0 >= Lc.n2 || j >= Lc.n1) return;
    T out[4];
    restrict4<T, D3>(u, f, Lf, t, b, w, dd, i, j, kc0, out);
    T *dst = rc + Lc.at(i, j, kc0);
    T *ez = ezero ? ezero + Lc.at(i, j, kc0) : nullptr;  // the coarse level's error starts from zero
    if (sizeof(T) == 4) {
        reinterpret_cast<float4 *>(dst)[0] = make_float4((float)out[0], (float)out[1], (float)out[2], (float)out[3]);
        if (ez) reinterpret_cast<float4 *>(ez)[0] = make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
        reinterpret_cast<double2 *>(dst)[0] = make_double2((double)out[0], (double)out[1]);
        reinterpret_cast<double2 *>(dst)[1] = make_double2((double)out[2], (double)out[3]);
        if (ez) {
            reinterpret_cast<double2 *>(ez)[0] = make_double2(0.0, 0.0);
            reinterpret_cast<double2 *>(ez)[1] = make_double2(0.0, 0.0);
        }
    }
}

// Fused FP32 residual and restriction, two coarse cells along k per thread
// (fine n_z a multiple of 8): the arithmetic of k_resid_restrict8 at 80
// registers instead of 128, so three blocks of eight warps per SM hide the
// loads' latency (256^3 -> 128^3: 52 us per launch against 73).
template <bool D3, bool RS>
__global__ void __launch_bounds__(256, 3) k_resid_restrict4(const float *__restrict__ u, const float *__restrict__ f,
                                                         Lay Lf, Tab3<float> t, Bnd b, WTab<float> w,
                                                         float *__restrict__ rc, Lay Lc, float *__restrict__ ezero) {
    pdl_enter();
    const int kc0 = 2 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = D3 ? (int)(blockIdx.y * blockDim.y + threadIdx.y) : 0;
    const int i = blockIdx.z;
    if (kc0 >= Lc.n2 || j >= Lc.n1) return;
    float out[2];
    restrict2<float, D3, RS>(u, f, Lf, t, b, w, (const float *)nullptr, i, j, kc0, out);
    const int64_t q = Lc.at(i, j, kc0);
    *reinterpret_cast<float2 *>(rc + q) = make_float2(out[0], out[1]);
    if (ezero) *reinterpret_cast<float2 *>(ezero + q) = make_float2(0.f, 0.f);  // the coarse error starts from zero
}

// The FP64 form's fused residual and restriction with the stored diagonal,
// two coarse cells along k per thread: k_resid_restrict8's arithmetic
// (restrict2 forms the same residuals and sums) at fewer registers.
template <bool D3>
__global__ void __launch_bounds__(128, 6) k_resid_restrict4d(const double *__restrict__ u,
                                                          const double *__restrict__ f, Lay Lf, Tab3<double> t,
                                                          Bnd b, WTab<double> w, double *__restrict__ rc, Lay Lc,
                                                          const double *__restrict__ dd,
                                                          double *__restrict__ ezero) {
    pdl_enter();
    const int kc0 = 2 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = D3 ? (int)(blockIdx.y * blockDim.y + threadIdx.y) : 0;
    const int i = blockIdx.z;
    if (kc0 >= Lc.n2 || j >= Lc.n1) return;
    double out[2];
    restrict2<double, D3>(u, f, Lf, t, b, w, dd, i, j, kc0, out);
    const int64_t q = Lc.at(i, j, kc0);
    *reinterpret_cast<double2 *>(rc + q) = make_double2(out[0], out[1]);
    if (ezero) *reinterpret_cast<double2 *>(ezero + q) = make_double2(0.0, 0.0);
}

// Injection prolongation and correction in place: fine += coarse(i/2,..).
template <class TF, class TC>
__global__ void k_prolong_add(TF *__restrict__ f, const TC *__restrict__ c, Lay Lf, Lay Lc, int d3) {
    pdl_enter();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    if (k >= Lf.n2) return;
    const int64_t q = Lf.at(i, j, k);
    f[q] = f[q] + (TF)c[Lc.at(i >> 1, d3 ? (j >> 1) : 0, k >> 1)];
}

// Injection prolongation and correction, eight fine cells along k per
// thread (n_z a multiple of 8): two aligned vector loads and stores of the
// fine row, one of the four coarse cells.
template <class T>
__global__ void k_prolong_add8(T *__restrict__ f, const T *__restrict__ c, Lay Lf, Lay Lc, int d3) {
    pdl_enter();
    const int k0 = 8 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y), i = blockIdx.z;
    if (k0 >= Lf.n2 || j >= Lf.n1) return;
    prolong8(f, c, Lf, Lc, d3, i, j, k0);
}

// k_prolong_add8 into a row-split FP32 level (3-D): fine cells k0 .. k0+7 of
// a row are its red and black halves at k0/2 .. k0/2+3, and both take the
// coarse cells (i/2, j/2, k0/2 .. k0/2+3), cell for cell what k_prolong_add8
// adds.
__global__ void k_prolong_add8_rs(float *__restrict__ f, const float *__restrict__ c, Lay Lf, Lay Lc) {
    pdl_enter();
    const int k0 = 8 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y), i = blockIdx.z;
    if (k0 >= Lf.n2 || j >= Lf.n1) return;
    const int h = k0 >> 1, H = Lf.n2 >> 1;
    float *row = f + Lf.at(i, j, 0);
    const float4 w = __ldg(reinterpret_cast<const float4 *>(c + Lc.at(i >> 1, j >> 1, h)));
    float4 *rd = reinterpret_cast<float4 *>(row + h), *bk = reinterpret_cast<float4 *>(row + H + h);
    const float4 a = *rd, d = *bk;
    *rd = make_float4(a.x + w.x, a.y + w.y, a.z + w.z, a.w + w.w);
    *bk = make_float4(d.x + w.x, d.y + w.y, d.z + w.z, d.w + w.w);
}

__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) {
        const double w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int NV>
__device__ __forceinline__ void block_store(double (&v)[NV], const bool (&is_max)[NV], double *part) {
    __shared__ double sh[NV][32];
    for (int q = 0; q < NV; q++) v[q] = is_max[q] ? warp_max(v[q]) : warp_sum(v[q]);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0)
        for (int q = 0; q < NV; q++) sh[q][wid] = v[q];
    __syncthreads();
    if (wid == 0) {
        for (int q = 0; q < NV; q++) {
            double x = lane < nw ? sh[q][lane] : 0.0;
            x = is_max[q] ? warp_max(x) : warp_sum(x);
            if (lane == 0) part[NV * blockIdx.x + q] = x;
        }
    }
}

// FP64 residual of the finest level with norm partials; optionally writes
// the residual in FP32 (MIXED form) and first applies u += e.
// For the L-infinity norm |r| and the running maximum use integer
// operations on the bit pattern (non-negative doubles order like their
// bits; a NaN sorts above infinity and reaches the host as non-finite), so
// the FP64 pipe only computes the stencil.  The RHS norm is taken once per
// solve (k_rhs_norm).
template <bool D3, bool MIX>
__global__ void k_resid_norm64(const double *__restrict__ u, const double *__restrict__ f,
                               const double *__restrict__ dd, Lay L, Tab3<double> t, Bnd b, int rtype,
                               double *__restrict__ part, float *__restrict__ r32, int rs) {
    unsigned long long mbits = 0ull;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for_core_rows(L, [&](int i, int j, int k) {
        const double r = resid<double, D3>(u, f, L, t, b, i, j, k, dd);
        if (MIX) r32[rs ? rs_at(L, i, j, k) : L.at(i, j, k)] = (float)r;
        if (rtype == 0) {
            const unsigned long long bits = (unsigned long long)__double_as_longlong(r) & 0x7fffffffffffffffull;
            mbits = bits > mbits ? bits : mbits;
        } else if (rtype == 1) {
            v[2] += fabs(r);
        } else {
            v[2] = fmat(r, r, v[2]);
        }
    });
    if (rtype == 0) {
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long w = __shfl_xor_sync(0xffffffffu, mbits, o);
            mbits = w > mbits ? w : mbits;
        }
        __shared__ unsigned long long shm[32];
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
        if (lane == 0) shm[wid] = mbits;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long m = 0ull;
            for (int q = 0; q < nw; q++) m = shm[q] > m ? shm[q] : m;
            part[4 * blockIdx.x] = __longlong_as_double((long long)m);
            part[4 * blockIdx.x + 1] = 0.0;
            part[4 * blockIdx.x + 2] = 0.0;
            part[4 * blockIdx.x + 3] = 0.0;
        }
        return;
    }
    const bool mx[4] = {true, true, false, false};
    block_store<4>(v, mx, part);
}

// RHS norm of the solve: max|f| (L-inf), sum|f| (L1) or sum f^2 (L2).
__global__ void k_rhs_norm(const double *__restrict__ f, Lay L, int rtype, double *__restrict__ part) {
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for_core_rows(L, [&](int i, int j, int k) {
        const double fv = f[L.at(i, j, k)];
        if (rtype == 0) {
            const double af = fabs(fv);
            if (af > v[1]) v[1] = af;
        } else if (rtype == 1) {
            v[3] += fabs(fv);
        } else {
            v[3] = fmat(fv, fv, v[3]);
        }
    });
    const bool mx[4] = {true, true, false, false};
    block_store<4>(v, mx, part);
}

// One warp: lane t reduces partials t, t+32, ... in order, then a fixed
// shuffle tree combines the lanes (the same order on every run).
__global__ void k_rhs_norm_final(const double *__restrict__ part, int nb, int rtype, double *__restrict__ out) {
    double m = 0.0, sm = 0.0;
    for (int q = threadIdx.x; q < nb; q += 32) {
        const double a = part[4 * q + 1];
        if (a > m) m = a;
        sm += part[4 * q + 3];
    }
    m = warp_max(m);
    sm = warp_sum(sm);
    if (threadIdx.x == 0) out[0] = rtype == 0 ? m : sm;
}

// A coarsest-level cell with its neighbours and folded coefficients, in the
// order offdiag applies them (x-, x+, y-, y+, z-, z+).  A wall neighbour is
// the cell itself (the mirror of its own value), its coefficient negated at a
// Dirichlet wall; a periodic neighbour wraps.
struct CCell {
    int c, nb[6];
    double cf[6];
};

template <bool D3>
__device__ __forceinline__ CCell ccell(const Lay &L, const Tab3<double> &t, const Bnd &b, int i, int j, int k) {
    CCell x;
    x.c = (int)L.at(i, j, k);
    const int ax[3] = {i, j, k}, nn[3] = {L.n0, L.n1, L.n2};
    const int st[3] = {(int)L.s0, (int)L.s1, 1};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const int lo = 2 * d, hi = 2 * d + 1;
        const double cm = D3 || d != 1 ? t.cm[d][ax[d]] : 0.0, cp = D3 || d != 1 ? t.cp[d][ax[d]] : 0.0;
        if (ax[d] > 0) {
            x.nb[lo] = x.c - st[d];
            x.cf[lo] = cm;
        } else if (b.per[d]) {
            x.nb[lo] = x.c + (nn[d] - 1) * st[d];
            x.cf[lo] = cm;
        } else {
            x.nb[lo] = x.c;
            x.cf[lo] = b.sg_lo[d] > 0 ? cm : -cm;
        }
        if (ax[d] < nn[d] - 1) {
            x.nb[hi] = x.c + st[d];
            x.cf[hi] = cp;
        } else if (b.per[d]) {
            x.nb[hi] = x.c - (nn[d] - 1) * st[d];
            x.cf[hi] = cp;
        } else {
            x.nb[hi] = x.c;
            x.cf[hi] = b.sg_hi[d] > 0 ? cp : -cp;
        }
    }
    return x;
}

// offdiag<double, D3> of a prepared cell: the same products and sums, in the
// same order.
template <bool D3>
__device__ __forceinline__ double ccell_offdiag(const double *u, const CCell &x) {
    double s = x.cf[0] * u[x.nb[0]];
    s = fmat(x.cf[1], u[x.nb[1]], s);
    if (D3) {
        s = fmat(x.cf[2], u[x.nb[2]], s);
        s = fmat(x.cf[3], u[x.nb[3]], s);
    }
    s = fmat(x.cf[4], u[x.nb[4]], s);
    s = fmat(x.cf[5], u[x.nb[5]], s);
    return s;
}

// The coarsest SOR red-black sweeps of k_coarsest_fast when every thread of
// the block owns at most one cell of each colour and two residual cells
// (n0 * n1 * ceil(n2/2) <= blockDim, cells <= 2 blockDim): u (zero), f, wd
// (omega/D) and dd (D) in shared memory; returns the sweeps run.
template <bool D3>
__device__ int coarsest_cached(double *u, const double *f, const double *wd, const double *dd, const Lay &L,
                               const Tab3<double> &t, const Bnd &b, double omc, double tol, int max_count,
                               int stall_check, unsigned long long *shm) {
    const int half = (L.n2 + 1) / 2;
    const int ncol = L.n0 * L.n1 * half;
    const int ncell = L.n0 * L.n1 * L.n2;
    int iter = 0, sweeps = 0;
    double stall_ref = __longlong_as_double(0x7ff0000000000000ll);  // +infinity
    // Every thread owns at most one cell of each colour and two residual
    // cells: their indices, neighbours and coefficients are formed once
    // and kept in registers, and a sweep is shared-memory loads and the
    // FMA chain.  A wall neighbour is the cell itself with the
    // coefficient negated at a Dirichlet wall (cf * -u and -cf * u are
    // the same bits), so the arithmetic is offdiag's and resid's.
    CCell col[2], res[2];
    bool has_col[2], has_res[2];
    double wdc[2], fcol[2], ddr[2], fres[2];
#pragma unroll
    for (int colour = 0; colour < 2; colour++) {
        const int q = threadIdx.x;
        has_col[colour] = false;
        if (q < ncol) {
            const int kk = q % half, rest = q / half, j = rest % L.n1, i = rest / L.n1;
            const int k = 2 * kk + ((i + j + colour) & 1);
            if (k < L.n2) {
                col[colour] = ccell<D3>(L, t, b, i, j, k);
                wdc[colour] = wd[col[colour].c];
                fcol[colour] = f[col[colour].c];
                has_col[colour] = true;
            }
        }
    }
#pragma unroll
    for (int r = 0; r < 2; r++) {
        const int q = threadIdx.x + r * blockDim.x;
        has_res[r] = q < ncell;
        if (has_res[r]) {
            const int k = q % L.n2, rest = q / L.n2, j = rest % L.n1, i = rest / L.n1;
            res[r] = ccell<D3>(L, t, b, i, j, k);
            ddr[r] = dd[res[r].c];
            fres[r] = f[res[r].c];
        }
    }
    // one warp (up to 64 cells): warp barriers, and the shuffle maximum
    // is already in every lane
    const bool one_warp = blockDim.x == 32;
    auto sync = [&]() {
        if (one_warp)
            __syncwarp();
        else
            __syncthreads();
    };
    for (;;) {
#pragma unroll
        for (int colour = 0; colour < 2; colour++) {
            if (has_col[colour]) {
                const CCell &x = col[colour];
                const double uc = u[x.c];
                const double sv = ccell_offdiag<D3>(u, x) - fcol[colour];
                u[x.c] = fmat(sv, wdc[colour], omc * uc);
            }
            sync();
        }
        unsigned long long m = 0ull;
#pragma unroll
        for (int r = 0; r < 2; r++) {
            if (!has_res[r]) continue;
            const CCell &x = res[r];
            const double rv = fres[r] - fmat(-ddr[r], u[x.c], ccell_offdiag<D3>(u, x));
            const unsigned long long bits = (unsigned long long)__double_as_longlong(rv) & 0x7fffffffffffffffull;
            m = bits > m ? bits : m;
        }
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long w2 = __shfl_xor_sync(0xffffffffu, m, o);
            m = w2 > m ? w2 : m;
        }
        unsigned long long mm = m;
        if (!one_warp) {
            if ((threadIdx.x & 31) == 0) shm[threadIdx.x >> 5] = m;
            __syncthreads();
            mm = 0ull;
            for (int q = 0; q < (int)(blockDim.x >> 5); q++) mm = shm[q] > mm ? shm[q] : mm;
            __syncthreads();
        }
        sweeps++;
        const double rn = __longlong_as_double((long long)mm);
        if (rn < tol) break;
        if (stall_check > 0 && iter % stall_check == 0) {
            if (rn > 0.999 * stall_ref) break;
            stall_ref = rn;
        }
        iter++;
        if (iter > max_count) break;
    }
    return sweeps;
}

// Coarsest level of the FP64 and MIXED forms: SOR red-black sweeps with
// omega/D stored per cell and the boundary folded into the stencil, run to
// the absolute tolerance or the iteration cap of poisson_d3.cc:249-432, by
// one block in shared memory.
template <bool D3>
__global__ void k_coarsest_fast(double *ug, const double *__restrict__ fg, const double *__restrict__ wdg,
                                const double *__restrict__ ddg, Lay L, Tab3<double> t, Bnd b, double omc, double tol,
                                int max_count, int stall_check, int *sweeps_out) {
    pdl_enter();
    extern __shared__ double stage[];
    __shared__ unsigned long long shm[32];
    double *u = stage, *f = stage + L.size, *wd = stage + 2 * L.size, *dd = stage + 3 * L.size;
    for (int64_t q = threadIdx.x; q < L.size; q += blockDim.x) {
        u[q] = 0.0;  // the coarsest solve starts from zero
        f[q] = fg[q];
        wd[q] = wdg[q];
        dd[q] = ddg[q];
    }
    __syncthreads();
    const int half = (L.n2 + 1) / 2;
    const int ncol = L.n0 * L.n1 * half;
    const int ncell = L.n0 * L.n1 * L.n2;
    int iter = 0, sweeps = 0;
    double stall_ref = __longlong_as_double(0x7ff0000000000000ll);  // +infinity
    if (ncol <= (int)blockDim.x && ncell <= 2 * (int)blockDim.x) {
        const int sweeps = coarsest_cached<D3>(u, f, wd, dd, L, t, b, omc, tol, max_count, stall_check, shm);
        for (int64_t q = threadIdx.x; q < L.size; q += blockDim.x) ug[q] = u[q];
        if (threadIdx.x == 0) *sweeps_out += sweeps;
        return;
    }
    for (;;) {
        for (int colour = 0; colour < 2; colour++) {
            for (int q = threadIdx.x; q < ncol; q += blockDim.x) {
                const int kk = q % half, rest = q / half, j = rest % L.n1, i = rest / L.n1;
                const int k = 2 * kk + ((i + j + colour) & 1);
                if (k >= L.n2) continue;
                const int64_t c = L.at(i, j, k);
                const double uc = u[c];
                const double sv = offdiag<double, D3>(u, L, t, b, i, j, k, c, uc) - f[c];
                u[c] = fmat(sv, wd[c], omc * uc);
            }
            __syncthreads();
        }
        unsigned long long m = 0ull;
        for (int q = threadIdx.x; q < ncell; q += blockDim.x) {
            const int k = q % L.n2, rest = q / L.n2, j = rest % L.n1, i = rest / L.n1;
            const double r = resid<double, D3>(u, f, L, t, b, i, j, k, dd);
            const unsigned long long bits = (unsigned long long)__double_as_longlong(r) & 0x7fffffffffffffffull;
            m = bits > m ? bits : m;
        }
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long w = __shfl_xor_sync(0xffffffffu, m, o);
            m = w > m ? w : m;
        }
        if ((threadIdx.x & 31) == 0) shm[threadIdx.x >> 5] = m;
        __syncthreads();
        unsigned long long mm = 0ull;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) mm = shm[q] > mm ? shm[q] : mm;
        __syncthreads();
        sweeps++;
        const double rn = __longlong_as_double((long long)mm);
        if (rn < tol) break;
        if (stall_check > 0 && iter % stall_check == 0) {
            // a singular coarsest problem whose restricted RHS is slightly
            // incompatible stops improving at the incompatible part: stop
            // once `stall_check` sweeps gain less than 0.1%
            if (rn > 0.999 * stall_ref) break;
            stall_ref = rn;
        }
        iter++;
        if (iter > max_count) break;
    }
    for (int64_t q = threadIdx.x; q < L.size; q += blockDim.x) ug[q] = u[q];
    if (threadIdx.x == 0) *sweeps_out += sweeps;
}

// ---- the bottom of the MIXED V-cycle in one block ----
//
// Below some size a level's kernels are launch latency: a colour sweep of
// 16^3 cells lasts a few microseconds.  k_bottom runs everything a V-cycle
// does from the first level it holds down to the coarsest and back up to
// that level again (pre-smoothing, residual and restriction, the coarsest
// solve, prolongation and correction, post-smoothing) in one block, each
// level's e and r and the coarsest u, f, omega/D and D in shared memory,
// the steps separated by block barriers.  Each step has the arithmetic of
// the kernel it replaces (k_rbgs32, k_resid_restrict, k_coarsest_fast,
// k_prolong_add), cell for cell, so the V-cycle's bits do not change.
//
// Inside the block everything is latency, so the block keeps every operand
// in shared memory: the levels' coefficient and restriction-weight tables
// and the coarsest level's tables are copied in, each level's colour cells
// are listed once as packed (i, j, k/2) (before the wait on the previous
// kernel), and a thread forms all of its cells of a sweep (at most BOT_CPT)
// before it writes any of them back.
constexpr int BOT_MAX = 4;  // FP32 levels above the coarsest
constexpr int BOT_THREADS = 512;
constexpr int BOT_CPT = 4;  // colour cells per thread and sweep

struct BotArgs {
    int nb;  // FP32 levels held: lb .. lb + nb - 1, then the coarsest
    Lay L[BOT_MAX];
    Tab3<float> t[BOT_MAX];
    WTab<float> w[BOT_MAX + 1];  // restriction weights of levels lb+1 .. the coarsest (index m+1)
    Lay Lc;
    Tab3<double> tc;
    const double *wdc, *ddc;  // the coarsest level's omega/D and D
    const float *r_top;       // r of level lb, formed by the restriction before
    float *e_top;             // e of level lb, read by the prolongation after
    Bnd b;
    float w32, omc32;
    double omc64, tol;
    int max_count, stall, pre, post;
    int *sweeps_out;
    // shared-memory byte offsets: e, r per level; u, f, wd, dd; the tables
    // of each level (coefficients, then the next level's restriction
    // weights), the coarsest level's tables; each level's colour-cell list
    unsigned off[2 * BOT_MAX + 4];
    unsigned toff[BOT_MAX], tcoff, loff[BOT_MAX];
};

// Asynchronous global -> shared copies (cp.async): a thread issues all of
// its copies back to back and waits once, so the block's set-up is one
// round trip to L2 however many arrays it gathers.
__device__ __forceinline__ void cpa(void *dst, const float *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(__cvta_generic_to_global(src))
                 : "memory");
}
__device__ __forceinline__ void cpa(void *dst, const double *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(__cvta_generic_to_global(src))
                 : "memory");
}
__device__ __forceinline__ void cpa_wait() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Shared-memory copies of a level's tables (every thread issues a share of
// the copies); the pointers go to the shared struct `s` (thread 0).
template <class T>
__device__ void bot_tab(const Tab3<T> &g, const Lay &L, T *p, Tab3<T> *s) {
    const int n[3] = {L.n0, L.n1, L.n2};
    for (int d = 0; d < 3; d++) {
        if (threadIdx.x == 0) {
            s->cm[d] = p;
            s->cp[d] = p + n[d];
            s->dg[d] = p + 2 * n[d];
        }
        for (int q = threadIdx.x; q < n[d]; q += blockDim.x) {
            cpa(p + q, g.cm[d] + q);
            cpa(p + n[d] + q, g.cp[d] + q);
            cpa(p + 2 * n[d] + q, g.dg[d] + q);
        }
        p += 3 * n[d];
    }
}
__device__ void bot_wtab(const WTab<float> &g, const Lay &Lc, float *p, WTab<float> *s) {
    const int n[3] = {Lc.n0, Lc.n1, Lc.n2};
    for (int d = 0; d < 3; d++) {
        if (threadIdx.x == 0) {
            s->w0[d] = p;
            s->w1[d] = p + n[d];
        }
        for (int q = threadIdx.x; q < n[d]; q += blockDim.x) {
            cpa(p + q, g.w0[d] + q);
            cpa(p + n[d] + q, g.w1[d] + q);
        }
        p += 2 * n[d];
    }
}

// Colour column q of a level (q < n0 n1 ceil(n2/2)) as (i << 20 | j << 10 | k/2).
__device__ __forceinline__ unsigned bot_pack(const Lay &L, int q) {
    const int half = (L.n2 + 1) / 2;
    const int kk = q % half, rest = q / half, j = rest % L.n1, i = rest / L.n1;
    return ((unsigned)i << 20) | ((unsigned)j << 10) | (unsigned)kk;
}

template <bool D3>
__device__ void bot_smooth(float *e, const float *r, const Lay &L, const Tab3<float> &ts, const Bnd &b, int count,
                           float w, float omc, const unsigned *lst) {
    const Tab3<float> t = ts;  // the table pointers in registers for the whole sweep
    const int half = (L.n2 + 1) / 2, ncol = L.n0 * L.n1 * half;
    for (int n = 0; n < count; n++)
        for (int colour = 0; colour < 2; colour++) {
            // the sweep's cells read only cells of the other colour: all
            // of a thread's cells are formed before any is written
            float nv[BOT_CPT];
            int cc[BOT_CPT];
#pragma unroll
            for (int m = 0; m < BOT_CPT; m++) {
                cc[m] = -1;
                const int q = threadIdx.x + m * blockDim.x;
                if (q >= ncol) continue;
                const unsigned pk = lst[q];
                const int i = (int)(pk >> 20), j = (int)((pk >> 10) & 1023u);
                const int k = 2 * (int)(pk & 1023u) + ((i + j + colour) & 1);
                if (k >= L.n2) continue;
                const int64_t c = L.at(i, j, k);
                const float uc = e[c];
                const float sv = offdiag<float, D3>(e, L, t, b, i, j, k, c, uc) - r[c];
                nv[m] = fmat(omc, uc, sweep_div(w * sv, diag<float, D3>(t, i, j, k)));
                cc[m] = (int)c;
            }
#pragma unroll
            for (int m = 0; m < BOT_CPT; m++)
                if (cc[m] >= 0) e[cc[m]] = nv[m];
            __syncthreads();
        }
}

template <class TO, bool D3>
__device__ void bot_restrict(const float *e, const float *r, const Lay &Lf, const Tab3<float> &ts, const Bnd &b,
                             const WTab<float> &ws, TO *rc, const Lay &Lc) {
    const Tab3<float> t = ts;  // the table pointers in registers
    const WTab<float> w = ws;
    const int ncell = Lc.n0 * Lc.n1 * Lc.n2;
    for (int q = threadIdx.x; q < ncell; q += blockDim.x) {
        const int k = q % Lc.n2, rest = q / Lc.n2, j = rest % Lc.n1, i = rest / Lc.n1;
        const int i2 = 2 * i, j2 = 2 * j, k2 = 2 * k;
        float sy[2];
        for (int a = 0; a < 2; a++) {
            float sz[2];
            for (int bb = 0; bb < 2; bb++) {
                const float r0 = resid<float, D3>(e, r, Lf, t, b, i2 + a, j2 + bb, k2);
                const float r1 = resid<float, D3>(e, r, Lf, t, b, i2 + a, j2 + bb, k2 + 1);
                sz[bb] = fmat(w.w1[2][k], r1, w.w0[2][k] * r0);
            }
            sy[a] = fmat(w.w1[1][j], sz[1], w.w0[1][j] * sz[0]);
        }
        rc[Lc.at(i, j, k)] = (TO)fmat(w.w1[0][i], sy[1], w.w0[0][i] * sy[0]);
    }
}

// e_fine += e_coarse of the parent cell, by coarse cells: the eight children
// are read before any is written.
template <class TC>
__device__ void bot_prolong(float *ef, const TC *ec, const Lay &Lf, const Lay &Lc) {
    const int ncell = Lc.n0 * Lc.n1 * Lc.n2;
    for (int q = threadIdx.x; q < ncell; q += blockDim.x) {
        const int k = q % Lc.n2, rest = q / Lc.n2, j = rest % Lc.n1, i = rest / Lc.n1;
        const float v = (float)ec[Lc.at(i, j, k)];
        float o[8];
        int cc[8];
#pragma unroll
        for (int x = 0; x < 8; x++) {
            const int fi = 2 * i + (x >> 2), fj = 2 * j + ((x >> 1) & 1), fk = 2 * k + (x & 1);
            cc[x] = -1;
            if (fi < Lf.n0 && fj < Lf.n1 && fk < Lf.n2) {
                cc[x] = (int)Lf.at(fi, fj, fk);
                o[x] = ef[cc[x]] + v;
            }
        }
#pragma unroll
        for (int x = 0; x < 8; x++)
            if (cc[x] >= 0) ef[cc[x]] = o[x];
    }
}

template <bool D3>
__global__ void __launch_bounds__(BOT_THREADS) k_bottom(const __grid_constant__ BotArgs a) {
    extern __shared__ __align__(16) unsigned char bsm[];
    __shared__ unsigned long long shm[32];
    // the levels' table pointers (the same for every thread) live in shared
    // memory, and the arrays' addresses are formed from the offsets where
    // they are used: nothing per level sits in per-thread local memory
    __shared__ Tab3<float> st[BOT_MAX];
    __shared__ WTab<float> sw[BOT_MAX];
    __shared__ Tab3<double> stc;
    auto E = [&](int m) { return reinterpret_cast<float *>(bsm + a.off[2 * m]); };
    auto R = [&](int m) { return reinterpret_cast<float *>(bsm + a.off[2 * m + 1]); };
    auto LST = [&](int m) { return reinterpret_cast<unsigned *>(bsm + a.loff[m]); };
    double *u = reinterpret_cast<double *>(bsm + a.off[2 * BOT_MAX]);
    double *f = reinterpret_cast<double *>(bsm + a.off[2 * BOT_MAX + 1]);
    double *wd = reinterpret_cast<double *>(bsm + a.off[2 * BOT_MAX + 2]);
    double *dd = reinterpret_cast<double *>(bsm + a.off[2 * BOT_MAX + 3]);
    // on-chip set-up before the wait on the previous kernels: cell lists
    // and zeroed arrays (every e starts from zero; the restriction into a
    // level clears it; ghosts stay zero and are never read)
    for (int m = 0; m < a.nb; m++) {
        unsigned *l = LST(m);
        const int ncol = a.L[m].n0 * a.L[m].n1 * ((a.L[m].n2 + 1) / 2);
        for (int q = threadIdx.x; q < ncol; q += blockDim.x) l[q] = bot_pack(a.L[m], q);
        float *em = E(m), *rm = R(m);
        for (int64_t q = threadIdx.x; q < a.L[m].size; q += blockDim.x) {
            em[q] = 0.f;
            if (m > 0) rm[q] = 0.f;
        }
    }
    for (int64_t q = threadIdx.x; q < a.Lc.size; q += blockDim.x) {
        u[q] = 0.0;
        f[q] = 0.0;
    }
    // global memory only after the wait (earlier kernels may still run
    // before it)
    pdl_enter();
    for (int m = 0; m < a.nb; m++) {
        float *tp = reinterpret_cast<float *>(bsm + a.toff[m]);
        bot_tab<float>(a.t[m], a.L[m], tp, &st[m]);
        const Lay &Ln = m + 1 < a.nb ? a.L[m + 1] : a.Lc;
        bot_wtab(a.w[m + 1], Ln, tp + 3 * (a.L[m].n0 + a.L[m].n1 + a.L[m].n2), &sw[m]);
    }
    bot_tab<double>(a.tc, a.Lc, reinterpret_cast<double *>(bsm + a.tcoff), &stc);
    for (int64_t q = threadIdx.x; q < a.Lc.size; q += blockDim.x) {
        cpa(wd + q, a.wdc + q);
        cpa(dd + q, a.ddc + q);
    }
    {
        float *r0 = R(0);
        for (int64_t q = threadIdx.x; q < a.L[0].size; q += blockDim.x) cpa(r0 + q, a.r_top + q);
    }
    cpa_wait();
    __syncthreads();
    for (int m = 0; m < a.nb; m++) {
        bot_smooth<D3>(E(m), R(m), a.L[m], st[m], a.b, a.pre, a.w32, a.omc32, LST(m));
        if (m + 1 < a.nb)
            bot_restrict<float, D3>(E(m), R(m), a.L[m], st[m], a.b, sw[m], R(m + 1), a.L[m + 1]);
        else
            bot_restrict<double, D3>(E(m), R(m), a.L[m], st[m], a.b, sw[m], f, a.Lc);
        __syncthreads();
    }
    const int sweeps = coarsest_cached<D3>(u, f, wd, dd, a.Lc, stc, a.b, a.omc64, a.tol, a.max_count, a.stall, shm);
    __syncthreads();
    for (int m = a.nb - 1; m >= 0; m--) {
        if (m == a.nb - 1)
            bot_prolong<double>(E(m), u, a.L[m], a.Lc);
        else
            bot_prolong<float>(E(m), E(m + 1), a.L[m], a.L[m + 1]);
        __syncthreads();
        bot_smooth<D3>(E(m), R(m), a.L[m], st[m], a.b, a.post, a.w32, a.omc32, LST(m));
    }
    {
        const float *e0 = E(0);
        for (int64_t q = threadIdx.x; q < a.L[0].size; q += blockDim.x) a.e_top[q] = e0[q];
    }
    if (threadIdx.x == 0) *a.sweeps_out += sweeps;
}

// Exact coarsest solve of the MIXED form (fd_solve), one block; dynamic
// shared memory holds two copies of the coarsest grid.
__global__ void k_coarsest_fd(double *ug, const double *__restrict__ fg, Lay L, FDiag F) {
    pdl_enter();
    extern __shared__ double fds[];
    const int ncell = L.n0 * L.n1 * L.n2;
    fd_solve(ug, fg, L, F, fds, fds + ncell);
}

// u += e over the core (MIXED form update, FP64 accumulate).
__global__ void k_update64(double *__restrict__ u, const float *__restrict__ e, Lay L, int rs) {
    pdl_enter();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    if (k >= L.n2) return;
    const int64_t q = L.at(i, j, k);
    u[q] = u[q] + (double)e[rs ? rs_at(L, i, j, k) : q];
}

__device__ __forceinline__ void two_sum(double a, double b, double &s, double &c) {
    s = a + b;
    const double bb = s - a;
    c = (a - (s - bb)) + (b - bb);
}

// Compensated (Neumaier) sum of the core of u: per-block (sum, error) pairs.
__global__ void k_csum(const double *__restrict__ u, Lay L, double *__restrict__ part) {
    double s = 0.0, c = 0.0;
    for_core_rows(L, [&](int i, int j, int k) {
        double t, e;
        two_sum(s, u[L.at(i, j, k)], t, e);
        s = t;
        c += e;
    });
    for (int o = 16; o > 0; o >>= 1) {
        const double s2 = __shfl_xor_sync(0xffffffffu, s, o), c2 = __shfl_xor_sync(0xffffffffu, c, o);
        double t, e;
        two_sum(s, s2, t, e);
        s = t;
        c += c2 + e;
    }
    __shared__ double sh[2][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) {
        sh[0][wid] = s;
        sh[1][wid] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double S = 0.0, Cc = 0.0;
        for (int w = 0; w < nw; w++) {
            double t, e;
            two_sum(S, sh[0][w], t, e);
            S = t;
            Cc += sh[1][w] + e;
        }
        part[2 * blockIdx.x] = S;
        part[2 * blockIdx.x + 1] = Cc;
    }
}

// Mean of u from the (sum, error) partials, in a fixed order; slot 0 of
// `out` receives the mean; with `sub` set, out[0] becomes mean - out[1].
// One warp, lanes over strided partials in order, then a fixed shuffle tree
// of compensated additions.
__global__ void k_csum_final(const double *__restrict__ part, int nb, double count, double *out, int slot) {
    double S = 0.0, Cc = 0.0;
    for (int q = threadIdx.x; q < nb; q += 32) {
        double t, e;
        two_sum(S, part[2 * q], t, e);
        S = t;
        Cc += part[2 * q + 1] + e;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double s2 = __shfl_xor_sync(0xffffffffu, S, o), c2 = __shfl_xor_sync(0xffffffffu, Cc, o);
        double t, e;
        two_sum(S, s2, t, e);
        S = t;
        Cc += c2 + e;
    }
    if (threadIdx.x == 0) out[slot] = (S + Cc) / count;
}

__global__ void k_shift(double *__restrict__ u, Lay L, const double *__restrict__ m) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    if (k >= L.n2) return;
    const int64_t q = L.at(i, j, k);
    u[q] = u[q] - (m[0] - m[1]);
}

// omega / D and D per cell for the FP64 kernels (either may be absent).
template <bool D3>
__global__ void k_inv_diag(double *__restrict__ wd, double *__restrict__ dd, Lay L, Tab3<double> t, double w) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = D3 ? (int)blockIdx.y : 0;
    const int i = blockIdx.z;
    if (k >= L.n2) return;
    const double d = diag<double, D3>(t, i, j, k);
    if (wd) wd[L.at(i, j, k)] = w / d;
    if (dd) dd[L.at(i, j, k)] = d;
}

// ------------------------------------------------------- host side ----

Tab3<double> tab64(const Level &v) {
    return Tab3<double>{{v.cm[0], v.cm[1], v.cm[2]}, {v.cp[0], v.cp[1], v.cp[2]}, {v.dg[0], v.dg[1], v.dg[2]}};
}
Tab3<float> tab32(const Level &v) {
    return Tab3<float>{{v.cm32[0], v.cm32[1], v.cm32[2]},
                       {v.cp32[0], v.cp32[1], v.cp32[2]},
                       {v.dg32[0], v.dg32[1], v.dg32[2]}};
}
WTab<double> wt64(const Level &v) { return WTab<double>{{v.w0[0], v.w0[1], v.w0[2]}, {v.w1[0], v.w1[1], v.w1[2]}}; }
WTab<float> wt32(const Level &v) {
    return WTab<float>{{v.w032[0], v.w032[1], v.w032[2]}, {v.w132[0], v.w132[1], v.w132[2]}};
}

Bnd bnd(const saras_mg *h) {
    Bnd b;
    for (int d = 0; d < 3; d++) {
        b.per[d] = h->ghost.per[d];
        b.sg_lo[d] = h->ghost.kind[2 * d] == SARAS_BC_NEUMANN ? 1 : -1;
        b.sg_hi[d] = h->ghost.kind[2 * d + 1] == SARAS_BC_NEUMANN ? 1 : -1;
    }
    return b;
}

inline dim3 cgrid(const Lay &L, bool d3, int kcount, int bx) {
    return dim3(cdiv(kcount, bx), d3 ? (unsigned)L.n1 : 1u, (unsigned)L.n0);
}
inline int bxfor(int n) { return std::min(BX, (n + 31) / 32 * 32); }

// The eight-cells-per-thread sweep needs rows of whole strips.
inline bool v8_ok(const Lay &L) { return L.n2 % 8 == 0 && L.n2 >= 16; }

template <class T, bool WD>
void colour_v8(saras_mg *h, cudaStream_t s, Level &v, T *u, const T *f, const T *wd, const Tab3<T> &tb, int colour,
               T w, T omc) {
    const Lay &L = v.lay;
    const int strips = L.n2 / 8;
    const int bx = std::min(strips, 32);
    const int by = h->d3 ? std::max(1, 128 / bx) : 1;
    const dim3 blk(bx, by);
    const dim3 g(cdiv(strips, bx), h->d3 ? cdiv(L.n1, by) : 1u, (unsigned)L.n0);
    const Bnd b = bnd(h);
    // the stored-omega/D form skips the (1 - omega) u term when it is zero
    const bool w1 = WD && h->prm.sor_param == 1.0;
    if (h->d3)
        launch_pdl(w1 ? k_rbgs_v8<T, true, WD, true> : k_rbgs_v8<T, true, WD>, g, blk, 0, s, u, f, wd, L, tb, b,
                   colour, w, omc);
    else
        launch_pdl(w1 ? k_rbgs_v8<T, false, WD, true> : k_rbgs_v8<T, false, WD>, g, blk, 0, s, u, f, wd, L, tb, b,
                   colour, w, omc);
}

void colour64(saras_mg *h, cudaStream_t s, int l, int colour) {
    Level &v = h->lv[(size_t)l];
    const Lay &L = v.lay;
    if (L.n2 % 4 == 0 && L.n2 >= 16 && (int64_t)L.n0 * L.n1 * L.n2 >= (int64_t(1) << 20)) {
        // the large levels: 4-cell strips, twice the resident warps
        kbegin(h, s, l == 0 ? KC_SMOOTH0 : -1);
        const int strips = L.n2 / 4, bx = std::min(strips, 64), by = h->d3 ? std::max(1, 128 / bx) : 1;
        const dim3 g(cdiv(strips, bx), h->d3 ? cdiv(L.n1, by) : 1u, (unsigned)L.n0);
        const bool w1 = h->prm.sor_param == 1.0;
        const double omc = 1.0 - h->prm.sor_param;
        if (h->d3)
            launch_pdl(w1 ? k_rbgs_v4wd<true, true> : k_rbgs_v4wd<true, false>, g, dim3(bx, by), 0, s, v.lhs,
                       (const double *)v.rhs, (const double *)v.inv_diag, L, tab64(v), bnd(h), colour, omc);
        else
            launch_pdl(w1 ? k_rbgs_v4wd<false, true> : k_rbgs_v4wd<false, false>, g, dim3(bx, by), 0, s, v.lhs,
                       (const double *)v.rhs, (const double *)v.inv_diag, L, tab64(v), bnd(h), colour, omc);
        kend(h, s, l == 0 ? KC_SMOOTH0 : -1);
        return;
    }
    if (v8_ok(L)) {
        kbegin(h, s, l == 0 ? KC_SMOOTH0 : -1);
        colour_v8<double, true>(h, s, v, v.lhs, v.rhs, v.inv_diag, tab64(v), colour, 0.0, 1.0 - h->prm.sor_param);
        kend(h, s, l == 0 ? KC_SMOOTH0 : -1);
        return;
    }
    const int half = (L.n2 + 1) / 2, bx = bxfor(half);
    const double omc = 1.0 - h->prm.sor_param;
    const bool w1 = h->prm.sor_param == 1.0;
    const Bnd b = bnd(h);
    kbegin(h, s, l == 0 ? KC_SMOOTH0 : -1);
    if (h->d3) {
        if (w1)
            launch_pdl(k_rbgs64<true, true>, cgrid(L, true, half, bx), bx, 0, s, v.lhs, v.rhs, v.inv_diag, L, tab64(v),
                                                                         b, colour, omc);
        else
            launch_pdl(k_rbgs64<true, false>, cgrid(L, true, half, bx), bx, 0, s, v.lhs, v.rhs, v.inv_diag, L, tab64(v),
                                                                          b, colour, omc);
    } else {
        if (w1)
            launch_pdl(k_rbgs64<false, true>, cgrid(L, false, half, bx), bx, 0, s, v.lhs, v.rhs, v.inv_diag, L,
                                                                           tab64(v), b, colour, omc);
        else
            launch_pdl(k_rbgs64<false, false>, cgrid(L, false, half, bx), bx, 0, s, v.lhs, v.rhs, v.inv_diag, L,
                                                                            tab64(v), b, colour, omc);
    }
    kend(h, s, l == 0 ? KC_SMOOTH0 : -1);
}

void colour32(saras_mg *h, cudaStream_t s, int l, int colour) {
    Level &v = h->lv[(size_t)l];
    const Lay &L = v.lay;
    if (v.tma.ok) {
        kbegin(h, s, l == 0 ? KC_SMOOTH0 : -1);
        tma_colour(h, s, v, colour);
        kend(h, s, l == 0 ? KC_SMOOTH0 : -1);
        return;
    }
    if (v8_ok(L)) {
        kbegin(h, s, l == 0 ? KC_SMOOTH0 : -1);
        colour_v8<float, false>(h, s, v, v.e32, v.r32, (const float *)nullptr, tab32(v), colour,
                                (float)h->prm.sor_param, (float)(1.0 - h->prm.sor_param));
        kend(h, s, l == 0 ? KC_SMOOTH0 : -1);
        return;
    }
    const int half = (L.n2 + 1) / 2, bx = bxfor(half);
    const float w = (float)h->prm.sor_param, omc = (float)(1.0 - h->prm.sor_param);
    const Bnd b = bnd(h);
    kbegin(h, s, l == 0 ? KC_SMOOTH0 : -1);
    if (h->d3)
        launch_pdl(k_rbgs32<true>, cgrid(L, true, half, bx), bx, 0, s, v.e32, v.r32, L, tab32(v), b, colour, w, omc);
    else
        launch_pdl(k_rbgs32<false>, cgrid(L, false, half, bx), bx, 0, s, v.e32, v.r32, L, tab32(v), b, colour, w, omc);
    kend(h, s, l == 0 ? KC_SMOOTH0 : -1);
}

// ---- one whole FP32 red-black iteration on a small 3-D level ----
//
// On the levels between the finest ones and the single-block bottom (rows
// of at most 64 cells, 64^3 and 32^3 at 256^3) a colour launch costs about
// the same whatever its size, so k_rbgs_pair runs both colours of an
// iteration in one launch, the way k_rbgs_fused does on the large levels: a
// block stages its tile (SP_TI planes x SP_TJ rows x the whole row) with two
// halo cells of e and one of r, and the tables, in shared memory, updates
// the first colour on the tile and one halo cell around it, meets at a block
// barrier, updates the second colour on the tile and stores the tile to the
// other buffer of a ping-pong pair (no block writes what another reads).
// Every cell's arithmetic is offdiag's and diag's in their order, so the
// launch gives the bits of the two colour launches.
// Tiles of 2 planes x 2 rows: the levels are L2-resident and each launch is
// latency, so many small blocks (1024 at 64^3) beat fewer large ones in
// spite of the recomputed halo (256^3 solve: 2x2 tiles 111.6 ms, 2x4 112.6,
// 4x8 117.7, the two colour launches 112.7).
constexpr int SP_TI = 2, SP_TJ = 2, SP_THREADS = 256;
constexpr int SP_EI = SP_TI + 4, SP_EJ = SP_TJ + 4, SP_RI = SP_TI + 2, SP_RJ = SP_TJ + 2;
constexpr int SP_MAXN2 = 64;  // longest row
// per thread at SP_MAXN2: e and r vectors staged, first- and second-colour cells
constexpr int SP_EV = (SP_EI * SP_EJ * (SP_MAXN2 / 4) + SP_THREADS - 1) / SP_THREADS;
constexpr int SP_RV = (SP_RI * SP_RJ * (SP_MAXN2 / 4) + SP_THREADS - 1) / SP_THREADS;
constexpr int SP_RC = (SP_RI * SP_RJ * (SP_MAXN2 / 2) + SP_THREADS - 1) / SP_THREADS;
constexpr int SP_KC = (SP_TI * SP_TJ * (SP_MAXN2 / 2) + SP_THREADS - 1) / SP_THREADS;
static_assert(SP_RI + SP_RJ + SP_MAXN2 <= SP_THREADS, "one table entry per thread");

__device__ __forceinline__ int wrapi(int a, int n) { return ((a % n) + n) % n; }

size_t pair_smem(int n2) {
    return ((size_t)(SP_EI * SP_EJ + SP_RI * SP_RJ) * n2 + 3 * (SP_RI + SP_RJ) + 3 * (size_t)n2) * sizeof(float);
}

// One colour cell at position c of the e tile (plane offset ti and row
// offset tj in the tables' index, k its own index): offdiag, then diag.
__device__ __forceinline__ float pair_cell(const float *es, int c, int n2, int iw, int jw, int k, int n0, int n1,
                                           const Bnd &b, const float *tx, const float *ty, const float *tz, int ti,
                                           int tj, float f, float w, float omc) {
    constexpr int RS1 = 1;
    const int sj = n2, si = SP_EJ * n2;
    const float uc = es[c];
    const float xm = iw > 0 || b.per[0] ? es[c - si] : (b.sg_lo[0] > 0 ? uc : -uc);
    const float xp = iw < n0 - 1 || b.per[0] ? es[c + si] : (b.sg_hi[0] > 0 ? uc : -uc);
    const float zm = k > 0 ? es[c - RS1] : (b.per[2] ? es[c + n2 - 1] : (b.sg_lo[2] > 0 ? uc : -uc));
    const float zp = k < n2 - 1 ? es[c + RS1] : (b.per[2] ? es[c - (n2 - 1)] : (b.sg_hi[2] > 0 ? uc : -uc));
    const float ym = jw > 0 || b.per[1] ? es[c - sj] : (b.sg_lo[1] > 0 ? uc : -uc);
    const float yp = jw < n1 - 1 || b.per[1] ? es[c + sj] : (b.sg_hi[1] > 0 ? uc : -uc);
    const int nx = SP_RI, ny = SP_RJ;
    float sm = tx[ti] * xm;
    sm = fmat(tx[nx + ti], xp, sm);
    sm = fmat(ty[tj], ym, sm);
    sm = fmat(ty[ny + tj], yp, sm);
    sm = fmat(tz[k], zm, sm);
    sm = fmat(tz[n2 + k], zp, sm);
    const float sv = sm - f;
    float d = tx[2 * nx + ti] + tz[2 * n2 + k];
    d += ty[2 * ny + tj];
    return fmat(omc, uc, sweep_div(w * sv, d + d));
}

__global__ void __launch_bounds__(SP_THREADS) k_rbgs_pair(const float *__restrict__ src, float *__restrict__ dst,
                                                          const float *__restrict__ r, Lay L, Tab3<float> t, Bnd b,
                                                          float w, float omc) {
    extern __shared__ __align__(16) float sp[];
    const int n0 = L.n0, n1 = L.n1, n2 = L.n2, n4 = n2 >> 2, h2 = n2 >> 1;
    float *es = sp;                             // planes i0-2 .. i0+TI+1, rows j0-2 .. j0+TJ+1
    float *rs = es + SP_EI * SP_EJ * n2;        // planes i0-1 .. i0+TI, rows j0-1 .. j0+TJ
    float *tx = rs + SP_RI * SP_RJ * n2;        // cm, cp, dg of planes i0-1 .. i0+TI
    float *ty = tx + 3 * SP_RI;                 // ... of rows j0-1 .. j0+TJ
    float *tz = ty + 3 * SP_RJ;                 // ... of k
    const int i0 = (int)blockIdx.y * SP_TI, j0 = (int)blockIdx.x * SP_TJ;
    const bool px = b.per[0] != 0, py = b.per[1] != 0;
    pdl_enter();
    // Staging: a thread issues all of its loads (at most SP_EV e vectors,
    // SP_RV r vectors and one table entry) before it stores any, so the
    // block waits for one round trip to L2.  Planes and rows outside a wall
    // are not loaded (the stencil mirrors); on a periodic axis they are the
    // wrapped ones.
    {
        float4 ev[SP_EV], rv[SP_RV];
        int eo[SP_EV], ro[SP_RV];
#pragma unroll
        for (int m = 0; m < SP_EV; m++) {
            const int x = threadIdx.x + m * SP_THREADS;
            eo[m] = -1;
            if (x >= SP_EI * SP_EJ * n4) continue;
            const int k4 = x % n4, row = x / n4, jj = row % SP_EJ, ii = row / SP_EJ;
            int ig = i0 - 2 + ii, jg = j0 - 2 + jj;
            if (px) ig = wrapi(ig, n0); else if (ig < 0 || ig >= n0) continue;
            if (py) jg = wrapi(jg, n1); else if (jg < 0 || jg >= n1) continue;
            ev[m] = __ldg(reinterpret_cast<const float4 *>(src + L.at(ig, jg, 4 * k4)));
            eo[m] = row * n2 + 4 * k4;
        }
#pragma unroll
        for (int m = 0; m < SP_RV; m++) {
            const int x = threadIdx.x + m * SP_THREADS;
            ro[m] = -1;
            if (x >= SP_RI * SP_RJ * n4) continue;
            const int k4 = x % n4, row = x / n4, jj = row % SP_RJ, ii = row / SP_RJ;
            int ig = i0 - 1 + ii, jg = j0 - 1 + jj;
            if (px) ig = wrapi(ig, n0); else if (ig < 0 || ig >= n0) continue;
            if (py) jg = wrapi(jg, n1); else if (jg < 0 || jg >= n1) continue;
            rv[m] = __ldg(reinterpret_cast<const float4 *>(r + L.at(ig, jg, 4 * k4)));
            ro[m] = row * n2 + 4 * k4;
        }
        // tables: entry x < SP_RI + SP_RJ + n2 (at most SP_THREADS)
        const int x = threadIdx.x;
        float tv[3];
        float *dt = nullptr;
        int st = 0;
        if (x < SP_RI) {
            const int q = px ? wrapi(i0 - 1 + x, n0) : min(max(i0 - 1 + x, 0), n0 - 1);
            tv[0] = __ldg(t.cm[0] + q), tv[1] = __ldg(t.cp[0] + q), tv[2] = __ldg(t.dg[0] + q);
            dt = tx + x, st = SP_RI;
        } else if (x < SP_RI + SP_RJ) {
            const int q = py ? wrapi(j0 - 1 + x - SP_RI, n1) : min(max(j0 - 1 + x - SP_RI, 0), n1 - 1);
            tv[0] = __ldg(t.cm[1] + q), tv[1] = __ldg(t.cp[1] + q), tv[2] = __ldg(t.dg[1] + q);
            dt = ty + (x - SP_RI), st = SP_RJ;
        } else if (x < SP_RI + SP_RJ + n2) {
            const int q = x - SP_RI - SP_RJ;
            tv[0] = __ldg(t.cm[2] + q), tv[1] = __ldg(t.cp[2] + q), tv[2] = __ldg(t.dg[2] + q);
            dt = tz + q, st = n2;
        }
#pragma unroll
        for (int m = 0; m < SP_EV; m++)
            if (eo[m] >= 0) *reinterpret_cast<float4 *>(es + eo[m]) = ev[m];
#pragma unroll
        for (int m = 0; m < SP_RV; m++)
            if (ro[m] >= 0) *reinterpret_cast<float4 *>(rs + ro[m]) = rv[m];
        if (dt) {
            dt[0] = tv[0];
            dt[st] = tv[1];
            dt[2 * st] = tv[2];
        }
    }
    __syncthreads();
    // first colour ((i + j + k) even) on the tile and one halo cell around
    // it; a colour's cells read only the other colour, so a thread forms all
    // of its cells before it writes any
    {
        float nv[SP_RC];
        int co[SP_RC];
#pragma unroll
        for (int m = 0; m < SP_RC; m++) {
            const int x = threadIdx.x + m * SP_THREADS;
            co[m] = -1;
            if (x >= SP_RI * SP_RJ * h2) continue;
            const int kk = x % h2, row = x / h2, jj = row % SP_RJ, ii = row / SP_RJ;
            int iw = i0 - 1 + ii, jw = j0 - 1 + jj;
            if (px) iw = wrapi(iw, n0); else if (iw < 0 || iw >= n0) continue;
            if (py) jw = wrapi(jw, n1); else if (jw < 0 || jw >= n1) continue;
            const int k = 2 * kk + ((iw + jw) & 1);
            if (k >= n2) continue;
            const int c = ((ii + 1) * SP_EJ + (jj + 1)) * n2 + k;
            nv[m] = pair_cell(es, c, n2, iw, jw, k, n0, n1, b, tx, ty, tz, ii, jj, rs[row * n2 + k], w, omc);
            co[m] = c;
        }
#pragma unroll
        for (int m = 0; m < SP_RC; m++)
            if (co[m] >= 0) es[co[m]] = nv[m];
    }
    __syncthreads();
    // second colour on the tile
    {
        float nv[SP_KC];
        int co[SP_KC];
#pragma unroll
        for (int m = 0; m < SP_KC; m++) {
            const int x = threadIdx.x + m * SP_THREADS;
            co[m] = -1;
            if (x >= SP_TI * SP_TJ * h2) continue;
            const int kk = x % h2, row = x / h2, jj = row % SP_TJ, ii = row / SP_TJ;
            const int iw = i0 + ii, jw = j0 + jj;
            const int k = 2 * kk + 1 - ((iw + jw) & 1);
            if (k >= n2) continue;
            const int c = ((ii + 2) * SP_EJ + (jj + 2)) * n2 + k;
            nv[m] = pair_cell(es, c, n2, iw, jw, k, n0, n1, b, tx, ty, tz, ii + 1, jj + 1,
                              rs[((ii + 1) * SP_RJ + (jj + 1)) * n2 + k], w, omc);
            co[m] = c;
        }
#pragma unroll
        for (int m = 0; m < SP_KC; m++)
            if (co[m] >= 0) es[co[m]] = nv[m];
    }
    __syncthreads();
    for (int x = threadIdx.x; x < SP_TI * SP_TJ * n4; x += blockDim.x) {
        const int k4 = x % n4, row = x / n4, jj = row % SP_TJ, ii = row / SP_TJ;
        *reinterpret_cast<float4 *>(dst + L.at(i0 + ii, j0 + jj, 4 * k4)) =
            *reinterpret_cast<const float4 *>(es + ((ii + 2) * SP_EJ + (jj + 2)) * n2 + 4 * k4);
    }
}

// Coarsest level: the FP64_EXACT single-block solve (or smoothing), shared
// by all forms; declared in mg.cu.
}  // namespace

namespace saras {
void coarsest_level(saras_mg *h, cudaStream_t s);
void norm_final(saras_mg *h, cudaStream_t s);
void ghost_all_level(saras_mg *h, cudaStream_t s, int l, bool zeroBC);

// Levels that take k_rbgs_pair (and hold a second e buffer for it): 3-D,
// rows of 8 to 64 cells in whole float4s, planes and rows that divide into
// tiles, not a level of the large fused iteration.
bool pair_sweep_fits(const Lay &L, bool d3) {
    return d3 && L.n2 >= 8 && L.n2 <= SP_MAXN2 && L.n2 % 4 == 0 && L.n0 % SP_TI == 0 && L.n1 % SP_TJ == 0 &&
           !fused_sweep_fits(L, d3);
}
}  // namespace saras

namespace {

void residual_restrict(saras_mg *h, cudaStream_t s, int l, bool mixed) {
    Level &f = h->lv[(size_t)l];
    Level &c = h->lv[(size_t)l + 1];
    const Lay &Lc = c.lay;
    const int bx = bxfor(Lc.n2);
    const Bnd b = bnd(h);
    const bool to64 = l + 1 == h->nl - 1;  // the coarsest level is FP64 in every form
    // the coarse level's iterate starts from zero; the restriction clears it
    // (the coarsest solve clears its own)
    double *z64 = to64 ? nullptr : c.lhs;
    float *z32 = to64 ? nullptr : c.e32;
    const dim3 gs = cgrid(Lc, h->d3, Lc.n2, bx);
    kbegin(h, s, l == 0 ? KC_RESTRICT : -1);
    if (v8_ok(f.lay) && (!mixed || !to64)) {
        const int strips = Lc.n2 / 4, bx4 = std::min(strips, 32), by = h->d3 ? std::max(1, 128 / bx4) : 1;
        const dim3 g4(cdiv(strips, bx4), h->d3 ? cdiv(Lc.n1, by) : 1u, (unsigned)Lc.n0);
        const dim3 blk(bx4, by);
        if (!mixed && h->d3 && (int64_t)Lc.n0 * Lc.n1 * Lc.n2 >= (int64_t(1) << 17)) {
            // the large levels: two coarse cells per thread
            const int pairs = Lc.n2 / 2, bx2 = std::min(pairs, 64), by2 = std::max(1, 128 / bx2);
            const dim3 g2(cdiv(pairs, bx2), cdiv(Lc.n1, by2), (unsigned)Lc.n0);
            launch_pdl(k_resid_restrict4d<true>, g2, dim3(bx2, by2), 0, s, (const double *)f.lhs,
                       (const double *)f.rhs, f.lay, tab64(f), b, wt64(c), c.rhs, Lc, (const double *)f.dd, z64);
        } else if (!mixed) {
            if (h->d3)
                launch_pdl(k_resid_restrict8<double, true>, g4, blk, 0, s, f.lhs, f.rhs, f.lay, tab64(f), b, wt64(c),
                           c.rhs, Lc, f.dd, z64);
            else
                launch_pdl(k_resid_restrict8<double, false>, g4, blk, 0, s, f.lhs, f.rhs, f.lay, tab64(f), b,
                           wt64(c), c.rhs, Lc, f.dd, z64);
        } else {
            // FP32: two coarse cells per thread
            const int pairs = Lc.n2 / 2, bx2 = std::min(pairs, 64), by2 = h->d3 ? std::max(1, 256 / bx2) : 1;
            const dim3 g2(cdiv(pairs, bx2), h->d3 ? cdiv(Lc.n1, by2) : 1u, (unsigned)Lc.n0);
            if (h->d3 && tma_resid_restrict(h, s, f, c, tab32(f), wt32(c), z32)) {
                // the large levels: planes through the TMA pipeline, the same bits
            } else if (h->d3)
                launch_pdl(f.rs ? k_resid_restrict4<true, true> : k_resid_restrict4<true, false>, g2, dim3(bx2, by2),
                           0, s, f.e32, f.r32, f.lay, tab32(f), b, wt32(c), c.r32, Lc, z32);
            else
                launch_pdl(k_resid_restrict4<false, false>, g2, dim3(bx2, by2), 0, s, f.e32, f.r32, f.lay, tab32(f),
                           b, wt32(c), c.r32, Lc, z32);
        }
    } else if (!mixed) {
        if (h->d3)
            launch_pdl(k_resid_restrict<double, double, true>, gs, bx, 0, s, f.lhs, f.rhs, f.lay, tab64(f), b,
                       wt64(c), c.rhs, Lc, f.dd, z64);
        else
            launch_pdl(k_resid_restrict<double, double, false>, gs, bx, 0, s, f.lhs, f.rhs, f.lay, tab64(f), b,
                       wt64(c), c.rhs, Lc, f.dd, z64);
    } else if (to64) {
        if (h->d3)
            launch_pdl(k_resid_restrict<float, double, true>, gs, bx, 0, s, f.e32, f.r32, f.lay, tab32(f), b,
                       wt32(c), c.rhs, Lc, (const float *)nullptr, (double *)nullptr);
        else
            launch_pdl(k_resid_restrict<float, double, false>, gs, bx, 0, s, f.e32, f.r32, f.lay, tab32(f), b,
                       wt32(c), c.rhs, Lc, (const float *)nullptr, (double *)nullptr);
    } else {
        if (h->d3)
            launch_pdl(k_resid_restrict<float, float, true>, gs, bx, 0, s, f.e32, f.r32, f.lay, tab32(f), b,
                       wt32(c), c.r32, Lc, (const float *)nullptr, z32);
        else
            launch_pdl(k_resid_restrict<float, float, false>, gs, bx, 0, s, f.e32, f.r32, f.lay, tab32(f), b,
                       wt32(c), c.r32, Lc, (const float *)nullptr, z32);
    }
    kend(h, s, l == 0 ? KC_RESTRICT : -1);
}

void prolong_add(saras_mg *h, cudaStream_t s, int l, bool mixed) {
    Level &c = h->lv[(size_t)l];
    Level &f = h->lv[(size_t)l - 1];
    const Lay &L = f.lay;
    const int bx = bxfor(L.n2);
    const dim3 g(cdiv(L.n2, bx), (unsigned)L.n1, (unsigned)L.n0);
    kbegin(h, s, l == 1 ? KC_PROLONG : -1);
    const bool to_top = l == h->nl - 1;
    if (v8_ok(L) && (!mixed || !to_top)) {
        const int strips = L.n2 / 8, bx8 = std::min(strips, 32), by = h->d3 ? std::max(1, 128 / bx8) : 1;
        const dim3 g8(cdiv(strips, bx8), cdiv(L.n1, by), (unsigned)L.n0);
        if (!mixed)
            launch_pdl(k_prolong_add8<double>, g8, dim3(bx8, by), 0, s, f.lhs, c.lhs, L, c.lay, h->d3 ? 1 : 0);
        else if (f.rs)
            launch_pdl(k_prolong_add8_rs, g8, dim3(bx8, by), 0, s, f.e32, c.e32, L, c.lay);
        else
            launch_pdl(k_prolong_add8<float>, g8, dim3(bx8, by), 0, s, f.e32, c.e32, L, c.lay, h->d3 ? 1 : 0);
    } else if (!mixed)
        launch_pdl(k_prolong_add<double, double>, g, bx, 0, s, f.lhs, c.lhs, L, c.lay, h->d3 ? 1 : 0);
    else if (l == h->nl - 1)
        launch_pdl(k_prolong_add<float, double>, g, bx, 0, s, f.e32, c.lhs, L, c.lay, h->d3 ? 1 : 0);
    else
        launch_pdl(k_prolong_add<float, float>, g, bx, 0, s, f.e32, c.e32, L, c.lay, h->d3 ? 1 : 0);
    kend(h, s, l == 1 ? KC_PROLONG : -1);
}

void smooth(saras_mg *h, cudaStream_t s, int l, int count, bool mixed) {
    int n = 0;
    Level &v = h->lv[(size_t)l];
    if (mixed && v.tma.fok) {
        // pairs of iterations through the fused kernel, e32 -> e32b -> e32;
        // an odd last one takes the colour sweeps below
        for (; n + 2 <= count; n += 2)
            for (int half = 0; half < 2; half++) {
                kbegin(h, s, l == 0 ? KC_SMOOTH0 : -1);
                tma_fused(h, s, v, half == 0);
                kend(h, s, l == 0 ? KC_SMOOTH0 : -1);
            }
    } else if (mixed && v.e32b && pair_sweep_fits(v.lay, h->d3)) {
        const Lay &L = v.lay;
        const dim3 grid((unsigned)(L.n1 / SP_TJ), (unsigned)(L.n0 / SP_TI));
        const float w = (float)h->prm.sor_param, omc = (float)(1.0 - h->prm.sor_param);
        for (; n + 2 <= count; n += 2)
            for (int half = 0; half < 2; half++) {
                kbegin(h, s, l == 0 ? KC_SMOOTH0 : -1);
                launch_pdl(k_rbgs_pair, grid, SP_THREADS, pair_smem(L.n2), s, half == 0 ? v.e32 : v.e32b,
                           half == 0 ? v.e32b : v.e32, v.r32, L, tab32(v), bnd(h), w, omc);
                kend(h, s, l == 0 ? KC_SMOOTH0 : -1);
            }
    }
    for (; n < count; n++) {
        if (mixed) {
            colour32(h, s, l, 0);
            colour32(h, s, l, 1);
        } else {
            colour64(h, s, l, 0);
            colour64(h, s, l, 1);
        }
    }
}

void resid_norm(saras_mg *h, cudaStream_t s, bool mixed) {
    Level &v = h->lv[0];
    const Bnd b = bnd(h);
    kbegin(h, s, KC_NORM);
    if (h->d3) {
        if (mixed)
            k_resid_norm64<true, true><<<h->norm_blocks, 256, 0, s>>>(v.lhs, v.rhs, v.dd, v.lay, tab64(v), b,
                                                                      h->prm.res_type, h->norm_part, v.r32, v.rs);
        else
            k_resid_norm64<true, false><<<h->norm_blocks, 256, 0, s>>>(v.lhs, v.rhs, v.dd, v.lay, tab64(v), b,
                                                                       h->prm.res_type, h->norm_part, nullptr, 0);
    } else {
        if (mixed)
            k_resid_norm64<false, true><<<h->norm_blocks, 256, 0, s>>>(v.lhs, v.rhs, v.dd, v.lay, tab64(v), b,
                                                                       h->prm.res_type, h->norm_part, v.r32, v.rs);
        else
            k_resid_norm64<false, false><<<h->norm_blocks, 256, 0, s>>>(v.lhs, v.rhs, v.dd, v.lay, tab64(v), b,
                                                                        h->prm.res_type, h->norm_part, nullptr, 0);
    }
    kend(h, s, KC_NORM);
    norm_final(h, s);
}

bool singular(const saras_mg *h) {
    for (int d = 0; d < 3; d++) {
        if (!h->grid.active(d) || h->ghost.per[d]) continue;
        if (h->ghost.kind[2 * d] != SARAS_BC_NEUMANN || h->ghost.kind[2 * d + 1] != SARAS_BC_NEUMANN) return false;
    }
    return true;
}

void csum(saras_mg *h, cudaStream_t s, const double *u, int slot) {
    const Lay &L = h->lv[0].lay;
    const double count = (double)L.n0 * L.n1 * L.n2;
    kbegin(h, s, -1);
    k_csum<<<h->norm_blocks, 256, 0, s>>>(u, L, h->norm_part);
    kbegin(h, s, -1);
    k_csum_final<<<1, 32, 0, s>>>(h->norm_part, h->norm_blocks, count, h->mix_scalar, slot);
}

}  // namespace

namespace saras {

// Tables of the MIXED form's exact coarsest solve: per axis the
// eigen-decomposition of the coarsest level's 1-D operator (coefficients as
// build_tables forms them, the handle's ghost rule folded in).  The exact
// solve stands in for sweeps run to a tight coarsest tolerance (at most
// FD_TOL_MAX) on a coarsest level of FD_MIN_CELLS or more cells, where the
// sweeps cost the most (12x12x6: about ten times the whole rest of the
// cycle) for the same outer iterations.  A looser tolerance keeps the sweeps,
// whose early stop damps the injection-prolonged correction (128^3,
// tolerance 1e-6: 4 outer iterations with the sweeps, 6 with the exact
// solve); so do small coarsest levels, where sweeps are cheap, and an axis
// that cannot be decomposed (a stretched periodic axis).
saras_status build_fd(saras_mg *h) {
    Level &c = h->lv[(size_t)h->nl - 1];
    c.fdv = FDiag{};
    if (!c.fd || h->prm.precision != SARAS_PREC_MIXED || h->prm.mg_tolerance > FD_TOL_MAX) return SARAS_OK;
    const HostGrid &g = h->grid;
    const int l = h->nl - 1;
    const int n[3] = {c.lay.n0, c.lay.n1, c.lay.n2};
    std::vector<double> host((size_t)fd_elems(c.lay), 0.0);
    FDiag f{};
    size_t off = 0;
    double lmax = 0.0;
    for (int d = 0; d < 3; d++) {
        const size_t nn = (size_t)n[d] * n[d];
        double *V = host.data() + off, *Vi = V + nn, *lam = Vi + nn;
        if (!g.active(d)) {
            V[0] = 1.0;
            Vi[0] = 1.0;
            lam[0] = 0.0;
        } else {
            const AxisLevel &a = g.lv[(size_t)l][(size_t)d];
            const double hx = (1 << l) * g.dxi[d];
            const double ih2 = 1.0 / std::pow(hx, 2), i2h = 0.5 / hx;
            std::vector<double> cm((size_t)n[d]), cp((size_t)n[d]), a2((size_t)n[d]);
            for (int i = 0; i < n[d]; i++) {
                const double A2 = a.at(a.xix2, i) * ih2, A1 = a.at(a.xixx, i) * i2h;
                cm[(size_t)i] = A2 - A1;
                cp[(size_t)i] = A2 + A1;
                a2[(size_t)i] = A2;
            }
            const int sl = h->ghost.kind[2 * d] == SARAS_BC_NEUMANN ? 1 : -1;
            const int sh = h->ghost.kind[2 * d + 1] == SARAS_BC_NEUMANN ? 1 : -1;
            if (!coarse_axis_eigen(n[d], cm.data(), cp.data(), a2.data(), h->ghost.per[d] != 0, sl, sh, V, Vi, lam))
                return SARAS_OK;
        }
        double m = 0.0;
        for (int k = 0; k < n[d]; k++) m = std::max(m, std::fabs(lam[k]));
        lmax += m;
        f.v[d] = c.fd + off;
        f.vi[d] = c.fd + off + nn;
        f.lam[d] = c.fd + off + 2 * nn;
        off += 2 * nn + (size_t)n[d];
    }
    const size_t bytes = host.size() * sizeof(double);
    if (h->tab_stage && h->tab_stage_bytes >= h->tab_stage_used + bytes) {
        // pinned staging of a re-pointed handle: no wait for the stream
        char *st = h->tab_stage + h->tab_stage_used;
        std::memcpy(st, host.data(), bytes);
        h->tab_stage_used += (bytes + 255) / 256 * 256;
        SARAS_CUDA(cudaMemcpyAsync(c.fd, st, bytes, cudaMemcpyHostToDevice, h->stream));
    } else {
        // pageable source: staged before the call returns, ordered on the stream
        SARAS_CUDA(cudaMemcpyAsync(c.fd, host.data(), bytes, cudaMemcpyHostToDevice, h->stream));
    }
    f.lam_tol = 1e-9 * lmax;
    f.ok = 1;
    c.fdv = f;
    return SARAS_OK;
}

void bottom_plan(saras_mg *h);

saras_status fast_setup(saras_mg *h) {
    for (int f = 0; f < 6; f++)
        if (h->prm.bc_kind[f] == SARAS_BC_DIRICHLET_TEST) {
            set_error("the TEST_POISSON wall kind is available in the FP64_EXACT form only");
            return SARAS_BAD_ARG;
        }
    for (int l = 0; l < h->nl; l++) {
        Level &v = h->lv[(size_t)l];
        if (!v.inv_diag && !v.dd) continue;
        const Lay &L = v.lay;
        const int bx = bxfor(L.n2);
        if (h->d3)
            k_inv_diag<true><<<cgrid(L, true, L.n2, bx), bx, 0, h->stream>>>(v.inv_diag, v.dd, L, tab64(v),
                                                                           h->prm.sor_param);
        else
            k_inv_diag<false><<<cgrid(L, false, L.n2, bx), bx, 0, h->stream>>>(v.inv_diag, v.dd, L, tab64(v),
                                                                            h->prm.sor_param);
    }
    if (h->prm.precision == SARAS_PREC_MIXED)
        for (int l = 0; l < h->nl; l++) tma_plan(h, h->lv[(size_t)l]);
    // the finest level's FP32 arrays are row-split when every smoothing
    // iteration there is a fused pair (even counts): its only other readers
    // and writers (FP64 residual, update, restriction, prolongation) follow
    {
        Level &v0 = h->lv[0];
        v0.rs = !h->no_rowsplit && h->prm.precision == SARAS_PREC_MIXED && h->d3 && v0.tma.fok &&
                        fused_rowsplit_fits(v0.lay, h->d3) &&
                        h->prm.pre_smooth % 2 == 0 && h->prm.post_smooth % 2 == 0
                    ? 1
                    : 0;
    }
    SARAS_TRY(build_fd(h));
    bottom_plan(h);
    SARAS_CUDA(cudaFuncSetAttribute(k_coarsest_fd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    2 * FD_MAX_CELLS * (int)sizeof(double)));
    SARAS_CUDA(cudaFuncSetAttribute(k_coarsest_fast<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    200 * 1024));
    SARAS_CUDA(cudaFuncSetAttribute(k_coarsest_fast<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    200 * 1024));
    SARAS_CUDA(cudaGetLastError());
    return SARAS_OK;
}

// The MIXED form's single-block bottom (k_bottom): the FP32 levels above
// the coarsest whose colour sweeps are at most BOT_CPT cells per thread, as
// long as everything the block keeps fits BOT_SMEM bytes of shared memory.
// Needs a 3-D hierarchy and a coarsest level swept in registers (no exact
// solve).  At 256^3 it holds 16^3, 8^3 and 4^3 and replaces twenty-one
// launches per V-cycle.
constexpr size_t BOT_SMEM = 160 * 1024;

int64_t bot_ncol(const Lay &L) { return (int64_t)L.n0 * L.n1 * ((L.n2 + 1) / 2); }

// k_bottom's shared memory when it holds levels lb .. the coarsest: the
// offsets go to `a`, the bytes are returned.
size_t bot_layout(const saras_mg *h, int lb, BotArgs *a) {
    const int top = h->nl - 1;
    auto al = [](size_t x) { return (x + 15) / 16 * 16; };
    size_t off = 0;
    for (int m = 0; m < top - lb; m++) {
        const Lay &L = h->lv[(size_t)(lb + m)].lay, &Ln = h->lv[(size_t)(lb + m + 1)].lay;
        a->off[2 * m] = (unsigned)off;
        off += al((size_t)L.size * sizeof(float));
        a->off[2 * m + 1] = (unsigned)off;
        off += al((size_t)L.size * sizeof(float));
        a->toff[m] = (unsigned)off;
        off += al((size_t)(3 * (L.n0 + L.n1 + L.n2) + 2 * (Ln.n0 + Ln.n1 + Ln.n2)) * sizeof(float));
        a->loff[m] = (unsigned)off;
        off += al((size_t)bot_ncol(L) * sizeof(unsigned));
    }
    const Lay &C = h->lv[(size_t)top].lay;
    for (int q = 0; q < 4; q++) {
        a->off[2 * BOT_MAX + q] = (unsigned)off;
        off += al((size_t)C.size * sizeof(double));
    }
    a->tcoff = (unsigned)off;
    off += al((size_t)3 * (C.n0 + C.n1 + C.n2) * sizeof(double));
    return off;
}

void bottom_plan(saras_mg *h) {
    h->bottom = -1;
    h->bottom_smem = 0;
    if (h->prm.precision != SARAS_PREC_MIXED || !h->d3 || h->nl < 3 || !h->prm.solve_flag) return;
    const int top = h->nl - 1;
    const Level &c = h->lv[(size_t)top];
    if (c.fdv.ok) return;
    const Lay &C = c.lay;
    // the coarsest solve keeps one cell of each colour and two residual
    // cells per thread in registers
    if (bot_ncol(C) > BOT_THREADS || (int64_t)C.n0 * C.n1 * C.n2 > 2 * BOT_THREADS) return;
    BotArgs tmp{};
    int lb = top;
    while (lb - 1 >= 1 && top - (lb - 1) <= BOT_MAX) {
        // a level joins while its colour sweep is at most BOT_CPT cells per
        // thread (the packed cell lists need i < 4096, j < 1024, k < 2048),
        // each of its cells has its parent on the next level, and the
        // block's shared memory stays within BOT_SMEM
        const Lay &L = h->lv[(size_t)lb - 1].lay, &Ln = h->lv[(size_t)lb].lay;
        if (bot_ncol(L) > (int64_t)BOT_CPT * BOT_THREADS || L.n0 >= 4096 || L.n1 >= 1024 || L.n2 >= 2048) break;
        if (L.n0 > 2 * Ln.n0 || L.n1 > 2 * Ln.n1 || L.n2 > 2 * Ln.n2) break;
        if (bot_layout(h, lb - 1, &tmp) > BOT_SMEM) break;
        lb--;
    }
    if (lb >= top) return;
    if (cudaFuncSetAttribute(k_bottom<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)BOT_SMEM) !=
        cudaSuccess) {
        cudaGetLastError();
        return;
    }
    h->bottom = lb;
    h->bottom_smem = bot_layout(h, lb, &tmp);
}

void bottom(saras_mg *h, cudaStream_t s) {
    const int lb = h->bottom, top = h->nl - 1;
    BotArgs a{};
    a.nb = top - lb;
    const size_t smem = bot_layout(h, lb, &a);
    for (int m = 0; m < a.nb; m++) {
        const Level &v = h->lv[(size_t)(lb + m)];
        a.L[m] = v.lay;
        a.t[m] = tab32(v);
        a.w[m + 1] = wt32(h->lv[(size_t)(lb + m + 1)]);
    }
    const Level &c = h->lv[(size_t)top];
    a.Lc = c.lay;
    a.tc = tab64(c);
    a.wdc = c.inv_diag;
    a.ddc = c.dd;
    a.r_top = h->lv[(size_t)lb].r32;
    a.e_top = h->lv[(size_t)lb].e32;
    a.b = bnd(h);
    a.w32 = (float)h->prm.sor_param;
    a.omc32 = (float)(1.0 - h->prm.sor_param);
    a.omc64 = 1.0 - h->prm.sor_param;
    a.tol = h->prm.mg_tolerance;
    a.max_count = h->maxCount();
    a.stall = COARSE_STALL_CHECK;
    a.pre = h->prm.pre_smooth;
    a.post = h->prm.post_smooth;
    a.sweeps_out = h->coarse_sweeps;
    kbegin(h, s, KC_COARSE);
    launch_pdl(k_bottom<true>, 1, BOT_THREADS, smem, s, a);
    kend(h, s, KC_COARSE);
}

// One V-cycle over the whole hierarchy: u (FP64 form) or e (MIXED form) at
// the finest level is smoothed from its current value.
void vcycle_fast(saras_mg *h, cudaStream_t s, bool mixed) {
    const int top = h->nl - 1;
    smooth(h, s, 0, h->prm.pre_smooth, mixed);
    const int lb = mixed ? h->bottom : -1;
    if (lb > 0) {
        // down to level lb, the bottom in one block, up from level lb
        for (int l = 0; l < lb; l++) {
            residual_restrict(h, s, l, mixed);
            if (l + 1 < lb) smooth(h, s, l + 1, h->prm.pre_smooth, mixed);
        }
        bottom(h, s);
        for (int l = lb; l > 0; l--) {
            prolong_add(h, s, l, mixed);
            smooth(h, s, l - 1, h->prm.post_smooth, mixed);
        }
        return;
    }
    for (int l = 0; l < top; l++) {
        residual_restrict(h, s, l, mixed);
        if (l + 1 == top)
            coarsest_level(h, s);
        else
            smooth(h, s, l + 1, h->prm.pre_smooth, mixed);
    }
    for (int l = top; l > 0; l--) {
        prolong_add(h, s, l, mixed);
        smooth(h, s, l - 1, h->prm.post_smooth, mixed);
    }
}

// One V-cycle of the FP64 form, or one outer iteration of the MIXED form:
// `inner_cycles` FP32 V-cycles on the error equation A e = r (the first from
// e = 0, the others from the current e), then the FP64 update and residual.
void fast_cycle(saras_mg *h, cudaStream_t s) {
    const bool mixed = h->prm.precision == SARAS_PREC_MIXED;
    if (!mixed) {
        vcycle_fast(h, s, false);
        resid_norm(h, s, false);
        return;
    }
    mixed_head(h, s);
    const int inner = mixed_inner(h);
    for (int q = 0; q < inner; q++) vcycle_fast(h, s, true);
    mixed_tail(h, s);
}

// FP32 V-cycles of the current outer iteration: inner_cycles, or with a
// negative inner_cycles (adaptive) the count the solve loop chose, at most
// -inner_cycles.
int mixed_inner(const saras_mg *h) {
    const int n = h->prm.inner_cycles;
    if (n > 0) return n;
    return h->inner_now > 0 ? h->inner_now : std::max(1, -n);
}

// The error equation at the finest level starts from zero.
void mixed_head(saras_mg *h, cudaStream_t s) {
    Level &v0 = h->lv[0];
    cudaMemsetAsync(v0.e32, 0, (size_t)v0.lay.size * sizeof(float), s);
}

// u += e (FP64), then the FP64 residual, its norm and the FP32 residual the
// next outer iteration starts from.
void mixed_tail(saras_mg *h, cudaStream_t s) {
    Level &v0 = h->lv[0];
    const Lay &L = v0.lay;
    const int bx = bxfor(L.n2);
    kbegin(h, s, -1);
    launch_pdl(k_update64, dim3(cdiv(L.n2, bx), (unsigned)L.n1, (unsigned)L.n0), bx, 0, s, v0.lhs, v0.e32, L,
               v0.rs);
    resid_norm(h, s, true);
}

void mixed_prepare(saras_mg *h, cudaStream_t s) {
    // residual of the initial guess feeds the first FP32 V-cycle; the mean
    // of the guess is kept for the null-space projection
    resid_norm(h, s, true);
    if (singular(h)) csum(h, s, h->lv[0].lhs, 1);
}

void final_ghosts(saras_mg *h, cudaStream_t s) { ghost_all_level(h, s, 0, false); }

void rhs_norm(saras_mg *h, cudaStream_t s) {
    Level &v = h->lv[0];
    kbegin(h, s, -1);
    k_rhs_norm<<<h->norm_blocks, 256, 0, s>>>(v.rhs, v.lay, h->prm.res_type, h->norm_part);
    kbegin(h, s, -1);
    k_rhs_norm_final<<<1, 32, 0, s>>>(h->norm_part, h->norm_blocks, h->prm.res_type, h->norm_out + 4);
}

void coarsest_fast(saras_mg *h, cudaStream_t s, Level &c) {
    const Lay &C = c.lay;
    if (h->prm.precision == SARAS_PREC_MIXED && c.fdv.ok) {
        // the MIXED form solves its coarsest level exactly (fd_solve)
        const int64_t cells = (int64_t)C.n0 * C.n1 * C.n2;
        const int threads = cells <= 512 ? 64 : 256;
        kbegin(h, s, KC_COARSE);
        launch_pdl(k_coarsest_fd, 1, threads, (size_t)(2 * cells) * sizeof(double), s, c.lhs, c.rhs, C, c.fdv);
        kend(h, s, KC_COARSE);
        return;
    }
    const size_t smem = (size_t)(4 * C.size) * sizeof(double);
    if (smem > 200 * 1024) {  // coarsest grid too large for one block's shared memory
        cudaMemsetAsync(c.lhs, 0, (size_t)C.size * sizeof(double), s);
        smooth(h, s, h->nl - 1, std::max(1, h->prm.pre_smooth), false);
        return;
    }
    const int64_t cells = (int64_t)C.n0 * C.n1 * C.n2;
    // up to 512 cells: one thread per cell of a colour (k_coarsest_fast's
    // register-cached sweeps); larger grids loop over their cells
    const int64_t ncol = (int64_t)C.n0 * C.n1 * ((C.n2 + 1) / 2);
    const int threads = ncol <= 256 ? (int)std::max<int64_t>(32, (ncol + 31) / 32 * 32)
                                    : (cells <= 4096 ? 128 : 256);
    const Bnd b = bnd(h);
    // the MIXED form also stops a stagnating coarsest solve; the FP64 form
    // keeps mgSolve's tolerance-or-cap rule
    const int stall = h->prm.precision == SARAS_PREC_MIXED ? COARSE_STALL_CHECK : 0;
    kbegin(h, s, KC_COARSE);
    if (h->d3)
        launch_pdl(k_coarsest_fast<true>, 1, threads, smem, s, c.lhs, c.rhs, c.inv_diag, c.dd, C, tab64(c), b,
                   1.0 - h->prm.sor_param, h->prm.mg_tolerance, h->maxCount(), stall, h->coarse_sweeps);
    else
        launch_pdl(k_coarsest_fast<false>, 1, threads, smem, s, c.lhs, c.rhs, c.inv_diag, c.dd, C, tab64(c), b,
                   1.0 - h->prm.sor_param, h->prm.mg_tolerance, h->maxCount(), stall, h->coarse_sweeps);
    kend(h, s, KC_COARSE);
}

void mixed_finish(saras_mg *h, cudaStream_t s) {
    if (singular(h)) {
        // remove the drift of the constant null-space component: the mean of
        // the result returns to the mean of the initial guess
        csum(h, s, h->lv[0].lhs, 0);
        const Lay &L = h->lv[0].lay;
        const int bx = bxfor(L.n2);
        kbegin(h, s, -1);
        k_shift<<<dim3(cdiv(L.n2, bx), (unsigned)L.n1, (unsigned)L.n0), bx, 0, s>>>(h->lv[0].lhs, L, h->mix_scalar);
    }
    final_ghosts(h, s);
}

double kernel_bytes(const saras_mg *h, int kclass) {
    const Lay &L = h->lv[0].lay;
    const double n = (double)L.n0 * L.n1 * L.n2;
    const bool mixed = h->prm.precision == SARAS_PREC_MIXED;
    const double sz = mixed ? 4.0 : 8.0;
    switch (kclass) {
    case KC_SMOOTH0: {
        // an RBGS iteration reads e and r and writes e (3 N s): a fused
        // launch is a whole iteration, a colour launch half of one; the
        // average over a V-cycle's launch mix (smooth() pairs iterations)
        const bool fused = mixed && (h->lv[0].tma.fok || (h->lv[0].e32b && pair_sweep_fits(h->lv[0].lay, h->d3)));
        int f = 0, k = 0;
        for (int c : {h->prm.pre_smooth, h->prm.post_smooth}) {
            const int fc = fused ? c / 2 * 2 : 0;
            f += fc;
            k += c - fc;
        }
        return f + 2 * k > 0 ? (f + k) * 3.0 * n * sz / (f + 2 * k) : 0.0;
    }
    case KC_RESTRICT:  // read u, f; write the coarse rhs
        return (2.0 + 0.125) * n * sz;
    case KC_PROLONG:  // read coarse, read and write fine
        return (0.125 + 2.0) * n * sz;
    case KC_NORM:  // read u, f (FP64); MIXED also writes r in FP32
        return mixed ? 20.0 * n : 16.0 * n;
    case KC_H2D:  // one dense padded box of the caller per copy
    case KC_D2H:
        return (double)h->stage_elems * sizeof(double);
    default:
        return 0.0;
    }
}

}  // namespace saras
