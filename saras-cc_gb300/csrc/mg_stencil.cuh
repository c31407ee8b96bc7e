// Device stencil helpers of the FP64 and MIXED forms, shared by the
// single-problem kernels (mg_fast.cu) and the batched serving kernels
// (serve.cu): the stretched 7-point operator with its ghost cells folded in.
#pragma once

#include "common.cuh"

namespace saras {

// Ghost rule folded into the stencil: per axis periodic flag and the sign
// of the mirrored value on the low and high faces (+1 Neumann, -1 Dirichlet).
struct Bnd {
    int per[3];
    int sg_lo[3], sg_hi[3];
};

template <class T>
struct Tab3 {
    const T *cm[3], *cp[3], *dg[3];
};

template <class T>
struct WTab {
    const T *w0[3], *w1[3];
};

__device__ __forceinline__ float fmat(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmat(double a, double b, double c) { return __fma_rn(a, b, c); }

// Sweeps between the stagnation checks of the MIXED form's coarsest solve.
constexpr int COARSE_STALL_CHECK = 8;

// Quotient of the FP32 colour sweeps: the hardware reciprocal path of
// __fdividef (about two ulp).  Every FP32 sweep kernel uses it, so the
// single-problem, TMA and batched sweeps produce identical bits.
__device__ __forceinline__ float sweep_div(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double sweep_div(double a, double b) { return a / b; }

// out = M applied along axis a of the dense n0 x n1 x n2 block `in`: for
// every cell, sum over m of M[o][m] * in(index m along a), o the cell's own
// index along a.  One thread per output cell, a fixed summation order.
__device__ __forceinline__ void fd_apply(const double *in, double *out, const double *__restrict__ M, int a, int n0,
                                         int n1, int n2) {
    const int ncell = n0 * n1 * n2;
    const int na = a == 0 ? n0 : (a == 1 ? n1 : n2);
    const int st = a == 0 ? n1 * n2 : (a == 1 ? n2 : 1);
    for (int q = threadIdx.x; q < ncell; q += blockDim.x) {
        const int o = (q / st) % na;
        const int base = q - o * st;
        const double *row = M + (int64_t)o * na;
        double s = 0.0;
        for (int m = 0; m < na; m++) s = fmat(row[m], in[base + m * st], s);
        out[q] = s;
    }
}

// Exact coarsest solve of the MIXED form (one block): u = (Vx (x) Vy (x) Vz)
// L^-1 (Vx^-1 (x) Vy^-1 (x) Vz^-1) f with the eigenvalue sums L; the null
// mode of a singular (all-Neumann or periodic) box is dropped, and with it
// the part of f outside the operator's range.  ug gets zero ghosts, as the
// sweeps leave them.  sa, sb: two buffers of n0*n1*n2 doubles.
__device__ __forceinline__ void fd_solve(double *ug, const double *fg, const Lay &L, const FDiag &F, double *sa,
                                         double *sb) {
    const int n0 = L.n0, n1 = L.n1, n2 = L.n2, ncell = n0 * n1 * n2;
    for (int q = threadIdx.x; q < ncell; q += blockDim.x) {
        const int k = q % n2, rest = q / n2, j = rest % n1, i = rest / n1;
        sa[q] = fg[L.at(i, j, k)];
    }
    __syncthreads();
    fd_apply(sa, sb, F.vi[2], 2, n0, n1, n2);
    __syncthreads();
    fd_apply(sb, sa, F.vi[1], 1, n0, n1, n2);
    __syncthreads();
    fd_apply(sa, sb, F.vi[0], 0, n0, n1, n2);
    __syncthreads();
    for (int q = threadIdx.x; q < ncell; q += blockDim.x) {
        const int k = q % n2, rest = q / n2, j = rest % n1, i = rest / n1;
        const double lam = (F.lam[0][i] + F.lam[1][j]) + F.lam[2][k];
        sb[q] = fabs(lam) > F.lam_tol ? sb[q] / lam : 0.0;
    }
    __syncthreads();
    fd_apply(sb, sa, F.v[0], 0, n0, n1, n2);
    __syncthreads();
    fd_apply(sa, sb, F.v[1], 1, n0, n1, n2);
    __syncthreads();
    fd_apply(sb, sa, F.v[2], 2, n0, n1, n2);
    __syncthreads();
    for (int64_t q = threadIdx.x; q < L.size; q += blockDim.x) ug[q] = 0.0;
    __syncthreads();
    for (int q = threadIdx.x; q < ncell; q += blockDim.x) {
        const int k = q % n2, rest = q / n2, j = rest % n1, i = rest / n1;
        ug[L.at(i, j, k)] = sa[q];
    }
}

template <class T>
__device__ __forceinline__ T nb_lo(const T *u, int64_t c, int i, int n, int64_t s, int per, int sg, T uc) {
    if (i > 0) return u[c - s];
    if (per) return u[c + (int64_t)(n - 1) * s];
    return sg > 0 ? uc : -uc;
}
template <class T>
__device__ __forceinline__ T nb_hi(const T *u, int64_t c, int i, int n, int64_t s, int per, int sg, T uc) {
    if (i < n - 1) return u[c + s];
    if (per) return u[c - (int64_t)(n - 1) * s];
    return sg > 0 ? uc : -uc;
}

// Off-diagonal part of the stretched 7-point operator at cell (i,j,k).
template <class T, bool D3>
__device__ __forceinline__ T offdiag(const T *u, const Lay &L, const Tab3<T> &t, const Bnd &b, int i, int j,
                                     int k, int64_t c, T uc) {
    const T xm = nb_lo(u, c, i, L.n0, L.s0, b.per[0], b.sg_lo[0], uc);
    const T xp = nb_hi(u, c, i, L.n0, L.s0, b.per[0], b.sg_hi[0], uc);
    const T zm = nb_lo(u, c, k, L.n2, (int64_t)1, b.per[2], b.sg_lo[2], uc);
    const T zp = nb_hi(u, c, k, L.n2, (int64_t)1, b.per[2], b.sg_hi[2], uc);
    T s = t.cm[0][i] * xm;
    s = fmat(t.cp[0][i], xp, s);
    if (D3) {
        const T ym = nb_lo(u, c, j, L.n1, L.s1, b.per[1], b.sg_lo[1], uc);
        const T yp = nb_hi(u, c, j, L.n1, L.s1, b.per[1], b.sg_hi[1], uc);
        s = fmat(t.cm[1][j], ym, s);
        s = fmat(t.cp[1][j], yp, s);
    }
    s = fmat(t.cm[2][k], zm, s);
    s = fmat(t.cp[2][k], zp, s);
    return s;
}

template <class T, bool D3>
__device__ __forceinline__ T diag(const Tab3<T> &t, int i, int j, int k) {
    T d = t.dg[0][i] + t.dg[2][k];
    if (D3) d += t.dg[1][j];
    return d + d;
}

// f - A u; with `dd` the diagonal is read per cell instead of rebuilt (it
// saves three FP64 additions per cell, the scarce resource on GB300).
template <class T, bool D3>
__device__ __forceinline__ T resid(const T *u, const T *f, const Lay &L, const Tab3<T> &t, const Bnd &b, int i,
                                   int j, int k, const T *dd = nullptr) {
    const int64_t c = L.at(i, j, k);
    const T uc = u[c];
    const T s = offdiag<T, D3>(u, L, t, b, i, j, k, c, uc);
    const T d = dd ? dd[c] : diag<T, D3>(t, i, j, k);
    return f[c] - fmat(-d, uc, s);
}

// ---- 8-cell strips along k (rows start on 32-byte boundaries, Lay) ----
// Shared by the single-problem kernels (mg_fast.cu) and the batched serving
// kernels (serve.cu), so both sweep with the same arithmetic.

template <class T>
__device__ __forceinline__ void ld8(const T *__restrict__ p, T (&o)[8]);
template <>
__device__ __forceinline__ void ld8<float>(const float *__restrict__ p, float (&o)[8]) {
    const float4 a = __ldg(reinterpret_cast<const float4 *>(p));
    const float4 b = __ldg(reinterpret_cast<const float4 *>(p + 4));
    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
    o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w;
}
template <>
__device__ __forceinline__ void ld8<double>(const double *__restrict__ p, double (&o)[8]) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const double2 a = __ldg(reinterpret_cast<const double2 *>(p + 2 * q));
        o[2 * q] = a.x;
        o[2 * q + 1] = a.y;
    }
}
// plain (coherent) vector load for the array being updated in place
template <class T>
__device__ __forceinline__ void ld8u(const T *p, T (&o)[8]);
template <>
__device__ __forceinline__ void ld8u<float>(const float *p, float (&o)[8]) {
    const float4 a = *reinterpret_cast<const float4 *>(p);
    const float4 b = *reinterpret_cast<const float4 *>(p + 4);
    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
    o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w;
}
template <>
__device__ __forceinline__ void ld8u<double>(const double *p, double (&o)[8]) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const double2 a = *reinterpret_cast<const double2 *>(p + 2 * q);
        o[2 * q] = a.x;
        o[2 * q + 1] = a.y;
    }
}

template <class T>
__device__ __forceinline__ void mirror8(const T (&cur)[8], int sg, T (&o)[8]) {
#pragma unroll
    for (int q = 0; q < 8; q++) o[q] = sg > 0 ? cur[q] : -cur[q];
}

// WD (the FP64 form, omega/D stored per cell): f enters the neighbour sum's
// chain as its first addend, and with W1 (SOR parameter 1) the (1 - omega) u
// term, zero, is not formed: seven FP64 operations per cell instead of nine,
// equal to the longer form to rounding.  Without WD (the FP32 sweeps, whose
// bits the served and single solves share) the chain is unchanged.
template <class T, bool D3, bool WD, int T0, bool W1 = false>
__device__ __forceinline__ void strip_update(T *u, const T (&cur)[8], const T (&xm)[8], const T (&xp)[8],
                                             const T (&ym)[8], const T (&yp)[8], const T (&fr)[8], const T (&wv)[8],
                                             T left, T right, const Tab3<T> &t, int i, int j, int k0, int64_t c0, T w,
                                             T omc) {
    const T cmx = t.cm[0][i], cpx = t.cp[0][i], dx = t.dg[0][i];
    T cmy = T(0), cpy = T(0), dy = T(0);
    if (D3) {
        cmy = t.cm[1][j];
        cpy = t.cp[1][j];
        dy = t.dg[1][j];
    }
#pragma unroll
    for (int q = T0; q < 8; q += 2) {
        const int k = k0 + q;
        const T zm = q > 0 ? cur[q - 1] : left;
        const T zp = q < 7 ? cur[q + 1] : right;
        T sm = WD ? fmat(cmx, xm[q], -fr[q]) : cmx * xm[q];
        sm = fmat(cpx, xp[q], sm);
        if (D3) {
            sm = fmat(cmy, ym[q], sm);
            sm = fmat(cpy, yp[q], sm);
        }
        sm = fmat(t.cm[2][k], zm, sm);
        sm = fmat(t.cp[2][k], zp, sm);
        if (!WD) sm = sm - fr[q];
        T v;
        if (WD) {
            v = W1 ? sm * wv[q] : fmat(sm, wv[q], omc * cur[q]);
        } else {
            T d = dx + t.dg[2][k];
            if (D3) d += dy;
            v = fmat(omc, cur[q], sweep_div(w * sm, d + d));
        }
        u[c0 + q] = v;
    }
}


template <class T>
__device__ __forceinline__ void st8(T *p, const T (&v)[8]);
template <>
__device__ __forceinline__ void st8<float>(float *p, const float (&v)[8]) {
    reinterpret_cast<float4 *>(p)[0] = make_float4(v[0], v[1], v[2], v[3]);
    reinterpret_cast<float4 *>(p)[1] = make_float4(v[4], v[5], v[6], v[7]);
}
template <>
__device__ __forceinline__ void st8<double>(double *p, const double (&v)[8]) {
#pragma unroll
    for (int q = 0; q < 4; q++) reinterpret_cast<double2 *>(p)[q] = make_double2(v[2 * q], v[2 * q + 1]);
}
template <class T>
__device__ __forceinline__ void ld4(const T *__restrict__ p, T (&o)[4]);
template <>
__device__ __forceinline__ void ld4<float>(const float *__restrict__ p, float (&o)[4]) {
    const float4 a = __ldg(reinterpret_cast<const float4 *>(p));
    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
}
template <>
__device__ __forceinline__ void ld4<double>(const double *__restrict__ p, double (&o)[4]) {
    const double2 a = __ldg(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldg(reinterpret_cast<const double2 *>(p + 2));
    o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
}


// One colour of the RBGS sweep on the 8-cell strip (i, j, k0 .. k0+7): the
// strip and its neighbour rows as vectors, boundary ghosts folded in, only
// the sweep's colour cells stored.
template <class T, bool D3, bool WD, bool W1 = false>
__device__ __forceinline__ void rbgs_strip8(T *u, const T *__restrict__ f, const T *__restrict__ wd, const Lay &L,
                                            const Tab3<T> &t, const Bnd &b, int colour, T w, T omc, int i, int j,
                                            int k0) {
    const int64_t c0 = L.at(i, j, k0);
    T cur[8], xm[8], xp[8], ym[8], yp[8], fr[8], wv[8];
    ld8u(u + c0, cur);
    if (i > 0) ld8u(u + c0 - L.s0, xm);
    else if (b.per[0]) ld8u(u + c0 + (int64_t)(L.n0 - 1) * L.s0, xm);
    else mirror8(cur, b.sg_lo[0], xm);
    if (i < L.n0 - 1) ld8u(u + c0 + L.s0, xp);
    else if (b.per[0]) ld8u(u + c0 - (int64_t)(L.n0 - 1) * L.s0, xp);
    else mirror8(cur, b.sg_hi[0], xp);
    if (D3) {
        if (j > 0) ld8u(u + c0 - L.s1, ym);
        else if (b.per[1]) ld8u(u + c0 + (int64_t)(L.n1 - 1) * L.s1, ym);
        else mirror8(cur, b.sg_lo[1], ym);
        if (j < L.n1 - 1) ld8u(u + c0 + L.s1, yp);
        else if (b.per[1]) ld8u(u + c0 - (int64_t)(L.n1 - 1) * L.s1, yp);
        else mirror8(cur, b.sg_hi[1], yp);
    }
    ld8(f + c0, fr);
    if (WD) ld8(wd + c0, wv);
    const T left = k0 > 0 ? u[c0 - 1]
                          : (b.per[2] ? u[c0 + L.n2 - 1] : (b.sg_lo[2] > 0 ? cur[0] : -cur[0]));
    const T right = k0 + 8 < L.n2 ? u[c0 + 8]
                                  : (b.per[2] ? u[c0 + 8 - L.n2] : (b.sg_hi[2] > 0 ? cur[7] : -cur[7]));
    if (((colour + i + j + k0) & 1) == 0)
        strip_update<T, D3, WD, 0, W1>(u, cur, xm, xp, ym, yp, fr, wv, left, right, t, i, j, k0, c0, w, omc);
    else
        strip_update<T, D3, WD, 1, W1>(u, cur, xm, xp, ym, yp, fr, wv, left, right, t, i, j, k0, c0, w, omc);
}

// Residuals of eight consecutive fine cells of one row (k_resid_restrict's
// resid() arithmetic, cell by cell) from vector loads of the row, its x and y
// neighbour rows, f and the stored diagonal.
template <class T, bool D3>
__device__ __forceinline__ void resid_row8(const T *__restrict__ u, const T *__restrict__ f, const Lay &L,
                                           const Tab3<T> &t, const Bnd &b, int i, int j, int k0,
                                           const T *__restrict__ dd, T (&r)[8]) {
    const int64_t c0 = L.at(i, j, k0);
    T cur[8], xm[8], xp[8], ym[8], yp[8], fr[8];
    ld8(u + c0, cur);
    if (i > 0) ld8(u + c0 - L.s0, xm);
    else if (b.per[0]) ld8(u + c0 + (int64_t)(L.n0 - 1) * L.s0, xm);
    else mirror8(cur, b.sg_lo[0], xm);
    if (i < L.n0 - 1) ld8(u + c0 + L.s0, xp);
    else if (b.per[0]) ld8(u + c0 - (int64_t)(L.n0 - 1) * L.s0, xp);
    else mirror8(cur, b.sg_hi[0], xp);
    if (D3) {
        if (j > 0) ld8(u + c0 - L.s1, ym);
        else if (b.per[1]) ld8(u + c0 + (int64_t)(L.n1 - 1) * L.s1, ym);
        else mirror8(cur, b.sg_lo[1], ym);
        if (j < L.n1 - 1) ld8(u + c0 + L.s1, yp);
        else if (b.per[1]) ld8(u + c0 - (int64_t)(L.n1 - 1) * L.s1, yp);
        else mirror8(cur, b.sg_hi[1], yp);
    }
    ld8(f + c0, fr);
    const T left = k0 > 0 ? __ldg(u + c0 - 1) : (b.per[2] ? __ldg(u + c0 + L.n2 - 1) : (b.sg_lo[2] > 0 ? cur[0] : -cur[0]));
    const T right = k0 + 8 < L.n2 ? __ldg(u + c0 + 8)
                                  : (b.per[2] ? __ldg(u + c0 + 8 - L.n2) : (b.sg_hi[2] > 0 ? cur[7] : -cur[7]));
    T dv[8];
    if (dd) ld8(dd + c0, dv);
    const T cmx = t.cm[0][i], cpx = t.cp[0][i];
    T cmy = T(0), cpy = T(0);
    if (D3) {
        cmy = t.cm[1][j];
        cpy = t.cp[1][j];
    }
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int k = k0 + q;
        const T zm = q > 0 ? cur[q - 1] : left;
        const T zp = q < 7 ? cur[q + 1] : right;
        T sm = cmx * xm[q];
        sm = fmat(cpx, xp[q], sm);
        if (D3) {
            sm = fmat(cmy, ym[q], sm);
            sm = fmat(cpy, yp[q], sm);
        }
        sm = fmat(t.cm[2][k], zm, sm);
        sm = fmat(t.cp[2][k], zp, sm);
        const T d = dd ? dv[q] : diag<T, D3>(t, i, j, k);
        r[q] = fr[q] - fmat(-d, cur[q], sm);
    }
}

// f - A u on the 4-cell row segment (i, j, k0 .. k0+3): resid_row8's
// arithmetic on half the cells (a kernel with half the registers per thread).
template <class T, bool D3, bool RS = false>
__device__ __forceinline__ void resid_row4(const T *__restrict__ u, const T *__restrict__ f, const Lay &L,
                                           const Tab3<T> &t, const Bnd &b, int i, int j, int k0,
                                           const T *__restrict__ dd, T (&r)[4]) {
    const int64_t c0 = RS ? L.at(i, j, 0) : L.at(i, j, k0);
    T cur[4], xm[4], xp[4], ym[4], yp[4], fr[4];
    auto mirror = [](const T (&c)[4], int sg, T (&o)[4]) {
#pragma unroll
        for (int q = 0; q < 4; q++) o[q] = sg > 0 ? c[q] : -c[q];
    };
    // RS: c0 is the row's start; cells k0 .. k0+3 of a row of parity pr are
    // its red and black halves at k0/2, k0/2 + 1, interleaved
    const int pr = (i + j) & 1, h = k0 >> 1, H = L.n2 >> 1;
    auto ld = [&](const T *p, int par, T (&o)[4]) {
        if (!RS) {
            ld4(p, o);
            return;
        }
        T rd[2], bk[2];
        if constexpr (RS && sizeof(T) == 4) {
            // h is even: 8-byte aligned pairs
            const float2 a = __ldg(reinterpret_cast<const float2 *>(p + h));
            const float2 c = __ldg(reinterpret_cast<const float2 *>(p + H + h));
            rd[0] = a.x; rd[1] = a.y; bk[0] = c.x; bk[1] = c.y;
        } else {
            rd[0] = __ldg(p + h);
            rd[1] = __ldg(p + h + 1);
            bk[0] = __ldg(p + H + h);
            bk[1] = __ldg(p + H + h + 1);
        }
        if (par == 0) {
            o[0] = rd[0]; o[1] = bk[0]; o[2] = rd[1]; o[3] = bk[1];
        } else {
            o[0] = bk[0]; o[1] = rd[0]; o[2] = bk[1]; o[3] = rd[1];
        }
    };
    // position of cell k of this row (RS) or its offset from c0
    auto at_k = [&](int k) -> int64_t { return RS ? (k >> 1) + (int64_t)(((pr + k) & 1) * H) : k - k0; };
    ld(u + c0, pr, cur);
    if (i > 0) ld(u + c0 - L.s0, 1 - pr, xm);
    else if (b.per[0]) ld(u + c0 + (int64_t)(L.n0 - 1) * L.s0, 1 - pr, xm);
    else mirror(cur, b.sg_lo[0], xm);
    if (i < L.n0 - 1) ld(u + c0 + L.s0, 1 - pr, xp);
    else if (b.per[0]) ld(u + c0 - (int64_t)(L.n0 - 1) * L.s0, 1 - pr, xp);
    else mirror(cur, b.sg_hi[0], xp);
    if (D3) {
        if (j > 0) ld(u + c0 - L.s1, 1 - pr, ym);
        else if (b.per[1]) ld(u + c0 + (int64_t)(L.n1 - 1) * L.s1, 1 - pr, ym);
        else mirror(cur, b.sg_lo[1], ym);
        if (j < L.n1 - 1) ld(u + c0 + L.s1, 1 - pr, yp);
        else if (b.per[1]) ld(u + c0 - (int64_t)(L.n1 - 1) * L.s1, 1 - pr, yp);
        else mirror(cur, b.sg_hi[1], yp);
    }
    ld(f + c0, pr, fr);
    const T left = k0 > 0 ? __ldg(u + c0 + at_k(k0 - 1))
                          : (b.per[2] ? __ldg(u + c0 + at_k(L.n2 - 1)) : (b.sg_lo[2] > 0 ? cur[0] : -cur[0]));
    const T right = k0 + 4 < L.n2 ? __ldg(u + c0 + at_k(k0 + 4))
                                  : (b.per[2] ? __ldg(u + c0 + at_k(0)) : (b.sg_hi[2] > 0 ? cur[3] : -cur[3]));
    T dv[4];
    if (dd) ld4(dd + c0, dv);
    const T cmx = t.cm[0][i], cpx = t.cp[0][i];
    T cmy = T(0), cpy = T(0);
    if (D3) {
        cmy = t.cm[1][j];
        cpy = t.cp[1][j];
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int k = k0 + q;
        const T zm = q > 0 ? cur[q - 1] : left;
        const T zp = q < 3 ? cur[q + 1] : right;
        T sm = cmx * xm[q];
        sm = fmat(cpx, xp[q], sm);
        if (D3) {
            sm = fmat(cmy, ym[q], sm);
            sm = fmat(cpy, yp[q], sm);
        }
        sm = fmat(t.cm[2][k], zm, sm);
        sm = fmat(t.cp[2][k], zp, sm);
        const T d = dd ? dv[q] : diag<T, D3>(t, i, j, k);
        r[q] = fr[q] - fmat(-d, cur[q], sm);
    }
}

// The two coarse cells (i, j, kc0, kc0+1) of the fused residual and
// restriction: restrict4's arithmetic from 4-cell fine rows.
template <class T, bool D3, bool RS = false>
__device__ __forceinline__ void restrict2(const T *__restrict__ u, const T *__restrict__ f, const Lay &Lf,
                                          const Tab3<T> &t, const Bnd &b, const WTab<T> &w,
                                          const T *__restrict__ dd, int i, int j, int kc0, T (&out)[2]) {
    if (D3) {
        T sy[2][2];
#pragma unroll
        for (int a = 0; a < 2; a++) {
            T sz[2][2];
#pragma unroll
            for (int bb = 0; bb < 2; bb++) {
                T r[4];
                resid_row4<T, true, RS>(u, f, Lf, t, b, 2 * i + a, 2 * j + bb, 2 * kc0, dd, r);
#pragma unroll
                for (int q = 0; q < 2; q++)
                    sz[bb][q] = fmat(w.w1[2][kc0 + q], r[2 * q + 1], w.w0[2][kc0 + q] * r[2 * q]);
            }
#pragma unroll
            for (int q = 0; q < 2; q++) sy[a][q] = fmat(w.w1[1][j], sz[1][q], w.w0[1][j] * sz[0][q]);
        }
#pragma unroll
        for (int q = 0; q < 2; q++) out[q] = fmat(w.w1[0][i], sy[1][q], w.w0[0][i] * sy[0][q]);
    } else {
        T r0[4], r1[4];
        resid_row4<T, false, RS>(u, f, Lf, t, b, 2 * i, 0, 2 * kc0, dd, r0);
        resid_row4<T, false, RS>(u, f, Lf, t, b, 2 * i + 1, 0, 2 * kc0, dd, r1);
#pragma unroll
        for (int q = 0; q < 2; q++) out[q] = ((r0[2 * q] + r0[2 * q + 1]) + (r1[2 * q] + r1[2 * q + 1])) * T(0.25);
    }
}

// The four coarse cells (i, j, kc0 .. kc0+3) of the fused residual and
// restriction: residuals of their 2x2x2 children from 8-cell fine rows,
// weighted by the coarsen factors v_abc / vTot (poisson_d3.cc:494-508) per
// axis, or the mean of four children in 2-D.
template <class T, bool D3>
__device__ __forceinline__ void restrict4(const T *__restrict__ u, const T *__restrict__ f, const Lay &Lf,
                                          const Tab3<T> &t, const Bnd &b, const WTab<T> &w,
                                          const T *__restrict__ dd, int i, int j, int kc0, T (&out)[4]) {
    if (D3) {
        T sy[2][4];
        for (int a = 0; a < 2; a++) {
            T sz[2][4];
            for (int bb = 0; bb < 2; bb++) {
                T r[8];
                resid_row8<T, true>(u, f, Lf, t, b, 2 * i + a, 2 * j + bb, 2 * kc0, dd, r);
#pragma unroll
                for (int q = 0; q < 4; q++)
                    sz[bb][q] = fmat(w.w1[2][kc0 + q], r[2 * q + 1], w.w0[2][kc0 + q] * r[2 * q]);
            }
#pragma unroll
            for (int q = 0; q < 4; q++) sy[a][q] = fmat(w.w1[1][j], sz[1][q], w.w0[1][j] * sz[0][q]);
        }
#pragma unroll
        for (int q = 0; q < 4; q++) out[q] = fmat(w.w1[0][i], sy[1][q], w.w0[0][i] * sy[0][q]);
    } else {
        T r0[8], r1[8];
        resid_row8<T, false>(u, f, Lf, t, b, 2 * i, 0, 2 * kc0, dd, r0);
        resid_row8<T, false>(u, f, Lf, t, b, 2 * i + 1, 0, 2 * kc0, dd, r1);
#pragma unroll
        for (int q = 0; q < 4; q++) out[q] = ((r0[2 * q] + r0[2 * q + 1]) + (r1[2 * q] + r1[2 * q + 1])) * T(0.25);
    }
}

// fine (i, j, k0 .. k0+7) += coarse (i/2, j/2, k0/2 ..): injection
// prolongation and correction with vector loads and stores.
template <class T>
__device__ __forceinline__ void prolong8(T *__restrict__ f, const T *__restrict__ c, const Lay &Lf, const Lay &Lc,
                                         int d3, int i, int j, int k0) {
    const int64_t q = Lf.at(i, j, k0);
    T v[8], w[4];
    ld8u(f + q, v);
    ld4(c + Lc.at(i >> 1, d3 ? (j >> 1) : 0, k0 >> 1), w);
#pragma unroll
    for (int s = 0; s < 8; s++) v[s] = v[s] + w[s >> 1];
    st8(f + q, v);
}

}  // namespace saras
