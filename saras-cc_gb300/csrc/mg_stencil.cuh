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

// Quotient of the FP32 colour sweeps: the hardware reciprocal path of
// __fdividef (about two ulp).  Every FP32 sweep kernel uses it, so the
// single-problem, TMA and batched sweeps produce identical bits.
__device__ __forceinline__ float sweep_div(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double sweep_div(double a, double b) { return a / b; }

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

}  // namespace saras
