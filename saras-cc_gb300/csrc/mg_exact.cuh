// Multigrid kernels of the FP64_EXACT form: every cell value is computed with
// the reference's operation order and separately rounded FP64 operations,
// and ghost cells are refreshed at the same points as the reference, so the
// results are bit-identical to lib/poisson's single-rank arithmetic.
#pragma once

#include "common.cuh"

namespace saras {

// Device pointers to the per-level 1-D coefficient tables (core indices).
// A2 = xix2*ihx2 and A1 = xixx*i2hx (poisson_d3.cc:110-116): the products
// are formed on the host in the same order as the reference forms them.
struct Coef {
    const double *A2x, *A1x, *A2y, *A1y, *A2z, *A1z;
};

// Restriction tables of a coarse level: r0 = xc(i) - xf(2i),
// r1 = xf(2i+1) - xc(i), rt = xf(2i+1) - xf(2i) (poisson_d3.cc:494-502).
struct RTab {
    const double *r0x, *r1x, *rtx, *r0y, *r1y, *rty, *r0z, *r1z, *rtz;
};

// Ghost-cell rules of one level: per axis periodic flag and per face kind
// (SARAS_BC_*); wall values of the TEST_POISSON branch at the finest level.
struct Ghost {
    int per[3];
    int kind[6];
    const double *wallx, *wally, *wallz;  // (n1+2)x(n2+2), (n0+2)x(n2+2), (n0+2)x(n1+2), or null
};

template <bool D3>
__device__ __forceinline__ double rbgs_exact(const double *__restrict__ u, const double *__restrict__ f,
                                             const Lay &L, const Coef &C, int i, int j, int k,
                                             double w, double omc) {
    const int64_t c = L.at(i, j, k);
    const double uc = u[c];
    const double xp = u[c + L.s0], xm = u[c - L.s0];
    const double zp = u[c + 1], zm = u[c - 1];
    const double a2x = C.A2x[i], a1x = C.A1x[i], a2z = C.A2z[k], a1z = C.A1z[k];
    double s = radd(rmul(a2x, radd(xp, xm)), rmul(a1x, rsub(xp, xm)));
    double den;
    if (D3) {
        const double yp = u[c + L.s1], ym = u[c - L.s1];
        const double a2y = C.A2y[j], a1y = C.A1y[j];
        s = radd(s, rmul(a2y, radd(yp, ym)));
        s = radd(s, rmul(a1y, rsub(yp, ym)));
        den = rmul(2.0, radd(radd(a2x, a2y), a2z));
    } else {
        den = rmul(2.0, radd(a2x, a2z));
    }
    s = radd(s, rmul(a2z, radd(zp, zm)));
    s = radd(s, rmul(a1z, rsub(zp, zm)));
    s = rsub(s, f[c]);
    return radd(rmul(omc, uc), rdiv(rmul(s, w), den));
}

// f - A u with the reference's association (poisson_d3.cc:81-87).
template <bool D3>
__device__ __forceinline__ double resid_exact(const double *__restrict__ u, const double *__restrict__ f,
                                              const Lay &L, const Coef &C, int i, int j, int k) {
    const int64_t c = L.at(i, j, k);
    const double uc = u[c];
    const double u2 = rmul(2.0, uc);
    const double xp = u[c + L.s0], xm = u[c - L.s0];
    const double zp = u[c + 1], zm = u[c - 1];
    double s = radd(rmul(C.A2x[i], radd(rsub(xp, u2), xm)), rmul(C.A1x[i], rsub(xp, xm)));
    if (D3) {
        const double yp = u[c + L.s1], ym = u[c - L.s1];
        s = radd(s, rmul(C.A2y[j], radd(rsub(yp, u2), ym)));
        s = radd(s, rmul(C.A1y[j], rsub(yp, ym)));
    }
    s = radd(s, rmul(C.A2z[k], radd(rsub(zp, u2), zm)));
    s = radd(s, rmul(C.A1z[k], rsub(zp, zm)));
    return rsub(f[c], s);
}

__device__ __forceinline__ double ghost_value(int kind, double u, double wall, bool zeroBC) {
    if (kind == SARAS_BC_NEUMANN) return u;
    if (kind == SARAS_BC_DIRICHLET) return -u;
    return zeroBC ? -u : rsub(rmul(2.0, wall), u);
}

// One axis of imposeBC / updateFace at plane position (a, b): a and b run
// over the full extents (-1..n) of the two other axes in (i,j,k) order.
// The wrap pass copies periodic planes (updateFace); the wall pass writes the
// ghosts of non-periodic faces.  imposeBC is the wrap pass over x, y, z
// followed by the wall pass over x, y, z.
__device__ __forceinline__ void ghost_axis_cell(double *u, const Lay &L, const Ghost &G, int axis,
                                                int a, int b, bool wall_pass, bool zeroBC, bool lvl0) {
    int lo[3], hi[3], in0[3], in1[3];
    const int n[3] = {L.n0, L.n1, L.n2};
    int o0 = axis == 0 ? 1 : 0;
    int o1 = axis == 2 ? 1 : 2;
    lo[axis] = -1;
    hi[axis] = n[axis];
    in0[axis] = 0;
    in1[axis] = n[axis] - 1;
    lo[o0] = hi[o0] = in0[o0] = in1[o0] = a;
    lo[o1] = hi[o1] = in0[o1] = in1[o1] = b;
    const int64_t glo = L.at(lo[0], lo[1], lo[2]), ghi = L.at(hi[0], hi[1], hi[2]);
    const int64_t ilo = L.at(in0[0], in0[1], in0[2]), ihi = L.at(in1[0], in1[1], in1[2]);
    if (!wall_pass) {
        if (!G.per[axis]) return;
        // self-exchange order of updateFace: plane 0 lands in ghost n, then
        // plane n-1 lands in ghost -1
        u[ghi] = u[ilo];
        u[glo] = u[ihi];
        return;
    }
    if (G.per[axis]) return;
    double w = 0.0;
    if (lvl0) {
        const double *wa = axis == 0 ? G.wallx : (axis == 1 ? G.wally : G.wallz);
        if (wa) {
            // wall arrays are indexed by the two other axes' full ranges
            const int m1 = (axis == 2 ? L.n1 : L.n2) + 2;
            w = wa[(int64_t)(a + 1) * m1 + (b + 1)];
        }
    }
    u[glo] = ghost_value(G.kind[2 * axis], u[ilo], w, zeroBC);
    u[ghi] = ghost_value(G.kind[2 * axis + 1], u[ihi], w, zeroBC);
}

}  // namespace saras
