// Cell-centred geometric multigrid for the SARAS pressure-Poisson equation on
// GB300 (sm_103a): hierarchy set-up, the FP64_EXACT kernels, the solve loop
// and the saras_mg_* C entry points.  The FP64 and MIXED forms live in
// mg_fast.cu and share this handle.
//
// Reference: lib/poisson/poisson.cc (mgSolve 109-189, vCycle 203-279,
// setStagBounds 358-441, setCoefficients 453-483, copyDerivs 501-622) and
// poisson_d3.cc / poisson_d2.cc (computeResidual, smooth, solve, coarsen,
// prolong, computeError, imposeBC, updateFace), single-rank semantics.
#include <algorithm>
#include <cmath>
#include <cstring>

#include <math_constants.h>

#include "mg_handle.cuh"
#include "mg_fast.cuh"

using namespace saras;

namespace {

constexpr int BX = 128;

inline dim3 cell_grid(const Lay &L, bool d3, int kcount, int bx) {
    return dim3(cdiv(kcount, bx), d3 ? (unsigned)L.n1 : 1u, (unsigned)L.n0);
}

// ------------------------------------------------------------ kernels ----

// One colour of the SOR red-black sweep: cells with (i+j+k) even are red,
// odd are black (the parity loops of poisson_d3.cc:104-242).
template <bool D3>
__global__ void k_rbgs_exact(double *u, const double *__restrict__ f, Lay L, Coef C, int colour,
                             double w, double omc) {
    const int kk = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = D3 ? (int)blockIdx.y : 0;
    const int i = blockIdx.z;
    const int k = 2 * kk + ((i + j + colour) & 1);
    if (k >= L.n2) return;
    u[L.at(i, j, k)] = rbgs_exact<D3>(u, f, L, C, i, j, k, w, omc);
}

template <bool D3>
__global__ void k_resid_exact(const double *__restrict__ u, const double *__restrict__ f,
                              double *__restrict__ t, Lay L, Coef C) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = D3 ? (int)blockIdx.y : 0;
    const int i = blockIdx.z;
    if (k >= L.n2) return;
    t[L.at(i, j, k)] = resid_exact<D3>(u, f, L, C, i, j, k);
}

// Restriction (multigrid_d3::coarsen regular branch, poisson_d3.cc:483-511;
// multigrid_d2::coarsen: mean of four).
template <bool D3>
__global__ void k_restrict_exact(const double *__restrict__ t, double *__restrict__ r, Lay Lf, Lay Lc,
                                 RTab R) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = D3 ? (int)blockIdx.y : 0;
    const int i = blockIdx.z;
    if (k >= Lc.n2) return;
    const int i2 = 2 * i, j2 = 2 * j, k2 = 2 * k;
    if (D3) {
        const double x0 = R.r0x[i], x1 = R.r1x[i], y0 = R.r0y[j], y1 = R.r1y[j], z0 = R.r0z[k],
                     z1 = R.r1z[k];
        const double v000 = rmul(rmul(x0, y0), z0);
        const double v100 = rmul(rmul(x1, y0), z0);
        const double v010 = rmul(rmul(x0, y1), z0);
        const double v001 = rmul(rmul(x0, y0), z1);
        const double v011 = rmul(rmul(x0, y1), z1);
        const double v101 = rmul(rmul(x1, y0), z1);
        const double v110 = rmul(rmul(x1, y1), z0);
        const double v111 = rmul(rmul(x1, y1), z1);
        const double vt = rmul(rmul(R.rtx[i], R.rty[j]), R.rtz[k]);
        double s = rmul(v111, t[Lf.at(i2 + 1, j2 + 1, k2 + 1)]);
        s = radd(s, rmul(v000, t[Lf.at(i2, j2, k2)]));
        s = radd(s, rmul(v110, t[Lf.at(i2 + 1, j2 + 1, k2)]));
        s = radd(s, rmul(v001, t[Lf.at(i2, j2, k2 + 1)]));
        s = radd(s, rmul(v101, t[Lf.at(i2 + 1, j2, k2 + 1)]));
        s = radd(s, rmul(v010, t[Lf.at(i2, j2 + 1, k2)]));
        s = radd(s, rmul(v011, t[Lf.at(i2, j2 + 1, k2 + 1)]));
        s = radd(s, rmul(v100, t[Lf.at(i2 + 1, j2, k2)]));
        r[Lc.at(i, j, k)] = rdiv(s, vt);
    } else {
        double s = radd(t[Lf.at(i2 + 1, 0, k2 + 1)], t[Lf.at(i2, 0, k2)]);
        s = radd(s, t[Lf.at(i2 + 1, 0, k2)]);
        s = radd(s, t[Lf.at(i2, 0, k2 + 1)]);
        r[Lc.at(i, 0, k)] = rdiv(s, 4.0);
    }
}

// Injection prolongation into a zeroed fine array followed by lhs += smd
// over the full padded array (poisson_d3.cc:516-560, poisson.cc:263-266).
__global__ void k_prolong_exact(const double *__restrict__ c, const double *__restrict__ smd,
                                double *__restrict__ f, Lay Lf, Lay Lc, int d3) {
    const int k = (int)(blockIdx.x * blockDim.x + threadIdx.x) - 1;
    const int j = (int)blockIdx.y - 1;
    const int i = (int)blockIdx.z - 1;
    if (k > Lf.n2) return;
    const bool core = i >= 0 && i < Lf.n0 && j >= 0 && j < Lf.n1 && k >= 0 && k < Lf.n2;
    const double v = core ? c[Lc.at(i / 2, d3 ? j / 2 : 0, k / 2)] : 0.0;
    const int64_t q = Lf.at(i, j, k);
    f[q] = radd(v, smd[q]);
}

// One axis of the ghost refresh over a plane range.
__global__ void k_ghost(double *u, Lay L, Ghost G, int axis, int wall_pass, int zeroBC, int lvl0,
                        int a_lo, int b_lo, int b_cnt) {
    const int b = b_lo + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int a = a_lo + (int)blockIdx.y;
    if (b >= b_lo + b_cnt) return;
    ghost_axis_cell(u, L, G, axis, a, b, wall_pass != 0, zeroBC != 0, lvl0 != 0);
}

__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) {
        const double w = __shfl_xor_sync(0xffffffffu, v, o);
        v = (w > v || w != w) ? w : v;
    }
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v = radd(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Residual norms of the finest level (multigrid_d3::computeError,
// poisson_d3.cc:563-663): per-block partials of max|r|, max|f|, and the
// sums of |r|,|f| (L1) or r^2, f^2 (L2).
template <bool D3>
__global__ void k_norm_exact(const double *__restrict__ u, const double *__restrict__ f, Lay L, Coef C,
                             int rtype, double *__restrict__ part) {
    double mr = 0.0, mf = 0.0, sr = 0.0, sf = 0.0;
    for_core_rows(L, [&](int i, int j, int k) {
        const double r = resid_exact<D3>(u, f, L, C, i, j, k);
        const double fv = f[L.at(i, j, k)];
        if (rtype == 0) {
            const double ar = fabs(r), af = fabs(fv);
            if (ar > mr) mr = ar;
            if (af > mf) mf = af;
            if (!isfinite(r)) mr = CUDART_INF;  // reported as SARAS_NAN by the host
        } else if (rtype == 1) {
            sr = radd(sr, fabs(r));
            sf = radd(sf, fabs(fv));
        } else {
            sr = radd(sr, rmul(r, r));
            sf = radd(sf, rmul(fv, fv));
        }
    });
    __shared__ double sh[4][32];
    mr = warp_max(mr);
    mf = warp_max(mf);
    sr = warp_sum(sr);
    sf = warp_sum(sf);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) {
        sh[0][wid] = mr;
        sh[1][wid] = mf;
        sh[2][wid] = sr;
        sh[3][wid] = sf;
    }
    __syncthreads();
    if (wid == 0) {
        mr = lane < nw ? sh[0][lane] : 0.0;
        mf = lane < nw ? sh[1][lane] : 0.0;
        sr = lane < nw ? sh[2][lane] : 0.0;
        sf = lane < nw ? sh[3][lane] : 0.0;
        mr = warp_max(mr);
        mf = warp_max(mf);
        sr = warp_sum(sr);
        sf = warp_sum(sf);
        if (lane == 0) {
            part[4 * blockIdx.x + 0] = mr;
            part[4 * blockIdx.x + 1] = mf;
            part[4 * blockIdx.x + 2] = sr;
            part[4 * blockIdx.x + 3] = sf;
        }
    }
}

// Combines the partials in a fixed order and forms residualVal.
__global__ void k_norm_final(const double *__restrict__ part, int nb, int rtype, double point_count,
                             double *__restrict__ out, const double *__restrict__ den_pre) {
    double mr = 0.0, mf = 0.0, sr = 0.0, sf = 0.0;
    for (int b = threadIdx.x; b < nb; b += 32) {
        const double a = part[4 * b], c = part[4 * b + 1];
        if (a > mr || a != a) mr = a;  // a NaN partial stays NaN (reported as SARAS_NAN)
        if (c > mf) mf = c;
        sr = radd(sr, part[4 * b + 2]);
        sf = radd(sf, part[4 * b + 3]);
    }
    mr = warp_max(mr);
    mf = warp_max(mf);
    sr = warp_sum(sr);
    sf = warp_sum(sf);
    if (threadIdx.x == 0) {
        double num, den, res;
        if (den_pre) {  // the RHS norm of the solve, taken once
            mf = den_pre[0];
            sf = den_pre[0];
        }
        if (rtype == 0) {
            num = mr;
            den = mf;
            res = den != 0.0 ? rdiv(num, den) : num;
        } else if (rtype == 1) {
            num = sr;
            den = sf;
            res = den != 0.0 ? rdiv(num, den) : rdiv(num, point_count);
        } else {
            num = sr;
            den = sf;
            res = den != 0.0 ? rdiv(__dsqrt_rn(rdiv(num, point_count)), __dsqrt_rn(rdiv(den, point_count)))
                             : __dsqrt_rn(rdiv(num, point_count));
        }
        out[0] = res;
        out[1] = num;
        out[2] = den;
    }
}

// ---- coarsest-level solve (multigrid_d3::solve, poisson_d3.cc:249-432) ----

__device__ void block_ghost_pass(double *u, const Lay &L, const Ghost &G, bool d3, bool wall_pass) {
    for (int axis = 0; axis < 3; axis++) {
        if (!d3 && axis == 1) continue;
        const int n[3] = {L.n0, L.n1, L.n2};
        const int o0 = axis == 0 ? 1 : 0, o1 = axis == 2 ? 1 : 2;
        int alo = -1, acnt = n[o0] + 2, blo = -1, bcnt = n[o1] + 2;
        if (!d3) {
            if (o0 == 1) { alo = 0; acnt = 1; }
            if (o1 == 1) { blo = 0; bcnt = 1; }
        }
        const int total = acnt * bcnt;
        for (int q = threadIdx.x; q < total; q += blockDim.x)
            ghost_axis_cell(u, L, G, axis, alo + q / bcnt, blo + q % bcnt, wall_pass, true, false);
        __syncthreads();
    }
}

template <bool D3>
__device__ void block_colour(double *u, const double *f, const Lay &L, const Coef &C, int colour, double w,
                             double omc) {
    const int half = (L.n2 + 1) / 2;
    const int total = L.n0 * L.n1 * half;
    for (int q = threadIdx.x; q < total; q += blockDim.x) {
        const int kk = q % half;
        const int rest = q / half;
        const int j = rest % L.n1;
        const int i = rest / L.n1;
        const int k = 2 * kk + ((i + j + colour) & 1);
        if (k < L.n2) u[L.at(i, j, k)] = rbgs_exact<D3>(u, f, L, C, i, j, k, w, omc);
    }
    __syncthreads();
}

// The whole coarsest level fits in shared memory when it is small (the
// usual 4^3 .. 12x12x6 grids): lhs and rhs are staged there, the iterations
// run out of shared memory, and blocks of one warp keep the barriers cheap.
template <bool D3, bool SMEM>
__global__ void k_coarsest_exact(double *ug, const double *__restrict__ fg, Lay L, Coef C, Ghost G, double w,
                                 double omc, double tol, int max_count, int *sweeps_out) {
    __shared__ double sh[32];
    extern __shared__ double stage[];
    double *u = ug;
    const double *f = fg;
    if (SMEM) {
        double *us = stage, *fs = stage + L.size;
        for (int64_t q = threadIdx.x; q < L.size; q += blockDim.x) {
            us[q] = ug[q];
            fs[q] = fg[q];
        }
        __syncthreads();
        u = us;
        f = fs;
    }
    int iter = 0, sweeps = 0;
    for (;;) {
        block_ghost_pass(u, L, G, D3, false);
        block_ghost_pass(u, L, G, D3, true);
        block_colour<D3>(u, f, L, C, 0, w, omc);
        block_ghost_pass(u, L, G, D3, false);
        block_colour<D3>(u, f, L, C, 1, w, omc);
        double m = -1.0e-10;
        const int total = L.n0 * L.n1 * L.n2;
        for (int q = threadIdx.x; q < total; q += blockDim.x) {
            const int k = q % L.n2;
            const int rest = q / L.n2;
            const int j = rest % L.n1;
            const int i = rest / L.n1;
            const double t = fabs(resid_exact<D3>(u, f, L, C, i, j, k));
            if (t > m) m = t;
        }
        m = warp_max(m);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
        __syncthreads();
        if (threadIdx.x < 32) {
            double v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : -1.0e-10;
            v = warp_max(v);
            if (threadIdx.x == 0) sh[0] = v;
        }
        __syncthreads();
        m = sh[0];
        __syncthreads();
        sweeps++;
        if (m < tol) break;
        iter++;
        if (iter > max_count) break;  // the reference warns and moves on
    }
    block_ghost_pass(u, L, G, D3, false);
    block_ghost_pass(u, L, G, D3, true);
    if (SMEM)
        for (int64_t q = threadIdx.x; q < L.size; q += blockDim.x) ug[q] = u[q];
    if (threadIdx.x == 0) *sweeps_out += sweeps;
}

constexpr int64_t COARSE_SMEM_LIMIT = 96 * 1024;  // bytes of lhs + rhs staged in shared memory

// ---- caller arrays ----

__global__ void k_scatter(const double *__restrict__ lhs_src, const double *__restrict__ rhs_src, int64_t s0,
                          int64_t s1, int64_t s2, double *__restrict__ lhs, double *__restrict__ rhs, Lay L) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    if (k >= L.n2) return;
    const int64_t q = (int64_t)i * s0 + (int64_t)j * s1 + (int64_t)k * s2;
    const int64_t d = L.at(i, j, k);
    lhs[d] = lhs_src[q];
    rhs[d] = rhs_src[q];
}

__global__ void k_gather(const double *__restrict__ lhs, Lay L, double *__restrict__ dst, int64_t s0, int64_t s1,
                         int64_t s2) {
    const int k = (int)(blockIdx.x * blockDim.x + threadIdx.x) - 1;
    const int j = (int)blockIdx.y - 1, i = (int)blockIdx.z - 1;
    if (k > L.n2) return;
    dst[(int64_t)i * s0 + (int64_t)j * s1 + (int64_t)k * s2] = lhs[L.at(i, j, k)];
}

}  // namespace

// ------------------------------------------------------- host helpers ----

namespace saras {

void kbegin(saras_mg *h, cudaStream_t s, int kc) {
    h->issued++;
    if (!h->timing || kc < 0) return;
    // in graph mode the graph's own event-record nodes time its launches;
    // a sequence issued directly beside it records marks of its own
    if (h->graph && !h->capturing && !h->timing_direct) return;
    if (h->ev_used + 2 > h->ev_pool.size()) {
        if (h->capturing) {  // no event creation inside a capture: stop timing this class
            return;
        }
        for (int q = 0; q < 64; q++) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            h->ev_pool.push_back(e);
        }
    }
    h->ev_marks.push_back({kc, h->ev_used});
    // inside a capture only an "external" record becomes an event-record node
    cudaEventRecordWithFlags(h->ev_pool[h->ev_used], s, h->capturing ? cudaEventRecordExternal : 0);
    h->ev_used += 2;
    h->mark_open = true;
}

void kend(saras_mg *h, cudaStream_t s, int kc) {
    if (!h->timing || kc < 0 || !h->mark_open) return;
    cudaEventRecordWithFlags(h->ev_pool[h->ev_marks.back().second + 1], s,
                             h->capturing ? cudaEventRecordExternal : 0);
    h->mark_open = false;
}

// Adds the elapsed times of the bracketed launches of the last sequence:
// a replay of the captured graph (its event-record nodes, whose marks stay
// valid for every replay) or a sequence issued directly (its own marks,
// recorded on events past the graph's).
void harvest_timing(saras_mg *h, bool from_graph) {
    if (!h->timing) return;
    auto &marks = from_graph ? h->graph_marks : h->ev_marks;
    for (auto &m : marks) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, h->ev_pool[m.second], h->ev_pool[m.second + 1]);
        h->kc_ms[m.first] += ms;
        h->kc_launches[m.first] += 1;
    }
    if (!from_graph) {
        h->ev_marks.clear();
        h->ev_used = h->graph ? h->ev_base : 0;
    }
    cudaGetLastError();  // a failed elapsed-time query must not surface as a solve error
}

static void ghost_axis_launch(saras_mg *h, cudaStream_t s, double *u, const Lay &L, int axis, bool wall_pass,
                              bool zeroBC, bool lvl0) {
    if (!h->d3 && axis == 1) return;
    if (wall_pass == (bool)h->ghost.per[axis]) return;  // nothing to do on this axis in this pass
    const int n[3] = {L.n0, L.n1, L.n2};
    const int o0 = axis == 0 ? 1 : 0, o1 = axis == 2 ? 1 : 2;
    int alo = -1, acnt = n[o0] + 2, blo = -1, bcnt = n[o1] + 2;
    if (!h->d3) {
        if (o0 == 1) { alo = 0; acnt = 1; }
        if (o1 == 1) { blo = 0; bcnt = 1; }
    }
    const int bx = std::min(128, (bcnt + 31) / 32 * 32);
    kbegin(h, s, -1);
    k_ghost<<<dim3(cdiv(bcnt, bx), (unsigned)acnt), bx, 0, s>>>(u, L, h->ghost, axis, wall_pass, zeroBC, lvl0,
                                                               alo, blo, bcnt);
}

// imposeBC: wrap pass over x, y, z, then wall pass over x, y, z.
static void ghost_all(saras_mg *h, cudaStream_t s, int l, bool zeroBC) {
    Level &v = h->lv[(size_t)l];
    for (int a = 0; a < 3; a++) ghost_axis_launch(h, s, v.lhs, v.lay, a, false, zeroBC, l == 0);
    for (int a = 0; a < 3; a++) ghost_axis_launch(h, s, v.lhs, v.lay, a, true, zeroBC, l == 0);
}

static void ghost_wrap(saras_mg *h, cudaStream_t s, int l) {
    Level &v = h->lv[(size_t)l];
    for (int a = 0; a < 3; a++) ghost_axis_launch(h, s, v.lhs, v.lay, a, false, true, l == 0);
}

static void colour_exact(saras_mg *h, cudaStream_t s, int l, int colour) {
    Level &v = h->lv[(size_t)l];
    const Lay &L = v.lay;
    const int half = (L.n2 + 1) / 2;
    const int bx = std::min(BX, (half + 31) / 32 * 32);
    const double w = h->prm.sor_param, omc = 1.0 - h->prm.sor_param;
    kbegin(h, s, l == 0 ? KC_SMOOTH0 : -1);
    if (h->d3)
        k_rbgs_exact<true><<<cell_grid(L, true, half, bx), bx, 0, s>>>(v.lhs, v.rhs, L, v.coef, colour, w, omc);
    else
        k_rbgs_exact<false><<<cell_grid(L, false, half, bx), bx, 0, s>>>(v.lhs, v.rhs, L, v.coef, colour, w, omc);
    kend(h, s, l == 0 ? KC_SMOOTH0 : -1);
}

// multigrid_d*::smooth
static void smooth_exact(saras_mg *h, cudaStream_t s, int l, int count, bool zeroBC) {
    for (int n = 0; n < count; n++) {
        ghost_all(h, s, l, zeroBC);
        colour_exact(h, s, l, 0);
        ghost_wrap(h, s, l);
        colour_exact(h, s, l, 1);
    }
    ghost_all(h, s, l, zeroBC);
}

static void norm_exact(saras_mg *h, cudaStream_t s) {
    Level &v = h->lv[0];
    const double pc = h->d3 ? (double)h->grid.N[0] * h->grid.N[1] * h->grid.N[2]
                            : (double)h->grid.N[0] * h->grid.N[2];
    kbegin(h, s, KC_NORM);
    if (h->d3)
        k_norm_exact<true><<<h->norm_blocks, 256, 0, s>>>(v.lhs, v.rhs, v.lay, v.coef, h->prm.res_type,
                                                           h->norm_part);
    else
        k_norm_exact<false><<<h->norm_blocks, 256, 0, s>>>(v.lhs, v.rhs, v.lay, v.coef, h->prm.res_type,
                                                            h->norm_part);
    kend(h, s, KC_NORM);
    kbegin(h, s, -1);
    k_norm_final<<<1, 32, 0, s>>>(h->norm_part, h->norm_blocks, h->prm.res_type, pc, h->norm_out, nullptr);
}

static void launch_coarsest(saras_mg *h, cudaStream_t s, Level &c) {
    const Lay &C = c.lay;
    const double w = h->prm.sor_param, omc = 1.0 - h->prm.sor_param;
    const int64_t cells = (int64_t)C.n0 * C.n1 * C.n2;
    const int threads = cells <= 1024 ? 32 : 256;
    const size_t smem = (size_t)(2 * C.size) * sizeof(double);
    const bool use_smem = (int64_t)smem <= COARSE_SMEM_LIMIT;
    kbegin(h, s, KC_COARSE);
    if (use_smem) {
        if (h->d3)
            k_coarsest_exact<true, true><<<1, threads, smem, s>>>(c.lhs, c.rhs, C, c.coef, h->ghost, w, omc,
                                                                  h->prm.mg_tolerance, h->maxCount(),
                                                                  h->coarse_sweeps);
        else
            k_coarsest_exact<false, true><<<1, threads, smem, s>>>(c.lhs, c.rhs, C, c.coef, h->ghost, w, omc,
                                                                   h->prm.mg_tolerance, h->maxCount(),
                                                                   h->coarse_sweeps);
    } else {
        if (h->d3)
            k_coarsest_exact<true, false><<<1, threads, 0, s>>>(c.lhs, c.rhs, C, c.coef, h->ghost, w, omc,
                                                                h->prm.mg_tolerance, h->maxCount(),
                                                                h->coarse_sweeps);
        else
            k_coarsest_exact<false, false><<<1, threads, 0, s>>>(c.lhs, c.rhs, C, c.coef, h->ghost, w, omc,
                                                                 h->prm.mg_tolerance, h->maxCount(),
                                                                 h->coarse_sweeps);
    }
    kend(h, s, KC_COARSE);
}

// poisson::vCycle in the FP64_EXACT form.
static void vcycle_exact(saras_mg *h, cudaStream_t s) {
    const int top = h->nl - 1;
    smooth_exact(h, s, 0, h->prm.pre_smooth, false);
    for (int l = 0; l < top; l++) {
        Level &f = h->lv[(size_t)l];
        Level &c = h->lv[(size_t)l + 1];
        const Lay &L = f.lay;
        const int bx = std::min(BX, (L.n2 + 31) / 32 * 32);
        kbegin(h, s, l == 0 ? KC_RESTRICT : -1);
        if (h->d3)
            k_resid_exact<true><<<cell_grid(L, true, L.n2, bx), bx, 0, s>>>(f.lhs, f.rhs, f.tmp, L, f.coef);
        else
            k_resid_exact<false><<<cell_grid(L, false, L.n2, bx), bx, 0, s>>>(f.lhs, f.rhs, f.tmp, L, f.coef);
        kend(h, s, l == 0 ? KC_RESTRICT : -1);
        cudaMemcpyAsync(f.smd, f.lhs, (size_t)L.size * sizeof(double), cudaMemcpyDeviceToDevice, s);
        const Lay &C = c.lay;
        const int cbx = std::min(BX, (C.n2 + 31) / 32 * 32);
        kbegin(h, s, -1);
        if (h->d3)
            k_restrict_exact<true><<<cell_grid(C, true, C.n2, cbx), cbx, 0, s>>>(f.tmp, c.rhs, L, C, c.rt);
        else
            k_restrict_exact<false><<<cell_grid(C, false, C.n2, cbx), cbx, 0, s>>>(f.tmp, c.rhs, L, C, c.rt);
        cudaMemsetAsync(c.lhs, 0, (size_t)C.size * sizeof(double), s);
        if (l + 1 == top && h->prm.solve_flag) {
            launch_coarsest(h, s, c);
        } else {
            smooth_exact(h, s, l + 1, h->prm.pre_smooth, true);
        }
    }
    for (int l = top; l > 0; l--) {
        Level &c = h->lv[(size_t)l];
        Level &f = h->lv[(size_t)l - 1];
        const Lay &L = f.lay;
        const int bx = std::min(BX, (L.n2 + 2 + 31) / 32 * 32);
        kbegin(h, s, l == 1 ? KC_PROLONG : -1);
        k_prolong_exact<<<dim3(cdiv(L.n2 + 2, bx), (unsigned)L.n1 + 2, (unsigned)L.n0 + 2), bx, 0, s>>>(
            c.lhs, f.smd, f.lhs, L, c.lay, h->d3 ? 1 : 0);
        kend(h, s, l == 1 ? KC_PROLONG : -1);
        smooth_exact(h, s, l - 1, h->prm.post_smooth, l - 1 != 0);
    }
    norm_exact(h, s);
}

// Hooks used by the FP64 and MIXED forms (mg_fast.cu).
void coarsest_level(saras_mg *h, cudaStream_t s) {
    const int top = h->nl - 1;
    Level &c = h->lv[(size_t)top];
    if (h->prm.solve_flag) {
        coarsest_fast(h, s, c);  // starts from zero itself
    } else {
        cudaMemsetAsync(c.lhs, 0, (size_t)c.lay.size * sizeof(double), s);
        smooth_exact(h, s, top, h->prm.pre_smooth, true);
    }
}

void norm_final(saras_mg *h, cudaStream_t s) {
    const double pc = h->d3 ? (double)h->grid.N[0] * h->grid.N[1] * h->grid.N[2]
                            : (double)h->grid.N[0] * h->grid.N[2];
    kbegin(h, s, -1);
    k_norm_final<<<1, 32, 0, s>>>(h->norm_part, h->norm_blocks, h->prm.res_type, pc, h->norm_out,
                                  h->norm_out + 4);
}

void ghost_all_level(saras_mg *h, cudaStream_t s, int l, bool zeroBC) { ghost_all(h, s, l, zeroBC); }

}  // namespace saras

int saras_mg::maxCount() const {
    // poisson::setStagBounds (poisson.cc:430-436)
    int cg[3];
    for (int d = 0; d < 3; d++) cg[d] = grid.N[d] / int(std::pow(2, nl - 1));
    return d3 ? int(2.5 * cg[0] * cg[1] * cg[2]) : int(2.5 * cg[0] * cg[2]);
}

// ------------------------------------------------------------ set-up ----

namespace {

// Device array of `count` elements: a 256-byte aligned piece of the
// handle's arena while saras_mg_create carves it (one cudaMalloc per
// hierarchy instead of about thirty: each cudaMalloc may wait for the whole
// device, which a serving engine creating hierarchies beside a running batch
// feels), otherwise its own allocation.
template <class T>
saras_status dalloc(saras_mg *h, T **p, int64_t count) {
    const size_t bytes = (size_t)std::max<int64_t>(count, 1) * sizeof(T);
    if (h->carving && h->arena) {
        const size_t off = (h->arena_used + 255) / 256 * 256;
        if (off + bytes <= h->arena_cap) {
            *p = reinterpret_cast<T *>(h->arena + off);
            h->arena_used = off + bytes;
            return SARAS_OK;
        }
    }
    cudaError_t e = cudaMalloc((void **)p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        set_error("cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? SARAS_OOM : SARAS_CUDA_ERR;
    }
    h->allocs.push_back((void *)*p);
    h->dev_bytes += (int64_t)bytes;
    return SARAS_OK;
}

// Builds the per-level 1-D tables.  On a retarget (new stretching, same
// extents) the device tables are reused and refilled asynchronously on the
// handle's stream from its pinned staging buffer.
saras_status build_tables(saras_mg *h, bool async = false) {
    const HostGrid &g = h->grid;
    for (int l = 0; l < h->nl; l++) {
        Level &v = h->lv[(size_t)l];
        // Per axis: A2, A1 (exact form), cm, cp, dg (FP64 form), r0, r1, rt, w
        // (restriction), each sized to the axis extent.
        int n[3] = {v.lay.n0, v.lay.n1, v.lay.n2};
        const int per_axis = 10;
        int64_t total = 0;
        for (int d = 0; d < 3; d++) total += (int64_t)per_axis * n[d];
        std::vector<double> host((size_t)total, 0.0);
        if (!v.tab) SARAS_TRY(dalloc(h, &v.tab, total));
        std::vector<float> host32((size_t)total, 0.f);
        if (!v.tab32) SARAS_TRY(dalloc(h, &v.tab32, total));
        int64_t off = 0;
        const double *dp[3][per_axis];
        const float *fp[3][per_axis];
        for (int d = 0; d < 3; d++) {
            const AxisLevel &a = g.lv[(size_t)l][(size_t)d];
            const int hInc = 1 << l;
            double ih2 = 0.0, i2h = 0.0;
            if (g.active(d)) {
                // poisson::setCoefficients (poisson.cc:463-482)
                const double hx = hInc * g.dxi[d];
                const double hx2 = std::pow(hx, 2);
                i2h = 0.5 / hx;
                ih2 = 1.0 / hx2;
            }
            for (int q = 0; q < per_axis; q++) {
                dp[d][q] = v.tab + off + (int64_t)q * n[d];
                fp[d][q] = v.tab32 + off + (int64_t)q * n[d];
            }
            for (int i = 0; i < n[d]; i++) {
                const double xix2 = a.at(a.xix2, i), xixx = a.at(a.xixx, i);
                const double A2 = xix2 * ih2, A1 = xixx * i2h;
                double vals[per_axis] = {A2, A1, A2 - A1, A2 + A1, A2, 0, 0, 0, 0.5, 0.5};
                if (l > 0 && g.active(d)) {
                    const AxisLevel &f = g.lv[(size_t)l - 1][(size_t)d];
                    const double xc = a.at(a.x, i), xf0 = f.at(f.x, 2 * i), xf1 = f.at(f.x, 2 * i + 1);
                    vals[5] = xc - xf0;
                    vals[6] = xf1 - xc;
                    vals[7] = xf1 - xf0;
                    vals[8] = vals[5] / vals[7];
                    vals[9] = vals[6] / vals[7];
                }
                for (int q = 0; q < per_axis; q++) {
                    host[(size_t)(off + (int64_t)q * n[d] + i)] = vals[q];
                    host32[(size_t)(off + (int64_t)q * n[d] + i)] = (float)vals[q];
                }
            }
            off += (int64_t)per_axis * n[d];
        }
        if (async) {
            const size_t b64 = host.size() * sizeof(double), b32 = host32.size() * sizeof(float);
            if (!h->tab_stage || h->tab_stage_bytes < h->tab_stage_used + b64 + b32) {
                set_error("table staging buffer too small");
                return SARAS_BAD_ARG;
            }
            char *st64 = h->tab_stage + h->tab_stage_used;
            std::memcpy(st64, host.data(), b64);
            std::memcpy(st64 + b64, host32.data(), b32);
            h->tab_stage_used += (b64 + b32 + 255) / 256 * 256;
            SARAS_CUDA(cudaMemcpyAsync(v.tab, st64, b64, cudaMemcpyHostToDevice, h->stream));
            SARAS_CUDA(cudaMemcpyAsync(v.tab32, st64 + b64, b32, cudaMemcpyHostToDevice, h->stream));
        } else {
            // pageable sources: staged before the calls return, ordered on the stream
            SARAS_CUDA(cudaMemcpyAsync(v.tab, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice,
                                       h->stream));
            SARAS_CUDA(cudaMemcpyAsync(v.tab32, host32.data(), host32.size() * sizeof(float),
                                       cudaMemcpyHostToDevice, h->stream));
        }
        v.coef = Coef{dp[0][0], dp[0][1], dp[1][0], dp[1][1], dp[2][0], dp[2][1]};
        v.rt = RTab{dp[0][5], dp[0][6], dp[0][7], dp[1][5], dp[1][6], dp[1][7], dp[2][5], dp[2][6], dp[2][7]};
        for (int d = 0; d < 3; d++) {
            v.cm[d] = dp[d][2];
            v.cp[d] = dp[d][3];
            v.dg[d] = dp[d][4];
            v.cm32[d] = fp[d][2];
            v.cp32[d] = fp[d][3];
            v.dg32[d] = fp[d][4];
            v.w0[d] = dp[d][8];
            v.w1[d] = dp[d][9];
            v.w032[d] = fp[d][8];
            v.w132[d] = fp[d][9];
        }
    }
    return SARAS_OK;
}

saras_status build_walls(saras_mg *h) {
    // multigrid_d3::initDirichlet / multigrid_d2::initDirichlet
    // (poisson_d3.cc:824-873): analytic r^2/6 (3D) or r^2/4 (2D) on the walls.
    const HostGrid &g = h->grid;
    bool any = false;
    for (int f = 0; f < 6; f++) any = any || h->prm.bc_kind[f] == SARAS_BC_DIRICHLET_TEST;
    if (!any) return SARAS_OK;
    const Lay &L = h->lv[0].lay;
    const int64_t nx = (int64_t)(L.n1 + 2) * (L.n2 + 2), ny = (int64_t)(L.n0 + 2) * (L.n2 + 2),
                  nz = (int64_t)(L.n0 + 2) * (L.n1 + 2);
    std::vector<double> w((size_t)(nx + ny + nz), 0.0);
    const AxisLevel &ax = g.lv[0][0], &ay = g.lv[0][1], &az = g.lv[0][2];
    if (h->d3) {
        const double xd = g.L[0] / 2.0, yd = g.L[1] / 2.0, zd = g.L[2] / 2.0;
        for (int j = 0; j < L.n1; j++)
            for (int k = 0; k < L.n2; k++) {
                const double y = ay.at(ay.x, j) - 0.5, z = az.at(az.x, k) - 0.5;
                w[(size_t)((j + 1) * (L.n2 + 2) + k + 1)] = (xd * xd + y * y + z * z) / 6.0;
            }
        for (int i = 0; i < L.n0; i++)
            for (int k = 0; k < L.n2; k++) {
                const double x = ax.at(ax.x, i) - 0.5, z = az.at(az.x, k) - 0.5;
                w[(size_t)(nx + (i + 1) * (L.n2 + 2) + k + 1)] = (x * x + yd * yd + z * z) / 6.0;
            }
        for (int i = 0; i < L.n0; i++)
            for (int j = 0; j < L.n1; j++) {
                const double x = ax.at(ax.x, i) - 0.5, y = ay.at(ay.x, j) - 0.5;
                w[(size_t)(nx + ny + (i + 1) * (L.n1 + 2) + j + 1)] = (x * x + y * y + zd * zd) / 6.0;
            }
    } else {
        const double xd = g.L[0] / 2.0, zd = g.L[2] / 2.0;
        for (int k = 0; k < L.n2; k++) {
            const double z = az.at(az.x, k) - 0.5;
            w[(size_t)((0 + 1) * (L.n2 + 2) + k + 1)] = (xd * xd + z * z) / 4.0;
        }
        for (int i = 0; i < L.n0; i++) {
            const double x = ax.at(ax.x, i) - 0.5;
            w[(size_t)(nx + ny + (i + 1) * (L.n1 + 2) + 0 + 1)] = (x * x + zd * zd) / 4.0;
        }
    }
    SARAS_TRY(dalloc(h, &h->walls, (int64_t)w.size()));
    SARAS_CUDA(cudaMemcpyAsync(h->walls, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    h->ghost.wallx = h->walls;
    h->ghost.wally = h->walls + nx;
    h->ghost.wallz = h->walls + nx + ny;
    return SARAS_OK;
}

saras_status check_params(const saras_mg_params &p) {
    if (p.vc_count < 1 || p.pre_smooth < 0 || p.post_smooth < 0 || p.res_type < 0 || p.res_type > 2 ||
        p.precision < 0 || p.precision > 2 || p.levels < 0 || p.inner_cycles < -4096 ||
        !(p.sor_param > 0.0 && p.sor_param < 2.0)) {
        set_error("invalid multigrid parameters");
        return SARAS_BAD_ARG;
    }
    for (int f = 0; f < 6; f++)
        if (p.bc_kind[f] < 0 || p.bc_kind[f] > 2) {
            set_error("invalid boundary kind on face %d", f);
            return SARAS_BAD_ARG;
        }
    return SARAS_OK;
}

void free_all(saras_mg *h) {
    // every device array came from dalloc: pieces of the arena or listed
    for (void *q : h->allocs) cudaFree(q);
    h->allocs.clear();
    if (h->arena) cudaFree(h->arena);
    h->arena = nullptr;
    if (h->norm_host) cudaFreeHost(h->norm_host);
    if (h->tab_stage) cudaFreeHost(h->tab_stage);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    if (h->graph_v) cudaGraphExecDestroy(h->graph_v);
    if (h->graph_tail) cudaGraphExecDestroy(h->graph_tail);
    for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
    for (cudaEvent_t e : h->copy_ev)
        if (e) cudaEventDestroy(e);
    if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
}

// Per-level device arrays of each form: FP64 u and f (every level in the
// FP64 forms; the finest and the coarsest in MIXED), FP64 scratch for the
// exact form's separate residual and smoothed copy, the FP32 error and
// residual of MIXED's inner levels, and the stored omega/D and D.
struct LevelArrays {
    bool u_f, scratch, e_r32, inv_diag, dd, fd;
};

LevelArrays level_arrays(int precision, int l, int nl) {
    const bool mixed = precision == SARAS_PREC_MIXED, fast = precision == SARAS_PREC_FP64;
    const bool coarsest = l == nl - 1;
    LevelArrays a;
    a.u_f = !mixed || l == 0 || coarsest;
    a.scratch = precision == SARAS_PREC_FP64_EXACT;
    a.e_r32 = mixed && !coarsest;
    a.inv_diag = fast || (mixed && coarsest);
    a.dd = fast || (mixed && (l == 0 || coarsest));
    a.fd = mixed && coarsest;
    return a;
}

// Pinned staging of the level tables (and exact-solve tables): their
// uploads are then asynchronous, never waiting for work already queued on
// the handle's stream.
saras_status ensure_tab_stage(saras_mg *h) {
    if (!h->tab_stage) {
        size_t bytes = 0;
        for (const Level &v : h->lv) bytes += (size_t)10 * (v.lay.n0 + v.lay.n1 + v.lay.n2) * 12 + 512;
        const Level &top = h->lv.back();
        if (top.fd) bytes += (size_t)fd_elems(top.lay) * sizeof(double) + 256;  // exact-solve tables
        SARAS_CUDA(cudaMallocHost((void **)&h->tab_stage, bytes));
        h->tab_stage_bytes = bytes;
    }
    h->tab_stage_used = 0;
    return SARAS_OK;
}

// `wait`: return with the set-up complete on the handle's stream.  Without
// it the set-up stays queued on that stream (ordered before any later work
// the caller puts there), so creating a handle never waits for other work
// already queued on the stream.
saras_status create(const saras_grid_desc *gd, const saras_mg_params *prm, void *stream, saras_mg *h,
                    bool wait = true) {
    SARAS_TRY(check_params(*prm));
    h->prm = *prm;
    SARAS_TRY(h->grid.build(*gd, prm->levels));
    h->d3 = h->grid.dims == 3;
    h->nl = h->grid.levels;
    h->stream = (cudaStream_t)stream;
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
        cudaGetLastError();
        set_error("no CUDA device");
        return SARAS_NO_DEVICE;
    }
    for (int d = 0; d < 3; d++) h->ghost.per[d] = h->grid.per[d] ? 1 : 0;
    for (int f = 0; f < 6; f++) h->ghost.kind[f] = prm->bc_kind[f];
    h->lv.resize((size_t)h->nl);
    if (prm->precision == SARAS_PREC_MIXED && h->nl < 2) {
        set_error("the MIXED form needs at least two levels");
        return SARAS_BAD_ARG;
    }
    {
        // one allocation for the hierarchy: the bytes the per-level rule
        // gives plus the alignment of every piece
        const int64_t est = mg_estimate_bytes(gd, prm);
        if (est > 0) {
            const size_t cap = (size_t)est + (size_t)256 * (16 * (size_t)h->nl + 32);
            if (cudaMalloc((void **)&h->arena, cap) == cudaSuccess) {
                h->arena_cap = cap;
                h->dev_bytes += (int64_t)cap;
                h->carving = true;
            } else {
                cudaGetLastError();
                h->arena = nullptr;
            }
        }
    }
    for (int l = 0; l < h->nl; l++) {
        Level &v = h->lv[(size_t)l];
        const AxisLevel *a = h->grid.lv[(size_t)l].data();
        v.lay = make_lay(a[0].n, h->d3 ? a[1].n : 1, a[2].n);
        const int64_t sz = v.lay.size;
        const LevelArrays use = level_arrays(prm->precision, l, h->nl);
        if (use.u_f) {
            SARAS_TRY(dalloc(h, &v.lhs, sz));
            SARAS_TRY(dalloc(h, &v.rhs, sz));
            SARAS_CUDA(cudaMemsetAsync(v.lhs, 0, (size_t)sz * sizeof(double), h->stream));
            SARAS_CUDA(cudaMemsetAsync(v.rhs, 0, (size_t)sz * sizeof(double), h->stream));
        }
        if (use.scratch) {
            SARAS_TRY(dalloc(h, &v.tmp, sz));
            SARAS_TRY(dalloc(h, &v.smd, sz));
        }
        if (use.e_r32) {
            SARAS_TRY(dalloc(h, &v.e32, sz));
            SARAS_TRY(dalloc(h, &v.r32, sz));
            SARAS_CUDA(cudaMemsetAsync(v.e32, 0, (size_t)sz * sizeof(float), h->stream));
            SARAS_CUDA(cudaMemsetAsync(v.r32, 0, (size_t)sz * sizeof(float), h->stream));
            if (fused_sweep_fits(v.lay, h->d3) || pair_sweep_fits(v.lay, h->d3)) SARAS_TRY(dalloc(h, &v.e32b, sz));
        }
        if (use.inv_diag) SARAS_TRY(dalloc(h, &v.inv_diag, sz));
        if (use.dd) SARAS_TRY(dalloc(h, &v.dd, sz));
        if (use.fd && fd_fits(v.lay)) SARAS_TRY(dalloc(h, &v.fd, fd_elems(v.lay)));
    }
    SARAS_TRY(ensure_tab_stage(h));
    SARAS_TRY(build_tables(h, true));
    SARAS_TRY(build_walls(h));
    const Lay &L0 = h->lv[0].lay;
    const int64_t cells = (int64_t)L0.n0 * L0.n1 * L0.n2;
    h->norm_blocks = (int)std::max<int64_t>(1, std::min<int64_t>(1216, (cells + 255) / 256));
    SARAS_TRY(dalloc(h, &h->norm_part, 4 * (int64_t)h->norm_blocks));
    SARAS_TRY(dalloc(h, &h->norm_out, 8));
    SARAS_TRY(dalloc(h, &h->coarse_sweeps, 4));
    SARAS_TRY(dalloc(h, &h->mix_scalar, 16));
    h->carving = false;  // later allocations (the host entry point's boxes) are their own
    SARAS_CUDA(cudaMemsetAsync(h->coarse_sweeps, 0, 4 * sizeof(int), h->stream));
    SARAS_CUDA(cudaMemsetAsync(h->norm_out, 0, 8 * sizeof(double), h->stream));
    SARAS_CUDA(cudaMallocHost((void **)&h->norm_host, 8 * sizeof(double)));
    // Dense padded box of a caller field for the host entry point.
    const int p = h->grid.pad, py = h->d3 ? p : 1;
    h->stage_st[2] = 1;
    h->stage_st[1] = L0.n2 + 2 * p;
    h->stage_st[0] = h->stage_st[1] * (L0.n1 + 2 * py);
    h->stage_elems = h->stage_st[0] * (L0.n0 + 2 * p);
    SARAS_CUDA(cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking));
    SARAS_CUDA(cudaFuncSetAttribute(k_coarsest_exact<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)COARSE_SMEM_LIMIT));
    SARAS_CUDA(cudaFuncSetAttribute(k_coarsest_exact<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)COARSE_SMEM_LIMIT));
    if (prm->precision != SARAS_PREC_FP64_EXACT) SARAS_TRY(fast_setup(h));
    // everything above is ordered on the handle's stream: wait for it alone,
    // not for other work on the device (a serving batch keeps running)
    if (wait) SARAS_CUDA(cudaStreamSynchronize(h->stream));
    return SARAS_OK;
}

// Issues one V-cycle (with its norm and the host copy of the norm).
void issue_cycle(saras_mg *h, cudaStream_t s) {
    h->issued = 0;
    if (h->prm.precision == SARAS_PREC_FP64_EXACT)
        vcycle_exact(h, s);
    else
        fast_cycle(h, s);
    cudaMemcpyAsync(h->norm_host, h->norm_out, 8 * sizeof(double), cudaMemcpyDeviceToHost, s);
}

saras_status ensure_graph(saras_mg *h) {
    if (h->graph && h->graph_timing != h->timing) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
        h->graph_marks.clear();
        h->ev_base = 0;
    }
    if (h->graph || !h->use_graph) return SARAS_OK;
    if (h->timing) {
        // events are created before capture; the marks recorded while
        // capturing become the graph's event-record nodes
        h->ev_marks.clear();
        h->ev_used = 0;
        if (h->ev_pool.size() < 4096) {
            while (h->ev_pool.size() < 4096) {
                cudaEvent_t e;
                SARAS_CUDA(cudaEventCreate(&e));
                h->ev_pool.push_back(e);
            }
        }
    }
    cudaGraph_t g = nullptr;
    SARAS_CUDA(cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal));
    h->capturing = true;
    issue_cycle(h, h->cap_stream);
    h->capturing = false;
    cudaError_t e = cudaStreamEndCapture(h->cap_stream, &g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        h->use_graph = false;  // fall back to direct launches
        return SARAS_OK;
    }
    h->launches_cycle = h->issued;
    h->graph_marks = h->ev_marks;
    h->ev_marks.clear();
    h->ev_base = h->ev_used;
    h->graph_timing = h->timing;
    e = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        h->graph = nullptr;
        h->use_graph = false;
    }
    return SARAS_OK;
}

// A MIXED outer iteration of n < the full count of V-cycles (adaptive inner
// counts): its head, n replays of a one-V-cycle graph and its tail with the
// norm's host copy.  The two graphs are captured on first use; with kernel
// timing on, or without graphs, the pieces are issued directly.
saras_status short_iteration(saras_mg *h, cudaStream_t s, int n) {
    const bool graphs = h->use_graph && !h->timing;
    if (graphs && !h->graph_v) {
        for (int q = 0; q < 2; q++) {
            cudaGraph_t g = nullptr;
            SARAS_CUDA(cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal));
            h->capturing = true;
            h->issued = 0;
            if (q == 0) {
                vcycle_fast(h, h->cap_stream, true);
            } else {
                mixed_tail(h, h->cap_stream);
                cudaMemcpyAsync(h->norm_host, h->norm_out, 8 * sizeof(double), cudaMemcpyDeviceToHost,
                                h->cap_stream);
            }
            h->capturing = false;
            SARAS_CUDA(cudaStreamEndCapture(h->cap_stream, &g));
            cudaGraphExec_t ge = nullptr;
            const cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
            SARAS_CUDA(e);
            (q == 0 ? h->graph_v : h->graph_tail) = ge;
            (q == 0 ? h->launches_v : h->launches_tail) = h->issued;
        }
    }
    mixed_head(h, s);
    h->last_launches += 1;
    if (graphs) {
        for (int q = 0; q < n; q++) SARAS_CUDA(cudaGraphLaunch(h->graph_v, s));
        SARAS_CUDA(cudaGraphLaunch(h->graph_tail, s));
        h->last_launches += n * h->launches_v + h->launches_tail;
    } else {
        h->issued = 0;
        h->timing_direct = true;
        for (int q = 0; q < n; q++) vcycle_fast(h, s, true);
        mixed_tail(h, s);
        h->timing_direct = false;
        cudaMemcpyAsync(h->norm_host, h->norm_out, 8 * sizeof(double), cudaMemcpyDeviceToHost, s);
        h->last_launches += h->issued;
    }
    return SARAS_OK;
}

// poisson::mgSolve on level-0 arrays already filled by the caller path.
saras_status solve_loop(saras_mg *h, double *res_hist, int32_t hist_cap, int32_t *n_cycles) {
    cudaStream_t s = h->stream;
    h->inner_now = 0;
    // the TMA sweeps' error word starts clear: an earlier solve whose wait
    // ran out leaves the handle usable
    SARAS_CUDA(cudaMemsetAsync(h->norm_out + 7, 0, sizeof(double), s));
    SARAS_TRY(ensure_graph(h));
    int cyc = 0;
    double r = 0.0;
    // MIXED form with a negative inner_cycles: outer iterations of up to
    // -inner_cycles V-cycles; once the residual is within reach, the next
    // iteration runs the V-cycles the last one's contraction says the
    // tolerance still needs (plus one) instead of the full count
    const bool mixed = h->prm.precision == SARAS_PREC_MIXED;
    const bool adapt = mixed && h->prm.inner_cycles < 0;
    const int full = mixed ? (adapt ? -h->prm.inner_cycles : std::max(1, h->prm.inner_cycles)) : 1;
    int n_next = full;
    double r_prev = -1.0;
    h->last_vcycles = 0;
    for (int c = 0; c < h->prm.vc_count; c++) {
        if (h->prm.precision != SARAS_PREC_FP64_EXACT && c == 0) rhs_norm(h, s);
        if (mixed && c == 0) {
            // the defect-correction loop starts from the residual of the guess
            mixed_prepare(h, s);
        }
        const int n_this = n_next;
        // whether this iteration's kernel-timing marks are the graph's
        bool from_graph = h->graph != nullptr;
        if (adapt && n_this < full) {
            from_graph = false;
            h->inner_now = n_this;
            const saras_status st = short_iteration(h, s, n_this);
            h->inner_now = 0;
            SARAS_TRY(st);
        } else if (h->graph) {
            SARAS_CUDA(cudaGraphLaunch(h->graph, s));
            h->last_launches += h->launches_cycle;
        } else {
            issue_cycle(h, s);
            h->last_launches += h->issued;
        }
        h->last_vcycles += n_this;
        SARAS_CUDA(cudaStreamSynchronize(s));
        harvest_timing(h, from_graph);
        r = h->norm_host[0];
        cyc++;
        int tma_err = 0;
        std::memcpy(&tma_err, h->norm_host + 7, sizeof(int));
        if (tma_err) {
            if (n_cycles) *n_cycles = cyc;
            set_error("a bounded wait of the TMA sweep ran out in V-cycle %d", c);
            return SARAS_TIMEOUT;
        }
        if (res_hist && c < hist_cap) res_hist[c] = r;
        if (h->prm.print_residual) std::printf("\nResidual after V Cycle %d is %.3e\n", c, r);
        if (!std::isfinite(r)) {
            if (n_cycles) *n_cycles = cyc;
            set_error("non-finite residual after V-cycle %d", c);
            return SARAS_NAN;
        }
        if (!h->prm.test_poisson && r < h->prm.vc_tolerance) break;
        if (adapt) {
            n_next = full;
            if (r_prev > 0.0 && r > 0.0 && r < r_prev) {
                const double rho = std::pow(r / r_prev, 1.0 / n_this);
                const double need = std::log(h->prm.vc_tolerance / r) / std::log(rho);
                if (need >= 0.0 && need + 1.0 < full) n_next = std::max(1, (int)std::ceil(need) + 1);
            }
            r_prev = r;
        }
    }
    if (h->prm.precision == SARAS_PREC_MIXED)
        mixed_finish(h, s);
    else if (h->prm.precision == SARAS_PREC_FP64)
        final_ghosts(h, s);
    if (n_cycles) *n_cycles = cyc;
    if (h->prm.test_poisson) return SARAS_OK;
    return r < h->prm.vc_tolerance ? SARAS_OK : SARAS_NOT_CONVERGED;
}

saras_status solve_common(saras_mg *h, double *lhs, const double *rhs, const int64_t st[3], double *res_hist,
                          int32_t hist_cap, int32_t *n_cycles) {
    cudaStream_t s = h->stream;
    Level &v0 = h->lv[0];
    const Lay &L = v0.lay;
    h->last_launches = 0;
    double *u0 = v0.lhs;
    double *f0 = v0.rhs;
    // mgSolve zeroes the finest arrays before copying the caller's core in
    SARAS_CUDA(cudaMemsetAsync(u0, 0, (size_t)L.size * sizeof(double), s));
    SARAS_CUDA(cudaMemsetAsync(f0, 0, (size_t)L.size * sizeof(double), s));
    const int bx = std::min(BX, (L.n2 + 31) / 32 * 32);
    k_scatter<<<dim3(cdiv(L.n2, bx), (unsigned)L.n1, (unsigned)L.n0), bx, 0, s>>>(lhs, rhs, st[0], st[1], st[2],
                                                                                u0, f0, L);
    h->last_launches += 1;
    saras_status status = solve_loop(h, res_hist, hist_cap, n_cycles);
    if (status != SARAS_OK && status != SARAS_NOT_CONVERGED) return status;
    const int gbx = std::min(BX, (L.n2 + 2 + 31) / 32 * 32);
    k_gather<<<dim3(cdiv(L.n2 + 2, gbx), (unsigned)L.n1 + 2, (unsigned)L.n0 + 2), gbx, 0, s>>>(u0, L, lhs, st[0],
                                                                                            st[1], st[2]);
    h->last_launches += 1;
    SARAS_CUDA(cudaGetLastError());
    return status;
}

}  // namespace

namespace saras {

// Device bytes saras_mg_create allocates for a grid and form (the host
// solve's staging boxes, made on first use, excluded), from the same
// per-level rule; the serving engine admits against it.
int64_t mg_estimate_bytes(const saras_grid_desc *gd, const saras_mg_params *prm) {
    HostGrid g;
    if (g.build(*gd, prm->levels) != SARAS_OK) return -1;
    const bool d3 = g.dims == 3;
    int64_t bytes = 0;
    int64_t cells0 = 0;
    for (int l = 0; l < g.levels; l++) {
        const AxisLevel *a = g.lv[(size_t)l].data();
        const Lay L = make_lay(a[0].n, d3 ? a[1].n : 1, a[2].n);
        if (l == 0) cells0 = (int64_t)L.n0 * L.n1 * L.n2;
        const LevelArrays u = level_arrays(prm->precision, l, g.levels);
        bytes += L.size * (16 * u.u_f + 16 * u.scratch + 8 * u.e_r32 + 8 * u.inv_diag + 8 * u.dd);
        if (u.e_r32 && (fused_sweep_fits(L, d3) || pair_sweep_fits(L, d3)))
            bytes += 4 * L.size;  // the fused iterations' second e buffer
        if (u.fd && fd_fits(L)) bytes += 8 * fd_elems(L);
        bytes += (int64_t)10 * (L.n0 + L.n1 + L.n2) * 12;  // 1-D tables, FP64 and FP32
        if (l == 0) {
            bool walls = false;
            for (int f = 0; f < 6; f++) walls = walls || prm->bc_kind[f] == SARAS_BC_DIRICHLET_TEST;
            if (walls)
                bytes += 8 * ((int64_t)(L.n1 + 2) * (L.n2 + 2) + (int64_t)(L.n0 + 2) * (L.n2 + 2) +
                              (int64_t)(L.n0 + 2) * (L.n1 + 2));
        }
    }
    const int64_t nb = std::max<int64_t>(1, std::min<int64_t>(1216, (cells0 + 255) / 256));
    bytes += 32 * nb + 8 * 8 + 4 * 4 + 16 * 8;
    return bytes;
}

// Re-points a handle at a grid with the same extents, periodicity and depth
// but other stretching (serving engine: hierarchies are reused across
// requests of one shape).  Tables and per-cell diagonals are refilled on the
// handle's stream; no allocation.
saras_status mg_retarget(saras_mg *h, const saras_grid_desc *gd) {
    HostGrid g;
    SARAS_TRY(g.build(*gd, h->prm.levels));
    if (g.levels != h->nl || g.dims != h->grid.dims || g.pad != h->grid.pad) return SARAS_BAD_ARG;
    for (int d = 0; d < 3; d++)
        if (g.N[d] != h->grid.N[d] || g.per[d] != h->grid.per[d]) return SARAS_BAD_ARG;
    SARAS_TRY(ensure_tab_stage(h));
    h->grid = g;
    SARAS_TRY(build_tables(h, true));
    return fast_setup(h);
}

// saras_mg_create whose set-up stays queued on `stream` (serving
// admissions: the handle's later work is ordered behind it on that stream).
saras_status mg_create_queued(const saras_grid_desc *gd, const saras_mg_params *prm, void *stream,
                              saras_mg **out) {
    *out = nullptr;
    saras_mg *h = new saras_mg();
    saras_status s = create(gd, prm, stream, h, false);
    if (s != SARAS_OK) {
        if (h->stream) cudaStreamSynchronize(h->stream);
        free_all(h);
        delete h;
        return s;
    }
    *out = h;
    return SARAS_OK;
}

// Finest-level fields of a resident handle: zero initial guess and the RHS
// core from a dense padded device box (serving admissions).
saras_status mg_load_rhs(saras_mg *h, const double *rhs_box_origin, const int64_t st[3]) {
    cudaStream_t s = h->stream;
    Level &v0 = h->lv[0];
    const Lay &L = v0.lay;
    SARAS_CUDA(cudaMemsetAsync(v0.lhs, 0, (size_t)L.size * sizeof(double), s));
    SARAS_CUDA(cudaMemsetAsync(v0.rhs, 0, (size_t)L.size * sizeof(double), s));
    const int bx = std::min(BX, (L.n2 + 31) / 32 * 32);
    k_scatter<<<dim3(cdiv(L.n2, bx), (unsigned)L.n1, (unsigned)L.n0), bx, 0, s>>>(
        rhs_box_origin, rhs_box_origin, st[0], st[1], st[2], v0.lhs, v0.rhs, L);
    SARAS_CUDA(cudaMemsetAsync(v0.lhs, 0, (size_t)L.size * sizeof(double), s));
    return SARAS_OK;
}

// Core plus one ghost layer of the finest lhs into a dense padded device box.
void mg_store_lhs(saras_mg *h, double *box_origin, const int64_t st[3]) {
    Level &v0 = h->lv[0];
    const Lay &L = v0.lay;
    const int gbx = std::min(BX, (L.n2 + 2 + 31) / 32 * 32);
    k_gather<<<dim3(cdiv(L.n2 + 2, gbx), (unsigned)L.n1 + 2, (unsigned)L.n0 + 2), gbx, 0, h->stream>>>(
        v0.lhs, L, box_origin, st[0], st[1], st[2]);
}

// mgSolve on the finest-level arrays as they stand: the caller has written
// the RHS core into lv[0].rhs and keeps the initial guess in lv[0].lhs.
// Used by the RK3 integrator, whose pressure correction lives there.
saras_status mg_solve_resident(saras_mg *h, int32_t *n_cycles) {
    h->last_launches = 0;
    return solve_loop(h, nullptr, 0, n_cycles);
}

}  // namespace saras

// ------------------------------------------------------- C entry points ----

extern "C" {

void saras_mg_default_params(saras_mg_params *p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    // Multigrid section of input/parameters.yaml
    p->vc_count = 20;
    p->vc_tolerance = 1.0e-6;
    p->solve_flag = 1;
    p->mg_tolerance = 1.0e-2;
    p->sor_param = 1.0;
    p->pre_smooth = 3;
    p->post_smooth = 6;
    p->res_type = 0;
    p->print_residual = 0;
    for (int f = 0; f < 6; f++) p->bc_kind[f] = SARAS_BC_NEUMANN;
    p->test_poisson = 0;
    p->precision = SARAS_PREC_FP64_EXACT;
    p->levels = 0;
    p->inner_cycles = 1;
}

saras_status saras_mg_create(const saras_grid_desc *grid, const saras_mg_params *prm, void *stream,
                             saras_mg **out) {
    if (!grid || !prm || !out) {
        set_error("null argument");
        return SARAS_BAD_ARG;
    }
    *out = nullptr;
    saras_mg *h = new saras_mg();
    saras_status s = create(grid, prm, stream, h);
    if (s != SARAS_OK) {
        free_all(h);
        delete h;
        return s;
    }
    *out = h;
    return SARAS_OK;
}

saras_status saras_mg_solve_dev(saras_mg *h, double *lhs, const double *rhs, const int64_t strides[3],
                                double *res_hist, int32_t hist_cap, int32_t *n_cycles) {
    if (!h || !lhs || !rhs || !strides) {
        set_error("null argument");
        return SARAS_BAD_ARG;
    }
    return solve_common(h, lhs, rhs, strides, res_hist, hist_cap, n_cycles);
}

saras_status saras_mg_solve(saras_mg *h, double *lhs, const double *rhs, const int64_t strides[3],
                            double *res_hist, int32_t hist_cap, int32_t *n_cycles) {
    if (!h || !lhs || !rhs || !strides) {
        set_error("null argument");
        return SARAS_BAD_ARG;
    }
    // Host fields must be dense padded boxes (the plainsf layout).
    for (int d = 0; d < 3; d++)
        if (strides[d] != h->stage_st[d]) {
            set_error("host fields must be C-contiguous padded arrays (stride %d is %lld, expected %lld)", d,
                      (long long)strides[d], (long long)h->stage_st[d]);
            return SARAS_BAD_ARG;
        }
    const int p = h->grid.pad, py = h->d3 ? p : 1;
    const int64_t origin = p * h->stage_st[0] + py * h->stage_st[1] + p;
    const size_t bytes = (size_t)h->stage_elems * sizeof(double);
    cudaStream_t s = h->stream;
    if (!h->stage_lhs) {  // device copies of the caller's boxes, made on first use
        SARAS_TRY(dalloc(h, &h->stage_lhs, h->stage_elems));
        SARAS_TRY(dalloc(h, &h->stage_rhs, h->stage_elems));
    }
    // with kernel timing on, the copies are bracketed by events too
    const bool tc = h->timing;
    if (tc && !h->copy_ev[0])
        for (int q = 0; q < 4; q++) SARAS_CUDA(cudaEventCreate(&h->copy_ev[q]));
    if (tc) SARAS_CUDA(cudaEventRecord(h->copy_ev[0], s));
    SARAS_CUDA(cudaMemcpyAsync(h->stage_lhs, lhs - origin, bytes, cudaMemcpyHostToDevice, s));
    SARAS_CUDA(cudaMemcpyAsync(h->stage_rhs, rhs - origin, bytes, cudaMemcpyHostToDevice, s));
    if (tc) SARAS_CUDA(cudaEventRecord(h->copy_ev[1], s));
    saras_status st = solve_common(h, h->stage_lhs + origin, h->stage_rhs + origin, h->stage_st, res_hist,
                                   hist_cap, n_cycles);
    if (st != SARAS_OK && st != SARAS_NOT_CONVERGED) return st;
    if (tc) SARAS_CUDA(cudaEventRecord(h->copy_ev[2], s));
    SARAS_CUDA(cudaMemcpyAsync(lhs - origin, h->stage_lhs, bytes, cudaMemcpyDeviceToHost, s));
    if (tc) SARAS_CUDA(cudaEventRecord(h->copy_ev[3], s));
    SARAS_CUDA(cudaStreamSynchronize(s));
    if (tc) {
        float a = 0.f, b = 0.f;
        SARAS_CUDA(cudaEventElapsedTime(&a, h->copy_ev[0], h->copy_ev[1]));
        SARAS_CUDA(cudaEventElapsedTime(&b, h->copy_ev[2], h->copy_ev[3]));
        h->kc_ms[KC_H2D] += a;
        h->kc_launches[KC_H2D] += 2;
        h->kc_ms[KC_D2H] += b;
        h->kc_launches[KC_D2H] += 1;
    }
    return st;
}

saras_status saras_mg_destroy(saras_mg *h) {
    if (!h) return SARAS_OK;
    cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
    return SARAS_OK;
}

int32_t saras_mg_num_levels(const saras_mg *h) { return h ? h->nl : -1; }

int64_t saras_mg_device_bytes(const saras_mg *h) { return h ? h->dev_bytes : -1; }

saras_status saras_mg_set_kernel_timing(saras_mg *h, int32_t enable) {
    if (!h) return SARAS_BAD_ARG;
    h->timing = enable != 0;
    for (int c = 0; c < KC_COUNT; c++) {
        h->kc_launches[c] = 0;
        h->kc_ms[c] = 0.0;
    }
    return SARAS_OK;
}

saras_status saras_mg_kernel_stats(saras_mg *h, int32_t kclass, int64_t *launches, double *total_ms,
                                   double *bytes_per_launch) {
    if (!h || kclass < 0 || kclass >= KC_COUNT) return SARAS_BAD_ARG;
    if (launches) *launches = h->kc_launches[kclass];
    if (total_ms) *total_ms = h->kc_ms[kclass];
    if (bytes_per_launch) *bytes_per_launch = kernel_bytes(h, kclass);
    return SARAS_OK;
}

saras_status saras_mg_set_wait_limit(saras_mg *h, int64_t polls) {
    if (!h || polls < 0 || polls > 0xffffffffLL) {
        set_error("invalid argument");
        return SARAS_BAD_ARG;
    }
    if ((unsigned)polls == h->wait_limit) return SARAS_OK;
    // the captured graphs hold the old bound: capture them again on next use
    SARAS_CUDA(cudaStreamSynchronize(h->stream));
    if (h->graph) cudaGraphExecDestroy(h->graph);
    if (h->graph_v) cudaGraphExecDestroy(h->graph_v);
    if (h->graph_tail) cudaGraphExecDestroy(h->graph_tail);
    h->graph = h->graph_v = h->graph_tail = nullptr;
    h->graph_marks.clear();
    h->ev_base = 0;
    h->wait_limit = (unsigned)polls;
    return SARAS_OK;
}

int64_t saras_mg_last_launches(const saras_mg *h) { return h ? h->last_launches : -1; }

int64_t saras_mg_last_vcycles(const saras_mg *h) { return h ? h->last_vcycles : -1; }

}  // extern "C"

// ------------------------------------------- solve in caller scratch ----

namespace saras {

// One mgSolve (FP64 or MIXED form) whose device working memory is carved
// out of `scratch` (scratch_bytes long, 256-byte aligned) instead of being
// allocated: the hierarchy, its 1-D tables and the residual-norm scratch.
// The call allocates no device or pinned memory; its host-side grid tables
// and the staging of their upload are ordinary host memory.  Nothing in the
// scratch needs to start at zero: the finest arrays are cleared by the solve
// itself, every coarse array is written before it is read, and the norm
// outputs and coarse-sweep counter are cleared here.  The work is ordered on
// `stream`; the scratch is reused by the next call, so calls that overlap in
// time (other streams, other host threads) race on it.
saras_status mg_solve_in_scratch(const saras_grid_desc *gd, const saras_mg_params *prm, cudaStream_t stream,
                                 char *scratch, size_t scratch_bytes, double *lhs, const double *rhs,
                                 const int64_t st[3], double *res_hist, int32_t hist_cap, int32_t *n_cycles) {
    SARAS_TRY(check_params(*prm));
    if (prm->precision != SARAS_PREC_FP64 && prm->precision != SARAS_PREC_MIXED) {
        set_error("the static-scratch solve runs the FP64 and MIXED forms only");
        return SARAS_BAD_ARG;
    }
    saras_mg h;
    h.prm = *prm;
    SARAS_TRY(h.grid.build(*gd, prm->levels));
    h.d3 = h.grid.dims == 3;
    h.nl = h.grid.levels;
    h.stream = stream;
    h.use_graph = false;
    if (prm->precision == SARAS_PREC_MIXED && h.nl < 2) {
        set_error("the MIXED form needs at least two levels");
        return SARAS_BAD_ARG;
    }
    for (int d = 0; d < 3; d++) h.ghost.per[d] = h.grid.per[d] ? 1 : 0;
    for (int f = 0; f < 6; f++) h.ghost.kind[f] = prm->bc_kind[f];
    h.lv.resize((size_t)h.nl);
    // carve the scratch: every array starts on a 256-byte boundary
    size_t off = 0;
    auto take = [&](auto **p, int64_t count) {
        using T = std::remove_reference_t<decltype(**p)>;
        off = (off + 255) / 256 * 256;
        const size_t bytes = (size_t)std::max<int64_t>(count, 1) * sizeof(T);
        *p = off + bytes <= scratch_bytes ? reinterpret_cast<T *>(scratch + off) : nullptr;
        off += bytes;
    };
    size_t stage_bytes = 0;
    for (int l = 0; l < h.nl; l++) {
        Level &v = h.lv[(size_t)l];
        const AxisLevel *a = h.grid.lv[(size_t)l].data();
        v.lay = make_lay(a[0].n, h.d3 ? a[1].n : 1, a[2].n);
        const int64_t sz = v.lay.size;
        const LevelArrays use = level_arrays(prm->precision, l, h.nl);
        if (use.u_f) {
            take(&v.lhs, sz);
            take(&v.rhs, sz);
        }
        if (use.e_r32) {
            take(&v.e32, sz);
            take(&v.r32, sz);
            if (fused_sweep_fits(v.lay, h.d3) || pair_sweep_fits(v.lay, h.d3)) take(&v.e32b, sz);
        }
        if (use.inv_diag) take(&v.inv_diag, sz);
        if (use.dd) take(&v.dd, sz);
        if (use.fd && fd_fits(v.lay)) take(&v.fd, fd_elems(v.lay));
        const int64_t total = (int64_t)10 * (v.lay.n0 + v.lay.n1 + v.lay.n2);
        take(&v.tab, total);
        take(&v.tab32, total);
        stage_bytes += (size_t)total * 12 + 256;
    }
    const Lay &L0 = h.lv[0].lay;
    const int64_t cells = (int64_t)L0.n0 * L0.n1 * L0.n2;
    h.norm_blocks = (int)std::max<int64_t>(1, std::min<int64_t>(1216, (cells + 255) / 256));
    take(&h.norm_part, 4 * (int64_t)h.norm_blocks);
    take(&h.norm_out, 8);
    take(&h.coarse_sweeps, 4);
    take(&h.mix_scalar, 16);
    if (off > scratch_bytes) {
        set_error("grid needs %zu bytes of solver scratch; the static scratch holds %zu bytes", off, scratch_bytes);
        return SARAS_BUDGET;
    }
    h.dev_bytes = 0;
    double norm_host[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    h.norm_host = norm_host;
    std::vector<char> stage(stage_bytes);
    h.tab_stage = stage.data();
    h.tab_stage_bytes = stage.size();
    h.tab_stage_used = 0;
    SARAS_CUDA(cudaMemsetAsync(h.norm_out, 0, 8 * sizeof(double), stream));
    SARAS_CUDA(cudaMemsetAsync(h.coarse_sweeps, 0, 4 * sizeof(int), stream));
    saras_status s = build_tables(&h, true);  // pageable sources: staged at the call, ordered on the stream
    h.tab_stage = nullptr;
    h.norm_host = norm_host;
    if (s == SARAS_OK) s = fast_setup(&h);
    if (s == SARAS_OK) s = solve_common(&h, lhs, rhs, st, res_hist, hist_cap, n_cycles);
    // whatever the outcome, work queued on the stream (the finishing kernels
    // and the gather) may still read the scratch: the call returns only once
    // it is done, so that the next call, on any stream, may reuse the scratch
    const cudaError_t e = cudaStreamSynchronize(stream);
    h.norm_host = nullptr;
    if (e != cudaSuccess && (s == SARAS_OK || s == SARAS_NOT_CONVERGED))
        return cuda_fail(e, "cudaStreamSynchronize", __FILE__, __LINE__);
    return s;
}

}  // namespace saras
