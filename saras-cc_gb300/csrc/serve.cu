// Serving engine: continuous batching of independent multigrid Poisson
// requests and time-step requests of uneven sizes on one GB300.
//
// Every admitted request keeps its MIXED-form hierarchy resident in HBM (a
// saras_mg handle taken from a per-shape pool and re-pointed at the
// request's stretching).  One outer iteration of ALL admitted requests runs
// as one CUDA-graph launch: each stage of the V-cycle is one batched,
// grid-stride kernel that walks a device table of work items (case, level,
// block of rows).  A graph is captured once per hierarchy depth; its kernels
// read the item tables and their lengths from device memory, so admitting or
// retiring a request only rewrites the tables between launches.
//
// A time-step request (one lsRK3 or eulerCN timeAdvance of its fields) runs
// its right-hand sides, Crank-Nicolson sweeps and corrections on the engine
// stream between batched iterations, and each of its pressure solves joins
// the batch as a case on the integrator's own hierarchy.
//
// A request's arithmetic never depends on the others or on the schedule:
// items touch only their own case, the colour sweeps update disjoint cells,
// and each case's L-infinity residual is a maximum over its own items.  A
// result is therefore the same alone and in any mix, and the same as the
// single-problem MIXED solve (mg_fast.cu) with the engine's parameters.
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "mg_fast.cuh"
#include "mg_stencil.cuh"

using namespace saras;

namespace {

constexpr int DMAX = 10;            // deepest hierarchy the graphs cover
constexpr int NREG = 3 * DMAX + 1;  // item regions: smooth[l], restrict[l], top[l], norm
constexpr int REG_SMOOTH = 0, REG_RESTRICT = DMAX, REG_TOP = 2 * DMAX, REG_NORM = 3 * DMAX;
constexpr int COARSE_THREADS = 128;
constexpr size_t COARSE_SMEM_CAP = 200 * 1024;  // single-problem coarsest-solve limit (mg_fast.cu)

// One level of one case as the batched kernels see it.
struct BLev {
    Lay lay;
    int d3;
    float *e, *r;             // FP32 error and right-hand side (levels above the coarsest)
    double *u, *f, *dd, *wd;  // FP64: finest (u, f, dd) or coarsest (u, f, dd, wd)
    Tab3<float> t32;
    WTab<float> w32;          // weights restricting into this level
    Tab3<double> t64;
    Bnd b;
    int top;                  // this level is the case's coarsest (FP64)
    int max_count;            // coarsest iteration limit
    int sweep_only;           // > 0: coarsest too large for one block; plain sweeps
    FDiag fd;                 // exact coarsest solve (fd.ok), as the single-problem MIXED form
    double tol;
    float w, omc;
    double omc64;
};

// A block of rows of one level (lev) with the next coarser level of the same
// case (clev).  Norm items reuse the fields: lev = slot, row0 = first finest
// item, nrows = number of finest items.
struct BItem {
    int lev, clev, row0, nrows;
};

__device__ __forceinline__ void row_ij(const Lay &L, int row, int &i, int &j) {
    i = row / L.n1;
    j = row - i * L.n1;
}

__device__ __forceinline__ unsigned long long abs_bits(double r) {
    return (unsigned long long)__double_as_longlong(r) & 0x7fffffffffffffffull;
}

// Block-wide maximum of non-negative doubles as bit patterns (NaN sorts last).
__device__ __forceinline__ unsigned long long block_max_bits(unsigned long long m, unsigned long long *shm) {
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, m, o);
        m = w > m ? w : m;
    }
    if ((threadIdx.x & 31) == 0) shm[threadIdx.x >> 5] = m;
    __syncthreads();
    unsigned long long mm = 0ull;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) mm = shm[q] > mm ? shm[q] : mm;
    __syncthreads();
    return mm;
}

// Rows of 8-cell strips (n_z a multiple of 8, at least 16): the vector
// paths of the single-problem kernels apply (same arithmetic).
__device__ __forceinline__ bool v8_level(const Lay &L) { return (L.n2 & 7) == 0 && L.n2 >= 16; }

// ---- batched stage kernels (grid-stride over items) ----

__global__ void __launch_bounds__(512) kb_zero(const BItem *__restrict__ items, const int *__restrict__ count,
                        const BLev *__restrict__ lv) {
    const int n = *count;
    for (int it = blockIdx.x; it < n; it += gridDim.x) {
        const BItem m = items[it];
        const BLev &L = lv[m.lev];
        const int n2 = L.lay.n2;
        if (v8_level(L.lay)) {
            const int s8 = n2 >> 3, strips = m.nrows * s8;
            for (int q = threadIdx.x; q < strips; q += blockDim.x) {
                int i, j;
                row_ij(L.lay, m.row0 + q / s8, i, j);
                float4 *p = reinterpret_cast<float4 *>(L.e + L.lay.at(i, j, (q % s8) * 8));
                p[0] = make_float4(0.f, 0.f, 0.f, 0.f);
                p[1] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            continue;
        }
        const int cells = m.nrows * n2;
        for (int q = threadIdx.x; q < cells; q += blockDim.x) {
            int i, j;
            row_ij(L.lay, m.row0 + q / n2, i, j);
            L.e[L.lay.at(i, j, q % n2)] = 0.f;
        }
    }
}

// FP32 colour sweep of the error equation (k_rbgs32 / k_rbgs_v8 arithmetic).
__global__ void __launch_bounds__(512) kb_rbgs(const BItem *__restrict__ items, const int *__restrict__ count,
                        const BLev *__restrict__ lv, int colour) {
    const int n = *count;
    for (int it = blockIdx.x; it < n; it += gridDim.x) {
        const BItem m = items[it];
        const BLev &L = lv[m.lev];
        if (v8_level(L.lay)) {
            const int s8 = L.lay.n2 >> 3, strips = m.nrows * s8;
            for (int q = threadIdx.x; q < strips; q += blockDim.x) {
                int i, j;
                row_ij(L.lay, m.row0 + q / s8, i, j);
                const int k0 = (q % s8) * 8;
                if (L.d3)
                    rbgs_strip8<float, true, false>(L.e, L.r, nullptr, L.lay, L.t32, L.b, colour, L.w, L.omc, i, j, k0);
                else
                    rbgs_strip8<float, false, false>(L.e, L.r, nullptr, L.lay, L.t32, L.b, colour, L.w, L.omc, i, j,
                                                     k0);
            }
            continue;
        }
        const int half = (L.lay.n2 + 1) / 2, cells = m.nrows * half;
        for (int q = threadIdx.x; q < cells; q += blockDim.x) {
            int i, j;
            row_ij(L.lay, m.row0 + q / half, i, j);
            const int k = 2 * (q % half) + ((i + j + colour) & 1);
            if (k >= L.lay.n2) continue;
            const int64_t c = L.lay.at(i, j, k);
            const float uc = L.e[c];
            float s, d;
            if (L.d3) {
                s = offdiag<float, true>(L.e, L.lay, L.t32, L.b, i, j, k, c, uc) - L.r[c];
                d = diag<float, true>(L.t32, i, j, k);
            } else {
                s = offdiag<float, false>(L.e, L.lay, L.t32, L.b, i, j, k, c, uc) - L.r[c];
                d = diag<float, false>(L.t32, i, j, k);
            }
            L.e[c] = fmat(L.omc, uc, sweep_div(L.w * s, d));
        }
    }
}

// Residual of the fine level restricted into the coarse one (items are rows
// of the coarse level; k_resid_restrict arithmetic).  The coarse target is
// FP64 when it is the case's coarsest level.
__global__ void __launch_bounds__(512) kb_restrict(const BItem *__restrict__ items, const int *__restrict__ count,
                            const BLev *__restrict__ lv) {
    const int n = *count;
    for (int it = blockIdx.x; it < n; it += gridDim.x) {
        const BItem m = items[it];
        const BLev &F = lv[m.lev];
        const BLev &C = lv[m.clev];
        const int n2 = C.lay.n2;
        if (v8_level(F.lay) && !C.top) {
            const int s4 = n2 >> 2, strips = m.nrows * s4;
            for (int q = threadIdx.x; q < strips; q += blockDim.x) {
                int i, j;
                row_ij(C.lay, m.row0 + q / s4, i, j);
                const int kc0 = (q % s4) * 4;
                float out[4];
                if (F.d3)
                    restrict4<float, true>(F.e, F.r, F.lay, F.t32, F.b, C.w32, nullptr, i, j, kc0, out);
                else
                    restrict4<float, false>(F.e, F.r, F.lay, F.t32, F.b, C.w32, nullptr, i, j, kc0, out);
                *reinterpret_cast<float4 *>(C.r + C.lay.at(i, j, kc0)) = make_float4(out[0], out[1], out[2], out[3]);
            }
            continue;
        }
        const int cells = m.nrows * n2;
        for (int q = threadIdx.x; q < cells; q += blockDim.x) {
            int i, j;
            row_ij(C.lay, m.row0 + q / n2, i, j);
            const int k = q % n2;
            const int i2 = 2 * i, j2 = 2 * j, k2 = 2 * k;
            float out;
            if (F.d3) {
                float sy[2];
                for (int a = 0; a < 2; a++) {
                    float sz[2];
                    for (int bb = 0; bb < 2; bb++) {
                        const float r0 = resid<float, true>(F.e, F.r, F.lay, F.t32, F.b, i2 + a, j2 + bb, k2);
                        const float r1 = resid<float, true>(F.e, F.r, F.lay, F.t32, F.b, i2 + a, j2 + bb, k2 + 1);
                        sz[bb] = fmat(C.w32.w1[2][k], r1, C.w32.w0[2][k] * r0);
                    }
                    sy[a] = fmat(C.w32.w1[1][j], sz[1], C.w32.w0[1][j] * sz[0]);
                }
                out = fmat(C.w32.w1[0][i], sy[1], C.w32.w0[0][i] * sy[0]);
            } else {
                const float r00 = resid<float, false>(F.e, F.r, F.lay, F.t32, F.b, i2, 0, k2);
                const float r01 = resid<float, false>(F.e, F.r, F.lay, F.t32, F.b, i2, 0, k2 + 1);
                const float r10 = resid<float, false>(F.e, F.r, F.lay, F.t32, F.b, i2 + 1, 0, k2);
                const float r11 = resid<float, false>(F.e, F.r, F.lay, F.t32, F.b, i2 + 1, 0, k2 + 1);
                out = ((r00 + r01) + (r10 + r11)) * 0.25f;
            }
            const int64_t cc = C.lay.at(i, j, k);
            if (C.top)
                C.f[cc] = (double)out;
            else
                C.r[cc] = out;
        }
    }
}

// Coarsest level of each listed case, one block per case: FP64 red-black
// sweeps from zero to the absolute tolerance, the iteration cap
// (poisson_d3.cc:249-432) or stagnation (k_coarsest_fast's MIXED-form
// rule), or a fixed number of sweeps when the level is too large for the
// single-problem block solve.
__global__ void kb_coarsest(const BItem *__restrict__ items, const int *__restrict__ count,
                            const BLev *__restrict__ lv) {
    __shared__ unsigned long long shm[32];
    extern __shared__ double fds[];
    const int n = *count;
    for (int it = blockIdx.x; it < n; it += gridDim.x) {
        const BLev &L = lv[items[it].lev];
        const Lay &Y = L.lay;
        const int ncell = Y.n0 * Y.n1 * Y.n2;
        if (L.fd.ok) {
            fd_solve(L.u, L.f, Y, L.fd, fds, fds + FD_MAX_CELLS);
            __syncthreads();
            continue;
        }
        for (int q = threadIdx.x; q < ncell; q += blockDim.x) {
            const int k = q % Y.n2, rest = q / Y.n2, j = rest % Y.n1, i = rest / Y.n1;
            L.u[Y.at(i, j, k)] = 0.0;
        }
        __syncthreads();
        const int half = (Y.n2 + 1) / 2, ncol = Y.n0 * Y.n1 * half;
        int iter = 0;
        double stall_ref = __longlong_as_double(0x7ff0000000000000ll);  // +infinity
        for (;;) {
            for (int colour = 0; colour < 2; colour++) {
                for (int q = threadIdx.x; q < ncol; q += blockDim.x) {
                    const int kk = q % half, rest = q / half, j = rest % Y.n1, i = rest / Y.n1;
                    const int k = 2 * kk + ((i + j + colour) & 1);
                    if (k >= Y.n2) continue;
                    const int64_t c = Y.at(i, j, k);
                    const double uc = L.u[c];
                    const double sv = (L.d3 ? offdiag<double, true>(L.u, Y, L.t64, L.b, i, j, k, c, uc)
                                            : offdiag<double, false>(L.u, Y, L.t64, L.b, i, j, k, c, uc)) -
                                      L.f[c];
                    L.u[c] = fmat(sv, L.wd[c], L.omc64 * uc);
                }
                __syncthreads();
            }
            if (L.sweep_only > 0) {
                if (++iter >= L.sweep_only) break;
                continue;
            }
            unsigned long long mx = 0ull;
            for (int q = threadIdx.x; q < ncell; q += blockDim.x) {
                const int k = q % Y.n2, rest = q / Y.n2, j = rest % Y.n1, i = rest / Y.n1;
                const double r = L.d3 ? resid<double, true>(L.u, L.f, Y, L.t64, L.b, i, j, k, L.dd)
                                      : resid<double, false>(L.u, L.f, Y, L.t64, L.b, i, j, k, L.dd);
                const unsigned long long bits = abs_bits(r);
                mx = bits > mx ? bits : mx;
            }
            const unsigned long long mm = block_max_bits(mx, shm);
            const double rn = __longlong_as_double((long long)mm);
            if (rn < L.tol) break;
            if (iter % COARSE_STALL_CHECK == 0) {  // MIXED form: stop a stagnating solve
                if (rn > 0.999 * stall_ref) break;
                stall_ref = rn;
            }
            iter++;
            if (iter > L.max_count) break;
        }
        __syncthreads();
    }
}

// e_fine += e_coarse (injection); the coarse source is FP64 at the coarsest.
__global__ void __launch_bounds__(512) kb_prolong(const BItem *__restrict__ items, const int *__restrict__ count,
                           const BLev *__restrict__ lv) {
    const int n = *count;
    for (int it = blockIdx.x; it < n; it += gridDim.x) {
        const BItem m = items[it];
        const BLev &F = lv[m.lev];
        const BLev &C = lv[m.clev];
        const int n2 = F.lay.n2;
        if (v8_level(F.lay) && !C.top) {
            const int s8 = n2 >> 3, strips = m.nrows * s8;
            for (int q = threadIdx.x; q < strips; q += blockDim.x) {
                int i, j;
                row_ij(F.lay, m.row0 + q / s8, i, j);
                prolong8(F.e, C.e, F.lay, C.lay, F.d3, i, j, (q % s8) * 8);
            }
            continue;
        }
        const int cells = m.nrows * n2;
        for (int q = threadIdx.x; q < cells; q += blockDim.x) {
            int i, j;
            row_ij(F.lay, m.row0 + q / n2, i, j);
            const int k = q % n2;
            const int64_t cc = C.lay.at(i >> 1, F.d3 ? (j >> 1) : 0, k >> 1);
            const int64_t cf = F.lay.at(i, j, k);
            F.e[cf] = F.e[cf] + (C.top ? (float)C.u[cc] : C.e[cc]);
        }
    }
}

// u += e over the finest level (FP64 accumulate).
__global__ void __launch_bounds__(512) kb_update(const BItem *__restrict__ items, const int *__restrict__ count,
                          const BLev *__restrict__ lv) {
    const int n = *count;
    for (int it = blockIdx.x; it < n; it += gridDim.x) {
        const BItem m = items[it];
        const BLev &L = lv[m.lev];
        const int n2 = L.lay.n2;
        if (v8_level(L.lay)) {
            const int s8 = n2 >> 3, strips = m.nrows * s8;
            for (int q = threadIdx.x; q < strips; q += blockDim.x) {
                int i, j;
                row_ij(L.lay, m.row0 + q / s8, i, j);
                const int64_t c = L.lay.at(i, j, (q % s8) * 8);
                double u[8];
                float e[8];
                ld8u(L.u + c, u);
                ld8(L.e + c, e);
#pragma unroll
                for (int t = 0; t < 8; t++) u[t] = u[t] + (double)e[t];
                st8(L.u + c, u);
            }
            continue;
        }
        const int cells = m.nrows * n2;
        for (int q = threadIdx.x; q < cells; q += blockDim.x) {
            int i, j;
            row_ij(L.lay, m.row0 + q / n2, i, j);
            const int64_t c = L.lay.at(i, j, q % n2);
            L.u[c] = L.u[c] + (double)L.e[c];
        }
    }
}

// FP64 residual of the finest level, its FP32 copy for the next outer
// iteration and one L-infinity partial per item.
__global__ void __launch_bounds__(512) kb_resid(const BItem *__restrict__ items, const int *__restrict__ count,
                         const BLev *__restrict__ lv, double *__restrict__ part) {
    __shared__ unsigned long long shm[32];
    const int n = *count;
    for (int it = blockIdx.x; it < n; it += gridDim.x) {
        const BItem m = items[it];
        const BLev &L = lv[m.lev];
        const int n2 = L.lay.n2, cells = m.nrows * n2;
        unsigned long long mx = 0ull;
        if (v8_level(L.lay)) {
            const int s8 = n2 >> 3, strips = m.nrows * s8;
            for (int q = threadIdx.x; q < strips; q += blockDim.x) {
                int i, j;
                row_ij(L.lay, m.row0 + q / s8, i, j);
                const int k0 = (q % s8) * 8;
                double r[8];
                if (L.d3)
                    resid_row8<double, true>(L.u, L.f, L.lay, L.t64, L.b, i, j, k0, L.dd, r);
                else
                    resid_row8<double, false>(L.u, L.f, L.lay, L.t64, L.b, i, j, k0, L.dd, r);
                float4 *p = reinterpret_cast<float4 *>(L.r + L.lay.at(i, j, k0));
                p[0] = make_float4((float)r[0], (float)r[1], (float)r[2], (float)r[3]);
                p[1] = make_float4((float)r[4], (float)r[5], (float)r[6], (float)r[7]);
#pragma unroll
                for (int t = 0; t < 8; t++) {
                    const unsigned long long bits = abs_bits(r[t]);
                    mx = bits > mx ? bits : mx;
                }
            }
        } else
        for (int q = threadIdx.x; q < cells; q += blockDim.x) {
            int i, j;
            row_ij(L.lay, m.row0 + q / n2, i, j);
            const int k = q % n2;
            const double r = L.d3 ? resid<double, true>(L.u, L.f, L.lay, L.t64, L.b, i, j, k, L.dd)
                                  : resid<double, false>(L.u, L.f, L.lay, L.t64, L.b, i, j, k, L.dd);
            L.r[L.lay.at(i, j, k)] = (float)r;
            const unsigned long long bits = abs_bits(r);
            mx = bits > mx ? bits : mx;
        }
        const unsigned long long mm = block_max_bits(mx, shm);
        if (threadIdx.x == 0) part[it] = __longlong_as_double((long long)mm);
    }
}

// Per case: maximum over its own items divided by max|f| (k_norm_final with
// the RHS norm taken once per solve).
__global__ void kb_norm(const BItem *__restrict__ items, const int *__restrict__ count,
                        const double *__restrict__ part, const double *__restrict__ fden,
                        double *__restrict__ res) {
    const int n = *count;
    for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < n; it += gridDim.x * blockDim.x) {
        const BItem m = items[it];
        double mx = 0.0;
        for (int q = 0; q < m.nrows; q++) {
            const double v = part[m.row0 + q];
            if (v > mx || v != v) mx = v;
        }
        const double den = fden[m.lev];
        res[m.lev] = den != 0.0 ? __ddiv_rn(mx, den) : mx;
    }
}

using Clock = std::chrono::steady_clock;

}  // namespace

// ------------------------------------------------------------- engine ----

struct ServeCase {
    int64_t id = 0;
    saras_mg *mg = nullptr;
    // time-step request: the integrator, its sub-stage, the caller's fields
    // (vx, vy, vz, p, t, pp at the core origin) and the V-cycles so far
    saras_rk3 *rk = nullptr;
    saras_rk3_params rprm{};
    int stage = 0;
    int total_cycles = 0;
    double tol = 0.0;  // relative residual that ends a solve (engine's, or the step request's)
    int cap = 0;       // outer iterations per solve
    int32_t step_status = SARAS_OK;
    double *fields[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    std::string shape;
    int slot = -1;
    int depth = 0;
    int cycles = 0;
    double res = 0.0;
    const double *in = nullptr;  // caller's host boxes, at the core origin
    double *out = nullptr;
    bool internal = false;       // synthetic request of the autotuner
    saras_grid_desc grid{};
    Clock::time_point t_submit;
    std::array<int, NREG> items{};
};

struct ServeDone {
    int64_t id;
    double res;
    int32_t cycles;
    int32_t status;
    double latency;
};

// Host copies of request boxes between the caller's pageable memory and the
// pinned staging ring, split across a few persistent worker threads: one
// host thread copies about 10 GB/s, a fraction of what the copy engines move,
// and a stream of requests arriving together spends its admissions and
// retirements in these copies.  copy() is called by the engine's thread
// alone and returns when every chunk is done.
class CopyPool {
  public:
    explicit CopyPool(int workers) {
        for (int w = 0; w < workers; w++) th_.emplace_back([this] { run(); });
    }
    ~CopyPool() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &t : th_) t.join();
    }
    void copy(void *dst, const void *src, size_t bytes) {
        constexpr size_t MIN_SPLIT = (size_t)2 << 20;
        if (th_.empty() || bytes < MIN_SPLIT) {
            std::memcpy(dst, src, bytes);
            return;
        }
        const size_t parts = th_.size() + 1;
        size_t chunk = (bytes + parts - 1) / parts;
        chunk = (chunk + 4095) / 4096 * 4096;
        {
            std::lock_guard<std::mutex> lk(mu_);
            dst_ = static_cast<char *>(dst);
            src_ = static_cast<const char *>(src);
            bytes_ = bytes;
            chunk_ = chunk;
            nchunks_ = (int)((bytes + chunk - 1) / chunk);
            next_.store(0);
            left_.store(nchunks_);
            gen_++;
        }
        cv_.notify_all();
        work();
        std::unique_lock<std::mutex> lk(mu_);
        done_cv_.wait(lk, [this] { return left_.load() == 0; });
    }

  private:
    // takes chunks of the current job until none is left
    void work() {
        for (;;) {
            const int c = next_.fetch_add(1);
            if (c >= nchunks_) return;
            const size_t lo = (size_t)c * chunk_, n = std::min(chunk_, bytes_ - lo);
            std::memcpy(dst_ + lo, src_ + lo, n);
            if (left_.fetch_sub(1) == 1) {
                std::lock_guard<std::mutex> lk(mu_);
                done_cv_.notify_all();
            }
        }
    }
    void run() {
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
            }
            work();
        }
    }
    std::vector<std::thread> th_;
    std::mutex mu_;
    std::condition_variable cv_, done_cv_;
    char *dst_ = nullptr;
    const char *src_ = nullptr;
    size_t bytes_ = 0, chunk_ = 0;
    int nchunks_ = 0;
    std::atomic<int> next_{0}, left_{0};
    uint64_t gen_ = 0;
    bool stop_ = false;
};

// Time-step work off the engine's thread.  Between its pressure solves a
// time-step request runs its right-hand sides, its Crank-Nicolson sweeps
// (each sweep's residual read on the host and compared with the tolerance,
// as the reference's solveVx loop does) and its correction.  On the
// engine's thread that work held up every batched iteration; here one
// worker thread runs it on the time-step stream while the engine goes on
// launching batches, and hands each case back with an event that the next
// batch waits on before the case's pressure solve joins it.
enum { STEP_ADMIT = 0, STEP_ADVANCE = 1 };

struct StepJob {
    ServeCase c;
    int kind = STEP_ADMIT;
    int32_t solve_status = SARAS_OK;  // STEP_ADVANCE: how the sub-stage's pressure solve ended
    bool retarget = false;            // STEP_ADMIT: a pooled integrator, to re-point at the request's grid
};

struct StepOut {
    ServeCase c;
    int32_t status = SARAS_OK;  // the request's outcome, when it leaves
    bool left = false;          // the request leaves the engine (done or failed)
    bool destroy = false;       // its integrator could not be re-pointed: free it
    cudaEvent_t ev = nullptr;   // the case's work on the time-step stream (when it rejoins)
    double secs = 0.0;          // wall time of the job
    std::string err;            // the worker's error message on failure
};

class StepWorker {
  public:
    using Fn = std::function<StepOut(StepJob &)>;
    StepWorker(int dev, Fn fn) : fn_(std::move(fn)) {
        th_ = std::thread([this, dev] { run(dev); });
    }
    ~StepWorker() { stop(); }
    void submit(StepJob j) {
        {
            std::lock_guard<std::mutex> lk(mu_);
            jobs_.push_back(std::move(j));
            held_++;
        }
        cv_.notify_all();
    }
    // Finished jobs; when none is ready and work is held, waits up to wait_s
    // seconds for one.
    std::vector<StepOut> take(double wait_s) {
        std::unique_lock<std::mutex> lk(mu_);
        if (outs_.empty() && held_ > 0 && wait_s > 0.0)
            done_cv_.wait_for(lk, std::chrono::duration<double>(wait_s), [this] { return !outs_.empty(); });
        std::vector<StepOut> r(std::make_move_iterator(outs_.begin()), std::make_move_iterator(outs_.end()));
        outs_.clear();
        held_ -= (int)r.size();
        return r;
    }
    // Requests the worker holds: queued, running, or finished and not taken.
    int held() {
        std::lock_guard<std::mutex> lk(mu_);
        return held_;
    }
    // Ends the thread after the job it is running; returns the cases of the
    // jobs it did not run and of the results nobody took.
    std::vector<ServeCase> stop() {
        std::vector<ServeCase> left;
        if (!th_.joinable()) return left;
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        th_.join();
        for (StepJob &j : jobs_) left.push_back(j.c);
        for (StepOut &o : outs_) {
            if (o.ev) cudaEventDestroy(o.ev);
            left.push_back(o.c);
        }
        jobs_.clear();
        outs_.clear();
        held_ = 0;
        return left;
    }

  private:
    void run(int dev) {
        cudaSetDevice(dev);
        for (;;) {
            StepJob j;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [this] { return stop_ || !jobs_.empty(); });
                if (stop_) return;
                j = std::move(jobs_.front());
                jobs_.pop_front();
            }
            StepOut o = fn_(j);
            {
                std::lock_guard<std::mutex> lk(mu_);
                outs_.push_back(std::move(o));
            }
            done_cv_.notify_all();
        }
    }
    Fn fn_;
    std::thread th_;
    std::mutex mu_;
    std::condition_variable cv_, done_cv_;
    std::deque<StepJob> jobs_;
    std::deque<StepOut> outs_;
    int held_ = 0;
    bool stop_ = false;
};

struct saras_serve {
    saras_serve_params prm{};
    std::unique_ptr<CopyPool> copies;  // host copies of request boxes (made with the pinned ring)
    cudaStream_t stream = nullptr;   // batched iterations, time-step work
    cudaStream_t adm = nullptr;      // Poisson admissions and retirements
    cudaStream_t stp = nullptr;      // time-step requests (integrators and their hierarchies)
    cudaEvent_t ev_adm = nullptr;    // admission work the next batch waits for
    cudaEvent_t ev_stp = nullptr;    // time-step work the next batch waits for (autotuning)
    std::unique_ptr<StepWorker> steps;  // time-step work, made with the first time-step request
    std::vector<cudaEvent_t> join_ev;   // cases back from the worker: the next batch waits for their work
    int dev = 0;
    std::vector<ServeCase> incoming; // admitted while a batch ran; join the next one
    std::deque<std::pair<ServeCase, int32_t>> finishing;  // finished by the last batch, retired during the next
    // pinned staging ring for admission uploads (copies from pageable memory
    // would wait for the admission stream, and so for the running batch)
    char *pin = nullptr;
    size_t pin_cap = 0, pin_head = 0;
    struct PinUse {
        size_t lo, hi;
        cudaEvent_t ev;
    };
    std::deque<PinUse> pin_busy;
    std::vector<cudaEvent_t> ev_pool;
    int sms = 152;
    std::deque<ServeCase> pending;
    std::vector<ServeCase> active;
    std::deque<ServeDone> done;
    std::map<std::string, std::vector<saras_mg *>> pool;
    std::map<std::string, std::vector<saras_rk3 *>> step_pool;  // idle integrators of time-step requests
    int64_t bytes_alloc = 0;
    std::vector<int> free_slots;
    std::array<int, NREG> used{};
    // device tables and their pinned staging
    BLev *d_lev = nullptr, *h_lev = nullptr;
    BItem *d_items = nullptr, *h_items = nullptr;
    int *d_counts = nullptr, *h_counts = nullptr;
    double *d_part = nullptr, *d_fden = nullptr, *d_res = nullptr, *h_res = nullptr;
    int lev_cap = 0;
    int reg_off[NREG] = {}, reg_cap[NREG] = {};  // fixed item regions (baked into the graphs)
    int64_t items_total = 0;
    double *d_box = nullptr;  // staging of one request's padded box
    int64_t box_cap = 0;
    cudaGraphExec_t graphs[DMAX + 1] = {};
    int64_t graph_launches[DMAX + 1] = {};
    bool dirty = true;
    // schedule
    int cells = 2048, threads = 256, bps = 2;
    // statistics
    int64_t cycles_run = 0, launches = 0, admitted = 0, retired = 0;
    int max_active = 0;
    double t_batch = 0.0, t_admit = 0.0, t_retire = 0.0, t_steps = 0.0;  // wall seconds by phase
};

namespace {

std::string shape_key(const saras_grid_desc &g, int levels) {
    char b[160];
    std::snprintf(b, sizeof(b), "%d:%d,%d,%d:%d%d%d:%d:%d", g.dims, g.n[0], g.n[1], g.n[2], g.periodic[0],
                  g.periodic[1], g.periodic[2], g.pad, levels);
    return b;
}

saras_mg_params case_params(const saras_serve *h) {
    saras_mg_params p;
    saras_mg_default_params(&p);
    p.vc_count = 1;
    p.vc_tolerance = h->prm.tolerance;
    p.solve_flag = 1;
    p.mg_tolerance = h->prm.mg_tolerance;
    p.sor_param = h->prm.sor_param;
    p.pre_smooth = h->prm.pre_smooth;
    p.post_smooth = h->prm.post_smooth;
    p.res_type = 0;
    p.precision = SARAS_PREC_MIXED;
    return p;
}

// A time-step request's integrator: its pressure solves run in the
// engine's MIXED form, so its multigrid takes the engine's parameters, with
// the outer-iteration cap of the engine.
saras_rk3_params step_params(const saras_serve *h, const saras_rk3_params &req) {
    saras_rk3_params r = req;
    r.mg = case_params(h);
    r.mg.vc_count = req.mg.vc_count;
    r.mg.vc_tolerance = req.mg.vc_tolerance;
    return r;
}

Bnd bnd_of(const saras_mg *m) {
    Bnd b;
    for (int d = 0; d < 3; d++) {
        b.per[d] = m->ghost.per[d];
        b.sg_lo[d] = m->ghost.kind[2 * d] == SARAS_BC_NEUMANN ? 1 : -1;
        b.sg_hi[d] = m->ghost.kind[2 * d + 1] == SARAS_BC_NEUMANN ? 1 : -1;
    }
    return b;
}

inline int rows_per_item(const saras_serve *h, const Lay &L) { return std::max(1, h->cells / std::max(1, L.n2)); }
inline int item_count(int rows, int per) { return (rows + per - 1) / per; }

// Items a case contributes to each region under the current schedule.
std::array<int, NREG> case_items(const saras_serve *h, const saras_mg *m) {
    std::array<int, NREG> c{};
    const int nl = m->nl;
    for (int l = 0; l + 1 < nl; l++) {
        const Lay &L = m->lv[(size_t)l].lay;
        const Lay &C = m->lv[(size_t)l + 1].lay;
        c[REG_SMOOTH + l] = item_count(L.n0 * L.n1, rows_per_item(h, L));
        c[REG_RESTRICT + l] = item_count(C.n0 * C.n1, rows_per_item(h, C));
    }
    c[REG_TOP + nl - 1] = 1;
    c[REG_NORM] = 1;
    return c;
}

bool fits(const saras_serve *h, const std::array<int, NREG> &c) {
    for (int r = 0; r < NREG; r++)
        if (h->used[r] + c[r] > h->reg_cap[r]) return false;
    return true;
}

// Region capacities: the finest level's items shrink about fourfold per
// coarser level (2-D) or eightfold (3-D); every case has one item per level
// at least, and one coarsest and one norm item.
void plan_regions(saras_serve *h) {
    const int per_case = 4 * h->prm.max_cases + 1024;
    int64_t off = 0;
    for (int r = 0; r < NREG; r++) {
        int cap;
        if (r >= REG_TOP)
            cap = h->prm.max_cases;
        else {
            const int l = r % DMAX;
            cap = std::max((1 << 18) >> (2 * l), per_case);
        }
        h->reg_off[r] = (int)off;
        h->reg_cap[r] = cap;
        off += cap;
    }
    h->items_total = off;
}

void recount(saras_serve *h) {
    h->used.fill(0);
    for (ServeCase &c : h->active) {
        c.items = case_items(h, c.mg);
        for (int r = 0; r < NREG; r++) h->used[r] += c.items[r];
    }
    h->dirty = true;
}

int active_depth(const saras_serve *h) {
    int d = 0;
    for (const ServeCase &c : h->active) d = std::max(d, c.depth);
    return d;
}

BLev level_desc(const saras_mg *m, int l) {
    const Level &v = m->lv[(size_t)l];
    BLev d{};
    d.lay = v.lay;
    d.d3 = m->d3 ? 1 : 0;
    d.e = v.e32;
    d.r = v.r32;
    d.u = v.lhs;
    d.f = v.rhs;
    d.dd = v.dd;
    d.wd = v.inv_diag;
    d.t32 = Tab3<float>{{v.cm32[0], v.cm32[1], v.cm32[2]}, {v.cp32[0], v.cp32[1], v.cp32[2]},
                        {v.dg32[0], v.dg32[1], v.dg32[2]}};
    d.w32 = WTab<float>{{v.w032[0], v.w032[1], v.w032[2]}, {v.w132[0], v.w132[1], v.w132[2]}};
    d.t64 = Tab3<double>{{v.cm[0], v.cm[1], v.cm[2]}, {v.cp[0], v.cp[1], v.cp[2]}, {v.dg[0], v.dg[1], v.dg[2]}};
    d.b = bnd_of(m);
    d.top = l == m->nl - 1 ? 1 : 0;
    d.fd = d.top ? v.fdv : FDiag{};
    d.max_count = m->maxCount();
    d.sweep_only = 0;
    if (d.top && (size_t)(4 * v.lay.size) * sizeof(double) > COARSE_SMEM_CAP)
        d.sweep_only = std::max(1, m->prm.pre_smooth);
    d.tol = m->prm.mg_tolerance;
    d.w = (float)m->prm.sor_param;
    d.omc = (float)(1.0 - m->prm.sor_param);
    d.omc64 = 1.0 - m->prm.sor_param;
    return d;
}

// Descriptors and item tables of the active cases into their fixed regions.
saras_status upload_tables(saras_serve *h) {
    int nlev = 0;
    int fill[NREG] = {};
    for (ServeCase &c : h->active) {
        saras_mg *m = c.mg;
        const int base = nlev;
        for (int l = 0; l < m->nl; l++) h->h_lev[nlev++] = level_desc(m, l);
        auto push = [&](int reg, BItem it) { h->h_items[(size_t)h->reg_off[reg] + fill[reg]++] = it; };
        const int first0 = fill[REG_SMOOTH];
        for (int l = 0; l + 1 < m->nl; l++) {
            const Lay &L = m->lv[(size_t)l].lay;
            const Lay &C = m->lv[(size_t)l + 1].lay;
            const int rows = L.n0 * L.n1, per = rows_per_item(h, L);
            for (int r0 = 0; r0 < rows; r0 += per)
                push(REG_SMOOTH + l, BItem{base + l, base + l + 1, r0, std::min(per, rows - r0)});
            const int crows = C.n0 * C.n1, cper = rows_per_item(h, C);
            for (int r0 = 0; r0 < crows; r0 += cper)
                push(REG_RESTRICT + l, BItem{base + l, base + l + 1, r0, std::min(cper, crows - r0)});
        }
        push(REG_TOP + m->nl - 1, BItem{base + m->nl - 1, -1, 0, 0});
        push(REG_NORM, BItem{c.slot, -1, first0, fill[REG_SMOOTH] - first0});
    }
    for (int r = 0; r < NREG; r++) h->h_counts[r] = fill[r];
    if (nlev > 0)
        SARAS_CUDA(cudaMemcpyAsync(h->d_lev, h->h_lev, (size_t)nlev * sizeof(BLev), cudaMemcpyHostToDevice,
                                   h->stream));
    for (int r = 0; r < NREG; r++)
        if (fill[r] > 0)
            SARAS_CUDA(cudaMemcpyAsync(h->d_items + h->reg_off[r], h->h_items + h->reg_off[r],
                                       (size_t)fill[r] * sizeof(BItem), cudaMemcpyHostToDevice, h->stream));
    SARAS_CUDA(cudaMemcpyAsync(h->d_counts, h->h_counts, NREG * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    h->dirty = false;
    return SARAS_OK;
}

// One outer iteration of every active case whose hierarchy has at most
// `depth` levels: the stage order of fast_cycle (mg_fast.cu) for the MIXED
// form, each stage one batched launch.
int64_t issue_batched(saras_serve *h, cudaStream_t s, int depth) {
    const int B = h->bps * h->sms, T = h->threads;
    const int pre = h->prm.pre_smooth, post = h->prm.post_smooth;
    int64_t n = 0;
    auto items = [&](int reg) { return h->d_items + h->reg_off[reg]; };
    auto cnt = [&](int reg) { return h->d_counts + reg; };
    auto sweeps = [&](int l, int count) {
        for (int q = 0; q < count; q++) {
            kb_rbgs<<<B, T, 0, s>>>(items(REG_SMOOTH + l), cnt(REG_SMOOTH + l), h->d_lev, 0);
            kb_rbgs<<<B, T, 0, s>>>(items(REG_SMOOTH + l), cnt(REG_SMOOTH + l), h->d_lev, 1);
            n += 2;
        }
    };
    kb_zero<<<B, T, 0, s>>>(items(REG_SMOOTH), cnt(REG_SMOOTH), h->d_lev);
    n++;
    sweeps(0, pre);
    for (int l = 0; l + 1 < depth; l++) {
        kb_restrict<<<B, T, 0, s>>>(items(REG_RESTRICT + l), cnt(REG_RESTRICT + l), h->d_lev);
        kb_coarsest<<<B, COARSE_THREADS, 2 * FD_MAX_CELLS * sizeof(double), s>>>(items(REG_TOP + l + 1),
                                                                                  cnt(REG_TOP + l + 1), h->d_lev);
        n += 2;
        if (l + 2 < depth) {
            kb_zero<<<B, T, 0, s>>>(items(REG_SMOOTH + l + 1), cnt(REG_SMOOTH + l + 1), h->d_lev);
            n++;
            sweeps(l + 1, pre);
        }
    }
    for (int l = depth - 2; l >= 0; l--) {
        kb_prolong<<<B, T, 0, s>>>(items(REG_SMOOTH + l), cnt(REG_SMOOTH + l), h->d_lev);
        n++;
        sweeps(l, post);
    }
    kb_update<<<B, T, 0, s>>>(items(REG_SMOOTH), cnt(REG_SMOOTH), h->d_lev);
    kb_resid<<<B, T, 0, s>>>(items(REG_SMOOTH), cnt(REG_SMOOTH), h->d_lev, h->d_part);
    kb_norm<<<cdiv(h->prm.max_cases, 128), 128, 0, s>>>(items(REG_NORM), cnt(REG_NORM), h->d_part, h->d_fden,
                                                         h->d_res);
    n += 3;
    cudaMemcpyAsync(h->h_res, h->d_res, (size_t)h->prm.max_cases * sizeof(double), cudaMemcpyDeviceToHost, s);
    return n;
}

void drop_graphs(saras_serve *h) {
    for (int d = 0; d <= DMAX; d++) {
        if (h->graphs[d]) cudaGraphExecDestroy(h->graphs[d]);
        h->graphs[d] = nullptr;
    }
}

saras_status graph_for(saras_serve *h, int depth, cudaGraphExec_t *out) {
    if (!h->graphs[depth]) {
        cudaStream_t cs;
        SARAS_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            h->graph_launches[depth] = issue_batched(h, cs, depth);
            e = cudaStreamEndCapture(cs, &g);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&h->graphs[depth], g, 0);
        if (g) cudaGraphDestroy(g);
        cudaStreamDestroy(cs);
        if (e != cudaSuccess) return cuda_fail(e, "serving graph capture", __FILE__, __LINE__);
    }
    *out = h->graphs[depth];
    return SARAS_OK;
}

// One batched outer iteration of the active cases; waits for its residuals.
// Launches one batched outer iteration of the active cases on the engine
// stream, after the admission work recorded so far.
saras_status launch_batched(saras_serve *h, int *depth_out) {
    SARAS_CUDA(cudaEventRecord(h->ev_adm, h->adm));
    SARAS_CUDA(cudaStreamWaitEvent(h->stream, h->ev_adm, 0));
    // time-step cases back from the worker: the work that set up their
    // pressure solves (the worker may meanwhile run other cases' work on the
    // time-step stream, which the batch does not wait for)
    for (cudaEvent_t e : h->join_ev) {
        const cudaError_t r = cudaStreamWaitEvent(h->stream, e, 0);
        cudaEventDestroy(e);
        if (r != cudaSuccess) {
            h->join_ev.clear();
            return cuda_fail(r, "cudaStreamWaitEvent", __FILE__, __LINE__);
        }
    }
    h->join_ev.clear();
    if (h->dirty) SARAS_TRY(upload_tables(h));
    cudaGraphExec_t g;
    const int depth = active_depth(h);
    SARAS_TRY(graph_for(h, depth, &g));
    SARAS_CUDA(cudaGraphLaunch(g, h->stream));
    *depth_out = depth;
    return SARAS_OK;
}

saras_status run_batched(saras_serve *h) {
    SARAS_CUDA(cudaEventRecord(h->ev_adm, h->adm));
    SARAS_CUDA(cudaStreamWaitEvent(h->stream, h->ev_adm, 0));
    SARAS_CUDA(cudaEventRecord(h->ev_stp, h->stp));
    SARAS_CUDA(cudaStreamWaitEvent(h->stream, h->ev_stp, 0));
    if (h->dirty) SARAS_TRY(upload_tables(h));
    cudaGraphExec_t g;
    const int depth = active_depth(h);
    SARAS_TRY(graph_for(h, depth, &g));
    SARAS_CUDA(cudaGraphLaunch(g, h->stream));
    SARAS_CUDA(cudaStreamSynchronize(h->stream));
    h->cycles_run++;
    h->launches += h->graph_launches[depth];
    return SARAS_OK;
}

saras_mg *take_handle(saras_serve *h, const std::string &key) {
    auto it = h->pool.find(key);
    if (it == h->pool.end() || it->second.empty()) return nullptr;
    saras_mg *m = it->second.back();
    it->second.pop_back();
    return m;
}

// Frees pooled (idle) hierarchies and integrators until `need` more bytes
// fit the budget.
void evict_pooled(saras_serve *h, int64_t need) {
    for (auto &kv : h->step_pool) {
        while (!kv.second.empty() && h->bytes_alloc + need > h->prm.hbm_budget_bytes) {
            saras_rk3 *rk = kv.second.back();
            kv.second.pop_back();
            h->bytes_alloc -= rk3_device_bytes(rk) + rk3_multigrid(rk)->dev_bytes;
            saras_rk3_destroy(rk);
        }
    }
    for (auto &kv : h->pool) {
        while (!kv.second.empty() && h->bytes_alloc + need > h->prm.hbm_budget_bytes) {
            saras_mg *m = kv.second.back();
            kv.second.pop_back();
            h->bytes_alloc -= m->dev_bytes;
            saras_mg_destroy(m);
        }
    }
}

struct Box {
    int64_t st[3];
    int64_t elems, origin;
};

Box box_of(const saras_grid_desc &g) {
    const int p0 = g.pad, py = g.dims == 3 ? p0 : 1;
    Box b;
    b.st[2] = 1;
    b.st[1] = g.n[2] + 2 * p0;
    b.st[0] = b.st[1] * ((g.dims == 3 ? g.n[1] : 1) + 2 * py);
    b.elems = b.st[0] * (g.n[0] + 2 * p0);
    b.origin = p0 * b.st[0] + py * b.st[1] + p0;
    return b;
}

saras_status stage_box(saras_serve *h, int64_t elems) {
    if (elems <= h->box_cap) return SARAS_OK;
    SARAS_CUDA(cudaStreamSynchronize(h->adm));
    cudaFree(h->d_box);
    h->d_box = nullptr;
    h->box_cap = 0;
    SARAS_CUDA(cudaMalloc((void **)&h->d_box, (size_t)elems * sizeof(double)));
    h->box_cap = elems;
    return SARAS_OK;
}

// Nothing resident: a request that does not fit now never will.
bool idle(saras_serve *h) {
    return h->active.empty() && h->incoming.empty() && h->finishing.empty() && (!h->steps || h->steps->held() == 0);
}

constexpr size_t PIN_BYTES = (size_t)256 << 20;

// Waits for (or retires) the oldest staged uploads until [lo, hi) of the
// ring is free.
void pin_wait(saras_serve *h, size_t lo, size_t hi) {
    auto overlaps = [&]() {
        for (const auto &u : h->pin_busy)
            if (u.lo < hi && lo < u.hi) return true;
        return false;
    };
    while (!h->pin_busy.empty() && overlaps()) {
        cudaEventSynchronize(h->pin_busy.front().ev);
        h->ev_pool.push_back(h->pin_busy.front().ev);
        h->pin_busy.pop_front();
    }
}

// The pinned staging ring and the copy threads, made on first use.
saras_status ensure_pin(saras_serve *h) {
    if (!h->pin && h->pin_cap == 0) {
        if (cudaMallocHost((void **)&h->pin, PIN_BYTES) == cudaSuccess) {
            h->pin_cap = PIN_BYTES;
        } else {
            cudaGetLastError();
            h->pin = nullptr;
            h->pin_cap = 1;  // do not retry
        }
    }
    if (!h->copies) {
        // every host core but the engine's thread and the step worker's
        // (the pool runs only while the engine's thread waits for a copy)
        const unsigned hw = std::thread::hardware_concurrency();
        h->copies.reset(new CopyPool((int)std::min(30u, hw > 3 ? hw - 3 : 1u)));
    }
    return SARAS_OK;
}

// Host box -> device staging box on the admission stream: through the
// pinned ring (a host copy by the copy threads, then an asynchronous DMA)
// when it fits, otherwise straight from the caller's pageable memory.
saras_status upload_box(saras_serve *h, double *dev, const double *host, size_t bytes) {
    SARAS_TRY(ensure_pin(h));
    const size_t need = (bytes + 255) / 256 * 256;
    if (!h->pin || need > h->pin_cap) {
        SARAS_CUDA(cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, h->adm));
        return SARAS_OK;
    }
    size_t lo = h->pin_head;
    if (lo + need > h->pin_cap) lo = 0;
    pin_wait(h, lo, lo + need);
    h->copies->copy(h->pin + lo, host, bytes);
    SARAS_CUDA(cudaMemcpyAsync(dev, h->pin + lo, bytes, cudaMemcpyHostToDevice, h->adm));
    cudaEvent_t ev = nullptr;
    if (!h->ev_pool.empty()) {
        ev = h->ev_pool.back();
        h->ev_pool.pop_back();
    } else {
        SARAS_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    }
    SARAS_CUDA(cudaEventRecord(ev, h->adm));
    h->pin_busy.push_back(saras_serve::PinUse{lo, lo + need, ev});
    h->pin_head = lo + need;
    return SARAS_OK;
}

double since(const ServeCase &c) { return std::chrono::duration<double>(Clock::now() - c.t_submit).count(); }

// Starts the pressure solve of the current sub-stage of a time-step case:
// its RHS is already in lv[0].rhs, the iterate lv[0].lhs holds the previous
// pressure correction (mgSolve's initial guess), as in saras_rk3_step.
saras_status start_solve(saras_serve *h, ServeCase &c) {
    saras_mg *m = c.mg;
    rhs_norm(m, m->stream);
    SARAS_CUDA(cudaMemcpyAsync(h->d_fden + c.slot, m->norm_out + 4, sizeof(double), cudaMemcpyDeviceToDevice,
                               m->stream));
    mixed_prepare(m, m->stream);
    SARAS_CUDA(cudaGetLastError());
    c.cycles = 0;
    return SARAS_OK;
}

// Returns a time-step case's integrator to its pool and records the
// outcome.
void drop_step(saras_serve *h, ServeCase &c, int32_t status) {
    if (c.rk) {
        h->step_pool[c.shape].push_back(c.rk);
        c.rk = nullptr;
        c.mg = nullptr;
    }
    h->done.push_back(ServeDone{c.id, c.res, c.total_cycles, status, since(c)});
    h->retired++;
}

enum AdmitStep { ADMIT_DONE = 0, ADMIT_WAIT = 1 };

// The worker's side of a time-step request, on the worker thread.  It
// touches the case's integrator and hierarchy, its slot's entry of d_fden
// and the time-step stream, nothing the engine's thread uses meanwhile.
//   STEP_ADMIT: re-point a pooled integrator at the request's grid, upload
//     the caller's fields, run the first sub-stage up to its pressure solve.
//   STEP_ADVANCE (the sub-stage's pressure solve has left the batch): finish
//     the solve, the sub-stage's correction, then either the next sub-stage
//     up to its pressure solve or the download of the fields.
// A case that goes on carries an event on the time-step stream after the
// work that set up its next pressure solve.
StepOut step_work(saras_serve *h, StepJob &j) {
    const auto t0 = Clock::now();
    StepOut o;
    o.c = j.c;
    ServeCase &c = o.c;
    saras_status s = SARAS_OK;
    bool rejoin = false;
    if (j.kind == STEP_ADMIT) {
        if (j.retarget) {
            const saras_rk3_params rp = step_params(h, c.rprm);
            s = rk3_retarget(c.rk, &c.grid, &rp);
            o.destroy = s != SARAS_OK;
        }
        const Box b = box_of(c.grid);
        if (s == SARAS_OK)
            s = saras_rk3_upload(c.rk, c.fields[0], c.fields[1], c.fields[2], c.fields[3], c.fields[4], c.fields[5],
                                 b.st);
        c.stage = 0;
        if (s == SARAS_OK) s = rk3_stage_begin(c.rk, 0);
        if (s == SARAS_OK) s = start_solve(h, c);
        rejoin = s == SARAS_OK;
    } else if (j.solve_status == SARAS_NAN) {
        s = SARAS_NAN;
    } else {
        // a pressure solve that stopped at its V-Cycle Count above the
        // tolerance is not a failure: mgSolve returns after vcCount cycles
        // (poisson.cc:182-188) and timeAdvance goes on; the request's
        // residual reports where the last solve stopped
        mixed_finish(c.mg, c.mg->stream);  // the integrator's stream: ordered before its correction
        s = rk3_stage_end(c.rk, c.stage);
        if (s == SARAS_OK && c.stage + 1 < rk3_stages(c.rk)) {
            c.stage++;
            s = rk3_stage_begin(c.rk, c.stage);
            if (s == SARAS_OK) s = start_solve(h, c);
            rejoin = s == SARAS_OK;
        } else if (s == SARAS_OK) {
            const Box b = box_of(c.grid);
            s = saras_rk3_download(c.rk, c.fields[0], c.fields[1], c.fields[2], c.fields[3], c.fields[4],
                                   c.fields[5], b.st);
        }
    }
    if (rejoin) {
        cudaError_t e = cudaEventCreateWithFlags(&o.ev, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(o.ev, c.mg->stream);
        if (e != cudaSuccess) {
            s = cuda_fail(e, "cudaEventRecord", __FILE__, __LINE__);
            if (o.ev) cudaEventDestroy(o.ev);
            o.ev = nullptr;
            rejoin = false;
        }
    }
    o.left = !rejoin;
    o.status = s;
    if (s != SARAS_OK) o.err = saras_last_error();
    o.secs = std::chrono::duration<double>(Clock::now() - t0).count();
    return o;
}

// Admission of a time-step request: its integrator (fields and hierarchy)
// inside the HBM budget, a slot and its work items.  The worker then
// uploads the caller's fields and runs the first sub-stage up to its
// pressure solve, which joins the batch when the worker hands the case back.
AdmitStep admit_step(saras_serve *h, ServeCase &c) {
    const saras_rk3_params rp = step_params(h, c.rprm);
    saras_rk3 *rk = nullptr;
    bool pooled = false;
    auto pit = h->step_pool.find(c.shape);
    if (pit != h->step_pool.end() && !pit->second.empty()) {
        rk = pit->second.back();
        pit->second.pop_back();
        pooled = true;
    } else {
        const int64_t est = rk3_estimate_bytes(&c.grid, &rp);
        if (h->bytes_alloc + est > h->prm.hbm_budget_bytes) evict_pooled(h, est);
        if (h->bytes_alloc + est > h->prm.hbm_budget_bytes) {
            if (!idle(h)) return ADMIT_WAIT;
            set_error("request %lld needs about %lld bytes, above the HBM budget", (long long)c.id,
                      (long long)est);
            h->done.push_back(ServeDone{c.id, 0.0, 0, SARAS_BUDGET, since(c)});
            return ADMIT_DONE;
        }
        const saras_status s = saras_rk3_create(&c.grid, &rp, h->stp, &rk);
        if (s != SARAS_OK) {
            h->done.push_back(ServeDone{c.id, 0.0, 0, (int32_t)s, since(c)});
            return ADMIT_DONE;
        }
        rk3_multigrid(rk)->no_rowsplit = true;
        rk3_multigrid(rk)->lv[0].rs = 0;
        h->bytes_alloc += rk3_device_bytes(rk) + rk3_multigrid(rk)->dev_bytes;
    }
    c.rk = rk;
    c.mg = rk3_multigrid(rk);
    // a pooled integrator has the request's shape, so its items are the
    // request's before it is re-pointed
    const std::array<int, NREG> items = case_items(h, c.mg);
    if (!fits(h, items)) {
        h->step_pool[c.shape].push_back(rk);
        c.rk = nullptr;
        c.mg = nullptr;
        if (!idle(h)) return ADMIT_WAIT;
        set_error("request %lld has more work items than the tables hold", (long long)c.id);
        h->done.push_back(ServeDone{c.id, 0.0, 0, SARAS_BUDGET, since(c)});
        return ADMIT_DONE;
    }
    if (!h->steps) h->steps.reset(new StepWorker(h->dev, [h](StepJob &j) { return step_work(h, j); }));
    c.items = items;
    c.slot = h->free_slots.back();
    h->free_slots.pop_back();
    for (int r = 0; r < NREG; r++) h->used[r] += items[r];
    StepJob j;
    j.c = c;
    j.kind = STEP_ADMIT;
    j.retarget = pooled;
    h->steps->submit(std::move(j));
    h->admitted++;
    return ADMIT_DONE;
}

// Cases the worker has finished with: back into the batch (the next batch
// waits for their work on the time-step stream) or out of the engine.
// Called between batches only, when the active list is not in use.
void collect_steps(saras_serve *h, double wait_s) {
    if (!h->steps) return;
    for (StepOut &o : h->steps->take(wait_s)) {
        h->t_steps += o.secs;
        ServeCase &c = o.c;
        if (!o.left) {
            h->join_ev.push_back(o.ev);
            h->active.push_back(c);
            h->dirty = true;
            continue;
        }
        if (o.status != SARAS_OK && !o.err.empty()) set_error("%s", o.err.c_str());
        h->free_slots.push_back(c.slot);
        for (int r = 0; r < NREG; r++) h->used[r] -= c.items[r];
        if (o.destroy) {
            h->bytes_alloc -= rk3_device_bytes(c.rk) + rk3_multigrid(c.rk)->dev_bytes;
            saras_rk3_destroy(c.rk);
            c.rk = nullptr;
            c.mg = nullptr;
        }
        drop_step(h, c, o.status);
    }
}

// Admits pending requests in order while slots, the item tables and the HBM
// budget allow.
saras_status admit(saras_serve *h, std::vector<ServeCase> &dst) {
    const saras_mg_params p = case_params(h);
    while (!h->pending.empty() && !h->free_slots.empty()) {
        ServeCase &c = h->pending.front();
        if (c.rk == nullptr && c.fields[0]) {
            const AdmitStep a = admit_step(h, c);
            if (a == ADMIT_WAIT) break;
            h->pending.pop_front();
            continue;
        }
        saras_mg *m = take_handle(h, c.shape);
        bool fresh = false;
        if (!m) {
            const int64_t est = mg_estimate_bytes(&c.grid, &p);
            if (h->bytes_alloc + est > h->prm.hbm_budget_bytes) evict_pooled(h, est);
            if (h->bytes_alloc + est > h->prm.hbm_budget_bytes) {
                if (idle(h)) {  // can never fit: fail the request rather than wait forever
                    set_error("request %lld needs about %lld bytes, above the HBM budget", (long long)c.id,
                              (long long)est);
                    h->done.push_back(ServeDone{c.id, 0.0, 0, SARAS_BUDGET, 0.0});
                    h->pending.pop_front();
                    continue;
                }
                break;  // wait for retirements to free memory
            }
            saras_status s = mg_create_queued(&c.grid, &p, h->adm, &m);
            if (s == SARAS_OK) {
                m->no_rowsplit = true;
                m->lv[0].rs = 0;
            }
            if (s != SARAS_OK) {
                h->done.push_back(ServeDone{c.id, 0.0, 0, (int32_t)s,
                                            std::chrono::duration<double>(Clock::now() - c.t_submit).count()});
                h->pending.pop_front();
                continue;
            }
            fresh = true;
            h->bytes_alloc += m->dev_bytes;
        }
        const std::array<int, NREG> items = case_items(h, m);
        if (!fits(h, items)) {
            h->pool[c.shape].push_back(m);
            if (idle(h)) {
                set_error("request %lld has more work items than the tables hold", (long long)c.id);
                h->done.push_back(ServeDone{c.id, 0.0, 0, SARAS_BUDGET, 0.0});
                h->pending.pop_front();
                continue;
            }
            break;
        }
        if (!fresh) SARAS_TRY(mg_retarget(m, &c.grid));
        c.mg = m;
        c.items = items;
        c.slot = h->free_slots.back();
        h->free_slots.pop_back();
        const Box b = box_of(c.grid);
        SARAS_TRY(stage_box(h, b.elems));
        SARAS_TRY(upload_box(h, h->d_box, c.in - b.origin, (size_t)b.elems * sizeof(double)));
        SARAS_TRY(mg_load_rhs(m, h->d_box + b.origin, b.st));
        rhs_norm(m, m->stream);
        SARAS_CUDA(cudaMemcpyAsync(h->d_fden + c.slot, m->norm_out + 4, sizeof(double), cudaMemcpyDeviceToDevice,
                                   m->stream));
        mixed_prepare(m, m->stream);
        SARAS_CUDA(cudaGetLastError());
        for (int r = 0; r < NREG; r++) h->used[r] += items[r];
        dst.push_back(c);
        h->pending.pop_front();
        h->admitted++;
        h->dirty = true;
    }
    h->max_active = std::max(h->max_active, (int)(h->active.size() + h->incoming.size() + h->finishing.size()) +
                                                (h->steps ? h->steps->held() : 0));
    return SARAS_OK;
}

// Retires a case that has left the batch: null-space projection, ghost
// layer, copy out, hierarchy back to its pool, slot and items free.
saras_status retire_case(saras_serve *h, const ServeCase &c, int32_t status) {
    saras_mg *m = c.mg;
    if (!c.internal) {
        mixed_finish(m, m->stream);
        const Box b = box_of(c.grid);
        SARAS_TRY(stage_box(h, b.elems));
        // a pad wider than one keeps the caller's outer layers
        if (c.grid.pad > 1)
            SARAS_CUDA(cudaMemcpyAsync(h->d_box, c.out - b.origin, (size_t)b.elems * sizeof(double),
                                       cudaMemcpyHostToDevice, m->stream));
        mg_store_lhs(m, h->d_box + b.origin, b.st);
        const size_t bytes = (size_t)b.elems * sizeof(double), need = (bytes + 255) / 256 * 256;
        SARAS_TRY(ensure_pin(h));
        if (h->pin && need <= h->pin_cap) {
            // through the pinned ring: a DMA at full speed, then the copy
            // threads into the caller's box; the ring part is free again
            // when this returns
            size_t lo = h->pin_head;
            if (lo + need > h->pin_cap) lo = 0;
            pin_wait(h, lo, lo + need);
            SARAS_CUDA(cudaMemcpyAsync(h->pin + lo, h->d_box, bytes, cudaMemcpyDeviceToHost, m->stream));
            SARAS_CUDA(cudaStreamSynchronize(m->stream));
            h->copies->copy(c.out - b.origin, h->pin + lo, bytes);
            h->pin_head = lo + need;
        } else {
            SARAS_CUDA(cudaMemcpyAsync(c.out - b.origin, h->d_box, bytes, cudaMemcpyDeviceToHost, m->stream));
            SARAS_CUDA(cudaStreamSynchronize(m->stream));
        }
        h->done.push_back(ServeDone{c.id, c.res, c.cycles, status,
                                    std::chrono::duration<double>(Clock::now() - c.t_submit).count()});
        h->retired++;
    }
    h->pool[c.shape].push_back(m);
    h->free_slots.push_back(c.slot);
    for (int r = 0; r < NREG; r++) h->used[r] -= c.items[r];
    return SARAS_OK;
}

// Retires active case idx at once.
saras_status retire(saras_serve *h, size_t idx, int32_t status) {
    const ServeCase c = h->active[idx];
    h->active.erase(h->active.begin() + (long)idx);
    h->dirty = true;
    return retire_case(h, c, status);
}

// Retires the cases the last batch finished.  Their copies out run on the
// admission stream and the host while the next batch runs.
saras_status flush_finishing(saras_serve *h) {
    const auto t0 = Clock::now();
    saras_status st = SARAS_OK;
    while (!h->finishing.empty()) {
        st = retire_case(h, h->finishing.front().first, h->finishing.front().second);
        // a retirement that failed has not released the case (its hierarchy,
        // slot and items are released last): it stays for destroy to free
        if (st != SARAS_OK) break;
        h->finishing.pop_front();
    }
    h->t_retire += std::chrono::duration<double>(Clock::now() - t0).count();
    return st;
}

saras_status enqueue(saras_serve *h, int64_t id, const saras_grid_desc *grid, const double *rhs, double *lhs,
                     bool internal) {
    HostGrid g;
    SARAS_TRY(g.build(*grid, 0));
    if (g.levels < 2 || g.levels > DMAX) {
        set_error("request depth %d outside 2..%d", g.levels, DMAX);
        return SARAS_BAD_ARG;
    }
    ServeCase c;
    c.id = id;
    c.grid = *grid;
    c.depth = g.levels;
    c.shape = shape_key(*grid, g.levels);
    const Box b = box_of(*grid);
    c.in = rhs + b.origin;
    c.out = lhs + b.origin;
    c.internal = internal;
    c.tol = h->prm.tolerance;
    c.cap = h->prm.max_cycles;
    c.t_submit = Clock::now();
    h->pending.push_back(c);
    return SARAS_OK;
}

void apply_schedule(saras_serve *h, int cells, int threads, int bps) {
    if (cells == h->cells && threads == h->threads && bps == h->bps) return;
    const bool relaunch = threads != h->threads || bps != h->bps;
    h->cells = cells;
    h->threads = threads;
    h->bps = bps;
    if (relaunch) drop_graphs(h);
    recount(h);
}

}  // namespace

extern "C" {

void saras_serve_default_params(saras_serve_params *p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->hbm_budget_bytes = (int64_t)40 << 30;
    p->max_cases = 256;
    p->max_cycles = 2000;
    p->tolerance = 1e-8;
    p->mg_tolerance = 1e-6;
    p->sor_param = 1.0;
    p->pre_smooth = 2;
    p->post_smooth = 2;
}

saras_status saras_serve_create(const saras_serve_params *prm, saras_serve **out) {
    if (!prm || !out || prm->max_cases < 1 || prm->max_cases > 4096 || !(prm->tolerance > 0.0) ||
        prm->max_cycles < 1 || prm->pre_smooth < 0 || prm->post_smooth < 0 || prm->hbm_budget_bytes <= 0 ||
        prm->cells_per_item < 0 || prm->threads < 0 || prm->threads > 1024 || prm->threads % 32 != 0 ||
        prm->blocks_per_sm < 0) {
        set_error("invalid serving parameters");
        return SARAS_BAD_ARG;
    }
    *out = nullptr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        set_error("no CUDA device");
        return SARAS_NO_DEVICE;
    }
    saras_serve *h = new saras_serve();
    h->prm = *prm;
    if (prm->cells_per_item) h->cells = prm->cells_per_item;
    if (prm->threads) h->threads = prm->threads;
    if (prm->blocks_per_sm) h->bps = prm->blocks_per_sm;
    cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, dev);
    h->dev = dev;
    h->lev_cap = prm->max_cases * DMAX;
    plan_regions(h);
    bool ok = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaStreamCreateWithFlags(&h->adm, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&h->ev_adm, cudaEventDisableTiming) == cudaSuccess;
    ok = ok && cudaStreamCreateWithFlags(&h->stp, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&h->ev_stp, cudaEventDisableTiming) == cudaSuccess;
    ok = ok && cudaMalloc((void **)&h->d_lev, (size_t)h->lev_cap * sizeof(BLev)) == cudaSuccess;
    ok = ok && cudaMalloc((void **)&h->d_items, (size_t)h->items_total * sizeof(BItem)) == cudaSuccess;
    ok = ok && cudaMalloc((void **)&h->d_counts, NREG * sizeof(int)) == cudaSuccess;
    ok = ok && cudaMalloc((void **)&h->d_part, (size_t)h->reg_cap[REG_SMOOTH] * sizeof(double)) == cudaSuccess;
    ok = ok && cudaMalloc((void **)&h->d_fden, (size_t)prm->max_cases * sizeof(double)) == cudaSuccess;
    ok = ok && cudaMalloc((void **)&h->d_res, (size_t)prm->max_cases * sizeof(double)) == cudaSuccess;
    ok = ok && cudaMallocHost((void **)&h->h_res, (size_t)prm->max_cases * sizeof(double)) == cudaSuccess;
    ok = ok && cudaMallocHost((void **)&h->h_lev, (size_t)h->lev_cap * sizeof(BLev)) == cudaSuccess;
    ok = ok && cudaMallocHost((void **)&h->h_items, (size_t)h->items_total * sizeof(BItem)) == cudaSuccess;
    ok = ok && cudaMallocHost((void **)&h->h_counts, NREG * sizeof(int)) == cudaSuccess;
    ok = ok && cudaMemsetAsync(h->d_counts, 0, NREG * sizeof(int), h->stream) == cudaSuccess;
    ok = ok && cudaMemsetAsync(h->d_res, 0, (size_t)prm->max_cases * sizeof(double), h->stream) == cudaSuccess;
    ok = ok && cudaMemsetAsync(h->d_fden, 0, (size_t)prm->max_cases * sizeof(double), h->stream) == cudaSuccess;
    ok = ok && cudaStreamSynchronize(h->stream) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        set_error("serving engine tables could not be allocated");
        saras_serve_destroy(h);
        return SARAS_OOM;
    }
    if (cudaFuncSetAttribute(kb_coarsest, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             2 * FD_MAX_CELLS * (int)sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        set_error("serving coarsest-solve kernel configuration failed");
        saras_serve_destroy(h);
        return SARAS_CUDA_ERR;
    }
    for (int s = prm->max_cases - 1; s >= 0; s--) h->free_slots.push_back(s);
    *out = h;
    return SARAS_OK;
}

saras_status saras_serve_submit(saras_serve *h, int64_t id, const saras_grid_desc *grid, const double *rhs,
                                double *lhs) {
    if (!h || !grid || !rhs || !lhs) {
        set_error("null argument");
        return SARAS_BAD_ARG;
    }
    return enqueue(h, id, grid, rhs, lhs, false);
}

saras_status saras_serve_submit_step(saras_serve *h, int64_t id, const saras_grid_desc *grid,
                                     const saras_rk3_params *prm, double *vx, double *vy, double *vz, double *p,
                                     double *t, double *pp) {
    if (!h || !grid || !prm || !vx || !vz || !p || !pp || (grid->dims == 3 && !vy) || (prm->with_scalar && !t)) {
        set_error("null argument");
        return SARAS_BAD_ARG;
    }
    if (prm->mg.vc_count < 1 || !(prm->mg.vc_tolerance > 0.0)) {
        set_error("a time-step request needs vc_count >= 1 and vc_tolerance > 0 for its pressure solves");
        return SARAS_BAD_ARG;
    }
    HostGrid g;
    SARAS_TRY(g.build(*grid, 0));
    if (g.levels < 2 || g.levels > DMAX) {
        set_error("request depth %d outside 2..%d", g.levels, DMAX);
        return SARAS_BAD_ARG;
    }
    ServeCase c;
    c.id = id;
    c.grid = *grid;
    c.depth = g.levels;
    c.shape = shape_key(*grid, g.levels);
    c.rprm = *prm;
    c.tol = prm->mg.vc_tolerance;
    c.cap = prm->mg.vc_count;
    double *f[6] = {vx, vy, vz, p, t, pp};
    const Box b = box_of(*grid);
    for (int q = 0; q < 6; q++) c.fields[q] = f[q] ? f[q] + b.origin : nullptr;
    c.t_submit = Clock::now();
    h->pending.push_back(c);
    return SARAS_OK;
}

saras_status saras_serve_step(saras_serve *h, int32_t *active, int32_t *pending) {
    if (!h) return SARAS_BAD_ARG;
    auto secs = [](Clock::time_point a, Clock::time_point b) { return std::chrono::duration<double>(b - a).count(); };
    collect_steps(h, 0.0);
    auto t0 = Clock::now();
    if (h->active.empty()) {
        // nothing to overlap with: retire what the last batch finished and
        // admit straight into the batch
        SARAS_TRY(flush_finishing(h));
        t0 = Clock::now();
        SARAS_TRY(admit(h, h->active));
        h->dirty = h->dirty || !h->active.empty();
    }
    auto t1 = Clock::now();
    h->t_admit += secs(t0, t1);
    if (!h->active.empty()) {
        // the batch runs on the engine stream while the requests that arrived
        // meanwhile are admitted on the admission stream; they join the next
        // batch, so the iterations of every request keep their arithmetic
        int depth = 0;
        SARAS_TRY(launch_batched(h, &depth));
        // meanwhile the cases the previous batch finished leave
        SARAS_TRY(flush_finishing(h));
        t0 = Clock::now();
        SARAS_TRY(admit(h, h->incoming));
        t1 = Clock::now();
        h->t_admit += secs(t0, t1);
        SARAS_CUDA(cudaStreamSynchronize(h->stream));
        t0 = Clock::now();
        h->t_batch += secs(t1, t0);
        h->cycles_run++;
        h->launches += h->graph_launches[depth];
        for (size_t q = 0; q < h->active.size();) {
            ServeCase &c = h->active[q];
            c.cycles++;
            c.res = h->h_res[c.slot];
            const bool bad = !std::isfinite(c.res);
            if (bad || c.res < c.tol || c.cycles >= c.cap) {
                const int32_t st = bad ? SARAS_NAN : (c.res < c.tol ? SARAS_OK : SARAS_NOT_CONVERGED);
                if (c.rk) {
                    // the sub-stage's end (and the next one's start) runs on
                    // the worker while the next batch runs; the case keeps
                    // its slot and items
                    c.total_cycles += c.cycles;
                    StepJob j;
                    j.c = c;
                    j.kind = STEP_ADVANCE;
                    j.solve_status = st;
                    h->active.erase(h->active.begin() + (long)q);
                    h->dirty = true;
                    h->steps->submit(std::move(j));
                    continue;
                }
                // out of the next batch's tables; retired while it runs
                h->finishing.emplace_back(c, st);
                h->active.erase(h->active.begin() + (long)q);
                h->dirty = true;
                continue;
            }
            q++;
        }
        if (!h->incoming.empty()) {
            for (ServeCase &c : h->incoming) h->active.push_back(c);
            h->incoming.clear();
            h->dirty = true;
        }
    } else if (h->steps && h->steps->held() > 0) {
        // nothing to batch until the worker hands a case back: wait for one
        // (briefly, so that the caller can submit meanwhile)
        collect_steps(h, 0.002);
    }
    // no batch follows to overlap the copies out with
    if (h->active.empty()) SARAS_TRY(flush_finishing(h));
    const int held = h->steps ? h->steps->held() : 0;
    if (active) *active = (int32_t)(h->active.size() + h->incoming.size() + h->finishing.size() + held);
    if (pending) *pending = (int32_t)h->pending.size();
    return SARAS_OK;
}

saras_status saras_serve_poll(saras_serve *h, int64_t *ids, double *residuals, int32_t *cycles, int32_t *status,
                              double *latency_s, int32_t cap, int32_t *n) {
    if (!h || !n || cap < 0) return SARAS_BAD_ARG;
    int32_t m = 0;
    while (m < cap && !h->done.empty()) {
        const ServeDone &d = h->done.front();
        if (ids) ids[m] = d.id;
        if (residuals) residuals[m] = d.res;
        if (cycles) cycles[m] = d.cycles;
        if (status) status[m] = d.status;
        if (latency_s) latency_s[m] = d.latency;
        h->done.pop_front();
        m++;
    }
    *n = m;
    return SARAS_OK;
}

saras_status saras_serve_autotune(saras_serve *h, const saras_grid_desc *grids, int32_t n, int32_t cycles,
                                  saras_serve_params *chosen) {
    if (!h || !grids || n < 1 || cycles < 1) {
        set_error("invalid autotune arguments");
        return SARAS_BAD_ARG;
    }
    if (!idle(h) || !h->pending.empty()) {
        set_error("autotune needs an idle engine");
        return SARAS_BAD_ARG;
    }
    // synthetic requests: a fixed pseudo-random RHS per shape
    std::vector<std::vector<double>> rhs((size_t)n), lhs((size_t)n);
    for (int q = 0; q < n; q++) {
        const Box b = box_of(grids[q]);
        rhs[(size_t)q].resize((size_t)b.elems);
        lhs[(size_t)q].assign((size_t)b.elems, 0.0);
        uint64_t x = 0x9e3779b97f4a7c15ull * (uint64_t)(q + 1);
        for (double &v : rhs[(size_t)q]) {
            x = x * 6364136223846793005ull + 1442695040888963407ull;
            v = (double)(x >> 11) * (2.0 / 9007199254740992.0) - 1.0;
        }
        SARAS_TRY(enqueue(h, -1 - q, &grids[q], rhs[(size_t)q].data(), lhs[(size_t)q].data(), true));
    }
    saras_status st = admit(h, h->active);
    while (!h->pending.empty()) h->pending.pop_front();  // what did not fit is not tuned for
    if (st == SARAS_OK && h->active.empty()) {
        set_error("no autotune request fits the engine's budget");
        st = SARAS_BUDGET;
    }
    const int cand_cells[] = {1024, 2048, 4096, 8192};
    const int cand_threads[] = {128, 256, 512};
    const int cand_bps[] = {1, 2, 4};
    int best[3] = {h->cells, h->threads, h->bps};
    float best_ms = 1e30f;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (st == SARAS_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
        st = cuda_fail(cudaGetLastError(), "cudaEventCreate", __FILE__, __LINE__);
    for (int ci : cand_cells) {
        for (int ti : cand_threads) {
            for (int bi : cand_bps) {
                if (st != SARAS_OK) break;
                apply_schedule(h, ci, ti, bi);
                bool ok = true;
                for (int r = 0; r < NREG; r++) ok = ok && h->used[r] <= h->reg_cap[r];
                if (!ok) continue;
                st = run_batched(h);  // warm-up (and graph capture)
                if (st != SARAS_OK) break;
                cudaGraphExec_t g;
                st = graph_for(h, active_depth(h), &g);
                if (st != SARAS_OK) break;
                cudaEventRecord(e0, h->stream);
                for (int q = 0; q < cycles; q++) cudaGraphLaunch(g, h->stream);
                cudaEventRecord(e1, h->stream);
                const cudaError_t e = cudaEventSynchronize(e1);
                if (e != cudaSuccess) {
                    st = cuda_fail(e, "autotune timing", __FILE__, __LINE__);
                    break;
                }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms < best_ms) {
                    best_ms = ms;
                    best[0] = ci;
                    best[1] = ti;
                    best[2] = bi;
                }
            }
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    apply_schedule(h, best[0], best[1], best[2]);
    while (!h->active.empty()) {
        const saras_status s2 = retire(h, h->active.size() - 1, SARAS_OK);
        if (st == SARAS_OK) st = s2;
    }
    if (chosen) {
        *chosen = h->prm;
        chosen->cells_per_item = h->cells;
        chosen->threads = h->threads;
        chosen->blocks_per_sm = h->bps;
    }
    return st;
}

saras_status saras_serve_get_stats(const saras_serve *h, saras_serve_stats *out) {
    if (!h || !out) return SARAS_BAD_ARG;
    std::memset(out, 0, sizeof(*out));
    out->bytes_allocated = h->bytes_alloc;
    out->batched_cycles = h->cycles_run;
    out->launches = h->launches;
    out->admitted = h->admitted;
    out->retired = h->retired;
    out->active = (int32_t)(h->active.size() + h->incoming.size() + h->finishing.size() +
                            (h->steps ? h->steps->held() : 0));
    out->pending = (int32_t)h->pending.size();
    int pooled = 0;
    for (const auto &kv : h->pool) pooled += (int)kv.second.size();
    for (const auto &kv : h->step_pool) pooled += (int)kv.second.size();
    out->pooled = pooled;
    out->max_active = h->max_active;
    out->t_batch_s = h->t_batch;
    out->t_admit_s = h->t_admit;
    out->t_retire_s = h->t_retire;
    out->t_steps_s = h->t_steps;
    return SARAS_OK;
}

saras_status saras_serve_destroy(saras_serve *h) {
    if (!h) return SARAS_OK;
    if (h->steps) {
        // the job the worker is running ends first; the cases it still
        // holds go with their integrators
        for (ServeCase &c : h->steps->stop())
            if (c.rk) saras_rk3_destroy(c.rk);
        h->steps.reset();
    }
    for (cudaEvent_t e : h->join_ev) cudaEventDestroy(e);
    h->join_ev.clear();
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->adm) cudaStreamSynchronize(h->adm);
    if (h->stp) cudaStreamSynchronize(h->stp);
    for (ServeCase &c : h->incoming) h->active.push_back(c);
    h->incoming.clear();
    for (auto &f : h->finishing) h->active.push_back(f.first);
    h->finishing.clear();
    for (ServeCase &c : h->active) {
        if (c.rk)
            saras_rk3_destroy(c.rk);  // owns its hierarchy
        else
            saras_mg_destroy(c.mg);
    }
    for (auto &kv : h->pool)
        for (saras_mg *m : kv.second) saras_mg_destroy(m);
    for (auto &kv : h->step_pool)
        for (saras_rk3 *rk : kv.second) saras_rk3_destroy(rk);
    drop_graphs(h);
    cudaFree(h->d_lev);
    cudaFree(h->d_items);
    cudaFree(h->d_counts);
    cudaFree(h->d_part);
    cudaFree(h->d_fden);
    cudaFree(h->d_res);
    cudaFree(h->d_box);
    if (h->h_res) cudaFreeHost(h->h_res);
    if (h->h_lev) cudaFreeHost(h->h_lev);
    if (h->h_items) cudaFreeHost(h->h_items);
    if (h->h_counts) cudaFreeHost(h->h_counts);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->adm) cudaStreamDestroy(h->adm);
    if (h->ev_adm) cudaEventDestroy(h->ev_adm);
    if (h->stp) cudaStreamDestroy(h->stp);
    if (h->ev_stp) cudaEventDestroy(h->ev_stp);
    for (auto &u : h->pin_busy) cudaEventDestroy(u.ev);
    for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
    if (h->pin) cudaFreeHost(h->pin);
    delete h;
    return SARAS_OK;
}

}  // extern "C"
