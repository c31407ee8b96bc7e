// TMA-staged colour sweep of the MIXED form's FP32 error equation on the
// large 3-D levels.
//
// A block owns a tile of `tj` rows (j) by the whole row (k) and marches
// through a chunk of planes (i).  Planes stream through a four-slot ring in
// shared memory: the tensor-memory accelerator (cp.async.bulk.tensor) loads
// the e tile with one halo row on each side and the r tile three planes
// ahead of the plane being updated, an mbarrier per slot signals arrival, the
// threads update the sweep's colour in place in shared memory, and a TMA
// store writes the tile's rows back whole.  Cells of the other colour are
// only read, so the in-place update needs no copy: every value a cell of the
// sweep's colour reads (its six neighbours) is of the other colour, within
// the block and across blocks.  The arithmetic per cell is that of
// k_rbgs_v8 (mg_fast.cu), so results are bit-identical.
//
// Every wait on an mbarrier is bounded; a wait that runs out sets an error
// word the host reads with the residual (norm_out[7]), waits (bounded) for
// the copies it issued and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>

#include "mg_fast.cuh"
#include "mg_stencil.cuh"

namespace saras {
namespace {

constexpr int TMA_THREADS = 256;
constexpr int TMA_SLOTS = 4;
constexpr unsigned TMA_WAIT_LIMIT = 1u << 24;

__device__ __forceinline__ uint32_t sa(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sa(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sa(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(sa(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// bounded wait; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (unsigned n = 0; n < TMA_WAIT_LIMIT; n++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void tma_load3(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(sa(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(sa(bar))
        : "memory");
}
__device__ __forceinline__ void tma_store3(const CUtensorMap *map, const void *src, int x, int y, int z) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(x), "r"(y), "r"(z), "r"(sa(src))
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }


// The colour cells of one 4-cell strip: k_rbgs_v8's strip_update (WD off),
// cell for cell.  Lanes of a warp own consecutive strips, so each quarter
// warp reads 128 contiguous bytes of shared memory per vector load.
template <int T0>
__device__ __forceinline__ void strip4(float *u, const float4 cur, const float4 xm, const float4 xp,
                                       const float4 ym, const float4 yp, const float4 fr, float left, float right,
                                       float cmx, float cpx, float dx, float cmy, float cpy, float dy,
                                       const float (&zc)[3][4], float w, float omc) {
    const float c[4] = {cur.x, cur.y, cur.z, cur.w};
    const float a[4] = {xm.x, xm.y, xm.z, xm.w}, bq[4] = {xp.x, xp.y, xp.z, xp.w};
    const float ya[4] = {ym.x, ym.y, ym.z, ym.w}, yb[4] = {yp.x, yp.y, yp.z, yp.w};
    const float f[4] = {fr.x, fr.y, fr.z, fr.w};
#pragma unroll
    for (int q = T0; q < 4; q += 2) {
        const float zm = q > 0 ? c[q - 1] : left;
        const float zp = q < 3 ? c[q + 1] : right;
        float sm = cmx * a[q];
        sm = fmat(cpx, bq[q], sm);
        sm = fmat(cmy, ya[q], sm);
        sm = fmat(cpy, yb[q], sm);
        sm = fmat(zc[0][q], zm, sm);
        sm = fmat(zc[1][q], zp, sm);
        sm = sm - f[q];
        float d = dx + zc[2][q];
        d += dy;
        u[q] = fmat(omc, c[q], sweep_div(w * sm, d + d));
    }
}

__device__ __forceinline__ float4 mirror4(float4 c, int sg) {
    return sg > 0 ? c : make_float4(-c.x, -c.y, -c.z, -c.w);
}
__device__ __forceinline__ float4 lds4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

__global__ void __launch_bounds__(TMA_THREADS) k_rbgs_tma(const __grid_constant__ CUtensorMap eld,
                                                          const __grid_constant__ CUtensorMap est,
                                                          const __grid_constant__ CUtensorMap rld,
                                                          const float *__restrict__ eg, Lay L, Tab3<float> t, Bnd b,
                                                          int colour, float w, float omc, int tj, int chunk,
                                                          int *err) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int s_fail;
    const int n2 = L.n2;
    const int e_slot = (tj + 2) * n2, r_slot = tj * n2;
    float *es = reinterpret_cast<float *>(smem);
    float *rs = es + TMA_SLOTS * e_slot;
    uint64_t *bar = reinterpret_cast<uint64_t *>(rs + TMA_SLOTS * r_slot);
    float *zt = reinterpret_cast<float *>(bar + TMA_SLOTS);  // c-, c+, d of the z axis
    for (int k = threadIdx.x; k < n2; k += blockDim.x) {
        zt[k] = t.cm[2][k];
        zt[n2 + k] = t.cp[2][k];
        zt[2 * n2 + k] = t.dg[2][k];
    }
    const int j0 = (int)blockIdx.x * tj;
    const int i0 = (int)blockIdx.y * chunk;
    const int i1 = min(L.n0, i0 + chunk);
    if (i0 >= i1) return;
    const uint32_t bytes = (uint32_t)((e_slot + r_slot) * sizeof(float));
    auto slot = [](int p) { return (p + 1) & (TMA_SLOTS - 1); };
    if (threadIdx.x == 0) {
        for (int s = 0; s < TMA_SLOTS; s++) mbar_init(&bar[s], 1);
        mbar_init_fence();
        s_fail = 0;
    }
    __syncthreads();
    // plane p: e rows j0-1 .. j0+tj (memory rows j0 .. j0+tj+1) and r rows j0 .. j0+tj-1
    auto issue = [&](int p) {
        const int s = slot(p);
        mbar_expect_tx(&bar[s], bytes);
        tma_load3(es + s * e_slot, &eld, &bar[s], KOFF, j0, p + 1);
        tma_load3(rs + s * r_slot, &rld, &bar[s], KOFF, j0 + 1, p + 1);
    };
    const int last = i1;  // planes i0-1 .. i1 are read
    int issued = i0 - 2;  // last plane issued
    if (threadIdx.x == 0)
        for (int p = i0 - 1; p <= min(i0 + 2, last); p++) issue(p);
    issued = min(i0 + 2, last);
    uint32_t phase = 0;
    int waited = i0 - 2;  // last plane waited for
    // one thread waits on the slot's mbarrier; the block barrier that follows
    // every wait releases the others (and orders the landed tile before
    // their reads)
    auto wait_plane = [&](int p) {
        const int s = slot(p);
        if (threadIdx.x == 0 && !mbar_wait(&bar[s], (phase >> s) & 1u)) s_fail = 1;
        phase ^= 1u << s;
        waited = p;
    };
    wait_plane(i0 - 1);
    wait_plane(i0);
    __syncthreads();
    // thread -> (row, 4-cell strip): rows jj = sj, sj + rstep, ...; the
    // z-axis coefficients of the thread's four cells stay in registers
    const int s4 = n2 >> 2;
    const int rstep = blockDim.x / s4;
    const int sj = threadIdx.x / s4;
    const int k0 = (threadIdx.x - sj * s4) * 4;
    float zc[3][4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        zc[0][q] = zt[k0 + q];
        zc[1][q] = zt[n2 + k0 + q];
        zc[2][q] = zt[2 * n2 + k0 + q];
    }
    const bool kfirst = k0 == 0, klast = k0 + 4 >= n2;
    // y-axis coefficients of the thread's rows (at most two with 256 threads)
    float ycm[2] = {0.f, 0.f}, ycp[2] = {0.f, 0.f}, ydg[2] = {0.f, 0.f};
    for (int m = 0, jj = sj; m < 2 && jj < tj; m++, jj += rstep) {
        ycm[m] = t.cm[1][j0 + jj];
        ycp[m] = t.cp[1][j0 + jj];
        ydg[m] = t.dg[1][j0 + jj];
    }
    for (int i = i0; i < i1 && !s_fail; i++) {
        wait_plane(i + 1);
        __syncthreads();
        if (s_fail) break;
        float *pc = es + slot(i) * e_slot;
        const float *pm = es + slot(i - 1) * e_slot;
        const float *pp = es + slot(i + 1) * e_slot;
        const float *rr = rs + slot(i) * r_slot;
        const float cmx = t.cm[0][i], cpx = t.cp[0][i], dx = t.dg[0][i];
#pragma unroll
        for (int m = 0; m < 2; m++) {
            const int jj = sj + m * rstep;
            if (jj >= tj) break;
            const int j = j0 + jj;
            float *row = pc + (jj + 1) * n2;
            const float4 cur = lds4(row + k0);
            float4 xm, xp, ym, yp;
            if (i > 0) xm = lds4(pm + (jj + 1) * n2 + k0);
            else if (b.per[0]) xm = *reinterpret_cast<const float4 *>(eg + L.at(L.n0 - 1, j, k0));
            else xm = mirror4(cur, b.sg_lo[0]);
            if (i < L.n0 - 1) xp = lds4(pp + (jj + 1) * n2 + k0);
            else if (b.per[0]) xp = *reinterpret_cast<const float4 *>(eg + L.at(0, j, k0));
            else xp = mirror4(cur, b.sg_hi[0]);
            if (j > 0) ym = lds4(row - n2 + k0);
            else if (b.per[1]) ym = *reinterpret_cast<const float4 *>(eg + L.at(i, L.n1 - 1, k0));
            else ym = mirror4(cur, b.sg_lo[1]);
            if (j < L.n1 - 1) yp = lds4(row + n2 + k0);
            else if (b.per[1]) yp = *reinterpret_cast<const float4 *>(eg + L.at(i, 0, k0));
            else yp = mirror4(cur, b.sg_hi[1]);
            const float4 fr = lds4(rr + jj * n2 + k0);
            const float left = !kfirst ? row[k0 - 1] : (b.per[2] ? row[n2 - 1] : (b.sg_lo[2] > 0 ? cur.x : -cur.x));
            const float right = !klast ? row[k0 + 4] : (b.per[2] ? row[0] : (b.sg_hi[2] > 0 ? cur.w : -cur.w));
            const float cmy = ycm[m], cpy = ycp[m], dy = ydg[m];
            if (((colour + i + j) & 1) == 0)
                strip4<0>(row + k0, cur, xm, xp, ym, yp, fr, left, right, cmx, cpx, dx, cmy, cpy, dy, zc, w, omc);
            else
                strip4<1>(row + k0, cur, xm, xp, ym, yp, fr, left, right, cmx, cpx, dx, cmy, cpy, dy, zc, w, omc);
        }
        fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            tma_store3(&est, pc + n2, KOFF, j0 + 1, i + 1);
            bulk_commit();
            if (i + 3 <= last) {
                bulk_wait_read1();  // the store of plane i-1 has read the slot plane i+3 reuses
                issue(i + 3);
            }
        }
        if (i + 3 <= last) issued = i + 3;
    }
    if (threadIdx.x == 0) {
        if (s_fail) {
            atomicExch(err, 1);
            // let every load still in flight land before the block's shared memory goes away
            for (int p = waited + 1; p <= issued; p++) {
                const int s = slot(p);
                mbar_wait(&bar[s], (phase >> s) & 1u);
                phase ^= 1u << s;
            }
        }
        bulk_wait_all();
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

bool encode3(CUtensorMap *m, const float *base, const Lay &L, int rows) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dim[3] = {(cuuint64_t)L.s1, (cuuint64_t)L.n1 + 2, (cuuint64_t)L.n0 + 2};
    const cuuint64_t stride[2] = {(cuuint64_t)L.s1 * sizeof(float), (cuuint64_t)L.s0 * sizeof(float)};
    const cuuint32_t box[3] = {(cuuint32_t)L.n2, (cuuint32_t)rows, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dim, stride, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

size_t tma_smem(int tj, int n2) {
    return (size_t)TMA_SLOTS * ((size_t)(tj + 2) * n2 + (size_t)tj * n2) * sizeof(float) + TMA_SLOTS * 8 +
           (size_t)3 * n2 * sizeof(float);
}

}  // namespace

// Plans the TMA sweep of one level: tile rows, plane chunk and the three
// tensor maps (e with halo rows, e without, r).  Levels that do not qualify
// keep the vector sweep.
void tma_plan(saras_mg *h, Level &v) {
    v.tma.ok = 0;
    const Lay &L = v.lay;
    if (!h->d3 || !v.e32 || !v.r32) return;
    // rows of 32..256 cells, a power of two: 256 threads cover a tile as
    // (row, 4-cell strip) pairs, two rows each
    if (L.n2 < 32 || L.n2 > 256 || 1024 % L.n2 != 0 || (int64_t)L.n0 * L.n1 * L.n2 < (1 << 20)) return;
    int tj = std::max(2, 2048 / L.n2);
    while (tj >= 2 && (L.n1 % tj != 0 || tj + 2 > 256)) tj /= 2;
    if (tj < 2) return;
    if (tma_smem(tj, L.n2) > 200 * 1024) return;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int jt = L.n1 / tj;
    const int want = 3 * sms;
    const int nchunks = std::max(1, want / jt);  // one wave: at most three blocks per SM
    const int chunk = std::max(4, (L.n0 + nchunks - 1) / nchunks);
    if (!encode3(&v.tma.eld, v.e32, L, tj + 2) || !encode3(&v.tma.est, v.e32, L, tj) ||
        !encode3(&v.tma.rld, v.r32, L, tj))
        return;
    // one attribute for every level and handle: the largest ring any plan may use
    if (cudaFuncSetAttribute(k_rbgs_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    v.tma.tj = tj;
    v.tma.chunk = chunk;
    v.tma.ok = 1;
}

// One colour sweep through the TMA path; false when the level has none.
bool tma_colour(saras_mg *h, cudaStream_t s, Level &v, int colour) {
    if (!v.tma.ok) return false;
    const Lay &L = v.lay;
    const dim3 grid((unsigned)(L.n1 / v.tma.tj), (unsigned)((L.n0 + v.tma.chunk - 1) / v.tma.chunk));
    const Tab3<float> t{{v.cm32[0], v.cm32[1], v.cm32[2]}, {v.cp32[0], v.cp32[1], v.cp32[2]},
                        {v.dg32[0], v.dg32[1], v.dg32[2]}};
    Bnd b;
    for (int d = 0; d < 3; d++) {
        b.per[d] = h->ghost.per[d];
        b.sg_lo[d] = h->ghost.kind[2 * d] == SARAS_BC_NEUMANN ? 1 : -1;
        b.sg_hi[d] = h->ghost.kind[2 * d + 1] == SARAS_BC_NEUMANN ? 1 : -1;
    }
    int *err = reinterpret_cast<int *>(h->norm_out + 7);
    k_rbgs_tma<<<grid, TMA_THREADS, tma_smem(v.tma.tj, L.n2), s>>>(
        v.tma.eld, v.tma.est, v.tma.rld, v.e32, L, t, b, colour, (float)h->prm.sor_param,
        (float)(1.0 - h->prm.sor_param), v.tma.tj, v.tma.chunk, err);
    return true;
}

}  // namespace saras
