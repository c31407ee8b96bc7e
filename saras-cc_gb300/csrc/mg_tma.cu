// TMA-staged colour sweep of the MIXED form's FP32 error equation on the
// large 3-D levels.
//
// A block owns a tile of `tj` rows (j) by the whole row (k) and marches
// through a chunk of planes (i).  Planes stream through a ring of slots in
// shared memory: a producer lane loads the e tile (with one halo row on each
// side) and the r tile with cp.async.bulk.tensor as soon as a slot is free,
// and eight consumer warps, each owning tj/8 rows, update the sweep's colour
// in place in shared memory and write their rows back whole with their own
// TMA stores.  Cells of the other colour are only read, so the in-place
// update needs no copy and the warps never wait for one another: every
// value a cell of the sweep's colour reads (its six neighbours) is of the
// other colour, within the block and across blocks.  The arithmetic per cell
// is that of k_rbgs_v8 (mg_fast.cu), so results are bit-identical.
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

constexpr int TMA_SLOTS = 5;
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

// Warp-specialised pipeline: warp 0 (one lane) loads planes into a ring of
// TMA_SLOTS slots, each with a "full" mbarrier (completed by the TMA
// transaction count) and an "empty" mbarrier (one arrival per consumer warp).
// Each of the TMA_CONSUMERS consumer warps owns tj / TMA_CONSUMERS rows of
// the tile: for plane i it waits for plane i+1 to land, updates the sweep's
// colour in its rows in place, stores its rows with its own TMA store, and
// releases plane i-1.  Warps never wait for one another: a warp reads other
// warps' rows only at cells of the other colour, which nobody writes in this
// sweep.
constexpr int TMA_CONSUMERS = 8;
constexpr int TMA_WS_THREADS = 32 * (TMA_CONSUMERS + 1);

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(sa(bar)) : "memory");
}

__global__ void __launch_bounds__(TMA_WS_THREADS) k_rbgs_tma(const __grid_constant__ CUtensorMap eld,
                                                             const __grid_constant__ CUtensorMap est,
                                                             const __grid_constant__ CUtensorMap rld,
                                                             const float *__restrict__ eg, Lay L, Tab3<float> t,
                                                             Bnd b, int colour, float w, float omc, int tj,
                                                             int chunk, int *err) {
    pdl_enter();
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int s_fail;
    const int n2 = L.n2;
    const int e_slot = (tj + 2) * n2, r_slot = tj * n2;
    float *es = reinterpret_cast<float *>(smem);
    float *rs = es + TMA_SLOTS * e_slot;
    uint64_t *full = reinterpret_cast<uint64_t *>(rs + TMA_SLOTS * r_slot);
    uint64_t *empty = full + TMA_SLOTS;
    const int j0 = (int)blockIdx.x * tj;
    const int i0 = (int)blockIdx.y * chunk;
    const int i1 = min(L.n0, i0 + chunk);
    if (i0 >= i1) return;
    if (threadIdx.x == 0) {
        for (int q = 0; q < TMA_SLOTS; q++) {
            mbar_init(&full[q], 1);
            mbar_init(&empty[q], TMA_CONSUMERS);
        }
        mbar_init_fence();
        s_fail = 0;
    }
    __syncthreads();
    // plane p (i0-1 .. i1) uses slot u % TMA_SLOTS for u = p - (i0-1); its
    // full phase is (u / TMA_SLOTS) & 1, and it may be loaded once the
    // previous occupant (u - TMA_SLOTS) has been released
    const int first = i0 - 1;
    auto slot_of = [&](int p) { return (p - first) % TMA_SLOTS; };
    auto par_of = [&](int p) { return (uint32_t)(((p - first) / TMA_SLOTS) & 1); };
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        // ---- producer ----
        if (lane == 0) {
            const uint32_t bytes = (uint32_t)((e_slot + r_slot) * sizeof(float));
            int p = first;
            for (; p <= i1; p++) {
                const int q = slot_of(p);
                if (p - first >= TMA_SLOTS && !s_fail) {
                    if (!mbar_wait(&empty[q], (uint32_t)(((p - first) / TMA_SLOTS - 1) & 1))) {
                        s_fail = 1;
                        atomicExch(err, 1);
                    }
                }
                if (s_fail) break;
                mbar_expect_tx(&full[q], bytes);
                tma_load3(es + q * e_slot, &eld, &full[q], KOFF, j0, p + 1);
                tma_load3(rs + q * r_slot, &rld, &full[q], KOFF, j0 + 1, p + 1);
            }
            // nothing may be in flight when the block exits: wait (bounded)
            // for the last planes issued to land
            for (int x = max(first, p - TMA_SLOTS); x < p; x++) mbar_wait(&full[slot_of(x)], par_of(x));
        }
        return;
    }
    // ---- consumers ----
    // A tile holds 2048 cells (tj * n2), so each lane owns exactly two
    // 4-cell strips per plane, at fixed (row, k) positions: their z and y
    // coefficients and boundary flags stay in registers for the whole chunk.
    const int cw = warp - 1;
    const int rows = tj / TMA_CONSUMERS;  // rows of this warp
    const int r0 = cw * rows;             // first tile row of this warp
    const int s4 = n2 >> 2;               // 4-cell strips per row
    int jj[2], k0[2];
    float zc[2][3][4], cmy[2], cpy[2], dy[2];
#pragma unroll
    for (int m = 0; m < 2; m++) {
        const int q = lane + 32 * m;
        jj[m] = r0 + q / s4;
        k0[m] = (q % s4) * 4;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            zc[m][0][c] = t.cm[2][k0[m] + c];
            zc[m][1][c] = t.cp[2][k0[m] + c];
            zc[m][2][c] = t.dg[2][k0[m] + c];
        }
        const int j = j0 + jj[m];
        cmy[m] = t.cm[1][j];
        cpy[m] = t.cp[1][j];
        dy[m] = t.dg[1][j];
    }
    auto wait_full = [&](int p) {
        if (s_fail) return false;
        if (!mbar_wait(&full[slot_of(p)], par_of(p))) {
            s_fail = 1;
            atomicExch(err, 1);
            return false;
        }
        return true;
    };
    bool ok = wait_full(first) && wait_full(i0);
    for (int i = i0; i < i1 && ok; i++) {
        ok = wait_full(i + 1);
        if (!ok) break;
        float *pc = es + slot_of(i) * e_slot;
        const float *pm = es + slot_of(i - 1) * e_slot;
        const float *pp = es + slot_of(i + 1) * e_slot;
        const float *rr = rs + slot_of(i) * r_slot;
        const float cmx = t.cm[0][i], cpx = t.cp[0][i], dx = t.dg[0][i];
#pragma unroll
        for (int m = 0; m < 2; m++) {
            const int j = j0 + jj[m], kk = k0[m];
            float *row = pc + (jj[m] + 1) * n2;
            const float4 cur = lds4(row + kk);
            float4 xm, xp, ym, yp;
            if (i > 0) xm = lds4(pm + (jj[m] + 1) * n2 + kk);
            else if (b.per[0]) xm = *reinterpret_cast<const float4 *>(eg + L.at(L.n0 - 1, j, kk));
            else xm = mirror4(cur, b.sg_lo[0]);
            if (i < L.n0 - 1) xp = lds4(pp + (jj[m] + 1) * n2 + kk);
            else if (b.per[0]) xp = *reinterpret_cast<const float4 *>(eg + L.at(0, j, kk));
            else xp = mirror4(cur, b.sg_hi[0]);
            if (j > 0) ym = lds4(row - n2 + kk);
            else if (b.per[1]) ym = *reinterpret_cast<const float4 *>(eg + L.at(i, L.n1 - 1, kk));
            else ym = mirror4(cur, b.sg_lo[1]);
            if (j < L.n1 - 1) yp = lds4(row + n2 + kk);
            else if (b.per[1]) yp = *reinterpret_cast<const float4 *>(eg + L.at(i, 0, kk));
            else yp = mirror4(cur, b.sg_hi[1]);
            const float4 fr = lds4(rr + jj[m] * n2 + kk);
            const float left = kk > 0 ? row[kk - 1] : (b.per[2] ? row[n2 - 1] : (b.sg_lo[2] > 0 ? cur.x : -cur.x));
            const float right = kk + 4 < n2 ? row[kk + 4] : (b.per[2] ? row[0] : (b.sg_hi[2] > 0 ? cur.w : -cur.w));
            if (((colour + i + j) & 1) == 0)
                strip4<0>(row + kk, cur, xm, xp, ym, yp, fr, left, right, cmx, cpx, dx, cmy[m], cpy[m], dy[m], zc[m],
                          w, omc);
            else
                strip4<1>(row + kk, cur, xm, xp, ym, yp, fr, left, right, cmx, cpx, dx, cmy[m], cpy[m], dy[m], zc[m],
                          w, omc);
        }
        fence_async_smem();
        __syncwarp();
        if (lane == 0) {
            tma_store3(&est, pc + (r0 + 1) * n2, KOFF, j0 + r0 + 1, i + 1);
            bulk_commit();
            if (i > i0 - 1) {
                bulk_wait_read1();  // this warp's store of plane i-1 has read the slot
                mbar_arrive(&empty[slot_of(i - 1)]);
            }
        }
        __syncwarp();
    }
    if (lane == 0) bulk_wait_all();
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
    return (size_t)TMA_SLOTS * ((size_t)(tj + 2) * n2 + (size_t)tj * n2) * sizeof(float) + 2 * TMA_SLOTS * 8;
}

}  // namespace

// Plans the TMA sweep of one level: tile rows, plane chunk and the three
// tensor maps (e with halo rows, e without, r).  Levels that do not qualify
// keep the vector sweep.
void tma_plan(saras_mg *h, Level &v) {
    v.tma.ok = 0;
    const Lay &L = v.lay;
    if (!h->d3 || !v.e32 || !v.r32) return;
    // rows of 32..256 cells (a power of two); tiles of 2048 cells shared by
    // the consumer warps row-wise
    if (L.n2 < 32 || L.n2 > 256 || 1024 % L.n2 != 0 || (int64_t)L.n0 * L.n1 * L.n2 < (1 << 20)) return;
    // tiles of exactly 2048 cells: two 4-cell strips per consumer lane
    const int tj = 2048 / L.n2;
    if (L.n1 % tj != 0 || tj % TMA_CONSUMERS != 0 || tj + 2 > 256) return;
    const size_t smem = tma_smem(tj, L.n2);
    if (smem > 200 * 1024) return;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int per_sm = std::max(1, (int)((227 * 1024) / smem));
    const int jt = L.n1 / tj;
    const int nchunks = std::max(1, per_sm * sms / jt);  // one wave
    const int chunk = std::max(4, (L.n0 + nchunks - 1) / nchunks);
    if (!encode3(&v.tma.eld, v.e32, L, tj + 2) || !encode3(&v.tma.est, v.e32, L, tj / TMA_CONSUMERS) ||
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
    launch_pdl(k_rbgs_tma, grid, dim3(TMA_WS_THREADS), tma_smem(v.tma.tj, L.n2), s, v.tma.eld, v.tma.est, v.tma.rld,
               (const float *)v.e32, L, t, b, colour, (float)h->prm.sor_param, (float)(1.0 - h->prm.sor_param),
               v.tma.tj, v.tma.chunk, err);
    return true;
}

}  // namespace saras
