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
// word the host reads with the residual (norm_out[7]); the block then stops
// issuing copies, waits (with the default bound) for the loads and stores it
// issued and returns.  The host may lower the pipeline waits' bound
// (saras_mg_set_wait_limit) to exercise that path.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <type_traits>

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
__device__ __forceinline__ bool mbar_test_wait(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(sa(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// bounded wait of at most `limit` polls (the first a non-blocking test, the
// others potentially blocking tries); false when the limit ran out.  The
// pipeline's waits take the handle's limit (TMA_WAIT_LIMIT unless the host
// set another); the waits that drain a block's own copies before it exits
// always take TMA_WAIT_LIMIT, so that no copy is in flight when the block's
// shared memory is released
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, unsigned limit = TMA_WAIT_LIMIT) {
    if (mbar_test_wait(bar, parity)) return true;
    for (unsigned n = 1; n < limit; n++)
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
__device__ __forceinline__ void tma_load4(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y, int z,
                                          int w) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(sa(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(sa(bar))
        : "memory");
}
__device__ __forceinline__ void tma_store4(const CUtensorMap *map, const void *src, int x, int y, int z, int w) {
    asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3, %4}], [%5];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(x), "r"(y), "r"(z), "r"(w), "r"(sa(src))
                 : "memory");
}
// Whole rows of a level between global and shared memory: rows of up to 256
// cells through a 3-D map (x = KOFF, the core's first cell); rows of 512
// (split) through a 4-D map that views each row's core as two halves of 256
// cells, box 256 x 2 x rows, which lands as rows of 512 contiguous cells.
// y and z are the row and plane coordinates (ghost layer at 0).
__device__ __forceinline__ void tma_rows(void *dst, const CUtensorMap *map, uint64_t *bar, int split, int y, int z) {
    if (split)
        tma_load4(dst, map, bar, 0, 0, y, z);
    else
        tma_load3(dst, map, bar, KOFF, y, z);
}
__device__ __forceinline__ void tma_rows_store(const CUtensorMap *map, const void *src, int split, int y, int z) {
    if (split)
        tma_store4(map, src, 0, 0, y, z);
    else
        tma_store3(map, src, KOFF, y, z);
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }


// The colour cells of one 4-cell strip: k_rbgs_v8's strip_update (WD off),
// cell for cell.  Lanes of a warp own consecutive strips, so each quarter
// warp reads 128 contiguous bytes of shared memory per vector load.
template <int T0, bool W1 = false>
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
        // W1: the SOR parameter is 1 and the blend returns s/(2d) unchanged
        u[q] = W1 ? sweep_div(sm, d + d) : fmat(omc, c[q], sweep_div(w * sm, d + d));
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
                                                             int chunk, int *err, unsigned wlim) {
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
                    if (!mbar_wait(&empty[q], (uint32_t)(((p - first) / TMA_SLOTS - 1) & 1), wlim)) {
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
        if (!mbar_wait(&full[slot_of(p)], par_of(p), wlim)) {
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

// ---- One whole red-black iteration per launch, out of place ----
//
// k_rbgs_tma moves e and r through HBM once per colour.  k_rbgs_fused runs
// both colours of an iteration in one pass: a block reads its tile of e
// (from the source buffer) and of r once, updates the first colour, then the
// second, and stores the tile into the destination buffer.  The second
// colour of a cell needs the first colour's new values around it, also those
// of the neighbouring tiles and chunks, which other blocks produce at times
// nobody orders; so the block recomputes the first colour itself on one halo
// row each side of its tile and one halo plane each side of its chunk, from
// the source buffer, which no block writes during the launch (two halo rows
// and planes of e, one of r).  The arithmetic per cell is strip4's, so one
// launch gives the bits of k_rbgs_tma's colour-0 launch followed by its
// colour-1 launch.
//
// Tiles: tj rows (FU_TILE cells) by the whole row; the block marches through
// planes i0-1 .. i1 of its chunk.  Per plane step q, every consumer thread:
//   R(q):   first colour on plane q, tile rows and halo rows;
//   barrier (consumer threads): R(q) and K(q-2) complete everywhere;
//   thread 0: TMA store of plane q-2, release of e(q-3) and r(q-2);
//   K(q-1): second colour on plane q-1, tile rows.
// R(q) reads the second colour on planes q-1..q+1 (old values) and K(q-1)
// the first colour on planes q-2..q (new values).  Between two barriers
// threads run K(q-1) and R(q+1), which update disjoint cells; a strip is
// written back whole, its cells of the other colour unchanged (the bits a
// concurrent reader expects).  A producer lane streams e planes through a
// ring of FU_ESLOTS slots and r planes through FU_RSLOTS slots, two steps
// ahead of their first use.
//
// Consumer warps: 12 on the plain layout; 9 on the row-split layout, whose
// strips carry fewer instructions, so that its per-step barrier waits on
// fewer warps (9 warps give every thread two of the 18 rows of R at 256-cell
// rows).
template <bool RS>
__host__ __device__ constexpr int fu_nt() {
    return 32 * (RS ? 9 : 12);
}
template <bool RS>
__host__ __device__ constexpr int fu_threads() {
    return fu_nt<RS>() + 32;
}
constexpr int FU_ESLOTS = 6, FU_RSLOTS = 4;
constexpr int FU_TILE = 4096;
constexpr int64_t FU_MIN_CELLS = int64_t(1) << 22;
// tile rows: FU_TILE cells, or four rows of 512 cells (the rings of 8-row
// tiles would not fit the shared memory)
__host__ __device__ constexpr int fu_tile_rows(int n2) { return n2 == 512 ? 4 : FU_TILE / n2; }
// head of the dynamic shared memory: mbarriers, the tile's y coefficients
// (from byte 256) and the chunk's x coefficients (from byte 1024, chunk + 2
// planes of three), rounded up to 1 KB and at least 4 KB
__host__ __device__ constexpr size_t fu_head(int chunk) {
    return ((1024 + 12 * (size_t)(chunk + 2) + 1023) / 1024 * 1024) > 4096
               ? (1024 + 12 * (size_t)(chunk + 2) + 1023) / 1024 * 1024
               : 4096;
}

template <int NT>
__device__ __forceinline__ void consumer_sync() {
    asm volatile("bar.sync 1, %0;" ::"r"(NT) : "memory");
}
__device__ __forceinline__ int wrap(int a, int n) { return ((a % n) + n) % n; }

// Colour cells of the strip at row[k0 .. k0+3] (a tile row of e in shared
// memory); xmr / xpr: the same row on the planes below and above, rrow: the
// row of r.  Mirrors at non-periodic walls as k_rbgs_tma forms them.
template <int PAR, bool W1>
__device__ __forceinline__ void fu_strip(float *row, const float *xmr, const float *xpr, const float *rrow, int n2,
                                         int k0, bool xlo, bool xhi, bool ylo, bool yhi, const Bnd &b, int li, int ri,
                                         bool lneg, bool rneg, float cmx, float cpx, float dx, float cmy, float cpy,
                                         float dy, const float (&zc)[3][4], float w, float omc) {
    const float4 cur = lds4(row + k0);
    // the neighbour rows always exist in the slots (halo rows, ghost or
    // out-of-range planes), so they are loaded unconditionally and replaced
    // by mirrors only on a wall (rare, and the same for a whole warp)
    float4 xm = lds4(xmr + k0), xp = lds4(xpr + k0), ym = lds4(row - n2 + k0), yp = lds4(row + n2 + k0);
    if (xlo | xhi | ylo | yhi) {
        if (xlo) xm = mirror4(cur, b.sg_lo[0]);
        if (xhi) xp = mirror4(cur, b.sg_hi[0]);
        if (ylo) ym = mirror4(cur, b.sg_lo[1]);
        if (yhi) yp = mirror4(cur, b.sg_hi[1]);
    }
    const float4 fr = lds4(rrow + k0);
    const float lv = row[li], rv = row[ri];
    const float left = lneg ? -lv : lv, right = rneg ? -rv : rv;
    float o[4] = {cur.x, cur.y, cur.z, cur.w};
    strip4<PAR, W1>(o, cur, xm, xp, ym, yp, fr, left, right, cmx, cpx, dx, cmy, cpy, dy, zc, w, omc);
    *reinterpret_cast<float4 *>(row + k0) = make_float4(o[0], o[1], o[2], o[3]);
}

// Row-split rows (each row: its red cells, then its black cells, in k
// order): the four cells of one colour at compact positions m .. m+3 of the
// half `own` (0 red, H black) of `row`, own k = 2 (m + q) + o.  Every x and y
// neighbour is the other colour at the same compact positions of the
// neighbouring rows' other half; the z neighbours are the other half of the
// same row at m .. m+3 shifted by one (left of it for o = 0, right for
// o = 1), with the row's wrap or wall mirror at its ends.  strip4's
// arithmetic, cell for cell, on four cells of one colour.
// The strip's neighbour outside its four z positions (left for o = 0, right
// for o = 1): `zo` indexes it in the row when it is a cell of the row (an
// interior neighbour or a periodic wrap), otherwise zmode is 1 (Neumann
// wall: the strip's own end cell) or 2 (Dirichlet wall: minus it).  The
// thread's strip position is fixed, so zo and zmode are set once per kernel.
// W1: the SOR parameter is 1, and (1 - w) u + w s/(2d) is s/(2d) (w s = s
// exactly; 0 u + v = v for finite u), so the multiply and the final FMA are
// skipped with the same values.
template <int o, bool W1>
__device__ __forceinline__ void fu_strip_rs(float *row, const float *xmr, const float *xpr, const float *rrow, int n2,
                                            int own, int oth, int m, int zo, int zmode, bool xlo, bool xhi, bool ylo,
                                            bool yhi, const Bnd &b, float cmx, float cpx, float dx, float cmy,
                                            float cpy, float dy, const float (&zc)[3][4], float w, float omc) {
    const float4 cur4 = lds4(row + own + m);
    // neighbour rows always exist in the slots; mirrors replace them on walls
    float4 xm4 = lds4(xmr + oth + m), xp4 = lds4(xpr + oth + m);
    float4 ym4 = lds4(row - n2 + oth + m), yp4 = lds4(row + n2 + oth + m);
    if (xlo | xhi | ylo | yhi) {
        if (xlo) xm4 = mirror4(cur4, b.sg_lo[0]);
        if (xhi) xp4 = mirror4(cur4, b.sg_hi[0]);
        if (ylo) ym4 = mirror4(cur4, b.sg_lo[1]);
        if (yhi) yp4 = mirror4(cur4, b.sg_hi[1]);
    }
    const float4 f4 = lds4(rrow + own + m);
    const float4 a4 = lds4(row + oth + m);
    const float c[4] = {cur4.x, cur4.y, cur4.z, cur4.w};
    const float xm[4] = {xm4.x, xm4.y, xm4.z, xm4.w}, xp[4] = {xp4.x, xp4.y, xp4.z, xp4.w};
    const float ym[4] = {ym4.x, ym4.y, ym4.z, ym4.w}, yp[4] = {yp4.x, yp4.y, yp4.z, yp4.w};
    const float f[4] = {f4.x, f4.y, f4.z, f4.w};
    const float zl = row[zo];
    const float end = o == 1 ? c[3] : c[0];
    const float outside = zmode == 0 ? zl : (zmode == 1 ? end : -end);
    float zm[4], zp[4];
    if (o == 1) {
        zm[0] = a4.x; zm[1] = a4.y; zm[2] = a4.z; zm[3] = a4.w;
        zp[0] = a4.y; zp[1] = a4.z; zp[2] = a4.w; zp[3] = outside;
    } else {
        zm[0] = outside; zm[1] = a4.x; zm[2] = a4.y; zm[3] = a4.z;
        zp[0] = a4.x; zp[1] = a4.y; zp[2] = a4.z; zp[3] = a4.w;
    }
    float u[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        float sm = cmx * xm[q];
        sm = fmat(cpx, xp[q], sm);
        sm = fmat(cmy, ym[q], sm);
        sm = fmat(cpy, yp[q], sm);
        sm = fmat(zc[0][q], zm[q], sm);
        sm = fmat(zc[1][q], zp[q], sm);
        sm = sm - f[q];
        float d = dx + zc[2][q];
        d += dy;
        u[q] = W1 ? sweep_div(sm, d + d) : fmat(omc, c[q], sweep_div(w * sm, d + d));
    }
    *reinterpret_cast<float4 *>(row + own + m) = make_float4(u[0], u[1], u[2], u[3]);
}

// esrc / esrc2: source e with boxes of tj rows and of two rows; edst:
// destination e, tj rows; rld / rld1: r with tj rows and one row.
template <bool RS, bool W1>
__global__ void __launch_bounds__(fu_threads<RS>(), 1)
    k_rbgs_fused(const __grid_constant__ CUtensorMap esrc, const __grid_constant__ CUtensorMap esrc2,
                 const __grid_constant__ CUtensorMap edst, const __grid_constant__ CUtensorMap rld,
                 const __grid_constant__ CUtensorMap rld1, Lay L, Tab3<float> t, Bnd b, float w, float omc, int tj,
                 int chunk, int *err, unsigned wlim, int split) {
    constexpr int NT = fu_nt<RS>();
    pdl_enter();
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int s_fail;
    const int n0 = L.n0, n1 = L.n1, n2 = L.n2;
    const int e_slot = (tj + 4) * n2, r_slot = (tj + 2) * n2;
    uint64_t *efull = reinterpret_cast<uint64_t *>(smem), *eempty = efull + FU_ESLOTS;
    uint64_t *rfull = eempty + FU_ESLOTS, *rempty = rfull + FU_RSLOTS;
    float *sy = reinterpret_cast<float *>(smem + 256);   // cm, cp, dg of y for rows j0-1 .. j0+tj
    float *sx = reinterpret_cast<float *>(smem + 1024);  // cm, cp, dg of x for planes i0-1 .. i1
    float *es = reinterpret_cast<float *>(smem + fu_head(chunk));
    float *rs = es + FU_ESLOTS * e_slot;
    const int j0 = (int)blockIdx.x * tj;
    const int i0 = (int)blockIdx.y * chunk;
    const int i1 = min(n0, i0 + chunk);
    if (i0 >= i1) return;
    if (threadIdx.x == 0) {
        for (int q = 0; q < FU_ESLOTS; q++) {
            mbar_init(&efull[q], 1);
            mbar_init(&eempty[q], 1);
        }
        for (int q = 0; q < FU_RSLOTS; q++) {
            mbar_init(&rfull[q], 1);
            mbar_init(&rempty[q], 1);
        }
        mbar_init_fence();
        s_fail = 0;
    }
    __syncthreads();
    // e planes i0-2 .. i1+1 and r planes i0-1 .. i1; plane p of e sits in
    // slot (p - P0) % FU_ESLOTS, of r in (p - Q0) % FU_RSLOTS.  Periodic
    // axes wrap the plane and halo-row coordinates; at walls the halo rows
    // and planes are the ghost layer or out of range (TMA fills zeros) and
    // are never read.
    const int P0 = i0 - 2, Q0 = i0 - 1;
    auto pco = [&](int p) { return (b.per[0] ? wrap(p, n0) : p) + 1; };
    auto rco = [&](int j) { return (b.per[1] ? wrap(j, n1) : j) + 1; };
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        // ---- producer ----
        if (lane == 0) {
            const uint32_t eb = (uint32_t)(e_slot * sizeof(float)), rb = (uint32_t)(r_slot * sizeof(float));
            int ne = 0, nr = 0;
            bool fail = false;
            for (int P = P0; P <= i1 + 1 && !fail; P++) {
                const int u = P - P0, s = u % FU_ESLOTS;
                if (u >= FU_ESLOTS && !mbar_wait(&eempty[s], (uint32_t)((u / FU_ESLOTS - 1) & 1), wlim)) {
                    fail = true;
                    break;
                }
                mbar_expect_tx(&efull[s], eb);
                float *d = es + s * e_slot;
                tma_rows(d, &esrc2, &efull[s], split, rco(j0 - 2), pco(P));
                tma_rows(d + 2 * n2, &esrc, &efull[s], split, j0 + 1, pco(P));
                tma_rows(d + (tj + 2) * n2, &esrc2, &efull[s], split, rco(j0 + tj), pco(P));
                ne++;
                const int Q = P - 1;
                if (Q < Q0 || Q > i1) continue;
                const int v = Q - Q0, sr = v % FU_RSLOTS;
                if (v >= FU_RSLOTS && !mbar_wait(&rempty[sr], (uint32_t)((v / FU_RSLOTS - 1) & 1), wlim)) {
                    fail = true;
                    break;
                }
                mbar_expect_tx(&rfull[sr], rb);
                float *d2 = rs + sr * r_slot;
                tma_rows(d2, &rld1, &rfull[sr], split, rco(j0 - 1), pco(Q));
                tma_rows(d2 + n2, &rld, &rfull[sr], split, j0 + 1, pco(Q));
                tma_rows(d2 + (tj + 1) * n2, &rld1, &rfull[sr], split, rco(j0 + tj), pco(Q));
                nr++;
            }
            if (fail) {
                s_fail = 1;
                atomicExch(err, 1);
            }
            // nothing may be in flight when the block exits: wait (bounded)
            // for the last planes issued to land
            for (int x = max(0, ne - FU_ESLOTS); x < ne; x++)
                mbar_wait(&efull[x % FU_ESLOTS], (uint32_t)((x / FU_ESLOTS) & 1));
            for (int x = max(0, nr - FU_RSLOTS); x < nr; x++)
                mbar_wait(&rfull[x % FU_RSLOTS], (uint32_t)((x / FU_RSLOTS) & 1));
        }
        return;
    }
    // ---- consumers ----
    // Thread ct owns the 4-cell strip at k0 of every rstep-th row it visits:
    // its z coefficients and z-wall handling stay in registers.
    const int ct = threadIdx.x - 32;
    // strips of four cells: of the row (both colours), or with RS of one
    // row half (one colour); a thread keeps its strip's z coefficients (for
    // RS those of both colour offsets o)
    const int H = n2 >> 1;
    const int s4 = RS ? (H >> 2) : (n2 >> 2);
    const int k0 = (ct % s4) * 4, ro = ct / s4, rstep = NT / s4;
    float zc[2][3][4];
#pragma unroll
    for (int oo = 0; oo < (RS ? 2 : 1); oo++)
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const int k = RS ? 2 * (k0 + c) + oo : k0 + c;
            zc[oo][0][c] = t.cm[2][k];
            zc[oo][1][c] = t.cp[2][k];
            zc[oo][2][c] = t.dg[2][k];
        }
    const int ny = tj + 2;
    for (int x = ct; x < ny; x += NT) {
        const int j = j0 - 1 + x;
        const int jw = b.per[1] ? wrap(j, n1) : min(max(j, 0), n1 - 1);
        sy[x] = t.cm[1][jw];
        sy[ny + x] = t.cp[1][jw];
        sy[2 * ny + x] = t.dg[1][jw];
    }
    // the x coefficients of every plane the chunk's steps visit, so that no
    // step waits on a global load after its ring wait
    const int nx = i1 - i0 + 2;
    for (int x = ct; x < nx; x += NT) {
        const int q = i0 - 1 + x;
        const int qw = b.per[0] ? wrap(q, n0) : min(max(q, 0), n0 - 1);
        sx[x] = t.cm[0][qw];
        sx[nx + x] = t.cp[0][qw];
        sx[2 * nx + x] = t.dg[0][qw];
    }
    consumer_sync<NT>();
    auto eptr = [&](int p) { return es + ((p - P0) % FU_ESLOTS) * e_slot; };
    auto rptr = [&](int p) { return rs + ((p - Q0) % FU_RSLOTS) * r_slot; };
    auto wait_e = [&](int p) {
        const int u = p - P0;
        if (!s_fail && !mbar_wait(&efull[u % FU_ESLOTS], (uint32_t)((u / FU_ESLOTS) & 1), wlim)) {
            s_fail = 1;
            atomicExch(err, 1);
        }
    };
    auto wait_r = [&](int p) {
        const int u = p - Q0;
        if (!s_fail && !mbar_wait(&rfull[u % FU_RSLOTS], (uint32_t)((u / FU_RSLOTS) & 1), wlim)) {
            s_fail = 1;
            atomicExch(err, 1);
        }
    };
    // the TMA store of plane q-2 and the slot releases, once the consumers
    // have met after R(q)
    auto store_release = [&](int q) {
        if (ct == 0 && !s_fail) {
            if (q - 2 >= i0) {
                tma_rows_store(&edst, eptr(q - 2) + 2 * n2, split, j0 + 1, q - 1);
                bulk_commit();
            }
            if (q - 3 >= P0) {
                if (q - 3 >= i0) bulk_wait_read1();  // the store of plane q-3 has read its slot
                mbar_arrive(&eempty[(q - 3 - P0) % FU_ESLOTS]);
            }
            if (q - 2 >= Q0) mbar_arrive(&rempty[(q - 2 - Q0) % FU_RSLOTS]);
        }
    };
    const bool px = b.per[0] != 0, py = b.per[1] != 0;
    wait_e(P0);
    wait_e(P0 + 1);
    if constexpr (RS) {
        // Row-split layout: every thread visits at most two rows of R (tile
        // rows and the halo row each side) and two of K per plane, the same
        // rows on every plane, so their offsets, wall flags, y coefficients
        // and row parities are formed once; so are the strip's z neighbours
        // outside it (zo: for R, whose own half is the red one, and for K).
        // Slot indices advance by one per plane instead of being recomputed.
        int r_off[2], r_jp[2];
        bool r_ok[2], r_lo[2], r_hi[2];
        float r_cm[2], r_cp[2], r_dg[2];
        int k_off[2], k_jp[2];
        bool k_ok[2], k_lo[2], k_hi[2];
        float k_cm[2], k_cp[2], k_dg[2];
#pragma unroll
        for (int v = 0; v < 2; v++) {
            const int x = ro + v * rstep;
            const int j = j0 - 1 + x;
            r_ok[v] = x < ny && (py || (j >= 0 && j < n1));
            const int jw = r_ok[v] ? (py ? wrap(j, n1) : j) : 0;
            const int xs = r_ok[v] ? x : 0;
            r_off[v] = xs;
            r_jp[v] = jw & 1;
            r_lo[v] = !py && jw == 0;
            r_hi[v] = !py && jw == n1 - 1;
            r_cm[v] = sy[xs];
            r_cp[v] = sy[ny + xs];
            r_dg[v] = sy[2 * ny + xs];
            const int xk = ro + v * rstep;
            k_ok[v] = xk < tj;
            const int xks = k_ok[v] ? xk : 0;
            const int jk = j0 + xks;
            k_off[v] = xks;
            k_jp[v] = jk & 1;
            k_lo[v] = !py && jk == 0;
            k_hi[v] = !py && jk == n1 - 1;
            k_cm[v] = sy[xks + 1];
            k_cp[v] = sy[ny + xks + 1];
            k_dg[v] = sy[2 * ny + xks + 1];
        }
        // z neighbours outside the strip: o = 0 the left one, o = 1 the right
        // one, in the other half (R: own 0, other H; K: own H, other 0)
        const int zmode0 = k0 > 0 || b.per[2] ? 0 : (b.sg_lo[2] > 0 ? 1 : 2);
        const int zmode1 = k0 + 4 < H || b.per[2] ? 0 : (b.sg_hi[2] > 0 ? 1 : 2);
        const int zl_oth = k0 > 0 ? k0 - 1 : H - 1, zr_oth = k0 + 4 < H ? k0 + 4 : 0;
        const int zoR0 = zmode0 == 0 ? H + zl_oth : k0, zoR1 = zmode1 == 0 ? H + zr_oth : k0;
        const int zoK0 = zmode0 == 0 ? zl_oth : H + k0, zoK1 = zmode1 == 0 ? zr_oth : H + k0;
        int se = (i0 - 1 - P0) % FU_ESLOTS;  // slot of e plane q
        int sr = 0;                          // slot of r plane q (q - Q0 = 0 at the start)
        for (int q = i0 - 1; q <= i1; q++) {
            wait_e(q + 1);
            wait_r(q);
            const int sm1 = se == 0 ? FU_ESLOTS - 1 : se - 1, sp1 = se == FU_ESLOTS - 1 ? 0 : se + 1;
            const int sm2 = sm1 == 0 ? FU_ESLOTS - 1 : sm1 - 1, srm1 = sr == 0 ? FU_RSLOTS - 1 : sr - 1;
            if (px || (q >= 0 && q < n0)) {
                // R(q): the red half of the tile rows and the halo rows
                const int qi = px ? wrap(q, n0) : q;
                float *pc = es + se * e_slot;
                const float *pm = es + sm1 * e_slot, *pp = es + sp1 * e_slot, *rr = rs + sr * r_slot;
                const int xq = q - (i0 - 1);
                const float cmx = sx[xq], cpx = sx[nx + xq], dx = sx[2 * nx + xq];
                const bool xlo = !px && qi == 0, xhi = !px && qi == n0 - 1;
#pragma unroll
                for (int v = 0; v < 2; v++) {
                    if (!r_ok[v]) continue;
                    const int off = (r_off[v] + 1) * n2;
                    const float *rrow = rr + r_off[v] * n2;
                    if (((qi + r_jp[v]) & 1) == 0)
                        fu_strip_rs<0, W1>(pc + off, pm + off, pp + off, rrow, n2, 0, H, k0, zoR0, zmode0, xlo, xhi,
                                           r_lo[v], r_hi[v], b, cmx, cpx, dx, r_cm[v], r_cp[v], r_dg[v], zc[0], w,
                                           omc);
                    else
                        fu_strip_rs<1, W1>(pc + off, pm + off, pp + off, rrow, n2, 0, H, k0, zoR1, zmode1, xlo, xhi,
                                           r_lo[v], r_hi[v], b, cmx, cpx, dx, r_cm[v], r_cp[v], r_dg[v], zc[1], w,
                                           omc);
                }
            }
            // this thread's writes (R(q), K(q-2)) before the async proxy reads them
            fence_async_smem();
            consumer_sync<NT>();
            store_release(q);
            const int p = q - 1;
            if (p >= i0) {
                // K(p): the black half of the tile rows
                float *pc = es + sm1 * e_slot;
                const float *pm = es + sm2 * e_slot, *pp = es + se * e_slot, *rr = rs + srm1 * r_slot;
                const int xp_ = p - (i0 - 1);
                const float cmx = sx[xp_], cpx = sx[nx + xp_], dx = sx[2 * nx + xp_];
                const bool xlo = !px && p == 0, xhi = !px && p == n0 - 1;
#pragma unroll
                for (int v = 0; v < 2; v++) {
                    if (!k_ok[v]) continue;
                    const int off = (k_off[v] + 2) * n2;
                    const float *rrow = rr + (k_off[v] + 1) * n2;
                    if (((p + k_jp[v]) & 1) == 1)
                        fu_strip_rs<0, W1>(pc + off, pm + off, pp + off, rrow, n2, H, 0, k0, zoK0, zmode0, xlo, xhi,
                                           k_lo[v], k_hi[v], b, cmx, cpx, dx, k_cm[v], k_cp[v], k_dg[v], zc[0], w,
                                           omc);
                    else
                        fu_strip_rs<1, W1>(pc + off, pm + off, pp + off, rrow, n2, H, 0, k0, zoK1, zmode1, xlo, xhi,
                                           k_lo[v], k_hi[v], b, cmx, cpx, dx, k_cm[v], k_cp[v], k_dg[v], zc[1], w,
                                           omc);
                }
            }
            se = sp1;
            sr = sr == FU_RSLOTS - 1 ? 0 : sr + 1;
        }
    } else {
        const int li = k0 > 0 ? k0 - 1 : (b.per[2] ? n2 - 1 : k0);
        const bool lneg = k0 == 0 && !b.per[2] && b.sg_lo[2] < 0;
        const int ri = k0 + 4 < n2 ? k0 + 4 : (b.per[2] ? 0 : k0 + 3);
        const bool rneg = k0 + 4 >= n2 && !b.per[2] && b.sg_hi[2] < 0;
        // A thread visits the same rows on every plane (at most FU_PROWS of
        // each colour phase), so their offsets, wall flags, y coefficients
        // and row parities are formed once, and the ring slots advance by
        // one per plane.
        constexpr int FU_PROWS = 3;
        int r_off[FU_PROWS], r_jp[FU_PROWS];
        bool r_ok[FU_PROWS], r_lo[FU_PROWS], r_hi[FU_PROWS];
        float r_cm[FU_PROWS], r_cp[FU_PROWS], r_dg[FU_PROWS];
        int k_off[FU_PROWS], k_jp[FU_PROWS];
        bool k_ok[FU_PROWS], k_lo[FU_PROWS], k_hi[FU_PROWS];
        float k_cm[FU_PROWS], k_cp[FU_PROWS], k_dg[FU_PROWS];
#pragma unroll
        for (int v = 0; v < FU_PROWS; v++) {
            const int x = ro + v * rstep;
            const int j = j0 - 1 + x;
            r_ok[v] = x < ny && (py || (j >= 0 && j < n1));
            const int jw = r_ok[v] ? (py ? wrap(j, n1) : j) : 0;
            const int xs = r_ok[v] ? x : 0;
            r_off[v] = xs;
            r_jp[v] = jw & 1;
            r_lo[v] = !py && jw == 0;
            r_hi[v] = !py && jw == n1 - 1;
            r_cm[v] = sy[xs];
            r_cp[v] = sy[ny + xs];
            r_dg[v] = sy[2 * ny + xs];
            k_ok[v] = x < tj;
            const int xk = k_ok[v] ? x : 0;
            const int jk = j0 + xk;
            k_off[v] = xk;
            k_jp[v] = jk & 1;
            k_lo[v] = !py && jk == 0;
            k_hi[v] = !py && jk == n1 - 1;
            k_cm[v] = sy[xk + 1];
            k_cp[v] = sy[ny + xk + 1];
            k_dg[v] = sy[2 * ny + xk + 1];
        }
        int se = (i0 - 1 - P0) % FU_ESLOTS;  // slot of e plane q
        int sr = 0;                          // slot of r plane q
        int qi = px ? wrap(i0 - 1, n0) : i0 - 1;  // plane q in the level
        // every consumer thread runs every step and barrier, failed or not
        for (int q = i0 - 1; q <= i1; q++) {
            wait_e(q + 1);
            wait_r(q);
            const int sm1 = se == 0 ? FU_ESLOTS - 1 : se - 1, sp1 = se == FU_ESLOTS - 1 ? 0 : se + 1;
            const int sm2 = sm1 == 0 ? FU_ESLOTS - 1 : sm1 - 1, srm1 = sr == 0 ? FU_RSLOTS - 1 : sr - 1;
            if (px || (q >= 0 && q < n0)) {
                // R(q): the first colour on the tile rows and the halo rows
                float *pc = es + se * e_slot;
                const float *pm = es + sm1 * e_slot, *pp = es + sp1 * e_slot, *rr = rs + sr * r_slot;
                const int xq = q - (i0 - 1);
                const float cmx = sx[xq], cpx = sx[nx + xq], dx = sx[2 * nx + xq];
                const bool xlo = !px && qi == 0, xhi = !px && qi == n0 - 1;
#pragma unroll
                for (int v = 0; v < FU_PROWS; v++) {
                    if (!r_ok[v]) continue;
                    const int off = (r_off[v] + 1) * n2;
                    const float *rrow = rr + r_off[v] * n2;
                    if (((qi + r_jp[v]) & 1) == 0)
                        fu_strip<0, W1>(pc + off, pm + off, pp + off, rrow, n2, k0, xlo, xhi, r_lo[v], r_hi[v], b,
                                        li, ri, lneg, rneg, cmx, cpx, dx, r_cm[v], r_cp[v], r_dg[v], zc[0], w, omc);
                    else
                        fu_strip<1, W1>(pc + off, pm + off, pp + off, rrow, n2, k0, xlo, xhi, r_lo[v], r_hi[v], b,
                                        li, ri, lneg, rneg, cmx, cpx, dx, r_cm[v], r_cp[v], r_dg[v], zc[0], w, omc);
                }
            }
            // this thread's writes (R(q), K(q-2)) before the async proxy reads them
            fence_async_smem();
            consumer_sync<NT>();
            store_release(q);
            const int p = q - 1;
            if (p >= i0) {
                // K(p): the second colour on the tile rows
                float *pc = es + sm1 * e_slot;
                const float *pm = es + sm2 * e_slot, *pp = es + se * e_slot, *rr = rs + srm1 * r_slot;
                const int xp_ = p - (i0 - 1);
                const float cmx = sx[xp_], cpx = sx[nx + xp_], dx = sx[2 * nx + xp_];
                const bool xlo = !px && p == 0, xhi = !px && p == n0 - 1;
#pragma unroll
                for (int v = 0; v < FU_PROWS; v++) {
                    if (!k_ok[v]) continue;
                    const int off = (k_off[v] + 2) * n2;
                    const float *rrow = rr + (k_off[v] + 1) * n2;
                    if (((1 + p + k_jp[v]) & 1) == 0)
                        fu_strip<0, W1>(pc + off, pm + off, pp + off, rrow, n2, k0, xlo, xhi, k_lo[v], k_hi[v], b,
                                        li, ri, lneg, rneg, cmx, cpx, dx, k_cm[v], k_cp[v], k_dg[v], zc[0], w, omc);
                    else
                        fu_strip<1, W1>(pc + off, pm + off, pp + off, rrow, n2, k0, xlo, xhi, k_lo[v], k_hi[v], b,
                                        li, ri, lneg, rneg, cmx, cpx, dx, k_cm[v], k_cp[v], k_dg[v], zc[0], w, omc);
                }
            }
            se = sp1;
            sr = sr == FU_RSLOTS - 1 ? 0 : sr + 1;
            qi = px ? (qi == n0 - 1 ? 0 : qi + 1) : qi + 1;
        }
    }
    fence_async_smem();
    consumer_sync<NT>();
    if (ct == 0) {
        if (!s_fail) {
            tma_rows_store(&edst, eptr(i1 - 1) + 2 * n2, split, j0 + 1, i1);
            bulk_commit();
        }
        bulk_wait_all();
    }
}

// ---- residual and restriction through the same kind of pipeline ----
//
// k_resid_restrict4's work on the large 3-D levels of the MIXED form, with
// the fine planes streamed through shared memory.  A block owns a tile of tj
// fine rows (tj/2 coarse rows) by the whole row and an even chunk of fine
// planes.  A producer lane loads e planes (the tile and one halo row on each
// side) and r planes (the tile) into rings of slots.  Each consumer thread
// owns two coarse cells of one coarse row: on fine plane p it forms the
// residuals of their eight children in that plane (two fine rows of four
// cells, resid_row4's arithmetic on the slots) and their weighted sums over
// k and j (restrict2's), and on the odd plane it combines the two planes'
// sums and stores the coarse cells.  Each consumer warp releases a plane's
// slots once its step no longer reads them; warps never wait for one
// another.  The same bits as k_resid_restrict4, the row-split layout
// included (a fine row of parity pr holds the cells of colour pr first).
constexpr int RR_ESLOTS = 5, RR_RSLOTS = 4;
constexpr int RR_WARPS = 8;
constexpr int RR_THREADS = 32 * (RR_WARPS + 1);
constexpr int RR_TILE = 2048;  // fine cells of a tile plane: tj = RR_TILE / n_z rows, 2 coarse cells a thread
constexpr int RR_SX_MAX = 64;  // fine planes of a chunk at most (their x coefficients are staged)
constexpr int64_t RR_MIN_CELLS = int64_t(1) << 20;
// head of the dynamic shared memory: mbarriers, then the chunk's x
// coefficients (from byte 256) and the coarse planes' x weights
constexpr size_t RR_HEAD = 2048;

template <bool RS>
__global__ void __launch_bounds__(RR_THREADS, 2) k_resid_restrict_tma(
    const __grid_constant__ CUtensorMap eld, const __grid_constant__ CUtensorMap eld1,
    const __grid_constant__ CUtensorMap rld, Lay Lf, Tab3<float> t, Bnd b, WTab<float> w, float *__restrict__ rc,
    Lay Lc, float *__restrict__ ezero, int tj, int chunk, int *err, unsigned wlim, int split) {
    pdl_enter();
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int s_fail;
    const int n0 = Lf.n0, n1 = Lf.n1, n2 = Lf.n2;
    const int e_slot = (tj + 2) * n2, r_slot = tj * n2;
    uint64_t *efull = reinterpret_cast<uint64_t *>(smem), *eempty = efull + RR_ESLOTS;
    uint64_t *rfull = eempty + RR_ESLOTS, *rempty = rfull + RR_RSLOTS;
    float *sx = reinterpret_cast<float *>(smem + 256);  // cm, cp, dg of x for planes i0 .. i1-1
    float *sw = sx + 3 * RR_SX_MAX;                     // w0, w1 of x for coarse planes i0/2 ..
    float *es = reinterpret_cast<float *>(smem + RR_HEAD);
    float *rs = es + RR_ESLOTS * e_slot;
    const int j0 = (int)blockIdx.x * tj;
    const int i0 = (int)blockIdx.y * chunk;  // even
    const int i1 = min(n0, i0 + chunk);
    if (i0 >= i1) return;
    if (threadIdx.x == 0) {
        for (int q = 0; q < RR_ESLOTS; q++) {
            mbar_init(&efull[q], 1);
            mbar_init(&eempty[q], RR_WARPS);
        }
        for (int q = 0; q < RR_RSLOTS; q++) {
            mbar_init(&rfull[q], 1);
            mbar_init(&rempty[q], RR_WARPS);
        }
        mbar_init_fence();
        s_fail = 0;
    }
    // the chunk's x coefficients and weights
    const int nx = i1 - i0;
    for (int x = threadIdx.x; x < nx; x += blockDim.x) {
        sx[x] = t.cm[0][i0 + x];
        sx[RR_SX_MAX + x] = t.cp[0][i0 + x];
        sx[2 * RR_SX_MAX + x] = t.dg[0][i0 + x];
        if ((x & 1) == 0) {
            sw[x >> 1] = w.w0[0][(i0 + x) >> 1];
            sw[RR_SX_MAX / 2 + (x >> 1)] = w.w1[0][(i0 + x) >> 1];
        }
    }
    __syncthreads();
    // e planes i0-1 .. i1 (plane P in slot (P - P0) % RR_ESLOTS) and r planes
    // i0 .. i1-1 (plane Q in slot (Q - i0) % RR_RSLOTS); periodic axes wrap
    // the halo planes and rows, at walls they are the ghost layer and never
    // read (mirrors replace them)
    const int P0 = i0 - 1;
    auto pco = [&](int q) { return (b.per[0] ? wrap(q, n0) : q) + 1; };
    auto rco = [&](int j) { return (b.per[1] ? wrap(j, n1) : j) + 1; };
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        if (lane == 0) {
            const uint32_t eb = (uint32_t)(e_slot * sizeof(float)), rb = (uint32_t)(r_slot * sizeof(float));
            int ne = 0, nr = 0;
            bool fail = false;
            for (int P = P0; P <= i1 && !fail; P++) {
                const int u = P - P0, se = u % RR_ESLOTS;
                if (u >= RR_ESLOTS && !mbar_wait(&eempty[se], (uint32_t)((u / RR_ESLOTS - 1) & 1), wlim)) {
                    fail = true;
                    break;
                }
                mbar_expect_tx(&efull[se], eb);
                float *d = es + se * e_slot;
                tma_rows(d, &eld1, &efull[se], split, rco(j0 - 1), pco(P));
                tma_rows(d + n2, &eld, &efull[se], split, j0 + 1, pco(P));
                tma_rows(d + (tj + 1) * n2, &eld1, &efull[se], split, rco(j0 + tj), pco(P));
                ne++;
                const int Q = P - 1;  // r of plane Q goes with e of plane Q + 1
                if (Q < i0 || Q >= i1) continue;
                const int v = Q - i0, sr = v % RR_RSLOTS;
                if (v >= RR_RSLOTS && !mbar_wait(&rempty[sr], (uint32_t)((v / RR_RSLOTS - 1) & 1), wlim)) {
                    fail = true;
                    break;
                }
                mbar_expect_tx(&rfull[sr], rb);
                tma_rows(rs + sr * r_slot, &rld, &rfull[sr], split, j0 + 1, pco(Q));
                nr++;
            }
            if (fail) {
                s_fail = 1;
                atomicExch(err, 1);
            }
            // nothing may be in flight when the block exits
            for (int x = max(0, ne - RR_ESLOTS); x < ne; x++)
                mbar_wait(&efull[x % RR_ESLOTS], (uint32_t)((x / RR_ESLOTS) & 1));
            for (int x = max(0, nr - RR_RSLOTS); x < nr; x++)
                mbar_wait(&rfull[x % RR_RSLOTS], (uint32_t)((x / RR_RSLOTS) & 1));
        }
        return;
    }
    // ---- consumers: two coarse cells (kc0, kc0 + 1) of coarse row cj ----
    const int ct = threadIdx.x - 32;
    const int cpr = n2 >> 2;  // threads per coarse row
    const int cjl = ct / cpr, kc0 = 2 * (ct % cpr), k0 = 2 * kc0;
    const int jc = (j0 >> 1) + cjl;
    const bool px = b.per[0] != 0, py = b.per[1] != 0;
    const int H = n2 >> 1, h2 = k0 >> 1;
    // per fine row bb: local row, wall flags, y coefficients, parity offset
    int jl[2];
    bool ylo[2], yhi[2];
    float cmy[2], cpy[2], dgy[2];
#pragma unroll
    for (int bb = 0; bb < 2; bb++) {
        jl[bb] = 2 * cjl + bb;
        const int j = j0 + jl[bb];
        ylo[bb] = !py && j == 0;
        yhi[bb] = !py && j == n1 - 1;
        cmy[bb] = t.cm[1][j];
        cpy[bb] = t.cp[1][j];
        dgy[bb] = t.dg[1][j];
    }
    float cmz[4], cpz[4], dgz[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        cmz[q] = t.cm[2][k0 + q];
        cpz[q] = t.cp[2][k0 + q];
        dgz[q] = t.dg[2][k0 + q];
    }
    const float w0z[2] = {w.w0[2][kc0], w.w0[2][kc0 + 1]}, w1z[2] = {w.w1[2][kc0], w.w1[2][kc0 + 1]};
    const float w0y = w.w0[1][jc], w1y = w.w1[1][jc];
    // ring positions, advanced by one per plane: the slot and fill parity
    // of the e plane the step reads as its centre and of the r plane
    int se = 1, ne_ph = 0;  // e(i0) is fill 1 of slot 1 (e(i0-1) fill 0 of slot 0)
    int sr = 0, nr_ph = 0;  // r(i0) is fill 0 of slot 0
    auto wait_slot = [&](uint64_t *bar, int phase) {
        if (!s_fail && !mbar_wait(bar, (uint32_t)(phase & 1), wlim)) {
            s_fail = 1;
            atomicExch(err, 1);
        }
    };
    // four cells k0 .. k0+3 of a row of parity PAR (RS: its two halves)
    auto ld = [&](const float *row, auto par_c, float (&o)[4]) {
        if constexpr (!RS) {
            const float4 v = lds4(row + k0);
            o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
        } else {
            const float2 a = *reinterpret_cast<const float2 *>(row + h2);
            const float2 c = *reinterpret_cast<const float2 *>(row + H + h2);
            if constexpr (decltype(par_c)::value == 0) {
                o[0] = a.x; o[1] = c.x; o[2] = a.y; o[3] = c.y;
            } else {
                o[0] = c.x; o[1] = a.x; o[2] = c.y; o[3] = a.y;
            }
        }
    };
    // e(i0 - 1) and e(i0) before the first step
    wait_slot(&efull[0], 0);
    wait_slot(&efull[1], 0);
    float sy0[2] = {0.f, 0.f};
    // One fine plane p of parity A (the child index along x of its coarse
    // plane): the residuals of the eight children in it, their weighted sums
    // over k and j, and on A = 1 the coarse cells.  Fine row j of the tile has
    // the parity of bb (j0 is even), so the row's colour parity is A ^ bb.
    auto step = [&](int p, auto a_c) {
        constexpr int A = decltype(a_c)::value;
        const int sp = se == RR_ESLOTS - 1 ? 0 : se + 1, sm1 = se == 0 ? RR_ESLOTS - 1 : se - 1;
        // e(p+1) is the fill after the centre's: the next slot, the same
        // phase unless the ring wrapped
        wait_slot(&efull[sp], sp == 0 ? ne_ph + 1 : ne_ph);
        wait_slot(&rfull[sr], nr_ph);
        const float *pc = es + se * e_slot, *pm = es + sm1 * e_slot, *pp = es + sp * e_slot;
        const float *rr = rs + sr * r_slot;
        const int xq = p - i0;
        const float cmx = sx[xq], cpx = sx[RR_SX_MAX + xq], dgx = sx[2 * RR_SX_MAX + xq];
        const bool xlo = !px && p == 0, xhi = !px && p == n0 - 1;
        float sz[2][2];
        auto row_sums = [&](auto bb_c) {
            constexpr int BB = decltype(bb_c)::value;
            constexpr int PR = A ^ BB;
            const std::integral_constant<int, PR> own{};
            const std::integral_constant<int, 1 - PR> oth{};
            const int off = (jl[BB] + 1) * n2;
            const float *row = pc + off;
            float cur[4], xm[4], xp[4], ym[4], yp[4], fr[4];
            ld(row, own, cur);
            if (xlo) {
#pragma unroll
                for (int q = 0; q < 4; q++) xm[q] = b.sg_lo[0] > 0 ? cur[q] : -cur[q];
            } else {
                ld(pm + off, oth, xm);
            }
            if (xhi) {
#pragma unroll
                for (int q = 0; q < 4; q++) xp[q] = b.sg_hi[0] > 0 ? cur[q] : -cur[q];
            } else {
                ld(pp + off, oth, xp);
            }
            if (ylo[BB]) {
#pragma unroll
                for (int q = 0; q < 4; q++) ym[q] = b.sg_lo[1] > 0 ? cur[q] : -cur[q];
            } else {
                ld(row - n2, oth, ym);
            }
            if (yhi[BB]) {
#pragma unroll
                for (int q = 0; q < 4; q++) yp[q] = b.sg_hi[1] > 0 ? cur[q] : -cur[q];
            } else {
                ld(row + n2, oth, yp);
            }
            ld(rr + jl[BB] * n2, own, fr);
            // position of cell k of this row
            auto at_k = [&](int k) { return RS ? (k >> 1) + ((PR + k) & 1) * H : k; };
            const float left =
                k0 > 0 ? row[at_k(k0 - 1)] : (b.per[2] ? row[at_k(n2 - 1)] : (b.sg_lo[2] > 0 ? cur[0] : -cur[0]));
            const float right = k0 + 4 < n2 ? row[at_k(k0 + 4)]
                                            : (b.per[2] ? row[at_k(0)] : (b.sg_hi[2] > 0 ? cur[3] : -cur[3]));
            float r[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float zm = q > 0 ? cur[q - 1] : left;
                const float zp = q < 3 ? cur[q + 1] : right;
                float sm = cmx * xm[q];
                sm = fmat(cpx, xp[q], sm);
                sm = fmat(cmy[BB], ym[q], sm);
                sm = fmat(cpy[BB], yp[q], sm);
                sm = fmat(cmz[q], zm, sm);
                sm = fmat(cpz[q], zp, sm);
                float d = dgx + dgz[q];
                d += dgy[BB];
                d = d + d;
                r[q] = fr[q] - fmat(-d, cur[q], sm);
            }
#pragma unroll
            for (int q = 0; q < 2; q++) sz[BB][q] = fmat(w1z[q], r[2 * q + 1], w0z[q] * r[2 * q]);
        };
        row_sums(std::integral_constant<int, 0>{});
        row_sums(std::integral_constant<int, 1>{});
        // this warp no longer reads e(p-1) and r(p)
        __syncwarp();
        if (lane == 0) {
            mbar_arrive(&eempty[sm1]);
            mbar_arrive(&rempty[sr]);
        }
        se = sp;
        if (sp == 0) ne_ph++;
        sr = sr == RR_RSLOTS - 1 ? 0 : sr + 1;
        if (sr == 0) nr_ph++;
        float sy[2];
#pragma unroll
        for (int q = 0; q < 2; q++) sy[q] = fmat(w1y, sz[1][q], w0y * sz[0][q]);
        if constexpr (A == 0) {
            sy0[0] = sy[0];
            sy0[1] = sy[1];
        } else {
            if (!s_fail) {
                const int ic = p >> 1;
                const float w0x = sw[xq >> 1], w1x = sw[RR_SX_MAX / 2 + (xq >> 1)];
                const int64_t q = Lc.at(ic, jc, kc0);
                *reinterpret_cast<float2 *>(rc + q) =
                    make_float2(fmat(w1x, sy[0], w0x * sy0[0]), fmat(w1x, sy[1], w0x * sy0[1]));
                if (ezero) *reinterpret_cast<float2 *>(ezero + q) = make_float2(0.f, 0.f);
            }
        }
    };
    // chunks are even and start on even planes
    for (int p = i0; p < i1; p += 2) {
        step(p, std::integral_constant<int, 0>{});
        step(p + 1, std::integral_constant<int, 1>{});
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

// Rows of `rows` of a level for tma_rows: encode3's map for rows of up to
// 256 cells; for rows of 512, a 4-D map of the core viewed as two halves of
// 256 cells (its base is the first core cell, 16-byte aligned: rows start
// their core at KOFF on a 32-byte boundary, and a half is 1 KB).
bool encode_rows(CUtensorMap *m, const float *base, const Lay &L, int rows) {
    if (L.n2 <= 256) return encode3(m, base, L, rows);
    if (L.n2 != 512) return false;
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dim[4] = {256, 2, (cuuint64_t)L.n1 + 2, (cuuint64_t)L.n0 + 2};
    const cuuint64_t stride[3] = {256 * sizeof(float), (cuuint64_t)L.s1 * sizeof(float),
                                  (cuuint64_t)L.s0 * sizeof(float)};
    const cuuint32_t box[4] = {256, 2, (cuuint32_t)rows, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float *>(base + KOFF), dim, stride, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

size_t tma_smem(int tj, int n2) {
    return (size_t)TMA_SLOTS * ((size_t)(tj + 2) * n2 + (size_t)tj * n2) * sizeof(float) + 2 * TMA_SLOTS * 8;
}

size_t fused_smem(int tj, int n2, int chunk) {
    return fu_head(chunk) + ((size_t)FU_ESLOTS * (tj + 4) + (size_t)FU_RSLOTS * (tj + 2)) * n2 * sizeof(float);
}

Tab3<float> sweep_tab(const Level &v) {
    return Tab3<float>{{v.cm32[0], v.cm32[1], v.cm32[2]}, {v.cp32[0], v.cp32[1], v.cp32[2]},
                       {v.dg32[0], v.dg32[1], v.dg32[2]}};
}

Bnd sweep_bnd(const saras_mg *h) {
    Bnd b;
    for (int d = 0; d < 3; d++) {
        b.per[d] = h->ghost.per[d];
        b.sg_lo[d] = h->ghost.kind[2 * d] == SARAS_BC_NEUMANN ? 1 : -1;
        b.sg_hi[d] = h->ghost.kind[2 * d + 1] == SARAS_BC_NEUMANN ? 1 : -1;
    }
    return b;
}

// The fused iteration's plan: tile rows, plane chunk (all blocks resident
// in one wave) and the six tensor maps.
void fused_plan(Level &v, int sms) {
    const Lay &L = v.lay;
    const int tj = fu_tile_rows(L.n2);
    TmaPlan &m = v.tma;
    if (!encode_rows(&m.fa, v.e32, L, tj) || !encode_rows(&m.fa2, v.e32, L, 2) || !encode_rows(&m.fb, v.e32b, L, tj) ||
        !encode_rows(&m.fb2, v.e32b, L, 2) || !encode_rows(&m.fr, v.r32, L, tj) || !encode_rows(&m.fr1, v.r32, L, 1))
        return;
    if (cudaFuncSetAttribute(k_rbgs_fused<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_rbgs_fused<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_rbgs_fused<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_rbgs_fused<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
            cudaSuccess) {
        cudaGetLastError();
        return;
    }
    // the block must fit an SM (registers and shared memory) or the level
    // keeps the colour sweeps; the occupancy is taken at the smallest head
    const size_t smem0 = fused_smem(tj, L.n2, 0);
    int per_sm = 0, per_sm_rs = 0;
    int per_sm_w1 = 0, per_sm_pw1 = 0;
    if (smem0 > 200 * 1024 ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rbgs_fused<false, false>, fu_threads<false>(),
                                                      smem0) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_pw1, k_rbgs_fused<false, true>, fu_threads<false>(),
                                                      smem0) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_rs, k_rbgs_fused<true, false>, fu_threads<true>(),
                                                      smem0) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_w1, k_rbgs_fused<true, true>, fu_threads<true>(),
                                                      smem0) != cudaSuccess ||
        per_sm_w1 < 1 || per_sm_pw1 < 1 || per_sm < 1 || per_sm_rs < 1) {
        cudaGetLastError();
        return;
    }
    per_sm = std::min(per_sm, per_sm_rs);
    // one wave: the chunks of every tile column fill the resident blocks
    const int nch = std::max(1, per_sm * sms / (L.n1 / tj));
    const int chunk = std::max(8, (L.n0 + nch - 1) / nch);
    // the chunk's x coefficients sit in the head: the ring must still fit
    if (fused_smem(tj, L.n2, chunk) > 200 * 1024) return;
    m.ftj = tj;
    m.fchunk = chunk;
    m.fok = 1;
}

size_t rr_smem(int tj, int n2) {
    return RR_HEAD + ((size_t)RR_ESLOTS * (tj + 2) + (size_t)RR_RSLOTS * tj) * n2 * sizeof(float);
}

// The TMA residual-restriction's plan for a fine level: tile rows, an even
// plane chunk (all blocks resident in one wave) and three tensor maps.
void rr_plan(Level &v, int sms) {
    const Lay &L = v.lay;
    const int tj = RR_TILE / L.n2;
    TmaPlan &m = v.tma;
    const size_t smem = rr_smem(tj, L.n2);
    if (smem > 200 * 1024 || !encode_rows(&m.rre, v.e32, L, tj) || !encode_rows(&m.rre1, v.e32, L, 1) ||
        !encode_rows(&m.rrr, v.r32, L, tj))
        return;
    // one attribute for every level and handle: the largest ring any plan may use
    if (cudaFuncSetAttribute(k_resid_restrict_tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_resid_restrict_tma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
            cudaSuccess) {
        cudaGetLastError();
        return;
    }
    int per_sm = 0, per_sm_rs = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_resid_restrict_tma<false>, RR_THREADS, smem) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_rs, k_resid_restrict_tma<true>, RR_THREADS, smem) !=
            cudaSuccess ||
        per_sm < 1 || per_sm_rs < 1) {
        cudaGetLastError();
        return;
    }
    per_sm = std::min(per_sm, per_sm_rs);
    const int nch = std::max(1, per_sm * sms / (L.n1 / tj));
    int chunk = (L.n0 + nch - 1) / nch;
    chunk = std::min(RR_SX_MAX, std::max(2, chunk + (chunk & 1)));
    m.rtj = tj;
    m.rchunk = chunk;
    m.rok = 1;
}

}  // namespace

// Levels that take the fused red-black iteration (and hold a second e
// buffer for it): 3-D, rows of 128, 256 or 512 cells, tiles of
// fu_tile_rows rows that divide the level's rows, at least FU_MIN_CELLS
// cells.
bool fused_sweep_fits(const Lay &L, bool d3) {
    // every consumer thread owns one strip of each row it visits: strips of
    // four cells of the row (plain layout)
    if (!d3 || (L.n2 != 512 && (L.n2 < 128 || L.n2 > 256 || FU_TILE % L.n2 != 0)) ||
        fu_nt<false>() % (L.n2 / 4) != 0)
        return false;
    const int tj = fu_tile_rows(L.n2);
    // the plain consumers visit at most three rows of each colour phase
    if (tj + 2 > 3 * (fu_nt<false>() / (L.n2 / 4))) return false;
    return L.n1 % tj == 0 && L.n0 >= 16 && (int64_t)L.n0 * L.n1 * L.n2 >= FU_MIN_CELLS;
}

// The row-split layout's fused iteration (strips of a row half): rows of up
// to 256 cells.
bool fused_rowsplit_fits(const Lay &L, bool d3) {
    if (!fused_sweep_fits(L, d3) || L.n2 > 256 || fu_nt<true>() % (L.n2 / 8) != 0) return false;
    // the row-split consumers visit at most two rows of each colour phase
    return fu_tile_rows(L.n2) + 2 <= 2 * (fu_nt<true>() / (L.n2 / 8));
}

// Levels that take the TMA residual-restriction: 3-D, at least
// RR_MIN_CELLS cells, rows of 128 or 256 cells, even extents, tiles of
// RR_TILE cells that divide the level's rows.
bool rr_fits(const Lay &L, bool d3) {
    if (!d3 || L.n2 < 128 || (L.n2 > 256 && L.n2 != 512) || RR_TILE % L.n2 != 0) return false;
    const int tj = RR_TILE / L.n2;
    // one consumer thread per pair of coarse cells of the tile's coarse rows
    if ((tj / 2) * (L.n2 / 4) != 32 * RR_WARPS) return false;
    return (tj & 1) == 0 && L.n1 % tj == 0 && (L.n0 & 1) == 0 && L.n0 >= 4 &&
           (int64_t)L.n0 * L.n1 * L.n2 >= RR_MIN_CELLS;
}

// Plans the TMA sweeps of one level: the fused iteration's (levels with a
// second e buffer) and the colour sweep's tile rows, plane chunk and three
// tensor maps (e with halo rows, e without, r).  Levels that do not qualify
// keep the vector sweep.
void tma_plan(saras_mg *h, Level &v) {
    v.tma.ok = 0;
    v.tma.fok = 0;
    const Lay &L = v.lay;
    if (!h->d3 || !v.e32 || !v.r32) return;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (v.e32b && fused_sweep_fits(L, h->d3)) fused_plan(v, sms);
    v.tma.rok = 0;
    if (rr_fits(L, h->d3)) rr_plan(v, sms);
    // rows of 32..256 cells (a power of two); tiles of 2048 cells shared by
    // the consumer warps row-wise
    if (L.n2 < 32 || L.n2 > 256 || 1024 % L.n2 != 0 || (int64_t)L.n0 * L.n1 * L.n2 < (1 << 20)) return;
    // tiles of exactly 2048 cells: two 4-cell strips per consumer lane
    const int tj = 2048 / L.n2;
    if (L.n1 % tj != 0 || tj % TMA_CONSUMERS != 0 || tj + 2 > 256) return;
    const size_t smem = tma_smem(tj, L.n2);
    if (smem > 200 * 1024) return;
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

// Polls of the pipeline waits: the handle's limit, or TMA_WAIT_LIMIT.
unsigned tma_wait_limit(const saras_mg *h) { return h->wait_limit > 0 ? h->wait_limit : TMA_WAIT_LIMIT; }

// One colour sweep through the TMA path; false when the level has none.
bool tma_colour(saras_mg *h, cudaStream_t s, Level &v, int colour) {
    if (!v.tma.ok) return false;
    const Lay &L = v.lay;
    const dim3 grid((unsigned)(L.n1 / v.tma.tj), (unsigned)((L.n0 + v.tma.chunk - 1) / v.tma.chunk));
    const Tab3<float> t = sweep_tab(v);
    const Bnd b = sweep_bnd(h);
    int *err = reinterpret_cast<int *>(h->norm_out + 7);
    launch_pdl(k_rbgs_tma, grid, dim3(TMA_WS_THREADS), tma_smem(v.tma.tj, L.n2), s, v.tma.eld, v.tma.est, v.tma.rld,
               (const float *)v.e32, L, t, b, colour, (float)h->prm.sor_param, (float)(1.0 - h->prm.sor_param),
               v.tma.tj, v.tma.chunk, err, tma_wait_limit(h));
    return true;
}

// One red-black iteration through the fused kernel, e32 -> e32b (to_b) or
// e32b -> e32; false when the level has no fused plan.
// The FP32 residual of fine level f restricted into coarse level c (not the
// coarsest) through the TMA pipeline, the coarse error cleared when z32 is
// given; false when the level has no plan.
bool tma_resid_restrict(saras_mg *h, cudaStream_t s, Level &f, Level &c, const Tab3<float> &t,
                        const WTab<float> &w, float *z32) {
    if (!f.tma.rok) return false;
    const Lay &L = f.lay;
    const TmaPlan &m = f.tma;
    const dim3 grid((unsigned)(L.n1 / m.rtj), (unsigned)((L.n0 + m.rchunk - 1) / m.rchunk));
    int *err = reinterpret_cast<int *>(h->norm_out + 7);
    launch_pdl(f.rs ? k_resid_restrict_tma<true> : k_resid_restrict_tma<false>, grid, dim3(RR_THREADS),
               rr_smem(m.rtj, L.n2), s, m.rre, m.rre1, m.rrr, L, t, sweep_bnd(h), w, c.r32, c.lay, z32, m.rtj,
               m.rchunk, err, tma_wait_limit(h), L.n2 > 256 ? 1 : 0);
    return true;
}

bool tma_fused(saras_mg *h, cudaStream_t s, Level &v, bool to_b) {
    if (!v.tma.fok) return false;
    const Lay &L = v.lay;
    const TmaPlan &m = v.tma;
    const dim3 grid((unsigned)(L.n1 / m.ftj), (unsigned)((L.n0 + m.fchunk - 1) / m.fchunk));
    int *err = reinterpret_cast<int *>(h->norm_out + 7);
    const dim3 block((unsigned)(v.rs ? fu_threads<true>() : fu_threads<false>()));
    // the kernels skip the SOR blend when the parameter is 1
    const bool w1 = h->prm.sor_param == 1.0;
    launch_pdl(v.rs ? (w1 ? k_rbgs_fused<true, true> : k_rbgs_fused<true, false>)
                    : (w1 ? k_rbgs_fused<false, true> : k_rbgs_fused<false, false>),
               grid,
               block, fused_smem(m.ftj, L.n2, m.fchunk), s,
               to_b ? m.fa : m.fb, to_b ? m.fa2 : m.fb2, to_b ? m.fb : m.fa, m.fr, m.fr1, L, sweep_tab(v), sweep_bnd(h),
               (float)h->prm.sor_param, (float)(1.0 - h->prm.sor_param), m.ftj, m.fchunk, err, tma_wait_limit(h),
               L.n2 > 256 ? 1 : 0);
    return true;
}

}  // namespace saras
