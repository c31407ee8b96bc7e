// Device-resident multigrid hierarchy behind the saras_mg_* entry points.
#pragma once

#include <cuda.h>

#include <vector>

#include "common.cuh"
#include "grid_host.h"
#include "mg_exact.cuh"

namespace saras {

// TMA plan of a level's FP32 colour sweep (mg_tma.cu): tensor maps of e
// (tile with one halo row each side, tile alone) and r, tile rows and planes
// per block.  The fused red-black iteration (fok) adds maps of e (tile rows,
// two halo rows) for both buffers of its ping-pong pair and of r (tile rows,
// one halo row), with its own tile rows and plane chunk.
struct TmaPlan {
    CUtensorMap eld, est, rld;
    int tj = 0, chunk = 0, ok = 0;
    CUtensorMap fa, fa2, fb, fb2, fr, fr1;
    int ftj = 0, fchunk = 0, fok = 0;
    CUtensorMap rre, rre1, rrr;  // the TMA residual-restriction's e (tile, one row) and r
    int rtj = 0, rchunk = 0, rok = 0;
};

// Per-level device state.  FP64 arrays serve the FP64_EXACT and FP64 forms
// and the finest level of the MIXED form; FP32 arrays hold the MIXED form's
// error hierarchy.
struct Level {
    Lay lay;
    double *lhs = nullptr, *rhs = nullptr, *tmp = nullptr, *smd = nullptr;
    float *e32 = nullptr, *r32 = nullptr;
    float *e32b = nullptr;  // second buffer of the fused red-black iteration's ping-pong
    double *tab = nullptr;  // all 1-D tables of the level in one allocation
    Coef coef{};
    RTab rt{};
    // FP64 form: folded stencil coefficients per axis, c_minus/c_plus
    // (xix2*ihx2 -/+ xixx*i2hx) and the diagonal half-sum d = xix2*ihx2.
    const double *cm[3] = {nullptr, nullptr, nullptr}, *cp[3] = {nullptr, nullptr, nullptr};
    const double *dg[3] = {nullptr, nullptr, nullptr};
    // restriction weights of the two children normalised by the parent
    // extent: w0 = r0/rt, w1 = r1/rt (so that v_abc/vTot = wx_a wy_b wz_c)
    const double *w0[3] = {nullptr, nullptr, nullptr}, *w1[3] = {nullptr, nullptr, nullptr};
    // FP32 copies of the folded tables for the MIXED form
    float *tab32 = nullptr;
    const float *cm32[3] = {nullptr, nullptr, nullptr}, *cp32[3] = {nullptr, nullptr, nullptr};
    const float *dg32[3] = {nullptr, nullptr, nullptr};
    const float *w032[3] = {nullptr, nullptr, nullptr}, *w132[3] = {nullptr, nullptr, nullptr};
    double *inv_diag = nullptr;  // FP64 form: omega / D per cell
    double *dd = nullptr;        // FP64 forms: the diagonal D = 2 sum(xix2*ihx2) per cell
    float *inv_diag32 = nullptr; // MIXED form: omega / D per cell
    double *fd = nullptr;        // MIXED form, coarsest level: V, V^-1, eigenvalues per axis
    FDiag fdv{};                 // their device view; fdv.ok = 0: red-black sweeps
    TmaPlan tma{};
    // MIXED form, finest level with the fused iteration and even smoothing
    // counts: e32, e32b and r32 are row-split, each row holding its red
    // cells, then its black cells (rs_at); the kernels that touch them
    // (fused sweep, FP64 residual, update, restriction from and
    // prolongation into the level) follow it
    int rs = 0;
};

// kernel classes timed with events (KC_H2D / KC_D2H: the host entry point's
// copies of the caller's boxes)
enum KClass {
    KC_SMOOTH0 = 0,
    KC_RESTRICT = 1,
    KC_PROLONG = 2,
    KC_NORM = 3,
    KC_COARSE = 4,
    KC_H2D = 5,
    KC_D2H = 6,
    KC_COUNT = 7
};

}  // namespace saras

struct saras_mg {
    saras::HostGrid grid;
    saras_mg_params prm{};
    bool d3 = true;
    int nl = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t cap_stream = nullptr;
    std::vector<saras::Level> lv;
    saras::Ghost ghost{};
    double *walls = nullptr;
    // residual-norm scratch
    double *norm_part = nullptr;
    double *norm_out = nullptr;   // device: [0] residualVal, [1] numerator, [2] denominator
    double *norm_host = nullptr;  // pinned mirror of norm_out
    int norm_blocks = 0;
    int *coarse_sweeps = nullptr;
    // staging of caller host fields (dense padded boxes)
    double *stage_lhs = nullptr, *stage_rhs = nullptr;
    int64_t stage_elems = 0;
    int64_t stage_st[3] = {0, 0, 0};
    // mixed form scratch
    double *mix_scalar = nullptr;
    // graph of one V-cycle (plus the norm and its host copy)
    cudaGraphExec_t graph = nullptr;
    bool use_graph = true;
    // MIXED form with adaptive inner counts: V-cycles of the current outer
    // iteration (0: the full count), graphs of one V-cycle and of the outer
    // iteration's tail for shortened iterations, and the V-cycles of the
    // last solve
    int inner_now = 0;
    cudaGraphExec_t graph_v = nullptr, graph_tail = nullptr;
    int64_t launches_v = 0, launches_tail = 0;
    int64_t last_vcycles = 0;
    // MIXED form: first level of the V-cycle's bottom run by one block in
    // shared memory (k_bottom, with the coarsest solve), -1 for none
    int bottom = -1;
    size_t bottom_smem = 0;
    // the serving engine's hierarchies: its batched kernels address the
    // FP32 arrays in the plain layout, so the finest level is never row-split
    bool no_rowsplit = false;
    int64_t launches_cycle = 0;
    int64_t last_launches = 0;
    int64_t dev_bytes = 0;
    // device memory: the hierarchy made by saras_mg_create is carved out of
    // one allocation (arena); allocations made later, or that do not fit it,
    // are listed in allocs
    char *arena = nullptr;
    size_t arena_cap = 0, arena_used = 0;
    bool carving = false;
    std::vector<void *> allocs;
    // polls of the TMA sweeps' pipeline waits (0: the kernels' default)
    unsigned wait_limit = 0;
    // kernel timing
    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    std::vector<std::pair<int, size_t>> ev_marks;  // (class, index of start event)
    std::vector<std::pair<int, size_t>> graph_marks;  // marks baked into the graph
    bool graph_timing = false;
    bool capturing = false;
    // a sequence issued directly while a timed graph exists (a shortened
    // MIXED iteration): its launches record their own marks
    bool timing_direct = false;
    size_t ev_base = 0;  // events [0, ev_base) are the graph's event-record nodes
    bool mark_open = false;
    int64_t kc_launches[saras::KC_COUNT] = {};
    double kc_ms[saras::KC_COUNT] = {};
    double kc_bytes[saras::KC_COUNT] = {};
    cudaEvent_t copy_ev[4] = {nullptr, nullptr, nullptr, nullptr};  // host entry point's copies
    int64_t issued = 0;  // launches issued while recording the current sequence
    int maxCount() const;  // coarsest-level iteration limit (poisson.cc:430-436)
    // pinned staging of table refills (serving retargets)
    char *tab_stage = nullptr;
    size_t tab_stage_bytes = 0, tab_stage_used = 0;
};
