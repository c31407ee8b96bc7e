// FP64 and MIXED forms of the multigrid solve (mg_fast.cu) and the host
// helpers the translation units share.
#pragma once

#include "mg_handle.cuh"

namespace saras {

// Kernel-class event timing (mg.cu)
void kbegin(saras_mg *h, cudaStream_t s, int kc);
void kend(saras_mg *h, cudaStream_t s, int kc);
void harvest_timing(saras_mg *h, bool from_graph);

// mg_fast.cu
saras_status fast_setup(saras_mg *h);          // per-cell inverse diagonals, checks
void fast_cycle(saras_mg *h, cudaStream_t s);  // one V-cycle / outer iteration + norm
// the MIXED outer iteration in pieces (adaptive inner counts)
void vcycle_fast(saras_mg *h, cudaStream_t s, bool mixed);
void mixed_head(saras_mg *h, cudaStream_t s);
void mixed_tail(saras_mg *h, cudaStream_t s);
int mixed_inner(const saras_mg *h);
void mixed_prepare(saras_mg *h, cudaStream_t s);
void mixed_finish(saras_mg *h, cudaStream_t s);
void final_ghosts(saras_mg *h, cudaStream_t s);
double kernel_bytes(const saras_mg *h, int kclass);
void rhs_norm(saras_mg *h, cudaStream_t s);       // max|f| (or sums) of the solve, once
void coarsest_fast(saras_mg *h, cudaStream_t s, Level &c);

template <class T>
struct Tab3;  // mg_stencil.cuh
template <class T>
struct WTab;

// mg_tma.cu: TMA-staged FP32 colour sweep of the large 3-D levels
void tma_plan(saras_mg *h, Level &v);
bool tma_colour(saras_mg *h, cudaStream_t s, Level &v, int colour);
bool tma_fused(saras_mg *h, cudaStream_t s, Level &v, bool to_b);
bool fused_sweep_fits(const Lay &L, bool d3);
bool fused_rowsplit_fits(const Lay &L, bool d3);
bool tma_resid_restrict(saras_mg *h, cudaStream_t s, Level &f, Level &c, const Tab3<float> &t,
                        const WTab<float> &w, float *z32);
bool pair_sweep_fits(const Lay &L, bool d3);  // mg_fast.cu: levels of k_rbgs_pair

// mg.cu: handle reuse by the serving engine
saras_status mg_retarget(saras_mg *h, const saras_grid_desc *gd);
saras_status mg_load_rhs(saras_mg *h, const double *rhs_box_origin, const int64_t st[3]);
void mg_store_lhs(saras_mg *h, double *box_origin, const int64_t st[3]);
int64_t mg_estimate_bytes(const saras_grid_desc *gd, const saras_mg_params *prm);
saras_status mg_create_queued(const saras_grid_desc *gd, const saras_mg_params *prm, void *stream,
                              saras_mg **out);

// rk3.cu: the time step in halves around its pressure solves, for the
// serving engine, which runs those solves in its batch
int rk3_stages(const saras_rk3 *h);                          // 3 (lsRK3) or 1 (eulerCN)
saras_status rk3_stage_begin(saras_rk3 *h, int stage);       // RHS, CN sweeps, divergence into lv[0].rhs
saras_status rk3_stage_end(saras_rk3 *h, int stage);         // P += Pp, V -= grad Pp, BCs
saras_mg *rk3_multigrid(saras_rk3 *h);
int64_t rk3_device_bytes(const saras_rk3 *h);                // the integrator's fields and tables
// re-points a handle at another stretching of the same shape (and new
// parameters); fields cleared as at creation
saras_status rk3_retarget(saras_rk3 *h, const saras_grid_desc *gd, const saras_rk3_params *prm);
int64_t rk3_estimate_bytes(const saras_grid_desc *gd, const saras_rk3_params *prm);  // with its hierarchy

}  // namespace saras
