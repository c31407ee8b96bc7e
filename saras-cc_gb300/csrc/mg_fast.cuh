// FP64 and MIXED forms of the multigrid solve (mg_fast.cu) and the host
// helpers the translation units share.
#pragma once

#include "mg_handle.cuh"

namespace saras {

// Kernel-class event timing (mg.cu)
void kbegin(saras_mg *h, cudaStream_t s, int kc);
void kend(saras_mg *h, cudaStream_t s, int kc);
void harvest_timing(saras_mg *h);

// mg_fast.cu
saras_status fast_setup(saras_mg *h);          // per-cell inverse diagonals, checks
void fast_cycle(saras_mg *h, cudaStream_t s);  // one V-cycle / outer iteration + norm
void mixed_prepare(saras_mg *h, cudaStream_t s);
void mixed_finish(saras_mg *h, cudaStream_t s);
void final_ghosts(saras_mg *h, cudaStream_t s);
double kernel_bytes(const saras_mg *h, int kclass);
void rhs_norm(saras_mg *h, cudaStream_t s);       // max|f| (or sums) of the solve, once
void coarsest_fast(saras_mg *h, cudaStream_t s, Level &c);

// mg_tma.cu: TMA-staged FP32 colour sweep of the large 3-D levels
void tma_plan(saras_mg *h, Level &v);
bool tma_colour(saras_mg *h, cudaStream_t s, Level &v, int colour);

// mg.cu: handle reuse by the serving engine
saras_status mg_retarget(saras_mg *h, const saras_grid_desc *gd);
saras_status mg_load_rhs(saras_mg *h, const double *rhs_box_origin, const int64_t st[3]);
void mg_store_lhs(saras_mg *h, double *box_origin, const int64_t st[3]);
int64_t mg_estimate_bytes(const saras_grid_desc *gd, const saras_mg_params *prm);

}  // namespace saras
