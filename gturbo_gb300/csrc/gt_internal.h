// gt_internal.h -- host helpers shared by the C-ABI translation units (not part of the ABI).
#pragma once

#include "../../include/gturbo.h"
#include "gt_kernels.cuh"

namespace gt {

// Arguments of one nonlinear-term evaluation of a field with the tables of handle h
// (epilogue defaults: EPI_NLT with h's integrating factor and time steps).
NltArgs handle_nlt_args(const gt_handle* h, const double* zin, double* q, double* u, double* v,
                        int* flag);

}  // namespace gt

namespace gt {

// Forced-mode table of a handle (device pointers) and its kick amplitude sqrt(dt)*famp.
struct ForcingView {
  const int* ikx;
  const int* iky;
  const int* jc;
  int nf;
  int nh;
  double sf;
  const uint32_t* lcga;  // LCG jump-ahead of the (k+1)-th draw
  const uint32_t* lcgb;
  uint32_t lcga_nf, lcgb_nf;  // jump-ahead of a whole kick (nf draws)
  double sdt;
};
ForcingView handle_forcing(const gt_handle* h);
// Launch one kernel of the handle's grid size.
cudaError_t handle_dispatch(const gt_handle* h, const struct GtOp& op);
// The LCG kick of gt_forcing with amplitude famp (the handle's own famp in gt_forcing);
// seed0 is the LCG state before the kick.
cudaError_t forcing_amp(gt_handle* h, double* z, uint32_t seed0, double famp);
// k^2 tables of the handle
void handle_k2(const gt_handle* h, const double** fkxs, const double** fkys);
// the handle's untruncated-input flag (used by its single-field nonlinear-term passes)
int* handle_flag(const gt_handle* h);

// Grid size, RK order and the parameters a handle was created with.
const gt_params* handle_params(const gt_handle* h);
int handle_rko(const gt_handle* h);
// Launch variants of the column and row passes (nonlinear term, tangent-linear, adjoint).
int handle_variant(const gt_handle* h);
int handle_row_variant(const gt_handle* h);
// whether the field-split column passes run for this handle (size, column variant, setting)
bool handle_col_split(const gt_handle* h);
// whether the split pass C runs as clusters (gt_set_col_split mode 2)
bool handle_col_cluster(const gt_handle* h);
// whether the pass kernels launch with programmatic dependent launch (setting, profiling off)
bool handle_pdl(const gt_handle* h);
// device memory gt_adj_gradient may hold for whole kept segments (gt_adj_set_memory)
int64_t handle_adj_memory(const gt_handle* h);
// Records msg as h's last error (h == NULL: the thread's create/no-handle error); returns code.
int set_error(gt_handle* h, int code, const char* msg);

}  // namespace gt

namespace gt {
cudaStream_t handle_stream(const gt_handle* h);
}  // namespace gt
