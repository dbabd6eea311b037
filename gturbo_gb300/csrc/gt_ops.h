// gt_ops.h -- host-side description of one kernel launch, dispatched to the per-N
// instantiation units (gt_inst_<N>.cu) so that every grid size compiles in parallel.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gt_adjoint.cuh"
#include "gt_kernels.cuh"

namespace gt {

enum OpKind : int {
  OP_NLT_COLINV = 0,  // pass A
  OP_NLT_ROW = 1,     // pass B
  OP_NLT_COLFWD = 2,  // pass C (+ epilogue)
  OP_COL_INV = 3,     // column inverse transform (fft_inv, first half)
  OP_COL_FWD = 4,     // column forward transform, scaled (fft_dir, second half)
  OP_ROW_C2R = 5,     // row C2R (fft_inv, second half)
  OP_ROW_R2C = 6,     // row R2C (fft_dir, first half)
  OP_TLM_COLINV = 7,  // tangent-linear passes (N <= 4096)
  OP_TLM_ROW = 8,
  OP_TLM_COLFWD = 9,
  OP_ADJ_COLINV = 10, // adjoint passes (N <= 4096)
  OP_ADJ_ROW = 11,
  OP_ADJ_COLFWD = 12,
  OP_NLT_COLFWD_INV = 13,  // pass C of stage nlt + pass A of stage nlt2
  OP_ROW_C2R_F32 = 14,     // row C2R of `a` written as floats to `f32` (dumps)
  OP_ROW_R2C_F32 = 15,     // row R2C of the floats `f32` into `a` (restarts)
  OP_NLT_COLINV_FS = 16,   // pass A split by field (q must not alias zin)
  OP_NLT_COLFWD_FS = 17,   // pass C split by field, epilogue by the column's second CTA (or,
                           // with GtOp::cluster, by both CTAs of the column's 2-CTA cluster)
  OP_ADJ_COLINV_FS = 18,   // transposed pass A split by field
  OP_ADJ_COLFWD_FS = 19,   // transposed pass C split by field, update by the column's third CTA
  OP_TLM_COLINV_FS = 20,   // tangent pass A split by field
  OP_TLM_COLFWD_FS = 21,   // tangent pass C split by field, update by the column's fourth CTA
};

struct GtOp {
  int kind;
  int variant;        // launch variant of the column passes (Var<N, V>, V in 0..4)
  int row_variant;    // launch variant of the row passes (0, 1, 2: 16, 8, 4 values per thread)
  cudaStream_t stream;
  NltArgs nlt;        // passes A, B, C
  NltArgs nlt2;       // the next stage (OP_NLT_COLFWD_INV)
  TlmArgs tlm;
  AdjArgs adj;
  double2* a;         // field of the standalone transforms
  float* f32;         // real(4) output of OP_ROW_C2R_F32
  const double2* tw;  // twiddle buffer of the column transforms (length NY)
  const double2* twr; // twiddle buffer of the row transforms (length NX)
  double scale;
  int nh;             // columns of the field, NX/2+1: the grid of the column passes
  int nrows;          // rows of the field, NY: the grid of the row passes
  bool rt;            // non-square grid: the column kernels with the column count at run time
  bool pdl;           // launch the pass kernels with programmatic dependent launch
  bool cluster;       // OP_NLT_COLFWD_FS: the column's two CTAs as one cluster
};

// Launches the pass kernel k on stream s. With `pdl` the launch may begin while the previous
// kernel on s drains (programmatic dependent launch); only kernels whose first statement is
// pdl_enter() are launched this way. The error, if any, is left for cudaGetLastError.
template <typename... KArgs, typename... Args>
inline void launch_pass(bool pdl, cudaStream_t s, void (*k)(KArgs...), unsigned grid, unsigned block, size_t smem,
                        Args... args) {
  cudaLaunchAttribute at;
  at.id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at.val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = &at;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, k, args...);
}

// CTAs of a column pass over nh columns, C per CTA, and of a row pass over nrows rows, ROWS per
// CTA (the handle keeps nrows a multiple of ROWS).
inline unsigned col_ctas(int nh, int cols) { return (unsigned)((nh + cols - 1) / cols); }
inline unsigned row_ctas(int nrows, int rows) { return (unsigned)(nrows / rows); }
// Row passes run in the instantiation of the row length NX, column passes in that of the column
// length NY.
inline bool is_row_op(int kind) {
  return kind == OP_NLT_ROW || kind == OP_ROW_C2R || kind == OP_ROW_R2C || kind == OP_ROW_C2R_F32 ||
         kind == OP_ROW_R2C_F32 || kind == OP_TLM_ROW || kind == OP_ADJ_ROW;
}

// Per-N entry points (defined in gt_inst_<N>.cu).
#define GT_DECLARE_N(NN)                              \
  cudaError_t prepare_##NN();                         \
  cudaError_t dispatch_##NN(const GtOp& op);
GT_DECLARE_N(16)
GT_DECLARE_N(32)
GT_DECLARE_N(64)
GT_DECLARE_N(128)
GT_DECLARE_N(256)
GT_DECLARE_N(512)
GT_DECLARE_N(1024)
GT_DECLARE_N(2048)
GT_DECLARE_N(4096)
GT_DECLARE_N(8192)
#undef GT_DECLARE_N

}  // namespace gt
