// gt_ens_kernels.cuh -- the pass kernels of the batched ensembles, by tile family.
//
// Each family is compiled in a translation unit of its own (gt_ens_r16.cu, gt_ens_r8.cu,
// gt_ens_r4.cu, which define GT_ENS_R) so that the three compile in parallel; gt_ens.cu launches
// them through ens_passes_r<R> and prepares them through ens_prepare_r<R>.
#pragma once

#include <cuda_runtime.h>

#include "gt_kernels.cuh"

namespace gt {

// One step's passes of an ensemble: work lists of the column and row passes, the per-stage
// arguments of every member ([stages][nm]).
struct EnsLaunch {
  int ncol, nrow, stages, nm;
  const NltArgs* args;
  const EnsTile* col;
  const EnsTile* row;
};

void ens_passes_r16(const EnsLaunch& l, cudaStream_t s);
void ens_passes_r8(const EnsLaunch& l, cudaStream_t s);
void ens_passes_r4(const EnsLaunch& l, cudaStream_t s);
cudaError_t ens_prepare_r16();
cudaError_t ens_prepare_r8();
cudaError_t ens_prepare_r4();

#ifdef GT_ENS_R
// Tile families of the ensemble passes: R complex values per thread and 2048 / R threads per CTA.
// Every CTA holds 2048 values (C = 2048/N columns or rows of a size-N member) in every family, so
// the work lists and the shared memory do not depend on the family; gt_ens_autotune times the
// families on the ensemble's own members and keeps the fastest. MINB: CTAs per SM requested from
// ptxas (3 for 256 threads caps a thread at 85 registers, as the 8-value tiles need).
template <int R>
struct EnsFam {
  static constexpr int THREADS = 2048 / R;
  static constexpr int MINB = R == 8 ? kEnsMinBlocks : R == 16 ? 3 : 2;
};

template <int R>
__global__ void __launch_bounds__(EnsFam<R>::THREADS, EnsFam<R>::MINB)
k_ens_colinv(const NltArgs* __restrict__ args, const EnsTile* __restrict__ tiles) {
  const EnsTile w = tiles[blockIdx.x];
  const NltArgs a = args[w.member];
  switch (a.n) {
    case 128: colinv_tile<128, 16, R>(a, w.tile); break;
    case 256: colinv_tile<256, 8, R>(a, w.tile); break;
    case 512: colinv_tile<512, 4, R>(a, w.tile); break;
    case 1024: colinv_tile<1024, 2, R>(a, w.tile); break;
    case 2048: colinv_tile<2048, 1, R>(a, w.tile); break;
    default: break;
  }
}

template <int R>
__global__ void __launch_bounds__(EnsFam<R>::THREADS, EnsFam<R>::MINB)
k_ens_row(const NltArgs* __restrict__ args, const EnsTile* __restrict__ tiles) {
  const EnsTile w = tiles[blockIdx.x];
  const NltArgs a = args[w.member];
  switch (a.n) {
    case 128: row_tile<128, 16, R>(a, w.tile); break;
    case 256: row_tile<256, 8, R>(a, w.tile); break;
    case 512: row_tile<512, 4, R>(a, w.tile); break;
    case 1024: row_tile<1024, 2, R>(a, w.tile); break;
    case 2048: row_tile<2048, 1, R>(a, w.tile); break;
    default: break;
  }
}

template <int R>
__global__ void __launch_bounds__(EnsFam<R>::THREADS, EnsFam<R>::MINB)
k_ens_colfwd(const NltArgs* __restrict__ args, const EnsTile* __restrict__ tiles) {
  const EnsTile w = tiles[blockIdx.x];
  const NltArgs a = args[w.member];
  switch (a.n) {
    case 128: colfwd_tile<128, 16, R>(a, w.tile); break;
    case 256: colfwd_tile<256, 8, R>(a, w.tile); break;
    case 512: colfwd_tile<512, 4, R>(a, w.tile); break;
    case 1024: colfwd_tile<1024, 2, R>(a, w.tile); break;
    case 2048: colfwd_tile<2048, 1, R>(a, w.tile); break;
    default: break;
  }
}

// pass C of stage cur[m] fused with pass A of stage next[m] (same tiles)
template <int R>
__global__ void __launch_bounds__(EnsFam<R>::THREADS, EnsFam<R>::MINB)
k_ens_colfwd_inv(const NltArgs* __restrict__ cur, const NltArgs* __restrict__ next,
                 const EnsTile* __restrict__ tiles) {
  const EnsTile w = tiles[blockIdx.x];
  const NltArgs a = cur[w.member];
  const NltArgs b = next[w.member];
  switch (a.n) {
    case 128: colfwd_colinv_tile<128, 16, R>(a, b, w.tile); break;
    case 256: colfwd_colinv_tile<256, 8, R>(a, b, w.tile); break;
    case 512: colfwd_colinv_tile<512, 4, R>(a, b, w.tile); break;
    case 1024: colfwd_colinv_tile<1024, 2, R>(a, b, w.tile); break;
    case 2048: colfwd_colinv_tile<2048, 1, R>(a, b, w.tile); break;
    default: break;
  }
}

// the passes of one step in tile family R: pass A of stage 0, then per stage pass B and pass C
// fused with the next stage's pass A
template <int R>
void ens_passes(const EnsLaunch& l, cudaStream_t s) {
  constexpr int TH = EnsFam<R>::THREADS;
  k_ens_colinv<R><<<l.ncol, TH, kEnsColSmem, s>>>(l.args, l.col);
  for (int st = 0; st < l.stages; ++st) {
    const NltArgs* a = l.args + (size_t)st * l.nm;
    k_ens_row<R><<<l.nrow, TH, kEnsRowSmem, s>>>(a, l.row);
    if (st + 1 < l.stages)
      k_ens_colfwd_inv<R><<<l.ncol, TH, kEnsColSmem, s>>>(a, a + l.nm, l.col);
    else
      k_ens_colfwd<R><<<l.ncol, TH, kEnsColSmem, s>>>(a, l.col);
  }
}

template <int R>
cudaError_t ens_prepare() {
  const cudaFuncAttribute attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
  cudaError_t c = cudaFuncSetAttribute(k_ens_colinv<R>, attr, (int)kEnsColSmem);
  if (c == cudaSuccess) c = cudaFuncSetAttribute(k_ens_colfwd<R>, attr, (int)kEnsColSmem);
  if (c == cudaSuccess) c = cudaFuncSetAttribute(k_ens_colfwd_inv<R>, attr, (int)kEnsColSmem);
  if (c == cudaSuccess) c = cudaFuncSetAttribute(k_ens_row<R>, attr, (int)kEnsRowSmem);
  return c;
}
#endif  // GT_ENS_R

}  // namespace gt
