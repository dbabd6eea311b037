// Ensemble pass kernels of the tile family with 8 values per thread.
#define GT_ENS_R 8
#include "gt_ens_kernels.cuh"

namespace gt {
void ens_passes_r8(const EnsLaunch& l, cudaStream_t s) { ens_passes<8>(l, s); }
cudaError_t ens_prepare_r8() { return ens_prepare<8>(); }
}  // namespace gt
