// Ensemble pass kernels of the tile family with 16 values per thread.
#define GT_ENS_R 16
#include "gt_ens_kernels.cuh"

namespace gt {
void ens_passes_r16(const EnsLaunch& l, cudaStream_t s) { ens_passes<16>(l, s); }
cudaError_t ens_prepare_r16() { return ens_prepare<16>(); }
}  // namespace gt
