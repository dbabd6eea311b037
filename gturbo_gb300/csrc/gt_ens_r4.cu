// Ensemble pass kernels of the tile family with 4 values per thread.
#define GT_ENS_R 4
#include "gt_ens_kernels.cuh"

namespace gt {
void ens_passes_r4(const EnsLaunch& l, cudaStream_t s) { ens_passes<4>(l, s); }
cudaError_t ens_prepare_r4() { return ens_prepare<4>(); }
}  // namespace gt
