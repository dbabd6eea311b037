// Kernels of the 512 x 512 grid.
#define GT_N 512
#include "gt_inst.inc"
