// Kernels of the 32 x 32 grid.
#define GT_N 32
#include "gt_inst.inc"
