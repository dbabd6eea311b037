// Kernels of the 128 x 128 grid.
#define GT_N 128
#include "gt_inst.inc"
