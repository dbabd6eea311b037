// Kernels of the 64 x 64 grid.
#define GT_N 64
#include "gt_inst.inc"
