// Kernels of the 2048 x 2048 grid.
#define GT_N 2048
#include "gt_inst.inc"
