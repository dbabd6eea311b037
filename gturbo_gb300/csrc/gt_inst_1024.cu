// Kernels of the 1024 x 1024 grid.
#define GT_N 1024
#include "gt_inst.inc"
