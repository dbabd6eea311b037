// Kernels of the 16 x 16 grid.
#define GT_N 16
#include "gt_inst.inc"
