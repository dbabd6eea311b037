// Kernels of the 8192 x 8192 grid.
#define GT_N 8192
#include "gt_inst.inc"
