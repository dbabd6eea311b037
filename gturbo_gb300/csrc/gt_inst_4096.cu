// Kernels of the 4096 x 4096 grid.
#define GT_N 4096
#include "gt_inst.inc"
