// Kernels of the 256 x 256 grid.
#define GT_N 256
#include "gt_inst.inc"
