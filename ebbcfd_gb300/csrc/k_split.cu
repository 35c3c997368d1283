// k_split.cu -- split-precision instantiation of the stage kernels (sm_103a): FP32
// face, flux, gradient and limiter arithmetic with multiply-add contraction and the
// approximate FP32 division and square root (a few units in the last place, FP32
// denormals flushed); the solution update and the grid-wide reductions inside
// k_update run in FP64.
#include "kernels.cuh"

EBB_INSTANTIATE(float)
