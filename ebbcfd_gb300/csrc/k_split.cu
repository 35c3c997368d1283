// k_split.cu -- split-precision instantiation of the stage kernels (sm_103a): FP32
// face, flux, gradient and limiter arithmetic with multiply-add contraction; the
// solution update and the reductions inside k_update run in FP64.
#include "kernels.cuh"

EBB_INSTANTIATE(float)
